"""CPU tests of the synthetic mesh generators and the OBJ reader."""
import numpy as np
import pytest

from conftest import REFERENCE_ASSETS, has_reference_assets, reference_meshes
from fea_gb300 import meshgen as mg


@pytest.mark.parametrize("level", [0, 1, 3, 5])
def test_icosphere_sizes_and_orientation(level):
    xyz, tri = mg.icosphere(level)
    assert xyz.shape == (10 * 4 ** level + 2, 3) and tri.shape == (20 * 4 ** level, 3)
    assert np.allclose(np.linalg.norm(xyz, axis=1), 1, atol=1e-6)
    v = xyz.astype(np.float64)
    a, b, c = v[tri[:, 0]], v[tri[:, 1]], v[tri[:, 2]]
    n = np.cross(b - a, c - a)
    assert np.all(np.einsum("ij,ij->i", n, a + b + c) > 0)  # outward winding


def test_icosphere_deterministic():
    a = mg.icosphere(3)
    b = mg.icosphere(3)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


@pytest.mark.parametrize("n", [2, 5, 64])
def test_grid_sizes(n):
    xyz, tri = mg.jittered_grid(n, seed=3)
    assert xyz.shape == (n * n, 3) and tri.shape == (2 * (n - 1) ** 2, 3)
    v = xyz.astype(np.float64)
    a, b, c = v[tri[:, 0]], v[tri[:, 1]], v[tri[:, 2]]
    area = 0.5 * np.cross(b - a, c - a)[:, 2]
    assert np.all(area > 0)
    assert abs(area.sum() - 1.0) < 1e-5
    assert xyz[:, 0].min() == 0 and xyz[:, 0].max() == 1


def test_grid_seed_changes_mesh():
    a = mg.jittered_grid(16, seed=1)
    b = mg.jittered_grid(16, seed=2)
    assert not np.array_equal(a[1], b[1])


def test_config2_grid_counts():
    """1024^2 grid: V 1,048,576, T 2,093,058 (nnz 7,331,842 = V + 2E)."""
    xyz, tri = mg.jittered_grid(1024, seed=0)
    assert xyz.shape[0] == 1048576 and tri.shape[0] == 2093058
    n = 1024
    assert xyz.shape[0] + 2 * (n - 1) * (3 * n - 1) == 7331842


def test_cylinder_boundary_loops():
    xyz, tri = mg.cylinder(24, 10)
    ob = mg.boundary_vertices(tri, xyz.shape[0])
    assert ob.sum() == 48


def test_initial_fields():
    xyz, _ = mg.jittered_grid(128, seed=0)
    u, v = mg.gray_scott_patches(xyz, seed=0)
    assert u.dtype == np.float32 and 0 <= u.min() and u.max() <= 1
    assert np.sum(v > 0.2) > 0 and np.mean(u) > 0.8


def test_reference_mesh_fixture():
    m = reference_meshes()
    xyz, tri = m["icosphere"]
    assert xyz.shape == (10242, 3) and tri.shape == (20480, 3)
    xyz, tri = m["tube"]
    assert xyz.shape == (4704, 3) and tri.shape == (9216, 3)
    assert mg.boundary_vertices(tri, xyz.shape[0]).sum() == 192


@pytest.mark.skipif(not has_reference_assets(), reason="FEA_REFERENCE_ASSETS not set")
def test_read_reference_obj():
    xyz, tri = mg.read_obj(REFERENCE_ASSETS + "/icosphere.obj")
    assert xyz.shape == (10242, 3) and tri.shape == (20480, 3)
    xyz, tri = mg.read_obj(REFERENCE_ASSETS + "/tube.obj")
    assert xyz.shape == (4704, 3) and tri.shape == (9216, 3)
    assert mg.boundary_vertices(tri, xyz.shape[0]).sum() == 192
