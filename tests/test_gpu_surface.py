"""The steps after the solve, through the C ABI against the oracle: extruded
smooth normals (shaders/FEM/smooth_normals.glsl) and the .ply export
(Surface::export_to_ply).  Both are float arithmetic rounded at every
operation in the reference's order, so the bar is bit-exact; the normals sum
in ascending triangle order on both sides."""
import numpy as np
import pytest

from fea_gb300 import meshgen as mg

pytestmark = pytest.mark.gpu


def _gs_handle(fea, xyz, tri, bc, u, v):
    p = fea.default_params(equation=fea.REACTION_DIFFUSION, reaction_mode=1)
    s = fea.CUDASolver(xyz, tri, boundary_condition=bc, params=p)
    s.set_fields(u, v)
    return s


def _cases():
    ico = mg.icosphere(3)
    grid = mg.jittered_grid(33, seed=5)
    return [("ico3", ico, 1, ico[0] / np.linalg.norm(ico[0], axis=1, keepdims=True)),
            ("grid33", grid, 0, np.tile([0.0, 0.0, 1.0], (len(grid[0]), 1)))]


@pytest.mark.parametrize("case", [0, 1])
@pytest.mark.parametrize("extrusion", [0.0, 0.35, 4.0])
def test_smooth_normals_bit_exact(fea, oracle_mod, case, extrusion):
    name, (xyz, tri), bc, nrm = _cases()[case]
    rng = np.random.default_rng(3)
    u = rng.uniform(0, 1, len(xyz)).astype(np.float32)
    v = rng.uniform(-0.5, 1, len(xyz)).astype(np.float32)
    s = _gs_handle(fea, xyz, tri, bc, u, v)
    vals = s.get_values()  # the displayed field (v), 0 on Dirichlet points
    got = s.smooth_normals(nrm, extrusion)
    ref = oracle_mod.smooth_normals(xyz, tri, nrm, vals, extrusion)
    np.testing.assert_array_equal(got, ref)


@pytest.mark.parametrize("case", [0, 1])
@pytest.mark.parametrize("mesh_type", [0, 1, 2])
@pytest.mark.parametrize("threshold", [-1.0, 0.3, 2.0])
def test_ply_geometry_bit_exact(fea, oracle_mod, case, mesh_type, threshold):
    name, (xyz, tri), bc, nrm = _cases()[case]
    rng = np.random.default_rng(4)
    u = rng.uniform(0, 1, len(xyz)).astype(np.float32)
    v = (0.5 + 0.4 * np.sin(4 * xyz[:, 0]) * np.cos(3 * xyz[:, 1])).astype(np.float32)
    s = _gs_handle(fea, xyz, tri, bc, u, v)
    vals = s.get_values()
    P, pv, T = s.ply_geometry(nrm, 0.25, threshold, mesh_type)
    Po, pvo, To = oracle_mod.ply_clip(xyz, tri, nrm, vals, 0.25, threshold, mesh_type)
    np.testing.assert_array_equal(P, Po)
    np.testing.assert_array_equal(pv, pvo)
    np.testing.assert_array_equal(T, To)
    if threshold > 1.5:
        assert len(P) == 0 and len(T) == 0


def test_export_ply_file(fea, oracle_mod, tmp_path):
    (xyz, tri) = mg.icosphere(2)
    nrm = xyz / np.linalg.norm(xyz, axis=1, keepdims=True)
    v = (0.5 + 0.5 * xyz[:, 2]).astype(np.float32)
    s = _gs_handle(fea, xyz, tri, 1, np.ones(len(xyz), np.float32), v)
    coeffs = np.random.default_rng(7).uniform(-1, 1, (7, 3)).astype(np.float32)
    path = tmp_path / "out.ply"
    s.export_ply(str(path), nrm, 0.25, 0.4, fea.binding.MESH_MIRRORED, coeffs)
    P, pv, T = oracle_mod.ply_clip(xyz, tri, nrm, s.get_values(), 0.25, 0.4, 2)
    lines = path.read_text().splitlines()
    header = ["ply", "format ascii 1.0", f"element vertex {len(P)}", "property float x", "property float y",
              "property float z", "property float red", "property float green", "property float blue",
              f"element face {len(T)}", "property list uchar uint vertex_indices", "end_header"]
    assert lines[:12] == header
    verts = np.array([[np.float32(x) for x in ln.split()] for ln in lines[12:12 + len(P)]], dtype=np.float32)
    np.testing.assert_array_equal(verts[:, :3], P)
    col = np.repeat(coeffs[6][None, :], len(pv), axis=0)
    for k in range(5, -1, -1):  # c0 + t (c1 + t (... + t c6)) in float32
        col = coeffs[k][None, :] + pv[:, None] * col
    np.testing.assert_array_equal(verts[:, 3:], col.astype(np.float32))
    faces = np.array([[int(x) for x in ln.split()] for ln in lines[12 + len(P):]], dtype=np.int64)
    assert np.all(faces[:, 0] == 3)
    np.testing.assert_array_equal(faces[:, 1:], T.astype(np.int64))


def test_export_arguments(fea, tmp_path):
    xyz, tri = mg.icosphere(1)
    s = _gs_handle(fea, xyz, tri, 1, np.ones(len(xyz), np.float32), np.zeros(len(xyz), np.float32))
    with pytest.raises(fea.FeaError):
        s.export_ply(str(tmp_path / "x.ply"), xyz, 0.25, 0.0, 7)
    with pytest.raises(fea.FeaError):
        s.export_ply(str(tmp_path / "missing_dir" / "x.ply"), xyz, 0.25, 0.0, 0)
