"""GPU tests on the reference's own meshes and on malformed meshes.

- icosphere.obj and tube.obj of the reference (committed as
  tests/golden/reference_meshes.npz) go through fea_create with
  on_boundary = NULL, so boundary detection runs on the device as
  Surface::init_from_obj does (Surface.cpp:104-122); the pattern is checked
  against the golden checksums (FEMContext.cpp:97-112) and a few steps
  against the oracle.
- Malformed meshes are refused with FEA_ERR_BAD_MESH and leave the device
  usable (the reference throws on malformed input, Surface.cpp:40-41, 59-74;
  it builds NaN element matrices from zero-area triangles).  A duplicated
  triangle is valid input and matches the oracle.
"""
import hashlib
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, device_field, oracle_step, reference_meshes, rel_l2
from fea_gb300 import meshgen as mg

pytestmark = pytest.mark.gpu

FEA_ERR_BAD_MESH = -4


def _gold():
    with open(os.path.join(GOLDEN, "reference_meshes.json")) as fh:
        return json.load(fh)["meshes"]


@pytest.mark.parametrize("name", ["icosphere", "tube"])
@pytest.mark.parametrize("bc", [0, 1])
def test_reference_mesh_on_device(fea, oracle_mod, name, bc):
    xyz, tri = reference_meshes()[name]
    s = fea.CUDASolver(xyz, tri, boundary_condition=bc, precision=fea.FP64,
                       params=fea.default_params(equation=fea.HEAT, heat_time_step=0.01, heat_conductivity=0.05,
                                                 cg_tolerance=1e-12))
    S = oracle_mod.System(xyz, tri, bc=bc)
    inf = s.info
    idx, ob = s.idx_map()
    np.testing.assert_array_equal(ob, S.on_boundary)
    np.testing.assert_array_equal(idx, S.idx)
    assert inf.num_boundary_points == S.num_boundary == (192 if name == "tube" else 0)
    assert (inf.num_unknowns, inf.nnz, inf.max_row_nonzeros) == (S.N, S.nnz, S.max_row_nonzeros)
    rp, col, _, _ = s.matrix(fea.STIFFNESS)
    np.testing.assert_array_equal(rp, S.row_ptr)
    np.testing.assert_array_equal(col, S.col)
    gold = _gold()[name]
    if gold["bc"] == bc:  # the golden summaries: icosphere Neumann, tube Dirichlet
        assert inf.nnz == gold["nnz"] == (71682 if name == "icosphere" else 31200)
        assert hashlib.sha256(rp.tobytes()).hexdigest() == gold["row_ptr_sha256"]
        assert hashlib.sha256(col.tobytes()).hexdigest() == gold["col_sha256"]
    # three heat steps from z^2, FP64 against the oracle
    u0 = (xyz[:, 2].astype(np.float64) ** 2).astype(np.float32)
    s.set_values(u0)
    s.advance_time(3)
    uo, *_ = oracle_step(oracle_mod, S, oracle_mod.HEAT, 0.01, S.gather(u0), np.zeros(S.N), 3, kappa=0.05)
    assert rel_l2(s.get_values(), S.scatter(uo)) < 1e-7  # float32 node values
    assert rel_l2(device_field(s, 0), uo) < 1e-9  # the FP64 state
    s.close()


def _bad(fea, xyz, tri):
    with pytest.raises(fea.FeaError) as e:
        fea.CUDASolver(xyz, tri, boundary_condition=fea.NEUMANN)
    return e.value


def _grid():
    return mg.jittered_grid(9, seed=1)


def test_bad_meshes_refused(fea, oracle_mod):
    cases = {}
    xyz, tri = _grid()
    t = tri.copy()
    t[5] = [t[5, 0], t[5, 0], t[5, 1]]  # repeated corner: zero area
    cases["repeated corner"] = (xyz, t)
    x = xyz.copy()
    a, b, c = tri[7]
    x[a], x[b], x[c] = (0.25, 0.25, 0.0), (0.5, 0.5, 0.0), (0.75, 0.75, 0.0)  # collinear, exact in binary
    cases["collinear"] = (x, tri)
    x = xyz.copy()
    a, b, c = tri[3]
    x[b] = x[a]
    x[c] = x[a]  # all corners at one point: zero area
    cases["zero area"] = (x, tri)
    x = xyz.copy()
    x[11, 1] = np.nan
    cases["nan coordinate"] = (x, tri)
    x = xyz.copy()
    x[4, 0] = np.inf
    cases["inf coordinate"] = (x, tri)
    t = tri.copy()
    t[2, 1] = xyz.shape[0]  # index >= V
    cases["index out of range"] = (xyz, t)
    msgs = {}
    for name, (xx, tt) in cases.items():
        err = _bad(fea, xx, tt)
        assert err.code == FEA_ERR_BAD_MESH, (name, err)
        msgs[name] = str(err)
    assert "zero area" in msgs["collinear"] and "zero area" in msgs["repeated corner"]
    assert "non-finite" in msgs["nan coordinate"] and "non-finite" in msgs["inf coordinate"]
    assert "out of range" in msgs["index out of range"]
    # the device is still usable: a valid mesh steps to the oracle's result
    s = fea.CUDASolver(xyz, tri, boundary_condition=fea.NEUMANN, precision=fea.FP64,
                       params=fea.default_params(equation=fea.HEAT, heat_time_step=0.01, heat_conductivity=1.0,
                                                 cg_tolerance=1e-12))
    S = oracle_mod.System(xyz, tri, bc=1)
    u0 = np.cos(3 * xyz[:, 0]).astype(np.float32)
    s.set_values(u0)
    s.advance_time(2)
    uo, *_ = oracle_step(oracle_mod, S, oracle_mod.HEAT, 0.01, S.gather(u0), np.zeros(S.N), 2, kappa=1.0)
    assert rel_l2(device_field(s, 0), uo) < 1e-9


@pytest.mark.parametrize("bc", [0, 1])
def test_duplicated_triangle(fea, oracle_mod, bc):
    """A triangle listed twice: its entries are summed twice (setFromTriplets)
    and its edges are used twice for the boundary count, on the device as in
    the oracle."""
    xyz, tri = _grid()
    k = int(np.flatnonzero(np.isin(tri, np.flatnonzero(mg.boundary_vertices(tri, xyz.shape[0]))).any(1))[0])
    tri2 = np.concatenate([tri, tri[k:k + 1]])  # a boundary triangle, twice
    s = fea.CUDASolver(xyz, tri2, boundary_condition=bc, precision=fea.FP64,
                       params=fea.default_params(equation=fea.HEAT, heat_time_step=0.01, heat_conductivity=1.0,
                                                 cg_tolerance=1e-12))
    S = oracle_mod.System(xyz, tri2, bc=bc)
    idx, ob = s.idx_map()
    np.testing.assert_array_equal(ob, S.on_boundary)
    np.testing.assert_array_equal(idx, S.idx)
    rp, col, val, _ = s.matrix(fea.STIFFNESS)
    np.testing.assert_array_equal(rp, S.row_ptr)
    np.testing.assert_array_equal(col, S.col)
    assert np.max(np.abs(val - S.K)) <= 1e-13 * np.abs(S.K).max()
    u0 = np.sin(2 * xyz[:, 1]).astype(np.float32) + 1.0
    s.set_values(u0)
    s.advance_time(2)
    uo, *_ = oracle_step(oracle_mod, S, oracle_mod.HEAT, 0.01, S.gather(u0), np.zeros(S.N), 2, kappa=1.0)
    assert rel_l2(device_field(s, 0), uo) < 1e-9


@pytest.mark.parametrize("bc", [0, 1])
def test_pslg_mesh_steps(fea, oracle_mod, bc):
    """A drawn domain (a square with a square hole, the reference's default
    triangle area 0.005) triangulated by fea_triangulate_pslg goes through
    fea_create with its boundary flags, as Surface::init_from_PSLG hands them
    on (Surface.cpp:472-478), and steps to the oracle's result."""
    sq = np.array([[0, 0], [1, 0], [1, 1], [0, 1]], float)
    hole = np.array([[0.4, 0.4], [0.6, 0.4], [0.6, 0.6], [0.4, 0.6]])
    ring = lambda n, s: np.array([[s + i, s + (i + 1) % n] for i in range(n)])  # noqa: E731
    xyz, tri, ob = fea.triangulate_pslg(np.vstack([sq, hole]), np.vstack([ring(4, 0), ring(4, 4)]), [[0.5, 0.5]],
                                        max_area=0.005)
    s = fea.CUDASolver(xyz, tri, boundary_condition=bc, precision=fea.FP64, on_boundary=ob,
                       params=fea.default_params(equation=fea.HEAT, heat_time_step=0.01, heat_conductivity=0.5,
                                                 cg_tolerance=1e-12))
    S = oracle_mod.System(xyz, tri, bc=bc, on_boundary=ob)
    assert s.info.num_boundary_points == int(ob.sum()) == S.num_boundary
    rp, col, _, _ = s.matrix(fea.STIFFNESS)
    np.testing.assert_array_equal(rp, S.row_ptr)
    np.testing.assert_array_equal(col, S.col)
    u0 = np.sin(np.pi * xyz[:, 0]) * np.sin(np.pi * xyz[:, 2]).astype(np.float32)
    s.set_values(u0.astype(np.float32))
    s.advance_time(3)
    uo, *_ = oracle_step(oracle_mod, S, oracle_mod.HEAT, 0.01, S.gather(u0.astype(np.float32)), np.zeros(S.N), 3,
                         kappa=0.5)
    assert rel_l2(device_field(s, 0), uo) < 1e-9
