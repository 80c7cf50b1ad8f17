"""CPU tests: pin the oracle (the CPU restatement in oracle/) against known answers.

The reference ships no golden vectors, so the oracle is pinned against
closed forms and mesh invariants derived from its source
(FEMContext.cpp:70-240, CPUSolver.cpp:64-146), against scipy for the
linear algebra, and against fixtures generated from the reference's own mesh
assets (tests/golden/, made by tests/golden/make_golden.py).
"""
import json
import os
import sys

import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from conftest import REFERENCE_ASSETS, has_reference_assets, reference_meshes, rel_l2
from fea_gb300 import meshgen as mg

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def unit_triangle():
    xyz = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], dtype=np.float32)
    tri = np.array([[0, 1, 2]], dtype=np.uint32)
    return xyz, tri


def test_single_element_closed_forms(oracle_mod):
    """Stiffness = area * g_i.g_j, mass = |J|/24 (1 + delta_ij) (FEMContext.cpp:103,127-132)."""
    xyz, tri = unit_triangle()
    K, M, A = oracle_mod.element_matrices(xyz, tri, velocity=(1, 0, 0))
    K_ref = 0.5 * np.array([[2, -1, -1], [-1, 1, 0], [-1, 0, 1]], dtype=np.float64)
    M_ref = (1.0 / 24.0) * np.array([[2, 1, 1], [1, 2, 1], [1, 1, 2]])
    np.testing.assert_allclose(K.reshape(3, 3), K_ref, atol=1e-15)
    np.testing.assert_allclose(M.reshape(3, 3), M_ref, atol=1e-15)
    # advection: |J|/6 * t.g_j with t = (1, 0, 0): g = (-1,-1,0), (1,0,0), (0,1,0)
    A_ref = (1.0 / 6.0) * np.array([[-1, 1, 0]] * 3, dtype=np.float64)
    np.testing.assert_allclose(A.reshape(3, 3), A_ref, atol=1e-15)


def test_element_invariance_and_float32(oracle_mod):
    """Rotated/scaled copies: K is scale- and rotation-invariant, M scales with area."""
    rng = np.random.default_rng(3)
    xyz = rng.normal(size=(3, 3)).astype(np.float32)
    tri = np.array([[0, 1, 2]], dtype=np.uint32)
    K, M, _ = oracle_mod.element_matrices(xyz, tri)
    Q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
    xyz2 = (2.0 * xyz.astype(np.float64) @ Q.T).astype(np.float32)
    K2, M2, _ = oracle_mod.element_matrices(xyz2, tri)
    np.testing.assert_allclose(K2, K, rtol=2e-6, atol=1e-7)
    np.testing.assert_allclose(M2, 4 * M, rtol=2e-6)
    K32, M32, _ = oracle_mod.element_matrices(xyz, tri, dtype=np.float32)
    np.testing.assert_allclose(K32, K, rtol=1e-5, atol=1e-6)
    assert abs(K.reshape(3, 3).sum(1)).max() < 1e-12


def test_zero_velocity_tangent_is_zero(oracle_mod):
    """Velocity along the normal: Eigen's normalized() keeps the zero vector (no NaN)."""
    xyz, tri = unit_triangle()
    _, _, A = oracle_mod.element_matrices(xyz, tri, velocity=(0, 0, 1))
    assert np.all(A == 0)


def test_boundary_and_idx_map(oracle_mod):
    n = 9
    xyz, tri = mg.jittered_grid(n, seed=1)
    ob, nb = oracle_mod.boundary(tri, n * n)
    ii, jj = np.meshgrid(np.arange(n), np.arange(n), indexing="xy")
    perim = ((ii == 0) | (jj == 0) | (ii == n - 1) | (jj == n - 1)).ravel()
    assert nb == 4 * (n - 1)
    np.testing.assert_array_equal(ob.astype(bool), perim)
    np.testing.assert_array_equal(ob, mg.boundary_vertices(tri, n * n))
    idx, N = oracle_mod.idx_map(ob, oracle_mod.DIRICHLET)
    assert N == (n - 2) ** 2
    assert np.all(idx[perim] == -1)
    np.testing.assert_array_equal(idx[~perim], np.arange(N))
    idx, N = oracle_mod.idx_map(ob, oracle_mod.NEUMANN)
    np.testing.assert_array_equal(idx, np.arange(n * n))


def test_closed_mesh_has_no_boundary(oracle_mod):
    xyz, tri = mg.icosphere(2)
    ob, nb = oracle_mod.boundary(tri, xyz.shape[0])
    assert nb == 0


def test_degenerate_edge_never_boundary(oracle_mod):
    tri = np.array([[0, 1, 2], [3, 3, 4]], dtype=np.uint32)
    ob, nb = oracle_mod.boundary(tri, 5)
    # triangle 0's three edges are used once; in (3, 3, 4) the edge 3-4 appears
    # twice (as 3->4 and 4->3) and 3-3 counts twice, so 3 and 4 stay interior
    assert list(ob) == [1, 1, 1, 0, 0]


@pytest.mark.parametrize("level", [0, 1, 2, 3])
def test_icosphere_pattern_counts(oracle_mod, level):
    """nnz = V + 2E on a closed mesh; symmetric, sorted columns."""
    xyz, tri = mg.icosphere(level)
    S = oracle_mod.System(xyz, tri, bc=oracle_mod.NEUMANN)
    V = 10 * 4 ** level + 2
    E = 30 * 4 ** level
    assert S.V == V and S.T == 20 * 4 ** level
    assert S.nnz == V + 2 * E
    for r in range(S.N):
        c = S.col[S.row_ptr[r]:S.row_ptr[r + 1]]
        assert np.all(np.diff(c) > 0)
    A = sp.csr_matrix((np.ones(S.nnz), S.col, S.row_ptr), shape=(S.N, S.N))
    assert (A - A.T).nnz == 0


def test_matrix_invariants(oracle_mod):
    """K 1 = 0 (Neumann), sum(M) = area, K x = 0 for linear x at interior points."""
    n = 17
    xyz, tri = mg.jittered_grid(n, seed=5)
    S = oracle_mod.System(xyz, tri, bc=oracle_mod.NEUMANN)
    K = S.scipy("K")
    M = S.scipy("M")
    assert abs(K @ np.ones(S.N)).max() < 1e-12
    assert abs(M.sum() - 1.0) < 1e-6  # float32 coordinates of the unit square
    lin = 0.3 * xyz[:, 0].astype(np.float64) - 0.7 * xyz[:, 1] + 0.1
    r = K @ lin
    assert abs(r[S.on_boundary == 0]).max() < 1e-6
    assert abs(K - K.T).max() == 0.0  # bit-symmetric: same summation order both ways
    assert abs(M - M.T).max() == 0.0


def test_explicit_zeros_kept(oracle_mod):
    """Right triangles: the stiffness coupling across the hypotenuse is exactly 0
    (cot 90 deg) but Eigen keeps the entry (setFromTriplets never prunes)."""
    xyz, tri = mg.jittered_grid(5, seed=0, jitter=0.0)
    S = oracle_mod.System(xyz, tri, bc=oracle_mod.NEUMANN)
    assert np.sum(S.K == 0.0) > 0
    t = tri.astype(np.int64)
    E = np.unique(np.sort(np.concatenate([t[:, [0, 1]], t[:, [1, 2]], t[:, [2, 0]]]), axis=1), axis=0)
    assert S.nnz == S.V + 2 * E.shape[0]


def test_advection_filter_ignores_bc(oracle_mod):
    """Under Neumann the advection triplets still skip boundary points (FEMContext.cpp:188)."""
    xyz, tri = mg.jittered_grid(9, seed=2)
    S = oracle_mod.System(xyz, tri, bc=oracle_mod.NEUMANN, velocity=(1.0, 0.5, 0.0))
    bnd = S.on_boundary.astype(bool)
    rows = np.repeat(np.arange(S.N), np.diff(S.row_ptr))
    touching = bnd[rows] | bnd[S.col]
    assert np.all(S.adv_present[touching] == 0)
    assert np.all(S.Adv[touching] == 0)
    assert np.all(S.adv_present[~touching] == 1)
    # Dirichlet: same pattern as K, all present
    Sd = oracle_mod.System(xyz, tri, bc=oracle_mod.DIRICHLET, velocity=(1.0, 0.5, 0.0))
    assert np.all(Sd.adv_present == 1)


def test_pcg_matches_direct_solve(oracle_mod):
    xyz, tri = mg.icosphere(3)
    S = oracle_mod.System(xyz, tri, bc=oracle_mod.NEUMANN)
    A = (S.M / 1e-2 + 0.3 * S.K)
    b = np.random.default_rng(0).normal(size=S.N)
    x, it, rr = S.pcg(A, b, tol=1e-13)
    xs = spla.spsolve(sp.csr_matrix((A, S.col, S.row_ptr), shape=(S.N, S.N)).tocsc(), b)
    assert rel_l2(x, xs) < 1e-11
    assert rr < 1e-13 and 0 < it < 2 * S.N
    # zero right-hand side -> zero solution, no iterations (Eigen's early exit)
    x0, it0, _ = S.pcg(A, np.zeros(S.N), x0=np.ones(S.N))
    assert it0 == 0 and np.all(x0 == 0)


def test_heat_decay_on_sphere(oracle_mod):
    """The l = 1 harmonic z decays like 1/(1 + 2 kappa dt)^n under implicit Euler."""
    xyz, tri = mg.icosphere(4)
    S = oracle_mod.System(xyz, tri, bc=oracle_mod.NEUMANN)
    u0 = S.gather(xyz[:, 2].astype(np.float64))
    kappa, dt, n = 1.0, 1e-2, 10
    p = oracle_mod.params(oracle_mod.HEAT, dt, kappa=kappa, tol=1e-14)
    u, _, _, _, flags = S.step(p, u0, np.zeros(S.N), nsteps=n)
    ratio = (u @ u0) / (u0 @ u0)
    assert abs(ratio - (1 + 2 * kappa * dt) ** -n) < 2e-3
    assert flags == 0


def test_neumann_heat_conserves_mass(oracle_mod):
    xyz, tri = mg.jittered_grid(17, seed=9)
    S = oracle_mod.System(xyz, tri, bc=oracle_mod.NEUMANN)
    u0 = np.random.default_rng(1).uniform(size=S.N)
    p = oracle_mod.params(oracle_mod.HEAT, 1e-3, kappa=0.5, tol=1e-14)
    u, *_ = S.step(p, u0, np.zeros(S.N), nsteps=5)
    M = S.scipy("M")
    assert abs(np.sum(M @ u) - np.sum(M @ u0)) < 1e-10


@pytest.mark.parametrize("mode", [0, 1])
def test_gray_scott_fixed_point(oracle_mod, mode):
    """(u, v) = (1, 0) is stationary for both reaction modes."""
    xyz, tri = mg.icosphere(2)
    S = oracle_mod.System(xyz, tri, bc=oracle_mod.NEUMANN)
    p = oracle_mod.params(oracle_mod.REACTION_DIFFUSION, 0.5, Du=2e-4, Dv=1e-4, F=0.04, k=0.06,
                          reaction_mode=mode, tol=1e-14)
    u, v, _, _, _ = S.step(p, np.ones(S.N), np.zeros(S.N), nsteps=3)
    assert abs(u - 1).max() < 1e-12 and abs(v).max() < 1e-12


def test_gray_scott_reference_rhs(oracle_mod):
    """Reference mode: b_u = (M/dt) u - u v^2 + F (1 - u), nodal (CPUSolver.cpp:134)."""
    xyz, tri = mg.icosphere(2)
    S = oracle_mod.System(xyz, tri, bc=oracle_mod.NEUMANN)
    rng = np.random.default_rng(4)
    u = rng.uniform(0.3, 1, S.N)
    v = rng.uniform(0, 0.4, S.N)
    dt, Du, Dv, F, k = 1e-3, 0.08, 0.04, 0.035, 0.06
    p = oracle_mod.params(oracle_mod.REACTION_DIFFUSION, dt, Du=Du, Dv=Dv, F=F, k=k, reaction_mode=0, tol=1e-15)
    u1, v1, *_ = S.step(p, u, v, nsteps=1)
    M, K = S.scipy("M"), S.scipy("K")
    bu = (M / dt) @ u - u * v * v + F * (1 - u)
    bv = (M / dt) @ v + u * v * v - (F + k) * v
    uu = spla.spsolve((M / dt + Du * K).tocsc(), bu)
    vv = spla.spsolve((M / dt + Dv * K).tocsc(), bv)
    assert rel_l2(u1, uu) < 1e-12 and rel_l2(v1, vv) < 1e-12


def test_wave_schemes(oracle_mod):
    """Reference semi-implicit wave (CPUSolver.cpp:113-118) and Newmark energy conservation."""
    xyz, tri = mg.icosphere(3)
    S = oracle_mod.System(xyz, tri, bc=oracle_mod.NEUMANN)
    u0 = S.gather(mg.gaussian_bumps(xyz, seed=1, n_bumps=2, width2=0.1))
    dt, c = 1e-2, 1.0
    p = oracle_mod.params(oracle_mod.WAVE, dt, kappa=c, wave_scheme=0, tol=1e-15)
    u1, v1, *_ = S.step(p, u0, np.zeros(S.N), nsteps=1)
    M, K = S.scipy("M"), S.scipy("K")
    vv = spla.spsolve((M / dt + c * c * K * dt).tocsc(), -c * c * (K @ u0))
    assert rel_l2(v1, vv) < 1e-12
    assert rel_l2(u1, u0 + dt * vv) < 1e-14
    # Newmark (beta = 1/4, gamma = 1/2) conserves E = v'Mv + c^2 u'Ku
    pn = oracle_mod.params(oracle_mod.WAVE, dt, kappa=c, wave_scheme=1, tol=1e-15)
    a0 = S.newmark_init(pn, u0)
    np.testing.assert_allclose(M @ a0, -c * c * (K @ u0), rtol=1e-9, atol=1e-12)
    E0 = u0 @ (K @ u0) * c * c
    u, v, a, _, _ = S.step(pn, u0, np.zeros(S.N), a0, nsteps=50)
    E1 = v @ (M @ v) + c * c * u @ (K @ u)
    assert abs(E1 - E0) / E0 < 1e-8


def test_advection_diffusion_schemes(oracle_mod):
    xyz, tri = mg.jittered_grid(17, seed=3)
    S = oracle_mod.System(xyz, tri, bc=oracle_mod.NEUMANN, velocity=(1.0, 0.2, 0.0))
    u0 = np.exp(-((xyz[:, 0] - 0.5) ** 2 + (xyz[:, 1] - 0.5) ** 2) / 0.02).astype(np.float64)
    dt, c = 1e-3, 0.25
    M, K, Adv = S.scipy("M"), S.scipy("K"), S.scipy("Adv")
    p0 = oracle_mod.params(oracle_mod.ADVECTION_DIFFUSION, dt, kappa=c, adv_scheme=0, tol=1e-15)
    u1, *_ = S.step(p0, u0, np.zeros(S.N), nsteps=1)
    ref = spla.spsolve((M / dt + c * K - Adv).tocsc(), (M / dt) @ u0)
    assert rel_l2(u1, ref) < 1e-10
    p1 = oracle_mod.params(oracle_mod.ADVECTION_DIFFUSION, dt, kappa=c, adv_scheme=1, adv_sign=-1.0, tol=1e-15)
    u2, *_ = S.step(p1, u0, np.zeros(S.N), nsteps=1)
    ref2 = spla.spsolve((M / dt + c * K).tocsc(), (M / dt) @ u0 - Adv @ u0)
    assert rel_l2(u2, ref2) < 1e-12


def test_instability_flags(oracle_mod):
    u = np.array([1.0, 2e4, 0.0])
    v = np.zeros(3)
    assert oracle_mod.lib().fo_instability_f64(3, u.ctypes.data, v.ctypes.data) == 1
    u[1] = np.nan
    assert oracle_mod.lib().fo_instability_f64(3, u.ctypes.data, v.ctypes.data) == 2


def test_fp32_port_tracks_fp64(oracle_mod):
    """The FP32 Eigen-semantics port (the CPU baseline) follows the FP64 oracle."""
    xyz, tri = mg.jittered_grid(33, seed=7)
    S64 = oracle_mod.System(xyz, tri, bc=oracle_mod.NEUMANN)
    S32 = oracle_mod.System(xyz, tri, bc=oracle_mod.NEUMANN, dtype=np.float32)
    u0, v0 = mg.gray_scott_patches(xyz, seed=1)
    kw = dict(Du=2e-5, Dv=1e-5, F=0.037, k=0.06, reaction_mode=1)
    p64 = oracle_mod.params(oracle_mod.REACTION_DIFFUSION, 1.0, tol=1e-14, **kw)
    p32 = oracle_mod.params(oracle_mod.REACTION_DIFFUSION, 1.0, tol=1.1920929e-07, warm_start=0, **kw)
    u64, v64, *_ = S64.step(p64, S64.gather(u0), S64.gather(v0), nsteps=3)
    u32, v32, *_ = S32.step(p32, S32.gather(u0), S32.gather(v0), nsteps=3)
    assert rel_l2(u32, u64) < 1e-5 and rel_l2(v32, v64) < 1e-5


def test_adjoint_matches_finite_differences(oracle_mod):
    """FP64 adjoint of the explicit advection-diffusion loss vs central differences."""
    n = 9
    xyz, tri = mg.jittered_grid(n, seed=4)
    cen = xyz[tri].mean(axis=1)
    vel = np.stack([-(cen[:, 1] - 0.5), cen[:, 0] - 0.5, np.zeros(len(tri))], 1) * 0.5
    S = oracle_mod.System(xyz, tri, bc=oracle_mod.NEUMANN, elem_vel=vel)
    rng = np.random.default_rng(0)
    D = 1e-3 * np.exp(0.5 * rng.normal(size=S.T))
    u0 = S.gather(np.exp(-((xyz[:, 0] - 0.4) ** 2 + (xyz[:, 1] - 0.5) ** 2) / 0.05))
    target = rng.uniform(size=S.N)
    p = oracle_mod.params(oracle_mod.ADVECTION_DIFFUSION, 1e-2, kappa=1.0, adv_scheme=1, adv_sign=-1.0,
                          tol=1e-15)
    nsteps, ck = 12, 5
    J, gu, gD = S.adjoint_advdiff(p, D, u0, target, nsteps, ck)

    def loss(u0_, D_):
        KD = oracle_mod.ordered_sum(S.slot, S.Kloc, S.nnz, D_)
        A = sp.csr_matrix((S.M / p.dt + KD, S.col, S.row_ptr), shape=(S.N, S.N)).tocsc()
        Mm, Adv = S.scipy("M"), S.scipy("Adv")
        lu = spla.splu(A)
        u = u0_.copy()
        for _ in range(nsteps):
            u = lu.solve((Mm / p.dt) @ u - Adv @ u)
        d = u - target
        return 0.5 * d @ (Mm @ d)

    assert abs(J - loss(u0, D)) < 1e-12 * max(1, abs(J))
    eps = 1e-6
    for k in range(4):
        du = rng.normal(size=S.N)
        fd = (loss(u0 + eps * du, D) - loss(u0 - eps * du, D)) / (2 * eps)
        assert abs(fd - gu @ du) < 1e-6 * max(1, abs(fd))
        dD = rng.normal(size=S.T) * D
        fd = (loss(u0, D + eps * dD) - loss(u0, D - eps * dD)) / (2 * eps)
        assert abs(fd - gD @ dD) < 1e-5 * max(abs(fd), 1e-8)


def test_reference_meshes_against_golden(oracle_mod):
    """The oracle on the reference's own meshes (committed fixture arrays)
    reproduces the committed summaries."""
    with open(os.path.join(GOLDEN, "reference_meshes.json")) as fh:
        gold = json.load(fh)
    from make_golden import summarise
    meshes = reference_meshes()
    for name, want in gold["meshes"].items():
        xyz, tri = meshes[name]
        got = summarise(oracle_mod, xyz, tri, want["bc"])
        want = {k: v for k, v in want.items() if k != "obj_sha256"}
        assert got == want, name


@pytest.mark.skipif(not has_reference_assets(), reason="FEA_REFERENCE_ASSETS not set")
def test_reference_fixture_matches_obj_files():
    """The committed fixture arrays are the reference's OBJ files as read."""
    import hashlib
    with open(os.path.join(GOLDEN, "reference_meshes.json")) as fh:
        gold = json.load(fh)
    meshes = reference_meshes()
    for name, want in gold["meshes"].items():
        path = os.path.join(REFERENCE_ASSETS, name + ".obj")
        with open(path, "rb") as fh:
            assert hashlib.sha256(fh.read()).hexdigest() == want["obj_sha256"], name
        xyz, tri = mg.read_obj(path)
        assert np.array_equal(xyz, meshes[name][0]) and np.array_equal(tri, meshes[name][1]), name


def test_golden_known_counts():
    """Counts of the reference's icosphere.obj (V 10,242, T 20,480, nnz 71,682, max row 7)."""
    with open(os.path.join(GOLDEN, "reference_meshes.json")) as fh:
        gold = json.load(fh)
    ico = gold["meshes"]["icosphere"]
    assert (ico["V"], ico["T"], ico["nnz"], ico["max_row"]) == (10242, 20480, 71682, 7)
    assert ico["num_boundary"] == 0
    tube = gold["meshes"]["tube"]
    assert tube["num_boundary"] == 192


def test_gray_scott_adjoint_matches_finite_differences(oracle_mod):
    """FP64 adjoint of the mass-weighted Gray-Scott loss vs central differences,
    for the initial fields and for F, k, Du, Dv."""
    xyz, tri = mg.jittered_grid(9, seed=3)
    S = oracle_mod.System(xyz, tri, bc=oracle_mod.NEUMANN)
    rng = np.random.default_rng(2)
    u0, v0 = mg.gray_scott_patches(xyz, seed=1, side=0.3)
    u0, v0 = S.gather(u0), S.gather(v0)
    tu, tv = rng.uniform(size=S.N), rng.uniform(size=S.N)
    base = dict(Du=2e-3, Dv=1e-3, F=0.04, k=0.06, reaction_mode=1, tol=1e-15)
    nsteps, ck = 6, 4

    def run(u, v, **over):
        kw = dict(base)
        kw.update(over)
        p = oracle_mod.params(oracle_mod.REACTION_DIFFUSION, 0.5, **kw)
        return S.adjoint_gray_scott(p, u, v, tu, tv, nsteps, ck)

    J, gu, gv, gp = run(u0, v0)
    eps = 1e-6
    for _ in range(3):
        du, dv = rng.normal(size=S.N), rng.normal(size=S.N)
        fd = (run(u0 + eps * du, v0 + eps * dv)[0] - run(u0 - eps * du, v0 - eps * dv)[0]) / (2 * eps)
        pred = gu @ du + gv @ dv
        assert abs(fd - pred) <= 1e-6 * abs(pred)
    for j, name in enumerate(("F", "k", "Du", "Dv")):
        h = 1e-5 * base[name]
        fd = (run(u0, v0, **{name: base[name] + h})[0] - run(u0, v0, **{name: base[name] - h})[0]) / (2 * h)
        assert abs(fd - gp[j]) <= 1e-5 * abs(gp[j]), name
    # a dropped target drops its term
    p = oracle_mod.params(oracle_mod.REACTION_DIFFUSION, 0.5, **base)
    J_u_only = S.adjoint_gray_scott(p, u0, v0, tu, None, nsteps, ck)[0]
    J_v_only = S.adjoint_gray_scott(p, u0, v0, None, tv, nsteps, ck)[0]
    assert abs(J_u_only + J_v_only - J) <= 1e-12 * J


def test_extrapolated_start_from_given_previous_state(oracle_mod):
    """warm_start 2 with prev: a one-step call from (u1, v1) with prev (u0, v0)
    takes the same route as the second step of a two-step call from (u0, v0)."""
    O = oracle_mod
    xyz, tri = mg.jittered_grid(17, seed=2)
    u0, v0 = mg.gray_scott_patches(xyz, seed=4, side=0.3)
    S = O.System(xyz, tri, bc=O.NEUMANN)
    p = O.params(O.REACTION_DIFFUSION, 1.0, Du=2e-4, Dv=1e-4, F=0.04, k=0.06, reaction_mode=1, tol=1e-5,
                 warm_start=2)
    u, v = S.gather(u0), S.gather(v0)
    u2, v2, _, it2, _ = S.step(p, u, v, nsteps=2)
    u1, v1, _, it1, _ = S.step(p, u, v, nsteps=1)
    ue, ve, _, ite, _ = S.step(p, u1, v1, nsteps=1, prev=(u, v))
    assert np.array_equal(ue, u2) and np.array_equal(ve, v2) and it1 + ite == it2
    uw, vw, *_ = S.step(p, u1, v1, nsteps=1)  # no prev: the previous-field start
    assert not np.array_equal(uw, u2)
