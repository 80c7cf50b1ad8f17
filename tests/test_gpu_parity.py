"""GPU parity tests: the CUDA path through the C ABI against the oracle.

Bars: the compressed pattern, boundary flags and idx_map are bit-exact; FP32
matrix values agree with the FP64 oracle to 2e-6 of the row's largest entry,
FP64 values to 1e-13; one time step agrees with the FP64 oracle (solved to
1e-14) to rel-L2 1e-5 per field for FP32 handles and 1e-9 for FP64 handles.
"""
import numpy as np
import pytest

from conftest import device_field, oracle_step, rel_l2
from fea_gb300 import meshgen as mg

pytestmark = pytest.mark.gpu

MESHES = {
    "ico3": (lambda: mg.icosphere(3)),
    "grid33": (lambda: mg.jittered_grid(33, seed=2)),
    "grid_right": (lambda: mg.jittered_grid(17, seed=0, jitter=0.0)),
    "cyl": (lambda: mg.cylinder(40, 15)),
}


def _solver(fea, xyz, tri, bc, precision=None, **kw):
    p = fea.default_params(**kw)
    return fea.CUDASolver(xyz, tri, boundary_condition=bc, precision=fea.FP32 if precision is None else precision,
                          params=p)


@pytest.mark.parametrize("name", list(MESHES))
@pytest.mark.parametrize("bc", [0, 1])
def test_pattern_and_boundary_bit_exact(fea, oracle_mod, name, bc):
    xyz, tri = MESHES[name]()
    s = _solver(fea, xyz, tri, bc)
    S = oracle_mod.System(xyz, tri, bc=bc)
    idx, ob = s.idx_map()
    np.testing.assert_array_equal(ob, S.on_boundary)
    np.testing.assert_array_equal(idx, S.idx)
    inf = s.info
    assert (inf.num_unknowns, inf.nnz, inf.max_row_nonzeros) == (S.N, S.nnz, S.max_row_nonzeros)
    assert inf.num_boundary_points == S.num_boundary
    rp, col, _, _ = s.matrix(fea.STIFFNESS)
    np.testing.assert_array_equal(rp, S.row_ptr)
    np.testing.assert_array_equal(col, S.col)
    _, _, _, pres = s.matrix(fea.ADVECTION)
    np.testing.assert_array_equal(pres, S.adv_present)


def _row_scale(S, val):
    rows = np.repeat(np.arange(S.N), np.diff(S.row_ptr))
    mx = np.zeros(S.N)
    np.maximum.at(mx, rows, np.abs(val))
    return mx[rows]


@pytest.mark.parametrize("name", list(MESHES))
@pytest.mark.parametrize("precision", [0, 1])
def test_matrix_values(fea, oracle_mod, name, precision):
    xyz, tri = MESHES[name]()
    vel = (0.3, 1.0, -0.2)
    s = _solver(fea, xyz, tri, 1, precision, advdiff_velocity=vel)
    S = oracle_mod.System(xyz, tri, bc=1, velocity=vel)
    tol = 2e-6 if precision == 0 else 1e-13
    for which, ref in ((fea.STIFFNESS, S.K), (fea.MASS, S.M), (fea.ADVECTION, S.Adv)):
        _, _, val, _ = s.matrix(which)
        err = np.abs(val.astype(np.float64) - ref) / np.maximum(_row_scale(S, ref), 1e-30)
        assert err.max() < tol, (which, err.max())


def test_assembly_deterministic(fea):
    xyz, tri = mg.jittered_grid(65, seed=4)
    a = _solver(fea, xyz, tri, 1).matrix(fea.STIFFNESS)[2]
    b = _solver(fea, xyz, tri, 1).matrix(fea.STIFFNESS)[2]
    assert np.array_equal(a, b)


def test_explicit_zeros_kept_on_device(fea, oracle_mod):
    xyz, tri = mg.jittered_grid(9, seed=0, jitter=0.0)
    s = _solver(fea, xyz, tri, 1)
    _, _, val, _ = s.matrix(fea.STIFFNESS)
    S = oracle_mod.System(xyz, tri, bc=1)
    assert np.array_equal(val == 0, S.K == 0) and np.sum(val == 0) > 0


_device_field = device_field


_oracle_step = oracle_step


@pytest.mark.parametrize("precision,tol", [(0, 1e-5), (1, 1e-9)])
@pytest.mark.parametrize("bc", [0, 1])
def test_heat_steps(fea, oracle_mod, precision, tol, bc):
    xyz, tri = mg.cylinder(48, 20) if bc == 0 else mg.icosphere(4)
    u0 = np.exp(-np.sum((xyz - xyz[7]) ** 2, axis=1) / 0.1).astype(np.float32)
    s = _solver(fea, xyz, tri, bc, precision, equation=fea.HEAT, heat_time_step=1e-2, heat_conductivity=1.0,
                cg_tolerance=1e-7 if precision == 0 else 1e-12)
    s.set_values(u0)
    S = oracle_mod.System(xyz, tri, bc=bc)
    u = S.gather(u0.astype(np.float64))
    for step in range(3):
        s.advance_time(1)
        u, *_ = _oracle_step(oracle_mod, S, oracle_mod.HEAT, 1e-2, u, np.zeros(S.N), 1, kappa=1.0)
        g = s.get_values()
        assert rel_l2(g, S.scatter(u)) < max(tol, 1e-7), step  # float32 node values
        if bc == 0:
            assert np.all(g[S.on_boundary == 1] == 0)  # map_vector_to_surface
        if precision == 1:  # full FP64 state through the device API
            assert rel_l2(_device_field(s, 0), u) < tol, step
    st = s.status()
    assert st.flags == 0 and st.steps_done == 1 and st.last_iterations[0] > 0


@pytest.mark.parametrize("mode", [0, 1])
def test_gray_scott_per_step(fea, oracle_mod, mode):
    """Per-step error from the oracle's state, and 20-step drift."""
    xyz, tri = mg.jittered_grid(65, seed=8)
    u0, v0 = mg.gray_scott_patches(xyz, seed=2, side=0.12)
    if mode == 1:
        kw = dict(rd_time_step=1.0, rd_Du=2e-5, rd_Dv=1e-5, rd_feed_rate=0.037, rd_kill_rate=0.06)
    else:  # the reference's own defaults (EquationParameters.hpp:37-49)
        kw = dict()
    s = _solver(fea, xyz, tri, 1, equation=fea.REACTION_DIFFUSION, reaction_mode=mode, cg_tolerance=1e-7, **kw)
    p = s.params
    S = oracle_mod.System(xyz, tri, bc=1)
    okw = dict(Du=p.rd_Du, Dv=p.rd_Dv, F=p.rd_feed_rate, k=p.rd_kill_rate, reaction_mode=mode)
    u, v = S.gather(u0), S.gather(v0)
    s.set_fields(u0, v0)
    for step in range(3):
        s.set_fields(S.scatter(u).astype(np.float32), S.scatter(v).astype(np.float32))
        uo, vo, *_ = _oracle_step(oracle_mod, S, oracle_mod.REACTION_DIFFUSION, p.rd_time_step,
                                  S.gather(S.scatter(u).astype(np.float32)),
                                  S.gather(S.scatter(v).astype(np.float32)), 1, **okw)
        s.advance_time(1)
        ug, vg = s.get_fields()
        assert rel_l2(ug, S.scatter(uo)) < 1e-5 and rel_l2(vg, S.scatter(vo)) < 1e-5, step
        np.testing.assert_array_equal(s.get_values(), vg)  # the surface shows v
        u, v = uo, vo
    # drift over 20 steps from the same start
    s.set_fields(u0, v0)
    s.advance_time(20)
    ug, vg = s.get_fields()
    uo, vo, *_ = _oracle_step(oracle_mod, S, oracle_mod.REACTION_DIFFUSION, p.rd_time_step, S.gather(u0),
                              S.gather(v0), 20, **okw)
    assert rel_l2(ug, S.scatter(uo)) < 1e-5 and rel_l2(vg, S.scatter(vo)) < 1e-5
    assert s.status().steps_done == 20


@pytest.mark.parametrize("refine", [0, 1, 2])
def test_refinement_modes(fea, oracle_mod, refine):
    """cg_refine 0 (no true-residual pass), 1 (float-float for FP32 handles)
    and 2 (FP64): Gray-Scott steps of an FP32 handle meet the same bar
    against the FP64 oracle, and modes 1 and 2 agree closely."""
    xyz, tri = mg.jittered_grid(65, seed=8)
    u0, v0 = mg.gray_scott_patches(xyz, seed=2, side=0.12)
    kw = dict(rd_time_step=1.0, rd_Du=2e-5, rd_Dv=1e-5, rd_feed_rate=0.037, rd_kill_rate=0.06)
    out = {}
    for mode in sorted({1, refine}):
        s = _solver(fea, xyz, tri, 1, equation=fea.REACTION_DIFFUSION, reaction_mode=1, cg_tolerance=1e-6,
                    cg_refine=mode, **kw)
        s.set_fields(u0, v0)
        s.advance_time(5)
        out[mode] = s.get_fields()
        assert s.status().flags == 0
        p = s.params
    S = oracle_mod.System(xyz, tri, bc=1)
    uo, vo, *_ = _oracle_step(oracle_mod, S, oracle_mod.REACTION_DIFFUSION, p.rd_time_step, S.gather(u0),
                              S.gather(v0), 5, Du=p.rd_Du, Dv=p.rd_Dv, F=p.rd_feed_rate, k=p.rd_kill_rate,
                              reaction_mode=1)
    ug, vg = out[refine]
    assert rel_l2(ug, S.scatter(uo)) < 1e-5 and rel_l2(vg, S.scatter(vo)) < 1e-5
    if refine != 1:
        assert rel_l2(ug, out[1][0]) < 1e-5 and rel_l2(vg, out[1][1]) < 1e-5


@pytest.mark.parametrize("precision", [0, 1])
def test_extrapolated_initial_guess(fea, oracle_mod, precision):
    """cg_initial_guess 1 starts each step's solves from 2 x_n - x_(n-1):
    the steps still meet the bar against the FP64 oracle, with fewer CG
    iterations than the previous-solution start; fields set from outside
    with new values restart the history (the first step after them takes
    the warm start; the FP64 handle's round trip through float32 changes
    them, the FP32 handle's does not)."""
    xyz, tri = mg.jittered_grid(65, seed=8)
    u0, v0 = mg.gray_scott_patches(xyz, seed=2, side=0.12)
    kw = dict(rd_time_step=1.0, rd_Du=2e-5, rd_Dv=1e-5, rd_feed_rate=0.037, rd_kill_rate=0.06)
    tol, bar = (1e-6, 1e-5) if precision == 0 else (1e-12, 1e-8)  # nine steps of drift
    res = {}
    for guess in (0, 1):
        s = _solver(fea, xyz, tri, 1, precision=precision, equation=fea.REACTION_DIFFUSION, reaction_mode=1,
                    cg_tolerance=tol, cg_initial_guess=guess, **kw)
        s.set_fields(u0, v0)
        s.advance_time(3)
        s.set_fields(*s.get_fields())
        s.advance_time(9)
        st = s.status()
        assert st.flags == 0
        res[guess] = (s.get_fields(), st.total_iterations, _device_field(s, 0), _device_field(s, 1))
        p = s.params
    S = oracle_mod.System(xyz, tri, bc=1)
    okw = dict(Du=p.rd_Du, Dv=p.rd_Dv, F=p.rd_feed_rate, k=p.rd_kill_rate, reaction_mode=1)
    u3, v3, *_ = _oracle_step(oracle_mod, S, oracle_mod.REACTION_DIFFUSION, p.rd_time_step, S.gather(u0),
                              S.gather(v0), 3, **okw)
    u3, v3 = S.gather(S.scatter(u3).astype(np.float32)), S.gather(S.scatter(v3).astype(np.float32))
    uo, vo, *_ = _oracle_step(oracle_mod, S, oracle_mod.REACTION_DIFFUSION, p.rd_time_step, u3, v3, 9, **okw)
    for guess in (0, 1):
        (ug, vg), _, ud, vd = res[guess]
        assert rel_l2(ud, uo) < bar and rel_l2(vd, vo) < bar, guess
    assert res[1][1] < res[0][1]  # fewer CG iterations
    print(f"iterations over 12 steps: previous solution {res[0][1]}, extrapolated {res[1][1]}")


def test_unchanged_fields_keep_history(fea):
    """A frame loop that writes the displayed field back unchanged
    (set_values after get_values, CPUSolver.cpp:130,144) keeps the
    extrapolation's history: the trajectory is bit-identical to the one
    without the round trips.  A field written with a changed value restarts
    it: the result is bit-identical to a fresh handle started from the
    changed state."""
    xyz, tri = mg.jittered_grid(49, seed=4)
    u0, v0 = mg.gray_scott_patches(xyz, seed=3, side=0.15)
    kw = dict(rd_time_step=1.0, rd_Du=2e-5, rd_Dv=1e-5, rd_feed_rate=0.037, rd_kill_rate=0.06)

    def handle():
        s = _solver(fea, xyz, tri, 1, equation=fea.REACTION_DIFFUSION, reaction_mode=1, cg_tolerance=1e-5,
                    cg_initial_guess=1, **kw)
        s.set_fields(u0, v0)
        return s

    def run(s, n, round_trip):
        for _ in range(n):
            if round_trip:
                s.set_values(s.get_values())
                s.set_fields(*s.get_fields())
            s.advance_time(1)

    a = handle()
    run(a, 6, False)
    b = handle()
    run(b, 6, True)
    assert a.status().total_iterations == b.status().total_iterations
    for f in (0, 1):
        assert np.array_equal(_device_field(a, f), _device_field(b, f))
    # a changed value: same as a fresh start from the changed state
    c = handle()
    run(c, 3, False)
    u3, v3 = c.get_fields()
    u3[len(u3) // 2] += 1e-3
    c.set_fields(u3, v3)
    it0 = c.status().total_iterations
    run(c, 3, False)
    d = handle()
    d.set_fields(u3, v3)
    run(d, 3, False)
    assert c.status().total_iterations - it0 == d.status().total_iterations
    for f in (0, 1):
        assert np.array_equal(_device_field(c, f), _device_field(d, f))


def test_extrapolation_matches_oracle_start(fea, oracle_mod):
    """The oracle's extrapolated start (warm_start 2) solves the same systems:
    with a loose tolerance both take the same route, so FP64 GPU and FP64
    oracle agree far below the tolerance-limited error."""
    xyz, tri = mg.jittered_grid(33, seed=3)
    u0, v0 = mg.gray_scott_patches(xyz, seed=1, side=0.2)
    kw = dict(rd_time_step=1.0, rd_Du=2e-4, rd_Dv=1e-4, rd_feed_rate=0.04, rd_kill_rate=0.06)
    s = _solver(fea, xyz, tri, 1, precision=1, equation=fea.REACTION_DIFFUSION, reaction_mode=1,
                cg_tolerance=1e-4, cg_initial_guess=1, cg_refine=0, **kw)
    s.set_fields(u0, v0)
    s.advance_time(6)
    p = s.params
    S = oracle_mod.System(xyz, tri, bc=1)
    f32 = lambda x: float(np.float32(x))  # noqa: E731
    po = oracle_mod.params(oracle_mod.REACTION_DIFFUSION, f32(p.rd_time_step), Du=f32(p.rd_Du), Dv=f32(p.rd_Dv),
                           F=f32(p.rd_feed_rate), k=f32(p.rd_kill_rate), reaction_mode=1, tol=1e-4, warm_start=2)
    uo, vo, *_ = S.step(po, S.gather(u0), S.gather(v0), nsteps=6)
    po.warm_start = 1
    uw, vw, *_ = S.step(po, S.gather(u0), S.gather(v0), nsteps=6)
    e_extrap = max(rel_l2(_device_field(s, 0), uo), rel_l2(_device_field(s, 1), vo))
    e_warm = max(rel_l2(_device_field(s, 0), uw), rel_l2(_device_field(s, 1), vw))
    assert e_extrap < 1e-9 < e_warm  # the GPU followed the extrapolated route, not the warm one


@pytest.mark.parametrize("scheme", [0, 1])
def test_wave_steps(fea, oracle_mod, scheme):
    xyz, tri = mg.icosphere(4)
    u0 = mg.gaussian_bumps(xyz, seed=5, n_bumps=3, width2=0.05, amplitude=(-1, 1)).astype(np.float32)
    dt, c = 2e-3, 1.0
    s = _solver(fea, xyz, tri, 1, equation=fea.WAVE, wave_time_step=dt, wave_c=c, wave_scheme=scheme,
                cg_tolerance=1e-7)
    s.set_fields(u0, np.zeros_like(u0))
    S = oracle_mod.System(xyz, tri, bc=1)
    s.advance_time(10)
    ug, vg = s.get_fields()
    uo, vo, *_ = _oracle_step(oracle_mod, S, oracle_mod.WAVE, dt, S.gather(u0), np.zeros(S.N), 10, kappa=c,
                              wave_scheme=scheme)
    assert rel_l2(ug, S.scatter(uo)) < 1e-5
    assert rel_l2(vg, S.scatter(vo)) < 1e-4


@pytest.mark.parametrize("scheme", [0, 1])
def test_advection_diffusion_steps(fea, oracle_mod, scheme):
    xyz, tri = mg.jittered_grid(41, seed=6)
    vel = (1.0, 0.3, 0.0)
    u0 = np.exp(-((xyz[:, 0] - 0.4) ** 2 + (xyz[:, 1] - 0.5) ** 2) / 0.01).astype(np.float32)
    sign = -1.0 if scheme == 1 else 1.0
    s = _solver(fea, xyz, tri, 1, equation=fea.ADVECTION_DIFFUSION, advdiff_time_step=1e-3, advdiff_c=0.05,
                advdiff_velocity=vel, advection_scheme=scheme, advection_sign=sign, cg_tolerance=1e-7,
                cg_max_iterations=2000)
    s.set_values(u0)
    S = oracle_mod.System(xyz, tri, bc=1, velocity=vel)
    s.advance_time(5)
    uo, *_ = _oracle_step(oracle_mod, S, oracle_mod.ADVECTION_DIFFUSION, 1e-3, S.gather(u0), np.zeros(S.N), 5,
                          kappa=0.05, adv_scheme=scheme, adv_sign=sign)
    assert rel_l2(s.get_values(), S.scatter(uo)) < 1e-5


def test_per_element_diffusivity(fea, oracle_mod):
    xyz, tri = mg.jittered_grid(33, seed=1)
    D = (1e-2 * np.exp(0.5 * mg.fourier_field(xyz[tri].mean(axis=1), seed=2))).astype(np.float32)
    s = _solver(fea, xyz, tri, 1, equation=fea.HEAT, heat_time_step=1e-2, heat_conductivity=1.0,
                cg_tolerance=1e-7)
    s.set_element_fields(diffusivity=D)
    S = oracle_mod.System(xyz, tri, bc=1, diffusivity=D.astype(np.float64))
    _, _, K, _ = s.matrix(fea.STIFFNESS)
    assert np.abs(K - S.K).max() / np.abs(S.K).max() < 2e-6
    u0 = np.sin(3 * xyz[:, 0]).astype(np.float32)
    s.set_values(u0)
    s.advance_time(4)
    uo, *_ = _oracle_step(oracle_mod, S, oracle_mod.HEAT, 1e-2, S.gather(u0), np.zeros(S.N), 4, kappa=1.0)
    assert rel_l2(s.get_values(), S.scatter(uo)) < 1e-5


def test_instability_detection(fea):
    """has_numerical_instability (CPUSolver.cpp:41-48): > 1e4 and non-finite values."""
    xyz, tri = mg.icosphere(2)
    s = _solver(fea, xyz, tri, 1, equation=fea.HEAT, heat_time_step=1e-2, heat_conductivity=1.0)
    u = np.zeros(xyz.shape[0], np.float32)
    s.set_values(u)
    s.advance_time(2)
    assert not s.has_numerical_instability()
    u[3] = 5e4
    s.set_values(u)
    s.advance_time(5)
    assert s.has_numerical_instability()
    st = s.status()
    assert st.flags & 1 and st.steps_done == 0  # stepping stopped before touching the state
    np.testing.assert_array_equal(s.get_values(), u)
    u[3] = np.nan
    s.set_values(u)
    s.advance_time(1)
    assert s.status().flags & 2
    s.clear_values()
    assert not s.has_numerical_instability()
    assert np.all(s.get_values() == 0)


def test_max_iterations_flag(fea):
    xyz, tri = mg.icosphere(3)
    s = _solver(fea, xyz, tri, 1, equation=fea.HEAT, heat_time_step=1.0, heat_conductivity=1.0,
                cg_max_iterations=2, cg_tolerance=1e-12)
    s.set_values(np.random.default_rng(0).uniform(size=xyz.shape[0]).astype(np.float32))
    s.advance_time(1)
    st = s.status()
    assert st.flags & 4 and st.last_iterations[0] == 2


def test_device_field_roundtrip(fea):
    import torch
    xyz, tri = mg.jittered_grid(17, seed=3)
    s = _solver(fea, xyz, tri, 0, equation=fea.REACTION_DIFFUSION)
    N = s.info.num_unknowns
    u = torch.rand(N, device="cuda", dtype=torch.float32)
    v = torch.rand(N, device="cuda", dtype=torch.float32)
    torch.cuda.synchronize()  # the handle runs on its own stream
    s.set_fields_device(u.data_ptr(), v.data_ptr())
    u2 = torch.empty_like(u)
    v2 = torch.empty_like(v)
    s.get_fields_device(u2.data_ptr(), v2.data_ptr())
    assert torch.equal(u, u2) and torch.equal(v, v2)
    idx, _ = s.idx_map()
    hu, hv = s.get_fields()
    m = idx >= 0
    assert np.array_equal(hu[m], u.cpu().numpy()[idx[m]])
    assert np.all(hu[~m] == 0)


def test_step_determinism(fea):
    xyz, tri = mg.jittered_grid(65, seed=2)
    u0, v0 = mg.gray_scott_patches(xyz, seed=1, side=0.1)
    outs = []
    for _ in range(2):
        s = _solver(fea, xyz, tri, 1, equation=fea.REACTION_DIFFUSION, reaction_mode=1, rd_time_step=1.0,
                    rd_Du=2e-5, rd_Dv=1e-5, rd_feed_rate=0.037, rd_kill_rate=0.06)
        s.set_fields(u0, v0)
        s.advance_time(5)
        outs.append(s.get_fields())
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])


@pytest.mark.parametrize("variant", [2, 4, 10, 11, 13, 14, 15])
def test_unrolled_loop_matches_stream_launches(fea, monkeypatch, variant):
    """The step graph chains 8 iteration kernels per pass of each CG loop; the
    copies that run after a solve has stopped change nothing.  The same steps
    launched kernel by kernel (loop conditions read on the host) give the
    same fields bit for bit and the same iteration counts, and launch exactly
    one kernel per iteration (deferred-finish variants 10 and 11: pairs of
    launches, one more launch per solve to finish its last iteration)."""
    xyz, tri = mg.jittered_grid(65, seed=2)
    u0, v0 = mg.gray_scott_patches(xyz, seed=1, side=0.1)
    res = {}
    for mode in ("graph", "stream"):
        if mode == "stream":
            monkeypatch.setenv("FEA_LAUNCH_MODE", "stream")
        else:
            monkeypatch.delenv("FEA_LAUNCH_MODE", raising=False)
        s = _solver(fea, xyz, tri, 1, equation=fea.REACTION_DIFFUSION, reaction_mode=1, rd_time_step=1.0,
                    rd_Du=2e-5, rd_Dv=1e-5, rd_feed_rate=0.037, rd_kill_rate=0.06)
        s.set_cg_variant(variant)
        s.set_fields(u0, v0)
        s.advance_time(4)
        st = s.status()
        res[mode] = (s.get_fields(), st.total_iterations, st.cg_launches, list(st.last_iterations))
    (fg, ig, lg, lig), (fs, is_, ls, lis) = res["graph"], res["stream"]
    assert np.array_equal(fg[0], fs[0]) and np.array_equal(fg[1], fs[1])
    assert ig == is_ and lig == lis and ig > 0
    if variant in fea.DEFERRED_VARIANTS:
        assert is_ < ls <= is_ + 4 * 2 * 2  # 4 steps, 2 solve loops each, at most 2 launches past the last iteration
        assert ig < lg <= ig + 4 * 2 * 8
    else:
        assert ls == is_
        assert ig <= lg <= ig + 4 * 2 * 7  # 4 steps, 2 solve loops each, at most 7 stopped copies per loop


@pytest.mark.parametrize("pair", [(2, 10), (7, 11)])
@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_deferred_finish_bit_identical(fea, pair, precision):
    """Variants 10 and 11 finish each iteration at the start of the next
    launch (every block merges the block partials) instead of in the last
    block of the launch; the partials, their merge order and the scalar
    arithmetic are the same, so the fields match variants 2 and 7 bit for
    bit, with the same iteration counts."""
    xyz, tri = mg.jittered_grid(97, seed=4)
    u0, v0 = mg.gray_scott_patches(xyz, seed=2, side=0.1)
    prec = fea.FP32 if precision == "fp32" else fea.FP64
    res = []
    for variant in pair:
        s = _solver(fea, xyz, tri, 0, precision=prec, equation=fea.REACTION_DIFFUSION, reaction_mode=1,
                    rd_time_step=1.0, rd_Du=2e-5, rd_Dv=1e-5, rd_feed_rate=0.037, rd_kill_rate=0.06,
                    cg_tolerance=1e-6 if precision == "fp32" else 1e-10)
        s.set_cg_variant(variant)
        s.set_fields(u0, v0)
        s.advance_time(6)
        st = s.status()
        res.append((s.get_fields(), st.total_iterations, list(st.last_iterations), st.flags))
    (fa, ia, la, ga), (fb, ib, lb, gb) = res
    assert np.array_equal(fa[0], fb[0]) and np.array_equal(fa[1], fb[1])
    assert ia == ib and la == lb and ga == gb and ia > 0


def test_autotune_choice_is_valid(fea):
    xyz, tri = mg.jittered_grid(129, seed=1)
    s = _solver(fea, xyz, tri, 1, equation=fea.REACTION_DIFFUSION)
    assert s.info.rows_per_warp_lanes in fea.DEFERRED_VARIANTS  # a deferred-finish kernel is the default
    assert s.autotune() in fea.CG_VARIANTS
    with pytest.raises(fea.FeaError):
        s.set_cg_variant(5)


@pytest.mark.parametrize("name", ["grid33", "ico3", "cyl"])
@pytest.mark.parametrize("bc", [0, 1])
def test_cg_variants_agree(fea, oracle_mod, name, bc):
    """Every CG kernel variant steps to the oracle's result (Gray-Scott, two fields)."""
    xyz, tri = MESHES[name]()
    u0, v0 = mg.gray_scott_patches(xyz, seed=6, side=0.3) if np.ptp(xyz[:, 2]) == 0 else \
        mg.sphere_patches(xyz / np.linalg.norm(xyz, axis=1, keepdims=True), seed=6, n_patches=5, radius=0.4)
    kw = dict(rd_time_step=0.5, rd_Du=2e-3, rd_Dv=1e-3, rd_feed_rate=0.04, rd_kill_rate=0.06)
    S = oracle_mod.System(xyz, tri, bc=bc)
    p = None
    outs = []
    for variant in fea.CG_VARIANTS:
        s = _solver(fea, xyz, tri, bc, equation=fea.REACTION_DIFFUSION, reaction_mode=1, cg_tolerance=1e-7, **kw)
        s.set_cg_variant(variant)
        s.set_fields(u0, v0)
        s.advance_time(2)
        outs.append(s.get_fields())
        p = s.params
    uo, vo, *_ = oracle_step(oracle_mod, S, oracle_mod.REACTION_DIFFUSION, p.rd_time_step, S.gather(u0),
                             S.gather(v0), 2, Du=p.rd_Du, Dv=p.rd_Dv, F=p.rd_feed_rate, k=p.rd_kill_rate,
                             reaction_mode=1)
    for variant, (ug, vg) in zip(fea.CG_VARIANTS, outs):
        assert rel_l2(ug, S.scatter(uo)) < 1e-5 and rel_l2(vg, S.scatter(vo)) < 1e-5, variant


def test_boundary_condition_switch(fea, oracle_mod):
    """update_boundary_conditions (FEMContext.cpp:224-240) rebuilds everything."""
    xyz, tri = mg.cylinder(24, 8)
    s = _solver(fea, xyz, tri, 1)
    assert s.info.num_unknowns == xyz.shape[0]
    s.set_boundary_condition(0)
    S = oracle_mod.System(xyz, tri, bc=0)
    assert s.info.num_unknowns == S.N
    rp, col, _, _ = s.matrix(fea.MASS)
    np.testing.assert_array_equal(col, S.col)


def test_page_locked_host_buffers(fea):
    """Page-locked host buffers are read and written in place by the node
    gather and scatter kernels (no staging copy).  Through set_values /
    get_values and set_fields / get_fields they give the same bits as
    pageable arrays, and a frame loop that writes the displayed field back
    from a page-locked buffer keeps the extrapolation's history."""
    import ctypes as C
    import torch
    xyz, tri = mg.jittered_grid(65, seed=6)
    u0, v0 = mg.gray_scott_patches(xyz, seed=5, side=0.15)
    kw = dict(rd_time_step=1.0, rd_Du=2e-5, rd_Dv=1e-5, rd_feed_rate=0.037, rd_kill_rate=0.06)
    lib = fea.load()
    V = xyz.shape[0]
    pinned = [torch.empty(V, dtype=torch.float32).pin_memory() for _ in range(2)]
    hu, hv = (t.numpy() for t in pinned)
    ptr = [C.c_void_p(a.ctypes.data) for a in (hu, hv)]

    def handle():
        s = _solver(fea, xyz, tri, 1, equation=fea.REACTION_DIFFUSION, reaction_mode=1, cg_tolerance=1e-5,
                    cg_initial_guess=1, **kw)
        return s

    a = handle()
    a.set_fields(u0, v0)
    b = handle()
    hu[:], hv[:] = u0, v0
    fea.binding.check(lib.fea_set_fields(b._h, ptr[0], ptr[1]))
    for f in (0, 1):
        assert np.array_equal(_device_field(a, f), _device_field(b, f))
    for _ in range(5):
        a.set_values(a.get_values())
        a.advance_time(1)
        fea.binding.check(lib.fea_get_values(b._h, ptr[1]))
        fea.binding.check(lib.fea_set_values(b._h, ptr[1]))
        fea.binding.check(lib.fea_advance_time(b._h, 1))
    assert a.status().total_iterations == b.status().total_iterations
    fea.binding.check(lib.fea_get_fields(b._h, ptr[0], ptr[1]))
    ua, va = a.get_fields()
    assert np.array_equal(ua, hu) and np.array_equal(va, hv)
    fea.binding.check(lib.fea_get_values(b._h, ptr[0]))
    assert np.array_equal(a.get_values(), hu)
