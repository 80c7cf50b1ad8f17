"""Full-size accuracy of the benchmark workloads.

Gray-Scott on the 1024 x 1024 jittered grid (1,048,576 vertices), the bench's
CG tolerance, FP32 fields: one step from a generic state (three FP64 oracle
steps after the initial condition) must stay within rel-L2 1e-5 of the FP64
oracle per field; the drift over ten steps from the initial condition is
checked too.

The advection-diffusion inverse problem on the 512 x 512 grid (200 steps,
checkpoints every 20, FP64): adjoint directional derivatives against central
finite differences (eps 1e-4) of the GPU forward model on 32 random
directions, to 1e-4.
"""
import os

import numpy as np
import pytest

from conftest import rel_l2
from fea_gb300 import meshgen as mg

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def workload(oracle_mod):
    import bench
    xyz, tri, u0, v0 = bench.workload()
    S = oracle_mod.System(xyz, tri, bc=oracle_mod.NEUMANN)
    f32 = lambda x: float(np.float32(x))  # noqa: E731
    p = oracle_mod.params(oracle_mod.REACTION_DIFFUSION, 1.0, Du=f32(2e-5), Dv=f32(1e-5), F=f32(0.037),
                          k=f32(0.06), reaction_mode=1, tol=1e-12, nthreads=os.cpu_count() or 1)
    return bench, xyz, tri, u0, v0, S, p


def _solver(fea, bench, xyz, tri):
    p = fea.default_params(equation=fea.REACTION_DIFFUSION, reaction_mode=1, cg_tolerance=bench.CG_TOL,
                           **bench.PARAMS)
    return fea.CUDASolver(xyz, tri, boundary_condition=fea.NEUMANN, precision=fea.FP32, params=p)


def test_one_step_error_full_size(fea, workload):
    bench, xyz, tri, u0, v0, S, p = workload
    u, v, *_ = S.step(p, S.gather(u0), S.gather(v0), nsteps=3)
    us, vs = S.scatter(u).astype(np.float32), S.scatter(v).astype(np.float32)
    uo, vo, *_ = S.step(p, S.gather(us), S.gather(vs), nsteps=1)
    s = _solver(fea, bench, xyz, tri)
    s.set_fields(us, vs)
    s.advance_time(1)
    ug, vg = s.get_fields()
    eu, ev = rel_l2(ug, S.scatter(uo)), rel_l2(vg, S.scatter(vo))
    print(f"one-step rel-L2: u {eu:.3e} v {ev:.3e}; iterations {list(s.status().last_iterations)}")
    assert eu < 1e-5 and ev < 1e-5


def test_ten_step_drift_full_size(fea, workload):
    bench, xyz, tri, u0, v0, S, p = workload
    s = _solver(fea, bench, xyz, tri)
    s.set_fields(u0, v0)
    s.advance_time(10)
    ug, vg = s.get_fields()
    uo, vo, *_ = S.step(p, S.gather(u0), S.gather(v0), nsteps=10)
    eu, ev = rel_l2(ug, S.scatter(uo)), rel_l2(vg, S.scatter(vo))
    print(f"ten-step drift rel-L2: u {eu:.3e} v {ev:.3e}")
    assert eu < 1e-5 and ev < 1e-5


def test_adjoint_inverse_problem_full_size(fea):
    import bench
    import torch
    s, u0, target, prior, _ = bench.adjoint_workload(fea, fea.FP64)
    steps, ck, eps = bench.ADJ_STEPS, bench.ADJ_CKPT, 1e-4
    J, gu, gD = s.adjoint_advdiff_device(u0, target, steps, ck)
    assert J > 0
    gen = torch.Generator(device="cuda").manual_seed(5)

    def loss(u, D):
        s.set_element_diffusivity_device(D)
        return s.adjoint_advdiff_device(u, target, steps, ck, grads=False)[0]

    worst = 0.0
    for k in range(32):
        du = torch.randn(u0.shape, generator=gen, device="cuda", dtype=torch.float64)
        dD = torch.randn(prior.shape, generator=gen, device="cuda", dtype=torch.float64)
        pred = float(gu @ du + gD @ (prior * dD))
        fd = (loss(u0 + eps * du, prior * (1 + eps * dD)) - loss(u0 - eps * du, prior * (1 - eps * dD))) / (2 * eps)
        worst = max(worst, abs(fd - pred) / abs(pred))
    print(f"adjoint vs central differences, 32 directions: worst relative error {worst:.2e}")
    assert worst < 1e-4


def test_heat_fp64_icosphere_level5(fea, oracle_mod):
    """Heat, FP64: icosphere level 5 (10,242 vertices), diffusivity 1, implicit
    Euler dt 1e-3 for 100 steps from a Gaussian bump exp(-|x - p|^2 / 0.02) at a
    seeded point, Jacobi-PCG to 1e-10; against the FP64 oracle solved to 1e-14."""
    from conftest import oracle_step
    xyz, tri = mg.icosphere(5)
    assert (len(xyz), len(tri)) == (10242, 20480)
    p0 = mg.sphere_point(np.random.default_rng(1))
    u0 = np.exp(-np.sum((xyz.astype(np.float64) - p0) ** 2, axis=1) / 0.02)
    p = fea.default_params(equation=fea.HEAT, heat_time_step=1e-3, heat_conductivity=1.0, cg_tolerance=1e-10)
    s = fea.CUDASolver(xyz, tri, boundary_condition=fea.NEUMANN, precision=fea.FP64, params=p)
    import torch
    S = oracle_mod.System(xyz, tri, bc=oracle_mod.NEUMANN)
    u = torch.tensor(S.gather(u0), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    s.set_fields_device(u.data_ptr(), u.data_ptr())
    s.advance_time(100)
    out = torch.zeros_like(u)
    other = torch.zeros_like(u)
    torch.cuda.synchronize()
    s.get_fields_device(out.data_ptr(), other.data_ptr())
    uo, *_ = oracle_step(oracle_mod, S, oracle_mod.HEAT, 1e-3, S.gather(u0), np.zeros(S.N), 100, kappa=1.0)
    err = rel_l2(out.cpu().numpy(), uo)
    print(f"heat L5 FP64, 100 steps: rel-L2 {err:.2e}")
    assert err < 1e-8
    assert s.status().steps_done == 100


def test_newmark_wave_icosphere_level8(fea, oracle_mod):
    """Wave, Newmark beta = 1/4, gamma = 1/2 on the level-8 icosphere (655,362
    vertices), c = 1, dt 2e-3, eight seeded bumps (width 0.05, amplitudes
    U(-1, 1)), zero initial velocity, FP32 fields.  Five steps against the FP64
    oracle; over 1,000 steps the discrete energy 1/2 v'Mv + 1/2 c^2 u'Ku, which
    this scheme conserves exactly, stays within 1e-3."""
    from conftest import oracle_step
    xyz, tri = mg.icosphere(8)
    assert len(xyz) == 655362
    u0 = mg.gaussian_bumps(xyz, seed=3, n_bumps=8, width2=0.05, amplitude=(-1, 1)).astype(np.float32)
    p = fea.default_params(equation=fea.WAVE, wave_time_step=2e-3, wave_c=1.0, wave_scheme=1, cg_tolerance=1e-7)
    s = fea.CUDASolver(xyz, tri, boundary_condition=fea.NEUMANN, params=p)
    s.set_fields(u0, np.zeros_like(u0))
    S = oracle_mod.System(xyz, tri, bc=oracle_mod.NEUMANN)
    s.advance_time(5)
    ug, vg = s.get_fields()
    uo, vo, *_ = oracle_step(oracle_mod, S, oracle_mod.WAVE, 2e-3, S.gather(u0.astype(np.float64)), np.zeros(S.N),
                             5, kappa=1.0, wave_scheme=1)
    eu, ev = rel_l2(ug, S.scatter(uo)), rel_l2(vg, S.scatter(vo))
    print(f"wave L8 Newmark, 5 steps: rel-L2 u {eu:.2e} v {ev:.2e}")
    assert eu < 1e-5 and ev < 1e-4
    rp, col, kv, _ = s.matrix(fea.STIFFNESS)
    _, _, mv, _ = s.matrix(fea.MASS)
    import scipy.sparse as sp
    K = sp.csr_matrix((kv.astype(np.float64), col, rp), shape=(S.N, S.N))
    M = sp.csr_matrix((mv.astype(np.float64), col, rp), shape=(S.N, S.N))

    def energy():
        u, v = (S.gather(f.astype(np.float64)) for f in s.get_fields())
        return 0.5 * v @ (M @ v) + 0.5 * u @ (K @ u)

    s.set_fields(u0, np.zeros_like(u0))
    e0 = energy()
    s.advance_time(1000)
    e1 = energy()
    print(f"wave L8 Newmark, 1000 steps: energy {e0:.6e} -> {e1:.6e} (rel {abs(e1 - e0) / e0:.2e})")
    assert s.status().steps_done == 1000 and not s.has_numerical_instability()
    assert abs(e1 - e0) <= 1e-3 * e0
