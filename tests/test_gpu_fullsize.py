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
