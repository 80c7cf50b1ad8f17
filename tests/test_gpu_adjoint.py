"""The hand-written adjoint of the explicit advection-diffusion step on the GPU.

Bars (FP64 handles): loss and gradients agree with the oracle's FP64 adjoint
to 1e-8 (relative); directional derivatives agree with central finite
differences of the GPU forward model (eps 1e-4) to 1e-4; the autograd bridge
returns the adjoint's gradients.
"""
import numpy as np
import pytest

from conftest import f32, rel_l2
from fea_gb300 import meshgen as mg

pytestmark = pytest.mark.gpu


def _problem(fea, oracle_mod, n=17, bc=1, sign=1.0, seed=4):
    """Jittered n x n grid, rotating velocity, smooth per-element diffusivity."""
    import torch
    xyz, tri = mg.jittered_grid(n, seed=seed)
    cen = xyz[tri].mean(axis=1)
    vel = (np.stack([-(cen[:, 1] - 0.5), cen[:, 0] - 0.5, np.zeros(len(tri))], 1) * 0.5).astype(np.float32)
    D = 1e-3 * np.exp(0.5 * mg.fourier_field(cen, seed=seed + 1))
    dt = 1e-2
    p = fea.default_params(equation=fea.ADVECTION_DIFFUSION, advection_scheme=1, advdiff_time_step=dt,
                           advdiff_c=1.0, advection_sign=sign, velocity_mode=1, cg_tolerance=1e-13)
    s = fea.CUDASolver(xyz, tri, boundary_condition=bc, precision=fea.FP64, params=p)
    s.set_element_fields(velocity=vel)
    Dt = torch.tensor(D, dtype=torch.float64, device="cuda")
    s.set_element_diffusivity_device(Dt)
    S = oracle_mod.System(xyz, tri, bc=bc, elem_vel=vel)
    op = oracle_mod.params(oracle_mod.ADVECTION_DIFFUSION, f32(dt), kappa=1.0, adv_scheme=1, adv_sign=sign,
                           tol=1e-15)
    rng = np.random.default_rng(seed)
    u0 = S.gather(np.exp(-((xyz[:, 0] - 0.4) ** 2 + (xyz[:, 1] - 0.5) ** 2) / 0.05))
    target = rng.uniform(size=S.N)
    return s, S, op, D, Dt, u0, target


@pytest.mark.parametrize("bc,sign", [(1, 1.0), (1, -1.0), (0, 1.0)])
def test_adjoint_matches_oracle(fea, oracle_mod, bc, sign):
    import torch
    s, S, op, D, Dt, u0, target = _problem(fea, oracle_mod, bc=bc, sign=sign)
    nsteps, ck = 12, 5
    J, gu, gD = s.adjoint_advdiff_device(torch.tensor(u0, device="cuda"), torch.tensor(target, device="cuda"),
                                         nsteps, ck)
    Jo, guo, gDo = S.adjoint_advdiff(op, D, u0, target, nsteps, ck)
    assert abs(J - Jo) <= 1e-8 * abs(Jo)
    assert rel_l2(gu.cpu().numpy(), guo) < 1e-8
    assert rel_l2(gD.cpu().numpy(), gDo) < 1e-8
    # the handle's field is left at u_N: the loss of the plain forward model agrees
    J2, _, _ = s.adjoint_advdiff_device(torch.tensor(u0, device="cuda"), torch.tensor(target, device="cuda"),
                                        nsteps, nsteps, grads=False)
    assert abs(J2 - J) <= 1e-11 * abs(J)


def test_adjoint_matches_finite_differences(fea, oracle_mod):
    import torch
    s, S, op, D, Dt, u0, target = _problem(fea, oracle_mod, n=25)
    nsteps, ck, eps = 20, 6, 1e-4
    u0t = torch.tensor(u0, device="cuda")
    tg = torch.tensor(target, device="cuda")
    J, gu, gD = s.adjoint_advdiff_device(u0t, tg, nsteps, ck)
    gu, gD = gu.cpu().numpy(), gD.cpu().numpy()
    rng = np.random.default_rng(1)

    def loss(u, Dv):
        s.set_element_diffusivity_device(torch.tensor(Dv, device="cuda"))
        return s.adjoint_advdiff_device(torch.tensor(u, device="cuda"), tg, nsteps, ck, grads=False)[0]

    for k in range(8):
        du = rng.normal(size=S.N)
        dD = rng.normal(size=S.T)
        pred = gu @ du + gD @ (D * dD)
        fd = (loss(u0 + eps * du, D * (1 + eps * dD)) - loss(u0 - eps * du, D * (1 - eps * dD))) / (2 * eps)
        assert abs(fd - pred) <= 1e-4 * abs(pred), (k, fd, pred)


def test_autograd_bridge(fea, oracle_mod):
    import torch
    from fea_gb300.autograd import advdiff_loss
    s, S, op, D, Dt, u0, target = _problem(fea, oracle_mod)
    u = torch.tensor(u0, device="cuda", requires_grad=True)
    Dg = torch.tensor(D, device="cuda", requires_grad=True)
    tg = torch.tensor(target, device="cuda")
    J = advdiff_loss(s, u, Dg, tg, 8, 3)
    (2.0 * J).backward()
    Jd, gu, gD = s.adjoint_advdiff_device(u.detach(), tg, 8, 3)
    assert abs(J.item() - Jd) <= 1e-12 * abs(Jd)
    torch.testing.assert_close(u.grad, 2.0 * gu, rtol=1e-12, atol=0)
    torch.testing.assert_close(Dg.grad, 2.0 * gD, rtol=1e-12, atol=0)


def test_adjoint_fp32_handle(fea, oracle_mod):
    """FP32 handles run the same adjoint; gradients within FP32 accuracy."""
    xyz, tri = mg.jittered_grid(17, seed=2)
    cen = xyz[tri].mean(axis=1)
    vel = (np.stack([-(cen[:, 1] - 0.5), cen[:, 0] - 0.5, np.zeros(len(tri))], 1) * 0.5).astype(np.float32)
    D = (1e-3 * np.exp(0.5 * mg.fourier_field(cen, seed=3))).astype(np.float32)
    p = fea.default_params(equation=fea.ADVECTION_DIFFUSION, advection_scheme=1, advdiff_time_step=1e-2,
                           advdiff_c=1.0, velocity_mode=1, cg_tolerance=1e-7)
    s = fea.CUDASolver(xyz, tri, boundary_condition=1, params=p)
    s.set_element_fields(diffusivity=D, velocity=vel)
    S = oracle_mod.System(xyz, tri, bc=1, elem_vel=vel)
    op = oracle_mod.params(oracle_mod.ADVECTION_DIFFUSION, f32(1e-2), kappa=1.0, adv_scheme=1, adv_sign=1.0,
                           tol=1e-15)
    u0 = np.exp(-((xyz[:, 0] - 0.5) ** 2 + (xyz[:, 1] - 0.4) ** 2) / 0.05).astype(np.float32)
    target = np.random.default_rng(0).uniform(size=len(xyz)).astype(np.float32)
    J, gu, gD = s.adjoint_advdiff(u0, target, 10, 4)
    Jo, guo, gDo = S.adjoint_advdiff(op, D.astype(np.float64), S.gather(u0.astype(np.float64)),
                                     S.gather(target.astype(np.float64)), 10, 4)
    assert abs(J - Jo) <= 1e-5 * abs(Jo)
    assert rel_l2(S.gather(gu), guo) < 1e-4
    assert rel_l2(gD, gDo) < 1e-4


def test_adjoint_argument_errors(fea):
    xyz, tri = mg.icosphere(2)
    s = fea.CUDASolver(xyz, tri, boundary_condition=1,
                       params=fea.default_params(equation=fea.HEAT))
    u = np.zeros(len(xyz), np.float32)
    with pytest.raises(fea.FeaError) as ei:
        s.adjoint_advdiff(u, u, 2, 1)  # not the explicit advection-diffusion model
    assert ei.value.code == -6
    with pytest.raises(fea.FeaError):
        s.adjoint_advdiff(u, u, 0, 1)


def _gs_problem(fea, oracle_mod, mesh, bc=1):
    import torch
    xyz, tri = mesh
    kw = dict(rd_time_step=0.5, rd_Du=2e-3, rd_Dv=1e-3, rd_feed_rate=0.04, rd_kill_rate=0.06)
    p = fea.default_params(equation=fea.REACTION_DIFFUSION, reaction_mode=1, cg_tolerance=1e-13, **kw)
    s = fea.CUDASolver(xyz, tri, boundary_condition=bc, precision=fea.FP64, params=p)
    S = oracle_mod.System(xyz, tri, bc=bc)
    planar = np.ptp(xyz[:, 2]) == 0
    u0, v0 = (mg.gray_scott_patches(xyz, seed=1, side=0.3) if planar else
              mg.sphere_patches(xyz / np.linalg.norm(xyz, axis=1, keepdims=True), seed=1, n_patches=4, radius=0.4))
    u0, v0 = S.gather(u0), S.gather(v0)
    rng = np.random.default_rng(9)
    tu, tv = rng.uniform(size=S.N), rng.uniform(size=S.N)
    op = oracle_mod.params(oracle_mod.REACTION_DIFFUSION, f32(0.5), Du=f32(2e-3), Dv=f32(1e-3), F=f32(0.04),
                           k=f32(0.06), reaction_mode=1, tol=1e-15)
    T = lambda a: torch.tensor(a, dtype=torch.float64, device="cuda")  # noqa: E731
    return s, S, op, p, (u0, v0, tu, tv), T


@pytest.mark.parametrize("mesh,bc", [("grid", 1), ("grid", 0), ("ico", 1)])
def test_gray_scott_adjoint_matches_oracle(fea, oracle_mod, mesh, bc):
    m = mg.jittered_grid(17, seed=2) if mesh == "grid" else mg.icosphere(3)
    s, S, op, p, (u0, v0, tu, tv), T = _gs_problem(fea, oracle_mod, m, bc)
    J, gu, gv, gp = s.adjoint_gray_scott_device(T(u0), T(v0), T(tu), T(tv), 7, 3)
    Jo, guo, gvo, gpo = S.adjoint_gray_scott(op, u0, v0, tu, tv, 7, 3)
    assert abs(J - Jo) <= 1e-9 * abs(Jo)
    assert rel_l2(gu.cpu().numpy(), guo) < 1e-8 and rel_l2(gv.cpu().numpy(), gvo) < 1e-8
    np.testing.assert_allclose(gp, gpo, rtol=1e-8)
    # a dropped target drops its term
    Ju = s.adjoint_gray_scott_device(T(u0), T(v0), T(tu), None, 7, 3, grads=False)[0]
    Jv = s.adjoint_gray_scott_device(T(u0), T(v0), None, T(tv), 7, 3, grads=False)[0]
    assert abs(Ju + Jv - J) <= 1e-11 * abs(J)


def test_gray_scott_adjoint_finite_differences(fea, oracle_mod):
    """Initial fields and (F, k, Du, Dv): central differences of the GPU forward."""
    s, S, op, p, (u0, v0, tu, tv), T = _gs_problem(fea, oracle_mod, mg.jittered_grid(21, seed=4))
    nsteps, ck = 10, 4
    J, gu, gv, gp = s.adjoint_gray_scott_device(T(u0), T(v0), T(tu), T(tv), nsteps, ck)
    gu, gv = gu.cpu().numpy(), gv.cpu().numpy()

    def loss(u, v):
        return s.adjoint_gray_scott_device(T(u), T(v), T(tu), T(tv), nsteps, ck, grads=False)[0]

    rng = np.random.default_rng(3)
    eps = 1e-4
    for _ in range(6):
        du, dv = rng.normal(size=S.N), rng.normal(size=S.N)
        fd = (loss(u0 + eps * du, v0 + eps * dv) - loss(u0 - eps * du, v0 - eps * dv)) / (2 * eps)
        pred = gu @ du + gv @ dv
        assert abs(fd - pred) <= 1e-4 * abs(pred)
    for j, name in enumerate(("rd_feed_rate", "rd_kill_rate", "rd_Du", "rd_Dv")):
        base = getattr(p, name)
        lo, hi = f32(base * (1 - 1e-3)), f32(base * (1 + 1e-3))  # the ABI holds float parameters
        setattr(p, name, hi)
        s.set_params(p)
        j_hi = loss(u0, v0)
        setattr(p, name, lo)
        s.set_params(p)
        j_lo = loss(u0, v0)
        setattr(p, name, base)
        s.set_params(p)
        fd = (j_hi - j_lo) / (hi - lo)
        assert abs(fd - gp[j]) <= 1e-4 * abs(gp[j]), (name, fd, gp[j])


def test_gray_scott_adjoint_state_check(fea):
    xyz, tri = mg.icosphere(2)
    s = fea.CUDASolver(xyz, tri, boundary_condition=1,
                       params=fea.default_params(equation=fea.REACTION_DIFFUSION, reaction_mode=0))
    u = np.ones(len(xyz), np.float32)
    with pytest.raises(fea.FeaError) as ei:
        s.adjoint_advdiff(u, u, 2, 1)
    assert ei.value.code == -6


def test_gray_scott_autograd_bridge(fea, oracle_mod):
    import torch
    from fea_gb300.autograd import gray_scott_loss
    s, S, op, p, (u0, v0, tu, tv), T = _gs_problem(fea, oracle_mod, mg.jittered_grid(17, seed=2))
    u = T(u0).requires_grad_()
    v = T(v0).requires_grad_()
    theta = torch.tensor([p.rd_feed_rate, p.rd_kill_rate, p.rd_Du, p.rd_Dv], dtype=torch.float64,
                         requires_grad=True)
    J = gray_scott_loss(s, u, v, theta, T(tu), T(tv), 5, 2)
    J.backward()
    Jd, gu, gv, gp = s.adjoint_gray_scott_device(T(u0), T(v0), T(tu), T(tv), 5, 2)
    assert abs(J.item() - Jd) <= 1e-12 * abs(Jd)
    torch.testing.assert_close(u.grad, gu, rtol=1e-12, atol=0)
    torch.testing.assert_close(v.grad, gv, rtol=1e-12, atol=0)
    np.testing.assert_allclose(theta.grad.numpy(), gp, rtol=1e-12)
