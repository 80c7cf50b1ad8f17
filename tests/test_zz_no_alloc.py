"""The solve that allocates no device memory (fea_pcg_solve_csr_noalloc).

It is meant for callers that cannot allocate on the device mid-run, such as a
render loop that must not stall on cudaMalloc/cudaFree or a host framework
that owns the GPU's memory pool.  Its results are checked against the
library's normal step loop (one implicit heat step of a solver handle, solved
twice in a row from the handle's own state) and against the oracle's CPU PCG
on the same matrix, in both precisions and on two calls in a row; its status
reporting is checked on a zero right-hand side, a matrix that is not SPD, a
NaN right-hand side and an iteration limit that runs out.  This file runs
last so that a failure here cannot hide another test's failure.
"""
import ctypes as C

import numpy as np
import pytest
import scipy.sparse as sp

from conftest import rel_l2
from fea_gb300 import meshgen as mg

pytestmark = pytest.mark.gpu

FEA_ERR_TOO_LARGE, FEA_ERR_SOLVE = -8, -9
NOT_CONVERGED, BREAKDOWN, NONFINITE = 4, 8, 2


def _unknown_field(s):
    import torch
    u = torch.zeros(s.info.num_unknowns, dtype=torch.float32, device="cuda")
    v = torch.zeros_like(u)
    torch.cuda.synchronize()
    s.get_fields_device(u.data_ptr(), v.data_ptr())
    return u


def _solve(fea, n, rp, col, A, b, x, precision, tol, max_iter=0):
    """One call through the C ABI on device tensors; returns (rc, iterations, rel_residual, flags)."""
    import torch
    lib = fea.load()
    torch.cuda.synchronize()
    iters, rel, flags = C.c_int(0), C.c_double(0), C.c_uint32(0)
    rc = lib.fea_pcg_solve_csr_noalloc(n, rp.data_ptr(), col.data_ptr(), A.data_ptr(), b.data_ptr(), x.data_ptr(),
                                       precision, tol, max_iter, None, C.byref(iters), C.byref(rel), C.byref(flags))
    return rc, iters.value, rel.value, flags.value


def test_noalloc_solve_matches_heat_step(fea):
    import torch
    xyz, tri = mg.jittered_grid(97, seed=21)
    p = fea.default_params(equation=fea.HEAT, heat_time_step=1e-2, heat_conductivity=0.5, cg_tolerance=1e-7)
    s = fea.CUDASolver(xyz, tri, boundary_condition=fea.NEUMANN, precision=fea.FP32, params=p)
    s.set_values(np.exp(-((xyz[:, 0] - 0.3) ** 2 + (xyz[:, 1] - 0.6) ** 2) / 0.02).astype(np.float32))
    rp, col, K, _ = s.matrix(fea.STIFFNESS)
    _, _, M, _ = s.matrix(fea.MASS)
    n = rp.shape[0] - 1
    dt, kappa = np.float32(p.heat_time_step), np.float32(p.heat_conductivity)
    A = (M / dt + kappa * K).astype(np.float32)  # the operator's per-entry float32 evaluation
    Mdt = sp.csr_matrix(((M / dt).astype(np.float64), col, rp), shape=(n, n))
    d_rp, d_col, d_A = (torch.from_numpy(a).cuda() for a in (rp, col, A))
    for call in range(2):
        u = _unknown_field(s)
        b = torch.from_numpy((Mdt @ u.cpu().numpy().astype(np.float64)).astype(np.float32)).cuda()
        x = u.clone()
        rc, iters, rel, flags = _solve(fea, n, d_rp, d_col, d_A, b, x, fea.FP32, 1e-7)
        assert rc == 0, fea.load().fea_last_error()
        assert flags == 0 and 0 < iters < 2 * n and rel < 1e-7
        s.advance_time(1)
        ref = _unknown_field(s)
        assert rel_l2(x.cpu().numpy(), ref.cpu().numpy()) < 1e-5, call


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_noalloc_matches_oracle_pcg(fea, oracle_mod, precision):
    """Two solves in a row, each from a nonzero initial guess, against the
    oracle's Jacobi-PCG (FP64, solved to 1e-13) on the same matrix: within
    1e-5 for FP32, 1e-9 for FP64 (the bars of the other parity tests)."""
    import torch
    xyz, tri = mg.icosphere(4)
    S = oracle_mod.System(xyz, tri, bc=oracle_mod.NEUMANN)
    dt, kappa = 0.01, 0.3
    A64 = S.M / dt + kappa * S.K
    fp64 = precision == "fp64"
    real, prec, tol, bar = (np.float64, fea.FP64, 1e-12, 1e-9) if fp64 else (np.float32, fea.FP32, 1e-7, 1e-5)
    Ar = A64.astype(real)
    Mdt = sp.csr_matrix((S.M / dt, S.col, S.row_ptr), shape=(S.N, S.N))
    d_rp, d_col, d_A = (torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (S.row_ptr, S.col, Ar))
    rng = np.random.default_rng(3)
    for call in range(2):
        u = np.exp(-np.sum((xyz - xyz[17 + 400 * call]) ** 2, axis=1) / 0.1).astype(np.float64)
        b = (Mdt @ u).astype(real)
        x0 = (u + 0.01 * rng.standard_normal(S.N)).astype(real)
        x = torch.from_numpy(x0.copy()).cuda()
        rc, iters, rel, flags = _solve(fea, S.N, d_rp, d_col, d_A, torch.from_numpy(b).cuda(), x, prec, tol)
        assert rc == 0 and flags == 0, fea.load().fea_last_error()
        assert 0 < iters < 2 * S.N and rel < tol
        xo, _, _ = S.pcg(Ar.astype(np.float64), b.astype(np.float64), x0.astype(np.float64), tol=1e-13)
        assert rel_l2(x.cpu().numpy(), xo) < bar, call


def test_noalloc_status(fea, oracle_mod):
    import torch
    xyz, tri = mg.jittered_grid(33, seed=5)
    S = oracle_mod.System(xyz, tri, bc=oracle_mod.NEUMANN)
    A = (S.M / 0.01 + S.K).astype(np.float32)
    d_rp, d_col = torch.from_numpy(S.row_ptr).cuda(), torch.from_numpy(S.col).cuda()
    d_A = torch.from_numpy(A).cuda()
    n = S.N
    # a zero right-hand side: x = 0 (Eigen's early exit), no iteration
    x = torch.ones(n, device="cuda")
    rc, iters, rel, flags = _solve(fea, n, d_rp, d_col, d_A, torch.zeros(n, device="cuda"), x, fea.FP32, 1e-7)
    assert rc == 0 and flags == 0 and iters == 0 and rel == 0.0
    assert torch.count_nonzero(x).item() == 0
    b = torch.from_numpy((sp.csr_matrix((A.astype(np.float64), S.col, S.row_ptr)) @ np.ones(n)).astype(np.float32))
    b = b.cuda()
    # the iteration limit runs out: FEA_OK with the flag, and the residual it reached
    x = torch.zeros(n, device="cuda")
    rc, iters, rel, flags = _solve(fea, n, d_rp, d_col, d_A, b, x, fea.FP32, 1e-7, max_iter=2)
    assert rc == 0 and flags == NOT_CONVERGED and iters == 2 and 1e-7 < rel < np.inf  # CG's |r| need not fall
    # a matrix that is not SPD (negated): p.Ap < 0 on the first iteration
    x = torch.zeros(n, device="cuda")
    rc, iters, rel, flags = _solve(fea, n, d_rp, d_col, -d_A, b, x, fea.FP32, 1e-7)
    assert rc == FEA_ERR_SOLVE and flags & BREAKDOWN
    assert b"breakdown" in fea.load().fea_last_error()
    # NaN in the right-hand side
    bn = b.clone()
    bn[n // 2] = float("nan")
    x = torch.zeros(n, device="cuda")
    rc, iters, rel, flags = _solve(fea, n, d_rp, d_col, d_A, bn, x, fea.FP32, 1e-7)
    assert rc == FEA_ERR_SOLVE and flags & NONFINITE
    # the scratch is still usable: a good solve right after the failed ones
    x = torch.zeros(n, device="cuda")
    rc, iters, rel, flags = _solve(fea, n, d_rp, d_col, d_A, b, x, fea.FP32, 1e-7)
    assert rc == 0 and flags == 0 and rel < 1e-7
    assert rel_l2(x.cpu().numpy(), np.ones(n)) < 1e-3


def test_noalloc_rejects_oversize(fea):
    lib = fea.load()
    rc = lib.fea_pcg_solve_csr_noalloc(1 << 21, None, None, None, None, None, fea.FP32, 0.0, 0, None, None, None,
                                       None)
    assert rc == FEA_ERR_TOO_LARGE
    assert b"no-allocation limit" in lib.fea_last_error()
    rc = lib.fea_pcg_solve_csr_noalloc((1 << 19) + 1, None, None, None, None, None, fea.FP64, 0.0, 0, None, None,
                                       None, None)
    assert rc == FEA_ERR_TOO_LARGE
