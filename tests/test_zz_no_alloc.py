"""The solve that allocates no device memory (fea_pcg_solve_csr_noalloc).

It is meant for callers that cannot allocate on the device mid-run, such as a
render loop that must not stall on cudaMalloc/cudaFree or a host framework
that owns the GPU's memory pool.  Its result must match the library's normal
step loop: here one implicit heat step of a solver handle, (M/dt + kappa K) u'
= (M/dt) u, solved twice in a row from the handle's own state.  This file
runs last so that a failure here cannot hide another test's failure.
"""
import ctypes as C

import numpy as np
import pytest
import scipy.sparse as sp

from conftest import rel_l2
from fea_gb300 import meshgen as mg

pytestmark = pytest.mark.gpu


def _unknown_field(s):
    import torch
    u = torch.zeros(s.info.num_unknowns, dtype=torch.float32, device="cuda")
    v = torch.zeros_like(u)
    torch.cuda.synchronize()
    s.get_fields_device(u.data_ptr(), v.data_ptr())
    return u


def test_noalloc_solve_matches_heat_step(fea):
    import torch
    lib = fea.load()
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
    d_rp = torch.from_numpy(rp).cuda()
    d_col = torch.from_numpy(col).cuda()
    d_A = torch.from_numpy(A).cuda()
    for call in range(2):
        u = _unknown_field(s)
        b = torch.from_numpy((Mdt @ u.cpu().numpy().astype(np.float64)).astype(np.float32)).cuda()
        x = u.clone()
        torch.cuda.synchronize()
        iters, rel = C.c_int(0), C.c_double(0)
        rc = lib.fea_pcg_solve_csr_noalloc(n, d_rp.data_ptr(), d_col.data_ptr(), d_A.data_ptr(), b.data_ptr(),
                                           x.data_ptr(), fea.FP32, 1e-7, 0, None, C.byref(iters), C.byref(rel))
        assert rc == 0, lib.fea_last_error()
        assert 0 < iters.value < 2 * n and rel.value < 1e-7
        s.advance_time(1)
        ref = _unknown_field(s)
        assert rel_l2(x.cpu().numpy(), ref.cpu().numpy()) < 1e-5, call


def test_noalloc_rejects_oversize(fea):
    lib = fea.load()
    rc = lib.fea_pcg_solve_csr_noalloc(1 << 21, None, None, None, None, None, fea.FP32, 0.0, 0, None, None, None)
    assert rc == -8
    assert b"no-allocation limit" in lib.fea_last_error()
    rc = lib.fea_pcg_solve_csr_noalloc((1 << 19) + 1, None, None, None, None, None, fea.FP64, 0.0, 0, None, None,
                                       None)
    assert rc == -8
