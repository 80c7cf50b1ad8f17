"""Benchmark: Gray-Scott on the 1024 x 1024 jittered grid (1,048,576 vertices).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

One step = the reference's Gray-Scott advance_time (CPUSolver.cpp:127-145):
mass-weighted reaction right-hand side for u and v, then the two SPD solves
(M/dt + D K) x = b with Jacobi-PCG, FP32 fields and float-float reductions.
Workload (synthetic, seeded): Du 2e-5, Dv 1e-5, F 0.037, k 0.06, dt 1, Neumann,
u = 1, v = 0 with 20 squares of side 0.05 at u = 0.5, v = 0.25, plus U(-0.01,
0.01) noise.  Timed steps continue from the warm-up state.

Prints one JSON line (rank 0).  `value` times each step on the device with
CUDA events on the solver's stream, with the L2 cache flushed (256 MiB write)
before every timed step; `e2e` times set_values (host -> device) +
advance_time(1) + get_values (device -> host) through the C ABI with a
page-locked host buffer, over the same steps (same start state and
extrapolation history).  With --gpus N > 1 (torchrun) every rank steps its
own replica of the workload: the path does not shard across GPUs.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "fea-visualizer_gb300"))

GRID_N = 1024
PARAMS = dict(rd_time_step=1.0, rd_Du=2e-5, rd_Dv=1e-5, rd_feed_rate=0.037, rd_kill_rate=0.06)
# CG stopping tolerance |r| < tol |b|: the loosest setting whose one-step error
# against the FP64 oracle stays below 1e-5 with margin (about 2.5e-6, set by the
# FP32 matrix values; tests/test_gpu_fullsize.py checks it on this workload)
CG_TOL = 1e-5
# the solves' start: 1 = 2 x_n - x_(n-1) from the last two steps (0: the
# previous solution)
CG_GUESS = 1
METRIC = "Gray-Scott 1M-vert steps/s at rel-L2<=1e-5, batched vs plain; CG SpMV HBM GB/s"


def workload():
    from fea_gb300 import meshgen as mg
    xyz, tri = mg.jittered_grid(GRID_N, seed=0)
    u0, v0 = mg.gray_scott_patches(xyz, seed=0)
    return xyz, tri, u0, v0


def config(V, T, nnz, extra=None):
    c = {"workload": f"gray-scott {GRID_N}x{GRID_N} jittered grid", "vertices": V, "triangles": T,
         "nnz": nnz, "reaction": "mass-weighted (consistent)", "bc": "neumann", "dt": 1.0, "Du": 2e-5,
         "Dv": 1e-5, "F": 0.037, "k": 0.06, "cg": f"jacobi-pcg, |r| < {CG_TOL:g} |b|, warm start, float-float dots and scalars",
         "l2": "flushed before every timed step (256 MiB write)"}
    if extra:
        c.update(extra)
    return c


class Clocks:
    """nvidia-smi samples during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        # raw samples: a temporary file unless FEA_CLOCKS_DIR names a folder to keep them in
        self.path = os.path.join(os.environ.get("FEA_CLOCKS_DIR") or tempfile.gettempdir(),
                                 f"fea_clocks_rank{index}.csv")

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        if not self.proc or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, val in zip(names, f[5:9]):
                if val.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# DRAM bytes (read + write) per in-loop launch of the CG iteration kernel, by
# variant: the mean of consecutive steady launches of the step loop of this
# workload in one ncu capture without cache control (the capture commands sit
# with the kernels' profile summaries).  A variant without an entry reports
# traffic null.
IN_LOOP_TRAFFIC = {10: 104.1e6, 11: 106.9e6, 14: 91.7e6, 15: 91.4e6}


def cg_kernel_name(variant):
    """The CG iteration kernel that runs for a variant (fea_set_cg_variant)."""
    if variant in (0, 1):
        return "k_cgcg_iter_ell"
    if variant in (2, 3, 6, 7):
        return "k_cgcg_iter_stream"
    if variant in (10, 11):
        return "k_cgcg_iter_stream (deferred finish)"
    if variant == 13:
        return "k_cgcg_iter_direct"
    if variant in (14, 15):
        return "k_cgcg_iter_ring"
    return "k_cgcg_iter"


def measured_peak_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as fh:
            return float(json.load(fh)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def iter_bytes(N, nnz, nfields=2):
    """Algorithmic bytes of one CG iteration launch (the step's dominant
    kernel: paired CSR SpMV with the vector updates fused): values (4 B per
    field) and a 4 B column index per stored entry, row pointers, and per row
    and field the reads of r, w, s, D^-1, x, p and the writes of x, p, r, s, w
    (11 x 4 B; the gathered vectors counted once)."""
    return nnz * (4 * nfields + 4) + 4 * (N + 1) + 11 * 4 * nfields * N


# Batched sweep: 256 Gray-Scott instances on icospheres of uneven size
BATCH_N = 256
# CG tolerance of the sweep: the loosest whose one step from the oracle's
# state stays within rel-L2 1e-5 on every instance (tests/test_gpu_batch_sweep.py)
BATCH_CG_TOL = 1e-6
BATCH_LEVELS = (3, 4, 5, 6)
BATCH_PARAMS = dict(time_step=0.5, Du=2e-4, Dv=1e-4)


def in_loop_iteration_ms(F, s, p, start_u, start_v, stream, counts=(40, 140), steps=3):
    """Device time per CG iteration inside the step graph, as the step loop
    runs it (the previous iteration's writes still in L2, written back while
    this one streams): steps whose iteration count is pinned by max_iter (the
    tolerance is unreachable), timed with CUDA events at two counts, the
    difference per iteration.  Every iteration streams more than the L2."""
    import torch
    ms, its = [], []
    for m in counts:
        q = F.binding.Params.from_buffer_copy(p)
        q.cg_tolerance = 1e-30
        q.cg_max_iterations = m
        s.set_params(q)
        s.set_fields(start_u, start_v)
        s.advance_time(1)
        s.synchronize()
        it0 = s.status().total_iterations
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            e0.record(stream)
            s.advance_time(steps)
            e1.record(stream)
        s.synchronize()
        ms.append(e0.elapsed_time(e1))
        its.append(s.status().total_iterations - it0)
    s.set_params(p)
    return (ms[1] - ms[0]) / max(1, its[1] - its[0]), its


def batch_workload(n=BATCH_N, seed=0):
    import numpy as np
    from fea_gb300 import meshgen as mg
    rng = np.random.default_rng(seed)
    meshes = {L: mg.icosphere(L) for L in BATCH_LEVELS}
    insts, starts = [], []
    for i in range(n):
        xyz, tri = meshes[int(rng.choice(BATCH_LEVELS))]
        insts.append(dict(vertices=xyz, triangles=tri, boundary_condition=1,
                          feed_rate=float(rng.uniform(0.01, 0.06)), kill_rate=float(rng.uniform(0.045, 0.07)),
                          **BATCH_PARAMS))
        starts.append(mg.sphere_patches(xyz, seed=1000 + i))
    return insts, starts


# Adjoint inverse problem: advection-diffusion on the 512 x 512 jittered grid
ADJ_GRID, ADJ_STEPS, ADJ_CKPT, ADJ_DT = 512, 200, 20, 1e-2


def adjoint_workload(F, precision):
    """Handle, initial field u0 and target (unknown-indexed CUDA tensors) and
    the prior diffusivity: rotating velocity (-(y-0.5), x-0.5) * 0.5 per
    element, hidden D_e = 1e-3 exp(0.5 g) with g a 16-mode Fourier field, a
    seeded Gaussian u0; the target is the hidden model's final field and the
    loss is evaluated at the prior D = 1e-3."""
    import numpy as np
    import torch
    from fea_gb300 import meshgen as mg
    xyz, tri = mg.jittered_grid(ADJ_GRID, seed=0)
    cen = xyz[tri].mean(axis=1)
    vel = (np.stack([-(cen[:, 1] - 0.5), cen[:, 0] - 0.5, np.zeros(len(tri))], 1) * 0.5).astype(np.float32)
    hidden = 1e-3 * np.exp(0.5 * mg.fourier_field(cen, seed=1, n_modes=16))
    rng = np.random.default_rng(2)
    c = rng.uniform(0.3, 0.7, 2)
    u0n = np.exp(-((xyz[:, 0] - c[0]) ** 2 + (xyz[:, 1] - c[1]) ** 2) / 0.02)
    p = F.default_params(equation=F.ADVECTION_DIFFUSION, advection_scheme=1, advdiff_time_step=ADJ_DT,
                         advdiff_c=1.0, velocity_mode=1, cg_tolerance=1e-12 if precision == F.FP64 else 1e-6)
    s = F.CUDASolver(xyz, tri, boundary_condition=F.NEUMANN, precision=precision, params=p)
    s.set_element_fields(velocity=vel)
    dt = torch.float64 if precision == F.FP64 else torch.float32
    u0 = torch.tensor(u0n, dtype=dt, device="cuda")  # Neumann: unknowns are the nodes
    s.set_element_diffusivity_device(torch.tensor(hidden, dtype=dt, device="cuda"))
    s.adjoint_advdiff_device(u0, torch.zeros_like(u0), ADJ_STEPS, ADJ_STEPS, grads=False)
    target = torch.zeros_like(u0)
    other = torch.zeros_like(u0)
    torch.cuda.synchronize()
    s.get_fields_device(target.data_ptr(), other.data_ptr())
    prior = torch.full((len(tri),), 1e-3, dtype=dt, device="cuda")
    s.set_element_diffusivity_device(prior)
    return s, u0, target, prior, hidden


def bench_adjoint(F):
    """One loss + gradients evaluation (forward, checkpointed reverse sweep) in
    FP64 and FP32, and the forward model alone."""
    import torch
    out = {"workload": f"advection-diffusion inverse problem, {ADJ_GRID}x{ADJ_GRID} jittered grid, rotating "
                       f"velocity, implicit diffusion dt {ADJ_DT:g}, {ADJ_STEPS} steps, checkpoints every "
                       f"{ADJ_CKPT}; loss 1/2 |u_N - target|_M^2, gradients w.r.t. u0 and per-element D"}
    for name, prec in (("fp64", F.FP64), ("fp32", F.FP32)):
        s, u0, target, prior, _ = adjoint_workload(F, prec)
        s.adjoint_advdiff_device(u0, target, ADJ_STEPS, ADJ_CKPT)  # warm-up (graphs, allocations)
        t0 = time.perf_counter()
        J, gu, gD = s.adjoint_advdiff_device(u0, target, ADJ_STEPS, ADJ_CKPT)
        t1 = time.perf_counter()
        s.adjoint_advdiff_device(u0, target, ADJ_STEPS, ADJ_CKPT, grads=False)
        t2 = time.perf_counter()
        st = s.status()
        out[name] = {"loss_and_gradients_ms": 1000 * (t1 - t0), "forward_only_ms": 1000 * (t2 - t1), "loss": J,
                     "grad_u0_norm": float(torch.linalg.norm(gu)), "grad_D_norm": float(torch.linalg.norm(gD)),
                     "cg_iterations_last_solve": int(st.last_iterations[0])}
        s.close()
    return out


def _timed_steps(s, nsteps):
    """Device time of advance_time(nsteps) on the handle's stream (CUDA events)
    and the CG iterations it took."""
    import torch
    st = torch.cuda.ExternalStream(s.stream())
    it0 = s.status().total_iterations
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(st):
        e0.record(st)
        s.advance_time(nsteps)
        e1.record(st)
    s.synchronize()
    return e0.elapsed_time(e1), s.status().total_iterations - it0


def bench_configs(F):
    """The other single-mesh workloads, device-timed: FP64 heat on the level-5
    icosphere (100 steps, PCG to 1e-10) and the Newmark wave on the level-8
    icosphere (1,000 steps, FP32)."""
    import numpy as np
    from fea_gb300 import meshgen as mg
    out = {}
    xyz, tri = mg.icosphere(5)
    p0 = mg.sphere_point(np.random.default_rng(1))
    u0 = np.exp(-np.sum((xyz.astype(np.float64) - p0) ** 2, axis=1) / 0.02).astype(np.float32)
    p = F.default_params(equation=F.HEAT, heat_time_step=1e-3, heat_conductivity=1.0, cg_tolerance=1e-10)
    s = F.CUDASolver(xyz, tri, boundary_condition=F.NEUMANN, precision=F.FP64, params=p)
    s.set_fields(u0, u0)
    s.advance_time(5)  # warm-up (graph instantiation)
    s.set_fields(u0, u0)
    ms, its = _timed_steps(s, 100)
    out["heat_fp64_icosphere5"] = {
        "workload": "heat, FP64, level-5 icosphere (10,242 vertices), kappa 1, dt 1e-3, Gaussian bump, "
                    "Jacobi-PCG to 1e-10", "steps": 100, "ms": ms, "steps_per_s": 100 / (ms / 1000),
        "cg_iterations_per_step": its / 100, "cg_variant": s.info.rows_per_warp_lanes}
    s.close()
    xyz, tri = mg.icosphere(8)
    w0 = mg.gaussian_bumps(xyz, seed=3, n_bumps=8, width2=0.05, amplitude=(-1, 1)).astype(np.float32)
    p = F.default_params(equation=F.WAVE, wave_time_step=2e-3, wave_c=1.0, wave_scheme=1, cg_tolerance=1e-7)
    s = F.CUDASolver(xyz, tri, boundary_condition=F.NEUMANN, params=p)
    s.set_fields(w0, np.zeros_like(w0))
    s.advance_time(5)
    s.set_fields(w0, np.zeros_like(w0))
    ms, its = _timed_steps(s, 1000)
    out["wave_newmark_icosphere8"] = {
        "workload": "wave, Newmark beta 1/4 gamma 1/2, FP32, level-8 icosphere (655,362 vertices), c 1, "
                    "dt 2e-3, eight bumps", "steps": 1000, "ms": ms, "steps_per_s": 1000 / (ms / 1000),
        "cg_iterations_per_step": its / 1000, "cg_variant": s.info.rows_per_warp_lanes,
        "status_flags": int(s.status().flags)}
    s.close()
    return out


# Gray-Scott adjoint: the (F, k, Du, Dv) gradients on the 512 x 512 jittered grid
GS_ADJ_GRID, GS_ADJ_STEPS, GS_ADJ_CKPT, GS_ADJ_F_TARGET = 512, 50, 10, 0.04


def bench_gs_adjoint(F):
    """One loss + gradients evaluation of the Gray-Scott adjoint (u0, v0, F,
    k, Du, Dv) in FP64 and FP32, and the forward model alone.  The target is
    the v field of the same run with the feed rate at 0.04; the loss is
    evaluated at 0.037."""
    import numpy as np
    import torch
    from fea_gb300 import meshgen as mg
    xyz, tri = mg.jittered_grid(GS_ADJ_GRID, seed=0)
    u0n, v0n = mg.gray_scott_patches(xyz, seed=0)
    out = {"workload": f"gray-scott inverse problem, {GS_ADJ_GRID}x{GS_ADJ_GRID} jittered grid, mass-weighted "
                       f"reaction, dt 1, {GS_ADJ_STEPS} steps, checkpoints every {GS_ADJ_CKPT}; loss "
                       f"1/2 |v_N - target|_M^2 (target: feed rate {GS_ADJ_F_TARGET}, evaluated at 0.037), "
                       f"gradients w.r.t. u0, v0, F, k, Du, Dv"}

    def handle(prec, feed):
        p = F.default_params(equation=F.REACTION_DIFFUSION, reaction_mode=1, rd_time_step=1.0, rd_Du=2e-5,
                             rd_Dv=1e-5, rd_feed_rate=feed, rd_kill_rate=0.06,
                             cg_tolerance=1e-12 if prec == F.FP64 else 1e-6)
        return F.CUDASolver(xyz, tri, boundary_condition=F.NEUMANN, precision=prec, params=p)

    for name, prec in (("fp64", F.FP64), ("fp32", F.FP32)):
        dt = torch.float64 if prec == F.FP64 else torch.float32
        u0 = torch.tensor(u0n, dtype=dt, device="cuda")  # Neumann: unknowns are the nodes
        v0 = torch.tensor(v0n, dtype=dt, device="cuda")
        h = handle(prec, GS_ADJ_F_TARGET)
        torch.cuda.synchronize()
        h.set_fields_device(u0.data_ptr(), v0.data_ptr())
        h.advance_time(GS_ADJ_STEPS)
        tu, tv = torch.zeros_like(u0), torch.zeros_like(v0)
        h.synchronize()
        h.get_fields_device(tu.data_ptr(), tv.data_ptr())
        h.synchronize()
        h.close()
        s = handle(prec, 0.037)
        s.adjoint_gray_scott_device(u0, v0, None, tv, GS_ADJ_STEPS, GS_ADJ_CKPT)  # warm-up
        t0 = time.perf_counter()
        J, gu, gv, gp = s.adjoint_gray_scott_device(u0, v0, None, tv, GS_ADJ_STEPS, GS_ADJ_CKPT)
        t1 = time.perf_counter()
        s.adjoint_gray_scott_device(u0, v0, None, tv, GS_ADJ_STEPS, GS_ADJ_CKPT, grads=False)
        t2 = time.perf_counter()
        out[name] = {"loss_and_gradients_ms": 1000 * (t1 - t0), "forward_only_ms": 1000 * (t2 - t1), "loss": J,
                     "grad_u0_norm": float(torch.linalg.norm(gu)), "grad_v0_norm": float(torch.linalg.norm(gv)),
                     "dJ_dF": float(gp[0]), "dJ_dk": float(gp[1]), "dJ_dDu": float(gp[2]),
                     "dJ_dDv": float(gp[3]), "status_flags": int(s.status().flags)}
        s.close()
    return out


def batch_iter_bytes(insts):
    """Algorithmic bytes of one CG iteration of every instance of a batch:
    iter_bytes of each instance's mesh (closed meshes: N = V, nnz = V + 2E)."""
    import numpy as np
    total = 0
    for d in insts:
        tri = np.asarray(d["triangles"], dtype=np.int64)
        e = np.sort(np.concatenate([tri[:, [0, 1]], tri[:, [1, 2]], tri[:, [2, 0]]]), axis=1)
        nedges = np.unique(e[:, 0] * (1 << 32) + e[:, 1]).size
        V = d["vertices"].shape[0]
        total += iter_bytes(V, V + 2 * nedges)
    return total


def bench_batched(F, steps, warmup, plain_steps):
    """The 256-instance sweep in one batch vs the plain loop of single-mesh
    handles (one after another, each advancing its own graph)."""
    import numpy as np
    insts, starts = batch_workload()
    t0 = time.perf_counter()
    B = F.BatchSolver(insts, cg_tolerance=BATCH_CG_TOL)
    setup_s = time.perf_counter() - t0
    B.set_initial_guess(CG_GUESS)  # the solves' start, as on the single-mesh handles
    for i, (u, v) in enumerate(starts):
        B.set_fields(i, u, v)
    B.advance_time(warmup)
    B.synchronize()
    it0, _ = B.counters()
    t0 = time.perf_counter()
    B.advance_time(steps)
    B.synchronize()
    batch_s = time.perf_counter() - t0
    it1, _ = B.counters()
    flags, iters = B.status()
    batch_variant = B.cg_variant
    handles = []
    for d in insts:
        p = F.default_params(equation=F.REACTION_DIFFUSION, reaction_mode=1, rd_time_step=d["time_step"],
                             rd_Du=d["Du"], rd_Dv=d["Dv"], rd_feed_rate=d["feed_rate"],
                             rd_kill_rate=d["kill_rate"], cg_tolerance=BATCH_CG_TOL, cg_initial_guess=CG_GUESS)
        handles.append(F.CUDASolver(d["vertices"], d["triangles"], boundary_condition=F.NEUMANN, params=p))
    plain = {}
    # the plain loop on the handles' default kernels, and on the batch's own kernel family
    for name, var in (("default", None), ("same_family", batch_variant)):
        for h, (u, v) in zip(handles, starts):
            if var is not None:
                h.set_cg_variant(var)
            h.set_fields(u, v)
            h.advance_time(1)
            h.synchronize()
        t0 = time.perf_counter()
        for h in handles:
            h.advance_time(plain_steps)
            h.synchronize()
        plain[name] = time.perf_counter() - t0
    plain_s = plain["default"]
    # roofline of the batched CG iteration kernel: one launch over every
    # instance, back to back (each launch streams more than the L2)
    it_ms = B.time_iteration(20)
    it_bytes = batch_iter_bytes(insts)
    peak, peak_kind = measured_peak_hbm()
    # the whole sweep's effective rate: the iterations it ran, per second
    sweep_bytes = float(np.sum((it1 - it0) * np.array([batch_iter_bytes([d]) for d in insts])))
    # accuracy of the batch against the plain handles: the same 5 steps from the start state
    for i, (h, (u, v)) in enumerate(zip(handles, starts)):
        h.set_fields(u, v)
        B.set_fields(i, u, v)
        h.advance_time(5)
    B.advance_time(5)
    err = 0.0
    for i, h in enumerate(handles):
        for a, b in zip(B.get_fields(i), h.get_fields()):
            err = max(err, float(np.linalg.norm(a.astype(np.float64) - b) / max(np.linalg.norm(b), 1e-30)))
        h.close()
    nverts = sum(d["vertices"].shape[0] for d in insts)
    batch_rate = BATCH_N * steps / batch_s
    plain_rate = BATCH_N * plain_steps / plain_s
    same_rate = BATCH_N * plain_steps / plain["same_family"]
    B.close()
    achieved = it_bytes / (it_ms * 1e-3) / 1e9
    return {"workload": f"{BATCH_N} gray-scott instances, icospheres of levels {list(BATCH_LEVELS)} drawn "
                        f"uniformly, F ~ U(0.01,0.06), k ~ U(0.045,0.07), Du 2e-4, Dv 1e-4, dt 0.5, "
                        f"CG |r| < {BATCH_CG_TOL:g} |b|",
            "vertices": nverts, "steps": steps, "instance_steps_per_s": batch_rate,
            "sweep_steps_per_s": steps / batch_s, "plain_instance_steps_per_s": plain_rate,
            "plain_steps_timed": plain_steps, "speedup_vs_plain": batch_rate / plain_rate,
            "plain_same_family_instance_steps_per_s": same_rate, "speedup_vs_plain_same_family": batch_rate / same_rate,
            "cg_variant": batch_variant, "initial_guess": GUESS_LABEL[CG_GUESS],
            "cg_iterations_per_sweep_step_mean_instance": float(np.mean(it1 - it0)) / steps,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "algorithmic_bytes_per_batched_iteration": it_bytes, "ms_per_batched_iteration": it_ms,
                         "how": "fea_batch_time_iteration: the iteration kernel over every instance, fields masked, "
                                "20 launches back to back (CUDA events); bytes: iter_bytes of each instance's mesh",
                         "peak_source": peak_kind,
                         "sweep_effective_GBps": sweep_bytes / batch_s / 1e9,
                         "sweep_effective_how": "algorithmic bytes of the CG iterations the timed sweep ran, over "
                                                "its wall time (right-hand sides, refinement and launches included)"},
            "max_rel_l2_vs_plain_after_5_steps": err, "setup_s": setup_s,
            "status_flags_or": int(np.bitwise_or.reduce(flags)),
            "max_iterations_last_solve": int(iters.max()), "min_iterations_last_solve": int(iters.min()),
            "timing": "wall clock around one advance_time(K) graph launch + synchronize; "
                      "every CG iteration touches more than the L2 size (~0.6 GB)"}


def max_over_ranks(value, dist=None, device="cpu"):
    """The largest of the ranks' values: a replica job takes as long as its
    slowest rank.  Without a process group, the value itself."""
    if dist is None:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


FLT_EPSILON = 1.1920928955078125e-07
# the reference's CG set-up (CPUSolver.cpp:65: Eigen's default tolerance, zero guess)
REF_CG = "jacobi-pcg, zero guess, |r| < FLT_EPSILON |b|, double dots, operator rebuilt every step"
EQ_CG = f"jacobi-pcg, |r| < {CG_TOL:g} |b| (the GPU arm's setting), double dots"
GUESS_LABEL = {0: "previous solution", 1: "2 x_n - x_(n-1) (extrapolated)"}


_CPU_SYSTEMS = {}


def cpu_system(xyz, tri):
    """The oracle's FP32 port of the reference's assembled system (cached per mesh)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    key = (xyz.shape[0], tri.shape[0])
    if key not in _CPU_SYSTEMS:
        _CPU_SYSTEMS[key] = O.System(xyz, tri, bc=O.NEUMANN, dtype="float32")
    return O, _CPU_SYSTEMS[key]


def cpu_sample(xyz, tri, u0, v0, nsteps, nthreads, tol=FLT_EPSILON, warm_start=0, prev=None):
    """The reference's Eigen-semantics CPU step (the oracle's FP32 port):
    A = M/dt + D K rebuilt every step; by default a zero initial guess and
    tol = FLT_EPSILON as Eigen's ConjugateGradient uses (CPUSolver.cpp:65).
    Without `prev` the timed steps follow one untimed step from (u0, v0);
    with prev (the state one step before u0, v0) they start at (u0, v0)
    itself, the first one extrapolated from prev (warm_start 2), after an
    untimed step from the same state.  Returns (steps/s, CG iterations,
    seconds, nnz)."""
    O, S = cpu_system(xyz, tri)
    p = O.params(O.REACTION_DIFFUSION, 1.0, Du=2e-5, Dv=1e-5, F=0.037, k=0.06, reaction_mode=1,
                 tol=tol, warm_start=warm_start, nthreads=nthreads)
    u, v = S.gather(u0), S.gather(v0)
    pv = None if prev is None else (S.gather(prev[0]), S.gather(prev[1]))
    u1, v1, *_ = S.step(p, u, v, nsteps=1, prev=pv)  # warm-up (page-in)
    if prev is None:
        u, v = u1, v1  # the warm start's first guess
    t0 = time.perf_counter()
    u, v, _, it, _ = S.step(p, u, v, nsteps=nsteps, prev=pv)
    dt = time.perf_counter() - t0
    return nsteps / dt, it, dt, int(S.nnz)


def cpu_baselines(xyz, tri, u0, v0, steps_all, steps_one, guess, eq_state):
    """The CPU figures beside the GPU arm: the reference's semantics on all
    host cores and on one (the reference builds without OpenMP,
    CMakeLists.txt:106), and the same step with the GPU arm's tolerance and
    initial guess on all cores (equal work), which splits the GPU/CPU ratio
    into algorithm and hardware.  The equal-work sample runs the GPU arm's
    timed steps themselves: from the state where its timed region starts,
    eq_state = (u, v, u_prev, v_prev), four times as many steps as the other
    samples (they are cheaper)."""
    nthreads = os.cpu_count() or 1
    out = {}
    eu, ev, pu, pv = eq_state
    for name, nt, n, tol, ws, cg, start, prev in (
            ("threads_all", nthreads, steps_all, FLT_EPSILON, 0, REF_CG, (u0, v0), None),
            ("threads_1", 1, steps_one, FLT_EPSILON, 0, REF_CG, (u0, v0), None),
            ("equal_work", nthreads, 4 * steps_all, CG_TOL, 1 + guess, f"{EQ_CG}, start: {GUESS_LABEL[guess]}",
             (eu, ev), (pu, pv) if guess == 1 else None)):
        sps, it, dt, nnz = cpu_sample(xyz, tri, start[0], start[1], n, nt, tol, ws, prev)
        out[name] = {"value": sps, "unit": "steps/s", "cores": nt, "steps": n, "seconds": dt,
                     "cg_iterations_per_step": it / n, "cg": cg}
    return out


def run_reference(args, rank, world):
    """--impl reference: the CPU path timed on the host cores (rank 0 only)."""
    if rank != 0:
        return
    xyz, tri, u0, v0 = workload()
    nthreads = os.cpu_count() or 1
    cpu_sample(xyz, tri, u0, v0, max(1, args.warmup), nthreads)  # warm-up steps
    sps, it, dt, nnz = cpu_sample(xyz, tri, u0, v0, args.steps, nthreads)
    value = args.steps / dt
    cfg = config(int(xyz.shape[0]), int(tri.shape[0]), nnz,
                 {"parallelism": f"cpu, OpenMP {nthreads} threads", "cg": REF_CG,
                  "cg_iterations_per_step": it / args.steps})
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 / value, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": cfg,
            "cpu_baseline": {"value": value, "unit": "steps/s", "cores": nthreads, "kind": "port",
                             "sample": f"{args.steps} full steps of the workload, oracle FP32 port of the "
                                       f"reference's CPU step ({REF_CG}), OpenMP {nthreads} threads"},
            "e2e": {"value": value, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_probe(kind, cg_variant=None):
    """Small fixed runs for profiler captures (no JSON line).

    batch-iteration: the 256-instance batch is created (its autotuner times one
      iteration of each variant), started, stepped twice, and
      fea_batch_time_iteration runs 5 launches;
    batch-step: the batch with the extrapolated start, 6 steps, then one step
      inside the NVTX range "capture";
    step: the 1024 x 1024 handle, 25 steps, then one step inside "capture"."""
    import torch
    import fea_gb300 as F
    if kind == "step":
        xyz, tri, u0, v0 = workload()
        p = F.default_params(equation=F.REACTION_DIFFUSION, reaction_mode=1, cg_tolerance=CG_TOL,
                             cg_initial_guess=CG_GUESS, **PARAMS)
        s = F.CUDASolver(xyz, tri, boundary_condition=F.NEUMANN, precision=F.FP32, params=p)
        if cg_variant is not None:
            s.set_cg_variant(cg_variant)
        s.set_fields(u0, v0)
        s.advance_time(25)
        s.synchronize()
        torch.cuda.nvtx.range_push("capture")
        s.advance_time(1)
        s.synchronize()
        torch.cuda.nvtx.range_pop()
        st = s.status()
        print("iterations per field", list(st.last_iterations), "flags", st.flags)
        return
    insts, starts = batch_workload()
    B = F.BatchSolver(insts, cg_tolerance=BATCH_CG_TOL)
    if cg_variant is not None:
        B.set_cg_variant(cg_variant)
    if kind == "batch-step":
        B.set_initial_guess(CG_GUESS)
    for i, (u, w) in enumerate(starts):
        B.set_fields(i, u, w)
    if kind == "batch-iteration":
        B.advance_time(2)
        print("variant", B.cg_variant, "ms per iteration launch", B.time_iteration(5))
        return
    B.advance_time(6)
    B.synchronize()
    torch.cuda.nvtx.range_push("capture")
    B.advance_time(1)
    B.synchronize()
    torch.cuda.nvtx.range_pop()
    _, it = B.status()
    print("variant", B.cg_variant, "iterations of the last solve: max", int(it.max()), "mean", float(it.mean()))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-steps", type=int, default=2, help="steps of the all-cores CPU baseline samples")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-batch", action="store_true", help="skip the 256-instance batched sweep")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the adjoint inverse-problem timing")
    ap.add_argument("--no-configs", action="store_true", help="skip the heat and wave workload timings")
    ap.add_argument("--batch-steps", type=int, default=50)
    ap.add_argument("--plain-steps", type=int, default=3)
    ap.add_argument("--cg-variant", type=int, default=None,
                    help="CG kernel variant instead of the autotuned one (profiling captures)")
    ap.add_argument("--initial-guess", type=int, default=CG_GUESS,
                    help="cg_initial_guess: 0 previous solution, 1 extrapolated from the last two steps")
    ap.add_argument("--grid", type=int, default=GRID_N,
                    help="vertices per side (other sizes are for profiling captures, not bench lines)")
    ap.add_argument("--probe", choices=["step", "batch-step", "batch-iteration"], default=None,
                    help="a small fixed run for profiler captures instead of the bench (no JSON line)")
    args = ap.parse_args()
    if args.probe:
        return run_probe(args.probe, args.cg_variant)
    args.warmup = max(args.warmup, 3)
    globals()["GRID_N"] = args.grid

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return run_reference(args, rank, world)

    import numpy as np
    import torch
    import fea_gb300 as F

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    xyz, tri, u0, v0 = workload()
    p = F.default_params(equation=F.REACTION_DIFFUSION, reaction_mode=1, cg_tolerance=CG_TOL,
                         cg_initial_guess=args.initial_guess, **PARAMS)
    s = F.CUDASolver(xyz, tri, boundary_condition=F.NEUMANN, precision=F.FP32, params=p)
    lanes = s.autotune()
    if args.cg_variant is not None:
        s.set_cg_variant(args.cg_variant)
        lanes = args.cg_variant
    info = s.info
    N, nnz, V = info.num_unknowns, info.nnz, info.num_vertices
    stream = torch.cuda.ExternalStream(s.stream())
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def warm_to_start():
        """The warm-up from the initial state.  The device-timed and the end-to-end
        loops both start where it ends, with the history it leaves for the next
        step's extrapolated start, so they run the same steps (the steps are
        bit-for-bit repeatable; the CG iteration count changes as the pattern
        evolves).  Returns the state one step before the timed region."""
        s.set_fields(u0, v0)
        s.advance_time(args.warmup - 1)
        pu, pv = s.get_fields()
        s.advance_time(1)
        s.synchronize()
        return pu, pv

    prev_u, prev_v = warm_to_start()
    st0 = s.status()
    start_u, start_v = s.get_fields()

    # timed: K steps, L2 flushed before each, CUDA events on the solver stream
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with Clocks(local) as clk:
        with torch.cuda.stream(stream):
            for k in range(args.steps):
                flush.fill_(k & 0xFF)
                ev[k][0].record(stream)
                s.advance_time(1)
                ev[k][1].record(stream)
        s.synchronize()
        torch.cuda.synchronize()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    total_ms = sum(step_ms)
    st1 = s.status()
    total_ms = max_over_ranks(total_ms, dist, "cuda")
    iters = st1.total_iterations - st0.total_iterations
    # per step: rhs, 2 x init, refine, stepctl; the CG iteration kernels (counted on the device,
    # with the copies that close an unrolled loop pass); per call: start, final check
    launches = args.steps * 5 + (st1.cg_launches - st0.cg_launches) + 2 * args.steps
    value = world * args.steps / (total_ms / 1000.0)

    # one K-step graph launch (no flush between steps) for reference
    s.set_fields(start_u, start_v)
    s.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        e0.record(stream)
        s.advance_time(args.steps)
        e1.record(stream)
    s.synchronize()
    one_launch_ms = e0.elapsed_time(e1)

    # dominant kernel: one CG iteration, timed alone on the same operator
    spmv_ms = s.time_spmv(reps=20, flush_l2=True)
    spmv_warm_ms = s.time_spmv(reps=20, flush_l2=False)
    # every CG kernel variant on the same operator (L2 flushed), then back to the autotuned one
    variant_ms = {}
    for var in F.CG_VARIANTS:
        try:
            s.set_cg_variant(var)
        except F.FeaError:
            continue
        variant_ms[str(var)] = s.time_spmv(reps=10, flush_l2=True)
    s.set_cg_variant(lanes)
    peak, peak_kind = measured_peak_hbm()
    bytes_spmv = iter_bytes(N, nnz)

    # end to end through the C ABI with a host buffer: like surface->values,
    # one page-locked array that every step reads (set_values) and rewrites
    # (get_values) (values = v, CPUSolver.cpp:130,144)
    hv = torch.empty(V, dtype=torch.float32).pin_memory()
    vals = hv.numpy()
    lib = F.load()
    import ctypes as C
    vals[:] = start_v  # one untimed pass through the calls
    F.binding.check(lib.fea_set_values(s._h, C.c_void_p(vals.ctypes.data)))
    F.binding.check(lib.fea_advance_time(s._h, 1))
    F.binding.check(lib.fea_get_values(s._h, C.c_void_p(vals.ctypes.data)))
    warm_to_start()  # back to the device-timed loop's start state and history
    e2e_same_start = all(np.array_equal(a, b) for a, b in zip(s.get_fields(), (start_u, start_v)))
    vals[:] = start_v  # the state's own bits: writing them back keeps the history
    it_e2e0 = s.status().total_iterations
    s.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        F.binding.check(lib.fea_set_values(s._h, C.c_void_p(vals.ctypes.data)))
        F.binding.check(lib.fea_advance_time(s._h, 1))
        F.binding.check(lib.fea_get_values(s._h, C.c_void_p(vals.ctypes.data)))
    e2e_s = max_over_ranks(time.perf_counter() - t0, dist, "cuda")
    e2e = world * args.steps / e2e_s
    e2e_iters = (s.status().total_iterations - it_e2e0) / args.steps

    flags = s.status().flags
    # the cost of the FP64 true-residual pass (cg_refine = 2) against the
    # default float-float pass: the same steps from the same state, device-timed
    refine_ms = {}
    for mode in (1, 2):
        q = F.binding.Params.from_buffer_copy(p)
        q.cg_refine = mode
        s.set_params(q)
        s.set_fields(start_u, start_v)
        s.advance_time(1)  # graph instantiation
        s.set_fields(start_u, start_v)
        ms, its = _timed_steps(s, args.steps)
        refine_ms[mode] = (ms / args.steps, its / args.steps)
    s.set_params(p)
    # the roofline's launch duration: one CG iteration as the step loop runs it
    iter_ms, pinned_iters = in_loop_iteration_ms(F, s, p, start_u, start_v, stream)
    achieved = bytes_spmv / (iter_ms * 1e-3) / 1e9
    batched = None
    if not args.no_batch:
        batched = bench_batched(F, args.batch_steps, 3, args.plain_steps)
    adjoint = None if args.no_adjoint else bench_adjoint(F)
    gs_adjoint = None if args.no_adjoint else bench_gs_adjoint(F)
    configs = None if args.no_configs else bench_configs(F)
    cpu = None
    if rank == 0 and not args.no_cpu:
        runs = cpu_baselines(xyz, tri, u0, v0, args.cpu_steps, 1, args.initial_guess,
                             (start_u, start_v, prev_u, prev_v))
        a = runs["threads_all"]
        cpu = {"value": a["value"], "unit": "steps/s", "cores": a["cores"], "kind": "port",
               "sample": f"{a['steps']} full steps of the same workload ({a['seconds']:.1f} s), oracle FP32 "
                         f"port of the reference's CPU step ({REF_CG}), "
                         f"{a['cg_iterations_per_step']:.0f} CG iterations per step",
               **runs,
               "split": {"gpu_vs_cpu_same_semantics": value / a["value"],
                         "algorithm (reference semantics vs equal work, CPU)": runs["equal_work"]["value"] / a["value"],
                         "hardware (GPU vs CPU, equal work)": value / runs["equal_work"]["value"]}}
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": config(int(V), int(tri.shape[0]), int(nnz),
                             {"parallelism": "replicas" if world > 1 else "single gpu", "cg_variant": lanes,
                              "cg": f"jacobi-pcg, |r| < {CG_TOL:g} |b|, start: {GUESS_LABEL[args.initial_guess]}, "
                                    "float-float dots and scalars",
                              "cg_iterations_per_step": iters / args.steps,
                              "one_launch_ms_per_step": one_launch_ms / args.steps}),
            "e2e": {"value": e2e, "unit": "steps/s", "h2d_bytes_per_step": 4 * V, "d2h_bytes_per_step": 4 * V,
                    "cg_iterations_per_step": e2e_iters, "same_start_and_history_as_value": e2e_same_start,
                    "how": "set_values (host -> device) + advance_time(1) + get_values (device -> host) per step "
                           "through the C ABI, one page-locked host array, wall clock; the same steps as `value` "
                           "(same start state and extrapolation history), no L2 flush"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": IN_LOOP_TRAFFIC.get(lanes),
                         "frac_algorithmic": achieved / peak,
                         "frac_dram": (IN_LOOP_TRAFFIC[lanes] / (iter_ms * 1e-3) / 1e9 / peak
                                       if lanes in IN_LOOP_TRAFFIC else None),
                         "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum, in-loop launches, "
                                           "--cache-control none" if lanes in IN_LOOP_TRAFFIC else
                                           "no capture of this variant",
                         "kernel": f"{cg_kernel_name(lanes)} (one CG iteration: paired u,v product with "
                                   f"fused vector updates)",
                         "algorithmic_bytes_per_launch": bytes_spmv, "ms_per_launch": iter_ms,
                         "ms_per_launch_how": "in the step graph: pinned iteration counts "
                                              f"{pinned_iters[0]} and {pinned_iters[1]}, difference per iteration",
                         "ms_per_launch_isolated": spmv_ms, "ms_per_launch_isolated_l2_warm": spmv_warm_ms,
                         "isolated_how": "one launch after a 256 MiB read evicting the L2; its own writes "
                                         "are written back after the timing, so it reads low",
                         "peak_source": peak_kind, "variant": lanes,
                         "ms_per_launch_isolated_by_variant": variant_ms},
            "cpu_baseline": cpu,
            "refinement": {"float_float_ms_per_step": refine_ms[1][0], "fp64_ms_per_step": refine_ms[2][0],
                           "float_float_cg_iterations_per_step": refine_ms[1][1],
                           "fp64_cg_iterations_per_step": refine_ms[2][1],
                           "how": "cg_refine 1 and 2, the same steps from the warm-up state, no L2 flush"},
            "batched": batched,
            "adjoint": adjoint,
            "gray_scott_adjoint": gs_adjoint,
            "other_workloads": configs,
            "clocks": clk.summary(),
            "gpu_launches": int(launches),
            "status_flags": int(flags),
        }
        print(json.dumps(line), flush=True)
    s.close()
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
