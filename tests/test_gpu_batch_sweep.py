"""The batched sweep at its full size: all 256 Gray-Scott instances of the
bench's batch (icospheres of levels 3 to 6, F ~ U(0.01, 0.06), k ~
U(0.045, 0.07), Du 2e-4, Dv 1e-4, dt 0.5, the bench's CG tolerance).

- One step of every instance from the oracle's state (two FP64 oracle steps
  after the instance's start, rounded to float32) against the oracle's step,
  within rel-L2 1e-5 per field, at the sweep's CG tolerance (1e-6: at 1e-5
  the worst instance measured 1.9e-5).
- 1,000 steps of the batch against 1,000 steps of single-mesh handles of the
  same instances (the configuration's horizon): printed and bounded.
"""
import os

import numpy as np
import pytest

from conftest import oracle_step, rel_l2

pytestmark = pytest.mark.gpu

HORIZON = 1000
# rel-L2 bound of batch vs single handles after HORIZON steps.  Both solve
# every step to the same tolerance, but their CG iterations sum the rows'
# inner products in per-thread groups of different rows (a batch group of at
# most 8 tiles; a single handle's block share), so alpha and beta differ in
# their last bits, and unstable patterns amplify that over the horizon.
# Measured on a GB300: median 1.3e-6, 95th percentile 1.6e-5, worst 1.2e-3,
# the order of the FP32 drift against the FP64 oracle (1.4e-3 after 2,000
# steps on the 1M-vertex workload).  Bound: about 4x the worst.
HORIZON_BOUND = 5e-3


@pytest.fixture(scope="module")
def sweep():
    import bench
    insts, starts = bench.batch_workload()
    return bench, insts, starts


def test_every_instance_one_step_from_oracle_state(fea, oracle_mod, sweep):
    bench, insts, starts = sweep
    B = fea.BatchSolver(insts, cg_tolerance=bench.BATCH_CG_TOL)
    systems = {}
    refs = []
    for i, (d, (u0, v0)) in enumerate(zip(insts, starts)):
        key = d["vertices"].shape[0]
        if key not in systems:
            systems[key] = oracle_mod.System(d["vertices"], d["triangles"], bc=oracle_mod.NEUMANN)
        S = systems[key]
        kw = dict(Du=d["Du"], Dv=d["Dv"], F=d["feed_rate"], k=d["kill_rate"], reaction_mode=1)
        u, v, *_ = oracle_step(oracle_mod, S, oracle_mod.REACTION_DIFFUSION, d["time_step"],
                               S.gather(u0.astype(np.float32)), S.gather(v0.astype(np.float32)), 2, **kw)
        us, vs = S.scatter(u).astype(np.float32), S.scatter(v).astype(np.float32)
        uo, vo, *_ = oracle_step(oracle_mod, S, oracle_mod.REACTION_DIFFUSION, d["time_step"], S.gather(us),
                                 S.gather(vs), 1, **kw)
        B.set_fields(i, us, vs)
        refs.append((S.scatter(uo), S.scatter(vo)))
    B.advance_time(1)
    flags, iters = B.status()
    assert np.all(flags == 0) and np.all(iters > 0)
    worst = (0.0, 0.0, -1)
    for i, (uo, vo) in enumerate(refs):
        ug, vg = B.get_fields(i)
        eu, ev = rel_l2(ug, uo), rel_l2(vg, vo)
        worst = max(worst, (eu, ev, i), key=lambda w: max(w[0], w[1]))
        assert eu < 1e-5 and ev < 1e-5, (i, eu, ev)
    print(f"256 instances, one step from the oracle's state: worst rel-L2 u {worst[0]:.3e} v {worst[1]:.3e} "
          f"(instance {worst[2]})")
    B.close()


def test_batch_vs_single_handles_over_the_horizon(fea, sweep):
    bench, insts, starts = sweep
    B = fea.BatchSolver(insts, cg_tolerance=bench.BATCH_CG_TOL)
    for i, (u, v) in enumerate(starts):
        B.set_fields(i, u, v)
    B.advance_time(HORIZON)
    flags, _ = B.status()
    assert np.all(flags == 0)
    worst, errs = 0.0, []
    for i, (d, (u, v)) in enumerate(zip(insts, starts)):
        p = fea.default_params(equation=fea.REACTION_DIFFUSION, reaction_mode=1, rd_time_step=d["time_step"],
                               rd_Du=d["Du"], rd_Dv=d["Dv"], rd_feed_rate=d["feed_rate"],
                               rd_kill_rate=d["kill_rate"], cg_tolerance=bench.BATCH_CG_TOL)
        s = fea.CUDASolver(d["vertices"], d["triangles"], boundary_condition=fea.NEUMANN, params=p)
        s.set_fields(u, v)
        s.advance_time(HORIZON)
        assert s.status().flags == 0
        us, vs = s.get_fields()
        ub, vb = B.get_fields(i)
        e = max(rel_l2(ub, us), rel_l2(vb, vs))
        errs.append(e)
        s.close()
    errs = np.array(errs)
    print(f"batch vs single handles after {HORIZON} steps: rel-L2 median {np.median(errs):.3e}, "
          f"95th percentile {np.percentile(errs, 95):.3e}, worst {errs.max():.3e} (instance {errs.argmax()})")
    assert errs.max() < HORIZON_BOUND
    B.close()
