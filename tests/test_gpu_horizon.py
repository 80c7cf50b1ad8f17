"""Accuracy of the 1M-vertex Gray-Scott workload (the bench's workload) over
its whole horizon of 2,000 steps, against the FP64 oracle.

The oracle's states come from tests/golden/make_gray_scott_states.py (CPU,
hours at full length; the fields stay out of git).  The tests skip, naming
that script, when its states are absent.
- Per step: from the oracle's state after k steps (rounded to float32, as the
  handle holds it), one GPU step must stay within rel-L2 1e-5 of the oracle's
  step per field -- the metric's accuracy bar -- for k from the bench's
  warm-up (5) and its timed steps (25, 55) to the end of the horizon (2,000).
  A state set from outside starts its first step from the previous
  solution; the bench's extrapolated start is exercised by the drift run.
- Drift: the GPU run from the initial state against the oracle's trajectory,
  with the bench's tolerance and initial guess.
  Gray-Scott patterns are unstable, so the drift grows with the horizon; it is
  printed and bounded, and the per-step bar is the contract.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN, rel_l2

pytestmark = pytest.mark.gpu

STATES = os.path.join(GOLDEN, "_states")
PER_STEP = (5, 25, 55, 100, 250, 500, 1000, 1500, 2000)
# rel-L2 drift bounds of the GPU run from the initial state, per horizon
# (u and v), with the bench's tolerance and extrapolated start.  Measured on
# a GB300 (u / v): 2.7e-6 / 1.7e-5 after 25 steps, 4.4e-6 / 2.3e-5 after 55,
# 7.4e-6 / 4.0e-5 after 100, 3.9e-5 / 1.2e-4 after 250, 7.6e-5 / 1.8e-4
# after 500, 2.4e-4 / 4.7e-4 after 1,000, 6.5e-4 / 1.2e-3 after 1,500 and
# 7.6e-4 / 1.4e-3 after 2,000.  The per-step error stays near 1e-6 (FP32
# operator values: the drift after 100 steps is the same at CG tolerances
# down to 1e-7), and the unstable pattern amplifies it.  Bounds: about 2.5x
# the measured drift.
DRIFT_BOUND = {25: 5e-5, 55: 6e-5, 100: 1e-4, 250: 3e-4, 500: 5e-4, 1000: 1.2e-3, 1500: 3e-3, 2000: 3.5e-3}


def _state(k):
    path = os.path.join(STATES, f"gray_scott_1024_k{k}.npz")
    if not os.path.exists(path):
        pytest.skip(f"oracle state after {k} steps absent: run tests/golden/make_gray_scott_states.py")
    return np.load(path)


@pytest.fixture(scope="module")
def handle(fea):
    import bench
    xyz, tri, u0, v0 = bench.workload()
    p = fea.default_params(equation=fea.REACTION_DIFFUSION, reaction_mode=1, cg_tolerance=bench.CG_TOL,
                           cg_initial_guess=bench.CG_GUESS, **bench.PARAMS)
    s = fea.CUDASolver(xyz, tri, boundary_condition=fea.NEUMANN, precision=fea.FP32, params=p)
    yield s, u0, v0
    s.close()


@pytest.mark.parametrize("k", PER_STEP)
def test_per_step_error_from_oracle_state(handle, k):
    s, _, _ = handle
    z = _state(k)
    s.set_fields(z["u"], z["v"])
    s.advance_time(1)
    ug, vg = s.get_fields()
    eu, ev = rel_l2(ug, z["next_u"]), rel_l2(vg, z["next_v"])
    print(f"step {k} -> {k + 1}: rel-L2 u {eu:.3e} v {ev:.3e}, CG iterations {list(s.status().last_iterations)}")
    assert s.status().flags == 0
    assert eu < 1e-5 and ev < 1e-5


def test_drift_over_the_horizon(handle):
    s, u0, v0 = handle
    horizons = [k for k in sorted(DRIFT_BOUND) if os.path.exists(os.path.join(STATES, f"gray_scott_1024_k{k}.npz"))]
    if not horizons:
        pytest.skip("no oracle states: run tests/golden/make_gray_scott_states.py")
    s.set_fields(u0, v0)
    done, report = 0, []
    for k in horizons:
        s.advance_time(k - done)
        done = k
        z = np.load(os.path.join(STATES, f"gray_scott_1024_k{k}.npz"))
        ug, vg = s.get_fields()
        eu, ev = rel_l2(ug, z["u"]), rel_l2(vg, z["v"])
        report.append((k, eu, ev))
        print(f"drift after {k} steps: rel-L2 u {eu:.3e} v {ev:.3e}")
    assert s.status().flags == 0
    for k, eu, ev in report:
        assert eu < DRIFT_BOUND[k] and ev < DRIFT_BOUND[k], (k, eu, ev)
