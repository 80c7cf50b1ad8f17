"""Batched Gray-Scott (fea_batch_*) against the oracle and the single-mesh path.

Every instance follows the mass-weighted Gray-Scott step of its own mesh and
parameters.  Bars: one step from the oracle's state agrees with the FP64
oracle (solved to 1e-14) to rel-L2 1e-5 per field for FP32 and 1e-9 for FP64;
ten steps agree with single-mesh handles of the same instances to 1e-5; runs
are bit-for-bit repeatable; an instance frozen by a blow-up leaves the others
bit-identical.
"""
import numpy as np
import pytest

from conftest import oracle_step, rel_l2
from fea_gb300 import meshgen as mg

pytestmark = pytest.mark.gpu


def _instances():
    """Uneven meshes and parameters, Neumann and Dirichlet."""
    rng = np.random.default_rng(11)
    meshes = [
        (mg.icosphere(2), 1), (mg.icosphere(3), 1), (mg.icosphere(4), 1),
        (mg.jittered_grid(33, seed=3), 0), (mg.cylinder(40, 15), 1), (mg.icosphere(3), 1),
    ]
    out = []
    for (xyz, tri), bc in meshes:
        planar = np.ptp(xyz[:, 2]) == 0
        out.append(dict(vertices=xyz, triangles=tri, boundary_condition=bc,
                        time_step=1.0 if planar else 0.5,
                        Du=2e-5 if planar else 2e-4, Dv=1e-5 if planar else 1e-4,
                        feed_rate=float(rng.uniform(0.01, 0.06)), kill_rate=float(rng.uniform(0.045, 0.07))))
    return out


def _start(inst, seed):
    xyz = inst["vertices"]
    if np.ptp(xyz[:, 2]) == 0:
        return mg.gray_scott_patches(xyz, seed=seed, side=0.15)
    return mg.sphere_patches(xyz / np.linalg.norm(xyz, axis=1, keepdims=True), seed=seed, n_patches=6,
                             radius=0.3)


def _okw(inst):
    return dict(Du=inst["Du"], Dv=inst["Dv"], F=inst["feed_rate"], k=inst["kill_rate"], reaction_mode=1)


@pytest.mark.parametrize("precision,tol,cg_tol", [(0, 1e-5, 1e-7), (1, 1e-9, 1e-12)])
def test_batched_steps_match_oracle(fea, oracle_mod, precision, tol, cg_tol):
    insts = _instances()
    B = fea.BatchSolver(insts, precision=precision, cg_tolerance=cg_tol)
    systems = [oracle_mod.System(d["vertices"], d["triangles"], bc=d["boundary_condition"]) for d in insts]
    states = []
    for i, (d, S) in enumerate(zip(insts, systems)):
        u0, v0 = _start(d, i)
        states.append((S.gather(u0.astype(np.float32)), S.gather(v0.astype(np.float32))))
    for step in range(2):
        for i, (S, (u, v)) in enumerate(zip(systems, states)):
            B.set_fields(i, S.scatter(u).astype(np.float32), S.scatter(v).astype(np.float32))
        B.advance_time(1)
        flags, iters = B.status()
        assert np.all(flags == 0) and np.all(iters > 0), (flags, iters)
        for i, (d, S, (u, v)) in enumerate(zip(insts, systems, states)):
            uf = S.gather(S.scatter(u).astype(np.float32))
            vf = S.gather(S.scatter(v).astype(np.float32))
            uo, vo, *_ = oracle_step(oracle_mod, S, oracle_mod.REACTION_DIFFUSION, d["time_step"], uf, vf, 1,
                                     **_okw(d))
            ug, vg = B.get_fields(i)
            # node values travel as float32: the bar is at least their resolution
            bar = max(tol, 1e-7)
            assert rel_l2(ug, S.scatter(uo)) < bar and rel_l2(vg, S.scatter(vo)) < bar, (step, i)
            if d["boundary_condition"] == 0:
                assert np.all(ug[S.on_boundary == 1] == 0)
            states[i] = (uo, vo)


def test_batched_matches_single_mesh_handles(fea):
    insts = _instances()
    B = fea.BatchSolver(insts, cg_tolerance=1e-6)
    singles = []
    for i, d in enumerate(insts):
        u0, v0 = _start(d, 100 + i)
        B.set_fields(i, u0, v0)
        p = fea.default_params(equation=fea.REACTION_DIFFUSION, reaction_mode=1, rd_time_step=d["time_step"],
                               rd_Du=d["Du"], rd_Dv=d["Dv"], rd_feed_rate=d["feed_rate"],
                               rd_kill_rate=d["kill_rate"], cg_tolerance=1e-6)
        s = fea.CUDASolver(d["vertices"], d["triangles"], boundary_condition=d["boundary_condition"], params=p)
        s.set_fields(u0, v0)
        singles.append(s)
    B.advance_time(10)
    for s in singles:
        s.advance_time(10)
    _, iters = B.status()
    for i, s in enumerate(singles):
        ub, vb = B.get_fields(i)
        us, vs = s.get_fields()
        assert rel_l2(ub, us) < 1e-5 and rel_l2(vb, vs) < 1e-5, i
        st = s.status()
        assert abs(int(iters[i, 0]) - st.last_iterations[0]) <= 1
        assert abs(int(iters[i, 1]) - st.last_iterations[1]) <= 1


@pytest.mark.parametrize("variant", [0, 14])
def test_batched_repeatable_and_masked(fea, variant):
    insts = _instances()
    runs = []
    for _ in range(2):
        B = fea.BatchSolver(insts, cg_tolerance=1e-6)
        B.set_cg_variant(variant)  # bit-for-bit comparisons need the same kernels
        for i, d in enumerate(insts):
            B.set_fields(i, *_start(d, 7 + i))
        B.advance_time(5)
        runs.append([np.concatenate(B.get_fields(i)) for i in range(len(insts))])
        _, iters = B.status()
        # the masks let every instance stop at its own iteration count
        assert len(set(iters[:, 0].tolist())) > 1, iters
        B.close()
    for a, b in zip(*runs):
        np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("variant", [0, 14])
def test_blowup_freezes_only_its_instance(fea, variant):
    insts = _instances()
    starts = [_start(d, 30 + i) for i, d in enumerate(insts)]
    ref = fea.BatchSolver(insts, cg_tolerance=1e-6)
    bad = fea.BatchSolver(insts, cg_tolerance=1e-6)
    ref.set_cg_variant(variant)
    bad.set_cg_variant(variant)
    for i, (u, v) in enumerate(starts):
        ref.set_fields(i, u, v)
        if i == 1:
            u = u.copy()
            u[5] = 2e4  # above the 1e4 instability threshold (CPUSolver.cpp:41-48)
        bad.set_fields(i, u, v)
    ref.advance_time(3)
    bad.advance_time(3)
    flags, _ = bad.status()
    assert flags[1] & fea.binding.STATUS_BLOWUP
    assert np.all(np.delete(flags, 1) == 0)
    u1, _ = bad.get_fields(1)
    assert u1[5] == np.float32(2e4)  # frozen: never stepped
    for i in range(len(insts)):
        if i == 1:
            continue
        for a, b in zip(ref.get_fields(i), bad.get_fields(i)):
            np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("variant", [0, 1, 4, 8, 14])
def test_batched_variants_match_oracle(fea, oracle_mod, variant):
    insts = _instances()
    B = fea.BatchSolver(insts, cg_tolerance=1e-7)
    B.set_cg_variant(variant)
    assert B.cg_variant == variant
    for i, d in enumerate(insts):
        B.set_fields(i, *_start(d, 50 + i))
    B.advance_time(2)
    for i, d in enumerate(insts):
        S = oracle_mod.System(d["vertices"], d["triangles"], bc=d["boundary_condition"])
        u0, v0 = _start(d, 50 + i)
        uo, vo, *_ = oracle_step(oracle_mod, S, oracle_mod.REACTION_DIFFUSION, d["time_step"],
                                 S.gather(u0.astype(np.float32)), S.gather(v0.astype(np.float32)), 2, **_okw(d))
        ug, vg = B.get_fields(i)
        assert rel_l2(ug, S.scatter(uo)) < 1e-5 and rel_l2(vg, S.scatter(vo)) < 1e-5, (variant, i)


def test_batch_arguments(fea):
    insts = _instances()[:2]
    B = fea.BatchSolver(insts)
    with pytest.raises(fea.FeaError):
        B.get_fields(2)
    with pytest.raises(fea.FeaError):
        B.advance_time(-1)
    with pytest.raises(fea.FeaError):
        B.set_cg_variant(2)
    with pytest.raises(fea.FeaError):
        B.set_initial_guess(2)


@pytest.mark.parametrize("variant", [0, 14])
def test_instance_independent_of_batch(fea, variant):
    """An instance's results do not depend on the other instances: each
    instance stepped alone in a batch of one matches its fields in the full
    batch bit for bit (its partial sums are grouped by its own tiles only)."""
    insts = _instances()
    B = fea.BatchSolver(insts, cg_tolerance=1e-6)
    B.set_cg_variant(variant)
    for i, d in enumerate(insts):
        B.set_fields(i, *_start(d, 60 + i))
    B.advance_time(3)
    for i, d in enumerate(insts):
        one = fea.BatchSolver([d], cg_tolerance=1e-6)
        one.set_cg_variant(variant)
        one.set_fields(0, *_start(d, 60 + i))
        one.advance_time(3)
        for a, b in zip(B.get_fields(i), one.get_fields(0)):
            np.testing.assert_array_equal(a, b)
        one.close()


@pytest.mark.parametrize("variant", [0, 14])
def test_batch_timing_probe_leaves_state(fea, variant):
    """fea_batch_time_iteration runs the iteration kernel over every instance
    with the fields masked: the steps that follow match an unprobed batch bit
    for bit."""
    insts = _instances()
    out = []
    for probe in (False, True):
        B = fea.BatchSolver(insts, cg_tolerance=1e-6)
        B.set_cg_variant(variant)
        for i, d in enumerate(insts):
            B.set_fields(i, *_start(d, 40 + i))
        B.advance_time(2)
        if probe:
            assert B.time_iteration(3) > 0
        B.advance_time(3)
        out.append([B.get_fields(i) for i in range(len(insts))])
        B.close()
    for (ua, va), (ub, vb) in zip(*out):
        assert np.array_equal(ua, ub) and np.array_equal(va, vb)


def _extrapolating_batch(fea, insts, seed, tol=1e-6, precision=0):
    B = fea.BatchSolver(insts, precision=precision, cg_tolerance=tol)
    B.set_cg_variant(14)
    B.set_initial_guess(1)
    for i, d in enumerate(insts):
        B.set_fields(i, *_start(d, seed + i))
    return B


def test_extrapolated_start_matches_single_mesh_handles(fea):
    """Rule 1 (solves started from 2 x_n - x_(n-1)) against single-mesh
    handles with cg_initial_guess 1: the same states to 1e-5 over ten steps
    and iteration counts within 2.  Against the rule-0 batch, whose solves
    start elsewhere and so stop at other points within the tolerance (1e-6
    per solve), the states agree to 5e-5 and rule 1 takes fewer iterations."""
    insts = _instances()
    B = _extrapolating_batch(fea, insts, 300)
    B0 = fea.BatchSolver(insts, cg_tolerance=1e-6)
    B0.set_cg_variant(14)
    singles = []
    for i, d in enumerate(insts):
        u0, v0 = _start(d, 300 + i)
        B0.set_fields(i, u0, v0)
        p = fea.default_params(equation=fea.REACTION_DIFFUSION, reaction_mode=1, rd_time_step=d["time_step"],
                               rd_Du=d["Du"], rd_Dv=d["Dv"], rd_feed_rate=d["feed_rate"],
                               rd_kill_rate=d["kill_rate"], cg_tolerance=1e-6, cg_initial_guess=1)
        s = fea.CUDASolver(d["vertices"], d["triangles"], boundary_condition=d["boundary_condition"], params=p)
        s.set_fields(u0, v0)
        singles.append(s)
    B.advance_time(10)
    B0.advance_time(10)
    for s in singles:
        s.advance_time(10)
    _, iters = B.status()
    for i, s in enumerate(singles):
        ub, vb = B.get_fields(i)
        us, vs = s.get_fields()
        assert rel_l2(ub, us) < 1e-5 and rel_l2(vb, vs) < 1e-5, i
        u0b, v0b = B0.get_fields(i)
        assert rel_l2(ub, u0b) < 5e-5 and rel_l2(vb, v0b) < 5e-5, i
        st = s.status()
        assert abs(int(iters[i, 0]) - st.last_iterations[0]) <= 2, (i, iters[i], st.last_iterations)
        assert abs(int(iters[i, 1]) - st.last_iterations[1]) <= 2, (i, iters[i], st.last_iterations)
    it1, steps1 = B.counters()
    it0, steps0 = B0.counters()
    assert np.all(steps1 == 10) and np.all(steps0 == 10)
    assert it1.sum() < it0.sum(), (it1, it0)


@pytest.mark.parametrize("precision,cg_tol,bar", [(0, 1e-7, 1e-5), (1, 1e-12, 1e-9)])
def test_extrapolated_start_matches_oracle(fea, oracle_mod, precision, cg_tol, bar):
    """Rule 1 over three steps against the FP64 oracle (solved to 1e-14),
    FP32 and FP64 batches: the start only changes where CG begins, not what
    it converges to."""
    insts = _instances()
    B = _extrapolating_batch(fea, insts, 320, tol=cg_tol, precision=precision)
    B.advance_time(3)
    for i, d in enumerate(insts):
        S = oracle_mod.System(d["vertices"], d["triangles"], bc=d["boundary_condition"])
        u0, v0 = _start(d, 320 + i)
        uo, vo, *_ = oracle_step(oracle_mod, S, oracle_mod.REACTION_DIFFUSION, d["time_step"],
                                 S.gather(u0.astype(np.float32)), S.gather(v0.astype(np.float32)), 3, **_okw(d))
        ug, vg = B.get_fields(i)
        # node values travel as float32: the bar is at least their resolution
        b = max(bar, 1e-7)
        assert rel_l2(ug, S.scatter(uo)) < b and rel_l2(vg, S.scatter(vo)) < b, i


def test_extrapolated_start_histories(fea):
    """Histories are per instance: new fields for one instance restart its
    history (its next step starts from x_n, bit-identical to a fresh batch),
    and an instance stepped alone matches the full batch bit for bit."""
    insts = _instances()
    B = _extrapolating_batch(fea, insts, 340)
    B.advance_time(3)
    u5, v5 = _start(insts[2], 999)
    B.set_fields(2, u5, v5)
    B.advance_time(2)
    one = fea.BatchSolver([insts[2]], cg_tolerance=1e-6)
    one.set_cg_variant(14)
    one.set_initial_guess(1)
    one.set_fields(0, u5, v5)
    one.advance_time(2)
    for a, b in zip(B.get_fields(2), one.get_fields(0)):
        np.testing.assert_array_equal(a, b)
    one.close()
    for i in (0, 4):
        one = _extrapolating_batch(fea, [insts[i]], 340 + i)
        one.advance_time(5)
        for a, b in zip(B.get_fields(i), one.get_fields(0)):
            np.testing.assert_array_equal(a, b)
        one.close()


def test_extrapolated_start_rule_switch(fea):
    """Switching rule 1 off returns to the x_n start: a batch stepped with
    rule 1, switched to rule 0, steps bit-identically to a rule-0 batch
    given the same state."""
    insts = _instances()[:3]
    B = _extrapolating_batch(fea, insts, 360)
    B.advance_time(3)
    states = [B.get_fields(i) for i in range(len(insts))]
    B.set_initial_guess(0)
    B.advance_time(2)
    R = fea.BatchSolver(insts, cg_tolerance=1e-6)
    R.set_cg_variant(14)
    for i, (u, v) in enumerate(states):
        R.set_fields(i, u, v)
    R.advance_time(2)
    for i in range(len(insts)):
        for a, b in zip(B.get_fields(i), R.get_fields(i)):
            np.testing.assert_array_equal(a, b)
