"""FP64 oracle states of the 1M-vertex Gray-Scott workload (the bench's
workload: 1024 x 1024 jittered grid, mass-weighted reaction, Du 2e-5, Dv 1e-5,
F 0.037, k 0.06, dt 1) along a long trajectory, for the accuracy tests of
tests/test_gpu_horizon.py.  CPU only; it takes hours at full length.

    python tests/golden/make_gray_scott_states.py [--steps 2000] [--threads N]

From the bench's initial state the oracle (the C restatement of the
reference's CPU step, FP64, Jacobi-PCG to |r| < 1e-12 |b|) steps forward.  At
each checkpoint step k it writes tests/golden/_states/gray_scott_1024_k{k}.npz
holding
  u, v           the state after k steps, rounded to float32 (the form the
                 GPU handle is given);
  next_u, next_v one oracle step from that rounded state (float32 storage).
The fields stay out of git (16 MB per checkpoint).  A resume file in the same
folder lets an interrupted run continue.
"""
import argparse
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "_states")
CHECKPOINTS = (5, 25, 55, 100, 250, 500, 1000, 1500, 2000)
ORACLE_TOL = 1e-12


def state_path(k):
    return os.path.join(OUT, f"gray_scott_1024_k{k}.npz")


def oracle_params(O, nthreads):
    f32 = lambda x: float(np.float32(x))  # noqa: E731  the ABI carries float parameters
    return O.params(O.REACTION_DIFFUSION, 1.0, Du=f32(2e-5), Dv=f32(1e-5), F=f32(0.037), k=f32(0.06),
                    reaction_mode=1, tol=ORACLE_TOL, nthreads=nthreads)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    args = ap.parse_args()
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "fea-visualizer_gb300"))
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import bench
    import oracle as O
    O.build()
    os.makedirs(OUT, exist_ok=True)
    xyz, tri, u0, v0 = bench.workload()
    S = O.System(xyz, tri, bc=O.NEUMANN)
    p = oracle_params(O, args.threads)
    resume = os.path.join(OUT, "resume.npz")
    log = os.path.join(OUT, "log.jsonl")
    if os.path.exists(resume):
        z = np.load(resume)
        k, u, v = int(z["k"]), z["u"], z["v"]
    else:
        k, u, v = 0, S.gather(u0.astype(np.float64)), S.gather(v0.astype(np.float64))
    while k < args.steps:
        t0 = time.time()
        u, v, _, it, flags = S.step(p, u, v, nsteps=1)
        k += 1
        rec = {"k": k, "iterations": it, "flags": flags, "seconds": round(time.time() - t0, 2)}
        if k in CHECKPOINTS:
            us, vs = S.scatter(u).astype(np.float32), S.scatter(v).astype(np.float32)
            nu, nv, *_ = S.step(p, S.gather(us), S.gather(vs), nsteps=1)
            np.savez(state_path(k), u=us, v=vs, next_u=S.scatter(nu).astype(np.float32),
                     next_v=S.scatter(nv).astype(np.float32), oracle_tol=ORACLE_TOL)
            rec["saved"] = os.path.basename(state_path(k))
        if k % 25 == 0 or k in CHECKPOINTS:
            np.savez(resume, k=k, u=u, v=v)
        with open(log, "a") as fh:
            fh.write(json.dumps(rec) + "\n")
    print(f"done: {k} steps")


if __name__ == "__main__":
    main()
