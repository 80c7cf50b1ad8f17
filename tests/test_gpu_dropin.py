"""The reference application's frame loop through the C++ drop-in shim
(fea-visualizer_gb300/host/cuda_solver.hpp), built with g++ against the C ABI."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, rel_l2
from fea_gb300 import meshgen as mg

HOST = os.path.join(ROOT, "fea-visualizer_gb300", "host")
LIBDIR = os.path.join(ROOT, "fea-visualizer_gb300", "lib")


def build_demo(tmp_path):
    exe = str(tmp_path / "drop_in_demo")
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), "-I", HOST,
                    os.path.join(HOST, "drop_in_demo.cpp"), "-L", LIBDIR, "-lfea_gb300",
                    f"-Wl,-rpath,{LIBDIR}", "-o", exe], check=True)
    return exe


def test_demo_compiles(tmp_path):
    """CPU: the shim and the demo compile and link against the library."""
    import __graft_entry__ as ge
    ge.build_library()
    assert os.path.exists(build_demo(tmp_path))


@pytest.mark.gpu
@pytest.mark.parametrize("bc", [0, 1])
def test_heat_frames_through_shim(fea, oracle_mod, tmp_path, bc):
    exe = build_demo(tmp_path)
    xyz, tri = mg.cylinder(36, 14)
    u0 = np.cos(2 * np.arctan2(xyz[:, 1], xyz[:, 0])).astype(np.float32) + 1.0
    mesh = tmp_path / "mesh.bin"
    with open(mesh, "wb") as fh:
        fh.write(np.array([xyz.shape[0], tri.shape[0]], np.int64).tobytes())
        fh.write(xyz.tobytes())
        fh.write(tri.astype(np.uint32).tobytes())
        fh.write(u0.tobytes())
    out = tmp_path / "out.bin"
    frames = 5
    ply = tmp_path / "out.ply"
    subprocess.run([exe, str(mesh), str(out), "0", str(bc), str(frames), str(ply)], check=True)
    raw = np.fromfile(out, dtype=np.float32)
    vals, unstable = raw[:-1], raw[-1:].view(np.int32)[0]
    assert unstable == 0
    S = oracle_mod.System(xyz, tri, bc=bc)
    # reference defaults: HeatParameters dt 0.01, conductivity 0.05 (float)
    p = oracle_mod.params(oracle_mod.HEAT, float(np.float32(0.01)), kappa=float(np.float32(0.05)), tol=1e-14)
    u = S.gather(u0)
    for _ in range(frames):
        u, *_ = S.step(p, u, np.zeros(S.N), nsteps=1)
        u = S.gather(S.scatter(u).astype(np.float32))  # the frame loop round-trips float values
    assert rel_l2(vals, S.scatter(u)) < 1e-5
    if bc == 0:
        assert np.all(vals[S.on_boundary == 1] == 0)
    # the export at the end of the loop (threshold 0, Open): geometry as the oracle's
    normals = np.tile(np.array([0.0, 0.0, 1.0], np.float32), (len(xyz), 1))
    P, _, T = oracle_mod.ply_clip(xyz, tri, normals, vals, 0.25, 0.0, 0)
    lines = ply.read_text().splitlines()
    assert lines[0] == "ply" and lines[2] == f"element vertex {len(P)}" and lines[9] == f"element face {len(T)}"
