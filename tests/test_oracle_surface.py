"""Known-answer checks of the oracle's post-solve steps (CPU only): extruded
smooth normals (shaders/FEM/smooth_normals.glsl) and the iso-clipped .ply
geometry (Surface::export_to_ply, Surface.cpp:138-285)."""
import numpy as np

from fea_gb300 import meshgen as mg


def _face_normals(xyz, tri):
    a, b, c = (xyz[tri[:, i]].astype(np.float64) for i in range(3))
    return np.cross(b - a, c - a)


def test_smooth_normals_without_extrusion_are_face_sums(oracle_mod):
    xyz, tri = mg.icosphere(3)
    nrm = xyz / np.linalg.norm(xyz, axis=1, keepdims=True)
    out = oracle_mod.smooth_normals(xyz, tri, nrm, np.zeros(len(xyz)), 0.7).astype(np.float64)
    ref = np.zeros_like(out)
    for i in range(3):
        np.add.at(ref, tri[:, i], _face_normals(xyz, tri))
    np.testing.assert_allclose(out, ref, rtol=1e-5, atol=1e-7)
    # outward orientation: every vertex normal points away from the centre
    assert np.all(np.sum(out * nrm, axis=1) > 0)
    # a closed surface's area vectors cancel
    assert np.abs(out.sum(axis=0)).max() < 1e-5


def test_smooth_normals_extrusion_is_clamped(oracle_mod):
    xyz, tri = mg.icosphere(2)
    nrm = xyz / np.linalg.norm(xyz, axis=1, keepdims=True)
    # value * extrusion clamps at 1 and negative values do not extrude: a
    # uniform value v gives the sphere of radius 1 + min(1, e * max(0, v))
    for v, e, r in ((0.5, 0.4, 1.2), (5.0, 0.4, 2.0), (-3.0, 0.4, 1.0)):
        out = oracle_mod.smooth_normals(xyz, tri, nrm, np.full(len(xyz), v), e).astype(np.float64)
        base = oracle_mod.smooth_normals(xyz, tri, nrm, np.zeros(len(xyz)), e).astype(np.float64)
        np.testing.assert_allclose(out, base * r * r, rtol=1e-4, atol=1e-6)


def test_ply_clip_everything_above(oracle_mod):
    xyz, tri = mg.icosphere(2)
    nrm = xyz / np.linalg.norm(xyz, axis=1, keepdims=True)
    vals = 0.5 + 0.1 * xyz[:, 0]
    P, pv, T = oracle_mod.ply_clip(xyz, tri, nrm, vals, 0.25, -1.0, 0)
    # every corner kept once, every triangle kept with its corners renumbered
    assert P.shape == (len(xyz), 3) and T.shape == tri.shape
    ext = xyz + (vals * 0.25)[:, None].astype(np.float32) * nrm.astype(np.float32)
    order = T.ravel()
    np.testing.assert_allclose(P[order], ext[tri.ravel()], rtol=1e-6, atol=1e-7)
    np.testing.assert_array_equal(pv[order], vals.astype(np.float32)[tri.ravel()])
    # closed: a second, projected copy of every triangle
    P2, _, T2 = oracle_mod.ply_clip(xyz, tri, nrm, vals, 0.25, -1.0, 1)
    assert len(P2) == 2 * len(xyz) and len(T2) == 2 * len(tri)


def test_ply_clip_nothing_above(oracle_mod):
    xyz, tri = mg.jittered_grid(9, seed=1)
    nrm = np.tile([0.0, 0.0, 1.0], (len(xyz), 1))
    P, pv, T = oracle_mod.ply_clip(xyz, tri, nrm, np.zeros(len(xyz)), 0.25, 0.5, 2)
    assert len(P) == 0 and len(T) == 0


def test_ply_clip_cut_lies_on_the_threshold(oracle_mod):
    """A linear field on a flat grid: cut vertices carry the threshold value
    and lie where the field equals it (extrusion 0 keeps the plane)."""
    xyz, tri = mg.jittered_grid(17, seed=2, jitter=0.0)
    nrm = np.tile([0.0, 0.0, 1.0], (len(xyz), 1))
    vals = xyz[:, 0].astype(np.float64)
    thr = 0.37
    P, pv, T = oracle_mod.ply_clip(xyz, tri, nrm, vals, 0.0, thr, 0)
    cut = pv == np.float32(thr)
    assert cut.sum() > 0
    np.testing.assert_allclose(P[cut, 0], thr, atol=1e-6)
    assert np.all(P[:, 0] >= thr - 1e-6)
    # the kept area is the part of the unit square with x >= thr
    a = P[T[:, 0]].astype(np.float64)
    b = P[T[:, 1]].astype(np.float64)
    c = P[T[:, 2]].astype(np.float64)
    area = 0.5 * np.abs(np.cross(b - a, c - a)[:, 2]).sum()
    assert abs(area - (1.0 - thr)) < 1e-6
