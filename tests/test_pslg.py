"""CPU tests of the PSLG triangulation (fea_triangulate_pslg), the replacement
of the reference's Triangle call (Surface::perform_triangulation,
Surface.cpp:431-486, switches "Qeqpza<area>").

Triangle is not part of the reference checkout, so nothing pins its exact
output; the tests check the invariants its switches promise: every angle at
least 20 degrees away from small input angles (q), every triangle's area at
most the bound (a), the input segments present as chains of mesh edges (p),
triangles inside the segments only and none in a hole, the boundary flags
(Triangle's point markers, Surface.cpp:472-478) equal to the vertices of
edges used once, and the reference's reversed corner order (Surface.cpp:468).
The library's triangulator is host code: these run without a GPU.
"""
import numpy as np
import pytest

from fea_gb300 import meshgen as mg


@pytest.fixture(scope="module")
def fea():
    import os
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import __graft_entry__ as ge
    ge.build_library()
    import fea_gb300
    return fea_gb300


def ring(pts, start=0):
    n = len(pts)
    return np.array([[start + i, start + (i + 1) % n] for i in range(n)])


SQUARE = np.array([[0, 0], [1, 0], [1, 1], [0, 1]], float)
HOLE = np.array([[0.4, 0.4], [0.6, 0.4], [0.6, 0.6], [0.4, 0.6]])
L_SHAPE = np.array([[0, 0], [2, 0], [2, 1], [1, 1], [1, 2], [0, 2]], float)
CIRCLE = np.stack([np.cos(np.linspace(0, 2 * np.pi, 40, endpoint=False)),
                   np.sin(np.linspace(0, 2 * np.pi, 40, endpoint=False))], 1)


def geometry(xyz, tri):
    x = xyz[:, [0, 2]].astype(np.float64)
    a, b, c = x[tri[:, 0]], x[tri[:, 1]], x[tri[:, 2]]
    signed = 0.5 * ((b[:, 0] - a[:, 0]) * (c[:, 1] - a[:, 1]) - (b[:, 1] - a[:, 1]) * (c[:, 0] - a[:, 0]))

    def angle(p, q, r):
        u, v = q - p, r - p
        cosv = (u * v).sum(1) / (np.linalg.norm(u, axis=1) * np.linalg.norm(v, axis=1))
        return np.degrees(np.arccos(np.clip(cosv, -1, 1)))

    angles = np.stack([angle(a, b, c), angle(b, c, a), angle(c, a, b)], 1)
    return x, signed, angles


def polygon_area(p):
    return 0.5 * abs(np.dot(p[:, 0], np.roll(p[:, 1], -1)) - np.dot(p[:, 1], np.roll(p[:, 0], -1)))


def segment_chain(x, edges, a, b):
    """Mesh vertices on the straight segment a-b, in order along it; every
    consecutive pair must be a mesh edge."""
    d = b - a
    t = ((x - a) @ d) / (d @ d)
    dist = np.abs((x[:, 0] - a[0]) * d[1] - (x[:, 1] - a[1]) * d[0]) / np.linalg.norm(d)
    tol_t = 4e-6 / np.linalg.norm(d)  # float32 vertices
    on = np.flatnonzero((dist < 2e-6) & (t > -tol_t) & (t < 1 + tol_t))
    on = on[np.argsort(t[on])]
    return all((min(u, v), max(u, v)) in edges for u, v in zip(on[:-1], on[1:])) and len(on) >= 2


def check_mesh(fea, pts, segs, holes, max_area, hole_polys=(), quality=True):
    xyz, tri, ob = fea.triangulate_pslg(pts, segs, holes, max_area=max_area)
    assert xyz.dtype == np.float32 and tri.dtype == np.uint32 and ob.dtype == np.uint8
    assert np.all(xyz[:, 1] == 0)  # the XZ plane (Surface.cpp:460-466)
    x, signed, angles = geometry(xyz, tri)
    # the reference reverses Triangle's counter-clockwise corners: every triangle turns clockwise in (x, z)
    assert np.all(signed < 0)
    assert np.all(-signed <= max_area * (1 + 1e-6))
    if quality:
        assert angles.min() >= 20.0 - 1e-6
    # area: the polygon minus its holes
    want = polygon_area(pts[:4] if len(hole_polys) else pts) - sum(polygon_area(h) for h in hole_polys)
    if not len(hole_polys):
        want = polygon_area(pts)
    assert abs(-signed.sum() - want) < 1e-6 * want
    # boundary flags: the vertices of edges used once (Surface.cpp:104-122)
    assert np.array_equal(ob, mg.boundary_vertices(tri, xyz.shape[0]))
    # segments present as chains of mesh edges
    e = np.concatenate([tri[:, [0, 1]], tri[:, [1, 2]], tri[:, [2, 0]]])
    edges = set(map(tuple, np.sort(e, axis=1).tolist()))
    for s0, s1 in segs:
        assert segment_chain(x, edges, pts[s0], pts[s1]), (s0, s1)
    # no triangle in a hole; Euler characteristic of a disc with holes
    cen = x[tri].mean(axis=1)
    for h in hole_polys:
        inside = (cen[:, 0] > h[:, 0].min()) & (cen[:, 0] < h[:, 0].max()) & (cen[:, 1] > h[:, 1].min()) & \
                 (cen[:, 1] < h[:, 1].max())
        assert not inside.any()
    assert xyz.shape[0] - len(edges) + tri.shape[0] == 1 - len(hole_polys)
    return xyz, tri, ob, angles


@pytest.mark.parametrize("area", [0.005, 0.0005])
def test_square(fea, area):
    xyz, tri, ob, _ = check_mesh(fea, SQUARE, ring(SQUARE), None, area)
    assert tri.shape[0] >= 1.0 / area


def test_l_shape_and_circle(fea):
    check_mesh(fea, L_SHAPE, ring(L_SHAPE), None, 0.005)
    check_mesh(fea, CIRCLE, ring(CIRCLE), None, 0.01)


def test_square_with_hole(fea):
    pts = np.vstack([SQUARE, HOLE])
    segs = np.vstack([ring(SQUARE), ring(HOLE, 4)])
    xyz, tri, ob, _ = check_mesh(fea, pts, segs, [[0.5, 0.5]], 0.005, hole_polys=(HOLE,))
    # both loops are boundary
    x = xyz[:, [0, 2]]
    on_hole = (np.abs(x - 0.5).max(axis=1) > 0.1 - 1e-7) & (np.abs(x - 0.5).max(axis=1) < 0.1 + 1e-7)
    assert np.all(ob[on_hole] == 1) and on_hole.sum() >= 8


@pytest.mark.parametrize("deg", [15, 5])
def test_small_input_angle(fea, deg):
    """Below 60 degrees Ruppert's guarantee stops at the input angle itself:
    the refinement ends (concentric-shell splits), and angles under 20 degrees
    appear only at the sharp corner."""
    a = np.radians(deg)
    pts = np.array([[0, 0], [1, 0], [np.cos(a), np.sin(a)]])
    xyz, tri, ob, angles = check_mesh(fea, pts, ring(pts), None, 0.005, quality=False)
    small = angles.min(axis=1) < 20.0 - 1e-6
    corner = int(np.flatnonzero(np.all(np.abs(xyz[:, [0, 2]]) < 1e-12, axis=1))[0])
    assert np.all(np.any(tri[small] == corner, axis=1))
    assert angles.min() >= deg - 1e-6


def test_random_star(fea):
    rng = np.random.default_rng(0)
    r = 1 + 0.3 * rng.uniform(-1, 1, 60)
    th = np.sort(rng.uniform(0, 2 * np.pi, 60))
    pts = np.stack([r * np.cos(th), r * np.sin(th)], 1)
    xyz, tri, ob, angles = check_mesh(fea, pts, ring(pts), None, 0.002, quality=False)
    assert np.percentile(angles.min(axis=1), 5) >= 20.0


def test_no_area_bound(fea):
    xyz, tri, ob = fea.triangulate_pslg(SQUARE, ring(SQUARE), None, max_area=0.0)
    assert tri.shape == (2, 3) and ob.sum() == 4


@pytest.mark.parametrize("case", ["open", "index", "duplicate", "nan", "crossing"])
def test_invalid_pslg(fea, case):
    pts, segs = SQUARE.copy(), ring(SQUARE)
    if case == "open":  # no enclosed region: Surface.cpp:40-41 throws "Invalid PSLG"
        segs = segs[:3]
    elif case == "index":
        segs = np.array([[0, 1], [1, 2], [2, 7]])
    elif case == "duplicate":
        pts = np.vstack([pts, pts[:1]])
        segs = np.vstack([segs, [[4, 1]]])
    elif case == "nan":
        pts[2, 0] = np.nan
    else:  # the diagonals cross
        segs = np.vstack([segs, [[0, 2], [1, 3]]])
    with pytest.raises(fea.FeaError) as e:
        fea.triangulate_pslg(pts, segs, None)
    assert e.value.code == -4
