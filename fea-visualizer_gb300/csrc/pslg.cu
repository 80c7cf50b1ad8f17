// pslg.cu -- quality triangulation of a planar straight line graph (PSLG):
// the input side of the reference's drawn-domain path.
//
// The reference meshes a user-drawn PSLG on the XZ plane with Shewchuk's
// Triangle (Surface::init_from_PSLG and perform_triangulation,
// src/Utils/Surface.cpp:25-49, 431-486), switches "Qeqpza<area>": a
// constrained, quality mesh (minimum angle 20 degrees) of the region enclosed
// by the segments, holes removed, every triangle's area at most
// PSLG::triangle_area (include/Utils/PSLG.hpp:29, default 0.005), zero-based
// indices; it then reverses each triangle's corner order (Surface.cpp:468)
// and takes the boundary flags from Triangle's point markers (:472-478).
//
// Triangle itself is not part of the reference checkout.  This file restates
// the published method it implements: Delaunay refinement (Ruppert 1995; the
// formulation of Shewchuk, "Delaunay Refinement Algorithms for Triangular
// Mesh Generation", 2002):
//  1. an incremental Delaunay triangulation of the points (Bowyer-Watson
//     insertion inside a bounding triangle);
//  2. segments recovered by inserting midpoints until every piece is a mesh
//     edge (a conforming triangulation); the pieces ("subsegments") are then
//     constraints that no later insertion's cavity crosses;
//  3. triangles outside the segments and inside holes removed by flood fill;
//  4. refinement: a subsegment with a vertex strictly inside its diametral
//     circle is split at its midpoint; a triangle with an angle below the bound
//     or an area above it gets its circumcentre inserted, unless that point
//     would encroach a subsegment (or lies beyond one), in which case those
//     subsegments are split instead.  An angle between two segments of the
//     input is not refined (it cannot be improved).
// Orientation and in-circle tests evaluate in double and fall back to
// double-double arithmetic (error-free sums and products, Dekker 1971) when
// the result is within the rounding bound of the fast evaluation.
//
// Output: the mesh's vertices (x, 0, z) as float32, triangles with the
// reference's reversed corner order, and a flag per vertex for vertices on a
// segment (Triangle's point markers for an unmarked PSLG).  Vertices that no
// triangle uses (input points inside holes or outside the domain) are left
// out, as Triangle's -j switch would.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <deque>
#include <new>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "fea_common.cuh"

struct fea_pslg_mesh {
    std::vector<float> xyz;
    std::vector<uint32_t> tri;
    std::vector<uint8_t> on_boundary;
};

namespace fea {
namespace {

// ---- predicates ---------------------------------------------------------------
struct DD {  // double-double: value = hi + lo
    double hi, lo;
};
inline DD two_sum(double a, double b) {
    const double s = a + b, bb = s - a;
    return {s, (a - (s - bb)) + (b - bb)};
}
inline DD two_prod(double a, double b) {
    const double p = a * b;
    return {p, std::fma(a, b, -p)};
}
inline DD dd_add(DD a, DD b) {
    DD s = two_sum(a.hi, b.hi);
    s.lo += a.lo + b.lo;
    return two_sum(s.hi, s.lo);
}
inline DD dd_neg(DD a) { return {-a.hi, -a.lo}; }
inline DD dd_mul(DD a, DD b) {
    DD p = two_prod(a.hi, b.hi);
    p.lo += a.hi * b.lo + a.lo * b.hi;
    return two_sum(p.hi, p.lo);
}
inline DD dd_sub_d(double a, double b) { return two_sum(a, -b); }

struct P2 {
    double x, y;
};

// > 0 when a, b, c turn counter-clockwise
double orient(const P2& a, const P2& b, const P2& c) {
    const double l = (a.x - c.x) * (b.y - c.y), r = (a.y - c.y) * (b.x - c.x);
    const double det = l - r;
    const double bound = 1e-15 * (std::fabs(l) + std::fabs(r));
    if (std::fabs(det) > bound) return det;
    const DD ax = dd_sub_d(a.x, c.x), ay = dd_sub_d(a.y, c.y), bx = dd_sub_d(b.x, c.x), by = dd_sub_d(b.y, c.y);
    const DD d = dd_add(dd_mul(ax, by), dd_neg(dd_mul(ay, bx)));
    return d.hi + d.lo;
}

// > 0 when d lies inside the circle through a, b, c (counter-clockwise)
double incircle(const P2& a, const P2& b, const P2& c, const P2& d) {
    const double adx = a.x - d.x, ady = a.y - d.y, bdx = b.x - d.x, bdy = b.y - d.y, cdx = c.x - d.x,
                 cdy = c.y - d.y;
    const double al = adx * adx + ady * ady, bl = bdx * bdx + bdy * bdy, cl = cdx * cdx + cdy * cdy;
    const double t1 = bdx * cdy - bdy * cdx, t2 = cdx * ady - cdy * adx, t3 = adx * bdy - ady * bdx;
    const double det = al * t1 + bl * t2 + cl * t3;
    const double perm = al * (std::fabs(bdx * cdy) + std::fabs(bdy * cdx)) +
                        bl * (std::fabs(cdx * ady) + std::fabs(cdy * adx)) +
                        cl * (std::fabs(adx * bdy) + std::fabs(ady * bdx));
    if (std::fabs(det) > 1e-14 * perm) return det;
    const DD ax = dd_sub_d(a.x, d.x), ay = dd_sub_d(a.y, d.y), bx = dd_sub_d(b.x, d.x), by = dd_sub_d(b.y, d.y),
             cx = dd_sub_d(c.x, d.x), cy = dd_sub_d(c.y, d.y);
    const DD aL = dd_add(dd_mul(ax, ax), dd_mul(ay, ay)), bL = dd_add(dd_mul(bx, bx), dd_mul(by, by)),
             cL = dd_add(dd_mul(cx, cx), dd_mul(cy, cy));
    const DD u1 = dd_add(dd_mul(bx, cy), dd_neg(dd_mul(by, cx)));
    const DD u2 = dd_add(dd_mul(cx, ay), dd_neg(dd_mul(cy, ax)));
    const DD u3 = dd_add(dd_mul(ax, by), dd_neg(dd_mul(ay, bx)));
    const DD r = dd_add(dd_add(dd_mul(aL, u1), dd_mul(bL, u2)), dd_mul(cL, u3));
    return r.hi + r.lo;
}

// ---- triangulation ------------------------------------------------------------
struct Tri {
    int v[3];  // counter-clockwise
    int n[3];  // neighbour across the edge opposite v[i]; -1 none
    bool alive;
};

inline uint64_t ekey(int a, int b) {
    const uint32_t lo = (uint32_t)std::min(a, b), hi = (uint32_t)std::max(a, b);
    return ((uint64_t)hi << 32) | lo;
}

struct Failure {
    int code;
    const char* msg;
};

class Mesher {
public:
    std::vector<P2> p;
    std::vector<Tri> t;
    std::unordered_set<uint64_t> seg;  // constrained subsegments
    std::unordered_set<int> seg_vertex;  // vertices on a segment
    int nsuper = 0;                    // first vertex of the bounding triangle
    size_t max_points = 0;
    int hint = 0;

    // edge index (0..2) of tri ti whose edge is (a, b) in either direction, -1 if none
    int edge_of(int ti, int a, int b) const {
        const Tri& T = t[ti];
        for (int i = 0; i < 3; i++) {
            const int x = T.v[(i + 1) % 3], y = T.v[(i + 2) % 3];
            if ((x == a && y == b) || (x == b && y == a)) return i;
        }
        return -1;
    }
    bool constrained(int ti, int e) const {
        const Tri& T = t[ti];
        return seg.count(ekey(T.v[(e + 1) % 3], T.v[(e + 2) % 3])) != 0;
    }

    // Walk from triangle `start` towards q.  Returns the triangle containing q
    // (on its boundary included); when `stop_at_seg`, a step that would cross
    // a subsegment (or leave the mesh) stops the walk: *blocked receives that
    // subsegment's key (0 when the mesh ends without one).
    int locate(int start, const P2& q, bool stop_at_seg, uint64_t* blocked) {
        int ti = start;
        if (ti < 0 || ti >= (int)t.size() || !t[ti].alive) ti = any_alive();
        if (blocked) *blocked = 0;
        for (size_t steps = 0; steps < 4 * t.size() + 16; steps++) {
            const Tri& T = t[ti];
            int best = -1;
            double worst = 0.0;
            for (int i = 0; i < 3; i++) {  // the edge q is most clearly beyond
                const double o = orient(p[T.v[(i + 1) % 3]], p[T.v[(i + 2) % 3]], q);
                if (o < worst) {
                    worst = o;
                    best = i;
                }
            }
            if (best < 0) return ti;
            if (stop_at_seg && constrained(ti, best)) {
                if (blocked) *blocked = ekey(T.v[(best + 1) % 3], T.v[(best + 2) % 3]);
                return -1;
            }
            const int nb = T.n[best];
            if (nb < 0) {
                if (blocked) *blocked = 0;
                return -1;
            }
            ti = nb;
        }
        // a walk that cycles (degenerate input): exhaustive search
        for (int i = 0; i < (int)t.size(); i++) {
            if (!t[i].alive) continue;
            const Tri& T = t[i];
            if (orient(p[T.v[0]], p[T.v[1]], q) >= 0 && orient(p[T.v[1]], p[T.v[2]], q) >= 0 &&
                orient(p[T.v[2]], p[T.v[0]], q) >= 0)
                return i;
        }
        return -1;
    }
    int any_alive() const {
        for (int i = (int)t.size() - 1; i >= 0; i--)
            if (t[i].alive) return i;
        return -1;
    }

    // The Bowyer-Watson cavity of point q from triangle ti: the triangles whose
    // circumcircle holds q, reached without crossing a subsegment.
    void cavity(int ti, const P2& q, std::vector<int>& out, std::vector<char>& mark, int ti2 = -1) const {
        out.clear();
        out.push_back(ti);
        mark[ti] = 1;
        if (ti2 >= 0 && !mark[ti2]) {  // a second seed: the other side of a subsegment being split
            out.push_back(ti2);
            mark[ti2] = 1;
        }
        for (size_t k = 0; k < out.size(); k++) {
            const Tri& T = t[out[k]];
            for (int e = 0; e < 3; e++) {
                const int nb = T.n[e];
                if (nb < 0 || mark[nb] || constrained(out[k], e)) continue;
                const Tri& N = t[nb];
                if (incircle(p[N.v[0]], p[N.v[1]], p[N.v[2]], q) > 0) {
                    mark[nb] = 1;
                    out.push_back(nb);
                }
            }
        }
    }

    struct BE {
        int a, b, outer;  // cavity boundary edge a -> b (counter-clockwise), the triangle beyond
    };
    std::vector<BE> be_;

    // The boundary of cavity `cav` (marked in `mark`) into be_; whether q sees
    // every boundary edge from its inner side, so that the fan of new
    // triangles is valid.  `split` is the subsegment being split at q (it may
    // lie on the boundary when the mesh ends there); 0 for none.
    bool boundary_ok(const P2& q, const std::vector<int>& cav, const std::vector<char>& mark, uint64_t split) {
        be_.clear();
        for (int ti : cav) {
            const Tri& T = t[ti];
            for (int e = 0; e < 3; e++) {
                const int nb = T.n[e];
                if (nb >= 0 && mark[nb]) continue;
                const int a = T.v[(e + 1) % 3], b = T.v[(e + 2) % 3];
                if (split && ekey(a, b) == split) continue;  // q lies on it: the edge is replaced
                if (!(orient(p[a], p[b], q) > 0)) return false;
                be_.push_back({a, b, nb});
            }
        }
        return true;
    }

    // Insert point qi into cavity `cav` whose boundary boundary_ok left in
    // be_; returns the new triangles.  A subsegment being split must have been
    // removed from `seg` by the caller.
    std::vector<int> fill(int qi, const std::vector<int>& cav, std::vector<char>& mark) {
        const std::vector<BE> be = be_;
        for (int ti : cav) {
            mark[ti] = 0;
            t[ti].alive = false;
        }
        std::vector<int> fresh;
        fresh.reserve(be.size());
        std::unordered_map<int, int> by_start;  // vertex a -> new triangle (q, a, b)
        for (const BE& e : be) {
            int id;
            if (!free_.empty()) {
                id = free_.back();
                free_.pop_back();
            } else {
                id = (int)t.size();
                t.push_back(Tri{});
            }
            Tri& N = t[id];
            N.v[0] = qi;
            N.v[1] = e.a;
            N.v[2] = e.b;
            N.n[0] = e.outer;  // across (a, b)
            N.n[1] = N.n[2] = -1;
            N.alive = true;
            if (e.outer >= 0) {
                Tri& O = t[e.outer];
                for (int k = 0; k < 3; k++)
                    if ((O.v[(k + 1) % 3] == e.b && O.v[(k + 2) % 3] == e.a)) O.n[k] = id;
            }
            by_start[e.a] = id;
            fresh.push_back(id);
        }
        for (int id : fresh) {  // fan neighbours: (q, a, b) meets (q, b, c) across (q, b)
            Tri& N = t[id];
            const auto it = by_start.find(N.v[2]);
            if (it != by_start.end()) {
                N.n[1] = it->second;              // edge opposite a: (b, q)
                t[it->second].n[2] = id;          // edge opposite c of the next: (q, b)
            }
        }
        for (int ti : cav) free_.push_back(ti);
        if (vtri.size() < p.size()) vtri.resize(2 * p.size() + 16, -1);
        for (int id : fresh)
            for (int k = 0; k < 3; k++) vtri[t[id].v[k]] = id;
        hint = fresh.empty() ? hint : fresh[0];
        return fresh;
    }

    std::vector<int> free_;
    std::vector<char> mark_;
    std::vector<int> vtri;  // an alive triangle at each vertex (-1 none)

    // An alive triangle with edge (a, b), found among the triangles around a
    // (reached through neighbours from vtri[a]); -1 when the edge is absent.
    int find_edge(int a, int b) {
        const int s0 = a < (int)vtri.size() ? vtri[a] : -1;
        if (s0 < 0 || !t[s0].alive) return -1;
        int stack[256], seen[256], ns = 0, nseen = 0;
        stack[ns++] = s0;
        seen[nseen++] = s0;
        while (ns > 0) {
            const int ti = stack[--ns];
            if (edge_of(ti, a, b) >= 0) return ti;
            const Tri& T = t[ti];
            for (int e = 0; e < 3; e++) {
                const int nb = T.n[e];
                if (nb < 0 || T.v[e] == a) continue;  // only edges through a lead around it
                bool known = false;
                for (int k = 0; k < nseen; k++) known |= seen[k] == nb;
                if (known || nseen >= 256) continue;
                seen[nseen++] = nb;
                stack[ns++] = nb;
            }
        }
        return -1;
    }

    // Insert point q; `start` is where to begin locating it; `split` the
    // subsegment q splits (0 for none).  Returns the new triangles.
    // A split (subsegment key) seeds the cavity with the one or two triangles
    // on that subsegment, `start` and `start2`, instead of locating q: the
    // midpoint lies on the subsegment up to rounding.
    std::vector<int> insert_point(const P2& q, int start, bool is_seg_vertex, uint64_t split = 0, int start2 = -1) {
        if (p.size() >= max_points) throw Failure{FEA_ERR_TOO_LARGE, "PSLG mesh exceeds the vertex limit"};
        const int ti = split ? start : locate(start, q, false, nullptr);
        if (ti < 0) throw Failure{FEA_ERR_BAD_MESH, "PSLG point outside the mesh"};
        const Tri& T = t[ti];
        for (int k = 0; k < 3; k++)
            if (p[T.v[k]].x == q.x && p[T.v[k]].y == q.y) throw Failure{FEA_ERR_BAD_MESH, "duplicate PSLG vertex"};
        if (mark_.size() < t.size() + 64) mark_.resize(2 * t.size() + 64, 0);
        std::vector<int> cav;
        cavity(ti, q, cav, mark_, split ? start2 : -1);
        if (!boundary_ok(q, cav, mark_, split)) {
            for (int ci : cav) mark_[ci] = 0;
            throw Failure{FEA_ERR_BAD_MESH, "PSLG insertion failed (degenerate or crossing segments)"};
        }
        const int qi = (int)p.size();
        p.push_back(q);
        if (is_seg_vertex) seg_vertex.insert(qi);
        return fill(qi, cav, mark_);
    }

    bool has_edge(int a, int b) { return find_edge(a, b) >= 0; }

    int first_input = 3, end_input = 3;  // mesh vertices [first_input, end_input) are the input points
    double min_seg = 0.0;                // subsegments shorter than this are not split
    std::unordered_set<uint64_t> frozen;  // subsegments that cannot be split any further

    // Split subsegment (a, b).  With exactly one endpoint an input point, the
    // split point lies at a power-of-two distance from it (the one nearest
    // half the length: concentric shells, so that subsegments meeting at a
    // small input angle stop encroaching on one another); else the midpoint.
    // Returns the new triangles (none when the subsegment is too short).
    std::vector<int> split_segment(int a, int b) {
        const double len = std::hypot(p[b].x - p[a].x, p[b].y - p[a].y);
        if (!(len > min_seg)) {
            frozen.insert(ekey(a, b));
            return {};
        }
        const bool ia = a >= first_input && a < end_input, ib = b >= first_input && b < end_input;
        double f = 0.5;
        if (ia != ib) {
            const double d = std::exp2(std::nearbyint(std::log2(0.5 * len)));
            f = ia ? d / len : 1.0 - d / len;
            if (!(f > 0.2 && f < 0.8)) f = 0.5;
        }
        seg.erase(ekey(a, b));
        const P2 m{p[a].x + f * (p[b].x - p[a].x), p[a].y + f * (p[b].y - p[a].y)};
        const int mi = (int)p.size();
        const int start = find_edge(a, b);  // the triangles on the subsegment
        if (start < 0) throw Failure{FEA_ERR_BAD_MESH, "PSLG subsegment lost"};
        const int start2 = t[start].n[edge_of(start, a, b)];
        std::vector<int> fresh = insert_point(m, start, true, ekey(a, b), start2);
        seg.insert(ekey(a, mi));
        seg.insert(ekey(mi, b));
        return fresh;
    }
};

double tri_area(const P2& a, const P2& b, const P2& c) {
    return 0.5 * ((b.x - a.x) * (c.y - a.y) - (b.y - a.y) * (c.x - a.x));
}

P2 circumcentre(const P2& a, const P2& b, const P2& c) {
    const double bx = b.x - a.x, by = b.y - a.y, cx = c.x - a.x, cy = c.y - a.y;
    const double d = 2.0 * (bx * cy - by * cx);
    const double b2 = bx * bx + by * by, c2 = cx * cx + cy * cy;
    return {a.x + (cy * b2 - by * c2) / d, a.y + (bx * c2 - cx * b2) / d};
}

bool in_diametral_circle(const P2& a, const P2& b, const P2& q) {
    return (a.x - q.x) * (b.x - q.x) + (a.y - q.y) * (b.y - q.y) < 0.0;
}

int run(const double* points, int64_t np, const int32_t* segs, int64_t ns, const double* holes, int64_t nh,
        double max_area, double min_angle_deg, fea_pslg_mesh* out) {
    if (np < 3 || ns < 3) throw Failure{FEA_ERR_BAD_MESH, "a PSLG needs at least 3 points and 3 segments"};
    if (!(min_angle_deg >= 0.0) || min_angle_deg > 30.0)
        throw Failure{FEA_ERR_INVALID_ARGUMENT, "minimum angle must lie in [0, 30] degrees"};
    if (!(max_area > 0.0) && max_area != 0.0) throw Failure{FEA_ERR_INVALID_ARGUMENT, "bad maximum area"};
    Mesher M;
    double x0 = INFINITY, y0 = INFINITY, x1 = -INFINITY, y1 = -INFINITY;
    for (int64_t i = 0; i < np; i++) {
        const double x = points[2 * i], y = points[2 * i + 1];
        if (!std::isfinite(x) || !std::isfinite(y)) throw Failure{FEA_ERR_BAD_MESH, "non-finite PSLG point"};
        x0 = std::min(x0, x);
        x1 = std::max(x1, x);
        y0 = std::min(y0, y);
        y1 = std::max(y1, y);
    }
    for (int64_t s = 0; s < 2 * ns; s++)
        if (segs[s] < 0 || segs[s] >= np) throw Failure{FEA_ERR_BAD_MESH, "PSLG segment index out of range"};
    const double size = std::max(x1 - x0, y1 - y0);
    if (!(size > 0.0)) throw Failure{FEA_ERR_BAD_MESH, "degenerate PSLG"};
    // vertex budget: the area bound sets the scale (about 2 / area triangles per unit area)
    const double domain = (x1 - x0) * (y1 - y0);
    const double est = max_area > 0.0 ? 8.0 * domain / max_area : 0.0;
    M.max_points = (size_t)std::min(4.0e6, 1.0e5 + 4.0 * est + 100.0 * (double)(np + ns));
    // bounding triangle, far outside the points
    const double cx = 0.5 * (x0 + x1), cy = 0.5 * (y0 + y1), R = 20.0 * size;
    M.p.push_back({cx - 2 * R, cy - R});
    M.p.push_back({cx + 2 * R, cy - R});
    M.p.push_back({cx, cy + 2 * R});
    M.t.push_back(Tri{{0, 1, 2}, {-1, -1, -1}, true});
    M.vtri.assign(3, 0);
    M.nsuper = 0;
    const int base = 3;  // input point i is mesh vertex base + i
    M.first_input = base;
    M.end_input = base + (int)np;
    M.min_seg = 1e-9 * size;
    for (int64_t i = 0; i < np; i++) M.insert_point({points[2 * i], points[2 * i + 1]}, M.hint, false);
    // segments: split at midpoints until every piece is a mesh edge
    std::vector<std::pair<int, int>> todo;
    for (int64_t s = 0; s < ns; s++) {
        const int a = base + segs[2 * s], b = base + segs[2 * s + 1];
        if (a == b) throw Failure{FEA_ERR_BAD_MESH, "zero-length PSLG segment"};
        todo.push_back({a, b});
        M.seg_vertex.insert(a);
        M.seg_vertex.insert(b);
    }
    while (!todo.empty()) {
        const auto [a, b] = todo.back();
        todo.pop_back();
        if (M.seg.count(ekey(a, b))) continue;
        if (M.has_edge(a, b)) {
            M.seg.insert(ekey(a, b));
            continue;
        }
        const P2 m{0.5 * (M.p[a].x + M.p[b].x), 0.5 * (M.p[a].y + M.p[b].y)};
        if (std::hypot(M.p[a].x - M.p[b].x, M.p[a].y - M.p[b].y) < 1e-12 * size)
            throw Failure{FEA_ERR_BAD_MESH, "PSLG segments cross or overlap"};
        const int mi = (int)M.p.size();
        M.insert_point(m, M.hint, true);
        todo.push_back({a, mi});
        todo.push_back({mi, b});
    }
    // remove the outside and the holes: flood fill without crossing subsegments
    std::vector<char> dead(M.t.size(), 0);
    std::deque<int> q;
    auto flood = [&](int start) {
        if (start < 0 || dead[start]) return;
        dead[start] = 1;
        q.push_back(start);
        while (!q.empty()) {
            const int ti = q.front();
            q.pop_front();
            for (int e = 0; e < 3; e++) {
                const int nb = M.t[ti].n[e];
                if (nb < 0 || dead[nb] || M.constrained(ti, e)) continue;
                dead[nb] = 1;
                q.push_back(nb);
            }
        }
    };
    for (int i = 0; i < (int)M.t.size(); i++)
        if (M.t[i].alive && (M.t[i].v[0] < base || M.t[i].v[1] < base || M.t[i].v[2] < base)) flood(i);
    for (int64_t h = 0; h < nh; h++) {
        const P2 hp{holes[2 * h], holes[2 * h + 1]};
        if (!std::isfinite(hp.x) || !std::isfinite(hp.y)) throw Failure{FEA_ERR_BAD_MESH, "non-finite hole point"};
        const int ti = M.locate(M.hint, hp, false, nullptr);
        if (ti >= 0) flood(ti);
    }
    for (int i = 0; i < (int)M.t.size(); i++) {
        if (!M.t[i].alive) continue;
        if (dead[i]) {
            M.t[i].alive = false;
            M.free_.push_back(i);
            continue;
        }
        for (int e = 0; e < 3; e++)
            if (M.t[i].n[e] >= 0 && dead[M.t[i].n[e]]) M.t[i].n[e] = -1;
    }
    if (M.any_alive() < 0)
        throw Failure{FEA_ERR_BAD_MESH, "invalid PSLG: no triangle lies inside its segments"};
    std::fill(M.vtri.begin(), M.vtri.end(), -1);
    for (int i = 0; i < (int)M.t.size(); i++)
        if (M.t[i].alive)
            for (int k = 0; k < 3; k++) M.vtri[M.t[i].v[k]] = i;
    // ---- refinement ----
    const double min_angle = min_angle_deg * 3.14159265358979323846 / 180.0;
    const double ratio = min_angle > 0.0 ? 2.0 * std::sin(min_angle) : 0.0;  // shortest edge / circumradius
    auto bad = [&](int ti) -> bool {
        const Tri& T = M.t[ti];
        const P2 &a = M.p[T.v[0]], &b = M.p[T.v[1]], &c = M.p[T.v[2]];
        const double area = tri_area(a, b, c);
        if (!(area > 0.0)) return false;  // degenerate: nothing to refine from
        if (max_area > 0.0 && area > max_area) return true;
        if (ratio <= 0.0) return false;
        const double la = std::hypot(b.x - c.x, b.y - c.y), lb = std::hypot(c.x - a.x, c.y - a.y),
                     lc = std::hypot(a.x - b.x, a.y - b.y);
        const double R = la * lb * lc / (4.0 * area);
        int k = 0;
        double lmin = la;
        if (lb < lmin) { lmin = lb; k = 1; }
        if (lc < lmin) { lmin = lc; k = 2; }
        if (lmin >= ratio * R) return false;
        // the smallest angle sits opposite the shortest edge: between two
        // segments of the input it cannot be improved
        const int v = T.v[k];
        const uint64_t e1 = ekey(v, T.v[(k + 1) % 3]), e2 = ekey(v, T.v[(k + 2) % 3]);
        return !(M.seg.count(e1) && M.seg.count(e2));
    };
    std::deque<uint64_t> enc;
    std::deque<std::pair<int, std::array<int, 3>>> badq;
    auto check_tri = [&](int ti) {
        const Tri& T = M.t[ti];
        for (int e = 0; e < 3; e++) {  // its subsegments, against the opposite corner
            const int a = T.v[(e + 1) % 3], b = T.v[(e + 2) % 3];
            if (M.seg.count(ekey(a, b)) && in_diametral_circle(M.p[a], M.p[b], M.p[T.v[e]])) enc.push_back(ekey(a, b));
        }
        if (bad(ti)) badq.push_back({ti, {T.v[0], T.v[1], T.v[2]}});
    };
    for (int i = 0; i < (int)M.t.size(); i++)
        if (M.t[i].alive) check_tri(i);
    auto after_insert = [&](const std::vector<int>& fresh) {
        for (int id : fresh) check_tri(id);
    };
    size_t guard = 0;
    const size_t guard_max = 64 * M.max_points;
    std::vector<int> cav;
    while (!enc.empty() || !badq.empty()) {
        if (++guard > guard_max) throw Failure{FEA_ERR_TOO_LARGE, "PSLG refinement did not finish"};
        if (!enc.empty()) {
            const uint64_t k = enc.front();
            enc.pop_front();
            if (!M.seg.count(k)) continue;
            const int a = (int)(k & 0xffffffffu), b = (int)(k >> 32);
            try {
                after_insert(M.split_segment(a, b));
            } catch (const Failure& f) {
                if (f.code != FEA_ERR_BAD_MESH) throw;
                M.seg.insert(k);  // a split point that coincides with a vertex: keep the subsegment
                M.frozen.insert(k);
            }
            continue;
        }
        const auto [ti, verts] = badq.front();
        badq.pop_front();
        const Tri& T = M.t[ti];
        if (!T.alive || T.v[0] != verts[0] || T.v[1] != verts[1] || T.v[2] != verts[2] || !bad(ti)) continue;
        const P2 c = circumcentre(M.p[T.v[0]], M.p[T.v[1]], M.p[T.v[2]]);
        if (!std::isfinite(c.x) || !std::isfinite(c.y)) continue;
        uint64_t blocked = 0;
        const int tc = M.locate(ti, c, true, &blocked);
        if (tc < 0) {  // beyond a subsegment: that subsegment is encroached
            if (blocked && !M.frozen.count(blocked)) {
                enc.push_back(blocked);
                badq.push_back({ti, verts});
            }
            continue;
        }
        // would the circumcentre encroach a subsegment of its cavity's boundary?
        if (M.mark_.size() < M.t.size() + 64) M.mark_.resize(2 * M.t.size() + 64, 0);
        M.cavity(tc, c, cav, M.mark_);
        bool encroaches = false, splittable = false;
        for (int cj : cav) {
            const Tri& C = M.t[cj];
            for (int e = 0; e < 3; e++) {
                const int a = C.v[(e + 1) % 3], b = C.v[(e + 2) % 3];
                if (M.seg.count(ekey(a, b)) && in_diametral_circle(M.p[a], M.p[b], c)) {
                    encroaches = true;
                    if (!M.frozen.count(ekey(a, b))) {
                        enc.push_back(ekey(a, b));
                        splittable = true;
                    }
                }
            }
        }
        if (encroaches || !M.boundary_ok(c, cav, M.mark_, 0)) {
            for (int cj : cav) M.mark_[cj] = 0;
            if (splittable) badq.push_back({ti, verts});  // refined again once the subsegments are split
            continue;
        }
        if (M.p.size() >= M.max_points) throw Failure{FEA_ERR_TOO_LARGE, "PSLG mesh exceeds the vertex limit"};
        const int qi = (int)M.p.size();
        M.p.push_back(c);
        after_insert(M.fill(qi, cav, M.mark_));
    }
    // ---- output ----
    std::vector<int> newid(M.p.size(), -1);
    int nv = 0;
    for (const Tri& T : M.t)
        if (T.alive)
            for (int k = 0; k < 3; k++)
                if (newid[T.v[k]] < 0) newid[T.v[k]] = nv++;
    out->xyz.assign(3 * (size_t)nv, 0.f);
    out->on_boundary.assign(nv, 0);
    for (int i = 0; i < (int)M.p.size(); i++) {
        const int j = newid[i];
        if (j < 0) continue;
        out->xyz[3 * j] = (float)M.p[i].x;  // (x, 0, z) on the XZ plane (Surface.cpp:460-466)
        out->xyz[3 * j + 1] = 0.f;
        out->xyz[3 * j + 2] = (float)M.p[i].y;
        out->on_boundary[j] = M.seg_vertex.count(i) ? 1 : 0;
    }
    out->tri.clear();
    for (const Tri& T : M.t)
        if (T.alive)  // counter-clockwise (a, b, c) written as (c, b, a), Surface.cpp:468
            for (int k = 2; k >= 0; k--) out->tri.push_back((uint32_t)newid[T.v[k]]);
    return FEA_OK;
}

}  // namespace
}  // namespace fea

extern "C" {

int fea_triangulate_pslg(const double* points, int64_t num_points, const int32_t* segments, int64_t num_segments,
                         const double* holes, int64_t num_holes, double max_area, double min_angle_deg,
                         fea_pslg_mesh** out) {
    using namespace fea;
    if (!out) return fail(FEA_ERR_INVALID_ARGUMENT, "null output");
    *out = nullptr;
    if (!points || !segments || (num_holes > 0 && !holes) || num_points < 0 || num_segments < 0 || num_holes < 0)
        return fail(FEA_ERR_INVALID_ARGUMENT, "bad PSLG arrays");
    if (num_points >= (int64_t)1 << 28 || num_segments >= (int64_t)1 << 28)
        return fail(FEA_ERR_TOO_LARGE, "PSLG too large");
    fea_pslg_mesh* m = nullptr;
    try {
        m = new fea_pslg_mesh();
        run(points, num_points, segments, num_segments, holes, num_holes, max_area, min_angle_deg, m);
        *out = m;
        return FEA_OK;
    } catch (const Failure& f) {
        delete m;
        return fail(f.code, f.msg);
    } catch (const std::bad_alloc&) {
        delete m;
        return fail(FEA_ERR_OUT_OF_MEMORY, "host allocation failed");
    }
}

int fea_pslg_mesh_sizes(const fea_pslg_mesh* m, int64_t* num_vertices, int64_t* num_triangles) {
    if (!m) return fea::fail(FEA_ERR_INVALID_ARGUMENT, "null mesh");
    if (num_vertices) *num_vertices = (int64_t)m->on_boundary.size();
    if (num_triangles) *num_triangles = (int64_t)(m->tri.size() / 3);
    return FEA_OK;
}

int fea_pslg_mesh_copy(const fea_pslg_mesh* m, float* vertices, uint32_t* triangles, uint8_t* on_boundary) {
    if (!m) return fea::fail(FEA_ERR_INVALID_ARGUMENT, "null mesh");
    if (vertices) std::copy(m->xyz.begin(), m->xyz.end(), vertices);
    if (triangles) std::copy(m->tri.begin(), m->tri.end(), triangles);
    if (on_boundary) std::copy(m->on_boundary.begin(), m->on_boundary.end(), on_boundary);
    return FEA_OK;
}

int fea_pslg_mesh_destroy(fea_pslg_mesh* m) {
    delete m;
    return FEA_OK;
}

}  // extern "C"
