// cg_device.cuh -- device building blocks shared by the single-mesh and the
// batched step loops: exact accumulators for FP32 inner products, cached and
// L2-only vector loads, block totals, loop signalling, and graph-node helpers.
#pragma once

#include <tuple>

#include "fea_internal.cuh"

namespace fea {
namespace {

// ---- accumulators -------------------------------------------------------------
template <typename R>
struct Acc;

template <>
struct Acc<double> {
    double s = 0.0;
    __device__ __forceinline__ void add(double x) { s += x; }
    __device__ __forceinline__ void add_prod(double a, double b) { s = fmar(a, b, s); }
    __device__ __forceinline__ void sub(const Acc& o) { s -= o.s; }
    __device__ __forceinline__ double value() const { return s; }
    __device__ __forceinline__ double rounded() const { return s; }
    __device__ __forceinline__ void merge(const Acc& o) { s += o.s; }
    __device__ __forceinline__ void shfl_add(int off) { s += __shfl_xor_sync(0xffffffffu, s, off); }
    // storage of a block's total in an 8-byte partial slot
    using Packed = double;
    __device__ __forceinline__ Packed pack() const { return s; }
    __device__ __forceinline__ static Acc unpack(Packed x) {
        Acc a;
        a.s = x;
        return a;
    }
};

// float-float: value = hi + lo with |lo| <= ulp(hi)/2 (Knuth two-sum plus the
// exact product error from fma); intrinsics keep the compiler from fusing.
template <>
struct Acc<float> {
    float hi = 0.f, lo = 0.f;
    __device__ __forceinline__ void add(float x) {
        const float s = __fadd_rn(hi, x);
        const float bb = __fsub_rn(s, hi);
        const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(x, bb));
        const float l = __fadd_rn(lo, err);
        hi = __fadd_rn(s, l);
        lo = __fsub_rn(l, __fsub_rn(hi, s));
    }
    __device__ __forceinline__ void add_prod(float a, float b) {
        const float p = __fmul_rn(a, b);
        const float e = __fmaf_rn(a, b, -p);
        add(p);
        lo = __fadd_rn(lo, e);
    }
    __device__ __forceinline__ void sub(const Acc& o) {
        add(-o.hi);
        lo = __fsub_rn(lo, o.lo);
    }
    __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
    // hi + lo rounded once to float.  The pair's exact sum fits a double, so
    // this equals (float)value() without touching the FP64 pipe.
    __device__ __forceinline__ float rounded() const { return __fadd_rn(hi, lo); }
    __device__ __forceinline__ void merge(const Acc& o) {
        add(o.hi);
        lo = __fadd_rn(lo, o.lo);
    }
    __device__ __forceinline__ void shfl_add(int off) {
        Acc o;
        o.hi = __shfl_xor_sync(0xffffffffu, hi, off);
        o.lo = __shfl_xor_sync(0xffffffffu, lo, off);
        merge(o);
    }
    using Packed = float2;
    __device__ __forceinline__ Packed pack() const { return make_float2(hi, lo); }
    __device__ __forceinline__ static Acc unpack(Packed x) {
        Acc a;
        a.hi = x.x;
        a.lo = x.y;
        return a;
    }
};

// ---- float-float scalars ------------------------------------------------------
// The CG scalars of FP32 solvers (alpha, beta, gamma, the convergence test)
// are computed in float-float arithmetic (about 48 significant bits), so that
// no FP64 instruction runs inside a CG iteration.  Knuth / Dekker error-free
// transformations, rounded intrinsics throughout.
using FF = Acc<float>;

__device__ __forceinline__ FF ff_quick(float a, float b) {  // |a| >= |b|
    FF r;
    r.hi = __fadd_rn(a, b);
    r.lo = __fsub_rn(b, __fsub_rn(r.hi, a));
    return r;
}
__device__ __forceinline__ FF ff_of(double x) {
    FF r;
    r.hi = __double2float_rn(x);
    r.lo = __double2float_rn(x - (double)r.hi);
    return r;
}
__device__ __forceinline__ FF ff_load(const volatile float (&p)[2]) {
    FF r;
    r.hi = p[0];
    r.lo = p[1];
    return r;
}
__device__ __forceinline__ void ff_store(volatile float (&p)[2], const FF& x) {
    p[0] = x.hi;
    p[1] = x.lo;
}
__device__ __forceinline__ FF ff_two(float a, float b) {  // any magnitudes
    FF r;
    r.hi = __fadd_rn(a, b);
    const float bb = __fsub_rn(r.hi, a);
    r.lo = __fadd_rn(__fsub_rn(a, __fsub_rn(r.hi, bb)), __fsub_rn(b, bb));
    return r;
}
// a - b with both pairs' errors carried (accurate under cancellation).
__device__ __forceinline__ FF ff_sub(const FF& a, const FF& b) {
    FF s = ff_two(a.hi, -b.hi);
    const FF t = ff_two(a.lo, -b.lo);
    s = ff_quick(s.hi, __fadd_rn(s.lo, t.hi));
    return ff_quick(s.hi, __fadd_rn(s.lo, t.lo));
}
__device__ __forceinline__ FF ff_mul(const FF& a, const FF& b) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    return ff_quick(p, e);
}
// Long division: q1 = a/b in float, then the quotient of the exact remainder.
__device__ __forceinline__ FF ff_div(const FF& a, const FF& b) {
    const float q1 = __fdiv_rn(a.hi, b.hi);
    FF q;
    q.hi = q1;
    q.lo = 0.f;
    const FF r = ff_sub(a, ff_mul(q, b));
    return ff_quick(q1, __fdiv_rn(r.hi, b.hi));
}
__device__ __forceinline__ FF ff_norm(const FF& a) { return ff_two(a.hi, a.lo); }
// a < b for normalised pairs
__device__ __forceinline__ bool ff_less(const FF& a, const FF& b) {
    return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo);
}

// Programmatic dependent launch.  wait: block until the kernel this one
// depends on programmatically has completed and its memory is visible (a
// no-op without such a dependency).  launch_dependents: this block no longer
// holds back the launch of kernels that depend on this one.
__device__ __forceinline__ void grid_dependency_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void grid_launch_dependents() {
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// Loop condition: stored for host-driven loops, and set on the graph's
// conditional node when the kernel runs inside the step graph.  Called by one
// thread only (concurrent cudaGraphSetConditional calls are undefined).
template <typename A>
__device__ __forceinline__ void signal_loop(const A& a, bool cont) {
    *a.cont = cont ? 1 : 0;
    if (a.use_graph) cudaGraphSetConditional(a.cond, cont ? 1u : 0u);
}

__device__ __forceinline__ void raise_flags(RunState* run, unsigned int f) {
    const unsigned int w = __reduce_or_sync(0xffffffffu, f);
    if (w && (threadIdx.x & 31) == 0) {
        atomicOr(&run->flags, w);
        __threadfence();
    }
}

template <typename R>
__device__ __forceinline__ unsigned int check_value(R x) {
    unsigned int f = 0;
    if (x > (R)1e4f) f |= FEA_STATUS_BLOWUP;  // CPUSolver.cpp:43
    if (!isfinite(x)) f |= FEA_STATUS_NONFINITE;
    return f;
}

template <typename R>
__device__ __forceinline__ R ldg(const R* p) {
    return __ldg(p);
}
// Load of a 4-, 8- or 16-byte value: through the read-only cache, or from L2
// only (l2only) for data that other blocks of the running kernel wrote.
template <typename T>
__device__ __forceinline__ T ldv(const T* p, bool l2only) {
    T o;
    if constexpr (sizeof(T) == 4) {
        const float* q = reinterpret_cast<const float*>(p);
        const float t = l2only ? __ldcg(q) : __ldg(q);
        memcpy(&o, &t, 4);
    } else if constexpr (sizeof(T) == 8) {
        const float2* q = reinterpret_cast<const float2*>(p);
        const float2 t = l2only ? __ldcg(q) : __ldg(q);
        memcpy(&o, &t, 8);
    } else {
        static_assert(sizeof(T) == 16, "4, 8 or 16 bytes");
        const float4* q = reinterpret_cast<const float4*>(p);
        const float4 t = l2only ? __ldcg(q) : __ldg(q);
        memcpy(&o, &t, 16);
    }
    return o;
}

template <typename R, int NF>
__device__ __forceinline__ FV<R, NF> ldfv(const FV<R, NF>* p) {
    return ldv(p, false);
}

// Block totals of NV accumulators: warp sums by shuffles, then a shuffle tree
// over the warps' sums in warp 0 (a fixed order).  The accumulator type carries through
// (float-float pairs for FP32 solvers: no FP64 instruction), and the result is
// valid in thread 0 (empty elsewhere).  sm holds 32 * NV packed values.
template <int NV, typename R>
__device__ __forceinline__ void block_totals(Acc<R> (&acc)[NV], typename Acc<R>::Packed* sm, Acc<R> (&blk)[NV]) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; k++) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc[k].shfl_add(o);
        if (lane == 0) sm[wid * NV + k] = acc[k].pack();
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < NV; k++) blk[k] = Acc<R>();
    if (wid == 0) {  // lane w holds warp w's sums; a shuffle tree over the warps
        const int nw = (blockDim.x + 31) >> 5;
        if (lane < nw)
#pragma unroll
            for (int k = 0; k < NV; k++) blk[k] = Acc<R>::unpack(sm[lane * NV + k]);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            if (o < nw)
#pragma unroll
                for (int k = 0; k < NV; k++) blk[k].shfl_add(o);
        if (lane != 0)
#pragma unroll
            for (int k = 0; k < NV; k++) blk[k] = Acc<R>();
    }
    __syncthreads();
}

// y[k] += partials p[k * vstride + b * pstride] for b in [b0, b1), thread t
// taking b0 + t, b0 + t + blockDim.x, ...  The loads of kMergeBatch partials
// per value are all issued before the first merge, so the block pays one L2
// round trip per batch rather than one per partial.
constexpr int kMergeBatch = 2;
template <int NV, typename R>
__device__ __forceinline__ void merge_partials(Acc<R> (&y)[NV], const typename Acc<R>::Packed* p, int64_t vstride,
                                               int64_t pstride, int64_t b0, int64_t b1) {
    using P = typename Acc<R>::Packed;
    const int64_t step = (int64_t)kMergeBatch * blockDim.x;
    for (int64_t base = b0 + threadIdx.x; base < b1; base += step) {
        P v[kMergeBatch][NV];
#pragma unroll
        for (int u = 0; u < kMergeBatch; u++) {
            const int64_t b = base + (int64_t)u * blockDim.x;
#pragma unroll
            for (int k = 0; k < NV; k++)
                if (b < b1) v[u][k] = __ldcg(&p[k * vstride + b * pstride]);
        }
#pragma unroll
        for (int u = 0; u < kMergeBatch; u++)
            if (base + (int64_t)u * blockDim.x < b1)
#pragma unroll
                for (int k = 0; k < NV; k++) y[k].merge(Acc<R>::unpack(v[u][k]));
    }
}

// Last-block-done reduction of block totals held in thread 0: every block
// stores its NV totals, packed, to part[k * stride + blockIdx.x] (8-byte
// slots); the block that finishes last merges all partials in a fixed order
// (the result does not depend on which block finished last) and returns true
// in all its threads with the totals in out[] (valid in thread 0).  The
// ticket counter is reset for the next launch.
template <int NV, typename R>
__device__ bool grid_commit(const Acc<R> (&blk)[NV], double* part, int stride, unsigned int* ticket,
                            typename Acc<R>::Packed* sm, Acc<R> (&out)[NV]) {
    using P = typename Acc<R>::Packed;
    static_assert(sizeof(P) == sizeof(double), "partials use 8-byte slots");
    P* pp = reinterpret_cast<P*>(part);
    __shared__ bool is_last;
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; k++) pp[k * stride + blockIdx.x] = blk[k].pack();
        __threadfence();
        const unsigned int t = atomicAdd(ticket, 1u);
        is_last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (!is_last) return false;
    __threadfence();
    Acc<R> y[NV];
    merge_partials<NV, R>(y, pp, stride, 1, 0, (int64_t)gridDim.x);
    block_totals<NV, R>(y, sm, out);
    if (threadIdx.x == 0) *ticket = 0u;
    return true;
}

// ---- CG building blocks ----------------------------------------------------------

// Control values of one CG phase, read once per phase by every thread.
template <typename R, int NF>
struct PhaseCtl {
    int par;  // iteration parity: which of the alternating buffers holds the old values
    int act[NF];
    bool fresh[NF];  // first iteration of a loop: p = u, s = w
    bool need_old;
    bool any;
    R beta[NF], alpha[NF];
    template <typename S>
    __device__ __forceinline__ void set(int iter, const volatile S* st) {
        par = iter & 1;
        need_old = false;
        any = false;
#pragma unroll
        for (int f = 0; f < NF; f++) {
            act[f] = st->active[f];
            fresh[f] = st->fresh[f] != 0;
            if constexpr (sizeof(R) == 4) {  // coefficients stored rounded: no conversion here
                beta[f] = fresh[f] ? (R)0 : st->fbeta[f];
                alpha[f] = act[f] ? st->falpha[f] : (R)0;
            } else {
                beta[f] = fresh[f] ? (R)0 : (R)st->beta[f];
                alpha[f] = act[f] ? (R)st->alpha[f] : (R)0;
            }
            need_old |= !fresh[f];
            any |= act[f] != 0;
        }
    }
    __device__ __forceinline__ void load(const CgState* cg) {
        const volatile CgState* v = cg;
        set(v->iter, v);
    }
};

// Warp-cooperative CSR product over the warp's 32 consecutive rows row0 ..
// row0+31 (rows >= N are empty): lane l returns sum_e A_e * g(col_e) of row
// row0 + l, per field.  The rows' stored entries form one contiguous range,
// streamed in windows of 32*WCH entries: every lane issues WCH coalesced
// value/column loads, then WCH independent gathers g(col), so each round trip
// to memory carries a whole window rather than one row.  Products go to the
// warp's shared-memory window smw[32*WCH] and each lane sums its own row in
// column order.
template <typename R, int NF, int WCH, typename G>
__device__ __forceinline__ FV<R, NF> warp_rows(const int32_t* __restrict__ rp, const int32_t* __restrict__ col,
                                               const FV<R, NF>* __restrict__ A, int64_t row0, int64_t N,
                                               FV<R, NF>* smw, G g) {
    constexpr int WIN = 32 * WCH;
    const int lane = threadIdx.x & 31;
    const int64_t row = row0 + lane;
    const int32_t rs = ldg(rp + (row < N ? row : N));
    int32_t re = __shfl_down_sync(0xffffffffu, rs, 1);
    if (lane == 31) re = ldg(rp + (row0 + 32 < N ? row0 + 32 : N));
    const int32_t e0 = __shfl_sync(0xffffffffu, rs, 0);
    const int32_t e1 = __shfl_sync(0xffffffffu, re, 31);
    FV<R, NF> acc;
#pragma unroll
    for (int f = 0; f < NF; f++) acc.v[f] = 0;
    for (int32_t wb = e0; wb < e1; wb += WIN) {
        FV<R, NF> av[WCH];
        int32_t cc[WCH];
#pragma unroll
        for (int k = 0; k < WCH; k++) {
            const int32_t idx = wb + k * 32 + lane;
            cc[k] = -1;
            if (idx < e1) {
                av[k] = ldv(A + idx, false);
                cc[k] = ldg(col + idx);
            }
        }
#pragma unroll
        for (int k = 0; k < WCH; k++) {
            FV<R, NF> prod;
#pragma unroll
            for (int f = 0; f < NF; f++) prod.v[f] = 0;
            if (cc[k] >= 0) {
                const FV<R, NF> gv = g(cc[k]);
#pragma unroll
                for (int f = 0; f < NF; f++) prod.v[f] = av[k].v[f] * gv.v[f];
            }
            smw[k * 32 + lane] = prod;
        }
        __syncwarp();
        const int32_t lo = (rs > wb ? rs : wb) - wb;
        const int32_t hi = (re < wb + WIN ? re : wb + WIN) - wb;
        for (int32_t k = lo; k < hi; k++) {
            const FV<R, NF> t = smw[k];
#pragma unroll
            for (int f = 0; f < NF; f++) acc.v[f] += t.v[f];
        }
        __syncwarp();
    }
    return acc;
}

// Set-up product of a Chronopoulos-Gear solve on one warp's rows: w = A z and
// z.w into dot[] (delta0).
template <typename R, int NF, int WCH>
__device__ __forceinline__ void init_rows(const int32_t* __restrict__ rp, const int32_t* __restrict__ col,
                                          const FV<R, NF>* __restrict__ A, const FV<R, NF>* __restrict__ z,
                                          FV<R, NF>* __restrict__ w, int64_t row0, int64_t N, FV<R, NF>* smw,
                                          Acc<R> (&dot)[NF]) {
    const FV<R, NF> wr =
        warp_rows<R, NF, WCH>(rp, col, A, row0, N, smw, [&](int32_t c) { return ldv(z + c, false); });
    const int64_t row = row0 + (threadIdx.x & 31);
    if (row < N) {
        const FV<R, NF> zr = ldv(z + row, false);
#pragma unroll
        for (int f = 0; f < NF; f++) dot[f].add_prod(zr.v[f], wr.v[f]);
        w[row] = wr;
    }
}

// The vectors of one Chronopoulos-Gear iteration: r, w and s alternate
// between two buffers with the iteration parity (old: 0 suffix, new: 1).
template <typename R, int NF>
struct CgVecs {
    const int32_t* rp;
    const int32_t* col;
    const FV<R, NF>* A;
    const FV<R, NF>* dinv;
    FV<R, NF>* x;
    FV<R, NF>* p;
    const FV<R, NF>* r0;
    const FV<R, NF>* w0;
    const FV<R, NF>* s0;
    FV<R, NF>* r1;
    FV<R, NF>* w1;
    FV<R, NF>* s1;
};

// New s, r and u = D^-1 r of one unknown from its old r, w, s (and D^-1).
template <typename R, int NF>
__device__ __forceinline__ void cg_advance(const PhaseCtl<R, NF>& c, const FV<R, NF>& ro, const FV<R, NF>& wo,
                                           const FV<R, NF>& so, const FV<R, NF>& d, FV<R, NF>& sn,
                                           FV<R, NF>& rn, FV<R, NF>& un) {
#pragma unroll
    for (int f = 0; f < NF; f++) {
        sn.v[f] = c.fresh[f] ? wo.v[f] : fmar(c.beta[f], so.v[f], wo.v[f]);
        rn.v[f] = c.act[f] ? fmar(-c.alpha[f], sn.v[f], ro.v[f]) : ro.v[f];
        un.v[f] = d.v[f] * rn.v[f];
    }
}

// One Chronopoulos-Gear iteration on a tile of blockDim.x consecutive rows
// starting at tile0 (one row per thread, 32 rows per warp), Jacobi-
// preconditioned CG rearranged (Chronopoulos & Gear 1989) so that an
// iteration needs one global reduction: with u = D^-1 r, w = A u, s = A p,
//   p = u + beta p,  s = w + beta s,  x += alpha p,  r -= alpha s,
//   u' = D^-1 r,  w' = A u',  gamma' = r.u',  delta' = w'.u'.
// Each thread first applies the vector updates to its own row and leaves u'
// in the tile's shared-memory slice ut[]; after a block barrier the SpMV
// takes u' of in-tile columns from there and recomputes it from the old r, w
// and s in global memory only for columns outside the tile (few, in the
// solver's Morton order).  dots[] receives gamma', delta' and |r'|^2 per
// field.  Every thread of the block must call it (it holds barriers).
template <typename R, int NF, int WCH>
__device__ __forceinline__ void cgcg_tile(const CgVecs<R, NF>& v, const PhaseCtl<R, NF>& c, int64_t tile0,
                                          int64_t N, FV<R, NF>* smw, FV<R, NF>* ut, Acc<R> (&dots)[3 * NF]) {
    const int t = threadIdx.x;
    const int64_t row = tile0 + t;
    FV<R, NF> un;
#pragma unroll
    for (int f = 0; f < NF; f++) un.v[f] = 0;
    if (row < N) {
        const FV<R, NF> ro = ldv(v.r0 + row, false), wo = ldv(v.w0 + row, false), d = ldv(v.dinv + row, false);
        FV<R, NF> so = wo;
        if (c.need_old) so = ldv(v.s0 + row, false);
        FV<R, NF> x = v.x[row], p = v.p[row];
        FV<R, NF> sn, rn;
        cg_advance(c, ro, wo, so, d, sn, rn, un);
#pragma unroll
        for (int f = 0; f < NF; f++) {
            if (c.act[f]) {
                const R ui = d.v[f] * ro.v[f];
                p.v[f] = c.fresh[f] ? ui : fmar(c.beta[f], p.v[f], ui);
                x.v[f] = fmar(c.alpha[f], p.v[f], x.v[f]);
            }
            dots[f].add_prod(rn.v[f], un.v[f]);
            dots[2 * NF + f].add_prod(rn.v[f], rn.v[f]);
        }
        v.x[row] = x;
        v.p[row] = p;
        v.r1[row] = rn;
        v.s1[row] = sn;
    }
    ut[t] = un;
    __syncthreads();
    const uint32_t span = blockDim.x;
    const FV<R, NF> wn = warp_rows<R, NF, WCH>(v.rp, v.col, v.A, tile0 + (t & ~31), N, smw, [&](int32_t col) {
        const uint32_t o = (uint32_t)(col - tile0);
        if (o < span) return ut[o];
        const FV<R, NF> ro = ldv(v.r0 + col, false), wo = ldv(v.w0 + col, false);
        const FV<R, NF> d = ldv(v.dinv + col, false);
        FV<R, NF> so = wo;
        if (c.need_old) so = ldv(v.s0 + col, false);
        FV<R, NF> sn, rn, u2;
        cg_advance(c, ro, wo, so, d, sn, rn, u2);
        return u2;
    });
    if (row < N) {
        v.w1[row] = wn;
#pragma unroll
        for (int f = 0; f < NF; f++) dots[NF + f].add_prod(wn.v[f], un.v[f]);
    }
    __syncthreads();  // the next tile reuses ut[]
}

// ---- tile-ELL bodies (layout: tile_ell.cu) -------------------------------------

template <typename R, int NF>
struct EllView {
    const FV<R, NF>* As;
    const uint16_t* lcol;
    const int32_t* slice_off;
    const int32_t* halo_off;
    const int32_t* halo_col;
};

// Where a warp's slice and its tile's halo sit in the layout: loaded one
// tile ahead, so no load of a tile waits on another.
struct EllTileRef {
    int32_t sb, sw;  // the warp's slice: first entry, width (entries per row)
    int32_t h0, h1;  // the tile's halo range
};

template <typename R, int NF>
__device__ __forceinline__ EllTileRef ell_ref(const EllView<R, NF>& e, int64_t tile, int64_t ntiles) {
    EllTileRef r{0, 0, 0, 0};
    if (tile < ntiles) {
        const int64_t s = tile * (kTileRows / 32) + (threadIdx.x >> 5);
        r.sb = ldg(e.slice_off + s);
        r.sw = (ldg(e.slice_off + s + 1) - r.sb) >> 5;
        r.h0 = ldg(e.halo_off + tile);
        r.h1 = ldg(e.halo_off + tile + 1);
    }
    return r;
}

// The first KPRE entries of the thread's row in its slice, loaded into
// registers before the tile's operand is staged (their loads do not depend on
// it); ell_finish multiplies them and any remaining entries with ut[].
template <typename R, int NF, int KPRE>
struct EllRow {
    FV<R, NF> a[KPRE];
    uint32_t l[KPRE];
    __device__ __forceinline__ void load(const EllView<R, NF>& e, const EllTileRef& r) {
        const int lane = threadIdx.x & 31;
#pragma unroll
        for (int k = 0; k < KPRE; k++) {
            if (k < r.sw) {
                a[k] = ldv(e.As + r.sb + 32 * k + lane, false);
                l[k] = __ldg(e.lcol + r.sb + 32 * k + lane);
            }
        }
    }
    __device__ __forceinline__ FV<R, NF> finish(const EllView<R, NF>& e, const EllTileRef& r,
                                                const FV<R, NF>* ut) const {
        const int lane = threadIdx.x & 31;
        FV<R, NF> acc;
#pragma unroll
        for (int f = 0; f < NF; f++) acc.v[f] = 0;
#pragma unroll
        for (int k = 0; k < KPRE; k++) {
            if (k < r.sw) {
                const FV<R, NF> g = ut[l[k]];
#pragma unroll
                for (int f = 0; f < NF; f++) acc.v[f] = fmar(a[k].v[f], g.v[f], acc.v[f]);
            }
        }
        for (int k = KPRE; k < r.sw; k++) {
            const FV<R, NF> av = ldv(e.As + r.sb + 32 * k + lane, false);
            const FV<R, NF> g = ut[__ldg(e.lcol + r.sb + 32 * k + lane)];
#pragma unroll
            for (int f = 0; f < NF; f++) acc.v[f] = fmar(av.v[f], g.v[f], acc.v[f]);
        }
        return acc;
    }
};

// u' of one unknown from the old r, w, s and D^-1 in global memory.
template <typename R, int NF>
__device__ __forceinline__ FV<R, NF> cg_u_at(const CgVecs<R, NF>& v, const PhaseCtl<R, NF>& c, int64_t i) {
    const FV<R, NF> ro = ldv(v.r0 + i, false), wo = ldv(v.w0 + i, false), d = ldv(v.dinv + i, false);
    FV<R, NF> so = wo;
    if (c.need_old) so = ldv(v.s0 + i, false);
    FV<R, NF> sn, rn, un;
    cg_advance(c, ro, wo, so, d, sn, rn, un);
    return un;
}

// One Chronopoulos-Gear iteration on tile `tile` in the tile-ELL layout (the
// recurrences as in cgcg_tile).  Each thread updates its row and stages u' in
// ut[] (this tile's buffer: kTileRows + the layout's largest halo); the
// tile's halo columns get u' recomputed from the old r, w, s; after one block
// barrier every gathered operand comes from shared memory.  All loads of the
// tile are issued before the barrier.  The caller alternates two ut buffers
// between consecutive tiles, which makes the one barrier enough.  Every
// thread of the block calls it.
template <typename R, int NF, int KPRE>
__device__ __forceinline__ void cgcg_tile_ell(const CgVecs<R, NF>& v, const EllView<R, NF>& e,
                                              const PhaseCtl<R, NF>& c, int64_t tile, const EllTileRef& ref,
                                              int64_t N, FV<R, NF>* ut, Acc<R> (&dots)[3 * NF]) {
    const int t = threadIdx.x;
    const int64_t row = tile * kTileRows + t;
    EllRow<R, NF, KPRE> er;
    er.load(e, ref);
    FV<R, NF> un;
#pragma unroll
    for (int f = 0; f < NF; f++) un.v[f] = 0;
    if (row < N) {
        const FV<R, NF> ro = ldv(v.r0 + row, false), wo = ldv(v.w0 + row, false), d = ldv(v.dinv + row, false);
        FV<R, NF> so = wo;
        if (c.need_old) so = ldv(v.s0 + row, false);
        FV<R, NF> x = v.x[row], p = v.p[row];
        FV<R, NF> sn, rn;
        cg_advance(c, ro, wo, so, d, sn, rn, un);
#pragma unroll
        for (int f = 0; f < NF; f++) {
            if (c.act[f]) {
                const R ui = d.v[f] * ro.v[f];
                p.v[f] = c.fresh[f] ? ui : fmar(c.beta[f], p.v[f], ui);
                x.v[f] = fmar(c.alpha[f], p.v[f], x.v[f]);
            }
            dots[f].add_prod(rn.v[f], un.v[f]);
            dots[2 * NF + f].add_prod(rn.v[f], rn.v[f]);
        }
        v.x[row] = x;
        v.p[row] = p;
        v.r1[row] = rn;
        v.s1[row] = sn;
    }
    ut[t] = un;
    for (int32_t h = ref.h0 + t; h < ref.h1; h += blockDim.x)
        ut[kTileRows + (h - ref.h0)] = cg_u_at(v, c, ldg(e.halo_col + h));
    __syncthreads();
    const FV<R, NF> wn = er.finish(e, ref, ut);
    if (row < N) {
        v.w1[row] = wn;
#pragma unroll
        for (int f = 0; f < NF; f++) dots[NF + f].add_prod(wn.v[f], un.v[f]);
    }
}

// Set-up product w = A z on tile `tile` in the tile-ELL layout, z.w into dot[]
// (same staging and buffer alternation as cgcg_tile_ell).
template <typename R, int NF, int KPRE>
__device__ __forceinline__ void init_tile_ell(const EllView<R, NF>& e, const FV<R, NF>* __restrict__ z,
                                              FV<R, NF>* __restrict__ w, int64_t tile, const EllTileRef& ref,
                                              int64_t N, FV<R, NF>* ut, Acc<R> (&dot)[NF]) {
    const int t = threadIdx.x;
    const int64_t row = tile * kTileRows + t;
    EllRow<R, NF, KPRE> er;
    er.load(e, ref);
    FV<R, NF> zr;
#pragma unroll
    for (int f = 0; f < NF; f++) zr.v[f] = 0;
    if (row < N) zr = ldv(z + row, false);
    ut[t] = zr;
    for (int32_t h = ref.h0 + t; h < ref.h1; h += blockDim.x)
        ut[kTileRows + (h - ref.h0)] = ldv(z + ldg(e.halo_col + h), false);
    __syncthreads();
    const FV<R, NF> wr = er.finish(e, ref, ut);
    if (row < N) {
        w[row] = wr;
#pragma unroll
        for (int f = 0; f < NF; f++) dot[f].add_prod(zr.v[f], wr.v[f]);
    }
}

// gamma = r.z of the running solve (and its float-float copy for FP32).
template <typename R, typename S>
__device__ __forceinline__ void set_gamma(volatile S* s, int f, const Acc<R>& g) {
    s->rz[f] = g.value();
    if constexpr (sizeof(R) == 4) ff_store(s->ffrz[f], ff_norm(g));
}

// CG scalars of a solve's start, per field: |b|^2, the threshold tol^2 |b|^2
// (at least the smallest normal number of R), |r|^2 and gamma = r.z.  The
// FP32 solver keeps float-float copies of gamma and the threshold for its
// iterations.  Returns whether the field iterates.
template <typename R, typename S>
__device__ __forceinline__ int start_solve(volatile S* s, int f, int stop, double tol, const Acc<R>& bb_a,
                                           const Acc<R>& rr_a, const Acc<R>& rz_a) {
    const double tiny = sizeof(R) == 4 ? 1.1754943508222875e-38 : 2.2250738585072014e-308;
    const double bb = bb_a.value(), rr = rr_a.value();
    double thr = tol * tol * bb;
    thr = thr < tiny ? tiny : thr;
    s->bb[f] = bb;
    s->thr[f] = thr;
    s->rr[f] = rr;
    set_gamma(s, f, rz_a);
    if constexpr (sizeof(R) == 4) ff_store(s->ffthr[f], ff_of(thr));
    s->iters[f] = 0;
    s->fresh[f] = 1;  // the first direction is p = z
    s->active[f] = (!stop && bb > 0.0 && rr >= thr) ? 1 : 0;
    return s->active[f];
}

// After the SpMV phase: alpha = r.z / p.q, or breakdown.
// (S: CgState or a batched instance's state; flags receives FEA_STATUS_*.)
template <typename R, int NF, typename S>
__device__ void finish_spmv(volatile S* cg, unsigned int* flags, const int (&act)[NF], const Acc<R>* tot) {
#pragma unroll
    for (int f = 0; f < NF; f++) {
        if (!act[f]) continue;
        bool ok;
        if constexpr (sizeof(R) == 4) {
            const FF pq = ff_norm(tot[f]);
            const FF al = ff_div(ff_load(cg->ffrz[f]), pq);
            ok = pq.hi > 0.f && isfinite(al.hi);
            if (ok) {
                ff_store(cg->ffalpha[f], al);
                cg->falpha[f] = al.rounded();
            }
        } else {
            const double al = cg->rz[f] / tot[f].s;
            ok = tot[f].s > 0.0 && isfinite(al);
            if (ok) cg->alpha[f] = al;
        }
        if (!ok) {
            cg->active[f] = 0;
            cg->iters[f] = cg->iter;
            atomicOr(flags, FEA_STATUS_BREAKDOWN);
        }
    }
}

// After a Chronopoulos-Gear iteration: convergence |r|^2 < tol^2 |b|^2, then
// beta = gamma'/gamma and alpha = gamma' / (delta' - beta gamma'/alpha) for
// the next iteration; iteration count and the max_iter limit.  tot holds
// gamma' = r.u, delta' = w.u and r.r per field.  Returns whether another
// iteration runs.  The FP32 solver does this in float-float arithmetic and
// stores |r|^2 as a double only when a field stops iterating.
template <typename R, int NF, typename S>
__device__ bool finish_cgcg(volatile S* cg, unsigned int* flags, const int (&act)[NF], const Acc<R>* tot) {
    const int it = cg->iter + 1;
    cg->iter = it;
    int any = 0;
#pragma unroll
    for (int f = 0; f < NF; f++) {
        cg->fresh[f] = 0;
        if (!act[f]) continue;
        const Acc<R>& rr = tot[2 * NF + f];
        int state;  // 0: iterates, 1: converged, 2: breakdown
        if constexpr (sizeof(R) == 4) {
            const FF r2 = ff_norm(rr);
            if (!isfinite(r2.hi)) {
                state = 2;
            } else if (ff_less(r2, ff_load(cg->ffthr[f]))) {
                state = 1;
            } else {
                const FF g = ff_norm(tot[f]), d = ff_norm(tot[NF + f]);
                const FF beta = ff_div(g, ff_load(cg->ffrz[f]));
                const FF den = ff_sub(d, ff_div(ff_mul(beta, g), ff_load(cg->ffalpha[f])));
                const FF alpha = ff_div(g, den);
                state = (!(den.hi > 0.f) || !isfinite(alpha.hi) || !isfinite(beta.hi)) ? 2 : 0;
                if (state == 0) {
                    cg->fbeta[f] = beta.rounded();
                    cg->falpha[f] = alpha.rounded();
                    ff_store(cg->ffalpha[f], alpha);
                    ff_store(cg->ffrz[f], g);
                }
            }
        } else {
            const double g = tot[f].s, d = tot[NF + f].s, r2 = rr.s;
            if (!isfinite(r2)) {
                state = 2;
            } else if (r2 < cg->thr[f]) {
                state = 1;
            } else {
                const double beta = g / cg->rz[f];
                const double den = d - beta * g / cg->alpha[f];
                const double alpha = g / den;
                state = (!(den > 0.0) || !isfinite(alpha) || !isfinite(beta)) ? 2 : 0;
                if (state == 0) {
                    cg->beta[f] = beta;
                    cg->alpha[f] = alpha;
                    cg->rz[f] = g;
                }
            }
            cg->rr[f] = r2;
        }
        if (state == 0) {
            any = 1;
            continue;
        }
        if constexpr (sizeof(R) == 4) cg->rr[f] = rr.value();
        cg->active[f] = 0;
        cg->iters[f] = it;
        if (state == 2) atomicOr(flags, FEA_STATUS_BREAKDOWN);
    }
    const bool cont = any && it < cg->max_iter;
    if (any && !cont) {
        atomicOr(flags, FEA_STATUS_NOT_CONVERGED);
#pragma unroll
        for (int f = 0; f < NF; f++)
            if (cg->active[f]) {
                if constexpr (sizeof(R) == 4) cg->rr[f] = tot[2 * NF + f].value();
                cg->active[f] = 0;
                cg->iters[f] = it;
            }
    }
    return cont;
}

// ---- standalone kernels (autotuning and timing probes) -------------------------------

// ---- graph construction helpers ---------------------------------------------------

template <typename... P>
cudaGraphNode_t add_kernel(cudaGraph_t g, cudaGraphNode_t dep, void (*fn)(P...), int grid, int block,
                           const typename std::tuple_element<0, std::tuple<P...>>::type& arg, size_t smem = 0) {
    auto local = arg;
    void* argv[] = {(void*)&local};
    cudaKernelNodeParams kp = {};
    kp.func = (void*)fn;
    kp.gridDim = dim3((unsigned)grid);
    kp.blockDim = dim3((unsigned)block);
    kp.sharedMemBytes = (unsigned int)smem;
    kp.kernelParams = argv;
    cudaGraphNode_t n;
    FEA_CUDA_TRY(cudaGraphAddKernelNode(&n, g, dep ? &dep : nullptr, dep ? 1 : 0, &kp));
    return n;
}

// from -> to as a programmatic dependency: `to` may be scheduled once every
// block of `from` has called grid_launch_dependents (or exited); it reads
// what `from` wrote only after grid_dependency_wait.
inline void add_programmatic_edge(cudaGraph_t g, cudaGraphNode_t from, cudaGraphNode_t to) {
    cudaGraphEdgeData ed = {};
    ed.from_port = cudaGraphKernelNodePortProgrammatic;
    ed.type = cudaGraphDependencyTypeProgrammatic;
    FEA_CUDA_TRY(cudaGraphAddDependencies(g, &from, &to, &ed, 1));
}

cudaGraphNode_t add_while(cudaGraph_t g, cudaGraphNode_t dep, cudaGraphConditionalHandle h, cudaGraph_t* body) {
    cudaGraphNodeParams np = {};
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = h;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    cudaGraphNode_t n;
    FEA_CUDA_TRY(cudaGraphAddNode(&n, g, dep ? &dep : nullptr, nullptr, dep ? 1 : 0, &np));
    *body = np.conditional.phGraph_out[0];
    return n;
}

// Opts `kernel` in to `smem` bytes of dynamic shared memory when that is above
// its current limit.  The limit is a property of the function, shared by
// every handle, so it only ever grows: a graph instantiated for a larger
// handle stays launchable after a smaller one is set up.
template <typename K>
void ensure_dyn_smem(K kernel, size_t smem) {
    if (smem <= 48 * 1024) return;
    cudaFuncAttributes fa{};
    FEA_CUDA_TRY(cudaFuncGetAttributes(&fa, kernel));
    if ((size_t)fa.maxDynamicSharedSizeBytes < smem)
        FEA_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
}

// Grid of one wave: SMs x resident blocks of this kernel (from the occupancy
// calculator, with `smem` bytes of dynamic shared memory, opted in above the
// default 48 KB), capped by the work and by the partial-sum stride.
template <typename K>
int wave_grid(K kernel, int64_t work_blocks, size_t smem = 0) {
    ensure_dyn_smem(kernel, smem);
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kBlock, smem) != cudaSuccess || per_sm < 1)
        per_sm = 1;
    int64_t g = (int64_t)num_sms() * per_sm;
    if (g > max_grid_blocks()) g = max_grid_blocks();
    if (g > work_blocks) g = work_blocks;
    return (int)(g < 1 ? 1 : g);
}

}  // namespace
}  // namespace fea
