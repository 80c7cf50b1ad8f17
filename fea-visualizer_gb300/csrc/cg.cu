// cg.cu -- the per-step hot path: fused right-hand side, Jacobi-preconditioned
// CG and the step loop, all inside one CUDA graph.
//
// Reference semantics: CPUSolver::advance_time (CPUSolver.cpp:64-146) solves
// A x = b with Eigen::ConjugateGradient<.., Lower|Upper> and its diagonal
// preconditioner (:65): stop when |r|^2 < tol^2 |b|^2, at most max_iter
// iterations.  The compute-shader path (cgm.glsl:104-149, GPUSolver.cpp:326-361)
// runs the same recurrences with a host round trip per stage; here the loop is
// a CUDA graph WHILE node over time steps with a WHILE node per solve whose
// body is ONE kernel per CG iteration (the Chronopoulos-Gear form below): the
// vector updates are fused into the SpMV, and a single grid-wide reduction
// gives every scalar of the next iteration.
// Inner products: FP32 products are accumulated exactly as float-float pairs
// per thread and per warp, then in FP64 across warps and blocks (the GB300's
// FP64 pipe is narrow, so FP64 arithmetic is kept off the per-element path).
// The block partials are combined by the last block to finish, in a fixed
// order, so every reduction is deterministic.
#include <algorithm>
#include <cmath>

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
    __device__ __forceinline__ void add_prod(double a, double b) { s = fma(a, b, s); }
    __device__ __forceinline__ void sub(const Acc& o) { s -= o.s; }
    __device__ __forceinline__ double value() const { return s; }
    __device__ __forceinline__ void shfl_add(int off) { s += __shfl_xor_sync(0xffffffffu, s, off); }
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
    __device__ __forceinline__ void shfl_add(int off) {
        const float oh = __shfl_xor_sync(0xffffffffu, hi, off);
        const float ol = __shfl_xor_sync(0xffffffffu, lo, off);
        add(oh);
        lo = __fadd_rn(lo, ol);
    }
};

// Block reduction of NV accumulators, then the grid-wide last-block step.
// Returns true in the last block, with totals in out[] valid in thread 0.
template <typename R, int NV>
__device__ __forceinline__ bool grid_reduce(Acc<R> (&acc)[NV], double* part, int stride, unsigned int* ticket,
                                            double (&out)[NV]) {
    __shared__ double sm[32 * NV];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; k++) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc[k].shfl_add(o);
        if (lane == 0) sm[wid * NV + k] = acc[k].value();
    }
    __syncthreads();
    double x[NV];
#pragma unroll
    for (int k = 0; k < NV; k++) x[k] = 0.0;
    if (threadIdx.x == 0) {
        const int nw = (blockDim.x + 31) >> 5;
        for (int w = 0; w < nw; w++)
#pragma unroll
            for (int k = 0; k < NV; k++) x[k] += sm[w * NV + k];
    }
    __syncthreads();
    // x[] holds the block totals in thread 0; the last block sums them.
    return last_block_commit<NV>(x, part, stride, ticket, sm, out);
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

// Threads are grouped LANES per CSR row; a warp covers 32/LANES consecutive
// rows per pass, so its loads of values and column indices are contiguous.
template <int LANES>
struct RowMap {
    static constexpr int RPW = 32 / LANES;
    int sub, grp;
    int64_t warp, nwarps;
    __device__ __forceinline__ RowMap() {
        const int lane = threadIdx.x & 31;
        sub = lane & (LANES - 1);
        grp = lane / LANES;
        warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
        nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    }
};

// ---- CSR SpMV building blocks ------------------------------------------------------
//
// Every kernel reads vectors that earlier launches wrote, so the read-only
// path (LoadRO) is valid for all of them.

struct LoadRO {
    template <typename T>
    static __device__ __forceinline__ T ld(const T* p) {
        return ldv<T>(p, false);
    }
};

// Control values of one phase, read once per phase by every thread.
template <typename R, int NF>
struct PhaseCtl {
    int par;          // iteration parity: p_old = pp[par], p_new = pp[par ^ 1]
    int act[NF];
    bool fresh[NF];
    bool need_old;
    bool any;
    R beta[NF], alpha[NF];
    __device__ __forceinline__ void load(const CgState* cg) {
        const volatile CgState* v = cg;
        par = v->iter & 1;
        need_old = false;
        any = false;
#pragma unroll
        for (int f = 0; f < NF; f++) {
            act[f] = v->active[f];
            fresh[f] = v->fresh[f] != 0;
            beta[f] = fresh[f] ? (R)0 : (R)v->beta[f];
            alpha[f] = act[f] ? (R)v->alpha[f] : (R)0;
            need_old |= !fresh[f];
            any |= act[f] != 0;
        }
    }
};

// q = A p_new with p_new = z + beta p_old computed for every gathered column
// (the direction update of the previous iteration, fused; the two p buffers
// alternate with the iteration parity), plus p_new.q into dot[].
//
// Warp-cooperative CSR: a warp owns 32 consecutive rows, whose stored entries
// form one contiguous range.  The warp streams that range in windows of
// 32*WCH entries: every lane issues WCH coalesced value/column loads, then WCH
// independent gathers, so each round trip to memory carries a whole window
// rather than one row.  Products go to shared memory and each lane sums its
// own row in column order.
template <typename R, int NF, int WCH, typename LP>
__device__ __forceinline__ void spmv_phase(const StepArgs<R, NF>& a, const PhaseCtl<R, NF>& c,
                                           FV<R, NF> (*sm)[32 * WCH], Acc<R> (&dot)[NF]) {
    constexpr int WIN = 32 * WCH;
    const FV<R, NF>* pold = a.pp[c.par];
    FV<R, NF>* pnew = a.pp[c.par ^ 1];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int64_t N = a.N;
    for (int64_t r0 = warp * 32; r0 < N; r0 += nwarps * 32) {
        const int64_t row = r0 + lane;
        const int32_t rs = ldg(a.rp + (row < N ? row : N));
        int32_t re = __shfl_down_sync(0xffffffffu, rs, 1);
        if (lane == 31) re = ldg(a.rp + (r0 + 32 < N ? r0 + 32 : N));
        const int32_t e0 = __shfl_sync(0xffffffffu, rs, 0);
        const int32_t e1 = __shfl_sync(0xffffffffu, re, 31);
        R acc[NF];
#pragma unroll
        for (int f = 0; f < NF; f++) acc[f] = 0;
        for (int32_t wb = e0; wb < e1; wb += WIN) {
            FV<R, NF> av[WCH];
            int32_t cc[WCH];
#pragma unroll
            for (int k = 0; k < WCH; k++) {
                const int32_t idx = wb + k * 32 + lane;
                cc[k] = -1;
                if (idx < e1) {
                    av[k] = ldv(a.A + idx, false);
                    cc[k] = ldg(a.col + idx);
                }
            }
#pragma unroll
            for (int k = 0; k < WCH; k++) {
                FV<R, NF> prod;
#pragma unroll
                for (int f = 0; f < NF; f++) prod.v[f] = 0;
                if (cc[k] >= 0) {
                    const FV<R, NF> zc = LP::ld(a.z + cc[k]);
                    FV<R, NF> pc = zc;
                    if (c.need_old) pc = LP::ld(pold + cc[k]);
#pragma unroll
                    for (int f = 0; f < NF; f++) {
                        const R pn = c.fresh[f] ? zc.v[f] : fma(c.beta[f], pc.v[f], zc.v[f]);
                        prod.v[f] = av[k].v[f] * pn;
                    }
                }
                sm[wib][k * 32 + lane] = prod;
            }
            __syncwarp();
            const int32_t lo = (rs > wb ? rs : wb) - wb;
            const int32_t hi = (re < wb + WIN ? re : wb + WIN) - wb;
            for (int32_t k = lo; k < hi; k++) {
                const FV<R, NF> t = sm[wib][k];
#pragma unroll
                for (int f = 0; f < NF; f++) acc[f] += t.v[f];
            }
            __syncwarp();
        }
        if (row < N) {
            const FV<R, NF> zr = LP::ld(a.z + row);
            FV<R, NF> pr = zr, qv;
            if (c.need_old) pr = LP::ld(pold + row);
#pragma unroll
            for (int f = 0; f < NF; f++) {
                const R pn = c.fresh[f] ? zr.v[f] : fma(c.beta[f], pr.v[f], zr.v[f]);
                pr.v[f] = pn;
                qv.v[f] = acc[f];
                dot[f].add_prod(pn, acc[f]);
            }
            pnew[row] = pr;
            a.q[row] = qv;
        }
    }
}

// After the SpMV phase: alpha = r.z / p.q, or breakdown.
template <typename R, int NF>
__device__ void finish_spmv(volatile CgState* cg, RunState* run, const int (&act)[NF], const double* tot) {
#pragma unroll
    for (int f = 0; f < NF; f++) {
        if (!act[f]) continue;
        cg->pq[f] = tot[f];
        const double al = cg->rz[f] / tot[f];
        if (!(tot[f] > 0.0) || !isfinite(al)) {
            cg->active[f] = 0;
            cg->iters[f] = cg->iter;
            atomicOr(&run->flags, FEA_STATUS_BREAKDOWN);
        } else {
            cg->alpha[f] = al;
        }
    }
}

// After a Chronopoulos-Gear iteration: convergence |r|^2 < tol^2 |b|^2, then
// beta = gamma'/gamma and alpha = gamma' / (delta' - beta gamma'/alpha) for
// the next iteration; iteration count and the max_iter limit.  tot holds
// gamma' = r.u, delta' = w.u and r.r per field.  Returns whether another
// iteration runs.
template <typename R, int NF>
__device__ bool finish_cgcg(volatile CgState* cg, RunState* run, const int (&act)[NF], const double* tot) {
    const int it = cg->iter + 1;
    cg->iter = it;
    int any = 0;
#pragma unroll
    for (int f = 0; f < NF; f++) {
        cg->fresh[f] = 0;
        if (!act[f]) continue;
        const double g = tot[f], d = tot[NF + f], rr = tot[2 * NF + f];
        cg->rr[f] = rr;
        if (!isfinite(rr)) {
            cg->active[f] = 0;
            cg->iters[f] = it;
            atomicOr(&run->flags, FEA_STATUS_BREAKDOWN);
            continue;
        }
        if (rr < cg->thr[f]) {
            cg->active[f] = 0;
            cg->iters[f] = it;
            continue;
        }
        const double beta = g / cg->rz[f];
        const double den = d - beta * g / cg->alpha[f];
        const double alpha = g / den;
        if (!(den > 0.0) || !isfinite(alpha) || !isfinite(beta)) {
            cg->active[f] = 0;
            cg->iters[f] = it;
            atomicOr(&run->flags, FEA_STATUS_BREAKDOWN);
            continue;
        }
        cg->beta[f] = beta;
        cg->alpha[f] = alpha;
        cg->rz[f] = g;
        any = 1;
    }
    const bool cont = any && it < cg->max_iter;
    if (any && !cont) {
        atomicOr(&run->flags, FEA_STATUS_NOT_CONVERGED);
#pragma unroll
        for (int f = 0; f < NF; f++)
            if (cg->active[f]) {
                cg->active[f] = 0;
                cg->iters[f] = it;
            }
    }
    return cont;
}

template <int NV, typename R>
__device__ __forceinline__ void block_totals(Acc<R> (&acc)[NV], double* sm, double (&blk)[NV]) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; k++) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc[k].shfl_add(o);
        if (lane == 0) sm[wid * NV + k] = acc[k].value();
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < NV; k++) blk[k] = 0.0;
    if (threadIdx.x == 0) {
        const int nw = (blockDim.x + 31) >> 5;
        for (int w = 0; w < nw; w++)
#pragma unroll
            for (int k = 0; k < NV; k++) blk[k] += sm[w * NV + k];
    }
    __syncthreads();
}

// ---- standalone kernels (autotuning and timing probes) -------------------------------

template <typename R, int NF, int WCH>
__global__ void __launch_bounds__(kBlock, (WCH <= 4 ? 6 : 4)) k_cg_spmv(StepArgs<R, NF> a) {
    __shared__ FV<R, NF> sm[kBlock / 32][32 * WCH];
    __shared__ double red[32 * NF];
    PhaseCtl<R, NF> c;
    c.load(a.cg);
    Acc<R> dot[NF];
    spmv_phase<R, NF, WCH, LoadRO>(a, c, sm, dot);
    double blk[NF], tot[NF];
    block_totals<NF>(dot, red, blk);
    if (last_block_commit<NF>(blk, a.part, a.part_stride, a.tickets + 0, red, tot) && threadIdx.x == 0)
        finish_spmv<R, NF>(a.cg, a.run, c.act, tot);
}

// ---- Chronopoulos-Gear iteration -----------------------------------------------------
//
// Jacobi-preconditioned CG rearranged (Chronopoulos & Gear, 1989) so that one
// iteration needs one global reduction: with u = D^-1 r, w = A u and s = A p,
//   p = u + beta p,  s = w + beta s,  x += alpha p,  r -= alpha s,
//   u' = D^-1 r,  w' = A u',  gamma' = r.u',  delta' = w'.u',
//   beta' = gamma'/gamma,  alpha' = gamma' / (delta' - beta' gamma'/alpha).
// It produces the same iterates as the textbook recurrence in exact
// arithmetic.  One kernel per iteration: every row owner applies the vector
// updates, and the SpMV recomputes u' at each gathered column from the old r,
// w and s there (so r, w and s alternate between two buffers).

// Set-up of a solve: w0 = A z (z = D^-1 r0 from k_rhs / k_refine), delta0 =
// z.w0 and alpha0 = r0.z / delta0.  The SpMV of the probe kernel with p = z.
template <typename R, int NF, int WCH>
__global__ void __launch_bounds__(kBlock, (WCH <= 4 ? 6 : 4)) k_cgcg_init(StepArgs<R, NF> a) {
    __shared__ FV<R, NF> sm[kBlock / 32][32 * WCH];
    __shared__ double red[32 * NF];
    PhaseCtl<R, NF> c;
    c.load(a.cg);
    c.need_old = false;
#pragma unroll
    for (int f = 0; f < NF; f++) {
        c.fresh[f] = true;
        c.beta[f] = 0;
    }
    StepArgs<R, NF> v = a;
    v.pp[c.par ^ 1] = a.pp[0];
    v.q = a.wb[c.par];
    Acc<R> dot[NF];
    spmv_phase<R, NF, WCH, LoadRO>(v, c, sm, dot);
    double blk[NF], tot[NF];
    block_totals<NF>(dot, red, blk);
    if (last_block_commit<NF>(blk, a.part, a.part_stride, a.tickets + 0, red, tot) && threadIdx.x == 0) {
        volatile CgState* cg = a.cg;
        finish_spmv<R, NF>(cg, a.run, c.act, tot);
        int any = 0;
#pragma unroll
        for (int f = 0; f < NF; f++) {
            cg->fresh[f] = 1;  // the first iteration takes p = u, s = w
            any |= cg->active[f];
        }
        signal_loop(a, any != 0);
    }
}

template <typename R, int NF, int WCH>
__global__ void __launch_bounds__(kBlock, (WCH <= 4 ? 6 : 4)) k_cgcg_iter(StepArgs<R, NF> a) {
    constexpr int WIN = 32 * WCH;
    __shared__ FV<R, NF> sm[kBlock / 32][WIN];
    __shared__ double red[32 * 3 * NF];
    PhaseCtl<R, NF> c;
    c.load(a.cg);
    const FV<R, NF>* __restrict__ r0 = a.rb[c.par];
    const FV<R, NF>* __restrict__ w0 = a.wb[c.par];
    const FV<R, NF>* __restrict__ s0 = a.sb[c.par];
    FV<R, NF>* __restrict__ r1 = a.rb[c.par ^ 1];
    FV<R, NF>* __restrict__ w1 = a.wb[c.par ^ 1];
    FV<R, NF>* __restrict__ s1 = a.sb[c.par ^ 1];
    // new residual and preconditioned residual of one unknown from its old r, w, s
    auto advance = [&](const FV<R, NF>& ro, const FV<R, NF>& wo, const FV<R, NF>& so, const FV<R, NF>& d,
                       FV<R, NF>& sn, FV<R, NF>& rn, FV<R, NF>& un) {
#pragma unroll
        for (int f = 0; f < NF; f++) {
            sn.v[f] = c.fresh[f] ? wo.v[f] : fma(c.beta[f], so.v[f], wo.v[f]);
            rn.v[f] = c.act[f] ? fma(-c.alpha[f], sn.v[f], ro.v[f]) : ro.v[f];
            un.v[f] = d.v[f] * rn.v[f];
        }
    };
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int64_t N = a.N;
    Acc<R> dots[3 * NF];  // gamma', delta', |r'|^2
    for (int64_t row0 = warp * 32; row0 < N; row0 += nwarps * 32) {
        const int64_t row = row0 + lane;
        const int32_t rs = ldg(a.rp + (row < N ? row : N));
        int32_t re = __shfl_down_sync(0xffffffffu, rs, 1);
        if (lane == 31) re = ldg(a.rp + (row0 + 32 < N ? row0 + 32 : N));
        const int32_t e0 = __shfl_sync(0xffffffffu, rs, 0);
        const int32_t e1 = __shfl_sync(0xffffffffu, re, 31);
        R acc[NF];
#pragma unroll
        for (int f = 0; f < NF; f++) acc[f] = 0;
        for (int32_t wb = e0; wb < e1; wb += WIN) {
            FV<R, NF> av[WCH];
            int32_t cc[WCH];
#pragma unroll
            for (int k = 0; k < WCH; k++) {
                const int32_t idx = wb + k * 32 + lane;
                cc[k] = -1;
                if (idx < e1) {
                    av[k] = ldv(a.A + idx, false);
                    cc[k] = ldg(a.col + idx);
                }
            }
#pragma unroll
            for (int k = 0; k < WCH; k++) {
                FV<R, NF> prod;
#pragma unroll
                for (int f = 0; f < NF; f++) prod.v[f] = 0;
                if (cc[k] >= 0) {
                    const int32_t col = cc[k];
                    const FV<R, NF> ro = ldv(r0 + col, false), wo = ldv(w0 + col, false);
                    const FV<R, NF> d = ldv(a.dinv + col, false);
                    FV<R, NF> so = wo;
                    if (c.need_old) so = ldv(s0 + col, false);
                    FV<R, NF> sn, rn, un;
                    advance(ro, wo, so, d, sn, rn, un);
#pragma unroll
                    for (int f = 0; f < NF; f++) prod.v[f] = av[k].v[f] * un.v[f];
                }
                sm[wib][k * 32 + lane] = prod;
            }
            __syncwarp();
            const int32_t lo = (rs > wb ? rs : wb) - wb;
            const int32_t hi = (re < wb + WIN ? re : wb + WIN) - wb;
            for (int32_t k = lo; k < hi; k++) {
                const FV<R, NF> t = sm[wib][k];
#pragma unroll
                for (int f = 0; f < NF; f++) acc[f] += t.v[f];
            }
            __syncwarp();
        }
        if (row < N) {
            const FV<R, NF> ro = ldv(r0 + row, false), wo = ldv(w0 + row, false), d = ldv(a.dinv + row, false);
            FV<R, NF> so = wo;
            if (c.need_old) so = ldv(s0 + row, false);
            FV<R, NF> x = a.x[row], p = a.pp[0][row];
            FV<R, NF> sn, rn, un, wn;
            advance(ro, wo, so, d, sn, rn, un);
#pragma unroll
            for (int f = 0; f < NF; f++) {
                if (c.act[f]) {
                    const R ui = d.v[f] * ro.v[f];
                    p.v[f] = c.fresh[f] ? ui : fma(c.beta[f], p.v[f], ui);
                    x.v[f] = fma(c.alpha[f], p.v[f], x.v[f]);
                }
                wn.v[f] = acc[f];
                dots[f].add_prod(rn.v[f], un.v[f]);
                dots[NF + f].add_prod(wn.v[f], un.v[f]);
                dots[2 * NF + f].add_prod(rn.v[f], rn.v[f]);
            }
            a.x[row] = x;
            a.pp[0][row] = p;
            r1[row] = rn;
            s1[row] = sn;
            w1[row] = wn;
        }
    }
    double blk[3 * NF], tot[3 * NF];
    block_totals<3 * NF>(dots, red, blk);
    if (last_block_commit<3 * NF>(blk, a.part, a.part_stride, a.tickets + 1, red, tot) && threadIdx.x == 0)
        signal_loop(a, finish_cgcg<R, NF>(a.cg, a.run, c.act, tot));
}

// Fused right-hand side + initial residual r = b - A x0 (warm start x0 = the
// previous solution), z = D^-1 r, p = z, and the CG set-up scalars.  Also the
// has_numerical_instability test of the state entering the step.
template <typename R, int NF, int EQ, int LANES>
__global__ void __launch_bounds__(kBlock) k_rhs(StepArgs<R, NF> a) {
    const StepParams P = *a.prm;
    const R dt = (R)P.dt;
    Acc<R> dots[3 * NF];  // |b|^2, |r|^2, r.z per field
    unsigned int flags = 0;
    RowMap<LANES> m;
    for (int64_t base = m.warp * m.RPW; base < a.N; base += m.nwarps * m.RPW) {
        const int64_t row = base + m.grp;
        Acc<R> bs[NF], ax[NF];
        if (row < a.N) {
            const int32_t e1 = ldg(a.rp + row + 1);
            for (int32_t e = ldg(a.rp + row) + m.sub; e < e1; e += LANES) {
                const int32_t c = ldg(a.col + e);
                const FV<R, NF> av = ldfv(a.A + e);
                const FV<R, NF> xc = a.x[c];
                const R me = ldg(a.M + e);
                if constexpr (EQ == EQ_HEAT) {
                    bs[0].add_prod(div_rn(me, dt), xc.v[0]);
                } else if constexpr (EQ == EQ_ADV_EXPLICIT) {
                    bs[0].add_prod(div_rn(me, dt), xc.v[0]);
                    bs[0].add_prod((R)P.adv_sign * ldg(a.Adv + e), xc.v[0]);
                } else if constexpr (EQ == EQ_WAVE_REF) {
                    bs[0].add_prod(div_rn(me, dt), xc.v[0]);
                    bs[0].add_prod(-(R)P.c2 * ldg(a.K + e), a.u[c]);
                } else if constexpr (EQ == EQ_WAVE_NEWMARK) {
                    const R uc = a.u[c], vc = a.v[c];
                    const R ut = uc + dt * vc + dt * dt * ((R)0.5 - (R)P.beta) * xc.v[0];
                    bs[0].add_prod(-(R)P.c2 * ldg(a.K + e), ut);
                } else if constexpr (EQ == EQ_NEWMARK_INIT) {
                    bs[0].add_prod(-(R)P.c2 * ldg(a.K + e), a.u[c]);
                } else if constexpr (EQ == EQ_GS_REF) {
#pragma unroll
                    for (int f = 0; f < NF; f++) bs[f].add_prod(div_rn(me, dt), xc.v[f]);
                } else {  // EQ_GS_CONSISTENT
                    const R u = xc.v[0], v = xc.v[NF - 1];
                    const R uvv = u * (v * v);
                    const R wu = u / dt - uvv + (R)P.F * ((R)1 - u);
                    const R wv = v / dt + uvv - ((R)P.F + (R)P.k) * v;
                    bs[0].add_prod(me, wu);
                    bs[NF - 1].add_prod(me, wv);
                }
#pragma unroll
                for (int f = 0; f < NF; f++) ax[f].add_prod(av.v[f], xc.v[f]);
            }
        }
#pragma unroll
        for (int o = LANES / 2; o > 0; o >>= 1)
#pragma unroll
            for (int f = 0; f < NF; f++) {
                bs[f].shfl_add(o);
                ax[f].shfl_add(o);
            }
        if (m.sub == 0 && row < a.N) {
            const FV<R, NF> xr = a.x[row];
            if constexpr (EQ == EQ_GS_REF) {  // nodal reaction, CPUSolver.cpp:134,137
                const R u = xr.v[0], v = xr.v[NF - 1];
                const R uvv = u * (v * v);
                bs[0].add(-uvv);
                bs[0].add((R)P.F * ((R)1 - u));
                bs[NF - 1].add(uvv);
                bs[NF - 1].add(-((R)P.F + (R)P.k) * v);
            }
            if constexpr (EQ == EQ_WAVE_REF || EQ == EQ_NEWMARK_INIT) {
                flags |= check_value(a.u[row]) | check_value(a.v[row]);
            } else if constexpr (EQ == EQ_WAVE_NEWMARK) {
                const R ur = a.u[row], vr = a.v[row], ar = xr.v[0];
                flags |= check_value(ur) | check_value(vr);
                a.ut[row] = ur + dt * vr + dt * dt * ((R)0.5 - (R)P.beta) * ar;
                a.vt[row] = vr + dt * ((R)1 - (R)P.gamma) * ar;
            } else {
#pragma unroll
                for (int f = 0; f < NF; f++) flags |= check_value(xr.v[f]);
            }
            const FV<R, NF> d = ldfv(a.dinv + row);
            FV<R, NF> bv, rv, pv;
#pragma unroll
            for (int f = 0; f < NF; f++) {
                bv.v[f] = (R)bs[f].value();
                bs[f].sub(ax[f]);
                rv.v[f] = (R)bs[f].value();
                pv.v[f] = d.v[f] * rv.v[f];
                dots[f].add_prod(bv.v[f], bv.v[f]);
                dots[NF + f].add_prod(rv.v[f], rv.v[f]);
                dots[2 * NF + f].add_prod(rv.v[f], pv.v[f]);
            }
            a.b[row] = bv;
            a.rb[0][row] = rv;  // iteration 0 reads parity 0
            a.z[row] = pv;
        }
    }
    raise_flags(a.run, flags);
    double tot[3 * NF];
    if (grid_reduce<R, 3 * NF>(dots, a.part, a.part_stride, a.tickets + 2, tot) && threadIdx.x == 0) {
        CgState* cg = a.cg;
        RunState* run = a.run;
        const int stop = (atomicOr(&run->flags, 0u) & (FEA_STATUS_BLOWUP | FEA_STATUS_NONFINITE)) != 0;
        cg->stop = stop;
        cg->iter = 0;
        cg->max_iter = run->max_iter;
        int any = 0;
        const double tiny = sizeof(R) == 4 ? 1.1754943508222875e-38 : 2.2250738585072014e-308;
#pragma unroll
        for (int f = 0; f < NF; f++) {
            const double bb = tot[f], rr = tot[NF + f], rz = tot[2 * NF + f];
            double thr = run->tol * run->tol * bb;
            cg->bb[f] = bb;
            cg->thr[f] = thr < tiny ? tiny : thr;
            cg->rr[f] = rr;
            cg->rz[f] = rz;
            cg->iters[f] = 0;
            cg->fresh[f] = 1;  // the first direction is p = z
            cg->active[f] = (!stop && bb > 0.0 && rr >= cg->thr[f]) ? 1 : 0;
            any |= cg->active[f];
        }
        signal_loop(a, any != 0);
    }
}

// After the first CG loop: zero right-hand sides give x = 0 (Eigen's
// early exit), then one FP64-accurate true-residual pass r = b - A x.  Fields
// whose true residual is still above the threshold restart CG from there.
template <typename R, int NF, int LANES>
__global__ void __launch_bounds__(kBlock) k_refine(StepArgs<R, NF> a) {
    CgState* cg = a.cg;
    const int stop = cg->stop;
    const int refine = a.run->refine && cg->iter < cg->max_iter && !stop;
    int zero[NF];
#pragma unroll
    for (int f = 0; f < NF; f++) zero[f] = !stop && !(cg->bb[f] > 0.0);
    Acc<R> dots[2 * NF];
    RowMap<LANES> m;
    for (int64_t base = m.warp * m.RPW; base < a.N; base += m.nwarps * m.RPW) {
        const int64_t row = base + m.grp;
        Acc<R> ax[NF];
        if (refine && row < a.N) {
            const int32_t e1 = ldg(a.rp + row + 1);
            for (int32_t e = ldg(a.rp + row) + m.sub; e < e1; e += LANES) {
                const FV<R, NF> av = ldfv(a.A + e);
                const FV<R, NF> xc = a.x[ldg(a.col + e)];
#pragma unroll
                for (int f = 0; f < NF; f++) ax[f].add_prod(av.v[f], xc.v[f]);
            }
        }
        if (refine) {
#pragma unroll
            for (int o = LANES / 2; o > 0; o >>= 1)
#pragma unroll
                for (int f = 0; f < NF; f++) ax[f].shfl_add(o);
        }
        if (m.sub == 0 && row < a.N) {
            bool zany = false;
#pragma unroll
            for (int f = 0; f < NF; f++) zany |= zero[f] != 0;
            if (zany) {
                FV<R, NF> xr = a.x[row];
#pragma unroll
                for (int f = 0; f < NF; f++)
                    if (zero[f]) xr.v[f] = 0;
                a.x[row] = xr;
            }
            if (refine) {
                const FV<R, NF> bv = a.b[row], d = ldfv(a.dinv + row);
                FV<R, NF> rv, pv;
#pragma unroll
                for (int f = 0; f < NF; f++) {
                    Acc<R> t;
                    t.add(bv.v[f]);
                    t.sub(ax[f]);
                    rv.v[f] = (R)t.value();
                    pv.v[f] = d.v[f] * rv.v[f];
                    dots[f].add_prod(rv.v[f], rv.v[f]);
                    dots[NF + f].add_prod(rv.v[f], pv.v[f]);
                }
                a.rb[cg->iter & 1][row] = rv;  // the restart continues the iteration parity
                a.z[row] = pv;
            }
        }
    }
    double tot[2 * NF];
    if (grid_reduce<R, 2 * NF>(dots, a.part, a.part_stride, a.tickets + 3, tot) && threadIdx.x == 0) {
        int any = 0;
#pragma unroll
        for (int f = 0; f < NF; f++) {
            cg->active[f] = 0;
            cg->fresh[f] = 1;
            if (refine && !zero[f] && cg->bb[f] > 0.0) {
                cg->rr[f] = tot[f];
                if (tot[f] >= cg->thr[f]) {
                    cg->rz[f] = tot[NF + f];
                    cg->active[f] = 1;
                    any = 1;
                }
            }
        }
        signal_loop(a, any != 0);
    }
}

// Wave updates after the solve.
template <typename R, int NF, int EQ>
__global__ void __launch_bounds__(kBlock) k_post(StepArgs<R, NF> a) {
    if (a.cg->stop) return;
    const StepParams P = *a.prm;
    const R dt = (R)P.dt;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < a.N; i += (int64_t)gridDim.x * blockDim.x) {
        if constexpr (EQ == EQ_WAVE_REF) {  // u = u + v dt, CPUSolver.cpp:118
            a.u[i] = a.u[i] + a.x[i].v[0] * dt;
        } else if constexpr (EQ == EQ_WAVE_NEWMARK) {
            const R acc = a.x[i].v[0];
            a.u[i] = a.ut[i] + (R)P.beta * dt * dt * acc;
            a.v[i] = a.vt[i] + (R)P.gamma * dt * acc;
        }
    }
}

// Step bookkeeping and the outer loop condition (single thread).
template <typename R, int NF>
__global__ void k_stepctl(StepArgs<R, NF> a) {
    CgState* cg = a.cg;
    RunState* run = a.run;
    if (!cg->stop) {
        run->steps_done += 1;
        run->steps_left -= 1;
        run->total_iters += cg->iter;
        for (int f = 0; f < NF; f++) {
            run->last_iters[f] = cg->iters[f];
            run->last_rel[f] = cg->bb[f] > 0.0 ? sqrt(cg->rr[f] / cg->bb[f]) : 0.0;
        }
    }
    const int cont = !cg->stop && run->steps_left > 0 &&
                     !(run->flags & (FEA_STATUS_BLOWUP | FEA_STATUS_NONFINITE));
    signal_loop(a, cont != 0);
}

template <typename R, int NF>
__global__ void k_start(StepArgs<R, NF> a) {
    signal_loop(a, a.run->steps_left > 0);
}

// has_numerical_instability of the state after the last step.
template <typename R, int NF, int EQ>
__global__ void __launch_bounds__(kBlock) k_final_check(StepArgs<R, NF> a) {
    unsigned int flags = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < a.N; i += (int64_t)gridDim.x * blockDim.x) {
        if constexpr (EQ == EQ_WAVE_REF || EQ == EQ_WAVE_NEWMARK || EQ == EQ_NEWMARK_INIT) {
            flags |= check_value(a.u[i]) | check_value(a.v[i]);
        } else {
            const FV<R, NF> x = a.x[i];
#pragma unroll
            for (int f = 0; f < NF; f++) flags |= check_value(x.v[f]);
        }
    }
    raise_flags(a.run, flags);
}

// ---- graph construction ----------------------------------------------------------

template <typename... P>
cudaGraphNode_t add_kernel(cudaGraph_t g, cudaGraphNode_t dep, void (*fn)(P...), int grid, int block,
                           const typename std::tuple_element<0, std::tuple<P...>>::type& arg) {
    auto local = arg;
    void* argv[] = {(void*)&local};
    cudaKernelNodeParams kp = {};
    kp.func = (void*)fn;
    kp.gridDim = dim3((unsigned)grid);
    kp.blockDim = dim3((unsigned)block);
    kp.sharedMemBytes = 0;
    kp.kernelParams = argv;
    cudaGraphNode_t n;
    FEA_CUDA_TRY(cudaGraphAddKernelNode(&n, g, dep ? &dep : nullptr, dep ? 1 : 0, &kp));
    return n;
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

int g_max_grid = 0;

// Grid of one wave: SMs x resident blocks of this kernel (from the occupancy
// calculator), capped by the work and by the partial-sum stride.
template <typename K>
int wave_grid(K kernel, int64_t work_blocks) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kBlock, 0) != cudaSuccess || per_sm < 1)
        per_sm = 1;
    int64_t g = (int64_t)num_sms() * per_sm;
    if (g > max_grid_blocks()) g = max_grid_blocks();
    if (g > work_blocks) g = work_blocks;
    return (int)(g < 1 ? 1 : g);
}

constexpr int kRowLanes = 8;  // lanes per row of the once-per-step kernels

template <typename R, int NF, int WCH>
struct Grids {
    int spmv, iter, rhs, stream;
    explicit Grids(int64_t N) {
        spmv = wave_grid(k_cgcg_init<R, NF, WCH>, ceil_div(N, kBlock));
        iter = wave_grid(k_cgcg_iter<R, NF, WCH>, ceil_div(N, kBlock));
        rhs = (int)std::min<int64_t>(max_grid_blocks(), std::max<int64_t>(1, ceil_div(N, (kBlock / kRowLanes))));
        stream = (int)std::min<int64_t>(max_grid_blocks(), std::max<int64_t>(1, ceil_div(N, kBlock)));
    }
};

// Argument sets of a step: the step loop (a) and the two CG loops (a1: after
// k_rhs, a2: after k_refine); each names the condition it sets.
template <typename R, int NF>
struct LoopArgs {
    StepArgs<R, NF> a, a1, a2;
    LoopArgs(const StepArgs<R, NF>& base, LoopFlags* lf, int use_graph) : a(base), a1(base), a2(base) {
        a.use_graph = a1.use_graph = a2.use_graph = use_graph;
        a.cont = &lf->step;
        a1.cont = &lf->cg1;
        a2.cont = &lf->cg2;
    }
};

// Step graph:  start -> WHILE(step) { rhs -> init -> WHILE(cg1) { iter }
//              -> refine -> init -> WHILE(cg2) { iter } -> [post] -> stepctl }
//              -> final_check
template <typename R, int NF, int EQ, int WCH>
void build_graph_t(StepGraph& G, const StepArgs<R, NF>& base, LoopFlags* lf) {
    LoopArgs<R, NF> L(base, lf, 1);
    const Grids<R, NF, WCH> g(base.N);
    cudaGraph_t top;
    FEA_CUDA_TRY(cudaGraphCreate(&top, 0));
    G.graph = top;
    FEA_CUDA_TRY(cudaGraphConditionalHandleCreate(&L.a.cond, top, 0, 0));
    cudaGraphNode_t n = add_kernel(top, nullptr, k_start<R, NF>, 1, 1, L.a);
    cudaGraph_t step_body;
    n = add_while(top, n, L.a.cond, &step_body);
    add_kernel(top, n, k_final_check<R, NF, EQ>, g.stream, kBlock, L.a);
    FEA_CUDA_TRY(cudaGraphConditionalHandleCreate(&L.a1.cond, step_body, 0, 0));
    FEA_CUDA_TRY(cudaGraphConditionalHandleCreate(&L.a2.cond, step_body, 0, 0));
    cudaGraphNode_t s = add_kernel(step_body, nullptr, k_rhs<R, NF, EQ, kRowLanes>, g.rhs, kBlock, L.a1);
    s = add_kernel(step_body, s, k_cgcg_init<R, NF, WCH>, g.spmv, kBlock, L.a1);
    cudaGraph_t body1, body2;
    s = add_while(step_body, s, L.a1.cond, &body1);
    add_kernel(body1, nullptr, k_cgcg_iter<R, NF, WCH>, g.iter, kBlock, L.a1);
    s = add_kernel(step_body, s, k_refine<R, NF, kRowLanes>, g.rhs, kBlock, L.a2);
    s = add_kernel(step_body, s, k_cgcg_init<R, NF, WCH>, g.spmv, kBlock, L.a2);
    s = add_while(step_body, s, L.a2.cond, &body2);
    add_kernel(body2, nullptr, k_cgcg_iter<R, NF, WCH>, g.iter, kBlock, L.a2);
    if constexpr (EQ == EQ_WAVE_REF || EQ == EQ_WAVE_NEWMARK)
        s = add_kernel(step_body, s, k_post<R, NF, EQ>, g.stream, kBlock, L.a);
    add_kernel(step_body, s, k_stepctl<R, NF>, 1, 1, L.a);
    FEA_CUDA_TRY(cudaGraphInstantiate(&G.exec, top, 0));
}

int read_flag(const int* d, cudaStream_t st) {
    int h = 0;
    FEA_CUDA_TRY(cudaMemcpyAsync(&h, d, sizeof(int), cudaMemcpyDeviceToHost, st));
    FEA_CUDA_TRY(cudaStreamSynchronize(st));
    return h;
}

// The same kernels launched one by one with the loop conditions read back
// on the host: every kernel is then visible to profilers (kernels inside
// graphs with conditional nodes are not).  Each loop is bounded by the
// kernels' own iteration and step limits.
template <typename R, int NF, int EQ, int WCH>
void run_stream_t(const StepArgs<R, NF>& base, LoopFlags* lf, cudaStream_t st) {
    LoopArgs<R, NF> L(base, lf, 0);
    const Grids<R, NF, WCH> g(base.N);
    k_start<R, NF><<<1, 1, 0, st>>>(L.a);
    FEA_CHECK_LAUNCH();
    while (read_flag(&lf->step, st)) {
        k_rhs<R, NF, EQ, kRowLanes><<<g.rhs, kBlock, 0, st>>>(L.a1);
        FEA_CHECK_LAUNCH();
        for (const StepArgs<R, NF>* la : {&L.a1, &L.a2}) {
            if (la == &L.a2) {
                k_refine<R, NF, kRowLanes><<<g.rhs, kBlock, 0, st>>>(L.a2);
                FEA_CHECK_LAUNCH();
            }
            k_cgcg_init<R, NF, WCH><<<g.spmv, kBlock, 0, st>>>(*la);
            FEA_CHECK_LAUNCH();
            while (read_flag(la->cont, st)) {
                k_cgcg_iter<R, NF, WCH><<<g.iter, kBlock, 0, st>>>(*la);
                FEA_CHECK_LAUNCH();
            }
        }
        if constexpr (EQ == EQ_WAVE_REF || EQ == EQ_WAVE_NEWMARK) {
            k_post<R, NF, EQ><<<g.stream, kBlock, 0, st>>>(L.a);
            FEA_CHECK_LAUNCH();
        }
        k_stepctl<R, NF><<<1, 1, 0, st>>>(L.a);
        FEA_CHECK_LAUNCH();
    }
    k_final_check<R, NF, EQ><<<g.stream, kBlock, 0, st>>>(L.a);
    FEA_CHECK_LAUNCH();
}

// SpMV variants: entries streamed per lane and window (the autotuned shape).
template <typename R, int NF, int EQ>
void dispatch_variant(StepGraph* G, const StepArgs<R, NF>& a, int wch, LoopFlags* lf, cudaStream_t st) {
    switch (wch) {
    case 4: G ? build_graph_t<R, NF, EQ, 4>(*G, a, lf) : run_stream_t<R, NF, EQ, 4>(a, lf, st); break;
    case 16: G ? build_graph_t<R, NF, EQ, 16>(*G, a, lf) : run_stream_t<R, NF, EQ, 16>(a, lf, st); break;
    default: G ? build_graph_t<R, NF, EQ, 8>(*G, a, lf) : run_stream_t<R, NF, EQ, 8>(a, lf, st); break;
    }
}

template <typename R, int NF>
void dispatch_kind(StepGraph* G, const StepArgs<R, NF>& a, int kind, int wch, LoopFlags* lf, cudaStream_t st) {
    if constexpr (NF == 1) {
        switch (kind) {
        case EQ_HEAT: dispatch_variant<R, 1, EQ_HEAT>(G, a, wch, lf, st); break;
        case EQ_ADV_EXPLICIT: dispatch_variant<R, 1, EQ_ADV_EXPLICIT>(G, a, wch, lf, st); break;
        case EQ_WAVE_REF: dispatch_variant<R, 1, EQ_WAVE_REF>(G, a, wch, lf, st); break;
        case EQ_WAVE_NEWMARK: dispatch_variant<R, 1, EQ_WAVE_NEWMARK>(G, a, wch, lf, st); break;
        case EQ_NEWMARK_INIT: dispatch_variant<R, 1, EQ_NEWMARK_INIT>(G, a, wch, lf, st); break;
        default: throw Error{FEA_ERR_UNSUPPORTED};
        }
    } else {
        switch (kind) {
        case EQ_GS_REF: dispatch_variant<R, 2, EQ_GS_REF>(G, a, wch, lf, st); break;
        case EQ_GS_CONSISTENT: dispatch_variant<R, 2, EQ_GS_CONSISTENT>(G, a, wch, lf, st); break;
        default: throw Error{FEA_ERR_UNSUPPORTED};
        }
    }
}

}  // namespace

int max_grid_blocks() {
    if (g_max_grid == 0) g_max_grid = num_sms() * 8;  // 8 resident 256-thread blocks per SM
    return g_max_grid;
}

template <typename R, int NF>
void build_step_graph(StepGraph& G, const StepArgs<R, NF>& a, int kind, int wch, LoopFlags* lf) {
    G.destroy();
    G.kind = kind;
    G.lanes = wch;
    dispatch_kind<R, NF>(&G, a, kind, wch, lf, nullptr);
}

template <typename R, int NF>
void run_steps_stream(const StepArgs<R, NF>& a, int kind, int wch, LoopFlags* lf, cudaStream_t st) {
    dispatch_kind<R, NF>(nullptr, a, kind, wch, lf, st);
}

template <typename R, int NF>
void launch_spmv_probe(const StepArgs<R, NF>& a, int wch, cudaStream_t st) {
    switch (wch) {
    case 4: k_cg_spmv<R, NF, 4><<<Grids<R, NF, 4>(a.N).spmv, kBlock, 0, st>>>(a); break;
    case 16: k_cg_spmv<R, NF, 16><<<Grids<R, NF, 16>(a.N).spmv, kBlock, 0, st>>>(a); break;
    default: k_cg_spmv<R, NF, 8><<<Grids<R, NF, 8>(a.N).spmv, kBlock, 0, st>>>(a); break;
    }
    FEA_CHECK_LAUNCH();
}

#define FEA_INST_STEP(R, NF)                                                                              \
    template void build_step_graph<R, NF>(StepGraph&, const StepArgs<R, NF>&, int, int, LoopFlags*);     \
    template void run_steps_stream<R, NF>(const StepArgs<R, NF>&, int, int, LoopFlags*, cudaStream_t);    \
    template void launch_spmv_probe<R, NF>(const StepArgs<R, NF>&, int, cudaStream_t);
FEA_INST_STEP(float, 1)
FEA_INST_STEP(float, 2)
FEA_INST_STEP(double, 1)
FEA_INST_STEP(double, 2)

}  // namespace fea
