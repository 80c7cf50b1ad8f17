// batched.cu -- many Gray-Scott instances stepped together.
//
// No reference counterpart: the reference steps one mesh.  Each instance is
// one mesh with its own (F, k, Du, Dv, dt) and follows the Gray-Scott step of
// CPUSolver.cpp:127-145 with the mass-weighted reaction, b = M (x/dt + f(x))
// for x = (u, v), solved with the single-mesh solver's CG: the Jacobi-
// preconditioned Chronopoulos-Gear iteration with float-float inner products
// and scalars, and one true-residual refinement pass per solve.
//
// Layout.  The instances' systems are stacked block-diagonally into one CSR
// matrix, each in its own solver order (a single-mesh handle built per
// instance supplies pattern, Morton ordering and FP64 matrices, then is
// released).  Every instance starts on a tile boundary (a tile is kTile rows:
// one pass of a kBlock-thread block, 32 rows per warp); the rows between
// instances are empty.  So a tile belongs to exactly one instance.
//
// Kernels walk the tiles with a grid-stride loop.  Each tile reduces its rows'
// inner products and stores them as the tile's partials; the tile that
// completes an instance last sums that instance's partials in tile order (the
// result does not depend on the schedule) and advances the instance's CG
// scalars.  An instance whose solves have converged, or that is frozen after a
// blow-up, is masked: its tiles are skipped.  A solve loop runs while any
// instance iterates; the step loop is one CUDA graph with conditional WHILE
// nodes, as in the single-mesh solver.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <type_traits>
#include <vector>

#include "cg_device.cuh"
#include "ring.cuh"
#include "tma.cuh"

namespace fea {
namespace {

constexpr int kTile = kBlock;  // rows per tile
constexpr int kNV = 6;         // partials per tile: 3 inner products x 2 fields
constexpr int kLanes = 1;      // threads per row of the once-per-step kernels (1: no shuffle reductions)

struct BPrm {
    double dt, F, k;
};

// CG and step state of one instance.
struct BInst {
    double rz[2], rr[2], pq[2], thr[2], bb[2], alpha[2], beta[2];
    float ffrz[2][2], ffalpha[2][2], ffthr[2][2];  // FP32: float-float copies
    float falpha[2], fbeta[2];                       // FP32: rounded coefficients
    int active[2], fresh[2], iters[2];
    int iter;  // iterations of the current solve
    int max_iter;
    int stop;            // frozen: its state was unstable at the start of a step
    unsigned int flags;  // FEA_STATUS_* since the last advance
    int last_iters[2];
    double last_rel[2];
    long long steps_done, total_iters;
    int prev_valid;  // xprev holds the state one step before x (the extrapolated start)
};

// Loop state shared by the instances.
struct BCtl {
    long long steps_left, steps_done;
    int iter;             // CG iteration of the running solve loop: buffer parity
    int n_next;           // (instance, field) solves left active by this phase
    int live;             // the same count after the last phase that ended
    unsigned int ticket;  // blocks finished in this phase
    int refine;
    double tol;
};

struct BFlags {
    int step, cg1, cg2, probe;
};

template <typename R>
struct BArgs {
    int64_t N;  // rows, padding included (= ntiles * kTile)
    int ntiles, ninst;
    const int32_t* rp;
    const int32_t* col;
    const FV<R, 2>* A;
    const FV<R, 2>* dinv;
    const R* M;
    FV<R, 2>* x;
    FV<R, 2>* b;
    FV<R, 2>* z;
    FV<R, 2>* p;
    FV<R, 2>* rb[2];
    FV<R, 2>* wb[2];
    FV<R, 2>* sb[2];
    const int32_t* tile_inst;  // [ntiles] instance of each tile
    const int32_t* inst_tile;  // [ninst + 1] first tile of each instance
    const BPrm* prm;           // [ninst]
    BInst* inst;               // [ninst]
    BCtl* ctl;
    double* part;           // [ntiles * kNV] tile partials
    unsigned int* iticket;  // [ninst] tiles finished per instance in this phase
    int probe;              // timing probe: every tile, no state update
    // tile-ELL copies of A (variants 0 and 1, the staged right-hand side and
    // refinement) and of M (the staged right-hand side)
    const FV<R, 2>* As;
    const R* Ms;
    const uint16_t* lcol;
    const uint32_t* lcol2;  // column pairs (TileEll::lcol2)
    const int32_t* slice_off;
    const int32_t* halo_off;
    const int32_t* halo_col;
    int hmax;
    // ring kernel (variant 14): the layout it streams (the tile-ELL copy
    // without diagonal entries; the diagonal term A_ii u'_i is the row's new
    // residual r'_i, as u' = D^-1 r'), its largest tile
    const FV<R, 2>* As_od;
    const uint16_t* lcol_od;
    const int32_t* slice_off_od;
    int emax, emax_od;         // stored entries of the largest tile of each layout
    int tcap;                  // tile-list capacity of a block
    const int32_t* inst_grp;   // [ninst + 1] first group slot of each instance
    double* gpart;             // [groups * kNV] group partials
    int32_t* act_pos;          // [ninst + 1] active-tile table (build_active_table); null: not kept
    // Extrapolated initial guess (variant 14; null otherwise): the state one
    // step back and the start 2 x_n - x_(n-1) the right-hand side formed.
    FV<R, 2>* xprev;
    FV<R, 2>* xg;
    cudaGraphConditionalHandle cond;
    int* cont;
    int use_graph;
};

// Thread 0 holds the tile's NV totals in blk.  They become the tile's
// partials; the tile that completes its instance last sums the instance's
// partials in tile order and returns true in all its threads, with the totals
// in out[] (valid in thread 0).  The instance's ticket is reset for the next
// phase.
template <int NV, typename R>
__device__ bool inst_commit(const Acc<R> (&blk)[NV], double* part, int tile, int t0, int nt, unsigned int* ticket,
                            typename Acc<R>::Packed* smem, Acc<R> (&out)[NV]) {
    using P = typename Acc<R>::Packed;
    static_assert(sizeof(P) == sizeof(double), "partials use 8-byte slots");
    P* pp = reinterpret_cast<P*>(part);
    __shared__ bool last;
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; k++) pp[(int64_t)tile * kNV + k] = blk[k].pack();
        __threadfence();
        last = atomicAdd(ticket, 1u) == (unsigned int)(nt - 1);
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    Acc<R> y[NV];
    merge_partials<NV, R>(y, pp, 1, kNV, t0, (int64_t)t0 + nt);  // tile t, value k at pp[t * kNV + k]
    block_totals<NV, R>(y, smem, out);
    if (threadIdx.x == 0) *ticket = 0u;
    return true;
}

enum { kIterKeep = 0, kIterNext = 1, kIterReset = 2 };

// Sum of v over the block, in every thread, and in `before` the sum over the
// threads below this one; wsum: kBlock / 32 ints.
__device__ __forceinline__ int block_sum_int(int v, int* wsum, int& before) {
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    int incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) wsum[wib] = incl;
    __syncthreads();
    int tot = 0;
    before = incl - v;
#pragma unroll
    for (int w = 0; w < kBlock / 32; w++) {
        const int s = wsum[w];
        tot += s;
        if (w < wib) before += s;
    }
    __syncthreads();  // wsum is reused
    return tot;
}

// The active-tile table of the ring kernel (act_pos): instance i's tiles
// start at act_pos[i] in the sequence of the active instances' tiles laid end
// to end; act_pos[ninst] is the total.  Built by the last block of a phase,
// when no block of the phase reads it any more and before the next phase can.
template <typename R>
__device__ void build_active_table(const BArgs<R>& a) {
    __shared__ int wsum[kBlock / 32];
    int base = 0;
    for (int i0 = 0; i0 < a.ninst; i0 += kBlock) {
        const int i = i0 + threadIdx.x;
        int nt = 0;
        if (i < a.ninst) {
            const volatile BInst* s = a.inst + i;
            if (s->active[0] || s->active[1]) nt = a.inst_tile[i + 1] - a.inst_tile[i];
        }
        int before;
        const int tot = block_sum_int(nt, wsum, before);
        if (i < a.ninst) a.act_pos[i] = base + before;
        base += tot;
    }
    if (threadIdx.x == 0) a.act_pos[a.ninst] = base;
}

// End of a phase: the block that finishes last publishes whether any
// (instance, field) solve is still active, resets the phase counter, moves the
// iteration counter and sets the loop condition; with the ring kernel it also
// builds the next phase's active-tile table.
template <typename R>
__device__ void phase_end(const BArgs<R>& a, int iter_mode) {
    __shared__ bool lastb;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        lastb = atomicAdd(&a.ctl->ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (threadIdx.x == 0 && lastb) {
        __threadfence();
        BCtl* c = a.ctl;
        const int n = atomicExch(&c->n_next, 0);
        c->live = n;
        c->ticket = 0u;
        if (iter_mode == kIterNext) c->iter = c->iter + 1;
        if (iter_mode == kIterReset) c->iter = 0;
        signal_loop(a, n > 0);
    }
    if (lastb && a.act_pos) {
        __threadfence();
        build_active_table(a);
    }
}

__device__ __forceinline__ void raise_inst(BInst* s, unsigned int f) {
    const unsigned int w = __reduce_or_sync(0xffffffffu, f);
    if (w && (threadIdx.x & 31) == 0) {
        atomicOr(&s->flags, w);
        __threadfence();
    }
}

template <typename R>
__device__ __forceinline__ int iter_of(const BArgs<R>& a) {
    return ((const volatile BCtl*)a.ctl)->iter;
}

// The CG loop body chains kBatchUnroll iteration kernels (each pass of a
// graph WHILE loop costs a few microseconds of relaunch).  A kernel that
// finds no solve left running is one of the extra copies of the last pass:
// it leaves the state alone and only confirms the loop's end.
constexpr int kBatchUnroll = 4;
template <typename R>
__device__ __forceinline__ bool batch_stopped(const BArgs<R>& a) {
    if (a.probe || ((const volatile BCtl*)a.ctl)->live > 0) return false;
    if (blockIdx.x == 0 && threadIdx.x == 0) signal_loop(a, false);
    return true;
}

// Timing probe of an iteration kernel: every tile iterates with its fields
// masked, so x and p are written back unchanged and only CG scratch (which
// the next step recomputes) changes; the instances' state is left alone.
template <typename R>
__device__ __forceinline__ void probe_mask(PhaseCtl<R, 2>& c) {
#pragma unroll
    for (int f = 0; f < 2; f++) {
        c.act[f] = 0;
        c.fresh[f] = false;
        c.alpha[f] = 0;
        c.beta[f] = 0;
    }
    c.need_old = true;
    c.any = false;
}

// Right-hand side b = M (x/dt + f(x)) of every unfrozen instance, initial
// residual r = b - A x (warm start), z = D^-1 r, and the set-up scalars;
// instances whose state entering the step is unstable are frozen.
template <typename R>
__global__ void __launch_bounds__(kBlock) kb_rhs(BArgs<R> a) {
    __shared__ typename Acc<R>::Packed red[32 * kNV];
    constexpr int RPW = 32 / kLanes;      // rows per warp pass
    constexpr int RPB = kBlock / kLanes;  // rows per block pass
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int sub = lane & (kLanes - 1), grp = lane / kLanes;
    for (int tile = blockIdx.x; tile < a.ntiles; tile += gridDim.x) {
        const int i = a.tile_inst[tile];
        BInst* s = a.inst + i;
        if (((const volatile BInst*)s)->stop) continue;
        const BPrm P = a.prm[i];
        const R dt = (R)P.dt, Fr = (R)P.F, Kr = (R)P.k;
        Acc<R> dots[kNV];  // |b|^2, |r|^2, r.z per field
        unsigned int flags = 0;
        for (int pass = 0; pass < kTile / RPB; pass++) {
            const int64_t row = (int64_t)tile * kTile + pass * RPB + wib * RPW + grp;
            Acc<R> bs[2], ax[2];
            const int32_t e1 = ldg(a.rp + row + 1);
            for (int32_t e = ldg(a.rp + row) + sub; e < e1; e += kLanes) {
                const int32_t c = ldg(a.col + e);
                const FV<R, 2> av = ldv(a.A + e, false);
                const FV<R, 2> xc = a.x[c];
                const R me = ldg(a.M + e);
                const R u = xc.v[0], v = xc.v[1];
                const R uvv = u * (v * v);
                const R wu = u / dt - uvv + Fr * ((R)1 - u);
                const R wv = v / dt + uvv - (Fr + Kr) * v;
                bs[0].add_prod(me, wu);
                bs[1].add_prod(me, wv);
                ax[0].add_prod(av.v[0], u);
                ax[1].add_prod(av.v[1], v);
            }
#pragma unroll
            for (int o = kLanes / 2; o > 0; o >>= 1)
#pragma unroll
                for (int f = 0; f < 2; f++) {
                    bs[f].shfl_add(o);
                    ax[f].shfl_add(o);
                }
            if (sub == 0) {
                const FV<R, 2> xr = a.x[row];
                flags |= check_value(xr.v[0]) | check_value(xr.v[1]);
                const FV<R, 2> d = ldv(a.dinv + row, false);
                FV<R, 2> bv, rv, zv;
#pragma unroll
                for (int f = 0; f < 2; f++) {
                    bv.v[f] = bs[f].rounded();
                    bs[f].sub(ax[f]);
                    rv.v[f] = bs[f].rounded();
                    zv.v[f] = d.v[f] * rv.v[f];
                    dots[f].add_prod(bv.v[f], bv.v[f]);
                    dots[2 + f].add_prod(rv.v[f], rv.v[f]);
                    dots[4 + f].add_prod(rv.v[f], zv.v[f]);
                }
                a.b[row] = bv;
                a.rb[0][row] = rv;  // the solve starts at iteration 0 (parity 0)
                a.z[row] = zv;
            }
        }
        raise_inst(s, flags);
        Acc<R> blk[kNV], tot[kNV];
        block_totals<kNV>(dots, red, blk);
        const int t0 = a.inst_tile[i], nt = a.inst_tile[i + 1] - t0;
        if (inst_commit<kNV>(blk, a.part, tile, t0, nt, a.iticket + i, red, tot) && threadIdx.x == 0) {
            volatile BInst* vs = s;
            const int stop = (atomicOr(&s->flags, 0u) & (FEA_STATUS_BLOWUP | FEA_STATUS_NONFINITE)) != 0;
            const double tol = a.ctl->tol;
            vs->stop = stop;
            vs->iter = 0;
            int nact = 0;
#pragma unroll
            for (int f = 0; f < 2; f++) nact += start_solve<R>(vs, f, stop, tol, tot[f], tot[2 + f], tot[4 + f]);
            if (nact) atomicAdd(&a.ctl->n_next, nact);
        }
    }
    phase_end(a, kIterReset);
}

// Set-up of a solve for every instance with an active field: w0 = A z,
// delta0 = z.w0, alpha0 = r0.z / delta0.  Also the SpMV timing probe.
template <typename R, int WCH>
__global__ void __launch_bounds__(kBlock, (WCH <= 4 ? 6 : 4)) kb_init(BArgs<R> a) {
    __shared__ FV<R, 2> sm[kBlock / 32][32 * WCH];
    __shared__ typename Acc<R>::Packed red[32 * kNV];
    const int wib = threadIdx.x >> 5;
    const int iter = iter_of(a);
    FV<R, 2>* w = a.wb[iter & 1];
    for (int tile = blockIdx.x; tile < a.ntiles; tile += gridDim.x) {
        const int i = a.tile_inst[tile];
        PhaseCtl<R, 2> c;
        c.set(iter, (const volatile BInst*)(a.inst + i));
        if (!c.any && !a.probe) continue;
        Acc<R> dot[2];
        init_rows<R, 2, WCH>(a.rp, a.col, a.A, a.z, w, (int64_t)tile * kTile + wib * 32, a.N, sm[wib], dot);
        Acc<R> blk[2], tot[2];
        block_totals<2>(dot, red, blk);
        const int t0 = a.inst_tile[i], nt = a.inst_tile[i + 1] - t0;
        if (inst_commit<2>(blk, a.part, tile, t0, nt, a.iticket + i, red, tot) && threadIdx.x == 0 && !a.probe) {
            volatile BInst* s = a.inst + i;
            finish_spmv<R, 2>(s, &a.inst[i].flags, c.act, tot);
            int nact = 0;
#pragma unroll
            for (int f = 0; f < 2; f++) {
                s->fresh[f] = 1;  // the first iteration takes p = u, s = w
                nact += s->active[f];
            }
            if (nact) atomicAdd(&a.ctl->n_next, nact);
        }
    }
    phase_end(a, kIterKeep);
}

// One Chronopoulos-Gear iteration of every instance that still iterates.
template <typename R, int WCH>
__global__ void __launch_bounds__(kBlock, (WCH <= 4 ? 6 : 4)) kb_iter(BArgs<R> a) {
    grid_dependency_wait();
    if (batch_stopped(a)) return;
    __shared__ FV<R, 2> sm[kBlock / 32][32 * WCH];
    __shared__ FV<R, 2> ut[kTile];
    __shared__ typename Acc<R>::Packed red[32 * kNV];
    const int wib = threadIdx.x >> 5;
    const int iter = iter_of(a), par = iter & 1;
    CgVecs<R, 2> v;
    v.rp = a.rp;
    v.col = a.col;
    v.A = a.A;
    v.dinv = a.dinv;
    v.x = a.x;
    v.p = a.p;
    v.r0 = a.rb[par];
    v.w0 = a.wb[par];
    v.s0 = a.sb[par];
    v.r1 = a.rb[par ^ 1];
    v.w1 = a.wb[par ^ 1];
    v.s1 = a.sb[par ^ 1];
    for (int tile = blockIdx.x; tile < a.ntiles; tile += gridDim.x) {
        const int i = a.tile_inst[tile];
        PhaseCtl<R, 2> c;
        c.set(iter, (const volatile BInst*)(a.inst + i));
        if (a.probe) probe_mask(c);
        if (!c.any && !a.probe) continue;
        Acc<R> dots[kNV];  // gamma', delta', |r'|^2
        cgcg_tile<R, 2, WCH>(v, c, (int64_t)tile * kTile, a.N, sm[wib], ut, dots);
        Acc<R> blk[kNV], tot[kNV];
        block_totals<kNV>(dots, red, blk);
        const int t0 = a.inst_tile[i], nt = a.inst_tile[i + 1] - t0;
        if (inst_commit<kNV>(blk, a.part, tile, t0, nt, a.iticket + i, red, tot) && threadIdx.x == 0 && !a.probe) {
            volatile BInst* s = a.inst + i;
            if (finish_cgcg<R, 2>(s, &a.inst[i].flags, c.act, tot))
                atomicAdd(&a.ctl->n_next, s->active[0] + s->active[1]);
        }
    }
    grid_launch_dependents();
    if (!a.probe) phase_end(a, kIterNext);
}

// The same two kernels on the tile-ELL layout of the stacked matrix (the
// instances' tiles are the layout's tiles): the tile's operand and halo staged
// in shared memory, two staging buffers alternating over processed tiles.
template <typename R>
__device__ __forceinline__ EllView<R, 2> bell_view(const BArgs<R>& a) {
    return EllView<R, 2>{a.As, a.lcol, a.slice_off, a.halo_off, a.halo_col};
}

template <typename R, int KPRE>
__global__ void __launch_bounds__(kBlock) kb_init_ell(BArgs<R> a) {
    extern __shared__ __align__(16) unsigned char dyn_smem[];
    FV<R, 2>* ut = reinterpret_cast<FV<R, 2>*>(dyn_smem);
    __shared__ typename Acc<R>::Packed red[32 * kNV];
    const int iter = iter_of(a);
    FV<R, 2>* w = a.wb[iter & 1];
    const EllView<R, 2> e = bell_view(a);
    const int stride = kTileRows + a.hmax;
    int buf = 0;
    for (int tile = blockIdx.x; tile < a.ntiles; tile += gridDim.x) {
        const int i = a.tile_inst[tile];
        PhaseCtl<R, 2> c;
        c.set(iter, (const volatile BInst*)(a.inst + i));
        if (!c.any && !a.probe) continue;
        Acc<R> dot[2];
        init_tile_ell<R, 2, KPRE>(e, a.z, w, tile, ell_ref(e, tile, a.ntiles), a.N, ut + buf * stride, dot);
        buf ^= 1;
        Acc<R> blk[2], tot[2];
        block_totals<2>(dot, red, blk);
        const int t0 = a.inst_tile[i], nt = a.inst_tile[i + 1] - t0;
        if (inst_commit<2>(blk, a.part, tile, t0, nt, a.iticket + i, red, tot) && threadIdx.x == 0 && !a.probe) {
            volatile BInst* s = a.inst + i;
            finish_spmv<R, 2>(s, &a.inst[i].flags, c.act, tot);
            int nact = 0;
#pragma unroll
            for (int f = 0; f < 2; f++) {
                s->fresh[f] = 1;
                nact += s->active[f];
            }
            if (nact) atomicAdd(&a.ctl->n_next, nact);
        }
    }
    phase_end(a, kIterKeep);
}

template <typename R, int KPRE>
__global__ void __launch_bounds__(kBlock) kb_iter_ell(BArgs<R> a) {
    grid_dependency_wait();
    if (batch_stopped(a)) return;
    extern __shared__ __align__(16) unsigned char dyn_smem[];
    FV<R, 2>* ut = reinterpret_cast<FV<R, 2>*>(dyn_smem);
    __shared__ typename Acc<R>::Packed red[32 * kNV];
    const int iter = iter_of(a), par = iter & 1;
    CgVecs<R, 2> v;
    v.rp = a.rp;
    v.col = a.col;
    v.A = a.A;
    v.dinv = a.dinv;
    v.x = a.x;
    v.p = a.p;
    v.r0 = a.rb[par];
    v.w0 = a.wb[par];
    v.s0 = a.sb[par];
    v.r1 = a.rb[par ^ 1];
    v.w1 = a.wb[par ^ 1];
    v.s1 = a.sb[par ^ 1];
    const EllView<R, 2> e = bell_view(a);
    const int stride = kTileRows + a.hmax;
    int buf = 0;
    for (int tile = blockIdx.x; tile < a.ntiles; tile += gridDim.x) {
        const int i = a.tile_inst[tile];
        PhaseCtl<R, 2> c;
        c.set(iter, (const volatile BInst*)(a.inst + i));
        if (a.probe) probe_mask(c);
        if (!c.any && !a.probe) continue;
        Acc<R> dots[kNV];
        cgcg_tile_ell<R, 2, KPRE>(v, e, c, tile, ell_ref(e, tile, a.ntiles), a.N, ut + buf * stride, dots);
        buf ^= 1;
        Acc<R> blk[kNV], tot[kNV];
        block_totals<kNV>(dots, red, blk);
        const int t0 = a.inst_tile[i], nt = a.inst_tile[i + 1] - t0;
        if (inst_commit<kNV>(blk, a.part, tile, t0, nt, a.iticket + i, red, tot) && threadIdx.x == 0 && !a.probe) {
            volatile BInst* s = a.inst + i;
            if (finish_cgcg<R, 2>(s, &a.inst[i].flags, c.act, tot))
                atomicAdd(&a.ctl->n_next, s->active[0] + s->active[1]);
        }
    }
    grid_launch_dependents();
    if (!a.probe) phase_end(a, kIterNext);
}

// After the right-hand side, with the extrapolated start: every unfrozen
// instance's state moves to xprev and the start 2 x_n - x_(n-1) the
// right-hand side formed (x_n itself where the instance had no history)
// becomes x, the start of its solves; its history is then valid.
template <typename R>
__global__ void __launch_bounds__(kBlock) kb_guess_move(BArgs<R> a) {
    // one tile per block pass, one row per thread; an instance's stop flag is
    // fixed while this kernel runs (no other kernel runs beside it)
    for (int tile = blockIdx.x; tile < a.ntiles; tile += gridDim.x) {
        if (a.inst[a.tile_inst[tile]].stop) continue;
        const int64_t r = (int64_t)tile * kTile + threadIdx.x;
        const FV<R, 2> xn = a.x[r], x0 = a.xg[r];
        a.xprev[r] = xn;
        a.x[r] = x0;
    }
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.ninst; i += gridDim.x * blockDim.x)
        if (!a.inst[i].stop) a.inst[i].prev_valid = 1;
}

// Histories of the extrapolated start cleared (instance `only`, or all when
// it is negative).
__global__ void kb_clear_history(BInst* inst, int n, int only) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        if (only < 0 || i == only) inst[i].prev_valid = 0;
}

// ---- variant 14: the ring pipeline -------------------------------------------------
//
// The single-mesh ring kernel's tile pipeline over the batch's tiles: thread
// 0 moves each tile's operator entries and 16-bit local columns with
// cp.async.bulk into a ring of S shared-memory stages, S - 1 tiles ahead of
// the product; the threads load their rows' values and their halo slot's
// operands one tile ahead; one block barrier per tile orders the staged
// vector.  The CG iteration, the right-hand side, the set-up product and the
// refinement all run on it (kb_ring's phases).
//
// Work.  Each instance's tiles are cut into groups of kGroupTiles consecutive
// tiles (an instance's last group may be shorter).  At the start of a launch
// every block lays the instances' tiles end to end (for the iteration only
// the active instances', from the table the previous phase's last block
// built) and takes the groups that start in its equal share of that
// sequence, so the blocks get equal work however many instances have
// converged.  The threads accumulate a group's inner products over its
// tiles; at the group's last tile the block reduces them into the group's
// partials, and the block that completes an instance's last group sums the
// instance's group partials in group order and advances its state.  The
// groups are fixed per instance, so an instance's results depend neither on
// the other instances nor on the schedule.
constexpr int kGroupTiles = 8;

// Phases of a batched solve that run on the ring pipeline: the CG iteration,
// the right-hand side with the initial residual, the set-up product of a
// solve, and the true-residual refinement.
enum { kPhIter = 0, kPhRhs = 1, kPhInit = 2, kPhRefine = 3 };

// An instance with groups in the block's share.
struct BRingInst {
    int inst, nt, t0, g0, ng;  // instance, tiles, first tile, first group slot, groups
    int u0, u1;                // its groups in the share
};

// What a phase needs of such an instance, read at the start of the launch:
// the CG phase control (iteration, set-up), the step's parameters (right-hand
// side), the refinement's decisions.
template <typename R>
struct BRingCtl {
    PhaseCtl<R, 2> c;
    R dt, F, k;
    int refine, zero[2];
    int extrap;  // right-hand side: the solve starts from 2 x_n - x_(n-1)
};

// One stage of the ring: a tile's operator entries, its entries of M (the
// right-hand side), then its local columns.
struct BStage {
    size_t A, M, L, bytes;
    __host__ __device__ BStage(int emax, size_t fv, size_t mv) {
        auto al = [](size_t x) { return (x + 127) & ~(size_t)127; };
        A = 0;
        M = al(fv * (size_t)emax);
        L = al(M + mv * (size_t)emax);
        bytes = al(L + 2 * (size_t)emax);
    }
};

// Dynamic shared memory of kb_ring: the ring, two staging buffers (u' of the
// tile and its halo; x and the nodal reaction for the right-hand side), then
// the block's instances, their controls and its tile list (tile, index of its
// instance in the block's list, group slot), each for up to tcap tiles.
template <typename R>
struct BRingLayout {
    size_t ubuf, ov, ctl, tl, tq, tg, total;
    __host__ __device__ BRingLayout(int emax, int hmax, int tcap, int stages, int ph) {
        auto al = [](size_t x) { return (x + 127) & ~(size_t)127; };
        const size_t mv = ph == kPhRhs ? sizeof(R) : 0;
        ubuf = al((size_t)stages * BStage(emax, sizeof(FV<R, 2>), mv).bytes);
        const size_t per = (size_t)(ph == kPhRhs ? 2 : 1) * sizeof(FV<R, 2>) * (size_t)(kTileRows + hmax);
        ov = al(ubuf + 2 * per);
        ctl = al(ov + sizeof(BRingInst) * (size_t)tcap);
        tl = al(ctl + sizeof(BRingCtl<R>) * (size_t)tcap);
        tq = al(tl + sizeof(int32_t) * (size_t)tcap);
        tg = al(tq + sizeof(int32_t) * (size_t)tcap);
        total = al(tg + sizeof(int32_t) * (size_t)tcap);
    }
};

// The nodal reaction of the mass-weighted Gray-Scott right-hand side,
// b = M w(x) (CPUSolver.cpp:134,137 with the mass weight).
template <typename R>
__device__ __forceinline__ FV<R, 2> gs_reaction(const FV<R, 2>& x, R dt, R F, R k) {
    const R u = x.v[0], v = x.v[1];
    const R uvv = u * (v * v);
    FV<R, 2> w;
    w.v[0] = u / dt - uvv + F * ((R)1 - u);
    w.v[1] = v / dt + uvv - (F + k) * v;
    return w;
}

// One phase over every participating instance on the ring pipeline.  The
// iteration streams the diagonal-free layout when it exists; the other phases
// stream the full one (the right-hand side also M's entries).  Per phase:
//   iteration   rows r, w, s, D^-1, x, p; stages u'; w' = A u'; finish_cgcg
//   rhs         rows x, D^-1; stages x and w(x); b = M w(x), r0 = b - A x
//               in float-float; start_solve (every unfrozen instance)
//   init        rows z; stages z; w0 = A z; finish_spmv (active instances)
//   refine      rows x, b, D^-1; stages x; r = b - A x in float-float;
//               the restart decision (instances to refine or to zero)
// The iteration shares out the active instances' tiles (the table its
// previous phase built); the others share out every instance's tiles and
// skip the groups of instances that do not take part, whose state no commit
// of the phase changes before those groups are read.
template <typename R, int S, int PH>
__global__ void __launch_bounds__(kBlock, 2) kb_ring(BArgs<R> a) {
    using V = FV<R, 2>;
    using Ctl = BRingCtl<R>;
    static_assert(S >= 2 && S <= 8, "ring depth");
    constexpr bool kIt = PH == kPhIter, kRhs = PH == kPhRhs, kIni = PH == kPhInit, kRef = PH == kPhRefine;
    constexpr int NVP = kIni ? 2 : kRef ? 4 : kNV;  // partials per group
    extern __shared__ __align__(16) unsigned char dyn_smem[];  // bulk copies need 16-byte destinations
    __shared__ __align__(8) uint64_t bars[S];
    __shared__ typename Acc<R>::Packed red[32 * kNV];
    __shared__ int s_nov, s_ntl;
    const bool od = kIt && a.As_od != nullptr;  // the streamed layout lacks the diagonal entries
    const V* const Aop = od ? a.As_od : a.As;
    const uint16_t* const lop = od ? a.lcol_od : a.lcol;
    const int32_t* const soff = od ? a.slice_off_od : a.slice_off;
    const int emx = od ? a.emax_od : a.emax;
    const BRingLayout<R> Lay(emx, a.hmax, a.tcap, S, PH);
    const BStage L(emx, sizeof(V), kRhs ? sizeof(R) : 0);
    unsigned char* const ring = dyn_smem;
    V* const ubuf = reinterpret_cast<V*>(dyn_smem + Lay.ubuf);
    BRingInst* const ov = reinterpret_cast<BRingInst*>(dyn_smem + Lay.ov);
    Ctl* const ovc = reinterpret_cast<Ctl*>(dyn_smem + Lay.ctl);
    int32_t* const tl = reinterpret_cast<int32_t*>(dyn_smem + Lay.tl);
    int32_t* const tq = reinterpret_cast<int32_t*>(dyn_smem + Lay.tq);
    int32_t* const tg = reinterpret_cast<int32_t*>(dyn_smem + Lay.tg);
    const int hstride = kTileRows + a.hmax;             // one staged vector: the tile's rows, then its halo
    const int bstride = (kRhs ? 2 : 1) * hstride;       // one staging buffer
    const int t = threadIdx.x, lane = t & 31, wib = t >> 5, j = halo_slot(t);
    const int ntiles = a.ntiles, tcap = a.tcap;
    if (t == 0) {
        for (int b = 0; b < S; b++) mbar_init(&bars[b], 1);
        mbar_fence_init();
        s_nov = 0;
    }
    grid_dependency_wait();
    if constexpr (kIt)
        if (batch_stopped(a)) return;
    const int iter = iter_of(a), par = iter & 1;
    const int refine_on = kRef ? a.ctl->refine : 0;
    // the tiles laid end to end (the active instances' for the iteration, from
    // the table the previous phase's last block built; every instance's
    // otherwise); this block's share [lo, hi) and the taking part instances
    // with a group starting in it
    const int32_t* pos_of = (kIt && !a.probe) ? a.act_pos : a.inst_tile;
    const int T = pos_of[a.ninst];
    const int lo = (int)((int64_t)T * blockIdx.x / gridDim.x);
    const int hi = (int)((int64_t)T * (blockIdx.x + 1) / gridDim.x);
    for (int i = t; i < a.ninst; i += kBlock) {
        const int pos = pos_of[i], nt = pos_of[i + 1] - pos;
        if (nt > 0 && pos + nt > lo && pos < hi) {
            const int ng = (nt + kGroupTiles - 1) / kGroupTiles;
            const int u0 = lo > pos ? (lo - pos + kGroupTiles - 1) / kGroupTiles : 0;
            const int u1 = min(ng, (hi - pos + kGroupTiles - 1) / kGroupTiles);
            if (u0 < u1) {
                const volatile BInst* s = a.inst + i;
                Ctl cc{};  // the members this phase does not set stay zero
                bool take = true;
                if constexpr (kIt || kIni) {
                    cc.c.set(iter, s);
                    if (a.probe) probe_mask(cc.c);
                    if constexpr (kIni) take = cc.c.any;
                } else if constexpr (kRhs) {
                    take = !s->stop;
                    cc.extrap = a.xg != nullptr && s->prev_valid != 0;
                    const BPrm P = a.prm[i];
                    cc.dt = (R)P.dt;
                    cc.F = (R)P.F;
                    cc.k = (R)P.k;
                } else {
                    const int stop = s->stop;
                    cc.refine = refine_on && s->iter < s->max_iter && !stop;
#pragma unroll
                    for (int f = 0; f < 2; f++) cc.zero[f] = !stop && !(s->bb[f] > 0.0);
                    take = cc.refine || cc.zero[0] || cc.zero[1];
                }
                if (take) {
                    const int q = atomicAdd(&s_nov, 1);
                    if (q < tcap) {
                        ov[q] = BRingInst{i, nt, a.inst_tile[i], a.inst_grp[i], ng, u0, u1};
                        ovc[q] = cc;
                    }
                }
            }
        }
    }
    __syncthreads();
    if (t == 0) {  // the block's tile list
        const int nov = min(s_nov, tcap);
        int k = 0;
        for (int q = 0; q < nov; q++) {
            const BRingInst o = ov[q];
            for (int u = o.u0; u < o.u1; u++) {
                const int x1 = min((u + 1) * kGroupTiles, o.nt);
                for (int x = u * kGroupTiles; x < x1; x++, k++)
                    if (k < tcap) {
                        tl[k] = o.t0 + x;
                        tq[k] = q;
                        tg[k] = o.g0 + u;
                    }
            }
        }
        s_ntl = k;
        if (k > tcap || s_nov > tcap) {  // the host sizes tcap for the largest share: not reached
            atomicOr(&a.inst[0].flags, FEA_STATUS_BREAKDOWN);
            s_ntl = 0;
        }
    }
    __syncthreads();
    const int ntl = s_ntl;
    auto tile_at = [&](int k) { return k < ntl ? tl[k] : ntiles; };
    auto halo_head = [&](int tile, int32_t& h0, int32_t& cnt) {
        h0 = cnt = 0;
        if (tile < ntiles) {
            h0 = a.halo_off[tile];
            cnt = a.halo_off[tile + 1] - h0;
        }
    };
    auto slice_ref = [&](int tile, int32_t& sb, int32_t& sw) {
        sb = sw = 0;
        if (tile < ntiles) {
            const int sl = tile * (kTileRows / 32) + wib;
            const int32_t s0 = soff[sl];
            sb = s0 - soff[tile * (kTileRows / 32)];
            sw = (soff[sl + 1] - s0) >> 5;
        }
    };
    auto tile_range = [&](int tile, int32_t& e0, int32_t& e1) {
        e0 = e1 = 0;
        if (tile < ntiles) {
            e0 = soff[tile * (kTileRows / 32)];
            e1 = soff[(tile + 1) * (kTileRows / 32)];
        }
    };
    auto stage_of = [&](int b) { return ring + (size_t)b * L.bytes; };
    auto issue = [&](int b, int32_t e0, int32_t e1) {
        uint64_t* bar = &bars[b];
        const uint32_t n = (uint32_t)(e1 - e0);  // a multiple of 32 entries
        if (n == 0) {
            mbar_arrive(bar);
            return;
        }
        mbar_arrive_expect_tx(bar, n * (uint32_t)(sizeof(V) + (kRhs ? sizeof(R) : 0) + 2));
        const uint64_t pol = l2_evict_first_policy();
        bulk_g2s_hint(stage_of(b) + L.A, Aop + e0, n * (uint32_t)sizeof(V), bar, pol);
        if constexpr (kRhs) bulk_g2s_hint(stage_of(b) + L.M, a.Ms + e0, n * (uint32_t)sizeof(R), bar, pol);
        bulk_g2s_hint(stage_of(b) + L.L, lop + e0, 2 * n, bar, pol);
    };
    uint32_t armed = 0;  // thread 0: bit b set while stage b has copies in flight
    int32_t re0 = 0, re1 = 0;
    if (t == 0) {
        for (int b = 0; b < S && b < ntl; b++) {
            int32_t e0, e1;
            tile_range(tl[b], e0, e1);
            issue(b, e0, e1);
            armed |= 1u << b;
        }
        tile_range(tile_at(S), re0, re1);
    }
    int32_t sb, sw, sbn, swn;
    slice_ref(tile_at(0), sb, sw);
    slice_ref(tile_at(1), sbn, swn);
    int32_t h0c, hcc, h0n, hcn, hh0, hhc;
    halo_head(tile_at(0), h0c, hcc);
    halo_head(tile_at(1), h0n, hcn);
    halo_head(tile_at(2), hh0, hhc);
    const int32_t fcol = j < hcc ? a.halo_col[h0c + j] : -1;
    int32_t hcoln = j < hcn ? a.halo_col[h0n + j] : -1;
    CgVecs<R, 2> v;
    v.rp = a.rp;
    v.col = a.col;
    v.A = a.A;
    v.dinv = a.dinv;
    v.x = a.x;
    v.p = a.p;
    v.r0 = a.rb[par];
    v.w0 = a.wb[par];
    v.s0 = a.sb[par];
    v.r1 = a.rb[par ^ 1];
    v.w1 = a.wb[par ^ 1];
    v.s1 = a.sb[par ^ 1];
    // the halo slot's staged vector: z (set-up) or x (right-hand side, refinement)
    const V* const hsrc = kIni ? a.z : a.x;
    // row values of the next tile: iteration r, w, s, D^-1, x, p; right-hand
    // side x, D^-1 and, with the extrapolated start, x_(n-1) (in cr); set-up z
    // (in cx); refinement x, b (in cw), D^-1
    const bool xp_on = kRhs && a.xg != nullptr;
    auto load_rows = [&](int tile, V& cr, V& cw, V& cs, V& cd, V& cx, V& cp) {
        const uint64_t pol_keep = l2_evict_last_policy();
        const int row = tile * kTileRows + t;  // every vector holds whole tiles
        if constexpr (kIt) {
            cr = ld_keep(v.r0 + row, pol_keep);
            cw = ld_keep(v.w0 + row, pol_keep);
            cs = ld_keep(v.s0 + row, pol_keep);
            cp = ld_keep(v.p + row, pol_keep);
        }
        if constexpr (kRhs)
            if (xp_on) cr = ld_keep(a.xprev + row, pol_keep);
        if constexpr (kRef) cw = ld_keep(a.b + row, pol_keep);
        if constexpr (!kIni) cd = ld_keep(v.dinv + row, pol_keep);
        cx = ld_keep((kIni ? a.z : v.x) + row, pol_keep);
    };
    auto load_halo = [&](int32_t col, V& hr, V& hw, V& hs, V& hd) {
        const uint64_t pol_keep = l2_evict_last_policy();
        if constexpr (kIt) {
            hr = ld_keep(v.r0 + col, pol_keep);
            hw = ld_keep(v.w0 + col, pol_keep);
            hs = ld_keep(v.s0 + col, pol_keep);
            hd = ld_keep(v.dinv + col, pol_keep);
        } else {
            hr = ld_keep(hsrc + col, pol_keep);
            if constexpr (kRhs)
                if (xp_on) hw = ld_keep(a.xprev + col, pol_keep);
        }
    };
    // the solve's start at an unknown: 2 x_n - x_(n-1) (one rounding; 2 x is
    // exact) with the extrapolated start, else x_n
    auto start_at = [&](const V& xn, const V& xp, bool extrap) {
        V g = xn;
        if (extrap)
#pragma unroll
            for (int f = 0; f < 2; f++) g.v[f] = fmar((R)2, xn.v[f], -xp.v[f]);
        return g;
    };
    V cr, cw, cs, cd, cx, cp, hr, hw, hs, hd;
    if (ntl > 0) load_rows(tl[0], cr, cw, cs, cd, cx, cp);
    if (fcol >= 0) load_halo(fcol, hr, hw, hs, hd);
    Ctl cc{};
    int cq = -1;
    // the iteration sums its rows' inner products per thread in R (fused
    // multiply-adds over at most a group's tiles), the other phases in the
    // handle's accumulators; the block and instance totals use the latter
    using DA = std::conditional_t<kIt, R, Acc<R>>;
    DA dots[NVP];
    if constexpr (kIt)
#pragma unroll
        for (int f = 0; f < NVP; f++) dots[f] = 0;
    unsigned int flags = 0;  // right-hand side: the instability test of the group's rows
    uint32_t phases = 0u;    // bit b: parity of stage b's next phase
    int bad_inst = -1;       // instance of a tile whose stage wait expired
    int buf = 0, b = 0;
    for (int k = 0; k < ntl; k++) {
        const int tile = tl[k], q = tq[k];
        if (q != cq) {
            cc = ovc[q];
            cq = q;
        }
        const PhaseCtl<R, 2>& c = cc.c;
        V* const ut = ubuf + buf * bstride;  // staged: u', z or x
        V* const uw = ut + hstride;          // right-hand side: the nodal reaction
        const int row = tile * kTileRows + t;
        V un, wn;  // iteration: u' and the product's start (the diagonal term in the diagonal-free layout)
        V x0r = cx;  // right-hand side: the solve's start at this row
#pragma unroll
        for (int f = 0; f < 2; f++) un.v[f] = wn.v[f] = 0;
        if constexpr (kIt) {
            V sn, rn;
            cg_advance(c, cr, cw, c.need_old ? cs : cw, cd, sn, rn, un);
            if (od) wn = rn;
#pragma unroll
            for (int f = 0; f < 2; f++) {
                if (c.act[f]) {
                    const R ui = cd.v[f] * cr.v[f];
                    cp.v[f] = c.fresh[f] ? ui : fmar(c.beta[f], cp.v[f], ui);
                    cx.v[f] = fmar(c.alpha[f], cp.v[f], cx.v[f]);
                }
                dots[f] = fmar(rn.v[f], un.v[f], dots[f]);
                dots[4 + f] = fmar(rn.v[f], rn.v[f], dots[4 + f]);
            }
            v.x[row] = cx;
            v.p[row] = cp;
            v.r1[row] = rn;
            v.s1[row] = sn;
            ut[t] = un;
        } else if constexpr (kRhs) {
            x0r = start_at(cx, cr, cc.extrap);
            ut[t] = x0r;                                 // A x0 with the solve's start
            uw[t] = gs_reaction(cx, cc.dt, cc.F, cc.k);  // b from x_n
            flags |= check_value(cx.v[0]) | check_value(cx.v[1]);
        } else {
            ut[t] = cx;
        }
        // the tile's own values this thread keeps past the loads of the next tile
        const V xr = cx, dr = cd, br = cw;
        const int nt = tile_at(k + 1);
        if (nt < ntiles) load_rows(nt, cr, cw, cs, cd, cx, cp);
        if (j < hcc) {
            if constexpr (kIt) {
                V sn, rn, u2;
                cg_advance(c, hr, hw, c.need_old ? hs : hw, hd, sn, rn, u2);
                ut[kTileRows + j] = u2;
            } else if constexpr (kRhs) {
                ut[kTileRows + j] = start_at(hr, hw, cc.extrap);
                uw[kTileRows + j] = gs_reaction(hr, cc.dt, cc.F, cc.k);
            } else {
                ut[kTileRows + j] = hr;
            }
        }
        if (hcoln >= 0) load_halo(hcoln, hr, hw, hs, hd);
        for (int32_t h = kBlock + t; h < hcc; h += kBlock) {
            const int32_t col = a.halo_col[h0c + h];
            if constexpr (kIt) {
                ut[kTileRows + h] = cg_u_at(v, c, col);
            } else if constexpr (kRhs) {
                const V g = hsrc[col];
                ut[kTileRows + h] = start_at(g, xp_on ? a.xprev[col] : g, cc.extrap);
                uw[kTileRows + h] = gs_reaction(g, cc.dt, cc.F, cc.k);
            } else {
                ut[kTileRows + h] = hsrc[col];
            }
        }
        __syncthreads();
        if (t == 0 && k > 0) {  // refill the previous tile's stage, S - 1 tiles ahead
            const int bp = b == 0 ? S - 1 : b - 1;
            if (k + S - 1 < ntl) {
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                issue(bp, re0, re1);
                armed |= 1u << bp;
            }
            tile_range(tile_at(k + S), re0, re1);
        }
        h0c = h0n;
        hcc = hcn;
        hcoln = j < hhc ? a.halo_col[hh0 + j] : -1;
        h0n = hh0;
        hcn = hhc;
        halo_head(tile_at(k + 3), hh0, hhc);
        int32_t sb2, sw2;
        slice_ref(tile_at(k + 2), sb2, sw2);
        // the product from the stage
        const bool got = mbar_wait(&bars[b], (phases >> b) & 1u);
        phases ^= 1u << b;
        if (!got) bad_inst = ov[q].inst;
        if (t == 0 && got) armed &= ~(1u << b);
        const V* As = reinterpret_cast<const V*>(stage_of(b) + L.A) + sb + lane;
        const uint16_t* Ls = reinterpret_cast<const uint16_t*>(stage_of(b) + L.L) + sb + lane;
        if constexpr (kIt || kIni) {
#pragma unroll 4
            for (int kk = 0; kk < sw; kk++) {
                const V av = As[32 * kk];
                const V g = ut[Ls[32 * kk]];
#pragma unroll
                for (int f = 0; f < 2; f++) wn.v[f] = fmar(av.v[f], g.v[f], wn.v[f]);
            }
            if constexpr (kIt) {
                v.w1[row] = wn;
#pragma unroll
                for (int f = 0; f < 2; f++) dots[2 + f] = fmar(wn.v[f], un.v[f], dots[2 + f]);
            } else {
                a.wb[par][row] = wn;
#pragma unroll
                for (int f = 0; f < 2; f++) dots[f].add_prod(xr.v[f], wn.v[f]);  // z.w0
            }
        } else if constexpr (kRhs) {
            const R* Ms = reinterpret_cast<const R*>(stage_of(b) + L.M) + sb + lane;
            Acc<R> bs[2], ax[2];
#pragma unroll 4
            for (int kk = 0; kk < sw; kk++) {
                const V av = As[32 * kk];
                const R me = Ms[32 * kk];
                const int l = Ls[32 * kk];
                const V w = uw[l], x = ut[l];
                bs[0].add_prod(me, w.v[0]);
                bs[1].add_prod(me, w.v[1]);
                ax[0].add_prod(av.v[0], x.v[0]);
                ax[1].add_prod(av.v[1], x.v[1]);
            }
            V bv, rv, zv;
#pragma unroll
            for (int f = 0; f < 2; f++) {
                bv.v[f] = bs[f].rounded();
                bs[f].sub(ax[f]);
                rv.v[f] = bs[f].rounded();
                zv.v[f] = dr.v[f] * rv.v[f];
                dots[f].add_prod(bv.v[f], bv.v[f]);
                dots[2 + f].add_prod(rv.v[f], rv.v[f]);
                dots[4 + f].add_prod(rv.v[f], zv.v[f]);
            }
            a.b[row] = bv;
            a.rb[0][row] = rv;  // the solve starts at iteration 0 (parity 0)
            a.z[row] = zv;
            if (xp_on) a.xg[row] = x0r;  // kb_guess_move makes it x
        } else {  // refinement
            Acc<R> ax[2];
            if (cc.refine) {
#pragma unroll 4
                for (int kk = 0; kk < sw; kk++) {
                    const V av = As[32 * kk];
                    const V x = ut[Ls[32 * kk]];
#pragma unroll
                    for (int f = 0; f < 2; f++) ax[f].add_prod(av.v[f], x.v[f]);
                }
            }
            if (cc.zero[0] || cc.zero[1]) {  // only zero fields change: their products go unused
                V xz = xr;
#pragma unroll
                for (int f = 0; f < 2; f++)
                    if (cc.zero[f]) xz.v[f] = 0;
                a.x[row] = xz;
            }
            if (cc.refine) {
                V rv, zv;
#pragma unroll
                for (int f = 0; f < 2; f++) {
                    Acc<R> tr;
                    tr.add(br.v[f]);
                    tr.sub(ax[f]);
                    rv.v[f] = tr.rounded();
                    zv.v[f] = dr.v[f] * rv.v[f];
                    dots[f].add_prod(rv.v[f], rv.v[f]);
                    dots[2 + f].add_prod(rv.v[f], zv.v[f]);
                }
                a.rb[par][row] = rv;  // the restart continues the iteration parity
                a.z[row] = zv;
            }
        }
        sb = sbn;
        sw = swn;
        sbn = sb2;
        swn = sw2;
        buf ^= 1;
        b = b + 1 == S ? 0 : b + 1;
        if (k + 1 == ntl || tg[k + 1] != tg[k]) {  // the group's last tile: its partials
            const BRingInst o = ov[q];
            BInst* const s = a.inst + o.inst;
            if constexpr (kRhs) {
                raise_inst(s, flags);
                flags = 0;
            }
            Acc<R> blk[NVP], tot[NVP], acc[NVP];
#pragma unroll
            for (int f = 0; f < NVP; f++) {
                if constexpr (kIt) acc[f].add(dots[f]);
                else acc[f] = dots[f];
            }
            block_totals<NVP>(acc, red, blk);
            if (inst_commit<NVP>(blk, a.gpart, tg[k], o.g0, o.ng, a.iticket + o.inst, red, tot) && t == 0 &&
                !a.probe) {
                volatile BInst* vs = s;
                if constexpr (kIt) {
                    if (finish_cgcg<R, 2>(vs, &s->flags, c.act, tot))
                        atomicAdd(&a.ctl->n_next, vs->active[0] + vs->active[1]);
                } else if constexpr (kRhs) {
                    const int stop = (atomicOr(&s->flags, 0u) & (FEA_STATUS_BLOWUP | FEA_STATUS_NONFINITE)) != 0;
                    const double tol = a.ctl->tol;
                    vs->stop = stop;
                    vs->iter = 0;
                    int nact = 0;
#pragma unroll
                    for (int f = 0; f < 2; f++)
                        nact += start_solve<R>(vs, f, stop, tol, tot[f], tot[2 + f], tot[4 + f]);
                    if (nact) atomicAdd(&a.ctl->n_next, nact);
                } else if constexpr (kIni) {
                    finish_spmv<R, 2>(vs, &s->flags, c.act, tot);
                    int nact = 0;
#pragma unroll
                    for (int f = 0; f < 2; f++) {
                        vs->fresh[f] = 1;  // the first iteration takes p = u, s = w
                        nact += vs->active[f];
                    }
                    if (nact) atomicAdd(&a.ctl->n_next, nact);
                } else {
                    int nact = 0;
#pragma unroll
                    for (int f = 0; f < 2; f++) {
                        vs->active[f] = 0;
                        vs->fresh[f] = 1;
                        if (cc.refine && !cc.zero[f] && vs->bb[f] > 0.0) {
                            const double rr = tot[f].value();
                            vs->rr[f] = rr;
                            if (rr >= vs->thr[f]) {
                                set_gamma(vs, f, tot[2 + f]);
                                vs->active[f] = 1;
                                nact++;
                            }
                        }
                    }
                    if (nact) atomicAdd(&a.ctl->n_next, nact);
                }
            }
#pragma unroll
            for (int f = 0; f < NVP; f++) dots[f] = DA();
        }
    }
    grid_launch_dependents();
    if (__syncthreads_or(bad_inst >= 0)) {
        if (bad_inst >= 0) atomicOr(&a.inst[bad_inst].flags, FEA_STATUS_BREAKDOWN);
        if (t == 0)
            for (int q2 = 0; q2 < S; q2++)  // copies still in flight land before the block leaves
                if (armed & (1u << q2)) mbar_wait(&bars[q2], (phases >> q2) & 1u);
    }
    if constexpr (kIt) {
        if (!a.probe) phase_end(a, kIterNext);
    } else {
        phase_end(a, kRhs ? kIterReset : kIterKeep);
    }
}

// ---- right-hand side and refinement on the tile-ELL layout ------------------------
//
// kb_rhs and kb_refine multiply by the whole operator once per step.  These
// forms stage the tile's x (and for the right-hand side the nodal reaction
// w(x), evaluated once per unknown instead of once per stored entry) for the
// tile's rows and its halo in shared memory, then each warp reads its 32-row
// slice of the tile-ELL copies of A and M with coalesced loads and gathers
// from shared memory.  Entries keep their CSR order within a row and padding
// entries hold 0, so the sums and their rounding are those of the CSR forms.

// x of the tile's rows and halo in g[0 .. kTileRows + halo); with `react`,
// the nodal reaction w(x) in gw[] too.  Every thread of the block calls it;
// a barrier follows in the caller.
template <typename R, typename F>
__device__ __forceinline__ void stage_tile_x(const BArgs<R>& a, int tile, FV<R, 2>* gx, FV<R, 2>* gw, F react) {
    const int t = threadIdx.x;
    const FV<R, 2> xr = a.x[(int64_t)tile * kTileRows + t];
    gx[t] = xr;
    if (gw) gw[t] = react(xr);
    const int32_t h0 = a.halo_off[tile], hn = a.halo_off[tile + 1] - h0;
    for (int h = t; h < hn; h += kBlock) {
        const FV<R, 2> xc = a.x[a.halo_col[h0 + h]];
        gx[kTileRows + h] = xc;
        if (gw) gw[kTileRows + h] = react(xc);
    }
}

// Right-hand side b = M w(x) and r0 = b - A x (warm start), z = D^-1 r0 and
// the set-up scalars of every unfrozen instance, as kb_rhs.
template <typename R>
__global__ void __launch_bounds__(kBlock) kb_rhs_ell(BArgs<R> a) {
    using V = FV<R, 2>;
    extern __shared__ __align__(16) unsigned char dyn_smem[];
    V* const gx = reinterpret_cast<V*>(dyn_smem);
    V* const gw = gx + (kTileRows + a.hmax);
    __shared__ typename Acc<R>::Packed red[32 * kNV];
    const int t = threadIdx.x, lane = t & 31, wib = t >> 5;
    for (int tile = blockIdx.x; tile < a.ntiles; tile += gridDim.x) {
        const int i = a.tile_inst[tile];
        BInst* s = a.inst + i;
        if (((const volatile BInst*)s)->stop) continue;
        const BPrm P = a.prm[i];
        const R dt = (R)P.dt, Fr = (R)P.F, Kr = (R)P.k;
        auto react = [&](const V& x) {  // CPUSolver.cpp:134,137 with the mass weight
            const R u = x.v[0], v = x.v[1];
            const R uvv = u * (v * v);
            V w;
            w.v[0] = u / dt - uvv + Fr * ((R)1 - u);
            w.v[1] = v / dt + uvv - (Fr + Kr) * v;
            return w;
        };
        stage_tile_x(a, tile, gx, gw, react);
        const int sl = tile * (kTileRows / 32) + wib;
        const int32_t sb = a.slice_off[sl], sw = (a.slice_off[sl + 1] - sb) >> 5;
        __syncthreads();
        Acc<R> bs[2], ax[2];
#pragma unroll 4
        for (int32_t k = 0; k < sw; k++) {
            const int32_t e = sb + 32 * k + lane;
            const V av = ldv(a.As + e, false);
            const R me = ldg(a.Ms + e);
            const int l = a.lcol[e];
            const V w = gw[l], x = gx[l];
            bs[0].add_prod(me, w.v[0]);
            bs[1].add_prod(me, w.v[1]);
            ax[0].add_prod(av.v[0], x.v[0]);
            ax[1].add_prod(av.v[1], x.v[1]);
        }
        const int64_t row = (int64_t)tile * kTileRows + t;
        const V xr = gx[t];
        const unsigned int flags = check_value(xr.v[0]) | check_value(xr.v[1]);
        const V d = ldv(a.dinv + row, false);
        Acc<R> dots[kNV];  // |b|^2, |r|^2, r.z per field
        V bv, rv, zv;
#pragma unroll
        for (int f = 0; f < 2; f++) {
            bv.v[f] = bs[f].rounded();
            bs[f].sub(ax[f]);
            rv.v[f] = bs[f].rounded();
            zv.v[f] = d.v[f] * rv.v[f];
            dots[f].add_prod(bv.v[f], bv.v[f]);
            dots[2 + f].add_prod(rv.v[f], rv.v[f]);
            dots[4 + f].add_prod(rv.v[f], zv.v[f]);
        }
        a.b[row] = bv;
        a.rb[0][row] = rv;  // the solve starts at iteration 0 (parity 0)
        a.z[row] = zv;
        raise_inst(s, flags);
        Acc<R> blk[kNV], tot[kNV];
        block_totals<kNV>(dots, red, blk);  // its barriers also free gx, gw for the next tile
        const int t0 = a.inst_tile[i], nt = a.inst_tile[i + 1] - t0;
        if (inst_commit<kNV>(blk, a.part, tile, t0, nt, a.iticket + i, red, tot) && t == 0) {
            volatile BInst* vs = s;
            const int stop = (atomicOr(&s->flags, 0u) & (FEA_STATUS_BLOWUP | FEA_STATUS_NONFINITE)) != 0;
            const double tol = a.ctl->tol;
            vs->stop = stop;
            vs->iter = 0;
            int nact = 0;
#pragma unroll
            for (int f = 0; f < 2; f++) nact += start_solve<R>(vs, f, stop, tol, tot[f], tot[2 + f], tot[4 + f]);
            if (nact) atomicAdd(&a.ctl->n_next, nact);
        }
    }
    phase_end(a, kIterReset);
}

// The refinement pass of kb_refine on the tile-ELL layout: zero right-hand
// sides give x = 0, then the float-float true residual r = b - A x; fields
// still above their threshold restart CG from there.
template <typename R>
__global__ void __launch_bounds__(kBlock) kb_refine_ell(BArgs<R> a) {
    using V = FV<R, 2>;
    extern __shared__ __align__(16) unsigned char dyn_smem[];
    V* const gx = reinterpret_cast<V*>(dyn_smem);
    __shared__ typename Acc<R>::Packed red[32 * kNV];
    const int t = threadIdx.x, lane = t & 31, wib = t >> 5;
    const int par = iter_of(a) & 1;
    const int refine_on = a.ctl->refine;
    for (int tile = blockIdx.x; tile < a.ntiles; tile += gridDim.x) {
        const int i = a.tile_inst[tile];
        const volatile BInst* s = a.inst + i;
        const int stop = s->stop;
        const int refine = refine_on && s->iter < s->max_iter && !stop;
        int zero[2];
#pragma unroll
        for (int f = 0; f < 2; f++) zero[f] = !stop && !(s->bb[f] > 0.0);
        if (!refine && !zero[0] && !zero[1]) continue;
        const int64_t row = (int64_t)tile * kTileRows + t;
        Acc<R> ax[2];
        if (refine) {  // uniform over the block (one instance per tile)
            stage_tile_x(a, tile, gx, (V*)nullptr, [](const V& x) { return x; });
            const int sl = tile * (kTileRows / 32) + wib;
            const int32_t sb = a.slice_off[sl], sw = (a.slice_off[sl + 1] - sb) >> 5;
            __syncthreads();
#pragma unroll 4
            for (int32_t k = 0; k < sw; k++) {
                const int32_t e = sb + 32 * k + lane;
                const V av = ldv(a.As + e, false);
                const V x = gx[a.lcol[e]];
#pragma unroll
                for (int f = 0; f < 2; f++) ax[f].add_prod(av.v[f], x.v[f]);
            }
        }
        Acc<R> dots[4];  // |r|^2, r.z per field
        if (zero[0] || zero[1]) {
            V xr = a.x[row];
#pragma unroll
            for (int f = 0; f < 2; f++)
                if (zero[f]) xr.v[f] = 0;
            a.x[row] = xr;
        }
        if (refine) {
            const V bv = a.b[row], d = ldv(a.dinv + row, false);
            V rv, zv;
#pragma unroll
            for (int f = 0; f < 2; f++) {
                Acc<R> tr;
                tr.add(bv.v[f]);
                tr.sub(ax[f]);
                rv.v[f] = tr.rounded();
                zv.v[f] = d.v[f] * rv.v[f];
                dots[f].add_prod(rv.v[f], rv.v[f]);
                dots[2 + f].add_prod(rv.v[f], zv.v[f]);
            }
            a.rb[par][row] = rv;  // the restart continues the iteration parity
            a.z[row] = zv;
        }
        Acc<R> blk[4], tot[4];
        block_totals<4>(dots, red, blk);  // its barriers also free gx for the next tile
        const int t0 = a.inst_tile[i], nt = a.inst_tile[i + 1] - t0;
        if (inst_commit<4>(blk, a.part, tile, t0, nt, a.iticket + i, red, tot) && t == 0) {
            volatile BInst* w = a.inst + i;
            int nact = 0;
#pragma unroll
            for (int f = 0; f < 2; f++) {
                w->active[f] = 0;
                w->fresh[f] = 1;
                if (refine && !zero[f] && w->bb[f] > 0.0) {
                    const double rr = tot[f].value();
                    w->rr[f] = rr;
                    if (rr >= w->thr[f]) {
                        set_gamma(w, f, tot[2 + f]);
                        w->active[f] = 1;
                        nact++;
                    }
                }
            }
            if (nact) atomicAdd(&a.ctl->n_next, nact);
        }
    }
    phase_end(a, kIterKeep);
}

// After the first solve loop: zero right-hand sides give x = 0, then one
// float-float true-residual pass r = b - A x; fields still above their
// threshold restart CG from there.
template <typename R>
__global__ void __launch_bounds__(kBlock) kb_refine(BArgs<R> a) {
    __shared__ typename Acc<R>::Packed red[32 * kNV];
    constexpr int RPW = 32 / kLanes;
    constexpr int RPB = kBlock / kLanes;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int sub = lane & (kLanes - 1), grp = lane / kLanes;
    const int par = iter_of(a) & 1;
    const int refine_on = a.ctl->refine;
    for (int tile = blockIdx.x; tile < a.ntiles; tile += gridDim.x) {
        const int i = a.tile_inst[tile];
        const volatile BInst* s = a.inst + i;
        const int stop = s->stop;
        const int refine = refine_on && s->iter < s->max_iter && !stop;
        int zero[2];
#pragma unroll
        for (int f = 0; f < 2; f++) zero[f] = !stop && !(s->bb[f] > 0.0);
        if (!refine && !zero[0] && !zero[1]) continue;
        Acc<R> dots[4];  // |r|^2, r.z per field
        for (int pass = 0; pass < kTile / RPB; pass++) {
            const int64_t row = (int64_t)tile * kTile + pass * RPB + wib * RPW + grp;
            Acc<R> ax[2];
            if (refine) {
                const int32_t e1 = ldg(a.rp + row + 1);
                for (int32_t e = ldg(a.rp + row) + sub; e < e1; e += kLanes) {
                    const FV<R, 2> av = ldv(a.A + e, false);
                    const FV<R, 2> xc = a.x[ldg(a.col + e)];
#pragma unroll
                    for (int f = 0; f < 2; f++) ax[f].add_prod(av.v[f], xc.v[f]);
                }
#pragma unroll
                for (int o = kLanes / 2; o > 0; o >>= 1)
#pragma unroll
                    for (int f = 0; f < 2; f++) ax[f].shfl_add(o);
            }
            if (sub == 0) {
                if (zero[0] || zero[1]) {
                    FV<R, 2> xr = a.x[row];
#pragma unroll
                    for (int f = 0; f < 2; f++)
                        if (zero[f]) xr.v[f] = 0;
                    a.x[row] = xr;
                }
                if (refine) {
                    const FV<R, 2> bv = a.b[row], d = ldv(a.dinv + row, false);
                    FV<R, 2> rv, zv;
#pragma unroll
                    for (int f = 0; f < 2; f++) {
                        Acc<R> t;
                        t.add(bv.v[f]);
                        t.sub(ax[f]);
                        rv.v[f] = t.rounded();
                        zv.v[f] = d.v[f] * rv.v[f];
                        dots[f].add_prod(rv.v[f], rv.v[f]);
                        dots[2 + f].add_prod(rv.v[f], zv.v[f]);
                    }
                    a.rb[par][row] = rv;  // the restart continues the iteration parity
                    a.z[row] = zv;
                }
            }
        }
        Acc<R> blk[4], tot[4];
        block_totals<4>(dots, red, blk);
        const int t0 = a.inst_tile[i], nt = a.inst_tile[i + 1] - t0;
        if (inst_commit<4>(blk, a.part, tile, t0, nt, a.iticket + i, red, tot) && threadIdx.x == 0) {
            volatile BInst* w = a.inst + i;
            int nact = 0;
#pragma unroll
            for (int f = 0; f < 2; f++) {
                w->active[f] = 0;
                w->fresh[f] = 1;
                if (refine && !zero[f] && w->bb[f] > 0.0) {
                    const double rr = tot[f].value();
                    w->rr[f] = rr;
                    if (rr >= w->thr[f]) {
                        set_gamma(w, f, tot[2 + f]);
                        w->active[f] = 1;
                        nact++;
                    }
                }
            }
            if (nact) atomicAdd(&a.ctl->n_next, nact);
        }
    }
    phase_end(a, kIterKeep);
}

// Step bookkeeping of every instance and the outer loop condition (one block).
template <typename R>
__global__ void __launch_bounds__(kBlock) kb_stepctl(BArgs<R> a) {
    __shared__ int alive;
    if (threadIdx.x == 0) alive = 0;
    __syncthreads();
    int mine = 0;
    for (int i = threadIdx.x; i < a.ninst; i += blockDim.x) {
        BInst* s = a.inst + i;
        if (!s->stop) {
            s->steps_done += 1;
            s->total_iters += s->iter;
            for (int f = 0; f < 2; f++) {
                s->last_iters[f] = s->iters[f];
                s->last_rel[f] = s->bb[f] > 0.0 ? sqrt(s->rr[f] / s->bb[f]) : 0.0;
            }
            mine++;
        }
    }
    if (mine) atomicAdd(&alive, mine);
    __syncthreads();
    if (threadIdx.x == 0) {
        BCtl* c = a.ctl;
        c->steps_left -= 1;
        c->steps_done += 1;
        signal_loop(a, c->steps_left > 0 && alive > 0);
    }
}

template <typename R>
__global__ void kb_start(BArgs<R> a) {
    signal_loop(a, a.ctl->steps_left > 0);
}

// Instability test of the state after the last step.
template <typename R>
__global__ void __launch_bounds__(kBlock) kb_final_check(BArgs<R> a) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < a.N; r += (int64_t)gridDim.x * blockDim.x) {
        const FV<R, 2> x = a.x[r];
        const unsigned int f = check_value(x.v[0]) | check_value(x.v[1]);
        if (f) atomicOr(&a.inst[a.tile_inst[r / kTile]].flags, f);
    }
}

// Start of an advance: every instance unfrozen with clear flags (a state
// that is still unstable is frozen again by the first step's check).
__global__ void kb_clear(BInst* inst, int n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        inst[i].stop = 0;
        inst[i].flags = 0u;
    }
}

// ---- set-up kernels ------------------------------------------------------------------

// Instance pattern -> stacked pattern: rows shifted by row0, slots by e0;
// the padding rows up to the next tile boundary are empty.
__global__ void kb_copy_pattern(const int32_t* __restrict__ rp, const int32_t* __restrict__ col, int64_t n,
                                int64_t nrows, int64_t nnz, int64_t row0, int64_t e0, int32_t* rp_out,
                                int32_t* col_out) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < nrows; r += stride)
        rp_out[row0 + r] = (int32_t)(e0 + (r <= n ? rp[r] : nnz));
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nnz; e += stride)
        col_out[e0 + e] = (int32_t)(row0 + col[e]);
}

__global__ void kb_node_map(const int32_t* __restrict__ idx_c, int64_t V, int64_t row0, int32_t* out) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < V; v += (int64_t)gridDim.x * blockDim.x)
        out[v] = idx_c[v] >= 0 ? (int32_t)(row0 + idx_c[v]) : -1;
}

// node-indexed float field -> field f of the stacked state
template <typename R>
__global__ void kb_gather(const float* __restrict__ vals, const int32_t* __restrict__ map, int64_t V,
                          FV<R, 2>* x, int f) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < V; v += (int64_t)gridDim.x * blockDim.x) {
        const int32_t r = map[v];
        if (r >= 0) x[r].v[f] = (R)vals[v];
    }
}

// field f of the stacked state -> node-indexed floats (Dirichlet points 0)
template <typename R>
__global__ void kb_scatter(const FV<R, 2>* __restrict__ x, const int32_t* __restrict__ map, int64_t V, float* out,
                           int f) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < V; v += (int64_t)gridDim.x * blockDim.x) {
        const int32_t r = map[v];
        out[v] = r >= 0 ? (float)x[r].v[f] : 0.f;
    }
}

}  // namespace
}  // namespace fea

using namespace fea;

struct fea_batch {
    int device = 0;
    cudaStream_t stream = nullptr;
    int precision = FEA_FP32;
    int ninst = 0, ntiles = 0;
    int64_t N = 0, nnz = 0;
    int wch = 8;  // CG kernel variant (autotuned): 0/1 tile-ELL (8/4 entries prefetched), 4/8 CSR window,
                  // 14 tile-ELL with the operator streamed by a bulk-copy ring
    TileEll ell;  // tile-ELL layout of the stacked matrix
    void* As = nullptr;
    void* Ms = nullptr;  // its copy of M
    TileEll ell_od;  // the same without diagonal entries (ring variant)
    void* As_od = nullptr;
    std::vector<int64_t> V, node_off;
    DeviceArena mem;
    int32_t *rp = nullptr, *col = nullptr, *tile_inst = nullptr, *inst_tile = nullptr, *node_map = nullptr;
    void *A = nullptr, *dinv = nullptr, *M = nullptr;
    void *x = nullptr, *b = nullptr, *z = nullptr, *p = nullptr, *rws = nullptr;
    BPrm* prm = nullptr;
    BInst* inst = nullptr;
    BCtl* ctl = nullptr;
    double* part = nullptr;
    unsigned int* iticket = nullptr;
    int ngroups = 0;               // groups of kGroupTiles tiles (variant 14)
    int32_t* inst_grp = nullptr;   // [ninst + 1] first group of each instance
    double* gpart = nullptr;       // [ngroups * kNV]
    int32_t* act_pos = nullptr;    // [ninst + 1] active-tile table
    BFlags* flags = nullptr;
    float* staging = nullptr;  // node-sized staging buffer (largest instance)
    int guess_rule = 0;        // start of the solves: 0 x_n, 1 2 x_n - x_(n-1) (variant 14)
    void *xprev = nullptr, *xg = nullptr;  // [N] x_(n-1) and the next start (allocated with rule 1)
    double tol = 0.0;
    int max_iter_cfg = 0;
    bool stream_mode = false;
    StepGraph graph;
};

namespace fea {
namespace {

template <typename R>
BArgs<R> make_bargs(fea_batch* B) {
    BArgs<R> a{};
    a.N = B->N;
    a.ntiles = B->ntiles;
    a.ninst = B->ninst;
    a.rp = B->rp;
    a.col = B->col;
    a.A = (const FV<R, 2>*)B->A;
    a.dinv = (const FV<R, 2>*)B->dinv;
    a.M = (const R*)B->M;
    a.x = (FV<R, 2>*)B->x;
    a.b = (FV<R, 2>*)B->b;
    a.z = (FV<R, 2>*)B->z;
    a.p = (FV<R, 2>*)B->p;
    FV<R, 2>* w = (FV<R, 2>*)B->rws;
    for (int k = 0; k < 2; k++) {
        a.rb[k] = w + k * B->N;
        a.wb[k] = w + (2 + k) * B->N;
        a.sb[k] = w + (4 + k) * B->N;
    }
    a.tile_inst = B->tile_inst;
    a.inst_tile = B->inst_tile;
    a.prm = B->prm;
    a.inst = B->inst;
    a.ctl = B->ctl;
    a.part = B->part;
    a.iticket = B->iticket;
    if (B->ell.ok) {
        a.As = (const FV<R, 2>*)B->As;
        a.Ms = (const R*)B->Ms;
        a.lcol = B->ell.lcol;
        a.lcol2 = B->ell.lcol2;
        a.slice_off = B->ell.slice_off;
        a.halo_off = B->ell.halo_off;
        a.halo_col = B->ell.halo_col;
        a.hmax = B->ell.hmax;
        a.emax = B->ell.emax;
        if (B->ell_od.ok) {
            a.As_od = (const FV<R, 2>*)B->As_od;
            a.lcol_od = B->ell_od.lcol;
            a.slice_off_od = B->ell_od.slice_off;
            a.emax_od = B->ell_od.emax;
        }
    }
    a.inst_grp = B->inst_grp;
    a.gpart = B->gpart;
    a.act_pos = B->wch == 14 ? B->act_pos : nullptr;
    if (B->guess_rule == 1 && B->wch == 14 && B->xprev) {
        a.xprev = (FV<R, 2>*)B->xprev;
        a.xg = (FV<R, 2>*)B->xg;
    }
    return a;
}

// Blocks of kb_guess_move: one per tile, up to 16 passes' worth per SM.
int move_grid(const fea_batch* B) { return std::max(1, std::min(B->ntiles, 16 * num_sms())); }

// Graph identity: the variant and whether the extrapolated start is on.
int graph_key(const fea_batch* B) { return B->wch + (B->guess_rule == 1 && B->wch == 14 ? 1000 : 0); }

template <typename R>
struct BLoop {
    BArgs<R> a, a1, a2;
    BLoop(const BArgs<R>& base, BFlags* fl, int use_graph) : a(base), a1(base), a2(base) {
        a.use_graph = a1.use_graph = a2.use_graph = use_graph;
        a.cont = &fl->step;
        a1.cont = &fl->cg1;
        a2.cont = &fl->cg2;
    }
};

// The CG kernels of a variant: 4 and 8 the windowed CSR kernels, 0 and 1 the
// tile-ELL kernels with 8 or 4 entries prefetched, 14 the tile-ELL ring kernel
// (its set-up product is variant 1's).
template <typename R, int V>
struct BKernels {
    static constexpr void (*init)(BArgs<R>) = kb_init<R, V>;
    static constexpr void (*iter)(BArgs<R>) = kb_iter<R, V>;
    static size_t smem(const fea_batch*) { return 0; }
};
template <typename R, int KPRE>
struct BEllKernels {
    static constexpr void (*init)(BArgs<R>) = kb_init_ell<R, KPRE>;
    static constexpr void (*iter)(BArgs<R>) = kb_iter_ell<R, KPRE>;
    static size_t smem(const fea_batch* B) { return 2 * sizeof(FV<R, 2>) * (size_t)(kTileRows + B->ell.hmax); }
};
template <typename R>
struct BKernels<R, 0> : BEllKernels<R, 8> {};
template <typename R>
struct BKernels<R, 1> : BEllKernels<R, 4> {};
constexpr int kBatchRingStages = 3;
template <typename R>
struct BKernels<R, 14> : BEllKernels<R, 4> {
    static constexpr void (*init)(BArgs<R>) = kb_ring<R, kBatchRingStages, kPhInit>;
    static constexpr void (*iter)(BArgs<R>) = kb_ring<R, kBatchRingStages, kPhIter>;
};

// Tile-list capacity of a ring-kernel block for a grid of `grid` blocks: a
// block's share is at most ceil(tiles / grid) tiles, and its last group may
// reach kGroupTiles - 1 tiles beyond it.
int ring_tcap(const fea_batch* B, int64_t grid) {
    return (int)(ceil_div(B->ntiles, std::max<int64_t>(grid, 1)) + kGroupTiles);
}

// Entries of the largest tile a ring phase streams (the iteration streams
// the diagonal-free layout when it exists).
int ring_emax(const fea_batch* B, int ph) { return ph == kPhIter && B->ell_od.ok ? B->ell_od.emax : B->ell.emax; }

template <typename R>
size_t ring_smem(const fea_batch* B, int tcap, int ph) {
    return BRingLayout<R>(ring_emax(B, ph), B->ell.hmax, tcap, kBatchRingStages, ph).total;
}

// The largest of the phases' shared memory.
template <typename R>
size_t ring_smem_max(const fea_batch* B, int tcap) {
    size_t m = 0;
    for (int ph : {kPhIter, kPhRhs, kPhInit, kPhRefine}) m = std::max(m, ring_smem<R>(B, tcap, ph));
    return m;
}

// Whether the ring kernel fits: the tile-ELL layout exists and a block's
// shared memory is within the opt-in limit for the largest tile list a grid
// can give it (a grid of min(SMs, groups) blocks).
template <typename R>
bool ring_fits(const fea_batch* B) {
    if (!B->ell.ok || B->ell.emax <= 0) return false;
    int dev = 0, lim = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&lim, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess)
        return false;
    const int64_t g = std::max<int64_t>(1, std::min<int64_t>(num_sms(), B->ngroups));
    return ring_smem_max<R>(B, ring_tcap(B, g)) + 2048 <= (size_t)lim;
}

template <typename R, int V>
struct BGrids {
    using K = BKernels<R, V>;
    using Fn = void (*)(BArgs<R>);
    int rhs, init, iter, stream, tcap = 0;
    size_t smem_init, smem_iter, smem_rhs = 0, smem_refine = 0;
    Fn rhs_k = kb_rhs<R>, refine_k = kb_refine<R>;  // the staged tile-ELL forms when the layout exists
    explicit BGrids(const fea_batch* B) {
        smem_init = smem_iter = K::smem(B);
        if constexpr (V == 14) {
            // Every phase on the ring pipeline, at one grid: the smallest of
            // the phases' one-wave grids at the tile-list capacity of one
            // block per SM; then the capacity of that grid (never larger, so
            // the occupancy holds; larger when fewer groups than SMs shrink
            // the grid) and each phase's shared memory for it.
            const Fn ks[4] = {K::iter, kb_ring<R, kBatchRingStages, kPhRhs>, K::init,
                              kb_ring<R, kBatchRingStages, kPhRefine>};
            const int phs[4] = {kPhIter, kPhRhs, kPhInit, kPhRefine};
            const int tcap0 = ring_tcap(B, num_sms());
            int g = INT32_MAX;
            for (int p = 0; p < 4; p++)
                g = std::min(g, wave_grid(ks[p], std::max(B->ngroups, 1), ring_smem<R>(B, tcap0, phs[p])));
            tcap = ring_tcap(B, g);
            size_t sm[4];
            for (int p = 0; p < 4; p++) {
                sm[p] = ring_smem<R>(B, tcap, phs[p]);
                ensure_dyn_smem(ks[p], sm[p]);
            }
            rhs_k = ks[1];
            refine_k = ks[3];
            smem_iter = sm[0];
            smem_rhs = sm[1];
            smem_init = sm[2];
            smem_refine = sm[3];
            rhs = init = iter = g;
        } else {
            if (B->ell.ok) {
                rhs_k = kb_rhs_ell<R>;
                refine_k = kb_refine_ell<R>;
                smem_rhs = smem_refine = 2 * sizeof(FV<R, 2>) * (size_t)(kTileRows + B->ell.hmax);
                ensure_dyn_smem(refine_k, smem_refine);
            }
            rhs = wave_grid(rhs_k, B->ntiles, smem_rhs);
            init = wave_grid(K::init, B->ntiles, smem_init);
            iter = wave_grid(K::iter, B->ntiles, smem_iter);
        }
        stream = (int)std::min<int64_t>(max_grid_blocks(), std::max<int64_t>(1, ceil_div(B->N, kBlock)));
    }
    void apply(BArgs<R>& a) const { a.tcap = tcap; }
};

// The iteration kernels of a loop pass, chained by programmatic edges.
template <typename R>
void add_batch_iterations(cudaGraph_t body, void (*iter)(BArgs<R>), int grid, const BArgs<R>& a, size_t smem) {
    cudaGraphNode_t prev = nullptr;
    for (int u = 0; u < kBatchUnroll; u++) {
        cudaGraphNode_t n = add_kernel(body, nullptr, iter, grid, kBlock, a, smem);
        if (prev) add_programmatic_edge(body, prev, n);
        prev = n;
    }
}

// start -> WHILE(step) { rhs -> init -> WHILE(cg1) { iter x 4 } -> refine -> init
//          -> WHILE(cg2) { iter x 4 } -> stepctl } -> final_check
template <typename R, int WCH>
void build_batch_graph_t(fea_batch* B) {
    BLoop<R> L(make_bargs<R>(B), B->flags, 1);
    const BGrids<R, WCH> g(B);
    for (BArgs<R>* x : {&L.a, &L.a1, &L.a2}) g.apply(*x);
    using K = BKernels<R, WCH>;
    StepGraph& G = B->graph;
    cudaGraph_t top;
    FEA_CUDA_TRY(cudaGraphCreate(&top, 0));
    G.graph = top;
    FEA_CUDA_TRY(cudaGraphConditionalHandleCreate(&L.a.cond, top, 0, 0));
    cudaGraphNode_t n = add_kernel(top, nullptr, kb_start<R>, 1, 1, L.a);
    cudaGraph_t step_body;
    n = add_while(top, n, L.a.cond, &step_body);
    add_kernel(top, n, kb_final_check<R>, g.stream, kBlock, L.a);
    FEA_CUDA_TRY(cudaGraphConditionalHandleCreate(&L.a1.cond, step_body, 0, 0));
    FEA_CUDA_TRY(cudaGraphConditionalHandleCreate(&L.a2.cond, step_body, 0, 0));
    cudaGraphNode_t s = add_kernel(step_body, nullptr, g.rhs_k, g.rhs, kBlock, L.a1, g.smem_rhs);
    if (L.a1.xg) s = add_kernel(step_body, s, kb_guess_move<R>, move_grid(B), kBlock, L.a1);
    s = add_kernel(step_body, s, K::init, g.init, kBlock, L.a1, g.smem_init);
    cudaGraph_t body1, body2;
    s = add_while(step_body, s, L.a1.cond, &body1);
    add_batch_iterations(body1, K::iter, g.iter, L.a1, g.smem_iter);
    s = add_kernel(step_body, s, g.refine_k, g.rhs, kBlock, L.a2, g.smem_refine);
    s = add_kernel(step_body, s, K::init, g.init, kBlock, L.a2, g.smem_init);
    s = add_while(step_body, s, L.a2.cond, &body2);
    add_batch_iterations(body2, K::iter, g.iter, L.a2, g.smem_iter);
    add_kernel(step_body, s, kb_stepctl<R>, 1, kBlock, L.a);
    FEA_CUDA_TRY(cudaGraphInstantiate(&G.exec, top, 0));
    G.lanes = graph_key(B);
}

int read_int(const int* d, cudaStream_t st) {
    int h = 0;
    FEA_CUDA_TRY(cudaMemcpyAsync(&h, d, sizeof(int), cudaMemcpyDeviceToHost, st));
    FEA_CUDA_TRY(cudaStreamSynchronize(st));
    return h;
}

// The same step loop launched kernel by kernel (profiling mode,
// FEA_LAUNCH_MODE=stream); each loop is bounded by the kernels' own limits.
template <typename R, int WCH>
void run_batch_stream_t(fea_batch* B) {
    BLoop<R> L(make_bargs<R>(B), B->flags, 0);
    const BGrids<R, WCH> g(B);
    for (BArgs<R>* x : {&L.a, &L.a1, &L.a2}) g.apply(*x);
    using K = BKernels<R, WCH>;
    cudaStream_t st = B->stream;
    kb_start<R><<<1, 1, 0, st>>>(L.a);
    FEA_CHECK_LAUNCH();
    while (read_int(&B->flags->step, st)) {
        g.rhs_k<<<g.rhs, kBlock, g.smem_rhs, st>>>(L.a1);
        FEA_CHECK_LAUNCH();
        if (L.a1.xg) {
            kb_guess_move<R><<<move_grid(B), kBlock, 0, st>>>(L.a1);
            FEA_CHECK_LAUNCH();
        }
        for (int loop = 0; loop < 2; loop++) {
            const BArgs<R>& la = loop ? L.a2 : L.a1;
            if (loop) {
                g.refine_k<<<g.rhs, kBlock, g.smem_refine, st>>>(L.a2);
                FEA_CHECK_LAUNCH();
            }
            K::init<<<g.init, kBlock, g.smem_init, st>>>(la);
            FEA_CHECK_LAUNCH();
            while (read_int(la.cont, st)) {
                K::iter<<<g.iter, kBlock, g.smem_iter, st>>>(la);
                FEA_CHECK_LAUNCH();
            }
        }
        kb_stepctl<R><<<1, kBlock, 0, st>>>(L.a);
        FEA_CHECK_LAUNCH();
    }
    kb_final_check<R><<<g.stream, kBlock, 0, st>>>(L.a);
    FEA_CHECK_LAUNCH();
}

template <typename R>
void run_batch(fea_batch* B) {
    if (B->stream_mode) {
        switch (B->wch) {
        case 0: run_batch_stream_t<R, 0>(B); break;
        case 1: run_batch_stream_t<R, 1>(B); break;
        case 4: run_batch_stream_t<R, 4>(B); break;
        case 14: run_batch_stream_t<R, 14>(B); break;
        default: run_batch_stream_t<R, 8>(B); break;
        }
        return;
    }
    if (!B->graph.exec || B->graph.lanes != graph_key(B)) {
        B->graph.destroy();
        switch (B->wch) {
        case 0: build_batch_graph_t<R, 0>(B); break;
        case 1: build_batch_graph_t<R, 1>(B); break;
        case 4: build_batch_graph_t<R, 4>(B); break;
        case 14: build_batch_graph_t<R, 14>(B); break;
        default: build_batch_graph_t<R, 8>(B); break;
        }
    }
    FEA_CUDA_TRY(cudaGraphLaunch(B->graph.exec, B->stream));
}

template <typename R, int V>
void batch_iter_probe_t(fea_batch* B, BArgs<R> a) {
    const BGrids<R, V> g(B);
    g.apply(a);
    BKernels<R, V>::iter<<<g.iter, kBlock, g.smem_iter, B->stream>>>(a);
    FEA_CHECK_LAUNCH();
}

// One iteration kernel of variant `var` over every tile, fields masked
// (probe_mask): x and p are written back unchanged and only CG scratch, which
// every solve recomputes, changes.  The timing probe of autotuning and of
// fea_batch_time_iteration.
template <typename R>
void batch_iter_probe(fea_batch* B, int var) {
    BArgs<R> a = make_bargs<R>(B);
    a.probe = 1;
    a.use_graph = 0;
    a.cont = &B->flags->probe;
    switch (var) {
    case 0: batch_iter_probe_t<R, 0>(B, a); break;
    case 1: batch_iter_probe_t<R, 1>(B, a); break;
    case 4: batch_iter_probe_t<R, 4>(B, a); break;
    case 14: batch_iter_probe_t<R, 14>(B, a); break;
    default: batch_iter_probe_t<R, 8>(B, a); break;
    }
}

// Whether variant v can run on this batch.
template <typename R>
bool batch_variant_ok(const fea_batch* B, int v) {
    if (v == 0 || v == 1) return B->ell.ok;
    if (v == 14) return ring_fits<R>(B);
    return v == 4 || v == 8;
}

// Pick the CG kernel variant by timing one iteration kernel of each candidate.
template <typename R>
void autotune_batch(fea_batch* B) {
    cudaEvent_t e0, e1;
    FEA_CUDA_TRY(cudaEventCreate(&e0));
    FEA_CUDA_TRY(cudaEventCreate(&e1));
    float best = 1e30f;
    int pick = 8;
    for (int w : {0, 1, 4, 8, 14}) {
        if (!batch_variant_ok<R>(B, w)) continue;
        for (int rep = 0; rep < 13; rep++) {
            if (rep == 3) FEA_CUDA_TRY(cudaEventRecord(e0, B->stream));
            batch_iter_probe<R>(B, w);
        }
        FEA_CUDA_TRY(cudaEventRecord(e1, B->stream));
        FEA_CUDA_TRY(cudaEventSynchronize(e1));
        float ms = 0.f;
        FEA_CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
        if (ms < best) {
            best = ms;
            pick = w;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    B->wch = pick;
}

void check_batch(const fea_batch* B) {
    if (!B) {
        set_error("null batch handle");
        throw Error{FEA_ERR_INVALID_ARGUMENT};
    }
    FEA_CUDA_TRY(cudaSetDevice(B->device));
}

void check_instance(const fea_batch* B, int i) {
    if (i < 0 || i >= B->ninst) {
        set_error("instance %d out of range [0, %d)", i, B->ninst);
        throw Error{FEA_ERR_INVALID_ARGUMENT};
    }
}

// A single-mesh handle per instance builds its boundary, pattern, solver
// order and FP64 matrices; they are copied into the stacked arrays and the
// handles released.
struct InstanceHandles {
    std::vector<fea_solver*> h;
    ~InstanceHandles() {
        for (fea_solver* p : h) fea_destroy(p);
    }
};

template <typename R>
void copy_instance(fea_batch* B, int i, fea_solver* h, const fea_instance_desc& d, int64_t row0, int64_t e0,
                   int64_t nrows) {
    const MeshView m = mesh_view(h);
    cudaStream_t st = m.stream;
    const int64_t n = m.N, nnz = m.Pc->nnz;
    kb_copy_pattern<<<launch_grid(std::max(nrows, nnz)), kBlock, 0, st>>>(m.Pc->row_ptr, m.Pc->col, n, nrows, nnz,
                                                                          row0, e0, B->rp, B->col);
    FEA_CHECK_LAUNCH();
    OpCoef<2> c{};
    c.f[0] = {(double)d.time_step, (double)d.Du, 1.0, 0.0};
    c.f[1] = {(double)d.time_step, (double)d.Dv, 1.0, 0.0};
    combine_operator<R, 2>(*m.Pc, m.emap, m.M64, m.K64, m.Adv64, c, (FV<R, 2>*)B->A + e0, (FV<R, 2>*)B->dinv + row0,
                           st);
    round_copy<R>(m.M64, m.emap, nnz, (R*)B->M + e0, st);
    kb_node_map<<<launch_grid(m.V), kBlock, 0, st>>>(m.idx_c, m.V, row0, B->node_map + B->node_off[i]);
    FEA_CHECK_LAUNCH();
    FEA_CUDA_TRY(cudaStreamSynchronize(st));
}

template <typename R>
void create_batch(fea_batch* B, const fea_instance_desc* inst, int n) {
    InstanceHandles H;
    H.h.assign(n, nullptr);
    std::vector<int64_t> N(n), NNZ(n);
    for (int i = 0; i < n; i++) {
        const fea_instance_desc& d = inst[i];
        fea_params prm;
        fea_params_default(&prm);
        prm.equation = FEA_REACTION_DIFFUSION;
        prm.reaction_mode = 1;
        prm.rd_time_step = d.time_step;
        prm.rd_Du = d.Du;
        prm.rd_Dv = d.Dv;
        prm.rd_feed_rate = d.feed_rate;
        prm.rd_kill_rate = d.kill_rate;
        const int rc = fea_create(d.vertices, d.num_vertices, d.triangles, d.num_triangles, nullptr,
                                  d.boundary_condition, B->precision, &prm, &H.h[i]);
        if (rc != FEA_OK) throw Error{rc};
        const MeshView m = mesh_view(H.h[i]);
        N[i] = m.N;
        NNZ[i] = m.Pc->nnz;
    }
    std::vector<int32_t> tile0(n + 1), tinst;
    std::vector<int64_t> e0(n + 1);
    B->V.resize(n);
    B->node_off.resize(n + 1);
    int64_t tiles = 0, nnz = 0, nodes = 0, vmax = 1;
    for (int i = 0; i < n; i++) {
        const int64_t nt = std::max<int64_t>(1, ceil_div(N[i], kTile));
        tile0[i] = (int32_t)tiles;
        e0[i] = nnz;
        B->V[i] = inst[i].num_vertices;
        B->node_off[i] = nodes;
        for (int64_t t = 0; t < nt; t++) tinst.push_back(i);
        tiles += nt;
        nnz += NNZ[i];
        nodes += inst[i].num_vertices;
        vmax = std::max<int64_t>(vmax, inst[i].num_vertices);
    }
    tile0[n] = (int32_t)tiles;
    e0[n] = nnz;
    B->node_off[n] = nodes;
    if (tiles * kTile >= (int64_t)INT32_MAX || nnz >= (int64_t)INT32_MAX) {
        set_error("batch exceeds int32 indexing (%lld rows, %lld entries)", (long long)(tiles * kTile),
                  (long long)nnz);
        throw Error{FEA_ERR_TOO_LARGE};
    }
    B->ntiles = (int)tiles;
    B->N = tiles * kTile;
    B->nnz = nnz;
    const int64_t Nr = B->N;
    cudaStream_t st = B->stream;
    B->rp = B->mem.alloc<int32_t>(Nr + 1);
    B->col = B->mem.alloc<int32_t>(nnz);
    B->tile_inst = B->mem.alloc<int32_t>(tiles);
    B->inst_tile = B->mem.alloc<int32_t>(n + 1);
    B->node_map = B->mem.alloc<int32_t>(nodes);
    B->A = B->mem.alloc<FV<R, 2>>(nnz);
    B->M = B->mem.alloc<R>(nnz);
    B->dinv = B->mem.alloc<FV<R, 2>>(Nr);
    B->x = B->mem.alloc<FV<R, 2>>(Nr);
    B->b = B->mem.alloc<FV<R, 2>>(Nr);
    B->z = B->mem.alloc<FV<R, 2>>(Nr);
    B->p = B->mem.alloc<FV<R, 2>>(Nr);
    B->rws = B->mem.alloc<FV<R, 2>>(6 * Nr);
    B->prm = B->mem.alloc<BPrm>(n);
    B->inst = B->mem.alloc<BInst>(n);
    B->ctl = B->mem.alloc<BCtl>(1);
    B->part = B->mem.alloc<double>(tiles * kNV);
    B->iticket = B->mem.alloc<unsigned int>(n);
    std::vector<int32_t> grp0(n + 1);  // groups of kGroupTiles tiles per instance (ring kernel)
    for (int i = 0; i < n; i++) grp0[i + 1] = grp0[i] + (int32_t)ceil_div(tile0[i + 1] - tile0[i], kGroupTiles);
    B->ngroups = grp0[n];
    B->inst_grp = B->mem.alloc<int32_t>(n + 1);
    B->gpart = B->mem.alloc<double>((int64_t)B->ngroups * kNV);
    B->act_pos = B->mem.alloc<int32_t>(n + 1);
    B->flags = B->mem.alloc<BFlags>(1);
    B->staging = B->mem.alloc<float>(vmax);
    const size_t fv = sizeof(FV<R, 2>);
    for (auto zv : {std::make_pair(B->dinv, Nr), std::make_pair(B->x, Nr), std::make_pair(B->b, Nr),
                    std::make_pair(B->z, Nr), std::make_pair(B->p, Nr), std::make_pair(B->rws, 6 * Nr)})
        FEA_CUDA_TRY(cudaMemsetAsync(zv.first, 0, fv * (size_t)zv.second, st));
    FEA_CUDA_TRY(cudaMemsetAsync(B->ctl, 0, sizeof(BCtl), st));
    FEA_CUDA_TRY(cudaMemsetAsync(B->iticket, 0, sizeof(unsigned int) * n, st));
    FEA_CUDA_TRY(cudaMemsetAsync(B->flags, 0, sizeof(BFlags), st));
    FEA_CUDA_TRY(cudaMemsetAsync(B->part, 0, sizeof(double) * tiles * kNV, st));
    FEA_CUDA_TRY(cudaMemsetAsync(B->gpart, 0, sizeof(double) * (size_t)B->ngroups * kNV, st));
    FEA_CUDA_TRY(cudaMemsetAsync(B->act_pos, 0, sizeof(int32_t) * (n + 1), st));
    FEA_CUDA_TRY(cudaMemcpyAsync(B->inst_grp, grp0.data(), sizeof(int32_t) * (n + 1), cudaMemcpyHostToDevice, st));
    FEA_CUDA_TRY(cudaMemcpyAsync(B->tile_inst, tinst.data(), sizeof(int32_t) * tiles, cudaMemcpyHostToDevice, st));
    FEA_CUDA_TRY(cudaMemcpyAsync(B->inst_tile, tile0.data(), sizeof(int32_t) * (n + 1), cudaMemcpyHostToDevice, st));
    std::vector<BPrm> hp(n);
    std::vector<BInst> hi(n);
    for (int i = 0; i < n; i++) {
        hp[i] = {(double)inst[i].time_step, (double)inst[i].feed_rate, (double)inst[i].kill_rate};
        memset(&hi[i], 0, sizeof(BInst));
        const int64_t lim = B->max_iter_cfg > 0 ? B->max_iter_cfg : 2 * N[i];
        hi[i].max_iter = (int)std::min<int64_t>(std::max<int64_t>(lim, 1), 0x7fffffff);
    }
    FEA_CUDA_TRY(cudaMemcpyAsync(B->prm, hp.data(), sizeof(BPrm) * n, cudaMemcpyHostToDevice, st));
    FEA_CUDA_TRY(cudaMemcpyAsync(B->inst, hi.data(), sizeof(BInst) * n, cudaMemcpyHostToDevice, st));
    BCtl hc{};
    hc.tol = B->tol;
    hc.refine = 1;
    FEA_CUDA_TRY(cudaMemcpyAsync(B->ctl, &hc, sizeof(hc), cudaMemcpyHostToDevice, st));
    // closing row pointer of the stacked matrix
    const int32_t last = (int32_t)nnz;
    FEA_CUDA_TRY(cudaMemcpyAsync(B->rp + Nr, &last, sizeof(int32_t), cudaMemcpyHostToDevice, st));
    FEA_CUDA_TRY(cudaStreamSynchronize(st));
    for (int i = 0; i < n; i++) {
        copy_instance<R>(B, i, H.h[i], inst[i], (int64_t)tile0[i] * kTile, e0[i],
                         (int64_t)(tile0[i + 1] - tile0[i]) * kTile);
        fea_destroy(H.h[i]);
        H.h[i] = nullptr;
    }
    {  // tile-ELL layout of the stacked matrix
        std::vector<int32_t> hrp(Nr + 1), hcol(nnz);
        FEA_CUDA_TRY(cudaMemcpyAsync(hrp.data(), B->rp, sizeof(int32_t) * (Nr + 1), cudaMemcpyDeviceToHost, st));
        if (nnz > 0)
            FEA_CUDA_TRY(cudaMemcpyAsync(hcol.data(), B->col, sizeof(int32_t) * nnz, cudaMemcpyDeviceToHost, st));
        FEA_CUDA_TRY(cudaStreamSynchronize(st));
        if (build_tile_ell(hrp, hcol, Nr, sizeof(FV<R, 2>), kEllSmemBudget, B->ell, B->mem, st)) {
            B->As = B->mem.alloc<FV<R, 2>>(B->ell.E);
            fill_tile_ell<R, 2>(B->ell, (const FV<R, 2>*)B->A, (FV<R, 2>*)B->As, st);
            B->Ms = B->mem.alloc<R>(B->ell.E);
            fill_tile_ell<R, 1>(B->ell, (const FV<R, 1>*)B->M, (FV<R, 1>*)B->Ms, st);
            if (build_tile_ell(hrp, hcol, Nr, sizeof(FV<R, 2>), kEllSmemBudget, B->ell_od, B->mem, st, true)) {
                B->As_od = B->mem.alloc<FV<R, 2>>(B->ell_od.E);
                fill_tile_ell<R, 2>(B->ell_od, (const FV<R, 2>*)B->A, (FV<R, 2>*)B->As_od, st);
            }
        }
    }
    autotune_batch<R>(B);
    FEA_CUDA_TRY(cudaStreamSynchronize(st));
}

}  // namespace
}  // namespace fea

#define BATCH_API_BEGIN try {
#define BATCH_API_END                                                    \
    }                                                                    \
    catch (const fea::Error& e) {                                        \
        return e.code;                                                   \
    }                                                                    \
    catch (const std::bad_alloc&) {                                      \
        return fea::fail(FEA_ERR_OUT_OF_MEMORY, "host allocation failed"); \
    }                                                                    \
    catch (...) {                                                        \
        return fea::fail(FEA_ERR_CUDA, "unexpected failure");            \
    }                                                                    \
    return FEA_OK;

extern "C" {

int fea_batch_create(const fea_instance_desc* instances, int num_instances, int precision, double cg_tolerance,
                     int cg_max_iterations, fea_batch** out) {
    if (!out) return fail(FEA_ERR_INVALID_ARGUMENT, "null output handle");
    *out = nullptr;
    if (!instances || num_instances <= 0) return fail(FEA_ERR_INVALID_ARGUMENT, "no instances");
    if (precision != FEA_FP32 && precision != FEA_FP64) return fail(FEA_ERR_INVALID_ARGUMENT, "bad precision");
    for (int i = 0; i < num_instances; i++) {
        const fea_instance_desc& d = instances[i];
        if (!d.vertices || !d.triangles || d.num_vertices <= 0 || d.num_triangles <= 0)
            return fail(FEA_ERR_BAD_MESH, "instance mesh must have vertices and triangles");
        if (!(d.time_step > 0.f)) return fail(FEA_ERR_INVALID_ARGUMENT, "instance time step must be positive");
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(FEA_ERR_NO_DEVICE, "no CUDA device");
    fea_batch* B = nullptr;
    try {
        B = new fea_batch();
        FEA_CUDA_TRY(cudaGetDevice(&B->device));
        FEA_CUDA_TRY(cudaStreamCreateWithFlags(&B->stream, cudaStreamNonBlocking));
        B->precision = precision;
        B->ninst = num_instances;
        B->tol = cg_tolerance > 0.0 ? cg_tolerance : (precision == FEA_FP64 ? 1e-10 : 1.1920928955078125e-07);
        B->max_iter_cfg = cg_max_iterations;
        const char* mode = getenv("FEA_LAUNCH_MODE");
        B->stream_mode = mode && strcmp(mode, "stream") == 0;
        if (precision == FEA_FP64) create_batch<double>(B, instances, num_instances);
        else create_batch<float>(B, instances, num_instances);
        *out = B;
        return FEA_OK;
    } catch (const fea::Error& e) {
        if (B) fea_batch_destroy(B);
        return e.code;
    } catch (const std::bad_alloc&) {
        if (B) fea_batch_destroy(B);
        return fail(FEA_ERR_OUT_OF_MEMORY, "host allocation failed");
    } catch (...) {
        if (B) fea_batch_destroy(B);
        return fail(FEA_ERR_CUDA, "unexpected failure");
    }
}

int fea_batch_destroy(fea_batch* B) {
    if (!B) return FEA_OK;
    cudaSetDevice(B->device);
    if (B->stream) cudaStreamSynchronize(B->stream);
    B->graph.destroy();
    B->mem.release();
    if (B->stream) cudaStreamDestroy(B->stream);
    delete B;
    return FEA_OK;
}

int fea_batch_set_fields(fea_batch* B, int instance, const float* u, const float* v) {
    BATCH_API_BEGIN
    check_batch(B);
    check_instance(B, instance);
    const int64_t V = B->V[instance];
    const int32_t* map = B->node_map + B->node_off[instance];
    const float* src[2] = {u, v};
    for (int f = 0; f < 2; f++) {
        if (!src[f]) continue;
        FEA_CUDA_TRY(cudaMemcpyAsync(B->staging, src[f], sizeof(float) * V, cudaMemcpyHostToDevice, B->stream));
        if (B->precision == FEA_FP64)
            kb_gather<double><<<launch_grid(V), kBlock, 0, B->stream>>>(B->staging, map, V, (FV<double, 2>*)B->x, f);
        else
            kb_gather<float><<<launch_grid(V), kBlock, 0, B->stream>>>(B->staging, map, V, (FV<float, 2>*)B->x, f);
        FEA_CHECK_LAUNCH();
    }
    kb_clear_history<<<1, kBlock, 0, B->stream>>>(B->inst, B->ninst, instance);  // a new state has no history
    FEA_CHECK_LAUNCH();
    FEA_CUDA_TRY(cudaStreamSynchronize(B->stream));
    BATCH_API_END
}

int fea_batch_get_fields(fea_batch* B, int instance, float* u, float* v) {
    BATCH_API_BEGIN
    check_batch(B);
    check_instance(B, instance);
    const int64_t V = B->V[instance];
    const int32_t* map = B->node_map + B->node_off[instance];
    float* dst[2] = {u, v};
    for (int f = 0; f < 2; f++) {
        if (!dst[f]) continue;
        if (B->precision == FEA_FP64)
            kb_scatter<double><<<launch_grid(V), kBlock, 0, B->stream>>>((const FV<double, 2>*)B->x, map, V,
                                                                          B->staging, f);
        else
            kb_scatter<float><<<launch_grid(V), kBlock, 0, B->stream>>>((const FV<float, 2>*)B->x, map, V,
                                                                         B->staging, f);
        FEA_CHECK_LAUNCH();
        FEA_CUDA_TRY(cudaMemcpyAsync(dst[f], B->staging, sizeof(float) * V, cudaMemcpyDeviceToHost, B->stream));
        FEA_CUDA_TRY(cudaStreamSynchronize(B->stream));
    }
    BATCH_API_END
}

int fea_batch_advance_time(fea_batch* B, int64_t nsteps) {
    BATCH_API_BEGIN
    check_batch(B);
    if (nsteps < 0) return fail(FEA_ERR_INVALID_ARGUMENT, "negative step count");
    if (nsteps == 0) return FEA_OK;
    long long ctl[2] = {nsteps, 0};  // steps_left, steps_done
    FEA_CUDA_TRY(cudaMemcpyAsync(B->ctl, ctl, sizeof(ctl), cudaMemcpyHostToDevice, B->stream));
    kb_clear<<<launch_grid(B->ninst), kBlock, 0, B->stream>>>(B->inst, B->ninst);
    FEA_CHECK_LAUNCH();
    if (B->precision == FEA_FP64) run_batch<double>(B);
    else run_batch<float>(B);
    BATCH_API_END
}

int fea_batch_synchronize(fea_batch* B) {
    BATCH_API_BEGIN
    check_batch(B);
    FEA_CUDA_TRY(cudaStreamSynchronize(B->stream));
    BATCH_API_END
}

int fea_batch_cg_variant(fea_batch* B, int set, int* variant) {
    BATCH_API_BEGIN
    check_batch(B);
    if (!variant) return fail(FEA_ERR_INVALID_ARGUMENT, "null variant");
    if (!set) {
        *variant = B->wch;
        return FEA_OK;
    }
    const int v = *variant;
    if (v != 0 && v != 1 && v != 4 && v != 8 && v != 14)
        return fail(FEA_ERR_INVALID_ARGUMENT, "batch CG variant must be 0, 1, 4, 8 or 14");
    const bool ok = B->precision == FEA_FP64 ? batch_variant_ok<double>(B, v) : batch_variant_ok<float>(B, v);
    if (!ok) {
        set_error("batch CG variant %d unavailable: no tile-ELL layout, or its shared memory does not fit", v);
        return FEA_ERR_UNSUPPORTED;
    }
    if (v != B->wch) {  // the histories of the extrapolated start are kept by variant 14 only
        kb_clear_history<<<launch_grid(B->ninst), kBlock, 0, B->stream>>>(B->inst, B->ninst, -1);
        FEA_CHECK_LAUNCH();
    }
    B->wch = v;
    BATCH_API_END
}

int fea_batch_set_initial_guess(fea_batch* B, int rule) {
    BATCH_API_BEGIN
    check_batch(B);
    if (rule != 0 && rule != 1) return fail(FEA_ERR_INVALID_ARGUMENT, "initial guess rule must be 0 or 1");
    if (rule == B->guess_rule) return FEA_OK;
    if (rule == 1 && !B->xprev) {
        const size_t nb = (B->precision == FEA_FP64 ? sizeof(FV<double, 2>) : sizeof(FV<float, 2>)) * (size_t)B->N;
        void* xp = B->mem.alloc<char>((int64_t)nb);
        void* xg = B->mem.alloc<char>((int64_t)nb);
        FEA_CUDA_TRY(cudaMemsetAsync(xp, 0, nb, B->stream));
        FEA_CUDA_TRY(cudaMemsetAsync(xg, 0, nb, B->stream));
        B->xprev = xp;
        B->xg = xg;
    }
    kb_clear_history<<<launch_grid(B->ninst), kBlock, 0, B->stream>>>(B->inst, B->ninst, -1);
    FEA_CHECK_LAUNCH();
    FEA_CUDA_TRY(cudaStreamSynchronize(B->stream));
    B->guess_rule = rule;
    BATCH_API_END
}

int fea_batch_set_cg(fea_batch* B, double cg_tolerance, int cg_max_iterations) {
    BATCH_API_BEGIN
    check_batch(B);
    if (!(cg_tolerance >= 0.0)) return fail(FEA_ERR_INVALID_ARGUMENT, "bad CG tolerance");
    const int n = B->ninst;
    FEA_CUDA_TRY(cudaStreamSynchronize(B->stream));
    std::vector<BInst> h(n);
    std::vector<int32_t> t0(n + 1);
    BCtl c{};
    FEA_CUDA_TRY(cudaMemcpy(h.data(), B->inst, sizeof(BInst) * n, cudaMemcpyDeviceToHost));
    FEA_CUDA_TRY(cudaMemcpy(t0.data(), B->inst_tile, sizeof(int32_t) * (n + 1), cudaMemcpyDeviceToHost));
    FEA_CUDA_TRY(cudaMemcpy(&c, B->ctl, sizeof(BCtl), cudaMemcpyDeviceToHost));
    B->tol = cg_tolerance > 0.0 ? cg_tolerance : (B->precision == FEA_FP64 ? 1e-10 : 1.1920928955078125e-07);
    B->max_iter_cfg = cg_max_iterations;
    for (int i = 0; i < n; i++) {  // default limit: twice the instance's rows (its tiles, padding included)
        const int64_t lim = cg_max_iterations > 0 ? cg_max_iterations : 2 * (int64_t)(t0[i + 1] - t0[i]) * kTile;
        h[i].max_iter = (int)std::min<int64_t>(std::max<int64_t>(lim, 1), 0x7fffffff);
    }
    c.tol = B->tol;
    FEA_CUDA_TRY(cudaMemcpy(B->inst, h.data(), sizeof(BInst) * n, cudaMemcpyHostToDevice));
    FEA_CUDA_TRY(cudaMemcpy(B->ctl, &c, sizeof(BCtl), cudaMemcpyHostToDevice));
    BATCH_API_END
}

int fea_batch_time_iteration(fea_batch* B, int reps, double* ms_per_launch) {
    BATCH_API_BEGIN
    check_batch(B);
    if (reps <= 0 || !ms_per_launch) return fail(FEA_ERR_INVALID_ARGUMENT, "bad arguments");
    cudaEvent_t e0, e1;
    FEA_CUDA_TRY(cudaEventCreate(&e0));
    FEA_CUDA_TRY(cudaEventCreate(&e1));
    auto launch = [&]() {
        if (B->precision == FEA_FP64) batch_iter_probe<double>(B, B->wch);
        else batch_iter_probe<float>(B, B->wch);
    };
    launch();  // warm-up
    FEA_CUDA_TRY(cudaEventRecord(e0, B->stream));
    for (int r = 0; r < reps; r++) launch();
    FEA_CUDA_TRY(cudaEventRecord(e1, B->stream));
    FEA_CUDA_TRY(cudaEventSynchronize(e1));
    float ms = 0.f;
    FEA_CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *ms_per_launch = ms / reps;
    BATCH_API_END
}

int fea_batch_get_counters(fea_batch* B, int64_t* total_iterations, int64_t* steps_done) {
    BATCH_API_BEGIN
    check_batch(B);
    const int n = B->ninst;
    std::vector<BInst> h(n);
    FEA_CUDA_TRY(cudaMemcpyAsync(h.data(), B->inst, sizeof(BInst) * n, cudaMemcpyDeviceToHost, B->stream));
    FEA_CUDA_TRY(cudaStreamSynchronize(B->stream));
    for (int i = 0; i < n; i++) {
        if (total_iterations) total_iterations[i] = h[i].total_iters;
        if (steps_done) steps_done[i] = h[i].steps_done;
    }
    BATCH_API_END
}

int fea_batch_get_status(fea_batch* B, uint32_t* flags, int32_t* iterations) {
    BATCH_API_BEGIN
    check_batch(B);
    const int n = B->ninst;
    std::vector<BInst> h(n);
    FEA_CUDA_TRY(cudaMemcpyAsync(h.data(), B->inst, sizeof(BInst) * n, cudaMemcpyDeviceToHost, B->stream));
    FEA_CUDA_TRY(cudaStreamSynchronize(B->stream));
    for (int i = 0; i < n; i++) {
        if (flags) flags[i] = h[i].flags;
        if (iterations) {
            iterations[2 * i] = h[i].last_iters[0];
            iterations[2 * i + 1] = h[i].last_iters[1];
        }
    }
    BATCH_API_END
}

}  // extern "C"
