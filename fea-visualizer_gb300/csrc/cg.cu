// cg.cu -- the per-step hot path: fused right-hand side, Jacobi-preconditioned
// CG and the step loop, all inside one CUDA graph.
//
// Reference semantics: CPUSolver::advance_time (CPUSolver.cpp:64-146) solves
// A x = b with Eigen::ConjugateGradient<.., Lower|Upper> and its diagonal
// preconditioner (:65): stop when |r|^2 < tol^2 |b|^2, at most max_iter
// iterations.  The compute-shader path (cgm.glsl:104-149, GPUSolver.cpp:326-361)
// runs the same recurrences with a host round trip per stage; here the loop is
// a CUDA graph WHILE node over time steps with a WHILE node per solve whose
// body chains eight copies of ONE kernel per CG iteration (the Chronopoulos-
// Gear form below): the vector updates are fused into the SpMV, and a single
// grid-wide reduction gives every scalar of the next iteration.
// Inner products: FP32 products are accumulated as float-float pairs (about
// 48 significant bits) per thread, warp, block and grid, and the CG scalars
// are updated in float-float arithmetic too: the GB300's FP64 pipe is narrow
// enough that a few FP64 instructions per warp at the end of every iteration
// cost microseconds, so the FP32 iteration runs none.  The block partials are
// combined by the last block to finish, in a fixed order, so every reduction
// is deterministic.
#include <algorithm>
#include <cmath>
#include <type_traits>

#include "cg_device.cuh"
#include "ring.cuh"
#include "tma.cuh"

namespace fea {

namespace {

// Block reduction of NV accumulators, then the grid-wide last-block step.
// Returns true in the last block, with totals in out[] valid in thread 0.
template <typename R, int NV>
__device__ __forceinline__ bool grid_reduce(Acc<R> (&acc)[NV], double* part, int stride, unsigned int* ticket,
                                            Acc<R> (&out)[NV]) {
    __shared__ typename Acc<R>::Packed sm[32 * NV];
    Acc<R> blk[NV];
    block_totals<NV, R>(acc, sm, blk);
    return grid_commit<NV, R>(blk, part, stride, ticket, sm, out);
}

// The loop body holds kLoopUnroll iteration kernels, since every pass of a
// graph WHILE loop costs a few microseconds of relaunch; a kernel that finds
// every field of its solve stopped is one of the extra copies of the last
// pass: it leaves the state alone and only confirms the loop's end.
constexpr int kLoopUnroll = 8;
template <typename R, int NF>
__device__ __forceinline__ bool solve_stopped(const StepArgs<R, NF>& a, const PhaseCtl<R, NF>& c) {
    if (a.probe) return false;
    if (blockIdx.x == 0 && threadIdx.x == 0) a.run->cg_launches += 1;
    if (c.any) return false;
    if (blockIdx.x == 0 && threadIdx.x == 0) signal_loop(a, false);
    return true;
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

// The set-up of a step's first solve (Gray-Scott with the guess buffers):
// the state becomes x_(n-1) and the start k_rhs formed becomes x (the two are
// equal without the extrapolation); a skipped step keeps both.  Every later
// step may then extrapolate.
template <typename R, int NF>
__device__ __forceinline__ void move_guess(const StepArgs<R, NF>& a) {
    if (((const volatile CgState*)a.cg)->stop) return;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < a.N; i += (int64_t)gridDim.x * blockDim.x) {
        const FV<R, NF> x = a.x[i];
        a.xprev[i] = x;
        a.x[i] = a.xg[i];
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) a.run->prev_valid = 1;
}

// Set-up of a solve: w0 = A z (z = D^-1 r0 from k_rhs / k_refine), delta0 =
// z.w0 and alpha0 = r0.z / delta0.
template <typename R, int NF, int WCH>
__global__ void __launch_bounds__(kBlock, (WCH <= 4 ? 6 : 4)) k_cgcg_init(StepArgs<R, NF> a) {
    __shared__ FV<R, NF> sm[kBlock / 32][32 * WCH];
    __shared__ typename Acc<R>::Packed red[32 * NF];
    if (a.guess_init && a.xg) move_guess(a);
    PhaseCtl<R, NF> c;
    c.load(a.cg);
    if (!c.any) {  // no field iterates (every solve converged or stopped): no product to set up
        if (blockIdx.x == 0 && threadIdx.x == 0) signal_loop(a, false);
        return;
    }
    FV<R, NF>* w = a.wb[a.defer ? 0 : c.par];
    const int wib = threadIdx.x >> 5;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    Acc<R> dot[NF];
    for (int64_t row0 = warp * 32; row0 < a.N; row0 += nwarps * 32)
        init_rows<R, NF, WCH>(a.rp, a.col, a.A, a.z, w, row0, a.N, sm[wib], dot);
    Acc<R> blk[NF], tot[NF];
    block_totals<NF>(dot, red, blk);
    if (grid_commit<NF>(blk, a.part, a.part_stride, a.tickets + 0, red, tot) && threadIdx.x == 0) {
        volatile CgState* cg = a.cg;
        finish_spmv<R, NF>(cg, &a.run->flags, c.act, tot);
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
    __shared__ FV<R, NF> sm[kBlock / 32][32 * WCH];
    __shared__ FV<R, NF> ut[kBlock];
    __shared__ typename Acc<R>::Packed red[32 * 3 * NF];
    grid_dependency_wait();
    PhaseCtl<R, NF> c;
    c.load(a.cg);
    if (solve_stopped(a, c)) return;
    CgVecs<R, NF> v;
    v.rp = a.rp;
    v.col = a.col;
    v.A = a.A;
    v.dinv = a.dinv;
    v.x = a.x;
    v.p = a.pp[0];
    v.r0 = a.rb[c.par];
    v.w0 = a.wb[c.par];
    v.s0 = a.sb[c.par];
    v.r1 = a.rb[c.par ^ 1];
    v.w1 = a.wb[c.par ^ 1];
    v.s1 = a.sb[c.par ^ 1];
    const int wib = threadIdx.x >> 5;
    Acc<R> dots[3 * NF];  // gamma', delta', |r'|^2
    for (int64_t tile0 = blockIdx.x * (int64_t)kBlock; tile0 < a.N; tile0 += (int64_t)gridDim.x * kBlock)
        cgcg_tile<R, NF, WCH>(v, c, tile0, a.N, sm[wib], ut, dots);
    grid_launch_dependents();
    Acc<R> blk[3 * NF], tot[3 * NF];
    block_totals<3 * NF>(dots, red, blk);
    if (grid_commit<3 * NF>(blk, a.part, a.part_stride, a.tickets + 1, red, tot) && threadIdx.x == 0)
        signal_loop(a, finish_cgcg<R, NF>(a.cg, &a.run->flags, c.act, tot));
}

// The same two kernels on the tile-ELL layout (variant 0): one block per
// 256-row tile (grid-stride), the tile's operand staged in dynamic shared
// memory (kTileRows + hmax entries).
template <typename R, int NF>
__device__ __forceinline__ EllView<R, NF> ell_view(const StepArgs<R, NF>& a) {
    return EllView<R, NF>{a.As, a.lcol, a.slice_off, a.halo_off, a.halo_col};
}

// Tile loop of the tile-ELL kernels: block b takes tiles b, b + G, ...;
// consecutive tiles alternate the two staging buffers of ut (each kTileRows +
// hmax entries of dynamic shared memory), and every tile's slice and halo
// references are loaded one tile ahead.
template <typename R, int NF, typename Body>
__device__ __forceinline__ void ell_tiles(const StepArgs<R, NF>& a, FV<R, NF>* ut, Body body) {
    const EllView<R, NF> e = ell_view(a);
    const int64_t ntiles = ceil_div(a.N, kTileRows);
    const int stride = kTileRows + a.hmax;
    EllTileRef ref = ell_ref(e, (int64_t)blockIdx.x, ntiles);
    int buf = 0;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const EllTileRef next = ell_ref(e, tile + gridDim.x, ntiles);
        body(e, tile, ref, ut + buf * stride);
        ref = next;
        buf ^= 1;
    }
}

template <typename R, int NF, int KPRE>
__global__ void __launch_bounds__(kBlock) k_cgcg_init_ell(StepArgs<R, NF> a) {
    extern __shared__ __align__(16) unsigned char dyn_smem[];
    FV<R, NF>* ut = reinterpret_cast<FV<R, NF>*>(dyn_smem);
    __shared__ typename Acc<R>::Packed red[32 * NF];
    if (a.guess_init && a.xg) move_guess(a);
    PhaseCtl<R, NF> c;
    c.load(a.cg);
    if (!c.any) {  // no field iterates (every solve converged or stopped): no product to set up
        if (blockIdx.x == 0 && threadIdx.x == 0) signal_loop(a, false);
        return;
    }
    FV<R, NF>* w = a.wb[a.defer ? 0 : c.par];
    Acc<R> dot[NF];
    ell_tiles(a, ut, [&](const EllView<R, NF>& e, int64_t tile, const EllTileRef& ref, FV<R, NF>* buf) {
        init_tile_ell<R, NF, KPRE>(e, a.z, w, tile, ref, a.N, buf, dot);
    });
    Acc<R> blk[NF], tot[NF];
    block_totals<NF>(dot, red, blk);
    if (grid_commit<NF>(blk, a.part, a.part_stride, a.tickets + 0, red, tot) && threadIdx.x == 0) {
        volatile CgState* cg = a.cg;
        finish_spmv<R, NF>(cg, &a.run->flags, c.act, tot);
        int any = 0;
#pragma unroll
        for (int f = 0; f < NF; f++) {
            cg->fresh[f] = 1;
            any |= cg->active[f];
        }
        signal_loop(a, any != 0);
    }
}

template <typename R, int NF, int KPRE>
__global__ void __launch_bounds__(kBlock) k_cgcg_iter_ell(StepArgs<R, NF> a) {
    extern __shared__ __align__(16) unsigned char dyn_smem[];
    FV<R, NF>* ut = reinterpret_cast<FV<R, NF>*>(dyn_smem);
    __shared__ typename Acc<R>::Packed red[32 * 3 * NF];
    grid_dependency_wait();
    PhaseCtl<R, NF> c;
    c.load(a.cg);
    if (solve_stopped(a, c)) return;
    CgVecs<R, NF> v;
    v.rp = a.rp;
    v.col = a.col;
    v.A = a.A;
    v.dinv = a.dinv;
    v.x = a.x;
    v.p = a.pp[0];
    v.r0 = a.rb[c.par];
    v.w0 = a.wb[c.par];
    v.s0 = a.sb[c.par];
    v.r1 = a.rb[c.par ^ 1];
    v.w1 = a.wb[c.par ^ 1];
    v.s1 = a.sb[c.par ^ 1];
    Acc<R> dots[3 * NF];
    ell_tiles(a, ut, [&](const EllView<R, NF>& e, int64_t tile, const EllTileRef& ref, FV<R, NF>* buf) {
        cgcg_tile_ell<R, NF, KPRE>(v, e, c, tile, ref, a.N, buf, dots);
    });
    grid_launch_dependents();
    Acc<R> blk[3 * NF], tot[3 * NF];
    block_totals<3 * NF>(dots, red, blk);
    if (grid_commit<3 * NF>(blk, a.part, a.part_stride, a.tickets + 1, red, tot) && threadIdx.x == 0)
        signal_loop(a, finish_cgcg<R, NF>(a.cg, &a.run->flags, c.act, tot));
}

// ---- variants 2, 3, 6, 7, 10, 11: tile-ELL streamed through shared memory -------
//
// Every input a tile streams is a few contiguous ranges: its operator values
// and 16-bit local columns (the tile's slices are consecutive) and its 256
// rows of r, w, s, D^-1, x and p.  Thread 0 moves them into one of NS stages
// of shared memory with bulk copies (cp.async.bulk, completing on the stage's
// mbarrier) stages ahead of the tile being computed, so the block computes on
// data already in shared memory while later tiles' data is in flight.  The
// halo operands of the next tile are gathered into registers during the
// current tile and staged after its product.  Every wait is bounded: on
// expiry the kernel raises FEA_STATUS_BREAKDOWN, waits (bounded) for the
// copies it issued and leaves the tile loop.  The template flags choose the
// refill point (LATE) and how an iteration is finished (DEFER: by the next
// launch, in every block; otherwise by this launch's last block).

// Byte offsets of one stage (all 16-byte aligned).
template <typename R, int NF>
struct StageLayout {
    size_t A, L, V, U, bar, bytes;
    __host__ __device__ StageLayout(int emax, int hmax) {
        const size_t fv = sizeof(FV<R, NF>);
        auto al = [](size_t x) { return (x + 15) & ~(size_t)15; };
        A = 0;
        L = al(A + fv * (size_t)emax);
        V = al(L + 2 * (size_t)emax);
        U = al(V + 6 * fv * (size_t)kTileRows);
        bar = al(U + fv * (size_t)(kTileRows + hmax));
        bytes = al(bar + 8);
    }
};

// The vectors a stage holds, in this order.
enum { kVr = 0, kVw = 1, kVs = 2, kVd = 3, kVx = 4, kVp = 5 };

// Thread 0: bulk copies of tile `tile` (entries e0 .. e1 of the tile-ELL
// arrays) into stage S, after the block's last read of S and a proxy fence.
template <typename R, int NF>
__device__ void stage_tile(unsigned char* S, const StageLayout<R, NF>& L, const StepArgs<R, NF>& a,
                           const CgVecs<R, NF>& v, int64_t tile, int32_t e0, int32_t e1) {
    uint64_t* bar = reinterpret_cast<uint64_t*>(S + L.bar);
    const uint32_t nA = (uint32_t)(e1 - e0) * (uint32_t)sizeof(FV<R, NF>);
    const uint32_t nL = (uint32_t)(e1 - e0) * 2u;
    const uint32_t nV = (uint32_t)kTileRows * (uint32_t)sizeof(FV<R, NF>);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    mbar_arrive_expect_tx(bar, nA + nL + 6 * nV);
    if (nA) {
        const uint64_t pol = l2_evict_first_policy();
        bulk_g2s_hint(S + L.A, a.As + e0, nA, bar, pol);
        bulk_g2s_hint(S + L.L, a.lcol + e0, nL, bar, pol);
    }
    const int64_t r0 = tile * kTileRows;
    const FV<R, NF>* src[6] = {v.r0 + r0, v.w0 + r0, v.s0 + r0, v.dinv + r0, v.x + r0, v.p + r0};
    const uint64_t vpol = l2_evict_last_policy();
#pragma unroll
    for (int k = 0; k < 6; k++) bulk_g2s_hint(S + L.V + (size_t)k * nV, src[k], nV, bar, vpol);
}

// The first copies of a stage in two parts: the tile's operator entries
// (constant through a solve; issued before the dependency wait) raise the
// expected bytes without arriving, and its rows of r, w, s, D^-1, x and p
// arrive with theirs once the previous iteration's vectors are visible.
template <typename R, int NF>
__device__ void stage_entries(unsigned char* S, const StageLayout<R, NF>& L, const StepArgs<R, NF>& a, int32_t e0,
                              int32_t e1) {
    uint64_t* bar = reinterpret_cast<uint64_t*>(S + L.bar);
    const uint32_t nA = (uint32_t)(e1 - e0) * (uint32_t)sizeof(FV<R, NF>);
    const uint32_t nL = (uint32_t)(e1 - e0) * 2u;
    if (!nA) return;
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    mbar_expect_tx(bar, nA + nL);
    const uint64_t pol = l2_evict_first_policy();
    bulk_g2s_hint(S + L.A, a.As + e0, nA, bar, pol);
    bulk_g2s_hint(S + L.L, a.lcol + e0, nL, bar, pol);
}
template <typename R, int NF>
__device__ void stage_rows(unsigned char* S, const StageLayout<R, NF>& L, const CgVecs<R, NF>& v, int64_t tile) {
    uint64_t* bar = reinterpret_cast<uint64_t*>(S + L.bar);
    const uint32_t nV = (uint32_t)kTileRows * (uint32_t)sizeof(FV<R, NF>);
    mbar_arrive_expect_tx(bar, 6 * nV);
    const int64_t r0 = tile * kTileRows;
    const FV<R, NF>* src[6] = {v.r0 + r0, v.w0 + r0, v.s0 + r0, v.dinv + r0, v.x + r0, v.p + r0};
    const uint64_t vpol = l2_evict_last_policy();
#pragma unroll
    for (int k = 0; k < 6; k++) bulk_g2s_hint(S + L.V + (size_t)k * nV, src[k], nV, bar, vpol);
}


// The per-tile references (entry ranges, slice offsets, halo lists) are loaded
// ahead of use in a software pipeline, so that no load waits on another
// within a tile: a tile's halo offset is loaded one tile before its halo
// column, which is loaded one tile before the column's operands are gathered,
// which happens one tile before the tile itself.
//
// LATE = false: thread 0 refills a stage after a third block barrier at the
// end of the tile that used it.  LATE = true: after the next tile's first
// barrier, which already orders every read of the stage before the refill;
// two barriers per tile.
template <typename R, int NF, int NS, bool LATE, bool DEFER>
__global__ void __launch_bounds__(kBlock) k_cgcg_iter_stream(StepArgs<R, NF> a) {
    extern __shared__ __align__(16) unsigned char dyn_smem[];
    __shared__ typename Acc<R>::Packed red[32 * 3 * NF];
    __shared__ int armed[NS];
    const StageLayout<R, NF> L(a.emax, a.hmax);
    const int t = threadIdx.x, lane = t & 31, wib = t >> 5, j = halo_slot(t);
    const int64_t ntiles = ceil_div(a.N, kTileRows), G = gridDim.x, t0 = blockIdx.x;
    auto stage = [&](int b) { return dyn_smem + (size_t)b * L.bytes; };
    auto bar_of = [&](int b) { return reinterpret_cast<uint64_t*>(stage(b) + L.bar); };
    auto ut_of = [&](int b) { return reinterpret_cast<FV<R, NF>*>(stage(b) + L.U); };
    // first halo entry and halo count of tile `tile` (0, 0 past the end)
    auto halo_head = [&](int64_t tile, int32_t& h0, int32_t& cnt) {
        h0 = cnt = 0;
        if (tile < ntiles) {
            h0 = a.halo_off[tile];
            cnt = a.halo_off[tile + 1] - h0;
        }
    };
    // halo column of this thread's slot (-1: none)
    auto halo_col = [&](int32_t h0, int32_t cnt) { return j < cnt ? a.halo_col[h0 + j] : -1; };
    // this warp's slice of tile `tile`: offset in the tile's entries, width
    auto slice_ref = [&](int64_t tile, int32_t& sb, int32_t& sw) {
        sb = sw = 0;
        if (tile < ntiles) {
            const int64_t sl = tile * (kTileRows / 32) + wib;
            const int32_t s0 = a.slice_off[sl];
            sb = s0 - a.slice_off[tile * (kTileRows / 32)];
            sw = (a.slice_off[sl + 1] - s0) >> 5;
        }
    };
    // entry range of tile `tile` (thread 0's copies)
    auto entries = [&](int64_t tile, int32_t& e0, int32_t& e1) {
        e0 = e1 = 0;
        if (tile < ntiles) {
            e0 = a.slice_off[tile * (kTileRows / 32)];
            e1 = a.slice_off[(tile + 1) * (kTileRows / 32)];
        }
    };
    // Before the dependency wait, only what no earlier kernel writes: the
    // stages' barriers, the first tiles' operator entries (bulk copies) and
    // the tile references.  Under a programmatic launch this overlaps the end
    // of the previous iteration.
    if (t == 0) {
        for (int b = 0; b < NS; b++) {
            mbar_init(bar_of(b), 1);
            armed[b] = 0;
        }
        mbar_fence_init();
        for (int b = 0; b < NS; b++)
            if (t0 + b * G < ntiles) {
                int32_t e0, e1;
                entries(t0 + b * G, e0, e1);
                stage_entries(stage(b), L, a, e0, e1);
                armed[b] = 1;
            }
    }
    // pipeline registers: halo column and count of the next tile, halo head
    // of the tile after next, this tile's slice, and (thread 0) the entry
    // range of the next refill
    int32_t hcol, hcnt, hh0, hhc, sb, sw, re0 = 0, re1 = 0;
    {
        int32_t h0;
        halo_head(t0 + G, h0, hcnt);
        hcol = halo_col(h0, hcnt);
    }
    halo_head(t0 + 2 * G, hh0, hhc);
    slice_ref(t0, sb, sw);
    if (t == 0) entries(t0 + NS * G, re0, re1);
    int32_t fh0, fcnt;  // the first tile's halo; this thread's slot t of it
    halo_head(t0, fh0, fcnt);
    const int32_t fcol = t < fcnt ? a.halo_col[fh0 + t] : -1;
    grid_dependency_wait();
    PhaseCtl<R, NF> c;
    CgVecs<R, NF> v;
    v.rp = a.rp;
    v.col = a.col;
    v.A = a.A;
    v.dinv = a.dinv;
    v.x = a.x;
    v.p = a.pp[0];
    if constexpr (!DEFER) {
        // the slot's operands from both parity buffers, in flight with the
        // state load that tells which parity is current
        FV<R, NF> fr[2], fw[2], fs[2], fd;
        if (fcol >= 0) {
            fd = ldv(a.dinv + fcol, false);
#pragma unroll
            for (int q = 0; q < 2; q++) {
                fr[q] = ldv(a.rb[q] + fcol, false);
                fw[q] = ldv(a.wb[q] + fcol, false);
                fs[q] = ldv(a.sb[q] + fcol, false);
            }
        }
        c.load(a.cg);
        if (solve_stopped(a, c)) {
            if (t == 0)  // the entry copies land before the block exits
                for (int b = 0; b < NS; b++)
                    if (armed[b]) {
                        mbar_arrive(bar_of(b));
                        mbar_wait(bar_of(b), 0u);
                    }
            return;
        }
        v.r0 = a.rb[c.par];
        v.w0 = a.wb[c.par];
        v.s0 = a.sb[c.par];
        v.r1 = a.rb[c.par ^ 1];
        v.w1 = a.wb[c.par ^ 1];
        v.s1 = a.sb[c.par ^ 1];
        if (t == 0)
            for (int b = 0; b < NS; b++)
                if (armed[b]) stage_rows(stage(b), L, v, t0 + b * G);
        // the first tile's halo, straight into stage 0 (slots beyond 256 directly)
        if (fcol >= 0) {
            const bool q = c.par != 0;  // selects, not a dynamic index (keeps the pairs in registers)
            const FV<R, NF> ro = q ? fr[1] : fr[0], wo = q ? fw[1] : fw[0], so = q ? fs[1] : fs[0];
            FV<R, NF> sn, rn, u2;
            cg_advance(c, ro, wo, c.need_old ? so : wo, fd, sn, rn, u2);
            ut_of(0)[kTileRows + t] = u2;
        }
    } else {
        // Deferred finish.  The node's buffer parity q is static, so the
        // rows' copies and the first halo loads start at once; meanwhile
        // every block reads the state of parity q ^ 1 and, when the previous
        // launch left an iteration pending, merges that launch's block
        // partials (fixed order: every block gets the same scalars) and
        // finishes it.  Block 0 publishes the state of parity q.
        const int q = a.par;
        v.r0 = a.rb[q];
        v.w0 = a.wb[q];
        v.s0 = a.sb[q];
        v.r1 = a.rb[q ^ 1];
        v.w1 = a.wb[q ^ 1];
        v.s1 = a.sb[q ^ 1];
        if (t == 0)
            for (int b = 0; b < NS; b++)
                if (armed[b]) stage_rows(stage(b), L, v, t0 + b * G);
        FV<R, NF> fr, fw, fs, fd;
        if (fcol >= 0) {
            fr = ldv(v.r0 + fcol, false);
            fw = ldv(v.w0 + fcol, false);
            fs = ldv(v.s0 + fcol, false);
            fd = ldv(v.dinv + fcol, false);
        }
        __shared__ CgState st;
        __shared__ unsigned int sflags;
        {
            const int* src = reinterpret_cast<const int*>(q ? a.cg_alt : a.cg);
            int* dst = reinterpret_cast<int*>(&st);
            for (int k = t; k < (int)(sizeof(CgState) / 4); k += kBlock) dst[k] = __ldcg(src + k);
        }
        if (t == 0) sflags = 0u;
        __syncthreads();
        const bool had_pending = st.pending != 0;
        if (had_pending && !a.probe) {
            Acc<R> y[3 * NF], tot[3 * NF];
            const auto* pp =
                reinterpret_cast<const typename Acc<R>::Packed*>(a.part + (q ? 8 * (int64_t)a.part_stride : 0));
            merge_partials<3 * NF, R>(y, pp, a.part_stride, 1, 0, (int64_t)gridDim.x);
            block_totals<3 * NF, R>(y, red, tot);
            if (t == 0) {
                int act[NF];
#pragma unroll
                for (int f = 0; f < NF; f++) act[f] = st.active[f];
                finish_cgcg<R, NF>((volatile CgState*)&st, &sflags, act, tot);
                st.pending = 0;
            }
            __syncthreads();
        }
        c.set(st.iter, (const volatile CgState*)&st);
        c.par = q;
        // Only a solve's first launch iterates without finishing one: a
        // launch that would iterate on a state with neither (an inconsistent
        // state) stops the solve instead, so the loop always ends.
        const bool stray = !a.probe && !had_pending && c.any && c.need_old;
        const bool go = c.any && !stray;
        if (t == 0 && blockIdx.x == 0 && !a.probe) {
            a.run->cg_launches += 1;
            if (sflags) atomicOr(&a.run->flags, sflags);
            CgState* out = q ? a.cg : a.cg_alt;
            const int* src = reinterpret_cast<const int*>(&st);
            int* dst = reinterpret_cast<int*>(out);
            for (int k = 0; k < (int)(sizeof(CgState) / 4); k++) dst[k] = src[k];
            if (go) {  // this launch iterates; the next one finishes it
                out->pending = 1;
#pragma unroll
                for (int f = 0; f < NF; f++) out->fresh[f] = 0;
            } else if (stray) {
#pragma unroll
                for (int f = 0; f < NF; f++) out->active[f] = 0;
                atomicOr(&a.run->flags, FEA_STATUS_BREAKDOWN);
            }
            signal_loop(a, go);
        }
        if (!go && !a.probe) {  // every field stopped: the stages' copies land, then the block leaves
            if (t == 0)
                for (int b = 0; b < NS; b++)
                    if (armed[b]) mbar_wait(bar_of(b), 0u);
            return;
        }
        if (fcol >= 0) {
            FV<R, NF> sn, rn, u2;
            cg_advance(c, fr, fw, c.need_old ? fs : fw, fd, sn, rn, u2);
            ut_of(0)[kTileRows + t] = u2;
        }
    }
    for (int32_t h = kBlock + t; h < fcnt; h += kBlock) ut_of(0)[kTileRows + h] = cg_u_at(v, c, a.halo_col[fh0 + h]);
    __syncthreads();
    Acc<R> dots[3 * NF];
    uint32_t phases = 0u;  // bit b: parity of stage b's next phase (a register, not a local array)
    bool ok = true;
    int b = 0;
    int64_t refill = -1;  // LATE: tile whose stage (the previous one) thread 0 refills next
    int bprev = 0;
    for (int64_t tile = t0; tile < ntiles; tile += G) {
        FV<R, NF>* ut = ut_of(b);
        const int bn = b + 1 == NS ? 0 : b + 1;
        // operands of the next tile's halo slot (column loaded one tile ago)
        FV<R, NF> hr, hw, hs, hd;
        if (hcol >= 0) {
            hr = ldv(v.r0 + hcol, false);
            hw = ldv(v.w0 + hcol, false);
            hd = ldv(v.dinv + hcol, false);
            hs = hw;
            if (c.need_old) hs = ldv(v.s0 + hcol, false);
        }
        // references further ahead, each from values already loaded
        const int32_t hcol2 = halo_col(hh0, hhc), hcnt2 = hhc;
        int32_t hh0n, hhcn, sb2, sw2;
        halo_head(tile + 3 * G, hh0n, hhcn);
        slice_ref(tile + G, sb2, sw2);
        const int32_t ce0 = re0, ce1 = re1;
        if (t == 0) entries((LATE ? tile : tile + G) + NS * G, re0, re1);  // the next refill
        const bool got = mbar_wait(bar_of(b), (phases >> b) & 1u);
        phases ^= 1u << b;
        if (!__syncthreads_and(got)) {
            ok = false;
            break;
        }
        if (t == 0) {
            armed[b] = 0;
            if (LATE && refill >= 0) {
                stage_tile(stage(bprev), L, a, v, refill, ce0, ce1);
                armed[bprev] = 1;
            }
        }
        if (LATE) {
            refill = tile + NS * G < ntiles ? tile + NS * G : -1;
            bprev = b;
        }
        const FV<R, NF>* V = reinterpret_cast<const FV<R, NF>*>(stage(b) + L.V);
        const int64_t row = tile * kTileRows + t;
        FV<R, NF> un;
#pragma unroll
        for (int f = 0; f < NF; f++) un.v[f] = 0;
        if (row < a.N) {
            const FV<R, NF> ro = V[kVr * kTileRows + t], wo = V[kVw * kTileRows + t], d = V[kVd * kTileRows + t];
            FV<R, NF> so = wo;
            if (c.need_old) so = V[kVs * kTileRows + t];
            FV<R, NF> x = V[kVx * kTileRows + t], p = V[kVp * kTileRows + t];
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
        const FV<R, NF>* As = reinterpret_cast<const FV<R, NF>*>(stage(b) + L.A) + sb + lane;
        const uint16_t* Ls = reinterpret_cast<const uint16_t*>(stage(b) + L.L) + sb + lane;
        FV<R, NF> wn;
#pragma unroll
        for (int f = 0; f < NF; f++) wn.v[f] = 0;
#pragma unroll 4
        for (int k = 0; k < sw; k++) {
            const FV<R, NF> av = As[32 * k];
            const FV<R, NF> g = ut[Ls[32 * k]];
#pragma unroll
            for (int f = 0; f < NF; f++) wn.v[f] = fmar(av.v[f], g.v[f], wn.v[f]);
        }
        if (row < a.N) {
            v.w1[row] = wn;
#pragma unroll
            for (int f = 0; f < NF; f++) dots[NF + f].add_prod(wn.v[f], un.v[f]);
        }
        // the next tile's halo into its stage (free since that stage's last tile)
        if (hcol >= 0) {
            FV<R, NF> sn, rn, u2;
            cg_advance(c, hr, hw, hs, hd, sn, rn, u2);
            ut_of(bn)[kTileRows + j] = u2;
        }
        if (hcnt > kBlock && tile + G < ntiles) {  // halos beyond 256 columns: the rest directly
            const int32_t h0 = a.halo_off[tile + G];
            for (int32_t h = kBlock + t; h < hcnt; h += kBlock)
                ut_of(bn)[kTileRows + h] = cg_u_at(v, c, a.halo_col[h0 + h]);
        }
        if (!LATE) {
            __syncthreads();  // this stage is free again
            if (t == 0 && tile + NS * G < ntiles) {
                stage_tile(stage(b), L, a, v, tile + NS * G, ce0, ce1);
                armed[b] = 1;
            }
        }
        hcol = hcol2;
        hcnt = hcnt2;
        hh0 = hh0n;
        hhc = hhcn;
        sb = sb2;
        sw = sw2;
        b = bn;
    }
    grid_launch_dependents();
    if (!ok) {
        if (t == 0) {
            atomicOr(&a.run->flags, FEA_STATUS_BREAKDOWN);
            for (int q = 0; q < NS; q++)  // copies still in flight land before the block exits
                if (armed[q]) mbar_wait(bar_of(q), (phases >> q) & 1u);
        }
        __syncthreads();
    }
    Acc<R> blk[3 * NF], tot[3 * NF];
    block_totals<3 * NF>(dots, red, blk);
    if constexpr (DEFER) {  // the block's partials of parity q; the next launch merges them
        if (t == 0 && !a.probe) {
            auto* pp = reinterpret_cast<typename Acc<R>::Packed*>(a.part + (a.par ? 0 : 8 * (int64_t)a.part_stride));
#pragma unroll
            for (int k = 0; k < 3 * NF; k++) pp[k * a.part_stride + blockIdx.x] = blk[k].pack();
        }
    } else if (grid_commit<3 * NF>(blk, a.part, a.part_stride, a.tickets + 1, red, tot) && threadIdx.x == 0) {
        signal_loop(a, finish_cgcg<R, NF>(a.cg, &a.run->flags, c.act, tot));
    }
}

// ---- variant 13: tile-ELL with direct loads, pipelined one tile ahead -------------
//
// Each warp multiplies its 32-row slice of a tile from registers.  The
// slice's operator entries and 16-bit local columns go straight from global
// memory into the registers of the row's thread (entry k of the slice's 32
// rows is one coalesced request), and each register takes the next tile's
// entry as soon as the product has used it, so a whole tile of work covers the
// DRAM latency of every entry.  The rows' r, w, s, D^-1, x, p and the operands
// of the thread's halo slot are loaded for the next tile as soon as this
// tile's row update and halo have used their registers; the per-tile
// references (slice offsets, halo heads and columns) run one and two tiles
// further ahead.  No thread copies for others: the only
// block barrier of a tile orders its u' slice, and two u' buffers alternate
// between consecutive tiles.  The iteration is finished by the next launch
// (deferred finish, as variants 10 and 11), and both block reductions give
// each value to one warp: at the start, warp k merges value k of every
// block's partials; at the end, value k of the block's threads.


// Totals of NV values over nb block partials p[k * stride + b]: warp k merges
// value k (lane l takes b = l, l + 32, ... with 16 loads in flight, then a
// shuffle tree), a fixed order; lane 0 of warp k leaves total k in sm[k].
// Needs NV <= the block's warps; every thread calls it (no barrier inside).
template <int NV, typename R>
__device__ __forceinline__ void merge_partials_by_warp(const typename Acc<R>::Packed* p, int64_t stride, int nb,
                                                       typename Acc<R>::Packed* sm) {
    using P = typename Acc<R>::Packed;
    constexpr int B = 16;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (w >= NV) return;
    Acc<R> y;
    for (int base = lane; base < nb; base += 32 * B) {
        P v[B];
#pragma unroll
        for (int u = 0; u < B; u++)
            if (base + 32 * u < nb) v[u] = __ldcg(&p[w * stride + base + 32 * u]);
#pragma unroll
        for (int u = 0; u < B; u++)
            if (base + 32 * u < nb) y.merge(Acc<R>::unpack(v[u]));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) y.shfl_add(o);
    if (lane == 0) sm[w] = y.pack();
}

// Deferred finish at the start of a launch of buffer parity q (variants 12 to
// 15): every block reads the state of parity q ^ 1 into st; when the previous
// launch left an iteration pending, warp k merges value k of that launch's
// block partials (a fixed order, so every block gets the same scalars) and
// thread 0 finishes the iteration.  Block 0 publishes the state of parity q
// and the loop condition.  Returns whether this launch iterates (c set).
// Only a solve's first launch iterates without finishing one: a launch that
// would iterate on a state with neither stops the solve instead.
template <typename R, int NF>
__device__ __forceinline__ bool deferred_head(const StepArgs<R, NF>& a, int q, CgState& st, unsigned int& sflags,
                                              typename Acc<R>::Packed* red, PhaseCtl<R, NF>& c) {
    using P = typename Acc<R>::Packed;
    constexpr int NV = 3 * NF;
    const int t = threadIdx.x;
    {
        const int* src = reinterpret_cast<const int*>(q ? a.cg_alt : a.cg);
        int* dst = reinterpret_cast<int*>(&st);
        for (int k = t; k < (int)(sizeof(CgState) / 4); k += blockDim.x) dst[k] = __ldcg(src + k);
    }
    if (t == 0) sflags = 0u;
    __syncthreads();
    const bool had_pending = st.pending != 0;
    if (had_pending && !a.probe) {
        const P* pp = reinterpret_cast<const P*>(a.part + (q ? 8 * (int64_t)a.part_stride : 0));
        merge_partials_by_warp<NV, R>(pp, a.part_stride, (int)gridDim.x, red);
        __syncthreads();
        if (t == 0) {
            Acc<R> tot[NV];
#pragma unroll
            for (int k = 0; k < NV; k++) tot[k] = Acc<R>::unpack(red[k]);
            int act[NF];
#pragma unroll
            for (int f = 0; f < NF; f++) act[f] = st.active[f];
            finish_cgcg<R, NF>((volatile CgState*)&st, &sflags, act, tot);
            st.pending = 0;
        }
        __syncthreads();
    }
    c.set(st.iter, (const volatile CgState*)&st);
    c.par = q;
    const bool stray = !a.probe && !had_pending && c.any && c.need_old;
    const bool go = c.any && !stray;
    if (t == 0 && blockIdx.x == 0 && !a.probe) {
        a.run->cg_launches += 1;
        if (sflags) atomicOr(&a.run->flags, sflags);
        CgState* out = q ? a.cg : a.cg_alt;
        const int* src = reinterpret_cast<const int*>(&st);
        int* dst = reinterpret_cast<int*>(out);
        for (int k = 0; k < (int)(sizeof(CgState) / 4); k++) dst[k] = src[k];
        if (go) {  // this launch iterates; the next one finishes it
            out->pending = 1;
#pragma unroll
            for (int f = 0; f < NF; f++) out->fresh[f] = 0;
        } else if (stray) {
#pragma unroll
            for (int f = 0; f < NF; f++) out->active[f] = 0;
            atomicOr(&a.run->flags, FEA_STATUS_BREAKDOWN);
        }
        signal_loop(a, go);
    }
    return go;
}

// The block's partials of parity q for the next launch to merge: every
// thread's accumulators through shared memory (red: NV * blockDim.x slots),
// value k summed by warp k.
template <typename R, int NV>
__device__ __forceinline__ void store_block_partials(const StepArgs<R, NV / 3>& a, int q, const Acc<R> (&dots)[NV],
                                                     typename Acc<R>::Packed* red) {
    using P = typename Acc<R>::Packed;
    const int t = threadIdx.x, lane = t & 31, wib = t >> 5;
#pragma unroll
    for (int k = 0; k < NV; k++) red[k * kBlock + t] = dots[k].pack();
    __syncthreads();
    if (wib < NV) {
        Acc<R> y = Acc<R>::unpack(red[wib * kBlock + lane]);
#pragma unroll
        for (int i = 1; i < kBlock / 32; i++) y.merge(Acc<R>::unpack(red[wib * kBlock + lane + 32 * i]));
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) y.shfl_add(o);
        if (lane == 0 && !a.probe) {
            P* pp = reinterpret_cast<P*>(a.part + (q ? 0 : 8 * (int64_t)a.part_stride));
            pp[wib * a.part_stride + blockIdx.x] = y.pack();
        }
    }
}

// PAR: the launch's buffer parity (a.par), a template argument so that the
// parity's vector pointers stay constant operands.  Indices are 32-bit (N and
// the layout's entry count are below 2^31).
template <typename R, int NF, int K, int PAR, int MINB>
__global__ void __launch_bounds__(kBlock, MINB) k_cgcg_iter_direct(StepArgs<R, NF> a) {
    using V = FV<R, NF>;
    using P = typename Acc<R>::Packed;
    constexpr int NV = 3 * NF;
    static_assert(NV <= kBlock / 32, "one warp per reduced value");
    static_assert(K % 2 == 0, "columns come in pairs");
    extern __shared__ __align__(16) unsigned char dyn_smem[];
    __shared__ P red[NV * kBlock];
    __shared__ CgState st;
    __shared__ unsigned int sflags;
    V* const ubuf = reinterpret_cast<V*>(dyn_smem);
    const int ustride = kTileRows + a.hmax;
    const int t = threadIdx.x, lane = t & 31, wib = t >> 5, j = halo_slot(t);
    const int ntiles = (int)ceil_div(a.N, kTileRows), G = (int)gridDim.x, t0 = (int)blockIdx.x;
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
            sb = a.slice_off[sl];
            sw = (a.slice_off[sl + 1] - sb) >> 5;
        }
    };
    // Before the dependency wait, only what no earlier kernel writes: the
    // tile references and the first tile's operator entries.
    int32_t sb, sw, sbn, swn;
    slice_ref(t0, sb, sw);
    slice_ref(t0 + G, sbn, swn);
    V av[K];
    uint32_t lc[K / 2];  // column pairs
    {
        const uint64_t pol_once = l2_evict_first_policy();
#pragma unroll
        for (int k = 0; k < K; k++)
            if (k < sw) av[k] = ld_once(a.As + sb + 32 * k + lane, pol_once);
#pragma unroll
        for (int m = 0; m < K / 2; m++)
            if (2 * m < sw) lc[m] = ld_once(a.lcol2 + sb + 32 * m + lane, pol_once);
    }
    // halo pipeline: this tile's head and slot column, the next tile's, and
    // the head of the tile after next
    int32_t h0c, hcc, h0n, hcn, hh0, hhc;
    halo_head(t0, h0c, hcc);
    halo_head(t0 + G, h0n, hcn);
    halo_head(t0 + 2 * G, hh0, hhc);
    const int32_t fcol = j < hcc ? a.halo_col[h0c + j] : -1;
    int32_t hcoln = j < hcn ? a.halo_col[h0n + j] : -1;
    grid_dependency_wait();
    constexpr int q = PAR;  // buffer parity of this launch (static per graph node)
    CgVecs<R, NF> v;
    v.rp = a.rp;
    v.col = a.col;
    v.A = a.A;
    v.dinv = a.dinv;
    v.x = a.x;
    v.p = a.pp[0];
    v.r0 = a.rb[q];
    v.w0 = a.wb[q];
    v.s0 = a.sb[q];
    v.r1 = a.rb[q ^ 1];
    v.w1 = a.wb[q ^ 1];
    v.s1 = a.sb[q ^ 1];
    // the first tile's rows and halo slot, in flight while the previous
    // iteration is finished
    V cr, cw, cs, cd, cx, cp, hr, hw, hs, hd;
    {
        const uint64_t pol_keep = l2_evict_last_policy();
        const int row = t0 * kTileRows + t;  // every vector holds whole tiles
        if (t0 < ntiles) {
            cr = ld_keep(v.r0 + row, pol_keep);
            cw = ld_keep(v.w0 + row, pol_keep);
            cs = ld_keep(v.s0 + row, pol_keep);
            cd = ld_keep(v.dinv + row, pol_keep);
            cx = ld_keep(v.x + row, pol_keep);
            cp = ld_keep(v.p + row, pol_keep);
        }
        if (fcol >= 0) {
            hr = ld_keep(v.r0 + fcol, pol_keep);
            hw = ld_keep(v.w0 + fcol, pol_keep);
            hs = ld_keep(v.s0 + fcol, pol_keep);
            hd = ld_keep(v.dinv + fcol, pol_keep);
        }
    }
    PhaseCtl<R, NF> c;
    const bool go = deferred_head<R, NF>(a, q, st, sflags, red, c);
    if (!go && !a.probe) return;  // every field stopped (plain loads in flight need no wait)
    Acc<R> dots[NV];  // gamma', delta', |r'|^2 per field
    int buf = 0;
    for (int tile = t0; tile < ntiles; tile += G) {
        V* ut = ubuf + buf * ustride;
        const int row = tile * kTileRows + t;
        V un;
#pragma unroll
        for (int f = 0; f < NF; f++) un.v[f] = 0;
        if (row < a.N) {
            V sn, rn;
            cg_advance(c, cr, cw, c.need_old ? cs : cw, cd, sn, rn, un);
#pragma unroll
            for (int f = 0; f < NF; f++) {
                if (c.act[f]) {
                    const R ui = cd.v[f] * cr.v[f];
                    cp.v[f] = c.fresh[f] ? ui : fmar(c.beta[f], cp.v[f], ui);
                    cx.v[f] = fmar(c.alpha[f], cp.v[f], cx.v[f]);
                }
                dots[f].add_prod(rn.v[f], un.v[f]);
                dots[2 * NF + f].add_prod(rn.v[f], rn.v[f]);
            }
            v.x[row] = cx;
            v.p[row] = cp;
            v.r1[row] = rn;
            v.s1[row] = sn;
        }
        ut[t] = un;
        // the row's registers are free: the next tile's rows go in flight
        // now, ahead of the halo, the barrier and the product
        const uint64_t pol_keep = l2_evict_last_policy();
        const int nt = tile + G;
        if (nt < ntiles) {
            const int nrow = nt * kTileRows + t;
            cr = ld_keep(v.r0 + nrow, pol_keep);
            cw = ld_keep(v.w0 + nrow, pol_keep);
            cs = ld_keep(v.s0 + nrow, pol_keep);
            cd = ld_keep(v.dinv + nrow, pol_keep);
            cx = ld_keep(v.x + nrow, pol_keep);
            cp = ld_keep(v.p + nrow, pol_keep);
        }
        if (j < hcc) {
            V sn, rn, u2;
            cg_advance(c, hr, hw, c.need_old ? hs : hw, hd, sn, rn, u2);
            ut[kTileRows + j] = u2;
        }
        if (hcoln >= 0) {  // the next tile's halo slot operands
            hr = ld_keep(v.r0 + hcoln, pol_keep);
            hw = ld_keep(v.w0 + hcoln, pol_keep);
            hs = ld_keep(v.s0 + hcoln, pol_keep);
            hd = ld_keep(v.dinv + hcoln, pol_keep);
        }
        for (int32_t h = kBlock + t; h < hcc; h += kBlock)  // halos beyond 256 columns: directly
            ut[kTileRows + h] = cg_u_at(v, c, a.halo_col[h0c + h]);
        __syncthreads();
        // references further ahead, each from values loaded a tile ago
        h0c = h0n;
        hcc = hcn;
        hcoln = j < hhc ? a.halo_col[hh0 + j] : -1;
        h0n = hh0;
        hcn = hhc;
        halo_head(tile + 3 * G, hh0, hhc);
        int32_t sb2, sw2;
        slice_ref(tile + 2 * G, sb2, sw2);
        // the product; each register takes the next tile's entry once used
        const uint64_t pol_once = l2_evict_first_policy();
        V wn;
#pragma unroll
        for (int f = 0; f < NF; f++) wn.v[f] = 0;
#pragma unroll
        for (int k = 0; k < K; k++) {
            if (k < sw) {
                const V g = ut[(k & 1) ? lc[k / 2] >> 16 : lc[k / 2] & 0xffffu];
#pragma unroll
                for (int f = 0; f < NF; f++) wn.v[f] = fmar(av[k].v[f], g.v[f], wn.v[f]);
            }
            if (k < swn) av[k] = ld_once(a.As + sbn + 32 * k + lane, pol_once);
            if ((k & 1) && k - 1 < swn) lc[k / 2] = ld_once(a.lcol2 + sbn + 32 * (k / 2) + lane, pol_once);
        }
        for (int k = K; k < sw; k++) {  // rows longer than the registers hold
            const V ak = ld_once(a.As + sb + 32 * k + lane, pol_once);
            const V g = ut[ld_once_u16(a.lcol + sb + 32 * k + lane, pol_once)];
#pragma unroll
            for (int f = 0; f < NF; f++) wn.v[f] = fmar(ak.v[f], g.v[f], wn.v[f]);
        }
        if (row < a.N) {
            v.w1[row] = wn;
#pragma unroll
            for (int f = 0; f < NF; f++) dots[NF + f].add_prod(wn.v[f], un.v[f]);
        }
        sb = sbn;
        sw = swn;
        sbn = sb2;
        swn = sw2;
        buf ^= 1;
    }
    grid_launch_dependents();
    __syncthreads();  // red[] held the start-of-launch totals
    store_block_partials<R, NV>(a, q, dots, red);
}

// ---- variants 14 and 15: direct row loads, operator streamed by a bulk-copy ring ---
//
// Variant 13's structure (rows, halo and references loaded by the threads a
// tile ahead, one block barrier per tile, deferred finish) with the operator
// entries and their 16-bit local columns moved by bulk copies (cp.async.bulk
// on an mbarrier per stage) into a ring of S shared-memory stages, S - 1 tiles
// ahead of the product: the DRAM stream holds no registers, so it runs further
// ahead than register prefetches can.  Thread 0 refills the stage of the
// previous tile after the current tile's barrier (every warp has finished
// that tile's product by then).  Each warp waits for its tile's stage on its
// own, with a bounded wait; an expired wait raises FEA_STATUS_BREAKDOWN at the
// end of the launch, after thread 0 has waited (bounded) for the copies it
// issued.

// Each thread sums its rows' inner products in R with fused multiply-adds (a
// dozen rows per launch on the benchmark mesh); the block and grid totals
// carry the handle's accumulators (float-float for FP32).  Against
// float-float sums per thread: the same iteration counts, 5% less time per
// launch.
template <typename R, int NF, int S, int PAR, int MINB>
__global__ void __launch_bounds__(kBlock, MINB) k_cgcg_iter_ring(StepArgs<R, NF> a) {
    using V = FV<R, NF>;
    using P = typename Acc<R>::Packed;
    constexpr int NV = 3 * NF;
    static_assert(NV <= kBlock / 32, "one warp per reduced value");
    static_assert(S >= 2 && S <= 8, "ring depth");
    extern __shared__ __align__(16) unsigned char dyn_smem[];  // bulk copies need 16-byte destinations
    __shared__ P mred[NV];
    __shared__ __align__(8) uint64_t bars[S];
    __shared__ CgState st;
    __shared__ unsigned int sflags;
    // the streamed layout: without the diagonal entries when it was built
    // (the diagonal term A_ii u'_i is then the row's new residual r'_i, as
    // u' = D^-1 r'), else the full one
    const bool od = a.As_od != nullptr;
    const V* const Aop = od ? a.As_od : a.As;
    const uint16_t* const lop = od ? a.lcol_od : a.lcol;
    const int32_t* const soff = od ? a.slice_off_od : a.slice_off;
    const int emx = od ? a.emax_od : a.emax;
    const RingStage L(emx, sizeof(V));
    unsigned char* const ring = dyn_smem;
    V* const ubuf = reinterpret_cast<V*>(dyn_smem + ring_bytes<R, NF>(emx, S));
    const int ustride = kTileRows + a.hmax;
    const int t = threadIdx.x, lane = t & 31, wib = t >> 5, j = halo_slot(t);
    const int ntiles = (int)ceil_div(a.N, kTileRows), G = (int)gridDim.x, t0 = (int)blockIdx.x;
    auto halo_head = [&](int tile, int32_t& h0, int32_t& cnt) {
        h0 = cnt = 0;
        if (tile < ntiles) {
            h0 = a.halo_off[tile];
            cnt = a.halo_off[tile + 1] - h0;
        }
    };
    // this warp's slice of a tile: offset in the tile's entries, width
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
    // thread 0: the bulk copies of one tile's entries and columns into stage b
    auto issue = [&](int b, int32_t e0, int32_t e1) {
        uint64_t* bar = &bars[b];
        const uint32_t n = (uint32_t)(e1 - e0);  // a multiple of 32 entries
        if (n == 0) {
            mbar_arrive(bar);
            return;
        }
        mbar_arrive_expect_tx(bar, n * (uint32_t)sizeof(V) + 2 * n);
        const uint64_t pol = l2_evict_first_policy();
        bulk_g2s_hint(stage_of(b) + L.A, Aop + e0, n * (uint32_t)sizeof(V), bar, pol);
        bulk_g2s_hint(stage_of(b) + L.L, lop + e0, 2 * n, bar, pol);
    };
    // Before the dependency wait, only what no earlier kernel writes: the
    // stages' barriers, the first S tiles' operator copies, the references.
    uint32_t armed = 0;  // thread 0: bit b set while stage b has copies in flight
    int32_t re0 = 0, re1 = 0;  // thread 0: entry range of the next refill
    if (t == 0) {
        for (int b = 0; b < S; b++) mbar_init(&bars[b], 1);
        mbar_fence_init();
        for (int b = 0; b < S; b++) {
            int32_t e0, e1;
            if (t0 + b * G < ntiles) {
                tile_range(t0 + b * G, e0, e1);
                issue(b, e0, e1);
                armed |= 1u << b;
            }
        }
        tile_range(t0 + S * G, re0, re1);
    }
    int32_t sb, sw, sbn, swn;
    slice_ref(t0, sb, sw);
    slice_ref(t0 + G, sbn, swn);
    int32_t h0c, hcc, h0n, hcn, hh0, hhc;
    halo_head(t0, h0c, hcc);
    halo_head(t0 + G, h0n, hcn);
    halo_head(t0 + 2 * G, hh0, hhc);
    const int32_t fcol = j < hcc ? a.halo_col[h0c + j] : -1;
    int32_t hcoln = j < hcn ? a.halo_col[h0n + j] : -1;
    grid_dependency_wait();
    constexpr int q = PAR;
    CgVecs<R, NF> v;
    v.rp = a.rp;
    v.col = a.col;
    v.A = a.A;
    v.dinv = a.dinv;
    v.x = a.x;
    v.p = a.pp[0];
    v.r0 = a.rb[q];
    v.w0 = a.wb[q];
    v.s0 = a.sb[q];
    v.r1 = a.rb[q ^ 1];
    v.w1 = a.wb[q ^ 1];
    v.s1 = a.sb[q ^ 1];
    V cr, cw, cs, cd, cx, cp, hr, hw, hs, hd;
    {
        const uint64_t pol_keep = l2_evict_last_policy();
        const int row = t0 * kTileRows + t;  // every vector holds whole tiles
        if (t0 < ntiles) {
            cr = ld_keep(v.r0 + row, pol_keep);
            cw = ld_keep(v.w0 + row, pol_keep);
            cs = ld_keep(v.s0 + row, pol_keep);
            cd = ld_keep(v.dinv + row, pol_keep);
            cx = ld_keep(v.x + row, pol_keep);
            cp = ld_keep(v.p + row, pol_keep);
        }
        if (fcol >= 0) {
            hr = ld_keep(v.r0 + fcol, pol_keep);
            hw = ld_keep(v.w0 + fcol, pol_keep);
            hs = ld_keep(v.s0 + fcol, pol_keep);
            hd = ld_keep(v.dinv + fcol, pol_keep);
        }
    }
    PhaseCtl<R, NF> c;
    const bool go = deferred_head<R, NF>(a, q, st, sflags, mred, c);
    if (!go && !a.probe) {  // every field stopped: the copies land, then the block leaves
        if (t == 0)
            for (int b = 0; b < S; b++)
                if (armed & (1u << b)) mbar_wait(&bars[b], 0u);
        return;
    }
    R dots[NV];
#pragma unroll
    for (int k = 0; k < NV; k++) dots[k] = 0;
    auto dot_add = [&](int k, R x, R y) { dots[k] = fmar(x, y, dots[k]); };
    uint32_t phases = 0u;  // bit b: parity of stage b's next phase
    bool bad = false;      // a stage wait expired
    int buf = 0, b = 0, k = 0;
    for (int tile = t0; tile < ntiles; tile += G, k++) {
        V* ut = ubuf + buf * ustride;
        const int row = tile * kTileRows + t;
        V un, wn;  // wn: the product's start, the diagonal term in the diagonal-free layout
#pragma unroll
        for (int f = 0; f < NF; f++) un.v[f] = wn.v[f] = 0;
        if (row < a.N) {
            V sn, rn;
            cg_advance(c, cr, cw, c.need_old ? cs : cw, cd, sn, rn, un);
            if (od) wn = rn;
#pragma unroll
            for (int f = 0; f < NF; f++) {
                if (c.act[f]) {
                    const R ui = cd.v[f] * cr.v[f];
                    cp.v[f] = c.fresh[f] ? ui : fmar(c.beta[f], cp.v[f], ui);
                    cx.v[f] = fmar(c.alpha[f], cp.v[f], cx.v[f]);
                }
                dot_add(f, rn.v[f], un.v[f]);
                dot_add(2 * NF + f, rn.v[f], rn.v[f]);
            }
            v.x[row] = cx;
            v.p[row] = cp;
            v.r1[row] = rn;
            v.s1[row] = sn;
        }
        ut[t] = un;
        const uint64_t pol_keep = l2_evict_last_policy();
        const int nt = tile + G;
        if (nt < ntiles) {
            const int nrow = nt * kTileRows + t;
            cr = ld_keep(v.r0 + nrow, pol_keep);
            cw = ld_keep(v.w0 + nrow, pol_keep);
            cs = ld_keep(v.s0 + nrow, pol_keep);
            cd = ld_keep(v.dinv + nrow, pol_keep);
            cx = ld_keep(v.x + nrow, pol_keep);
            cp = ld_keep(v.p + nrow, pol_keep);
        }
        if (j < hcc) {
            V sn, rn, u2;
            cg_advance(c, hr, hw, c.need_old ? hs : hw, hd, sn, rn, u2);
            ut[kTileRows + j] = u2;
        }
        if (hcoln >= 0) {
            hr = ld_keep(v.r0 + hcoln, pol_keep);
            hw = ld_keep(v.w0 + hcoln, pol_keep);
            hs = ld_keep(v.s0 + hcoln, pol_keep);
            hd = ld_keep(v.dinv + hcoln, pol_keep);
        }
        for (int32_t h = kBlock + t; h < hcc; h += kBlock)
            ut[kTileRows + h] = cg_u_at(v, c, a.halo_col[h0c + h]);
        __syncthreads();
        if (t == 0 && k > 0) {  // refill the previous tile's stage, S - 1 tiles ahead
            const int bp = b == 0 ? S - 1 : b - 1;
            const int target = tile + (S - 1) * G;
            if (target < ntiles) {
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                issue(bp, re0, re1);
                armed |= 1u << bp;
            }
            tile_range(target + G, re0, re1);
        }
        h0c = h0n;
        hcc = hcn;
        hcoln = j < hhc ? a.halo_col[hh0 + j] : -1;
        h0n = hh0;
        hcn = hhc;
        halo_head(tile + 3 * G, hh0, hhc);
        int32_t sb2, sw2;
        slice_ref(tile + 2 * G, sb2, sw2);
        // the product from the stage
        const bool got = mbar_wait(&bars[b], (phases >> b) & 1u);
        phases ^= 1u << b;
        bad |= !got;
        if (t == 0 && got) armed &= ~(1u << b);
        const V* As = reinterpret_cast<const V*>(stage_of(b) + L.A) + sb + lane;
        const uint16_t* Ls = reinterpret_cast<const uint16_t*>(stage_of(b) + L.L) + sb + lane;
#pragma unroll 4
        for (int kk = 0; kk < sw; kk++) {
            const V av = As[32 * kk];
            const V g = ut[Ls[32 * kk]];
#pragma unroll
            for (int f = 0; f < NF; f++) wn.v[f] = fmar(av.v[f], g.v[f], wn.v[f]);
        }
        if (row < a.N) {
            v.w1[row] = wn;
#pragma unroll
            for (int f = 0; f < NF; f++) dot_add(NF + f, wn.v[f], un.v[f]);
        }
        sb = sbn;
        sw = swn;
        sbn = sb2;
        swn = sw2;
        buf ^= 1;
        b = b + 1 == S ? 0 : b + 1;
    }
    grid_launch_dependents();
    // every thread is done with the ring before it holds the reduction
    if (__syncthreads_or(bad)) {
        if (t == 0) {
            atomicOr(&a.run->flags, FEA_STATUS_BREAKDOWN);
            for (int q2 = 0; q2 < S; q2++)  // copies still in flight land before the ring is reused
                if (armed & (1u << q2)) mbar_wait(&bars[q2], (phases >> q2) & 1u);
        }
        __syncthreads();
    }
    Acc<R> acc[NV];
#pragma unroll
    for (int k = 0; k < NV; k++) acc[k].add(dots[k]);
    store_block_partials<R, NV>(a, q, acc, reinterpret_cast<P*>(ring));
}

// The tile loop of the ring kernels that run once per solve or step
// (variants 14 and 15): the full tile-ELL layout (with kM, also the mass
// matrix's copy) streamed through S bulk-copy stages, the block's tiles
// strided by the grid.  Per tile, thread t loads load_raw(index, policy) of
// its row and of its halo slot one tile ahead and stages make(raw) once;
// after the block barrier each thread sums its row's entries against the
// staged values in CSR order (Sum::add from a value-initialised Sum; padding
// entries hold 0) and row_done(row, raw, extra, sum) finishes the row, with
// `extra` fetched by load_extra(row, policy) one tile ahead.  Returns false
// when a stage wait expired; the copies in flight have landed by then.  smem
// holds the ring (ring_bytes) and two staging buffers of kTileRows + hmax
// staged values.
template <typename R, int NF, int S, typename Sum, bool kM, typename LoadRaw, typename Make, typename LoadExtra,
          typename RowDone>
__device__ bool ring_product_tiles(const StepArgs<R, NF>& a, unsigned char* smem, uint64_t* bars, LoadRaw load_raw,
                                   Make make, LoadExtra load_extra, RowDone row_done) {
    using V = FV<R, NF>;
    using Raw = decltype(load_raw(0, uint64_t{}));
    using Gv = decltype(make(Raw{}));
    static_assert(S >= 2 && S <= 8, "ring depth");
    constexpr size_t mv = kM ? sizeof(R) : 0;
    const RingStage L(a.emax, sizeof(V), mv);
    Gv* const ubuf = reinterpret_cast<Gv*>(smem + ring_bytes<R, NF>(a.emax, S, mv));
    const int ustride = kTileRows + a.hmax;
    const int t = threadIdx.x, lane = t & 31, wib = t >> 5, j = halo_slot(t);
    const int ntiles = (int)ceil_div(a.N, kTileRows), G = (int)gridDim.x, t0 = (int)blockIdx.x;
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
            const int32_t s0 = a.slice_off[sl];
            sb = s0 - a.slice_off[tile * (kTileRows / 32)];
            sw = (a.slice_off[sl + 1] - s0) >> 5;
        }
    };
    auto tile_range = [&](int tile, int32_t& e0, int32_t& e1) {
        e0 = e1 = 0;
        if (tile < ntiles) {
            e0 = a.slice_off[tile * (kTileRows / 32)];
            e1 = a.slice_off[(tile + 1) * (kTileRows / 32)];
        }
    };
    auto stage_of = [&](int b) { return smem + (size_t)b * L.bytes; };
    auto issue = [&](int b, int32_t e0, int32_t e1) {  // thread 0
        uint64_t* bar = &bars[b];
        const uint32_t n = (uint32_t)(e1 - e0);  // a multiple of 32 entries
        if (n == 0) {
            mbar_arrive(bar);
            return;
        }
        mbar_arrive_expect_tx(bar, n * (uint32_t)(sizeof(V) + mv + 2));
        const uint64_t pol = l2_evict_first_policy();
        bulk_g2s_hint(stage_of(b) + L.A, a.As + e0, n * (uint32_t)sizeof(V), bar, pol);
        if constexpr (kM) bulk_g2s_hint(stage_of(b) + L.M, a.Ms + e0, n * (uint32_t)mv, bar, pol);
        bulk_g2s_hint(stage_of(b) + L.L, a.lcol + e0, 2 * n, bar, pol);
    };
    uint32_t armed = 0;        // thread 0: bit b set while stage b has copies in flight
    int32_t re0 = 0, re1 = 0;  // thread 0: entry range of the next refill
    if (t == 0) {
        for (int b = 0; b < S; b++) mbar_init(&bars[b], 1);
        mbar_fence_init();
        for (int b = 0; b < S; b++) {
            if (t0 + b * G < ntiles) {
                int32_t e0, e1;
                tile_range(t0 + b * G, e0, e1);
                issue(b, e0, e1);
                armed |= 1u << b;
            }
        }
        tile_range(t0 + S * G, re0, re1);
    }
    __syncthreads();  // the barriers are initialised before any thread waits on them
    int32_t sb, sw, sbn, swn;
    slice_ref(t0, sb, sw);
    slice_ref(t0 + G, sbn, swn);
    int32_t h0c, hcc, h0n, hcn, hh0, hhc;
    halo_head(t0, h0c, hcc);
    halo_head(t0 + G, h0n, hcn);
    halo_head(t0 + 2 * G, hh0, hhc);
    const int32_t hcol = j < hcc ? a.halo_col[h0c + j] : -1;
    int32_t hcoln = j < hcn ? a.halo_col[h0n + j] : -1;
    const uint64_t pol_keep = l2_evict_last_policy();
    Raw cv{}, hv{};
    decltype(load_extra(0, uint64_t{})) ce{};
    if (t0 < ntiles) {
        const int row = t0 * kTileRows + t;  // every vector holds whole tiles
        cv = load_raw(row, pol_keep);
        ce = load_extra(row, pol_keep);
    }
    if (hcol >= 0) hv = load_raw(hcol, pol_keep);
    uint32_t phases = 0u;  // bit b: parity of stage b's next phase
    bool bad = false;      // a stage wait expired
    int buf = 0, b = 0, k = 0;
    for (int tile = t0; tile < ntiles; tile += G, k++) {
        Gv* ut = ubuf + buf * ustride;
        const int row = tile * kTileRows + t;
        const Raw vr = cv;
        const auto er = ce;
        ut[t] = make(vr);
        if (j < hcc) ut[kTileRows + j] = make(hv);
        const int nt = tile + G;
        if (nt < ntiles) {
            const int nrow = nt * kTileRows + t;
            cv = load_raw(nrow, pol_keep);
            ce = load_extra(nrow, pol_keep);
        }
        if (hcoln >= 0) hv = load_raw(hcoln, pol_keep);
        for (int32_t h = kBlock + t; h < hcc; h += kBlock) ut[kTileRows + h] = make(load_raw(a.halo_col[h0c + h], pol_keep));
        __syncthreads();
        if (t == 0 && k > 0) {  // refill the previous tile's stage, S - 1 tiles ahead
            const int bp = b == 0 ? S - 1 : b - 1;
            const int target = tile + (S - 1) * G;
            if (target < ntiles) {
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                issue(bp, re0, re1);
                armed |= 1u << bp;
            }
            tile_range(target + G, re0, re1);
        }
        h0c = h0n;
        hcc = hcn;
        hcoln = j < hhc ? a.halo_col[hh0 + j] : -1;
        h0n = hh0;
        hcn = hhc;
        halo_head(tile + 3 * G, hh0, hhc);
        int32_t sb2, sw2;
        slice_ref(tile + 2 * G, sb2, sw2);
        const bool got = mbar_wait(&bars[b], (phases >> b) & 1u);
        phases ^= 1u << b;
        bad |= !got;
        if (t == 0 && got) armed &= ~(1u << b);
        const V* As = reinterpret_cast<const V*>(stage_of(b) + L.A) + sb + lane;
        const uint16_t* Ls = reinterpret_cast<const uint16_t*>(stage_of(b) + L.L) + sb + lane;
        Sum sum{};
        if constexpr (kM) {
            const R* Ms = reinterpret_cast<const R*>(stage_of(b) + L.M) + sb + lane;
#pragma unroll 4
            for (int kk = 0; kk < sw; kk++) sum.add(As[32 * kk], Ms[32 * kk], ut[Ls[32 * kk]]);
        } else {
#pragma unroll 4
            for (int kk = 0; kk < sw; kk++) sum.add(As[32 * kk], ut[Ls[32 * kk]]);
        }
        if (row < a.N) row_done(row, vr, er, sum);
        sb = sbn;
        sw = swn;
        sbn = sb2;
        swn = sw2;
        buf ^= 1;
        b = b + 1 == S ? 0 : b + 1;
    }
    if (__syncthreads_or(bad)) {
        if (t == 0)
            for (int q2 = 0; q2 < S; q2++)  // copies still in flight land before the block leaves
                if (armed & (1u << q2)) mbar_wait(&bars[q2], (phases >> q2) & 1u);
        return false;
    }
    return true;
}

// Row sums of the ring set-up product: R with fused multiply-adds, as the
// tile-ELL product (EllRow::finish) sums them.
template <typename R, int NF>
struct FmaRowSum {
    FV<R, NF> w{};
    __device__ __forceinline__ void add(const FV<R, NF>& av, const FV<R, NF>& g) {
#pragma unroll
        for (int f = 0; f < NF; f++) w.v[f] = fmar(av.v[f], g.v[f], w.v[f]);
    }
};
struct NoExtra {};

// Set-up of a solve for variants 14 and 15: w0 = A z, delta0 = z.w0 and
// alpha0 = r0.z / delta0, bit for bit as k_cgcg_init_ell computes them (the
// full tile-ELL layout, each row's entries summed in CSR order from 0), with
// the operator streamed through a ring of bulk-copy stages as in the
// iteration (ring_product_tiles).  (Starting from the residual on the
// diagonal-free layout, as the iteration does, changes w0's rounding and
// cost about two CG iterations per step on the 1M-vertex workload.)
template <typename R, int NF, int S>
__global__ void __launch_bounds__(kBlock, 2) k_cgcg_init_ring(StepArgs<R, NF> a) {
    using V = FV<R, NF>;
    extern __shared__ __align__(16) unsigned char dyn_smem[];  // bulk copies need 16-byte destinations
    __shared__ typename Acc<R>::Packed red[32 * NF];
    __shared__ __align__(8) uint64_t bars[S];
    if (a.guess_init && a.xg) move_guess(a);
    PhaseCtl<R, NF> c;
    c.load(a.cg);
    if (!c.any) {  // no field iterates (every solve converged or stopped): no product to set up
        if (blockIdx.x == 0 && threadIdx.x == 0) signal_loop(a, false);
        return;
    }
    V* const w = a.wb[a.defer ? 0 : c.par];
    Acc<R> dot[NF];
    const bool ok = ring_product_tiles<R, NF, S, FmaRowSum<R, NF>, false>(
        a, dyn_smem, bars, [&](int i, uint64_t pol) { return ld_keep(a.z + i, pol); }, [](const V& g) { return g; },
        [](int, uint64_t) { return NoExtra{}; },
        [&](int row, const V& zr, const NoExtra&, const FmaRowSum<R, NF>& sum) {
            w[row] = sum.w;
#pragma unroll
            for (int f = 0; f < NF; f++) dot[f].add_prod(zr.v[f], sum.w.v[f]);
        });
    if (!ok && threadIdx.x == 0) atomicOr(&a.run->flags, FEA_STATUS_BREAKDOWN);
    Acc<R> blk[NF], tot[NF];
    block_totals<NF>(dot, red, blk);
    if (grid_commit<NF>(blk, a.part, a.part_stride, a.tickets + 0, red, tot) && threadIdx.x == 0) {
        volatile CgState* cg = a.cg;
        finish_spmv<R, NF>(cg, &a.run->flags, c.act, tot);
        int any = 0;
#pragma unroll
        for (int f = 0; f < NF; f++) {
            cg->fresh[f] = 1;
            any |= cg->active[f];
        }
        signal_loop(a, any != 0);
    }
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
    // Gray-Scott: the solve starts from x0 = 2 x_n - x_(n-1) (one rounding;
    // 2 x is exact) when the extrapolation is on and x_(n-1) is the previous
    // step's state; b still comes from x_n
    constexpr bool kGS = EQ == EQ_GS_REF || EQ == EQ_GS_CONSISTENT;
    const bool extrap = kGS && a.xprev != nullptr && a.run->guess == 1 && a.run->prev_valid != 0;
    auto guess_at = [&](const FV<R, NF>& xn, int64_t i) {
        FV<R, NF> g = xn;
        if (extrap) {
            const FV<R, NF> xp = a.xprev[i];
#pragma unroll
            for (int f = 0; f < NF; f++) g.v[f] = fmar((R)2, xn.v[f], -xp.v[f]);
        }
        return g;
    };
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
                const FV<R, NF> x0c = kGS ? guess_at(xc, c) : xc;  // the solve's start at column c
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
                } else if constexpr (EQ == EQ_GIVEN) {
                    (void)me;  // b is given; only A x0 is gathered
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
                for (int f = 0; f < NF; f++) ax[f].add_prod(av.v[f], x0c.v[f]);
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
            if constexpr (kGS)
                if (a.xg) a.xg[row] = guess_at(xr, row);  // the set-up kernel makes it x
            if constexpr (EQ == EQ_GS_REF) {  // nodal reaction, CPUSolver.cpp:134,137
                const R u = xr.v[0], v = xr.v[NF - 1];
                const R uvv = u * (v * v);
                bs[0].add(-uvv);
                bs[0].add((R)P.F * ((R)1 - u));
                bs[NF - 1].add(uvv);
                bs[NF - 1].add(-((R)P.F + (R)P.k) * v);
            }
            if constexpr (EQ == EQ_GIVEN) {  // adjoint values may be large: only non-finite stops
                const FV<R, NF> g = a.rhs[row];
#pragma unroll
                for (int f = 0; f < NF; f++) {
                    bs[f].add(g.v[f]);
                    if (!isfinite(xr.v[f])) flags |= FEA_STATUS_NONFINITE;
                }
            } else if constexpr (EQ == EQ_WAVE_REF || EQ == EQ_NEWMARK_INIT) {
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
                bv.v[f] = bs[f].rounded();
                bs[f].sub(ax[f]);
                rv.v[f] = bs[f].rounded();
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
    Acc<R> tot[3 * NF];
    if (grid_reduce<R, 3 * NF>(dots, a.part, a.part_stride, a.tickets + 2, tot) && threadIdx.x == 0) {
        CgState* cg = a.cg;
        RunState* run = a.run;
        const int stop = (atomicOr(&run->flags, 0u) & (FEA_STATUS_BLOWUP | FEA_STATUS_NONFINITE)) != 0;
        cg->stop = stop;
        cg->iter = 0;
        cg->max_iter = run->max_iter;
        int any = 0;
#pragma unroll
        for (int f = 0; f < NF; f++)
            any |= start_solve<R>((volatile CgState*)cg, f, stop, run->tol, tot[f], tot[NF + f], tot[2 * NF + f]);
        cg->pending = 0;
        signal_loop(a, any != 0);
    }
}

// The mass-weighted Gray-Scott right-hand side of k_rhs on the tile-ELL
// layout.  Per tile (one row per thread): the state x, the solve's start x0
// (extrapolated when the rule asks) and the nodal reaction w(x) of the
// tile's rows and halo are staged in shared memory once per unknown; each
// warp then reads its 32-row slice of the tile-ELL copies of A and M with
// coalesced loads.  Entries keep their CSR order within a row and padding
// entries hold 0, so b, r0 and their rounding are those of k_rhs.
template <typename R, int NF>
__global__ void __launch_bounds__(kBlock) k_rhs_gs_ell(StepArgs<R, NF> a) {
    static_assert(NF == 2, "the paired Gray-Scott solve");
    using V = FV<R, NF>;
    extern __shared__ __align__(16) unsigned char dyn_smem[];
    const int hs = kTileRows + a.hmax;
    V* const gw = reinterpret_cast<V*>(dyn_smem);  // w(x) of the tile's rows, then its halo
    V* const g0 = gw + hs;                          // x0
    const StepParams P = *a.prm;
    const R dt = (R)P.dt, Fr = (R)P.F, Kr = (R)P.k;
    const bool extrap = a.xprev != nullptr && a.run->guess == 1 && a.run->prev_valid != 0;
    auto guess_at = [&](const V& xn, int64_t i) {
        V g = xn;
        if (extrap) {
            const V xp = a.xprev[i];
#pragma unroll
            for (int f = 0; f < NF; f++) g.v[f] = fmar((R)2, xn.v[f], -xp.v[f]);
        }
        return g;
    };
    auto react = [&](const V& x) {
        const R u = x.v[0], v = x.v[1];
        const R uvv = u * (v * v);
        V w;
        w.v[0] = u / dt - uvv + Fr * ((R)1 - u);
        w.v[1] = v / dt + uvv - (Fr + Kr) * v;
        return w;
    };
    const int t = threadIdx.x, lane = t & 31, wib = t >> 5;
    const int ntiles = (int)ceil_div(a.N, kTileRows);
    Acc<R> dots[3 * NF];  // |b|^2, |r|^2, r.z per field
    unsigned int flags = 0;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int64_t row = (int64_t)tile * kTileRows + t;  // every vector holds whole tiles
        const V xr = a.x[row];
        const int32_t h0 = a.halo_off[tile], hn = a.halo_off[tile + 1] - h0;
        const int sl = tile * (kTileRows / 32) + wib;
        const int32_t sb = a.slice_off[sl], sw = (a.slice_off[sl + 1] - sb) >> 5;
        const V d = ldfv(a.dinv + row);
        const V x0r = guess_at(xr, row);
        gw[t] = react(xr);
        g0[t] = x0r;
        for (int h = t; h < hn; h += kBlock) {
            const int32_t c = a.halo_col[h0 + h];
            const V xc = a.x[c];
            gw[kTileRows + h] = react(xc);
            g0[kTileRows + h] = guess_at(xc, c);
        }
        __syncthreads();
        Acc<R> bs[NF], ax[NF];
#pragma unroll 4
        for (int32_t k = 0; k < sw; k++) {
            const int32_t e = sb + 32 * k + lane;
            const V av = ldfv(a.As + e);
            const R me = ldg(a.Ms + e);
            const int l = a.lcol[e];
            const V w = gw[l], x0 = g0[l];
#pragma unroll
            for (int f = 0; f < NF; f++) {
                bs[f].add_prod(me, w.v[f]);
                ax[f].add_prod(av.v[f], x0.v[f]);
            }
        }
        if (row < a.N) {
            if (a.xg) a.xg[row] = x0r;  // the set-up kernel makes it x
#pragma unroll
            for (int f = 0; f < NF; f++) flags |= check_value(xr.v[f]);
            V bv, rv, pv;
#pragma unroll
            for (int f = 0; f < NF; f++) {
                bv.v[f] = bs[f].rounded();
                bs[f].sub(ax[f]);
                rv.v[f] = bs[f].rounded();
                pv.v[f] = d.v[f] * rv.v[f];
                dots[f].add_prod(bv.v[f], bv.v[f]);
                dots[NF + f].add_prod(rv.v[f], rv.v[f]);
                dots[2 * NF + f].add_prod(rv.v[f], pv.v[f]);
            }
            a.b[row] = bv;
            a.rb[0][row] = rv;  // iteration 0 reads parity 0
            a.z[row] = pv;
        }
        __syncthreads();  // the next tile restages gw, g0
    }
    raise_flags(a.run, flags);
    Acc<R> tot[3 * NF];
    if (grid_reduce<R, 3 * NF>(dots, a.part, a.part_stride, a.tickets + 2, tot) && threadIdx.x == 0) {
        CgState* cg = a.cg;
        RunState* run = a.run;
        const int stop = (atomicOr(&run->flags, 0u) & (FEA_STATUS_BLOWUP | FEA_STATUS_NONFINITE)) != 0;
        cg->stop = stop;
        cg->iter = 0;
        cg->max_iter = run->max_iter;
        int any = 0;
#pragma unroll
        for (int f = 0; f < NF; f++)
            any |= start_solve<R>((volatile CgState*)cg, f, stop, run->tol, tot[f], tot[NF + f], tot[2 * NF + f]);
        cg->pending = 0;
        signal_loop(a, any != 0);
    }
}

// Staged values and row sums of the ring Gray-Scott right-hand side.
template <typename R, int NF>
struct GsRaw {
    FV<R, NF> x, xp;  // the state and, for the extrapolated start, the state one step before
};
template <typename R, int NF>
struct GsStaged {
    FV<R, NF> w, x0;  // the nodal reaction w(x) and the solve's start
};
template <typename R, int NF>
struct GsRowSum {
    Acc<R> bs[NF], ax[NF];
    __device__ __forceinline__ void add(const FV<R, NF>& av, R me, const GsStaged<R, NF>& g) {
#pragma unroll
        for (int f = 0; f < NF; f++) {
            bs[f].add_prod(me, g.w.v[f]);
            ax[f].add_prod(av.v[f], g.x0.v[f]);
        }
    }
};

// k_rhs_gs_ell on the ring of variants 14 and 15: the nodal reaction and the
// solve's start of each tile's rows and halo are staged once, A and the mass
// matrix's tile-ELL copy stream through the bulk-copy stages
// (ring_product_tiles), and each row sums the same products in the same
// order, so b, r0, z and the set-up sums are bit-identical.
template <typename R, int NF, int S>
__global__ void __launch_bounds__(kBlock, 2) k_rhs_gs_ring(StepArgs<R, NF> a) {
    static_assert(NF == 2, "the paired Gray-Scott solve");
    using V = FV<R, NF>;
    using Raw = GsRaw<R, NF>;
    using Gv = GsStaged<R, NF>;
    extern __shared__ __align__(16) unsigned char dyn_smem[];  // bulk copies need 16-byte destinations
    __shared__ __align__(8) uint64_t bars[S];
    const StepParams P = *a.prm;
    const R dt = (R)P.dt, Fr = (R)P.F, Kr = (R)P.k;
    const bool extrap = a.xprev != nullptr && a.run->guess == 1 && a.run->prev_valid != 0;
    auto start = [&](const Raw& r) {
        V g = r.x;
        if (extrap)
#pragma unroll
            for (int f = 0; f < NF; f++) g.v[f] = fmar((R)2, r.x.v[f], -r.xp.v[f]);
        return g;
    };
    auto react = [&](const V& x) {
        const R u = x.v[0], v = x.v[1];
        const R uvv = u * (v * v);
        V w;
        w.v[0] = u / dt - uvv + Fr * ((R)1 - u);
        w.v[1] = v / dt + uvv - (Fr + Kr) * v;
        return w;
    };
    Acc<R> dots[3 * NF];  // |b|^2, |r|^2, r.z per field
    unsigned int flags = 0;
    const bool ok = ring_product_tiles<R, NF, S, GsRowSum<R, NF>, true>(
        a, dyn_smem, bars,
        [&](int i, uint64_t pol) {
            Raw r;
            r.x = ld_keep(a.x + i, pol);
            r.xp = extrap ? ld_keep(a.xprev + i, pol) : r.x;
            return r;
        },
        [&](const Raw& r) { return Gv{react(r.x), start(r)}; },
        [&](int row, uint64_t pol) { return ld_keep(a.dinv + row, pol); },
        [&](int row, const Raw& xr, const V& d, GsRowSum<R, NF> sum) {
            if (a.xg) a.xg[row] = start(xr);  // the set-up kernel makes it x
#pragma unroll
            for (int f = 0; f < NF; f++) flags |= check_value(xr.x.v[f]);
            V bv, rv, pv;
#pragma unroll
            for (int f = 0; f < NF; f++) {
                bv.v[f] = sum.bs[f].rounded();
                sum.bs[f].sub(sum.ax[f]);
                rv.v[f] = sum.bs[f].rounded();
                pv.v[f] = d.v[f] * rv.v[f];
                dots[f].add_prod(bv.v[f], bv.v[f]);
                dots[NF + f].add_prod(rv.v[f], rv.v[f]);
                dots[2 * NF + f].add_prod(rv.v[f], pv.v[f]);
            }
            a.b[row] = bv;
            a.rb[0][row] = rv;  // iteration 0 reads parity 0
            a.z[row] = pv;
        });
    if (!ok) flags |= FEA_STATUS_BREAKDOWN;
    raise_flags(a.run, flags);
    Acc<R> tot[3 * NF];
    if (grid_reduce<R, 3 * NF>(dots, a.part, a.part_stride, a.tickets + 2, tot) && threadIdx.x == 0) {
        CgState* cg = a.cg;
        RunState* run = a.run;
        const int stop = (atomicOr(&run->flags, 0u) & (FEA_STATUS_BLOWUP | FEA_STATUS_NONFINITE)) != 0;
        cg->stop = stop;
        cg->iter = 0;
        cg->max_iter = run->max_iter;
        int any = 0;
#pragma unroll
        for (int f = 0; f < NF; f++)
            any |= start_solve<R>((volatile CgState*)cg, f, stop, run->tol, tot[f], tot[NF + f], tot[2 * NF + f]);
        cg->pending = 0;
        signal_loop(a, any != 0);
    }
}

// Dynamic shared memory of k_rhs_gs_ring: the ring with the mass entries and
// two staging buffers of kTileRows + hmax (reaction, start) pairs.
template <typename R, int NF>
size_t rhs_ring_smem_bytes(int emax, int hmax, int stages) {
    return ring_bytes<R, NF>(emax, stages, sizeof(R)) + 2 * sizeof(GsStaged<R, NF>) * (size_t)(kTileRows + hmax);
}

// After the first CG loop: zero right-hand sides give x = 0 (Eigen's
// early exit), then one true-residual pass r = b - A x.  Fields whose true
// residual is still above the threshold restart CG from there.  The pass
// accumulates in the handle's accumulators (float-float pairs for FP32
// handles, about 48 significant bits) or, with RunState::refine == 2, in
// FP64: A x, r and the norms r.r, r.z in double, r rounded once to R.
template <typename A, typename R, int NF, int LANES>
__device__ __forceinline__ void refine_rows(const StepArgs<R, NF>& a, bool refine, const int (&zero)[NF],
                                            int parity, A (&dots)[2 * NF]) {
    RowMap<LANES> m;
    for (int64_t base = m.warp * m.RPW; base < a.N; base += m.nwarps * m.RPW) {
        const int64_t row = base + m.grp;
        A ax[NF];
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
                    A t;
                    t.add(bv.v[f]);
                    t.sub(ax[f]);
                    rv.v[f] = (R)t.rounded();
                    pv.v[f] = d.v[f] * rv.v[f];
                    dots[f].add_prod(rv.v[f], rv.v[f]);
                    dots[NF + f].add_prod(rv.v[f], pv.v[f]);
                }
                a.rb[parity][row] = rv;  // the restart's buffer parity
                a.z[row] = pv;
            }
        }
    }
}

// Row sums of the ring refinement: the handle's accumulators (float-float
// pairs for FP32 handles, or FP64), in CSR order as refine_rows sums them.
template <typename A, typename R, int NF>
struct AccRowSum {
    A ax[NF];
    __device__ __forceinline__ void add(const FV<R, NF>& av, const FV<R, NF>& g) {
#pragma unroll
        for (int f = 0; f < NF; f++) ax[f].add_prod(av.v[f], g.v[f]);
    }
};

// refine_rows on the ring layout of variants 14 and 15: the same sums in the
// same order (padding entries add exact zeros), so r, z and the norms are
// bit-identical; x of each tile and its halo is staged once and the operator
// streamed through bulk-copy stages (ring_product_tiles).
template <typename A, typename R, int NF, int S>
__device__ __forceinline__ void refine_rows_ring(const StepArgs<R, NF>& a, bool refine, const int (&zero)[NF],
                                                 int parity, A (&dots)[2 * NF], unsigned char* smem,
                                                 uint64_t* bars) {
    using V = FV<R, NF>;
    bool zany = false;
#pragma unroll
    for (int f = 0; f < NF; f++) zany |= zero[f] != 0;
    auto zeroed = [&](V x) {
#pragma unroll
        for (int f = 0; f < NF; f++)
            if (zero[f]) x.v[f] = 0;
        return x;
    };
    if (!refine) {  // no products: only the zero fields' unknowns are set to 0
        if (zany)
            for (int64_t row = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; row < a.N;
                 row += (int64_t)gridDim.x * blockDim.x)
                a.x[row] = zeroed(a.x[row]);
        return;
    }
    struct Extra {
        V b, d;
    };
    // x is staged before this kernel zeroes a field: only zero fields change,
    // and their residuals go unused
    const bool ok = ring_product_tiles<R, NF, S, AccRowSum<A, R, NF>, false>(
        a, smem, bars, [&](int i, uint64_t pol) { return ld_keep(a.x + i, pol); }, [](const V& g) { return g; },
        [&](int row, uint64_t pol) { return Extra{ld_keep(a.b + row, pol), ld_keep(a.dinv + row, pol)}; },
        [&](int row, const V& xr, const Extra& e, const AccRowSum<A, R, NF>& sum) {
            if (zany) a.x[row] = zeroed(xr);
            V rv, pv;
#pragma unroll
            for (int f = 0; f < NF; f++) {
                A t;
                t.add(e.b.v[f]);
                t.sub(sum.ax[f]);
                rv.v[f] = (R)t.rounded();
                pv.v[f] = e.d.v[f] * rv.v[f];
                dots[f].add_prod(rv.v[f], rv.v[f]);
                dots[NF + f].add_prod(rv.v[f], pv.v[f]);
            }
            a.rb[parity][row] = rv;  // the restart's buffer parity
            a.z[row] = pv;
        });
    if (!ok && threadIdx.x == 0) atomicOr(&a.run->flags, FEA_STATUS_BREAKDOWN);
}

// The true-residual pass; S > 0: on the ring layout of variants 14 and 15
// (dynamic shared memory ring_smem_bytes(emax, hmax, S)).
template <typename R, int NF, int LANES, int S = 0>
__global__ void __launch_bounds__(kBlock) k_refine(StepArgs<R, NF> a) {
    extern __shared__ __align__(16) unsigned char dyn_smem[];
    __shared__ __align__(8) uint64_t bars[S > 0 ? S : 1];
    CgState* cg = a.cg;
    const int stop = cg->stop;
    const int mode = a.run->refine;
    const bool refine = mode && cg->iter < cg->max_iter && !stop;
    const bool fp64 = sizeof(R) == 4 && mode == 2;
    const int parity = a.defer ? 0 : (cg->iter & 1);
    int zero[NF];
#pragma unroll
    for (int f = 0; f < NF; f++) zero[f] = !stop && !(cg->bb[f] > 0.0);
    double rr[NF], rz[NF];
    bool last;
    if (fp64) {
        Acc<double> dots[2 * NF], tot[2 * NF];
        if constexpr (S > 0) refine_rows_ring<Acc<double>, R, NF, S>(a, refine, zero, parity, dots, dyn_smem, bars);
        else refine_rows<Acc<double>, R, NF, LANES>(a, refine, zero, parity, dots);
        last = grid_reduce<double, 2 * NF>(dots, a.part, a.part_stride, a.tickets + 3, tot);
#pragma unroll
        for (int f = 0; f < NF; f++) {
            rr[f] = tot[f].value();
            rz[f] = tot[NF + f].value();
        }
    } else {
        Acc<R> dots[2 * NF], tot[2 * NF];
        if constexpr (S > 0) refine_rows_ring<Acc<R>, R, NF, S>(a, refine, zero, parity, dots, dyn_smem, bars);
        else refine_rows<Acc<R>, R, NF, LANES>(a, refine, zero, parity, dots);
        last = grid_reduce<R, 2 * NF>(dots, a.part, a.part_stride, a.tickets + 3, tot);
#pragma unroll
        for (int f = 0; f < NF; f++) {
            rr[f] = tot[f].value();
            rz[f] = tot[NF + f].value();
            if (last && threadIdx.x == 0 && refine && !zero[f] && cg->bb[f] > 0.0 && rr[f] >= cg->thr[f])
                set_gamma((volatile CgState*)cg, f, tot[NF + f]);  // the pair itself for FP32 handles
        }
    }
    if (last && threadIdx.x == 0) {
        int any = 0;
#pragma unroll
        for (int f = 0; f < NF; f++) {
            cg->active[f] = 0;
            cg->fresh[f] = 1;
            if (refine && !zero[f] && cg->bb[f] > 0.0) {
                cg->rr[f] = rr[f];
                if (rr[f] >= cg->thr[f]) {
                    if (fp64) {  // gamma = r.z from the FP64 sum (float-float copy for the iterations)
                        cg->rz[f] = rz[f];
                        if constexpr (sizeof(R) == 4) ff_store(cg->ffrz[f], ff_of(rz[f]));
                    }
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
        } else if constexpr (EQ == EQ_GIVEN) {
            const FV<R, NF> x = a.x[i];
#pragma unroll
            for (int f = 0; f < NF; f++)
                if (!isfinite(x.v[f])) flags |= FEA_STATUS_NONFINITE;
        } else {
            const FV<R, NF> x = a.x[i];
#pragma unroll
            for (int f = 0; f < NF; f++) flags |= check_value(x.v[f]);
        }
    }
    raise_flags(a.run, flags);
}

// ---- graph construction ----------------------------------------------------------

int g_max_grid = 0;

constexpr int kRowLanes = 1;  // threads per row of the once-per-step kernels (1: no shuffle reductions)

// The CG kernels of a variant: WCH > 0 the windowed CSR kernels (entries per
// lane and window), 0 the tile-ELL kernels with their dynamic shared memory.
template <typename R, int NF, int WCH>
struct CgKernels {
    using Fn = void (*)(StepArgs<R, NF>);
    static constexpr Fn init = k_cgcg_init<R, NF, WCH>;
    static constexpr Fn iter = k_cgcg_iter<R, NF, WCH>;
    // the iteration kernel of a launch with buffer parity `par`
    static Fn iter_par(int) { return iter; }
    static size_t smem_init(const StepArgs<R, NF>&) { return 0; }
    static size_t smem_iter(const StepArgs<R, NF>&) { return 0; }
    static constexpr int kPassStages = 0;  // ring stages of the once-per-step passes (0: CSR / tile-ELL forms)
};
// Variants 0 and 1: the tile-ELL kernels with 8 or 4 entries per row
// prefetched into registers; two staging buffers of kTileRows + hmax entries.
template <typename R, int NF, int KPRE>
struct EllKernels {
    using Fn = void (*)(StepArgs<R, NF>);
    static constexpr Fn init = k_cgcg_init_ell<R, NF, KPRE>;
    static constexpr Fn iter = k_cgcg_iter_ell<R, NF, KPRE>;
    static Fn iter_par(int) { return iter; }
    static size_t smem_init(const StepArgs<R, NF>& a) {
        return 2 * sizeof(FV<R, NF>) * (size_t)(kTileRows + a.hmax);
    }
    static size_t smem_iter(const StepArgs<R, NF>& a) { return smem_init(a); }
    static constexpr int kPassStages = 0;
};
template <typename R, int NF>
struct CgKernels<R, NF, 0> : EllKernels<R, NF, 8> {};
template <typename R, int NF>
struct CgKernels<R, NF, 1> : EllKernels<R, NF, 4> {};
// Variants 2 and 3: the streamed iteration with 2 or 3 stages, refilled
// after a third barrier per tile; 6 and 7: the same, refilled after the next
// tile's first barrier.  The set-up product is variant 1's.
template <typename R, int NF, int NS, bool LATE, bool DEFER = false>
struct StreamKernels : EllKernels<R, NF, 4> {
    using Fn = void (*)(StepArgs<R, NF>);
    static constexpr Fn iter = k_cgcg_iter_stream<R, NF, NS, LATE, DEFER>;
    static Fn iter_par(int) { return iter; }
    static size_t smem_iter(const StepArgs<R, NF>& a) { return NS * StageLayout<R, NF>(a.emax, a.hmax).bytes; }
};
template <typename R, int NF>
struct CgKernels<R, NF, 2> : StreamKernels<R, NF, 2, false> {};
template <typename R, int NF>
struct CgKernels<R, NF, 3> : StreamKernels<R, NF, 3, false> {};
template <typename R, int NF>
struct CgKernels<R, NF, 6> : StreamKernels<R, NF, 2, true> {};
template <typename R, int NF>
struct CgKernels<R, NF, 7> : StreamKernels<R, NF, 3, true> {};
// Variants 10 and 11: variants 2 and 7 with the deferred finish: no grid-wide
// last-block step at the end of an iteration; the next launch merges the
// block partials in every block and finishes the iteration at its start.
template <typename R, int NF>
struct CgKernels<R, NF, 10> : StreamKernels<R, NF, 2, false, true> {};
template <typename R, int NF>
struct CgKernels<R, NF, 11> : StreamKernels<R, NF, 3, true, true> {};
// Variant 12: the tile-ELL iteration with direct, register-pipelined loads
// and the deferred finish (two u' buffers of kTileRows + hmax entries); one
// kernel per buffer parity.
template <typename R, int NF, int MINB>
struct DirectKernels : EllKernels<R, NF, 4> {
    using Fn = void (*)(StepArgs<R, NF>);
    static constexpr int K = sizeof(FV<R, NF>) <= 8 ? 8 : 4;
    static constexpr Fn iter = k_cgcg_iter_direct<R, NF, K, 0, MINB>;
    static Fn iter_par(int par) { return par ? k_cgcg_iter_direct<R, NF, K, 1, MINB> : iter; }
};
// Variants 14 and 15: direct row loads with the operator in a ring of 3 or 4
// bulk-copy stages.
template <typename R, int NF, int S, int MINB>
struct RingKernels {
    using Fn = void (*)(StepArgs<R, NF>);
    static constexpr Fn init = k_cgcg_init_ring<R, NF, S>;
    static constexpr Fn iter = k_cgcg_iter_ring<R, NF, S, 0, MINB>;
    static Fn iter_par(int par) { return par ? k_cgcg_iter_ring<R, NF, S, 1, MINB> : iter; }
    static size_t smem_iter(const StepArgs<R, NF>& a) {
        return ring_smem_bytes<R, NF>(a.As_od ? a.emax_od : a.emax, a.hmax, S);
    }
    static size_t smem_init(const StepArgs<R, NF>& a) { return ring_smem_bytes<R, NF>(a.emax, a.hmax, S); }
    static constexpr int kPassStages = S;  // right-hand side and true-residual pass on the ring too
};
template <typename R, int NF>
struct CgKernels<R, NF, 14> : RingKernels<R, NF, 3, 2> {};
template <typename R, int NF>
struct CgKernels<R, NF, 15> : RingKernels<R, NF, 4, 2> {};
// Variant 13: registers for two resident blocks per SM (FP32 pairs: no spills).
template <typename R, int NF>
struct CgKernels<R, NF, 13> : DirectKernels<R, NF, (sizeof(FV<R, NF>) <= 8 ? 2 : 1)> {};

// The right-hand side kernel of an equation: for the mass-weighted
// Gray-Scott step on the tile-ELL layout, the ring form when the variant's
// once-per-step passes run on the ring (ring_stages 3 or 4) and its shared
// memory fits, else the staged tile-ELL form; otherwise k_rhs.
template <typename R, int NF, int EQ>
struct RhsKernel {
    using Fn = void (*)(StepArgs<R, NF>);
    Fn fn = k_rhs<R, NF, EQ, kRowLanes>;
    int grid = 0;
    size_t smem = 0;
    explicit RhsKernel(const StepArgs<R, NF>& a, int ring_stages = 0) {
        grid = (int)std::min<int64_t>(max_grid_blocks(), std::max<int64_t>(1, ceil_div(a.N, (kBlock / kRowLanes))));
        if constexpr (EQ == EQ_GS_CONSISTENT && NF == 2) {
            if (a.Ms && a.As) {
                const size_t ring = ring_stages ? rhs_ring_smem_bytes<R, NF>(a.emax, a.hmax, ring_stages) : 0;
                if (ring_stages && ring <= kStreamSmemLimit) {
                    fn = ring_stages == 4 ? k_rhs_gs_ring<R, NF, 4> : k_rhs_gs_ring<R, NF, 3>;
                    smem = ring;
                } else {
                    fn = k_rhs_gs_ell<R, NF>;
                    smem = 2 * sizeof(FV<R, NF>) * (size_t)(kTileRows + a.hmax);
                }
                grid = wave_grid(fn, ceil_div(a.N, kTileRows), smem);
            }
        }
    }
};

template <typename R, int NF, int WCH>
struct Grids {
    using K = CgKernels<R, NF, WCH>;
    using Fn = void (*)(StepArgs<R, NF>);
    int spmv, iter, rhs, stream, refine;
    size_t smem_init, smem_iter, smem_refine = 0;
    Fn refine_k = k_refine<R, NF, kRowLanes, K::kPassStages>;
    explicit Grids(const StepArgs<R, NF>& a) {
        const int64_t N = a.N;
        smem_init = K::smem_init(a);
        smem_iter = K::smem_iter(a);
        spmv = wave_grid(K::init, ceil_div(N, kBlock), smem_init);
        iter = wave_grid(K::iter, ceil_div(N, kBlock), smem_iter);
        if (K::iter_par(1) != K::iter) ensure_dyn_smem(K::iter_par(1), smem_iter);  // the other parity's kernel
        rhs = (int)std::min<int64_t>(max_grid_blocks(), std::max<int64_t>(1, ceil_div(N, (kBlock / kRowLanes))));
        stream = (int)std::min<int64_t>(max_grid_blocks(), std::max<int64_t>(1, ceil_div(N, kBlock)));
        refine = rhs;
        if constexpr (K::kPassStages > 0) {
            smem_refine = ring_smem_bytes<R, NF>(a.emax, a.hmax, K::kPassStages);
            refine = wave_grid(refine_k, ceil_div(N, kTileRows), smem_refine);
        }
    }
};

// Argument sets of a step: the step loop (a) and the two CG loops (a1: after
// k_rhs, a2: after k_refine); each names the condition it sets.
template <typename R, int NF>
struct LoopArgs {
    StepArgs<R, NF> a, a1, a2;
    LoopArgs(const StepArgs<R, NF>& base, LoopFlags* lf, int use_graph) : a(base), a1(base), a2(base) {
        a.use_graph = a1.use_graph = a2.use_graph = use_graph;
        a1.guess_init = 1;  // the set-up of a step's first solve takes the right-hand side's guess
        a.cont = &lf->step;
        a1.cont = &lf->cg1;
        a2.cont = &lf->cg2;
    }
};

// A CG loop body: kLoopUnroll iteration kernels in a chain whose edges are
// programmatic, so that each launch is scheduled while the previous one
// finishes its reduction (the kernels wait for it before reading its output).
// Deferred-finish variants get node u the buffer parity u & 1 (kLoopUnroll
// is even, so every pass starts at parity 0 as every solve does).
static_assert(kLoopUnroll % 2 == 0, "loop passes keep the buffer parity");
template <typename K, typename R, int NF>
void add_iterations(cudaGraph_t body, int grid, const StepArgs<R, NF>& a, size_t smem) {
    cudaGraphNode_t prev = nullptr;
    for (int u = 0; u < kLoopUnroll; u++) {
        StepArgs<R, NF> au = a;
        au.par = a.defer ? (u & 1) : 0;
        cudaGraphNode_t n = add_kernel(body, nullptr, K::iter_par(au.par), grid, kBlock, au, smem);
        if (prev) add_programmatic_edge(body, prev, n);
        prev = n;
    }
}

// Step graph:  start -> WHILE(step) { rhs -> init -> WHILE(cg1) { iter x 8 }
//              -> refine -> init -> WHILE(cg2) { iter x 8 } -> [post] -> stepctl }
//              -> final_check
template <typename R, int NF, int EQ, int WCH>
void build_graph_t(StepGraph& G, const StepArgs<R, NF>& base, LoopFlags* lf) {
    LoopArgs<R, NF> L(base, lf, 1);
    const Grids<R, NF, WCH> g(base);
    using K = CgKernels<R, NF, WCH>;
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
    const RhsKernel<R, NF, EQ> rk(base, K::kPassStages);
    cudaGraphNode_t s = add_kernel(step_body, nullptr, rk.fn, rk.grid, kBlock, L.a1, rk.smem);
    s = add_kernel(step_body, s, K::init, g.spmv, kBlock, L.a1, g.smem_init);
    cudaGraph_t body1, body2;
    s = add_while(step_body, s, L.a1.cond, &body1);
    add_iterations<K>(body1, g.iter, L.a1, g.smem_iter);
    s = add_kernel(step_body, s, g.refine_k, g.refine, kBlock, L.a2, g.smem_refine);
    s = add_kernel(step_body, s, K::init, g.spmv, kBlock, L.a2, g.smem_init);
    s = add_while(step_body, s, L.a2.cond, &body2);
    add_iterations<K>(body2, g.iter, L.a2, g.smem_iter);
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
    using K = CgKernels<R, NF, WCH>;
    const Grids<R, NF, WCH> g(base);
    const RhsKernel<R, NF, EQ> rk(base, K::kPassStages);
    k_start<R, NF><<<1, 1, 0, st>>>(L.a);
    FEA_CHECK_LAUNCH();
    while (read_flag(&lf->step, st)) {
        rk.fn<<<rk.grid, kBlock, rk.smem, st>>>(L.a1);
        FEA_CHECK_LAUNCH();
        for (const StepArgs<R, NF>* la : {&L.a1, &L.a2}) {
            if (la == &L.a2) {
                g.refine_k<<<g.refine, kBlock, g.smem_refine, st>>>(L.a2);
                FEA_CHECK_LAUNCH();
            }
            K::init<<<g.spmv, kBlock, g.smem_init, st>>>(*la);
            FEA_CHECK_LAUNCH();
            while (read_flag(la->cont, st)) {
                if (la->defer) {  // parities 0 and 1, so the final state lands in parity 1 as in the graph
                    StepArgs<R, NF> aq = *la;
                    for (int q = 0; q < 2; q++) {
                        aq.par = q;
                        K::iter_par(q)<<<g.iter, kBlock, g.smem_iter, st>>>(aq);
                        FEA_CHECK_LAUNCH();
                    }
                } else {
                    K::iter<<<g.iter, kBlock, g.smem_iter, st>>>(*la);
                    FEA_CHECK_LAUNCH();
                }
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
    case 0: G ? build_graph_t<R, NF, EQ, 0>(*G, a, lf) : run_stream_t<R, NF, EQ, 0>(a, lf, st); break;
    case 1: G ? build_graph_t<R, NF, EQ, 1>(*G, a, lf) : run_stream_t<R, NF, EQ, 1>(a, lf, st); break;
    case 2: G ? build_graph_t<R, NF, EQ, 2>(*G, a, lf) : run_stream_t<R, NF, EQ, 2>(a, lf, st); break;
    case 3: G ? build_graph_t<R, NF, EQ, 3>(*G, a, lf) : run_stream_t<R, NF, EQ, 3>(a, lf, st); break;
    case 6: G ? build_graph_t<R, NF, EQ, 6>(*G, a, lf) : run_stream_t<R, NF, EQ, 6>(a, lf, st); break;
    case 7: G ? build_graph_t<R, NF, EQ, 7>(*G, a, lf) : run_stream_t<R, NF, EQ, 7>(a, lf, st); break;
    case 10: G ? build_graph_t<R, NF, EQ, 10>(*G, a, lf) : run_stream_t<R, NF, EQ, 10>(a, lf, st); break;
    case 11: G ? build_graph_t<R, NF, EQ, 11>(*G, a, lf) : run_stream_t<R, NF, EQ, 11>(a, lf, st); break;
    case 13: G ? build_graph_t<R, NF, EQ, 13>(*G, a, lf) : run_stream_t<R, NF, EQ, 13>(a, lf, st); break;
    case 14: G ? build_graph_t<R, NF, EQ, 14>(*G, a, lf) : run_stream_t<R, NF, EQ, 14>(a, lf, st); break;
    case 15: G ? build_graph_t<R, NF, EQ, 15>(*G, a, lf) : run_stream_t<R, NF, EQ, 15>(a, lf, st); break;
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
        case EQ_GIVEN: dispatch_variant<R, 1, EQ_GIVEN>(G, a, wch, lf, st); break;
        default: throw Error{FEA_ERR_UNSUPPORTED};
        }
    } else {
        switch (kind) {
        case EQ_GS_REF: dispatch_variant<R, 2, EQ_GS_REF>(G, a, wch, lf, st); break;
        case EQ_GS_CONSISTENT: dispatch_variant<R, 2, EQ_GS_CONSISTENT>(G, a, wch, lf, st); break;
        case EQ_GIVEN: dispatch_variant<R, 2, EQ_GIVEN>(G, a, wch, lf, st); break;
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

// Probe state: every field masked, so an iteration writes x and p back
// unchanged and leaves only CG scratch behind, while keeping the loads and
// stores of a steady-state iteration (fresh = 0: the old s is gathered too).
template <typename R, int NF>
__global__ void k_probe_state(CgState* cg) {
    for (int f = 0; f < NF; f++) {
        cg->active[f] = 0;
        cg->fresh[f] = 0;
        cg->alpha[f] = 0.0;
        cg->beta[f] = 0.0;
        cg->falpha[f] = 0.f;
        cg->fbeta[f] = 0.f;
    }
    cg->pending = 0;
}

template <typename R, int NF>
void prepare_probe(const StepArgs<R, NF>& a, cudaStream_t st) {
    k_probe_state<R, NF><<<1, 1, 0, st>>>(a.cg);
    FEA_CHECK_LAUNCH();
}

template <typename R, int NF, int WCH>
void probe_t(const StepArgs<R, NF>& a, cudaStream_t st) {
    const Grids<R, NF, WCH> g(a);
    CgKernels<R, NF, WCH>::iter_par(a.par)<<<g.iter, kBlock, g.smem_iter, st>>>(a);
    FEA_CHECK_LAUNCH();
}

template <typename R, int NF>
void launch_spmv_probe(const StepArgs<R, NF>& a, int wch, cudaStream_t st) {
    switch (wch) {
    case 0: probe_t<R, NF, 0>(a, st); break;
    case 1: probe_t<R, NF, 1>(a, st); break;
    case 2: probe_t<R, NF, 2>(a, st); break;
    case 3: probe_t<R, NF, 3>(a, st); break;
    case 6: probe_t<R, NF, 6>(a, st); break;
    case 7: probe_t<R, NF, 7>(a, st); break;
    case 10: probe_t<R, NF, 10>(a, st); break;
    case 11: probe_t<R, NF, 11>(a, st); break;
    case 13: probe_t<R, NF, 13>(a, st); break;
    case 14: probe_t<R, NF, 14>(a, st); break;
    case 15: probe_t<R, NF, 15>(a, st); break;
    case 4: probe_t<R, NF, 4>(a, st); break;
    case 16: probe_t<R, NF, 16>(a, st); break;
    default: probe_t<R, NF, 8>(a, st); break;
    }
}

// Shared memory of one stage of the streamed iteration on this layout.
template <typename R, int NF>
size_t stream_stage_bytes(int emax, int hmax) {
    return StageLayout<R, NF>(emax, hmax).bytes;
}
template <typename R, int NF>
size_t ring_smem_bytes(int emax, int hmax, int stages) {
    return ring_bytes<R, NF>(emax, stages) + 2 * sizeof(FV<R, NF>) * (size_t)(kTileRows + hmax);
}
template size_t ring_smem_bytes<float, 1>(int, int, int);
template size_t ring_smem_bytes<float, 2>(int, int, int);
template size_t ring_smem_bytes<double, 1>(int, int, int);
template size_t ring_smem_bytes<double, 2>(int, int, int);
template size_t stream_stage_bytes<float, 1>(int, int);
template size_t stream_stage_bytes<float, 2>(int, int);
template size_t stream_stage_bytes<double, 1>(int, int);
template size_t stream_stage_bytes<double, 2>(int, int);

#define FEA_INST_STEP(R, NF)                                                                              \
    template void build_step_graph<R, NF>(StepGraph&, const StepArgs<R, NF>&, int, int, LoopFlags*);     \
    template void run_steps_stream<R, NF>(const StepArgs<R, NF>&, int, int, LoopFlags*, cudaStream_t);    \
    template void launch_spmv_probe<R, NF>(const StepArgs<R, NF>&, int, cudaStream_t);                 \
    template void prepare_probe<R, NF>(const StepArgs<R, NF>&, cudaStream_t);
FEA_INST_STEP(float, 1)
FEA_INST_STEP(float, 2)
FEA_INST_STEP(double, 1)
FEA_INST_STEP(double, 2)

}  // namespace fea
