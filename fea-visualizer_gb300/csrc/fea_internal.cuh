// fea_internal.cuh -- types shared by the translation units of libfea_gb300.
#pragma once

#include <vector>

#include "fea_common.cuh"

namespace fea {

// Compressed sparsity pattern of the stiffness/mass matrices plus the data
// that sums element entries into it in triplet order.
struct Pattern {
    int64_t N = 0, nnz = 0, ntrip = 0;
    int32_t* row_ptr = nullptr;    // [N+1]
    int32_t* col = nullptr;        // [nnz], sorted within a row
    int32_t* seg_start = nullptr;  // [nnz+1]: first bucket position of each slot
    int32_t* seg_id = nullptr;     // [ntrip]: triplet id (9k+3i+j) at each bucket position
    int32_t* slot_of = nullptr;    // [9T]: slot of each triplet id, -1 if filtered out
    int32_t* diag = nullptr;       // [N]: slot of the diagonal entry, -1 if absent
    int32_t* tpos = nullptr;       // [nnz]: slot of the transposed entry
    int32_t max_row = 0;
};

int launch_grid(int64_t n);
// Copy of P with the unknowns renumbered (pos[u] = new index, inv = inverse);
// emap[e'] receives the original slot of every new slot.
void build_permuted(const Pattern& P, const int32_t* pos, const int32_t* inv, Pattern& Pc, int32_t* emap,
                    DeviceArena& keep, cudaStream_t st);
void detect_boundary(const uint32_t* tri, int64_t T, int64_t V, uint8_t* ob, cudaStream_t st);
// Bit 0: a triangle index >= V; bit 1: a non-finite vertex coordinate; bit 2:
// a zero-area triangle (FP64 cross product of its edges is zero).  0: valid.
int check_mesh(const float* xyz, const uint32_t* tri, int64_t T, int64_t V, cudaStream_t st);
int64_t build_idx_map(const uint8_t* ob, int64_t V, int bc, int32_t* idx, cudaStream_t st);
void build_pattern(Pattern& P, DeviceArena& keep, const uint32_t* tri, int64_t T, const uint8_t* ob,
                   const int32_t* idx, int bc, int64_t N, cudaStream_t st);

// ---- tile-ELL operator layout (tile_ell.cu) ----------------------------------------
// Tiles of kTileRows solver-order rows (one row per thread of a kBlock-thread
// block), 32-row slices stored column by column, 16-bit tile-local column
// indices into [tile rows | tile halo].
constexpr int kTileRows = kBlock;
constexpr size_t kEllSmemBudget = 96 * 1024;  // largest staged operand per block
struct TileEll {
    int64_t E = 0;  // stored entries, padding included
    int ntiles = 0, hmax = 0;
    int emax = 0;                  // stored entries of the largest tile
    int32_t* slice_off = nullptr;  // [ntiles * 8 + 1] first entry of each slice
    int32_t* halo_off = nullptr;   // [ntiles + 1]
    int32_t* halo_col = nullptr;   // sorted distinct out-of-tile columns per tile
    uint16_t* lcol = nullptr;      // [E] local column index
    // [E] the same columns in pairs: slot sb + 32 m + lane of a slice that
    // starts at entry sb holds the local columns of its row's entries 2m (low
    // half) and 2m + 1 (high half) for m < ceil(width / 2); the slice's other
    // slots are unused.  One 32-bit load then brings two columns.
    uint32_t* lcol2 = nullptr;
    int32_t* emap = nullptr;       // [E] CSR slot of each entry, -1 for padding
    bool ok = false;
};
// From host copies of a solver-order CSR pattern.  Returns false (L.ok false)
// when a tile's halo does not fit the 16-bit indices or `smem_budget` bytes of
// shared memory at fv_bytes per operand.
// skip_diag: each row's diagonal entry is left out (a kernel that adds the
// diagonal term from the row's own values reads the rest); no lcol2.
bool build_tile_ell(const std::vector<int32_t>& rp, const std::vector<int32_t>& col, int64_t N, size_t fv_bytes,
                    size_t smem_budget, TileEll& L, DeviceArena& keep, cudaStream_t st, bool skip_diag = false);
// As[k] = A[emap[k]] (0 for padding): the layout's copy of operator values.
template <typename R, int NF>
void fill_tile_ell(const TileEll& L, const FV<R, NF>* A, FV<R, NF>* As, cudaStream_t st);

// ---- assembly (assemble.cu) ---------------------------------------------------
template <typename R>
void element_matrices(const float* xyz, const uint32_t* tri, int64_t T, int vel_mode, const float vel[3],
                      const float* elem_vel, R* Kloc, R* Mloc, R* Aloc, cudaStream_t st);
template <typename R>
void ordered_sum(const Pattern& P, const R* loc, const R* elem_scale, R* out, cudaStream_t st);
template <typename R>
void ordered_sum_adv(const Pattern& P, const R* loc, const uint32_t* tri, const uint8_t* ob, R* out,
                     uint8_t* present, cudaStream_t st);

// Operator values for NF fields: A_f = M / md_f + (k1_f * K) * k2_f + a1_f * Adv,
// evaluated per entry in FP64 from the FP64 matrices, then rounded once to R
// (FP32 handles store FP32 operators assembled in FP64).  dinv is the inverse
// of the stored (rounded) diagonal.
struct OpCoef1 {
    double md, k1, k2, a1;
};
template <int NF>
struct OpCoef {
    OpCoef1 f[NF];
};
// P is the pattern the operator is stored on; with emap, its slot e' takes the
// matrix values of slot emap[e'] (the matrices stay in the assembly order).
template <typename R, int NF>
void combine_operator(const Pattern& P, const int32_t* emap, const double* M, const double* K, const double* Adv,
                      const OpCoef<NF>& c, FV<R, NF>* A, FV<R, NF>* dinv, cudaStream_t st);
// out[i] = (R)in[map ? map[i] : i]
template <typename R>
void round_copy(const double* in, const int32_t* map, int64_t n, R* out, cudaStream_t st);

// ---- time stepping (cg.cu) ------------------------------------------------------
enum StepKind : int {
    EQ_HEAT = 0,         // b = (M/dt) u, also implicit advection-diffusion
    EQ_ADV_EXPLICIT = 1, // b = (M/dt) u + s Adv u
    EQ_WAVE_REF = 2,     // solve for v: b = (M/dt) v - c^2 K u; then u += dt v
    EQ_WAVE_NEWMARK = 3, // solve for a: b = -c^2 K u~; then u, v updates
    EQ_GS_REF = 4,       // (u, v): b = (M/dt) x + f(x) nodal
    EQ_GS_CONSISTENT = 5, // (u, v): b = M (x/dt + f(x))
    EQ_NEWMARK_INIT = 6,  // solve M a0 = -c^2 K u0 for Newmark's starting acceleration
    EQ_GIVEN = 7          // solve A x = rhs for a given right-hand side (the adjoint solve)
};

// Scalars of the step loop, device resident.
struct StepParams {
    double dt, F, k, c2, beta, gamma, adv_sign;
};

struct CgState {
    double rz[2], rr[2], pq[2], thr[2], bb[2], alpha[2], beta[2];
    // FP32 solvers: float-float (hi, lo) gamma, alpha and threshold, and the
    // coefficients alpha, beta rounded to float for the vector updates
    float ffrz[2][2], ffalpha[2][2], ffthr[2][2];
    float falpha[2], fbeta[2];
    int active[2];
    int fresh[2];  // the next direction is p = z (first iteration of a loop)
    int iters[2];
    int iter;
    int max_iter;
    int stop;     // this step is skipped (bad state detected at its start)
    int pending;  // deferred-finish kernels: the last kernel's iteration awaits its scalars
};

struct RunState {
    long long steps_left, steps_done, total_iters;
    long long cg_launches;  // iteration kernels run (timing probes excluded)
    unsigned int flags;
    int last_iters[2];
    double last_rel[2];
    double tol;
    int max_iter;
    int refine;
    int guess;       // Gray-Scott: 1 starts each step's CG from 2 x_n - x_(n-1)
    int prev_valid;  // x_(n-1) of the extrapolation is the previous step's state
};

// Everything a step-loop kernel needs, passed by value.
template <typename R, int NF>
struct StepArgs {
    int N;
    const int32_t* rp;
    const int32_t* col;
    const FV<R, NF>* A;     // operator values [nnz]
    const FV<R, NF>* dinv;  // [N]
    const R* M;             // mass values [nnz]
    const R* K;             // stiffness values [nnz] (diffusivity-scaled)
    const R* Adv;           // advection values [nnz]
    // Per-row vectors hold whole tiles: ceil(N / kTileRows) * kTileRows rows
    // (the streamed CG kernels copy 256-row tiles of them).
    FV<R, NF>* x;           // unknown of the solve (warm start and result)
    FV<R, NF>* b;
    FV<R, NF>* z;           // D^-1 r of the initial residual
    FV<R, NF>* pp[2];       // search direction (pp[0]; pp[1] only for the SpMV probe)
    FV<R, NF>* q;           // SpMV probe output
    FV<R, NF>* rb[2];       // residual r, w = A D^-1 r and s = A p, each in two
    FV<R, NF>* wb[2];       // buffers that alternate with the iteration parity
    FV<R, NF>* sb[2];       // (an iteration gathers the old and writes the new)
    R* u;                   // NF == 1 equations: displacement / field
    R* v;                   // velocity (wave)
    R* a;                   // acceleration (Newmark)
    R* ut;                  // Newmark predictors
    R* vt;
    const FV<R, NF>* rhs;   // EQ_GIVEN: right-hand side [N]
    // Gray-Scott initial-guess extrapolation (nullptr otherwise): the
    // previous step's state and the guess k_rhs formed; the set-up kernel
    // of a step's first solve (guess_init) moves x to xprev and the guess to x.
    FV<R, NF>* xprev;
    FV<R, NF>* xg;
    int guess_init;
    // tile-ELL copy of A (the CG kernels' layout when ell.ok)
    const FV<R, NF>* As;
    const uint16_t* lcol;
    const uint32_t* lcol2;  // column pairs (TileEll::lcol2)
    const int32_t* slice_off;
    const int32_t* halo_off;
    const int32_t* halo_col;
    int hmax, emax;
    // The same layout without the diagonal entries (ring kernels, when built):
    // the iteration adds the diagonal term A_ii u'_i = r'_i from the row's
    // own residual (u' = D^-1 r'), so the operator stream carries one entry
    // less per row.  Same halo lists.  Null: the full layout above.
    const FV<R, NF>* As_od;
    const uint16_t* lcol_od;
    const int32_t* slice_off_od;
    int emax_od;
    const R* Ms;  // tile-ELL copy of M (the staged Gray-Scott right-hand side), or null
    const StepParams* prm;
    CgState* cg;
    // Deferred-finish variants: the state is double-buffered (cg and cg_alt),
    // the partials too (part and part + 8 * part_stride); the iteration kernel
    // with node parity `par` reads state and partials of parity par ^ 1 and
    // writes parity par, where parity 1 is `cg` / `part`.  Every solve's
    // iterations then start at buffer parity 0 (defer = 1).
    CgState* cg_alt;
    int defer, par;
    RunState* run;
    double* part;           // block partials [16 * part_stride]
    int part_stride;
    unsigned int* tickets;  // [8]
    cudaGraphConditionalHandle cond;  // loop condition set by this kernel (graph mode)
    int* cont;              // the same condition, also stored here for host-driven loops
    int use_graph;          // 1: kernels run as graph nodes and set `cond`
    int probe;              // 1: a timing probe (iterates with every field masked)
};

// Loop-condition slots in device memory for host-driven (stream) execution.
struct LoopFlags {
    int cg1, cg2, step, probe;
};

// A built step-loop graph for one (precision, fields, equation, lanes) plan.
struct StepGraph {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int kind = -1, lanes = 0;
    void destroy() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        exec = nullptr;
        graph = nullptr;
    }
};

template <typename R, int NF>
void build_step_graph(StepGraph& g, const StepArgs<R, NF>& base, int kind, int lanes, LoopFlags* lf);

// The same step loop launched kernel by kernel, conditions read on the host
// (profiling mode: FEA_LAUNCH_MODE=stream).
template <typename R, int NF>
void run_steps_stream(const StepArgs<R, NF>& base, int kind, int lanes, LoopFlags* lf, cudaStream_t st);

// Timing and autotuning probe: one CG iteration kernel with the given window
// size, after prepare_probe has masked every field (x and p are written back
// unchanged; only CG scratch changes, which the next step recomputes).
// a.x and a.cont must be set.
template <typename R, int NF>
void prepare_probe(const StepArgs<R, NF>& a, cudaStream_t st);
template <typename R, int NF>
void launch_spmv_probe(const StepArgs<R, NF>& a, int lanes, cudaStream_t st);
// Dynamic shared memory of one stage of the streamed CG iteration (variants
// 2 and 3 hold 2 and 3 stages) for a tile-ELL layout with the given largest
// tile and halo.
template <typename R, int NF>
size_t stream_stage_bytes(int emax, int hmax);
constexpr size_t kStreamSmemLimit = 220 * 1024;  // per block, below the 227 KB opt-in maximum
// Dynamic shared memory of the ring iteration kernels (variants 14 and 15)
// with `stages` operator stages.
template <typename R, int NF>
size_t ring_smem_bytes(int emax, int hmax, int stages);

int max_grid_blocks();

// CG variants whose iteration kernels finish the previous launch's iteration
// at their start (deferred finish; see StepArgs::defer).
constexpr bool is_deferred_variant(int l) { return l >= 10 && l <= 15 && l != 12; }

// ---- adjoint of the explicit advection-diffusion step (adjoint.cu) ----------------
// lam = M (u - t), *J = 1/2 (u - t).lam  (exact accumulators; one block-partial
// reduction through part/ticket).
template <typename R>
void adjoint_loss(const Pattern& P, const R* M, const R* u, const R* t, R* lam, double* part, int stride,
                  unsigned int* ticket, double* J, cudaStream_t st);
// lam = (M/dt) mu + s Adv^T mu
template <typename R>
void adjoint_lambda(const Pattern& P, const R* M, const R* Adv, double dt, double adv_sign, const R* mu, R* lam,
                    cudaStream_t st);
// gD[e] -= c * mu_e^T K_e u_e for every element (K_e: unscaled element
// stiffness, FP64; idx_c maps nodes to solver rows, -1 on Dirichlet points)
template <typename R>
void adjoint_grad_D(const double* Kloc, const uint32_t* tri, const int32_t* idx_c, int64_t T, double c, const R* mu,
                    const R* u, double* gD, cudaStream_t st);

// ---- after the solve (surface.cu) ------------------------------------------------
// Vertex -> incident triangles (vt_ptr [V+1], vt_tri [3T], ascending per vertex).
void build_vertex_triangles(const uint32_t* tri, int64_t T, int64_t V, int32_t* vt_ptr, int32_t* vt_tri,
                            cudaStream_t st);
// Extruded smooth normals: face[3T] scratch, out[3V].
void smooth_normals(const float* xyz, const uint32_t* tri, int64_t T, int64_t V, const int32_t* vt_ptr,
                    const int32_t* vt_tri, const float* nrm, const float* val, float e, float* face, float* out,
                    cudaStream_t st);
// Export clipping: slots pos[18T], pval[6T], used[6T]; triangles otri[12T]
// (slot numbers, -1 when not emitted).
void ply_clip(const float* xyz, const uint32_t* tri, int64_t T, const float* nrm, const float* val, float e,
              float threshold, int mesh_type, float* pos, float* pval, uint8_t* used, int32_t* otri,
              cudaStream_t st);

// Gray-Scott (mass-weighted reaction) adjoint: lam = M (x - t) for the fields
// whose use flag is set, *J = 1/2 (x - t).lam; and one reverse step from
// mu = A^-1 lam (x0/x1: the step's input and output), accumulating
// g[4] += (dJ/dF, dJ/dk, dJ/dDu, dJ/dDv) of the step.
template <typename R>
void adjoint_gs_loss(const Pattern& P, const R* M, const FV<R, 2>* x, const FV<R, 2>* t, int use_u, int use_v,
                     FV<R, 2>* lam, double* part, int stride, unsigned int* ticket, double* J, cudaStream_t st);
template <typename R>
void adjoint_gs_step(const Pattern& P, const R* M, const R* K, const FV<R, 2>* mu, const FV<R, 2>* x0,
                     const FV<R, 2>* x1, double dt, double F, double k, FV<R, 2>* lam, double* part, int stride,
                     unsigned int* ticket, double* g, cudaStream_t st);

// Solver-order view of a handle's assembled mesh: what the batched solver
// copies out of a single-mesh handle built for each of its instances.
struct MeshView {
    int64_t V = 0, T = 0, N = 0;
    const Pattern* Pc = nullptr;    // pattern in solver order (diag filled)
    const int32_t* emap = nullptr;  // solver slot -> assembly slot
    const double* M64 = nullptr;    // FP64 matrices in assembly order
    const double* K64 = nullptr;
    const double* Adv64 = nullptr;
    const int32_t* idx_c = nullptr;  // node -> solver index, -1 on Dirichlet points
    cudaStream_t stream = nullptr;
};
MeshView mesh_view(const fea_solver* s);

}  // namespace fea
