// solver.cu -- the fea_solver handle and the C ABI of include/fea_gpu.h.
//
// A handle holds one mesh and plays the roles of the reference's FEMContext
// (mesh, idx_map, assembled matrices; src/FEM/FEMContext.cpp) and of a Solver
// implementation (state fields u, v and advance_time; include/FEM/Solver.hpp).
#include <algorithm>
#include <charconv>
#include <cstdio>
#include <unordered_map>
#include <cstdarg>
#include <cstring>
#include <new>
#include <utility>

#include "fea_internal.cuh"

namespace fea {

namespace {
thread_local char g_err[512] = "";
}

void set_error(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

int num_sms() {
    static int n = 0;
    if (n == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 152;
    }
    return n;
}

namespace {

// ---- node <-> unknown maps (CPUSolver.cpp:13-37) --------------------------------
// Stores a state value; a store that changes its bits clears *prev_valid (the
// extrapolated initial guess needs the state the loop itself produced, so a
// field written back unchanged between frames keeps the history).
template <typename R>
__device__ __forceinline__ void store_state(R* dst, R val, int* prev_valid) {
    if (prev_valid) {
        const R old = *dst;
        bool same;
        if constexpr (sizeof(R) == 8) same = __double_as_longlong(old) == __double_as_longlong(val);
        else same = __float_as_uint(old) == __float_as_uint(val);
        if (!same) *prev_valid = 0;
    }
    *dst = val;
}

template <typename R>
__global__ void k_gather_nodes(const float* __restrict__ vals, const int32_t* __restrict__ idx, int64_t V, R* out,
                               int stride, int off, int* prev_valid) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < V; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t k = idx[i];
        if (k >= 0) store_state(out + (int64_t)k * stride + off, (R)vals[i], prev_valid);
    }
}

template <typename R>
__global__ void k_scatter_nodes(const R* __restrict__ in, const int32_t* __restrict__ idx, int64_t V, float* out,
                                int stride, int off) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < V; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t k = idx[i];
        out[i] = k >= 0 ? (float)in[(int64_t)k * stride + off] : 0.0f;
    }
}

template <typename R>
__global__ void k_interleave(const R* __restrict__ u, const R* __restrict__ v, int64_t N, R* uv) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
        uv[2 * i] = u[i];
        uv[2 * i + 1] = v[i];
    }
}

template <typename R>
__global__ void k_deinterleave(const R* __restrict__ uv, int64_t N, R* u, R* v) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
        u[i] = uv[2 * i];
        v[i] = uv[2 * i + 1];
    }
}

// Caller-order unknown u <-> solver-order index pos[u].
template <typename R>
__global__ void k_copy_to_state(const R* __restrict__ in, const int32_t* __restrict__ pos, int64_t N, R* out,
                                int stride, int off, int* prev_valid) {
    for (int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; u < N; u += (int64_t)gridDim.x * blockDim.x)
        store_state(out + (int64_t)pos[u] * stride + off, in[u], prev_valid);
}

template <typename R>
__global__ void k_copy_from_state(const R* __restrict__ in, const int32_t* __restrict__ pos, int64_t N, R* out,
                                  int stride, int off) {
    for (int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; u < N; u += (int64_t)gridDim.x * blockDim.x)
        out[u] = in[(int64_t)pos[u] * stride + off];
}

__global__ void k_compose_idx(const int32_t* __restrict__ idx, const int32_t* __restrict__ pos, int64_t V,
                              int32_t* idx_c) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < V; i += (int64_t)gridDim.x * blockDim.x)
        idx_c[i] = idx[i] >= 0 ? pos[idx[i]] : -1;
}

template <typename R>
__global__ void k_float_to(const float* __restrict__ in, int64_t n, R* out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = (R)in[i];
}

// Reads n 16-byte words (evicting the L2 with clean lines); the sink is
// written only for an all-ones word, which the buffer (zeroed) never holds.
__global__ void k_read_flush(const uint4* __restrict__ p, int64_t n, unsigned int* sink) {
    unsigned int acc = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const uint4 v = __ldcg(p + i);
        acc |= v.x & v.y & v.z & v.w;
    }
    if (acc == 0xffffffffu) *sink = acc;
}

template <typename A, typename B>
__global__ void k_convert(const A* __restrict__ in, int64_t n, B* out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = (B)in[i];
}

}  // namespace

// Everything that depends on the arithmetic type.
struct Fields {
    int64_t N = 0;
    void* u = nullptr;   // R[N]
    void* v = nullptr;   // R[N]
    void* a = nullptr;   // R[N]  Newmark acceleration
    void* ut = nullptr;  // R[N]  Newmark predictors
    void* vt = nullptr;
    void* uv = nullptr;  // R[2N] interleaved (Gray-Scott)
    bool interleaved = false;  // (u, v) currently live in uv
    // solver work, one field (p1 holds the two alternating direction buffers)
    // r1/r2 hold the alternating r, w, s buffers of the Chronopoulos-Gear loop
    void *A1 = nullptr, *d1 = nullptr, *b1 = nullptr, *r1 = nullptr, *z1 = nullptr, *p1 = nullptr, *q1 = nullptr;
    void *A0 = nullptr, *d0 = nullptr;  // Newmark start-up operator (M)
    // two fields
    void *A2 = nullptr, *d2 = nullptr, *b2 = nullptr, *r2 = nullptr, *z2 = nullptr, *p2 = nullptr, *q2 = nullptr;
    void *xprev2 = nullptr, *xg2 = nullptr;  // Gray-Scott: previous state, extrapolated guess
};

}  // namespace fea

using namespace fea;

struct fea_solver {
    int device = 0;
    cudaStream_t stream = nullptr;
    int precision = FEA_FP32;
    int bc = FEA_DIRICHLET;
    int64_t V = 0, T = 0, nb = 0, N = 0;
    fea_params prm{};
    // mesh
    DeviceArena mesh_mem;
    float* xyz = nullptr;
    uint32_t* tri = nullptr;
    uint8_t* ob = nullptr;
    float* elem_D = nullptr;    // [T] per-element diffusivity (null: 1)
    float* elem_vel = nullptr;  // [3T]
    double* elem_Dr = nullptr;  // diffusivity widened to FP64 for assembly
    // FEMContext state (rebuilt on BC change)
    DeviceArena mat_mem;
    int32_t* idx = nullptr;
    Pattern P;
    double *Kloc = nullptr, *Mloc = nullptr, *Aloc = nullptr;  // element blocks [9T], FP64
    double *K64 = nullptr, *M64 = nullptr, *Adv64 = nullptr;   // assembled in FP64
    void *K = nullptr, *M = nullptr, *Adv = nullptr;           // in the handle's type (export)
    // the solver's ordering of the unknowns (Morton order of their points)
    Pattern Pc;                     // pattern in solver order
    int32_t* pos = nullptr;         // [N] unknown -> solver index
    int32_t* inv = nullptr;         // [N] solver index -> unknown
    int32_t* emap = nullptr;        // [nnz] solver slot -> assembly slot
    int32_t* idx_c = nullptr;       // [V] node -> solver index (-1 on Dirichlet points)
    void *Kc = nullptr, *Mc = nullptr, *Advc = nullptr;        // values in solver order
    TileEll ell;                    // the CG kernels' layout of Pc (tile_ell.cu)
    int stream_stages = 0;          // stages of the streamed iteration that fit in shared memory (0, 2 or 3)
    void *S1 = nullptr, *S0 = nullptr, *S2 = nullptr;          // tile-ELL copies of A1, A0, A2
    void* Ms_ell = nullptr;                                    // tile-ELL copy of M
    TileEll ell_od;                                            // the layout without diagonal entries (ring kernels)
    void *S1d = nullptr, *S0d = nullptr, *S2d = nullptr;       // its copies of A1, A0, A2
    std::vector<float> h_xyz;       // host copy of the points (ordering keys)
    uint8_t* adv_present = nullptr;
    Fields F;
    // loop state
    DeviceArena run_mem;
    StepParams* d_prm = nullptr;
    CgState* d_cg = nullptr;
    RunState* d_run = nullptr;
    double* d_part = nullptr;
    unsigned int* d_tickets = nullptr;
    LoopFlags* d_flags = nullptr;
    bool stream_mode = false;  // FEA_LAUNCH_MODE=stream: kernel-by-kernel launches
    RunState* h_run = nullptr;  // pinned
    StepGraph graph, init_graph;
    int lanes = 8;  // CG kernel variant: 0/1 tile-ELL (8/4 entries prefetched), 2/3 streamed (stages), 4/8/16 CSR window
    bool op_dirty = true;
    int op_kind = -1;
    bool acc_valid = false;
    float cur_vel[3] = {1.f, 0.f, 0.f};
    int cur_vel_mode = 0;
    float* d_nodes = nullptr;  // node-indexed staging buffer [V] for host field copies
    int32_t* vt_ptr = nullptr;  // vertex -> triangles (built on first use)
    int32_t* vt_tri = nullptr;
};

namespace fea {
namespace {

size_t rsize(const fea_solver* s) { return s->precision == FEA_FP64 ? 8 : 4; }

// Entries of the largest tile the ring kernels stream (the diagonal-free
// layout when it was built).
// The widest tile of the ring kernels' layouts: the set-up product streams
// the full layout, the iteration the one without the diagonal.
int ring_emax(const fea_solver* s) { return s->ell.emax; }

int64_t pad_tiles(int64_t n) { return ceil_div(n, kTileRows) * kTileRows; }

void* ralloc(DeviceArena& ar, const fea_solver* s, int64_t n) {
    if (s->precision == FEA_FP64) return ar.alloc<double>(n);
    return ar.alloc<float>(n);
}

int step_kind(const fea_params& p) {
    switch (p.equation) {
    case FEA_HEAT: return EQ_HEAT;
    case FEA_ADVECTION_DIFFUSION: return p.advection_scheme == 1 ? EQ_ADV_EXPLICIT : EQ_HEAT;
    case FEA_WAVE: return p.wave_scheme == 1 ? EQ_WAVE_NEWMARK : EQ_WAVE_REF;
    case FEA_REACTION_DIFFUSION: return p.reaction_mode == 1 ? EQ_GS_CONSISTENT : EQ_GS_REF;
    default: return -1;
    }
}

bool two_fields(int kind) { return kind == EQ_GS_REF || kind == EQ_GS_CONSISTENT; }

double time_step(const fea_params& p) {
    switch (p.equation) {
    case FEA_HEAT: return p.heat_time_step;
    case FEA_ADVECTION_DIFFUSION: return p.advdiff_time_step;
    case FEA_WAVE: return p.wave_time_step;
    default: return p.rd_time_step;
    }
}

// Assembly runs in FP64 for both precisions (once per mesh or parameter
// change); FP32 handles then round the assembled values once, so their
// matrices carry only the final FP32 rounding.
void assemble(fea_solver* s) {
    const bool vel_elem = s->prm.velocity_mode == 1 && s->elem_vel;
    element_matrices<double>(s->xyz, s->tri, s->T, vel_elem ? 1 : 0, s->prm.advdiff_velocity, s->elem_vel,
                             s->Kloc, s->Mloc, s->Aloc, s->stream);
    ordered_sum<double>(s->P, s->Kloc, s->elem_Dr, s->K64, s->stream);
    ordered_sum<double>(s->P, s->Mloc, nullptr, s->M64, s->stream);
    ordered_sum_adv<double>(s->P, s->Aloc, s->tri, s->ob, s->Adv64, s->adv_present, s->stream);
    if (s->precision == FEA_FP32) {
        round_copy<float>(s->K64, nullptr, s->P.nnz, (float*)s->K, s->stream);
        round_copy<float>(s->M64, nullptr, s->P.nnz, (float*)s->M, s->stream);
        round_copy<float>(s->Adv64, nullptr, s->P.nnz, (float*)s->Adv, s->stream);
        round_copy<float>(s->K64, s->emap, s->P.nnz, (float*)s->Kc, s->stream);
        round_copy<float>(s->M64, s->emap, s->P.nnz, (float*)s->Mc, s->stream);
        round_copy<float>(s->Adv64, s->emap, s->P.nnz, (float*)s->Advc, s->stream);
        fill_tile_ell<float, 1>(s->ell, (const FV<float, 1>*)s->Mc, (FV<float, 1>*)s->Ms_ell, s->stream);
    } else {
        round_copy<double>(s->K64, s->emap, s->P.nnz, (double*)s->Kc, s->stream);
        round_copy<double>(s->M64, s->emap, s->P.nnz, (double*)s->Mc, s->stream);
        round_copy<double>(s->Adv64, s->emap, s->P.nnz, (double*)s->Advc, s->stream);
        fill_tile_ell<double, 1>(s->ell, (const FV<double, 1>*)s->Mc, (FV<double, 1>*)s->Ms_ell, s->stream);
    }
    memcpy(s->cur_vel, s->prm.advdiff_velocity, sizeof(s->cur_vel));
    s->cur_vel_mode = s->prm.velocity_mode;
    s->op_dirty = true;
}

uint64_t spread3(uint32_t x) {  // 21 bits -> every third bit of 63
    uint64_t v = x & 0x1fffffu;
    v = (v | (v << 32)) & 0x1f00000000ffffull;
    v = (v | (v << 16)) & 0x1f0000ff0000ffull;
    v = (v | (v << 8)) & 0x100f00f00f00f00full;
    v = (v | (v << 4)) & 0x10c30c30c30c30c3ull;
    v = (v | (v << 2)) & 0x1249249249249249ull;
    return v;
}

// The solver's ordering of the unknowns: sorted by the 63-bit Morton key of
// their points (coordinates quantised to 21 bits over the bounding box), ties
// by unknown number, then by stored-entry count within each tile of
// kTileRows rows.  Neighbouring points get nearby numbers, so a tile is a
// compact patch whose rows mostly reference each other.  Computed on the host
// once per mesh and boundary condition.
void build_ordering(fea_solver* s) {
    cudaStream_t st = s->stream;
    const int64_t V = s->V, N = s->N;
    std::vector<int32_t> idx(V);
    FEA_CUDA_TRY(cudaMemcpyAsync(idx.data(), s->idx, sizeof(int32_t) * V, cudaMemcpyDeviceToHost, st));
    FEA_CUDA_TRY(cudaStreamSynchronize(st));
    float lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    for (int d = 0; d < 3; d++) {
        lo[d] = hi[d] = V ? s->h_xyz[d] : 0.f;
        for (int64_t i = 0; i < V; i++) {
            lo[d] = std::min(lo[d], s->h_xyz[3 * i + d]);
            hi[d] = std::max(hi[d], s->h_xyz[3 * i + d]);
        }
    }
    std::vector<std::pair<uint64_t, int32_t>> key;
    key.reserve(N);
    for (int64_t i = 0; i < V; i++) {
        if (idx[i] < 0) continue;
        uint64_t m = 0;
        for (int d = 0; d < 3; d++) {
            const double ext = (double)hi[d] - (double)lo[d];
            double t = ext > 0 ? ((double)s->h_xyz[3 * i + d] - lo[d]) / ext : 0.0;
            t = t < 0 ? 0 : (t > 1 ? 1 : t);
            m |= spread3((uint32_t)(t * 2097151.0)) << d;
        }
        key.emplace_back(m, idx[i]);
    }
    std::sort(key.begin(), key.end());
    // within each tile of kTileRows rows, rows by stored-entry count, so the
    // 32-row slices of the tile-ELL layout carry little padding (the tile's
    // row set, hence its locality, is that of the Morton order)
    std::vector<int32_t> rp(N + 1);
    FEA_CUDA_TRY(cudaMemcpyAsync(rp.data(), s->P.row_ptr, sizeof(int32_t) * (N + 1), cudaMemcpyDeviceToHost, st));
    FEA_CUDA_TRY(cudaStreamSynchronize(st));
    std::vector<int32_t> pos(N), inv(N);
    for (int64_t c = 0; c < N; c++) inv[c] = key[c].second;
    for (int64_t t0 = 0; t0 < N; t0 += kTileRows)
        std::stable_sort(inv.begin() + t0, inv.begin() + std::min<int64_t>(N, t0 + kTileRows),
                         [&](int32_t a, int32_t b) { return rp[a + 1] - rp[a] < rp[b + 1] - rp[b]; });
    for (int64_t c = 0; c < N; c++) pos[inv[c]] = (int32_t)c;
    s->pos = s->mat_mem.alloc<int32_t>(N);
    s->inv = s->mat_mem.alloc<int32_t>(N);
    s->emap = s->mat_mem.alloc<int32_t>(s->P.nnz);
    s->idx_c = s->mat_mem.alloc<int32_t>(V);
    if (N > 0) {
        FEA_CUDA_TRY(cudaMemcpyAsync(s->pos, pos.data(), sizeof(int32_t) * N, cudaMemcpyHostToDevice, st));
        FEA_CUDA_TRY(cudaMemcpyAsync(s->inv, inv.data(), sizeof(int32_t) * N, cudaMemcpyHostToDevice, st));
    }
    k_compose_idx<<<launch_grid(V), kBlock, 0, st>>>(s->idx, s->pos, V, s->idx_c);
    FEA_CHECK_LAUNCH();
    build_permuted(s->P, s->pos, s->inv, s->Pc, s->emap, s->mat_mem, st);
}

// FEMContext::update_boundary_conditions + assemble_matrices and the state.
void build_context(fea_solver* s) {
    s->graph.destroy();
    s->init_graph.destroy();
    s->mat_mem.release();
    s->P = Pattern{};
    s->Pc = Pattern{};
    s->ell = TileEll{};
    s->ell_od = TileEll{};
    s->stream_stages = 0;
    s->S1 = s->S0 = s->S2 = nullptr;
    s->S1d = s->S0d = s->S2d = nullptr;
    s->Ms_ell = nullptr;
    s->F = Fields{};
    cudaStream_t st = s->stream;
    s->idx = s->mat_mem.alloc<int32_t>(s->V);
    s->N = build_idx_map(s->ob, s->V, s->bc, s->idx, st);
    build_pattern(s->P, s->mat_mem, s->tri, s->T, s->ob, s->idx, s->bc, s->N, st);
    const int64_t N = s->N, nnz = s->P.nnz, T = s->T;
    build_ordering(s);
    {
        std::vector<int32_t> rp(N + 1), col(nnz);
        FEA_CUDA_TRY(cudaMemcpyAsync(rp.data(), s->Pc.row_ptr, sizeof(int32_t) * (N + 1), cudaMemcpyDeviceToHost, st));
        if (nnz > 0)
            FEA_CUDA_TRY(cudaMemcpyAsync(col.data(), s->Pc.col, sizeof(int32_t) * nnz, cudaMemcpyDeviceToHost, st));
        FEA_CUDA_TRY(cudaStreamSynchronize(st));
        build_tile_ell(rp, col, N, 2 * rsize(s), kEllSmemBudget, s->ell, s->mat_mem, st);
        if (s->ell.ok) {
            s->S1 = ralloc(s->mat_mem, s, s->ell.E);
            s->S0 = ralloc(s->mat_mem, s, s->ell.E);
            s->S2 = ralloc(s->mat_mem, s, 2 * s->ell.E);
            s->Ms_ell = ralloc(s->mat_mem, s, s->ell.E);
            if (build_tile_ell(rp, col, N, 2 * rsize(s), kEllSmemBudget, s->ell_od, s->mat_mem, st, true)) {
                s->S1d = ralloc(s->mat_mem, s, s->ell_od.E);
                s->S0d = ralloc(s->mat_mem, s, s->ell_od.E);
                s->S2d = ralloc(s->mat_mem, s, 2 * s->ell_od.E);
            }
        }
        // both field counts fit when the two-field stages do
        const size_t stage = s->precision == FEA_FP64 ? stream_stage_bytes<double, 2>(s->ell.emax, s->ell.hmax)
                                                      : stream_stage_bytes<float, 2>(s->ell.emax, s->ell.hmax);
        s->stream_stages = !s->ell.ok ? 0 : 3 * stage <= kStreamSmemLimit ? 3 : 2 * stage <= kStreamSmemLimit ? 2 : 0;
        // default variant: direct row loads with the operator ring (14) when
        // its stages fit, else the streamed deferred-finish kernel with as
        // many stages as fit, else the tile-ELL kernel, else windowed CSR
        const int remax = ring_emax(s);
        const size_t ring = s->precision == FEA_FP64 ? ring_smem_bytes<double, 2>(remax, s->ell.hmax, 3)
                                                     : ring_smem_bytes<float, 2>(remax, s->ell.hmax, 3);
        s->lanes = !s->ell.ok ? 8
                   : ring <= kStreamSmemLimit ? 14
                   : s->stream_stages >= 3    ? 11
                   : s->stream_stages >= 2    ? 10
                                              : 0;
    }
    s->Kloc = s->mat_mem.alloc<double>(9 * T);
    s->Mloc = s->mat_mem.alloc<double>(9 * T);
    s->Aloc = s->mat_mem.alloc<double>(9 * T);
    s->K64 = s->mat_mem.alloc<double>(nnz);
    s->M64 = s->mat_mem.alloc<double>(nnz);
    s->Adv64 = s->mat_mem.alloc<double>(nnz);
    if (s->precision == FEA_FP64) {
        s->K = s->K64;
        s->M = s->M64;
        s->Adv = s->Adv64;
    } else {
        s->K = ralloc(s->mat_mem, s, nnz);
        s->M = ralloc(s->mat_mem, s, nnz);
        s->Adv = ralloc(s->mat_mem, s, nnz);
    }
    s->Kc = ralloc(s->mat_mem, s, nnz);
    s->Mc = ralloc(s->mat_mem, s, nnz);
    s->Advc = ralloc(s->mat_mem, s, nnz);
    s->adv_present = s->mat_mem.alloc<uint8_t>(nnz);
    Fields& F = s->F;
    F.N = N;
    // every per-row vector holds whole tiles (Nt rows, zero beyond N): the
    // streamed CG kernels copy 256-row tiles of them into shared memory
    const int64_t Nt = ceil_div(N, kTileRows) * kTileRows;
    F.u = ralloc(s->mat_mem, s, Nt);
    F.v = ralloc(s->mat_mem, s, Nt);
    F.a = ralloc(s->mat_mem, s, Nt);
    F.ut = ralloc(s->mat_mem, s, Nt);
    F.vt = ralloc(s->mat_mem, s, Nt);
    F.uv = ralloc(s->mat_mem, s, 2 * Nt);
    F.A1 = ralloc(s->mat_mem, s, nnz);
    F.d1 = ralloc(s->mat_mem, s, Nt);
    F.b1 = ralloc(s->mat_mem, s, Nt);
    const int64_t Np = Nt;  // every buffer of a group starts on a tile boundary
    F.r1 = ralloc(s->mat_mem, s, 6 * Np);  // r, w, s: two buffers each
    F.z1 = ralloc(s->mat_mem, s, Nt);
    F.p1 = ralloc(s->mat_mem, s, 2 * Np);
    F.q1 = ralloc(s->mat_mem, s, Nt);
    F.A0 = ralloc(s->mat_mem, s, nnz);
    F.d0 = ralloc(s->mat_mem, s, Nt);
    F.A2 = ralloc(s->mat_mem, s, 2 * nnz);
    F.d2 = ralloc(s->mat_mem, s, 2 * Nt);
    F.b2 = ralloc(s->mat_mem, s, 2 * Nt);
    F.r2 = ralloc(s->mat_mem, s, 12 * Np);
    F.z2 = ralloc(s->mat_mem, s, 2 * Nt);
    F.p2 = ralloc(s->mat_mem, s, 4 * Np);
    F.q2 = ralloc(s->mat_mem, s, 2 * Nt);
    F.xprev2 = ralloc(s->mat_mem, s, 2 * Nt);
    F.xg2 = ralloc(s->mat_mem, s, 2 * Nt);
    // every vector starts at zero (the direction buffers are read with weight
    // beta = 0 only after a write, but a zero start keeps them finite)
    const std::pair<void*, int64_t> zeroed[] = {
        {F.u, Nt}, {F.v, Nt}, {F.a, Nt}, {F.ut, Nt}, {F.vt, Nt}, {F.uv, 2 * Nt}, {F.d1, Nt}, {F.b1, Nt},
        {F.r1, 6 * Np}, {F.z1, Nt}, {F.p1, 2 * Np}, {F.q1, Nt}, {F.d0, Nt}, {F.d2, 2 * Nt}, {F.b2, 2 * Nt},
        {F.r2, 12 * Np}, {F.z2, 2 * Nt}, {F.p2, 4 * Np}, {F.q2, 2 * Nt}, {F.xprev2, 2 * Nt}, {F.xg2, 2 * Nt}};
    for (const auto& zv : zeroed)
        FEA_CUDA_TRY(cudaMemsetAsync(zv.first, 0, rsize(s) * (size_t)(zv.second > 0 ? zv.second : 1), st));
    F.interleaved = false;
    s->acc_valid = false;
    assemble(s);
    FEA_CUDA_TRY(cudaStreamSynchronize(st));
}

// r, w and s of the Chronopoulos-Gear iteration, two buffers each, carved
// from one allocation of 6 * Np unknowns.
template <typename R, int NF>
void set_rws(StepArgs<R, NF>& a, FV<R, NF>* base, int64_t Np) {
    for (int k = 0; k < 2; k++) {
        a.rb[k] = base + k * Np;
        a.wb[k] = base + (2 + k) * Np;
        a.sb[k] = base + (4 + k) * Np;
    }
}

template <typename R, int NF>
StepArgs<R, NF> make_args(fea_solver* s, bool init_op) {
    StepArgs<R, NF> a{};
    Fields& F = s->F;
    a.N = (int)s->N;
    a.rp = s->Pc.row_ptr;
    a.col = s->Pc.col;
    a.M = (const R*)s->Mc;
    a.K = (const R*)s->Kc;
    a.Adv = (const R*)s->Advc;
    if constexpr (NF == 1) {
        a.A = (const FV<R, 1>*)(init_op ? F.A0 : F.A1);
        a.dinv = (const FV<R, 1>*)(init_op ? F.d0 : F.d1);
        a.b = (FV<R, 1>*)F.b1;
        set_rws(a, (FV<R, 1>*)F.r1, pad_tiles(s->N));
        a.z = (FV<R, 1>*)F.z1;
        a.pp[0] = (FV<R, 1>*)F.p1;
        a.pp[1] = a.pp[0] + pad_tiles(s->N);
        a.q = (FV<R, 1>*)F.q1;
    } else {
        a.A = (const FV<R, 2>*)F.A2;
        a.dinv = (const FV<R, 2>*)F.d2;
        a.b = (FV<R, 2>*)F.b2;
        set_rws(a, (FV<R, 2>*)F.r2, pad_tiles(s->N));
        a.z = (FV<R, 2>*)F.z2;
        a.pp[0] = (FV<R, 2>*)F.p2;
        a.pp[1] = a.pp[0] + pad_tiles(s->N);
        a.q = (FV<R, 2>*)F.q2;
    }
    a.u = (R*)F.u;
    a.v = (R*)F.v;
    a.a = (R*)F.a;
    a.ut = (R*)F.ut;
    a.vt = (R*)F.vt;
    if (s->ell.ok) {
        if constexpr (NF == 1) a.As = (const FV<R, 1>*)(init_op ? s->S0 : s->S1);
        else a.As = (const FV<R, 2>*)s->S2;
        a.lcol = s->ell.lcol;
        a.lcol2 = s->ell.lcol2;
        a.slice_off = s->ell.slice_off;
        a.halo_off = s->ell.halo_off;
        a.halo_col = s->ell.halo_col;
        a.hmax = s->ell.hmax;
        a.emax = s->ell.emax;
        a.Ms = (const R*)s->Ms_ell;
        if (s->ell_od.ok) {
            if constexpr (NF == 1) a.As_od = (const FV<R, 1>*)(init_op ? s->S0d : s->S1d);
            else a.As_od = (const FV<R, 2>*)s->S2d;
            a.lcol_od = s->ell_od.lcol;
            a.slice_off_od = s->ell_od.slice_off;
            a.emax_od = s->ell_od.emax;
        }
    }
    a.prm = s->d_prm;
    a.cg = s->d_cg + 1;
    a.cg_alt = s->d_cg;
    a.defer = is_deferred_variant(s->lanes) ? 1 : 0;
    a.run = s->d_run;
    a.part = s->d_part;
    a.part_stride = max_grid_blocks();
    a.tickets = s->d_tickets;
    return a;
}

// Unknown vector of the solve for each kind.
template <typename R, int NF>
void set_x(fea_solver* s, StepArgs<R, NF>& a, int kind) {
    Fields& F = s->F;
    if constexpr (NF == 2) {
        a.x = (FV<R, 2>*)F.uv;
        if (kind == EQ_GS_REF || kind == EQ_GS_CONSISTENT) {  // the initial-guess extrapolation's buffers
            a.xprev = (FV<R, 2>*)F.xprev2;
            a.xg = (FV<R, 2>*)F.xg2;
        }
    } else {
        if (kind == EQ_WAVE_REF) a.x = (FV<R, 1>*)F.v;
        else if (kind == EQ_WAVE_NEWMARK || kind == EQ_NEWMARK_INIT) a.x = (FV<R, 1>*)F.a;
        else a.x = (FV<R, 1>*)F.u;
    }
}

template <typename R>
void upload_params(fea_solver* s) {
    const fea_params& p = s->prm;
    StepParams h{};
    h.dt = time_step(p);
    h.F = p.rd_feed_rate;
    h.k = p.rd_kill_rate;
    const R c = (R)p.wave_c;
    h.c2 = (double)(R)(c * c);
    h.beta = p.newmark_beta;
    h.gamma = p.newmark_gamma;
    h.adv_sign = p.advection_sign;
    FEA_CUDA_TRY(cudaMemcpyAsync(s->d_prm, &h, sizeof(h), cudaMemcpyHostToDevice, s->stream));
    RunState r{};
    FEA_CUDA_TRY(cudaMemcpyAsync(&r, s->d_run, sizeof(r), cudaMemcpyDeviceToHost, s->stream));
    FEA_CUDA_TRY(cudaStreamSynchronize(s->stream));
    double tol = p.cg_tolerance;
    if (!(tol > 0.0)) tol = s->precision == FEA_FP64 ? 1e-10 : 1.1920928955078125e-07;
    r.tol = tol;
    r.max_iter = p.cg_max_iterations > 0 ? p.cg_max_iterations : (int)(2 * s->N > 0x7fffffff ? 0x7fffffff : 2 * s->N);
    r.refine = p.cg_refine;
    if (r.guess != p.cg_initial_guess) r.prev_valid = 0;  // a new rule starts from the warm start
    r.guess = p.cg_initial_guess;
    FEA_CUDA_TRY(cudaMemcpyAsync(s->d_run, &r, sizeof(r), cudaMemcpyHostToDevice, s->stream));
    FEA_CUDA_TRY(cudaStreamSynchronize(s->stream));
}

// Operator coefficients (the float parameters widened to double; the
// operator is evaluated in FP64 and rounded once to the handle's type).
template <typename R>
void update_operator(fea_solver* s, int kind) {
    const fea_params& p = s->prm;
    const double dt = time_step(p);
    if (kind == EQ_GS_REF || kind == EQ_GS_CONSISTENT) {
        OpCoef<2> c{};
        c.f[0] = {dt, (double)p.rd_Du, 1.0, 0.0};
        c.f[1] = {dt, (double)p.rd_Dv, 1.0, 0.0};
        combine_operator<R, 2>(s->Pc, s->emap, s->M64, s->K64, s->Adv64, c, (FV<R, 2>*)s->F.A2, (FV<R, 2>*)s->F.d2,
                               s->stream);
        fill_tile_ell<R, 2>(s->ell, (const FV<R, 2>*)s->F.A2, (FV<R, 2>*)s->S2, s->stream);
        fill_tile_ell<R, 2>(s->ell_od, (const FV<R, 2>*)s->F.A2, (FV<R, 2>*)s->S2d, s->stream);
    } else {
        OpCoef<1> c{};
        c.f[0] = {dt, 0.0, 1.0, 0.0};
        if (kind == EQ_HEAT && p.equation == FEA_HEAT) {
            c.f[0].k1 = p.heat_conductivity;
        } else if (kind == EQ_HEAT) {  // implicit advection-diffusion, CPUSolver.cpp:95
            c.f[0].k1 = p.advdiff_c;
            c.f[0].a1 = -1.0;
        } else if (kind == EQ_ADV_EXPLICIT) {
            c.f[0].k1 = p.advdiff_c;
        } else if (kind == EQ_WAVE_REF) {  // M/dt + (c^2 K) dt, CPUSolver.cpp:113
            const double cc = p.wave_c;
            c.f[0].k1 = cc * cc;
            c.f[0].k2 = dt;
        } else {  // Newmark: M + (beta dt^2 c^2) K
            const double cc = p.wave_c;
            c.f[0].md = 1.0;
            c.f[0].k1 = p.newmark_beta * dt * dt * (cc * cc);
            OpCoef<1> m{};
            m.f[0] = {1.0, 0.0, 1.0, 0.0};
            combine_operator<R, 1>(s->Pc, s->emap, s->M64, s->K64, s->Adv64, m, (FV<R, 1>*)s->F.A0, (FV<R, 1>*)s->F.d0,
                                   s->stream);
            fill_tile_ell<R, 1>(s->ell, (const FV<R, 1>*)s->F.A0, (FV<R, 1>*)s->S0, s->stream);
            fill_tile_ell<R, 1>(s->ell_od, (const FV<R, 1>*)s->F.A0, (FV<R, 1>*)s->S0d, s->stream);
        }
        combine_operator<R, 1>(s->Pc, s->emap, s->M64, s->K64, s->Adv64, c, (FV<R, 1>*)s->F.A1, (FV<R, 1>*)s->F.d1,
                               s->stream);
        fill_tile_ell<R, 1>(s->ell, (const FV<R, 1>*)s->F.A1, (FV<R, 1>*)s->S1, s->stream);
        fill_tile_ell<R, 1>(s->ell_od, (const FV<R, 1>*)s->F.A1, (FV<R, 1>*)s->S1d, s->stream);
    }
}

// Fields changed from outside the step loop: the next step starts its solves
// from the previous solution (the initial-guess extrapolation needs two steps
// of the loop's own history).
void invalidate_guess(fea_solver* s) {
    if (s->d_run) FEA_CUDA_TRY(cudaMemsetAsync(&s->d_run->prev_valid, 0, sizeof(int), s->stream));
}

// Forces the previous-solution start while it lives (the adjoints recompute
// forward states from checkpoints and must reproduce them exactly), then
// restores the handle's rule.
struct GuessOff {
    fea_solver* s;
    explicit GuessOff(fea_solver* h) : s(h) {
        const int zero = 0;
        FEA_CUDA_TRY(cudaMemcpyAsync(&s->d_run->guess, &zero, sizeof(int), cudaMemcpyHostToDevice, s->stream));
        FEA_CUDA_TRY(cudaStreamSynchronize(s->stream));
    }
    ~GuessOff() {
        const int g = s->prm.cg_initial_guess;
        cudaMemcpyAsync(&s->d_run->guess, &g, sizeof(int), cudaMemcpyHostToDevice, s->stream);
        cudaMemsetAsync(&s->d_run->prev_valid, 0, sizeof(int), s->stream);
        cudaStreamSynchronize(s->stream);
    }
};

template <typename R>
void ensure_layout(fea_solver* s, bool interleaved) {
    Fields& F = s->F;
    if (F.interleaved == interleaved || F.N == 0) {
        F.interleaved = interleaved;
        return;
    }
    if (interleaved)
        k_interleave<R><<<launch_grid(F.N), kBlock, 0, s->stream>>>((R*)F.u, (R*)F.v, F.N, (R*)F.uv);
    else
        k_deinterleave<R><<<launch_grid(F.N), kBlock, 0, s->stream>>>((R*)F.uv, F.N, (R*)F.u, (R*)F.v);
    FEA_CHECK_LAUNCH();
    invalidate_guess(s);
    F.interleaved = interleaved;
}

template <typename R, int NF>
void run_graph(fea_solver* s, StepGraph& g, int kind, bool init_op, int64_t nsteps) {
    const bool stream_mode = s->stream_mode;
    if (!stream_mode && (!g.exec || g.kind != kind || g.lanes != s->lanes)) {
        StepArgs<R, NF> a = make_args<R, NF>(s, init_op);
        set_x<R, NF>(s, a, kind);
        build_step_graph<R, NF>(g, a, kind, s->lanes, s->d_flags);
    }
    long long ctl[2] = {nsteps, 0};  // steps_left, steps_done
    FEA_CUDA_TRY(cudaMemcpyAsync(s->d_run, ctl, sizeof(ctl), cudaMemcpyHostToDevice, s->stream));
    FEA_CUDA_TRY(cudaMemsetAsync(&s->d_run->flags, 0, sizeof(unsigned int), s->stream));
    if (stream_mode) {
        StepArgs<R, NF> a = make_args<R, NF>(s, init_op);
        set_x<R, NF>(s, a, kind);
        run_steps_stream<R, NF>(a, kind, s->lanes, s->d_flags, s->stream);
    } else {
        FEA_CUDA_TRY(cudaGraphLaunch(g.exec, s->stream));
    }
}

template <typename R>
void advance(fea_solver* s, int64_t nsteps) {
    const int kind = step_kind(s->prm);
    if (kind < 0) throw Error{FEA_ERR_INVALID_ARGUMENT};
    const bool vel_changed = s->prm.velocity_mode != s->cur_vel_mode ||
                             memcmp(s->cur_vel, s->prm.advdiff_velocity, sizeof(s->cur_vel)) != 0;
    if (vel_changed) assemble(s);
    if (s->op_dirty || s->op_kind != kind) {
        update_operator<R>(s, kind);
        s->op_dirty = false;
        s->op_kind = kind;
    }
    ensure_layout<R>(s, two_fields(kind));
    if (kind == EQ_WAVE_NEWMARK && !s->acc_valid) {
        // a0 from M a0 = -c^2 K u0
        FEA_CUDA_TRY(cudaMemsetAsync(s->F.a, 0, rsize(s) * (size_t)(s->N > 0 ? s->N : 1), s->stream));
        run_graph<R, 1>(s, s->init_graph, EQ_NEWMARK_INIT, true, 1);
        s->acc_valid = true;
    }
    if (two_fields(kind)) run_graph<R, 2>(s, s->graph, kind, false, nsteps);
    else run_graph<R, 1>(s, s->graph, kind, false, nsteps);
}

void check_handle(const fea_solver* s) {
    if (!s) {
        set_error("null handle");
        throw Error{FEA_ERR_INVALID_ARGUMENT};
    }
    FEA_CUDA_TRY(cudaSetDevice(s->device));
}

// The device alias of a page-locked host buffer, or nullptr for pageable
// memory.  Page-locked host memory is mapped into the device's address space
// (unified addressing), so the node gather and scatter kernels read and write
// it directly over the host link, in one pass and without the staging copy.
const void* mapped_alias(const void* host) {
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, host) != cudaSuccess) {
        (void)cudaGetLastError();  // an unknown pointer is pageable memory
        return nullptr;
    }
    return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
}

// Host fields travel through the handle's node-sized staging buffer, or are
// read and written in place when the caller's buffer is page-locked.
template <typename R>
void set_node_field(fea_solver* s, const float* host, int which /*0 u, 1 v*/) {
    const float* d = static_cast<const float*>(mapped_alias(host));
    if (!d) {
        FEA_CUDA_TRY(cudaMemcpyAsync(s->d_nodes, host, sizeof(float) * s->V, cudaMemcpyHostToDevice, s->stream));
        d = s->d_nodes;
    }
    Fields& F = s->F;
    int* pv = s->d_run ? &s->d_run->prev_valid : nullptr;
    if (F.interleaved)
        k_gather_nodes<R><<<launch_grid(s->V), kBlock, 0, s->stream>>>(d, s->idx_c, s->V, (R*)F.uv, 2, which, pv);
    else
        k_gather_nodes<R><<<launch_grid(s->V), kBlock, 0, s->stream>>>(d, s->idx_c, s->V,
                                                                        (R*)(which ? F.v : F.u), 1, 0, pv);
    FEA_CHECK_LAUNCH();
    FEA_CUDA_TRY(cudaStreamSynchronize(s->stream));
}

template <typename R>
void get_node_field(fea_solver* s, float* host, int which) {
    float* mapped = static_cast<float*>(const_cast<void*>(mapped_alias(host)));
    float* d = mapped ? mapped : s->d_nodes;
    Fields& F = s->F;
    if (F.interleaved)
        k_scatter_nodes<R><<<launch_grid(s->V), kBlock, 0, s->stream>>>((R*)F.uv, s->idx_c, s->V, d, 2, which);
    else
        k_scatter_nodes<R><<<launch_grid(s->V), kBlock, 0, s->stream>>>((R*)(which ? F.v : F.u), s->idx_c, s->V, d,
                                                                         1, 0);
    FEA_CHECK_LAUNCH();
    if (!mapped)
        FEA_CUDA_TRY(cudaMemcpyAsync(host, d, sizeof(float) * s->V, cudaMemcpyDeviceToHost, s->stream));
    FEA_CUDA_TRY(cudaStreamSynchronize(s->stream));
}

template <typename R>
void copy_field_device(fea_solver* s, const void* src, void* dst, int which, bool to_state) {
    Fields& F = s->F;
    const int64_t N = s->N;
    if (N == 0) return;
    R* state = F.interleaved ? (R*)F.uv : (R*)(which ? F.v : F.u);
    const int st = F.interleaved ? 2 : 1, off = F.interleaved ? which : 0;
    if (to_state) {
        int* pv = s->d_run ? &s->d_run->prev_valid : nullptr;
        k_copy_to_state<R><<<launch_grid(N), kBlock, 0, s->stream>>>((const R*)src, s->pos, N, state, st, off, pv);
    } else
        k_copy_from_state<R><<<launch_grid(N), kBlock, 0, s->stream>>>(state, s->pos, N, (R*)dst, st, off);
    FEA_CHECK_LAUNCH();
}

int displayed_field(const fea_params& p) { return p.equation == FEA_REACTION_DIFFUSION ? 1 : 0; }

// Arguments of the timing probe on the current equation's operator.
template <typename R, int NF>
StepArgs<R, NF> probe_args(fea_solver* s, int kind) {
    StepArgs<R, NF> a = make_args<R, NF>(s, false);
    set_x<R, NF>(s, a, kind);
    a.cont = &s->d_flags->probe;
    a.use_graph = 0;
    a.probe = 1;
    return a;
}

// One probe launch (prepare: mask the fields first, outside any timing).
template <typename R>
void probe(fea_solver* s, int kind, int lanes, bool prepare) {
    if (two_fields(kind)) {
        const StepArgs<R, 2> a = probe_args<R, 2>(s, kind);
        if (prepare) prepare_probe<R, 2>(a, s->stream);
        else launch_spmv_probe<R, 2>(a, lanes, s->stream);
    } else {
        const StepArgs<R, 1> a = probe_args<R, 1>(s, kind);
        if (prepare) prepare_probe<R, 1>(a, s->stream);
        else launch_spmv_probe<R, 1>(a, lanes, s->stream);
    }
}

void probe_any(fea_solver* s, int kind, int lanes, bool prepare) {
    if (s->precision == FEA_FP64) probe<double>(s, kind, lanes, prepare);
    else probe<float>(s, kind, lanes, prepare);
}

// The operator of `kind` up to date (the probe times the current equation).
void ensure_operator(fea_solver* s, int kind) {
    if (s->op_dirty || s->op_kind != kind) {
        if (s->precision == FEA_FP64) update_operator<double>(s, kind);
        else update_operator<float>(s, kind);
        s->op_dirty = false;
        s->op_kind = kind;
    }
}

// ---- adjoint of the explicit advection-diffusion step -------------------------------
// (recurrences in adjoint.cu).  The transposed solves mu = A^-1 lam run the
// forward operator (A is symmetric) through the step graph with a given
// right-hand side; forward states are recomputed from checkpoints taken every
// `ckpt` steps.

// One solve A mu = lam with the graph g (built on first use).
template <typename R, int NF>
void run_given(fea_solver* s, StepGraph& g, const StepArgs<R, NF>& a) {
    long long ctl[2] = {1, 0};  // steps_left, steps_done
    FEA_CUDA_TRY(cudaMemcpyAsync(s->d_run, ctl, sizeof(ctl), cudaMemcpyHostToDevice, s->stream));
    FEA_CUDA_TRY(cudaMemsetAsync(&s->d_run->flags, 0, sizeof(unsigned int), s->stream));
    if (s->stream_mode) {
        run_steps_stream<R, NF>(a, EQ_GIVEN, s->lanes, s->d_flags, s->stream);
        return;
    }
    if (!g.exec) build_step_graph<R, NF>(g, a, EQ_GIVEN, s->lanes, s->d_flags);
    FEA_CUDA_TRY(cudaGraphLaunch(g.exec, s->stream));
}

// u0, t: solver-order device arrays.  Leaves lam = dJ/du0 (solver order) and
// gD = dJ/dD (FP64, per element) when `grads`, and the handle's field at u_N.
template <typename R>
double adjoint_core(fea_solver* s, const R* u0, const R* t, int64_t nsteps, int64_t ckpt, bool grads, R* lam,
                    double* gD) {
    if (step_kind(s->prm) != EQ_ADV_EXPLICIT) {
        set_error("the adjoint needs equation FEA_ADVECTION_DIFFUSION with advection_scheme 1");
        throw Error{FEA_ERR_STATE};
    }
    cudaStream_t st = s->stream;
    const int64_t N = s->N;
    const size_t rb = sizeof(R) * (size_t)N;
    const auto d2d = cudaMemcpyDeviceToDevice;
    ckpt = std::min(ckpt, nsteps);
    const int64_t nck = ceil_div(nsteps, ckpt);
    ensure_layout<R>(s, false);
    DeviceArena tmp;
    R* ck = tmp.alloc<R>(nck * N);
    R* seg = tmp.alloc<R>((ckpt + 1) * N);
    R* mu = tmp.alloc<R>(pad_tiles(N));  // x of the solves: whole tiles
    R* uN = tmp.alloc<R>(N);
    R* lam_f = lam ? lam : tmp.alloc<R>(N);
    double* J = tmp.alloc<double>(1);
    R* u = (R*)s->F.u;
    FEA_CUDA_TRY(cudaMemcpyAsync(u, u0, rb, d2d, st));
    for (int64_t sg = 0; sg < nck; sg++) {  // forward sweep, a checkpoint per segment
        FEA_CUDA_TRY(cudaMemcpyAsync(ck + sg * N, u, rb, d2d, st));
        advance<R>(s, std::min(ckpt, nsteps - sg * ckpt));
    }
    FEA_CUDA_TRY(cudaMemcpyAsync(uN, u, rb, d2d, st));
    adjoint_loss<R>(s->Pc, (const R*)s->Mc, u, t, lam_f, s->d_part, max_grid_blocks(), s->d_tickets + 5, J, st);
    if (grads) {
        FEA_CUDA_TRY(cudaMemsetAsync(gD, 0, sizeof(double) * (size_t)s->T, st));
        FEA_CUDA_TRY(cudaMemsetAsync(mu, 0, sizeof(R) * (size_t)pad_tiles(N), st));
        StepArgs<R, 1> a = make_args<R, 1>(s, false);
        a.x = (FV<R, 1>*)mu;
        a.rhs = (const FV<R, 1>*)lam_f;
        StepGraph g;
        const double dt = time_step(s->prm), c = s->prm.advdiff_c, sign = s->prm.advection_sign;
        try {
            for (int64_t sg = nck - 1; sg >= 0; sg--) {
                const int64_t n0 = sg * ckpt, n1 = std::min(n0 + ckpt, nsteps);
                FEA_CUDA_TRY(cudaMemcpyAsync(u, ck + sg * N, rb, d2d, st));
                for (int64_t n = n0; n < n1; n++) {  // u^{n0+1} .. u^{n1}
                    advance<R>(s, 1);
                    FEA_CUDA_TRY(cudaMemcpyAsync(seg + (n - n0 + 1) * N, u, rb, d2d, st));
                }
                for (int64_t n = n1 - 1; n >= n0; n--) {
                    run_given<R, 1>(s, g, a);  // mu = A^-1 lam, warm-started from the previous mu
                    adjoint_grad_D<R>(s->Kloc, s->tri, s->idx_c, s->T, c, mu, seg + (n - n0 + 1) * N, gD, st);
                    adjoint_lambda<R>(s->Pc, (const R*)s->Mc, (const R*)s->Advc, dt, sign, mu, lam_f, st);
                }
            }
        } catch (...) {
            cudaStreamSynchronize(st);
            g.destroy();
            throw;
        }
        FEA_CUDA_TRY(cudaStreamSynchronize(st));
        g.destroy();
    }
    FEA_CUDA_TRY(cudaMemcpyAsync(u, uN, rb, d2d, st));
    double h = 0;
    FEA_CUDA_TRY(cudaMemcpyAsync(&h, J, sizeof(double), cudaMemcpyDeviceToHost, st));
    FEA_CUDA_TRY(cudaStreamSynchronize(st));
    return h;
}

// ---- adjoint of the mass-weighted Gray-Scott step (kernels in adjoint.cu) ---------
// x0, t: solver-order (u, v) pairs; use_u / use_v select the loss terms.
// Leaves lam = (dJ/du0, dJ/dv0) in solver order, adds (dJ/dF, dJ/dk, dJ/dDu,
// dJ/dDv) into g[4] (device), and the handle's fields at the final state.
template <typename R>
double adjoint_gs_core(fea_solver* s, const FV<R, 2>* x0, const FV<R, 2>* t, int use_u, int use_v, int64_t nsteps,
                       int64_t ckpt, bool grads, FV<R, 2>* lam, double* g) {
    if (step_kind(s->prm) != EQ_GS_CONSISTENT) {
        set_error("the Gray-Scott adjoint needs equation FEA_REACTION_DIFFUSION with reaction_mode 1");
        throw Error{FEA_ERR_STATE};
    }
    const GuessOff guess_off(s);  // recomputed forward states must equal the forward sweep's
    cudaStream_t st = s->stream;
    const int64_t N = s->N;
    const size_t xb = sizeof(FV<R, 2>) * (size_t)N;
    const auto d2d = cudaMemcpyDeviceToDevice;
    ckpt = std::min(ckpt, nsteps);
    const int64_t nck = ceil_div(nsteps, ckpt);
    ensure_layout<R>(s, true);  // the forward steps update the operator to the current parameters
    DeviceArena tmp;
    FV<R, 2>* ck = tmp.alloc<FV<R, 2>>(nck * N);
    FV<R, 2>* seg = tmp.alloc<FV<R, 2>>((ckpt + 1) * N);
    FV<R, 2>* mu = tmp.alloc<FV<R, 2>>(pad_tiles(N));  // x of the solves: whole tiles
    FV<R, 2>* xN = tmp.alloc<FV<R, 2>>(N);
    double* J = tmp.alloc<double>(1);
    FV<R, 2>* x = (FV<R, 2>*)s->F.uv;
    FEA_CUDA_TRY(cudaMemcpyAsync(x, x0, xb, d2d, st));
    for (int64_t sg = 0; sg < nck; sg++) {  // forward sweep, a checkpoint per segment
        FEA_CUDA_TRY(cudaMemcpyAsync(ck + sg * N, x, xb, d2d, st));
        advance<R>(s, std::min(ckpt, nsteps - sg * ckpt));
    }
    FEA_CUDA_TRY(cudaMemcpyAsync(xN, x, xb, d2d, st));
    adjoint_gs_loss<R>(s->Pc, (const R*)s->Mc, x, t, use_u, use_v, lam, s->d_part, max_grid_blocks(),
                       s->d_tickets + 5, J, st);
    if (grads) {
        FEA_CUDA_TRY(cudaMemsetAsync(mu, 0, sizeof(FV<R, 2>) * (size_t)pad_tiles(N), st));
        StepArgs<R, 2> a = make_args<R, 2>(s, false);
        a.x = mu;
        a.rhs = lam;
        StepGraph gr;
        const fea_params& p = s->prm;
        const double dt = p.rd_time_step, F = p.rd_feed_rate, kr = p.rd_kill_rate;
        try {
            for (int64_t sg = nck - 1; sg >= 0; sg--) {
                const int64_t n0 = sg * ckpt, n1 = std::min(n0 + ckpt, nsteps);
                FEA_CUDA_TRY(cudaMemcpyAsync(x, ck + sg * N, xb, d2d, st));
                FEA_CUDA_TRY(cudaMemcpyAsync(seg, x, xb, d2d, st));
                for (int64_t n = n0; n < n1; n++) {  // x^{n0+1} .. x^{n1}
                    advance<R>(s, 1);
                    FEA_CUDA_TRY(cudaMemcpyAsync(seg + (n - n0 + 1) * N, x, xb, d2d, st));
                }
                for (int64_t n = n1 - 1; n >= n0; n--) {
                    run_given<R, 2>(s, gr, a);  // mu = A^-1 lam (both fields), warm-started
                    adjoint_gs_step<R>(s->Pc, (const R*)s->Mc, (const R*)s->Kc, mu, seg + (n - n0) * N,
                                       seg + (n - n0 + 1) * N, dt, F, kr, lam, s->d_part, max_grid_blocks(),
                                       s->d_tickets + 6, g, st);
                }
            }
        } catch (...) {
            cudaStreamSynchronize(st);
            gr.destroy();
            throw;
        }
        FEA_CUDA_TRY(cudaStreamSynchronize(st));
        gr.destroy();
    }
    FEA_CUDA_TRY(cudaMemcpyAsync(x, xN, xb, d2d, st));
    double h = 0;
    FEA_CUDA_TRY(cudaMemcpyAsync(&h, J, sizeof(double), cudaMemcpyDeviceToHost, st));
    FEA_CUDA_TRY(cudaStreamSynchronize(st));
    return h;
}

// Node-indexed float arrays (NULL targets drop their loss terms).
template <typename R>
void adjoint_gs_host(fea_solver* s, const float* u0, const float* v0, const float* tu, const float* tv,
                     int64_t nsteps, int64_t ckpt, double* loss, float* gu, float* gv, double* gparams) {
    cudaStream_t st = s->stream;
    const int64_t N = s->N, V = s->V;
    DeviceArena tmp;
    FV<R, 2>* x0 = tmp.alloc<FV<R, 2>>(N);
    FV<R, 2>* t = tmp.alloc<FV<R, 2>>(N);
    FV<R, 2>* lam = tmp.alloc<FV<R, 2>>(N);
    double* g = tmp.alloc<double>(4);
    FEA_CUDA_TRY(cudaMemsetAsync(t, 0, sizeof(FV<R, 2>) * (size_t)N, st));
    FEA_CUDA_TRY(cudaMemsetAsync(g, 0, 4 * sizeof(double), st));
    const std::pair<const float*, std::pair<R*, int>> ins[4] = {
        {u0, {(R*)x0, 0}}, {v0, {(R*)x0, 1}}, {tu, {(R*)t, 0}}, {tv, {(R*)t, 1}}};
    for (const auto& in : ins) {
        if (!in.first) continue;
        FEA_CUDA_TRY(cudaMemcpyAsync(s->d_nodes, in.first, sizeof(float) * V, cudaMemcpyHostToDevice, st));
        k_gather_nodes<R><<<launch_grid(V), kBlock, 0, st>>>(s->d_nodes, s->idx_c, V, in.second.first, 2,
                                                              in.second.second, nullptr);
        FEA_CHECK_LAUNCH();
    }
    const bool grads = gu || gv || gparams;
    const double J = adjoint_gs_core<R>(s, x0, t, tu != nullptr, tv != nullptr, nsteps, ckpt, grads, lam, g);
    if (loss) *loss = J;
    float* outs[2] = {gu, gv};
    for (int f = 0; f < 2; f++) {
        if (!outs[f]) continue;
        k_scatter_nodes<R><<<launch_grid(V), kBlock, 0, st>>>((const R*)lam, s->idx_c, V, s->d_nodes, 2, f);
        FEA_CHECK_LAUNCH();
        FEA_CUDA_TRY(cudaMemcpyAsync(outs[f], s->d_nodes, sizeof(float) * V, cudaMemcpyDeviceToHost, st));
        FEA_CUDA_TRY(cudaStreamSynchronize(st));
    }
    if (gparams) FEA_CUDA_TRY(cudaMemcpyAsync(gparams, g, 4 * sizeof(double), cudaMemcpyDeviceToHost, st));
    FEA_CUDA_TRY(cudaStreamSynchronize(st));
}

// Unknown-indexed device arrays in the handle's precision.
template <typename R>
void adjoint_gs_device(fea_solver* s, const void* u0, const void* v0, const void* tu, const void* tv,
                       int64_t nsteps, int64_t ckpt, double* loss, void* gu, void* gv, double* gparams) {
    cudaStream_t st = s->stream;
    const int64_t N = s->N;
    DeviceArena tmp;
    FV<R, 2>* x0 = tmp.alloc<FV<R, 2>>(N);
    FV<R, 2>* t = tmp.alloc<FV<R, 2>>(N);
    FV<R, 2>* lam = tmp.alloc<FV<R, 2>>(N);
    double* g = tmp.alloc<double>(4);
    FEA_CUDA_TRY(cudaMemsetAsync(t, 0, sizeof(FV<R, 2>) * (size_t)N, st));
    FEA_CUDA_TRY(cudaMemsetAsync(g, 0, 4 * sizeof(double), st));
    const std::pair<const void*, std::pair<R*, int>> ins[4] = {
        {u0, {(R*)x0, 0}}, {v0, {(R*)x0, 1}}, {tu, {(R*)t, 0}}, {tv, {(R*)t, 1}}};
    if (N > 0)
        for (const auto& in : ins) {
            if (!in.first) continue;
            k_copy_to_state<R><<<launch_grid(N), kBlock, 0, st>>>((const R*)in.first, s->pos, N, in.second.first, 2,
                                                                   in.second.second, nullptr);
            FEA_CHECK_LAUNCH();
        }
    const bool grads = gu || gv || gparams;
    const double J = adjoint_gs_core<R>(s, x0, t, tu != nullptr, tv != nullptr, nsteps, ckpt, grads, lam, g);
    if (loss) *loss = J;
    void* outs[2] = {gu, gv};
    for (int f = 0; f < 2; f++)
        if (outs[f] && N > 0) {
            k_copy_from_state<R><<<launch_grid(N), kBlock, 0, st>>>((const R*)lam, s->pos, N, (R*)outs[f], 2, f);
            FEA_CHECK_LAUNCH();
        }
    if (gparams) FEA_CUDA_TRY(cudaMemcpyAsync(gparams, g, 4 * sizeof(double), cudaMemcpyDeviceToHost, st));
    FEA_CUDA_TRY(cudaStreamSynchronize(st));
}

// Node-indexed float inputs and outputs (the host entry point).
template <typename R>
void adjoint_host(fea_solver* s, const float* u0, const float* target, int64_t nsteps, int64_t ckpt, double* loss,
                  float* grad_u0, float* grad_D) {
    cudaStream_t st = s->stream;
    const int64_t N = s->N, V = s->V, T = s->T;
    DeviceArena tmp;
    R* u0s = tmp.alloc<R>(N);
    R* ts = tmp.alloc<R>(N);
    R* lam = tmp.alloc<R>(N);
    double* gD = tmp.alloc<double>(T);
    float* gDf = tmp.alloc<float>(T);
    const std::pair<const float*, R*> ins[2] = {{u0, u0s}, {target, ts}};
    for (const auto& in : ins) {
        FEA_CUDA_TRY(cudaMemcpyAsync(s->d_nodes, in.first, sizeof(float) * V, cudaMemcpyHostToDevice, st));
        k_gather_nodes<R><<<launch_grid(V), kBlock, 0, st>>>(s->d_nodes, s->idx_c, V, in.second, 1, 0, nullptr);
        FEA_CHECK_LAUNCH();
    }
    const bool grads = grad_u0 || grad_D;
    const double J = adjoint_core<R>(s, u0s, ts, nsteps, ckpt, grads, lam, gD);
    if (loss) *loss = J;
    if (grad_u0) {
        k_scatter_nodes<R><<<launch_grid(V), kBlock, 0, st>>>(lam, s->idx_c, V, s->d_nodes, 1, 0);
        FEA_CHECK_LAUNCH();
        FEA_CUDA_TRY(cudaMemcpyAsync(grad_u0, s->d_nodes, sizeof(float) * V, cudaMemcpyDeviceToHost, st));
    }
    if (grad_D) {
        k_convert<double, float><<<launch_grid(T), kBlock, 0, st>>>(gD, T, gDf);
        FEA_CHECK_LAUNCH();
        FEA_CUDA_TRY(cudaMemcpyAsync(grad_D, gDf, sizeof(float) * T, cudaMemcpyDeviceToHost, st));
    }
    FEA_CUDA_TRY(cudaStreamSynchronize(st));
}

// Unknown-indexed device arrays in the handle's precision.
template <typename R>
void adjoint_device(fea_solver* s, const void* u0, const void* target, int64_t nsteps, int64_t ckpt, double* loss,
                    void* grad_u0, void* grad_D) {
    cudaStream_t st = s->stream;
    const int64_t N = s->N, T = s->T;
    DeviceArena tmp;
    R* u0s = tmp.alloc<R>(N);
    R* ts = tmp.alloc<R>(N);
    R* lam = tmp.alloc<R>(N);
    double* gD = tmp.alloc<double>(T);
    if (N > 0) {
        k_copy_to_state<R><<<launch_grid(N), kBlock, 0, st>>>((const R*)u0, s->pos, N, u0s, 1, 0, nullptr);
        k_copy_to_state<R><<<launch_grid(N), kBlock, 0, st>>>((const R*)target, s->pos, N, ts, 1, 0, nullptr);
        FEA_CHECK_LAUNCH();
    }
    const bool grads = grad_u0 || grad_D;
    const double J = adjoint_core<R>(s, u0s, ts, nsteps, ckpt, grads, lam, gD);
    if (loss) *loss = J;
    if (grad_u0 && N > 0) {
        k_copy_from_state<R><<<launch_grid(N), kBlock, 0, st>>>(lam, s->pos, N, (R*)grad_u0, 1, 0);
        FEA_CHECK_LAUNCH();
    }
    if (grad_D) {
        k_convert<double, R><<<launch_grid(T), kBlock, 0, st>>>(gD, T, (R*)grad_D);
        FEA_CHECK_LAUNCH();
    }
    FEA_CUDA_TRY(cudaStreamSynchronize(st));
}

}  // namespace

MeshView mesh_view(const fea_solver* s) {
    MeshView m;
    m.V = s->V;
    m.T = s->T;
    m.N = s->N;
    m.Pc = &s->Pc;
    m.emap = s->emap;
    m.M64 = s->M64;
    m.K64 = s->K64;
    m.Adv64 = s->Adv64;
    m.idx_c = s->idx_c;
    m.stream = s->stream;
    return m;
}

// ---- after the solve: smooth normals and the .ply export ----------------------------

// The displayed field (v for Gray-Scott, u otherwise; 0 on Dirichlet points),
// node-indexed, into the handle's staging buffer.
void stage_node_values(fea_solver* s) {
    const int which = displayed_field(s->prm);
    Fields& F = s->F;
    const int64_t V = s->V;
    if (s->precision == FEA_FP64) {
        if (F.interleaved)
            k_scatter_nodes<double><<<launch_grid(V), kBlock, 0, s->stream>>>((double*)F.uv, s->idx_c, V, s->d_nodes,
                                                                               2, which);
        else
            k_scatter_nodes<double><<<launch_grid(V), kBlock, 0, s->stream>>>(
                (double*)(which ? F.v : F.u), s->idx_c, V, s->d_nodes, 1, 0);
    } else {
        if (F.interleaved)
            k_scatter_nodes<float><<<launch_grid(V), kBlock, 0, s->stream>>>((float*)F.uv, s->idx_c, V, s->d_nodes, 2,
                                                                              which);
        else
            k_scatter_nodes<float><<<launch_grid(V), kBlock, 0, s->stream>>>((float*)(which ? F.v : F.u), s->idx_c,
                                                                              V, s->d_nodes, 1, 0);
    }
    FEA_CHECK_LAUNCH();
}

void ensure_vertex_triangles(fea_solver* s) {
    if (s->vt_ptr) return;
    s->vt_ptr = s->mesh_mem.alloc<int32_t>(s->V + 1);
    s->vt_tri = s->mesh_mem.alloc<int32_t>(3 * s->T);
    build_vertex_triangles(s->tri, s->T, s->V, s->vt_ptr, s->vt_tri, s->stream);
}

// nrm and out: device float[3V]
void smooth_normals_dev(fea_solver* s, const float* nrm, float e, float* out) {
    ensure_vertex_triangles(s);
    stage_node_values(s);
    DeviceArena tmp;
    float* face = tmp.alloc<float>(3 * s->T);
    smooth_normals(s->xyz, s->tri, s->T, s->V, s->vt_ptr, s->vt_tri, nrm, s->d_nodes, e, face, out, s->stream);
    FEA_CUDA_TRY(cudaStreamSynchronize(s->stream));
}

struct PlyGeometry {
    std::vector<float> pos, val;
    std::vector<uint32_t> tri;
};

struct PosKey {
    uint32_t b[3];
    bool operator==(const PosKey& o) const { return b[0] == o.b[0] && b[1] == o.b[1] && b[2] == o.b[2]; }
};
struct PosKeyHash {
    size_t operator()(const PosKey& k) const {
        uint64_t h = 1469598103934665603ull;
        for (uint32_t x : k.b) h = (h ^ x) * 1099511628211ull;
        return (size_t)h;
    }
};

uint32_t key_bits(float f) {
    if (f == 0.0f) f = 0.0f;  // -0 and +0 are the same position
    uint32_t u;
    memcpy(&u, &f, 4);
    return u;
}

// Clipping on the device, then the reference's first-seen numbering of the
// positions (an exact-equality position map) on the host.
void ply_geometry(fea_solver* s, const float* nrm_host, float e, float thr, int mesh_type, PlyGeometry& g) {
    const int64_t V = s->V, T = s->T;
    cudaStream_t st = s->stream;
    DeviceArena tmp;
    float* nrm = tmp.alloc<float>(3 * V);
    float* pos = tmp.alloc<float>(18 * T);
    float* pval = tmp.alloc<float>(6 * T);
    uint8_t* used = tmp.alloc<uint8_t>(6 * T);
    int32_t* otri = tmp.alloc<int32_t>(12 * T);
    FEA_CUDA_TRY(cudaMemcpyAsync(nrm, nrm_host, sizeof(float) * 3 * V, cudaMemcpyHostToDevice, st));
    stage_node_values(s);
    ply_clip(s->xyz, s->tri, T, nrm, s->d_nodes, e, thr, mesh_type, pos, pval, used, otri, st);
    std::vector<float> hpos(18 * T), hval(6 * T);
    std::vector<uint8_t> hused(6 * T);
    std::vector<int32_t> htri(12 * T);
    FEA_CUDA_TRY(cudaMemcpyAsync(hpos.data(), pos, sizeof(float) * 18 * T, cudaMemcpyDeviceToHost, st));
    FEA_CUDA_TRY(cudaMemcpyAsync(hval.data(), pval, sizeof(float) * 6 * T, cudaMemcpyDeviceToHost, st));
    FEA_CUDA_TRY(cudaMemcpyAsync(hused.data(), used, 6 * T, cudaMemcpyDeviceToHost, st));
    FEA_CUDA_TRY(cudaMemcpyAsync(htri.data(), otri, sizeof(int32_t) * 12 * T, cudaMemcpyDeviceToHost, st));
    FEA_CUDA_TRY(cudaStreamSynchronize(st));
    std::unordered_map<PosKey, uint32_t, PosKeyHash> map;
    std::vector<uint32_t> slot_idx(6 * T, 0);
    g.pos.clear();
    g.val.clear();
    g.tri.clear();
    for (int64_t k = 0; k < T; k++) {
        for (int j = 0; j < 6; j++) {  // the order of the reference's add_clipped_position calls
            const int64_t q = 6 * k + j;
            if (!hused[q]) continue;
            const float* p = &hpos[3 * q];
            const PosKey key{{key_bits(p[0]), key_bits(p[1]), key_bits(p[2])}};
            auto it = map.find(key);
            if (it == map.end()) {
                const uint32_t idx = (uint32_t)g.val.size();
                map.emplace(key, idx);
                g.pos.insert(g.pos.end(), p, p + 3);
                g.val.push_back(hval[q]);
                slot_idx[q] = idx;
            } else {
                slot_idx[q] = it->second;
            }
        }
        for (int m = 0; m < 4; m++) {
            const int32_t* t3 = &htri[12 * k + 3 * m];
            if (t3[0] < 0) continue;
            for (int i = 0; i < 3; i++) g.tri.push_back(slot_idx[t3[i]]);
        }
    }
}

void append_float(std::string& out, float x) {
    char buf[64];
    const auto r = std::to_chars(buf, buf + sizeof(buf), x);  // shortest round-trip form, as std::format("{}")
    out.append(buf, r.ptr);
}

// Surface::export_to_ply's file (Surface.cpp:254-284): ASCII PLY, float
// x y z red green blue per vertex (color from the polynomial color map,
// ColorMap::get_color, ColorMap.cpp:12-14), "3 a b c" per face.
void write_ply(const char* path, const PlyGeometry& g, const float* coeffs) {
    std::string out;
    const size_t nv = g.val.size(), nf = g.tri.size() / 3;
    out.reserve(64 * nv + 24 * nf + 256);
    out += "ply\nformat ascii 1.0\nelement vertex " + std::to_string(nv) +
           "\nproperty float x\nproperty float y\nproperty float z\nproperty float red\nproperty float green\n"
           "property float blue\nelement face " +
           std::to_string(nf) + "\nproperty list uchar uint vertex_indices\nend_header\n";
    for (size_t i = 0; i < nv; i++) {
        const float t = g.val[i];
        float col[3];
        for (int ch = 0; ch < 3; ch++) {  // c0 + t (c1 + t (c2 + ... + t c6))
            float acc = coeffs[3 * 6 + ch];
            for (int k = 5; k >= 0; k--) acc = coeffs[3 * k + ch] + t * acc;
            col[ch] = acc;
        }
        const float v6[6] = {g.pos[3 * i], g.pos[3 * i + 1], g.pos[3 * i + 2], col[0], col[1], col[2]};
        for (int j = 0; j < 6; j++) {
            append_float(out, v6[j]);
            out += j < 5 ? ' ' : '\n';
        }
    }
    for (size_t f = 0; f < nf; f++)
        out += "3 " + std::to_string(g.tri[3 * f]) + " " + std::to_string(g.tri[3 * f + 1]) + " " +
               std::to_string(g.tri[3 * f + 2]) + "\n";
    FILE* fh = fopen(path, "wb");
    if (!fh) {
        set_error("cannot open %s for writing", path);
        throw Error{FEA_ERR_INVALID_ARGUMENT};
    }
    const size_t wrote = fwrite(out.data(), 1, out.size(), fh);
    const int closed = fclose(fh);
    if (wrote != out.size() || closed != 0) {
        set_error("writing %s failed", path);
        throw Error{FEA_ERR_INVALID_ARGUMENT};
    }
}

// Device partial-reduction storage sized for the widest grid.
void alloc_run_state(fea_solver* s) {
    s->d_prm = s->run_mem.alloc<StepParams>(1);
    s->d_cg = s->run_mem.alloc<CgState>(2);
    s->d_run = s->run_mem.alloc<RunState>(1);
    s->d_part = s->run_mem.alloc<double>(16 * (int64_t)max_grid_blocks());
    s->d_tickets = s->run_mem.alloc<unsigned int>(8);
    s->d_flags = s->run_mem.alloc<LoopFlags>(1);
    FEA_CUDA_TRY(cudaMemsetAsync(s->d_flags, 0, sizeof(LoopFlags), s->stream));
    const char* mode = getenv("FEA_LAUNCH_MODE");
    s->stream_mode = mode && strcmp(mode, "stream") == 0;
    FEA_CUDA_TRY(cudaMemsetAsync(s->d_cg, 0, 2 * sizeof(CgState), s->stream));
    FEA_CUDA_TRY(cudaMemsetAsync(s->d_run, 0, sizeof(RunState), s->stream));
    FEA_CUDA_TRY(cudaMemsetAsync(s->d_tickets, 0, 8 * sizeof(unsigned int), s->stream));
    FEA_CUDA_TRY(cudaMallocHost(&s->h_run, sizeof(RunState)));
}

}  // namespace fea

#define API_BEGIN try {
#define API_END                                                          \
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

const char* fea_last_error(void) { return fea::g_err; }
const char* fea_version(void) { return "fea_gb300 1.0 (sm_103a)"; }

int fea_params_default(fea_params* o) {
    if (!o) return fail(FEA_ERR_INVALID_ARGUMENT, "null params");
    memset(o, 0, sizeof(*o));
    o->equation = FEA_WAVE;  // FEMContext.hpp:31
    o->heat_time_step = 0.01f;
    o->heat_conductivity = 0.05f;
    o->advdiff_time_step = 0.001f;
    o->advdiff_c = 0.25f;
    o->advdiff_velocity[0] = 1.0f;
    o->wave_time_step = 0.05f;
    o->wave_c = 0.05f;
    o->rd_time_step = 0.001f;
    o->rd_Du = 0.08f;
    o->rd_Dv = 0.04f;
    o->rd_feed_rate = 0.035f;
    o->rd_kill_rate = 0.06f;
    o->reaction_mode = 0;
    o->wave_scheme = 0;
    o->newmark_beta = 0.25;
    o->newmark_gamma = 0.5;
    o->advection_scheme = 0;
    o->advection_sign = 1.0f;
    o->velocity_mode = 0;
    o->cg_tolerance = 0.0;
    o->cg_max_iterations = 0;
    o->cg_refine = 1;
    o->cg_initial_guess = 0;
    return FEA_OK;
}

int fea_create(const float* vertices, int64_t V, const uint32_t* triangles, int64_t T, const uint8_t* on_boundary,
               int bc, int precision, const fea_params* params, fea_solver** out) {
    if (!out) return fail(FEA_ERR_INVALID_ARGUMENT, "null output handle");
    *out = nullptr;
    if (!vertices || !triangles || V <= 0 || T <= 0)
        return fail(FEA_ERR_BAD_MESH, "mesh must have vertices and triangles");
    if (bc != FEA_DIRICHLET && bc != FEA_NEUMANN) return fail(FEA_ERR_INVALID_ARGUMENT, "bad boundary condition");
    if (precision != FEA_FP32 && precision != FEA_FP64) return fail(FEA_ERR_INVALID_ARGUMENT, "bad precision");
    if (V >= (int64_t)INT32_MAX || 9 * T >= (int64_t)INT32_MAX) return fail(FEA_ERR_TOO_LARGE, "mesh exceeds int32 indexing");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(FEA_ERR_NO_DEVICE, "no CUDA device");
    fea_solver* s = nullptr;
    API_BEGIN
    s = new fea_solver();
    FEA_CUDA_TRY(cudaGetDevice(&s->device));
    FEA_CUDA_TRY(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
    s->precision = precision;
    s->bc = bc;
    s->V = V;
    s->T = T;
    if (params) s->prm = *params;
    else fea_params_default(&s->prm);
    s->h_xyz.assign(vertices, vertices + 3 * V);
    s->xyz = s->mesh_mem.alloc<float>(3 * V);
    s->tri = s->mesh_mem.alloc<uint32_t>(3 * T);
    s->ob = s->mesh_mem.alloc<uint8_t>(V);
    s->d_nodes = s->mesh_mem.alloc<float>(V);
    FEA_CUDA_TRY(cudaMemcpyAsync(s->xyz, vertices, sizeof(float) * 3 * V, cudaMemcpyHostToDevice, s->stream));
    FEA_CUDA_TRY(cudaMemcpyAsync(s->tri, triangles, sizeof(uint32_t) * 3 * T, cudaMemcpyHostToDevice, s->stream));
    if (const int bad = check_mesh(s->xyz, s->tri, T, V, s->stream)) {
        fea_destroy(s);
        return fail(FEA_ERR_BAD_MESH, (bad & 1)   ? "triangle index out of range"
                                      : (bad & 2) ? "non-finite vertex coordinate"
                                                  : "degenerate triangle (zero area)");
    }
    if (on_boundary) {
        FEA_CUDA_TRY(cudaMemcpyAsync(s->ob, on_boundary, V, cudaMemcpyHostToDevice, s->stream));
    } else {
        detect_boundary(s->tri, T, V, s->ob, s->stream);
    }
    {
        std::vector<uint8_t> h(V);
        FEA_CUDA_TRY(cudaMemcpyAsync(h.data(), s->ob, V, cudaMemcpyDeviceToHost, s->stream));
        FEA_CUDA_TRY(cudaStreamSynchronize(s->stream));
        int64_t nb = 0;
        for (int64_t i = 0; i < V; i++) nb += h[i] ? 1 : 0;
        s->nb = nb;
    }
    alloc_run_state(s);
    build_context(s);
    if (precision == FEA_FP64) upload_params<double>(s);
    else upload_params<float>(s);
    *out = s;
    return FEA_OK;
    }
    catch (const fea::Error& e) {
        if (s) fea_destroy(s);
        return e.code;
    }
    catch (const std::bad_alloc&) {
        if (s) fea_destroy(s);
        return fail(FEA_ERR_OUT_OF_MEMORY, "host allocation failed");
    }
    catch (...) {
        if (s) fea_destroy(s);
        return fail(FEA_ERR_CUDA, "unexpected failure");
    }
}

int fea_destroy(fea_solver* s) {
    if (!s) return FEA_OK;
    cudaSetDevice(s->device);
    if (s->stream) cudaStreamSynchronize(s->stream);
    s->graph.destroy();
    s->init_graph.destroy();
    s->mat_mem.release();
    s->run_mem.release();
    s->mesh_mem.release();
    if (s->h_run) cudaFreeHost(s->h_run);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
    return FEA_OK;
}

int fea_set_boundary_condition(fea_solver* s, int bc) {
    API_BEGIN
    check_handle(s);
    if (bc != FEA_DIRICHLET && bc != FEA_NEUMANN) return fail(FEA_ERR_INVALID_ARGUMENT, "bad boundary condition");
    FEA_CUDA_TRY(cudaStreamSynchronize(s->stream));
    s->bc = bc;
    build_context(s);
    s->op_dirty = true;
    if (s->precision == FEA_FP64) upload_params<double>(s);
    else upload_params<float>(s);
    API_END
}

int fea_set_params(fea_solver* s, const fea_params* p) {
    API_BEGIN
    check_handle(s);
    if (!p) return fail(FEA_ERR_INVALID_ARGUMENT, "null params");
    if (p->equation < FEA_HEAT || p->equation > FEA_REACTION_DIFFUSION)
        return fail(FEA_ERR_INVALID_ARGUMENT, "bad equation");
    FEA_CUDA_TRY(cudaStreamSynchronize(s->stream));
    const bool wave_changed = p->wave_c != s->prm.wave_c || p->wave_time_step != s->prm.wave_time_step ||
                              p->newmark_beta != s->prm.newmark_beta;
    if (wave_changed) s->acc_valid = false;
    s->prm = *p;
    s->op_dirty = true;
    if (s->precision == FEA_FP64) upload_params<double>(s);
    else upload_params<float>(s);
    API_END
}

int fea_set_element_fields(fea_solver* s, const float* diffusivity, const float* velocity) {
    API_BEGIN
    check_handle(s);
    FEA_CUDA_TRY(cudaStreamSynchronize(s->stream));
    if (diffusivity) {
        if (!s->elem_D) {
            s->elem_D = s->mesh_mem.alloc<float>(s->T);
            s->elem_Dr = s->mesh_mem.alloc<double>(s->T);
        }
        FEA_CUDA_TRY(cudaMemcpyAsync(s->elem_D, diffusivity, sizeof(float) * s->T, cudaMemcpyHostToDevice, s->stream));
        k_float_to<double><<<launch_grid(s->T), kBlock, 0, s->stream>>>(s->elem_D, s->T, s->elem_Dr);
        FEA_CHECK_LAUNCH();
    }
    if (velocity) {
        if (!s->elem_vel) s->elem_vel = s->mesh_mem.alloc<float>(3 * s->T);
        FEA_CUDA_TRY(cudaMemcpyAsync(s->elem_vel, velocity, sizeof(float) * 3 * s->T, cudaMemcpyHostToDevice,
                                     s->stream));
    }
    assemble(s);
    FEA_CUDA_TRY(cudaStreamSynchronize(s->stream));
    API_END
}

int fea_set_element_diffusivity_device(fea_solver* s, const void* diffusivity) {
    API_BEGIN
    check_handle(s);
    if (!diffusivity) return fail(FEA_ERR_INVALID_ARGUMENT, "null diffusivity");
    FEA_CUDA_TRY(cudaStreamSynchronize(s->stream));
    if (!s->elem_D) {
        s->elem_D = s->mesh_mem.alloc<float>(s->T);
        s->elem_Dr = s->mesh_mem.alloc<double>(s->T);
    }
    if (s->precision == FEA_FP64) {
        FEA_CUDA_TRY(cudaMemcpyAsync(s->elem_Dr, diffusivity, sizeof(double) * s->T, cudaMemcpyDeviceToDevice,
                                     s->stream));
        k_convert<double, float><<<launch_grid(s->T), kBlock, 0, s->stream>>>(s->elem_Dr, s->T, s->elem_D);
    } else {
        FEA_CUDA_TRY(cudaMemcpyAsync(s->elem_D, diffusivity, sizeof(float) * s->T, cudaMemcpyDeviceToDevice,
                                     s->stream));
        k_float_to<double><<<launch_grid(s->T), kBlock, 0, s->stream>>>(s->elem_D, s->T, s->elem_Dr);
    }
    FEA_CHECK_LAUNCH();
    assemble(s);
    FEA_CUDA_TRY(cudaStreamSynchronize(s->stream));
    API_END
}

int fea_adjoint_advdiff(fea_solver* s, const float* u0, const float* target, int64_t nsteps,
                        int64_t checkpoint_every, double* loss, float* grad_u0, float* grad_D) {
    API_BEGIN
    check_handle(s);
    if (!u0 || !target || nsteps < 1 || checkpoint_every < 1)
        return fail(FEA_ERR_INVALID_ARGUMENT, "adjoint needs u0, target, nsteps >= 1 and checkpoint_every >= 1");
    if (s->precision == FEA_FP64) adjoint_host<double>(s, u0, target, nsteps, checkpoint_every, loss, grad_u0, grad_D);
    else adjoint_host<float>(s, u0, target, nsteps, checkpoint_every, loss, grad_u0, grad_D);
    API_END
}

int fea_adjoint_advdiff_device(fea_solver* s, const void* u0, const void* target, int64_t nsteps,
                               int64_t checkpoint_every, double* loss, void* grad_u0, void* grad_D) {
    API_BEGIN
    check_handle(s);
    if (!u0 || !target || nsteps < 1 || checkpoint_every < 1)
        return fail(FEA_ERR_INVALID_ARGUMENT, "adjoint needs u0, target, nsteps >= 1 and checkpoint_every >= 1");
    if (s->precision == FEA_FP64)
        adjoint_device<double>(s, u0, target, nsteps, checkpoint_every, loss, grad_u0, grad_D);
    else adjoint_device<float>(s, u0, target, nsteps, checkpoint_every, loss, grad_u0, grad_D);
    API_END
}

int fea_smooth_normals(fea_solver* s, const float* normals, float vertex_extrusion, float* out) {
    API_BEGIN
    check_handle(s);
    if (!normals || !out) return fail(FEA_ERR_INVALID_ARGUMENT, "null normals or output");
    DeviceArena tmp;
    float* nrm = tmp.alloc<float>(3 * s->V);
    float* res = tmp.alloc<float>(3 * s->V);
    FEA_CUDA_TRY(cudaMemcpyAsync(nrm, normals, sizeof(float) * 3 * s->V, cudaMemcpyHostToDevice, s->stream));
    smooth_normals_dev(s, nrm, vertex_extrusion, res);
    FEA_CUDA_TRY(cudaMemcpyAsync(out, res, sizeof(float) * 3 * s->V, cudaMemcpyDeviceToHost, s->stream));
    FEA_CUDA_TRY(cudaStreamSynchronize(s->stream));
    API_END
}

int fea_smooth_normals_device(fea_solver* s, const float* normals, float vertex_extrusion, float* out) {
    API_BEGIN
    check_handle(s);
    if (!normals || !out) return fail(FEA_ERR_INVALID_ARGUMENT, "null normals or output");
    smooth_normals_dev(s, normals, vertex_extrusion, out);
    API_END
}

int fea_ply_geometry(fea_solver* s, const float* normals, float vertex_extrusion, float threshold, int mesh_type,
                     float* positions, float* values, int64_t max_vertices, uint32_t* triangles,
                     int64_t max_triangles, int64_t* num_vertices, int64_t* num_triangles) {
    API_BEGIN
    check_handle(s);
    if (!normals || !num_vertices || !num_triangles) return fail(FEA_ERR_INVALID_ARGUMENT, "null argument");
    if (mesh_type < FEA_MESH_OPEN || mesh_type > FEA_MESH_MIRRORED) return fail(FEA_ERR_INVALID_ARGUMENT, "bad mesh type");
    PlyGeometry g;
    ply_geometry(s, normals, vertex_extrusion, threshold, mesh_type, g);
    const int64_t nv = (int64_t)g.val.size(), nt = (int64_t)g.tri.size() / 3;
    *num_vertices = nv;
    *num_triangles = nt;
    if (positions && values && nv <= max_vertices) {
        memcpy(positions, g.pos.data(), sizeof(float) * 3 * nv);
        memcpy(values, g.val.data(), sizeof(float) * nv);
    }
    if (triangles && nt <= max_triangles) memcpy(triangles, g.tri.data(), sizeof(uint32_t) * 3 * nt);
    API_END
}

int fea_export_ply(fea_solver* s, const char* path, const float* normals, float vertex_extrusion, float threshold,
                   int mesh_type, const float* color_coeffs) {
    API_BEGIN
    check_handle(s);
    if (!path || !normals) return fail(FEA_ERR_INVALID_ARGUMENT, "null path or normals");
    if (mesh_type < FEA_MESH_OPEN || mesh_type > FEA_MESH_MIRRORED) return fail(FEA_ERR_INVALID_ARGUMENT, "bad mesh type");
    float gray[21] = {0.f};
    gray[3] = gray[4] = gray[5] = 1.0f;  // color = (t, t, t)
    PlyGeometry g;
    ply_geometry(s, normals, vertex_extrusion, threshold, mesh_type, g);
    write_ply(path, g, color_coeffs ? color_coeffs : gray);
    API_END
}

int fea_adjoint_gray_scott(fea_solver* s, const float* u0, const float* v0, const float* target_u,
                           const float* target_v, int64_t nsteps, int64_t checkpoint_every, double* loss,
                           float* grad_u0, float* grad_v0, double* grad_params) {
    API_BEGIN
    check_handle(s);
    if (!u0 || !v0 || nsteps < 1 || checkpoint_every < 1)
        return fail(FEA_ERR_INVALID_ARGUMENT, "adjoint needs u0, v0, nsteps >= 1 and checkpoint_every >= 1");
    if (s->precision == FEA_FP64)
        adjoint_gs_host<double>(s, u0, v0, target_u, target_v, nsteps, checkpoint_every, loss, grad_u0, grad_v0,
                                grad_params);
    else
        adjoint_gs_host<float>(s, u0, v0, target_u, target_v, nsteps, checkpoint_every, loss, grad_u0, grad_v0,
                               grad_params);
    API_END
}

int fea_adjoint_gray_scott_device(fea_solver* s, const void* u0, const void* v0, const void* target_u,
                                  const void* target_v, int64_t nsteps, int64_t checkpoint_every, double* loss,
                                  void* grad_u0, void* grad_v0, double* grad_params) {
    API_BEGIN
    check_handle(s);
    if (!u0 || !v0 || nsteps < 1 || checkpoint_every < 1)
        return fail(FEA_ERR_INVALID_ARGUMENT, "adjoint needs u0, v0, nsteps >= 1 and checkpoint_every >= 1");
    if (s->precision == FEA_FP64)
        adjoint_gs_device<double>(s, u0, v0, target_u, target_v, nsteps, checkpoint_every, loss, grad_u0, grad_v0,
                                  grad_params);
    else
        adjoint_gs_device<float>(s, u0, v0, target_u, target_v, nsteps, checkpoint_every, loss, grad_u0, grad_v0,
                                 grad_params);
    API_END
}

int fea_clear_values(fea_solver* s) {
    API_BEGIN
    check_handle(s);
    Fields& F = s->F;
    const size_t n = rsize(s) * (size_t)(s->N > 0 ? s->N : 1);
    for (void* p : {F.u, F.v, F.a}) FEA_CUDA_TRY(cudaMemsetAsync(p, 0, n, s->stream));
    FEA_CUDA_TRY(cudaMemsetAsync(F.uv, 0, 2 * n, s->stream));
    FEA_CUDA_TRY(cudaMemsetAsync(&s->d_run->flags, 0, sizeof(unsigned int), s->stream));
    s->acc_valid = false;
    invalidate_guess(s);
    FEA_CUDA_TRY(cudaStreamSynchronize(s->stream));
    API_END
}

int fea_set_values(fea_solver* s, const float* values) {
    API_BEGIN
    check_handle(s);
    if (!values) return fail(FEA_ERR_INVALID_ARGUMENT, "null values");
    if (s->precision == FEA_FP64) set_node_field<double>(s, values, displayed_field(s->prm));
    else set_node_field<float>(s, values, displayed_field(s->prm));
    if (displayed_field(s->prm) == 0) s->acc_valid = false;
    API_END
}

int fea_get_values(fea_solver* s, float* values) {
    API_BEGIN
    check_handle(s);
    if (!values) return fail(FEA_ERR_INVALID_ARGUMENT, "null values");
    if (s->precision == FEA_FP64) get_node_field<double>(s, values, displayed_field(s->prm));
    else get_node_field<float>(s, values, displayed_field(s->prm));
    API_END
}

int fea_set_fields(fea_solver* s, const float* u, const float* v) {
    API_BEGIN
    check_handle(s);
    if (s->precision == FEA_FP64) {
        if (u) set_node_field<double>(s, u, 0);
        if (v) set_node_field<double>(s, v, 1);
    } else {
        if (u) set_node_field<float>(s, u, 0);
        if (v) set_node_field<float>(s, v, 1);
    }
    s->acc_valid = false;
    API_END
}

int fea_get_fields(fea_solver* s, float* u, float* v) {
    API_BEGIN
    check_handle(s);
    if (s->precision == FEA_FP64) {
        if (u) get_node_field<double>(s, u, 0);
        if (v) get_node_field<double>(s, v, 1);
    } else {
        if (u) get_node_field<float>(s, u, 0);
        if (v) get_node_field<float>(s, v, 1);
    }
    API_END
}

int fea_set_fields_device(fea_solver* s, const void* u, const void* v) {
    API_BEGIN
    check_handle(s);
    if (s->precision == FEA_FP64) {
        if (u) copy_field_device<double>(s, u, nullptr, 0, true);
        if (v) copy_field_device<double>(s, v, nullptr, 1, true);
    } else {
        if (u) copy_field_device<float>(s, u, nullptr, 0, true);
        if (v) copy_field_device<float>(s, v, nullptr, 1, true);
    }
    s->acc_valid = false;
    FEA_CUDA_TRY(cudaStreamSynchronize(s->stream));
    API_END
}

int fea_get_fields_device(fea_solver* s, void* u, void* v) {
    API_BEGIN
    check_handle(s);
    if (s->precision == FEA_FP64) {
        if (u) copy_field_device<double>(s, nullptr, u, 0, false);
        if (v) copy_field_device<double>(s, nullptr, v, 1, false);
    } else {
        if (u) copy_field_device<float>(s, nullptr, u, 0, false);
        if (v) copy_field_device<float>(s, nullptr, v, 1, false);
    }
    FEA_CUDA_TRY(cudaStreamSynchronize(s->stream));
    API_END
}

int fea_advance_time(fea_solver* s, int64_t nsteps) {
    API_BEGIN
    check_handle(s);
    if (nsteps < 0) return fail(FEA_ERR_INVALID_ARGUMENT, "negative step count");
    if (nsteps == 0 || s->N == 0) return FEA_OK;
    if (s->precision == FEA_FP64) advance<double>(s, nsteps);
    else advance<float>(s, nsteps);
    API_END
}

int fea_synchronize(fea_solver* s) {
    API_BEGIN
    check_handle(s);
    FEA_CUDA_TRY(cudaStreamSynchronize(s->stream));
    API_END
}

int fea_get_status(fea_solver* s, fea_status* out) {
    API_BEGIN
    check_handle(s);
    if (!out) return fail(FEA_ERR_INVALID_ARGUMENT, "null status");
    FEA_CUDA_TRY(cudaMemcpyAsync(s->h_run, s->d_run, sizeof(RunState), cudaMemcpyDeviceToHost, s->stream));
    FEA_CUDA_TRY(cudaStreamSynchronize(s->stream));
    const RunState& r = *s->h_run;
    out->flags = r.flags;
    out->last_iterations[0] = r.last_iters[0];
    out->last_iterations[1] = r.last_iters[1];
    out->last_rel_residual[0] = r.last_rel[0];
    out->last_rel_residual[1] = r.last_rel[1];
    out->steps_done = r.steps_done;
    out->total_iterations = r.total_iters;
    out->cg_launches = r.cg_launches;
    API_END
}

int fea_has_numerical_instability(fea_solver* s, int* out) {
    fea_status st;
    int rc = fea_get_status(s, &st);
    if (rc != FEA_OK) return rc;
    if (out) *out = (st.flags & (FEA_STATUS_BLOWUP | FEA_STATUS_NONFINITE)) ? 1 : 0;
    return FEA_OK;
}

int fea_get_info(fea_solver* s, fea_info* out) {
    API_BEGIN
    check_handle(s);
    if (!out) return fail(FEA_ERR_INVALID_ARGUMENT, "null info");
    out->num_vertices = s->V;
    out->num_triangles = s->T;
    out->num_boundary_points = s->nb;
    out->num_unknowns = s->N;
    out->nnz = s->P.nnz;
    out->max_row_nonzeros = s->P.max_row;
    out->precision = s->precision;
    out->boundary_condition = s->bc;
    out->rows_per_warp_lanes = s->lanes;
    out->device_bytes = s->mesh_mem.bytes + s->mat_mem.bytes + s->run_mem.bytes;
    API_END
}

int fea_get_matrix(fea_solver* s, int which, int32_t* row_ptr, int32_t* col, void* values, uint8_t* present) {
    API_BEGIN
    check_handle(s);
    const void* src = which == FEA_MATRIX_STIFFNESS ? s->K : which == FEA_MATRIX_MASS ? s->M
                    : which == FEA_MATRIX_ADVECTION ? s->Adv : nullptr;
    if (!src) return fail(FEA_ERR_INVALID_ARGUMENT, "bad matrix selector");
    FEA_CUDA_TRY(cudaStreamSynchronize(s->stream));
    if (row_ptr)
        FEA_CUDA_TRY(cudaMemcpy(row_ptr, s->P.row_ptr, sizeof(int32_t) * (s->N + 1), cudaMemcpyDeviceToHost));
    if (col && s->P.nnz) FEA_CUDA_TRY(cudaMemcpy(col, s->P.col, sizeof(int32_t) * s->P.nnz, cudaMemcpyDeviceToHost));
    if (values && s->P.nnz) FEA_CUDA_TRY(cudaMemcpy(values, src, rsize(s) * s->P.nnz, cudaMemcpyDeviceToHost));
    if (present && s->P.nnz) {
        if (which == FEA_MATRIX_ADVECTION)
            FEA_CUDA_TRY(cudaMemcpy(present, s->adv_present, s->P.nnz, cudaMemcpyDeviceToHost));
        else
            memset(present, 1, s->P.nnz);
    }
    API_END
}

int fea_get_idx_map(fea_solver* s, int32_t* idx_map, uint8_t* on_boundary) {
    API_BEGIN
    check_handle(s);
    FEA_CUDA_TRY(cudaStreamSynchronize(s->stream));
    if (idx_map) FEA_CUDA_TRY(cudaMemcpy(idx_map, s->idx, sizeof(int32_t) * s->V, cudaMemcpyDeviceToHost));
    if (on_boundary) FEA_CUDA_TRY(cudaMemcpy(on_boundary, s->ob, s->V, cudaMemcpyDeviceToHost));
    API_END
}

// Whether CG variant l runs on this handle: FEA_OK, FEA_ERR_INVALID_ARGUMENT
// (no such variant) or FEA_ERR_UNSUPPORTED (its layout or shared memory does
// not fit this mesh).
static int variant_check(const fea_solver* s, int l) {
    const bool csr = l == 4 || l == 8 || l == 16;
    const int stages = (l == 2 || l == 6 || l == 10) ? 2 : (l == 3 || l == 7 || l == 11) ? 3 : 0;
    const int ring = l == 14 ? 3 : l == 15 ? 4 : 0;
    if (!csr && l != 0 && l != 1 && l != 13 && stages == 0 && ring == 0) return FEA_ERR_INVALID_ARGUMENT;
    if (!csr && !s->ell.ok) return FEA_ERR_UNSUPPORTED;
    if (s->stream_stages < stages) return FEA_ERR_UNSUPPORTED;
    if (ring) {
        const size_t need = s->precision == FEA_FP64 ? ring_smem_bytes<double, 2>(ring_emax(s), s->ell.hmax, ring)
                                                     : ring_smem_bytes<float, 2>(ring_emax(s), s->ell.hmax, ring);
        if (need > kStreamSmemLimit) return FEA_ERR_UNSUPPORTED;
    }
    return FEA_OK;
}

int fea_autotune(fea_solver* s) {
    API_BEGIN
    check_handle(s);
    if (s->N == 0) return FEA_OK;
    const int kind = step_kind(s->prm);
    if (kind < 0) return fail(FEA_ERR_INVALID_ARGUMENT, "bad equation");
    ensure_operator(s, kind);
    cudaEvent_t e0, e1;
    FEA_CUDA_TRY(cudaEventCreate(&e0));
    FEA_CUDA_TRY(cudaEventCreate(&e1));
    const int cand[14] = {0, 1, 2, 3, 6, 7, 10, 11, 13, 14, 15, 4, 8, 16};
    float best = 1e30f;
    int best_l = s->lanes;
    for (int l : cand) {
        if (variant_check(s, l)) continue;
        probe_any(s, kind, l, true);
        for (int rep = 0; rep < 23; rep++) {
            if (rep == 3) FEA_CUDA_TRY(cudaEventRecord(e0, s->stream));
            probe_any(s, kind, l, false);
        }
        FEA_CUDA_TRY(cudaEventRecord(e1, s->stream));
        FEA_CUDA_TRY(cudaEventSynchronize(e1));
        float ms = 0;
        FEA_CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
        if (ms < best) {
            best = ms;
            best_l = l;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    s->lanes = best_l;
    API_END
}

int fea_set_cg_variant(fea_solver* s, int variant) {
    API_BEGIN
    check_handle(s);
    switch (variant_check(s, variant)) {
    case FEA_ERR_INVALID_ARGUMENT:
        return fail(FEA_ERR_INVALID_ARGUMENT, "CG variant must be 0 to 4, 6 to 8, 10, 11 or 13 to 16");
    case FEA_ERR_UNSUPPORTED:
        return fail(FEA_ERR_UNSUPPORTED, s->ell.ok ? "streamed tiles exceed the shared memory on this mesh"
                                                   : "tile-ELL layout unavailable on this mesh");
    default: break;
    }
    s->lanes = variant;
    API_END
}

int fea_get_stream(fea_solver* s, void** stream) {
    API_BEGIN
    check_handle(s);
    if (!stream) return fail(FEA_ERR_INVALID_ARGUMENT, "null stream output");
    *stream = (void*)s->stream;
    API_END
}

int fea_time_spmv(fea_solver* s, int reps, int flush_l2, double* ms_per_launch) {
    API_BEGIN
    check_handle(s);
    if (reps <= 0 || !ms_per_launch) return fail(FEA_ERR_INVALID_ARGUMENT, "bad arguments");
    if (s->N == 0) {
        *ms_per_launch = 0;
        return FEA_OK;
    }
    const int kind = step_kind(s->prm);
    if (kind < 0) return fail(FEA_ERR_INVALID_ARGUMENT, "bad equation");
    ensure_operator(s, kind);
    DeviceArena tmp;
    const size_t flush_bytes = (size_t)256 << 20;
    uint4* junk = nullptr;
    unsigned int* sink = nullptr;
    if (flush_l2) {
        junk = tmp.alloc<uint4>((int64_t)(flush_bytes / sizeof(uint4)));
        sink = tmp.alloc<unsigned int>(1);
        FEA_CUDA_TRY(cudaMemsetAsync(junk, 0, flush_bytes, s->stream));
    }
    auto flush = [&]() {
        if (!junk) return;
        k_read_flush<<<max_grid_blocks(), kBlock, 0, s->stream>>>(junk, (int64_t)(flush_bytes / sizeof(uint4)), sink);
        FEA_CHECK_LAUNCH();
    };
    flush();  // the memset's dirty lines leave the L2 before the first timing
    cudaEvent_t e0, e1;
    FEA_CUDA_TRY(cudaEventCreate(&e0));
    FEA_CUDA_TRY(cudaEventCreate(&e1));
    probe_any(s, kind, s->lanes, true);
    double total = 0;
    for (int rep = 0; rep < reps + 1; rep++) {  // the first launch is a warm-up
        flush();
        FEA_CUDA_TRY(cudaEventRecord(e0, s->stream));
        probe_any(s, kind, s->lanes, false);
        FEA_CUDA_TRY(cudaEventRecord(e1, s->stream));
        FEA_CUDA_TRY(cudaEventSynchronize(e1));
        float ms = 0;
        FEA_CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
        if (rep > 0) total += ms;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *ms_per_launch = total / reps;
    API_END
}

}  // extern "C"
