// pattern.cu -- mesh ingest and the compressed sparsity pattern, on the device.
//
//   boundary points   Surface.cpp:104-122 (edge used by exactly one triangle)
//   idx_map           FEMContext.cpp:224-240
//   CSR pattern       FEMContext.cpp:97-112 + Eigen setFromTriplets/makeCompressed:
//                     one entry per distinct (row, col), sorted columns, explicit
//                     zeros kept, duplicates summed in triplet order.
//
// Both the boundary detection and the pattern are "bucket sorts by row":
// count per row (atomics), exclusive scan, scatter into row buckets with an
// atomic cursor (arbitrary order), then sort every bucket by a 64-bit key whose
// low half is a unique id.  The per-row sort removes the arbitrary order of the
// scatter, so the result is deterministic.  Rows of up to 32 keys (every row of
// a mesh with vertex valence <= 10) sort in registers with warp shuffles;
// larger rows sort in shared memory, one block per row.
#include <vector>

#include "fea_common.cuh"
#include <algorithm>

#include "fea_internal.cuh"

namespace fea {

namespace {

constexpr uint64_t kPad = ~0ull;

__global__ void k_count_rows(const int32_t* rows, int64_t n, int32_t* cnt) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int32_t r = rows[i];
        if (r >= 0) atomicAdd(&cnt[r], 1);
    }
}

__global__ void k_scatter_rows(const int32_t* rows, const uint64_t* keys, int64_t n, int32_t* cursor,
                               uint64_t* out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int32_t r = rows[i];
        if (r >= 0) {
            int32_t pos = atomicAdd(&cursor[r], 1);
            out[pos] = keys[i];
        }
    }
}

// Warp-per-row bitonic sort for buckets of <= 32 keys; larger buckets are
// listed in `big` for k_sort_big.
__global__ void k_sort_small(const int32_t* bstart, int64_t nrows, uint64_t* keys, int32_t* big,
                             int32_t* nbig) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t r = warp; r < nrows; r += nwarps) {
        const int32_t s = bstart[r], len = bstart[r + 1] - s;
        if (len > 32) {
            if (lane == 0) big[atomicAdd(nbig, 1)] = (int32_t)r;
            continue;
        }
        if (len <= 1) continue;
        uint64_t key = lane < len ? keys[s + lane] : kPad;
#pragma unroll
        for (int k = 2; k <= 32; k <<= 1) {
#pragma unroll
            for (int j = k >> 1; j > 0; j >>= 1) {
                uint64_t other = __shfl_xor_sync(0xffffffffu, key, j);
                bool up = (lane & k) == 0;
                bool lower = (lane & j) == 0;
                uint64_t mn = key < other ? key : other;
                uint64_t mx = key < other ? other : key;
                key = (lower == up) ? mn : mx;
            }
        }
        if (lane < len) keys[s + lane] = key;
    }
}

constexpr int kBigSort = 4096;  // keys per block-sorted bucket (32 KB of shared memory)

// One block per large bucket: bitonic sort in shared memory up to kBigSort
// keys; beyond that thread 0 insertion-sorts in global memory (a vertex of
// valence > 1365; correct but slow).
__global__ void k_sort_big(const int32_t* bstart, const int32_t* big, const int32_t* nbig, uint64_t* keys) {
    __shared__ uint64_t sk[kBigSort];
    const int nb = *nbig;
    for (int b = blockIdx.x; b < nb; b += gridDim.x) {
        const int32_t r = big[b];
        const int32_t s = bstart[r], len = bstart[r + 1] - s;
        if (len <= kBigSort) {
            int P = 64;
            while (P < len) P <<= 1;
            for (int i = threadIdx.x; i < P; i += blockDim.x) sk[i] = i < len ? keys[s + i] : kPad;
            __syncthreads();
            for (int k = 2; k <= P; k <<= 1) {
                for (int j = k >> 1; j > 0; j >>= 1) {
                    for (int i = threadIdx.x; i < P; i += blockDim.x) {
                        int l = i ^ j;
                        if (l > i) {
                            bool up = (i & k) == 0;
                            uint64_t a = sk[i], c = sk[l];
                            if ((a > c) == up) {
                                sk[i] = c;
                                sk[l] = a;
                            }
                        }
                    }
                    __syncthreads();
                }
            }
            for (int i = threadIdx.x; i < len; i += blockDim.x) keys[s + i] = sk[i];
            __syncthreads();
        } else if (threadIdx.x == 0) {
            for (int32_t a = s + 1; a < s + len; a++) {
                uint64_t kk = keys[a];
                int32_t c = a - 1;
                while (c >= s && keys[c] > kk) {
                    keys[c + 1] = keys[c];
                    c--;
                }
                keys[c + 1] = kk;
            }
        }
    }
}

// Count distinct high halves per sorted bucket.
__global__ void k_count_unique(const int32_t* bstart, int64_t nrows, const uint64_t* keys, int32_t* ucnt) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t r = warp; r < nrows; r += nwarps) {
        const int32_t s = bstart[r], len = bstart[r + 1] - s;
        int32_t count = 0;
        uint32_t carry = 0xffffffffu;
        for (int32_t base = 0; base < len; base += 32) {
            const int32_t i = base + lane;
            uint32_t hi = i < len ? (uint32_t)(keys[s + i] >> 32) : 0xffffffffu;
            uint32_t prev = __shfl_up_sync(0xffffffffu, hi, 1);
            if (lane == 0) prev = carry;
            bool flag = i < len && (i == 0 || hi != prev);
            count += __popc(__ballot_sync(0xffffffffu, flag));
            carry = __shfl_sync(0xffffffffu, hi, 31);
        }
        if (lane == 0) ucnt[r] = count;
    }
}

// Emit the compressed pattern: col[slot] for the first key of every run,
// seg_start[slot] = bucket position of that key, seg_id[pos] = id of the key
// at bucket position pos, slot_of[id] = the slot the key sums into.
__global__ void k_emit(const int32_t* bstart, int64_t nrows, const uint64_t* keys, const int32_t* row_ptr,
                       int32_t* col, int32_t* seg_start, int32_t* seg_id, int32_t* slot_of) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const uint32_t lt = (1u << lane) - 1u;
    for (int64_t r = warp; r < nrows; r += nwarps) {
        const int32_t s = bstart[r], len = bstart[r + 1] - s;
        int32_t run = row_ptr[r];
        uint32_t carry = 0xffffffffu;
        for (int32_t base = 0; base < len; base += 32) {
            const int32_t i = base + lane;
            uint64_t key = i < len ? keys[s + i] : kPad;
            uint32_t hi = (uint32_t)(key >> 32);
            uint32_t prev = __shfl_up_sync(0xffffffffu, hi, 1);
            if (lane == 0) prev = carry;
            bool flag = i < len && (i == 0 || hi != prev);
            uint32_t bal = __ballot_sync(0xffffffffu, flag);
            int32_t slot = run + __popc(bal & lt) + (flag ? 1 : 0) - 1;
            if (i < len) {
                if (flag) {
                    col[slot] = (int32_t)hi;
                    seg_start[slot] = s + i;
                }
                uint32_t id = (uint32_t)(key & 0xffffffffu);
                seg_id[s + i] = (int32_t)id;
                if (slot_of) slot_of[id] = slot;
            }
            run += __popc(bal);
            carry = __shfl_sync(0xffffffffu, hi, 31);
        }
    }
}

// Triplet rows/keys of FEMContext.cpp:97-107: entry (k, i, j) has id 9k+3i+j,
// row idx[t_i], column idx[t_j], kept when bc is Neumann or both points are
// off the boundary.
__global__ void k_triplet_keys(const uint32_t* tri, int64_t T, const uint8_t* ob, const int32_t* idx, int bc,
                               int32_t* rows, uint64_t* keys) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < 9 * T; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t k = t / 9;
        const int e = (int)(t - 9 * k);
        const uint32_t vi = tri[3 * k + e / 3], vj = tri[3 * k + e % 3];
        const bool keep = bc == FEA_NEUMANN || (!ob[vi] && !ob[vj]);
        rows[t] = keep ? idx[vi] : -1;
        keys[t] = ((uint64_t)(uint32_t)idx[vj] << 32) | (uint64_t)t;
    }
}

// Undirected edges of every triangle for boundary detection: row = lower
// vertex, key = (upper vertex << 32 | edge id).  Degenerate edges never count
// once (Surface.cpp counts a == b twice per use) and are dropped.
__global__ void k_edge_keys(const uint32_t* tri, int64_t T, int32_t* rows, uint64_t* keys) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < 3 * T; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t k = t / 3;
        const int j = (int)(t - 3 * k);
        const uint32_t a = tri[3 * k + j], b = tri[3 * k + (j + 1) % 3];
        const uint32_t lo = a < b ? a : b, hi = a < b ? b : a;
        rows[t] = a == b ? -1 : (int32_t)lo;
        keys[t] = ((uint64_t)hi << 32) | (uint64_t)t;
    }
}

// Both ends of every edge seen once are boundary points.
__global__ void k_mark_boundary(const int32_t* bstart, int64_t nrows, const uint64_t* keys, uint8_t* ob) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t r = warp; r < nrows; r += nwarps) {
        const int32_t s = bstart[r], len = bstart[r + 1] - s;
        for (int32_t i = lane; i < len; i += 32) {
            uint32_t hi = (uint32_t)(keys[s + i] >> 32);
            bool first = i == 0 || (uint32_t)(keys[s + i - 1] >> 32) != hi;
            bool last = i == len - 1 || (uint32_t)(keys[s + i + 1] >> 32) != hi;
            if (first && last) {
                ob[r] = 1;
                ob[hi] = 1;
            }
        }
    }
}

__global__ void k_not_boundary(const uint8_t* ob, int64_t V, int32_t* flag) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < V; v += (int64_t)gridDim.x * blockDim.x)
        flag[v] = ob[v] ? 0 : 1;
}

__global__ void k_idx_map(const uint8_t* ob, const int32_t* scan, int64_t V, int bc, int32_t* idx) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < V; v += (int64_t)gridDim.x * blockDim.x)
        idx[v] = bc == FEA_NEUMANN ? (int32_t)v : (ob[v] ? -1 : scan[v]);
}

// Mesh checks: bit 0 an index >= V, bit 1 a non-finite coordinate, bit 2 a
// triangle whose edge vectors have a zero cross product in FP64 (zero area:
// collinear or repeated corners; the element matrices would divide by it).
__global__ void k_check_mesh(const float* xyz, const uint32_t* tri, int64_t T, int64_t V, int32_t* bad) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < 3 * V; i += stride)
        if (!isfinite(xyz[i])) atomicOr(bad, 2);
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < T; k += stride) {
        const uint32_t a = tri[3 * k], b = tri[3 * k + 1], c = tri[3 * k + 2];
        if ((int64_t)a >= V || (int64_t)b >= V || (int64_t)c >= V) {
            atomicOr(bad, 1);
            continue;
        }
        double e1[3], e2[3];
        for (int d = 0; d < 3; d++) {
            e1[d] = (double)xyz[3 * b + d] - (double)xyz[3 * a + d];
            e2[d] = (double)xyz[3 * c + d] - (double)xyz[3 * a + d];
        }
        const double n0 = e1[1] * e2[2] - e1[2] * e2[1];
        const double n1 = e1[2] * e2[0] - e1[0] * e2[2];
        const double n2 = e1[0] * e2[1] - e1[1] * e2[0];
        if (n0 == 0.0 && n1 == 0.0 && n2 == 0.0) atomicOr(bad, 4);
    }
}

__global__ void k_find_diag(const int32_t* rp, const int32_t* col, int64_t N, int32_t* diag) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < N; r += (int64_t)gridDim.x * blockDim.x) {
        int32_t d = -1;
        for (int32_t e = rp[r]; e < rp[r + 1]; e++)
            if (col[e] == (int32_t)r) d = e;
        diag[r] = d;
    }
}

// Index of the transposed entry of every slot (the pattern is symmetric).
__global__ void k_transpose_index(const int32_t* rp, const int32_t* col, int64_t N, int32_t* tpos) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < N; r += (int64_t)gridDim.x * blockDim.x) {
        for (int32_t e = rp[r]; e < rp[r + 1]; e++) {
            const int32_t c = col[e];
            int32_t lo = rp[c], hi = rp[c + 1] - 1, found = -1;
            while (lo <= hi) {
                int32_t m = (lo + hi) >> 1;
                if (col[m] == (int32_t)r) {
                    found = m;
                    break;
                }
                if (col[m] < (int32_t)r) lo = m + 1;
                else hi = m - 1;
            }
            tpos[e] = found;
        }
    }
}

int grid_for(int64_t n, int block = kBlock) {
    int64_t g = ceil_div(n, block);
    int64_t cap = (int64_t)num_sms() * 32;
    if (g > cap) g = cap;
    return (int)(g < 1 ? 1 : g);
}

// Sorts (row, key) pairs into per-row buckets.  Returns bucket starts [nrows+1]
// and the sorted keys (length = number of pairs with row >= 0).
struct Buckets {
    int32_t* start = nullptr;
    uint64_t* keys = nullptr;
    int64_t total = 0;
};

Buckets bucket_sort(DeviceArena& tmp, const int32_t* rows, const uint64_t* keys, int64_t n, int64_t nrows,
                    cudaStream_t st) {
    Buckets b;
    int32_t* cnt = tmp.alloc<int32_t>(nrows + 1);
    FEA_CUDA_TRY(cudaMemsetAsync(cnt, 0, sizeof(int32_t) * (nrows + 1), st));
    k_count_rows<<<grid_for(n), kBlock, 0, st>>>(rows, n, cnt);
    FEA_CHECK_LAUNCH();
    b.start = tmp.alloc<int32_t>(nrows + 1);
    b.total = exclusive_scan_i32(cnt, b.start, nrows, st);
    int32_t* cursor = tmp.alloc<int32_t>(nrows + 1);
    FEA_CUDA_TRY(cudaMemcpyAsync(cursor, b.start, sizeof(int32_t) * (nrows + 1), cudaMemcpyDeviceToDevice, st));
    b.keys = tmp.alloc<uint64_t>(b.total);
    k_scatter_rows<<<grid_for(n), kBlock, 0, st>>>(rows, keys, n, cursor, b.keys);
    FEA_CHECK_LAUNCH();
    int32_t* big = tmp.alloc<int32_t>(nrows + 1);
    int32_t* nbig = tmp.alloc<int32_t>(1);
    FEA_CUDA_TRY(cudaMemsetAsync(nbig, 0, sizeof(int32_t), st));
    k_sort_small<<<grid_for(nrows * 32), kBlock, 0, st>>>(b.start, nrows, b.keys, big, nbig);
    FEA_CHECK_LAUNCH();
    k_sort_big<<<num_sms() * 2, 256, 0, st>>>(b.start, big, nbig, b.keys);
    FEA_CHECK_LAUNCH();
    return b;
}

}  // namespace

int launch_grid(int64_t n) { return grid_for(n); }

// Boundary detection on the device (Surface.cpp:104-122).
void detect_boundary(const uint32_t* tri, int64_t T, int64_t V, uint8_t* ob, cudaStream_t st) {
    DeviceArena tmp;
    int32_t* rows = tmp.alloc<int32_t>(3 * T);
    uint64_t* keys = tmp.alloc<uint64_t>(3 * T);
    k_edge_keys<<<grid_for(3 * T), kBlock, 0, st>>>(tri, T, rows, keys);
    FEA_CHECK_LAUNCH();
    Buckets b = bucket_sort(tmp, rows, keys, 3 * T, V, st);
    FEA_CUDA_TRY(cudaMemsetAsync(ob, 0, V, st));
    k_mark_boundary<<<grid_for(V * 32), kBlock, 0, st>>>(b.start, V, b.keys, ob);
    FEA_CHECK_LAUNCH();
    FEA_CUDA_TRY(cudaStreamSynchronize(st));
}

int check_mesh(const float* xyz, const uint32_t* tri, int64_t T, int64_t V, cudaStream_t st) {
    DeviceArena tmp;
    int32_t* bad = tmp.alloc<int32_t>(1);
    FEA_CUDA_TRY(cudaMemsetAsync(bad, 0, sizeof(int32_t), st));
    k_check_mesh<<<grid_for(std::max(3 * V, T)), kBlock, 0, st>>>(xyz, tri, T, V, bad);
    FEA_CHECK_LAUNCH();
    int32_t h = 0;
    FEA_CUDA_TRY(cudaMemcpyAsync(&h, bad, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    FEA_CUDA_TRY(cudaStreamSynchronize(st));
    return h;
}

// idx_map and the number of unknowns (FEMContext.cpp:46-48, 224-240).
int64_t build_idx_map(const uint8_t* ob, int64_t V, int bc, int32_t* idx, cudaStream_t st) {
    DeviceArena tmp;
    int32_t* flag = tmp.alloc<int32_t>(V);
    int32_t* scan = tmp.alloc<int32_t>(V + 1);
    k_not_boundary<<<grid_for(V), kBlock, 0, st>>>(ob, V, flag);
    FEA_CHECK_LAUNCH();
    int64_t interior = exclusive_scan_i32(flag, scan, V, st);
    k_idx_map<<<grid_for(V), kBlock, 0, st>>>(ob, scan, V, bc, idx);
    FEA_CHECK_LAUNCH();
    FEA_CUDA_TRY(cudaStreamSynchronize(st));
    return bc == FEA_NEUMANN ? V : interior;
}

// CSR pattern + ordered-sum segments (see the file comment).
void build_pattern(Pattern& P, DeviceArena& keep, const uint32_t* tri, int64_t T, const uint8_t* ob,
                   const int32_t* idx, int bc, int64_t N, cudaStream_t st) {
    DeviceArena tmp;
    const int64_t n = 9 * T;
    int32_t* rows = tmp.alloc<int32_t>(n);
    uint64_t* keys = tmp.alloc<uint64_t>(n);
    k_triplet_keys<<<grid_for(n), kBlock, 0, st>>>(tri, T, ob, idx, bc, rows, keys);
    FEA_CHECK_LAUNCH();
    Buckets b = bucket_sort(tmp, rows, keys, n, N, st);
    int32_t* ucnt = tmp.alloc<int32_t>(N + 1);
    k_count_unique<<<grid_for(N * 32), kBlock, 0, st>>>(b.start, N, b.keys, ucnt);
    FEA_CHECK_LAUNCH();
    P.N = N;
    P.ntrip = b.total;
    P.row_ptr = keep.alloc<int32_t>(N + 1);
    P.nnz = exclusive_scan_i32(ucnt, P.row_ptr, N, st);
    P.col = keep.alloc<int32_t>(P.nnz);
    P.seg_start = keep.alloc<int32_t>(P.nnz + 1);
    P.seg_id = keep.alloc<int32_t>(P.ntrip);
    P.slot_of = keep.alloc<int32_t>(n);
    FEA_CUDA_TRY(cudaMemsetAsync(P.slot_of, 0xff, sizeof(int32_t) * n, st));
    k_emit<<<grid_for(N * 32), kBlock, 0, st>>>(b.start, N, b.keys, P.row_ptr, P.col, P.seg_start, P.seg_id,
                                                 P.slot_of);
    FEA_CHECK_LAUNCH();
    int32_t tot = (int32_t)P.ntrip;
    FEA_CUDA_TRY(cudaMemcpyAsync(P.seg_start + P.nnz, &tot, sizeof(int32_t), cudaMemcpyHostToDevice, st));
    P.diag = keep.alloc<int32_t>(N);
    k_find_diag<<<grid_for(N), kBlock, 0, st>>>(P.row_ptr, P.col, N, P.diag);
    FEA_CHECK_LAUNCH();
    P.tpos = keep.alloc<int32_t>(P.nnz);
    k_transpose_index<<<grid_for(N), kBlock, 0, st>>>(P.row_ptr, P.col, N, P.tpos);
    FEA_CHECK_LAUNCH();
    int32_t mx = 0;
    {
        std::vector<int32_t> h(N + 1);
        FEA_CUDA_TRY(cudaMemcpyAsync(h.data(), P.row_ptr, sizeof(int32_t) * (N + 1), cudaMemcpyDeviceToHost, st));
        FEA_CUDA_TRY(cudaStreamSynchronize(st));
        for (int64_t r = 0; r < N; r++) mx = h[r + 1] - h[r] > mx ? h[r + 1] - h[r] : mx;
    }
    P.max_row = mx;
}

// ---- computational ordering --------------------------------------------------------
//
// The solver iterates on a copy of the pattern whose unknowns are renumbered
// along a Morton (Z-order) curve of their coordinates, so that the rows a
// warp processes together have their columns in a few nearby ranges and the
// gathered vector entries hit in L1.  pos[u] is the new index of unknown u,
// inv its inverse; emap[e'] is the original slot of new slot e'.  Within a
// row the columns are sorted again, so the copy is a valid CSR matrix.

namespace {

__global__ void k_perm_rowlen(const int32_t* rp, const int32_t* inv, int64_t N, int32_t* len) {
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < N; c += (int64_t)gridDim.x * blockDim.x) {
        const int32_t u = inv[c];
        len[c] = rp[u + 1] - rp[u];
    }
}

__global__ void k_perm_fill(const int32_t* rp, const int32_t* col, const int32_t* pos, const int32_t* inv,
                            int64_t N, const int32_t* rpc, int32_t* colc, int32_t* emap) {
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < N; c += (int64_t)gridDim.x * blockDim.x) {
        const int32_t u = inv[c];
        const int32_t s = rp[u], n = rp[u + 1] - s, o = rpc[c];
        // insertion sort by new column, written straight to the output row
        for (int32_t k = 0; k < n; k++) {
            const int32_t nc = pos[col[s + k]];
            int32_t j = k - 1;
            while (j >= 0 && colc[o + j] > nc) {
                colc[o + j + 1] = colc[o + j];
                emap[o + j + 1] = emap[o + j];
                j--;
            }
            colc[o + j + 1] = nc;
            emap[o + j + 1] = s + k;
        }
    }
}

}  // namespace

void build_permuted(const Pattern& P, const int32_t* pos, const int32_t* inv, Pattern& Pc, int32_t* emap,
                    DeviceArena& keep, cudaStream_t st) {
    DeviceArena tmp;
    const int64_t N = P.N;
    Pc.N = N;
    Pc.nnz = P.nnz;
    Pc.max_row = P.max_row;
    int32_t* len = tmp.alloc<int32_t>(N + 1);
    k_perm_rowlen<<<grid_for(N), kBlock, 0, st>>>(P.row_ptr, inv, N, len);
    FEA_CHECK_LAUNCH();
    Pc.row_ptr = keep.alloc<int32_t>(N + 1);
    exclusive_scan_i32(len, Pc.row_ptr, N, st);
    Pc.col = keep.alloc<int32_t>(P.nnz);
    k_perm_fill<<<grid_for(N), kBlock, 0, st>>>(P.row_ptr, P.col, pos, inv, N, Pc.row_ptr, Pc.col, emap);
    FEA_CHECK_LAUNCH();
    Pc.diag = keep.alloc<int32_t>(N);
    k_find_diag<<<grid_for(N), kBlock, 0, st>>>(Pc.row_ptr, Pc.col, N, Pc.diag);
    FEA_CHECK_LAUNCH();
    Pc.tpos = keep.alloc<int32_t>(P.nnz);
    k_transpose_index<<<grid_for(N), kBlock, 0, st>>>(Pc.row_ptr, Pc.col, N, Pc.tpos);
    FEA_CHECK_LAUNCH();
    FEA_CUDA_TRY(cudaStreamSynchronize(st));
}

}  // namespace fea
