// tile_ell.cu -- the CG kernels' operator layout: tile-ELL with halo lists.
//
// The solver-order matrix is cut into tiles of kTileRows consecutive rows,
// each tile into 32-row slices.  A slice stores its rows' entries column by
// column (entry k of the slice's row `lane` at slice_off[s] + 32 k + lane),
// padded to the slice's longest row, so a warp reads one slice with fully
// coalesced loads and no row-pointer round trip.  Column indices are 16-bit
// and local to the tile: c - tile0 for rows of the tile, kTileRows + h for the
// tile's h-th halo column (the sorted distinct columns outside the tile).  The
// CG kernels place the vector they multiply for the tile's rows and its halo
// in shared memory, so every gathered operand is a shared-memory load.
// Entries keep their CSR order within a row (same summation order), and
// padding entries hold 0 with the row's own local index.  The diagonal-free
// variant of the layout leaves each row's diagonal entry out.
#include <algorithm>
#include <vector>

#include "fea_internal.cuh"

namespace fea {
namespace {

template <typename R, int NF>
__global__ void k_fill_tile_ell(int64_t E, const int32_t* __restrict__ emap, const FV<R, NF>* __restrict__ A,
                                FV<R, NF>* As) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < E; k += (int64_t)gridDim.x * blockDim.x) {
        const int32_t e = emap[k];
        FV<R, NF> v;
#pragma unroll
        for (int f = 0; f < NF; f++) v.v[f] = 0;
        if (e >= 0) v = A[e];
        As[k] = v;
    }
}

}  // namespace

bool build_tile_ell(const std::vector<int32_t>& rp, const std::vector<int32_t>& col, int64_t N, size_t fv_bytes,
                    size_t smem_budget, TileEll& L, DeviceArena& keep, cudaStream_t st, bool skip_diag) {
    L = TileEll{};
    if (N <= 0) return false;
    const int64_t ntiles = ceil_div(N, kTileRows), nslices = ntiles * (kTileRows / 32);
    std::vector<int32_t> slice_off(nslices + 1, 0), halo_off(ntiles + 1, 0), halo_col;
    // the stored entries of row r, in CSR order: rows[r] .. rows[r + 1] of `ents`
    std::vector<int32_t> rows(N + 1, 0), ents;
    ents.reserve(rp[N]);
    for (int64_t r = 0; r < N; r++) {
        for (int32_t e = rp[r]; e < rp[r + 1]; e++)
            if (!skip_diag || col[e] != r) ents.push_back(e);
        rows[r + 1] = (int32_t)ents.size();
    }
    int64_t E = 0;
    for (int64_t s = 0; s < nslices; s++) {
        int32_t w = 0;
        for (int64_t r = s * 32; r < std::min<int64_t>(N, s * 32 + 32); r++) w = std::max(w, rows[r + 1] - rows[r]);
        slice_off[s] = (int32_t)E;
        E += 32 * (int64_t)w;
        if (E >= (int64_t)INT32_MAX) return false;
    }
    slice_off[nslices] = (int32_t)E;
    int64_t hmax = 0;
    std::vector<int32_t> h;
    for (int64_t t = 0; t < ntiles; t++) {
        const int64_t t0 = t * kTileRows, t1 = std::min<int64_t>(N, t0 + kTileRows);
        h.clear();
        for (int64_t e = rp[t0]; e < rp[t1]; e++)
            if (col[e] < t0 || col[e] >= t1) h.push_back(col[e]);
        std::sort(h.begin(), h.end());
        h.erase(std::unique(h.begin(), h.end()), h.end());
        halo_off[t] = (int32_t)halo_col.size();
        halo_col.insert(halo_col.end(), h.begin(), h.end());
        hmax = std::max<int64_t>(hmax, (int64_t)h.size());
    }
    halo_off[ntiles] = (int32_t)halo_col.size();
    // 16-bit local indices and the shared-memory slice of the tile's operand
    if (kTileRows + hmax > 65535 || (size_t)(kTileRows + hmax) * fv_bytes > smem_budget) return false;
    std::vector<uint16_t> lcol(E);
    std::vector<int32_t> emap(E);
    for (int64_t s = 0; s < nslices; s++) {
        const int64_t t = s / (kTileRows / 32), t0 = t * kTileRows;
        const int32_t w = (slice_off[s + 1] - slice_off[s]) / 32;
        const int32_t* hb = halo_col.data() + halo_off[t];
        const int32_t* he = halo_col.data() + halo_off[t + 1];
        for (int lane = 0; lane < 32; lane++) {
            const int64_t r = s * 32 + lane;
            const int32_t len = r < N ? rows[r + 1] - rows[r] : 0;
            for (int32_t k = 0; k < w; k++) {
                const int64_t at = slice_off[s] + 32 * (int64_t)k + lane;
                if (k < len) {
                    const int32_t e = ents[rows[r] + k], c = col[e];
                    int64_t lc;
                    if (c >= t0 && c < t0 + kTileRows && c < N) lc = c - t0;
                    else lc = kTileRows + (std::lower_bound(hb, he, c) - hb);
                    lcol[at] = (uint16_t)lc;
                    emap[at] = e;
                } else {
                    lcol[at] = (uint16_t)(r - t0);  // padding: the row's own slot, value 0
                    emap[at] = -1;
                }
            }
        }
    }
    std::vector<uint32_t> lcol2(skip_diag ? 0 : E, 0u);
    for (int64_t s = 0; s < (skip_diag ? 0 : nslices); s++) {
        const int64_t sb = slice_off[s];
        const int32_t w = (slice_off[s + 1] - slice_off[s]) / 32;
        for (int32_t m = 0; 2 * m < w; m++)
            for (int lane = 0; lane < 32; lane++) {
                const uint32_t lo = lcol[sb + 32 * (2 * m) + lane];
                const uint32_t hi = 2 * m + 1 < w ? lcol[sb + 32 * (2 * m + 1) + lane] : lo;
                lcol2[sb + 32 * m + lane] = lo | (hi << 16);
            }
    }
    int64_t emax = 0;
    for (int64_t t = 0; t < ntiles; t++)
        emax = std::max<int64_t>(emax, slice_off[(t + 1) * (kTileRows / 32)] - slice_off[t * (kTileRows / 32)]);
    L.E = E;
    L.ntiles = (int)ntiles;
    L.hmax = (int)hmax;
    L.emax = (int)emax;
    L.slice_off = keep.alloc<int32_t>(nslices + 1);
    L.halo_off = keep.alloc<int32_t>(ntiles + 1);
    L.halo_col = keep.alloc<int32_t>(std::max<int64_t>(1, (int64_t)halo_col.size()));
    L.lcol = keep.alloc<uint16_t>(std::max<int64_t>(1, E));
    if (!skip_diag) L.lcol2 = keep.alloc<uint32_t>(std::max<int64_t>(1, E));
    L.emap = keep.alloc<int32_t>(std::max<int64_t>(1, E));
    FEA_CUDA_TRY(cudaMemcpyAsync(L.slice_off, slice_off.data(), sizeof(int32_t) * (nslices + 1),
                                 cudaMemcpyHostToDevice, st));
    FEA_CUDA_TRY(cudaMemcpyAsync(L.halo_off, halo_off.data(), sizeof(int32_t) * (ntiles + 1), cudaMemcpyHostToDevice,
                                 st));
    if (!halo_col.empty())
        FEA_CUDA_TRY(cudaMemcpyAsync(L.halo_col, halo_col.data(), sizeof(int32_t) * halo_col.size(),
                                     cudaMemcpyHostToDevice, st));
    if (E > 0) {
        FEA_CUDA_TRY(cudaMemcpyAsync(L.lcol, lcol.data(), sizeof(uint16_t) * E, cudaMemcpyHostToDevice, st));
        if (!skip_diag)
            FEA_CUDA_TRY(cudaMemcpyAsync(L.lcol2, lcol2.data(), sizeof(uint32_t) * E, cudaMemcpyHostToDevice, st));
        FEA_CUDA_TRY(cudaMemcpyAsync(L.emap, emap.data(), sizeof(int32_t) * E, cudaMemcpyHostToDevice, st));
    }
    FEA_CUDA_TRY(cudaStreamSynchronize(st));  // the host vectors go out of scope
    L.ok = true;
    return true;
}

template <typename R, int NF>
void fill_tile_ell(const TileEll& L, const FV<R, NF>* A, FV<R, NF>* As, cudaStream_t st) {
    if (!L.ok || L.E == 0) return;
    k_fill_tile_ell<R, NF><<<launch_grid(L.E), kBlock, 0, st>>>(L.E, L.emap, A, As);
    FEA_CHECK_LAUNCH();
}

template void fill_tile_ell<float, 1>(const TileEll&, const FV<float, 1>*, FV<float, 1>*, cudaStream_t);
template void fill_tile_ell<float, 2>(const TileEll&, const FV<float, 2>*, FV<float, 2>*, cudaStream_t);
template void fill_tile_ell<double, 1>(const TileEll&, const FV<double, 1>*, FV<double, 1>*, cudaStream_t);
template void fill_tile_ell<double, 2>(const TileEll&, const FV<double, 2>*, FV<double, 2>*, cudaStream_t);

}  // namespace fea
