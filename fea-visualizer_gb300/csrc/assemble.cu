// assemble.cu -- element-parallel P1 assembly (FEMContext.cpp:70-202).
//
// One thread per triangle computes the local 3x3 stiffness, mass and
// advection blocks from the vertex coordinates; a thread per CSR slot then
// sums the entries of its segment in triplet order (the duplicate summation
// order of Eigen's setFromTriplets), so assembly is deterministic.
#include "fea_internal.cuh"

namespace fea {

namespace {

// Gradients of the barycentric basis on triangle (a, b, c): with
// e1 = b - a, e2 = c - a, n the unit normal and |J| = |e1 x e2|, the rows of
// [e1 e2 n]^-1 are (e2 x n)/|J|, (n x e1)/|J| and n, so the reference
// gradients (-1,-1,0), (1,0,0), (0,1,0) map to
//   g_a = -(g_b + g_c),  g_b = (e2 x n)/|J|,  g_c = (n x e1)/|J|.
// This is the closed form of the inverse-transpose of FEMContext.cpp:85-95.
template <typename R>
__global__ void k_element(const float* __restrict__ xyz, const uint32_t* __restrict__ tri, int64_t T,
                          int vel_mode, R vx, R vy, R vz, const float* __restrict__ ev, R* Kloc, R* Mloc,
                          R* Aloc) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < T; k += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t ia = tri[3 * k], ib = tri[3 * k + 1], ic = tri[3 * k + 2];
        const R ax = xyz[3 * ia], ay = xyz[3 * ia + 1], az = xyz[3 * ia + 2];
        const R e1x = (R)xyz[3 * ib] - ax, e1y = (R)xyz[3 * ib + 1] - ay, e1z = (R)xyz[3 * ib + 2] - az;
        const R e2x = (R)xyz[3 * ic] - ax, e2y = (R)xyz[3 * ic + 1] - ay, e2z = (R)xyz[3 * ic + 2] - az;
        const R cx = e1y * e2z - e1z * e2y, cy = e1z * e2x - e1x * e2z, cz = e1x * e2y - e1y * e2x;
        const R jac = sqrt(cx * cx + cy * cy + cz * cz);
        const R il = (R)1 / jac;
        const R nx = cx * il, ny = cy * il, nz = cz * il;
        const R area = (R)0.5 * jac;
        R g[3][3];
        g[1][0] = (e2y * nz - e2z * ny) * il;
        g[1][1] = (e2z * nx - e2x * nz) * il;
        g[1][2] = (e2x * ny - e2y * nx) * il;
        g[2][0] = (ny * e1z - nz * e1y) * il;
        g[2][1] = (nz * e1x - nx * e1z) * il;
        g[2][2] = (nx * e1y - ny * e1x) * il;
        for (int d = 0; d < 3; d++) g[0][d] = -(g[1][d] + g[2][d]);
        // tangential velocity (FEMContext.cpp:179-180)
        R wx = vx, wy = vy, wz = vz;
        if (vel_mode == 1) {
            wx = ev[3 * k];
            wy = ev[3 * k + 1];
            wz = ev[3 * k + 2];
        }
        const R wn = wx * nx + wy * ny + wz * nz;
        const R nn = nx * nx + ny * ny + nz * nz;
        R tx = wx - wn / nn * nx, ty = wy - wn / nn * ny, tz = wz - wn / nn * nz;
        if (vel_mode == 0) {
            const R tl = sqrt(tx * tx + ty * ty + tz * tz);
            if (tl > (R)0) {
                tx /= tl;
                ty /= tl;
                tz /= tl;
            }
        }
        const R ms = (R)((double)jac / 24.0);
        const R as = jac / (R)6;
        R tg[3];
        for (int j = 0; j < 3; j++) tg[j] = as * (tx * g[j][0] + ty * g[j][1] + tz * g[j][2]);
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = 0; j < 3; j++) {
                const int64_t e = 9 * k + 3 * i + j;
                Kloc[e] = area * (g[i][0] * g[j][0] + g[i][1] * g[j][1] + g[i][2] * g[j][2]);
                Mloc[e] = ms * (R)(i == j ? 2 : 1);
                Aloc[e] = tg[j];
            }
    }
}

template <typename R>
__global__ void k_ordered_sum(const int32_t* __restrict__ seg_start, const int32_t* __restrict__ seg_id,
                              int64_t nnz, const R* __restrict__ loc, const R* __restrict__ scale, R* out) {
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < nnz; s += (int64_t)gridDim.x * blockDim.x) {
        R acc = 0;
        for (int32_t p = seg_start[s]; p < seg_start[s + 1]; p++) {
            const int32_t id = seg_id[p];
            R val = loc[id];
            if (scale) val = mul_rn(scale[id / 9], val);
            acc = add_rn(acc, val);
        }
        out[s] = acc;
    }
}

// Advection keeps only entries whose two points are off the boundary
// (FEMContext.cpp:188, independent of the BC).
template <typename R>
__global__ void k_ordered_sum_adv(const int32_t* __restrict__ seg_start, const int32_t* __restrict__ seg_id,
                                  int64_t nnz, const R* __restrict__ loc, const uint32_t* __restrict__ tri,
                                  const uint8_t* __restrict__ ob, R* out, uint8_t* present) {
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < nnz; s += (int64_t)gridDim.x * blockDim.x) {
        R acc = 0;
        uint8_t pres = 0;
        for (int32_t p = seg_start[s]; p < seg_start[s + 1]; p++) {
            const int32_t id = seg_id[p];
            const int32_t k = id / 9, e = id - 9 * (id / 9);
            const uint32_t vi = tri[3 * k + e / 3], vj = tri[3 * k + e % 3];
            if (!ob[vi] && !ob[vj]) {
                acc = add_rn(acc, loc[id]);
                pres = 1;
            }
        }
        out[s] = acc;
        if (present) present[s] = pres;
    }
}

template <typename R, int NF>
__global__ void k_combine(int64_t nnz, const int32_t* __restrict__ emap, const double* __restrict__ M,
                          const double* __restrict__ K, const double* __restrict__ Adv, OpCoef<NF> c, FV<R, NF>* A) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nnz; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t src = emap ? emap[e] : e;
        const double m = M[src], kk = K[src];
        const double ad = Adv ? Adv[src] : 0.0;
        FV<R, NF> out;
#pragma unroll
        for (int f = 0; f < NF; f++) {
            const OpCoef1& cf = c.f[f];
            double v = add_rn(div_rn(m, cf.md), mul_rn(mul_rn(cf.k1, kk), cf.k2));
            if (cf.a1 != 0.0) v = add_rn(v, mul_rn(cf.a1, ad));
            out.v[f] = (R)v;
        }
        A[e] = out;
    }
}

template <typename R>
__global__ void k_round_copy(const double* __restrict__ in, const int32_t* __restrict__ map, int64_t n, R* out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = (R)in[map ? map[i] : i];
}

// Inverse diagonal (Eigen's DiagonalPreconditioner: 1 where the diagonal is 0).
template <typename R, int NF>
__global__ void k_dinv(int64_t N, const int32_t* __restrict__ diag, const FV<R, NF>* __restrict__ A,
                       FV<R, NF>* dinv) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < N; r += (int64_t)gridDim.x * blockDim.x) {
        FV<R, NF> out;
        const int32_t d = diag[r];
#pragma unroll
        for (int f = 0; f < NF; f++) {
            const R dv = d >= 0 ? A[d].v[f] : (R)0;
            out.v[f] = dv != (R)0 ? (R)1 / dv : (R)1;
        }
        dinv[r] = out;
    }
}

}  // namespace

template <typename R>
void element_matrices(const float* xyz, const uint32_t* tri, int64_t T, int vel_mode, const float vel[3],
                      const float* elem_vel, R* Kloc, R* Mloc, R* Aloc, cudaStream_t st) {
    if (T <= 0) return;
    k_element<R><<<launch_grid(T), kBlock, 0, st>>>(xyz, tri, T, vel_mode, (R)vel[0], (R)vel[1], (R)vel[2], elem_vel,
                                                     Kloc, Mloc, Aloc);
    FEA_CHECK_LAUNCH();
}

template <typename R>
void ordered_sum(const Pattern& P, const R* loc, const R* elem_scale, R* out, cudaStream_t st) {
    if (P.nnz <= 0) return;
    k_ordered_sum<R><<<launch_grid(P.nnz), kBlock, 0, st>>>(P.seg_start, P.seg_id, P.nnz, loc, elem_scale, out);
    FEA_CHECK_LAUNCH();
}

template <typename R>
void ordered_sum_adv(const Pattern& P, const R* loc, const uint32_t* tri, const uint8_t* ob, R* out,
                     uint8_t* present, cudaStream_t st) {
    if (P.nnz <= 0) return;
    k_ordered_sum_adv<R><<<launch_grid(P.nnz), kBlock, 0, st>>>(P.seg_start, P.seg_id, P.nnz, loc, tri, ob, out,
                                                                 present);
    FEA_CHECK_LAUNCH();
}

template <typename R, int NF>
void combine_operator(const Pattern& P, const int32_t* emap, const double* M, const double* K, const double* Adv,
                      const OpCoef<NF>& c, FV<R, NF>* A, FV<R, NF>* dinv, cudaStream_t st) {
    if (P.nnz > 0) {
        k_combine<R, NF><<<launch_grid(P.nnz), kBlock, 0, st>>>(P.nnz, emap, M, K, Adv, c, A);
        FEA_CHECK_LAUNCH();
    }
    if (P.N > 0) {
        k_dinv<R, NF><<<launch_grid(P.N), kBlock, 0, st>>>(P.N, P.diag, A, dinv);
        FEA_CHECK_LAUNCH();
    }
}

template <typename R>
void round_copy(const double* in, const int32_t* map, int64_t n, R* out, cudaStream_t st) {
    if (n <= 0) return;
    k_round_copy<R><<<launch_grid(n), kBlock, 0, st>>>(in, map, n, out);
    FEA_CHECK_LAUNCH();
}

#define FEA_INST_R(R)                                                                                       \
    template void element_matrices<R>(const float*, const uint32_t*, int64_t, int, const float*, const float*, \
                                      R*, R*, R*, cudaStream_t);                                           \
    template void ordered_sum<R>(const Pattern&, const R*, const R*, R*, cudaStream_t);                    \
    template void ordered_sum_adv<R>(const Pattern&, const R*, const uint32_t*, const uint8_t*, R*, uint8_t*, \
                                     cudaStream_t);                                                        \
    template void combine_operator<R, 1>(const Pattern&, const int32_t*, const double*, const double*,     \
                                         const double*, const OpCoef<1>&, FV<R, 1>*, FV<R, 1>*, cudaStream_t); \
    template void combine_operator<R, 2>(const Pattern&, const int32_t*, const double*, const double*,     \
                                         const double*, const OpCoef<2>&, FV<R, 2>*, FV<R, 2>*, cudaStream_t); \
    template void round_copy<R>(const double*, const int32_t*, int64_t, R*, cudaStream_t);
FEA_INST_R(float)
FEA_INST_R(double)

}  // namespace fea
