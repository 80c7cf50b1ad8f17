// adjoint.cu -- kernels of the hand-written adjoints: the explicit
// advection-diffusion step and the mass-weighted Gray-Scott step.
//
// Forward step (the SPD form of CPUSolver.cpp:90-103 with the advection term
// on the right-hand side and a per-element diffusivity D_e):
//     A u' = B u,   A = M/dt + c K_D,  K_D = sum_e D_e K_e,  B = M/dt + s Adv.
// Loss J = 1/2 (u_N - t)^T M (u_N - t).  Reverse sweep, n = N-1 .. 0:
//     mu = A^-1 lam          (A is symmetric: the forward operator is reused)
//     dJ/dD_e -= c mu_e^T K_e u_e^{n+1}
//     lam = B^T mu = (M/dt) mu + s Adv^T mu
// with lam = M (u_N - t) at the start and dJ/du_0 = lam at the end.  The
// driver (fea_adjoint_advdiff in solver.cu) runs the solves through the step
// graph and recomputes forward states from checkpoints.
#include "cg_device.cuh"

namespace fea {
namespace {

template <typename R>
__global__ void __launch_bounds__(kBlock) k_adj_loss(int64_t N, const int32_t* __restrict__ rp,
                                                     const int32_t* __restrict__ col, const R* __restrict__ M,
                                                     const R* __restrict__ u, const R* __restrict__ t, R* lam,
                                                     double* part, int stride, unsigned int* ticket, double* J) {
    __shared__ typename Acc<R>::Packed red[32];
    Acc<R> acc[1];
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
        Acc<R> s;
        for (int32_t e = rp[i]; e < rp[i + 1]; e++) {
            const int32_t c = col[e];
            s.add_prod(M[e], u[c] - t[c]);
        }
        const R l = s.rounded();
        lam[i] = l;
        acc[0].add_prod(u[i] - t[i], l);
    }
    Acc<R> blk[1], tot[1];
    block_totals<1>(acc, red, blk);
    if (grid_commit<1>(blk, part, stride, ticket, red, tot) && threadIdx.x == 0) *J = 0.5 * tot[0].value();
}

// lam_i = (sum_e M_e mu_c) / dt + s sum_e Adv_{c,i} mu_c over row i's entries
// e (column c); Adv_{c,i} is the transposed slot tpos[e].
template <typename R>
__global__ void __launch_bounds__(kBlock) k_adj_lambda(int64_t N, const int32_t* __restrict__ rp,
                                                       const int32_t* __restrict__ col,
                                                       const int32_t* __restrict__ tpos, const R* __restrict__ M,
                                                       const R* __restrict__ Adv, double dt, double adv_sign,
                                                       const R* __restrict__ mu, R* lam) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
        Acc<R> m, a;
        for (int32_t e = rp[i]; e < rp[i + 1]; e++) {
            const R mc = mu[col[e]];
            m.add_prod(M[e], mc);
            a.add_prod(Adv[tpos[e]], mc);
        }
        lam[i] = (R)(m.value() / dt + adv_sign * a.value());
    }
}

template <typename R>
__global__ void __launch_bounds__(kBlock) k_adj_grad_D(const double* __restrict__ Kloc,
                                                       const uint32_t* __restrict__ tri,
                                                       const int32_t* __restrict__ idx_c, int64_t T, double c,
                                                       const R* __restrict__ mu, const R* __restrict__ u,
                                                       double* gD) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < T; k += (int64_t)gridDim.x * blockDim.x) {
        int32_t r[3];
#pragma unroll
        for (int i = 0; i < 3; i++) r[i] = idx_c[tri[3 * k + i]];
        double acc = 0.0;
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
            for (int j = 0; j < 3; j++) {
                if (r[i] < 0 || r[j] < 0) continue;  // the boundary filter of the stiffness triplets
                acc += (double)mu[r[i]] * Kloc[9 * k + 3 * i + j] * (double)u[r[j]];
            }
        gD[k] -= c * acc;
    }
}

// ---- Gray-Scott (reaction_mode 1) ------------------------------------------------
// Forward: A_f x_f' = M w_f(u, v), A_f = M/dt + D_f K, with the nodal
// w_u = u/dt - u v^2 + F (1 - u) and w_v = v/dt + u v^2 - (F + k) v.
// Reverse, with mu = A^-1 lam (the paired solve) and p_f = M mu_f:
//   lam_u = (1/dt - v^2 - F) p_u + v^2 p_v,  lam_v = -2uv p_u + (1/dt + 2uv - F - k) p_v
// at the step's input (u, v); dJ/dF += p_u (1 - u) - p_v v, dJ/dk -= p_v v,
// dJ/dD_f -= mu_f . K x_f' with x' the step's output.

template <typename R>
__global__ void __launch_bounds__(kBlock) k_gs_adj_loss(int64_t N, const int32_t* __restrict__ rp,
                                                        const int32_t* __restrict__ col, const R* __restrict__ M,
                                                        const FV<R, 2>* __restrict__ x,
                                                        const FV<R, 2>* __restrict__ tg, int use_u, int use_v,
                                                        FV<R, 2>* lam, double* part, int stride,
                                                        unsigned int* ticket, double* J) {
    __shared__ typename Acc<R>::Packed red[32];
    Acc<R> acc[1];
    const int use[2] = {use_u, use_v};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
        Acc<R> s[2];
        for (int32_t e = rp[i]; e < rp[i + 1]; e++) {
            const int32_t c = col[e];
            const FV<R, 2> xc = x[c], tc = tg[c];
#pragma unroll
            for (int f = 0; f < 2; f++)
                if (use[f]) s[f].add_prod(M[e], xc.v[f] - tc.v[f]);
        }
        const FV<R, 2> xi = x[i], ti = tg[i];
        FV<R, 2> l;
#pragma unroll
        for (int f = 0; f < 2; f++) {
            l.v[f] = use[f] ? s[f].rounded() : (R)0;
            if (use[f]) acc[0].add_prod(xi.v[f] - ti.v[f], l.v[f]);
        }
        lam[i] = l;
    }
    Acc<R> blk[1], tot[1];
    block_totals<1>(acc, red, blk);
    if (grid_commit<1>(blk, part, stride, ticket, red, tot) && threadIdx.x == 0) *J = 0.5 * tot[0].value();
}

template <typename R>
__global__ void __launch_bounds__(kBlock) k_gs_adj_step(int64_t N, const int32_t* __restrict__ rp,
                                                        const int32_t* __restrict__ col, const R* __restrict__ M,
                                                        const R* __restrict__ K, const FV<R, 2>* __restrict__ mu,
                                                        const FV<R, 2>* __restrict__ x0,
                                                        const FV<R, 2>* __restrict__ x1, double dt, double F,
                                                        double kr, FV<R, 2>* lam, double* part, int stride,
                                                        unsigned int* ticket, double* g) {
    __shared__ double red[32 * 4];
    double gp[4] = {0.0, 0.0, 0.0, 0.0};  // dF, dk, dDu, dDv of this thread's rows
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
        Acc<R> pu, pv, ku, kv;
        for (int32_t e = rp[i]; e < rp[i + 1]; e++) {
            const int32_t c = col[e];
            const FV<R, 2> mc = mu[c], xc = x1[c];
            const R m = M[e], k = K[e];
            pu.add_prod(m, mc.v[0]);
            pv.add_prod(m, mc.v[1]);
            ku.add_prod(k, xc.v[0]);
            kv.add_prod(k, xc.v[1]);
        }
        const double Pu = pu.value(), Pv = pv.value();
        const double u = (double)x0[i].v[0], v = (double)x0[i].v[1];
        const FV<R, 2> mi = mu[i];
        FV<R, 2> l;
        l.v[0] = (R)((1.0 / dt - v * v - F) * Pu + v * v * Pv);
        l.v[1] = (R)(-2.0 * u * v * Pu + (1.0 / dt + 2.0 * u * v - F - kr) * Pv);
        lam[i] = l;
        gp[0] += Pu * (1.0 - u) - Pv * v;
        gp[1] -= Pv * v;
        gp[2] -= (double)mi.v[0] * ku.value();
        gp[3] -= (double)mi.v[1] * kv.value();
    }
    block_sum<4>(gp, red);
    double tot[4];
    if (last_block_commit<4>(gp, part, stride, ticket, red, tot) && threadIdx.x == 0)
        for (int j = 0; j < 4; j++) g[j] += tot[j];
}

}  // namespace

template <typename R>
void adjoint_loss(const Pattern& P, const R* M, const R* u, const R* t, R* lam, double* part, int stride,
                  unsigned int* ticket, double* J, cudaStream_t st) {
    const int grid = (int)std::min<int64_t>(max_grid_blocks(), std::max<int64_t>(1, ceil_div(P.N, kBlock)));
    k_adj_loss<R><<<grid, kBlock, 0, st>>>(P.N, P.row_ptr, P.col, M, u, t, lam, part, stride, ticket, J);
    FEA_CHECK_LAUNCH();
}

template <typename R>
void adjoint_lambda(const Pattern& P, const R* M, const R* Adv, double dt, double adv_sign, const R* mu, R* lam,
                    cudaStream_t st) {
    if (P.N == 0) return;
    k_adj_lambda<R><<<launch_grid(P.N), kBlock, 0, st>>>(P.N, P.row_ptr, P.col, P.tpos, M, Adv, dt, adv_sign, mu,
                                                         lam);
    FEA_CHECK_LAUNCH();
}

template <typename R>
void adjoint_grad_D(const double* Kloc, const uint32_t* tri, const int32_t* idx_c, int64_t T, double c, const R* mu,
                    const R* u, double* gD, cudaStream_t st) {
    if (T == 0) return;
    k_adj_grad_D<R><<<launch_grid(T), kBlock, 0, st>>>(Kloc, tri, idx_c, T, c, mu, u, gD);
    FEA_CHECK_LAUNCH();
}

template <typename R>
void adjoint_gs_loss(const Pattern& P, const R* M, const FV<R, 2>* x, const FV<R, 2>* t, int use_u, int use_v,
                     FV<R, 2>* lam, double* part, int stride, unsigned int* ticket, double* J, cudaStream_t st) {
    const int grid = (int)std::min<int64_t>(max_grid_blocks(), std::max<int64_t>(1, ceil_div(P.N, kBlock)));
    k_gs_adj_loss<R><<<grid, kBlock, 0, st>>>(P.N, P.row_ptr, P.col, M, x, t, use_u, use_v, lam, part, stride,
                                              ticket, J);
    FEA_CHECK_LAUNCH();
}

template <typename R>
void adjoint_gs_step(const Pattern& P, const R* M, const R* K, const FV<R, 2>* mu, const FV<R, 2>* x0,
                     const FV<R, 2>* x1, double dt, double F, double k, FV<R, 2>* lam, double* part, int stride,
                     unsigned int* ticket, double* g, cudaStream_t st) {
    const int grid = (int)std::min<int64_t>(max_grid_blocks(), std::max<int64_t>(1, ceil_div(P.N, kBlock)));
    k_gs_adj_step<R><<<grid, kBlock, 0, st>>>(P.N, P.row_ptr, P.col, M, K, mu, x0, x1, dt, F, k, lam, part, stride,
                                              ticket, g);
    FEA_CHECK_LAUNCH();
}

#define FEA_INST_ADJ(R)                                                                                         \
    template void adjoint_loss<R>(const Pattern&, const R*, const R*, const R*, R*, double*, int, unsigned int*, \
                                  double*, cudaStream_t);                                                       \
    template void adjoint_lambda<R>(const Pattern&, const R*, const R*, double, double, const R*, R*,          \
                                    cudaStream_t);                                                              \
    template void adjoint_grad_D<R>(const double*, const uint32_t*, const int32_t*, int64_t, double, const R*,   \
                                    const R*, double*, cudaStream_t);                                           \
    template void adjoint_gs_loss<R>(const Pattern&, const R*, const FV<R, 2>*, const FV<R, 2>*, int, int,     \
                                     FV<R, 2>*, double*, int, unsigned int*, double*, cudaStream_t);            \
    template void adjoint_gs_step<R>(const Pattern&, const R*, const R*, const FV<R, 2>*, const FV<R, 2>*,     \
                                     const FV<R, 2>*, double, double, double, FV<R, 2>*, double*, int,        \
                                     unsigned int*, double*, cudaStream_t);
FEA_INST_ADJ(float)
FEA_INST_ADJ(double)

}  // namespace fea
