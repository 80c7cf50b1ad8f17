/*
 * fea_oracle_adjoint.c -- FP64 adjoint of the explicit advection-diffusion step
 * (test infrastructure only; see fea_oracle.h).
 *
 * Forward step (the SPD form of CPUSolver.cpp:90-103 with the advection term
 * moved to the right-hand side and a per-element diffusivity):
 *     A u^{n+1} = B u^n,   A = M/dt + K_D,  K_D = sum_e D_e K_e,  B = M/dt + s Adv
 * Loss J = 1/2 (u^N - t)^T M (u^N - t).
 * Reverse sweep: lambda^N = M (u^N - t); for n = N-1 .. 0:
 *     mu = A^{-1} lambda^{n+1}            (A is symmetric)
 *     dJ/dD_e -= mu_e^T K_e u_e^{n+1}
 *     lambda^n = B^T mu
 * dJ/du^0 = lambda^0.  States are recomputed from checkpoints every `ckpt`
 * steps.  All solves use Jacobi-PCG to |r| <= tol |b|.
 */
#include "fea_oracle.h"

#include <stdlib.h>
#include <string.h>

static void axT(int64_t N, const int32_t* rp, const int32_t* col, const double* val, const double* x,
                double* y) {
    memset(y, 0, sizeof(double) * (size_t)N);
    for (int64_t i = 0; i < N; i++)
        for (int32_t e = rp[i]; e < rp[i + 1]; e++) y[col[e]] += val[e] * x[i];
}

static void fwd_step(int64_t N, const int32_t* rp, const int32_t* col, const double* A, const double* M,
                     const double* Adv, const fo_params* prm, const double* u, double* un, double* b,
                     double* w) {
    double dt = prm->dt;
    fo_spmv_f64(N, rp, col, M, u, b);
    fo_spmv_f64(N, rp, col, Adv, u, w);
    for (int64_t i = 0; i < N; i++) b[i] = b[i] / dt + prm->adv_sign * w[i];
    memcpy(un, u, sizeof(double) * (size_t)N);
    double rr;
    fo_pcg_f64(N, rp, col, A, b, un, prm->tol, prm->max_iter, 0, 1, &rr);
}

double fo_adjoint_advdiff_f64(int64_t N, int64_t T, const int32_t* rp, const int32_t* col,
                              const int32_t* slot, const double* M, const double* Adv,
                              const double* Kloc, const double* D, const int32_t* idx_node,
                              const uint32_t* tri, const fo_params* prm, const double* u0,
                              const double* target, int64_t nsteps, int64_t ckpt, double* grad_u0,
                              double* grad_D) {
    int64_t nnz = rp[N];
    double dt = prm->dt;
    if (ckpt < 1) ckpt = 1;
    double* KD = (double*)malloc(sizeof(double) * (size_t)nnz);
    double* A = (double*)malloc(sizeof(double) * (size_t)nnz);
    fo_sum_f64(T, slot, Kloc, D, nnz, KD);
    for (int64_t e = 0; e < nnz; e++) A[e] = M[e] / dt + KD[e];
    int64_t nck = (nsteps + ckpt - 1) / ckpt + 1;
    double* cks = (double*)malloc(sizeof(double) * (size_t)(nck * N));
    double* seg = (double*)malloc(sizeof(double) * (size_t)((ckpt + 1) * N));
    double* b = (double*)malloc(sizeof(double) * (size_t)N);
    double* w = (double*)malloc(sizeof(double) * (size_t)N);
    double* cur = (double*)malloc(sizeof(double) * (size_t)N);
    double* lam = (double*)malloc(sizeof(double) * (size_t)N);
    double* mu = (double*)malloc(sizeof(double) * (size_t)N);
    /* forward sweep, keeping a checkpoint every ckpt steps */
    memcpy(cur, u0, sizeof(double) * (size_t)N);
    for (int64_t n = 0; n < nsteps; n++) {
        if (n % ckpt == 0) memcpy(cks + (n / ckpt) * N, cur, sizeof(double) * (size_t)N);
        fwd_step(N, rp, col, A, M, Adv, prm, cur, lam, b, w);
        memcpy(cur, lam, sizeof(double) * (size_t)N);
    }
    /* loss and its gradient at the final state */
    for (int64_t i = 0; i < N; i++) w[i] = cur[i] - target[i];
    fo_spmv_f64(N, rp, col, M, w, lam);
    double J = 0;
    for (int64_t i = 0; i < N; i++) J += 0.5 * w[i] * lam[i];
    memset(grad_D, 0, sizeof(double) * (size_t)T);
    /* reverse sweep over the segments */
    int64_t last_seg = (nsteps - 1) / ckpt;
    for (int64_t sg = last_seg; sg >= 0; sg--) {
        int64_t n0 = sg * ckpt;
        int64_t n1 = n0 + ckpt < nsteps ? n0 + ckpt : nsteps;
        memcpy(seg, cks + sg * N, sizeof(double) * (size_t)N);
        for (int64_t n = n0; n < n1; n++)
            fwd_step(N, rp, col, A, M, Adv, prm, seg + (n - n0) * N, seg + (n - n0 + 1) * N, b, w);
        for (int64_t n = n1 - 1; n >= n0; n--) {
            const double* unext = seg + (n - n0 + 1) * N;
            memset(mu, 0, sizeof(double) * (size_t)N);
            double rr;
            fo_pcg_f64(N, rp, col, A, lam, mu, prm->tol, prm->max_iter, 1, 1, &rr);
            for (int64_t k = 0; k < T; k++) {
                double acc = 0;
                for (int i = 0; i < 3; i++)
                    for (int j = 0; j < 3; j++) {
                        if (slot[9 * k + 3 * i + j] < 0) continue;
                        int32_t ri = idx_node[tri[3 * k + i]], cj = idx_node[tri[3 * k + j]];
                        acc += mu[ri] * Kloc[9 * k + 3 * i + j] * unext[cj];
                    }
                grad_D[k] -= acc;
            }
            fo_spmv_f64(N, rp, col, M, mu, b);
            axT(N, rp, col, Adv, mu, w);
            for (int64_t i = 0; i < N; i++) lam[i] = b[i] / dt + prm->adv_sign * w[i];
        }
    }
    memcpy(grad_u0, lam, sizeof(double) * (size_t)N);
    free(KD);
    free(A);
    free(cks);
    free(seg);
    free(b);
    free(w);
    free(cur);
    free(lam);
    free(mu);
    return J;
}

/*
 * FP64 adjoint of the Gray-Scott step with the mass-weighted reaction
 * (CPUSolver.cpp:127-145, reaction_mode 1):
 *     A_f x_f' = M w_f(u, v),  A_f = M/dt + D_f K,
 *     w_u = u/dt - u v^2 + F (1 - u),  w_v = v/dt + u v^2 - (F + k) v.
 * Loss J = 1/2 |u_N - t_u|_M^2 + 1/2 |v_N - t_v|_M^2 (a NULL target drops
 * its term).  Reverse sweep, with mu_f = A_f^-1 lam_f and p_f = M mu_f:
 *     lam_u = (1/dt - v^2 - F) p_u + v^2 p_v
 *     lam_v = -2uv p_u + (1/dt + 2uv - F - k) p_v        (at the step's input)
 *     dJ/dF += p_u.(1 - u) - p_v.v,   dJ/dk -= p_v.v,
 *     dJ/dD_f -= mu_f . K x_f'                             (x' the step's output)
 * dJ/du0 = lam_u, dJ/dv0 = lam_v at the end; states recomputed from
 * checkpoints every `ckpt` steps.  grad_params: dF, dk, dDu, dDv.
 */
double fo_adjoint_gray_scott_f64(int64_t N, const int32_t* rp, const int32_t* col, const double* M,
                                 const double* K, const fo_params* prm, const double* u0, const double* v0,
                                 const double* tu, const double* tv, int64_t nsteps, int64_t ckpt,
                                 double* grad_u0, double* grad_v0, double* grad_params) {
    int64_t nnz = rp[N];
    const double dt = prm->dt, F = prm->F, kk = prm->k;
    if (ckpt < 1) ckpt = 1;
    if (ckpt > nsteps) ckpt = nsteps;
    fo_params fp = *prm;
    fp.equation = 3;
    fp.reaction_mode = 1;
    double* A1 = (double*)malloc(sizeof(double) * (size_t)nnz);
    double* A2 = (double*)malloc(sizeof(double) * (size_t)nnz);
    for (int64_t e = 0; e < nnz; e++) {
        A1[e] = M[e] / dt + prm->Du * K[e];
        A2[e] = M[e] / dt + prm->Dv * K[e];
    }
    const int64_t nck = (nsteps + ckpt - 1) / ckpt;
    const size_t vb = sizeof(double) * (size_t)N;
    double* cku = (double*)malloc(vb * (size_t)nck);
    double* ckv = (double*)malloc(vb * (size_t)nck);
    double* su = (double*)malloc(vb * (size_t)(ckpt + 1));
    double* sv = (double*)malloc(vb * (size_t)(ckpt + 1));
    double* u = (double*)malloc(vb);
    double* v = (double*)malloc(vb);
    double* lu = (double*)calloc((size_t)N, sizeof(double));
    double* lv = (double*)calloc((size_t)N, sizeof(double));
    double* mu = (double*)calloc((size_t)N, sizeof(double));
    double* mv = (double*)calloc((size_t)N, sizeof(double));
    double* pu = (double*)malloc(vb);
    double* pv = (double*)malloc(vb);
    double* t = (double*)malloc(vb);
    int64_t it = 0;
    memcpy(u, u0, vb);
    memcpy(v, v0, vb);
    for (int64_t sg = 0; sg < nck; sg++) {
        memcpy(cku + sg * N, u, vb);
        memcpy(ckv + sg * N, v, vb);
        const int64_t n = (sg + 1) * ckpt < nsteps ? ckpt : nsteps - sg * ckpt;
        fo_step_f64(N, rp, col, M, K, NULL, &fp, u, v, NULL, n, &it);
    }
    double J = 0.0;
    if (tu) {
        for (int64_t i = 0; i < N; i++) t[i] = u[i] - tu[i];
        fo_spmv_f64(N, rp, col, M, t, lu);
        for (int64_t i = 0; i < N; i++) J += 0.5 * t[i] * lu[i];
    }
    if (tv) {
        for (int64_t i = 0; i < N; i++) t[i] = v[i] - tv[i];
        fo_spmv_f64(N, rp, col, M, t, lv);
        for (int64_t i = 0; i < N; i++) J += 0.5 * t[i] * lv[i];
    }
    double gF = 0.0, gk = 0.0, gDu = 0.0, gDv = 0.0;
    for (int64_t sg = nck - 1; sg >= 0; sg--) {
        const int64_t n0 = sg * ckpt, n1 = n0 + ckpt < nsteps ? n0 + ckpt : nsteps;
        memcpy(su, cku + sg * N, vb);
        memcpy(sv, ckv + sg * N, vb);
        for (int64_t n = n0; n < n1; n++) {
            double* uo = su + (n - n0 + 1) * N;
            double* vo = sv + (n - n0 + 1) * N;
            memcpy(uo, su + (n - n0) * N, vb);
            memcpy(vo, sv + (n - n0) * N, vb);
            fo_step_f64(N, rp, col, M, K, NULL, &fp, uo, vo, NULL, 1, &it);
        }
        for (int64_t n = n1 - 1; n >= n0; n--) {
            const double* ui = su + (n - n0) * N;
            const double* vi = sv + (n - n0) * N;
            const double* un = su + (n - n0 + 1) * N;
            const double* vn = sv + (n - n0 + 1) * N;
            double rr;
            fo_pcg_f64(N, rp, col, A1, lu, mu, prm->tol, prm->max_iter, 0, 1, &rr);
            fo_pcg_f64(N, rp, col, A2, lv, mv, prm->tol, prm->max_iter, 0, 1, &rr);
            fo_spmv_f64(N, rp, col, K, un, t);
            for (int64_t i = 0; i < N; i++) gDu -= mu[i] * t[i];
            fo_spmv_f64(N, rp, col, K, vn, t);
            for (int64_t i = 0; i < N; i++) gDv -= mv[i] * t[i];
            fo_spmv_f64(N, rp, col, M, mu, pu);
            fo_spmv_f64(N, rp, col, M, mv, pv);
            for (int64_t i = 0; i < N; i++) {
                const double uu = ui[i], vv = vi[i];
                gF += pu[i] * (1.0 - uu) - pv[i] * vv;
                gk -= pv[i] * vv;
                lu[i] = (1.0 / dt - vv * vv - F) * pu[i] + vv * vv * pv[i];
                lv[i] = -2.0 * uu * vv * pu[i] + (1.0 / dt + 2.0 * uu * vv - F - kk) * pv[i];
            }
        }
    }
    memcpy(grad_u0, lu, vb);
    memcpy(grad_v0, lv, vb);
    grad_params[0] = gF;
    grad_params[1] = gk;
    grad_params[2] = gDu;
    grad_params[3] = gDv;
    free(A1);
    free(A2);
    free(cku);
    free(ckv);
    free(su);
    free(sv);
    free(u);
    free(v);
    free(lu);
    free(lv);
    free(mu);
    free(mv);
    free(pu);
    free(pv);
    free(t);
    return J;
}
