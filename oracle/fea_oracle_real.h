/*
 * fea_oracle_real.h -- numeric half of the CPU restatement (test infrastructure
 * only; see fea_oracle.h).  Included by fea_oracle_f64.c and fea_oracle_f32.c
 * with R (the arithmetic type) and S (the symbol suffix) defined.
 */
#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "fea_oracle.h"

#define FO_CAT2(a, b) a##_##b
#define FO_CAT(a, b) FO_CAT2(a, b)
#define FN(name) FO_CAT(name, S)

/* Local matrices of FEMContext.cpp:70-202 for every triangle k; entry (i, j)
 * of element k goes to index 9k + 3i + j.
 *   stiffness: A = [b-a, c-a, n]^-T maps the reference gradients (-1,-1,0),
 *              (1,0,0), (0,1,0) to physical ones; K_ij = area * g_i . g_j  (:76-104)
 *   mass:      M_ij = |J|/24 * (1 + delta_ij)                               (:126-140)
 *   advection: Adv_ij = |J|/6 * t . g_j, t the tangential part of the
 *              velocity, normalised when vel_mode == 0 (:179-192; Eigen's
 *              normalized() leaves a zero vector unchanged).  vel_mode == 1
 *              takes a per-element velocity and keeps its magnitude.        */
void FN(fo_element_matrices)(int64_t T, const float* xyz, const uint32_t* tri, int vel_mode,
                             const float* velocity, const float* elem_vel, R* Kloc, R* Mloc,
                             R* Aloc) {
    static const R ref_g[3][3] = {{-1, -1, 0}, {1, 0, 0}, {0, 1, 0}};
    for (int64_t k = 0; k < T; k++) {
        R p[3][3];
        for (int v = 0; v < 3; v++)
            for (int d = 0; d < 3; d++) p[v][d] = (R)xyz[3 * (int64_t)tri[3 * k + v] + d];
        R e1[3], e2[3], cr[3], n[3];
        for (int d = 0; d < 3; d++) {
            e1[d] = p[1][d] - p[0][d];
            e2[d] = p[2][d] - p[0][d];
        }
        cr[0] = e1[1] * e2[2] - e1[2] * e2[1];
        cr[1] = e1[2] * e2[0] - e1[0] * e2[2];
        cr[2] = e1[0] * e2[1] - e1[1] * e2[0];
        R len = (R)sqrt((double)(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]));
        R inv_len = (R)1 / len;
        for (int d = 0; d < 3; d++) n[d] = cr[d] * inv_len;
        R area = (R)0.5 * len;
        /* A = [e1 e2 n] (columns), inverted through its adjugate */
        R m[3][3] = {{e1[0], e2[0], n[0]}, {e1[1], e2[1], n[1]}, {e1[2], e2[2], n[2]}};
        R c00 = m[1][1] * m[2][2] - m[1][2] * m[2][1];
        R c01 = m[1][2] * m[2][0] - m[1][0] * m[2][2];
        R c02 = m[1][0] * m[2][1] - m[1][1] * m[2][0];
        R det = m[0][0] * c00 + m[0][1] * c01 + m[0][2] * c02;
        R id = (R)1 / det;
        R inv[3][3];
        inv[0][0] = c00 * id;
        inv[0][1] = (m[0][2] * m[2][1] - m[0][1] * m[2][2]) * id;
        inv[0][2] = (m[0][1] * m[1][2] - m[0][2] * m[1][1]) * id;
        inv[1][0] = c01 * id;
        inv[1][1] = (m[0][0] * m[2][2] - m[0][2] * m[2][0]) * id;
        inv[1][2] = (m[0][2] * m[1][0] - m[0][0] * m[1][2]) * id;
        inv[2][0] = c02 * id;
        inv[2][1] = (m[0][1] * m[2][0] - m[0][0] * m[2][1]) * id;
        inv[2][2] = (m[0][0] * m[1][1] - m[0][1] * m[1][0]) * id;
        /* physical gradient g_i = inv^T * ref_i */
        R g[3][3];
        for (int i = 0; i < 3; i++)
            for (int r = 0; r < 3; r++)
                g[i][r] = inv[0][r] * ref_g[i][0] + inv[1][r] * ref_g[i][1] + inv[2][r] * ref_g[i][2];
        R jac = len;
        R mscale = (R)((double)jac / 24.0);
        R ascale = jac / (R)6;
        R vel[3];
        for (int d = 0; d < 3; d++) vel[d] = (R)(vel_mode == 0 ? velocity[d] : elem_vel[3 * k + d]);
        R vn = vel[0] * n[0] + vel[1] * n[1] + vel[2] * n[2];
        R nn = n[0] * n[0] + n[1] * n[1] + n[2] * n[2];
        R t[3];
        for (int d = 0; d < 3; d++) t[d] = vel[d] - vn / nn * n[d];
        if (vel_mode == 0) {
            R tl = (R)sqrt((double)(t[0] * t[0] + t[1] * t[1] + t[2] * t[2]));
            if (tl > 0)
                for (int d = 0; d < 3; d++) t[d] = t[d] / tl;
        }
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) {
                int64_t e = 9 * k + 3 * i + j;
                Kloc[e] = area * (g[i][0] * g[j][0] + g[i][1] * g[j][1] + g[i][2] * g[j][2]);
                Mloc[e] = mscale * (R)(i == j ? 2 : 1);
                Aloc[e] = ascale * (t[0] * g[j][0] + t[1] * g[j][1] + t[2] * g[j][2]);
            }
    }
}

/* Duplicate summation of setFromTriplets: out[slot] accumulates the local
 * entries in triplet order (elements ascending, then i, then j).  With
 * elem_scale the entry of element k is scaled first (per-element diffusivity). */
void FN(fo_sum)(int64_t T, const int32_t* slot, const R* loc, const R* elem_scale, int64_t nnz,
                R* out) {
    memset(out, 0, sizeof(R) * (size_t)nnz);
    for (int64_t k = 0; k < T; k++)
        for (int e = 0; e < 9; e++) {
            int32_t s = slot[9 * k + e];
            if (s < 0) continue;
            R val = elem_scale ? elem_scale[k] * loc[9 * k + e] : loc[9 * k + e];
            out[s] = out[s] + val;
        }
}

/* y = A x; each row sums in increasing column order, the order Eigen's
 * column-major sparse * dense product reaches row i in. */
void FN(fo_spmv)(int64_t N, const int32_t* rp, const int32_t* col, const R* val, const R* x, R* y) {
    for (int64_t i = 0; i < N; i++) {
        R acc = 0;
        for (int32_t e = rp[i]; e < rp[i + 1]; e++) acc += val[e] * x[col[e]];
        y[i] = acc;
    }
}

static void FN(spmv_mt)(int64_t N, const int32_t* rp, const int32_t* col, const R* val, const R* x,
                        R* y, int nt) {
#pragma omp parallel for schedule(static) num_threads(nt) if (nt > 1)
    for (int64_t i = 0; i < N; i++) {
        R acc = 0;
        for (int32_t e = rp[i]; e < rp[i + 1]; e++) acc += val[e] * x[col[e]];
        y[i] = acc;
    }
}

static double FN(dot_mt)(int64_t N, const R* a, const R* b, int nt) {
    double acc = 0;
#pragma omp parallel for schedule(static) reduction(+ : acc) num_threads(nt) if (nt > 1)
    for (int64_t i = 0; i < N; i++) acc += (double)a[i] * (double)b[i];
    return acc;
}

/* Jacobi-preconditioned CG with the semantics of Eigen::ConjugateGradient
 * (CPUSolver.cpp:65): inverse-diagonal preconditioner (1 where the diagonal
 * is 0), stop when |r|^2 < max(tol^2 |b|^2, smallest normal), at most max_iter
 * iterations (2N when max_iter <= 0).  Inner products accumulate in double.
 * Returns the number of A*p products; *rel_res = |r| / |b|. */
int64_t FN(fo_pcg)(int64_t N, const int32_t* rp, const int32_t* col, const R* val, const R* b, R* x,
                   double tol, int64_t max_iter, int zero_guess, int nt, double* rel_res) {
    if (max_iter <= 0) max_iter = 2 * N;
    if (nt < 1) nt = 1;
    R* r = (R*)malloc(sizeof(R) * (size_t)N);
    R* z = (R*)malloc(sizeof(R) * (size_t)N);
    R* p = (R*)malloc(sizeof(R) * (size_t)N);
    R* q = (R*)malloc(sizeof(R) * (size_t)N);
    R* dinv = (R*)malloc(sizeof(R) * (size_t)N);
    for (int64_t i = 0; i < N; i++) {
        R d = 0;
        for (int32_t e = rp[i]; e < rp[i + 1]; e++)
            if (col[e] == i) d += val[e];
        dinv[i] = d != 0 ? (R)1 / d : (R)1;
    }
    if (zero_guess) memset(x, 0, sizeof(R) * (size_t)N);
    FN(spmv_mt)(N, rp, col, val, x, q, nt);
#pragma omp parallel for schedule(static) num_threads(nt) if (nt > 1)
    for (int64_t i = 0; i < N; i++) r[i] = b[i] - q[i];
    double rhs2 = FN(dot_mt)(N, b, b, nt);
    int64_t it = 0;
    double rn2 = 0;
    if (rhs2 == 0) {
        memset(x, 0, sizeof(R) * (size_t)N);
        if (rel_res) *rel_res = 0;
        goto done;
    }
    {
        double thr = tol * tol * rhs2;
        double tiny = (sizeof(R) == sizeof(float)) ? (double)FLT_MIN : DBL_MIN;
        if (thr < tiny) thr = tiny;
        rn2 = FN(dot_mt)(N, r, r, nt);
        if (rn2 < thr) goto fin;
#pragma omp parallel for schedule(static) num_threads(nt) if (nt > 1)
        for (int64_t i = 0; i < N; i++) p[i] = dinv[i] * r[i];
        double abs_new = FN(dot_mt)(N, r, p, nt);
        while (it < max_iter) {
            FN(spmv_mt)(N, rp, col, val, p, q, nt);
            it++;
            R alpha = (R)(abs_new / FN(dot_mt)(N, p, q, nt));
#pragma omp parallel for schedule(static) num_threads(nt) if (nt > 1)
            for (int64_t i = 0; i < N; i++) {
                x[i] += alpha * p[i];
                r[i] -= alpha * q[i];
            }
            rn2 = FN(dot_mt)(N, r, r, nt);
            if (rn2 < thr) break;
#pragma omp parallel for schedule(static) num_threads(nt) if (nt > 1)
            for (int64_t i = 0; i < N; i++) z[i] = dinv[i] * r[i];
            double abs_old = abs_new;
            abs_new = FN(dot_mt)(N, r, z, nt);
            R beta = (R)(abs_new / abs_old);
#pragma omp parallel for schedule(static) num_threads(nt) if (nt > 1)
            for (int64_t i = 0; i < N; i++) p[i] = z[i] + beta * p[i];
        }
    fin:
        if (rel_res) *rel_res = sqrt(rn2 / rhs2);
    }
done:
    free(r);
    free(z);
    free(p);
    free(q);
    free(dinv);
    return it;
}

/* Operator values on the shared pattern: am*M + ak*K + aa*Adv, evaluated per
 * entry as the reference's sparse sums do. */
static void FN(combine)(int64_t nnz, const R* M, R am_div, const R* K, R ak, const R* Adv, R aa, R* out,
                        int nt) {
#pragma omp parallel for schedule(static) num_threads(nt) if (nt > 1)
    for (int64_t e = 0; e < nnz; e++) {
        R v = M[e] / am_div + ak * K[e];
        if (Adv && aa != 0) v = v + aa * Adv[e];
        out[e] = v;
    }
}

/* y = (M/dt) x, the scaled-matrix product of CPUSolver.cpp:78. */
static void FN(mass_dt)(int64_t N, const int32_t* rp, const int32_t* col, const R* M, R dt, const R* x,
                        R* y, int nt) {
#pragma omp parallel for schedule(static) num_threads(nt) if (nt > 1)
    for (int64_t i = 0; i < N; i++) {
        R acc = 0;
        for (int32_t e = rp[i]; e < rp[i + 1]; e++) acc += (M[e] / dt) * x[col[e]];
        y[i] = acc;
    }
}

int FN(fo_newmark_init)(int64_t N, const int32_t* rp, const int32_t* col, const R* M, const R* K,
                        const fo_params* prm, const R* u, R* a) {
    R* b = (R*)malloc(sizeof(R) * (size_t)N);
    R c2 = (R)(prm->kappa * prm->kappa);
    FN(fo_spmv)(N, rp, col, K, u, b);
    for (int64_t i = 0; i < N; i++) b[i] = -c2 * b[i];
    double rr;
    FN(fo_pcg)(N, rp, col, M, b, a, prm->tol, prm->max_iter, 1, prm->nthreads, &rr);
    free(b);
    return 0;
}

/* CPUSolver::advance_time (CPUSolver.cpp:64-146) for `nsteps` steps, plus the
 * extensions selected in prm.  u, v, a are unknown-indexed fields; *iters
 * accumulates A*p products.  Returns has_numerical_instability flags of the
 * final state. */
int64_t FN(fo_step)(int64_t N, const int32_t* rp, const int32_t* col, const R* M, const R* K,
                    const R* Adv, const fo_params* prm, R* u, R* v, R* a, int64_t nsteps,
                    int64_t* iters) {
    int64_t nnz = rp[N];
    int nt = prm->nthreads < 1 ? 1 : prm->nthreads;
    R dt = (R)prm->dt;
    R* A1 = (R*)malloc(sizeof(R) * (size_t)nnz);
    R* A2 = (R*)malloc(sizeof(R) * (size_t)nnz);
    R* b1 = (R*)malloc(sizeof(R) * (size_t)N);
    R* b2 = (R*)malloc(sizeof(R) * (size_t)N);
    R* w1 = (R*)malloc(sizeof(R) * (size_t)N);
    R* w2 = (R*)malloc(sizeof(R) * (size_t)N);
    R* x1 = (R*)malloc(sizeof(R) * (size_t)N);
    R* x2 = (R*)malloc(sizeof(R) * (size_t)N);
    R* up = (R*)malloc(sizeof(R) * (size_t)N);  /* the previous step's state (warm_start 2) */
    R* vp = (R*)malloc(sizeof(R) * (size_t)N);
    int zg = prm->warm_start ? 0 : 1;
    int have_prev = prm->warm_start == 2 && prm->prev_u && prm->prev_v;
    if (have_prev) {
        memcpy(up, prm->prev_u, sizeof(R) * (size_t)N);
        memcpy(vp, prm->prev_v, sizeof(R) * (size_t)N);
    }
    double rr;
    int64_t total = 0;
    R kap = (R)prm->kappa;
    for (int64_t s = 0; s < nsteps; s++) {
        switch (prm->equation) {
        case 0: { /* heat, CPUSolver.cpp:72-85 */
            FN(combine)(nnz, M, dt, K, prm->k_scaled ? (R)1 : kap, NULL, 0, A1, nt);
            FN(mass_dt)(N, rp, col, M, dt, u, b1, nt);
            memcpy(x1, u, sizeof(R) * (size_t)N);
            total += FN(fo_pcg)(N, rp, col, A1, b1, x1, prm->tol, prm->max_iter, zg, nt, &rr);
            memcpy(u, x1, sizeof(R) * (size_t)N);
        } break;
        case 2: { /* advection-diffusion, CPUSolver.cpp:90-103 */
            R kd = prm->k_scaled ? (R)1 : kap;
            FN(mass_dt)(N, rp, col, M, dt, u, b1, nt);
            if (prm->adv_scheme == 0) {
                FN(combine)(nnz, M, dt, K, kd, Adv, (R)-1, A1, nt);
            } else {
                FN(combine)(nnz, M, dt, K, kd, NULL, 0, A1, nt);
                FN(spmv_mt)(N, rp, col, Adv, u, w1, nt);
                R sg = (R)prm->adv_sign;
                for (int64_t i = 0; i < N; i++) b1[i] = b1[i] + sg * w1[i];
            }
            memcpy(x1, u, sizeof(R) * (size_t)N);
            total += FN(fo_pcg)(N, rp, col, A1, b1, x1, prm->tol, prm->max_iter, zg, nt, &rr);
            memcpy(u, x1, sizeof(R) * (size_t)N);
        } break;
        case 1: { /* wave */
            R c2 = kap * kap;
            if (prm->wave_scheme == 0) { /* CPUSolver.cpp:108-122 */
#pragma omp parallel for schedule(static) num_threads(nt) if (nt > 1)
                for (int64_t e = 0; e < nnz; e++) A1[e] = M[e] / dt + (c2 * K[e]) * dt;
                FN(mass_dt)(N, rp, col, M, dt, v, b1, nt);
                FN(spmv_mt)(N, rp, col, K, u, w1, nt);
                for (int64_t i = 0; i < N; i++) b1[i] = b1[i] - c2 * w1[i];
                memcpy(x1, v, sizeof(R) * (size_t)N);
                total += FN(fo_pcg)(N, rp, col, A1, b1, x1, prm->tol, prm->max_iter, zg, nt, &rr);
                memcpy(v, x1, sizeof(R) * (size_t)N);
                for (int64_t i = 0; i < N; i++) u[i] = u[i] + v[i] * dt;
            } else { /* Newmark-beta, acceleration form */
                R be = (R)prm->beta, ga = (R)prm->gamma;
                R bdt2 = be * dt * dt;
#pragma omp parallel for schedule(static) num_threads(nt) if (nt > 1)
                for (int64_t e = 0; e < nnz; e++) A1[e] = M[e] + (bdt2 * c2) * K[e];
                for (int64_t i = 0; i < N; i++) {
                    w1[i] = u[i] + dt * v[i] + dt * dt * ((R)0.5 - be) * a[i];
                    w2[i] = v[i] + dt * ((R)1 - ga) * a[i];
                }
                FN(spmv_mt)(N, rp, col, K, w1, b1, nt);
                for (int64_t i = 0; i < N; i++) b1[i] = -c2 * b1[i];
                memcpy(x1, a, sizeof(R) * (size_t)N);
                total += FN(fo_pcg)(N, rp, col, A1, b1, x1, prm->tol, prm->max_iter, zg, nt, &rr);
                for (int64_t i = 0; i < N; i++) {
                    a[i] = x1[i];
                    u[i] = w1[i] + bdt2 * a[i];
                    v[i] = w2[i] + ga * dt * a[i];
                }
            }
        } break;
        case 3: { /* Gray-Scott, CPUSolver.cpp:127-145 */
            R F = (R)prm->F, kk = (R)prm->k;
            FN(combine)(nnz, M, dt, K, (R)prm->Du, NULL, 0, A1, nt);
            FN(combine)(nnz, M, dt, K, (R)prm->Dv, NULL, 0, A2, nt);
            if (prm->reaction_mode == 0) {
                FN(mass_dt)(N, rp, col, M, dt, u, b1, nt);
                FN(mass_dt)(N, rp, col, M, dt, v, b2, nt);
                for (int64_t i = 0; i < N; i++) {
                    R uvv = u[i] * (v[i] * v[i]);
                    R bu = b1[i] - uvv;
                    b1[i] = bu + F * ((R)1 - u[i]);
                    R bv = b2[i] + uvv;
                    b2[i] = bv - (F + kk) * v[i];
                }
            } else {
                for (int64_t i = 0; i < N; i++) {
                    R uvv = u[i] * (v[i] * v[i]);
                    w1[i] = u[i] / dt - uvv + F * ((R)1 - u[i]);
                    w2[i] = v[i] / dt + uvv - (F + kk) * v[i];
                }
                FN(spmv_mt)(N, rp, col, M, w1, b1, nt);
                FN(spmv_mt)(N, rp, col, M, w2, b2, nt);
            }
            if (prm->warm_start == 2 && (s > 0 || have_prev)) {  /* extrapolated start, as the GPU's cg_initial_guess 1 */
                for (int64_t i = 0; i < N; i++) {
                    x1[i] = (R)2 * u[i] - up[i];
                    x2[i] = (R)2 * v[i] - vp[i];
                }
            } else {
                memcpy(x1, u, sizeof(R) * (size_t)N);
                memcpy(x2, v, sizeof(R) * (size_t)N);
            }
            memcpy(up, u, sizeof(R) * (size_t)N);
            memcpy(vp, v, sizeof(R) * (size_t)N);
            total += FN(fo_pcg)(N, rp, col, A1, b1, x1, prm->tol, prm->max_iter, zg, nt, &rr);
            total += FN(fo_pcg)(N, rp, col, A2, b2, x2, prm->tol, prm->max_iter, zg, nt, &rr);
            memcpy(u, x1, sizeof(R) * (size_t)N);
            memcpy(v, x2, sizeof(R) * (size_t)N);
        } break;
        default:
            break;
        }
    }
    free(A1);
    free(A2);
    free(b1);
    free(b2);
    free(w1);
    free(w2);
    free(x1);
    free(x2);
    free(up);
    free(vp);
    if (iters) *iters += total;
    return FN(fo_instability)(N, u, v);
}

/* has_numerical_instability (CPUSolver.cpp:41-48): bit 0 = some u_i or v_i
 * above 1e4; bit 1 (extension) = a NaN or infinity in either field. */
int FN(fo_instability)(int64_t N, const R* u, const R* v) {
    int f = 0;
    for (int64_t i = 0; i < N; i++) {
        if (u[i] > (R)1e4f || (v && v[i] > (R)1e4f)) f |= 1;
        if (!isfinite((double)u[i]) || (v && !isfinite((double)v[i]))) f |= 2;
    }
    return f;
}
