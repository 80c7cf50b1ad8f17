/*
 * fea_oracle.h -- CPU restatement of the reference's FEM hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA path and
 * the CPU baseline timed beside it; the product never links, loads or calls it.
 *
 * What it restates (paths are relative to the reference project):
 *   - boundary detection            src/Utils/Surface.cpp:104-122
 *   - idx_map / num_unknowns        src/FEM/FEMContext.cpp:46-48, 224-240
 *   - stiffness / mass / advection  src/FEM/FEMContext.cpp:70-202
 *     assembly, including the boundary filters (Adv ignores the BC, :188)
 *   - Eigen::SparseMatrix::setFromTriplets + makeCompressed: duplicates summed
 *     in triplet order, compressed storage with sorted inner indices and
 *     explicit zeros kept (restated from Eigen's documented behaviour; Eigen is
 *     not vendored with the reference and its pinned commit is unknown)
 *   - CPUSolver::advance_time for heat / advection-diffusion / wave /
 *     Gray-Scott, CPUSolver.cpp:64-146, and has_numerical_instability :41-48
 *   - Eigen::ConjugateGradient<.., Lower|Upper> with the default diagonal
 *     preconditioner: zero initial guess, stop when |r|^2 < tol^2 |b|^2,
 *     at most 2N iterations (Eigen's documented defaults)
 * plus the extensions the GPU path implements (consistent Gray-Scott reaction,
 * explicit advection, Newmark-beta wave, per-element diffusivity/velocity),
 * an FP64 adjoint of the implicit advection-diffusion step, and the steps
 * after the solve: extruded smooth normals (shaders/FEM/smooth_normals.glsl)
 * and the iso-clipped .ply geometry (src/Utils/Surface.cpp:138-285).
 *
 * Parity status: UNPINNED against reference outputs -- the reference publishes
 * no golden vectors and cannot be compiled here (Eigen and glm are absent).
 * The restatement is pinned instead against derived known-answer tests
 * (closed-form element matrices, K*1 = 0, sum(M) = area, nnz = V + 2E on the
 * reference's icosphere.obj, heat-kernel decay on the sphere).
 *
 * Numeric functions exist in two precisions: suffix _f64 (double) and _f32
 * (float, the reference's arithmetic type).
 */
#ifndef FEA_ORACLE_H
#define FEA_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- integer / pattern work (precision independent) ---------------------- */

/* on_boundary[v] = 1 for vertices of an edge used by exactly one triangle.
 * Returns the number of boundary points.  Surface.cpp:104-122. */
int64_t fo_boundary(int64_t V, int64_t T, const uint32_t* tri, uint8_t* on_boundary);

/* idx_map for bc (0 Dirichlet, 1 Neumann); returns num_unknowns.
 * FEMContext.cpp:224-240 and :46-48. */
int64_t fo_idx_map(int64_t V, const uint8_t* on_boundary, int bc, int32_t* idx_map);

/* Eigen-compressed pattern of the stiffness/mass triplets.  The build is
 * two-phase: fo_pattern_build returns an opaque object, fo_pattern_nnz its
 * size, fo_pattern_copy writes row_ptr[N+1], col[nnz], and for every local
 * entry (k, i, j) -> index 9k+3i+j the CSR slot it sums into (slot, -1 when the
 * BC filter drops it) and the slot under the advection filter (adv_slot). */
void* fo_pattern_build(int64_t V, int64_t T, const uint32_t* tri, const uint8_t* on_boundary,
                       const int32_t* idx_map, int bc);
int64_t fo_pattern_nnz(const void* p);
int64_t fo_pattern_rows(const void* p);
void fo_pattern_copy(const void* p, int32_t* row_ptr, int32_t* col, int32_t* slot, int32_t* adv_slot);
void fo_pattern_free(void* p);

/* ---- numeric work (instantiated for double and float) --------------------- */

typedef struct {
    int equation;       /* 0 heat, 1 wave, 2 advection-diffusion, 3 Gray-Scott */
    double dt;
    double kappa;       /* heat conductivity / advection-diffusion c / wave c */
    double Du, Dv, F, k;
    int reaction_mode;  /* 0 reference (nodal reaction), 1 consistent (M-weighted) */
    int wave_scheme;    /* 0 reference semi-implicit, 1 Newmark-beta */
    double beta, gamma; /* Newmark */
    int adv_scheme;     /* 0 implicit (A = M/dt + cK - Adv), 1 explicit (b += s*Adv*u) */
    double adv_sign;    /* s for the explicit scheme */
    int k_scaled;       /* 1: K already carries the diffusivity (per-element D) */
    double tol;         /* CG relative tolerance */
    int max_iter;       /* <= 0: 2N (Eigen default) */
    int warm_start;     /* 0: zero guess (Eigen solve()), 1: previous field,
                           2 (Gray-Scott): 2 x_n - x_(n-1) from the call's own
                           previous step; on its first step from prev_u/prev_v
                           when given, else the previous field */
    int nthreads;       /* OpenMP threads for SpMV/dots (1 = serial, deterministic) */
    const void* prev_u; /* warm_start 2: the state one step before u, v (R[N]) or NULL */
    const void* prev_v;
} fo_params;

#define FO_DECL(R, S) \
    void fo_element_matrices_##S(int64_t T, const float* xyz, const uint32_t* tri, int vel_mode, \
                                 const float* velocity, const float* elem_vel, \
                                 R* Kloc, R* Mloc, R* Aloc); \
    void fo_sum_##S(int64_t T, const int32_t* slot, const R* loc, const R* elem_scale, \
                    int64_t nnz, R* out); \
    void fo_spmv_##S(int64_t N, const int32_t* row_ptr, const int32_t* col, const R* val, \
                     const R* x, R* y); \
    int64_t fo_pcg_##S(int64_t N, const int32_t* row_ptr, const int32_t* col, const R* val, \
                       const R* b, R* x, double tol, int64_t max_iter, int zero_guess, \
                       int nthreads, double* rel_res); \
    int64_t fo_step_##S(int64_t N, const int32_t* row_ptr, const int32_t* col, \
                        const R* M, const R* K, const R* Adv, const fo_params* prm, \
                        R* u, R* v, R* a, int64_t nsteps, int64_t* iters); \
    int fo_newmark_init_##S(int64_t N, const int32_t* row_ptr, const int32_t* col, \
                            const R* M, const R* K, const fo_params* prm, const R* u, R* a); \
    int fo_instability_##S(int64_t N, const R* u, const R* v);

FO_DECL(double, f64)
FO_DECL(float, f32)

/* FP64 adjoint of J = 1/2 |u_N - target|_M^2 for the explicit advection-diffusion
 * step (M/dt + K_D) u' = (M/dt + s Adv) u with K_D = sum_e D_e K_e.  Returns the
 * loss; writes dJ/du0 [N] and dJ/dD [T].  Forward states are recomputed from
 * checkpoints every `ckpt` steps.  Kloc: per-element stiffness blocks [9T]. */
double fo_adjoint_advdiff_f64(int64_t N, int64_t T, const int32_t* row_ptr, const int32_t* col,
                              const int32_t* slot, const double* M, const double* Adv,
                              const double* Kloc, const double* D, const int32_t* idx_node,
                              const uint32_t* tri, const fo_params* prm, const double* u0,
                              const double* target, int64_t nsteps, int64_t ckpt,
                              double* grad_u0, double* grad_D);

/* FP64 adjoint of the mass-weighted Gray-Scott step (the loss 1/2 |x_N - t|_M^2
 * over the fields whose target is not NULL).  Returns the loss; writes dJ/du0,
 * dJ/dv0 [N] and grad_params[4] = dJ/dF, dJ/dk, dJ/dDu, dJ/dDv.  prm: the
 * Gray-Scott parameters (dt, Du, Dv, F, k, tol, max_iter, warm_start). */
double fo_adjoint_gray_scott_f64(int64_t N, const int32_t* row_ptr, const int32_t* col, const double* M,
                                 const double* K, const fo_params* prm, const double* u0, const double* v0,
                                 const double* target_u, const double* target_v, int64_t nsteps, int64_t ckpt,
                                 double* grad_u0, double* grad_v0, double* grad_params);

/* Extruded smooth normals (shaders/FEM/smooth_normals.glsl:30-57): for each
 * triangle, cross(b' - a', c' - a') of its corners moved along `normals` by
 * min(1, extrusion * max(0, value)), added to its three vertices (in triangle
 * order).  out: float[3V]. */
void fo_smooth_normals_f32(int64_t V, int64_t T, const float* xyz, const uint32_t* tri, const float* normals,
                           const float* values, float extrusion, float* out);

/* Geometry of Surface::export_to_ply (Surface.cpp:138-285): clipped
 * positions (first-seen order, exact-equality dedup), their values, and the
 * output triangles.  mesh_type 0 Open, 1 Closed, 2 Mirrored.  Returns the
 * vertex count; *ntri receives the triangle count (arrays hold at most
 * cap_v / cap_t). */
int64_t fo_ply_clip(int64_t V, int64_t T, const float* xyz, const uint32_t* tri, const float* normals,
                    const float* values, float extrusion, float threshold, int mesh_type, float* pos_out,
                    float* val_out, int64_t cap_v, uint32_t* tri_out, int64_t cap_t, int64_t* ntri);

#ifdef __cplusplus
}
#endif
#endif
