/*
 * fea_gpu.h -- C ABI of the GB300 FEM time-stepping library (libfea_gb300.so).
 *
 * It replaces the reference's solver layer for triangle meshes: the Solver
 * interface (include/FEM/Solver.hpp:8-14) with its CPU implementation
 * (src/FEM/CPUSolver.cpp) and compute-shader implementation
 * (src/FEM/GPUSolver.cpp, shaders/FEM/cgm.glsl, shaders/FEM/cgm_helper.glsl),
 * and the matrix assembly of FEMContext (src/FEM/FEMContext.cpp:57-240).
 * Paths are relative to the reference project.
 *
 * Conventions
 *   - Plain C types only.  Host pointers unless a name ends in _device.
 *   - Every function returns an int status: FEA_OK (0) or a negative FEA_ERR_*
 *     code; fea_last_error() gives a one-line message for the calling thread.
 *     No C++ exception crosses this boundary.
 *   - A handle owns one CUDA stream on the device that was current when it
 *     was created.  Calls on one handle must not run concurrently; distinct
 *     handles are independent.  Calls that return host data synchronise.
 *   - Fields are node-indexed float arrays of length num_vertices, like the
 *     reference's Surface::values (include/Utils/Surface.hpp:38).
 */
#ifndef FEA_GPU_H
#define FEA_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif
#if defined(__GNUC__)
#pragma GCC visibility push(default)
#endif

/* ---- status codes -------------------------------------------------------- */
#define FEA_OK 0
#define FEA_ERR_INVALID_ARGUMENT (-1)
#define FEA_ERR_CUDA (-2)
#define FEA_ERR_NO_DEVICE (-3)
#define FEA_ERR_BAD_MESH (-4)    /* Surface.cpp:40-41, 59-74 throw runtime_error */
#define FEA_ERR_OUT_OF_MEMORY (-5)
#define FEA_ERR_STATE (-6)       /* call order violated (e.g. step before assemble) */
#define FEA_ERR_UNSUPPORTED (-7)
#define FEA_ERR_TOO_LARGE (-8)
#define FEA_ERR_SOLVE (-9)       /* a solve broke down or met NaN/Inf (fea_pcg_solve_csr_noalloc) */

/* ---- step status flags (fea_get_status) ---------------------------------- */
#define FEA_STATUS_BLOWUP 1u       /* some u_i or v_i > 1e4 (CPUSolver.cpp:41-48) */
#define FEA_STATUS_NONFINITE 2u    /* NaN or Inf in a field */
#define FEA_STATUS_NOT_CONVERGED 4u /* a CG solve hit max_iter before tol */
#define FEA_STATUS_BREAKDOWN 8u    /* CG breakdown: p.Ap <= 0 or non-finite */

/* ---- enums mirroring the reference --------------------------------------- */
/* Equation, include/FEM/FEMContext.hpp:9-14 (same order and values) */
#define FEA_HEAT 0
#define FEA_WAVE 1
#define FEA_ADVECTION_DIFFUSION 2
#define FEA_REACTION_DIFFUSION 3
/* BoundaryCondition, include/FEM/FEMContext.hpp:16-19 */
#define FEA_DIRICHLET 0
#define FEA_NEUMANN 1
/* arithmetic type of matrix values and fields */
#define FEA_FP32 0
#define FEA_FP64 1
/* matrices for fea_get_matrix */
#define FEA_MATRIX_STIFFNESS 0
#define FEA_MATRIX_MASS 1
#define FEA_MATRIX_ADVECTION 2

/* Parameters: the four structs of include/FEM/EquationParameters.hpp:8-49
 * (same fields, same defaults from fea_params_default) plus the extensions
 * this library adds.  Extensions default to the reference's behaviour. */
typedef struct {
    int equation;                 /* FEA_HEAT .. FEA_REACTION_DIFFUSION */
    /* HeatParameters (EquationParameters.hpp:8-15) */
    float heat_time_step;         /* 0.01 */
    float heat_conductivity;      /* 0.05 */
    /* AdvectionDiffusionParameters (:17-26) */
    float advdiff_time_step;      /* 0.001 */
    float advdiff_c;              /* 0.25 */
    float advdiff_velocity[3];    /* (1, 0, 0) */
    /* WaveParameters (:28-35) */
    float wave_time_step;         /* 0.05 */
    float wave_c;                 /* 0.05 */
    /* ReactionDiffusionParameters (:37-49) */
    float rd_time_step;           /* 0.001 */
    float rd_Du;                  /* 0.08 */
    float rd_Dv;                  /* 0.04 */
    float rd_feed_rate;           /* 0.035 */
    float rd_kill_rate;           /* 0.06 */
    /* --- extensions --- */
    int reaction_mode;   /* 0: reaction added nodally (CPUSolver.cpp:134,137);
                            1: mass-weighted, b = M (u/dt + f(u, v)) */
    int wave_scheme;     /* 0: semi-implicit velocity form (CPUSolver.cpp:113-118);
                            1: Newmark-beta, solve (M + beta dt^2 c^2 K) a = -c^2 K u~ */
    double newmark_beta;  /* 0.25 */
    double newmark_gamma; /* 0.5 */
    int advection_scheme; /* 0: implicit, A = M/dt + cK - Adv (CPUSolver.cpp:95);
                             1: explicit, A = M/dt + K_D, b = (M/dt) u + s Adv u (SPD) */
    float advection_sign; /* s for the explicit scheme (1 = the reference's sign) */
    int velocity_mode;    /* 0: constant velocity, tangential part normalised
                             (FEMContext.cpp:180); 1: per-element velocity from
                             fea_set_element_fields, magnitude kept */
    double cg_tolerance;  /* relative: stop when |r| < tol |b|.  0 -> FLT_EPSILON
                             for FP32 handles, 1e-10 for FP64 (Eigen's default is
                             the type's epsilon) */
    int cg_max_iterations; /* 0 -> 2N (Eigen's default) */
    int cg_refine;         /* after each solve's CG loop, one true-residual pass
                              r = b - A x (CG restarts from it when |r| is still
                              above the tolerance): 1 accumulates it in the
                              handle's accumulators (FP64 for FP64 handles,
                              float-float pairs of about 48 significant bits
                              for FP32 handles), 2 in FP64 for FP32 handles
                              too, 0 skips it.  Default 1. */
    int cg_initial_guess;  /* Gray-Scott: the CG start of each step's solves.
                              0: the previous solution (warm start; the
                              reference's Eigen solve starts from zero,
                              CPUSolver.cpp:140-142); 1: the linear
                              extrapolation 2 x_n - x_(n-1) of the last two
                              steps (the previous solution on a handle's
                              first step and after fields are set to values
                              that differ from the state; writing back the
                              values just read keeps the history).  The
                              stopping rule is the same.  Default 0. */
} fea_params;

typedef struct {
    int64_t num_vertices;        /* FEMContext::num_nodes (FEMContext.cpp:33-35) */
    int64_t num_triangles;
    int64_t num_boundary_points; /* Surface::num_boundary_points */
    int64_t num_unknowns;        /* FEMContext::num_unknowns (:46-48) */
    int64_t nnz;                 /* entries of the compressed stiffness/mass pattern */
    int64_t max_row_nonzeros;    /* FEMContext::compute_max_row_nonzeros (:207-219) */
    int precision;               /* FEA_FP32 / FEA_FP64 */
    int boundary_condition;
    int rows_per_warp_lanes;     /* CG kernel variant (fea_set_cg_variant, fea_autotune) */
    int64_t device_bytes;        /* device memory held by the handle */
} fea_info;

typedef struct {
    uint32_t flags;              /* FEA_STATUS_* accumulated since the last clear */
    int32_t last_iterations[2];  /* CG iterations of the last solve of field 0/1 */
    double last_rel_residual[2]; /* |r| / |b| at exit of that solve */
    int64_t steps_done;          /* steps completed by the last fea_advance_time */
    int64_t total_iterations;    /* CG iterations summed over all solves */
    int64_t cg_launches;         /* CG iteration kernels launched, including the copies
                                    that close an unrolled loop pass without iterating */
} fea_status;

typedef struct fea_solver fea_solver;

/* Defaults of EquationParameters.hpp:8-49 plus reference-behaviour extensions. */
int fea_params_default(fea_params* out);

/* Mesh in, assembly included: replaces FEMContext::init_from_surface
 * (FEMContext.cpp:21-27) -> update_boundary_conditions (:224-240) ->
 * assemble_matrices (:57-64).  vertices: xyz float[3V]; triangles: uint32[3T];
 * on_boundary: uint8[V] or NULL to detect boundary points on the device as
 * Surface::init_from_obj does (Surface.cpp:104-122).  params may be NULL
 * (defaults).  Returns FEA_ERR_BAD_MESH (nothing allocated, no kernel fault)
 * for an empty mesh, a triangle index >= V, a non-finite coordinate, or a
 * zero-area triangle (collinear or repeated corners): the reference builds
 * NaN element matrices from such triangles (glm::normalize of a zero normal,
 * FEMContext.cpp:76) and solves on; here they are refused up front.  A
 * triangle listed twice is valid input: its entries are summed twice, as
 * Eigen's setFromTriplets does, and its edges count twice for the boundary. */
int fea_create(const float* vertices, int64_t num_vertices, const uint32_t* triangles,
               int64_t num_triangles, const uint8_t* on_boundary, int boundary_condition,
               int precision, const fea_params* params, fea_solver** out);
int fea_destroy(fea_solver* s);

/* FEMContext::update_boundary_conditions (FEMContext.cpp:224-240): rebuild
 * idx_map, pattern and matrices for a new BC.  Fields are cleared. */
int fea_set_boundary_condition(fea_solver* s, int boundary_condition);

/* Equation and parameters (FEMContext::equation, FEMContext::parameters).
 * A changed advection velocity re-assembles Adv, as the reference's velocity
 * slider does (Application.cpp:393-394). */
int fea_set_params(fea_solver* s, const fea_params* params);

/* Per-element diffusivity D_e (K_D = sum_e D_e K_e; float[T], NULL = 1) and
 * per-element velocity (float[3T], used when velocity_mode == 1). */
int fea_set_element_fields(fea_solver* s, const float* diffusivity, const float* velocity);

/* Solver::clear_values (CPUSolver.cpp:54-59): u = v = 0 (and Newmark a = 0). */
int fea_clear_values(fea_solver* s);

/* Surface::values in/out.  The displayed field is u for heat, wave and
 * advection-diffusion and v for Gray-Scott, as in CPUSolver.cpp:75/130;
 * set copies values[idx] of unknown points in (get_surface_value_vector,
 * CPUSolver.cpp:13-21), get writes every point, Dirichlet points as 0
 * (map_vector_to_surface, CPUSolver.cpp:28-37).  Both return once the
 * values are in place.  A page-locked host buffer that the device can map
 * (cudaHostAlloc, cudaHostRegister with cudaHostRegisterMapped) is read or
 * written in place by the device; other host memory goes through a staging
 * copy. */
int fea_set_values(fea_solver* s, const float* values);
int fea_get_values(fea_solver* s, float* values);

/* Both state fields at once (node-indexed, float[V] each; NULL leaves a field
 * unchanged).  u/v are the solver-private vectors of CPUSolver.hpp:17-18; for
 * the wave equation v is the velocity.  Setting fields resets Newmark's
 * acceleration, recomputed from M a = -c^2 K u at the next step. */
int fea_set_fields(fea_solver* s, const float* u, const float* v);
int fea_get_fields(fea_solver* s, float* u, float* v);

/* Device-resident variants: pointers to device memory of the handle's
 * device, unknown-indexed, in the handle's precision (float or double).
 * Ordered on the handle's stream and synchronised before returning. */
int fea_set_fields_device(fea_solver* s, const void* u, const void* v);
int fea_get_fields_device(fea_solver* s, void* u, void* v);

/* Solver::advance_time (CPUSolver.cpp:64-146) nsteps times.  The whole step
 * loop runs as one CUDA graph launch; stepping stops early once
 * FEA_STATUS_BLOWUP or FEA_STATUS_NONFINITE is raised (the application pauses
 * there, Application.cpp:532-538).  Asynchronous: returns after the launch. */
int fea_advance_time(fea_solver* s, int64_t nsteps);
/* Wait for the handle's stream. */
int fea_synchronize(fea_solver* s);

/* Solver::has_numerical_instability (CPUSolver.cpp:41-48): *out = 1 when a
 * field value exceeds 1e4 (or is not finite).  Synchronises. */
int fea_has_numerical_instability(fea_solver* s, int* out);
int fea_get_status(fea_solver* s, fea_status* out);
int fea_get_info(fea_solver* s, fea_info* out);

/* Assembled matrix in compressed-row form: row_ptr int32[N+1], col int32[nnz],
 * values in the handle's precision (float or double) [nnz].  The index arrays
 * equal Eigen's compressed column-major storage of the reference's matrices
 * (FEMContext.cpp:110-112) because the pattern is symmetric.  For
 * FEA_MATRIX_ADVECTION the values live on the stiffness pattern; `present`
 * (uint8[nnz], may be NULL) marks the entries that exist in the reference's
 * advection matrix, whose filter ignores the BC (FEMContext.cpp:188). */
int fea_get_matrix(fea_solver* s, int which, int32_t* row_ptr, int32_t* col, void* values,
                   uint8_t* present);

/* Node -> unknown map (FEMContext::idx_map, int32[V]) and boundary flags. */
int fea_get_idx_map(fea_solver* s, int32_t* idx_map, uint8_t* on_boundary);

/* CG kernel variants: 0 and 1 = tile-ELL layout (256-row tiles, 32-row
 * slices stored column-wise, operand and halo staged in shared memory; the
 * first 8 (variant 0) or 4 (variant 1) entries of each row prefetched into
 * registers), 2 and 3 = the same layout
 * with each tile's operator entries and row vectors moved into 2 or 3
 * shared-memory stages by bulk asynchronous copies ahead of the tile being
 * computed, 6 and 7 = variants 2 and 3 with each stage refilled after the
 * next tile's first block barrier (two barriers per tile instead of three),
 * 10 and 11 = variants 2 and 7 whose iterations are finished by the next
 * launch (every block merges the block partials at its start) instead of
 * by the last block to end, 13 = tile-ELL with every load issued by the
 * threads (operator entries into registers one tile ahead, rows half a tile
 * ahead) and the deferred finish, 14 and 15 = variant 13 with the operator
 * entries and columns moved by bulk copies into a ring of 3 or 4
 * shared-memory stages, 4 / 8 / 16 = warp-cooperative CSR with that many
 * entries per lane and window.  A new handle starts on variant 14 (11 when
 * its ring does not fit in shared memory, 10 when only two streamed stages
 * fit, 0 when none do, 8 without the tile-ELL layout).  fea_autotune times
 * one CG iteration of each candidate on this mesh and keeps the fastest
 * (fea_info.rows_per_warp_lanes); the fields are left unchanged. */
int fea_autotune(fea_solver* s);
/* Select a variant explicitly (FEA_ERR_INVALID_ARGUMENT for another value,
 * FEA_ERR_UNSUPPORTED for the tile-ELL variants when the layout, or for the
 * streamed and ring variants the shared memory of their stages, is
 * unavailable on this mesh). */
int fea_set_cg_variant(fea_solver* s, int variant);

/* The CUDA stream (cudaStream_t) the handle runs on, for callers that order
 * their own work or events after it. */
int fea_get_stream(fea_solver* s, void** stream);

/* Diagnostics: mean device time in ms of one CG iteration kernel (the step
 * loop's dominant kernel: the CSR SpMV with the vector updates fused) over
 * `reps` launches on the current operator of the current equation, each
 * launch preceded by a 256 MiB read that evicts the L2 cache (leaving clean
 * lines) when flush_l2 != 0.  CUDA events on the handle's stream.  The probe masks every
 * field, so the fields are written back unchanged; only CG scratch, which the
 * next step recomputes, changes. */
int fea_time_spmv(fea_solver* s, int reps, int flush_l2, double* ms_per_launch);

/* ---- after the solve: extruded smooth normals, .ply export ---------------
 * Smooth normals of the extruded surface (shaders/FEM/smooth_normals.glsl:
 * 30-57, Surface::calculate_normals, Surface.cpp:287-306): every triangle's
 * corners move along `normals` by min(1, vertex_extrusion * max(0, value)) of
 * the displayed field (as fea_get_values); the cross product of the moved
 * triangle's edges is added to its three vertices, unnormalised.  The sums
 * run in ascending triangle order (the shader's atomics have no fixed order).
 * normals, out: float[3V], host (or device for the _device variant). */
int fea_smooth_normals(fea_solver* s, const float* normals, float vertex_extrusion, float* out);
int fea_smooth_normals_device(fea_solver* s, const float* normals, float vertex_extrusion, float* out);

/* MeshType, include/Utils/Surface.hpp:25-29 */
#define FEA_MESH_OPEN 0
#define FEA_MESH_CLOSED 1
#define FEA_MESH_MIRRORED 2

/* Surface::export_to_ply (Surface.cpp:138-285) of the displayed field: the
 * triangles clipped at `threshold` on the extruded surface (plus the
 * projected copies for FEA_MESH_CLOSED / FEA_MESH_MIRRORED), positions
 * numbered in the reference's first-seen order, written as ASCII PLY with the
 * color of each vertex's value from the polynomial color map
 * c0 + t (c1 + t (... + t c6)) (ColorMap::get_color, ColorMap.cpp:12-14);
 * color_coeffs: float[21] (7 RGB coefficients), NULL for gray (t, t, t).
 * normals: host float[3V]. */
int fea_export_ply(fea_solver* s, const char* path, const float* normals, float vertex_extrusion, float threshold,
                   int mesh_type, const float* color_coeffs);
/* The same geometry in memory: positions float[3 n], values float[n],
 * triangles uint32[3 m]; *num_vertices = n, *num_triangles = m (the arrays
 * are filled when n <= max_vertices and m <= max_triangles; call with NULL
 * arrays to size them). */
int fea_ply_geometry(fea_solver* s, const float* normals, float vertex_extrusion, float threshold, int mesh_type,
                     float* positions, float* values, int64_t max_vertices, uint32_t* triangles,
                     int64_t max_triangles, int64_t* num_vertices, int64_t* num_triangles);

/* ---- adjoint (explicit advection-diffusion) ------------------------------
 * Model: nsteps steps of the advection-diffusion equation with
 * advection_scheme 1 (A u' = B u, A = M/dt + c K_D, B = M/dt + s Adv, with
 * c = advdiff_c, s = advection_sign and K_D = sum_e D_e K_e over the current
 * per-element diffusivity) from u0.  Loss J = 1/2 (u_N - target)^T M
 * (u_N - target).  Writes J, dJ/du0 and dJ/dD (per element) from the
 * hand-written adjoint: each reverse step solves with the forward operator
 * (A is symmetric) and back-propagates through the advection term; forward
 * states are recomputed from checkpoints every `checkpoint_every` steps.
 * Gradient outputs may be NULL (NULL for both: forward and loss only).  The
 * handle's field is left at u_N.  FEA_ERR_STATE for another equation or
 * scheme.  No reference counterpart: the reference has no differentiation.
 * Host variant: node-indexed float[V] u0, target and dJ/du0 (0 on Dirichlet
 * points), dJ/dD float[T]. */
int fea_adjoint_advdiff(fea_solver* s, const float* u0, const float* target, int64_t nsteps,
                        int64_t checkpoint_every, double* loss, float* grad_u0, float* grad_D);
/* Device-resident variant: unknown-indexed [N] u0, target and dJ/du0 and
 * per-element [T] dJ/dD, all in the handle's precision. */
int fea_adjoint_advdiff_device(fea_solver* s, const void* u0, const void* target, int64_t nsteps,
                               int64_t checkpoint_every, double* loss, void* grad_u0, void* grad_D);
/* ---- adjoint (mass-weighted Gray-Scott) ------------------------------------
 * Model: nsteps Gray-Scott steps with reaction_mode 1 (A_f x_f' = M w_f(u, v),
 * A_f = M/dt + D_f K; CPUSolver.cpp:127-145 with the mass-weighted reaction)
 * from (u0, v0).  Loss J = 1/2 |u_N - target_u|_M^2 + 1/2 |v_N - target_v|_M^2
 * (a NULL target drops its term).  Writes J, dJ/du0, dJ/dv0 and
 * grad_params[4] = dJ/dF, dJ/dk, dJ/dDu, dJ/dDv from the hand-written
 * adjoint: each reverse step solves with the forward operators (the paired
 * SPD solve) and back-propagates through the reaction's Jacobian; forward
 * states are recomputed from checkpoints.  Outputs may be NULL.  The handle's
 * fields are left at the final state.  FEA_ERR_STATE for another equation or
 * reaction mode.  No reference counterpart.  Host variant: node-indexed
 * float[V] arrays (gradients 0 on Dirichlet points). */
int fea_adjoint_gray_scott(fea_solver* s, const float* u0, const float* v0, const float* target_u,
                           const float* target_v, int64_t nsteps, int64_t checkpoint_every, double* loss,
                           float* grad_u0, float* grad_v0, double* grad_params);
/* Device-resident variant: unknown-indexed [N] arrays in the handle's
 * precision. */
int fea_adjoint_gray_scott_device(fea_solver* s, const void* u0, const void* v0, const void* target_u,
                                  const void* target_v, int64_t nsteps, int64_t checkpoint_every, double* loss,
                                  void* grad_u0, void* grad_v0, double* grad_params);

/* Per-element diffusivity D_e from device memory in the handle's precision
 * ([T]); like fea_set_element_fields without the float rounding for FP64
 * handles.  No reference counterpart. */
int fea_set_element_diffusivity_device(fea_solver* s, const void* diffusivity);

/* ---- batched Gray-Scott ---------------------------------------------------
 * Many independent meshes with their own (F, k, Du, Dv, dt), stepped together:
 * the instances' systems are stacked into one block-diagonal matrix and every
 * CG phase is one persistent kernel over all instances, with per-instance
 * scalars and convergence masks; the whole step loop is one CUDA graph.  No
 * reference counterpart (the reference steps one mesh); each instance follows
 * the Gray-Scott step of CPUSolver.cpp:127-145 with reaction_mode 1 and the
 * single-mesh solver's CG (cg_tolerance 0 -> FLT_EPSILON / 1e-10, max
 * iterations 0 -> 2N of the instance).  A state that exceeds 1e4 freezes only
 * its own instance (FEA_STATUS_BLOWUP in its flags). */
typedef struct {
    const float* vertices;      /* xyz float[3V] */
    int64_t num_vertices;
    const uint32_t* triangles;  /* uint32[3T] */
    int64_t num_triangles;
    int boundary_condition;
    float time_step, Du, Dv, feed_rate, kill_rate;
} fea_instance_desc;

typedef struct fea_batch fea_batch;

int fea_batch_create(const fea_instance_desc* instances, int num_instances, int precision,
                     double cg_tolerance, int cg_max_iterations, fea_batch** out);
int fea_batch_destroy(fea_batch* b);
/* u, v: node-indexed float[V] of instance i */
int fea_batch_set_fields(fea_batch* b, int instance, const float* u, const float* v);
int fea_batch_get_fields(fea_batch* b, int instance, float* u, float* v);
int fea_batch_advance_time(fea_batch* b, int64_t nsteps);
int fea_batch_synchronize(fea_batch* b);
/* flags: uint32[num_instances]; iterations: int32[2*num_instances] (last solve) */
int fea_batch_get_status(fea_batch* b, uint32_t* flags, int32_t* iterations);
/* No reference counterpart.  New CG stopping rule of every instance:
 * tolerance (0 -> FLT_EPSILON, 1e-10 for FP64) and iteration limit (0 ->
 * twice the instance's rows, whole tiles). */
int fea_batch_set_cg(fea_batch* b, double cg_tolerance, int cg_max_iterations);
/* No reference counterpart.  Per instance, int64[num_instances] each (NULL to
 * skip): CG iterations and steps since the batch was created. */
int fea_batch_get_counters(fea_batch* b, int64_t* total_iterations, int64_t* steps_done);
/* No reference counterpart.  Device time of one CG iteration kernel of the
 * batch's variant over every instance (fields masked: x and the instances'
 * state are unchanged; only CG scratch that the next step recomputes is
 * written), averaged over reps back-to-back launches after one warm-up. */
int fea_batch_time_iteration(fea_batch* b, int reps, double* ms_per_launch);
/* CG kernel variant of the batch: 0 / 1 tile-ELL (8 / 4 entries prefetched),
 * 4 / 8 windowed CSR, 14 tile-ELL with the operator streamed through a ring
 * of shared-memory stages by bulk copies, the work shared out evenly over the
 * blocks in groups of 8 tiles of an instance.  FEA_ERR_UNSUPPORTED when a
 * variant's layout or shared memory does not fit the batch.
 * fea_batch_create picks the fastest by timing one iteration of each;
 * *variant receives the current one when `set` is 0. */
int fea_batch_cg_variant(fea_batch* b, int set, int* variant);
/* No reference counterpart.  Start of every instance's solves: rule 0 its
 * state x_n (the default); rule 1 the extrapolated state 2 x_n - x_(n-1)
 * once the instance has stepped since its fields were last set (the
 * single-mesh cg_initial_guess 1).  Rule 1 takes effect with CG variant 14;
 * the other variants start from x_n.  Setting a rule, a new variant or an
 * instance's fields clears the histories it concerns.  Rule 1 allocates two
 * more state-sized vectors on first use. */
int fea_batch_set_initial_guess(fea_batch* b, int rule);

/* ---- solve without device allocation ---------------------------------------
 * No counterpart in the reference.  Solves A x = b with Jacobi-preconditioned
 * CG (the solver of the step loop) on a caller's compressed-row matrix, for
 * callers that cannot allocate device memory mid-run: a render loop where a
 * cudaMalloc/cudaFree would stall the frame (cudaFree synchronises the
 * device), a host framework that has reserved the GPU's memory up front, or
 * code that must not hit out-of-memory half way through a step.  All
 * pointers are device pointers: row_ptr int32[n+1], col int32[nnz], values,
 * b and x of the given precision; x holds the initial guess on entry and the
 * solution on return.  tolerance <= 0 and max_iterations <= 0 select the
 * defaults of fea_params (type epsilon or 1e-10, and 2n).  stream may be
 * NULL (the default stream); the call returns after the solve finished.
 * The work vectors live in one static device array of 16 MiB + 64 KiB that
 * every GPU loading the library holds until exit, so n is limited to
 * 1,048,576 (FP32) or 524,288 (FP64); larger n returns FEA_ERR_TOO_LARGE.
 * The first call on a device looks up that array's device address.  The
 * call reads the loop condition back to the host (a copy and a stream
 * synchronisation every 8 CG iterations), so it cannot be called while its
 * stream is being captured into a graph.  Calls share the array: calls that
 * overlap on the GPU race, so serialise them per device.
 * Outcome: *status_flags (may be NULL) receives FEA_STATUS_* bits --
 * FEA_STATUS_NOT_CONVERGED when max_iterations ran out above the tolerance
 * (the call still returns FEA_OK; *rel_residual tells how far it got),
 * FEA_STATUS_BREAKDOWN when p.Ap <= 0 (A is not SPD), FEA_STATUS_NONFINITE
 * for NaN or Inf in A, b, x or the iterates.  The last two return
 * FEA_ERR_SOLVE: x is then no solution.  A zero b gives x = 0 (Eigen's early
 * exit), 0 iterations and FEA_OK. */
int fea_pcg_solve_csr_noalloc(int64_t n, const int32_t* row_ptr, const int32_t* col, const void* values,
                              const void* b, void* x, int precision, double tolerance, int max_iterations,
                              void* stream, int* iterations, double* rel_residual, unsigned int* status_flags);

/* ---- drawn domains: PSLG -> quality triangle mesh ----------------------------
 * Replaces Surface::init_from_PSLG + Surface::perform_triangulation
 * (src/Utils/Surface.cpp:25-49, 431-486), which call Triangle with the
 * switches "Qeqpza<area>": a conforming quality mesh (minimum angle
 * min_angle_deg, Triangle's default 20; max_area = PSLG::triangle_area,
 * include/Utils/PSLG.hpp:29, default 0.005; 0 for no area bound) of the
 * region enclosed by the segments, with the triangles around each hole point
 * removed.  points: double[2 * num_points], the (x, z) coordinates on the XZ
 * plane (Surface.cpp:28-31); segments: int32[2 * num_segments] point index
 * pairs; holes: double[2 * num_holes] (x, z) or NULL.  Host code (no GPU).
 * The result holds vertices (x, 0, z), triangles with the reference's
 * reversed corner order (Surface.cpp:468) and on_boundary = 1 for vertices on
 * a segment (Triangle's point markers, Surface.cpp:472-478), ready for
 * fea_create.  FEA_ERR_BAD_MESH for an invalid PSLG (no triangle inside its
 * segments -- Surface.cpp:40-41 throws -- crossing or duplicate input,
 * indices out of range), FEA_ERR_TOO_LARGE when refinement would exceed its
 * vertex budget. */
typedef struct fea_pslg_mesh fea_pslg_mesh;
int fea_triangulate_pslg(const double* points, int64_t num_points, const int32_t* segments, int64_t num_segments,
                         const double* holes, int64_t num_holes, double max_area, double min_angle_deg,
                         fea_pslg_mesh** out);
int fea_pslg_mesh_sizes(const fea_pslg_mesh* m, int64_t* num_vertices, int64_t* num_triangles);
/* vertices: float[3V], triangles: uint32[3T], on_boundary: uint8[V] (each may be NULL) */
int fea_pslg_mesh_copy(const fea_pslg_mesh* m, float* vertices, uint32_t* triangles, uint8_t* on_boundary);
int fea_pslg_mesh_destroy(fea_pslg_mesh* m);

/* ---- misc ----------------------------------------------------------------- */
const char* fea_last_error(void);
const char* fea_version(void);

#if defined(__GNUC__)
#pragma GCC visibility pop
#endif
#ifdef __cplusplus
}
#endif
#endif /* FEA_GPU_H */
