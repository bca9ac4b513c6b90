/*
 * s4g.h -- C ABI of the GB300 segregated finite-volume solid solver.
 *
 * The library replaces, for one mesh region, the outer-corrector loop of
 * solids4foam's linearGeometryTotalDisplacement and
 * nonLinearGeometryTotalLagrangian solid models together with the OpenFOAM
 * finite-volume operators and the PCG/DIC linear solver they call.  Every
 * entry point is plain C: pointers, sizes and status codes, no exceptions,
 * no C++ or torch types.  Each declaration names the reference interface it
 * stands in for (paths relative to the solids4foam source tree).
 *
 * Ownership: the caller owns every host array it passes; the library copies
 * what it needs during the call and never keeps the pointer.  The library
 * owns all device memory of a context and frees it in the *_destroy calls.
 * Output arrays are caller-allocated and use the caller's cell order (the
 * library undoes its internal renumbering).
 *
 * Threading: a context is used by one host thread at a time.
 */
#ifndef S4G_H
#define S4G_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define S4G_ABI_VERSION 7

/* Status codes.  Reference convention for errors is FatalError (abort), see
 * src/solids4FoamModels/solidModels/solidModel/solidModel.C:1735-1742; a
 * drop-in maps every code but S4G_NOT_CONVERGED to FatalErrorIn, and
 * S4G_NOT_CONVERGED to the "Max iterations reached within momentum loop"
 * warning of solidModelTemplates.C:180-185 (the result is still returned). */
typedef enum s4g_status {
  S4G_OK = 0,
  S4G_BAD_ARG = 1,            /* invalid argument or inconsistent mesh */
  S4G_OOM = 2,                /* device allocation failed */
  S4G_NOT_CONVERGED = 3,      /* nCorrectors reached; results returned */
  S4G_NAN_DETECTED = 4,       /* non-finite value in the iteration */
  S4G_INDEFINITE = 5,         /* PCG found p.Ap <= 0 */
  S4G_TIMEOUT = 6,            /* a bounded device wait gave up */
  S4G_CUDA_ERROR = 7,         /* CUDA runtime error */
  S4G_NO_DEVICE = 8,          /* no CUDA device */
  S4G_ADMISSION_REJECTED = 9, /* server: footprint can never fit */
  S4G_PENDING = 10,           /* server: request not finished yet */
  S4G_CANCELLED = 11,         /* server: request was cancelled */
  S4G_NOT_BUILT = 12          /* feature not compiled into this library */
} s4g_status;

/* Human-readable name of a status code (never NULL). */
const char* s4g_status_str(s4g_status st);

/* ABI version of the loaded library (S4G_ABI_VERSION at build time). */
int s4g_abi_version(void);

/* Message of the last failing call on this host thread ("" if none). */
const char* s4g_last_error(void);

/* ------------------------------------------------------------ context -- */

typedef struct s4g_ctx s4g_ctx;

typedef struct s4g_ctx_opts {
  int device;   /* CUDA device ordinal */
  int verbose;  /* 1: print the reference's residual table every
                   infoFrequency correctors */
  int profile;  /* 1: time every kernel kind with CUDA events on the
                   library's stream (s4g_perf.kernel_ms / kernel_launches_by);
                   PCG batches are then launched kernel by kernel */
  int no_graphs; /* 1: launch PCG batches kernel by kernel instead of
                   replaying captured CUDA graphs (same results) */
  int spin_limit; /* polls a bounded device wait (the exact-DIC sweeps'
                   wait for the parts they depend on) makes before it gives
                   up: the kernel then sets an error bit, returns, and the
                   call reports S4G_TIMEOUT with the context still usable.
                   0: the default, 4,194,304 (seconds of waiting) */
} s4g_ctx_opts;

/* Kernel kinds of the per-kernel timers. */
enum {
  S4G_K_RHS = 0,       /* right-hand side: div(sigma), Rhie-Chow, BC terms */
  S4G_K_POST = 1,      /* post-solve: gradient, law, boundary, convergence */
  S4G_K_SWEEP_FWD = 2, /* DIC forward substitution */
  S4G_K_SWEEP_BWD = 3, /* DIC backward substitution */
  S4G_K_DIAG = 4,      /* diagonal preconditioner */
  S4G_K_PUPDATE = 5,   /* p = w + beta p */
  S4G_K_SPMV = 6,      /* q = A p */
  S4G_K_UPDATE = 7,    /* x, r update and residual */
  S4G_K_LOC_PRECOND = 8, /* fused x, r update + processor-local DIC (both sweeps) */
  S4G_K_LOC_SPMV = 9,  /* fused p = w + beta p and q = A p */
  S4G_K_KINDS = 10
};

/* Creates a context on one GPU.  Stands in for the per-run state the
 * reference keeps in the OpenFOAM Time/objectRegistry
 * (applications/solvers/solids4Foam/solids4Foam.C:36-43). */
s4g_status s4g_ctx_create(s4g_ctx** out, const s4g_ctx_opts* opts);
s4g_status s4g_ctx_destroy(s4g_ctx* ctx);

/* --------------------------------------------------------------- mesh -- */

/* An OpenFOAM fvMesh in its primitive form: upper-triangular internal faces
 * first (owner < neighbour, area vector owner -> neighbour), then boundary
 * faces grouped by patch, area vectors pointing out of the domain. */
typedef struct s4g_mesh_desc {
  int n_cells;
  int n_faces;            /* internal + boundary */
  int n_internal_faces;
  const int* owner;       /* [n_faces] */
  const int* neighbour;   /* [n_internal_faces] */
  const double* C;        /* [n_cells][3] cell centres */
  const double* V;        /* [n_cells] cell volumes */
  const double* Cf;       /* [n_faces][3] face centres */
  const double* Sf;       /* [n_faces][3] face area vectors */
  int n_patches;
  const int* patch_start; /* [n_patches] first face of each patch */
  const int* patch_size;  /* [n_patches] */
} s4g_mesh_desc;

/* Cell numbering used by the DIC preconditioner.  DIC depends on the cell
 * order exactly as OpenFOAM's does; every choice is an exact DIC of the
 * renumbered matrix (as after OpenFOAM's renumberMesh). */
typedef enum s4g_renumber {
  S4G_RENUMBER_NONE = 0,  /* the caller's numbering */
  S4G_RENUMBER_RCM = 1,   /* reverse Cuthill-McKee */
  S4G_RENUMBER_TILED = 2  /* coordinate-bisection parts, part-major order */
} s4g_renumber;

typedef struct s4g_mesh_opts {
  s4g_renumber renumber;
  int part_size;          /* rows per scheduling part (0: default 512) */
  int ls_boundary_delta;  /* leastSquares boundary d: 0 patch-normal
                             n(n.(Cf-C)) (OpenFOAM.com/.org fvPatch::delta),
                             1 full Cf-C (foam-extend) */
  int dic_subdomains;     /* 0: exact global DIC; 1: DIC restricted to each
                             part (processor-local DIC of a decomposed run) */
  int no_autotune;        /* 1: skip the kernel-variant autotuner of the
                             processor-local PCG (results are identical
                             either way; only the speed differs) */
  int empty_direction;    /* 2-D cases: 1, 2 or 3 for an x, y or z empty
                             direction, whose empty patches' faces the caller
                             leaves out of the mesh description (they have no
                             faces in OpenFOAM's discretisation either).  The
                             leastSquares tensor is inverted as OpenFOAM's
                             inv() does with an empty direction, and that
                             displacement component is not solved (plane
                             strain).  0: 3-D. */
  const int* part_of_cell; /* optional [n_cells]: the caller's decomposition
                             of the cells into DIC subdomains (the
                             counterpart of decomposePar's cellDecomposition),
                             subdomain ids 0..n-1, every id used; a
                             subdomain must fit the preconditioner kernel's
                             shared memory (about 2,000 cells).  Needs
                             renumber = S4G_RENUMBER_NONE and
                             dic_subdomains = 1: each subdomain's DIC then
                             runs in the caller's cell order, as a decomposed
                             run's processor does.  NULL: the library's
                             parts.  Read during s4g_mesh_upload only. */
} s4g_mesh_opts;

typedef struct s4g_mesh s4g_mesh;

typedef struct s4g_mesh_info {
  int n_cells, n_internal_faces, n_boundary_faces;
  int n_parts;            /* scheduling parts */
  int part_depth;         /* longest chain of dependent parts (DIC sweep) */
  int max_local_levels;   /* deepest in-part level count */
  int n_levels_global;    /* level count of the whole lower-triangular DAG */
  long long device_bytes; /* device memory held by this mesh */
  long long n_local_entries; /* processor-local DIC table entries (with padding);
                                0 unless dic_subdomains */
  int local_slots;        /* 1: the processor-local tables have fixed 3 + 3 slots per
                             row (every row has at most three lower and three upper
                             in-part neighbours); 0: generic tables */
} s4g_mesh_info;

/* Uploads the mesh once: validation, renumbering, cell-to-face CSR in the
 * solver order, then derived geometry on the device (weights, deltaCoeffs,
 * nonOrthDeltaCoeffs, nonOrthCorrectionVectors, patch correction vectors,
 * leastSquares tensors).  Stands in for the lazily built OpenFOAM fvMesh
 * geometry used by solidModel (solidModel.C:954-1330) and
 * patchCorrectionVectors.C:24-36. */
s4g_status s4g_mesh_upload(s4g_ctx* ctx, const s4g_mesh_desc* desc,
                           const s4g_mesh_opts* opts, s4g_mesh** out);
/* Host-only planning (no GPU needed): the DIC order and scheduling figures
 * s4g_mesh_upload would use.  perm_out [n_cells] (may be NULL): perm[i] =
 * caller cell of solver cell i; a caller can renumber its own mesh with it
 * (OpenFOAM renumberMesh) to run the identical DIC on the CPU. */
s4g_status s4g_mesh_plan(const s4g_mesh_desc* desc, const s4g_mesh_opts* opts,
                         int* perm_out, s4g_mesh_info* info);
/* perm[i] = caller cell of solver cell i (the DIC order). */
s4g_status s4g_mesh_get_permutation(const s4g_mesh* mesh, int* perm);
/* part_of_cell [n_cells] (caller order): the scheduling part of each cell;
 * with dic_subdomains these are the DIC subdomains (the counterpart of a
 * decomposePar cell decomposition). */
s4g_status s4g_mesh_get_parts(const s4g_mesh* mesh, int* part_of_cell);
s4g_status s4g_mesh_get_info(const s4g_mesh* mesh, s4g_mesh_info* info);
s4g_status s4g_mesh_destroy(s4g_mesh* mesh);

/* ----------------------------------------------------------- material -- */

typedef enum s4g_law_type {
  S4G_LINEAR_ELASTIC = 0,  /* materialModels/.../linearElastic/linearElastic.C */
  S4G_NEO_HOOKEAN = 1      /* .../neoHookeanElastic/neoHookeanElastic.C */
} s4g_law_type;

typedef struct s4g_law {
  s4g_law_type type;
  int use_mu_K;     /* 0: E, nu given; 1: mu, K given */
  double E, nu;
  double mu, K;
  double rho;       /* unused by the steady solve; kept for the drop-in */
} s4g_law;

/* One mechanical law for the whole mesh (mechanicalModel with a single law
 * forwards to laws[0]: mechanicalModel.C:476-498,571-582). */
s4g_status s4g_material_set(s4g_mesh* mesh, const s4g_law* law);

/* ---------------------------------------------------------------- BCs -- */

typedef enum s4g_bc_type {
  S4G_FIXED_DISPLACEMENT = 0, /* fixedDisplacementFvPatchVectorField.C:258-356 */
  S4G_SOLID_TRACTION = 1      /* solidTractionFvPatchVectorField.C:321-463 */
} s4g_bc_type;

/* vec3 [patch_size][3]: total displacement (fixedDisplacement) or traction
 * (solidTraction); NULL means zero.  pressure [patch_size] (solidTraction
 * only), NULL means zero.  Loads of the nonLinearGeometryTotalLagrangian
 * model ramp linearly over the load increments, as a tractionSeries /
 * pressureSeries table from zero would. */
s4g_status s4g_bc_set(s4g_mesh* mesh, int patch, s4g_bc_type type,
                      const double* vec3, const double* pressure);

/* relaxationFactor of a solidTraction patch (solidTractionFvPatchVectorField.C:82,
 * 387-392): each update of the traction gradient becomes
 * g = factor * g_new + (1 - factor) * g.  factor in (0, 1]; 1 (the default)
 * is no relaxation.  Kept across s4g_bc_set calls; ignored on
 * fixedDisplacement patches. */
s4g_status s4g_bc_set_relaxation(s4g_mesh* mesh, int patch, double factor);

/* ------------------------------------------------------------- solver -- */

typedef enum s4g_precond {
  S4G_PRECOND_DIC = 0,      /* OpenFOAM DIC / FDIC */
  S4G_PRECOND_DIAGONAL = 1  /* OpenFOAM diagonal */
} s4g_precond;

/* fvSolution solvers { "D|DD" { solver PCG; preconditioner; tolerance;
 * relTol; maxIter; } } */
typedef struct s4g_lin_solver {
  s4g_precond preconditioner;
  double tolerance;
  double rel_tol;
  int max_iter;
} s4g_lin_solver;

/* solidProperties <model>Coeffs (solidModel.C:1138-1243,1307-1323). */
typedef struct s4g_outer {
  int n_correctors;        /* nCorrectors */
  double solution_tol;     /* solutionTolerance */
  double alternative_tol;  /* alternativeTolerance */
  double material_tol;     /* materialTolerance */
  double stab_scale;       /* stabilisation { type RhieChow; scaleFactor; } */
  int info_frequency;      /* infoFrequency */
  double field_relaxation; /* fvSolution relaxationFactors { fields { D (DD for
                              the incremental TL model) f; } }: after each
                              solve D == D.prevIter + f (D - D.prevIter) on
                              the cells and the boundary faces (relaxField
                              "fixed", solidModel.C:837-841); f in (0, 1],
                              0 or 1: no relaxation */
  int relaxation_method;   /* <model>Coeffs relaxationMethod: 0 fixed, 1
                              Aitken (solidModel.C:842-896): a factor per
                              cell and boundary face, field_relaxation (or 1)
                              at each increment's first corrector, then
                              alpha (r_prev . dr) / (|dr|^2 + SMALL) bounded
                              to [0, 2], r = D.prevIter - D; D -= alpha r */
} s4g_outer;

typedef enum s4g_precision {
  S4G_FP64 = 0,           /* everything in FP64 */
  S4G_FP32_REFINE = 1     /* PCG/SpMV in FP32 with compensated dots; the
                             outer correctors refine in FP64 */
} s4g_precision;

s4g_status s4g_solver_set(s4g_mesh* mesh, const s4g_lin_solver* lin,
                          const s4g_outer* outer, s4g_precision precision);

/* Fills the reference defaults: PCG+DIC tol 1e-9 relTol 0.1 maxIter 1000;
 * nCorrectors 10000, solutionTolerance 1e-6, alternativeTolerance 1e-7,
 * materialTolerance 1e-5, RhieChow 0.1, infoFrequency 100, no field
 * relaxation (1), relaxationMethod fixed. */
void s4g_default_controls(s4g_lin_solver* lin, s4g_outer* outer);

/* -------------------------------------------------------------- solve -- */

typedef enum s4g_model {
  S4G_LIN_GEOM_TOTAL_DISP = 0,   /* linGeomTotalDispSolid.C:111-232 */
  S4G_NONLIN_GEOM_TOTAL_LAG = 1, /* nonLinGeomTotalLagSolid.C:125-260 */
  S4G_NONLIN_GEOM_TOTAL_LAG_TOTAL_DISP = 2 /* nonLinGeomTotalLagTotalDispSolid.C:173-328 */
} s4g_model;

typedef struct s4g_perf {
  int n_correctors;           /* outer correctors run (all increments) */
  int converged;              /* last increment converged */
  long long total_lin_iters;  /* PCG iterations summed over components */
  int last_max_lin_iters;     /* cmptMax(nIterations) of the last corrector */
  double initial_residual;    /* mag(initialResidual) of the last corrector */
  double rel_residual;        /* relative displacement residual, last */
  double solve_ms;            /* device time of the solve (CUDA events) */
  double h2d_ms, d2h_ms;      /* copies inside s4g_solve */
  long long kernel_launches;  /* kernels launched by the library */
  int enforce_linear;         /* TL: linear geometry was enforced */
  int device_status;          /* raw device status word (0 = clean) */
  int part_threads;           /* processor-local PCG: threads per part of the
                                 preconditioner kernel in use (autotuned) */
  int spmv_unroll;            /* processor-local PCG: SpMV form in use: entries
                                 unrolled in the fused p-update + SpMV (1 or
                                 6), or 0 for the split form */
  double tune_us[6];          /* autotuner timings (us): the two
                                 preconditioner variants, then the SpMV
                                 step plain/unrolled/split; the rest 0 */
  /* per kernel kind (S4G_K_*), only with s4g_ctx_opts.profile: summed
   * CUDA-event time and number of launches that did work */
  double kernel_ms[S4G_K_KINDS];
  long long kernel_launches_by[S4G_K_KINDS];
  int device_loop;            /* 1: the corrector loop ran device-resident (one
                                 CUDA graph launch per increment, its loops
                                 decided on the device); 0: driven from the host
                                 (profile, verbose or no_graphs) */
} s4g_perf;

/* Runs the solid model's evolve() for n_increments load increments (1 for
 * the linear model) on the device: every corrector, PCG iteration and
 * convergence test stays on the GPU; only the final fields come back.
 * D_out [n_cells][3]; sigma_out [n_cells][6] (XX XY XZ YY YZ ZZ); either may
 * be NULL.  Replaces solidModel::evolve (solidModel.H:759) of the
 * models named above, with tractionBoundarySnGrad evaluated on the device. */
s4g_status s4g_solve(s4g_mesh* mesh, s4g_model model, int n_increments,
                     double* D_out, double* sigma_out, s4g_perf* perf);

/* One time step: the solid model's evolve() as solids4Foam's time loop calls
 * it once per step (applications/solvers/solids4Foam/solids4Foam.C:58 ->
 * solidModel::evolve, solidModel.H:759), with the boundary values last set
 * by s4g_bc_set taken as they are (load factor 1: the caller evaluates its
 * load series, e.g. tractionSeries, at the step's time).  The step starts
 * from the state the previous step of the same model left on the device:
 * the linear model takes that step's D as D.oldTime; the total Lagrangian
 * forms continue from their shifted old-time fields.  The first step, a step
 * after s4g_state_reset, s4g_solve, s4g_solve_cases or s4g_solve_batch, or a
 * step of another model starts from zero.  A sequence of steps with boundary
 * values (n/N) b equals s4g_solve with N increments.  perf counts this
 * step's correctors and PCG iterations. */
s4g_status s4g_solve_step(s4g_mesh* mesh, s4g_model model, double* D_out, double* sigma_out,
                          s4g_perf* perf);
/* Forget the state s4g_solve_step continues from: the next step starts from
 * zero. */
s4g_status s4g_state_reset(s4g_mesh* mesh);

/* Batched load cases: n_cases independent solves of the
 * linearGeometryTotalDisplacement model on this mesh, advanced together with
 * every kernel launched once for all cases still running.  Replaces running
 * solidModel::evolve (linGeomTotalDispSolid.C:111-232) once per load case.
 * The cases share the mesh, the material, the solver controls and the
 * boundary-condition types set by s4g_bc_set; each case has its own
 * boundary values: bval [n_cases][n_boundary_faces][3] (fixedDisplacement:
 * displacement; solidTraction: traction) and bpress
 * [n_cases][n_boundary_faces] (solidTraction pressure, may be NULL), in the
 * caller's boundary-face order (faces n_internal_faces .. n_faces-1).  Each
 * case converges on its own, and its result is bit-identical to s4g_solve
 * with its boundary values.  Requires dic_subdomains = 1 and the DIC
 * preconditioner.  D_out [n_cases][n_cells][3], sigma_out
 * [n_cases][n_cells][6], perf [n_cases]; any may be NULL.  Returns
 * S4G_NOT_CONVERGED if any case did not converge. */
s4g_status s4g_solve_cases(s4g_mesh* mesh, int n_cases, const double* bval,
                           const double* bpress, double* D_out,
                           double* sigma_out, s4g_perf* perf);

/* Many meshes in one launch: the linearGeometryTotalDisplacement solve of
 * each mesh, with its own material, boundary conditions, controls and
 * precision as set on it, all advanced by one CUDA-graph launch in which
 * every mesh's device-resident corrector loop is an independent branch.
 * Replaces running solidModel::evolve (linGeomTotalDispSolid.C:111-232)
 * once per case, one case after another (applications/solvers/solids4Foam/
 * solids4Foam.C:36-81 runs one case per process).  Each mesh's result is
 * bit-identical to its s4g_solve.  The meshes belong to one context, which
 * must not set profile, verbose or no_graphs.  D_out[i] [n_cells_i][3],
 * sigma_out[i] [n_cells_i][6] (either array, or an entry, may be NULL),
 * perf [n_meshes] (solve_ms: the whole launch) may be NULL.  Returns
 * S4G_NOT_CONVERGED if a mesh did not converge, another status if one
 * failed. */
s4g_status s4g_solve_batch(s4g_mesh* const* meshes, int n_meshes, double* const* D_out,
                           double* const* sigma_out, s4g_perf* perf);

/* The mesh's points for the device step after the loop: points
 * [n_points][3] and the cells of every point as s4g_point_cells returns
 * them (caller cell ids; point_cell_start [n_points + 1]).  Copied once. */
s4g_status s4g_mesh_set_points(s4g_mesh* mesh, int n_points, const double* points,
                               const int* point_cell_start, const int* point_cells);
/* pointD [n_points][3] of the last solve, computed on the device from the D
 * and gradD the solve left there (total D and gradD for the total
 * Lagrangian models), as mechanical().interpolate(D, gradD, pointD) does
 * after each evolve() (linGeomTotalDispSolid.C:212, mechanicalModel.C:
 * 829-841, enhancedVolPointInterpolate.C:351-423); bit-identical to
 * s4g_point_interpolate on the same fields. */
s4g_status s4g_get_pointD(s4g_mesh* mesh, double* pointD_out);

/* Cell gradient of D from the last solve, [n_cells][9] row-major,
 * grad(D)_ij = dD_j/dx_i (the reference's gradD field). */
s4g_status s4g_get_gradD(s4g_mesh* mesh, double* gradD_out);

/* -------------------------------------------- operator-level entry points
 * For kernel-by-kernel parity checks.  Vectors are in the caller's cell
 * order, k columns stored row-interleaved [n_cells][k], k in 1..3. */

/* Scalar momentum matrix (fvm::laplacian(impKf, D) negated to SPD form),
 * diag [n_cells] and upper [n_internal_faces] in the caller's face order.
 * Requires material and BCs. */
s4g_status s4g_op_matrix(s4g_mesh* mesh, double* diag, double* upper);
/* y = A x. */
s4g_status s4g_op_amul(s4g_mesh* mesh, int k, const double* x, double* y);
/* w = DIC^-1 r (or diagonal). */
s4g_status s4g_op_precondition(s4g_mesh* mesh, int k, const double* r,
                               double* w);

/* y = A x and, per column j, xAx[j] = sum_i x_ij (A x)_ij; x, y [n_cells][k]
 * in the caller's cell order, xAx [k]; k in 1..3.  No counterpart in the
 * reference: an operator product for callers that must not allocate (a
 * server that has given the free device memory to admitted solves, a
 * latency-bound loop that must stay out of the CUDA allocator).  It
 * allocates nothing: it works in the mesh's work vectors and in one fixed
 * scratch block of static device memory.  Limits: meshes of at most 262,144
 * cells (larger ones get S4G_BAD_ARG); the matrix must already be assembled
 * (s4g_op_matrix or s4g_solve ran on this mesh); the scratch is shared by
 * every mesh on the device, so calls that overlap in time on one device
 * race and must be ordered by the caller; the first call on a device does a
 * one-time set-up (a symbol-address lookup) and belongs before any stream
 * capture; the looked-up address is kept for the process, so the entry
 * point must not be used after a cudaDeviceReset (or any destruction of the
 * device's primary context) in the same process. */
s4g_status s4g_op_amul_dot_noalloc(s4g_mesh* mesh, int k, const double* x,
                                   double* y, double* xAx);

/* ----------------------------------------------------------- serving --
 * Continuous admission of solves of uneven sizes onto one GPU.  No single
 * counterpart in the reference (one solids4Foam run is one solve); it
 * replaces running many solids4Foam cases one after another.  The server's
 * worker slots each own a context (a CUDA stream) and run one request at a
 * time; a free slot takes the first queued request whose device footprint
 * fits in the memory budget that running requests leave, so requests that
 * arrive while others run are admitted as slots and memory free up, and
 * their work overlaps on the device.  Each request computes exactly what a
 * lone s4g_solve of its inputs computes.  All s4g_server_* calls may be made
 * from any host thread. */
typedef struct s4g_server s4g_server;

typedef struct s4g_server_opts {
  int device;
  int max_slots;              /* requests running at once (0: 8; at most 64) */
  long long memory_budget;    /* device bytes running requests may hold
                                 (0: 80% of the free memory at creation) */
  int dry_run;                /* 1: no GPU work; a request "runs" for
                                 dry_run_us_per_kcell us per 1000 cells and
                                 returns zero fields (scheduler tests) */
  double dry_run_us_per_kcell;
} s4g_server_opts;

/* One solve: the mesh, its upload options, the law, boundary conditions
 * (n_bc patches: index, type, vec3 [patch_size][3] or NULL, pressure
 * [patch_size] or NULL), controls and the model.  Everything is copied at
 * submit. */
typedef struct s4g_request {
  const s4g_mesh_desc* mesh;
  s4g_mesh_opts mesh_opts;
  s4g_law law;
  int n_bc;
  const int* bc_patch;
  const s4g_bc_type* bc_type;
  const double* const* bc_vec3;
  const double* const* bc_pressure;
  s4g_lin_solver lin;
  s4g_outer outer;
  s4g_precision precision;
  s4g_model model;
  int n_increments;
  const double* bc_relaxation; /* [n_bc] relaxationFactor of each solidTraction
                                  patch (s4g_bc_set_relaxation), or NULL: 1 */
} s4g_request;

typedef struct s4g_server_stats {
  long long submitted, completed, rejected, cancelled;
  int running, queued;
  long long bytes_in_use, memory_budget;  /* estimated footprints */
  double p50_ms, p99_ms, mean_ms;         /* submit -> results ready */
  double solves_per_s;                    /* completed / (last finish - first submit) */
} s4g_server_stats;

s4g_status s4g_server_create(const s4g_server_opts* opts, s4g_server** out);
/* Queues a request; S4G_ADMISSION_REJECTED if its footprint exceeds the
 * whole budget (it could never run). */
s4g_status s4g_server_submit(s4g_server* server, const s4g_request* request,
                             uint64_t* id);
/* Result of request id: S4G_PENDING while queued or running (wait = 0), or
 * the solve's status with D_out [n_cells][3], sigma_out [n_cells][6] and
 * perf filled (each may be NULL); with wait = 1 it blocks until the request
 * ends.  A finished or cancelled request is forgotten once polled. */
s4g_status s4g_server_poll(s4g_server* server, uint64_t id, int wait,
                           double* D_out, double* sigma_out, s4g_perf* perf);
/* Removes a queued request (S4G_BAD_ARG once it runs); polling it then
 * returns S4G_CANCELLED. */
s4g_status s4g_server_cancel(s4g_server* server, uint64_t id);
s4g_status s4g_server_get_stats(s4g_server* server, s4g_server_stats* out);
/* Cancels queued requests, lets running ones finish, frees everything. */
s4g_status s4g_server_destroy(s4g_server* server);

/* ------------------------------------------------ after the solve loop --
 * Host-only steps the reference runs after evolve()'s corrector loop. */

/* The cells of every point (OpenFOAM pointCells), from the faces:
 * point_cell_start [n_points + 1]; point_cells [point_cell_start[n_points]]
 * in increasing cell order, or NULL to get the sizes only. */
s4g_status s4g_point_cells(int n_points, int n_faces, const int* face_start,
                           const int* face_points, int n_internal_faces, const int* owner,
                           const int* neighbour, int* point_cell_start, int* point_cells);
/* pointD [n_points][3] as enhancedVolPointInterpolation::interpolate(D,
 * gradD, pointD) computes it (enhancedVolPointInterpolate.C:351-423, from
 * mechanicalModel.C:829-841 after each evolve(), linGeomTotalDispSolid.C:212):
 * the inverse-distance-weighted average over the point's cells of
 * D_c + (x_p - C_c) . gradD_c.  D [n_cells][3], gradD [n_cells][9]
 * (s4g_get_gradD), C [n_cells][3] the cell centres. */
s4g_status s4g_point_interpolate(int n_points, const double* points, const int* point_cell_start,
                                 const int* point_cells, int n_cells, const double* C,
                                 const double* D, const double* gradD, double* pointD);
/* tractionBoundarySnGrad of the three models on the host, for a drop-in's
 * own override (boundary evaluations outside evolve(); inside s4g_solve the
 * same formula runs on the device): per face
 *   g = ((t - n_c p) - n_c . sigma_b + impK n . gradD_b) / impK,
 * with n_c = n for linear geometry (linGeomTotalDispSolid.C:235-271, whose
 * n . (sigma_b - impK gradD_b) is the same expression) and for an enforced
 * linear geometry, and n_c = Finv^T n / |Finv^T n| for the total Lagrangian
 * forms (nonLinGeomTotalLagSolid.C:263-325,
 * nonLinGeomTotalLagTotalDispSolid.C:284-328; gradD_b is then grad(DD) or
 * grad(D)).  traction [n][3] and pressure [n] may be NULL (zero);
 * normal [n][3]; sigma_b [n][6]; gradD_b, Finv_b [n][9] (Finv_b NULL:
 * n_c = n); g_out [n][3]. */
s4g_status s4g_traction_sngrad(int n_faces, const double* traction, const double* pressure,
                               const double* normal, const double* sigma_b, const double* gradD_b,
                               const double* Finv_b, double impK, double* g_out);
/* solidModel::writeFields (solidModel.C:1936-1962): sigmaEq [n] =
 * sqrt(3/2 |dev sigma|^2); epsilon [n][6] = symm(gradD) and epsilonEq [n]
 * = sqrt(2/3 |dev epsilon|^2) (written by the reference for the
 * linear-geometry model).  Any output may be NULL. */
s4g_status s4g_derived_fields(int n, const double* sigma, const double* gradD, double* sigmaEq,
                              double* epsilon, double* epsilonEq);

/* ---------------------------------------------------- case generation --
 * Seeded hexahedral box meshes (blockMesh + perturbMeshPoints stand-in,
 * applications/utilities/perturbMeshPoints/perturbMeshPoints.C:244-330):
 * patches xmin, xmax, ymin, ymax, zmin, zmax; interior vertices jittered by
 * up to jitter*h per axis.  Host-only helpers of the standalone driver. */
s4g_status s4g_box_mesh_sizes(int nx, int ny, int nz, int* n_cells,
                              int* n_faces, int* n_internal_faces,
                              int* n_points);
s4g_status s4g_box_mesh_build(int nx, int ny, int nz, double lx, double ly,
                              double lz, double jitter, uint64_t seed,
                              int* owner, int* neighbour, double* C, double* V,
                              double* Cf, double* Sf, int* patch_start,
                              int* patch_size, double* points);
/* Point ids of each face [n_faces][4] in the storage order of
 * s4g_box_mesh_build (right-hand rule: the area vector points out of the
 * owner), e.g. to write the box as an OpenFOAM polyMesh. */
s4g_status s4g_box_mesh_faces(int nx, int ny, int nz, int* face_points);

/* -------------------------------------------------- OpenFOAM case files --
 * Host-only reading of an OpenFOAM case's mesh and D boundary conditions
 * (ASCII format), for a caller without OpenFOAM: the reference builds the
 * same data with OpenFOAM's polyMesh/fvMesh constructors and the D
 * volVectorField's boundaryField (solidModel.C:954-1330); these entry
 * points hand the same arrays to s4g_mesh_upload and s4g_bc_set. */
typedef struct s4g_foam_case s4g_foam_case;

/* Reads <polymesh_dir>/{points,faces,owner,neighbour,boundary}: faces as a
 * faceList or a faceCompactList; any patch types.  C, V, Cf and Sf are
 * computed as OpenFOAM's primitiveMesh does: triangles directly, other
 * faces by a triangle fan about the average point; cells by pyramids about
 * the average face centre. */
s4g_status s4g_foam_read_mesh(const char* polymesh_dir, s4g_foam_case** out);
/* The mesh as an s4g_mesh_desc (pointers valid until s4g_foam_free) and
 * its number of points. */
s4g_status s4g_foam_mesh_desc(const s4g_foam_case* fc, s4g_mesh_desc* desc, int* n_points);
/* The points [n_points][3] and faces (face f has the points
 * face_points[face_start[f] .. face_start[f+1])) as read; pointers valid
 * until s4g_foam_free. */
s4g_status s4g_foam_mesh_points(const s4g_foam_case* fc, const double** points,
                                const int** face_start, const int** face_points);
/* Patch name and OpenFOAM patch type ("patch", "wall", "empty", ...), or
 * NULL for an index out of range. */
const char* s4g_foam_patch_name(const s4g_foam_case* fc, int patch);
const char* s4g_foam_patch_type(const s4g_foam_case* fc, int patch);
/* Reads the boundaryField of a D file: per patch fixedDisplacement (value,
 * or displacementSeries) or solidTraction (traction or tractionSeries,
 * pressure or pressureSeries, relaxationFactor), uniform or nonuniform;
 * series as s4g_foam_load_ramp describes.  Another type, a *Field input, a
 * missing patch or a malformed entry is S4G_BAD_ARG, named in
 * s4g_last_error. */
s4g_status s4g_foam_read_d(s4g_foam_case* fc, const char* d_file);
/* The condition read for a patch: type; vec3 [patch_size][3] (value or
 * traction); pressure [patch_size] (NULL for fixedDisplacement);
 * relaxation factor.  Pointers valid until s4g_foam_free. */
s4g_status s4g_foam_bc(const s4g_foam_case* fc, int patch, s4g_bc_type* type,
                       const double** vec3, const double** pressure,
                       double* relaxation_factor);
/* Load series read by s4g_foam_read_d: tractionSeries, pressureSeries and
 * displacementSeries (interpolationTable files of (time value) pairs,
 * linear interpolation; outOfBounds clamp, warn, error or repeat;
 * solidTraction...C:105-193,357-369, fixedDisplacement...C:174-185).
 * s4g_foam_bc returns a series' end value.  When every series is a linear
 * ramp from zero at time 0 and they end together, the load increments of
 * s4g_solve apply them (load factor n/N): end_time is that end, and
 * constant_loads is 1 if a constant nonzero load sits beside them (the
 * increments would ramp it as well).  Otherwise end_time is 0: a case with
 * other tables is stepped in time (s4g_foam_apply_bcs_at, s4g_solve_step). */
s4g_status s4g_foam_load_ramp(const s4g_foam_case* fc, double* end_time, int* constant_loads);
/* kind: 0 no load series, 1 linear ramps from zero with a common end (see
 * s4g_foam_load_ramp), 2 other tables. */
s4g_status s4g_foam_series_kind(const s4g_foam_case* fc, int* kind);
/* The condition of a patch at a time: the series evaluated at `time` as
 * the reference's boundary conditions evaluate them at the time step's time
 * (tractionSeries_(time) etc.), constant values as read.  vec3
 * [patch_size][3] (value or traction) and pressure [patch_size] are the
 * caller's buffers (either may be NULL).  A time outside a series with
 * outOfBounds error is S4G_BAD_ARG. */
s4g_status s4g_foam_bc_at(const s4g_foam_case* fc, int patch, double time, s4g_bc_type* type,
                          double* vec3, double* pressure, double* relaxation_factor);
/* s4g_bc_set and s4g_bc_set_relaxation on every patch with the conditions
 * at `time` (s4g_foam_bc_at): the boundary values of one time step. */
s4g_status s4g_foam_apply_bcs_at(const s4g_foam_case* fc, s4g_mesh* mesh, double time);
/* startTime (default 0), endTime and deltaT of a system/controlDict: the
 * time steps the reference's loop takes, which a caller maps to load
 * increments, (endTime - startTime) / deltaT. */
s4g_status s4g_foam_read_time(const char* control_dict, double* start_time, double* end_time,
                              double* delta_t);
/* The model, law and controls of a case directory, from
 * constant/solidProperties (solidModel and its <model>Coeffs, with the
 * stabilisation sub-dictionary and relaxationMethod:
 * solidModel.C:909-912,1138-1243,1305-1323), constant/mechanicalProperties
 * (one linearElastic or neoHookeanElastic law, planeStress no) and
 * system/fvSolution (the PCG solver of D, or DD for the incremental total
 * Lagrangian model, and that field's relaxationFactors field factor).
 * Entries that are not set keep the reference defaults
 * (s4g_default_controls).  Anything not built -- another model, law or
 * solver, plane stress, several laws, sigma0, predictor, solvePressureEqn --
 * is S4G_BAD_ARG, named in s4g_last_error. */
s4g_status s4g_foam_read_controls(const char* case_dir, s4g_model* model, s4g_law* law,
                                  s4g_lin_solver* lin, s4g_outer* outer);
/* relaxationFactors of a system/fvSolution for one field ("D" or "DD"):
 * field_factor from fields { } (or the older flat form), equation_factor
 * from equations { }; 1 where none is set.  Field relaxation (the
 * reference's "fixed" relaxField, D == D.prevIter + f (D - D.prevIter),
 * solidModel.C:837-841) is built: s4g_foam_read_controls puts the factor in
 * s4g_outer.field_relaxation.  Equation relaxation (fvMatrix::relax) is not
 * built on the device path, so a caller refuses a case that sets it below 1. */
s4g_status s4g_foam_read_relaxation(const char* fv_solution, const char* field,
                                    double* field_factor, double* equation_factor);
/* The leastSquares boundary delta of a system/fvSchemes for the gradient of
 * one field ("D" or "DD"): gradSchemes grad(<field>) (else default)
 * leastSquares gives 0 (OpenFOAM's patch-normal delta), extendedLeastSquares
 * <minDet> gives 1 (the full face-centre delta, as the reference's
 * cooksMembrane tutorial selects, tutorials/solids/linearElasticity/
 * cooksMembrane/system/fvSchemes) -- the value of
 * s4g_mesh_opts.ls_boundary_delta.  Other schemes are S4G_BAD_ARG. */
s4g_status s4g_foam_read_grad_scheme(const char* fv_schemes, const char* field,
                                     int* ls_boundary_delta);
/* s4g_bc_set and s4g_bc_set_relaxation on every patch of an uploaded mesh
 * (uploaded from this case's s4g_mesh_desc). */
s4g_status s4g_foam_apply_bcs(const s4g_foam_case* fc, s4g_mesh* mesh);
void s4g_foam_free(s4g_foam_case* fc);
/* Boundary values of D for writing results, Db [n_boundary_faces][3]:
 * fixedDisplacement faces take the value read from the D file; every other
 * face the cell value extrapolated with the cell gradient,
 * D_P + (C_f - C_P) . gradD_P. */
s4g_status s4g_foam_boundary_D(const s4g_foam_case* fc, const double* D, const double* gradD,
                               double* Db);
/* Writes <dir>/<name> as an ASCII volScalarField (width 1), volVectorField
 * (3) or volSymmTensorField (6, XX XY XZ YY YZ ZZ), as the reference's time
 * directories hold them: cell values [n_cells][width] and, per patch, a
 * calculated value per face from boundary_values [n_boundary_faces][width]
 * or, if that is NULL, the adjacent cell's value (empty patches: type
 * empty).  The directory's last component names the time. */
s4g_status s4g_foam_write_field(const s4g_foam_case* fc, const char* dir, const char* name,
                                int width, const char* dimensions, const double* cell_values,
                                const double* boundary_values);
/* Writes an ASCII polyMesh (points, faces, owner, neighbour, boundary) into
 * an existing directory; face f has the points
 * face_points[face_start[f] .. face_start[f+1]); patch_types (NULL, or a
 * NULL entry: "patch") names each patch's type, e.g. "empty". */
s4g_status s4g_foam_write_mesh(const char* polymesh_dir, int n_points, const double* points,
                               int n_faces, const int* face_start, const int* face_points,
                               int n_internal_faces, const int* owner, const int* neighbour,
                               int n_patches, const char* const* patch_names,
                               const int* patch_start, const int* patch_size,
                               const char* const* patch_types);
/* 2-D cases: a polyMesh with `empty` patches is read without their faces
 * (they have none in OpenFOAM's discretisation either); every s4g_foam_*
 * patch index, the s4g_mesh_desc and the faces then refer to the mesh
 * without them.  This is the empty direction (1, 2, 3: x, y, z) to pass as
 * s4g_mesh_opts.empty_direction; 0 for a 3-D mesh.  The empty patches must
 * be normal to an axis, one cell across. */
int s4g_foam_empty_direction(const s4g_foam_case* fc);
/* Writes <dir>/<name> as an ASCII pointVectorField (values [n_points][3],
 * patches calculated, empty patches empty). */
s4g_status s4g_foam_write_point_field(const s4g_foam_case* fc, const char* dir, const char* name,
                                      const char* dimensions, const double* values);

#ifdef __cplusplus
}
#endif

#endif /* S4G_H */
