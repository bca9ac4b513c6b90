/*
 * CPU FP64 oracle for the segregated finite-volume solid solve.
 *
 * TEST INFRASTRUCTURE ONLY.  Only the tests, the smoke check and the CPU
 * baseline leg of the benchmark may load this library; the product never
 * links or calls it.
 *
 * It restates, in plain C++, the arithmetic of solids4foam's
 * linearGeometryTotalDisplacement and nonLinearGeometryTotalLagrangian
 * outer-corrector loops together with the OpenFOAM finite-volume operators
 * they call (Gauss linear corrected laplacian, Gauss linear divergence,
 * leastSquares gradient, PCG with DIC).  Parity against a real OpenFOAM run is
 * unpinned: OpenFOAM is not available, so the OpenFOAM operators are written
 * from the published finite-volume formulation.  The solids4foam-side
 * algorithms follow the cited reference files line by line.
 */
#ifndef S4G_ORACLE_H
#define S4G_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  int n_cells;
  int n_faces;           /* internal + boundary */
  int n_internal_faces;
  const int* owner;      /* [n_faces] */
  const int* neighbour;  /* [n_internal_faces] */
  const double* C;       /* [n_cells][3] */
  const double* V;       /* [n_cells] */
  const double* Cf;      /* [n_faces][3] */
  const double* Sf;      /* [n_faces][3] */
  int n_patches;
  const int* patch_start;
  const int* patch_size;
} orc_mesh_desc;

enum { ORC_FIXED_DISPLACEMENT = 0, ORC_SOLID_TRACTION = 1 };
enum { ORC_LINEAR_ELASTIC = 0, ORC_NEO_HOOKEAN = 1 };
enum { ORC_LIN_GEOM_TOTAL_DISP = 0, ORC_NONLIN_GEOM_TOTAL_LAG = 1,
       ORC_NONLIN_GEOM_TOTAL_LAG_TOTAL_DISP = 2 };
enum { ORC_DIC = 0, ORC_DIAGONAL = 1 };

typedef struct {
  int type;               /* ORC_FIXED_DISPLACEMENT or ORC_SOLID_TRACTION */
  const double* value;    /* [size][3]: total displacement or traction; NULL = 0 */
  const double* pressure; /* [size]: traction patches only; NULL = 0 */
  double relaxation_factor; /* traction patches: relaxationFactor of the
                               traction gradient; 0 means 1, the reference's
                               default (solidTractionFvPatchVectorField.C:82) */
} orc_bc;

typedef struct {
  int model;              /* ORC_LIN_GEOM_TOTAL_DISP / ORC_NONLIN_GEOM_TOTAL_LAG /
                             ORC_NONLIN_GEOM_TOTAL_LAG_TOTAL_DISP */
  int law;                /* ORC_LINEAR_ELASTIC / ORC_NEO_HOOKEAN */
  double E, nu;           /* used when use_mu_K == 0 */
  double mu, K;           /* used when use_mu_K == 1 */
  int use_mu_K;
  int preconditioner;     /* ORC_DIC / ORC_DIAGONAL */
  double tolerance, rel_tol;
  int max_iter;
  int n_correctors;
  double solution_tol, alternative_tol, material_tol;
  double stab_scale;      /* RhieChow scaleFactor */
  int ls_boundary_delta;  /* 0: patch-normal d (OpenFOAM.com/.org), 1: d = Cf - C */
  int n_increments;       /* load increments (time steps), loads ramp linearly */
  int n_threads;          /* >1: OpenMP, DIC restricted to thread subdomains */
  int max_correctors_run; /* >0: stop after this many correctors (timing samples) */
  const int* dic_domain;  /* optional [n_cells] subdomain of each cell (caller
                             order): DIC restricted to each subdomain */
  double max_seconds;     /* >0: stop after the corrector that passes this wall
                             time (bounded timing samples) */
  int empty_direction;    /* 2-D cases (empty patches, whose faces the caller
                             leaves out of the mesh): 1, 2 or 3 for x, y or z;
                             0: 3-D.  The leastSquares tensor is inverted with
                             OpenFOAM's treatment of the empty direction and
                             that displacement component is not solved */
  double field_relaxation; /* fvSolution relaxationFactors { fields { "D|DD" f; } }:
                             after each solve D == D.prevIter + f (D - D.prevIter),
                             cells and boundary faces (solidModel.C:837-841,
                             GeometricField::relax); 0 or 1: none */
  int relaxation_method;  /* 0 "fixed" (field_relaxation above); 1 "Aitken"
                             (solidModel.C:842-896): a per-cell (and per
                             boundary face) factor alpha, field_relaxation
                             (or 1) at the first corrector of each
                             increment */
} orc_settings;

typedef struct {
  int n_correctors;       /* total over all increments */
  int converged;          /* last increment converged */
  long long total_lin_iters;
  double initial_residual;/* last corrector: mag of the 3 initial residuals */
  double rel_residual;    /* last corrector: relative displacement residual */
  double seconds;         /* wall time of the solve loop */
  int enforce_linear;     /* TL: linear geometry was enforced */
  int nan_detected;       /* a corrector produced a non-finite D: the solve
                             stopped there, unconverged (the library's
                             S4G_NAN_DETECTED) */
} orc_perf;

void orc_default_settings(orc_settings* s);

/*
 * Full solve.  `perm` (optional, [n_cells]) renumbers the mesh before the
 * solve: new cell i is old cell perm[i], as OpenFOAM's renumberMesh would;
 * faces are re-sorted upper-triangular.  Outputs are in the caller's
 * (un-permuted) cell order.  D_out [n_cells][3], sigma_out [n_cells][6]
 * (XX XY XZ YY YZ ZZ), gradD_out [n_cells][9] may be NULL.
 * Returns 0 on success, nonzero on bad input.
 */
int orc_solve(const orc_mesh_desc* mesh, const orc_bc* bcs,
              const orc_settings* s, const int* perm, double* D_out,
              double* sigma_out, double* gradD_out, orc_perf* perf);

/* ---- operator-level entry points, for kernel-by-kernel parity tests ---- */

/* Scalar LDU matrix of the implicit laplacian (negated to SPD form): diag
 * [n_cells] (with fixedDisplacement boundary diagonal) and upper
 * [n_internal_faces], with impK = 2mu+lambda from (E, nu). */
int orc_assemble_matrix(const orc_mesh_desc* mesh, const orc_bc* bcs,
                        double impK, double* diag, double* upper);

/* y = A x for the LDU matrix above (face-order accumulation). */
int orc_amul(const orc_mesh_desc* mesh, const double* diag,
             const double* upper, const double* x, double* y);

/* DIC preconditioner w = M^-1 r (OpenFOAM face order). */
int orc_dic_precondition(const orc_mesh_desc* mesh, const double* diag,
                         const double* upper, const double* r, double* w);

/* leastSquares gradient of a cell vector field with boundary values Db
 * [n_boundary_faces][3] and boundary snGrad [n_boundary_faces][3]:
 * cell gradient G [n_cells][9] and corrected boundary gradient Gb. */
int orc_ls_grad(const orc_mesh_desc* mesh, int ls_boundary_delta,
                const double* D, const double* Db, const double* snGradB,
                double* G, double* Gb);

#ifdef __cplusplus
}
#endif

#endif
