/* CPU oracle for the AFEPack elliptic-solve path -- TEST INFRASTRUCTURE.
 *
 * A plain-C restatement of the reference algorithms, loop for loop and in the
 * same floating-point operation order, so that its results can be pinned
 * against AFEPack compiled from its own sources (oracle/_ref) and then used
 * as the checker for the GPU path wherever the reference tree is absent.
 * Only the tests, the smoke check and the bench's CPU-baseline leg load it;
 * the product never does.
 *
 * CSR matrices use AFEPack's SparsityPattern layout: int64 row starts and
 * column numbers, and for square matrices the diagonal entry first in every
 * row followed by the other columns in ascending order
 * (include/AFEPack/SparsityPattern.h:76-126,193-237).
 */
#ifndef AFP_ORACLE_H
#define AFP_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  int64_t m, n;
  int64_t *rowptr; /* m+1 */
  int64_t *cols;   /* rowptr[m] */
  double *vals;    /* rowptr[m] */
} orc_csr;

void orc_csr_free(orc_csr *a);

/* StiffMatrix/MassMatrix::build (BilinearOperator.templates.h:56-255) for
 * Lagrange P1/P2 on triangles (dim 2) or tetrahedra (dim 3).
 * coords [n_vertex*dim], cells [n_cell*(dim+1)], elem_dof [n_cell*nd].
 * The stiffness element matrix is multiplied by coef[e] when coef != NULL.
 * Both matrices share one pattern: mass_vals receives the mass values in the
 * stiffness pattern's order (pass NULL to skip).  Returns 0 on success. */
/* quadrature points [n_cell*nq*dim] of the rule of accuracy acc; returns nq
 * (points may be NULL) or -1 */
int orc_quadrature_points(int dim, const double *coords, int64_t n_cell, const int64_t *cells, int acc,
                          double *points);
/* Operator::L2Discretize of point values fq [n_cell*nq] or of a FEM function
 * u [n_dof] (exactly one non-NULL) into f1 [n_dof] */
int orc_l2_discretize(int dim, int degree, const double *coords, int64_t n_cell, const int64_t *cells,
                      const int32_t *elem_dof, int64_t n_dof, int acc, const double *fq, const double *u,
                      double *f1);
int orc_assemble(int dim, int degree, const double *coords, int64_t n_cell,
                 const int64_t *cells, const int32_t *elem_dof, int64_t n_dof,
                 int acc_stiff, int acc_mass, const double *coef,
                 orc_csr *stiff, double *mass_vals);

/* dst = A src  (SparseMatrix::vmult, SparseMatrix.h:100-114) */
void orc_vmult(const orc_csr *a, const double *src, double *dst);

/* BoundaryConditionAdmin::apply with preserve_symmetry (FEMSpace.templates.h:1338-1366).
 * dirichlet[i] != 0 marks a Dirichlet DOF, g[i] its value (g may be NULL: zero). */
void orc_apply_dirichlet(orc_csr *a, double *f, const int32_t *dirichlet, const double *g);

/* AMG hierarchy (AMGSolver::reinit, src/AMGSolver.cpp:384-438). */
typedef struct {
  int n_level;          /* number of projections */
  int most_project_full;
  orc_csr *A;           /* n_level+1 matrices; A[0] is a copy of the input */
  orc_csr *P;           /* n_level projections (n_coarse x n_fine) */
  int64_t n_coarse;     /* order of the coarsest matrix */
  double *coarse_inv;   /* explicit inverse of A[n_level], row-major */
  int smooth_step;
  double alpha;
  orc_csr *Pt;          /* lazy hierarchy only: lazyProject's own P^T per level */
} orc_amg;

/* lazyProject (src/AMGSolver.cpp:235-284) */
int orc_lazy_project(const orc_csr *m, orc_csr *p, orc_csr *pt);
/* lazyInit (src/AMGSolver.cpp:442-503) */
int orc_amg_setup_lazy(const orc_csr *a, int smooth_step, int64_t max_coarse, double min_density, orc_amg *out);
/* lazyReinit on an initialised lazy hierarchy (src/AMGSolver.cpp:505-545):
 * recomputes every level from a (same pattern) with the stored P, Pt. */
int orc_amg_lazy_reinit(orc_amg *h, const orc_csr *a);

int orc_amg_setup(const orc_csr *a, int smooth_step, int64_t max_coarse, double min_density,
                  double alpha, orc_amg *out);
/* A hierarchy from given level matrices A[0..n_level] and projections
 * P[0..n_level-1] (copied); the coarsest inverse is computed here when
 * most_project_full.  Used to time the reference's solve phase on a
 * hierarchy that was built (and checked equal to the reference's) elsewhere. */
int orc_amg_from_levels(int n_level, const orc_csr *A, const orc_csr *P, int most_project_full,
                        int smooth_step, orc_amg *out);
/* Replaces the coarsest inverse of a hierarchy with a given row-major
 * n_coarse x n_coarse array (copied), for coarsest levels too large for the
 * single-threaded inverse above to be practical. */
int orc_amg_set_coarse_inverse(orc_amg *h, const double *inv);
void orc_amg_free(orc_amg *h);
/* Project() alone: C/F split and projection P for one level.
 * cf_out[i] = -1 for C-points, 1 for F-points (may be NULL). */
int orc_project(const orc_csr *m, double alpha, orc_csr *p, int32_t *cf_out);
/* getPMPt: A_c = P M P^T with the reference's pattern and accumulation order. */
int orc_rap(const orc_csr *p, const orc_csr *m, orc_csr *out);

/* AMGSolver::solve(x, r, 0, cycles-1, mode): runs `cycles` V-cycles from x. */
void orc_amg_vcycles(const orc_amg *h, double *x, const double *r, int cycles);

/* Example-style CG preconditioned by one V-cycle per iteration
 * (examples/FAST/src/poisson_solver_comparison_afepack.cpp:197-253).
 * Returns the iteration count; *relres receives ||b-Ax||_2/||b||_2. */
int orc_pcg(const orc_csr *a, const orc_amg *h, const double *b, double *x, double tol,
            int maxit, double *relres);

#ifdef __cplusplus
}
#endif
#endif
