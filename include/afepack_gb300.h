/*
 * afepack_gb300 -- C ABI of a GB300-native (sm_103a) implementation of
 * AFEPack's elliptic-solve path: P1/P2 stiffness/mass assembly into AFEPack's
 * CSR sparsity pattern, Dirichlet elimination, the classical C/F AMG
 * hierarchy with a GPU Galerkin product, the V-cycle with a multicolour
 * Gauss-Seidel smoother, and an outer preconditioned CG.
 *
 * Every entry point returns an afp_status; afp_last_error() gives the message
 * of the calling thread's last failure.  Objects are opaque handles owning
 * device memory.  Unless stated otherwise a double / int32 array argument may
 * live in host memory or in device memory of the context's GPU (copies go
 * through unified addressing); all work is ordered on the context's stream and
 * every call returns only after its results are visible to the caller.
 *
 * Matrices use AFEPack's SparsityPattern convention
 * (include/AFEPack/SparsityPattern.h:76-126,193-237): for a square matrix the
 * diagonal entry is the first of its row and the remaining column numbers are
 * ascending.  Row starts and column numbers are 32-bit here (AFEPack uses
 * size_t); afp_matrix_download widens nothing, callers widen if they need to.
 *
 * Reference interfaces each group replaces are cited beside it (paths within
 * the AFEPack source tree).
 */
#ifndef AFEPACK_GB300_H
#define AFEPACK_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define AFP_VERSION 1

typedef enum afp_status {
  AFP_OK = 0,
  AFP_ERR_INVALID = 1,        /* bad argument (null handle, size, option)      */
  AFP_ERR_CUDA = 2,           /* CUDA runtime failure                          */
  AFP_ERR_NO_DEVICE = 3,      /* no usable sm_103 GPU                          */
  AFP_ERR_OUT_OF_MEMORY = 4,  /* device or host allocation failed              */
  AFP_ERR_NOT_CONVERGED = 5,  /* iteration limit reached above the tolerance   */
  AFP_ERR_BREAKDOWN = 6,      /* NaN/Inf or a zero denominator in a recurrence */
  AFP_ERR_SINGULAR = 7,       /* singular coarsest matrix                      */
  AFP_ERR_TIMEOUT = 8,        /* a bounded wait ran out                        */
  AFP_ERR_UNSUPPORTED = 9,    /* input outside what the kernels handle         */
  AFP_ERR_CAPACITY = 10       /* request cannot be admitted (memory/slots)     */
} afp_status;

typedef struct afp_context afp_context;
typedef struct afp_space afp_space;
typedef struct afp_matrix afp_matrix;
typedef struct afp_amg afp_amg;

/* ---------------------------------------------------------------- misc */
int afp_version(void);
const char *afp_status_string(afp_status s);
const char *afp_last_error(void);

/* ------------------------------------------------------------- context */
/* A context binds one GPU and one CUDA stream (a new non-blocking stream). */
afp_status afp_context_create(int device, afp_context **out);
afp_status afp_context_destroy(afp_context *ctx);
afp_status afp_context_synchronize(afp_context *ctx);
/* The context's CUDA stream (a cudaStream_t), for callers that order their
 * own work or timing events with the library's. */
afp_status afp_context_stream(const afp_context *ctx, void **stream);
/* Number of this library's kernel launches issued on the context so far. */
afp_status afp_context_launch_count(const afp_context *ctx, int64_t *count);

/* --------------------------------------------------------------- space */
/* Mesh and DOF map of a Lagrange P1/P2 space on triangles (dim 2) or
 * tetrahedra (dim 3): the data AFEPack's FEMSpace holds after
 * buildElement/buildDof (include/AFEPack/FEMSpace.templates.h:884-1003).
 * coords [n_vertex*dim]; cells [n_cell*(dim+1)] positively oriented vertex
 * lists; elem_dof [n_cell*nd] global DOF of each template DOF (nd = 3,6 in
 * 2D, 4,10 in 3D, template order of triangle.{1,2}.tmp_dof /
 * tetrahedron.{1,2}.tmp_dof). */
afp_status afp_space_create(afp_context *ctx, int dim, int degree, int64_t n_vertex,
                            const double *coords, int64_t n_cell, const int32_t *cells,
                            int64_t n_dof, const int32_t *elem_dof, afp_space **out);
/* FEMSpace::buildDof on the device (include/AFEPack/FEMSpace.templates.h:884-1003):
 * the same space with the DOFs numbered as AFEPack numbers them -- elements
 * in order, inside an element the template's vertices, then (P2) its edges,
 * each geometry getting the next numbers the first time it is touched.
 * Edges are identified by their vertex pairs.  vertex_bmark [n_vertex]
 * (NULL: no boundary) gives each vertex a bit mask of the boundary pieces it
 * lies on; a vertex DOF is on the boundary when its mask is nonzero, an edge
 * DOF when its two vertices' masks share a bit. */
afp_status afp_space_create_numbered(afp_context *ctx, int dim, int degree, int64_t n_vertex,
                                     const double *coords, int64_t n_cell, const int32_t *cells,
                                     const int32_t *vertex_bmark, afp_space **out);
afp_status afp_space_info(const afp_space *sp, int64_t *n_dof, int *nd);
/* elem_dof [n_cell*nd]; dof_bmark [n_dof] (1 on the boundary) and dof_point
 * [n_dof*dim] (interpolation points) for spaces from
 * afp_space_create_numbered; any pointer may be NULL. */
afp_status afp_space_download_dofs(const afp_space *sp, int32_t *elem_dof, int32_t *dof_bmark,
                                   double *dof_point);
afp_status afp_space_destroy(afp_space *sp);

/* ------------------------------------------------------------ assembly */
typedef struct afp_assemble_opts {
  int acc_stiff;        /* algebraic accuracy of the stiffness quadrature  */
  int acc_mass;         /* algebraic accuracy of the mass quadrature       */
  const double *coef;   /* per-cell coefficient a_e of -div(a grad u), or NULL */
} afp_assemble_opts;

/* StiffMatrix<DIM,double>::build and MassMatrix<DIM,double>::build
 * (include/AFEPack/BilinearOperator.templates.h:56-255, element matrices of
 * :343-406): builds the sparsity pattern once and fills the stiffness matrix
 * (scaled per cell by coef when given) and, if mass != NULL, the mass matrix
 * in the same pattern. */
afp_status afp_assemble(afp_space *sp, const afp_assemble_opts *opts, afp_matrix **stiff,
                        afp_matrix **mass);

/* ------------------------------------------------------------- matrices */
/* A device copy of a CSR matrix given in AFEPack's layout. */
afp_status afp_matrix_create_csr(afp_context *ctx, int64_t m, int64_t n, int64_t nnz,
                                 const int32_t *rowptr, const int32_t *cols, const double *vals,
                                 afp_matrix **out);
afp_status afp_matrix_info(const afp_matrix *a, int64_t *m, int64_t *n, int64_t *nnz);
/* Overwrites all nnz stored values, keeping the pattern (what writing
 * SparseMatrix::global_entry(k) does in the reference). */
afp_status afp_matrix_set_values(afp_matrix *a, const double *vals);
/* Copies the pattern and values out (any argument may be NULL to skip). */
afp_status afp_matrix_download(const afp_matrix *a, int32_t *rowptr, int32_t *cols, double *vals);
/* y = A x  (SparseMatrix::vmult, include/AFEPack/SparseMatrix.h:100-114) */
afp_status afp_matrix_vmult(afp_matrix *a, const double *x, double *y);
/* y = A x without allocating device memory.  No counterpart in the
 * reference: it exists for callers that cannot let a library allocate on the
 * device when they call it (device memory already reserved by their own
 * arena, a hard device-memory cap, or a time-step loop whose allocator must
 * not grow).  x and y are staged in a fixed static device array of
 * 2 x AFP_NOALLOC_MAX_ENTRIES doubles (32 MiB), so matrices with more rows or
 * columns than that are refused with AFP_ERR_UNSUPPORTED.  The array is
 * reserved on a GPU by the first afp_context_create for that GPU (create the
 * context before an arena takes the rest of the device) and kept until the
 * process exits; its device address is looked up there too, once per device
 * ordinal, which assumes the device's primary context is never reset
 * (cudaDeviceReset) while the library is in use.  All calls share the array:
 * calls whose GPU work overlaps race.  Nothing in it needs to start at zero. */
#define AFP_NOALLOC_MAX_ENTRIES (1 << 21)
afp_status afp_matrix_vmult_noalloc(afp_matrix *a, const double *x, double *y);
afp_status afp_matrix_destroy(afp_matrix *a);

/* Operator::L2Discretize(f, fem_space, f1, algebric_accuracy)
 * (include/AFEPack/Operator.discretize.templates.h): f1_i = the sum, over
 * the cells around DOF i and their quadrature points, of Jxw f(q) phi_i(q),
 * added in the reference's order (bitwise its result for the first two
 * sources).  source selects what f is:
 *   AFP_SOURCE_POINT_VALUES  data = f at the quadrature points of
 *       afp_quadrature_points, [n_cell*n_q] (the reference's function-pointer
 *       form evaluates f at exactly these points, lines 151-183);
 *   AFP_SOURCE_FEM_FUNCTION  data = a FEM function's DOF values [n_dof]
 *       (L2Discretize(const FEMFunction&, f1, acc), lines 18-47);
 *   AFP_SOURCE_GAUSSIANS     data = [centre (dim), width s, amplitude a] per
 *       Gaussian: f = sum of a exp(-|x - c|^2 / (2 s^2)), evaluated on the
 *       device (the CUDA exp, within an ulp of the host's).
 * data and f1 may be host or device memory. */
typedef enum afp_source {
  AFP_SOURCE_POINT_VALUES = 0,
  AFP_SOURCE_FEM_FUNCTION = 1,
  AFP_SOURCE_GAUSSIANS = 2
} afp_source;
/* the global quadrature points [n_cell*n_q*dim] of the rule of accuracy acc
 * (points may be NULL to query n_q) */
afp_status afp_quadrature_points(afp_space *sp, int acc, int *n_q, double *points);
afp_status afp_l2_discretize(afp_space *sp, int acc, int source, const double *data, int64_t n_data,
                             double *f1);

/* BoundaryConditionAdmin::apply(A, u, f, preserve_symmetry)
 * (include/AFEPack/FEMSpace.templates.h:1338-1366): for every DOF i with
 * dirichlet[i] != 0, f_i = a_ii g_i and row i's off-diagonal entries become 0;
 * with preserve_symmetry the column entries a_ki become 0 too after
 * f_k -= a_ki f_i / a_ii.  The pattern is kept.  g == NULL means zero data. */
afp_status afp_apply_dirichlet(afp_matrix *a, double *f, const int32_t *dirichlet,
                               const double *g, int preserve_symmetry);

/* ------------------------------------------------------------------ AMG */
typedef enum afp_precision {
  AFP_PRECISION_FP64 = 0,   /* V-cycle in FP64                                   */
  AFP_PRECISION_MIXED = 1   /* V-cycle in FP32, FP64 outer recurrences           */
} afp_precision;

typedef struct afp_amg_opts {
  double tolerance;     /* AMGSolver toler (default 1e-12)                      */
  int smooth_step;      /* Gauss-Seidel sweeps per smoothing (default 3)        */
  int max_coarse;       /* n_most_project_order (default 50)                    */
  double min_density;   /* n_most_project_sparse_degree (default 0.382)         */
  double alpha;         /* strong-connection threshold (default 0.25)           */
  int precision;        /* afp_precision of the V-cycle (default FP64)          */
  int dense_tail;       /* coarsening stops at the first coarse level with at
                           most this many rows (default 4096, max 16384), or
                           with at most 16384 rows and at least 5% of its
                           entries nonzero; that level is solved with a dense
                           inverse instead of smoothed (0 keeps the
                           reference's full depth).  The inverse costs 2 n^3
                           FP64 operations (0.1 s at 4096 rows), so a sparse
                           level of more rows (a 33K-DOF 2D problem's
                           7,644-row third level: 1 s) is coarsened further
                           instead; dense coarse levels of 3D and 2D P2
                           hierarchies (6,744 rows at 12%, 12,588 at 11%)
                           stop by density */
  int max_colors;       /* colour classes of the smoother before rows fall into
                           an l1-Jacobi overflow class (default 32)             */
  int symmetric;        /* post-smoothing visits colours in reverse order so the
                           V-cycle is a symmetric preconditioner (default 1)    */
  int coarse_colors;    /* colour-class cap on levels >= 1 (default 4; 0 = use
                           max_colors): their long rows would otherwise need
                           dozens of sequential classes, one launch each; the
                           rows beyond the cap form one l1-Jacobi class.  On
                           the 3D P1 64^3 hierarchy caps of 8, 4 and 2 give
                           21, 21 and 22 PCG iterations (CPU restatement of
                           the V-cycle)                                         */
  int interp_bf16;      /* mixed precision only: keep P and P^T in BF16 (1) or
                           in FP32 (0, default: BF16 interpolation weights cost
                           the 3D P1 solve about 1.5x the PCG iterations)       */
  int fused_vcycle;     /* mixed precision: run each V-cycle as one persistent
                           kernel (1) instead of a chain of ~100 PDL launches
                           (0, default: on the 3D P1 64^3 hierarchy the chain
                           takes 0.80 ms per V-cycle and the persistent kernel
                           0.93 ms -- both are bound by ~100 dependent steps,
                           a launch or a grid-wide wait of ~2.5 us each).  The kernel keeps one CTA per SM and
                           streams every CTA's share of the level operators
                           through a ring of shared-memory slots with bulk
                           async copies; colour classes wait only for the CTAs
                           that own coupled rows, level changes for the whole
                           grid.  It needs the whole GPU, so the server's
                           concurrent workers use the chain.  Where the plan
                           does not apply (BF16 interpolation, a row longer
                           than ~3000 entries, a single-level hierarchy) the
                           chain runs. */
  double wait_limit_s;  /* bound on every wait of the persistent kernel (grid
                           barriers, neighbour waits, shared-memory slots);
                           past it the kernel stops and the call returns
                           AFP_ERR_TIMEOUT (default 2 s, at most 60) */
  int inject_barrier_stall; /* fault injection for tests: the first grid
                           barrier of each persistent V-cycle waits for one
                           arrival more than the grid has, so every wait runs
                           out after wait_limit_s (default 0) */
  int gpu_coarsen;      /* classical hierarchy: C/F splitting and P on the GPU
                           (1, default), with the host routine's flags and P
                           bit for bit, or on the host (0) */
} afp_amg_opts;

typedef struct afp_solve_info {
  int iterations;       /* V-cycles (stationary solve) or CG iterations        */
  int converged;        /* 1 when the stopping test was met                    */
  double initial_residual;
  double final_residual;   /* l1 norm (stationary) or relative l2 (PCG)        */
  double seconds;          /* device time of the call                          */
} afp_solve_info;

void afp_amg_default_opts(afp_amg_opts *opts);

/* AMGSolver::reinit (src/AMGSolver.cpp:384-438): the C/F splitting of
 * Project (:18-226) runs on the host, the Galerkin product P A P^T of
 * getPMPt (:288-358) on the GPU, level by level, until the reference's stop
 * rule (order <= max_coarse and density >= min_density) holds. */
afp_status afp_amg_setup(afp_matrix *a, const afp_amg_opts *opts, afp_amg **out);
/* AMGSolver::lazyReinit on a fresh solver, i.e. lazyInit (src/AMGSolver.cpp:442-503):
 * the hierarchy of lazyProject (:235-284, aggregation-like P with 1/count
 * weights), which AMGPreconditioner uses. */
afp_status afp_amg_setup_lazy(afp_matrix *a, const afp_amg_opts *opts, afp_amg **out);
/* AMGSolver::lazyReinit on an initialised lazy solver (:505-545): the same
 * projections applied to new matrix values.  `a` must share the pattern
 * object the solver was set up with -- the same matrix after
 * afp_matrix_set_values, or the stiffness/mass pair of one afp_assemble
 * call -- otherwise AFP_ERR_INVALID, as the reference aborts.  Only the GPU
 * Galerkin products run; no host C/F splitting. */
afp_status afp_amg_lazy_reinit(afp_amg *amg, afp_matrix *a);
afp_status afp_amg_destroy(afp_amg *amg);
afp_status afp_amg_num_levels(const afp_amg *amg, int *n_project, int *solve_levels);
/* level l (0 = fine): order, stored entries, smoother colour classes
 * (-1 for the dense tail level) */
afp_status afp_amg_level_info(const afp_amg *amg, int level, int64_t *n, int64_t *nnz, int *colors);
/* Downloads level l's Galerkin matrix (l >= 1) or projection P_l (l >= 0) in
 * the reference's orientation (P is n_{l+1} x n_l) and the reference's row
 * order; pass NULL to skip an array. */
afp_status afp_amg_download_level(const afp_amg *amg, int level, int32_t *rowptr, int32_t *cols,
                                  double *vals);
afp_status afp_amg_download_projection(const afp_amg *amg, int level, int32_t *rowptr,
                                       int32_t *cols, double *vals);

/* Measurement hook (no reference counterpart): runs `reps` times one unit of
 * work on device-resident data and reports its mean device time (CUDA events
 * on the context's stream) and its algorithmic bytes (compulsory traffic:
 * each array once per pass).  kind: 0 = one Gauss-Seidel sweep over all
 * colour classes of `level`, 1 = the residual SpMV of `level`, 2 = one
 * V-cycle, 3 = the FP64 fine-level SpMV of the CG; at the width of the last
 * batched solve (afp_pcg_solve_multi or a batch server), 4 = one batched
 * V-cycle and 5 = one batched sweep of `level`.  The precision is the
 * solver's. */
afp_status afp_amg_time_kernel(afp_amg *amg, int kind, int level, int reps, double *ms, double *bytes);

/* AMGSolver::solve(x, r, tol, step, mode) (src/AMGSolver.cpp:549-639):
 * step+1 V-cycles starting from x; tol only decides `converged`
 * (l1 residual < tol * initial l1 residual; tol == 0 uses the solver's). */
afp_status afp_amg_solve(afp_amg *amg, double *x, const double *r, double tol, int64_t step,
                         int mode, afp_solve_info *info);
/* AMGPreconditioner::vmult(x, b) (include/AFEPack/AMGSolver.h:193-195):
 * iterate_step+1 V-cycles from the given x. */
afp_status afp_amg_precondition(afp_amg *amg, double *x, const double *b, int iterate_step);

/* Conjugate gradients preconditioned by one V-cycle per iteration, the
 * solver shape of examples/FAST/src/poisson_solver_comparison_afepack.cpp:197-253
 * (which the library itself does not provide): stops when
 * ||b - A x||_2 <= tol ||b||_2.  x holds the initial guess on entry.
 * With a mixed-precision hierarchy the V-cycle runs in FP32 and the CG
 * recurrences, residuals and dot products in FP64. */
afp_status afp_pcg_solve(afp_amg *amg, double *x, const double *b, double tol, int maxit,
                         afp_solve_info *info);
/* nrhs systems with the same matrix; X and B are n x nrhs row-major.  One
 * batched launch per kernel serves all right-hand sides; every column has
 * its own CG recurrences and stopping test. info may be NULL or nrhs long. */
afp_status afp_pcg_solve_multi(afp_amg *amg, double *X, const double *B, int nrhs, double tol,
                               int maxit, afp_solve_info *info);

/* -------------------------------------------------------------- serving */
/* A solve server: continuous batching of independent requests on one GPU
 * (no counterpart in the reference, which solves one system per call).  Each
 * request carries its own mesh and data and runs the whole path --
 * afp_space_create, afp_assemble, b = M f, afp_apply_dirichlet (zero data),
 * afp_amg_setup, afp_pcg_solve -- in one of `workers` execution slots, each
 * with its own stream, so admitted requests overlap on the device and their
 * host C/F work runs in parallel.  A request is admitted, in arrival order,
 * when a slot is free and its estimated device footprint fits the budget. */
typedef struct afp_server afp_server;

typedef struct afp_server_opts {
  int workers;                 /* execution slots (default 8)                   */
  int64_t hbm_budget_bytes;    /* admission budget; 0 = 80% of free memory      */
  int precision;               /* afp_precision of the V-cycle (default MIXED)  */
  double tol;                  /* relative residual of the CG (default 1e-10)   */
  int maxit;                   /* CG iteration limit (default 500)              */
  int dense_tail;              /* afp_amg_opts.dense_tail, -1 = its default      */
} afp_server_opts;

typedef struct afp_request {
  int dim, degree, acc_stiff, acc_mass;
  int64_t n_vertex;
  const double *coords;        /* [n_vertex*dim]                                */
  int64_t n_cell;
  const int32_t *cells;        /* [n_cell*(dim+1)]                              */
  int64_t n_dof;
  const int32_t *elem_dof;     /* [n_cell*nd]                                   */
  const int32_t *dirichlet;    /* [n_dof] nonzero on Dirichlet DOFs (zero data) */
  const double *coef;          /* [n_cell] coefficient or NULL                   */
  const double *f;             /* [n_dof] nodal data, b = M f                    */
} afp_request;                 /* host arrays; copied by afp_server_submit       */

typedef struct afp_request_result {
  int status;                  /* afp_status of the request                     */
  int iterations;
  double rel_residual;
  double queue_seconds;        /* submit -> admission                           */
  double setup_seconds;        /* admission -> hierarchy ready                  */
  double latency_seconds;      /* submit -> solution ready                      */
  double device_seconds;       /* device time of the CG                         */
  int64_t estimate_bytes;      /* footprint charged at admission (estimate)     */
  int64_t measured_bytes;      /* peak device bytes the request held; the
                                  server charges this instead of the estimate
                                  once the request's setup is done (0 for the
                                  batch server)                                 */
} afp_request_result;

typedef struct afp_server_stats {
  int64_t completed, failed, queued;
  double p50_seconds, p99_seconds;   /* latency percentiles of completed requests */
  double solves_per_second;          /* completed / (last completion - stats start) */
  int64_t budget_bytes, in_use_bytes;
} afp_server_stats;

void afp_server_default_opts(afp_server_opts *opts);
afp_status afp_server_create(int device, const afp_server_opts *opts, afp_server **out);
afp_status afp_server_submit(afp_server *s, const afp_request *req, int64_t *ticket);
/* Blocks until the request is done; copies its solution (n_dof doubles) to x
 * when x != NULL and releases the ticket. */
afp_status afp_server_wait(afp_server *s, int64_t ticket, double *x, afp_request_result *res);
afp_status afp_server_poll(afp_server *s, int64_t ticket, int *done);
afp_status afp_server_get_stats(afp_server *s, afp_server_stats *stats);
afp_status afp_server_reset_stats(afp_server *s);
/* Finishes queued requests, then stops the slots. */
afp_status afp_server_destroy(afp_server *s);

/* A batching server for many right-hand sides against one resident
 * hierarchy (no counterpart in the reference): requests carry only b; the
 * server keeps `width` CG columns of the hierarchy's batched solver in flight
 * and, between two CG iterations, admits queued requests into free columns
 * and returns the ones that reached tol, so requests join and leave while
 * others are being solved (every iteration is one batched V-cycle over all
 * columns).  A request's solution does not depend on the other columns.
 * While a server exists, the hierarchy must not be used by other calls. */
typedef struct afp_batch_server afp_batch_server;

typedef struct afp_batch_opts {
  int width;                   /* columns (execution slots), 1..64 (default 32) */
  double tol;                  /* relative residual of each CG (default 1e-10) */
  int maxit;                   /* CG iteration limit (default 500)             */
} afp_batch_opts;

void afp_batch_default_opts(afp_batch_opts *opts);
afp_status afp_batch_server_create(afp_amg *amg, const afp_batch_opts *opts, afp_batch_server **out);
/* b: host array of n doubles (reference order), copied before returning. */
afp_status afp_batch_server_submit(afp_batch_server *s, const double *b, int64_t *ticket);
/* Blocks until the request is done; x (n doubles) receives its solution. */
afp_status afp_batch_server_wait(afp_batch_server *s, int64_t ticket, double *x, afp_request_result *res);
afp_status afp_batch_server_get_stats(afp_batch_server *s, afp_server_stats *stats);
afp_status afp_batch_server_reset_stats(afp_batch_server *s);
/* Finishes queued and running requests, then stops. */
afp_status afp_batch_server_destroy(afp_batch_server *s);

/* ----------------------------------------------------------- host logic */
/* The C/F splitting and projection of one level (Project, src/AMGSolver.cpp:18-226),
 * run on the host on a host CSR; no GPU needed.  cf receives -1 for C and 1
 * for F points.  P (n_coarse x m, sorted columns) is returned through
 * buffers the library allocates; release them with afp_host_free. */
afp_status afp_host_coarsen(int64_t m, const int32_t *rowptr, const int32_t *cols,
                            const double *vals, double alpha, int32_t *cf, int64_t *n_coarse,
                            int32_t **p_rowptr, int32_t **p_cols, double **p_vals);
void afp_host_free(void *p);

#ifdef __cplusplus
}
#endif
#endif /* AFEPACK_GB300_H */
