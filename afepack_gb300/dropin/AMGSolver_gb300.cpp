// Drop-in replacement for AFEPack's src/AMGSolver.cpp that runs the solver on
// a GB300 through the afepack_gb300 C ABI.  It is compiled inside AFEPack's
// own build in place of src/AMGSolver.cpp, against the UNCHANGED header
// include/AFEPack/AMGSolver.h, and linked with dropin_core.cpp and
// libafepack_gb300.so.
//
// The header has no spare member for a device handle, so the device solver
// of each AMGSolver object lives in dropin_core's table keyed by `this`,
// created by reinit() (the classical hierarchy) or lazyReinit() (lazyInit's
// hierarchy on first use, a numeric re-setup when the same SparsityPattern
// object returns with new values -- what AMGPreconditioner relies on,
// AMGSolver.h:179-190) and removed by clear() (the destructor calls clear(),
// as in the reference).  AMGPreconditioner is header-only in the reference
// and reaches the device through lazyReinit() and solve().  Errors abort with
// a message, which is what the reference does for its own failures.
#include <AFEPack/AMGSolver.h>

#include <iostream>
#include <stdexcept>
#include <vector>

#include "dropin_core.h"

AFEPACK_OPEN_NAMESPACE

namespace {

// AFEPack's CSR (size_t row starts and columns) as 32-bit arrays
struct Csr32 {
  std::vector<int32_t> rowptr, cols;
  std::vector<double> vals;
  afp_dropin::Matrix view(const AMGSolver::Matrix& M) {
    const SparsityPattern& sp = M.get_sparsity_pattern();
    const size_t m = M.m(), nnz = M.n_nonzero_elements();
    const size_t* rs = sp.get_rowstart_indices();
    const size_t* cn = sp.get_column_numbers();
    rowptr.assign(rs, rs + m + 1);
    cols.assign(cn, cn + nnz);
    vals.resize(nnz);
    for (size_t k = 0; k < nnz; ++k) vals[k] = M.global_entry(k);
    afp_dropin::Matrix v;
    v.m = (int64_t)m;
    v.n = (int64_t)M.n();
    v.nnz = (int64_t)nnz;
    v.rowptr = rowptr.data();
    v.cols = cols.data();
    v.vals = vals.data();
    return v;
  }
};

template <class F>
void or_abort(F&& f) {
  try {
    f();
  } catch (const std::exception& e) {
    std::cerr << e.what() << std::endl;
    abort();
  }
}

}  // namespace

namespace {
afp_dropin::Options options_of(double toler, u_int smooth_step, u_int nmpo, double nmpsd, double alpha) {
  afp_dropin::Options o;
  o.tol = toler;
  o.smooth_step = (int)smooth_step;
  o.max_coarse = (int)nmpo;
  o.min_density = nmpsd;
  o.alpha = alpha;
  return o;
}
}  // namespace

void AMGSolver::reinit(const Matrix& M) {
  clear();
  std::cerr << "AMGSolver initializing on the GPU ..." << std::flush;
  assert(M.get_sparsity_pattern().is_compressed());
  assert(M.m() == M.n());
  Csr32 c;
  or_abort([&] {
    afp_dropin::reinit(this, c.view(M),
                       options_of(toler, smooth_step, n_most_project_order, n_most_project_sparse_degree, alpha));
    n_project = (u_int)afp_dropin::n_project(this);
  });
  is_initialized = true;
  std::cerr << " OK! grid levels: " << n_project << std::endl;
}

// lazyInit (src/AMGSolver.cpp:442-503): a new lazyProject hierarchy for M
void AMGSolver::lazyInit(const Matrix& M) {
  clear();
  Csr32 c;
  or_abort([&] {
    afp_dropin::lazy_reinit(this, &M.get_sparsity_pattern(), c.view(M),
                            options_of(toler, smooth_step, n_most_project_order, n_most_project_sparse_degree, alpha));
    n_project = (u_int)afp_dropin::n_project(this);
  });
  is_initialized = true;
}

// lazyReinit (src/AMGSolver.cpp:505-545): lazyInit on first use, afterwards
// the same projections applied to M's new values (M must keep the pattern
// object the solver was set up with, or the call aborts as the reference does)
void AMGSolver::lazyReinit(const Matrix& M) {
  if (!is_initialized) {
    lazyInit(M);
    return;
  }
  Csr32 c;
  or_abort([&] {
    afp_dropin::lazy_reinit(this, &M.get_sparsity_pattern(), c.view(M),
                            options_of(toler, smooth_step, n_most_project_order, n_most_project_sparse_degree, alpha));
  });
}

void AMGSolver::solve(Vector<double>& x, const Vector<double>& r, double tol, size_t s1, int mode) const {
  assert(is_initialized == true);
  assert(x.size() == r.size());
  afp_solve_info info{};
  or_abort([&] { info = afp_dropin::solve(this, x.data(), r.begin(), tol, (int64_t)s1, mode); });
  if ((mode & 0x0001) == 0) {
    std::cerr << "AMGSolver begin with initial residual " << info.initial_residual << " ..." << std::endl;
    if (info.converged)
      std::cerr << "\r\tconverge with residual " << info.final_residual << " at step " << info.iterations << "."
                << std::endl;
    else
      std::cerr << "\r\tfailed to converge with residual " << info.final_residual << " at step "
                << info.iterations << "." << std::endl;
  }
}

void AMGSolver::clear() {
  if (!is_initialized) return;
  afp_dropin::clear(this);
  project_matrix.clear();
  projected_matrix.clear();
  project_matrix_r.clear();
  is_initialized = false;
}

AMGSolver::AMGSolver()
    : is_initialized(false), n_project(0), is_solve_most_project_exactly(true), toler(1.e-12), alpha(0.25),
      smooth_step(3), n_most_project_order(50), n_most_project_sparse_degree(0.382) {}

AMGSolver::AMGSolver(const Matrix& m, double tol, u_int s, u_int nmpo, double nmpsd, double alp)
    : is_initialized(false), n_project(0), is_solve_most_project_exactly(true), toler(tol), alpha(alp),
      smooth_step(s), n_most_project_order(nmpo), n_most_project_sparse_degree(nmpsd) {
  reinit(m);
}

AMGSolver::~AMGSolver() { clear(); }

AFEPACK_CLOSE_NAMESPACE
