// Drop-in replacement for AFEPack's src/AMGSolver.cpp that runs the solver on
// a GB300 through the afepack_gb300 C ABI.  It is compiled inside AFEPack's
// own build in place of src/AMGSolver.cpp, against the UNCHANGED header
// include/AFEPack/AMGSolver.h, and linked with libafepack_gb300.so.
//
// The header has no spare member for a device handle, so the handle of each
// AMGSolver object lives in a mutex-guarded side table keyed by `this`,
// created by reinit()/lazyReinit() and removed by clear() (the destructor
// calls clear(), as in the reference).  Errors abort with a message, which is
// what the reference does for its own failures (assert/abort).
//
// Environment: AFP_DEVICE selects the GPU (default 0); AFP_PRECISION=mixed
// selects the FP32 V-cycle; AFP_DENSE_TAIL overrides the dense-tail size
// (0 keeps the reference's full depth, which is the default here so that
// solve() iterates exactly the reference's hierarchy).
#include <AFEPack/AMGSolver.h>

#include <cstdlib>
#include <iostream>
#include <mutex>
#include <unordered_map>
#include <vector>

#include "afepack_gb300.h"

AFEPACK_OPEN_NAMESPACE

namespace {

struct DeviceSolver {
  afp_matrix* A = nullptr;
  afp_amg* amg = nullptr;
  const SparsityPattern* pattern = nullptr;
};

std::mutex g_mutex;
std::unordered_map<const AMGSolver*, DeviceSolver> g_table;
afp_context* g_ctx = nullptr;

void check(afp_status s, const char* what) {
  if (s == AFP_OK) return;
  std::cerr << "afepack_gb300: " << what << " failed: " << afp_status_string(s) << " (" << afp_last_error()
            << ")" << std::endl;
  abort();
}

afp_context* context() {
  if (g_ctx == nullptr) {
    const char* dev = std::getenv("AFP_DEVICE");
    check(afp_context_create(dev ? std::atoi(dev) : 0, &g_ctx), "afp_context_create");
  }
  return g_ctx;
}

afp_matrix* upload(const AMGSolver::Matrix& M) {
  const SparsityPattern& sp = M.get_sparsity_pattern();
  const size_t m = M.m(), nnz = M.n_nonzero_elements();
  const size_t* rs = sp.get_rowstart_indices();
  const size_t* cn = sp.get_column_numbers();
  std::vector<int32_t> rowptr(rs, rs + m + 1), cols(cn, cn + nnz);
  std::vector<double> vals(nnz);
  for (size_t k = 0; k < nnz; ++k) vals[k] = M.global_entry(k);
  afp_matrix* A = nullptr;
  check(afp_matrix_create_csr(context(), (int64_t)m, (int64_t)M.n(), (int64_t)nnz, rowptr.data(), cols.data(),
                              vals.data(), &A),
        "afp_matrix_create_csr");
  return A;
}

}  // namespace

void AMGSolver::reinit(const Matrix& M) {
  clear();
  std::cerr << "AMGSolver initializing on the GPU ..." << std::flush;
  assert(M.get_sparsity_pattern().is_compressed());
  assert(M.m() == M.n());
  afp_amg_opts o;
  afp_amg_default_opts(&o);
  o.tolerance = toler;
  o.smooth_step = (int)smooth_step;
  o.max_coarse = (int)n_most_project_order;
  o.min_density = n_most_project_sparse_degree;
  o.alpha = alpha;
  const char* prec = std::getenv("AFP_PRECISION");
  o.precision = (prec && std::string(prec) == "mixed") ? AFP_PRECISION_MIXED : AFP_PRECISION_FP64;
  const char* tail = std::getenv("AFP_DENSE_TAIL");
  o.dense_tail = tail ? std::atoi(tail) : 0;
  o.symmetric = 0;  // the reference smooths forward before and after the coarse correction
  DeviceSolver d;
  d.A = upload(M);
  d.pattern = &M.get_sparsity_pattern();
  check(afp_amg_setup(d.A, &o, &d.amg), "afp_amg_setup");
  int levels = 0, solve_levels = 0;
  check(afp_amg_num_levels(d.amg, &levels, &solve_levels), "afp_amg_num_levels");
  {
    std::lock_guard<std::mutex> lock(g_mutex);
    g_table[this] = d;
  }
  n_project = (u_int)levels;
  is_initialized = true;
  std::cerr << " OK! grid levels: " << n_project << std::endl;
}

void AMGSolver::lazyReinit(const Matrix& M) {
  if (is_initialized) {
    std::lock_guard<std::mutex> lock(g_mutex);
    auto it = g_table.find(this);
    if (it != g_table.end() && it->second.pattern != &M.get_sparsity_pattern()) {
      std::cerr << "The solver is not initialized with the same sparsity pattern." << std::endl;
      abort();
    }
  }
  reinit(M);
}

void AMGSolver::solve(Vector<double>& x, const Vector<double>& r, double tol, size_t s1, int mode) const {
  assert(is_initialized == true);
  assert(x.size() == r.size());
  afp_amg* amg = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_mutex);
    amg = g_table.at(this).amg;
  }
  afp_solve_info info;
  check(afp_amg_solve(amg, x.data(), r.begin(), tol, (int64_t)s1, mode, &info), "afp_amg_solve");
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
  DeviceSolver d;
  {
    std::lock_guard<std::mutex> lock(g_mutex);
    auto it = g_table.find(this);
    if (it != g_table.end()) {
      d = it->second;
      g_table.erase(it);
    }
  }
  if (d.amg) afp_amg_destroy(d.amg);
  if (d.A) afp_matrix_destroy(d.A);
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
