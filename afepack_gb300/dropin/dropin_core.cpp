// See dropin_core.h.
#include "dropin_core.h"

#include <cstdlib>
#include <mutex>
#include <stdexcept>
#include <string>
#include <unordered_map>

namespace afp_dropin {
namespace {

struct Solver {
  afp_matrix* A = nullptr;
  afp_amg* amg = nullptr;
  const void* pattern = nullptr;  // the SparsityPattern the solver was set up with
  bool lazy = false;
};

std::mutex g_mu;
std::unordered_map<const void*, Solver> g_solvers;
afp_context* g_ctx = nullptr;

void check(afp_status s, const char* what) {
  if (s == AFP_OK) return;
  throw std::runtime_error(std::string("afepack_gb300: ") + what + " failed: " + afp_status_string(s) + " (" +
                           afp_last_error() + ")");
}

afp_context* context() {
  if (g_ctx == nullptr) {
    const char* dev = std::getenv("AFP_DEVICE");
    check(afp_context_create(dev ? std::atoi(dev) : 0, &g_ctx), "afp_context_create");
  }
  return g_ctx;
}

afp_amg_opts device_opts(const Options& o) {
  afp_amg_opts d;
  afp_amg_default_opts(&d);
  d.tolerance = o.tol;
  d.smooth_step = o.smooth_step;
  d.max_coarse = o.max_coarse;
  d.min_density = o.min_density;
  d.alpha = o.alpha;
  const char* prec = std::getenv("AFP_PRECISION");
  d.precision = (prec && std::string(prec) == "mixed") ? AFP_PRECISION_MIXED : AFP_PRECISION_FP64;
  const char* tail = std::getenv("AFP_DENSE_TAIL");
  d.dense_tail = tail ? std::atoi(tail) : 0;
  d.symmetric = 0;  // the reference smooths forward before and after the coarse correction
  return d;
}

void release(Solver& s) {
  if (s.amg) afp_amg_destroy(s.amg);
  if (s.A) afp_matrix_destroy(s.A);
  s = Solver();
}

Solver& get(const void* owner) {
  auto it = g_solvers.find(owner);
  if (it == g_solvers.end()) throw std::runtime_error("afepack_gb300: the solver is not initialized");
  return it->second;
}

}  // namespace

void reinit(const void* owner, const Matrix& M, const Options& o) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (M.m != M.n) throw std::runtime_error("afepack_gb300: AMGSolver needs a square matrix");
  auto it = g_solvers.find(owner);
  if (it != g_solvers.end()) {
    release(it->second);
    g_solvers.erase(it);
  }
  Solver s;
  check(afp_matrix_create_csr(context(), M.m, M.n, M.nnz, M.rowptr, M.cols, M.vals, &s.A), "afp_matrix_create_csr");
  const afp_amg_opts d = device_opts(o);
  const afp_status st = afp_amg_setup(s.A, &d, &s.amg);
  if (st != AFP_OK) {
    afp_matrix_destroy(s.A);
    check(st, "afp_amg_setup");
  }
  g_solvers[owner] = s;
}

void lazy_reinit(const void* owner, const void* pattern, const Matrix& M, const Options& o) {
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_solvers.find(owner);
  if (it == g_solvers.end()) {  // lazyInit: the lazyProject hierarchy
    Solver s;
    s.pattern = pattern;
    s.lazy = true;
    check(afp_matrix_create_csr(context(), M.m, M.n, M.nnz, M.rowptr, M.cols, M.vals, &s.A), "afp_matrix_create_csr");
    const afp_amg_opts d = device_opts(o);
    const afp_status st = afp_amg_setup_lazy(s.A, &d, &s.amg);
    if (st != AFP_OK) {
      afp_matrix_destroy(s.A);
      check(st, "afp_amg_setup_lazy");
    }
    g_solvers[owner] = s;
    return;
  }
  Solver& s = it->second;
  if (!s.lazy || s.pattern != pattern)
    throw std::runtime_error("The solver is not initialized with the same sparsity pattern.");
  int64_t m = 0, nnz = 0;
  check(afp_matrix_info(s.A, &m, nullptr, &nnz), "afp_matrix_info");
  if (m != M.m || nnz != M.nnz) throw std::runtime_error("The solver is not initialized with the same sparsity pattern.");
  // new values into the same device pattern, then the Galerkin products again
  check(afp_matrix_set_values(s.A, M.vals), "afp_matrix_set_values");
  check(afp_amg_lazy_reinit(s.amg, s.A), "afp_amg_lazy_reinit");
}

afp_solve_info solve(const void* owner, double* x, const double* r, double tol, int64_t step, int mode) {
  afp_amg* amg;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    amg = get(owner).amg;
  }
  afp_solve_info info{};
  check(afp_amg_solve(amg, x, r, tol, step, mode, &info), "afp_amg_solve");
  return info;
}

void precondition(const void* owner, double* x, const double* b, int iterate_step) {
  afp_amg* amg;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    amg = get(owner).amg;
  }
  check(afp_amg_precondition(amg, x, b, iterate_step), "afp_amg_precondition");
}

void clear(const void* owner) {
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_solvers.find(owner);
  if (it == g_solvers.end()) return;
  release(it->second);
  g_solvers.erase(it);
}

bool initialized(const void* owner) {
  std::lock_guard<std::mutex> lk(g_mu);
  return g_solvers.count(owner) != 0;
}

int n_project(const void* owner) {
  afp_amg* amg;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    amg = get(owner).amg;
  }
  int np = 0, sl = 0;
  check(afp_amg_num_levels(amg, &np, &sl), "afp_amg_num_levels");
  return np;
}

afp_amg* handle(const void* owner) {
  std::lock_guard<std::mutex> lk(g_mu);
  return get(owner).amg;
}

}  // namespace afp_dropin
