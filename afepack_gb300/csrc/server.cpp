// Solve server: continuous batching of independent elliptic solves on one GPU.
//
// Requests (a mesh/DOF map, per-cell coefficient, nodal data, Dirichlet
// flags) enter a FIFO queue.  A request is admitted when an execution slot is
// free and its estimated device footprint fits the HBM budget; once its
// setup is done, the request's measured peak (its allocations on the slot's
// context) replaces the estimate in the budget.  Each slot is a host
// thread with its own afp_context, hence its own CUDA stream, so the GPU work
// of all admitted requests overlaps on the device while their host work (the
// colouring of the AMG setup) runs in parallel on the host cores.  Requests
// that arrive while others are running are admitted as soon as a slot and
// memory free up.  All device state of a request -- space, matrices,
// hierarchy, iterates -- stays resident for its whole life.
//
// Kernels are deterministic and every request owns its context's reduction
// scratch, so a request's solution does not depend on what else is running.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "common.cuh"

using Clock = std::chrono::steady_clock;

namespace {

struct Job {
  int64_t ticket = 0;
  // owned copies of the request arrays
  int dim = 2, degree = 1, acc_stiff = 4, acc_mass = 4;
  int64_t n_vertex = 0, n_cell = 0, n_dof = 0;
  std::vector<double> coords, coef, f;
  std::vector<int32_t> cells, elem_dof, dirichlet;
  std::vector<double> x;
  int64_t estimate = 0;
  int64_t charged = 0;     // bytes held against the budget: the estimate, then the measured setup peak
  int64_t base_bytes = 0;  // the worker context's DevBuf bytes before the request
  Clock::time_point t_submit, t_admit, t_setup, t_done;
  afp_request_result result{};
  bool done = false;
};

double secs(Clock::time_point a, Clock::time_point b) { return std::chrono::duration<double>(b - a).count(); }

}  // namespace

struct afp_server {
  afp_server_opts opts{};
  int device = 0;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Job*> queue;
  std::unordered_map<int64_t, std::unique_ptr<Job>> jobs;
  std::vector<std::thread> workers;
  int64_t next_ticket = 1;
  int64_t budget = 0, in_use = 0;
  bool stop = false;
  // statistics
  std::vector<double> latencies;
  int64_t completed = 0, failed = 0;
  Clock::time_point t_start = Clock::now(), t_last = Clock::now();
};

namespace {

// Device bytes a request is expected to hold at its peak (assembly + setup).
int64_t estimate_bytes(const Job& j) {
  const int nd = j.dim == 2 ? 3 * j.degree : (j.degree == 1 ? 4 : 10);
  const int64_t nnz = std::min<int64_t>(j.n_dof * j.n_dof, j.n_cell * nd * nd / (j.dim + 1) + j.n_dof);
  int64_t b = 0;
  b += j.n_vertex * j.dim * 8 + j.n_cell * (j.dim + 1 + nd) * 4 * 2;  // mesh, DOF map, incidence
  b += j.n_cell * nd * nd * 8 * 2;                                      // element matrices
  b += nnz * (8 + 4) * 2 + j.n_dof * 4 * 2;                             // stiffness + mass
  b += nnz * 20 * 4;                                                    // hierarchy (operator complexity ~2-3, x2 layouts)
  b += j.n_dof * 8 * 24;                                                // vectors
  return b + (64 << 20);
}

// the request's peak device bytes so far (its allocations on the worker's context)
int64_t request_peak(const afp_context* ctx, const Job& j) { return ctx->dev_peak.load() - j.base_bytes; }

afp_status run(afp_server* s, afp_context* ctx, Job& j, const afp_server_opts& o) {
  afp_space* sp = nullptr;
  afp_matrix *K = nullptr, *M = nullptr;
  afp_amg* amg = nullptr;
  afp_status st = AFP_OK;
  std::vector<double> b(j.n_dof);
  auto cleanup = [&]() {
    if (amg) afp_amg_destroy(amg);
    if (K) afp_matrix_destroy(K);
    if (M) afp_matrix_destroy(M);
    if (sp) afp_space_destroy(sp);
  };
#define AFP_TRY(call)      \
  do {                     \
    st = (call);           \
    if (st != AFP_OK) {    \
      cleanup();           \
      return st;           \
    }                      \
  } while (0)
  AFP_TRY(afp_space_create(ctx, j.dim, j.degree, j.n_vertex, j.coords.data(), j.n_cell, j.cells.data(), j.n_dof,
                           j.elem_dof.data(), &sp));
  afp_assemble_opts ao{j.acc_stiff, j.acc_mass, j.coef.empty() ? nullptr : j.coef.data()};
  AFP_TRY(afp_assemble(sp, &ao, &K, &M));
  AFP_TRY(afp_matrix_vmult(M, j.f.data(), b.data()));
  afp_matrix_destroy(M);
  M = nullptr;
  AFP_TRY(afp_apply_dirichlet(K, b.data(), j.dirichlet.data(), nullptr, 1));
  afp_amg_opts mo;
  afp_amg_default_opts(&mo);
  mo.fused_vcycle = 0;  // workers solve concurrently: no grid-wide cooperative kernels
  mo.precision = o.precision;
  if (o.dense_tail >= 0) mo.dense_tail = o.dense_tail;
  AFP_TRY(afp_amg_setup(K, &mo, &amg));
  j.t_setup = Clock::now();
  {
    // the footprint is known now (the CG adds only its vectors): charge the
    // measured peak instead of the estimate, and let waiting requests in if
    // that freed budget
    const int64_t measured = request_peak(ctx, j);
    std::lock_guard<std::mutex> lk(s->mu);
    s->in_use += measured - j.charged;
    j.charged = measured;
    s->cv_work.notify_all();
  }
  j.x.assign(j.n_dof, 0.0);
  afp_solve_info info{};
  st = afp_pcg_solve(amg, j.x.data(), b.data(), o.tol, o.maxit, &info);
  j.result.iterations = info.iterations;
  j.result.rel_residual = info.final_residual;
  j.result.device_seconds = info.seconds;
  if (st == AFP_OK && !info.converged) st = AFP_ERR_NOT_CONVERGED;
  cleanup();
  return st;
#undef AFP_TRY
}

void worker_main(afp_server* s) {
  afp_context* ctx = nullptr;
  if (afp_context_create(s->device, &ctx) != AFP_OK) return;
  for (;;) {
    Job* j = nullptr;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      s->cv_work.wait(lk, [&] {
        if (s->stop) return true;
        if (s->queue.empty()) return false;
        Job* head = s->queue.front();
        // admit in arrival order when the footprint fits; a request larger
        // than the whole budget is admitted alone
        return s->in_use + head->estimate <= s->budget || s->in_use == 0;
      });
      if (s->stop && s->queue.empty()) break;
      j = s->queue.front();
      s->queue.pop_front();
      s->in_use += j->estimate;
      j->charged = j->estimate;
      j->t_admit = Clock::now();
    }
    j->base_bytes = ctx->dev_bytes.load();
    ctx->dev_peak.store(j->base_bytes);
    afp_status st = run(s, ctx, *j, s->opts);
    {
      std::lock_guard<std::mutex> lk(s->mu);
      j->t_done = Clock::now();
      s->in_use -= j->charged;
      j->result.measured_bytes = request_peak(ctx, *j);
      j->result.status = st;
      j->result.queue_seconds = secs(j->t_submit, j->t_admit);
      j->result.setup_seconds = st == AFP_OK ? secs(j->t_admit, j->t_setup) : 0.0;
      j->result.latency_seconds = secs(j->t_submit, j->t_done);
      j->result.estimate_bytes = j->estimate;
      j->done = true;
      if (st == AFP_OK) {
        s->completed++;
        s->latencies.push_back(j->result.latency_seconds);
      } else {
        s->failed++;
      }
      s->t_last = j->t_done;
    }
    s->cv_done.notify_all();
    s->cv_work.notify_all();
  }
  afp_context_destroy(ctx);
}

double percentile(std::vector<double> v, double p) {
  if (v.empty()) return 0.0;
  std::sort(v.begin(), v.end());
  const double pos = p / 100.0 * (v.size() - 1);
  const size_t i = (size_t)pos;
  const double frac = pos - i;
  return i + 1 < v.size() ? v[i] * (1 - frac) + v[i + 1] * frac : v[i];
}

}  // namespace

using namespace afp;

extern "C" {

void afp_server_default_opts(afp_server_opts* o) {
  if (!o) return;
  o->workers = 8;
  o->hbm_budget_bytes = 0;
  o->precision = AFP_PRECISION_MIXED;
  o->tol = 1e-10;
  o->maxit = 500;
  o->dense_tail = -1;
}

afp_status afp_server_create(int device, const afp_server_opts* opts, afp_server** out) {
  return guarded([&] {
    AFP_REQUIRE(out, AFP_ERR_INVALID, "null argument");
    auto s = std::make_unique<afp_server>();
    if (opts) s->opts = *opts;
    else afp_server_default_opts(&s->opts);
    AFP_REQUIRE(s->opts.workers >= 1 && s->opts.workers <= 64, AFP_ERR_INVALID, "workers must be in [1, 64]");
    s->device = device;
    AFP_CUDA(cudaSetDevice(device));
    size_t free_b = 0, total_b = 0;
    AFP_CUDA(cudaMemGetInfo(&free_b, &total_b));
    s->budget = s->opts.hbm_budget_bytes > 0 ? (int64_t)s->opts.hbm_budget_bytes : (int64_t)(0.8 * (double)free_b);
    for (int w = 0; w < s->opts.workers; ++w) s->workers.emplace_back(worker_main, s.get());
    *out = s.release();
  });
}

afp_status afp_server_submit(afp_server* s, const afp_request* r, int64_t* ticket) {
  return guarded([&] {
    AFP_REQUIRE(s && r && ticket, AFP_ERR_INVALID, "null argument");
    AFP_REQUIRE((r->dim == 2 || r->dim == 3) && (r->degree == 1 || r->degree == 2), AFP_ERR_UNSUPPORTED,
                "only P1/P2 on triangles and tetrahedra");
    AFP_REQUIRE(r->coords && r->cells && r->elem_dof && r->dirichlet && r->f && r->n_dof > 0, AFP_ERR_INVALID,
                "incomplete request");
    auto j = std::make_unique<Job>();
    const int nd = r->dim == 2 ? 3 * r->degree : (r->degree == 1 ? 4 : 10);
    j->dim = r->dim;
    j->degree = r->degree;
    j->acc_stiff = r->acc_stiff;
    j->acc_mass = r->acc_mass;
    j->n_vertex = r->n_vertex;
    j->n_cell = r->n_cell;
    j->n_dof = r->n_dof;
    j->coords.assign(r->coords, r->coords + r->n_vertex * r->dim);
    j->cells.assign(r->cells, r->cells + r->n_cell * (r->dim + 1));
    j->elem_dof.assign(r->elem_dof, r->elem_dof + r->n_cell * nd);
    j->dirichlet.assign(r->dirichlet, r->dirichlet + r->n_dof);
    j->f.assign(r->f, r->f + r->n_dof);
    if (r->coef) j->coef.assign(r->coef, r->coef + r->n_cell);
    j->estimate = estimate_bytes(*j);
    j->t_submit = Clock::now();
    std::lock_guard<std::mutex> lk(s->mu);
    AFP_REQUIRE(!s->stop, AFP_ERR_INVALID, "server is shutting down");
    j->ticket = s->next_ticket++;
    *ticket = j->ticket;
    s->queue.push_back(j.get());
    s->jobs[j->ticket] = std::move(j);
    s->cv_work.notify_all();
  });
}

afp_status afp_server_wait(afp_server* s, int64_t ticket, double* x, afp_request_result* res) {
  return guarded([&] {
    AFP_REQUIRE(s, AFP_ERR_INVALID, "null server");
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->jobs.find(ticket);
    AFP_REQUIRE(it != s->jobs.end(), AFP_ERR_INVALID, "unknown ticket");
    Job* j = it->second.get();
    s->cv_done.wait(lk, [&] { return j->done; });
    if (res) *res = j->result;
    if (x && !j->x.empty()) std::memcpy(x, j->x.data(), sizeof(double) * j->n_dof);
    s->jobs.erase(it);
  });
}

afp_status afp_server_poll(afp_server* s, int64_t ticket, int* done) {
  return guarded([&] {
    AFP_REQUIRE(s && done, AFP_ERR_INVALID, "null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->jobs.find(ticket);
    AFP_REQUIRE(it != s->jobs.end(), AFP_ERR_INVALID, "unknown ticket");
    *done = it->second->done ? 1 : 0;
  });
}

afp_status afp_server_get_stats(afp_server* s, afp_server_stats* st) {
  return guarded([&] {
    AFP_REQUIRE(s && st, AFP_ERR_INVALID, "null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    st->completed = s->completed;
    st->failed = s->failed;
    st->queued = (int64_t)s->queue.size();
    st->p50_seconds = percentile(s->latencies, 50);
    st->p99_seconds = percentile(s->latencies, 99);
    const double span = secs(s->t_start, s->t_last);
    st->solves_per_second = span > 0 ? s->completed / span : 0.0;
    st->budget_bytes = s->budget;
    st->in_use_bytes = s->in_use;
  });
}

afp_status afp_server_reset_stats(afp_server* s) {
  return guarded([&] {
    AFP_REQUIRE(s, AFP_ERR_INVALID, "null server");
    std::lock_guard<std::mutex> lk(s->mu);
    s->latencies.clear();
    s->completed = s->failed = 0;
    s->t_start = s->t_last = Clock::now();
  });
}

afp_status afp_server_destroy(afp_server* s) {
  return guarded([&] {
    if (!s) return;
    {
      std::lock_guard<std::mutex> lk(s->mu);
      s->stop = true;
    }
    s->cv_work.notify_all();
    for (auto& t : s->workers) t.join();
    delete s;
  });
}

}  // extern "C"
