// AMG hierarchy, V-cycle and preconditioned CG (AMGSolver::reinit / solve,
// src/AMGSolver.cpp:384-639, and the CG of
// examples/FAST/src/poisson_solver_comparison_afepack.cpp:197-253).
//
// Setup reproduces the reference hierarchy: per level the host runs the C/F
// splitting (host_project) on the level matrix, the GPU forms P A P^T
// (galerkin_product), and the coarse matrix comes back to the host for the
// next splitting, until the reference's stop rule holds -- or, GB300-side,
// until a level is small enough (opts.dense_tail) to be solved through a
// dense inverse, the reference's own coarsest-level treatment.
//
// For the solve every smoothed level is colour-permuted: rows are grouped by
// greedy colour class so that a Gauss-Seidel class is a contiguous row
// range.  P and P^T are stored explicitly in the permuted numbering, so
// restriction and prolongation are gathers without atomics.  The V-cycle is
// captured once into a CUDA graph and replayed.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <numeric>

#include "amg_internal.cuh"
#include "launch.cuh"

using namespace afp;

namespace afp {
namespace {

// A level of at most kDenseTailMax rows whose matrix is at least
// kDenseTailDensity nonzero becomes the dense tail even above dense_tail
// rows.  Measured on the 2D P2 512^2 hierarchy: the 12,554-row level is 12%
// nonzero and the product that would coarsen it yields a 7,093-row level
// that is 68% nonzero (the reference algorithm spends 411 s of 8-thread CPU
// time on that one product); 3D P1 64^3 and 3D P2 tails are 9-14% nonzero.
constexpr int64_t kDenseTailMax = 16384;
constexpr double kDenseTailDensity = 0.05;


// Setup trace: with AFP_SETUP_TRACE set, each setup step prints its wall
// time (after a stream sync) to stderr.
struct SetupTrace {
  bool on = std::getenv("AFP_SETUP_TRACE") != nullptr;
  std::chrono::steady_clock::time_point t = std::chrono::steady_clock::now();
  void mark(const afp_context* ctx, const char* what, int level, int64_t n, int64_t nnz) {
    if (!on) return;
    sync(ctx);
    const auto now = std::chrono::steady_clock::now();
    std::fprintf(stderr, "[afp setup] level %d (n %lld, nnz %lld) %s: %.3f s\n", level, (long long)n,
                 (long long)nnz, what, std::chrono::duration<double>(now - t).count());
    t = now;
  }
};

void upload_host_csr(const afp_context* ctx, const HostCSR& H, DevCSR& D) {
  D.m = H.m;
  D.n = H.n;
  D.nnz = H.nnz();
  D.rp.alloc(ctx, H.m + 1);
  D.ci.alloc(ctx, D.nnz);
  D.va.alloc(ctx, D.nnz);
  D.rp.upload(H.rowptr.data(), H.m + 1);
  D.ci.upload(H.cols.data(), D.nnz);
  D.va.upload(H.vals.data(), D.nnz);
}

void download_host_csr(const afp_context* ctx, int64_t m, int64_t n, int64_t nnz, const int* rp, const int* ci,
                       const double* va, HostCSR& H) {
  H.m = m;
  H.n = n;
  H.rowptr.resize(m + 1);
  H.cols.resize(nnz);
  H.vals.resize(nnz);
  copy(ctx, H.rowptr.data(), rp, sizeof(int) * (m + 1));
  copy(ctx, H.cols.data(), ci, sizeof(int) * nnz);
  copy(ctx, H.vals.data(), va, sizeof(double) * nnz);
  sync(ctx);
}

template <class X>
X* lvx(afp_amg* h, int l);
template <>
double* lvx<double>(afp_amg* h, int l) {
  return h->lv[l].x.get();
}
template <>
float* lvx<float>(afp_amg* h, int l) {
  return h->lv[l].x32.get();
}
template <class X>
X* lvr(afp_amg* h, int l);
template <>
double* lvr<double>(afp_amg* h, int l) {
  return h->lv[l].r.get();
}
template <>
float* lvr<float>(afp_amg* h, int l) {
  return h->lv[l].r32.get();
}
template <class X>
X* lvt(afp_amg* h, int l);
template <>
double* lvt<double>(afp_amg* h, int l) {
  return h->lv[l].tmp.get();
}
template <>
float* lvt<float>(afp_amg* h, int l) {
  return h->lv[l].tmp32.get();
}
template <class X>
const X* l1(const Level& L);
template <>
const double* l1<double>(const Level& L) {
  return L.l1d.get();
}
template <>
const float* l1<float>(const Level& L) {
  return L.l1d32.get();
}

template <class X>
void smooth(afp_amg* h, int l, X* x, const X* r, bool backward) {
  const Level& L = h->lv[l];
  CSRView<X> A = L.A<X>();
  const int K = (int)L.cls.size() - 1;
  for (int s = 0; s < h->opts.smooth_step; ++s) {
    for (int q = 0; q < K; ++q) {
      const int c = backward ? K - 1 - q : q;
      const int64_t r0 = L.cls[c], r1 = L.cls[c + 1];
      if (L.overflow && c == K - 1)
        jacobi_l1_class<X>(h->ctx, A, r0, r1, x, r, l1<X>(L), lvt<X>(h, l));
      else
        gs_class<X>(h->ctx, A, r0, r1, x, r);
    }
  }
}

// One V-cycle on x0 (level-0 solve order) for right-hand side r0.
template <class X, class PV>
void vcycle(afp_amg* h, X* x0, const X* r0, bool zero_init) {
  const afp_context* ctx = h->ctx;
  const int t = h->t;
  for (int l = 0; l < t; ++l) {
    Level& L = h->lv[l];
    X* x = l == 0 ? x0 : lvx<X>(h, l);
    const X* r = l == 0 ? r0 : lvr<X>(h, l);
    if (l > 0 || zero_init) fill_zero<X>(ctx, L.n, x);
    smooth<X>(h, l, x, r, false);
    residual<X>(ctx, L.A<X>(), x, r, lvt<X>(h, l));
    CSRView<PV> P{h->lv[l + 1].n, L.prp.get(), L.pci.get(), p_vals<PV>(L), L.pvec};
    spmv<PV, X>(ctx, P, lvt<X>(h, l), lvr<X>(h, l + 1), false);
  }
  X* xt = t == 0 ? x0 : lvx<X>(h, t);
  const X* rt = t == 0 ? r0 : lvr<X>(h, t);
  if (h->tail_dense) {
    if constexpr (std::is_same<X, double>::value) dense_gemv<double>(ctx, h->lv[t].n, h->tail_inv.get(), rt, xt);
    else dense_gemv_df(ctx, h->lv[t].n, h->tail_ld, h->tail_hi.get(), h->tail_lo.get(), rt, xt);
  } else {
    diag_solve<X>(ctx, h->lv[t].A<X>(), rt, xt);
  }
  for (int l = t - 1; l >= 0; --l) {
    Level& L = h->lv[l];
    X* x = l == 0 ? x0 : lvx<X>(h, l);
    const X* r = l == 0 ? r0 : lvr<X>(h, l);
    CSRView<PV> T{L.n, L.trp.get(), L.tci.get(), pt_vals<PV>(L), L.tvec};
    spmv<PV, X>(ctx, T, lvx<X>(h, l + 1), x, true);
    smooth<X>(h, l, x, r, h->opts.symmetric != 0);
  }
}

// Mixed-precision V-cycle as the launch chain: FP32 levels, P / P^T in BF16
// or FP32 (opts.interp_bf16).
void vcycle_mixed(afp_amg* h, float* x0, const float* r0) {
  if (h->opts.interp_bf16) vcycle<float, __nv_bfloat16>(h, x0, r0, true);
  else vcycle<float, float>(h, x0, r0, true);
}

// z = V(r) on the solver's level-0 buffers (FP64 in and out): the streamed
// kernel when its plan exists (it converts r and z itself), else the chain.
void vcycle_level0(afp_amg* h) {
  afp_context* ctx = h->ctx;
  const int64_t n = h->lv[0].n;
  if (h->opts.precision != AFP_PRECISION_MIXED) {
    vcycle<double, double>(h, h->z.get(), h->r.get(), true);
  } else if (h->fused) {
    fused_vcycle(h, h->r.get(), h->z.get());
  } else {
    convert<double, float>(ctx, n, h->r.get(), h->r32.get());
    vcycle_mixed(h, h->z32.get(), h->r32.get());
    convert<float, double>(ctx, n, h->z32.get(), h->z.get());
  }
}

// Runs a graph build; if it fails while the streamed V-cycle is in use (a
// graph that cannot hold a cooperative kernel), drops its plan and retries
// with the launch chain.
void drop_fused(afp_amg* h) {
  // graphs captured with the fused kernel refer to the plan's buffers
  if (h->graph32) cudaGraphExecDestroy(h->graph32);
  if (h->loop32) cudaGraphExecDestroy(h->loop32);
  h->graph32 = h->loop32 = nullptr;
  h->fused.reset();
}

template <class F>
void with_chain_fallback(afp_amg* h, F&& build) {
  try {
    build();
  } catch (const Error&) {
    if (!h->fused) throw;
    cudaGetLastError();
    drop_fused(h);
    build();
  }
}

void check_fused(afp_amg* h) {
  if (fused_timed_out(h)) fail(AFP_ERR_TIMEOUT, "streamed V-cycle: a bounded wait ran out");
}

// Captures (once) and replays the preconditioner z = V(r) on the solver's
// own level-0 buffers (r, z).
void precondition(afp_amg* h) {
  afp_context* ctx = h->ctx;
  const bool mixed = h->opts.precision == AFP_PRECISION_MIXED;
  cudaGraphExec_t& exec = mixed ? h->graph32 : h->graph64;
  int64_t& nodes = mixed ? h->graph32_nodes : h->graph64_nodes;
  if (exec == nullptr) {
    with_chain_fallback(h, [&] {
      cudaGraph_t g = nullptr;
      const int64_t before = ctx->launches.n;
      AFP_CUDA(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
      try {
        vcycle_level0(h);
      } catch (...) {
        cudaStreamEndCapture(ctx->stream, &g);
        if (g) cudaGraphDestroy(g);
        ctx->launches.n = before;
        throw;
      }
      const int64_t captured = ctx->launches.n - before;
      ctx->launches.n = before;
      AFP_CUDA(cudaStreamEndCapture(ctx->stream, &g));
      const cudaError_t ie = cudaGraphInstantiate(&exec, g, 0);
      cudaGraphDestroy(g);
      if (ie != cudaSuccess) exec = nullptr;
      AFP_CUDA(ie);
      nodes = captured;
    });
  }
  AFP_CUDA(cudaGraphLaunch(exec, ctx->stream));
  ctx->launches.n += nodes;
}

__global__ void k_abs_residual_sum(int64_t m, const int* __restrict__ rp, const int* __restrict__ ci,
                                   const double* __restrict__ va, const double* __restrict__ x,
                                   const double* __restrict__ r, double* __restrict__ out) {
  // out[i] = |(A x)_i - r_i| (then summed by dot with ones)
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  double s = 0;
  for (int k = rp[i]; k < rp[i + 1]; ++k) s += va[k] * x[ci[k]];
  out[i] = fabs(s - r[i]);
}

__global__ void k_fill(int64_t n, double v, double* __restrict__ x) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) x[i] = v;
}

double l1_residual(afp_amg* h, const double* x, const double* r) {
  afp_context* ctx = h->ctx;
  const Level& L = h->lv[0];
  k_abs_residual_sum<<<grid_for(L.n, 256), 256, 0, ctx->stream>>>(L.n, L.rp.get(), L.ci.get(), L.va.get(), x, r,
                                                                  h->tmp.get());
  check_launch(ctx, "abs residual");
  k_fill<<<grid_for(L.n, 256), 256, 0, ctx->stream>>>(L.n, 1.0, h->q.get());
  check_launch(ctx, "ones");
  dot(ctx, L.n, h->tmp.get(), h->q.get(), ctx->d_scalars + 10);
  double v;
  copy(ctx, &v, ctx->d_scalars + 10, sizeof(double));
  sync(ctx);
  return v;
}

void build_solve_layout(afp_amg* h, std::vector<DevCSR>& refDev, const afp_matrix* A0) {
  afp_context* ctx = h->ctx;
  const int t = h->t;
  const bool mixed = h->opts.precision == AFP_PRECISION_MIXED;
  SetupTrace tr;
  h->lv.resize(t + 1);
  std::vector<std::vector<int>> perm(t + 1), iperm(t + 1);
  for (int l = 0; l <= t; ++l) {
    const HostCSR& H = h->refA[l];
    const int64_t n = H.m;
    perm[l].resize(n);
    iperm[l].resize(n);
    Level& L = h->lv[l];
    L.n = n;
    L.nnz = H.nnz();
    if (l < t) {
      std::vector<int> color;
      const int cap = (l > 0 && h->opts.coarse_colors > 0) ? h->opts.coarse_colors : h->opts.max_colors;
      int K = host_color(H, cap, color);
      const int nclass = K;
      std::vector<int64_t> cnt(nclass + 1, 0);
      for (int64_t i = 0; i < n; ++i) cnt[color[i] + 1]++;
      for (int c = 0; c < nclass; ++c) cnt[c + 1] += cnt[c];
      L.cls.assign(cnt.begin(), cnt.end());
      L.overflow = (K == cap + 1);
      std::vector<int64_t> cur(cnt.begin(), cnt.end() - 1);
      for (int64_t i = 0; i < n; ++i) perm[l][cur[color[i]]++] = (int)i;
    } else {
      std::iota(perm[l].begin(), perm[l].end(), 0);
      L.cls = {0, n};
    }
    for (int64_t i = 0; i < n; ++i) iperm[l][perm[l][i]] = (int)i;
  }
  for (int l = 0; l <= t; ++l) {
    Level& L = h->lv[l];
    const int* rp = l == 0 ? A0->pat->rowptr.get() : refDev[l].rp.get();
    const int* ci = l == 0 ? A0->pat->cols.get() : refDev[l].ci.get();
    const double* va = l == 0 ? A0->vals.get() : refDev[l].va.get();
    DevBuf<int> dperm(ctx, L.n), diperm(ctx, L.n);
    dperm.upload(perm[l].data(), L.n);
    diperm.upload(iperm[l].data(), L.n);
    permute_csr(ctx, L.n, rp, ci, va, dperm.get(), diperm.get(), L.nnz, L.rp, L.ci, L.va);
    L.vec = pick_vec((double)L.nnz / (double)L.n);
    L.perm = std::move(dperm);
    if (l < t && L.overflow) {
      const int K = (int)L.cls.size() - 1;
      const int64_t r0 = L.cls[K - 1], r1 = L.cls[K];
      L.l1d.alloc(ctx, std::max<int64_t>(1, r1 - r0));
      l1_diag(ctx, L.A<double>(), r0, r1, L.l1d.get());
      if (mixed) {
        L.l1d32.alloc(ctx, std::max<int64_t>(1, r1 - r0));
        convert<double, float>(ctx, r1 - r0, L.l1d.get(), L.l1d32.get());
      }
    }
    if (mixed) {
      L.va32.alloc(ctx, L.nnz);
      convert<double, float>(ctx, L.nnz, L.va.get(), L.va32.get());
    }
    L.x.alloc(ctx, L.n);
    L.r.alloc(ctx, L.n);
    L.tmp.alloc(ctx, L.n);
    if (mixed) {
      // four spare zeros: the streamed dense tail reads r in float4 runs up
      // to the tail's padded row length
      L.x32.alloc(ctx, L.n + 4);
      L.r32.alloc(ctx, L.n + 4);
      L.tmp32.alloc(ctx, L.n + 4);
      L.x32.zero();
      L.r32.zero();
      L.tmp32.zero();
    }
    (void)diperm;
  }
  tr.mark(ctx, "colouring + level permutation", t, h->lv[t].n, 0);
  // projections in the permuted numbering
  for (int l = 0; l < t; ++l) {
    Level& L = h->lv[l];
    const HostCSR& P = h->refP[l];
    HostCSR Pt;
    // transpose on the host (cheap: P has few entries per row)
    Pt.m = P.n;
    Pt.n = P.m;
    Pt.rowptr.assign(P.n + 1, 0);
    for (int q = 0; q < P.nnz(); ++q) Pt.rowptr[P.cols[q] + 1]++;
    for (int64_t i = 0; i < P.n; ++i) Pt.rowptr[i + 1] += Pt.rowptr[i];
    Pt.cols.resize(P.nnz());
    Pt.vals.resize(P.nnz());
    {
      std::vector<int> cur(Pt.rowptr.begin(), Pt.rowptr.end() - 1);
      for (int64_t c = 0; c < P.m; ++c)
        for (int q = P.rowptr[c]; q < P.rowptr[c + 1]; ++q) {
          const int k = cur[P.cols[q]]++;
          Pt.cols[k] = (int)c;
          Pt.vals[k] = P.vals[q];
        }
    }
    DevCSR dP, dT;
    upload_host_csr(ctx, P, dP);
    upload_host_csr(ctx, Pt, dT);
    DevBuf<int> pr(ctx, P.m), ic(ctx, P.n), tr(ctx, P.n), itc(ctx, P.m);
    pr.upload(perm[l + 1].data(), P.m);
    ic.upload(iperm[l].data(), P.n);
    tr.upload(perm[l].data(), P.n);
    itc.upload(iperm[l + 1].data(), P.m);
    permute_csr(ctx, P.m, dP.rp.get(), dP.ci.get(), dP.va.get(), pr.get(), ic.get(), P.nnz(), L.prp, L.pci, L.pva);
    permute_csr(ctx, P.n, dT.rp.get(), dT.ci.get(), dT.va.get(), tr.get(), itc.get(), P.nnz(), L.trp, L.tci, L.tva);
    L.pnnz = P.nnz();
    L.pvec = pick_vec((double)P.nnz() / (double)P.m);
    L.tvec = pick_vec((double)P.nnz() / (double)P.n);
    if (mixed && h->opts.interp_bf16) {
      L.pva16.alloc(ctx, P.nnz());
      L.tva16.alloc(ctx, P.nnz());
      convert<double, __nv_bfloat16>(ctx, P.nnz(), L.pva.get(), L.pva16.get());
      convert<double, __nv_bfloat16>(ctx, P.nnz(), L.tva.get(), L.tva16.get());
    } else if (mixed) {
      L.pva32.alloc(ctx, P.nnz());
      L.tva32.alloc(ctx, P.nnz());
      convert<double, float>(ctx, P.nnz(), L.pva.get(), L.pva32.get());
      convert<double, float>(ctx, P.nnz(), L.tva.get(), L.tva32.get());
    }
    sync(ctx);
  }
  tr.mark(ctx, "P / P^T permutation", t, h->lv[t].n, 0);
  // tail
  Level& T = h->lv[t];
  if (h->tail_dense) {
    h->tail_inv.alloc(ctx, T.n * T.n);
    if (!dense_inverse(ctx, T.A<double>(), h->tail_inv.get()))
      fail(AFP_ERR_SINGULAR, "coarsest matrix is singular");
    if (mixed) {
      // FP32 pair with FP64-class accuracy: a plain FP32 inverse summed in
      // FP32 loses the coarse correction on ill-conditioned 3D tails
      h->tail_ld = (T.n + 3) / 4 * 4;
      h->tail_hi.alloc(ctx, T.n * h->tail_ld);
      h->tail_lo.alloc(ctx, T.n * h->tail_ld);
      split_df(ctx, T.n, h->tail_ld, h->tail_inv.get(), h->tail_hi.get(), h->tail_lo.get());
      sync(ctx);
      h->tail_inv = DevBuf<double>();  // the FP64 V-cycle is not used at this precision
    }
  }
  if (mixed && !h->tail_dense) {
    T.va32.alloc(ctx, T.nnz);
    convert<double, float>(ctx, T.nnz, T.va.get(), T.va32.get());
  }
  tr.mark(ctx, "dense tail inverse", t, h->lv[t].n, 0);
  const int64_t n0 = h->lv[0].n;
  h->b.alloc(ctx, n0);
  h->x.alloc(ctx, n0);
  h->r.alloc(ctx, n0);
  h->z.alloc(ctx, n0);
  h->p.alloc(ctx, n0);
  h->q.alloc(ctx, n0);
  h->tmp.alloc(ctx, n0);
  if (mixed) {
    h->r32.alloc(ctx, n0);
    h->z32.alloc(ctx, n0);
  }
  sync(ctx);
  if (mixed && h->opts.fused_vcycle) fused_build(h);
  else h->fused.reset();
}

void setup(afp_amg* h, afp_matrix* A, bool lazy) {
  afp_context* ctx = h->ctx;
  h->lazy = lazy;
  h->pat0 = A->pat;
  const afp_amg_opts& o = h->opts;
  AFP_REQUIRE(A->pat->m == A->pat->n, AFP_ERR_INVALID, "matrix is not square");
  SetupTrace tr;
  HostCSR H0;
  download_host_csr(ctx, A->pat->m, A->pat->n, A->pat->nnz, A->pat->rowptr.get(), A->pat->cols.get(), A->vals.get(),
                    H0);
  h->refA.push_back(std::move(H0));
  std::vector<DevCSR> refDev(1);  // refDev[0] unused: the input matrix
  uint64_t k = (uint64_t)A->pat->m, m = k;
  float sparse_degree = (float)A->pat->nnz / ((float)m * m);
  h->most_full = true;
  int l = 0;
  while (m > (uint64_t)o.max_coarse || sparse_degree < o.min_density) {
    // the dense tail starts here: at most dense_tail rows, or a level already
    // dense enough (coarse levels of 2D P2 / 3D hierarchies) that the next
    // Galerkin product would cost far more than inverting this level
    if (o.dense_tail > 0 && l > 0) {
      const double density = (double)h->refA[l].nnz() / ((double)m * (double)m);
      if (m <= (uint64_t)o.dense_tail || (m <= (uint64_t)kDenseTailMax && density >= kDenseTailDensity)) break;
    }
    const HostCSR& M = h->refA[l];
    const int* arp = l == 0 ? A->pat->rowptr.get() : refDev[l].rp.get();
    const int* aci = l == 0 ? A->pat->cols.get() : refDev[l].ci.get();
    const double* ava = l == 0 ? A->vals.get() : refDev[l].va.get();
    HostCSR P, Pt;
    DevCSR dP, dT;
    tr.mark(ctx, "previous level done", l, M.m, M.nnz());
    if (!lazy && o.gpu_coarsen) {
      GpuProjection g;
      gpu_project(ctx, M.m, arp, aci, ava, o.alpha, g);
      dP = std::move(g.P);
      dT = std::move(g.Pt);
      download_host_csr(ctx, dP.m, dP.n, dP.nnz, dP.rp.get(), dP.ci.get(), dP.va.get(), P);
      if (tr.on)
        std::fprintf(stderr, "[afp setup] level %d: C/F rounds %d + %d\n", l, g.rounds1, g.rounds2);
      tr.mark(ctx, "GPU C/F + P", l, P.m, P.nnz());
    } else {
      std::vector<int> cf;
      if (lazy) host_lazy_project(M, P, Pt);
      else host_project(M, o.alpha, cf, P, Pt);
      tr.mark(ctx, "host C/F + P", l, P.m, P.nnz());
      upload_host_csr(ctx, P, dP);
      upload_host_csr(ctx, Pt, dT);
    }
    Pattern cpat;
    DevBuf<double> cvals;
    // A coarse level that may be the dense tail (by rows, or by density up
    // to kDenseTailMax rows) is formed through the dense product; if it then
    // turns out not to be the tail, the reference-order product is formed
    // after all (the next splitting needs getPMPt's values).  Whether a
    // level above dense_tail rows can reach the density rule is first
    // estimated from the symbolic count of an evenly spaced sample of its
    // rows (with a margin), so that sparse levels never build the
    // n_f x n_c intermediate.
    bool dense_done = false;
    bool try_dense = o.dense_tail > 0 && P.m <= kDenseTailMax;
    if (try_dense && P.m > (int64_t)o.dense_tail) {
      const int64_t ns = std::min<int64_t>(P.m, 256);
      std::vector<int> srp(ns + 1, 0), sci;
      for (int64_t t = 0; t < ns; ++t) {
        const int64_t i = t * P.m / ns;
        sci.insert(sci.end(), P.cols.begin() + P.rowptr[i], P.cols.begin() + P.rowptr[i + 1]);
        srp[t + 1] = (int)sci.size();
      }
      DevBuf<int> drp(ctx, ns + 1), dci(ctx, sci.size());
      drp.upload(srp.data(), ns + 1);
      dci.upload(sci.data(), sci.size());
      const int64_t nnz_s = galerkin_nnz(ctx, ns, P.m, drp.get(), dci.get(), arp, aci, dT.rp.get(), dT.ci.get());
      try_dense = (double)nnz_s / ((double)ns * (double)P.m) >= 0.5 * kDenseTailDensity;
    }
    if (try_dense) {
      galerkin_product_dense(ctx, P.m, P.n, dP.rp.get(), dP.ci.get(), dP.va.get(), arp, aci, ava, dT.rp.get(),
                             dT.ci.get(), dT.va.get(), cpat, cvals);
      const double density = (double)cpat.nnz / ((double)P.m * (double)P.m);
      dense_done = P.m <= o.dense_tail || density >= kDenseTailDensity;
      tr.mark(ctx, dense_done ? "GPU Galerkin product (dense, tail)" : "GPU Galerkin product (dense, discarded)",
              l + 1, cpat.m, cpat.nnz);
    }
    if (!dense_done)
      galerkin_product(ctx, P.m, P.n, dP.rp.get(), dP.ci.get(), dP.va.get(), arp, aci, ava, dT.rp.get(), dT.ci.get(),
                       dT.va.get(), cpat, cvals);
    tr.mark(ctx, "GPU Galerkin product", l + 1, cpat.m, cpat.nnz);
    HostCSR C;
    download_host_csr(ctx, cpat.m, cpat.n, cpat.nnz, cpat.rowptr.get(), cpat.cols.get(), cvals.get(), C);
    m = (uint64_t)C.m;
    if (k == m) {
      h->most_full = false;
      break;
    }
    k = m;
    DevCSR dc;
    dc.m = cpat.m;
    dc.n = cpat.n;
    dc.nnz = cpat.nnz;
    dc.rp = std::move(cpat.rowptr);
    dc.ci = std::move(cpat.cols);
    dc.va = std::move(cvals);
    refDev.push_back(std::move(dc));
    h->refP.push_back(std::move(P));
    if (lazy) h->refPt.push_back(std::move(Pt));
    sparse_degree = (float)C.nnz() / ((float)m * m);
    h->refA.push_back(std::move(C));
    ++l;
  }
  h->n_project = l;
  h->t = l;
  h->tail_dense = h->most_full;
  tr.mark(ctx, "hierarchy done", l, (int64_t)m, 0);
  build_solve_layout(h, refDev, A);
  tr.mark(ctx, "solve layout (colouring, permutation, tail inverse)", h->t, h->lv[h->t].n, 0);
}

// AMGSolver::lazyReinit on an initialised solver (src/AMGSolver.cpp:505-545):
// same projections, new matrix values -- every Galerkin level is recomputed
// on the GPU from the stored P and P^T; no host C/F work.
void lazy_reinit(afp_amg* h, afp_matrix* A) {
  afp_context* ctx = h->ctx;
  AFP_REQUIRE(h->lazy, AFP_ERR_INVALID, "solver was not set up in lazy mode");
  AFP_REQUIRE(A->pat == h->pat0, AFP_ERR_INVALID, "The solver is not initialized with the same sparsity pattern.");
  std::vector<DevCSR> refDev(1);
  HostCSR H0;
  download_host_csr(ctx, A->pat->m, A->pat->n, A->pat->nnz, A->pat->rowptr.get(), A->pat->cols.get(), A->vals.get(),
                    H0);
  h->refA[0] = std::move(H0);
  for (int l = 0; l < h->n_project; ++l) {
    DevCSR dP, dT;
    upload_host_csr(ctx, h->refP[l], dP);
    upload_host_csr(ctx, h->refPt[l], dT);
    const int* arp = l == 0 ? A->pat->rowptr.get() : refDev[l].rp.get();
    const int* aci = l == 0 ? A->pat->cols.get() : refDev[l].ci.get();
    const double* ava = l == 0 ? A->vals.get() : refDev[l].va.get();
    Pattern cpat;
    DevBuf<double> cvals;
    galerkin_product(ctx, dP.m, dP.n, dP.rp.get(), dP.ci.get(), dP.va.get(), arp, aci, ava, dT.rp.get(), dT.ci.get(),
                     dT.va.get(), cpat, cvals);
    HostCSR C;
    download_host_csr(ctx, cpat.m, cpat.n, cpat.nnz, cpat.rowptr.get(), cpat.cols.get(), cvals.get(), C);
    h->refA[l + 1] = std::move(C);
    DevCSR dc;
    dc.m = cpat.m;
    dc.n = cpat.n;
    dc.nnz = cpat.nnz;
    dc.rp = std::move(cpat.rowptr);
    dc.ci = std::move(cpat.cols);
    dc.va = std::move(cvals);
    refDev.push_back(std::move(dc));
  }
  // every captured graph refers to the level buffers rebuilt below
  if (h->graph64) cudaGraphExecDestroy(h->graph64);
  if (h->graph32) cudaGraphExecDestroy(h->graph32);
  if (h->loop64) cudaGraphExecDestroy(h->loop64);
  if (h->loop32) cudaGraphExecDestroy(h->loop32);
  h->graph64 = h->graph32 = h->loop64 = h->loop32 = nullptr;
  h->multi.reset();
  h->lv.clear();
  build_solve_layout(h, refDev, A);
}

void check_finite(double v, const char* what) {
  if (!std::isfinite(v)) fail(AFP_ERR_BREAKDOWN, std::string("non-finite ") + what);
}

// ------------------------------------------------------------------------
// CG as one CUDA graph: the first iteration, then a conditional WHILE node
// whose body is a whole iteration (V-cycle included); a one-thread kernel at
// the end of each iteration sets the loop condition from r.r, so the host
// synchronises once per solve instead of once per iteration.
// Device scalars: s[0] rz, s[1] p.q, s[2] r.r, s[3] rz', s[4] b.b,
// s[6] tol^2 b.b; loopvars = [iterations done, limit].
__global__ void k_pcg_check(const double* __restrict__ s, int* __restrict__ it, cudaGraphConditionalHandle handle) {
  pdl_wait();
  const int k = ++it[0];
  const double rr = s[2];
  const bool cont = (rr > s[6]) && (k < it[1]) && isfinite(rr);
  cudaGraphSetConditional(handle, cont ? 1u : 0u);
}

__global__ void k_copy_scalar(double* s, int from, int to) {
  pdl_wait();
  s[to] = s[from];
}

// z = M r on the solver's level-0 buffers, launched into the current capture
void precondition_inline(afp_amg* h) { vcycle_level0(h); }

void pcg_iteration_tail(afp_amg* h, double* s, cudaGraphConditionalHandle handle) {
  afp_context* ctx = h->ctx;
  const Level& L0 = h->lv[0];
  spmv_dot(ctx, L0.A<double>(), h->p.get(), h->q.get(), s + 1);
  cg_update_xr(ctx, L0.n, s, 0, 1, h->x.get(), h->r.get(), h->p.get(), h->q.get(), s + 2);
  launch_pdl(ctx->stream, 1, 1, 0, k_pcg_check, (const double*)s, h->loopvars.get(), handle);
  check_launch(ctx, "cg check");
}

cudaGraphExec_t& loop_graph(afp_amg* h) {
  afp_context* ctx = h->ctx;
  const int pi = h->opts.precision == AFP_PRECISION_MIXED ? 1 : 0;
  cudaGraphExec_t& exec = pi ? h->loop32 : h->loop64;
  if (exec != nullptr) return exec;
  const int64_t n = h->lv[0].n;
  double* s = ctx->d_scalars;
  if (h->loopvars.size() == 0) h->loopvars.alloc(ctx, 2);
  cudaGraph_t g;
  AFP_CUDA(cudaGraphCreate(&g, 0));
  cudaGraphConditionalHandle handle;
  AFP_CUDA(cudaGraphConditionalHandleCreate(&handle, g, 0, 0));
  const int64_t n0 = ctx->launches.n;
  AFP_CUDA(cudaStreamBeginCaptureToGraph(ctx->stream, g, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
  cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};
  try {
    precondition_inline(h);
    dot(ctx, n, h->r.get(), h->z.get(), s + 0);
    AFP_CUDA(cudaMemcpyAsync(h->p.get(), h->z.get(), sizeof(double) * n, cudaMemcpyDeviceToDevice, ctx->stream));
    pcg_iteration_tail(h, s, handle);
    cudaStreamCaptureStatus st;
    cudaGraph_t cg;
    const cudaGraphNode_t* deps = nullptr;
    size_t nd = 0;
    AFP_CUDA(cudaStreamGetCaptureInfo(ctx->stream, &st, nullptr, &cg, &deps, nullptr, &nd));
    cp.conditional.handle = handle;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t node;
    AFP_CUDA(cudaGraphAddNode(&node, cg, deps, nullptr, nd, &cp));
    AFP_CUDA(cudaStreamUpdateCaptureDependencies(ctx->stream, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
  } catch (...) {
    cudaStreamEndCapture(ctx->stream, &g);
    cudaGraphDestroy(g);
    throw;
  }
  AFP_CUDA(cudaStreamEndCapture(ctx->stream, &g));
  const int64_t n1 = ctx->launches.n;
  cudaGraph_t body = cp.conditional.phGraph_out[0];
  AFP_CUDA(cudaStreamBeginCaptureToGraph(ctx->stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
  try {
    precondition_inline(h);
    dot(ctx, n, h->r.get(), h->z.get(), s + 3);
    cg_update_p(ctx, n, s, 3, 0, h->z.get(), h->p.get());
    launch_pdl(ctx->stream, 1, 1, 0, k_copy_scalar, s, 3, 0);
    check_launch(ctx, "copy scalar");
    pcg_iteration_tail(h, s, handle);
  } catch (...) {
    cudaStreamEndCapture(ctx->stream, &body);
    cudaGraphDestroy(g);
    throw;
  }
  AFP_CUDA(cudaStreamEndCapture(ctx->stream, &body));
  AFP_CUDA(cudaGraphInstantiate(&exec, g, 0));
  AFP_CUDA(cudaGraphDestroy(g));
  h->loop_pre_nodes[pi] = n1 - n0;
  h->loop_body_nodes[pi] = ctx->launches.n - n1;
  ctx->launches.n = n0;
  return exec;
}

void pcg(afp_amg* h, double* x_user, const double* b_user, double tol, int maxit, afp_solve_info* info) {
  afp_context* ctx = h->ctx;
  const Level& L0 = h->lv[0];
  const int64_t n = L0.n;
  double* s = ctx->d_scalars;
  cudaEvent_t e0, e1;
  AFP_CUDA(cudaEventCreate(&e0));
  AFP_CUDA(cudaEventCreate(&e1));
  // inputs into solve order
  copy(ctx, h->tmp.get(), b_user, sizeof(double) * n);
  AFP_CUDA(cudaEventRecord(e0, ctx->stream));
  permute_gather(ctx, n, L0.perm.get(), h->tmp.get(), h->b.get());
  copy(ctx, h->tmp.get(), x_user, sizeof(double) * n);
  permute_gather(ctx, n, L0.perm.get(), h->tmp.get(), h->x.get());
  const CSRView<double> A = L0.A<double>();
  residual<double>(ctx, A, h->x.get(), h->b.get(), h->r.get());
  dot(ctx, n, h->b.get(), h->b.get(), s + 4);
  dot(ctx, n, h->r.get(), h->r.get(), s + 2);
  double hs[5];
  copy(ctx, hs, s, sizeof(double) * 5);
  sync(ctx);
  const double bn = std::max(std::sqrt(hs[4]), 1e-30);
  double rel = std::sqrt(hs[2]) / bn;
  check_finite(rel, "initial residual");
  const double init = rel;
  int it = 0;
  bool conv = rel <= tol;
  static const bool host_loop = std::getenv("AFP_HOST_LOOP") != nullptr;
  if (!conv && maxit > 0 && !host_loop) {
    const int pi = h->opts.precision == AFP_PRECISION_MIXED ? 1 : 0;
    cudaGraphExec_t exec = nullptr;
    with_chain_fallback(h, [&] { exec = loop_graph(h); });
    ctx->h_scalars[0] = tol * tol * hs[4];
    copy(ctx, s + 6, ctx->h_scalars, sizeof(double));
    int lv[2] = {0, maxit};
    h->loopvars.upload(lv, 2);
    AFP_CUDA(cudaGraphLaunch(exec, ctx->stream));
    double rr;
    copy(ctx, &rr, s + 2, sizeof(double));
    h->loopvars.download(lv, 2);
    sync(ctx);
    it = lv[0];
    ctx->launches.n += h->loop_pre_nodes[pi] + (int64_t)(it - 1) * h->loop_body_nodes[pi];
    check_fused(h);  // a V-cycle that gave up leaves z undefined: report that first
    rel = std::sqrt(rr) / bn;
    check_finite(rel, "residual");
    conv = rel <= tol;
  } else if (!conv) {
    precondition(h);  // z = M r
    dot(ctx, n, h->r.get(), h->z.get(), s + 0);
    AFP_CUDA(cudaMemcpyAsync(h->p.get(), h->z.get(), sizeof(double) * n, cudaMemcpyDeviceToDevice, ctx->stream));
    int cur = 0, nxt = 3;
    for (it = 1; it <= maxit; ++it) {
      spmv_dot(ctx, A, h->p.get(), h->q.get(), s + 1);
      cg_update_xr(ctx, n, s, cur, 1, h->x.get(), h->r.get(), h->p.get(), h->q.get(), s + 2);
      double rr;
      copy(ctx, &rr, s + 2, sizeof(double));
      sync(ctx);
      rel = std::sqrt(rr) / bn;
      check_fused(h);
      check_finite(rel, "residual");
      if (rel <= tol) {
        conv = true;
        break;
      }
      precondition(h);
      dot(ctx, n, h->r.get(), h->z.get(), s + nxt);
      cg_update_p(ctx, n, s, nxt, cur, h->z.get(), h->p.get());
      std::swap(cur, nxt);
    }
    if (it > maxit) it = maxit;
  }
  permute_scatter(ctx, n, L0.perm.get(), h->x.get(), h->tmp.get());
  AFP_CUDA(cudaEventRecord(e1, ctx->stream));
  copy(ctx, x_user, h->tmp.get(), sizeof(double) * n);
  sync(ctx);
  check_fused(h);
  float ms = 0;
  AFP_CUDA(cudaEventElapsedTime(&ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (info) {
    info->iterations = it;
    info->converged = conv;
    info->initial_residual = init;
    info->final_residual = rel;
    info->seconds = ms * 1e-3;
  }
  if (!conv)
    fail(AFP_ERR_NOT_CONVERGED, "CG reached its iteration limit (" + std::to_string(maxit) +
                                    ") above the tolerance; x holds the last iterate");
}

}  // namespace
}  // namespace afp

extern "C" {

void afp_amg_default_opts(afp_amg_opts* o) {
  if (!o) return;
  o->tolerance = 1.0e-12;
  o->smooth_step = 3;
  o->max_coarse = 50;
  o->min_density = 0.382;
  o->alpha = 0.25;
  o->precision = AFP_PRECISION_FP64;
  o->dense_tail = 4096;
  o->max_colors = 32;
  o->symmetric = 1;
  o->coarse_colors = 4;
  o->interp_bf16 = 0;
  o->fused_vcycle = 0;
  o->wait_limit_s = 2.0;
  o->inject_barrier_stall = 0;
  o->gpu_coarsen = 1;
}

afp_status afp_amg_setup(afp_matrix* a, const afp_amg_opts* opts, afp_amg** out) {
  return guarded([&] {
    AFP_REQUIRE(a && out, AFP_ERR_INVALID, "null argument");
    bind(a->ctx);
    auto h = std::make_unique<afp_amg>();
    h->ctx = a->ctx;
    if (opts) h->opts = *opts;
    else afp_amg_default_opts(&h->opts);
    const afp_amg_opts& o = h->opts;
    AFP_REQUIRE(o.smooth_step >= 0 && o.max_coarse >= 1 && o.alpha >= 0 && o.max_colors >= 1 && o.dense_tail >= 0 &&
                    (o.precision == AFP_PRECISION_FP64 || o.precision == AFP_PRECISION_MIXED) &&
                    o.wait_limit_s > 0 && o.wait_limit_s <= 60 && (o.gpu_coarsen == 0 || o.gpu_coarsen == 1),
                AFP_ERR_INVALID, "invalid AMG options");
    AFP_REQUIRE(o.dense_tail <= 16384, AFP_ERR_UNSUPPORTED, "dense_tail above 16384 rows");
    setup(h.get(), a, false);
    *out = h.release();
  });
}

afp_status afp_amg_setup_lazy(afp_matrix* a, const afp_amg_opts* opts, afp_amg** out) {
  return guarded([&] {
    AFP_REQUIRE(a && out, AFP_ERR_INVALID, "null argument");
    bind(a->ctx);
    auto h = std::make_unique<afp_amg>();
    h->ctx = a->ctx;
    if (opts) h->opts = *opts;
    else afp_amg_default_opts(&h->opts);
    setup(h.get(), a, true);
    *out = h.release();
  });
}

afp_status afp_amg_lazy_reinit(afp_amg* h, afp_matrix* a) {
  return guarded([&] {
    AFP_REQUIRE(h && a, AFP_ERR_INVALID, "null argument");
    bind(h->ctx);
    lazy_reinit(h, a);
  });
}

afp_status afp_amg_destroy(afp_amg* h) {
  return guarded([&] {
    if (!h) return;
    bind(h->ctx);
    sync(h->ctx);
    delete h;
  });
}

afp_status afp_amg_num_levels(const afp_amg* h, int* n_project, int* solve_levels) {
  return guarded([&] {
    AFP_REQUIRE(h, AFP_ERR_INVALID, "null solver");
    if (n_project) *n_project = h->n_project;
    if (solve_levels) *solve_levels = h->t + 1;
  });
}

afp_status afp_amg_level_info(const afp_amg* h, int level, int64_t* n, int64_t* nnz, int* colors) {
  return guarded([&] {
    AFP_REQUIRE(h && level >= 0 && level <= h->t, AFP_ERR_INVALID, "bad level");
    const Level& L = h->lv[level];
    if (n) *n = L.n;
    if (nnz) *nnz = L.nnz;
    if (colors) *colors = level < h->t ? (int)L.cls.size() - 1 : -1;
  });
}

afp_status afp_amg_download_level(const afp_amg* h, int level, int32_t* rowptr, int32_t* cols, double* vals) {
  return guarded([&] {
    AFP_REQUIRE(h && level >= 0 && level <= h->n_project, AFP_ERR_INVALID, "bad level");
    const HostCSR& H = h->refA[level];
    if (rowptr) std::copy(H.rowptr.begin(), H.rowptr.end(), rowptr);
    if (cols) std::copy(H.cols.begin(), H.cols.end(), cols);
    if (vals) std::copy(H.vals.begin(), H.vals.end(), vals);
  });
}

afp_status afp_amg_download_projection(const afp_amg* h, int level, int32_t* rowptr, int32_t* cols, double* vals) {
  return guarded([&] {
    AFP_REQUIRE(h && level >= 0 && level < h->n_project, AFP_ERR_INVALID, "bad level");
    const HostCSR& H = h->refP[level];
    if (rowptr) std::copy(H.rowptr.begin(), H.rowptr.end(), rowptr);
    if (cols) std::copy(H.cols.begin(), H.cols.end(), cols);
    if (vals) std::copy(H.vals.begin(), H.vals.end(), vals);
  });
}

afp_status afp_amg_solve(afp_amg* h, double* x, const double* r, double tol, int64_t step, int mode,
                         afp_solve_info* info) {
  return guarded([&] {
    AFP_REQUIRE(h && x && r && step >= 0, AFP_ERR_INVALID, "bad argument");
    (void)mode;
    afp_context* ctx = h->ctx;
    bind(ctx);
    if (tol == 0.0) tol = h->opts.tolerance;
    const Level& L0 = h->lv[0];
    const int64_t n = L0.n;
    cudaEvent_t e0, e1;
    AFP_CUDA(cudaEventCreate(&e0));
    AFP_CUDA(cudaEventCreate(&e1));
    copy(ctx, h->tmp.get(), r, sizeof(double) * n);
    AFP_CUDA(cudaEventRecord(e0, ctx->stream));
    permute_gather(ctx, n, L0.perm.get(), h->tmp.get(), h->b.get());
    copy(ctx, h->tmp.get(), x, sizeof(double) * n);
    permute_gather(ctx, n, L0.perm.get(), h->tmp.get(), h->x.get());
    const double init = l1_residual(h, h->x.get(), h->b.get());
    for (int64_t it = 0; it <= step; ++it) {
      // x <- x + V(b - A x): the same iterate as a V-cycle started from x
      residual<double>(ctx, L0.A<double>(), h->x.get(), h->b.get(), h->r.get());
      precondition(h);
      axpy(ctx, n, 1.0, h->z.get(), h->x.get());
    }
    const double fin = l1_residual(h, h->x.get(), h->b.get());
    permute_scatter(ctx, n, L0.perm.get(), h->x.get(), h->tmp.get());
    AFP_CUDA(cudaEventRecord(e1, ctx->stream));
    copy(ctx, x, h->tmp.get(), sizeof(double) * n);
    sync(ctx);
    check_fused(h);
    float ms = 0;
    AFP_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (info) {
      info->iterations = (int)(step + 1);
      info->converged = fin < tol * init;
      info->initial_residual = init;
      info->final_residual = fin;
      info->seconds = ms * 1e-3;
    }
  });
}

afp_status afp_amg_time_kernel(afp_amg* h, int kind, int level, int reps, double* ms, double* bytes) {
  return guarded([&] {
    AFP_REQUIRE(h && ms && bytes && reps > 0 && kind >= 0 && kind <= 5, AFP_ERR_INVALID, "bad argument");
    if (kind >= 4) {
      bind(h->ctx);
      time_multi(h, kind, level, reps, ms, bytes);
      return;
    }
    AFP_REQUIRE(level >= 0 && level < std::max(1, h->t), AFP_ERR_INVALID, "level is not a smoothed level");
    afp_context* ctx = h->ctx;
    bind(ctx);
    const bool mixed = h->opts.precision == AFP_PRECISION_MIXED;
    const Level& L = h->lv[level];
    const double v = mixed ? 4.0 : 8.0;
    // inputs: r = 1, x = 0 on the level (level 0 uses the solver's vectors)
    const int64_t n = L.n;
    if (mixed) {
      std::vector<float> one(n, 1.0f);
      copy(ctx, level == 0 ? h->r32.get() : L.r32.get(), one.data(), sizeof(float) * n);
      fill_zero<float>(ctx, n, level == 0 ? h->z32.get() : L.x32.get());
      if (level == 0) {  // the streamed V-cycle reads the FP64 r
        std::vector<double> one64(n, 1.0);
        copy(ctx, h->r.get(), one64.data(), sizeof(double) * n);
        sync(ctx);
      }
    } else {
      std::vector<double> one(n, 1.0);
      copy(ctx, level == 0 ? h->r.get() : L.r.get(), one.data(), sizeof(double) * n);
      fill_zero<double>(ctx, n, level == 0 ? h->z.get() : L.x.get());
    }
    auto unit = [&]() {
      if (kind == 0 || kind == 1) {
        if (mixed) {
          float* x = level == 0 ? h->z32.get() : L.x32.get();
          const float* r = level == 0 ? h->r32.get() : L.r32.get();
          if (kind == 0) {
            afp_amg_opts keep = h->opts;
            h->opts.smooth_step = 1;
            smooth<float>(h, level, x, r, false);
            h->opts = keep;
          } else {
            residual<float>(ctx, L.A<float>(), x, r, L.tmp32.get());
          }
        } else {
          double* x = level == 0 ? h->z.get() : L.x.get();
          const double* r = level == 0 ? h->r.get() : L.r.get();
          if (kind == 0) {
            afp_amg_opts keep = h->opts;
            h->opts.smooth_step = 1;
            smooth<double>(h, level, x, r, false);
            h->opts = keep;
          } else {
            residual<double>(ctx, L.A<double>(), x, r, L.tmp.get());
          }
        }
      } else if (kind == 2) {
        if (mixed && h->fused) fused_vcycle(h, h->r.get(), h->z.get());
        else if (mixed) vcycle_mixed(h, h->z32.get(), h->r32.get());
        else vcycle<double, double>(h, h->z.get(), h->r.get(), true);
      } else {
        spmv<double, double>(ctx, h->lv[0].A<double>(), h->p.get(), h->q.get(), false);
      }
    };
    unit();  // warm
    cudaEvent_t e0, e1;
    AFP_CUDA(cudaEventCreate(&e0));
    AFP_CUDA(cudaEventCreate(&e1));
    AFP_CUDA(cudaEventRecord(e0, ctx->stream));
    for (int i = 0; i < reps; ++i) unit();
    AFP_CUDA(cudaEventRecord(e1, ctx->stream));
    sync(ctx);
    check_fused(h);
    float t = 0;
    AFP_CUDA(cudaEventElapsedTime(&t, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *ms = t / reps;
    if (kind == 2) fused_print_trace(h);  // AFP_VCYCLE_TRACE: per-phase times of the last V-cycle
    const double mat = (double)L.nnz * (v + 4) + 4.0 * (n + 1);
    if (kind == 0) *bytes = mat + 3.0 * n * v;           // read r, x gathers once, write x
    else if (kind == 1) *bytes = mat + 3.0 * n * v;      // read x, r, write out
    else if (kind == 3) *bytes = (double)h->lv[0].nnz * 12 + 4.0 * (h->lv[0].n + 1) + 2.0 * h->lv[0].n * 8;
    else {
      const double s = h->opts.smooth_step, vp = mixed ? (h->opts.interp_bf16 ? 2.0 : 4.0) : 8.0;
      double b = 0;
      for (int l = 0; l < h->t; ++l) {
        const Level& Q = h->lv[l];
        const double m = (double)Q.nnz * (v + 4) + 4.0 * (Q.n + 1);
        b += (2 * s + 1) * m + 2 * s * 3 * Q.n * v + 2 * Q.n * v;
        b += 2.0 * Q.pnnz * (vp + 4) + 4.0 * (h->lv[l + 1].n + 1) + 4.0 * (Q.n + 1) + 3.0 * Q.n * v +
             2.0 * h->lv[l + 1].n * v;
      }
      const double nt = (double)h->lv[h->t].n;
      b += h->tail_dense ? nt * nt * 8.0 : 0.0;  // FP64 inverse, or its FP32 hi + lo pair
      *bytes = b;
    }
  });
}

afp_status afp_amg_precondition(afp_amg* h, double* x, const double* b, int iterate_step) {
  return afp_amg_solve(h, x, b, 0.0, iterate_step, 1, nullptr);
}

afp_status afp_pcg_solve(afp_amg* h, double* x, const double* b, double tol, int maxit, afp_solve_info* info) {
  return guarded([&] {
    AFP_REQUIRE(h && x && b && maxit >= 0 && tol >= 0, AFP_ERR_INVALID, "bad argument");
    bind(h->ctx);
    pcg(h, x, b, tol, maxit, info);
  });
}

afp_status afp_pcg_solve_multi(afp_amg* h, double* X, const double* B, int nrhs, double tol, int maxit,
                               afp_solve_info* info) {
  return guarded([&] {
    AFP_REQUIRE(h && X && B && nrhs > 0, AFP_ERR_INVALID, "bad argument");
    afp_context* ctx = h->ctx;
    bind(ctx);
    const int64_t n = h->lv[0].n;
    bool all = true;
    if (nrhs <= 64) {
      all = pcg_multi(h, X, B, nrhs, tol, maxit, info);
      if (!all) fail(AFP_ERR_NOT_CONVERGED, "a column reached the CG iteration limit above the tolerance");
      return;
    }
    // wider blocks: batches of 64 columns through contiguous staging blocks
    DevBuf<double> bB(ctx, n * 64), bX(ctx, n * 64);
    for (int c0 = 0; c0 < nrhs; c0 += 64) {
      const int kc = std::min(64, nrhs - c0);
      AFP_CUDA(cudaMemcpy2DAsync(bB.get(), kc * sizeof(double), B + c0, nrhs * sizeof(double), kc * sizeof(double), n,
                                 cudaMemcpyDefault, ctx->stream));
      AFP_CUDA(cudaMemcpy2DAsync(bX.get(), kc * sizeof(double), X + c0, nrhs * sizeof(double), kc * sizeof(double), n,
                                 cudaMemcpyDefault, ctx->stream));
      all = pcg_multi(h, bX.get(), bB.get(), kc, tol, maxit, info ? info + c0 : nullptr) && all;
      AFP_CUDA(cudaMemcpy2DAsync(X + c0, nrhs * sizeof(double), bX.get(), kc * sizeof(double), kc * sizeof(double), n,
                                 cudaMemcpyDefault, ctx->stream));
    }
    sync(ctx);
    if (!all) fail(AFP_ERR_NOT_CONVERGED, "a column reached the CG iteration limit above the tolerance");
  });
}

}  // extern "C"
