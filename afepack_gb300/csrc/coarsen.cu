// C/F splitting and projection on the GPU: AMGSolver::Project
// (src/AMGSolver.cpp:18-226) with the reference's flags and P bit for bit.
//
// The reference's two passes are sequential sweeps in row order.  Both have
// a parallel restatement with the same result:
//
// * Pass 1 (lines 39-68) makes row i a C point iff no earlier C point j < i
//   holds i as a strong neighbour in its own row (|a_ji| >= beta_j).  That
//   is the lexicographically first independent set of the graph j -> i
//   (j < i, strong in row j); it is computed in rounds: a row becomes F as
//   soon as one such j is C, and C once all of them are F.  The lowest
//   undecided row decides in every round, so the rounds end; on mesh
//   matrices they number a few times the mesh's grid width.
// * Pass 2 (lines 74-126) promotes an F point i to C when some strong F
//   neighbour k > i has no C point in its row that is also a strong C
//   neighbour of i.  The C points i sees are the pass-1 C points and the
//   promoted strong neighbours j < i.  A promotion of j < i can only add to
//   that set, which can only turn i's answer from "promote" to "keep", so a
//   row that would not be promoted against the pass-1 C points alone is
//   final, and a remaining candidate is decided once its candidate strong
//   neighbours below it are decided.  Again rounds, over the (few) candidates.
// * P and P^T (lines 127-216): every fine row's weights are accumulated by
//   one thread in the reference's order (the same additions into the same
//   entries), so the values are the reference's.
//
// Compiled with -fmad=false: every product and quotient rounds as on the host.
#include <cstdint>

#include "common.cuh"
#include "kernels.cuh"

namespace afp {

namespace {

constexpr int kRoundsPerCheck = 16;

// the reference's strength test: "if (fabs(a) < beta) continue" skips weak entries
__device__ __forceinline__ bool strong(double a, double beta) { return !(fabs(a) < beta); }

// position of column j among the off-diagonal entries of row i ([diag, ascending others]), or -1
__device__ __forceinline__ int find_offd(const int* __restrict__ rp, const int* __restrict__ ci, int i, int j) {
  int lo = rp[i] + 1, hi = rp[i + 1];
  const int end = hi;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (ci[mid] < j) lo = mid + 1;
    else hi = mid;
  }
  return (lo < end && ci[lo] == j) ? lo : -1;
}

// position of column c in a fully ascending row [b, e), or -1
__device__ __forceinline__ int find_sorted(const int* __restrict__ ci, int b, int e, int c) {
  const int end = e;
  while (b < e) {
    const int mid = (b + e) >> 1;
    if (ci[mid] < c) b = mid + 1;
    else e = mid;
  }
  return (b < end && ci[b] == c) ? b : -1;
}

__device__ __forceinline__ int8_t vload(const int8_t* p) { return *(const volatile int8_t*)p; }

// beta_i = alpha * max_j |a_ij| over the off-diagonal entries; one warp per row
__global__ void k_cf_beta(int m, const int* __restrict__ rp, const double* __restrict__ va, double alpha,
                          double* __restrict__ beta) {
  const int i = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (i >= m) return;
  double b = 0.0;
  for (int j = rp[i] + 1 + lane; j < rp[i + 1]; j += 32) {
    const double a = fabs(va[j]);
    b = (a < b) ? b : a;
  }
  for (int o = 16; o > 0; o >>= 1) {
    const double a = __shfl_xor_sync(0xffffffffu, b, o);
    b = (a < b) ? b : a;
  }
  if (lane == 0) beta[i] = b * alpha;
}

// in_edge[e] for an off-diagonal entry e = (i, j), j < i: row j holds i as a
// strong neighbour, so a C point j makes i an F point in pass 1
__global__ void k_cf_in_edges(int m, const int* __restrict__ rp, const int* __restrict__ ci,
                              const double* __restrict__ va, const double* __restrict__ beta,
                              uint8_t* __restrict__ in_edge) {
  const int i = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (i >= m) return;
  for (int e = rp[i] + 1 + lane; e < rp[i + 1]; e += 32) {
    const int j = ci[e];
    uint8_t f = 0;
    if (j < i) {
      const int p = find_offd(rp, ci, j, i);
      f = (p >= 0 && strong(va[p], beta[j])) ? 1 : 0;
    }
    in_edge[e] = f;
  }
}

// one round of pass 1; st: 0 undecided, -1 C, 1 F.  Rows read their lower
// neighbours' states while those may be written in the same round: a state
// only ever leaves 0 once, so a stale read delays a decision but never changes it.
__global__ void k_cf_pass1(int m, const int* __restrict__ rp, const int* __restrict__ ci,
                           const uint8_t* __restrict__ in_edge, int8_t* st, int* undecided) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  bool pending = false;
  if (i < m && vload(st + i) == 0) {
    int8_t out = -1;
    for (int e = rp[i] + 1; e < rp[i + 1]; ++e) {
      const int j = ci[e];
      if (j >= i) break;
      if (!in_edge[e]) continue;
      const int8_t s = vload(st + j);
      if (s == -1) {
        out = 1;
        pending = false;
        break;
      }
      if (s == 0) pending = true;
    }
    if (!pending) st[i] = out;
  }
  if (undecided != nullptr) {
    const unsigned b = __ballot_sync(0xffffffffu, pending);
    if ((threadIdx.x & 31) == 0 && b) atomicAdd(undecided, __popc(b));
  }
}

// Pass 2's test for an F point i (one warp): is there a strong neighbour
// k > i, F after pass 1, whose row has no C point that is also a strong C
// neighbour of i?  C points below i are the pass-1 ones and the promoted
// (s2 == 2); above i only the pass-1 ones count (the reference has not
// reached them yet).  With s2 == nullptr no promotion is counted.
__device__ bool cf_promote(int i, const int* __restrict__ rp, const int* __restrict__ ci,
                           const double* __restrict__ va, const double* __restrict__ beta,
                           const int8_t* __restrict__ st1, const int8_t* s2, int lane) {
  const double bi = beta[i];
  for (int e = rp[i] + 1; e < rp[i + 1]; ++e) {
    const int k = ci[e];
    if (k < i || st1[k] == -1 || !strong(va[e], bi)) continue;
    bool common = false;
    for (int b0 = rp[k] + 1; b0 < rp[k + 1] && !common; b0 += 32) {
      bool hit = false;
      const int j1 = b0 + lane;
      if (j1 < rp[k + 1]) {
        const int k1 = ci[j1];
        bool c = st1[k1] == -1;
        if (!c && s2 != nullptr && k1 < i) c = vload(s2 + k1) == 2;
        if (c) {
          const int p = find_offd(rp, ci, i, k1);
          hit = p >= 0 && strong(va[p], bi);
        }
      }
      common = __any_sync(0xffffffffu, hit);
    }
    if (!common) return true;
  }
  return false;
}

// s2 for every pass-1 F point: 1 (candidate) if it would be promoted against
// the pass-1 C points alone, else 0 (final: promotions below can only add C points)
__global__ void k_cf_pass2_candidates(int m, const int* __restrict__ rp, const int* __restrict__ ci,
                                      const double* __restrict__ va, const double* __restrict__ beta,
                                      const int8_t* __restrict__ st1, int8_t* __restrict__ s2) {
  const int i = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (i >= m) return;
  bool cand = false;
  if (st1[i] == 1) cand = cf_promote(i, rp, ci, va, beta, st1, nullptr, lane);
  if (lane == 0) s2[i] = cand ? 1 : 0;
}

// one round of pass 2 over the candidates (s2 == 1); s2 becomes 2 (promoted)
// or 0 once every candidate strong neighbour below i is decided
__global__ void k_cf_pass2_round(int m, const int* __restrict__ rp, const int* __restrict__ ci,
                                 const double* __restrict__ va, const double* __restrict__ beta,
                                 const int8_t* __restrict__ st1, int8_t* s2, int* undecided) {
  const int i = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (i >= m || vload(s2 + i) != 1) return;
  const double bi = beta[i];
  bool wait = false;
  for (int e = rp[i] + 1 + lane; e < rp[i + 1]; e += 32) {
    const int j = ci[e];
    if (j < i && strong(va[e], bi) && vload(s2 + j) == 1) wait = true;
  }
  if (__any_sync(0xffffffffu, wait)) {
    if (lane == 0 && undecided != nullptr) atomicAdd(undecided, 1);
    return;
  }
  const bool p = cf_promote(i, rp, ci, va, beta, st1, s2, lane);
  if (lane == 0) s2[i] = p ? 2 : 0;
}

__global__ void k_cf_flags(int m, const int8_t* __restrict__ st1, const int8_t* __restrict__ s2,
                           int* __restrict__ is_c) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < m) is_c[i] = (st1[i] == -1 || s2[i] == 2) ? 1 : 0;
}

// core_point[c] = i for the C points in ascending order (core_at = scan of is_c)
__global__ void k_cf_core_points(int m, const int* __restrict__ is_c, const int* __restrict__ core_at,
                                 int* __restrict__ core_point) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < m && is_c[i]) core_point[core_at[i]] = i;
}

// P row c: the core point k and the non-C points of its row, ascending
__global__ void k_cf_p_len(int nc, const int* __restrict__ rp, const int* __restrict__ ci,
                           const int* __restrict__ core_point, const int* __restrict__ is_c, int* __restrict__ len) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  const int k = core_point[c];
  int n = 1;
  for (int e = rp[k] + 1; e < rp[k + 1]; ++e) n += !is_c[ci[e]];
  len[c] = n;
}

__global__ void k_cf_p_fill(int nc, const int* __restrict__ rp, const int* __restrict__ ci,
                            const int* __restrict__ core_point, const int* __restrict__ is_c,
                            const int* __restrict__ p_rp, int* __restrict__ p_ci, int* __restrict__ pt_len) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  const int k = core_point[c];
  int q = p_rp[c];
  bool placed = false;
  for (int e = rp[k] + 1; e < rp[k + 1]; ++e) {
    const int l = ci[e];
    if (is_c[l]) continue;
    if (!placed && l > k) {
      p_ci[q++] = k;
      placed = true;
    }
    p_ci[q++] = l;
    atomicAdd(pt_len + l, 1);
  }
  if (!placed) p_ci[q++] = k;
  atomicAdd(pt_len + k, 1);
}

// P^T pattern: counted, filled in any order, then each row sorted (the rows
// are short) -- the result does not depend on the order of the fill
__global__ void k_cf_pt_fill(int nc, const int* __restrict__ p_rp, const int* __restrict__ p_ci,
                             int* __restrict__ cursor, int* __restrict__ pt_ci) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  for (int q = p_rp[c]; q < p_rp[c + 1]; ++q) pt_ci[atomicAdd(cursor + p_ci[q], 1)] = c;
}

__global__ void k_cf_pt_sort(int m, const int* __restrict__ pt_rp, int* __restrict__ pt_ci) {
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= m) return;
  const int b = pt_rp[l], e = pt_rp[l + 1];
  for (int q = b + 1; q < e; ++q) {
    const int v = pt_ci[q];
    int r = q - 1;
    while (r >= b && pt_ci[r] > v) {
      pt_ci[r + 1] = pt_ci[r];
      --r;
    }
    pt_ci[r + 1] = v;
  }
}

// a_lc[q] = M(l, core_point[c]) for the P^T entry q = (l, c)
__global__ void k_cf_a_lc(int m, const int* __restrict__ rp, const int* __restrict__ ci, const double* __restrict__ va,
                          const int* __restrict__ pt_rp, const int* __restrict__ pt_ci,
                          const int* __restrict__ core_point, double* __restrict__ a_lc) {
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= m) return;
  for (int q = pt_rp[l]; q < pt_rp[l + 1]; ++q) {
    const int k = core_point[pt_ci[q]];
    double a = 0.0;
    if (rp[l] < rp[l + 1] && ci[rp[l]] == k) a = va[rp[l]];
    else {
      const int p = find_offd(rp, ci, l, k);
      if (p >= 0) a = va[p];
    }
    a_lc[q] = a;
  }
}

// P^T values of fine row i, one thread per row, in the reference's order
__global__ void k_cf_weights(int m, const int* __restrict__ rp, const int* __restrict__ ci,
                             const double* __restrict__ va, const double* __restrict__ beta,
                             const int* __restrict__ is_c, const int* __restrict__ core_at,
                             const int* __restrict__ pt_rp, const int* __restrict__ pt_ci,
                             const double* __restrict__ a_lc, double* __restrict__ pt_va) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  const int tb = pt_rp[i], te = pt_rp[i + 1];
  if (is_c[i]) {
    const int q = find_sorted(pt_ci, tb, te, core_at[i]);
    if (q >= 0) pt_va[q] += 1.0;
    return;
  }
  const double bi = beta[i];
  double aii = rp[i] < rp[i + 1] ? va[rp[i]] : 0.0;
  for (int e = rp[i] + 1; e < rp[i + 1]; ++e)
    if (fabs(va[e]) < bi) aii += va[e];
  for (int e = rp[i] + 1; e < rp[i + 1]; ++e) {
    const int l = ci[e];
    if (fabs(va[e]) < bi) continue;
    if (is_c[l]) {
      const int q = find_sorted(pt_ci, tb, te, core_at[l]);
      if (q >= 0) pt_va[q] += fabs(va[e] / aii);
    } else {
      double d = 0.0;
      for (int i1 = pt_rp[l]; i1 < pt_rp[l + 1]; ++i1)
        if (find_sorted(pt_ci, tb, te, pt_ci[i1]) >= 0) d += a_lc[i1];
      if (fabs(d * aii) < 1e-16) continue;
      for (int i1 = pt_rp[l]; i1 < pt_rp[l + 1]; ++i1) {
        const int q = find_sorted(pt_ci, tb, te, pt_ci[i1]);
        if (q >= 0) pt_va[q] += fabs(va[e] * a_lc[i1] / (d * aii));
      }
    }
  }
}

// P(c, i) received the same additions as P^T(i, c)
__global__ void k_cf_p_vals(int nc, const int* __restrict__ p_rp, const int* __restrict__ p_ci,
                            const int* __restrict__ pt_rp, const int* __restrict__ pt_ci,
                            const double* __restrict__ pt_va, double* __restrict__ p_va) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  for (int q = p_rp[c]; q < p_rp[c + 1]; ++q) {
    const int i = p_ci[q];
    const int t = find_sorted(pt_ci, pt_rp[i], pt_rp[i + 1], c);
    p_va[q] = t >= 0 ? pt_va[t] : 0.0;
  }
}

// launches `launch(counter)` in batches, the last of each batch counting the
// rows left; returns the number of rounds run
template <class F>
int run_rounds(const afp_context* ctx, int m, DevBuf<int>& counter, F launch, const char* what) {
  int rounds = 0;
  for (;;) {
    counter.zero();
    for (int r = 0; r < kRoundsPerCheck; ++r) launch(r + 1 == kRoundsPerCheck ? counter.get() : nullptr);
    rounds += kRoundsPerCheck;
    check_launch(ctx, what);
    int left = 0;
    copy(ctx, &left, counter.get(), sizeof(int));
    sync(ctx);
    if (left == 0) return rounds;
    // the lowest undecided row decides in every round
    if (rounds > m + kRoundsPerCheck) fail(AFP_ERR_CUDA, std::string(what) + ": rounds did not settle");
  }
}

}  // namespace

int gpu_project(const afp_context* ctx, int64_t m64, const int* rp, const int* ci, const double* va, double alpha,
                GpuProjection& out) {
  const int m = (int)m64;
  const cudaStream_t s = ctx->stream;
  int nnz = 0;
  copy(ctx, &nnz, rp + m, sizeof(int));
  sync(ctx);
  const unsigned warp_grid = grid_for((int64_t)m * 32, 256);
  DevBuf<double> beta(ctx, m);
  DevBuf<uint8_t> in_edge(ctx, nnz > 0 ? nnz : 1);
  DevBuf<int8_t> st1(ctx, m), s2(ctx, m);
  DevBuf<int> counter(ctx, 1);
  k_cf_beta<<<warp_grid, 256, 0, s>>>(m, rp, va, alpha, beta.get());
  k_cf_in_edges<<<warp_grid, 256, 0, s>>>(m, rp, ci, va, beta.get(), in_edge.get());
  st1.zero();
  out.rounds1 = run_rounds(
      ctx, m, counter,
      [&](int* cnt) { k_cf_pass1<<<grid_for(m, 256), 256, 0, s>>>(m, rp, ci, in_edge.get(), st1.get(), cnt); },
      "C/F pass 1");
  k_cf_pass2_candidates<<<warp_grid, 256, 0, s>>>(m, rp, ci, va, beta.get(), st1.get(), s2.get());
  out.rounds2 = run_rounds(
      ctx, m, counter,
      [&](int* cnt) {
        k_cf_pass2_round<<<warp_grid, 256, 0, s>>>(m, rp, ci, va, beta.get(), st1.get(), s2.get(), cnt);
      },
      "C/F pass 2");
  DevBuf<int> is_c(ctx, m), core_at(ctx, m + 1);
  k_cf_flags<<<grid_for(m, 256), 256, 0, s>>>(m, st1.get(), s2.get(), is_c.get());
  const int nc = (int)exclusive_scan(ctx, is_c.get(), core_at.get(), m);
  out.cf.alloc(ctx, m);
  AFP_CUDA(cudaMemcpyAsync(out.cf.get(), is_c.get(), sizeof(int) * m, cudaMemcpyDeviceToDevice, s));
  DevBuf<int> core_point(ctx, nc > 0 ? nc : 1);
  k_cf_core_points<<<grid_for(m, 256), 256, 0, s>>>(m, is_c.get(), core_at.get(), core_point.get());

  DevCSR& P = out.P;
  DevCSR& T = out.Pt;
  P.m = nc;
  P.n = m;
  T.m = m;
  T.n = nc;
  DevBuf<int> plen(ctx, nc > 0 ? nc : 1);
  k_cf_p_len<<<grid_for(nc, 256), 256, 0, s>>>(nc, rp, ci, core_point.get(), is_c.get(), plen.get());
  P.rp.alloc(ctx, nc + 1);
  P.nnz = exclusive_scan(ctx, plen.get(), P.rp.get(), nc);
  P.ci.alloc(ctx, P.nnz);
  DevBuf<int> tlen(ctx, m);
  tlen.zero();
  k_cf_p_fill<<<grid_for(nc, 256), 256, 0, s>>>(nc, rp, ci, core_point.get(), is_c.get(), P.rp.get(), P.ci.get(),
                                                tlen.get());
  T.rp.alloc(ctx, m + 1);
  T.nnz = exclusive_scan(ctx, tlen.get(), T.rp.get(), m);
  T.ci.alloc(ctx, T.nnz);
  DevBuf<int> cursor(ctx, m);
  AFP_CUDA(cudaMemcpyAsync(cursor.get(), T.rp.get(), sizeof(int) * m, cudaMemcpyDeviceToDevice, s));
  k_cf_pt_fill<<<grid_for(nc, 256), 256, 0, s>>>(nc, P.rp.get(), P.ci.get(), cursor.get(), T.ci.get());
  k_cf_pt_sort<<<grid_for(m, 128), 128, 0, s>>>(m, T.rp.get(), T.ci.get());
  DevBuf<double> a_lc(ctx, T.nnz > 0 ? T.nnz : 1);
  k_cf_a_lc<<<grid_for(m, 128), 128, 0, s>>>(m, rp, ci, va, T.rp.get(), T.ci.get(), core_point.get(), a_lc.get());
  T.va.alloc(ctx, T.nnz);
  T.va.zero();
  k_cf_weights<<<grid_for(m, 128), 128, 0, s>>>(m, rp, ci, va, beta.get(), is_c.get(), core_at.get(), T.rp.get(),
                                                T.ci.get(), a_lc.get(), T.va.get());
  P.va.alloc(ctx, P.nnz);
  k_cf_p_vals<<<grid_for(nc, 128), 128, 0, s>>>(nc, P.rp.get(), P.ci.get(), T.rp.get(), T.ci.get(), T.va.get(),
                                                P.va.get());
  check_launch(ctx, "GPU C/F splitting");
  return nc;
}

}  // namespace afp
