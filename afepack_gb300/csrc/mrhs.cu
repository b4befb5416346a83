// Batched multi-right-hand-side V-cycle and CG: k systems with one matrix
// and hierarchy, all advanced by the same launches.
//
// Blocks are n x k row-major (the k values of one DOF are contiguous).  Every
// row kernel gives a matrix row to one warp whose lanes own the columns: a
// stored entry a_ij is read once and applied to all k columns of row j of the
// block, a 128/256-byte coalesced segment.  Relative to k single solves the
// matrix traffic drops k-fold and the arithmetic per matrix byte grows k-fold.
//
// CG keeps its recurrences per column: column scalars live on the device, a
// column stops updating once its relative residual meets the tolerance, and
// the iteration ends when every column has.
#include <cmath>

#include "amg_internal.cuh"
#include "df32.cuh"

namespace afp {
namespace {

constexpr int BLK = 256;
constexpr int WPB = BLK / 32;
constexpr int MAXK = 64;
constexpr int RED_GRID = 304;

template <class X>
struct AccT {
  using type = float;
};
template <>
struct AccT<double> {
  using type = double;
};
template <class A, class V>
__device__ __forceinline__ A as(V v) {
  return (A)v;
}
template <>
__device__ __forceinline__ float as<float, __nv_bfloat16>(__nv_bfloat16 v) {
  return __bfloat162float(v);
}

__device__ __forceinline__ int64_t warp_id() { return ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; }
__device__ __forceinline__ int64_t n_warps() { return ((int64_t)gridDim.x * blockDim.x) >> 5; }

template <class X>
__global__ void k_copy(int64_t n, const X* __restrict__ s, X* __restrict__ d) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) d[i] = s[i];
}

template <int KPL, class X>
__global__ void k_dense_gemm(int64_t n, const X* __restrict__ M, const X* __restrict__ r, X* __restrict__ x, int k) {
  using A = typename AccT<X>::type;
  const int lane = threadIdx.x & 31;
  for (int64_t row = warp_id(); row < n; row += n_warps()) {
    A acc[KPL];
#pragma unroll
    for (int q = 0; q < KPL; ++q) acc[q] = 0;
    for (int64_t j = 0; j < n; ++j) {
      const A a = (A)M[row * n + j];
#pragma unroll
      for (int q = 0; q < KPL; ++q) {
        const int c = lane + 32 * q;
        if (c < k) acc[q] += a * (A)r[j * k + c];
      }
    }
#pragma unroll
    for (int q = 0; q < KPL; ++q) {
      const int c = lane + 32 * q;
      if (c < k) x[row * k + c] = (X)acc[q];
    }
  }
}

// --------------------------------------------------- V-cycle row kernels
// One kernel for every row operation of the batched V-cycle on rows [r0, r1)
// of an n x k block: a sub-warp of W lanes (a power of two, W >= k up to 32)
// takes one row, lane l owning columns l, l + W, ... (KPL of them).  The
// row's (column, value) pairs are loaded W at a time, one per lane, and
// broadcast with shuffles; the gathers of x rows they address are issued four
// entries ahead (unrolled), so a row costs about two dependent memory round
// trips whatever its length.
enum RowOp { RO_SPMM = 0, RO_SPMM_ADD, RO_RES, RO_GS, RO_JAC };

template <int W, int KPL, class V, class X, int OP>
__global__ void k_rows_m(int64_t r0, int64_t r1, const int* __restrict__ rp, const int* __restrict__ ci,
                         const V* __restrict__ va, const X* x, X* y, const X* __restrict__ r,
                         const X* __restrict__ d, int k) {
  using A = typename AccT<X>::type;
  const int64_t row = r0 + ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / W;
  if (row >= r1) return;  // a whole sub-warp leaves together
  const int lane = threadIdx.x & (W - 1);
  const unsigned mask = W >= 32 ? 0xffffffffu : (((1u << W) - 1u) << ((threadIdx.x & 31) & ~(W - 1)));
  A acc[KPL];
#pragma unroll
  for (int q = 0; q < KPL; ++q) acc[q] = 0;
  int b = rp[row];
  const int e = rp[row + 1];
  A diag = 1;
  if (OP == RO_GS) {  // the diagonal is the row's first entry
    diag = as<A>(va[b]);
    ++b;
  }
  if (W == 1) {
#pragma unroll 4
    for (int j = b; j < e; ++j) {
      const A val = as<A>(va[j]);
      const X* xr = x + (int64_t)ci[j] * k;
#pragma unroll
      for (int q = 0; q < KPL; ++q)
        if (q < k) acc[q] += val * (A)xr[q];
    }
  } else {
    for (int base = b; base < e; base += W) {
      const int my = base + lane;
      const int cc = my < e ? ci[my] : 0;
      const A vv = my < e ? as<A>(va[my]) : A(0);
      const int cnt = min(W, e - base);
#pragma unroll 4
      for (int jj = 0; jj < cnt; ++jj) {
        const int col = __shfl_sync(mask, cc, jj, W);
        const A val = __shfl_sync(mask, vv, jj, W);
        const X* xr = x + (int64_t)col * k;
#pragma unroll
        for (int q = 0; q < KPL; ++q) {
          const int c = lane + W * q;
          if (c < k) acc[q] += val * (A)xr[c];
        }
      }
    }
  }
#pragma unroll
  for (int q = 0; q < KPL; ++q) {
    const int c = lane + W * q;
    if (c >= k) continue;
    const int64_t o = row * k + c;
    if (OP == RO_SPMM) y[o] = (X)acc[q];
    else if (OP == RO_SPMM_ADD) y[o] = (X)((A)y[o] + acc[q]);
    else if (OP == RO_RES) y[o] = (X)((A)r[o] - acc[q]);
    else if (OP == RO_GS) y[o] = (X)(((A)r[o] - acc[q]) / diag);
    else y[(row - r0) * k + c] = (X)((A)x[o] + ((A)r[o] - acc[q]) / (A)d[row - r0]);  // RO_JAC into tmp
  }
}

// Launches k_rows_m with W = the smallest power of two >= k (at most 32) and
// KPL = columns per lane.
template <class V, class X, int OP>
void rows_m(const afp_context* ctx, int64_t r0, int64_t r1, const int* rp, const int* ci, const V* va, const X* x,
            X* y, const X* r, const X* d, int k, const char* what) {
  if (r1 <= r0) return;
  auto go = [&](auto Wc, auto Kc) {
    constexpr int W = decltype(Wc)::value, KPL = decltype(Kc)::value;
    k_rows_m<W, KPL, V, X, OP><<<grid_for((r1 - r0) * W, 256), 256, 0, ctx->stream>>>(r0, r1, rp, ci, va, x, y, r, d,
                                                                                     k);
  };
  using I1 = std::integral_constant<int, 1>;
  using I2 = std::integral_constant<int, 2>;
  if (k == 1) go(I1(), I1());
  else if (k == 2) go(std::integral_constant<int, 2>(), I1());
  else if (k <= 4) go(std::integral_constant<int, 4>(), I1());
  else if (k <= 8) go(std::integral_constant<int, 8>(), I1());
  else if (k <= 16) go(std::integral_constant<int, 16>(), I1());
  else if (k <= 32) go(std::integral_constant<int, 32>(), I1());
  else go(std::integral_constant<int, 32>(), I2());
  check_launch(ctx, what);
}

// X = (hi + lo) R for the dense tail: an n x n double-float pair (rows of
// stride ld) times an n x k FP32 block, accumulated in double-float.  A block
// of 256 threads computes TR rows x k columns; R and the rows' hi/lo are
// staged in shared memory TJ columns at a time.  When there are fewer outputs
// than threads, S threads share an output, each taking every S-th inner
// index, and their pairs are summed in a fixed order at the end.
template <int TR>
__global__ void __launch_bounds__(256) k_tail_gemm_df(int64_t n, int64_t ld, const float* __restrict__ hi,
                                                       const float* __restrict__ lo, const float* __restrict__ R,
                                                       float* __restrict__ X, int k) {
  constexpr int BT = 256, TJ = 64, MAXO = TR * MAXK / BT;
  __shared__ float sR[TJ * MAXK];
  __shared__ float sH[TR * TJ], sL[TR * TJ];
  __shared__ float2 red[BT];
  const int64_t row0 = (int64_t)blockIdx.x * TR;
  const int O = TR * k;
  const int S = O >= BT ? 1 : BT / O;
  const int per = BT / S;  // outputs in flight at once
  const int tid = threadIdx.x, ob = tid / S, s = tid % S;
  const bool busy = tid < per * S;
  float sh[MAXO > 0 ? MAXO : 1], sl[MAXO > 0 ? MAXO : 1];
#pragma unroll
  for (int q = 0; q < (MAXO > 0 ? MAXO : 1); ++q) sh[q] = sl[q] = 0.f;
  for (int64_t j0 = 0; j0 < n; j0 += TJ) {  // columns [n, ld) of hi / lo are zeros: stop at n (R has n rows)
    const int tj = (int)(n - j0 < TJ ? n - j0 : TJ);
    __syncthreads();
    for (int t = tid; t < tj * k; t += BT) sR[t] = R[j0 * k + t];
    for (int t = tid; t < TR * TJ; t += BT) {
      const int rr = t / TJ, jj = t % TJ;
      const bool on = row0 + rr < n && jj < tj;
      sH[t] = on ? hi[(row0 + rr) * ld + j0 + jj] : 0.f;
      sL[t] = on ? lo[(row0 + rr) * ld + j0 + jj] : 0.f;
    }
    __syncthreads();
    if (busy) {
#pragma unroll
      for (int q = 0; q < (MAXO > 0 ? MAXO : 1); ++q) {
        const int o = ob + q * per;
        if (o >= O) break;
        const int rr = o / k, c = o % k;
        for (int jj = s; jj < tj; jj += S) df_add_prod(sh[q], sl[q], sH[rr * TJ + jj], sL[rr * TJ + jj], sR[jj * k + c]);
      }
    }
  }
  if (S > 1) {
    red[tid] = make_float2(sh[0], sl[0]);
    __syncthreads();
    if (busy && s == 0 && ob < O) {
      float h = red[tid].x, l = red[tid].y;
      for (int u = 1; u < S; ++u) df_add(h, l, red[tid + u].x, red[tid + u].y);
      const int rr = ob / k, c = ob % k;
      if (row0 + rr < n) X[(row0 + rr) * k + c] = __fadd_rn(h, l);
    }
  } else if (busy) {
#pragma unroll
    for (int q = 0; q < (MAXO > 0 ? MAXO : 1); ++q) {
      const int o = ob + q * per;
      if (o >= O) break;
      const int rr = o / k, c = o % k;
      if (row0 + rr < n) X[(row0 + rr) * k + c] = __fadd_rn(sh[q], sl[q]);
    }
  }
}

template <class X>
__global__ void k_diag_solve_m(int64_t n, const int* __restrict__ rp, const X* __restrict__ va,
                               const X* __restrict__ r, X* __restrict__ x, int k) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n * k) x[t] = r[t] / va[rp[t / k]];
}

template <class A, class B>
__global__ void k_conv(int64_t n, const A* __restrict__ in, B* __restrict__ out) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = (B)in[i];
}

template <class X>
__global__ void k_zero_m(int64_t n, X* __restrict__ x) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) x[i] = (X)0;
}

// out row i = in row perm[i] (gather) or out row perm[i] = in row i (scatter)
__global__ void k_rows_gather(int64_t n, int k, const int* __restrict__ perm, const double* __restrict__ in,
                              int64_t ld_in, double* __restrict__ out) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n * k) return;
  const int64_t i = t / k;
  const int c = (int)(t % k);
  out[t] = in[(int64_t)perm[i] * ld_in + c];
}
__global__ void k_rows_scatter(int64_t n, int k, const int* __restrict__ perm, const double* __restrict__ in,
                               double* __restrict__ out, int64_t ld_out) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n * k) return;
  const int64_t i = t / k;
  const int c = (int)(t % k);
  out[(int64_t)perm[i] * ld_out + c] = in[t];
}

// ------------------------------------------------------ column reductions
// Per-column sums of a.b over n x k blocks; deterministic (block partials,
// last block adds them in block order).
// partials: the batch's [RED_GRID x MAXK] scratch, followed in memory by the
// batch's retire counter (an unsigned in the next double slot)
template <int KPL>
__device__ void col_finish(double (&part)[KPL], int k, double* partials, double* dst) {
  unsigned* retire = reinterpret_cast<unsigned*>(partials + (int64_t)RED_GRID * MAXK);
  __shared__ double sm[WPB][MAXK];
  __shared__ bool last;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < KPL; ++q) {
    const int c = lane + 32 * q;
    if (c < MAXK) sm[w][c] = part[q];
  }
  __syncthreads();
  for (int c = threadIdx.x; c < k; c += blockDim.x) {
    double s = 0;
    for (int ww = 0; ww < WPB; ++ww) s += sm[ww][c];
    partials[(int64_t)blockIdx.x * MAXK + c] = s;
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = (atomicInc(retire, gridDim.x - 1) == gridDim.x - 1);
  __syncthreads();
  if (last) {
    for (int c = threadIdx.x; c < k; c += blockDim.x) {
      double s = 0;
      for (unsigned b = 0; b < gridDim.x; ++b) s += ((volatile double*)partials)[(int64_t)b * MAXK + c];
      dst[c] = s;
    }
  }
}

template <int KPL>
__global__ void k_col_dot(int64_t n, const double* __restrict__ a, const double* __restrict__ b, int k,
                          double* partials, double* dst) {
  const int lane = threadIdx.x & 31;
  double part[KPL];
#pragma unroll
  for (int q = 0; q < KPL; ++q) part[q] = 0;
  for (int64_t row = warp_id(); row < n; row += n_warps()) {
#pragma unroll
    for (int q = 0; q < KPL; ++q) {
      const int c = lane + 32 * q;
      if (c < k) part[q] += a[row * k + c] * b[row * k + c];
    }
  }
  col_finish<KPL>(part, k, partials, dst);
}

template <int KPL>
__global__ void k_spmm_dot(int64_t m, const int* __restrict__ rp, const int* __restrict__ ci,
                           const double* __restrict__ va, const double* __restrict__ p, double* __restrict__ q_out,
                           int k, double* partials, double* dst) {
  const int lane = threadIdx.x & 31;
  double part[KPL];
#pragma unroll
  for (int q = 0; q < KPL; ++q) part[q] = 0;
  for (int64_t row = warp_id(); row < m; row += n_warps()) {
    double acc[KPL];
#pragma unroll
    for (int q = 0; q < KPL; ++q) acc[q] = 0;
    for (int j = rp[row]; j < rp[row + 1]; ++j) {
      const double a = va[j];
      const double* pr = p + (int64_t)ci[j] * k;
#pragma unroll
      for (int q = 0; q < KPL; ++q) {
        const int c = lane + 32 * q;
        if (c < k) acc[q] += a * pr[c];
      }
    }
#pragma unroll
    for (int q = 0; q < KPL; ++q) {
      const int c = lane + 32 * q;
      if (c < k) {
        q_out[row * k + c] = acc[q];
        part[q] += acc[q] * p[row * k + c];
      }
    }
  }
  col_finish<KPL>(part, k, partials, dst);
}

// x += alpha_c p, r -= alpha_c q for active columns; rr_c = r.r
template <int KPL>
__global__ void k_update_xr(int64_t n, int k, const double* __restrict__ num, const double* __restrict__ den,
                            const int* __restrict__ active, double* __restrict__ x, double* __restrict__ r,
                            const double* __restrict__ p, const double* __restrict__ q, double* partials,
                            double* dst) {
  const int lane = threadIdx.x & 31;
  double alpha[KPL], part[KPL];
#pragma unroll
  for (int t = 0; t < KPL; ++t) {
    const int c = lane + 32 * t;
    alpha[t] = (c < k && active[c]) ? num[c] / den[c] : 0.0;
    part[t] = 0;
  }
  for (int64_t row = warp_id(); row < n; row += n_warps()) {
#pragma unroll
    for (int t = 0; t < KPL; ++t) {
      const int c = lane + 32 * t;
      if (c < k) {
        const int64_t o = row * k + c;
        x[o] += alpha[t] * p[o];
        const double rv = r[o] - alpha[t] * q[o];
        r[o] = rv;
        part[t] += rv * rv;
      }
    }
  }
  col_finish<KPL>(part, k, partials, dst);
}

template <int KPL>
__global__ void k_update_p(int64_t n, int k, const double* __restrict__ num, const double* __restrict__ den,
                           const int* __restrict__ active, const double* __restrict__ z, double* __restrict__ p) {
  const int lane = threadIdx.x & 31;
  double beta[KPL];
  bool act[KPL];
#pragma unroll
  for (int t = 0; t < KPL; ++t) {
    const int c = lane + 32 * t;
    act[t] = c < k && active[c];
    beta[t] = act[t] ? num[c] / den[c] : 0.0;
  }
  for (int64_t row = warp_id(); row < n; row += n_warps()) {
#pragma unroll
    for (int t = 0; t < KPL; ++t) {
      const int c = lane + 32 * t;
      if (c < k && act[t]) p[row * k + c] = z[row * k + c] + beta[t] * p[row * k + c];
    }
  }
}

unsigned rows_grid(const afp_context* ctx, int64_t rows) {
  const int64_t want = (rows + WPB - 1) / WPB;
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)ctx->sm_count * 16));
}

template <class F>
void with_kpl(int k, F&& f) {
  if (k <= 32) f(std::integral_constant<int, 1>());
  else f(std::integral_constant<int, 2>());
}

// ---------------------------------------------------------------- V-cycle
template <class X>
X* blk(MultiState& S, int which, int l);
template <>
double* blk<double>(MultiState& S, int which, int l) {
  return (which == 0 ? S.X : which == 1 ? S.R : S.T)[l].get();
}
template <>
float* blk<float>(MultiState& S, int which, int l) {
  return (which == 0 ? S.X32 : which == 1 ? S.R32 : S.T32)[l].get();
}

template <class X, class PV>
void vcycle_m(afp_amg* h, MultiState& S) {
  const afp_context* ctx = h->ctx;
  const int k = S.k, t = h->t;
  auto smooth = [&](int l, X* x, const X* r, bool backward) {
    const Level& L = h->lv[l];
    CSRView<X> A = L.A<X>();
    const int K = (int)L.cls.size() - 1;
    for (int s = 0; s < h->opts.smooth_step; ++s)
      for (int q = 0; q < K; ++q) {
        const int c = backward ? K - 1 - q : q;
        const int64_t r0 = L.cls[c], r1 = L.cls[c + 1];
        if (r1 <= r0) continue;
        if (L.overflow && c == K - 1) {
          const X* d;
          if constexpr (std::is_same<X, double>::value) d = L.l1d.get();
          else d = L.l1d32.get();
          X* tmp = blk<X>(S, 2, l);
          rows_m<X, X, RO_JAC>(ctx, r0, r1, A.rowptr, A.cols, A.vals, x, tmp, r, d, k, "mrhs l1-jacobi");
          k_copy<X><<<grid_for((r1 - r0) * k, BLK), BLK, 0, ctx->stream>>>((r1 - r0) * k, tmp, x + r0 * k);
          check_launch(ctx, "mrhs copy");
        } else {
          rows_m<X, X, RO_GS>(ctx, r0, r1, A.rowptr, A.cols, A.vals, x, x, r, nullptr, k, "mrhs gauss-seidel class");
        }
      }
  };
  for (int l = 0; l < t; ++l) {
    Level& L = h->lv[l];
    X* x = blk<X>(S, 0, l);
    const X* r = blk<X>(S, 1, l);
    k_zero_m<X><<<grid_for(L.n * k, BLK), BLK, 0, ctx->stream>>>(L.n * k, x);
    check_launch(ctx, "mrhs zero");
    smooth(l, x, r, false);
    CSRView<X> A = L.A<X>();
    rows_m<X, X, RO_RES>(ctx, 0, L.n, A.rowptr, A.cols, A.vals, x, blk<X>(S, 2, l), r, nullptr, k, "mrhs residual");
    const int64_t nc = h->lv[l + 1].n;
    rows_m<PV, X, RO_SPMM>(ctx, 0, nc, L.prp.get(), L.pci.get(), p_vals<PV>(L), blk<X>(S, 2, l), blk<X>(S, 1, l + 1),
                           nullptr, nullptr, k, "mrhs restriction");
  }
  const Level& T = h->lv[t];
  if (h->tail_dense) {
    if constexpr (std::is_same<X, double>::value) {
      with_kpl(k, [&](auto KPLc) {
        constexpr int KPL = decltype(KPLc)::value;
        k_dense_gemm<KPL, X><<<rows_grid(ctx, T.n), BLK, 0, ctx->stream>>>(T.n, h->tail_inv.get(), blk<X>(S, 1, t),
                                                                          blk<X>(S, 0, t), k);
      });
    } else {
      constexpr int TR = 16;
      k_tail_gemm_df<TR><<<(unsigned)((T.n + TR - 1) / TR), 256, 0, ctx->stream>>>(
          T.n, h->tail_ld, h->tail_hi.get(), h->tail_lo.get(), blk<X>(S, 1, t), blk<X>(S, 0, t), k);
    }
    check_launch(ctx, "mrhs dense tail");
  } else {
    CSRView<X> A = T.A<X>();
    k_diag_solve_m<X><<<grid_for(T.n * k, BLK), BLK, 0, ctx->stream>>>(T.n, A.rowptr, A.vals, blk<X>(S, 1, t),
                                                                       blk<X>(S, 0, t), k);
    check_launch(ctx, "mrhs diagonal tail");
  }
  for (int l = t - 1; l >= 0; --l) {
    Level& L = h->lv[l];
    rows_m<PV, X, RO_SPMM_ADD>(ctx, 0, L.n, L.trp.get(), L.tci.get(), pt_vals<PV>(L), blk<X>(S, 0, l + 1),
                               blk<X>(S, 0, l), nullptr, nullptr, k, "mrhs prolongation");
    smooth(l, blk<X>(S, 0, l), blk<X>(S, 1, l), h->opts.symmetric != 0);
  }
}

void ensure_state(afp_amg* h, int k) {
  const bool mixed = h->opts.precision == AFP_PRECISION_MIXED;
  if (h->multi && h->multi->k == k && h->multi->mixed == mixed) return;
  afp_context* ctx = h->ctx;
  auto S = std::make_unique<MultiState>();
  S->k = k;
  S->mixed = mixed;
  const int L = h->t + 1;
  if (mixed) {
    S->X32.resize(L);
    S->R32.resize(L);
    S->T32.resize(L);
  } else {
    S->X.resize(L);
    S->R.resize(L);
    S->T.resize(L);
  }
  for (int l = 0; l < L; ++l) {
    const int64_t nk = h->lv[l].n * k;
    if (mixed) {
      S->X32[l].alloc(ctx, nk);
      S->R32[l].alloc(ctx, nk);
      S->T32[l].alloc(ctx, nk);
    } else {
      S->X[l].alloc(ctx, nk);
      S->R[l].alloc(ctx, nk);
      S->T[l].alloc(ctx, nk);
    }
  }
  const int64_t n0k = h->lv[0].n * k;
  S->B.alloc(ctx, n0k);
  S->Xs.alloc(ctx, n0k);
  S->Rs.alloc(ctx, n0k);
  S->Z.alloc(ctx, n0k);
  S->P.alloc(ctx, n0k);
  S->Q.alloc(ctx, n0k);
  S->Tmp.alloc(ctx, n0k);
  S->scal.alloc(ctx, 8 * MAXK + (int64_t)RED_GRID * MAXK + 1);  // scalars, partials, retire counter
  S->scal.zero();
  S->active.alloc(ctx, MAXK);
  h->multi = std::move(S);
}

// Z = V(R) for all columns, through a captured graph.
void precondition_m(afp_amg* h) {
  afp_context* ctx = h->ctx;
  MultiState& S = *h->multi;
  const int64_t n0k = h->lv[0].n * S.k;
  if (S.graph == nullptr) {
    cudaGraph_t g;
    const int64_t before = ctx->launches.n;
    AFP_CUDA(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    try {
      if (S.mixed) {
        k_conv<double, float><<<grid_for(n0k, BLK), BLK, 0, ctx->stream>>>(n0k, S.Rs.get(), S.R32[0].get());
        check_launch(ctx, "mrhs to fp32");
        if (h->opts.interp_bf16) vcycle_m<float, __nv_bfloat16>(h, S);
        else vcycle_m<float, float>(h, S);
        k_conv<float, double><<<grid_for(n0k, BLK), BLK, 0, ctx->stream>>>(n0k, S.X32[0].get(), S.Z.get());
        check_launch(ctx, "mrhs to fp64");
      } else {
        k_copy<double><<<grid_for(n0k, BLK), BLK, 0, ctx->stream>>>(n0k, S.Rs.get(), S.R[0].get());
        check_launch(ctx, "mrhs copy r");
        vcycle_m<double, double>(h, S);
        k_copy<double><<<grid_for(n0k, BLK), BLK, 0, ctx->stream>>>(n0k, S.X[0].get(), S.Z.get());
        check_launch(ctx, "mrhs copy z");
      }
    } catch (...) {
      cudaStreamEndCapture(ctx->stream, &g);
      throw;
    }
    AFP_CUDA(cudaStreamEndCapture(ctx->stream, &g));
    AFP_CUDA(cudaGraphInstantiate(&S.graph, g, 0));
    AFP_CUDA(cudaGraphDestroy(g));
    S.graph_nodes = ctx->launches.n - before;
    ctx->launches.n = before;
  }
  AFP_CUDA(cudaGraphLaunch(S.graph, ctx->stream));
  ctx->launches.n += S.graph_nodes;
}

}  // namespace

// Batched CG over up to 64 columns (callers chunk wider blocks).
bool pcg_multi(afp_amg* h, double* X_user, const double* B_user, int nrhs, double tol, int maxit,
               afp_solve_info* info) {
  afp_context* ctx = h->ctx;
  const int k = nrhs;
  AFP_REQUIRE(k >= 1 && k <= MAXK, AFP_ERR_INVALID, "at most 64 columns per batch");
  ensure_state(h, k);
  MultiState& S = *h->multi;
  const Level& L0 = h->lv[0];
  const int64_t n = L0.n, nk = n * k;
  double* sc = S.scal.get();  // rows: 0 rz_a, 1 pq, 2 rr, 3 rz_b, 4 bb
  double* partials = sc + 8 * MAXK;
  cudaEvent_t e0, e1;
  AFP_CUDA(cudaEventCreate(&e0));
  AFP_CUDA(cudaEventCreate(&e1));
  // inputs into solve order (caller's arrays may be host or device)
  copy(ctx, S.Tmp.get(), B_user, sizeof(double) * nk);
  AFP_CUDA(cudaEventRecord(e0, ctx->stream));
  k_rows_gather<<<grid_for(nk, BLK), BLK, 0, ctx->stream>>>(n, k, L0.perm.get(), S.Tmp.get(), k, S.B.get());
  check_launch(ctx, "mrhs gather b");
  copy(ctx, S.Tmp.get(), X_user, sizeof(double) * nk);
  k_rows_gather<<<grid_for(nk, BLK), BLK, 0, ctx->stream>>>(n, k, L0.perm.get(), S.Tmp.get(), k, S.Xs.get());
  check_launch(ctx, "mrhs gather x");
  std::vector<int> act(k, 1);
  S.active.upload(act.data(), k);
  const CSRView<double> A = L0.A<double>();
  const unsigned rg = std::min<unsigned>(RED_GRID, rows_grid(ctx, n));
  rows_m<double, double, RO_RES>(ctx, 0, n, A.rowptr, A.cols, A.vals, S.Xs.get(), S.Rs.get(), S.B.get(), nullptr, k,
                                 "mrhs residual");
  with_kpl(k, [&](auto KPLc) {
    constexpr int KPL = decltype(KPLc)::value;
    k_col_dot<KPL><<<rg, BLK, 0, ctx->stream>>>(n, S.B.get(), S.B.get(), k, partials, sc + 4 * MAXK);
    check_launch(ctx, "mrhs dot");
    k_col_dot<KPL><<<rg, BLK, 0, ctx->stream>>>(n, S.Rs.get(), S.Rs.get(), k, partials, sc + 2 * MAXK);
    check_launch(ctx, "mrhs dot");
  });
  std::vector<double> hb(k), hr(k), init(k), rel(k);
  copy(ctx, hb.data(), sc + 4 * MAXK, sizeof(double) * k);
  copy(ctx, hr.data(), sc + 2 * MAXK, sizeof(double) * k);
  sync(ctx);
  std::vector<double> bn(k);
  int n_active = 0;
  std::vector<int> iters(k, 0);
  for (int c = 0; c < k; ++c) {
    bn[c] = std::max(std::sqrt(hb[c]), 1e-30);
    rel[c] = init[c] = std::sqrt(hr[c]) / bn[c];
    if (!std::isfinite(rel[c])) fail(AFP_ERR_BREAKDOWN, "non-finite initial residual");
    act[c] = rel[c] > tol;
    n_active += act[c];
  }
  S.active.upload(act.data(), k);
  int it = 0;
  if (n_active > 0) {
    precondition_m(h);
    int cur = 0, nxt = 3;
    with_kpl(k, [&](auto KPLc) {
      constexpr int KPL = decltype(KPLc)::value;
      k_col_dot<KPL><<<rg, BLK, 0, ctx->stream>>>(n, S.Rs.get(), S.Z.get(), k, partials, sc + cur * MAXK);
      check_launch(ctx, "mrhs dot");
    });
    AFP_CUDA(cudaMemcpyAsync(S.P.get(), S.Z.get(), sizeof(double) * nk, cudaMemcpyDeviceToDevice, ctx->stream));
    for (it = 1; it <= maxit; ++it) {
      with_kpl(k, [&](auto KPLc) {
        constexpr int KPL = decltype(KPLc)::value;
        k_spmm_dot<KPL><<<rg, BLK, 0, ctx->stream>>>(n, A.rowptr, A.cols, A.vals, S.P.get(), S.Q.get(), k, partials,
                                                     sc + 1 * MAXK);
        check_launch(ctx, "mrhs spmm+dot");
        k_update_xr<KPL><<<rg, BLK, 0, ctx->stream>>>(n, k, sc + cur * MAXK, sc + 1 * MAXK, S.active.get(),
                                                      S.Xs.get(), S.Rs.get(), S.P.get(), S.Q.get(), partials,
                                                      sc + 2 * MAXK);
        check_launch(ctx, "mrhs update x r");
      });
      copy(ctx, hr.data(), sc + 2 * MAXK, sizeof(double) * k);
      sync(ctx);
      n_active = 0;
      for (int c = 0; c < k; ++c) {
        if (!act[c]) continue;
        rel[c] = std::sqrt(hr[c]) / bn[c];
        if (!std::isfinite(rel[c])) fail(AFP_ERR_BREAKDOWN, "non-finite residual");
        iters[c] = it;
        if (rel[c] <= tol) act[c] = 0;
        n_active += act[c];
      }
      if (n_active == 0) break;
      S.active.upload(act.data(), k);
      precondition_m(h);
      with_kpl(k, [&](auto KPLc) {
        constexpr int KPL = decltype(KPLc)::value;
        k_col_dot<KPL><<<rg, BLK, 0, ctx->stream>>>(n, S.Rs.get(), S.Z.get(), k, partials, sc + nxt * MAXK);
        check_launch(ctx, "mrhs dot");
        k_update_p<KPL><<<rows_grid(ctx, n), BLK, 0, ctx->stream>>>(n, k, sc + nxt * MAXK, sc + cur * MAXK,
                                                                     S.active.get(), S.Z.get(), S.P.get());
        check_launch(ctx, "mrhs update p");
      });
      std::swap(cur, nxt);
    }
    if (it > maxit) it = maxit;
  }
  k_rows_scatter<<<grid_for(nk, BLK), BLK, 0, ctx->stream>>>(n, k, L0.perm.get(), S.Xs.get(), S.Tmp.get(), k);
  check_launch(ctx, "mrhs scatter x");
  AFP_CUDA(cudaEventRecord(e1, ctx->stream));
  copy(ctx, X_user, S.Tmp.get(), sizeof(double) * nk);
  sync(ctx);
  float ms = 0;
  AFP_CUDA(cudaEventElapsedTime(&ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (info)
    for (int c = 0; c < k; ++c) {
      info[c].iterations = iters[c];
      info[c].converged = rel[c] <= tol;
      info[c].initial_residual = init[c];
      info[c].final_residual = rel[c];
      info[c].seconds = ms * 1e-3;
    }
  for (int c = 0; c < k; ++c)
    if (!(rel[c] <= tol)) return false;
  return true;
}

}  // namespace afp
