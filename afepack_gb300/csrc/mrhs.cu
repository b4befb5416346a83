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
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <type_traits>
#include <unordered_map>

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
// of an n x k block.  A group of W lanes (a power of two) holds the row's k
// columns, KPL per lane: with VEC, lane l owns the contiguous columns
// l*KPL .. l*KPL+KPL-1 (k == W*KPL) and gathers them with one vector load;
// otherwise lane l owns columns l, l + W, ... (W >= k up to 32, scalar
// loads).  SPL groups share one row, group p taking the row's entries in chunks
// p, p + SPL, ... of W (long coarse-level rows: enough groups in flight to
// cover the gather latency).  A chunk's (column, value) pairs are loaded one
// per lane and broadcast with shuffles; the gathers of the x rows of U = 8
// entries are issued before any of their products is summed.  The groups'
// partial sums meet in shared memory and are added in group order, so the
// result does not depend on timing.
enum RowOp { RO_SPMM = 0, RO_SPMM_ADD, RO_RES, RO_GS, RO_JAC };

constexpr int ROWS_BLK = 256;

// KPL consecutive values at p (16-byte aligned) into v: one vector load
template <int KPL, class X>
__device__ __forceinline__ void load_vec(const X* p, X (&v)[KPL]) {
  if constexpr (std::is_same_v<X, float> && KPL == 4) {
    const float4 t = *reinterpret_cast<const float4*>(p);
    v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
  } else if constexpr (std::is_same_v<X, double> && KPL == 2) {
    const double2 t = *reinterpret_cast<const double2*>(p);
    v[0] = t.x; v[1] = t.y;
  } else {
#pragma unroll
    for (int q = 0; q < KPL; ++q) v[q] = p[q];
  }
}

template <int W, int KPL, int SPL, class V, class X, int OP, bool VEC>
__global__ void __launch_bounds__(ROWS_BLK) k_rows_m(int64_t r0, int64_t r1, const int* __restrict__ rp,
                                                     const int* __restrict__ ci, const V* __restrict__ va, const X* x,
                                                     X* y, const X* __restrict__ r, const X* __restrict__ d, int k) {
  using A = typename AccT<X>::type;
  constexpr int GPB = ROWS_BLK / W;  // groups per block
  __shared__ A part[SPL > 1 ? GPB : 1][SPL > 1 ? W : 1][KPL];
  const int grp = threadIdx.x / W, lane = threadIdx.x & (W - 1);
  const int64_t row = r0 + (int64_t)blockIdx.x * (GPB / SPL) + grp / SPL;
  const int pidx = grp % SPL;
  const bool on = row < r1;
  const unsigned mask = W >= 32 ? 0xffffffffu : (((1u << W) - 1u) << ((threadIdx.x & 31) & ~(W - 1)));
  A acc[KPL];
#pragma unroll
  for (int q = 0; q < KPL; ++q) acc[q] = 0;
  A diag = 1;
  if (on) {
    int b = rp[row];
    const int e = rp[row + 1];
    if (OP == RO_GS) {  // the diagonal is the row's first entry
      diag = as<A>(va[b]);
      ++b;
    }
    constexpr int U = 8;
    if (W == 1) {
      for (int j0 = b + pidx * U; j0 < e; j0 += SPL * U) {
        A vals[U];
        X xv[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const bool in = j0 + u < e;
          vals[u] = in ? as<A>(va[j0 + u]) : A(0);
          xv[u] = in ? x[(int64_t)ci[j0 + u] * k] : X(0);
        }
#pragma unroll
        for (int u = 0; u < U; ++u) acc[0] += vals[u] * (A)xv[u];
      }
    } else {
      for (int base = b + pidx * W; base < e; base += SPL * W) {
        const int my = base + lane;
        const int cc = my < e ? ci[my] : 0;
        const A vv = my < e ? as<A>(va[my]) : A(0);
        const int cnt = min(W, e - base);
        for (int jj = 0; jj < cnt; jj += U) {
          A vals[U];
          X xv[U][KPL];
#pragma unroll
          for (int u = 0; u < U; ++u) {
            const bool in = jj + u < cnt;  // the same for the whole group
            const int col = __shfl_sync(mask, cc, in ? jj + u : 0, W);
            const A val = __shfl_sync(mask, vv, in ? jj + u : 0, W);
            vals[u] = in ? val : A(0);
            const X* xr = x + (int64_t)col * k;
            if constexpr (VEC) {
              if (in) load_vec<KPL>(xr + lane * KPL, xv[u]);
              else
#pragma unroll
                for (int q = 0; q < KPL; ++q) xv[u][q] = X(0);
            } else {
#pragma unroll
              for (int q = 0; q < KPL; ++q) {
                const int c = lane + W * q;
                xv[u][q] = (in && c < k) ? xr[c] : X(0);
              }
            }
          }
#pragma unroll
          for (int u = 0; u < U; ++u)
#pragma unroll
            for (int q = 0; q < KPL; ++q) acc[q] += vals[u] * (A)xv[u][q];
        }
      }
    }
  }
  if (SPL > 1) {
#pragma unroll
    for (int q = 0; q < KPL; ++q) part[grp][lane][q] = acc[q];
    __syncthreads();
    if (pidx != 0) return;
#pragma unroll
    for (int q = 0; q < KPL; ++q) {
      A s = part[grp][lane][q];
      for (int p = 1; p < SPL; ++p) s += part[grp + p][lane][q];
      acc[q] = s;
    }
  }
  if (!on) return;
#pragma unroll
  for (int q = 0; q < KPL; ++q) {
    const int c = VEC ? lane * KPL + q : lane + W * q;
    if (c >= k) continue;
    const int64_t o = row * k + c;
    if (OP == RO_SPMM) y[o] = (X)acc[q];
    else if (OP == RO_SPMM_ADD) y[o] = (X)((A)y[o] + acc[q]);
    else if (OP == RO_RES) y[o] = (X)((A)r[o] - acc[q]);
    else if (OP == RO_GS) y[o] = (X)(((A)r[o] - acc[q]) / diag);
    else y[(row - r0) * k + c] = (X)((A)x[o] + ((A)r[o] - acc[q]) / (A)d[row - r0]);  // RO_JAC into tmp
  }
}

// Launches k_rows_m with 16-byte vector gathers (KPL = 16 bytes of columns
// per lane, W = k / KPL lanes) when k allows them and x is aligned, else
// with W = the smallest power of two >= k (at most 32) and KPL = columns per
// lane; SPL groups per row for rows of about `row_len` entries (about 48
// entries per group).
template <class V, class X, int OP>
void rows_m(const afp_context* ctx, int64_t r0, int64_t r1, const int* rp, const int* ci, const V* va, const X* x,
            X* y, const X* r, const X* d, int k, double row_len, const char* what) {
  if (r1 <= r0) return;
  auto go = [&](auto Wc, auto Kc, auto Vc) {
    constexpr int W = decltype(Wc)::value, KPL = decltype(Kc)::value;
    constexpr bool VEC = decltype(Vc)::value;
    // groups per row: enough for the row's gathers to overlap (about 48
    // entries per group), and for short row ranges (small colour classes of
    // coarse levels) enough lanes to fill about half the GPU
    int spl = 1;
    while (spl < 8 && spl * 48 < row_len) spl *= 2;
    while (spl < 16 && spl * W < row_len && (double)(r1 - r0) * W * spl < 1024.0 * ctx->sm_count) spl *= 2;
    spl = std::min(spl, ROWS_BLK / W);
    auto launch = [&](auto Sc) {
      constexpr int SPL = decltype(Sc)::value;
      if constexpr (ROWS_BLK / W >= SPL) {  // a block holds whole rows
        constexpr int rows_per_blk = ROWS_BLK / W / SPL;
        const unsigned grid = (unsigned)((r1 - r0 + rows_per_blk - 1) / rows_per_blk);
        k_rows_m<W, KPL, SPL, V, X, OP, VEC><<<grid, ROWS_BLK, 0, ctx->stream>>>(r0, r1, rp, ci, va, x, y, r, d, k);
      }
    };
    if (spl == 1) launch(std::integral_constant<int, 1>());
    else if (spl == 2) launch(std::integral_constant<int, 2>());
    else if (spl == 4) launch(std::integral_constant<int, 4>());
    else if (spl == 8) launch(std::integral_constant<int, 8>());
    else launch(std::integral_constant<int, 16>());
  };
  using I1 = std::integral_constant<int, 1>;
  using I2 = std::integral_constant<int, 2>;
  using NV = std::false_type;
  using VV = std::true_type;
  constexpr int KV = 16 / (int)sizeof(X);  // columns in one 16-byte load
  const bool vec = k % KV == 0 && k / KV >= 4 && k / KV <= 32 && ((k / KV) & (k / KV - 1)) == 0 &&
                   reinterpret_cast<uintptr_t>(x) % 16 == 0;
  if (vec) {
    constexpr std::integral_constant<int, KV> KVc{};
    if (k / KV == 4) go(std::integral_constant<int, 4>(), KVc, VV());
    else if (k / KV == 8) go(std::integral_constant<int, 8>(), KVc, VV());
    else if (k / KV == 16) go(std::integral_constant<int, 16>(), KVc, VV());
    else go(std::integral_constant<int, 32>(), KVc, VV());
  } else if (k == 1) go(I1(), I1(), NV());
  else if (k == 2) go(std::integral_constant<int, 2>(), I1(), NV());
  else if (k <= 4) go(std::integral_constant<int, 4>(), I1(), NV());
  else if (k <= 8) go(std::integral_constant<int, 8>(), I1(), NV());
  else if (k <= 16) go(std::integral_constant<int, 16>(), I1(), NV());
  else if (k <= 32) go(std::integral_constant<int, 32>(), I1(), NV());
  else go(std::integral_constant<int, 32>(), I2(), NV());
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

// The same product for wide blocks (k a multiple of 4, at most 64), register
// tiled: 256 threads = 16 row groups x 16 column groups, each thread a 4 x 4
// tile of a 64-row x 64-column block tile, so one 16-byte shared load of hi,
// lo and R each feeds 16 products.  The inner dimension is split into
// gridDim.y parts of jlen; part s writes its pair sums to part[s] and
// k_tail_reduce_df adds the parts in s order (the result does not depend on
// timing).
constexpr int TG_R = 64, TG_J = 32;
__global__ void __launch_bounds__(256) k_tail_gemm_df_tiled(int64_t n, int64_t ld, const float* __restrict__ hi,
                                                             const float* __restrict__ lo,
                                                             const float* __restrict__ R, int k, int64_t jlen,
                                                             float2* __restrict__ part) {
  __shared__ __align__(16) float sH[TG_J][TG_R + 4], sL[TG_J][TG_R + 4];
  __shared__ __align__(16) float sR[TG_J][MAXK];
  const int tid = threadIdx.x, cg = tid & 15, rg = tid >> 4;
  const int64_t row0 = (int64_t)blockIdx.x * TG_R;
  const int64_t jb = (int64_t)blockIdx.y * jlen;
  const int64_t je = jb + jlen < n ? jb + jlen : n;
  float sh[4][4], sl[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int c = 0; c < 4; ++c) sh[i][c] = sl[i][c] = 0.f;
  for (int64_t j0 = jb; j0 < je; j0 += TG_J) {
    const int tj = (int)(je - j0 < TG_J ? je - j0 : TG_J);
    __syncthreads();
    for (int t = tid; t < TG_R * TG_J; t += 256) {
      const int r = t / TG_J, jj = t % TG_J;
      const bool on = row0 + r < n && jj < tj;
      sH[jj][r] = on ? hi[(row0 + r) * ld + j0 + jj] : 0.f;
      sL[jj][r] = on ? lo[(row0 + r) * ld + j0 + jj] : 0.f;
    }
    for (int t = tid; t < TG_J * MAXK; t += 256) {
      const int jj = t / MAXK, c = t % MAXK;
      sR[jj][c] = (jj < tj && c < k) ? R[(j0 + jj) * k + c] : 0.f;
    }
    __syncthreads();
    for (int jj = 0; jj < tj; ++jj) {
      const float4 h4 = *reinterpret_cast<const float4*>(&sH[jj][rg * 4]);
      const float4 l4 = *reinterpret_cast<const float4*>(&sL[jj][rg * 4]);
      const float4 v4 = *reinterpret_cast<const float4*>(&sR[jj][cg * 4]);
      const float h[4] = {h4.x, h4.y, h4.z, h4.w}, l[4] = {l4.x, l4.y, l4.z, l4.w};
      const float v[4] = {v4.x, v4.y, v4.z, v4.w};
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int c = 0; c < 4; ++c) df_add_prod(sh[i][c], sl[i][c], h[i], l[i], v[c]);
    }
  }
  float2* out = part + (int64_t)blockIdx.y * n * k;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int64_t row = row0 + rg * 4 + i;
    if (row >= n) continue;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const int col = cg * 4 + c;
      if (col < k) out[row * k + col] = make_float2(sh[i][c], sl[i][c]);
    }
  }
}

__global__ void k_tail_reduce_df(int64_t nk, int parts, const float2* __restrict__ part, float* __restrict__ X) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nk) return;
  float h = part[t].x, l = part[t].y;
  for (int s = 1; s < parts; ++s) df_add(h, l, part[s * nk + t].x, part[s * nk + t].y);
  X[t] = __fadd_rn(h, l);
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
    // a chunk of 32 (column, value) pairs, one per lane, broadcast with
    // shuffles; the gathers of U entries are issued before their products
    // are summed (entries still added in row order)
    const int e = rp[row + 1];
    for (int base = rp[row]; base < e; base += 32) {
      const int my = base + lane;
      const int cc = my < e ? ci[my] : 0;
      const double vv = my < e ? va[my] : 0.0;
      const int cnt = min(32, e - base);
      constexpr int U = 8;
      for (int jj = 0; jj < cnt; jj += U) {
        double vals[U], pv[U][KPL];
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const bool in = jj + u < cnt;  // the same for the whole warp
          const int col = __shfl_sync(0xffffffffu, cc, in ? jj + u : 0);
          vals[u] = __shfl_sync(0xffffffffu, vv, in ? jj + u : 0);
          const double* pr = p + (int64_t)col * k;
#pragma unroll
          for (int q = 0; q < KPL; ++q) {
            const int c = lane + 32 * q;
            pv[u][q] = (in && c < k) ? pr[c] : 0.0;
          }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
          if (jj + u >= cnt) break;
#pragma unroll
          for (int q = 0; q < KPL; ++q)
            if (lane + 32 * q < k) acc[q] += vals[u] * pv[u][q];
        }
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
    const double len = (double)L.nnz / (double)L.n;
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
          rows_m<X, X, RO_JAC>(ctx, r0, r1, A.rowptr, A.cols, A.vals, x, tmp, r, d, k, len, "mrhs l1-jacobi");
          k_copy<X><<<grid_for((r1 - r0) * k, BLK), BLK, 0, ctx->stream>>>((r1 - r0) * k, tmp, x + r0 * k);
          check_launch(ctx, "mrhs copy");
        } else {
          rows_m<X, X, RO_GS>(ctx, r0, r1, A.rowptr, A.cols, A.vals, x, x, r, nullptr, k, len,
                              "mrhs gauss-seidel class");
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
    rows_m<X, X, RO_RES>(ctx, 0, L.n, A.rowptr, A.cols, A.vals, x, blk<X>(S, 2, l), r, nullptr, k,
                         (double)L.nnz / L.n, "mrhs residual");
    const int64_t nc = h->lv[l + 1].n;
    rows_m<PV, X, RO_SPMM>(ctx, 0, nc, L.prp.get(), L.pci.get(), p_vals<PV>(L), blk<X>(S, 2, l), blk<X>(S, 1, l + 1),
                           nullptr, nullptr, k, (double)L.pnnz / nc, "mrhs restriction");
  }
  const Level& T = h->lv[t];
  if (h->tail_dense) {
    if constexpr (std::is_same<X, double>::value) {
      with_kpl(k, [&](auto KPLc) {
        constexpr int KPL = decltype(KPLc)::value;
        k_dense_gemm<KPL, X><<<rows_grid(ctx, T.n), BLK, 0, ctx->stream>>>(T.n, h->tail_inv.get(), blk<X>(S, 1, t),
                                                                          blk<X>(S, 0, t), k);
      });
    } else if (S.tail_split > 0 && S.tail_part.size() > 0) {
      const int64_t rb = (T.n + TG_R - 1) / TG_R;
      const int64_t jlen = ((T.n + S.tail_split - 1) / S.tail_split + TG_J - 1) / TG_J * TG_J;
      const int parts = (int)((T.n + jlen - 1) / jlen);
      k_tail_gemm_df_tiled<<<dim3((unsigned)rb, (unsigned)parts), 256, 0, ctx->stream>>>(
          T.n, h->tail_ld, h->tail_hi.get(), h->tail_lo.get(), blk<X>(S, 1, t), k, jlen, S.tail_part.get());
      k_tail_reduce_df<<<grid_for(T.n * k, BLK), BLK, 0, ctx->stream>>>(T.n * k, parts, S.tail_part.get(),
                                                                        blk<X>(S, 0, t));
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
                               blk<X>(S, 0, l), nullptr, nullptr, k, (double)L.pnnz / L.n, "mrhs prolongation");
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
  // the register-tiled tail product for wide FP32 blocks: split its inner
  // dimension so that the grid covers about four waves of the GPU
  const Level& T = h->lv[h->t];
  if (mixed && h->tail_dense && k >= 32 && k % 4 == 0) {
    const int64_t rb = (T.n + TG_R - 1) / TG_R;
    S->tail_split = (int)std::max<int64_t>(1, std::min<int64_t>(8, (4 * ctx->sm_count + rb - 1) / rb));
    S->tail_part.alloc(ctx, (int64_t)S->tail_split * T.n * k);
  } else {
    S->tail_split = 0;
  }
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
                                 (double)L0.nnz / n, "mrhs residual");
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

// ==================================================================== serving
// Continuous batching of solves against one resident hierarchy.
//
// The server owns the hierarchy's batched CG state at a fixed width of k
// columns; each column is an execution slot.  One driver thread runs CG
// iterations over all k columns (one batched V-cycle, one FP64 A p, the
// column recurrences) and, between two iterations, admits queued requests
// into free columns and retires the ones that converged, so requests arrive
// and leave while others are in flight.  A request's column starts with
// x = 0, r = b, p = 0 and an old r.z of 1, so its first step is the plain
// CG start p = z.  Free columns hold r = p = 0 and are masked out of every
// update; the batched kernels are deterministic and each column's arithmetic
// uses only its own entries, so a request's solution does not depend on the
// other columns.
namespace afp {
namespace {

// column c of the solve-order block <- src[perm[i]] (b), x = 0, r = b, p = 0
__global__ void k_col_admit(int64_t n, int k, int c, const int* __restrict__ perm, const double* __restrict__ src,
                            double* __restrict__ B, double* __restrict__ X, double* __restrict__ R,
                            double* __restrict__ P) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double v = src[perm[i]];
  const int64_t o = i * k + c;
  B[o] = v;
  X[o] = 0.0;
  R[o] = v;
  P[o] = 0.0;
}

// dst[perm[i]] = X column c; then r = p = 0 in that column (a free slot)
__global__ void k_col_retire(int64_t n, int k, int c, const int* __restrict__ perm, const double* __restrict__ X,
                             double* __restrict__ dst, double* __restrict__ R, double* __restrict__ P) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t o = i * k + c;
  dst[perm[i]] = X[o];
  R[o] = 0.0;
  P[o] = 0.0;
}

}  // namespace
}  // namespace afp

struct afp_batch_server {
  afp_amg* amg = nullptr;
  afp_batch_opts opts{};
  struct Req {
    int64_t ticket = 0;
    std::vector<double> b, x;
    afp_request_result res{};
    std::chrono::steady_clock::time_point t_submit, t_admit;
    bool done = false;
  };
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Req*> queue;
  std::unordered_map<int64_t, std::unique_ptr<Req>> reqs;
  std::thread driver;
  bool stop = false;
  int64_t next_ticket = 1;
  std::string fatal;  // a driver failure fails every request after it
  // statistics
  std::vector<double> latencies;
  int64_t completed = 0, failed = 0, iterations = 0;
  std::chrono::steady_clock::time_point t_start = std::chrono::steady_clock::now(), t_last = t_start;
};

namespace {

using SClock = std::chrono::steady_clock;
double s_secs(SClock::time_point a, SClock::time_point b) { return std::chrono::duration<double>(b - a).count(); }

// Pinned host staging of the driver: k columns in, k columns out, and the
// column scalars read after every iteration.
struct PinnedStage {
  double* in = nullptr;
  double* out = nullptr;
  double* scal = nullptr;
  PinnedStage(int64_t n, int k) {
    AFP_CUDA(cudaMallocHost(&in, sizeof(double) * n * k));
    AFP_CUDA(cudaMallocHost(&out, sizeof(double) * n * k));
    AFP_CUDA(cudaMallocHost(&scal, sizeof(double) * 5 * afp::MAXK));
  }
  ~PinnedStage() {
    cudaFreeHost(in);
    cudaFreeHost(out);
    cudaFreeHost(scal);
  }
};

// The driver keeps the GPU busy between CG iterations: admissions copy the
// right-hand side through pinned memory (one asynchronous copy each), and a
// retired column's solution is copied out asynchronously and handed to its
// waiter while the next iteration runs.
void batch_driver(afp_batch_server* s) {
  using namespace afp;
  afp_amg* h = s->amg;
  afp_context* ctx = h->ctx;
  const int k = s->opts.width;
  std::vector<afp_batch_server::Req*> slot(k, nullptr);
  std::vector<int> iters(k, 0), act(k, 0);
  std::vector<double> rz_one(afp::MAXK, 1.0);
  // retired columns whose solutions are on their way to pinned memory
  std::vector<std::pair<int, afp_batch_server::Req*>> leaving;
  cudaEvent_t out_done = nullptr;
  auto hand_over = [&](double* pin_out, int64_t n) {
    if (leaving.empty()) return;
    AFP_CUDA(cudaEventSynchronize(out_done));
    for (auto& [c, r] : leaving) r->x.assign(pin_out + (int64_t)c * n, pin_out + (int64_t)(c + 1) * n);
    const auto now = SClock::now();
    std::lock_guard<std::mutex> lk(s->mu);
    for (auto& [c, r] : leaving) {
      r->res.queue_seconds = s_secs(r->t_submit, r->t_admit);
      r->res.latency_seconds = s_secs(r->t_submit, now);
      r->done = true;
      if (r->res.status == AFP_OK) {
        s->completed++;
        s->latencies.push_back(r->res.latency_seconds);
      } else {
        s->failed++;
      }
      s->t_last = now;
    }
    leaving.clear();
    s->cv_done.notify_all();
  };
  try {
    bind(ctx);
    ensure_state(h, k);
    MultiState& S = *h->multi;
    const Level& L0 = h->lv[0];
    const int64_t n = L0.n;
    PinnedStage pin(n, k);
    AFP_CUDA(cudaEventCreateWithFlags(&out_done, cudaEventDisableTiming));
    double* sc = S.scal.get();  // rows: 0 rz (old), 1 pq, 2 rr, 3 rz (new), 4 bb
    double* partials = sc + 8 * MAXK;
    const CSRView<double> A = L0.A<double>();
    const unsigned rg = std::min<unsigned>(RED_GRID, rows_grid(ctx, n));
    AFP_CUDA(cudaMemsetAsync(S.Rs.get(), 0, sizeof(double) * n * k, ctx->stream));
    AFP_CUDA(cudaMemsetAsync(S.P.get(), 0, sizeof(double) * n * k, ctx->stream));
    AFP_CUDA(cudaMemsetAsync(S.B.get(), 0, sizeof(double) * n * k, ctx->stream));
    S.active.upload(act.data(), k);
    sync(ctx);
    for (;;) {
      // ---- admission: queued requests into free columns
      std::vector<std::pair<int, afp_batch_server::Req*>> admit;
      {
        std::unique_lock<std::mutex> lk(s->mu);
        const bool any_active = std::find(act.begin(), act.end(), 1) != act.end();
        if (!any_active && !leaving.empty()) {
          lk.unlock();
          hand_over(pin.out, n);
          lk.lock();
        }
        if (!any_active) s->cv_work.wait(lk, [&] { return s->stop || !s->queue.empty(); });
        if (s->stop && s->queue.empty() && !any_active) break;
        for (int c = 0; c < k && !s->queue.empty(); ++c)
          if (!act[c]) {
            afp_batch_server::Req* r = s->queue.front();
            s->queue.pop_front();
            r->t_admit = SClock::now();
            admit.push_back({c, r});
          }
      }
      if (!admit.empty()) {
        for (auto& [c, r] : admit) {
          double* stage = pin.in + (int64_t)c * n;
          std::memcpy(stage, r->b.data(), sizeof(double) * n);
          std::vector<double>().swap(r->b);
          AFP_CUDA(cudaMemcpyAsync(S.Tmp.get() + (int64_t)c * n, stage, sizeof(double) * n, cudaMemcpyHostToDevice,
                                   ctx->stream));
          k_col_admit<<<grid_for(n, BLK), BLK, 0, ctx->stream>>>(n, k, c, L0.perm.get(), S.Tmp.get() + (int64_t)c * n,
                                                                S.B.get(), S.Xs.get(), S.Rs.get(), S.P.get());
          check_launch(ctx, "batch admit");
          // old r.z of a fresh column: 1
          AFP_CUDA(cudaMemcpyAsync(sc + c, rz_one.data(), sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
          slot[c] = r;
          iters[c] = 0;
          act[c] = 1;
        }
        S.active.upload(act.data(), k);
        with_kpl(k, [&](auto KPLc) {
          constexpr int KPL = decltype(KPLc)::value;
          k_col_dot<KPL><<<rg, BLK, 0, ctx->stream>>>(n, S.B.get(), S.B.get(), k, partials, sc + 4 * MAXK);
          check_launch(ctx, "batch b.b");
        });
      }
      // ---- one CG iteration over every column (free ones are masked)
      precondition_m(h);  // Z = V(R)
      with_kpl(k, [&](auto KPLc) {
        constexpr int KPL = decltype(KPLc)::value;
        k_col_dot<KPL><<<rg, BLK, 0, ctx->stream>>>(n, S.Rs.get(), S.Z.get(), k, partials, sc + 3 * MAXK);
        check_launch(ctx, "batch r.z");
        k_update_p<KPL><<<rows_grid(ctx, n), BLK, 0, ctx->stream>>>(n, k, sc + 3 * MAXK, sc, S.active.get(),
                                                                     S.Z.get(), S.P.get());
        check_launch(ctx, "batch p");
        k_spmm_dot<KPL><<<rg, BLK, 0, ctx->stream>>>(n, A.rowptr, A.cols, A.vals, S.P.get(), S.Q.get(), k, partials,
                                                     sc + 1 * MAXK);
        check_launch(ctx, "batch A p");
        k_update_xr<KPL><<<rg, BLK, 0, ctx->stream>>>(n, k, sc + 3 * MAXK, sc + 1 * MAXK, S.active.get(), S.Xs.get(),
                                                      S.Rs.get(), S.P.get(), S.Q.get(), partials, sc + 2 * MAXK);
        check_launch(ctx, "batch x r");
      });
      AFP_CUDA(cudaMemcpyAsync(sc, sc + 3 * MAXK, sizeof(double) * k, cudaMemcpyDeviceToDevice, ctx->stream));
      AFP_CUDA(cudaMemcpyAsync(pin.scal + 2 * MAXK, sc + 2 * MAXK, sizeof(double) * 3 * MAXK,
                               cudaMemcpyDeviceToHost, ctx->stream));  // rr, rz, bb
      // the previous retirements' solutions arrived before this iteration started
      hand_over(pin.out, n);
      sync(ctx);
      // ---- retire converged (or failed) columns
      const double* host = pin.scal;
      bool retired = false;
      for (int c = 0; c < k; ++c) {
        if (!act[c]) continue;
        ++iters[c];
        const double bn = std::max(std::sqrt(host[4 * MAXK + c]), 1e-300);
        const double rel = std::sqrt(host[2 * MAXK + c]) / bn;
        afp_batch_server::Req* r = slot[c];
        r->res.rel_residual = rel;
        int st = -1;
        if (!std::isfinite(rel)) st = AFP_ERR_BREAKDOWN;
        else if (rel <= s->opts.tol) st = AFP_OK;
        else if (iters[c] >= s->opts.maxit) st = AFP_ERR_NOT_CONVERGED;
        if (st < 0) continue;
        k_col_retire<<<grid_for(n, BLK), BLK, 0, ctx->stream>>>(n, k, c, L0.perm.get(), S.Xs.get(),
                                                               S.Tmp.get() + (int64_t)c * n, S.Rs.get(), S.P.get());
        check_launch(ctx, "batch retire");
        AFP_CUDA(cudaMemcpyAsync(pin.out + (int64_t)c * n, S.Tmp.get() + (int64_t)c * n, sizeof(double) * n,
                                 cudaMemcpyDeviceToHost, ctx->stream));
        r->res.status = st;
        r->res.iterations = iters[c];
        leaving.push_back({c, r});
        slot[c] = nullptr;
        act[c] = 0;
        retired = true;
      }
      if (retired) {
        AFP_CUDA(cudaEventRecord(out_done, ctx->stream));
        S.active.upload(act.data(), k);
      }
      {
        std::lock_guard<std::mutex> lk(s->mu);
        s->iterations++;
      }
    }
    hand_over(pin.out, n);
  } catch (const Error& e) {
    std::lock_guard<std::mutex> lk(s->mu);
    s->fatal = e.msg;
    for (auto& kv : s->reqs)
      if (!kv.second->done) {
        kv.second->res.status = e.status;
        kv.second->done = true;
        s->failed++;
      }
    s->queue.clear();
    s->cv_done.notify_all();
  }
  if (out_done) cudaEventDestroy(out_done);
}

double s_percentile(std::vector<double> v, double p) {
  if (v.empty()) return 0.0;
  std::sort(v.begin(), v.end());
  const double pos = p / 100.0 * (v.size() - 1);
  const size_t i = (size_t)pos;
  const double frac = pos - i;
  return i + 1 < v.size() ? v[i] * (1 - frac) + v[i + 1] * frac : v[i];
}

}  // namespace

extern "C" {

void afp_batch_default_opts(afp_batch_opts* o) {
  if (!o) return;
  o->width = 32;
  o->tol = 1e-10;
  o->maxit = 500;
}

afp_status afp_batch_server_create(afp_amg* amg, const afp_batch_opts* opts, afp_batch_server** out) {
  return afp::guarded([&] {
    AFP_REQUIRE(amg && out, AFP_ERR_INVALID, "null argument");
    auto s = std::make_unique<afp_batch_server>();
    if (opts) s->opts = *opts;
    else afp_batch_default_opts(&s->opts);
    AFP_REQUIRE(s->opts.width >= 1 && s->opts.width <= afp::MAXK, AFP_ERR_INVALID, "width must be in [1, 64]");
    AFP_REQUIRE(s->opts.tol > 0 && s->opts.maxit >= 1, AFP_ERR_INVALID, "bad tolerance or iteration limit");
    s->amg = amg;
    s->driver = std::thread(batch_driver, s.get());
    *out = s.release();
  });
}

afp_status afp_batch_server_submit(afp_batch_server* s, const double* b, int64_t* ticket) {
  return afp::guarded([&] {
    AFP_REQUIRE(s && b && ticket, AFP_ERR_INVALID, "null argument");
    const int64_t n = s->amg->lv[0].n;
    auto r = std::make_unique<afp_batch_server::Req>();
    r->b.assign(b, b + n);
    r->t_submit = SClock::now();
    std::lock_guard<std::mutex> lk(s->mu);
    AFP_REQUIRE(!s->stop, AFP_ERR_INVALID, "server is shutting down");
    AFP_REQUIRE(s->fatal.empty(), AFP_ERR_CUDA, "the server failed: " + s->fatal);
    r->ticket = s->next_ticket++;
    *ticket = r->ticket;
    s->queue.push_back(r.get());
    s->reqs[r->ticket] = std::move(r);
    s->cv_work.notify_all();
  });
}

afp_status afp_batch_server_wait(afp_batch_server* s, int64_t ticket, double* x, afp_request_result* res) {
  return afp::guarded([&] {
    AFP_REQUIRE(s, AFP_ERR_INVALID, "null server");
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->reqs.find(ticket);
    AFP_REQUIRE(it != s->reqs.end(), AFP_ERR_INVALID, "unknown ticket");
    afp_batch_server::Req* r = it->second.get();
    s->cv_done.wait(lk, [&] { return r->done; });
    if (res) *res = r->res;
    if (x && !r->x.empty()) std::memcpy(x, r->x.data(), sizeof(double) * r->x.size());
    s->reqs.erase(it);
  });
}

afp_status afp_batch_server_get_stats(afp_batch_server* s, afp_server_stats* st) {
  return afp::guarded([&] {
    AFP_REQUIRE(s && st, AFP_ERR_INVALID, "null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    st->completed = s->completed;
    st->failed = s->failed;
    st->queued = (int64_t)s->queue.size();
    st->p50_seconds = s_percentile(s->latencies, 50);
    st->p99_seconds = s_percentile(s->latencies, 99);
    const double span = s_secs(s->t_start, s->t_last);
    st->solves_per_second = span > 0 ? s->completed / span : 0.0;
    st->budget_bytes = 0;
    st->in_use_bytes = 0;
  });
}

afp_status afp_batch_server_reset_stats(afp_batch_server* s) {
  return afp::guarded([&] {
    AFP_REQUIRE(s, AFP_ERR_INVALID, "null server");
    std::lock_guard<std::mutex> lk(s->mu);
    s->latencies.clear();
    s->completed = s->failed = 0;
    s->t_start = s->t_last = SClock::now();
  });
}

afp_status afp_batch_server_destroy(afp_batch_server* s) {
  return afp::guarded([&] {
    if (!s) return;
    {
      std::lock_guard<std::mutex> lk(s->mu);
      s->stop = true;
    }
    s->cv_work.notify_all();
    if (s->driver.joinable()) s->driver.join();
    delete s;
  });
}

}  // extern "C"

namespace afp {
// Measurement of the batched V-cycle at the width of the last batched solve:
// kind 4 = one batched V-cycle, kind 5 = one batched Gauss-Seidel sweep of
// `level` (every colour class once); mean device time over reps and the
// algorithmic bytes (each array once per pass, the k columns of a vector
// block counted once per pass).
void time_multi(afp_amg* h, int kind, int level, int reps, double* ms, double* bytes) {
  AFP_REQUIRE(h->multi && h->multi->k > 0, AFP_ERR_INVALID, "no batched state: run a batched solve first");
  afp_context* ctx = h->ctx;
  MultiState& S = *h->multi;
  const int k = S.k;
  const bool mixed = S.mixed;
  const double v = mixed ? 4.0 : 8.0, vp = mixed ? (h->opts.interp_bf16 ? 2.0 : 4.0) : 8.0;
  auto unit = [&]() {
    if (kind == 4) {
      precondition_m(h);
      return;
    }
    const Level& L = h->lv[level];
    const double len = (double)L.nnz / (double)L.n;
    const int K = (int)L.cls.size() - 1;
    for (int q = 0; q < K; ++q) {
      const int64_t r0 = L.cls[q], r1 = L.cls[q + 1];
      if (mixed) {
        CSRView<float> A = L.A<float>();
        if (L.overflow && q == K - 1) {
          rows_m<float, float, RO_JAC>(ctx, r0, r1, A.rowptr, A.cols, A.vals, S.X32[level].get(), S.T32[level].get(),
                                       S.R32[level].get(), L.l1d32.get(), k, len, "mrhs l1-jacobi");
          k_copy<float><<<grid_for((r1 - r0) * k, BLK), BLK, 0, ctx->stream>>>((r1 - r0) * k, S.T32[level].get(),
                                                                               S.X32[level].get() + r0 * k);
          check_launch(ctx, "mrhs copy");
        } else {
          rows_m<float, float, RO_GS>(ctx, r0, r1, A.rowptr, A.cols, A.vals, S.X32[level].get(), S.X32[level].get(),
                                      S.R32[level].get(), nullptr, k, len, "mrhs gauss-seidel class");
        }
      } else {
        CSRView<double> A = L.A<double>();
        if (L.overflow && q == K - 1) {
          rows_m<double, double, RO_JAC>(ctx, r0, r1, A.rowptr, A.cols, A.vals, S.X[level].get(), S.T[level].get(),
                                         S.R[level].get(), L.l1d.get(), k, len, "mrhs l1-jacobi");
          k_copy<double><<<grid_for((r1 - r0) * k, BLK), BLK, 0, ctx->stream>>>((r1 - r0) * k, S.T[level].get(),
                                                                                S.X[level].get() + r0 * k);
          check_launch(ctx, "mrhs copy");
        } else {
          rows_m<double, double, RO_GS>(ctx, r0, r1, A.rowptr, A.cols, A.vals, S.X[level].get(), S.X[level].get(),
                                        S.R[level].get(), nullptr, k, len, "mrhs gauss-seidel class");
        }
      }
    }
  };
  AFP_REQUIRE(kind == 4 || (level >= 0 && level < h->t), AFP_ERR_INVALID, "level is not a smoothed level");
  unit();  // warm
  cudaEvent_t e0, e1;
  AFP_CUDA(cudaEventCreate(&e0));
  AFP_CUDA(cudaEventCreate(&e1));
  AFP_CUDA(cudaEventRecord(e0, ctx->stream));
  for (int i = 0; i < reps; ++i) unit();
  AFP_CUDA(cudaEventRecord(e1, ctx->stream));
  sync(ctx);
  float t = 0;
  AFP_CUDA(cudaEventElapsedTime(&t, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *ms = t / reps;
  auto pass = [&](const Level& Q) { return (double)Q.nnz * (v + 4) + 4.0 * (Q.n + 1) + 3.0 * Q.n * v * k; };
  if (kind == 5) {
    *bytes = pass(h->lv[level]);
    return;
  }
  const double s = h->opts.smooth_step;
  double b = 0;
  for (int l = 0; l < h->t; ++l) {
    const Level& Q = h->lv[l];
    const double nn = (double)Q.n, nc = (double)h->lv[l + 1].n;
    b += (2 * s + 1) * pass(Q) + 2.0 * nn * v * k;                          // sweeps, residual, zero
    b += 2.0 * Q.pnnz * (vp + 4) + 4.0 * (nc + 1) + 4.0 * (nn + 1) + 3.0 * nn * v * k + 2.0 * nc * v * k;  // P, P^T
  }
  const double nt = (double)h->lv[h->t].n;
  b += h->tail_dense ? nt * nt * 8.0 + 2.0 * nt * v * k : 0.0;
  *bytes = b;
}
}  // namespace afp
