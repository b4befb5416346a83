// Sparse kernels of the V-cycle and the outer CG.
//
// Every row kernel assigns a group of VEC consecutive threads to one CSR row
// (VEC from the level's mean row length), so the row's column numbers and
// values are read as contiguous, coalesced segments; partial sums are
// combined with warp shuffles.  Colour classes are contiguous row ranges
// (the hierarchy is stored colour-permuted), so a Gauss-Seidel class is one
// launch over a dense range without an index list.
//
// Reductions are deterministic: each block writes a partial sum and the last
// block to finish adds the partials in block order.
#include <cstdlib>

#include "df32.cuh"
#include "kernels.cuh"
#include "launch.cuh"
#include "solve.cuh"

namespace afp {

// Lanes per row: the smallest power of two in [4, 32] with at most
// `entries per lane` of the level's mean row length on each lane.  Four per
// lane (AFP_ENTRIES_PER_LANE overrides it for tuning) measured fastest on the
// 64^3 P1 level 0 (15 entries per row, 4 lanes): its FP32 Gauss-Seidel sweep
// 20 us against 32 us with one entry per lane, the residual 7 us against 19.
int pick_vec(double avg) {
  static const double epl = [] {
    const char* e = std::getenv("AFP_ENTRIES_PER_LANE");
    const double v = e ? std::atof(e) : 0.0;
    return v > 0.0 ? v : 4.0;
  }();
  int vec = 4;
  while (vec < 32 && vec * epl < avg) vec *= 2;
  return vec;
}

namespace {

constexpr int BLK = 256;

template <class X>
struct Acc {
  using type = float;
};
template <>
struct Acc<double> {
  using type = double;
};

template <class V>
__device__ __forceinline__ float tof(V v) {
  return (float)v;
}
template <>
__device__ __forceinline__ float tof<__nv_bfloat16>(__nv_bfloat16 v) {
  return __bfloat162float(v);
}

template <class A, class V>
__device__ __forceinline__ A val_as(V v) {
  return (A)v;
}
template <>
__device__ __forceinline__ float val_as<float, __nv_bfloat16>(__nv_bfloat16 v) {
  return __bfloat162float(v);
}

template <int VEC, class T>
__device__ __forceinline__ T group_sum(T s) {
#pragma unroll
  for (int o = VEC / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o, VEC);
  return s;
}

// Row loads ahead of griddepcontrol.wait.  The matrices of a solve are not
// written by any kernel of the V-cycle / CG chain, so each thread loads its
// row bounds and its first PF (column, value) pairs before waiting for the
// predecessor grid; only the gathers of x (and reads of r) wait.  Under PDL
// this overlaps two of the three dependent memory round trips of a row with
// the predecessor's drain.  The products are summed in the same order as a
// plain k = begin + lane, begin + lane + VEC, ... loop.
// Pairs loaded ahead per lane.  FP64 keeps it short: each guarded product
// of the unrolled loop costs an FP64 instruction slot whether or not the
// entry exists, and FP64 instruction throughput is what bounds the FP64
// kernels on this GPU.
template <int VEC, class V>
constexpr int prefetch_depth() {
  return sizeof(V) == 8 ? (VEC >= 32 ? 2 : 1) : (VEC >= 32 ? 8 : 4);
}

template <int VEC, class V>
struct RowAhead {
  static constexpr int PF = prefetch_depth<VEC, V>();
  int k, e;  // first entry of this lane, row end
  int c[PF];
  V v[PF];
  __device__ __forceinline__ void load(const int* __restrict__ ci, const V* __restrict__ va, int k0, int e0) {
    k = k0;
    e = e0;
#pragma unroll
    for (int q = 0; q < PF; ++q) {
      const int kk = k + q * VEC;
      c[q] = kk < e ? ci[kk] : 0;
      v[q] = kk < e ? va[kk] : V(0);
    }
  }
  template <class A, class X>
  __device__ __forceinline__ A dot(const int* __restrict__ ci, const V* __restrict__ va,
                                   const X* __restrict__ x) const {
    A s = 0;
#pragma unroll
    for (int q = 0; q < PF; ++q)
      if (k + q * VEC < e) s += val_as<A>(v[q]) * (A)x[c[q]];
    for (int kk = k + PF * VEC; kk < e; kk += VEC) s += val_as<A>(va[kk]) * (A)x[ci[kk]];
    return s;
  }
};

template <int VEC, class V, class X, bool ADD>
__global__ void k_spmv(int64_t m, const int* __restrict__ rp, const int* __restrict__ ci, const V* __restrict__ va,
                       const X* __restrict__ x, X* __restrict__ y) {
  using A = typename Acc<X>::type;
  const int64_t g = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / VEC;
  const int lane = threadIdx.x % VEC;
  RowAhead<VEC, V> row;
  row.load(ci, va, g < m ? rp[g] + lane : 0, g < m ? rp[g + 1] : 0);
  pdl_wait();
  A s = row.template dot<A>(ci, va, x);
  s = group_sum<VEC>(s);
  if (g < m && lane == 0) y[g] = ADD ? (X)((A)y[g] + s) : (X)s;
}

template <int VEC, class X>
__global__ void k_residual(int64_t m, const int* __restrict__ rp, const int* __restrict__ ci, const X* __restrict__ va,
                           const X* __restrict__ x, const X* __restrict__ r, X* __restrict__ out) {
  using A = typename Acc<X>::type;
  const int64_t g = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / VEC;
  const int lane = threadIdx.x % VEC;
  RowAhead<VEC, X> row;
  row.load(ci, va, g < m ? rp[g] + lane : 0, g < m ? rp[g + 1] : 0);
  pdl_wait();
  A s = row.template dot<A>(ci, va, x);
  s = group_sum<VEC>(s);
  if (g < m && lane == 0) out[g] = (X)((A)r[g] - s);
}

template <int VEC, class X>
__global__ void k_gs_class(int64_t r0, int64_t r1, const int* __restrict__ rp, const int* __restrict__ ci,
                           const X* __restrict__ va, X* __restrict__ x, const X* __restrict__ r) {
  using A = typename Acc<X>::type;
  const int64_t row = r0 + ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / VEC;
  const int lane = threadIdx.x % VEC;
  const bool on = row < r1;
  const int d = on ? rp[row] : 0;
  const X diag = on ? va[d] : X(1);
  RowAhead<VEC, X> ahead;
  ahead.load(ci, va, d + 1 + lane, on ? rp[row + 1] : 0);
  pdl_wait();
  A s = ahead.template dot<A>(ci, va, (const X*)x);
  s = group_sum<VEC>(s);
  if (on && lane == 0) x[row] = (X)(((A)r[row] - s) / (A)diag);
}

template <int VEC, class X>
__global__ void k_jacobi_l1(int64_t r0, int64_t r1, const int* __restrict__ rp, const int* __restrict__ ci,
                            const X* __restrict__ va, const X* __restrict__ x, const X* __restrict__ r,
                            const X* __restrict__ d, X* __restrict__ tmp) {
  using A = typename Acc<X>::type;
  const int64_t row = r0 + ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / VEC;
  const int lane = threadIdx.x % VEC;
  const bool on = row < r1;
  RowAhead<VEC, X> ahead;
  ahead.load(ci, va, on ? rp[row] + lane : 0, on ? rp[row + 1] : 0);
  pdl_wait();
  A s = ahead.template dot<A>(ci, va, x);
  s = group_sum<VEC>(s);
  if (on && lane == 0) tmp[row - r0] = (X)((A)x[row] + ((A)r[row] - s) / (A)d[row - r0]);
}

template <class X>
__global__ void k_copy_range(int64_t n, const X* __restrict__ src, X* __restrict__ dst) {
  pdl_wait();
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = src[i];
}

template <class X>
__global__ void k_dense_gemv(int64_t n, const X* __restrict__ M, const X* __restrict__ r, X* __restrict__ x) {
  pdl_wait();
  using A = typename Acc<X>::type;
  const int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32;
  const int lane = threadIdx.x & 31;
  A s = 0;
  if (row < n)
    for (int64_t j = lane; j < n; j += 32) s += (A)M[row * n + j] * (A)r[j];
  s = group_sum<32>(s);
  if (row < n && lane == 0) x[row] = (X)s;
}

__global__ void k_split_df(int64_t n, int64_t ld, const double* __restrict__ in, float* __restrict__ hi,
                           float* __restrict__ lo) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n * ld) return;
  const int64_t i = t / ld, j = t % ld;
  const double d = j < n ? in[i * n + j] : 0.0;
  const float h = __double2float_rn(d);
  hi[t] = h;
  lo[t] = __double2float_rn(d - (double)h);
}

// One warp per row; each lane walks the row with stride 32 (coalesced loads of
// hi and lo), accumulating a double-float pair; the pairs are merged across
// the warp with TwoSum.
__global__ void k_dense_gemv_df(int64_t n, int64_t ld, const float* __restrict__ hi, const float* __restrict__ lo,
                                const float* __restrict__ r, float* __restrict__ x) {
  pdl_wait();
  const int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32;
  const int lane = threadIdx.x & 31;
  if (row >= n) return;  // whole warps leave together
  const float* h = hi + row * ld;
  const float* l = lo + row * ld;
  float sh = 0.f, sl = 0.f;
  int64_t j = lane;
  for (; j + 96 < n; j += 128) {
    const float h0 = h[j], h1 = h[j + 32], h2 = h[j + 64], h3 = h[j + 96];
    const float l0 = l[j], l1 = l[j + 32], l2 = l[j + 64], l3 = l[j + 96];
    const float v0 = r[j], v1 = r[j + 32], v2 = r[j + 64], v3 = r[j + 96];
    df_add_prod(sh, sl, h0, l0, v0);
    df_add_prod(sh, sl, h1, l1, v1);
    df_add_prod(sh, sl, h2, l2, v2);
    df_add_prod(sh, sl, h3, l3, v3);
  }
  for (; j < n; j += 32) df_add_prod(sh, sl, h[j], l[j], r[j]);
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    const float oh = __shfl_xor_sync(0xffffffffu, sh, off);
    const float ol = __shfl_xor_sync(0xffffffffu, sl, off);
    df_add(sh, sl, oh, ol);
  }
  if (lane == 0) x[row] = __fadd_rn(sh, sl);
}

template <class X>
__global__ void k_diag_solve(int64_t n, const int* __restrict__ rp, const X* __restrict__ va, const X* __restrict__ r,
                             X* __restrict__ x) {
  pdl_wait();
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) x[i] = r[i] / va[rp[i]];
}

template <class A, class B>
__global__ void k_convert(int64_t n, const A* __restrict__ in, B* __restrict__ out) {
  pdl_wait();
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = (B)in[i];
}
template <>
__global__ void k_convert<double, __nv_bfloat16>(int64_t n, const double* __restrict__ in,
                                                 __nv_bfloat16* __restrict__ out) {
  pdl_wait();
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = __double2bfloat16(in[i]);
}

__global__ void k_gather(int64_t n, const int* __restrict__ perm, const double* __restrict__ in,
                         double* __restrict__ out) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = in[perm[i]];
}
__global__ void k_scatter(int64_t n, const int* __restrict__ perm, const double* __restrict__ in,
                          double* __restrict__ out) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[perm[i]] = in[i];
}

__global__ void k_axpy(int64_t n, double alpha, const double* __restrict__ x, double* __restrict__ y) {
  pdl_wait();
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] += alpha * x[i];
}

__global__ void k_strided_copy(int64_t n, const double* __restrict__ src, int64_t ss, double* __restrict__ dst,
                               int64_t ds) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i * ds] = src[i * ss];
}

template <class X>
__global__ void k_zero(int64_t n, X* __restrict__ x) {
  pdl_wait();
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) x[i] = (X)0;
}

// ------------------------------------------------------------ reductions
constexpr int RED_BLOCKS = 512;

// the context's partials array (RED_BLOCKS entries) and retire counter
struct RedScratch {
  double* partials;
  unsigned* retire;
};

__device__ __forceinline__ double block_sum(double v) {
  __shared__ double ws[BLK / 32];
  v = group_sum<32>(v);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) ws[w] = v;
  __syncthreads();
  double s = 0;
  if (w == 0) {
    s = lane < BLK / 32 ? ws[lane] : 0.0;
    s = group_sum<32>(s);
  }
  __syncthreads();
  return s;  // valid in thread 0
}

// Partial of this block -> scratch; the last block sums them in order.
__device__ __forceinline__ void finish_reduction(double partial, double* dst, RedScratch rs) {
  __shared__ bool last;
  if (threadIdx.x == 0) {
    rs.partials[blockIdx.x] = partial;
    __threadfence();
    unsigned done = atomicInc(rs.retire, gridDim.x - 1);  // wraps to 0 for the last block
    last = (done == gridDim.x - 1);
  }
  __syncthreads();
  if (last) {
    double s = 0;
    for (unsigned b = threadIdx.x; b < gridDim.x; b += BLK) s += ((volatile double*)rs.partials)[b];
    s = block_sum(s);
    if (threadIdx.x == 0) *dst = s;
  }
}

__global__ void k_dot(int64_t n, const double* __restrict__ a, const double* __restrict__ b, double* dst,
                      RedScratch rs) {
  pdl_wait();
  double s = 0;
  for (int64_t i = (int64_t)blockIdx.x * BLK + threadIdx.x; i < n; i += (int64_t)gridDim.x * BLK) s += a[i] * b[i];
  s = block_sum(s);
  finish_reduction(s, dst, rs);
}

template <int VEC>
__global__ void k_spmv_dot(int64_t m, const int* __restrict__ rp, const int* __restrict__ ci,
                           const double* __restrict__ va, const double* __restrict__ p, double* __restrict__ y,
                           double* dst, RedScratch rs) {
  pdl_wait();
  // warps stride over the rows uniformly so every lane joins each shuffle
  constexpr int GPW = 32 / VEC;
  const int lane = threadIdx.x % VEC, sub = (threadIdx.x & 31) / VEC;
  const int64_t nwarps = (int64_t)gridDim.x * (BLK / 32);
  double part = 0;
  for (int64_t w = ((int64_t)blockIdx.x * BLK + threadIdx.x) / 32; w * GPW < m; w += nwarps) {
    const int64_t g = w * GPW + sub;
    double s = 0;
    if (g < m)
      for (int k = rp[g] + lane; k < rp[g + 1]; k += VEC) s += va[k] * p[ci[k]];
    s = group_sum<VEC>(s);
    if (g < m && lane == 0) {
      y[g] = s;
      part += s * p[g];
    }
  }
  part = block_sum(part);
  finish_reduction(part, dst, rs);
}

__global__ void k_cg_update_xr(int64_t n, const double* __restrict__ sc, int num, int den, double* __restrict__ x,
                               double* __restrict__ r, const double* __restrict__ p, const double* __restrict__ q,
                               double* dst, RedScratch rs) {
  pdl_wait();
  const double alpha = sc[num] / sc[den];
  double s = 0;
  for (int64_t i = (int64_t)blockIdx.x * BLK + threadIdx.x; i < n; i += (int64_t)gridDim.x * BLK) {
    x[i] += alpha * p[i];
    const double ri = r[i] - alpha * q[i];
    r[i] = ri;
    s += ri * ri;
  }
  s = block_sum(s);
  finish_reduction(s, dst, rs);
}

__global__ void k_cg_update_p(int64_t n, const double* __restrict__ sc, int num, int den, const double* __restrict__ z,
                              double* __restrict__ p) {
  pdl_wait();
  const double beta = sc[num] / sc[den];
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = z[i] + beta * p[i];
}

// ----------------------------------------------------------- setup kernels
__global__ void k_perm_row_len(int64_t m, const int* __restrict__ rp, const int* __restrict__ rperm,
                               int* __restrict__ len) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < m) len[i] = rp[rperm[i] + 1] - rp[rperm[i]];
}

__global__ void k_perm_fill(int64_t m, const int* __restrict__ rp, const int* __restrict__ ci,
                            const double* __restrict__ va, const int* __restrict__ rperm, const int* __restrict__ cmap,
                            const int* __restrict__ orp, int* __restrict__ oci, double* __restrict__ ova) {
  const int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32;
  const int lane = threadIdx.x & 31;
  if (row >= m) return;
  const int src = rp[rperm[row]], len = rp[rperm[row] + 1] - src, dst = orp[row];
  for (int k = lane; k < len; k += 32) {
    oci[dst + k] = cmap[ci[src + k]];
    ova[dst + k] = va[src + k];
  }
}

__global__ void k_l1_diag(int64_t r0, int64_t r1, const int* __restrict__ rp, const int* __restrict__ ci,
                          const double* __restrict__ va, double* __restrict__ d) {
  int64_t j = r0 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= r1) return;
  double s = va[rp[j]];
  for (int k = rp[j] + 1; k < rp[j + 1]; ++k)
    if (ci[k] >= r0 && ci[k] < r1) s += fabs(va[k]);
  d[j - r0] = s;
}

__global__ void k_csr_to_dense(int64_t n, const int* __restrict__ rp, const int* __restrict__ ci,
                               const double* __restrict__ va, double* __restrict__ M) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int k = rp[i]; k < rp[i + 1]; ++k) M[i * n + ci[k]] = va[k];
}

__global__ void k_identity(int64_t n, double* __restrict__ M) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n * n) M[t] = (t / n == t % n) ? 1.0 : 0.0;
}

// pivot search and row swap/scale for column c (one block)
__global__ void k_gj_pivot(int64_t n, int64_t c, double* __restrict__ M, double* __restrict__ I,
                           double* __restrict__ colc, int* __restrict__ singular) {
  __shared__ double bv[1024];
  __shared__ int bi[1024];
  double best = -1.0;
  int arg = (int)c;
  for (int64_t r = c + threadIdx.x; r < n; r += blockDim.x) {
    double a = fabs(M[r * n + c]);
    if (a > best) { best = a; arg = (int)r; }
  }
  bv[threadIdx.x] = best;
  bi[threadIdx.x] = arg;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      double o = bv[threadIdx.x + s];
      int oi = bi[threadIdx.x + s];
      if (o > bv[threadIdx.x] || (o == bv[threadIdx.x] && oi < bi[threadIdx.x])) {
        bv[threadIdx.x] = o;
        bi[threadIdx.x] = oi;
      }
    }
    __syncthreads();
  }
  const int p = bi[0];
  if (bv[0] == 0.0) {
    if (threadIdx.x == 0) *singular = 1;
    return;
  }
  if (p != c)
    for (int64_t k = threadIdx.x; k < n; k += blockDim.x) {
      double t = M[c * n + k]; M[c * n + k] = M[p * n + k]; M[p * n + k] = t;
      t = I[c * n + k]; I[c * n + k] = I[p * n + k]; I[p * n + k] = t;
    }
  __syncthreads();
  const double d = M[c * n + c];
  __syncthreads();
  for (int64_t k = threadIdx.x; k < n; k += blockDim.x) {
    M[c * n + k] /= d;
    I[c * n + k] /= d;
  }
  __syncthreads();
  for (int64_t r = threadIdx.x; r < n; r += blockDim.x) colc[r] = (r == c) ? 0.0 : M[r * n + c];
}

__global__ void k_gj_eliminate(int64_t n, int64_t c, double* __restrict__ M, double* __restrict__ I,
                               const double* __restrict__ colc, const int* __restrict__ singular) {
  if (*singular) return;
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 2 * n * n) return;
  const bool inv = t >= n * n;
  const int64_t u = inv ? t - n * n : t;
  const int64_t r = u / n, k = u % n;
  const double f = colc[r];
  if (f == 0.0) return;
  double* A = inv ? I : M;
  A[r * n + k] -= f * A[c * n + k];
}

// C = alpha A B + beta C in FP64 (row-major, leading dimensions lda, ldb,
// ldc): 64 x 64 output tiles, 16-deep steps of k staged in shared memory,
// 4 x 4 outputs per thread (rows ty + 16a, columns tx + 16b).
__global__ void __launch_bounds__(256) k_dgemm(int64_t m, int64_t n, int64_t k, double alpha,
                                               const double* __restrict__ A, int64_t lda,
                                               const double* __restrict__ B, int64_t ldb, double beta,
                                               double* __restrict__ C, int64_t ldc) {
  __shared__ double As[16][65];
  __shared__ double Bs[16][64];
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  const int64_t row0 = (int64_t)blockIdx.y * 64, col0 = (int64_t)blockIdx.x * 64;
  double acc[4][4] = {};
  for (int64_t k0 = 0; k0 < k; k0 += 16) {
    for (int q = threadIdx.x; q < 64 * 16; q += 256) {
      const int r = q / 16, c = q % 16;
      As[c][r] = (row0 + r < m && k0 + c < k) ? A[(row0 + r) * lda + k0 + c] : 0.0;
      const int br = q / 64, bc = q % 64;
      Bs[br][bc] = (k0 + br < k && col0 + bc < n) ? B[(k0 + br) * ldb + col0 + bc] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < 16; ++kk) {
      double a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int64_t r = row0 + ty + 16 * i, c = col0 + tx + 16 * j;
      if (r < m && c < n) C[r * ldc + c] = alpha * acc[i][j] + (beta == 0.0 ? 0.0 : beta * C[r * ldc + c]);
    }
}

// dst[i][j] = src[i][j] for i < rows, j < cols (row-major, leading dims);
// rows [z0, z1) of dst get zeros instead (z1 <= z0: none).
__global__ void k_copy2d(int64_t rows, int64_t cols, const double* __restrict__ src, int64_t lds,
                         double* __restrict__ dst, int64_t ldd, int64_t z0, int64_t z1) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= rows * cols) return;
  const int64_t i = t / cols, j = t % cols;
  dst[i * ldd + j] = (i >= z0 && i < z1) ? 0.0 : src[i * lds + j];
}

// columns [c0, c1) of a rows x cols row-major block set to zero
__global__ void k_zero_cols(int64_t rows, int64_t cols, double* __restrict__ M, int64_t c0, int64_t c1) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t w = c1 - c0;
  if (t >= rows * w) return;
  M[(t / w) * cols + c0 + t % w] = 0.0;
}

template <class F>
void launch_vec(int vec, F&& f) {
  switch (vec) {
    case 4: f(std::integral_constant<int, 4>()); break;
    case 8: f(std::integral_constant<int, 8>()); break;
    case 16: f(std::integral_constant<int, 16>()); break;
    default: f(std::integral_constant<int, 32>()); break;
  }
}

unsigned red_grid(const afp_context* ctx, int64_t n) {
  int64_t g = (n + BLK - 1) / BLK;
  int64_t cap = std::min<int64_t>(RED_BLOCKS, (int64_t)ctx->sm_count * 2);
  return (unsigned)std::max<int64_t>(1, std::min(g, cap));
}

}  // namespace

template <class V, class X>
void spmv(const afp_context* ctx, const CSRView<V>& A, const X* x, X* y, bool add) {
  launch_vec(A.vec, [&](auto VEC) {
    constexpr int W = decltype(VEC)::value;
    unsigned grid = grid_for(A.m * W, BLK);
    if (add) launch_pdl(ctx->stream, grid, BLK, 0, k_spmv<W, V, X, true>, A.m, A.rowptr, A.cols, A.vals, x, y);
    else launch_pdl(ctx->stream, grid, BLK, 0, k_spmv<W, V, X, false>, A.m, A.rowptr, A.cols, A.vals, x, y);
  });
  check_launch(ctx, "spmv");
}

template <class X>
void residual(const afp_context* ctx, const CSRView<X>& A, const X* x, const X* r, X* out) {
  launch_vec(A.vec, [&](auto VEC) {
    constexpr int W = decltype(VEC)::value;
    launch_pdl(ctx->stream, grid_for(A.m * W, BLK), BLK, 0, k_residual<W, X>, A.m, A.rowptr, A.cols, A.vals, x, r,
               out);
  });
  check_launch(ctx, "residual");
}

template <class X>
void gs_class(const afp_context* ctx, const CSRView<X>& A, int64_t r0, int64_t r1, X* x, const X* r) {
  if (r1 <= r0) return;
  launch_vec(A.vec, [&](auto VEC) {
    constexpr int W = decltype(VEC)::value;
    launch_pdl(ctx->stream, grid_for((r1 - r0) * W, BLK), BLK, 0, k_gs_class<W, X>, r0, r1, A.rowptr, A.cols, A.vals,
               x, r);
  });
  check_launch(ctx, "gauss-seidel class");
}

template <class X>
void jacobi_l1_class(const afp_context* ctx, const CSRView<X>& A, int64_t r0, int64_t r1, X* x, const X* r,
                     const X* l1diag, X* tmp) {
  if (r1 <= r0) return;
  launch_vec(A.vec, [&](auto VEC) {
    constexpr int W = decltype(VEC)::value;
    launch_pdl(ctx->stream, grid_for((r1 - r0) * W, BLK), BLK, 0, k_jacobi_l1<W, X>, r0, r1, A.rowptr, A.cols,
               A.vals, (const X*)x, r, l1diag, tmp);
  });
  check_launch(ctx, "l1-jacobi class");
  launch_pdl(ctx->stream, grid_for(r1 - r0, BLK), BLK, 0, k_copy_range<X>, r1 - r0, (const X*)tmp, x + r0);
  check_launch(ctx, "l1-jacobi copy");
}

template <class X>
void dense_gemv(const afp_context* ctx, int64_t n, const X* Ainv, const X* r, X* x) {
  launch_pdl(ctx->stream, grid_for(n * 32, BLK), BLK, 0, k_dense_gemv<X>, n, Ainv, r, x);
  check_launch(ctx, "dense gemv");
}

void split_df(const afp_context* ctx, int64_t n, int64_t ld, const double* inv, float* hi, float* lo) {
  if (n == 0) return;
  k_split_df<<<grid_for(n * ld, BLK), BLK, 0, ctx->stream>>>(n, ld, inv, hi, lo);
  check_launch(ctx, "double-float split");
}

void dense_gemv_df(const afp_context* ctx, int64_t n, int64_t ld, const float* hi, const float* lo, const float* r,
                   float* x) {
  if (n == 0) return;
  launch_pdl(ctx->stream, grid_for(n * 32, BLK), BLK, 0, k_dense_gemv_df, n, ld, hi, lo, r, x);
  check_launch(ctx, "dense gemv (double-float)");
}

template <class X>
void diag_solve(const afp_context* ctx, const CSRView<X>& A, const X* r, X* x) {
  launch_pdl(ctx->stream, grid_for(A.m, BLK), BLK, 0, k_diag_solve<X>, A.m, A.rowptr, A.vals, r, x);
  check_launch(ctx, "diagonal solve");
}

template <class A, class B>
void convert(const afp_context* ctx, int64_t n, const A* in, B* out) {
  launch_pdl(ctx->stream, grid_for(n, BLK), BLK, 0, k_convert<A, B>, n, in, out);
  check_launch(ctx, "convert");
}

void permute_gather(const afp_context* ctx, int64_t n, const int* perm, const double* in, double* out) {
  k_gather<<<grid_for(n, BLK), BLK, 0, ctx->stream>>>(n, perm, in, out);
  check_launch(ctx, "permute gather");
}

void permute_scatter(const afp_context* ctx, int64_t n, const int* perm, const double* in, double* out) {
  k_scatter<<<grid_for(n, BLK), BLK, 0, ctx->stream>>>(n, perm, in, out);
  check_launch(ctx, "permute scatter");
}

void axpy(const afp_context* ctx, int64_t n, double alpha, const double* x, double* y) {
  k_axpy<<<grid_for(n, BLK), BLK, 0, ctx->stream>>>(n, alpha, x, y);
  check_launch(ctx, "axpy");
}

void strided_copy(const afp_context* ctx, int64_t n, const double* src, int64_t ss, double* dst, int64_t ds) {
  k_strided_copy<<<grid_for(n, BLK), BLK, 0, ctx->stream>>>(n, src, ss, dst, ds);
  check_launch(ctx, "strided copy");
}

template <class X>
void fill_zero(const afp_context* ctx, int64_t n, X* x) {
  launch_pdl(ctx->stream, grid_for(n, BLK), BLK, 0, k_zero<X>, n, x);
  check_launch(ctx, "zero");
}

void dot(const afp_context* ctx, int64_t n, const double* a, const double* b, double* dst) {
  launch_pdl(ctx->stream, red_grid(ctx, n), BLK, 0, k_dot, n, a, b, dst, RedScratch{ctx->d_partials, ctx->d_retire});
  check_launch(ctx, "dot");
}

void spmv_dot(const afp_context* ctx, const CSRView<double>& A, const double* p, double* y, double* dst) {
  launch_vec(A.vec, [&](auto VEC) {
    constexpr int W = decltype(VEC)::value;
    launch_pdl(ctx->stream, red_grid(ctx, A.m * W), BLK, 0, k_spmv_dot<W>, A.m, A.rowptr, A.cols, A.vals, p, y, dst,
               RedScratch{ctx->d_partials, ctx->d_retire});
  });
  check_launch(ctx, "spmv+dot");
}

void cg_update_xr(const afp_context* ctx, int64_t n, const double* s, int num, int den, double* x, double* r,
                  const double* p, const double* q, double* dst) {
  launch_pdl(ctx->stream, red_grid(ctx, n), BLK, 0, k_cg_update_xr, n, s, num, den, x, r, p, q, dst,
             RedScratch{ctx->d_partials, ctx->d_retire});
  check_launch(ctx, "cg update x r");
}

void cg_update_p(const afp_context* ctx, int64_t n, const double* s, int num, int den, const double* z, double* p) {
  launch_pdl(ctx->stream, grid_for(n, BLK), BLK, 0, k_cg_update_p, n, s, num, den, z, p);
  check_launch(ctx, "cg update p");
}

void permute_csr(const afp_context* ctx, int64_t m, const int* rowptr, const int* cols, const double* vals,
                 const int* rperm, const int* cmap, int64_t nnz, DevBuf<int>& orp, DevBuf<int>& oci,
                 DevBuf<double>& ova) {
  DevBuf<int> len(ctx, m);
  k_perm_row_len<<<grid_for(m, BLK), BLK, 0, ctx->stream>>>(m, rowptr, rperm, len.get());
  check_launch(ctx, "permute row lengths");
  orp.alloc(ctx, m + 1);
  int64_t total = exclusive_scan(ctx, len.get(), orp.get(), m);
  AFP_REQUIRE(total == nnz, AFP_ERR_CUDA, "permutation lost entries");
  oci.alloc(ctx, nnz);
  ova.alloc(ctx, nnz);
  k_perm_fill<<<grid_for(m * 32, BLK), BLK, 0, ctx->stream>>>(m, rowptr, cols, vals, rperm, cmap, orp.get(),
                                                              oci.get(), ova.get());
  check_launch(ctx, "permute fill");
}

void l1_diag(const afp_context* ctx, const CSRView<double>& A, int64_t r0, int64_t r1, double* d) {
  if (r1 <= r0) return;
  k_l1_diag<<<grid_for(r1 - r0, BLK), BLK, 0, ctx->stream>>>(r0, r1, A.rowptr, A.cols, A.vals, d);
  check_launch(ctx, "l1 diagonal");
}

namespace {

// inv = M^-1 for a dense n x n row-major M (overwritten) by Gauss-Jordan
// elimination with partial pivoting, two launches per column; false when a
// pivot is zero.
bool gj_inverse(const afp_context* ctx, int64_t n, double* M, double* inv) {
  DevBuf<double> colc(ctx, n);
  DevBuf<int> singular(ctx, 1);
  singular.zero();
  k_identity<<<grid_for(n * n, BLK), BLK, 0, ctx->stream>>>(n, inv);
  check_launch(ctx, "identity");
  for (int64_t c = 0; c < n; ++c) {
    k_gj_pivot<<<1, 1024, 0, ctx->stream>>>(n, c, M, inv, colc.get(), singular.get());
    check_launch(ctx, "gauss-jordan pivot");
    k_gj_eliminate<<<grid_for(2 * n * n, BLK), BLK, 0, ctx->stream>>>(n, c, M, inv, colc.get(), singular.get());
    check_launch(ctx, "gauss-jordan eliminate");
  }
  int hs = 0;
  singular.download(&hs, 1);
  sync(ctx);
  return hs == 0;
}

void dgemm(const afp_context* ctx, int64_t m, int64_t n, int64_t k, double alpha, const double* A, int64_t lda,
           const double* B, int64_t ldb, double beta, double* C, int64_t ldc) {
  if (m == 0 || n == 0) return;
  dim3 grid((unsigned)((n + 63) / 64), (unsigned)((m + 63) / 64));
  k_dgemm<<<grid, 256, 0, ctx->stream>>>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
  check_launch(ctx, "dgemm");
}

void copy2d(const afp_context* ctx, int64_t rows, int64_t cols, const double* src, int64_t lds, double* dst,
            int64_t ldd, int64_t z0 = 0, int64_t z1 = 0) {
  if (rows * cols == 0) return;
  k_copy2d<<<grid_for(rows * cols, BLK), BLK, 0, ctx->stream>>>(rows, cols, src, lds, dst, ldd, z0, z1);
  check_launch(ctx, "copy block");
}

}  // namespace

// Dense inverse of an SPD matrix (the coarsest level of the hierarchy).  Up
// to kPanel rows: Gauss-Jordan with partial pivoting.  Larger: the blocked
// sweep in place on the output, kPanel pivots at a time -- with the block
// pivot P, the panel rows R, the panel columns C and the rest S,
//   P <- P^-1,  R <- P^-1 R,  S <- S - C P^-1 R,  C <- -C P^-1,
// which after every panel leaves the inverse; the updates are FP64 GEMMs
// (2 n^3 flops in all).  A symmetric positive definite matrix needs no
// pivoting across panels (every block pivot is a Schur complement of it,
// itself SPD); within a pivot block the Gauss-Jordan pivots rows.
bool dense_inverse(const afp_context* ctx, const CSRView<double>& A, double* inv) {
  constexpr int64_t kPanel = 512;
  const int64_t n = A.m;
  if (n <= kPanel) {
    DevBuf<double> M(ctx, n * n);
    M.zero();
    k_csr_to_dense<<<grid_for(n, BLK), BLK, 0, ctx->stream>>>(n, A.rowptr, A.cols, A.vals, M.get());
    check_launch(ctx, "dense copy");
    return gj_inverse(ctx, n, M.get(), inv);
  }
  AFP_CUDA(cudaMemsetAsync(inv, 0, sizeof(double) * n * n, ctx->stream));
  k_csr_to_dense<<<grid_for(n, BLK), BLK, 0, ctx->stream>>>(n, A.rowptr, A.cols, A.vals, inv);
  check_launch(ctx, "dense copy");
  const int64_t b = kPanel;
  DevBuf<double> Pm(ctx, b * b), Pi(ctx, b * b), Rnew(ctx, b * n), Ccol(ctx, n * b), Crow(ctx, b * n);
  for (int64_t k0 = 0; k0 < n; k0 += b) {
    const int64_t k1 = std::min(n, k0 + b), pb = k1 - k0;
    copy2d(ctx, pb, pb, inv + k0 * n + k0, n, Pm.get(), pb);                   // P
    if (!gj_inverse(ctx, pb, Pm.get(), Pi.get())) return false;                 // P^-1
    copy2d(ctx, pb, n, inv + k0 * n, n, Crow.get(), n);                         // R (whole panel rows)
    copy2d(ctx, n, pb, inv + k0, n, Ccol.get(), pb, k0, k1);                    // C (panel rows zeroed)
    dgemm(ctx, pb, n, pb, 1.0, Pi.get(), pb, Crow.get(), n, 0.0, Rnew.get(), n);  // P^-1 R
    k_zero_cols<<<grid_for(pb * pb, BLK), BLK, 0, ctx->stream>>>(pb, n, Rnew.get(), k0, k1);
    check_launch(ctx, "zero panel columns");
    dgemm(ctx, n, n, pb, -1.0, Ccol.get(), pb, Rnew.get(), n, 1.0, inv, n);    // S - C P^-1 R
    copy2d(ctx, pb, n, Rnew.get(), n, inv + k0 * n, n);                         // panel rows
    copy2d(ctx, pb, pb, Pi.get(), pb, inv + k0 * n + k0, n);                    // pivot block
    dgemm(ctx, n, pb, pb, -1.0, Ccol.get(), pb, Pi.get(), pb, 0.0, Crow.get(), pb);  // -C P^-1 (into Crow)
    copy2d(ctx, n, pb, Crow.get(), pb, inv + k0, n, k0, k1);                    // panel columns...
    copy2d(ctx, pb, pb, Pi.get(), pb, inv + k0 * n + k0, n);                    // ...except the pivot block
  }
  sync(ctx);
  return true;
}

void csr_spmv(const afp_context* ctx, int64_t m, const int* rowptr, const int* cols, const double* vals,
              const double* x, double* y) {
  // A plain launch, without the PDL attribute: k_spmv loads the matrix before
  // griddepcontrol.wait, and the caller's preceding kernel on this stream
  // (assembly, Dirichlet rows, a value upload) may be the one writing it.
  if (m == 0) return;
  k_spmv<8, double, double, false><<<grid_for(m * 8, BLK), BLK, 0, ctx->stream>>>(m, rowptr, cols, vals, x, y);
  check_launch(ctx, "spmv");
}

// explicit instantiations
template void spmv<double, double>(const afp_context*, const CSRView<double>&, const double*, double*, bool);
template void spmv<float, float>(const afp_context*, const CSRView<float>&, const float*, float*, bool);
template void spmv<__nv_bfloat16, float>(const afp_context*, const CSRView<__nv_bfloat16>&, const float*, float*,
                                         bool);
template void residual<double>(const afp_context*, const CSRView<double>&, const double*, const double*, double*);
template void residual<float>(const afp_context*, const CSRView<float>&, const float*, const float*, float*);
template void gs_class<double>(const afp_context*, const CSRView<double>&, int64_t, int64_t, double*, const double*);
template void gs_class<float>(const afp_context*, const CSRView<float>&, int64_t, int64_t, float*, const float*);
template void jacobi_l1_class<double>(const afp_context*, const CSRView<double>&, int64_t, int64_t, double*,
                                      const double*, const double*, double*);
template void jacobi_l1_class<float>(const afp_context*, const CSRView<float>&, int64_t, int64_t, float*,
                                     const float*, const float*, float*);
template void dense_gemv<double>(const afp_context*, int64_t, const double*, const double*, double*);
template void dense_gemv<float>(const afp_context*, int64_t, const float*, const float*, float*);
template void diag_solve<double>(const afp_context*, const CSRView<double>&, const double*, double*);
template void diag_solve<float>(const afp_context*, const CSRView<float>&, const float*, float*);
template void convert<double, float>(const afp_context*, int64_t, const double*, float*);
template void convert<float, double>(const afp_context*, int64_t, const float*, double*);
template void convert<double, __nv_bfloat16>(const afp_context*, int64_t, const double*, __nv_bfloat16*);
template void fill_zero<double>(const afp_context*, int64_t, double*);
template void fill_zero<float>(const afp_context*, int64_t, float*);

}  // namespace afp
