// Galerkin coarse operator A_c = P A P^T on the GPU (AMGSolver::getPMPt,
// src/AMGSolver.cpp:288-358).
//
// Symbolic phase: one warp (or, for long rows, one block) per coarse row
// collects the column set {c : c in Pt[b], b in A[a], a in P[i]} in a
// shared-memory hash set, then sorts it and writes the row as
// [i, ascending others] -- the pattern getPMPt builds and compresses.
//
// Numeric phase: one warp per coarse row walks the (j, k) pairs of the
// triple loop in the reference's order (P row ascending, A row in stored
// order), and the lanes take the entries l of the Pt row, whose columns are
// distinct, so every output entry receives its products in exactly the
// reference's order: row_entry[c] += P(i,a)*A(a,b)*Pt(b,c).  Compiled with
// -fmad=false, the result is bitwise that of getPMPt.
#include <algorithm>
#include <climits>
#include <vector>

#include "common.cuh"
#include "kernels.cuh"

namespace afp {
namespace {

constexpr int WARP_CAP = 1024;      // hash slots of the warp-level symbolic pass
constexpr int BLOCK_CAP = 16384;    // hash slots of the block-level pass (2 x 64 KB of shared memory)
constexpr size_t NUM_SMEM_MAX = 200 * 1024;  // shared memory the numeric pass may use per block

__device__ __forceinline__ unsigned hash_slot(int key, int cap) {
  return ((unsigned)key * 2654435761u) & (unsigned)(cap - 1);
}

// Inserts key; returns 1 if it was new.  cap is a power of two.
__device__ __forceinline__ int hash_insert(int* table, int cap, int key) {
  unsigned s = hash_slot(key, cap);
  for (int probe = 0; probe < cap; ++probe) {
    int prev = atomicCAS(&table[s], -1, key);
    if (prev == -1) return 1;
    if (prev == key) return 0;
    s = (s + 1) & (unsigned)(cap - 1);
  }
  return 0;  // table full: caller checks the count against the capacity
}

template <int GROUP>
__device__ __forceinline__ void group_bitonic_sort(int* buf, int P, int tid) {
  for (int k = 2; k <= P; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int t = tid; t < P; t += GROUP) {
        int ixj = t ^ j;
        if (ixj > t) {
          int a = buf[t], b = buf[ixj];
          bool up = (t & k) == 0;
          if ((a > b) == up) {
            buf[t] = b;
            buf[ixj] = a;
          }
        }
      }
      if (GROUP == 32) __syncwarp(); else __syncthreads();
    }
  }
}

// Collects the coarse row's column set with GROUP threads (a warp or a block).
// Returns the unique count (may exceed 0.75*cap: the caller re-routes the row).
template <int GROUP>
__device__ int collect_row(int64_t i, const int* __restrict__ prp, const int* __restrict__ pc,
                           const int* __restrict__ arp, const int* __restrict__ ac, const int* __restrict__ trp,
                           const int* __restrict__ tc, int* table, int cap, int tid, int* red) {
  for (int t = tid; t < cap; t += GROUP) table[t] = -1;
  if (GROUP == 32) __syncwarp(); else __syncthreads();
  int mine = 0;
  const int limit = (cap * 3) / 4;
  for (int j = prp[i]; j < prp[i + 1]; ++j) {
    const int a = pc[j];
    const int kb = arp[a], ke = arp[a + 1];
    for (int k = kb + tid; k < ke; k += GROUP) {
      const int b = ac[k];
      for (int l = trp[b]; l < trp[b + 1]; ++l) mine += hash_insert(table, cap, tc[l]);
    }
    if (GROUP == 32) {
      // a row that outgrows the warp's table goes to the block pass: stop
      // here instead of probing a full table for the rest of its products
      int c = mine;
      for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
      if (c > limit) return c;
    }
  }
  // reduce the count
  int cnt = mine;
  if (GROUP == 32) {
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_down_sync(0xffffffffu, cnt, o);
    cnt = __shfl_sync(0xffffffffu, cnt, 0);
  } else {
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_down_sync(0xffffffffu, cnt, o);
    if ((tid & 31) == 0) atomicAdd(red, cnt);
    __syncthreads();
    cnt = *red;
    __syncthreads();
  }
  return cnt;
}

// Sorts the collected set into `out` as [i, ascending others].
template <int GROUP>
__device__ void emit_row(int64_t i, int* table, int* buf, int cap, int cnt, int tid, int* out, int* red) {
  // compact the table into buf
  if (GROUP == 32) {
    int base = 0;
    for (int t0 = 0; t0 < cap; t0 += 32) {
      int t = t0 + tid;
      int key = table[t];
      bool keep = key >= 0 && key != (int)i;
      unsigned mask = __ballot_sync(0xffffffffu, keep);
      if (keep) buf[base + __popc(mask & ((1u << tid) - 1u))] = key;
      base += __popc(mask);
    }
    __syncwarp();
  } else {
    if (tid == 0) *red = 0;
    __syncthreads();
    for (int t = tid; t < cap; t += GROUP) {
      int key = table[t];
      if (key >= 0 && key != (int)i) buf[atomicAdd(red, 1)] = key;
    }
    __syncthreads();
  }
  const int m = cnt - 1;
  int P = 1;
  while (P < m) P <<= 1;
  for (int t = m + tid; t < P; t += GROUP) buf[t] = INT_MAX;
  if (GROUP == 32) __syncwarp(); else __syncthreads();
  group_bitonic_sort<GROUP>(buf, P, tid);
  if (tid == 0) out[0] = (int)i;
  for (int t = tid; t < m; t += GROUP) out[1 + t] = buf[t];
  if (GROUP == 32) __syncwarp(); else __syncthreads();
}

// Warp-level symbolic pass over all rows.  count mode (rowptr == nullptr):
// row_len[i] = unique count, or -1 when the row needs the block-level pass.
__global__ void k_rap_symbolic_warp(int64_t n_c, const int* prp, const int* pc, const int* arp, const int* ac,
                                    const int* trp, const int* tc, int* row_len, const int* rowptr, int* cols,
                                    const unsigned char* big_flag) {
  extern __shared__ int sm_rap[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, wpb = blockDim.x >> 5;
  int* table = sm_rap + warp * 2 * WARP_CAP;
  int* buf = table + WARP_CAP;
  for (int64_t i = (int64_t)blockIdx.x * wpb + warp; i < n_c; i += (int64_t)gridDim.x * wpb) {
    if (rowptr != nullptr && big_flag[i]) continue;  // handled by the block pass
    int cnt = collect_row<32>(i, prp, pc, arp, ac, trp, tc, table, WARP_CAP, lane, nullptr);
    if (rowptr == nullptr) {
      if (lane == 0) row_len[i] = (cnt > (WARP_CAP * 3) / 4) ? -1 : cnt;
    } else {
      emit_row<32>(i, table, buf, WARP_CAP, cnt, lane, cols + rowptr[i], nullptr);
    }
    __syncwarp();
  }
}

// Block-level symbolic pass over the rows listed in `rows`.
__global__ void k_rap_symbolic_block(const int* rows, int n_rows, int cap, const int* prp, const int* pc,
                                     const int* arp, const int* ac, const int* trp, const int* tc, int* row_len,
                                     const int* rowptr, int* cols, int* overflow) {
  extern __shared__ int sm_rapb[];
  __shared__ int red;
  int* table = sm_rapb;
  int* buf = sm_rapb + cap;
  for (int r = blockIdx.x; r < n_rows; r += gridDim.x) {
    const int64_t i = rows[r];
    if (threadIdx.x == 0) red = 0;
    __syncthreads();
    int cnt = collect_row<256>(i, prp, pc, arp, ac, trp, tc, table, cap, threadIdx.x, &red);
    if (rowptr == nullptr) {
      if (threadIdx.x == 0) {
        if (cnt > (cap * 3) / 4) atomicExch(overflow, 1);
        row_len[i] = cnt;
      }
    } else {
      emit_row<256>(i, table, buf, cap, cnt, threadIdx.x, cols + rowptr[i], &red);
    }
    __syncthreads();
  }
}

__global__ void k_collect_big(const int* row_len, int64_t n, int* rows, int* count, unsigned char* big_flag) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const bool big = row_len[i] < 0;
  big_flag[i] = big;
  if (big) rows[atomicAdd(count, 1)] = (int)i;
}

__device__ __forceinline__ int find_slot(const int* c, int R, int key, int row) {
  if (key == row) return 0;
  int lo = 1, hi = R;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (c[mid] < key) lo = mid + 1; else hi = mid;
  }
  return lo;
}

// Numeric pass: exact reference accumulation order (see file comment).
// Rows of up to acc_cap entries accumulate in the warp's slice of shared
// memory (their column list too, for the slot searches); longer rows in
// place in global memory.  acc_cap is sized by the host from the product's
// longest row, so the nearly dense coarse levels of 3D hierarchies stay in
// shared memory as well.  With MAP (coarse levels of at most a few ten
// thousand rows), each warp also keeps a column -> slot table of n_c
// entries, so a product finds its entry with one shared load instead of a
// binary search over the row.
template <bool MAP>
__global__ void k_rap_numeric(int64_t n_c, const int* __restrict__ prp, const int* __restrict__ pc,
                              const double* __restrict__ pv, const int* __restrict__ arp, const int* __restrict__ ac,
                              const double* __restrict__ av, const int* __restrict__ trp, const int* __restrict__ tc,
                              const double* __restrict__ tv, const int* __restrict__ rowptr,
                              const int* __restrict__ cols, double* __restrict__ vals, int acc_cap) {
  extern __shared__ __align__(16) unsigned char sm_num[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, wpb = blockDim.x >> 5;
  double* sacc = reinterpret_cast<double*>(sm_num) + (size_t)warp * acc_cap;
  int* scol = reinterpret_cast<int*>(reinterpret_cast<double*>(sm_num) + (size_t)wpb * acc_cap) + warp * acc_cap;
  unsigned short* smap = reinterpret_cast<unsigned short*>(reinterpret_cast<int*>(
                             reinterpret_cast<double*>(sm_num) + (size_t)wpb * acc_cap) + (size_t)wpb * acc_cap) +
                         (size_t)warp * (MAP ? n_c : 0);
  if (MAP) {
    for (int64_t t = lane; t < n_c; t += 32) smap[t] = 0xFFFFu;
    __syncwarp();
  }
  for (int64_t i = (int64_t)blockIdx.x * wpb + warp; i < n_c; i += (int64_t)gridDim.x * wpb) {
    const int r0 = rowptr[i], R = rowptr[i + 1] - r0;
    const bool in_smem = R <= acc_cap;
    double* acc = in_smem ? sacc : vals + r0;
    const int* rc = in_smem ? scol : cols + r0;
    for (int t = lane; t < R; t += 32) {
      acc[t] = 0.0;
      if (in_smem) scol[t] = cols[r0 + t];
      if (MAP) smap[cols[r0 + t]] = (unsigned short)t;
    }
    __syncwarp();
    for (int j = prp[i]; j < prp[i + 1]; ++j) {
      const int a = pc[j];
      const double p = pv[j];
      for (int k = arp[a]; k < arp[a + 1]; ++k) {
        const int b = ac[k];
        const double pm = p * av[k];
        for (int l = trp[b] + lane; l < trp[b + 1]; l += 32) {
          const int slot = MAP ? (int)smap[tc[l]] : find_slot(rc, R, tc[l], (int)i);
          acc[slot] += pm * tv[l];
        }
        __syncwarp();
      }
    }
    if (in_smem)
      for (int t = lane; t < R; t += 32) vals[r0 + t] = sacc[t];
    if (MAP)
      for (int t = lane; t < R; t += 32) smap[cols[r0 + t]] = 0xFFFFu;
    __syncwarp();
  }
}

// The symbolic count of the product: row_len[i] = the unique columns of
// coarse row i, found by warps, or by blocks for rows that outgrow a warp's
// table (listed in big, flagged in big_flag).
struct SymbolicCount {
  DevBuf<int> row_len, big;
  DevBuf<unsigned char> big_flag;
  int hbig = 0, bcap = 1;
  size_t smem_w = 0, smem_b = 0;
  unsigned grid = 1;
};
constexpr int SYM_WPB = 4;

// n_c rows of P; n_cols = columns of the product (sizes the block-level table)
void symbolic_count(const afp_context* ctx, int64_t n_c, int64_t n_cols, const int* prp, const int* pc,
                    const int* arp, const int* ac, const int* trp, const int* tc, SymbolicCount& sc) {
  sc.smem_w = (size_t)SYM_WPB * 2 * WARP_CAP * sizeof(int);
  AFP_CUDA(cudaFuncSetAttribute(k_rap_symbolic_warp, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sc.smem_w));
  sc.grid = (unsigned)std::min<int64_t>((n_c + SYM_WPB - 1) / SYM_WPB, (int64_t)ctx->sm_count * 16);
  sc.row_len.alloc(ctx, n_c);
  k_rap_symbolic_warp<<<sc.grid, SYM_WPB * 32, sc.smem_w, ctx->stream>>>(n_c, prp, pc, arp, ac, trp, tc,
                                                                         sc.row_len.get(), nullptr, nullptr, nullptr);
  check_launch(ctx, "rap symbolic count");
  // rows whose column set does not fit the warp table go to the block pass
  DevBuf<int> nbig(ctx, 1), overflow(ctx, 1);
  sc.big.alloc(ctx, n_c);
  sc.big_flag.alloc(ctx, n_c);
  nbig.zero();
  overflow.zero();
  k_collect_big<<<grid_for(n_c, 256), 256, 0, ctx->stream>>>(sc.row_len.get(), n_c, sc.big.get(), nbig.get(),
                                                             sc.big_flag.get());
  check_launch(ctx, "rap big rows");
  nbig.download(&sc.hbig, 1);
  sync(ctx);
  while (sc.bcap < 2 * n_cols && sc.bcap < BLOCK_CAP) sc.bcap <<= 1;
  sc.smem_b = (size_t)2 * sc.bcap * sizeof(int);
  if (sc.hbig > 0) {
    AFP_CUDA(cudaFuncSetAttribute(k_rap_symbolic_block, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sc.smem_b));
    k_rap_symbolic_block<<<(unsigned)std::min(sc.hbig, ctx->sm_count * 2), 256, sc.smem_b, ctx->stream>>>(
        sc.big.get(), sc.hbig, sc.bcap, prp, pc, arp, ac, trp, tc, sc.row_len.get(), nullptr, nullptr,
        overflow.get());
    check_launch(ctx, "rap symbolic count (block)");
    int hov = 0;
    overflow.download(&hov, 1);
    sync(ctx);
    AFP_REQUIRE(!hov, AFP_ERR_UNSUPPORTED, "Galerkin product row longer than the block-level table");
  }
}

}  // namespace

int64_t galerkin_nnz(const afp_context* ctx, int64_t n_rows, int64_t n_c, const int* prp, const int* pc,
                     const int* arp, const int* ac, const int* trp, const int* tc) {
  SymbolicCount sc;
  symbolic_count(ctx, n_rows, n_c, prp, pc, arp, ac, trp, tc, sc);
  DevBuf<int> rowptr(ctx, n_rows + 1);
  return exclusive_scan(ctx, sc.row_len.get(), rowptr.get(), n_rows);
}

void galerkin_product(const afp_context* ctx, int64_t n_c, int64_t n_f, const int* prp, const int* pc,
                      const double* pv, const int* arp, const int* ac, const double* av, const int* trp,
                      const int* tc, const double* tv, Pattern& out, DevBuf<double>& vals) {
  (void)n_f;
  SymbolicCount sc;
  symbolic_count(ctx, n_c, n_c, prp, pc, arp, ac, trp, tc, sc);
  const int hbig = sc.hbig, bcap = sc.bcap;
  const size_t smem_w = sc.smem_w, smem_b = sc.smem_b;
  const unsigned grid = sc.grid;
  const int wpb = SYM_WPB;
  DevBuf<int>& row_len = sc.row_len;
  DevBuf<int>& big = sc.big;
  DevBuf<unsigned char>& big_flag = sc.big_flag;
  DevBuf<int> overflow(ctx, 1);
  overflow.zero();
  out.m = out.n = n_c;
  out.rowptr.alloc(ctx, n_c + 1);
  out.nnz = exclusive_scan(ctx, row_len.get(), out.rowptr.get(), n_c);
  out.cols.alloc(ctx, out.nnz);
  if (hbig > 0) {
    k_rap_symbolic_block<<<(unsigned)std::min(hbig, ctx->sm_count * 2), 256, smem_b, ctx->stream>>>(
        big.get(), hbig, bcap, prp, pc, arp, ac, trp, tc, row_len.get(), out.rowptr.get(), out.cols.get(),
        overflow.get());
    check_launch(ctx, "rap symbolic fill (block)");
  }
  k_rap_symbolic_warp<<<grid, wpb * 32, smem_w, ctx->stream>>>(n_c, prp, pc, arp, ac, trp, tc, row_len.get(),
                                                               out.rowptr.get(), out.cols.get(), big_flag.get());
  check_launch(ctx, "rap symbolic fill");
  vals.alloc(ctx, out.nnz);
  // shared-memory accumulator per warp: the longest row (at least 1024
  // entries), with fewer warps per block when rows are long
  int rmax = 0;
  {
    std::vector<int> rp(n_c + 1);
    out.rowptr.download(rp.data(), n_c + 1);
    sync(ctx);
    for (int64_t i = 0; i < n_c; ++i) rmax = std::max(rmax, rp[i + 1] - rp[i]);
  }
  const size_t per_entry = sizeof(double) + sizeof(int);
  int acc_cap = std::max(1024, (rmax + 31) / 32 * 32);
  // the column -> slot table: rows long enough for the binary search to
  // matter (a hundred entries and more) on levels small enough for a table
  // of n_c 16-bit slots per warp, as long as the table costs no warps per
  // block or the rows are long enough (a thousand entries) that one lookup
  // instead of a deep search is worth fewer warps
  auto warps_for = [&](size_t extra) {
    int w = 4;
    while (w > 1 && (size_t)w * (acc_cap * per_entry + extra) > NUM_SMEM_MAX) --w;
    return w;
  };
  const size_t map_bytes = (size_t)n_c * sizeof(unsigned short);
  const size_t map_extra = (map_bytes + 15) / 16 * 16;
  const bool map = rmax >= 128 && rmax < 65535 && map_bytes <= 64 * 1024 &&
                   (warps_for(map_extra) == warps_for(0) || rmax >= 1024);
  const size_t per_warp_extra = map ? map_extra : 0;
  const int wpn = warps_for(per_warp_extra);
  if ((size_t)acc_cap * per_entry + per_warp_extra > NUM_SMEM_MAX)  // longest rows accumulate in global memory
    acc_cap = (int)((NUM_SMEM_MAX - per_warp_extra) / per_entry) / 32 * 32;
  const size_t smem_n = (size_t)wpn * (acc_cap * per_entry + per_warp_extra);
  const unsigned grid_n = (unsigned)std::min<int64_t>((n_c + wpn - 1) / wpn, (int64_t)ctx->sm_count * 16);
  if (map) {
    AFP_CUDA(cudaFuncSetAttribute(k_rap_numeric<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_n));
    k_rap_numeric<true><<<grid_n, wpn * 32, smem_n, ctx->stream>>>(
        n_c, prp, pc, pv, arp, ac, av, trp, tc, tv, out.rowptr.get(), out.cols.get(), vals.get(), acc_cap);
  } else {
    AFP_CUDA(cudaFuncSetAttribute(k_rap_numeric<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_n));
    k_rap_numeric<false><<<grid_n, wpn * 32, smem_n, ctx->stream>>>(
        n_c, prp, pc, pv, arp, ac, av, trp, tc, tv, out.rowptr.get(), out.cols.get(), vals.get(), acc_cap);
  }
  check_launch(ctx, "rap numeric");
}

}  // namespace afp

// ------------------------------------------------------------------------
// Galerkin product of the dense tail.  The coarsest level is only inverted,
// never split again, so it does not need getPMPt's accumulation order; with
// at most a few thousand coarse rows it is formed through a dense
// intermediate instead: T = A P^T (n_f x n_c, one thread per row of A,
// accumulating in A's and then P^T's entry order), then A_c = P T (one block
// per coarse row, P's entry order), both FP64 and deterministic.  The result
// is returned in AFEPack's CSR layout (diagonal first, then ascending),
// keeping the entries that are not exactly zero.
namespace afp {
namespace {

__global__ void k_rap_dense_t(int64_t nf, int64_t nc, const int* __restrict__ arp, const int* __restrict__ ac,
                              const double* __restrict__ av, const int* __restrict__ trp,
                              const int* __restrict__ tc, const double* __restrict__ tv, double* __restrict__ T) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nf) return;
  double* Ti = T + i * nc;
  for (int q = arp[i]; q < arp[i + 1]; ++q) {
    const double a = av[q];
    const int k = ac[q];
    for (int s = trp[k]; s < trp[k + 1]; ++s) Ti[tc[s]] += a * tv[s];
  }
}

__global__ void k_rap_dense_pt(int64_t nc, const int* __restrict__ prp, const int* __restrict__ pc,
                               const double* __restrict__ pv, const double* __restrict__ T, double* __restrict__ Ac) {
  const int64_t c = blockIdx.x;
  const int b = prp[c], e = prp[c + 1];
  for (int64_t j = threadIdx.x; j < nc; j += blockDim.x) {
    double s = 0.0;
    for (int q = b; q < e; ++q) s += pv[q] * T[(int64_t)pc[q] * nc + j];
    Ac[c * nc + j] = s;
  }
}

// entries of dense row c that are kept: the diagonal always, others if != 0
__global__ void k_dense_row_count(int64_t n, const double* __restrict__ D, int* __restrict__ cnt) {
  const int64_t c = blockIdx.x;
  int local = 0;
  for (int64_t j = threadIdx.x; j < n; j += blockDim.x) local += (j == c || D[c * n + j] != 0.0) ? 1 : 0;
  __shared__ int red[256];
  red[threadIdx.x] = local;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) cnt[c] = red[0];
}

// one thread per row: the diagonal first, then the others in ascending order
__global__ void k_dense_row_fill(int64_t n, const double* __restrict__ D, const int* __restrict__ rp,
                                 int* __restrict__ ci, double* __restrict__ va) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  int o = rp[c];
  ci[o] = (int)c;
  va[o] = D[c * n + c];
  ++o;
  for (int64_t j = 0; j < n; ++j)
    if (j != c && D[c * n + j] != 0.0) {
      ci[o] = (int)j;
      va[o] = D[c * n + j];
      ++o;
    }
}

}  // namespace

void galerkin_product_dense(const afp_context* ctx, int64_t n_c, int64_t n_f, const int* prp, const int* pc,
                            const double* pv, const int* arp, const int* ac, const double* av, const int* trp,
                            const int* tc, const double* tv, Pattern& out, DevBuf<double>& vals) {
  DevBuf<double> T(ctx, n_f * n_c), D(ctx, n_c * n_c);
  T.zero();
  k_rap_dense_t<<<grid_for(n_f, 128), 128, 0, ctx->stream>>>(n_f, n_c, arp, ac, av, trp, tc, tv, T.get());
  check_launch(ctx, "dense Galerkin A P^T");
  k_rap_dense_pt<<<(unsigned)n_c, 256, 0, ctx->stream>>>(n_c, prp, pc, pv, T.get(), D.get());
  check_launch(ctx, "dense Galerkin P (A P^T)");
  T = DevBuf<double>();
  DevBuf<int> cnt(ctx, n_c);
  k_dense_row_count<<<(unsigned)n_c, 256, 0, ctx->stream>>>(n_c, D.get(), cnt.get());
  check_launch(ctx, "dense row count");
  out.m = out.n = n_c;
  out.rowptr.alloc(ctx, n_c + 1);
  out.nnz = exclusive_scan(ctx, cnt.get(), out.rowptr.get(), n_c);
  out.cols.alloc(ctx, out.nnz);
  vals.alloc(ctx, out.nnz);
  k_dense_row_fill<<<grid_for(n_c, 128), 128, 0, ctx->stream>>>(n_c, D.get(), out.rowptr.get(), out.cols.get(),
                                                                 vals.get());
  check_launch(ctx, "dense row fill");
  sync(ctx);
}

}  // namespace afp
