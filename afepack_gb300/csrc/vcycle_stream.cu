// The FP32 V-cycle as one persistent kernel that streams its operators
// through shared memory.
//
// As a chain of kernels the V-cycle is ~130 dependent launches (one per
// Gauss-Seidel colour class and sweep), each moving 2-20 MB: launch gaps and
// the dependent round trips at the start of each kernel (row bounds, then
// columns and values, then x) dominate.  Here one co-resident grid (one CTA
// per SM) walks a phase program built at setup
//
//   start (x0 = 0, r0 = FP32(r)) | GS class | l1-Jacobi class | residual |
//   restriction (+ next level's x = 0) | dense tail | prolongation | finish
//
// The operators are constant during a solve, so each CTA's share of every
// phase -- tiles of up to 256 CSR rows, each a blob of row offsets and
// 32-byte groups of four (column, value) pairs -- is copied global -> shared
// by the bulk-copy engine (cp.async.bulk, completion on an mbarrier) into a
// ring of slots by one producer warp.  The producer runs ahead of the 16
// consumer warps by up to the ring's depth and keeps streaming while they
// wait between phases.  Consumers take a phase's tiles in waves of up to
// three, flatten their rows, read each group as two 128-bit shared loads,
// gather its four x values (sixteen gathers in flight per lane), and reduce a
// row's products over its lanes with warp shuffles.
//
// Each colour class is split into one run of rows per CTA, balanced by
// stored entries; a CTA keeps the same runs in every phase, so every entry of
// x has one owner.  Between two colour classes of a level a CTA waits only
// for the CTAs whose rows are coupled to its own (nb_sync); level changes,
// the tail and the start and end use a grid barrier.  The l1-Jacobi overflow
// class couples its own rows: it reads their old values from a snapshot that
// the owning CTA writes for its own overflow rows at the end of the phase
// before (a Gauss-Seidel class, or the prolongation, which writes those rows),
// so the Jacobi phase updates x in place without a copy-back phase.
//
// Every wait is bounded (wait_limit_s on %globaltimer): a CTA that gives up
// raises the error word, every CTA stops at its next wait, the copies already
// issued into its ring are waited for (bounded too), and the host turns the
// word into AFP_ERR_TIMEOUT.  A test option makes the first grid barrier of a
// V-cycle wait for one arrival more than the grid has, so that every wait runs
// out.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "amg_internal.cuh"
#include "df32.cuh"

namespace afp {
namespace {

constexpr int kConsumerWarps = 16;
constexpr int kConsumers = kConsumerWarps * 32;
constexpr int kThreads = kConsumers + 32;  // + one producer warp
constexpr int kSlots = 8;
constexpr int kSlotBytes = 24 * 1024;
constexpr int kHdr = 32;                          // the entry's descriptor, written by the producer
constexpr int kBlobMax = kSlotBytes - kHdr;       // one tile's blob
constexpr int kMaxRows = 256;                     // rows per tile
constexpr int kWave = 3;                          // entries processed together (the other slots keep streaming)
constexpr int kTailSeg = (kBlobMax / 8) / 4 * 4;  // floats of hi (and of lo) per tail entry
constexpr int kRingBytes = kSlots * kSlotBytes;
constexpr int kPhaseBits = 12;                    // progress flags: epoch << 12 | phase
constexpr int kNbLevels = 16;                     // levels whose neighbour lists sit in shared memory
constexpr int kTailRows = 128;                    // dense tail rows per CTA (row partials in shared memory)

enum Op : int { OP_START = 0, OP_GS, OP_JAC, OP_RES, OP_RESTRICT, OP_TAIL, OP_TAIL_DIAG, OP_PROLONG, OP_FINISH };

// ------------------------------------------------------------ PTX helpers
__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* b, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* b, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.release.cta.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* b) {
  asm volatile("mbarrier.arrive.release.cta.shared::cta.b64 _, [%0];" ::"r"(smem_u32(b)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* b, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.acquire.cta.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(b)), "r"(parity)
      : "memory");
  return ok != 0;
}
// global -> shared bulk copy completing on mbarrier b (bytes a multiple of 16,
// both addresses 16-byte aligned)
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, uint64_t* b) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(b))
               : "memory");
}
__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release(unsigned* p, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned long long now_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// the consumer warps only (named barrier 1; the producer warp never joins it)
__device__ __forceinline__ void consumers_sync() { asm volatile("bar.sync 1, %0;" ::"n"(kConsumers) : "memory"); }

struct Shared {
  uint64_t full[kSlots];
  uint64_t empty[kSlots];
  float red[2 * kConsumerWarps];
  int abort;     // set by any thread (consumer or producer) that gives up
  int go;        // the consumers' common decision after a wait between phases
  int start_ok;  // no earlier V-cycle left the error word set
  int issued;
  unsigned base;
  unsigned epoch;
  int nnb[kNbLevels];       // this CTA's neighbour CTAs per level (count, list)
  int nbr[kNbLevels][32];
  float2 tailp[kTailRows][kConsumerWarps];  // per tail row, each warp's double-float partial
};

// Raises the error word (with `where`, the phase that gave up) and the
// CTA's abort flag.
__device__ __forceinline__ void give_up(const StreamArgs& a, Shared& s, int where) {
  if (atomicExch(&a.bar[2], 1u) == 0u) atomicExch(&a.bar[3], (unsigned)where);
  *(volatile int*)&s.abort = 1;
}

// Bounded wait for phase `parity` of mbarrier b; false after the limit or
// when the CTA is aborting (if `abortable`).
__device__ bool wait_slot(uint64_t* b, unsigned parity, const StreamArgs& a, Shared& s, bool abortable, int where) {
  unsigned long long t0 = 0;
  unsigned spins = 0;
  while (!mbar_try_wait(b, parity)) {
    if ((++spins & 63u) == 0) {
      if (abortable && *(volatile int*)&s.abort) return false;
      const unsigned long long t = now_ns();
      if (t0 == 0) {
        t0 = t;
      } else if (t - t0 > (unsigned long long)a.limit_ns) {
        give_up(a, s, where);
        return false;
      }
    }
  }
  return true;
}

// Grid barrier of the consumers: arrivals count up monotonically from the
// base this launch read at its start, so the k-th barrier waits for
// base + k * grid arrivals (wrap-safe).  The CTA also publishes that it
// finished phase `done`.  Returns the same decision to every consumer thread
// (false once the kernel must stop): only thread 0 writes s.go, between the
// two consumer barriers.
__device__ bool grid_sync(const StreamArgs& a, Shared& s, unsigned target, unsigned done, int where) {
  consumers_sync();
  if (threadIdx.x == 0) st_release(&a.prog[32 * blockIdx.x], done);
  if (threadIdx.x == 0 && *(volatile int*)&s.abort == 0) {
    // the release covers the CTA's writes (ordered before by the consumer
    // barrier); the acquire loads below make the other CTAs' writes visible
    asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(&a.bar[0]) : "memory");
    const unsigned long long t0 = now_ns();
    unsigned spins = 0;
    while ((int)(ld_acquire(&a.bar[0]) - target) < 0) {
      if ((++spins & 31u) == 0) {
        if (ld_acquire(&a.bar[2]) != 0u) {
          *(volatile int*)&s.abort = 1;
          break;
        }
        if (now_ns() - t0 > (unsigned long long)a.limit_ns) {
          give_up(a, s, where);
          break;
        }
      }
    }
  }
  if (threadIdx.x == 0) s.go = *(volatile int*)&s.abort == 0;
  consumers_sync();
  return s.go != 0;
}

// Wait between two colour classes of one level: this CTA publishes that it
// finished phase `done`, then waits only until each CTA whose rows are
// coupled to its rows on this level has finished it too (warp 0, one
// neighbour per lane).  The matrix pattern is symmetric and every x entry
// keeps one owner, so the CTAs this one reads from are exactly the ones that
// read its rows; neighbours thus stay within one phase of each other, which
// covers both orders of hazard (their new values read here, and old values
// of this CTA's rows read there before being overwritten).  Returns the same
// decision to every consumer thread.
__device__ bool nb_sync(const StreamArgs& a, Shared& s, int level, unsigned done, int where) {
  consumers_sync();
  if (threadIdx.x == 0) st_release(&a.prog[32 * blockIdx.x], done);
  if (threadIdx.x < 32) {
    const bool run = __shfl_sync(0xffffffffu, *(volatile int*)&s.abort == 0 ? 1 : 0, 0) != 0;
    if (run && (int)threadIdx.x < s.nnb[level]) {
      const unsigned* f = &a.prog[32 * s.nbr[level][threadIdx.x]];
      const unsigned long long t0 = now_ns();
      unsigned spins = 0;
      while ((int)(ld_acquire(f) - done) < 0) {
        if ((++spins & 31u) == 0) {
          if (*(volatile int*)&s.abort || ld_acquire(&a.bar[2]) != 0u) {
            *(volatile int*)&s.abort = 1;
            break;
          }
          if (now_ns() - t0 > (unsigned long long)a.limit_ns) {
            give_up(a, s, where);
            break;
          }
        }
      }
    }
    __syncwarp();
  }
  if (threadIdx.x == 0) s.go = *(volatile int*)&s.abort == 0;
  consumers_sync();
  return s.go != 0;
}

// x values gathered by the l1-Jacobi class: its own rows from the snapshot
__device__ __forceinline__ float jac_x(const StreamLevel& L, int c) {
  const float* base = c >= L.ov0 ? L.snap - L.ov0 : L.x;  // one load either way
  return base[c];
}

__device__ __forceinline__ const StreamTile& hdr(const char* slot) { return *(const StreamTile*)slot; }

// One row: lanes [0, vec) of its group take groups gb + lane, gb + lane + vec,
// ... four at a time (sixteen gathers in flight per lane); the row's sum is
// reduced over the group with shuffles and lane 0 applies the operation.
template <int OP>
__device__ __forceinline__ void row_apply(int row, const char* __restrict__ grp, int gb, int ge, int lane, int vec,
                                          unsigned gmask, const StreamLevel& L, const StreamLevel& Ln) {
  const float* xin = OP == OP_RESTRICT ? L.tmp : OP == OP_PROLONG ? Ln.x : L.x;
  // per-row operands first, so that their loads overlap the gathers
  float pr = 0.f, pa = 0.f, pb = 0.f;
  if (lane == 0) {
    if (OP == OP_GS || OP == OP_RES) pr = L.r[row];
    if (OP == OP_JAC) {
      pr = L.r[row];
      pa = L.snap[row - L.ov0];
      pb = L.l1d[row - L.ov0];
    }
    if (OP == OP_PROLONG) pa = L.x[row];
  }
  float s = 0.f, diag = 1.f;
  for (int g = gb + lane; g < ge; g += 4 * vec) {
    int4 c[4];
    float4 v[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int gg = g + u * vec;
      if (u == 0 || gg < ge) {
        const char* p = grp + (size_t)gg * 32;
        c[u] = *(const int4*)p;
        v[u] = *(const float4*)(p + 16);
      } else {
        c[u] = c[0];
        v[u] = make_float4(0.f, 0.f, 0.f, 0.f);
      }
    }
    if (OP == OP_GS && g == gb) {  // the diagonal is the row's first entry
      diag = v[0].x;
      v[0].x = 0.f;
    }
    float xv[16];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      if (OP == OP_JAC) {
        xv[4 * u] = jac_x(L, c[u].x);
        xv[4 * u + 1] = jac_x(L, c[u].y);
        xv[4 * u + 2] = jac_x(L, c[u].z);
        xv[4 * u + 3] = jac_x(L, c[u].w);
      } else {
        xv[4 * u] = xin[c[u].x];
        xv[4 * u + 1] = xin[c[u].y];
        xv[4 * u + 2] = xin[c[u].z];
        xv[4 * u + 3] = xin[c[u].w];
      }
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      s = fmaf(v[u].x, xv[4 * u], s);
      s = fmaf(v[u].y, xv[4 * u + 1], s);
      s = fmaf(v[u].z, xv[4 * u + 2], s);
      s = fmaf(v[u].w, xv[4 * u + 3], s);
    }
  }
  for (int o = vec >> 1; o > 0; o >>= 1) s += __shfl_xor_sync(gmask, s, o, vec);
  if (lane == 0) {
    if (OP == OP_GS) {
      L.x[row] = (pr - s) / diag;
    } else if (OP == OP_JAC) {
      L.x[row] = pa + (pr - s) / pb;
    } else if (OP == OP_RES) {
      L.tmp[row] = pr - s;
    } else if (OP == OP_RESTRICT) {
      Ln.r[row] = s;
      Ln.x[row] = 0.f;
    } else {  // OP_PROLONG
      L.x[row] = pa + s;
    }
  }
}

// The rows of a wave of nw entries (slots sl[0..nw)), flattened: row group
// (vec lanes) f takes flat rows f, f + 512/vec, ...
template <int OP>
__device__ void wave_rows(const char* const* sl, int nw, int vec, const StreamLevel& L, const StreamLevel& Ln) {
  int pre[kWave + 1];
  pre[0] = 0;
#pragma unroll
  for (int j = 0; j < kWave; ++j) pre[j + 1] = pre[j] + (j < nw ? hdr(sl[j]).n : 0);
  const int R = pre[nw];
  const int ct = threadIdx.x;
  const int lane = ct & (vec - 1);
  const int nslot = kConsumers / vec;
  const unsigned gmask = vec >= 32 ? 0xffffffffu : (((1u << vec) - 1u) << ((ct & 31) & ~(vec - 1)));
  for (int f = ct / vec; f < R; f += nslot) {
    int j = 0;
#pragma unroll
    for (int q = 1; q < kWave; ++q) j += (q < nw && f >= pre[q]) ? 1 : 0;
    const char* slot = sl[j];
    const StreamTile& T = hdr(slot);
    const int q = f - pre[j];
    const unsigned short* off = (const unsigned short*)(slot + kHdr);
    const char* grp = slot + kHdr + (T.meta >> 16);
    row_apply<OP>(T.row0 + q, grp, off[q], off[q + 1], lane, vec, gmask, L, Ln);
  }
}

// One segment [T.n, T.n + T.bytes/4) of tail row T.row0: hi then lo in the
// slot; (sh, sl) accumulate over the row's segments.
__device__ void tail_tile(const StreamLevel& Lt, const char* __restrict__ slot, float& sh, float& sl) {
  const StreamTile& T = hdr(slot);
  const int n4 = T.bytes / 16;
  const float* rt = Lt.r + T.n;
  const char* hi = slot + kHdr;
  for (int q = threadIdx.x; q < n4; q += kConsumers) {
    const float4 h = *(const float4*)(hi + 16 * q);
    const float4 l = *(const float4*)(hi + T.bytes + 16 * q);
    const float4 v = *(const float4*)(rt + 4 * q);
    df_add_prod(sh, sl, h.x, l.x, v.x);
    df_add_prod(sh, sl, h.y, l.y, v.y);
    df_add_prod(sh, sl, h.z, l.z, v.z);
    df_add_prod(sh, sl, h.w, l.w, v.w);
  }
}

// After a tail row's last segment: each warp reduces its lanes' (sh, sl) and
// parks the pair in shared memory (no CTA-wide wait per row).
__device__ __forceinline__ void tail_row_end(int rl, float& sh, float& sl, Shared& s) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    const float oh = __shfl_xor_sync(0xffffffffu, sh, off);
    const float ol = __shfl_xor_sync(0xffffffffu, sl, off);
    df_add(sh, sl, oh, ol);
  }
  if ((threadIdx.x & 31) == 0) s.tailp[rl][threadIdx.x >> 5] = make_float2(sh, sl);
  sh = sl = 0.f;
}

// After the CTA's last tail row: every row's warp pairs summed in warp order.
__device__ void tail_rows_finish(const StreamLevel& Lt, int row0, int nrows, Shared& s) {
  consumers_sync();
  for (int rl = threadIdx.x; rl < nrows; rl += kConsumers) {
    float h = s.tailp[rl][0].x, l = s.tailp[rl][0].y;
    for (int w = 1; w < kConsumerWarps; ++w) df_add(h, l, s.tailp[rl][w].x, s.tailp[rl][w].y);
    Lt.x[row0 + rl] = __fadd_rn(h, l);
  }
}

__global__ void __launch_bounds__(kThreads, 1) k_vcycle_stream(StreamArgs a) {
  extern __shared__ __align__(128) char dyn[];
  __shared__ Shared s;
  // slots start 128-byte aligned whatever the dynamic region's base alignment
  char* ring = (char*)(((uintptr_t)dyn + 127) & ~(uintptr_t)127);
  const int cta = blockIdx.x;
  const StreamPhase* ph = a.ph + (size_t)cta * a.nphase;
  const StreamTile* tiles = a.tiles + a.tile_off[cta];
  const int ntiles = a.tile_off[cta + 1] - a.tile_off[cta];
  if (threadIdx.x == 0) {
    for (int i = 0; i < kSlots; ++i) {
      mbar_init(&s.full[i], 1);
      mbar_init(&s.empty[i], kConsumerWarps);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    s.start_ok = ld_acquire(&a.bar[2]) == 0u;  // an earlier V-cycle gave up: do nothing
    s.abort = !s.start_ok;
    s.go = s.start_ok;
    s.issued = 0;
    s.base = ld_acquire(&a.bar[1]);
    s.epoch = ld_acquire(&a.bar[4]);
  }
  if (threadIdx.x < 32)  // neighbour lists (at most 32 per level) into shared memory
    for (int l = 0; l < kNbLevels && l <= a.t; ++l) {
      const int o = l * (gridDim.x + 1) + cta;
      const int b = a.nb_off[o], e = a.nb_off[o + 1];
      if (threadIdx.x == 0) s.nnb[l] = min(e - b, 32);
      if ((int)threadIdx.x < e - b) s.nbr[l][threadIdx.x] = a.nb[b + threadIdx.x];
    }
  __syncthreads();

  if (threadIdx.x >= kConsumers) {
    // ---------------------------------------------------------- producer
    if (threadIdx.x == kConsumers) {
      for (int i = 0; i < ntiles; ++i) {
        const int k = i % kSlots;
        if (i >= kSlots && !wait_slot(&s.empty[k], ((i / kSlots) - 1) & 1, a, s, true, -1)) break;
        if (*(volatile int*)&s.abort) break;
        const StreamTile T = tiles[i];
        char* slot = ring + (size_t)k * kSlotBytes;
        *(StreamTile*)slot = T;  // the descriptor travels with the data
        mbar_arrive_expect_tx(&s.full[k], T.src2 ? 2u * T.bytes : (unsigned)T.bytes);
        bulk_g2s(slot + kHdr, T.src, T.bytes, &s.full[k]);
        if (T.src2) bulk_g2s(slot + kHdr + T.bytes, T.src2, T.bytes, &s.full[k]);
        *(volatile int*)&s.issued = i + 1;
      }
    }
  } else if (s.start_ok) {
    // ---------------------------------------------------------- consumers
    const int G = gridDim.x;
    unsigned nbar = 0;
    float sh = 0.f, sl = 0.f;
    // diagnostic timestamps: phase start, work done, wait done (CTAs 0, G/2, G-1)
    const int tslot = cta == 0 ? 0 : cta == G / 2 ? 1 : cta == G - 1 ? 2 : -1;
    unsigned long long* tr = (a.trace && tslot >= 0 && threadIdx.x == 0) ? a.trace + (size_t)tslot * a.nphase * 3
                                                                          : nullptr;
    for (int p = 0; p < a.nphase; ++p) {
      if (tr) tr[3 * p] = now_ns();
      const StreamPhase P = ph[p];
      // level descriptors by value: register copies that stores through their
      // pointers cannot alias
      const StreamLevel L = a.L[P.level];
      switch (P.op) {
        case OP_START: {
          for (int64_t i = (int64_t)cta * kConsumers + threadIdx.x; i < L.n; i += (int64_t)G * kConsumers) {
            L.x[i] = 0.f;
            L.r[i] = (float)a.r64[i];
          }
          break;
        }
        case OP_FINISH: {
          for (int64_t i = (int64_t)cta * kConsumers + threadIdx.x; i < L.n; i += (int64_t)G * kConsumers)
            a.z64[i] = (double)L.x[i];
          break;
        }
        case OP_TAIL_DIAG: {
          for (int64_t i = (int64_t)cta * kConsumers + threadIdx.x; i < L.n; i += (int64_t)G * kConsumers)
            L.x[i] = L.r[i] / L.va[L.rp[i]];
          break;
        }
        default: {
          const StreamLevel Ln = a.L[P.level + 1 <= a.t ? P.level + 1 : P.level];
          int i = P.tile0;
          const int end = P.tile0 + P.ntiles;
          const int tail_row0 = (P.op == OP_TAIL && P.ntiles > 0) ? tiles[P.tile0].row0 : 0;
          int tail_rows = 0;
          while (i < end) {
            // a thread whose wait fails (abort) skips the work but keeps every
            // consumer barrier of the schedule; the next wait stops all
            bool ok = wait_slot(&s.full[i % kSlots], (i / kSlots) & 1, a, s, true, p);
            const char* slot0 = ring + (size_t)(i % kSlots) * kSlotBytes;
            const int meta = ok ? hdr(slot0).meta : tiles[i].meta;  // the same value, uniform either way
            const int nw = max(1, min(meta & 15, end - i));
            const int vec = max(1, (meta >> 4) & 63);
            const char* sls[kWave];
#pragma unroll
            for (int j = 0; j < kWave; ++j) {
              sls[j] = ring + (size_t)((i + j) % kSlots) * kSlotBytes;
              if (j > 0 && j < nw && ok)
                ok = wait_slot(&s.full[(i + j) % kSlots], ((i + j) / kSlots) & 1, a, s, true, p);
            }
            const bool tail = P.op == OP_TAIL;
            // a tail wave is segments of one row; the row ends with the wave's last
            const char* slast = ring + (size_t)((i + nw - 1) % kSlots) * kSlotBytes;
            const int tmeta = tail ? (ok ? hdr(slast).meta : tiles[i + nw - 1].meta) : 0;
            const int trow = tail ? (ok ? hdr(slast).row0 : tiles[i + nw - 1].row0) : 0;
            if (ok) {
              switch (P.op) {
                case OP_GS: wave_rows<OP_GS>(sls, nw, vec, L, Ln); break;
                case OP_JAC: wave_rows<OP_JAC>(sls, nw, vec, L, Ln); break;
                case OP_RES: wave_rows<OP_RES>(sls, nw, vec, L, Ln); break;
                case OP_RESTRICT: wave_rows<OP_RESTRICT>(sls, nw, vec, L, Ln); break;
                case OP_PROLONG: wave_rows<OP_PROLONG>(sls, nw, vec, L, Ln); break;
                default:
                  for (int j = 0; j < nw; ++j) tail_tile(L, sls[j], sh, sl);
                  break;
              }
            }
            __syncwarp();
            if ((threadIdx.x & 31) == 0)
              for (int j = 0; j < nw; ++j) mbar_arrive(&s.empty[(i + j) % kSlots]);
            if (tail && ((tmeta >> 10) & 1)) {
              tail_row_end(trow - tail_row0, sh, sl, s);
              tail_rows = trow - tail_row0 + 1;
            }
            i += nw;
          }
          if (P.op == OP_TAIL) tail_rows_finish(L, tail_row0, tail_rows, s);
          break;
        }
      }
      if (tr) tr[3 * p + 1] = now_ns();
      if (P.snap1 > P.snap0) {  // own overflow rows -> snapshot, for the Jacobi phase next
        consumers_sync();
        for (int i = P.snap0 + threadIdx.x; i < P.snap1; i += kConsumers) L.snap[i - L.ov0] = L.x[i];
      }
      if (p + 1 < a.nphase) {
        const unsigned done = (s.epoch << kPhaseBits) + (unsigned)p;
        if (P.sync == 1) {
          if (!nb_sync(a, s, P.level, done, p)) break;
        } else {
          ++nbar;
          const unsigned target = s.base + nbar * (unsigned)G + ((a.stall && nbar == 1) ? 1u : 0u);
          if (!grid_sync(a, s, target, done, p)) break;
        }
      }
      if (tr) tr[3 * p + 2] = now_ns();
    }
    if (cta == 0 && threadIdx.x == 0 && s.go) {
      a.bar[1] = s.base + nbar * (unsigned)G;
      a.bar[4] = s.epoch + 1;
    }
  }
  __syncthreads();
  // copies still in flight (only after an abort) must land before the CTA exits
  if (threadIdx.x == 0) {
    const int issued = *(volatile int*)&s.issued;
    for (int i = max(0, issued - kSlots); i < issued; ++i)
      wait_slot(&s.full[i % kSlots], (i / kSlots) & 1, a, s, false, -2);
  }
}

// ---------------------------------------------------------- plan building
__global__ void k_group_len(int64_t m, const int* __restrict__ rp, int* __restrict__ len) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < m) len[i] = (rp[i + 1] - rp[i] + 3) / 4;
}

__host__ __device__ inline int offset_bytes(int nrows) { return (2 * (nrows + 1) + 15) / 16 * 16; }

// Tile blobs of one operator: block b packs tile b (rows [row0[b], +nrows[b]))
// at blob offset off[b]: the rows' group offsets (uint16), then their groups.
__global__ void k_pack_tiles(const int* __restrict__ rp, const int* __restrict__ ci, const float* __restrict__ va,
                             const int* __restrict__ gp, const int* __restrict__ row0, const int* __restrict__ nrows,
                             const int64_t* __restrict__ off, char* __restrict__ blob) {
  const int b = blockIdx.x;
  const int r0 = row0[b], nr = nrows[b];
  char* base = blob + off[b];
  unsigned short* ro = (unsigned short*)base;
  const int g0 = gp[r0];
  const int obytes = offset_bytes(nr);
  for (int q = threadIdx.x; q <= nr; q += blockDim.x) ro[q] = (unsigned short)(gp[r0 + q] - g0);
  for (int q = nr + 1 + threadIdx.x; q < obytes / 2; q += blockDim.x) ro[q] = 0;
  int4* grp = (int4*)(base + obytes);
  for (int q = threadIdx.x; q < nr; q += blockDim.x) {
    const int i = r0 + q;
    const int e0 = rp[i], e1 = rp[i + 1];
    const int last = e1 > e0 ? ci[e1 - 1] : 0;
    for (int g = gp[i]; g < gp[i + 1]; ++g) {
      int c[4];
      float v[4];
      for (int j = 0; j < 4; ++j) {
        const int k = e0 + 4 * (g - gp[i]) + j;
        c[j] = k < e1 ? ci[k] : last;
        v[j] = k < e1 ? va[k] : 0.f;
      }
      grp[2 * (g - g0)] = make_int4(c[0], c[1], c[2], c[3]);
      grp[2 * (g - g0) + 1] =
          make_int4(__float_as_int(v[0]), __float_as_int(v[1]), __float_as_int(v[2]), __float_as_int(v[3]));
    }
  }
}

// Tiles of an m-row FP32 CSR operator (device arrays) whose rows are
// partitioned by `runs`: runs[c][k] .. runs[c][k+1] are the rows of class c
// handled by CTA k (G CTAs).  Returns false if a row does not fit a slot.
bool tile_operator(const afp_context* ctx, int64_t m, const int* rp, const int* ci, const float* va,
                   const std::vector<std::vector<int64_t>>& runs, int G, TiledOp& op) {
  DevBuf<int> len(ctx, std::max<int64_t>(m, 1)), gp(ctx, m + 1);
  k_group_len<<<grid_for(m, 256), 256, 0, ctx->stream>>>(m, rp, len.get());
  check_launch(ctx, "group lengths");
  exclusive_scan(ctx, len.get(), gp.get(), m);
  std::vector<int> hgp(m + 1);
  copy(ctx, hgp.data(), gp.get(), sizeof(int) * (m + 1));
  sync(ctx);
  op.m = m;
  op.first.assign(runs.size() * G + 1, 0);
  int64_t bytes = 0;
  for (size_t c = 0; c < runs.size(); ++c)
    for (int k = 0; k < G; ++k) {
      op.first[c * G + k] = (int)op.row0.size();
      int64_t a = runs[c][k];
      const int64_t b = runs[c][k + 1];
      while (a < b) {
        int64_t e = a;
        while (e < b && e - a < kMaxRows &&
               offset_bytes((int)(e + 1 - a)) + 32 * (int64_t)(hgp[e + 1] - hgp[a]) <= kBlobMax)
          ++e;
        if (e == a) return false;  // one row longer than a slot
        op.row0.push_back((int)a);
        op.nrows.push_back((int)(e - a));
        op.ngroups.push_back(hgp[e] - hgp[a]);
        op.off.push_back(bytes);
        bytes += offset_bytes((int)(e - a)) + 32 * (int64_t)(hgp[e] - hgp[a]);
        a = e;
      }
    }
  op.first[runs.size() * G] = (int)op.row0.size();
  const int nt = (int)op.row0.size();
  op.blob.alloc(ctx, std::max<int64_t>(bytes, 16));
  if (nt > 0) {
    DevBuf<int> d0(ctx, nt), dn(ctx, nt);
    DevBuf<int64_t> doff(ctx, nt);
    d0.upload(op.row0.data(), nt);
    dn.upload(op.nrows.data(), nt);
    doff.upload(op.off.data(), nt);
    k_pack_tiles<<<nt, 128, 0, ctx->stream>>>(rp, ci, va, gp.get(), d0.get(), dn.get(), doff.get(), op.blob.get());
    check_launch(ctx, "pack tiles");
    sync(ctx);
  }
  return true;
}

// Lanes per row for a wave of R rows with `groups` groups: the fewest rounds
// of dependent gathers, a round being one pass of the 512 consumer threads
// over their rows with four groups per lane per step.
int wave_lanes(int64_t R, int64_t groups) {
  int best = 1;
  double best_cost = 1e30;
  const double per_row = R > 0 ? (double)groups / (double)R : 1.0;
  for (int v = 1; v <= 32; v *= 2) {
    const double passes = std::ceil((double)R * v / kConsumers);
    const double steps = std::ceil(std::ceil(per_row / v) / 4.0);
    const double cost = passes * steps + 0.02 * v;  // ties: fewer lanes (fewer shuffles)
    if (cost < best_cost) {
      best_cost = cost;
      best = v;
    }
  }
  return best;
}

}  // namespace

void fused_build(afp_amg* h) {
  afp_context* ctx = h->ctx;
  h->fused.reset();
  const int t = h->t;
  if (t == 0 || h->opts.precision != AFP_PRECISION_MIXED || h->opts.interp_bf16) return;
  if (h->lv[t].n >= (int64_t)INT32_MAX / 2) return;
  int per_sm = 0;
  AFP_CUDA(cudaFuncSetAttribute(k_vcycle_stream, cudaFuncAttributeMaxDynamicSharedMemorySize, kRingBytes + 128));
  AFP_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_vcycle_stream, kThreads, kRingBytes + 128));
  if (per_sm < 1) return;
  const int G = ctx->sm_count;
  if (h->tail_dense && (h->lv[t].n + G - 1) / G > kTailRows) return;
  auto F = std::make_unique<FusedPlan>();
  F->grid = G;
  // Row runs: each colour class of a smoothed level is split into G runs of
  // about equal stored entries (rows of a class are uncoupled, so any split
  // works); the tail level into G runs of rows.  A CTA keeps the same runs in
  // every phase (its overflow-class rows in particular, which it snapshots).
  std::vector<std::vector<std::vector<int64_t>>> runs(t + 1);
  std::vector<std::vector<int>> hrp(t);
  for (int l = 0; l <= t; ++l) {
    const Level& L = h->lv[l];
    const std::vector<int64_t> cls = l < t ? L.cls : std::vector<int64_t>{0, L.n};
    if (l < t) {
      hrp[l].resize(L.n + 1);
      copy(ctx, hrp[l].data(), L.rp.get(), sizeof(int) * (L.n + 1));
      sync(ctx);
    }
    for (size_t c = 0; c + 1 < cls.size(); ++c) {
      std::vector<int64_t> st(G + 1, cls[c + 1]);
      st[0] = cls[c];
      auto weight = [&](int64_t i) { return l < t ? (double)hrp[l][i] : (double)i; };
      const double w0 = weight(cls[c]);
      const double total = weight(cls[c + 1]) - w0;
      int k = 1;
      for (int64_t i = cls[c]; i < cls[c + 1] && k < G; ++i) {
        const double w = weight(i + 1) - w0;
        while (k < G && w >= total * k / G) st[k++] = i + 1;
      }
      runs[l].push_back(st);
    }
  }
  // tiled operators: A_l, P_l (rows of level l+1), P^T_l (rows of level l)
  F->ops.resize(3 * t);
  for (int l = 0; l < t; ++l) {
    const Level& L = h->lv[l];
    if (!tile_operator(ctx, L.n, L.rp.get(), L.ci.get(), L.va32.get(), runs[l], G, F->ops[3 * l]) ||
        !tile_operator(ctx, h->lv[l + 1].n, L.prp.get(), L.pci.get(), L.pva32.get(), runs[l + 1], G,
                       F->ops[3 * l + 1]) ||
        !tile_operator(ctx, L.n, L.trp.get(), L.tci.get(), L.tva32.get(), runs[l], G, F->ops[3 * l + 2]))
      return;  // a row longer than a slot: keep the launch chain
  }
  // the phase program
  struct GPhase {
    int op, level, cls;
    bool snap;
  };
  std::vector<GPhase> prog;
  auto smooth = [&](int l, bool backward) {
    const Level& L = h->lv[l];
    const int K = (int)L.cls.size() - 1;
    for (int sw = 0; sw < h->opts.smooth_step; ++sw)
      for (int q = 0; q < K; ++q) {
        const int c = backward ? K - 1 - q : q;
        if (L.cls[c + 1] <= L.cls[c]) continue;
        prog.push_back({(L.overflow && c == K - 1) ? OP_JAC : OP_GS, l, c, false});
      }
  };
  prog.push_back({OP_START, 0, 0, false});
  for (int l = 0; l < t; ++l) {
    smooth(l, false);
    prog.push_back({OP_RES, l, -1, false});
    prog.push_back({OP_RESTRICT, l, -1, false});
  }
  prog.push_back({h->tail_dense ? OP_TAIL : OP_TAIL_DIAG, t, 0, false});
  for (int l = t - 1; l >= 0; --l) {
    prog.push_back({OP_PROLONG, l, -1, false});
    smooth(l, h->opts.symmetric != 0);
  }
  prog.push_back({OP_FINISH, 0, 0, false});
  for (size_t p = 1; p < prog.size(); ++p)
    if (prog[p].op == OP_JAC) {
      GPhase& q = prog[p - 1];
      if (!((q.op == OP_GS || q.op == OP_PROLONG) && q.level == prog[p].level)) return;  // no place for the snapshot
      q.snap = true;
    }
  const int nphase = (int)prog.size();
  if (nphase >= (1 << kPhaseBits)) return;
  // neighbour CTAs per smoothed level: the owners of the columns of a CTA's
  // rows and the CTAs whose rows have columns it owns.  Levels where some CTA
  // has more than 32 neighbours keep grid barriers between colour classes.
  std::vector<int> nb, nb_off((size_t)(t + 1) * (G + 1), 0);
  std::vector<char> nb_ok(t + 1, 0);
  for (int l = 0; l <= t; ++l) {
    std::vector<std::vector<int>> sets(G);
    if (l < t) {
      const Level& L = h->lv[l];
      std::vector<int> owner(L.n, 0), ci(L.nnz);
      for (size_t c = 0; c < runs[l].size(); ++c)
        for (int k = 0; k < G; ++k)
          for (int64_t i = runs[l][c][k]; i < runs[l][c][k + 1]; ++i) owner[i] = k;
      copy(ctx, ci.data(), L.ci.get(), sizeof(int) * L.nnz);
      sync(ctx);
      std::vector<char> mark((size_t)G * G, 0);
      for (int64_t i = 0; i < L.n; ++i)
        for (int q = hrp[l][i]; q < hrp[l][i + 1]; ++q) {
          const int a0 = owner[i], b0 = owner[ci[q]];
          if (a0 != b0) mark[(size_t)a0 * G + b0] = mark[(size_t)b0 * G + a0] = 1;
        }
      bool ok = true;
      for (int k = 0; k < G; ++k) {
        for (int j = 0; j < G; ++j)
          if (mark[(size_t)k * G + j]) sets[k].push_back(j);
        ok = ok && sets[k].size() <= 32;
      }
      nb_ok[l] = ok && l < kNbLevels;
    }
    for (int k = 0; k < G; ++k) {
      nb_off[(size_t)l * (G + 1) + k] = (int)nb.size();
      if (nb_ok[l]) nb.insert(nb.end(), sets[k].begin(), sets[k].end());
    }
    nb_off[(size_t)l * (G + 1) + G] = (int)nb.size();
  }
  auto smoothing = [](int op) { return op == OP_GS || op == OP_JAC; };
  std::vector<StreamPhase> phases((size_t)G * nphase);
  std::vector<StreamTile> stream;
  std::vector<int> tile_off(G + 1, 0);
  const int64_t ld = h->tail_ld;
  // appends op's tiles of classes [c0, c1) for CTA k, in waves
  auto add_tiles = [&](const TiledOp& op, int c0, int c1, int k, std::vector<StreamTile>& out) {
    std::vector<int> ids;
    for (int c = c0; c < c1; ++c)
      for (int q = op.first[c * G + k]; q < op.first[c * G + k + 1]; ++q) ids.push_back(q);
    for (size_t w = 0; w < ids.size(); w += kWave) {
      const int nw = (int)std::min<size_t>(kWave, ids.size() - w);
      int64_t R = 0, gsum = 0;
      for (int j = 0; j < nw; ++j) {
        R += op.nrows[ids[w + j]];
        gsum += op.ngroups[ids[w + j]];
      }
      const int vec = wave_lanes(R, gsum);
      for (int j = 0; j < nw; ++j) {
        const int q = ids[w + j];
        StreamTile T{};
        T.src = op.blob.get() + op.off[q];
        T.src2 = nullptr;
        T.bytes = offset_bytes(op.nrows[q]) + 32 * op.ngroups[q];
        T.row0 = op.row0[q];
        T.n = op.nrows[q];
        T.meta = (j == 0 ? nw : 0) | (vec << 4) | (offset_bytes(op.nrows[q]) << 16);
        out.push_back(T);
      }
    }
  };
  for (int k = 0; k < G; ++k) {
    tile_off[k] = (int)stream.size();
    std::vector<StreamTile> mine;
    for (int p = 0; p < nphase; ++p) {
      const GPhase& g = prog[p];
      StreamPhase& P = phases[(size_t)k * nphase + p];
      P.op = g.op;
      P.level = g.level;
      P.tile0 = (int)mine.size();
      P.snap0 = P.snap1 = 0;
      const int Kl = g.level < t ? (int)h->lv[g.level].cls.size() - 1 : 1;
      switch (g.op) {
        case OP_GS:
        case OP_JAC: add_tiles(F->ops[3 * g.level], g.cls, g.cls + 1, k, mine); break;
        case OP_RES: add_tiles(F->ops[3 * g.level], 0, Kl, k, mine); break;
        case OP_RESTRICT: {
          const int Kn = g.level + 1 < t ? (int)h->lv[g.level + 1].cls.size() - 1 : 1;
          add_tiles(F->ops[3 * g.level + 1], 0, Kn, k, mine);
          break;
        }
        case OP_PROLONG: add_tiles(F->ops[3 * g.level + 2], 0, Kl, k, mine); break;
        case OP_TAIL: {
          // one tail row's segments in waves of up to kWave
          const int nseg = (int)((ld + kTailSeg - 1) / kTailSeg);
          for (int64_t i = runs[t][0][k]; i < runs[t][0][k + 1]; ++i)
            for (int sg = 0; sg < nseg; ++sg) {
              const int64_t c0 = (int64_t)sg * kTailSeg;
              const int64_t cnt = std::min<int64_t>(kTailSeg, ld - c0);
              StreamTile T{};
              T.src = h->tail_hi.get() + i * ld + c0;
              T.src2 = h->tail_lo.get() + i * ld + c0;
              T.bytes = (int)(4 * cnt);
              T.row0 = (int)i;
              T.n = (int)c0;
              T.meta = (sg % kWave == 0 ? std::min(kWave, nseg - sg) : 0) | (1 << 4) | (sg == nseg - 1 ? (1 << 10) : 0);
              mine.push_back(T);
            }
          break;
        }
        default: break;
      }
      P.ntiles = (int)mine.size() - P.tile0;
      P.sync = (p + 1 < nphase && smoothing(g.op) && smoothing(prog[p + 1].op) && prog[p + 1].level == g.level &&
                nb_ok[g.level])
                   ? 1
                   : 0;
      if (g.snap) {
        const int K = (int)h->lv[g.level].cls.size() - 1;
        P.snap0 = (int)runs[g.level][K - 1][k];
        P.snap1 = (int)runs[g.level][K - 1][k + 1];
      }
    }
    stream.insert(stream.end(), mine.begin(), mine.end());
  }
  tile_off[G] = (int)stream.size();
  // device level descriptors
  std::vector<StreamLevel> lv(t + 1);
  F->snap.resize(t);
  for (int l = 0; l <= t; ++l) {
    const Level& L = h->lv[l];
    StreamLevel& d = lv[l];
    d.n = L.n;
    d.x = l == 0 ? h->z32.get() : L.x32.get();
    d.r = l == 0 ? h->r32.get() : L.r32.get();
    d.tmp = L.tmp32.get();
    d.rp = L.rp.get();
    d.va = L.va32.get();
    d.ov0 = (int)L.n;
    if (l < t && L.overflow) {
      const int K = (int)L.cls.size() - 1;
      d.ov0 = (int)L.cls[K - 1];
      F->snap[l].alloc(ctx, std::max<int64_t>(1, L.n - d.ov0));
      d.snap = F->snap[l].get();
      d.l1d = L.l1d32.get();
    }
  }
  F->levels.alloc(ctx, lv.size());
  F->levels.upload(lv.data(), lv.size());
  F->phases.alloc(ctx, phases.size());
  F->phases.upload(phases.data(), phases.size());
  F->tiles.alloc(ctx, std::max<size_t>(1, stream.size()));
  F->tiles.upload(stream.data(), stream.size());
  F->tile_off.alloc(ctx, G + 1);
  F->tile_off.upload(tile_off.data(), G + 1);
  F->nb.alloc(ctx, std::max<size_t>(1, nb.size()));
  F->nb.upload(nb.data(), nb.size());
  F->nb_off.alloc(ctx, nb_off.size());
  F->nb_off.upload(nb_off.data(), nb_off.size());
  F->prog.alloc(ctx, (size_t)32 * G);
  F->prog.zero();
  F->bar.alloc(ctx, 8);
  static const unsigned bar0[8] = {0, 0, 0, 0, 1, 0, 0, 0};  // epoch 1: the zeroed progress flags are older
  F->bar.upload(bar0, 8);
  if (std::getenv("AFP_VCYCLE_TRACE")) {
    F->trace.alloc(ctx, (size_t)9 * nphase);
    F->trace.zero();
  }
  F->nphase = nphase;
  F->ntiles = (int64_t)stream.size();
  sync(ctx);
  h->fused = std::move(F);
}

void fused_vcycle(afp_amg* h, const double* r64, double* z64) {
  afp_context* ctx = h->ctx;
  FusedPlan& F = *h->fused;
  StreamArgs a{};
  a.L = F.levels.get();
  a.ph = F.phases.get();
  a.tiles = F.tiles.get();
  a.tile_off = F.tile_off.get();
  a.nphase = F.nphase;
  a.t = h->t;
  a.bar = F.bar.get();
  a.prog = F.prog.get();
  a.nb = F.nb.get();
  a.nb_off = F.nb_off.get();
  a.limit_ns = (long long)(h->opts.wait_limit_s * 1e9);
  a.stall = h->opts.inject_barrier_stall;
  a.r64 = r64;
  a.z64 = z64;
  a.trace = F.trace.size() ? F.trace.get() : nullptr;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)F.grid);
  cfg.blockDim = dim3(kThreads);
  cfg.dynamicSmemBytes = kRingBytes + 128;
  cfg.stream = ctx->stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  AFP_CUDA(cudaLaunchKernelEx(&cfg, k_vcycle_stream, a));
  check_launch(ctx, "streamed V-cycle");
}

void fused_print_trace(afp_amg* h) {
  if (!h->fused || h->fused->trace.size() == 0) return;
  FusedPlan& F = *h->fused;
  const int n = F.nphase;
  std::vector<unsigned long long> t((size_t)9 * n);
  std::vector<StreamPhase> ph(n);
  copy(h->ctx, t.data(), F.trace.get(), sizeof(unsigned long long) * t.size());
  copy(h->ctx, ph.data(), F.phases.get(), sizeof(StreamPhase) * n);  // CTA 0's records
  sync(h->ctx);
  static const char* names[] = {"start", "gs", "jacobi", "residual", "restrict", "tail", "tail-diag", "prolong",
                                "finish"};
  for (int c = 0; c < 3; ++c) {
    const unsigned long long* r = t.data() + (size_t)c * n * 3;
    double work[9] = {0}, wait[9] = {0};
    int cnt[9] = {0};
    for (int p = 0; p < n; ++p) {
      const int op = ph[p].op;
      work[op] += (r[3 * p + 1] - r[3 * p]) * 1e-3;
      if (p + 1 < n) wait[op] += (r[3 * p + 2] - r[3 * p + 1]) * 1e-3;
      cnt[op]++;
    }
    for (int o = 0; o < 9; ++o)
      if (cnt[o])
        std::fprintf(stderr, "[afp vcycle] cta-slot %d %-9s x%3d work %8.1f us  wait %8.1f us\n", c, names[o], cnt[o],
                     work[o], wait[o]);
    std::fprintf(stderr, "[afp vcycle] cta-slot %d span %.1f us\n", c, (r[3 * (n - 1) + 1] - r[0]) * 1e-3);
  }
}

bool fused_timed_out(afp_amg* h) {
  if (!h->fused) return false;
  unsigned w[8] = {0};
  copy(h->ctx, w, h->fused->bar.get(), sizeof(w));
  sync(h->ctx);
  if (w[2]) {  // restart every count: arrivals, epoch, progress flags
    static const unsigned bar0[8] = {0, 0, 0, 0, 1, 0, 0, 0};
    h->fused->bar.upload(bar0, 8);
    h->fused->prog.zero();
    sync(h->ctx);
  }
  return w[2] != 0;
}

}  // namespace afp
