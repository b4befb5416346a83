// The FP32 V-cycle as one persistent cooperative kernel.
//
// Launched as a chain, the V-cycle is ~150-200 dependent kernels (one per
// colour class and sweep), each moving ~1-10 MB: at HBM speed a class takes
// about a microsecond, so launch gaps and the dependent memory round trips
// at the start of every kernel dominate.  Here one grid, co-resident by a
// cooperative launch, walks a phase program built at setup
//
//   GS class | l1-Jacobi class + copy-back | residual (+ zero of the next
//   level's x) | restriction | dense tail | prolongation
//
// with a grid barrier between dependent phases.  Before arriving at a
// barrier each thread loads the row bounds and first (column, value) pairs
// of the rows it will update in the next phase (the matrices are constant
// during a solve), so after the barrier only the gathers of x remain.
//
// Rows are processed by groups of `vec` lanes exactly as in the launch-chain
// kernels (lane-strided products, xor-shuffle reduction over the group), so
// the two forms of the V-cycle give bitwise the same result.
//
// Every barrier wait is bounded (kBarrierTimeoutNs on %globaltimer): a block
// that times out raises the error word, every block leaves the kernel at its
// next barrier, and the host turns the flag into AFP_ERR_TIMEOUT.
#include <algorithm>

#include "amg_internal.cuh"
#include "df32.cuh"

namespace afp {
namespace {

constexpr int kBlock = 512;
constexpr int kPF = 8;                                // (column, value) pairs loaded ahead per lane
constexpr unsigned long long kBarrierTimeoutNs = 2000000000ull;  // 2 s

enum Op : int { OP_ZERO = 0, OP_GS, OP_JAC, OP_COPY, OP_RES, OP_RESTRICT, OP_TAIL, OP_PROLONG };

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ unsigned long long now_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ unsigned atom_add_acq_rel(unsigned* p, unsigned v) {
  unsigned old;
  asm volatile("atom.add.acq_rel.gpu.global.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
  return old;
}

__device__ __forceinline__ void red_add_release(unsigned* p, unsigned v) {
  asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Sense-by-generation grid barrier: bar[0] arrivals, bar[1] generation,
// bar[2] error word.  Ordering comes from the atomics themselves: thread 0
// arrives with an acquire-release add after the block's bar.sync (its
// release covers the block's writes), the last arriver resets the count and
// publishes the next generation with a release add, and the others wait on
// it with acquire loads -- no separate sequentially consistent fences.
// Returns false (for every thread of the block) once the error word is set.
__device__ __forceinline__ bool grid_barrier(unsigned* bar, unsigned nblocks, unsigned& gen, int* s_ok) {
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned arrived = atom_add_acq_rel(&bar[0], 1u);
    if (arrived == nblocks - 1) {
      atomicExch(&bar[0], 0u);
      red_add_release(&bar[1], 1u);
    } else {
      const unsigned long long t0 = now_ns();
      unsigned spins = 0;
      while (ld_acquire(&bar[1]) == gen) {
        if ((++spins & 255u) == 0) {
          if (ld_acquire(&bar[2]) != 0u) break;
          if (now_ns() - t0 > kBarrierTimeoutNs) {
            atomicExch(&bar[2], 1u);
            break;
          }
        }
      }
    }
    *s_ok = ld_acquire(&bar[2]) == 0u;
  }
  ++gen;
  __syncthreads();
  return *s_ok != 0;
}

// Rows of one CSR operator handled by groups of `vec` lanes.
struct Rows {
  const int* rp;
  const int* ci;
  const float* va;
  int vec;
};

// One lane's view of one row: bounds and the first kPF pairs, loaded ahead.
struct Ahead {
  int k, e;
  float diag;
  int c[kPF];
  float v[kPF];
};

__device__ __forceinline__ void load_row(Ahead& a, const Rows& R, int64_t row, bool on, int lane, bool skip_diag) {
  int b = on ? R.rp[row] : 0;
  const int e = on ? R.rp[row + 1] : 0;
  a.diag = (on && skip_diag) ? R.va[b] : 1.f;
  if (skip_diag) b += 1;
  a.k = b + lane;
  a.e = e;
#pragma unroll
  for (int q = 0; q < kPF; ++q) {
    const int kk = a.k + q * R.vec;
    a.c[q] = kk < e ? R.ci[kk] : 0;
    a.v[q] = kk < e ? R.va[kk] : 0.f;
  }
}

// x is written by other blocks in earlier phases of the same launch: it must be
// read through the coherent path (no __restrict__ / read-only loads).
__device__ __forceinline__ float row_dot(const Ahead& a, const Rows& R, const float* x) {
  float s = 0.f;
#pragma unroll
  for (int q = 0; q < kPF; ++q)
    if (a.k + q * R.vec < a.e) s += a.v[q] * x[a.c[q]];
  for (int kk = a.k + kPF * R.vec; kk < a.e; kk += R.vec) s += R.va[kk] * x[R.ci[kk]];
  return s;
}

__device__ __forceinline__ float group_reduce(float s, int vec) {
  for (int o = vec / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o, vec);
  return s;
}

struct Ctx {
  const FusedLevel* L;
  const FusedPhase* ph;
  FusedTail tail;
  float* x0;
  const float* r0;
};

__device__ __forceinline__ float* lx(const Ctx& c, int l) { return l == 0 ? c.x0 : c.L[l].x; }
__device__ __forceinline__ const float* lr(const Ctx& c, int l) { return l == 0 ? c.r0 : c.L[l].r; }

// The operator a phase walks (null rp for phases without one).
__device__ __forceinline__ Rows phase_rows(const Ctx& c, const FusedPhase& p) {
  const FusedLevel& L = c.L[p.level];
  switch (p.op) {
    case OP_GS:
    case OP_JAC:
    case OP_RES:
      return {L.rp, L.ci, L.va, L.vec};
    case OP_RESTRICT:
      return {L.prp, L.pci, L.pva, L.pvec};
    case OP_PROLONG:
      return {L.trp, L.tci, L.tva, L.tvec};
    default:
      return {nullptr, nullptr, nullptr, 32};
  }
}

__global__ void __launch_bounds__(kBlock) k_vcycle_fused(const FusedLevel* __restrict__ levels,
                                                         const FusedPhase* __restrict__ phases, int nphase,
                                                         FusedTail tail, float* x0, const float* r0,
                                                         unsigned* bar) {
  __shared__ int s_ok;
  __shared__ unsigned s_gen;
  if (threadIdx.x == 0) s_gen = ld_acquire(&bar[1]);
  __syncthreads();
  unsigned gen = s_gen;
  const Ctx c{levels, phases, tail, x0, r0};
  const int64_t gtid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t nthr = (int64_t)gridDim.x * blockDim.x;
  const int64_t gwarp = gtid >> 5, nwarp = nthr >> 5;
  const int wl = threadIdx.x & 31;

  Ahead ahead;
  bool have_ahead = false;
  for (int p = 0; p < nphase; ++p) {
    const FusedPhase ph = phases[p];
    const Rows R = phase_rows(c, ph);
    const int vec = R.vec;
    const int lane = wl & (vec - 1);
    const int sub = wl / vec;
    const int64_t rpw = 32 / vec;
    switch (ph.op) {
      case OP_ZERO: {
        float* x = lx(c, ph.level);
        for (int64_t i = ph.r0 + gtid; i < ph.r1; i += nthr) x[i] = 0.f;
        break;
      }
      case OP_COPY: {  // l1-Jacobi values back into x
        const FusedLevel& L = c.L[ph.level];
        float* x = lx(c, ph.level);
        for (int64_t i = gtid; i < ph.r1 - ph.r0; i += nthr) x[ph.r0 + i] = L.tmp[i];
        break;
      }
      case OP_TAIL: {  // x_t = (hi + lo) r_t, one warp per row (as k_dense_gemv_df)
        const int64_t n = c.tail.n;
        for (int64_t row = gwarp; row < n; row += nwarp) {
          const float* h = c.tail.hi + row * n;
          const float* l = c.tail.lo + row * n;
          const float* r = c.tail.r;
          float sh = 0.f, sl = 0.f;
          int64_t j = wl;
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
          if (wl == 0) c.tail.x[row] = __fadd_rn(sh, sl);
        }
        break;
      }
      default: {  // row phases
        const FusedLevel& L = c.L[ph.level];
        const bool skip_diag = ph.op == OP_GS;
        const float* xin;  // the vector the rows are applied to
        float* out;
        switch (ph.op) {
          case OP_GS:
          case OP_JAC:
          case OP_RES:
            xin = lx(c, ph.level);
            break;
          case OP_RESTRICT:
            xin = L.tmp;
            break;
          default:  // OP_PROLONG
            xin = lx(c, ph.level + 1);
            break;
        }
        out = ph.op == OP_RESTRICT ? c.L[ph.level + 1].r : (ph.op == OP_RES ? L.tmp : lx(c, ph.level));
        const float* r = lr(c, ph.level);
        if (ph.op == OP_RES && ph.level + 1 < c.tail.level) {
          // the next level's x starts at zero; nothing reads it before its first class
          float* xn = c.L[ph.level + 1].x;
          for (int64_t i = gtid; i < c.L[ph.level + 1].n; i += nthr) xn[i] = 0.f;
        }
        bool first = true;
        for (int64_t base = ph.r0 + gwarp * rpw; base < ph.r1; base += nwarp * rpw) {
          const int64_t row = base + sub;
          const bool on = row < ph.r1;
          if (!(first && have_ahead)) load_row(ahead, R, row, on, lane, skip_diag);
          first = false;
          float s = row_dot(ahead, R, xin);
          s = group_reduce(s, vec);
          if (on && lane == 0) {
            switch (ph.op) {
              case OP_GS:
                out[row] = (r[row] - s) / ahead.diag;
                break;
              case OP_JAC:
                L.tmp[row - ph.r0] = xin[row] + (r[row] - s) / L.l1d[row - ph.r0];
                break;
              case OP_RES:
                out[row] = r[row] - s;
                break;
              case OP_RESTRICT:
                out[row] = s;
                break;
              default:  // OP_PROLONG
                out[row] = out[row] + s;
                break;
            }
          }
        }
        break;
      }
    }
    if (p + 1 == nphase) break;
    // load the next phase's first rows for this thread, then wait for the grid
    const FusedPhase nx = phases[p + 1];
    have_ahead = false;
    if (nx.op == OP_GS || nx.op == OP_JAC || nx.op == OP_RES || nx.op == OP_RESTRICT || nx.op == OP_PROLONG) {
      const Rows NR = phase_rows(c, nx);
      const int nlane = wl & (NR.vec - 1);
      const int64_t row = nx.r0 + gwarp * (32 / NR.vec) + wl / NR.vec;
      load_row(ahead, NR, row, row < nx.r1, nlane, nx.op == OP_GS);
      have_ahead = true;
    }
    if (!grid_barrier(bar, gridDim.x, gen, &s_ok)) return;
  }
}

}  // namespace

void fused_build(afp_amg* h) {
  afp_context* ctx = h->ctx;
  h->fused.reset();
  const int t = h->t;
  if (t == 0 || !h->tail_dense || h->opts.precision != AFP_PRECISION_MIXED || h->opts.interp_bf16) return;
  auto F = std::make_unique<FusedPlan>();
  std::vector<FusedLevel> lv(t);
  for (int l = 0; l < t; ++l) {
    const Level& L = h->lv[l];
    FusedLevel& f = lv[l];
    f.n = L.n;
    f.rp = L.rp.get();
    f.ci = L.ci.get();
    f.va = L.va32.get();
    f.vec = L.vec;
    f.l1d = L.l1d32.get();
    f.x = L.x32.get();
    f.r = L.r32.get();
    f.tmp = L.tmp32.get();
    f.prp = L.prp.get();
    f.pci = L.pci.get();
    f.pva = L.pva32.get();
    f.pvec = L.pvec;
    f.trp = L.trp.get();
    f.tci = L.tci.get();
    f.tva = L.tva32.get();
    f.tvec = L.tvec;
  }
  // level t (the tail) has x / r too: prolongation from it and restriction into it
  FusedLevel ft{};
  ft.n = h->lv[t].n;
  ft.x = h->lv[t].x32.get();
  ft.r = h->lv[t].r32.get();
  ft.vec = 32;
  lv.push_back(ft);
  std::vector<FusedPhase> ph;
  auto smooth = [&](int l, bool backward) {
    const Level& L = h->lv[l];
    const int K = (int)L.cls.size() - 1;
    for (int s = 0; s < h->opts.smooth_step; ++s)
      for (int q = 0; q < K; ++q) {
        const int cc = backward ? K - 1 - q : q;
        const int64_t r0 = L.cls[cc], r1 = L.cls[cc + 1];
        if (r1 <= r0) continue;
        if (L.overflow && cc == K - 1) {
          ph.push_back({OP_JAC, l, r0, r1});
          ph.push_back({OP_COPY, l, r0, r1});
        } else {
          ph.push_back({OP_GS, l, r0, r1});
        }
      }
  };
  ph.push_back({OP_ZERO, 0, 0, h->lv[0].n});
  for (int l = 0; l < t; ++l) {
    smooth(l, false);
    ph.push_back({OP_RES, l, 0, h->lv[l].n});
    ph.push_back({OP_RESTRICT, l, 0, h->lv[l + 1].n});
  }
  ph.push_back({OP_TAIL, t, 0, h->lv[t].n});
  for (int l = t - 1; l >= 0; --l) {
    ph.push_back({OP_PROLONG, l, 0, h->lv[l].n});
    smooth(l, h->opts.symmetric != 0);
  }
  F->levels.alloc(ctx, lv.size());
  F->levels.upload(lv.data(), lv.size());
  F->phases.alloc(ctx, ph.size());
  F->phases.upload(ph.data(), ph.size());
  F->nphase = (int)ph.size();
  F->tail = {h->lv[t].n, t, h->tail_hi.get(), h->tail_lo.get(), h->lv[t].x32.get(), h->lv[t].r32.get()};
  F->bar.alloc(ctx, 4);
  AFP_CUDA(cudaMemsetAsync(F->bar.get(), 0, 4 * sizeof(unsigned), ctx->stream));
  int per_sm = 0;
  AFP_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_vcycle_fused, kBlock, 0));
  AFP_REQUIRE(per_sm > 0, AFP_ERR_UNSUPPORTED, "fused V-cycle kernel does not fit on an SM");
  F->grid = per_sm * ctx->sm_count;
  sync(ctx);
  h->fused = std::move(F);
}

void fused_vcycle(afp_amg* h, float* x0, const float* r0) {
  afp_context* ctx = h->ctx;
  FusedPlan& F = *h->fused;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)F.grid);
  cfg.blockDim = dim3(kBlock);
  cfg.stream = ctx->stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  AFP_CUDA(cudaLaunchKernelEx(&cfg, k_vcycle_fused, (const FusedLevel*)F.levels.get(),
                              (const FusedPhase*)F.phases.get(), F.nphase, F.tail, x0, r0, F.bar.get()));
  check_launch(ctx, "fused V-cycle");
}

bool fused_timed_out(afp_amg* h) {
  if (!h->fused) return false;
  unsigned err = 0;
  copy(h->ctx, &err, h->fused->bar.get() + 2, sizeof(unsigned));
  sync(h->ctx);
  if (err) AFP_CUDA(cudaMemsetAsync(h->fused->bar.get(), 0, 4 * sizeof(unsigned), h->ctx->stream));
  return err != 0;
}

}  // namespace afp
