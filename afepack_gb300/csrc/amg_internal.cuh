// Internal layout of an AMG hierarchy (shared by amg.cu and mrhs.cu).
#pragma once

#include <memory>

#include "kernels.cuh"
#include "solve.cuh"

namespace afp {

// One level of the solve layout (colour-permuted numbering).
struct Level {
  int64_t n = 0, nnz = 0;
  DevBuf<int> rp, ci;
  DevBuf<double> va;
  DevBuf<float> va32;
  int vec = 8;
  std::vector<int64_t> cls;  // class boundaries (cls.size()-1 classes)
  bool overflow = false;     // the last class is the l1-Jacobi overflow class
  DevBuf<double> l1d;
  DevBuf<float> l1d32;
  // restriction P (n_{l+1} x n_l) and prolongation P^T (n_l x n_{l+1})
  DevBuf<int> prp, pci, trp, tci;
  DevBuf<double> pva, tva;
  DevBuf<__nv_bfloat16> pva16, tva16;
  DevBuf<float> pva32, tva32;
  int64_t pnnz = 0;
  int pvec = 8, tvec = 8;
  DevBuf<int> perm;  // solve order -> reference order
  DevBuf<double> x, r, tmp;
  DevBuf<float> x32, r32, tmp32;

  template <class X>
  CSRView<X> A() const;
};

template <>
inline CSRView<double> Level::A<double>() const {
  return {n, rp.get(), ci.get(), va.get(), vec};
}
template <>
inline CSRView<float> Level::A<float>() const {
  return {n, rp.get(), ci.get(), va32.get(), vec};
}

// values of P (restriction) and P^T (prolongation) in the V-cycle's storage type
template <class PV>
const PV* p_vals(const Level& L);
template <class PV>
const PV* pt_vals(const Level& L);
template <>
inline const double* p_vals<double>(const Level& L) { return L.pva.get(); }
template <>
inline const float* p_vals<float>(const Level& L) { return L.pva32.get(); }
template <>
inline const __nv_bfloat16* p_vals<__nv_bfloat16>(const Level& L) { return L.pva16.get(); }
template <>
inline const double* pt_vals<double>(const Level& L) { return L.tva.get(); }
template <>
inline const float* pt_vals<float>(const Level& L) { return L.tva32.get(); }
template <>
inline const __nv_bfloat16* pt_vals<__nv_bfloat16>(const Level& L) { return L.tva16.get(); }

// Work space of the batched multi-right-hand-side solver for k columns.
struct MultiState {
  int k = 0;
  bool mixed = false;
  std::vector<DevBuf<double>> X, R, T;      // per level, n_l x k (FP64 V-cycle)
  std::vector<DevBuf<float>> X32, R32, T32; // per level, n_l x k (FP32 V-cycle)
  DevBuf<double> B, Xs, Rs, Z, P, Q, Tmp;   // level-0 CG blocks, n x k
  DevBuf<double> scal;                      // column scalars, 8 x k
  DevBuf<int> active;                       // k flags
  DevBuf<float2> tail_part;                 // split-inner-dimension partial pairs of the dense tail
  int tail_split = 1;
  cudaGraphExec_t graph = nullptr;
  int64_t graph_nodes = 0;
  ~MultiState() {
    if (graph) cudaGraphExecDestroy(graph);
  }
};

// ------------------------------------------------ streamed V-cycle (vcycle_stream.cu)
// An FP32 CSR operator cut into tiles for the streamed V-cycle.  A tile is a
// run of at most 256 rows stored as one contiguous, 16-byte aligned blob: the
// rows' start offsets (uint16, in groups, nrows + 1 of them, padded to 16
// bytes) followed by the rows' groups of four (column, value) pairs, 32 bytes
// each (four int32 columns, then four FP32 values); rows are padded to whole
// groups with entries that repeat the row's last column with value 0.  Each
// colour class is split into one run of rows per CTA, balanced by stored
// entries, and each run into tiles that fit a shared-memory slot.
struct TiledOp {
  int64_t m = 0;
  DevBuf<char> blob;
  std::vector<int64_t> off;              // blob offset of each tile
  std::vector<int> row0, nrows, ngroups; // per tile
  std::vector<int> first;                // tiles of (class c, CTA k): [first[c*G+k], first[c*G+k+1])
};

// Device view of one level of the FP32 V-cycle.
struct StreamLevel {
  int64_t n = 0;
  float* x = nullptr;
  float* r = nullptr;
  float* tmp = nullptr;
  float* snap = nullptr;        // old values of the overflow class rows
  const float* l1d = nullptr;   // l1 diagonal of the overflow class (row - ov0)
  int ov0 = 0;                  // first row of the overflow class (n: none)
  const int* rp = nullptr;      // FP32 CSR of the level (diagonal tail solve)
  const float* va = nullptr;
};
// One phase as one CTA sees it: its stream entries [tile0, tile0 + ntiles);
// when the next phase is the level's l1-Jacobi class, its own overflow rows
// [snap0, snap1) to copy into the snapshot at the end; and how the next phase
// waits for this one: a grid barrier (sync 0) or only the CTAs whose rows are
// coupled to this CTA's rows on this level (sync 1, between colour classes).
struct StreamPhase {
  int op = 0, level = 0, tile0 = 0, ntiles = 0, snap0 = 0, snap1 = 0, sync = 0;
};
// One entry of a CTA's stream: a row tile (blob at src; rows [row0, row0 + n))
// or a segment of one dense tail row (row0; first column n; hi at src, lo at
// src2).  meta: bits 0-3 entries in the wave that starts here (0 inside a
// wave), bits 4-9 lanes per row for that wave, bit 10 last segment of a tail
// row, bits 16-31 bytes of the blob's row-offset table.
struct StreamTile {
  const void* src;
  const void* src2;
  int bytes, row0, n, meta;
};
struct StreamArgs {
  const StreamLevel* L;
  const StreamPhase* ph;    // [grid][nphase]
  const StreamTile* tiles;  // every CTA's stream, CTA k's from tile_off[k]
  const int* tile_off;
  int nphase, t;
  unsigned* bar;            // [arrivals, arrival base, error word, phase that gave up, launch epoch]
  unsigned* prog;           // per CTA (stride 32 words): epoch * 4096 + last phase finished
  const int* nb;            // neighbour CTAs of each CTA on each level
  const int* nb_off;        // [level * (grid + 1) + cta]: its range in nb
  long long limit_ns;
  int stall;                // fault injection: the first grid barrier never completes
  const double* r64;        // level-0 right-hand side (FP64, solve order)
  double* z64;              // the V-cycle's result (FP64, solve order)
  unsigned long long* trace;  // per-phase timestamps of three CTAs (diagnostic), or null
};
struct FusedPlan {
  std::vector<TiledOp> ops;  // per level: A, P, P^T
  std::vector<DevBuf<float>> snap;
  DevBuf<StreamLevel> levels;
  DevBuf<StreamPhase> phases;
  DevBuf<StreamTile> tiles;
  DevBuf<int> tile_off;
  DevBuf<unsigned> bar;
  DevBuf<unsigned> prog;
  DevBuf<int> nb, nb_off;
  DevBuf<unsigned long long> trace;
  int nphase = 0;
  int64_t ntiles = 0;
  int64_t grid = 0;
};

}  // namespace afp

struct afp_amg {
  afp_context* ctx = nullptr;
  afp_amg_opts opts{};
  int n_project = 0;   // levels built (projections)
  bool most_full = true;
  int t = 0;           // smoothed levels 0..t-1, level t is the tail
  bool tail_dense = true;
  std::vector<afp::Level> lv;
  std::vector<afp::HostCSR> refA, refP;  // reference-order copies for download
  bool lazy = false;                      // hierarchy from lazyProject (AMGPreconditioner)
  std::vector<afp::HostCSR> refPt;        // lazyProject's own P^T, used by the Galerkin product
  std::shared_ptr<afp::Pattern> pat0;     // the fine matrix's pattern object (lazy re-setup check)
  afp::DevBuf<double> tail_inv;           // FP64 dense inverse (FP64 precision)
  afp::DevBuf<float> tail_hi, tail_lo;    // the same as an FP32 pair hi + lo (mixed precision)
  int64_t tail_ld = 0;                    // row stride of hi / lo (a multiple of 4 floats)
  // solver vectors (level-0 solve order)
  afp::DevBuf<double> b, x, r, z, p, q, tmp;
  afp::DevBuf<float> r32, z32;
  cudaGraphExec_t graph64 = nullptr, graph32 = nullptr;
  int64_t graph64_nodes = 0, graph32_nodes = 0;
  std::unique_ptr<afp::MultiState> multi;
  // whole-CG graphs (first iteration + conditional while loop), per precision
  cudaGraphExec_t loop64 = nullptr, loop32 = nullptr;
  int64_t loop_pre_nodes[2] = {0, 0}, loop_body_nodes[2] = {0, 0};
  afp::DevBuf<int> loopvars;  // [iterations done, iteration limit]
  std::unique_ptr<afp::FusedPlan> fused;  // set when the FP32 V-cycle runs as one streamed persistent kernel

  ~afp_amg() {
    if (graph64) cudaGraphExecDestroy(graph64);
    if (graph32) cudaGraphExecDestroy(graph32);
    if (loop64) cudaGraphExecDestroy(loop64);
    if (loop32) cudaGraphExecDestroy(loop32);
  }
};

namespace afp {
// Batched CG over nrhs columns (mrhs.cu); false when a column stopped at
// the iteration limit above the tolerance.
void time_multi(afp_amg* h, int kind, int level, int reps, double* ms, double* bytes);
bool pcg_multi(afp_amg* h, double* X_user, const double* B_user, int nrhs, double tol, int maxit,
               afp_solve_info* info);
// Streamed FP32 V-cycle (vcycle_stream.cu): plan from the solve layout
// (leaves h->fused empty when it does not apply), launch z64 = V(r64) on the
// level-0 solve order, the bounded-wait error flag (read and cleared), and,
// with AFP_VCYCLE_TRACE set, per-phase times of the last launch on stderr.
void fused_build(afp_amg* h);
void fused_vcycle(afp_amg* h, const double* r64, double* z64);
bool fused_timed_out(afp_amg* h);
void fused_print_trace(afp_amg* h);
}  // namespace afp
