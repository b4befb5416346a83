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
  cudaGraphExec_t graph = nullptr;
  int64_t graph_nodes = 0;
  ~MultiState() {
    if (graph) cudaGraphExecDestroy(graph);
  }
};

// Device-side description of the FP32 V-cycle for the fused cooperative
// kernel (vcycle_fused.cu): one entry per smoothed level plus the tail level.
struct FusedLevel {
  int64_t n = 0;
  const int* rp = nullptr;
  const int* ci = nullptr;
  const float* va = nullptr;
  int vec = 32;
  const float* l1d = nullptr;  // l1 diagonal of the overflow class
  float* x = nullptr;          // level vectors (level 0 uses the launch's x0 / r0)
  float* r = nullptr;
  float* tmp = nullptr;
  const int* prp = nullptr;    // restriction P (rows = next level)
  const int* pci = nullptr;
  const float* pva = nullptr;
  int pvec = 32;
  const int* trp = nullptr;    // prolongation P^T (rows = this level)
  const int* tci = nullptr;
  const float* tva = nullptr;
  int tvec = 32;
};
struct FusedPhase {
  int op;
  int level;
  int64_t r0, r1;
};
struct FusedTail {
  int64_t n;
  int level;
  const float* hi;
  const float* lo;
  float* x;
  const float* r;
};
struct FusedPlan {
  DevBuf<FusedLevel> levels;
  DevBuf<FusedPhase> phases;
  int nphase = 0;
  FusedTail tail{};
  DevBuf<unsigned> bar;  // [arrivals, generation, error word, unused]
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
  std::unique_ptr<afp::FusedPlan> fused;  // set when the FP32 V-cycle runs as one cooperative kernel

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
bool pcg_multi(afp_amg* h, double* X_user, const double* B_user, int nrhs, double tol, int maxit,
               afp_solve_info* info);
// Fused FP32 V-cycle (vcycle_fused.cu): plan from the solve layout (leaves
// h->fused empty when it does not apply), launch, and the barrier-timeout flag.
void fused_build(afp_amg* h);
void fused_vcycle(afp_amg* h, float* x0, const float* r0);
bool fused_timed_out(afp_amg* h);
}  // namespace afp
