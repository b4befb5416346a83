// Declarations shared between the library's translation units.
#pragma once

#include "common.cuh"

namespace afp {

// y = A x over a CSR (any row order); one launch.
void csr_spmv(const afp_context* ctx, int64_t m, const int* rowptr, const int* cols, const double* vals,
              const double* x, double* y);

// Galerkin product A_c = P A P^T with AFEPack's pattern (diagonal first,
// then ascending) and getPMPt's accumulation order.  P is n_c x n_f with
// ascending columns, Pt its transpose with ascending columns.
void galerkin_product(const afp_context* ctx, int64_t n_c, int64_t n_f, const int* p_rowptr, const int* p_cols,
                      const double* p_vals, const int* a_rowptr, const int* a_cols, const double* a_vals,
                      const int* pt_rowptr, const int* pt_cols, const double* pt_vals, Pattern& out_pat,
                      DevBuf<double>& out_vals);

// Stored entries of the n_rows rows of P A P^T that the given rows of P
// produce (its symbolic count alone; n_c = columns of the product), to
// decide how to form a level before forming it.
int64_t galerkin_nnz(const afp_context* ctx, int64_t n_rows, int64_t n_c, const int* p_rowptr, const int* p_cols,
                     const int* a_rowptr, const int* a_cols, const int* pt_rowptr, const int* pt_cols);

// Reserves afp_matrix_vmult_noalloc's static staging array on `device` (the
// current device); called once per context creation (noalloc.cu).
void noalloc_reserve(int device);

// The same product through a dense intermediate (n_f x n_c and n_c x n_c
// FP64 arrays), for the dense-tail level only: deterministic, but not
// getPMPt's accumulation order; exact zeros other than the diagonal dropped.
void galerkin_product_dense(const afp_context* ctx, int64_t n_c, int64_t n_f, const int* p_rowptr,
                            const int* p_cols, const double* p_vals, const int* a_rowptr, const int* a_cols,
                            const double* a_vals, const int* pt_rowptr, const int* pt_cols, const double* pt_vals,
                            Pattern& out_pat, DevBuf<double>& out_vals);

// Host CSR (AFEPack layout) used by the coarsening.
struct HostCSR {
  int64_t m = 0, n = 0;
  std::vector<int> rowptr, cols;
  std::vector<double> vals;
  int64_t nnz() const { return rowptr.empty() ? 0 : rowptr[m]; }
};

// A device CSR (AFEPack layout for square levels, ascending rows for P, P^T).
struct DevCSR {
  int64_t m = 0, n = 0, nnz = 0;
  DevBuf<int> rp, ci;
  DevBuf<double> va;
};

// Project() on the GPU (coarsen.cu): flags and P, P^T bitwise the host
// routine's; cf[i] = 1 for C points, 0 for F points; rounds of the two
// passes for the trace.
struct GpuProjection {
  DevCSR P, Pt;
  DevBuf<int> cf;
  int rounds1 = 0, rounds2 = 0;
};
int gpu_project(const afp_context* ctx, int64_t m, const int* rowptr, const int* cols, const double* vals,
                double alpha, GpuProjection& out);

// Project(): C/F splitting and projection P (n_c x m) of one level, with
// its transpose; cf[i] = -1 (C) or 1 (F).
void host_project(const HostCSR& M, double alpha, std::vector<int>& cf, HostCSR& P, HostCSR& Pt);

// lazyProject(): aggregation-like projection P (n_c x m) and its transpose.
void host_lazy_project(const HostCSR& M, HostCSR& P, HostCSR& Pt);

// Greedy colouring of a square matrix's graph (nonzero off-diagonal entries
// couple rows): colour[i] < max_colors, or max_colors for rows that found no
// free colour (the overflow class).  Returns the number of classes used.
int host_color(const HostCSR& A, int max_colors, std::vector<int>& color);

}  // namespace afp
