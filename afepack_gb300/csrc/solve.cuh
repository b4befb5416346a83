// Sparse kernels of the V-cycle and the outer CG (declarations).
#pragma once

#include <cuda_bf16.h>

#include "common.cuh"

namespace afp {

// Read-only CSR view; V is the stored value type (double, float, bf16).
template <class V>
struct CSRView {
  int64_t m = 0;
  const int* rowptr = nullptr;
  const int* cols = nullptr;
  const V* vals = nullptr;
  int vec = 8;  // threads per row
};

int pick_vec(double avg_row_len);

// y = A x (add == false) or y += A x (add == true); X is the vector type.
template <class V, class X>
void spmv(const afp_context* ctx, const CSRView<V>& A, const X* x, X* y, bool add);

// out = r - A x
template <class X>
void residual(const afp_context* ctx, const CSRView<X>& A, const X* x, const X* r, X* out);

// One Gauss-Seidel colour class: rows [r0, r1) are mutually uncoupled,
// x_j = (r_j - sum_{k != j} a_jk x_k) / a_jj with the diagonal stored first.
template <class X>
void gs_class(const afp_context* ctx, const CSRView<X>& A, int64_t r0, int64_t r1, X* x, const X* r);

// l1-Jacobi on the overflow class [r0, r1): x_j += (r_j - (A x)_j) / d_j,
// d_j = a_jj + sum of |a_jk| over the class's other rows; tmp holds r1-r0 values.
template <class X>
void jacobi_l1_class(const afp_context* ctx, const CSRView<X>& A, int64_t r0, int64_t r1, X* x, const X* r,
                     const X* l1diag, X* tmp);

// x = Ainv r for a dense n x n row-major inverse.
template <class X>
void dense_gemv(const afp_context* ctx, int64_t n, const X* Ainv, const X* r, X* x);

// FP64 n x n inverse -> FP32 pair (hi, lo) with hi + lo == inv to ~2^-48;
// the pair's rows have stride ld >= n (a multiple of 4, so that every row
// starts 16-byte aligned) and zeros in columns [n, ld).
void split_df(const afp_context* ctx, int64_t n, int64_t ld, const double* inv, float* hi, float* lo);

// x = (hi + lo) r in FP32 with double-float accumulation (the FP32 V-cycle's
// dense coarsest solve; see df32.cuh); rows of the pair have stride ld.
void dense_gemv_df(const afp_context* ctx, int64_t n, int64_t ld, const float* hi, const float* lo, const float* r,
                   float* x);

// x_j = r_j / a_jj (coarsest level when it is not full).
template <class X>
void diag_solve(const afp_context* ctx, const CSRView<X>& A, const X* r, X* x);

// ----------------------------------------------------------- vector ops
template <class A, class B>
void convert(const afp_context* ctx, int64_t n, const A* in, B* out);
void permute_gather(const afp_context* ctx, int64_t n, const int* perm, const double* in, double* out);   // out[i] = in[perm[i]]
void permute_scatter(const afp_context* ctx, int64_t n, const int* perm, const double* in, double* out);  // out[perm[i]] = in[i]
// y += alpha x
void axpy(const afp_context* ctx, int64_t n, double alpha, const double* x, double* y);
// dst[i*ds] = src[i*ss]
void strided_copy(const afp_context* ctx, int64_t n, const double* src, int64_t ss, double* dst, int64_t ds);
template <class X>
void fill_zero(const afp_context* ctx, int64_t n, X* x);

// Deterministic FP64 reductions into dst (device scalar).
void dot(const afp_context* ctx, int64_t n, const double* a, const double* b, double* dst);
// y = A p and dst = p . y in one pass
void spmv_dot(const afp_context* ctx, const CSRView<double>& A, const double* p, double* y, double* dst);
// x += alpha p, r -= alpha q, alpha = s[num] / s[den]; dst = r . r
void cg_update_xr(const afp_context* ctx, int64_t n, const double* s, int num, int den, double* x, double* r,
                  const double* p, const double* q, double* dst);
// p = z + beta p, beta = s[num] / s[den]
void cg_update_p(const afp_context* ctx, int64_t n, const double* s, int num, int den, const double* z, double* p);

// --------------------------------------------------------- setup helpers
// Builds B with rows B[i] = A[rperm[i]] and columns mapped through cmap
// (the diagonal stays first when rperm and cmap agree).
void permute_csr(const afp_context* ctx, int64_t m, const int* rowptr, const int* cols, const double* vals,
                 const int* rperm, const int* cmap, int64_t nnz, DevBuf<int>& out_rowptr, DevBuf<int>& out_cols,
                 DevBuf<double>& out_vals);
// d_j = a_jj + sum_{k in [r0,r1), k != j} |a_jk| for j in [r0, r1)
void l1_diag(const afp_context* ctx, const CSRView<double>& A, int64_t r0, int64_t r1, double* d);
// Dense inverse of the n x n CSR matrix by Gauss-Jordan elimination with
// partial pivoting; returns false when a pivot is zero.
bool dense_inverse(const afp_context* ctx, const CSRView<double>& A, double* inv);

}  // namespace afp
