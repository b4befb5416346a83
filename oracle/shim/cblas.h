/* Minimal CBLAS declarations so the reference sources compile against the
 * OpenBLAS build that ships inside SciPy (its symbols carry a scipy_ prefix).
 * Test infrastructure for the oracle only; never linked into the product. */
#pragma once
#include <cstddef>
enum CBLAS_ORDER { CblasRowMajor = 101, CblasColMajor = 102 };
enum CBLAS_TRANSPOSE { CblasNoTrans = 111, CblasTrans = 112 };
#define AFP_CBLAS(ret, name, ...) extern "C" ret scipy_cblas_##name(__VA_ARGS__);
AFP_CBLAS(double, ddot, int, const double*, int, const double*, int)
AFP_CBLAS(float, sdot, int, const float*, int, const float*, int)
AFP_CBLAS(void, daxpy, int, double, const double*, int, double*, int)
AFP_CBLAS(void, saxpy, int, float, const float*, int, float*, int)
AFP_CBLAS(void, dscal, int, double, double*, int)
AFP_CBLAS(void, sscal, int, float, float*, int)
AFP_CBLAS(double, dasum, int, const double*, int)
AFP_CBLAS(float, sasum, int, const float*, int)
AFP_CBLAS(double, dnrm2, int, const double*, int)
AFP_CBLAS(float, snrm2, int, const float*, int)
AFP_CBLAS(size_t, idamax, int, const double*, int)
AFP_CBLAS(size_t, isamax, int, const float*, int)
AFP_CBLAS(void, dgemv, CBLAS_ORDER, CBLAS_TRANSPOSE, int, int, double, const double*, int, const double*, int, double, double*, int)
AFP_CBLAS(void, sgemv, CBLAS_ORDER, CBLAS_TRANSPOSE, int, int, float, const float*, int, const float*, int, float, float*, int)
AFP_CBLAS(void, dgemm, CBLAS_ORDER, CBLAS_TRANSPOSE, CBLAS_TRANSPOSE, int, int, int, double, const double*, int, const double*, int, double, double*, int)
AFP_CBLAS(void, sgemm, CBLAS_ORDER, CBLAS_TRANSPOSE, CBLAS_TRANSPOSE, int, int, int, float, const float*, int, const float*, int, float, float*, int)
#define cblas_ddot scipy_cblas_ddot
#define cblas_sdot scipy_cblas_sdot
#define cblas_daxpy scipy_cblas_daxpy
#define cblas_saxpy scipy_cblas_saxpy
#define cblas_dscal scipy_cblas_dscal
#define cblas_sscal scipy_cblas_sscal
#define cblas_dasum scipy_cblas_dasum
#define cblas_sasum scipy_cblas_sasum
#define cblas_dnrm2 scipy_cblas_dnrm2
#define cblas_snrm2 scipy_cblas_snrm2
#define cblas_idamax scipy_cblas_idamax
#define cblas_isamax scipy_cblas_isamax
#define cblas_dgemv scipy_cblas_dgemv
#define cblas_sgemv scipy_cblas_sgemv
#define cblas_dgemm scipy_cblas_dgemm
#define cblas_sgemm scipy_cblas_sgemm
