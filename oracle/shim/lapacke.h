/* Minimal LAPACKE declarations mapped onto SciPy's bundled OpenBLAS.
 * Test infrastructure for the oracle only; never linked into the product. */
#pragma once
typedef int lapack_int;
#define LAPACK_ROW_MAJOR 101
#define LAPACK_COL_MAJOR 102
#define AFP_LAPACKE(name, ...) extern "C" lapack_int scipy_LAPACKE_##name(__VA_ARGS__);
AFP_LAPACKE(dgetrf, int, lapack_int, lapack_int, double*, lapack_int, lapack_int*)
AFP_LAPACKE(sgetrf, int, lapack_int, lapack_int, float*, lapack_int, lapack_int*)
AFP_LAPACKE(dgetri, int, lapack_int, double*, lapack_int, const lapack_int*)
AFP_LAPACKE(sgetri, int, lapack_int, float*, lapack_int, const lapack_int*)
AFP_LAPACKE(dgesv, int, lapack_int, lapack_int, double*, lapack_int, lapack_int*, double*, lapack_int)
AFP_LAPACKE(sgesv, int, lapack_int, lapack_int, float*, lapack_int, lapack_int*, float*, lapack_int)
AFP_LAPACKE(dgeqrf, int, lapack_int, lapack_int, double*, lapack_int, double*)
AFP_LAPACKE(dormqr, int, char, char, lapack_int, lapack_int, lapack_int, const double*, lapack_int, const double*, double*, lapack_int)
AFP_LAPACKE(dtrtrs, int, char, char, char, lapack_int, lapack_int, const double*, lapack_int, double*, lapack_int)
AFP_LAPACKE(dgeqrf_work, int, lapack_int, lapack_int, double*, lapack_int, double*, double*, lapack_int)
AFP_LAPACKE(sgeqrf_work, int, lapack_int, lapack_int, float*, lapack_int, float*, float*, lapack_int)
AFP_LAPACKE(dormqr_work, int, char, char, lapack_int, lapack_int, lapack_int, const double*, lapack_int, const double*, double*, lapack_int, double*, lapack_int)
AFP_LAPACKE(sormqr_work, int, char, char, lapack_int, lapack_int, lapack_int, const float*, lapack_int, const float*, float*, lapack_int, float*, lapack_int)
#define LAPACKE_dgetrf scipy_LAPACKE_dgetrf
#define LAPACKE_sgetrf scipy_LAPACKE_sgetrf
#define LAPACKE_dgetri scipy_LAPACKE_dgetri
#define LAPACKE_sgetri scipy_LAPACKE_sgetri
#define LAPACKE_dgesv scipy_LAPACKE_dgesv
#define LAPACKE_sgesv scipy_LAPACKE_sgesv
#define LAPACKE_dgeqrf scipy_LAPACKE_dgeqrf
#define LAPACKE_dormqr scipy_LAPACKE_dormqr
#define LAPACKE_dtrtrs scipy_LAPACKE_dtrtrs
#define LAPACKE_dgeqrf_work scipy_LAPACKE_dgeqrf_work
#define LAPACKE_sgeqrf_work scipy_LAPACKE_sgeqrf_work
#define LAPACKE_dormqr_work scipy_LAPACKE_dormqr_work
#define LAPACKE_sormqr_work scipy_LAPACKE_sormqr_work
/* only the unused least-squares helper refers to these */
inline lapack_int LAPACKE_dtrsv(...) { return 0; }
inline lapack_int LAPACKE_strsv(...) { return 0; }
