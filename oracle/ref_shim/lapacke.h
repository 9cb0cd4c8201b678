/* LAPACKE interface (the row-major C declarations pyLOM's compiled path
 * calls) mapped onto the prefixed symbols of the OpenBLAS build that SciPy
 * bundles (scipy_LAPACKE_*, LP64).  Test infrastructure for the CPU
 * baseline. */
#ifndef PLOM_REF_LAPACKE_SHIM_H
#define PLOM_REF_LAPACKE_SHIM_H
#include <complex.h>
typedef int lapack_int;
typedef float _Complex lapack_complex_float;
typedef double _Complex lapack_complex_double;
#define LAPACK_ROW_MAJOR 101
#define LAPACK_COL_MAJOR 102

#define LAPACKE_sgeqrf scipy_LAPACKE_sgeqrf
#define LAPACKE_dgeqrf scipy_LAPACKE_dgeqrf
#define LAPACKE_cgeqrf scipy_LAPACKE_cgeqrf
#define LAPACKE_zgeqrf scipy_LAPACKE_zgeqrf
#define LAPACKE_sorgqr scipy_LAPACKE_sorgqr
#define LAPACKE_dorgqr scipy_LAPACKE_dorgqr
#define LAPACKE_cungqr scipy_LAPACKE_cungqr
#define LAPACKE_zungqr scipy_LAPACKE_zungqr
#define LAPACKE_sgesvd scipy_LAPACKE_sgesvd
#define LAPACKE_dgesvd scipy_LAPACKE_dgesvd
#define LAPACKE_cgesvd scipy_LAPACKE_cgesvd
#define LAPACKE_zgesvd scipy_LAPACKE_zgesvd
#define LAPACKE_sgesdd scipy_LAPACKE_sgesdd
#define LAPACKE_dgesdd scipy_LAPACKE_dgesdd
#define LAPACKE_cgesdd scipy_LAPACKE_cgesdd
#define LAPACKE_zgesdd scipy_LAPACKE_zgesdd
#define LAPACKE_sgetrf scipy_LAPACKE_sgetrf
#define LAPACKE_dgetrf scipy_LAPACKE_dgetrf
#define LAPACKE_cgetrf scipy_LAPACKE_cgetrf
#define LAPACKE_zgetrf scipy_LAPACKE_zgetrf
#define LAPACKE_sgetri scipy_LAPACKE_sgetri
#define LAPACKE_dgetri scipy_LAPACKE_dgetri
#define LAPACKE_cgetri scipy_LAPACKE_cgetri
#define LAPACKE_zgetri scipy_LAPACKE_zgetri
#define LAPACKE_strtri scipy_LAPACKE_strtri
#define LAPACKE_dtrtri scipy_LAPACKE_dtrtri
#define LAPACKE_ctrtri scipy_LAPACKE_ctrtri
#define LAPACKE_ztrtri scipy_LAPACKE_ztrtri
#define LAPACKE_cpotrf scipy_LAPACKE_cpotrf
#define LAPACKE_zpotrf scipy_LAPACKE_zpotrf
#define LAPACKE_sgeev scipy_LAPACKE_sgeev
#define LAPACKE_dgeev scipy_LAPACKE_dgeev

#define PLOM_QR_DECL(p, T, Q)                                                                 \
  lapack_int LAPACKE_##p##geqrf(int l, lapack_int m, lapack_int n, T* a, lapack_int lda, T* tau); \
  lapack_int LAPACKE_##p##Q(int l, lapack_int m, lapack_int n, lapack_int k, T* a,               \
                            lapack_int lda, const T* tau);
PLOM_QR_DECL(s, float, orgqr)
PLOM_QR_DECL(d, double, orgqr)
PLOM_QR_DECL(c, lapack_complex_float, ungqr)
PLOM_QR_DECL(z, lapack_complex_double, ungqr)

#define PLOM_SVD_DECL(p, T, RT)                                                                  \
  lapack_int LAPACKE_##p##gesvd(int l, char ju, char jvt, lapack_int m, lapack_int n, T* a,      \
                                lapack_int lda, RT* s, T* u, lapack_int ldu, T* vt,             \
                                lapack_int ldvt, RT* superb);                                    \
  lapack_int LAPACKE_##p##gesdd(int l, char jz, lapack_int m, lapack_int n, T* a, lapack_int lda, \
                                RT* s, T* u, lapack_int ldu, T* vt, lapack_int ldvt);            \
  lapack_int LAPACKE_##p##getrf(int l, lapack_int m, lapack_int n, T* a, lapack_int lda,         \
                                lapack_int* ipiv);                                               \
  lapack_int LAPACKE_##p##getri(int l, lapack_int n, T* a, lapack_int lda,                       \
                                const lapack_int* ipiv);                                         \
  lapack_int LAPACKE_##p##trtri(int l, char uplo, char diag, lapack_int n, T* a, lapack_int lda);
PLOM_SVD_DECL(s, float, float)
PLOM_SVD_DECL(d, double, double)
PLOM_SVD_DECL(c, lapack_complex_float, float)
PLOM_SVD_DECL(z, lapack_complex_double, double)

lapack_int LAPACKE_cpotrf(int l, char uplo, lapack_int n, lapack_complex_float* a, lapack_int lda);
lapack_int LAPACKE_zpotrf(int l, char uplo, lapack_int n, lapack_complex_double* a, lapack_int lda);
lapack_int LAPACKE_sgeev(int l, char jvl, char jvr, lapack_int n, float* a, lapack_int lda,
                         float* wr, float* wi, float* vl, lapack_int ldvl, float* vr,
                         lapack_int ldvr);
lapack_int LAPACKE_dgeev(int l, char jvl, char jvr, lapack_int n, double* a, lapack_int lda,
                         double* wr, double* wi, double* vl, lapack_int ldvl, double* vr,
                         lapack_int ldvr);
#endif
