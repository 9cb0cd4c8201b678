/* CBLAS interface (the netlib CBLAS declarations pyLOM's compiled path calls)
 * mapped onto the prefixed symbols of the OpenBLAS build that SciPy bundles
 * (scipy_cblas_*, LP64).  Test infrastructure for the CPU baseline. */
#ifndef PLOM_REF_CBLAS_SHIM_H
#define PLOM_REF_CBLAS_SHIM_H
enum CBLAS_ORDER { CblasRowMajor = 101, CblasColMajor = 102 };
enum CBLAS_TRANSPOSE { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 };
typedef enum CBLAS_ORDER CBLAS_ORDER;
typedef enum CBLAS_TRANSPOSE CBLAS_TRANSPOSE;
#define CBLAS_INDEX size_t
#include <stddef.h>

#define cblas_sgemm scipy_cblas_sgemm
#define cblas_dgemm scipy_cblas_dgemm
#define cblas_cgemm scipy_cblas_cgemm
#define cblas_zgemm scipy_cblas_zgemm
#define cblas_sscal scipy_cblas_sscal
#define cblas_dscal scipy_cblas_dscal
#define cblas_cscal scipy_cblas_cscal
#define cblas_zscal scipy_cblas_zscal

void cblas_sgemm(enum CBLAS_ORDER o, enum CBLAS_TRANSPOSE ta, enum CBLAS_TRANSPOSE tb, int m, int n,
                 int k, float alpha, const float* a, int lda, const float* b, int ldb, float beta,
                 float* c, int ldc);
void cblas_dgemm(enum CBLAS_ORDER o, enum CBLAS_TRANSPOSE ta, enum CBLAS_TRANSPOSE tb, int m, int n,
                 int k, double alpha, const double* a, int lda, const double* b, int ldb,
                 double beta, double* c, int ldc);
void cblas_cgemm(enum CBLAS_ORDER o, enum CBLAS_TRANSPOSE ta, enum CBLAS_TRANSPOSE tb, int m, int n,
                 int k, const void* alpha, const void* a, int lda, const void* b, int ldb,
                 const void* beta, void* c, int ldc);
void cblas_zgemm(enum CBLAS_ORDER o, enum CBLAS_TRANSPOSE ta, enum CBLAS_TRANSPOSE tb, int m, int n,
                 int k, const void* alpha, const void* a, int lda, const void* b, int ldb,
                 const void* beta, void* c, int ldc);
void cblas_sscal(int n, float alpha, float* x, int incx);
void cblas_dscal(int n, double alpha, double* x, int incx);
void cblas_cscal(int n, const void* alpha, void* x, int incx);
void cblas_zscal(int n, const void* alpha, void* x, int incx);
#endif
