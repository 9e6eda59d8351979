// CBLAS declarations of the calls that the reference's core/krylov/piram/piram/blitzblas.h
// makes, bound to the BLAS that ships inside scipy (its symbols carry a "scipy_" prefix):
// each cblas_<name> is a macro for scipy_cblas_<name>. Standard CBLAS signatures, 32-bit
// integers. Test infrastructure of the oracle only.
#ifndef ORACLE_REF_CBLAS_SHIM_H
#define ORACLE_REF_CBLAS_SHIM_H

enum CBLAS_ORDER { CblasRowMajor = 101, CblasColMajor = 102 };
enum CBLAS_TRANSPOSE { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 };
enum CBLAS_UPLO { CblasUpper = 121, CblasLower = 122 };
enum CBLAS_DIAG { CblasNonUnit = 131, CblasUnit = 132 };
enum CBLAS_SIDE { CblasLeft = 141, CblasRight = 142 };

#define cblas_dznrm2 scipy_cblas_dznrm2
#define cblas_zaxpy scipy_cblas_zaxpy
#define cblas_zcopy scipy_cblas_zcopy
#define cblas_zdotc_sub scipy_cblas_zdotc_sub
#define cblas_zgemm scipy_cblas_zgemm
#define cblas_zgemv scipy_cblas_zgemv
#define cblas_zgbmv scipy_cblas_zgbmv
#define cblas_zhbmv scipy_cblas_zhbmv
#define cblas_zscal scipy_cblas_zscal
#define cblas_ztbmv scipy_cblas_ztbmv
#define cblas_ztbsv scipy_cblas_ztbsv

double cblas_dznrm2(const int N, const void *X, const int incX);
void cblas_zaxpy(const int N, const void *alpha, const void *X, const int incX, void *Y, const int incY);
void cblas_zcopy(const int N, const void *X, const int incX, void *Y, const int incY);
void cblas_zdotc_sub(const int N, const void *X, const int incX, const void *Y, const int incY, void *dotc);
void cblas_zgemm(enum CBLAS_ORDER Order, enum CBLAS_TRANSPOSE TransA, enum CBLAS_TRANSPOSE TransB, const int M,
                 const int N, const int K, const void *alpha, const void *A, const int lda, const void *B,
                 const int ldb, const void *beta, void *C, const int ldc);
void cblas_zgemv(enum CBLAS_ORDER order, enum CBLAS_TRANSPOSE TransA, const int M, const int N, const void *alpha,
                 const void *A, const int lda, const void *X, const int incX, const void *beta, void *Y,
                 const int incY);
void cblas_zgbmv(enum CBLAS_ORDER order, enum CBLAS_TRANSPOSE TransA, const int M, const int N, const int KL,
                 const int KU, const void *alpha, const void *A, const int lda, const void *X, const int incX,
                 const void *beta, void *Y, const int incY);
void cblas_zhbmv(enum CBLAS_ORDER order, enum CBLAS_UPLO Uplo, const int N, const int K, const void *alpha,
                 const void *A, const int lda, const void *X, const int incX, const void *beta, void *Y,
                 const int incY);
void cblas_zscal(const int N, const void *alpha, void *X, const int incX);
void cblas_ztbmv(enum CBLAS_ORDER order, enum CBLAS_UPLO Uplo, enum CBLAS_TRANSPOSE TransA, enum CBLAS_DIAG Diag,
                 const int N, const int K, const void *A, const int lda, void *X, const int incX);
void cblas_ztbsv(enum CBLAS_ORDER order, enum CBLAS_UPLO Uplo, enum CBLAS_TRANSPOSE TransA, enum CBLAS_DIAG Diag,
                 const int N, const int K, const void *A, const int lda, void *X, const int incX);
#endif
