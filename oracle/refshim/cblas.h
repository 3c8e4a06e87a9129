/* Minimal CBLAS declarations for the reference's BLAS path, bound to the
 * OpenBLAS build that ships inside scipy (its exported symbols carry a
 * "scipy_" prefix; LP64 integers). */
#ifndef ORACLE_CBLAS_SHIM_H
#define ORACLE_CBLAS_SHIM_H
#ifdef __cplusplus
extern "C" {
#endif
enum CBLAS_ORDER { CblasRowMajor = 101, CblasColMajor = 102 };
enum CBLAS_TRANSPOSE { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 };
void scipy_cblas_sgemm(enum CBLAS_ORDER, enum CBLAS_TRANSPOSE, enum CBLAS_TRANSPOSE,
                       int M, int N, int K, float alpha, const float *A, int lda,
                       const float *B, int ldb, float beta, float *C, int ldc);
void scipy_cblas_sgemv(enum CBLAS_ORDER, enum CBLAS_TRANSPOSE, int M, int N,
                       float alpha, const float *A, int lda, const float *X, int incX,
                       float beta, float *Y, int incY);
void scipy_openblas_set_num_threads(int);
char *scipy_openblas_get_corename(void);
#ifdef __cplusplus
}
#endif
#define cblas_sgemm scipy_cblas_sgemm
#define cblas_sgemv scipy_cblas_sgemv
#define openblas_set_num_threads scipy_openblas_set_num_threads
#define openblas_get_corename scipy_openblas_get_corename
#endif
