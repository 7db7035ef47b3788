/* Build-only stand-in for <cblas.h>: declares the one routine the reference
 * calls (src/core/matrix_funs.cpp:152).  Its definition is oracle/ref_sgemm.c.
 * TEST INFRASTRUCTURE ONLY. */
#ifndef BM4DOF_REF_STUB_CBLAS_H
#define BM4DOF_REF_STUB_CBLAS_H
#ifdef __cplusplus
extern "C" {
#endif
enum CBLAS_ORDER { CblasRowMajor = 101, CblasColMajor = 102 };
enum CBLAS_TRANSPOSE { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 };
void cblas_sgemm(enum CBLAS_ORDER order, enum CBLAS_TRANSPOSE transA,
                 enum CBLAS_TRANSPOSE transB, int M, int N, int K, float alpha,
                 const float *A, int lda, const float *B, int ldb, float beta,
                 float *C, int ldc);
#ifdef __cplusplus
}
#endif
#endif
