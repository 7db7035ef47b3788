/*
 * ref_sgemm.c -- TEST INFRASTRUCTURE ONLY.
 *
 * A project-written cblas_sgemm for linking the reference's own sources
 * (no CBLAS/OpenBLAS is installed).  It defines the summation order that the
 * reference's productMatrix (src/core/matrix_funs.cpp:136-164) then follows:
 * every C(i,j) is accumulated from 0 over the inner index in increasing order,
 * one rounded product and one rounded sum per term (build with
 * -ffp-contract=off), and the result is alpha*sum + beta*C, except that
 * alpha == 1, beta == 0 -- the only case the reference uses -- stores the sum.
 */
#include "ref_stubs/cblas.h"

static float elem(const float *M, int ld, int colmajor, int r, int c)
{
	return colmajor ? M[(long)c * ld + r] : M[(long)r * ld + c];
}

void cblas_sgemm(enum CBLAS_ORDER order, enum CBLAS_TRANSPOSE transA,
                 enum CBLAS_TRANSPOSE transB, int M, int N, int K, float alpha,
                 const float *A, int lda, const float *B, int ldb, float beta,
                 float *C, int ldc)
{
	const int cm = order == CblasColMajor;
	for (int j = 0; j < N; j++)
		for (int i = 0; i < M; i++) {
			float acc = 0.f;
			for (int p = 0; p < K; p++) {
				const float a = transA == CblasNoTrans ? elem(A, lda, cm, i, p) : elem(A, lda, cm, p, i);
				const float b = transB == CblasNoTrans ? elem(B, ldb, cm, p, j) : elem(B, ldb, cm, j, p);
				acc = acc + a * b;
			}
			float *c = cm ? &C[(long)j * ldc + i] : &C[(long)i * ldc + j];
			if (alpha == 1.f && beta == 0.f) *c = acc;
			else *c = alpha * acc + (beta == 0.f ? 0.f : beta * *c);
		}
}
