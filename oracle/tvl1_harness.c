/* TEST INFRASTRUCTURE ONLY: a C entry point over the reference's own TV-L1
 * code (lib/tvl1flow/tvl1flow_lib.c and the files it includes), compiled from
 * the reference tree into oracle/_ref/libtvl1_ref.so.  It mirrors what the
 * tvl1flow program does between reading and writing its files
 * (lib/tvl1flow/main.c:147-176): cap the number of scales, then call
 * Dual_TVL1_optic_flow_multiscale.  One OpenMP thread, so that the stopping
 * test's float sum is taken in pixel order. */
#include <math.h>
#include <omp.h>

#include "tvl1flow_lib.c"

void ref_tvl1(const float *I0, const float *I1, int nx, int ny, float tau, float lambda, float theta,
              int nscales, int fscale, float zfactor, int nwarps, float epsilon, float *u, float *v)
{
	const float N = 1 + log(hypot(nx, ny) / 16.0) / log(1 / zfactor);
	if (N < nscales) nscales = N;
	if (nscales < fscale) fscale = nscales;
	omp_set_num_threads(1);
	Dual_TVL1_optic_flow_multiscale((float *)I0, (float *)I1, u, v, nx, ny, tau, lambda, theta, nscales, fscale,
	                                zfactor, nwarps, epsilon, false);
}
