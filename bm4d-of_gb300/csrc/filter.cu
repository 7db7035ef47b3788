// filter.cu -- collaborative filtering of each patch group, exact FP32.
//
// Restates VideoNLB::computeBayesEstimateStep1/2 and their _vbm3d bodies
// (src/core/nldct.cpp:1799-2006, 2015-2242) bit for bit:
//   * all-members-equal groups are left untouched and keep the previous
//     group's aggregation weights (1986-1999, 2222-2235) -- flagged here and
//     completed by fixup_equal_kernel;
//   * Z = G.B, the dense sPC x sPC patch transform, accumulated over the inner
//     index in increasing order with one rounded multiply and one rounded add
//     per term -- the order of the sequential sgemm the reference is built
//     with (productMatrix, src/core/matrix_funs.cpp:136-164);
//   * orthonormal Haar along the member axis (1846-1860), hard threshold at
//     (beta*sigma)^2 keeping coefficient (0,0) (1901-1908) or the empirical
//     Wiener gain against the basic estimate (2123-2135), inverse Haar, and
//     the inverse transform Z.Binv^T (1926-1931, 2155-2159);
//   * group weight 1/sigma^2/#kept in float (1935) or 1/sigma^2/sum(w^2) in
//     double (2167), the Wiener sum taken in the reference's order.
// The result is written as per-member aggregation terms (w*window[p])*g, the
// exact float product the reference adds into its image (2296-2297, 2385-2386).
#include <cuda_runtime.h>
#include <cstdint>

#include "common.cuh"

namespace bm4dof {

namespace {

constexpr int kFilterThreads = 256;

__device__ __forceinline__ int nsp_of(int np)
{
	// member stride of the shared-memory group tiles: a multiple of 4 (float4
	// access) plus 4, which spreads consecutive rows over distinct banks
	return ((np + 3) / 4) * 4 + 4;
}

template <int NS>
__device__ __forceinline__ void haar_forward(float (&z)[NS], float is2)
{
#pragma unroll
	for (int s = 2, h = 1; s <= NS; s *= 2, h *= 2)
#pragma unroll
		for (int n = 0; n < NS; n += s) {
			const float z0 = __fmul_rn(z[n], is2);
			const float z1 = __fmul_rn(z[n + h], is2);
			z[n] = __fadd_rn(z0, z1);
			z[n + h] = __fsub_rn(z0, z1);
		}
}

template <int NS>
__device__ __forceinline__ void haar_inverse(float (&z)[NS], float is2)
{
#pragma unroll
	for (int s = NS, h = NS / 2; s >= 2; s /= 2, h /= 2)
#pragma unroll
		for (int n = 0; n < NS; n += s) {
			const float z0 = __fmul_rn(z[n], is2);
			const float z1 = __fmul_rn(z[n + h], is2);
			z[n] = __fadd_rn(z0, z1);
			z[n + h] = __fsub_rn(z0, z1);
		}
}

// std::max(a, 0.f) as libstdc++ evaluates it ((a < 0) ? 0 : a, NaN kept)
__device__ __forceinline__ float max0(float a) { return a < 0.f ? 0.f : a; }

// One transform coefficient k of one channel: Haar over the NS members,
// shrinkage, inverse Haar.  Returns the number of kept coefficients (step 1).
// With order invariance (nldct.cpp:1865-1900, 2101-2122) one Wiener gain
// serves the mean row and one all other rows; the coefficient's share of the
// group weight, w0^2 + (NS-1) wi^2, goes to *contrib.
template <int NS, int STEP>
__device__ int shrink_column(float *zcol, const float *ycol, float *w2col, int k, float bs2,
                             float is2, bool oinv, float sigma2, float bm2, float *contrib)
{
	float z[NS];
#pragma unroll
	for (int n = 0; n < NS; n++) z[n] = zcol[n];
	haar_forward<NS>(z, is2);
	int kept = 0;
	if (oinv) {
		float y[NS];
#pragma unroll
		for (int n = 0; n < NS; n++) y[n] = STEP == 1 ? z[n] : ycol[n];
		if (STEP == 2) haar_forward<NS>(y, is2);
		float vi = 0.f;
#pragma unroll
		for (int n = 1; n < NS; n++) vi = __fadd_rn(vi, __fmul_rn(y[n], y[n]));
		vi = __fdiv_rn(vi, (float)(NS - 1));
		const float v0 = STEP == 1 ? max0(__fsub_rn(__fmul_rn(y[0], y[0]), sigma2)) : __fmul_rn(y[0], y[0]);
		const float w0 = __fdiv_rn(v0, __fadd_rn(v0, bm2));
		z[0] = __fmul_rn(z[0], w0);
		if (STEP == 1) vi = max0(__fsub_rn(vi, sigma2));
		const float wi = __fdiv_rn(vi, __fadd_rn(vi, bs2));
#pragma unroll
		for (int n = 1; n < NS; n++) z[n] = __fmul_rn(z[n], wi);
		*contrib = __fadd_rn(__fmul_rn(w0, w0), __fmul_rn(__fmul_rn((float)(NS - 1), wi), wi));
	} else if (STEP == 1) {
#pragma unroll
		for (int n = 0; n < NS; n++) {
			if (__fmul_rn(z[n], z[n]) > bs2 || (k == 0 && n == 0)) kept++;
			else z[n] = 0.f;
		}
	} else {
		float y[NS];
#pragma unroll
		for (int n = 0; n < NS; n++) y[n] = ycol[n];
		haar_forward<NS>(y, is2);
#pragma unroll
		for (int n = 0; n < NS; n++) {
			const float yy = __fmul_rn(y[n], y[n]);
			const float w = __fdiv_rn(yy, __fadd_rn(yy, bs2));
			z[n] = __fmul_rn(z[n], w);
			w2col[n] = __fmul_rn(w, w);
		}
	}
	haar_inverse<NS>(z, is2);
#pragma unroll
	for (int n = 0; n < NS; n++) zcol[n] = z[n];
	return kept;
}

template <int STEP>
__device__ int shrink_dispatch(int ns, float *zcol, const float *ycol, float *w2col, int k,
                               float bs2, float is2, bool oinv, float sigma2, float bm2, float *contrib)
{
#define SHRINK(N) shrink_column<N, STEP>(zcol, ycol, w2col, k, bs2, is2, oinv, sigma2, bm2, contrib)
	switch (ns) {
	case 1: return SHRINK(1);
	case 2: return SHRINK(2);
	case 4: return SHRINK(4);
	case 8: return SHRINK(8);
	case 16: return SHRINK(16);
	default: return SHRINK(32);
	}
#undef SHRINK
}

// out(n, q) = sum_r in(n, r) * M[r*spc + q], r increasing, for a block of 4
// members starting at n0.  in is a [r][nsp] tile, out a [q][nsp] tile.
__device__ __forceinline__ void product4(const float *in, const float *M, float *out, int spc,
                                         int nsp, int q, int n0)
{
	float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f;
	for (int r = 0; r < spc; r++) {
		const float4 g = *reinterpret_cast<const float4 *>(in + r * nsp + n0);
		const float b = M[r * spc + q];
		a0 = __fadd_rn(a0, __fmul_rn(g.x, b));
		a1 = __fadd_rn(a1, __fmul_rn(g.y, b));
		a2 = __fadd_rn(a2, __fmul_rn(g.z, b));
		a3 = __fadd_rn(a3, __fmul_rn(g.w, b));
	}
	*reinterpret_cast<float4 *>(out + q * nsp + n0) = make_float4(a0, a1, a2, a3);
}

// PX, PT, CC: patch size, patch frames and channels when known at compile
// time (0: taken from sp), so that the index arithmetic of the per-element
// loops folds into shifts and multiplies.
template <int STEP, int PX, int PT, int CC>
__global__ void __launch_bounds__(kFilterThreads, STEP == 2 ? 3 : 4)
filter_exact_kernel(Image noisy, Image basic, const Tile *__restrict__ tiles, int ntiles,
                    StepParams sp, const float *__restrict__ basis, const float *__restrict__ binv,
                    const float *__restrict__ win, long long g_begin, long long g_end,
                    const uint8_t *__restrict__ nsimp, const uint32_t *__restrict__ idx,
                    const uint8_t *__restrict__ alive, float *__restrict__ vals,
                    float *__restrict__ wslot, float *__restrict__ wgroup, uint8_t *__restrict__ eq)
{
	extern __shared__ __align__(16) float sm[];
	const int px = PX ? PX : sp.px, pt = PT ? PT : sp.pt, C = CC ? CC : sp.C;
	const int spc = px * px * pt, np = sp.np;
	const int nsp = nsp_of(np);
	const int tile_f = C * spc * nsp;          // floats of one group tile (all channels)
	const int bsz = ((spc * spc + 3) / 4) * 4; // basis sizes padded: the group tiles
	                                           // below must start on 16-byte boundaries
	float *Bt = sm;                            // Bt[p*spc + k] = basis[k*spc + p]
	float *Bi = Bt + bsz;                      // Bi[k*spc + p] = binv[k*spc + p]
	float *wn = Bi + bsz;                      // window
	float *Gn = wn + ((spc + 3) / 4) * 4;      // noisy group   [c][p][n]
	float *Zn = Gn + tile_f;                   // its transform [c][k][n]
	float *Gb = Zn + tile_f;                   // basic group (step 2); later Wiener w^2
	float *Zb = Gb + tile_f;
	__shared__ int s_mx[kMaxNp], s_my[kMaxNp], s_mt[kMaxNp];
	__shared__ int s_kept, s_ns, s_tile, s_equal;
	__shared__ float s_w;

	const int tid = threadIdx.x;
	for (int i = tid; i < spc * spc; i += blockDim.x) {
		const int k = i / spc, p = i % spc;
		Bt[p * spc + k] = basis[i];
		Bi[i] = binv[i];
	}
	for (int i = tid; i < spc; i += blockDim.x) wn[i] = win[i];

	const float sigma2 = __fmul_rn(sp.sigma, sp.sigma);
	const float bsig = __fmul_rn(sp.beta, sp.sigma);
	const float bs2 = __fmul_rn(bsig, bsig);
	const float bmsig = __fmul_rn(sp.beta_mean, sp.sigma);
	const float bm2 = __fmul_rn(bmsig, bmsig);
	const bool oinv = sp.order_inv != 0;
	const float is2 = (float)(1.0 / sqrt(2.0));

	for (long long g = g_begin + blockIdx.x; g < g_end; g += gridDim.x) {
		__syncthreads();
		if (!alive[g]) continue;
		if (tid == 0) {
			const int ti = tile_of(tiles, ntiles, g);
			s_tile = ti;
			s_ns = nsimp[g];
			s_kept = 0;
			s_equal = 0;
		}
		__syncthreads();
		const int ns = s_ns;
		const Tile T = tiles[s_tile];
		if (tid < ns) {
			const uint32_t lin = idx[g * np + tid];
			const uint32_t whl = (uint32_t)T.w * T.h;
			s_mt[tid] = (int)(lin / whl);
			s_my[tid] = (int)((lin % whl) / T.w);
			s_mx[tid] = (int)(lin % T.w);
		}
		__syncthreads();

		// gather the group: member-fastest tiles G[c][p][n] (nldct.cpp:1334-1339)
		const int per = C * spc;
		for (int it = tid; it < ns * per; it += blockDim.x) {
			const int n = it / per, r = it % per;
			const int c = r / spc, p = r % spc;
			const int ht = p / (px * px), hy = (p / px) % px, hx = p % px;
			const size_t a = noisy.at(T.ox + s_mx[n] + hx, T.oy + s_my[n] + hy, s_mt[n] + ht, c);
			Gn[(c * spc + p) * nsp + n] = __ldg(noisy.p + a);
			if (STEP == 2) Gb[(c * spc + p) * nsp + n] = __ldg(basic.p + a);
		}
		__syncthreads();

		const long long slot0 = (g - g_begin) * np;   // slots are chunk-relative
		// all-equal test (nldct.cpp:1986-1999, 2222-2235)
		int differs = 0;
		if (ns > 1)
			for (int r = tid; r < per; r += blockDim.x) {
				const float *row = Gn + r * nsp;
				for (int n = 1; n < ns; n++) differs |= row[n] != row[0];
			}
		const int any = __syncthreads_or(differs);
		if (ns > 1 && !any) {
			for (int it = tid; it < ns * per; it += blockDim.x) {
				const int n = it / per, r = it % per;
				vals[(slot0 + n) * per + r] = Gn[r * nsp + n];
			}
			if (tid == 0) eq[g] = 1;
			continue;
		}

		// forward transform(s): Z(n,k) = sum_p G(n,p) B(p,k)
		const int nblk = (ns + 3) / 4;
		const int nprod = (STEP == 2 ? 2 : 1) * C * spc * nblk;
		for (int it = tid; it < nprod; it += blockDim.x) {
			int r = it;
			const int k = r % spc; r /= spc;
			const int nb = r % nblk; r /= nblk;
			const int c = r % C; r /= C;
			const float *in = (r == 0 ? Gn : Gb) + c * spc * nsp;
			float *out = (r == 0 ? Zn : Zb) + c * spc * nsp;
			product4(in, Bt, out, spc, nsp, k, nb * 4);
		}
		__syncthreads();

		// Haar, shrinkage, inverse Haar per (channel, coefficient)
		int kept = 0;
		for (int it = tid; it < C * spc; it += blockDim.x) {
			const int k = it % spc;
			kept += shrink_dispatch<STEP>(ns, Zn + it * nsp, Zb + it * nsp, Gb + it * ns, k, bs2, is2, oinv,
			                              sigma2, bm2, Gb + it);
		}
		if (STEP == 1 && kept) atomicAdd(&s_kept, kept);
		__syncthreads();

		// inverse transform Ghat(n,p) = sum_k Z(n,k) Binv[k*spc + p] into Gn,
		// while one lane forms the group weight
		if (tid < 32) {
			if (tid == 0) {
				if (oinv) {
					// float sum of the coefficients' shares in (c, k) order
					float v = 0.f;
					for (int i = 0; i < C * spc; i++) v = __fadd_rn(v, Gb[i]);
					s_w = STEP == 1 ? __fdiv_rn(__fdiv_rn(1.f, sigma2), v) : (float)(1.0 / (double)sigma2 / (double)v);
				} else if (STEP == 1) {
					s_w = __fdiv_rn(__fdiv_rn(1.f, sigma2), (float)s_kept);
				} else {
					float v = 0.f;   // sum of w^2 in the reference's (c, k, n) order
					for (int i = 0; i < C * spc * ns; i++) v = __fadd_rn(v, Gb[i]);
					s_w = (float)(1.0 / (double)sigma2 / (double)v);
				}
			}
		} else {
			const int ninv = C * spc * nblk;
			for (int it = tid - 32; it < ninv; it += blockDim.x - 32) {
				int r = it;
				const int p = r % spc; r /= spc;
				const int nb = r % nblk; r /= nblk;
				const int c = r;
				product4(Zn + c * spc * nsp, Bi, Gn + c * spc * nsp, spc, nsp, p, nb * 4);
			}
		}
		__syncthreads();

		// aggregation terms (w * window[p]) * ghat (nldct.cpp:2296-2297, 2385-2386)
		const float w = s_w;
		for (int it = tid; it < ns * per; it += blockDim.x) {
			const int n = it / per, r = it % per;
			const int p = r % spc;
			vals[(slot0 + n) * per + r] = __fmul_rn(__fmul_rn(w, wn[p]), Gn[r * nsp + n]);
		}
		if (tid < ns) wslot[slot0 + tid] = w;
		if (tid == 0) { wgroup[g] = w; eq[g] = 0; }
	}
}

// Groups whose members are all equal keep the aggregation weights left by the
// previous processed groups of their tile (the reference's aggreWeights vector
// is not rewritten, nldct.cpp:1998, 2234): member n takes the weight of the
// latest earlier group with more than n members, or 1 if there is none
// (its initial value, nldct.cpp:754, 824).
__global__ void fixup_equal_kernel(const Tile *__restrict__ tiles, int ntiles, StepParams sp,
                                   const float *__restrict__ win, long long g_begin, long long g_end,
                                   const uint8_t *__restrict__ nsimp, const uint8_t *__restrict__ alive,
                                   const uint8_t *__restrict__ eq, const float *__restrict__ wgroup,
                                   float *__restrict__ vals, float *__restrict__ wslot)
{
	const int per = sp.C * sp.spc;
	for (long long g = g_begin + blockIdx.x * (long long)blockDim.x + threadIdx.x; g < g_end;
	     g += (long long)gridDim.x * blockDim.x) {
		if (!alive[g] || !eq[g]) continue;
		const Tile T = tiles[tile_of(tiles, ntiles, g)];
		const int ns = nsimp[g];
		const long long slot0 = (g - g_begin) * sp.np;
		for (int n = 0; n < ns; n++) {
			float w = 1.f;
			for (long long q = g - 1; q >= T.g0; q--)
				if (alive[q] && !eq[q] && nsimp[q] > n) { w = wgroup[q]; break; }
			wslot[slot0 + n] = w;
			float *v = vals + (slot0 + n) * per;
			for (int r = 0; r < per; r++) v[r] = __fmul_rn(__fmul_rn(w, win[r % sp.spc]), v[r]);
		}
	}
}

}  // namespace

size_t filter_smem_bytes(const StepParams &sp)
{
	const int nsp = ((sp.np + 3) / 4) * 4 + 4;
	const size_t tile_f = (size_t)sp.C * sp.spc * nsp;
	const size_t bsz = ((size_t)sp.spc * sp.spc + 3) / 4 * 4;
	return sizeof(float) * (2 * bsz + ((sp.spc + 3) / 4) * 4 + 4 * tile_f);
}

namespace {

template <int STEP, int PX, int PT, int CC>
cudaError_t launch_exact(int blocks, size_t smem, cudaStream_t st, const Image &noisy, const Image &basic,
                         const Tile *tiles, int ntiles, const StepParams &sp, const float *basis, const float *binv,
                         const float *win, long long g_begin, long long g_end, const uint8_t *nsimp,
                         const uint32_t *idx, const uint8_t *alive, float *vals, float *wslot, float *wgroup,
                         uint8_t *eq)
{
	auto kern = filter_exact_kernel<STEP, PX, PT, CC>;
	cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
	if (e != cudaSuccess) return e;
	kern<<<blocks, kFilterThreads, smem, st>>>(noisy, basic, tiles, ntiles, sp, basis, binv, win, g_begin, g_end,
	                                          nsimp, idx, alive, vals, wslot, wgroup, eq);
	return cudaGetLastError();
}

#define FILTER_ARGS                                                                                   \
	blocks, smem, st, noisy, basic, tiles, ntiles, sp, basis, binv, win, g_begin, g_end, nsimp, idx, alive, \
	    vals, wslot, wgroup, eq

}  // namespace

cudaError_t launch_filter(const Image &noisy, const Image &basic, const Tile *tiles, int ntiles,
                          const StepParams &sp, const float *basis, const float *binv,
                          const float *win, long long g_begin, long long g_end,
                          const uint8_t *nsimp, const uint32_t *idx, const uint8_t *alive,
                          float *vals, float *wslot, float *wgroup, uint8_t *eq, int nsm,
                          cudaStream_t st)
{
	if (g_end <= g_begin) return cudaSuccess;
	const size_t smem = filter_smem_bytes(sp);
	const long long n = g_end - g_begin;
	const int blocks = (int)(n < (long long)nsm * 8 ? n : (long long)nsm * 8);
	cudaError_t e;
	if (sp.C == 1 && sp.px == 4 && sp.pt == 4)
		e = sp.step1 ? launch_exact<1, 4, 4, 1>(FILTER_ARGS) : launch_exact<2, 4, 4, 1>(FILTER_ARGS);
	else if (sp.C == 1 && sp.px == 8 && sp.pt == 1)
		e = sp.step1 ? launch_exact<1, 8, 1, 1>(FILTER_ARGS) : launch_exact<2, 8, 1, 1>(FILTER_ARGS);
	else
		e = sp.step1 ? launch_exact<1, 0, 0, 0>(FILTER_ARGS) : launch_exact<2, 0, 0, 0>(FILTER_ARGS);
	if (e != cudaSuccess) return e;
	e = cudaGetLastError();
	if (e != cudaSuccess) return e;
	const int fb = (int)((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096);
	fixup_equal_kernel<<<fb, 256, 0, st>>>(tiles, ntiles, sp, win, g_begin, g_end, nsimp, alive, eq,
	                                       wgroup, vals, wslot);
	return cudaGetLastError();
}

}  // namespace bm4dof
