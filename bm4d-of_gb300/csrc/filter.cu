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
#include <algorithm>
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
                    float *__restrict__ wgroup, uint8_t *__restrict__ eq)
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
		const int ts = term_stride(C);
		if (ns > 1 && !any) {
			// unweighted: the weights are set later (fixup_equal_kernel)
			for (int it = tid; it < ns * per; it += blockDim.x) {
				const int n = it / per, r = it % per;
				const int c = r / spc, p = r % spc;
				vals[((slot0 + n) * spc + p) * ts + c] = Gn[r * nsp + n];
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
			const int c = r / spc, p = r % spc;
			vals[((slot0 + n) * spc + p) * ts + c] = __fmul_rn(__fmul_rn(w, wn[p]), Gn[r * nsp + n]);
		}
		for (int it = tid; it < ns * spc; it += blockDim.x) {
			const int n = it / spc, p = it % spc;
			vals[((slot0 + n) * spc + p) * ts + C] = __fmul_rn(w, wn[p]);
		}
		if (tid == 0) { wgroup[g] = w; eq[g] = 0; }
	}
}

// ---------------------------------------------------------------------------
// The same filter for one-channel groups of 64-element patches, four groups
// per CTA (64 threads each, sharing the bases in shared memory).  Each thread
// of a product forms a 4-member x 4-coefficient block, so that two vector
// loads feed 16 multiply-add pairs; every output is still accumulated over the
// inner index in increasing order with separately rounded products and sums,
// so the results are the generic kernel's, bit for bit.
// ---------------------------------------------------------------------------
constexpr int kQuadSub = 64, kQuadGroups = 4;

__device__ __forceinline__ void quad_sync(int id)
{
	asm volatile("bar.sync %0, %1;\n" ::"r"(id), "r"(kQuadSub) : "memory");
}

// (x0 * y0, x1 * y1), each rounded as __fmul_rn (mul.rn.f32x2)
__device__ __forceinline__ void mul2(float x0, float x1, float y0, float y1, float &p0, float &p1)
{
	unsigned long long x, y, z;
	asm("mov.b64 %0, {%1, %2};" : "=l"(x) : "f"(x0), "f"(x1));
	asm("mov.b64 %0, {%1, %2};" : "=l"(y) : "f"(y0), "f"(y1));
	asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(z) : "l"(x), "l"(y));
	asm("mov.b64 {%0, %1}, %2;" : "=f"(p0), "=f"(p1) : "l"(z));
}

// out[(q0 + c) * nsp + n0 + m] = sum_r in[r * nsp + n0 + m] * M[r * 64 + q0 + c]
__device__ __forceinline__ void product4x4(const float *in, const float *M, float *out, int nsp, int q0, int n0)
{
	float a[4][4];
#pragma unroll
	for (int m = 0; m < 4; m++)
#pragma unroll
		for (int c = 0; c < 4; c++) a[m][c] = 0.f;
#pragma unroll 4
	for (int r = 0; r < 64; r++) {
		const float4 g = *reinterpret_cast<const float4 *>(in + r * nsp + n0);
		const float4 b = *reinterpret_cast<const float4 *>(M + r * 64 + q0);
		// the 16 products as 8 packed multiplies of member pairs (m, m+1) by
		// coefficient pairs taken straight and swapped; each sum still takes
		// one rounded add per term in r order (a packed multiply whose lanes
		// are added one at a time rounds exactly as the scalar pair)
		float p[4][4];
		mul2(g.x, g.y, b.x, b.y, p[0][0], p[1][1]);
		mul2(g.x, g.y, b.y, b.x, p[0][1], p[1][0]);
		mul2(g.x, g.y, b.z, b.w, p[0][2], p[1][3]);
		mul2(g.x, g.y, b.w, b.z, p[0][3], p[1][2]);
		mul2(g.z, g.w, b.x, b.y, p[2][0], p[3][1]);
		mul2(g.z, g.w, b.y, b.x, p[2][1], p[3][0]);
		mul2(g.z, g.w, b.z, b.w, p[2][2], p[3][3]);
		mul2(g.z, g.w, b.w, b.z, p[2][3], p[3][2]);
#pragma unroll
		for (int m = 0; m < 4; m++)
#pragma unroll
			for (int c = 0; c < 4; c++) a[m][c] = __fadd_rn(a[m][c], p[m][c]);
	}
#pragma unroll
	for (int c = 0; c < 4; c++)
		*reinterpret_cast<float4 *>(out + (q0 + c) * nsp + n0) = make_float4(a[0][c], a[1][c], a[2][c], a[3][c]);
}

template <int STEP, int PX, int PT>
__global__ void __launch_bounds__(kQuadSub *kQuadGroups, 2)
filter_quad_kernel(Image noisy, Image basic, const Tile *__restrict__ tiles, int ntiles, StepParams sp,
                   const float *__restrict__ basis, const float *__restrict__ binv, const float *__restrict__ win,
                   long long g_begin, long long g_end, const uint8_t *__restrict__ nsimp,
                   const uint32_t *__restrict__ idx, const uint8_t *__restrict__ alive, float *__restrict__ vals,
                   float *__restrict__ wgroup, uint8_t *__restrict__ eq)
{
	constexpr int SPC = PX * PX * PT;
	static_assert(SPC == 64, "four-group filter: 64-element patches");
	extern __shared__ __align__(16) float sm[];
	float *Bt = sm;                 // Bt[p][k] = basis[k][p]
	float *Bi = Bt + SPC * SPC;     // Bi[k][p] = binv[k][p]
	float *wn = Bi + SPC * SPC;
	const int np = sp.np, nsp = nsp_of(np), tile_f = SPC * nsp;
	const int sub = threadIdx.x / kQuadSub, t = threadIdx.x % kQuadSub;
	// three tiles per group: the noisy group's pixels are dead once it is
	// transformed, so the basic group's transform and then the estimate reuse
	// their tile
	float *Gn = wn + SPC + sub * 3 * tile_f;   // noisy group [p][n]; basic transform; estimate
	float *Zn = Gn + tile_f;                   // noisy transform [k][n]
	float *Gb = Zn + tile_f;                   // basic group; later w^2 / weight shares
	float *Zb = Gn;
	__shared__ int s_mx[kQuadGroups][kMaxNp], s_my[kQuadGroups][kMaxNp], s_mt[kQuadGroups][kMaxNp];
	__shared__ int s_flag[kQuadGroups][2];
	__shared__ float s_w[kQuadGroups];

	for (int i = threadIdx.x; i < SPC * SPC; i += blockDim.x) {
		const int k = i / SPC, p = i % SPC;
		Bt[p * SPC + k] = basis[i];
		Bi[i] = binv[i];
	}
	for (int i = threadIdx.x; i < SPC; i += blockDim.x) wn[i] = win[i];
	__syncthreads();

	const float sigma2 = __fmul_rn(sp.sigma, sp.sigma);
	const float bsig = __fmul_rn(sp.beta, sp.sigma);
	const float bs2 = __fmul_rn(bsig, bsig);
	const float bmsig = __fmul_rn(sp.beta_mean, sp.sigma);
	const float bm2 = __fmul_rn(bmsig, bmsig);
	const bool oinv = sp.order_inv != 0;
	const float is2 = (float)(1.0 / sqrt(2.0));
	const int bar = 1 + sub, lane = t & 31, w = t >> 5;
	const int ht = t / (PX * PX), hy = (t / PX) % PX, hx = t % PX;

	for (long long g = g_begin + (long long)blockIdx.x * kQuadGroups + sub; g < g_end;
	     g += (long long)gridDim.x * kQuadGroups) {
		if (!alive[g]) continue;
		const int ns = nsimp[g];
		const Tile T = tiles[tile_of(tiles, ntiles, g)];
		if (t < ns) {
			const uint32_t lin = idx[g * np + t];
			const uint32_t whl = (uint32_t)T.w * T.h;
			s_mt[sub][t] = (int)(lin / whl);
			s_my[sub][t] = (int)((lin % whl) / T.w);
			s_mx[sub][t] = (int)(lin % T.w);
		}
		quad_sync(bar);
		// gather the group, thread t holding patch element t of every member
		for (int n = 0; n < ns; n++) {
			const size_t a = noisy.at(T.ox + s_mx[sub][n] + hx, T.oy + s_my[sub][n] + hy, s_mt[sub][n] + ht, 0);
			Gn[t * nsp + n] = __ldg(noisy.p + a);
			if (STEP == 2) Gb[t * nsp + n] = __ldg(basic.p + a);
		}
		quad_sync(bar);
		const long long slot0 = (g - g_begin) * np;
		// all-equal test (nldct.cpp:1986-1999, 2222-2235), row t
		int differs = 0;
		for (int n = 1; n < ns; n++) differs |= Gn[t * nsp + n] != Gn[t * nsp];
		differs = __any_sync(0xffffffffu, differs);
		if (lane == 0) s_flag[sub][w] = differs;
		quad_sync(bar);
		if (ns > 1 && !(s_flag[sub][0] | s_flag[sub][1])) {
			for (int n = 0; n < ns; n++)
				reinterpret_cast<float2 *>(vals)[(slot0 + n) * SPC + t] = make_float2(Gn[t * nsp + n], 0.f);
			if (t == 0) eq[g] = 1;
			quad_sync(bar);
			continue;
		}
		// forward transform(s) in 4 x 4 blocks: noisy, then basic (over the
		// noisy pixels)
		const int nblk = (ns + 3) / 4;
		for (int it = t; it < nblk * 16; it += kQuadSub) product4x4(Gn, Bt, Zn, nsp, (it % 16) * 4, (it / 16) * 4);
		quad_sync(bar);
		if (STEP == 2) {
			for (int it = t; it < nblk * 16; it += kQuadSub) product4x4(Gb, Bt, Zb, nsp, (it % 16) * 4, (it / 16) * 4);
			quad_sync(bar);
		}
		// Haar, shrinkage, inverse Haar of coefficient t
		int kept = shrink_dispatch<STEP>(ns, Zn + t * nsp, Zb + t * nsp, Gb + t * ns, t, bs2, is2, oinv, sigma2, bm2,
		                                 Gb + t);
		if (STEP == 1 && !oinv) {
#pragma unroll
			for (int o = 16; o > 0; o >>= 1) kept += __shfl_xor_sync(0xffffffffu, kept, o);
			if (lane == 0) s_flag[sub][w] = kept;
		}
		quad_sync(bar);
		if (t == 0) {
			if (oinv) {
				float v = 0.f;   // float sum of the coefficients' shares in k order
				for (int i = 0; i < SPC; i++) v = __fadd_rn(v, Gb[i]);
				s_w[sub] = STEP == 1 ? __fdiv_rn(__fdiv_rn(1.f, sigma2), v) : (float)(1.0 / (double)sigma2 / (double)v);
			} else if (STEP == 1) {
				s_w[sub] = __fdiv_rn(__fdiv_rn(1.f, sigma2), (float)(s_flag[sub][0] + s_flag[sub][1]));
			} else {
				float v = 0.f;   // sum of w^2 in the reference's (k, n) order
				for (int i = 0; i < SPC * ns; i++) v = __fadd_rn(v, Gb[i]);
				s_w[sub] = (float)(1.0 / (double)sigma2 / (double)v);
			}
		}
		// inverse transform into Gn
		for (int it = t; it < nblk * 16; it += kQuadSub) product4x4(Zn, Bi, Gn, nsp, (it % 16) * 4, (it / 16) * 4);
		quad_sync(bar);
		const float wg = s_w[sub];
		const float wp = __fmul_rn(wg, wn[t]);
		for (int n = 0; n < ns; n++)
			reinterpret_cast<float2 *>(vals)[(slot0 + n) * SPC + t] = make_float2(__fmul_rn(wp, Gn[t * nsp + n]), wp);
		if (t == 0) { wgroup[g] = wg; eq[g] = 0; }
		quad_sync(bar);
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
                                   float *__restrict__ vals)
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
			const int ts = term_stride(sp.C);
			float *v = vals + (slot0 + n) * sp.spc * ts;
			for (int p = 0; p < sp.spc; p++) {
				const float wp = __fmul_rn(w, win[p]);
				for (int c = 0; c < sp.C; c++) v[p * ts + c] = __fmul_rn(wp, v[p * ts + c]);
				v[p * ts + sp.C] = wp;
			}
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
                         const uint32_t *idx, const uint8_t *alive, float *vals, float *wgroup,
                         uint8_t *eq)
{
	auto kern = filter_exact_kernel<STEP, PX, PT, CC>;
	cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
	if (e != cudaSuccess) return e;
	kern<<<blocks, kFilterThreads, smem, st>>>(noisy, basic, tiles, ntiles, sp, basis, binv, win, g_begin, g_end,
	                                          nsimp, idx, alive, vals, wgroup, eq);
	return cudaGetLastError();
}

template <int STEP, int PX, int PT>
cudaError_t launch_quad(int blocks, size_t smem, cudaStream_t st, const Image &noisy, const Image &basic,
                        const Tile *tiles, int ntiles, const StepParams &sp, const float *basis, const float *binv,
                        const float *win, long long g_begin, long long g_end, const uint8_t *nsimp,
                        const uint32_t *idx, const uint8_t *alive, float *vals, float *wgroup,
                        uint8_t *eq)
{
	auto kern = filter_quad_kernel<STEP, PX, PT>;
	cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
	if (e != cudaSuccess) return e;
	kern<<<blocks, kQuadSub * kQuadGroups, smem, st>>>(noisy, basic, tiles, ntiles, sp, basis, binv, win, g_begin,
	                                                  g_end, nsimp, idx, alive, vals, wgroup, eq);
	return cudaGetLastError();
}

#define FILTER_ARGS_NB noisy, basic, tiles, ntiles, sp, basis, binv, win, g_begin, g_end, nsimp, idx, alive, vals, \
	    wgroup, eq

#define FILTER_ARGS                                                                                   \
	blocks, smem, st, noisy, basic, tiles, ntiles, sp, basis, binv, win, g_begin, g_end, nsimp, idx, alive, \
	    vals, wgroup, eq

}  // namespace

cudaError_t launch_filter(const Image &noisy, const Image &basic, const Tile *tiles, int ntiles,
                          const StepParams &sp, const float *basis, const float *binv,
                          const float *win, long long g_begin, long long g_end,
                          const uint8_t *nsimp, const uint32_t *idx, const uint8_t *alive,
                          float *vals, float *wgroup, uint8_t *eq, int nsm,
                          cudaStream_t st)
{
	if (g_end <= g_begin) return cudaSuccess;
	const size_t smem = filter_smem_bytes(sp);
	const long long n = g_end - g_begin;
	const int blocks = (int)(n < (long long)nsm * 8 ? n : (long long)nsm * 8);
	cudaError_t e;
	if (sp.C == 1 && sp.spc == 64 && ((sp.px == 4 && sp.pt == 4) || (sp.px == 8 && sp.pt == 1))) {
		const size_t qsmem = sizeof(float) * (2 * 64 * 64 + 64 + (size_t)kQuadGroups * 3 * 64 * (((sp.np + 3) / 4) * 4 + 4));
		const long long need = (n + kQuadGroups - 1) / kQuadGroups;
		const int qb = (int)std::min<long long>(need, (long long)nsm * 2);
		if (sp.px == 4)
			e = sp.step1 ? launch_quad<1, 4, 4>(qb, qsmem, st, FILTER_ARGS_NB) : launch_quad<2, 4, 4>(qb, qsmem, st, FILTER_ARGS_NB);
		else
			e = sp.step1 ? launch_quad<1, 8, 1>(qb, qsmem, st, FILTER_ARGS_NB) : launch_quad<2, 8, 1>(qb, qsmem, st, FILTER_ARGS_NB);
	} else if (sp.C == 1 && sp.px == 4 && sp.pt == 4)
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
	                                       wgroup, vals);
	return cudaGetLastError();
}

}  // namespace bm4dof
