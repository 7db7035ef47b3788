// learned.cu -- the group filter of the learned form (no step-1 pass).
//
// Each group (found on the noisy video with the step-2 geometry) is taken to
// the 3-D transform domain: the patch transform Z = G.B per member, then the
// orthonormal Haar transform along the members, as the reference's step 2
// does (src/core/nldct.cpp:2015-2174).  Where the reference's step 2 takes
// its Wiener gains w = y^2 / (y^2 + (beta2 sigma)^2) from the basic estimate
// y, the learned form takes the gains of the member-mean row (Haar
// coefficient 0) of every patch coefficient k from the gain network, whose
// inputs are the log-variances of the 64 coefficients across the members and
// sigma/255.  The other Haar rows take the Wiener gains of their own pilot,
// hard-thresholded at (beta1 sigma)^2 by the reference's step-1 rule
// (nldct.cpp:1901-1908).  The group weight is 1/(sigma^2 * sum of squared
// gains), the step-2 weight (nldct.cpp:2167).
//
// Fallback: when the residual variance of a filtered group (noisy minus
// estimate, over its members and pixels) exceeds kappa*sigma^2 the estimate
// removed signal, and the group is filtered again by the two-step shrinkage:
// a hard-thresholded pilot of its own coefficients, then the empirical Wiener
// gains of that pilot (the step-1 then step-2 rules on the same group).
//
// Three kernels share the per-group body:
//   MODE_FEATURES  gains-network inputs of every group of a chunk (bf16 rows)
//   MODE_APPLY     shrinkage, inverse transforms, aggregation terms
//   MODE_SAMPLES   training pairs: inputs from the noisy group, targets = the
//                  step-2 Wiener gains of the mean row computed from the
//                  basic estimate of the same members
// Four groups are filtered at once per CTA, 64 threads each (one thread per
// transform coefficient / patch element).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "common.cuh"
#include "internal.hpp"

namespace bm4dof {

namespace {

constexpr int kSub = 64;                // threads per group
constexpr int kGroupsPerCta = 4;
constexpr int kSpc = 64;

__device__ __forceinline__ void sub_sync(int id)
{
	asm volatile("bar.sync %0, %1;\n" ::"r"(id), "r"(kSub) : "memory");
}

template <int NS>
__device__ __forceinline__ void haar_fwd(float (&z)[NS])
{
	const float is2 = 0.70710678118654752f;
#pragma unroll
	for (int s = 2, h = 1; s <= NS; s *= 2, h *= 2)
#pragma unroll
		for (int n = 0; n < NS; n += s) {
			const float a = z[n], b = z[n + h];
			z[n] = (a + b) * is2;
			z[n + h] = (a - b) * is2;
		}
}

template <int NS>
__device__ __forceinline__ void haar_inv(float (&z)[NS])
{
	const float is2 = 0.70710678118654752f;
#pragma unroll
	for (int s = NS, h = NS / 2; s >= 2; s /= 2, h /= 2)
#pragma unroll
		for (int n = 0; n < NS; n += s) {
			const float a = z[n], b = z[n + h];
			z[n] = (a + b) * is2;
			z[n + h] = (a - b) * is2;
		}
}

// z[m] = sum_p G[m][p] * Bs[p][k]
template <int NS>
__device__ __forceinline__ void forward_col(const float *G, const float *Bs, int k, float (&z)[NS])
{
#pragma unroll
	for (int m = 0; m < NS; m++) z[m] = 0.f;
#pragma unroll 4
	for (int p = 0; p < kSpc; p += 4) {
		const float b0 = Bs[p * kSpc + k], b1 = Bs[(p + 1) * kSpc + k];
		const float b2 = Bs[(p + 2) * kSpc + k], b3 = Bs[(p + 3) * kSpc + k];
#pragma unroll
		for (int m = 0; m < NS; m++) {
			const float4 v = *reinterpret_cast<const float4 *>(G + m * kSpc + p);
			z[m] = fmaf(v.x, b0, z[m]);
			z[m] = fmaf(v.y, b1, z[m]);
			z[m] = fmaf(v.z, b2, z[m]);
			z[m] = fmaf(v.w, b3, z[m]);
		}
	}
}

// out[m] = sum_k Z[m][k] * Bi[k][p]
template <int NS>
__device__ __forceinline__ void inverse_px(const float *Z, const float *Bi, int p, float (&o)[NS])
{
#pragma unroll
	for (int m = 0; m < NS; m++) o[m] = 0.f;
#pragma unroll 4
	for (int k = 0; k < kSpc; k += 4) {
		const float b0 = Bi[k * kSpc + p], b1 = Bi[(k + 1) * kSpc + p];
		const float b2 = Bi[(k + 2) * kSpc + p], b3 = Bi[(k + 3) * kSpc + p];
#pragma unroll
		for (int m = 0; m < NS; m++) {
			const float4 v = *reinterpret_cast<const float4 *>(Z + m * kSpc + k);
			o[m] = fmaf(v.x, b0, o[m]);
			o[m] = fmaf(v.y, b1, o[m]);
			o[m] = fmaf(v.z, b2, o[m]);
			o[m] = fmaf(v.w, b3, o[m]);
		}
	}
}

__device__ __forceinline__ float sub_sum(float v, float *red, int bar)
{
	// sum over the 64 threads of a group (two warps)
#pragma unroll
	for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
	const int k = threadIdx.x & (kSub - 1);
	if ((k & 31) == 0) red[k >> 5] = v;
	sub_sync(bar);
	const float s = red[0] + red[1];
	sub_sync(bar);
	return s;
}

__device__ __forceinline__ float feature_of(float var, float sigma2)
{
	return logf(fmaxf(var, 1e-6f * sigma2) / sigma2);
}

template <int NS, int MODE>
__device__ void group_body(const LearnedArgs &a, const StepParams &sp, long long g, float *Gs, float *Zs,
                           const float *Bs, const float *Bi, const float *win, float *red, int bar)
{
	const int k = threadIdx.x & (kSub - 1);   // coefficient (transform) / pixel (inverse)
	const float sigma2 = sp.sigma * sp.sigma;
	const long long r = g - a.ga;             // chunk-relative row
	float z[NS];
	forward_col<NS>(Gs, Bs, k, z);

	if (MODE == kLearnedFeatures || MODE == kLearnedSamples) {
		float var = 0.f;
#pragma unroll
		for (int m = 0; m < NS; m++) var = fmaf(z[m], z[m], var);
		const float f = feature_of(var / (float)NS, sigma2);
		if (MODE == kLearnedFeatures) {
			__nv_bfloat16 *row = a.feat + r * kMlpInPad;
			row[k] = __float2bfloat16_rn(f);
			if (k == 0) row[kSpc] = __float2bfloat16_rn(sp.sigma / 255.f);
			if (k < kMlpInPad - kSpc - 1) row[kSpc + 1 + k] = __float2bfloat16_rn(0.f);
		} else {
			float *row = a.sfeat + g * kMlpIn;
			row[k] = f;
			if (k == 0) row[kSpc] = sp.sigma / 255.f;
			// target: the step-2 Wiener gain of the mean row, from the basic estimate
			float y[NS];
			forward_col<NS>(Zs, Bs, k, y);
			haar_fwd<NS>(y);
			const float bs = sp.beta * sp.sigma;
			const float yy = y[0] * y[0];
			a.starget[g * kSpc + k] = yy / (yy + bs * bs);
			if (k == 0) a.svalid[g] = 1;
		}
		return;
	}

	// ---- MODE_APPLY --------------------------------------------------------
	float zh[NS];
#pragma unroll
	for (int m = 0; m < NS; m++) zh[m] = z[m];
	haar_fwd<NS>(zh);
	const float bs2 = (sp.beta * sp.sigma) * (sp.beta * sp.sigma);      // Wiener
	const float bt2 = (sp.beta1 * sp.sigma) * (sp.beta1 * sp.sigma);    // hard threshold
	float gain;
	if (a.gains) {
		gain = a.gains[r * kSpc + k];
	} else {
		// without the network: empirical Wiener gain of the noisy mean row
		const float dd = zh[0] * zh[0];
		gain = dd > bs2 ? (dd - bs2) / dd : 0.f;
	}
	float w2 = gain * gain;
	z[0] = zh[0] * gain;
	// other rows: Wiener gains of their hard-thresholded pilot
#pragma unroll
	for (int m = 1; m < NS; m++) {
		const float pilot = zh[m] * zh[m] > bt2 ? zh[m] : 0.f;
		const float pp = pilot * pilot;
		const float w = pp / (pp + bs2);
		z[m] = zh[m] * w;
		w2 = fmaf(w, w, w2);
	}
	haar_inv<NS>(z);
#pragma unroll
	for (int m = 0; m < NS; m++) Zs[m * kSpc + k] = z[m];
	sub_sync(bar);
	float est[NS];
	inverse_px<NS>(Zs, Bi, k, est);
	float res = 0.f;
#pragma unroll
	for (int m = 0; m < NS; m++) {
		const float d = Gs[m * kSpc + k] - est[m];
		res = fmaf(d, d, res);
	}
	const float rsum = sub_sum(res, red, bar);
	float w2sum = sub_sum(w2, red, bar);
	if (rsum > a.kappa * sigma2 * (float)(NS * kSpc)) {
		// fallback: two-step shrinkage of the group's own coefficients
		float wv = 0.f;
#pragma unroll
		for (int m = 0; m < NS; m++) {
			const float pilot = (zh[m] * zh[m] > bt2 || (k == 0 && m == 0)) ? zh[m] : 0.f;
			const float pp = pilot * pilot;
			const float w = pp / (pp + bs2);
			z[m] = zh[m] * w;
			wv = fmaf(w, w, wv);
		}
		haar_inv<NS>(z);
#pragma unroll
		for (int m = 0; m < NS; m++) Zs[m * kSpc + k] = z[m];
		sub_sync(bar);
		inverse_px<NS>(Zs, Bi, k, est);
		w2sum = sub_sum(wv, red, bar);
		if (k == 0) atomicAdd(a.nfallback, 1u);
	}
	const float wgt = 1.f / (sigma2 * fmaxf(w2sum, 1e-3f));
	const long long slot0 = r * sp.np;
	const float wp = wgt * win[k];
#pragma unroll
	for (int m = 0; m < NS; m++)
		reinterpret_cast<float2 *>(a.vals)[(slot0 + m) * kSpc + k] = make_float2(wp * est[m], wp);
}

template <int MODE>
__global__ void __launch_bounds__(kSub *kGroupsPerCta, 2)
learned_kernel(LearnedArgs a, StepParams sp)
{
	extern __shared__ __align__(16) float lsm[];
	float *Bs = lsm;                    // Bs[p][k] = basis[k][p]
	float *Bi = Bs + kSpc * kSpc;       // Bi[k][p] = binv[k][p]
	float *win = Bi + kSpc * kSpc;
	const int sub = threadIdx.x / kSub, k = threadIdx.x % kSub;
	float *Gs = win + kSpc + sub * 2 * sp.np * kSpc;
	float *Zs = Gs + sp.np * kSpc;
	__shared__ int s_mx[kGroupsPerCta][kMaxNp], s_my[kGroupsPerCta][kMaxNp], s_mt[kGroupsPerCta][kMaxNp];
	__shared__ float s_red[kGroupsPerCta][2];
	for (int i = threadIdx.x; i < kSpc * kSpc; i += blockDim.x) {
		const int kk = i / kSpc, p = i % kSpc;
		Bs[p * kSpc + kk] = a.basis[i];
		Bi[i] = a.binv[i];
	}
	for (int i = threadIdx.x; i < kSpc; i += blockDim.x) win[i] = a.win[i];
	__syncthreads();
	const int bar = 1 + sub;
	const int px = sp.px;
	for (long long g = a.ga + (long long)blockIdx.x * kGroupsPerCta + sub; g < a.gb;
	     g += (long long)gridDim.x * kGroupsPerCta) {
		if (!a.alive[g]) continue;
		const int ns = a.nsimp[g];
		const Tile T = a.tiles[tile_of(a.tiles, a.ntiles, g)];
		if (k < ns) {
			const uint32_t lin = a.idx[g * sp.np + k];
			const uint32_t whl = (uint32_t)T.w * T.h;
			s_mt[sub][k] = (int)(lin / whl);
			s_my[sub][k] = (int)((lin % whl) / T.w);
			s_mx[sub][k] = (int)(lin % T.w);
		}
		sub_sync(bar);
		const int ht = k / (px * px), hy = (k / px) % px, hx = k % px;
		for (int m = 0; m < ns; m++) {
			const size_t ad = a.noisy.at(T.ox + s_mx[sub][m] + hx, T.oy + s_my[sub][m] + hy, s_mt[sub][m] + ht, 0);
			Gs[m * kSpc + k] = __ldg(a.noisy.p + ad);
			if (MODE == kLearnedSamples) Zs[m * kSpc + k] = __ldg(a.basic.p + ad);
		}
		sub_sync(bar);
		switch (ns) {
		case 1: group_body<1, MODE>(a, sp, g, Gs, Zs, Bs, Bi, win, s_red[sub], bar); break;
		case 2: group_body<2, MODE>(a, sp, g, Gs, Zs, Bs, Bi, win, s_red[sub], bar); break;
		case 4: group_body<4, MODE>(a, sp, g, Gs, Zs, Bs, Bi, win, s_red[sub], bar); break;
		case 8: group_body<8, MODE>(a, sp, g, Gs, Zs, Bs, Bi, win, s_red[sub], bar); break;
		case 16: group_body<16, MODE>(a, sp, g, Gs, Zs, Bs, Bi, win, s_red[sub], bar); break;
		default: group_body<32, MODE>(a, sp, g, Gs, Zs, Bs, Bi, win, s_red[sub], bar); break;
		}
		sub_sync(bar);
	}
}

// ---------------------------------------------------------------------------
// Tensor-core form of the features and apply kernels (groups of at most 16
// members): one warp per group; the patch transform and its inverse are
// m16n8k16 BF16 products with FP32 accumulation (members x 64 coefficients, K =
// 64), the Haar transform and the shrinkage stay in FP32 on the coefficients,
// one or two columns per lane.
// ---------------------------------------------------------------------------
constexpr int kTcWarps = 8;
constexpr int kBP = 72;    // bf16 row pitch of the 64-wide tiles
constexpr int kZP = 17;    // fp32 pitch of the [coefficient][member] tile

struct TcWarp {
	__nv_bfloat16 A[16][kBP];   // members x pixels, then members x shrunk coefficients
	float G[16][64];            // the group's pixels (FP32)
	float Z[64][kZP];           // coefficients x members, then pixels x members (estimate)
};

__device__ __forceinline__ void mma_bf16_tc(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                            uint32_t b0, uint32_t b1)
{
	asm volatile(
	    "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
	    "{%0,%1,%2,%3};\n"
	    : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
	    : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// OUT[row m][col n] = sum_k A[m][k] * Bt[n][k]; result rows scattered into
// Z[n][m] (m < 16, n < 64)
__device__ __forceinline__ void tc_product(const __nv_bfloat16 (*A)[kBP], const __nv_bfloat16 *Bt, float (*Z)[kZP])
{
	const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
	float acc[8][4];
#pragma unroll
	for (int j = 0; j < 8; j++) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
#pragma unroll
	for (int k0 = 0; k0 < 64; k0 += 16) {
		const uint32_t a0 = *reinterpret_cast<const uint32_t *>(&A[g][k0 + 2 * t]);
		const uint32_t a1 = *reinterpret_cast<const uint32_t *>(&A[g + 8][k0 + 2 * t]);
		const uint32_t a2 = *reinterpret_cast<const uint32_t *>(&A[g][k0 + 8 + 2 * t]);
		const uint32_t a3 = *reinterpret_cast<const uint32_t *>(&A[g + 8][k0 + 8 + 2 * t]);
#pragma unroll
		for (int j = 0; j < 8; j++) {
			const __nv_bfloat16 *b = Bt + (j * 8 + g) * kBP + k0 + 2 * t;
			mma_bf16_tc(acc[j], a0, a1, a2, a3, *reinterpret_cast<const uint32_t *>(b),
			            *reinterpret_cast<const uint32_t *>(b + 8));
		}
	}
#pragma unroll
	for (int j = 0; j < 8; j++) {
		const int n = j * 8 + 2 * t;
		Z[n][g] = acc[j][0];
		Z[n + 1][g] = acc[j][1];
		Z[n][g + 8] = acc[j][2];
		Z[n + 1][g + 8] = acc[j][3];
	}
}

template <int NS>
__device__ __forceinline__ void tc_column(const LearnedArgs &a, const StepParams &sp, long long r, int k,
                                          TcWarp &W, float &w2, float (&zh)[NS], bool fallback)
{
	const float bs2 = (sp.beta * sp.sigma) * (sp.beta * sp.sigma);
	const float bt2 = (sp.beta1 * sp.sigma) * (sp.beta1 * sp.sigma);
	float z[NS];
	if (!fallback) {
#pragma unroll
		for (int m = 0; m < NS; m++) zh[m] = W.Z[k][m];
		haar_fwd<NS>(zh);
		float gain;
		if (a.gains) {
			gain = a.gains[r * kSpc + k];
		} else {
			const float dd = zh[0] * zh[0];
			gain = dd > bs2 ? (dd - bs2) / dd : 0.f;
		}
		w2 = gain * gain;
		z[0] = zh[0] * gain;
#pragma unroll
		for (int m = 1; m < NS; m++) {
			const float pilot = zh[m] * zh[m] > bt2 ? zh[m] : 0.f;
			const float pp = pilot * pilot;
			const float w = pp / (pp + bs2);
			z[m] = zh[m] * w;
			w2 = fmaf(w, w, w2);
		}
	} else {
		w2 = 0.f;
#pragma unroll
		for (int m = 0; m < NS; m++) {
			const float pilot = (zh[m] * zh[m] > bt2 || (k == 0 && m == 0)) ? zh[m] : 0.f;
			const float pp = pilot * pilot;
			const float w = pp / (pp + bs2);
			z[m] = zh[m] * w;
			w2 = fmaf(w, w, w2);
		}
	}
	haar_inv<NS>(z);
#pragma unroll
	for (int m = 0; m < NS; m++) W.A[m][k] = __float2bfloat16_rn(z[m]);
}

template <int NS, int MODE>
__device__ void tc_group(const LearnedArgs &a, const StepParams &sp, long long g, TcWarp &W,
                         const __nv_bfloat16 *Bs, const __nv_bfloat16 *Bit, const float *win)
{
	const int lane = threadIdx.x & 31;
	const float sigma2 = sp.sigma * sp.sigma;
	const long long r = g - a.ga;
	tc_product(W.A, Bs, W.Z);
	__syncwarp();
	if (MODE == kLearnedFeatures) {
		__nv_bfloat16 *row = a.feat + r * kMlpInPad;
#pragma unroll
		for (int h = 0; h < 2; h++) {
			const int k = lane + 32 * h;
			float var = 0.f;
#pragma unroll
			for (int m = 0; m < NS; m++) var = fmaf(W.Z[k][m], W.Z[k][m], var);
			row[k] = __float2bfloat16_rn(feature_of(var / (float)NS, sigma2));
		}
		if (lane == 0) row[kSpc] = __float2bfloat16_rn(sp.sigma / 255.f);
		if (lane < kMlpInPad - kSpc - 1) row[kSpc + 1 + lane] = __float2bfloat16_rn(0.f);
		return;
	}
	float zh0[NS], zh1[NS], w2a, w2b;
	tc_column<NS>(a, sp, r, lane, W, w2a, zh0, false);
	tc_column<NS>(a, sp, r, lane + 32, W, w2b, zh1, false);
	__syncwarp();
	tc_product(W.A, Bit, W.Z);   // estimate, [pixel][member]
	__syncwarp();
	float res = 0.f;
#pragma unroll
	for (int h = 0; h < 2; h++) {
		const int p = lane + 32 * h;
#pragma unroll
		for (int m = 0; m < NS; m++) {
			const float d = W.G[m][p] - W.Z[p][m];
			res = fmaf(d, d, res);
		}
	}
	float w2 = w2a + w2b;
#pragma unroll
	for (int o = 16; o > 0; o >>= 1) {
		res += __shfl_xor_sync(0xffffffffu, res, o);
		w2 += __shfl_xor_sync(0xffffffffu, w2, o);
	}
	if (res > a.kappa * sigma2 * (float)(NS * kSpc)) {
		// fallback: two-step shrinkage of the group's own coefficients
		__syncwarp();
		tc_column<NS>(a, sp, r, lane, W, w2a, zh0, true);
		tc_column<NS>(a, sp, r, lane + 32, W, w2b, zh1, true);
		__syncwarp();
		tc_product(W.A, Bit, W.Z);
		__syncwarp();
		w2 = w2a + w2b;
#pragma unroll
		for (int o = 16; o > 0; o >>= 1) w2 += __shfl_xor_sync(0xffffffffu, w2, o);
		if (lane == 0) atomicAdd(a.nfallback, 1u);
	}
	const float wgt = 1.f / (sigma2 * fmaxf(w2, 1e-3f));
	const long long slot0 = r * sp.np;
#pragma unroll
	for (int h = 0; h < 2; h++) {
		const int p = lane + 32 * h;
		const float wp = wgt * win[p];
#pragma unroll
		for (int m = 0; m < NS; m++)
			reinterpret_cast<float2 *>(a.vals)[(slot0 + m) * kSpc + p] = make_float2(wp * W.Z[p][m], wp);
	}
}

template <int MODE>
__global__ void __launch_bounds__(32 * kTcWarps, 2)
learned_tc_kernel(LearnedArgs a, StepParams sp)
{
	extern __shared__ __align__(16) unsigned char tsm[];
	__nv_bfloat16 *Bs = reinterpret_cast<__nv_bfloat16 *>(tsm);    // [k][p] = basis[k][p]
	__nv_bfloat16 *Bit = Bs + 64 * kBP;                             // [p][k] = binv[k][p]
	float *win = reinterpret_cast<float *>(Bit + 64 * kBP);
	TcWarp *Ws = reinterpret_cast<TcWarp *>(win + 64);
	__shared__ int s_m[kTcWarps][3][16];
	for (int i = threadIdx.x; i < 64 * 64; i += blockDim.x) {
		const int k = i / 64, p = i % 64;
		Bs[k * kBP + p] = __float2bfloat16_rn(a.basis[i]);
		Bit[p * kBP + k] = __float2bfloat16_rn(a.binv[i]);
	}
	for (int i = threadIdx.x; i < 64; i += blockDim.x) win[i] = a.win[i];
	__syncthreads();
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	TcWarp &W = Ws[warp];
	const int px = sp.px;
	for (long long g = a.ga + (long long)blockIdx.x * kTcWarps + warp; g < a.gb;
	     g += (long long)gridDim.x * kTcWarps) {
		if (!a.alive[g]) continue;
		const int ns = a.nsimp[g];
		const Tile T = a.tiles[tile_of(a.tiles, a.ntiles, g)];
		if (lane < ns) {
			const uint32_t lin = a.idx[g * sp.np + lane];
			const uint32_t whl = (uint32_t)T.w * T.h;
			s_m[warp][2][lane] = (int)(lin / whl);
			s_m[warp][1][lane] = (int)((lin % whl) / T.w);
			s_m[warp][0][lane] = (int)(lin % T.w);
		}
		__syncwarp();
		for (int m = 0; m < 16; m++)
#pragma unroll
			for (int h = 0; h < 2; h++) {
				const int p = lane + 32 * h;
				float v = 0.f;
				if (m < ns) {
					const int ht = p / (px * px), hy = (p / px) % px, hx = p % px;
					v = __ldg(a.noisy.p + a.noisy.at(T.ox + s_m[warp][0][m] + hx, T.oy + s_m[warp][1][m] + hy,
					                                   s_m[warp][2][m] + ht, 0));
				}
				W.G[m][p] = v;
				W.A[m][p] = __float2bfloat16_rn(v);
			}
		__syncwarp();
		switch (ns) {
		case 1: tc_group<1, MODE>(a, sp, g, W, Bs, Bit, win); break;
		case 2: tc_group<2, MODE>(a, sp, g, W, Bs, Bit, win); break;
		case 4: tc_group<4, MODE>(a, sp, g, W, Bs, Bit, win); break;
		case 8: tc_group<8, MODE>(a, sp, g, W, Bs, Bit, win); break;
		default: tc_group<16, MODE>(a, sp, g, W, Bs, Bit, win); break;
		}
		__syncwarp();
	}
}

template <int MODE>
cudaError_t launch_tc(const LearnedArgs &a, const StepParams &sp, int nsm, cudaStream_t st)
{
	const size_t smem = sizeof(__nv_bfloat16) * 2 * 64 * kBP + sizeof(float) * 64 + sizeof(TcWarp) * kTcWarps;
	cudaError_t e = cudaFuncSetAttribute(learned_tc_kernel<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
	if (e != cudaSuccess) return e;
	int per_sm = 0;
	e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, learned_tc_kernel<MODE>, 32 * kTcWarps, smem);
	if (e != cudaSuccess) return e;
	const long long need = (a.gb - a.ga + kTcWarps - 1) / kTcWarps;
	const long long nb = std::min<long long>(need, (long long)nsm * std::max(per_sm, 1) * 4);
	learned_tc_kernel<MODE><<<(int)std::max<long long>(nb, 1), 32 * kTcWarps, smem, st>>>(a, sp);
	return cudaGetLastError();
}

template <int MODE>
cudaError_t launch_mode(const LearnedArgs &a, const StepParams &sp, int nsm, cudaStream_t st)
{
	const size_t smem = sizeof(float) * (2 * kSpc * kSpc + kSpc + (size_t)kGroupsPerCta * 2 * sp.np * kSpc);
	cudaError_t e = cudaFuncSetAttribute(learned_kernel<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
	if (e != cudaSuccess) return e;
	int per_sm = 0;
	e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, learned_kernel<MODE>, kSub * kGroupsPerCta, smem);
	if (e != cudaSuccess) return e;
	const long long need = (a.gb - a.ga + kGroupsPerCta - 1) / kGroupsPerCta;
	const long long nb = std::min<long long>(need, (long long)nsm * std::max(per_sm, 1) * 4);
	learned_kernel<MODE><<<(int)std::max<long long>(nb, 1), kSub * kGroupsPerCta, smem, st>>>(a, sp);
	return cudaGetLastError();
}

}  // namespace

bool learned_supported(const StepParams &sp)
{
	// 64-element patches (the network's width), one channel, power-of-two
	// member counts up to 32
	return sp.spc == kSpc && sp.C == 1 && sp.np <= kMaxNp;
}

cudaError_t launch_learned(int mode, const LearnedArgs &a, const StepParams &sp, int nsm, cudaStream_t st)
{
	if (a.gb <= a.ga) return cudaSuccess;
	// groups of up to 16 members: BF16 tensor-core transforms
	const bool tc = sp.np <= 16;
	switch (mode) {
	case kLearnedFeatures: return tc ? launch_tc<kLearnedFeatures>(a, sp, nsm, st) : launch_mode<kLearnedFeatures>(a, sp, nsm, st);
	case kLearnedApply: return tc ? launch_tc<kLearnedApply>(a, sp, nsm, st) : launch_mode<kLearnedApply>(a, sp, nsm, st);
	default: return launch_mode<kLearnedSamples>(a, sp, nsm, st);
	}
}

}  // namespace bm4dof
