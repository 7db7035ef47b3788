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
	for (int m = 0; m < NS; m++) a.vals[(slot0 + m) * kSpc + k] = wp * est[m];
	if (k < NS) a.wslot[slot0 + k] = wgt;
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
	switch (mode) {
	case kLearnedFeatures: return launch_mode<kLearnedFeatures>(a, sp, nsm, st);
	case kLearnedApply: return launch_mode<kLearnedApply>(a, sp, nsm, st);
	default: return launch_mode<kLearnedSamples>(a, sp, nsm, st);
	}
}

}  // namespace bm4dof
