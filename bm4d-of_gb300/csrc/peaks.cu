// peaks.cu -- measured FP32 rate of the exact search's instruction mix, the
// denominator of that kernel's roofline.
//
// The exact distance (nldct.cpp:1261-1274) is one rounded subtract, multiply
// and add per patch element, no FMA.  The search issues them as one packed
// subtract and one packed multiply per two elements (sub/mul.rn.f32x2) and
// two scalar adds (search_common.cuh, sqdiff2); the GPU's nominal FP32 rate
// (one operation per lane and clock) says nothing about how fast that mix
// issues.  fp32_mix_kernel runs the same mix from registers only, with eight
// independent chains per thread and 64 warps per SM, and counts 3 operations
// per element, the unit of the search's algorithmic work.
#include <cuda_runtime.h>
#include <cstdint>

#include "../../include/bm4dof.h"
#include "internal.hpp"
#include "search_common.cuh"

namespace bm4dof {

namespace {

constexpr int kChains = 8;
constexpr int kMixThreads = 256;

__global__ void __launch_bounds__(kMixThreads) fp32_mix_kernel(float *out, int iters, float seed)
{
	float acc[kChains], ref[kChains];
#pragma unroll
	for (int j = 0; j < kChains; j++) {
		acc[j] = seed * (float)(threadIdx.x + j);
		ref[j] = seed + (float)j;
	}
	for (int i = 0; i < iters; i++) {
#pragma unroll
		for (int j = 0; j < kChains; j++) {
			// two elements: (ref - acc)^2 and (ref + 1 - acc)^2, added in order
			float m0, m1;
			sqdiff2(ref[j], ref[j] + 1.f, acc[j], acc[j], m0, m1);
			acc[j] = __fadd_rn(__fadd_rn(acc[j], m0), m1);
		}
	}
	float s = 0.f;
#pragma unroll
	for (int j = 0; j < kChains; j++) s += acc[j];
	if (s == 1.2345f) out[blockIdx.x] = s;   // keeps the chains live, never true in practice
}

}  // namespace

}  // namespace bm4dof

using namespace bm4dof;

extern "C" bm4dof_status bm4dof_fp32_mix_rate(int device, float *tops, float *ms)
{
	clear_error();
	if (!tops) {
		set_error("bm4dof_fp32_mix_rate: null argument");
		return BM4DOF_ERR_ARGUMENT;
	}
	cudaError_t e = cudaSetDevice(device);
	int nsm = 0;
	if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device);
	cudaStream_t st = nullptr;
	cudaEvent_t a = nullptr, b = nullptr;
	float *out = nullptr;
	if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
	if (e == cudaSuccess) e = cudaEventCreate(&a);
	if (e == cudaSuccess) e = cudaEventCreate(&b);
	if (e == cudaSuccess) e = cudaMalloc(&out, sizeof(float) * 8 * (size_t)nsm);
	const int blocks = 8 * nsm, iters = 4096;
	float t = 0.f;
	if (e == cudaSuccess) {
		fp32_mix_kernel<<<blocks, kMixThreads, 0, st>>>(out, iters, 1e-3f);   // warm-up
		cudaEventRecord(a, st);
		for (int r = 0; r < 4; r++) fp32_mix_kernel<<<blocks, kMixThreads, 0, st>>>(out, iters, 1e-3f);
		cudaEventRecord(b, st);
		e = cudaEventSynchronize(b);
		if (e == cudaSuccess) e = cudaEventElapsedTime(&t, a, b);
		if (e == cudaSuccess) e = cudaGetLastError();
	}
	if (out) cudaFree(out);
	if (a) cudaEventDestroy(a);
	if (b) cudaEventDestroy(b);
	if (st) cudaStreamDestroy(st);
	if (e != cudaSuccess) {
		set_error(std::string("bm4dof_fp32_mix_rate: ") + cudaGetErrorString(e));
		return BM4DOF_ERR_CUDA;
	}
	// per chain and iteration: two elements, 3 operations each
	const double ops = 4.0 * blocks * (double)kMixThreads * iters * kChains * 6.0;
	*tops = (float)(ops / (t * 1e-3) / 1e12);
	if (ms) *ms = t / 4.f;
	return BM4DOF_OK;
}
