// mlp.cu -- the gain network of the learned form and its training.
//
// Network: 65 -> 256 -> 256 -> 64, GELU (erf form) after the two hidden
// layers, sigmoid on the output.  Weights and activations are BF16 with FP32
// accumulation on the tensor cores (mma.sync m16n8k16); FP32 master weights,
// biases, pre-activations, gradients and AdamW moments.
//
// Layouts (all row-major):
//   public parameter blob (host, float): W1[65][256] b1[256] W2[256][256]
//     b2[256] W3[256][64] b3[64]  -- W[in][out]
//   device master (float): the same with W1 padded to [80][256] (rows 65..79
//     stay zero: their inputs are zero, so their gradients are zero)
//   device working copy (bf16): Wt1[256][80] Wt2[256][256] Wt3[64][256] --
//     transposed so that the two k-adjacent elements of an MMA B fragment are
//     one 32-bit load
//   features: bf16 [rows][80] (65 used), gains: float [rows][64]
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/bm4dof.h"
#include "internal.hpp"

namespace bm4dof {

namespace {

using bf16 = __nv_bfloat16;

constexpr int kIn = 65, kInP = 80, kHid = 256, kOut = 64;
constexpr int kRowsPerCta = 64;          // 4 warps x 16 rows
constexpr int kActStride = kHid + 8;     // bf16 row pitch: conflict-free fragment loads

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1)
{
	asm volatile(
	    "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
	    "{%0,%1,%2,%3};\n"
	    : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
	    : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ float gelu(float x)
{
	return 0.5f * x * (1.f + erff(x * 0.70710678118654752f));
}

__device__ __forceinline__ float gelu_grad(float x)
{
	// d/dx x*Phi(x) = Phi(x) + x*phi(x)
	const float cdf = 0.5f * (1.f + erff(x * 0.70710678118654752f));
	const float pdf = 0.39894228040143268f * expf(-0.5f * x * x);
	return cdf + x * pdf;
}

__device__ __forceinline__ uint32_t ld_u32(const bf16 *p) { return *reinterpret_cast<const uint32_t *>(p); }

// One dense layer for the 16 rows [wr, wr+16) of a warp: out = act(in . W + b)
// with in a bf16 shared tile of K columns and Wt[N][K] in global memory.
// ACT 0: GELU into the bf16 shared tile `out` (and, when training, the
// pre-activations to P and the activations to H in global memory);
// ACT 1: sigmoid into the float rows of `gout`.
template <int K, int N, int ACT, bool TRAIN>
__device__ __forceinline__ void dense(const bf16 *in, bf16 *out, const bf16 *__restrict__ Wt,
                                      const float *__restrict__ bias, int wr, long long row0, long long n,
                                      float *gout, float *P, bf16 *H)
{
	const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll 1
	for (int nc = 0; nc < N; nc += 64) {
		float acc[8][4];
#pragma unroll
		for (int j = 0; j < 8; j++) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
#pragma unroll 4
		for (int k0 = 0; k0 < K; k0 += 16) {
			uint32_t a[4];
			a[0] = ld_u32(in + (wr + g) * kActStride + k0 + 2 * t);
			a[1] = ld_u32(in + (wr + g + 8) * kActStride + k0 + 2 * t);
			a[2] = ld_u32(in + (wr + g) * kActStride + k0 + 8 + 2 * t);
			a[3] = ld_u32(in + (wr + g + 8) * kActStride + k0 + 8 + 2 * t);
#pragma unroll
			for (int j = 0; j < 8; j++) {
				const bf16 *wp = Wt + (size_t)(nc + j * 8 + g) * K + k0 + 2 * t;
				mma_bf16(acc[j], a, __ldg(reinterpret_cast<const unsigned *>(wp)),
				         __ldg(reinterpret_cast<const unsigned *>(wp + 8)));
			}
		}
#pragma unroll
		for (int j = 0; j < 8; j++) {
			const int c = nc + j * 8 + 2 * t;
			const float b0 = __ldg(bias + c), b1 = __ldg(bias + c + 1);
#pragma unroll
			for (int h = 0; h < 2; h++) {
				const int r = wr + g + 8 * h;
				const long long row = row0 + r;
				const float v0 = acc[j][2 * h] + b0, v1 = acc[j][2 * h + 1] + b1;
				if (ACT == 0) {
					const bf16 o0 = __float2bfloat16_rn(gelu(v0)), o1 = __float2bfloat16_rn(gelu(v1));
					out[r * kActStride + c] = o0;
					out[r * kActStride + c + 1] = o1;
					if (TRAIN && row < n) {
						P[row * N + c] = v0;
						P[row * N + c + 1] = v1;
						H[row * N + c] = o0;
						H[row * N + c + 1] = o1;
					}
				} else if (row < n) {
					gout[row * N + c] = 1.f / (1.f + expf(-v0));
					gout[row * N + c + 1] = 1.f / (1.f + expf(-v1));
				}
			}
		}
	}
}

// Forward pass over n feature rows.  Each warp owns 16 rows of the CTA's two
// activation tiles, so the layers need only warp-level synchronisation.
template <bool TRAIN>
__global__ void __launch_bounds__(128)
mlp_forward_kernel(const bf16 *__restrict__ X, long long n, MlpWeights w, float *__restrict__ out,
                   float *P1, bf16 *H1, float *P2, bf16 *H2)
{
	extern __shared__ __align__(16) unsigned char msm[];
	bf16 *A = reinterpret_cast<bf16 *>(msm);
	bf16 *B = A + kRowsPerCta * kActStride;
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	const int wr = warp * 16;
	for (long long r0 = (long long)blockIdx.x * kRowsPerCta; r0 < n; r0 += (long long)gridDim.x * kRowsPerCta) {
		// features of the warp's rows: 16 rows x 80 bf16 = 160 16-byte pieces
		for (int i = lane; i < 16 * (kInP / 8); i += 32) {
			const int rr = i / (kInP / 8), c8 = i % (kInP / 8);
			const long long row = r0 + wr + rr;
			uint4 v = make_uint4(0, 0, 0, 0);
			if (row < n) v = __ldg(reinterpret_cast<const uint4 *>(X + row * kInP) + c8);
			*reinterpret_cast<uint4 *>(B + (wr + rr) * kActStride + c8 * 8) = v;
		}
		__syncwarp();
		dense<kInP, kHid, 0, TRAIN>(B, A, w.wt1, w.b1, wr, r0, n, nullptr, P1, H1);
		__syncwarp();
		dense<kHid, kHid, 0, TRAIN>(A, B, w.wt2, w.b2, wr, r0, n, nullptr, P2, H2);
		__syncwarp();
		dense<kHid, kOut, 1, TRAIN>(B, nullptr, w.wt3, w.b3, wr, r0, n, out, nullptr, nullptr);
		__syncwarp();
	}
}

constexpr size_t kForwardSmem = sizeof(bf16) * 2 * kRowsPerCta * kActStride;

// C[m][n] = sum_k A(m,k) B(k,n) with A(m,k) = a[m*am + k*ak], B(k,n) = b[k*bk + n*bn],
// bf16 operands, float result (ldc).  64 x 64 tiles, k in steps of 32.
__global__ void __launch_bounds__(128)
gemm_bf16_kernel(const bf16 *__restrict__ a, long long am, long long ak, const bf16 *__restrict__ b,
                 long long bk, long long bn, float *__restrict__ c, int ldc, int M, int N, long long K)
{
	constexpr int S = 40;   // bf16 pitch of the k-major shared tiles
	__shared__ __align__(16) bf16 As[64 * S];
	__shared__ __align__(16) bf16 Bs[64 * S];
	const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, g = lane >> 2, t = lane & 3;
	const int m0 = blockIdx.y * 64, n0 = blockIdx.x * 64;
	float acc[8][4];
#pragma unroll
	for (int j = 0; j < 8; j++) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
	const bf16 zero = __float2bfloat16_rn(0.f);
	for (long long k0 = 0; k0 < K; k0 += 32) {
		__syncthreads();
		for (int i = tid; i < 64 * 32; i += 128) {
			// consecutive threads along whichever index has unit stride
			int r, kk;
			if (ak == 1) { r = i / 32; kk = i % 32; } else { r = i % 64; kk = i / 64; }
			const long long m = m0 + r, k = k0 + kk;
			As[r * S + kk] = (m < M && k < K) ? a[m * am + k * ak] : zero;
			int q, kb;
			if (bk == 1) { q = i / 32; kb = i % 32; } else { q = i % 64; kb = i / 64; }
			const long long nn = n0 + q, k2 = k0 + kb;
			Bs[q * S + kb] = (nn < N && k2 < K) ? b[k2 * bk + nn * bn] : zero;
		}
		__syncthreads();
#pragma unroll
		for (int ks = 0; ks < 32; ks += 16) {
			uint32_t af[4];
			af[0] = ld_u32(As + (warp * 16 + g) * S + ks + 2 * t);
			af[1] = ld_u32(As + (warp * 16 + g + 8) * S + ks + 2 * t);
			af[2] = ld_u32(As + (warp * 16 + g) * S + ks + 8 + 2 * t);
			af[3] = ld_u32(As + (warp * 16 + g + 8) * S + ks + 8 + 2 * t);
#pragma unroll
			for (int j = 0; j < 8; j++)
				mma_bf16(acc[j], af, ld_u32(Bs + (j * 8 + g) * S + ks + 2 * t),
				         ld_u32(Bs + (j * 8 + g) * S + ks + 8 + 2 * t));
		}
	}
#pragma unroll
	for (int j = 0; j < 8; j++)
#pragma unroll
		for (int h = 0; h < 2; h++) {
			const int m = m0 + warp * 16 + g + 8 * h;
			const int nn = n0 + j * 8 + 2 * t;
			if (m >= M) continue;
			if (nn < N) c[(long long)m * ldc + nn] = acc[j][2 * h];
			if (nn + 1 < N) c[(long long)m * ldc + nn + 1] = acc[j][2 * h + 1];
		}
}

// float features [n][65] -> bf16 [n][80] (zero padded)
__global__ void pack_features_kernel(const float *__restrict__ f, long long n, bf16 *__restrict__ X)
{
	for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n * kInP;
	     i += (long long)gridDim.x * blockDim.x) {
		const long long r = i / kInP;
		const int c = (int)(i % kInP);
		X[i] = __float2bfloat16_rn(c < kIn ? f[r * kIn + c] : 0.f);
	}
}

// master (float, W[in][out]) -> transposed bf16 working copy
__global__ void pack_weights_kernel(const float *__restrict__ m, bf16 *__restrict__ wt)
{
	const int n1 = kHid * kInP, n2 = kHid * kHid, n3 = kOut * kHid;
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n1 + n2 + n3; i += gridDim.x * blockDim.x) {
		float v;
		if (i < n1) {
			const int o = i / kInP, k = i % kInP;
			v = m[kMlpOffW1 + k * kHid + o];
		} else if (i < n1 + n2) {
			const int j = i - n1, o = j / kHid, k = j % kHid;
			v = m[kMlpOffW2 + k * kHid + o];
		} else {
			const int j = i - n1 - n2, o = j / kHid, k = j % kHid;
			v = m[kMlpOffW3 + k * kOut + o];
		}
		wt[i] = __float2bfloat16_rn(v);
	}
}

// dL/dz3 of the mean squared error through the sigmoid, and per-block loss sums
__global__ void out_grad_kernel(const float *__restrict__ y, const float *__restrict__ tgt, long long n,
                                float *__restrict__ dP, bf16 *__restrict__ dPb, float *__restrict__ partial)
{
	__shared__ float red[256];
	const float scale = 2.f / (float)(n * kOut);
	float s = 0.f;
	for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n * kOut;
	     i += (long long)gridDim.x * blockDim.x) {
		const float e = y[i] - tgt[i];
		s += e * e;
		const float d = scale * e * y[i] * (1.f - y[i]);
		dP[i] = d;
		dPb[i] = __float2bfloat16_rn(d);
	}
	red[threadIdx.x] = s;
	__syncthreads();
	for (int h = blockDim.x / 2; h > 0; h >>= 1) {
		if ((int)threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
		__syncthreads();
	}
	if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

// dP = dH * GELU'(P)
__global__ void gelu_back_kernel(const float *__restrict__ dH, const float *__restrict__ P, long long cnt,
                                 float *__restrict__ dP, bf16 *__restrict__ dPb)
{
	for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < cnt;
	     i += (long long)gridDim.x * blockDim.x) {
		const float d = dH[i] * gelu_grad(P[i]);
		dP[i] = d;
		dPb[i] = __float2bfloat16_rn(d);
	}
}

// bias gradient: column sums of dP [n][N] (one thread per column, fixed order)
__global__ void colsum_kernel(const float *__restrict__ dP, long long n, int N, float *__restrict__ out)
{
	const int c = blockIdx.x * blockDim.x + threadIdx.x;
	if (c >= N) return;
	float s = 0.f;
	for (long long r = 0; r < n; r++) s += dP[r * N + c];
	out[c] = s;
}

__global__ void sum_kernel(const float *__restrict__ part, int n, float *__restrict__ out)
{
	if (threadIdx.x == 0 && blockIdx.x == 0) {
		double s = 0.0;
		for (int i = 0; i < n; i++) s += part[i];
		*out = (float)s;
	}
}

// AdamW on the master weights; weight decay on the matrices, not the biases
__global__ void adamw_kernel(float *__restrict__ p, const float *__restrict__ gr, float *__restrict__ m,
                             float *__restrict__ v, int n, float lr, float b1, float b2, float eps, float wd,
                             float c1, float c2)
{
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
		const bool bias = (i >= kMlpOffB1 && i < kMlpOffW2) || (i >= kMlpOffB2 && i < kMlpOffW3) || i >= kMlpOffB3;
		const float g = gr[i];
		const float mi = b1 * m[i] + (1.f - b1) * g;
		const float vi = b2 * v[i] + (1.f - b2) * g * g;
		m[i] = mi;
		v[i] = vi;
		float q = p[i];
		if (!bias) q -= lr * wd * q;
		q -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
		p[i] = q;
	}
}

int blocks_for(long long n, int threads, int cap = 4096)
{
	long long b = (n + threads - 1) / threads;
	return (int)std::max<long long>(1, std::min<long long>(b, cap));
}

}  // namespace

cudaError_t launch_mlp_forward(const uint16_t *X, long long n, const MlpWeights &w, float *out, int nsm,
                               cudaStream_t st)
{
	if (n <= 0) return cudaSuccess;
	cudaError_t e = cudaFuncSetAttribute(mlp_forward_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
	                                     (int)kForwardSmem);
	if (e != cudaSuccess) return e;
	const long long need = (n + kRowsPerCta - 1) / kRowsPerCta;
	const int nb = (int)std::min<long long>(need, (long long)nsm * 3);
	mlp_forward_kernel<false><<<nb, 128, kForwardSmem, st>>>(reinterpret_cast<const bf16 *>(X), n, w, out,
	                                                         nullptr, nullptr, nullptr, nullptr);
	return cudaGetLastError();
}

cudaError_t launch_pack_weights(const float *master, uint16_t *wt, cudaStream_t st)
{
	pack_weights_kernel<<<256, 256, 0, st>>>(master, reinterpret_cast<bf16 *>(wt));
	return cudaGetLastError();
}

MlpWeights mlp_weights(const uint16_t *wt, const float *master)
{
	MlpWeights w;
	const bf16 *b = reinterpret_cast<const bf16 *>(wt);
	w.wt1 = b;
	w.wt2 = b + kHid * kInP;
	w.wt3 = b + kHid * kInP + kHid * kHid;
	w.b1 = master + kMlpOffB1;
	w.b2 = master + kMlpOffB2;
	w.b3 = master + kMlpOffB3;
	return w;
}

void mlp_public_to_master(const float *pub, float *master)
{
	std::memset(master, 0, sizeof(float) * kMlpMasterSize);
	for (int k = 0; k < kIn; k++)
		for (int o = 0; o < kHid; o++) master[kMlpOffW1 + k * kHid + o] = pub[k * kHid + o];
	std::memcpy(master + kMlpOffB1, pub + kIn * kHid, sizeof(float) * (kMlpMasterSize - kMlpOffB1));
}

void mlp_master_to_public(const float *master, float *pub)
{
	for (int k = 0; k < kIn; k++)
		for (int o = 0; o < kHid; o++) pub[k * kHid + o] = master[kMlpOffW1 + k * kHid + o];
	std::memcpy(pub + kIn * kHid, master + kMlpOffB1, sizeof(float) * (kMlpMasterSize - kMlpOffB1));
}

}  // namespace bm4dof

using namespace bm4dof;

// ---------------------------------------------------------------------------
// trainer

struct bm4dof_trainer {
	int device = 0, nsm = 0;
	unsigned batch = 0;
	long long step = 0;
	cudaStream_t st = nullptr;
	float *master = nullptr, *grad = nullptr, *m1 = nullptr, *m2 = nullptr;
	uint16_t *wt = nullptr;
	// activations of one batch
	bf16 *X = nullptr, *H1 = nullptr, *H2 = nullptr, *dPb = nullptr;
	float *P1 = nullptr, *P2 = nullptr, *Y = nullptr, *dP = nullptr, *dH = nullptr, *part = nullptr,
	      *loss = nullptr;
};

namespace {

#define TCK(expr)                                                                            \
	do {                                                                                     \
		cudaError_t e_ = (expr);                                                             \
		if (e_ != cudaSuccess) {                                                             \
			set_error(std::string("CUDA error: ") + cudaGetErrorString(e_) + " at " #expr);  \
			return e_ == cudaErrorMemoryAllocation ? BM4DOF_ERR_NO_MEMORY : BM4DOF_ERR_CUDA; \
		}                                                                                    \
	} while (0)

constexpr int kPartBlocks = 512;

void free_trainer(bm4dof_trainer *t)
{
	void *ps[] = {t->master, t->grad, t->m1, t->m2, t->wt, t->X, t->H1, t->H2, t->dPb,
	              t->P1, t->P2, t->Y, t->dP, t->dH, t->part, t->loss};
	for (void *p : ps)
		if (p) cudaFree(p);
	if (t->st) cudaStreamDestroy(t->st);
	delete t;
}

// forward + backward of n rows (n <= batch): gradients into t->grad, loss into t->loss
bm4dof_status forward_backward(bm4dof_trainer *t, const float *feat, const float *target, long long n)
{
	cudaStream_t st = t->st;
	const MlpWeights w = mlp_weights(t->wt, t->master);
	pack_features_kernel<<<blocks_for(n * kInP, 256), 256, 0, st>>>(feat, n, t->X);
	TCK(cudaFuncSetAttribute(mlp_forward_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
	                         (int)kForwardSmem));
	const int nb = (int)std::min<long long>((n + kRowsPerCta - 1) / kRowsPerCta, (long long)t->nsm * 3);
	mlp_forward_kernel<true><<<nb, 128, kForwardSmem, st>>>(t->X, n, w, t->Y, t->P1, t->H1, t->P2, t->H2);
	out_grad_kernel<<<kPartBlocks, 256, 0, st>>>(t->Y, target, n, t->dP, t->dPb, t->part);
	sum_kernel<<<1, 32, 0, st>>>(t->part, kPartBlocks, t->loss);
	const bf16 *wt = reinterpret_cast<const bf16 *>(t->wt);
	const bf16 *wt2 = wt + kHid * kInP, *wt3 = wt2 + kHid * kHid;
	auto gemm = [&](const bf16 *a, long long am, long long ak, const bf16 *b, long long bk, long long bn,
	                float *c, int ldc, int M, int N, long long K) {
		dim3 grid((N + 63) / 64, (M + 63) / 64);
		gemm_bf16_kernel<<<grid, 128, 0, st>>>(a, am, ak, b, bk, bn, c, ldc, M, N, K);
	};
	// layer 3: dW3[i][j] = sum_b H2[b][i] dP3[b][j]; db3; dH2 = dP3 . W3^T
	gemm(t->H2, 1, kHid, t->dPb, kOut, 1, t->grad + kMlpOffW3, kOut, kHid, kOut, n);
	colsum_kernel<<<1, kOut, 0, st>>>(t->dP, n, kOut, t->grad + kMlpOffB3);
	gemm(t->dPb, kOut, 1, wt3, kHid, 1, t->dH, kHid, (int)n, kHid, kOut);
	gelu_back_kernel<<<blocks_for(n * kHid, 256), 256, 0, st>>>(t->dH, t->P2, n * kHid, t->dP, t->dPb);
	// layer 2
	gemm(t->H1, 1, kHid, t->dPb, kHid, 1, t->grad + kMlpOffW2, kHid, kHid, kHid, n);
	colsum_kernel<<<1, kHid, 0, st>>>(t->dP, n, kHid, t->grad + kMlpOffB2);
	gemm(t->dPb, kHid, 1, wt2, kHid, 1, t->dH, kHid, (int)n, kHid, kHid);
	gelu_back_kernel<<<blocks_for(n * kHid, 256), 256, 0, st>>>(t->dH, t->P1, n * kHid, t->dP, t->dPb);
	// layer 1 (rows 65..79 of dW1 come out zero: their inputs are zero)
	gemm(t->X, 1, kInP, t->dPb, kHid, 1, t->grad + kMlpOffW1, kHid, kInP, kHid, n);
	colsum_kernel<<<1, kHid, 0, st>>>(t->dP, n, kHid, t->grad + kMlpOffB1);
	TCK(cudaGetLastError());
	return BM4DOF_OK;
}

bool trainer_ok(bm4dof_trainer *t, const void *feat, const void *target, unsigned n)
{
	if (!t || !feat || !target || n == 0 || n > t->batch) {
		set_error("bm4dof_trainer: bad argument (null pointer or n outside [1, batch])");
		return false;
	}
	return true;
}

}  // namespace

extern "C" {

bm4dof_status bm4dof_trainer_create(bm4dof_trainer **out, int device, unsigned batch, unsigned seed)
{
	clear_error();
	if (!out || batch == 0) { set_error("bm4dof_trainer_create: bad argument"); return BM4DOF_ERR_ARGUMENT; }
	*out = nullptr;
	int ndev = 0;
	if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
		cudaGetLastError();
		set_error("bm4dof_trainer_create: no CUDA device");
		return BM4DOF_ERR_NO_DEVICE;
	}
	if (device < 0 || device >= ndev) { set_error("bm4dof_trainer_create: bad device"); return BM4DOF_ERR_ARGUMENT; }
	TCK(cudaSetDevice(device));
	bm4dof_trainer *t = new bm4dof_trainer();
	t->device = device;
	t->batch = batch;
	cudaDeviceGetAttribute(&t->nsm, cudaDevAttrMultiProcessorCount, device);
	const size_t B = batch;
	bool ok = cudaStreamCreateWithFlags(&t->st, cudaStreamNonBlocking) == cudaSuccess &&
	          cudaMalloc(&t->master, sizeof(float) * kMlpMasterSize) == cudaSuccess &&
	          cudaMalloc(&t->grad, sizeof(float) * kMlpMasterSize) == cudaSuccess &&
	          cudaMalloc(&t->m1, sizeof(float) * kMlpMasterSize) == cudaSuccess &&
	          cudaMalloc(&t->m2, sizeof(float) * kMlpMasterSize) == cudaSuccess &&
	          cudaMalloc(&t->wt, sizeof(uint16_t) * kMlpWtSize) == cudaSuccess &&
	          cudaMalloc(&t->X, sizeof(bf16) * B * kInP) == cudaSuccess &&
	          cudaMalloc(&t->H1, sizeof(bf16) * B * kHid) == cudaSuccess &&
	          cudaMalloc(&t->H2, sizeof(bf16) * B * kHid) == cudaSuccess &&
	          cudaMalloc(&t->dPb, sizeof(bf16) * B * kHid) == cudaSuccess &&
	          cudaMalloc(&t->P1, sizeof(float) * B * kHid) == cudaSuccess &&
	          cudaMalloc(&t->P2, sizeof(float) * B * kHid) == cudaSuccess &&
	          cudaMalloc(&t->Y, sizeof(float) * B * kOut) == cudaSuccess &&
	          cudaMalloc(&t->dP, sizeof(float) * B * kHid) == cudaSuccess &&
	          cudaMalloc(&t->dH, sizeof(float) * B * kHid) == cudaSuccess &&
	          cudaMalloc(&t->part, sizeof(float) * kPartBlocks) == cudaSuccess &&
	          cudaMalloc(&t->loss, sizeof(float)) == cudaSuccess;
	if (!ok) {
		cudaGetLastError();
		free_trainer(t);
		set_error("bm4dof_trainer_create: device allocation failed");
		return BM4DOF_ERR_NO_MEMORY;
	}
	// He-style uniform initialisation from a fixed LCG (host), zero biases
	std::vector<float> pub(kMlpPublicSize, 0.f);
	uint64_t s = 0x9E3779B97F4A7C15ull ^ seed;
	auto uni = [&s]() {
		s = s * 6364136223846793005ull + 1442695040888963407ull;
		return (float)((s >> 40) * (1.0 / 16777216.0)) * 2.f - 1.f;
	};
	const int fan[3] = {kIn, kHid, kHid}, outs[3] = {kHid, kHid, kOut};
	size_t o = 0;
	for (int l = 0; l < 3; l++) {
		const float a = std::sqrt(3.f / (float)fan[l]);
		for (int i = 0; i < fan[l] * outs[l]; i++) pub[o + i] = a * uni();
		o += (size_t)fan[l] * outs[l] + outs[l];
	}
	std::vector<float> master(kMlpMasterSize);
	mlp_public_to_master(pub.data(), master.data());
	TCK(cudaMemcpyAsync(t->master, master.data(), sizeof(float) * kMlpMasterSize, cudaMemcpyHostToDevice, t->st));
	TCK(cudaMemsetAsync(t->m1, 0, sizeof(float) * kMlpMasterSize, t->st));
	TCK(cudaMemsetAsync(t->m2, 0, sizeof(float) * kMlpMasterSize, t->st));
	TCK(cudaMemsetAsync(t->grad, 0, sizeof(float) * kMlpMasterSize, t->st));
	TCK(launch_pack_weights(t->master, t->wt, t->st));
	TCK(cudaStreamSynchronize(t->st));
	*out = t;
	return BM4DOF_OK;
}

bm4dof_status bm4dof_trainer_get_stream(bm4dof_trainer *t, void **stream)
{
	clear_error();
	if (!t || !stream) { set_error("bm4dof_trainer_get_stream: null argument"); return BM4DOF_ERR_ARGUMENT; }
	*stream = static_cast<void *>(t->st);
	return BM4DOF_OK;
}

void bm4dof_trainer_destroy(bm4dof_trainer *t)
{
	if (!t) return;
	cudaSetDevice(t->device);
	cudaStreamSynchronize(t->st);
	free_trainer(t);
}

bm4dof_status bm4dof_trainer_params(bm4dof_trainer *t, float *params, size_t n, int set)
{
	clear_error();
	if (!t || !params || n != (size_t)kMlpPublicSize) {
		set_error("bm4dof_trainer_params: bad argument (the blob holds " + std::to_string(kMlpPublicSize) + " floats)");
		return BM4DOF_ERR_ARGUMENT;
	}
	TCK(cudaSetDevice(t->device));
	std::vector<float> master(kMlpMasterSize);
	if (set) {
		mlp_public_to_master(params, master.data());
		TCK(cudaMemcpyAsync(t->master, master.data(), sizeof(float) * kMlpMasterSize, cudaMemcpyHostToDevice, t->st));
		TCK(launch_pack_weights(t->master, t->wt, t->st));
		TCK(cudaStreamSynchronize(t->st));
	} else {
		TCK(cudaMemcpyAsync(master.data(), t->master, sizeof(float) * kMlpMasterSize, cudaMemcpyDeviceToHost, t->st));
		TCK(cudaStreamSynchronize(t->st));
		mlp_master_to_public(master.data(), params);
	}
	return BM4DOF_OK;
}

bm4dof_status bm4dof_trainer_state(bm4dof_trainer *t, float *moment1, float *moment2, size_t n,
                                   unsigned long long *steps, int set)
{
	clear_error();
	if (!t || !moment1 || !moment2 || !steps || n != (size_t)kMlpPublicSize) {
		set_error("bm4dof_trainer_state: bad argument (each moment holds " + std::to_string(kMlpPublicSize) +
		          " floats)");
		return BM4DOF_ERR_ARGUMENT;
	}
	TCK(cudaSetDevice(t->device));
	std::vector<float> m1(kMlpMasterSize), m2(kMlpMasterSize);
	if (set) {
		// the padded inputs of W1 never receive a gradient: their moments stay 0
		mlp_public_to_master(moment1, m1.data());
		mlp_public_to_master(moment2, m2.data());
		TCK(cudaMemcpyAsync(t->m1, m1.data(), sizeof(float) * kMlpMasterSize, cudaMemcpyHostToDevice, t->st));
		TCK(cudaMemcpyAsync(t->m2, m2.data(), sizeof(float) * kMlpMasterSize, cudaMemcpyHostToDevice, t->st));
		TCK(cudaStreamSynchronize(t->st));
		t->step = (long long)*steps;
	} else {
		TCK(cudaMemcpyAsync(m1.data(), t->m1, sizeof(float) * kMlpMasterSize, cudaMemcpyDeviceToHost, t->st));
		TCK(cudaMemcpyAsync(m2.data(), t->m2, sizeof(float) * kMlpMasterSize, cudaMemcpyDeviceToHost, t->st));
		TCK(cudaStreamSynchronize(t->st));
		mlp_master_to_public(m1.data(), moment1);
		mlp_master_to_public(m2.data(), moment2);
		*steps = (unsigned long long)t->step;
	}
	return BM4DOF_OK;
}

bm4dof_status bm4dof_trainer_grad(bm4dof_trainer *t, const float *feat, const float *target, unsigned n,
                                  float *grads, float *loss)
{
	clear_error();
	if (!trainer_ok(t, feat, target, n)) return BM4DOF_ERR_ARGUMENT;
	TCK(cudaSetDevice(t->device));
	bm4dof_status s = forward_backward(t, feat, target, n);
	if (s != BM4DOF_OK) return s;
	std::vector<float> g(kMlpMasterSize);
	float l = 0.f;
	TCK(cudaMemcpyAsync(g.data(), t->grad, sizeof(float) * kMlpMasterSize, cudaMemcpyDeviceToHost, t->st));
	TCK(cudaMemcpyAsync(&l, t->loss, sizeof(float), cudaMemcpyDeviceToHost, t->st));
	TCK(cudaStreamSynchronize(t->st));
	if (grads) mlp_master_to_public(g.data(), grads);
	if (loss) *loss = l / (float)((size_t)n * kOut);
	return BM4DOF_OK;
}

bm4dof_status bm4dof_trainer_step(bm4dof_trainer *t, const float *feat, const float *target, unsigned n,
                                  float lr, float weight_decay, float *loss)
{
	clear_error();
	if (!trainer_ok(t, feat, target, n)) return BM4DOF_ERR_ARGUMENT;
	TCK(cudaSetDevice(t->device));
	bm4dof_status s = forward_backward(t, feat, target, n);
	if (s != BM4DOF_OK) return s;
	t->step++;
	const float b1 = 0.9f, b2 = 0.999f;
	const float c1 = 1.f - std::pow(b1, (float)t->step), c2 = 1.f - std::pow(b2, (float)t->step);
	adamw_kernel<<<blocks_for(kMlpMasterSize, 256), 256, 0, t->st>>>(t->master, t->grad, t->m1, t->m2,
	                                                                   kMlpMasterSize, lr, b1, b2, 1e-8f,
	                                                                   weight_decay, c1, c2);
	TCK(launch_pack_weights(t->master, t->wt, t->st));
	if (loss) {
		float l = 0.f;
		TCK(cudaMemcpyAsync(&l, t->loss, sizeof(float), cudaMemcpyDeviceToHost, t->st));
		TCK(cudaStreamSynchronize(t->st));
		*loss = l / (float)((size_t)n * kOut);
	}
	return BM4DOF_OK;
}

bm4dof_status bm4dof_trainer_predict(bm4dof_trainer *t, const float *feat, unsigned n, float *gains)
{
	clear_error();
	if (!t || !feat || !gains || n == 0 || n > t->batch) {
		set_error("bm4dof_trainer_predict: bad argument");
		return BM4DOF_ERR_ARGUMENT;
	}
	TCK(cudaSetDevice(t->device));
	pack_features_kernel<<<blocks_for((long long)n * kInP, 256), 256, 0, t->st>>>(feat, n, t->X);
	TCK(launch_mlp_forward(reinterpret_cast<const uint16_t *>(t->X), n, mlp_weights(t->wt, t->master), gains,
	                       t->nsm, t->st));
	TCK(cudaStreamSynchronize(t->st));
	return BM4DOF_OK;
}

}  // extern "C"
