// search_tc.cu -- mixed-precision patch search on the Blackwell tensor cores
// (tcgen05), with a certified exact re-rank.
//
// Same candidates and the same result as VideoNLB::estimateSimilarPatchesStep1
// (src/core/nldct.cpp:1143-1348; the step-2 search of grey video compares one
// channel as well): flow-chained windows, frames in the reference's visiting
// order, the k nearest by the reference's FP32 distance, the tau rule.
//
// 1. search_tc_kernel (pre-screen).  One CTA holds 128 reference patches (a
//    16 x 8 block of grid positions of one frame of one tile) as the MMA's A
//    operand, FP16, centred at 128.  For every candidate frame it stages the
//    union of their 128 search windows (4 patch frames, FP16) in shared
//    memory, builds the candidate patches 256 at a time as the B operand and
//    lets tcgen05.mma form all 128 x 256 cross terms <p', q'> in tensor
//    memory (FP32 accumulation).  Four selection warps read them back with
//    tcgen05.ld, one reference per thread (its TMEM lane):
//        a(p, q) = |p'|^2 + |q'|^2 - 2 <p', q'>   (the rounded patches),
//    test the candidate against the thread's own window and keep the 32
//    smallest a(p, q): candidates under the current 32nd smallest wait in a
//    list of up to 32 per reference, which the warp merges into the sorted
//    kept list with bitonic networks when it fills.  Four staging warps build the
//    next chunk's operands while the selection warps work on the current
//    one (two operand buffers, two TMEM accumulators of 256 columns,
//    mbarriers between them).  Per reference it writes the 32 candidates and
//    a lower bound L on the exact distance of every candidate it dropped:
//    each of those had a(p, q) >= A32, the 32nd smallest, and
//        |p - q| >= sqrt(A32 - E) - delta,
//    delta bounding the FP16 rounding of both patches (2^-11 of their norms)
//    and E the FP32 evaluation error of the split (norm bound max |q'|^2 over
//    the block's windows).
// 2. rerank_kernel.  One warp per reference: the exact FP32 distance of the
//    32 candidates in the reference's summation order, sorted.  When the k
//    smallest are pairwise distinct, below the next one and below L, no
//    dropped candidate can be among them or tie with them, so they are
//    exactly what std::partial_sort returns; the tau rule follows.  A
//    reference whose pre-screen did not finish (a NaN, a value beyond FP16,
//    or a block whose windows do not fit the staging buffer) goes on a list
//    for the exact search (search.cu).  One that is merely not certified (a
//    tie, or L too low: near-equal candidates, as in flat regions of the
//    basic estimate) keeps the order of its re-ranked 32 by default, or goes
//    on that list too when every neighbour list must be the exact path's
//    (BM4DOF_MIXED_CERTIFIED).
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <cstdint>
#include <vector>

#include "common.cuh"
#include "internal.hpp"
#include "search_common.cuh"
#include "umma.cuh"

namespace bm4dof {

namespace {

constexpr int kRefs = 128;            // references per CTA (MMA M, TMEM lanes)
constexpr int kBX = 16, kBY = 8;      // ... as a 16 x 8 block of grid positions
constexpr int kN = 256;               // candidates per chunk (MMA N)
constexpr int kK = 64;                // patch elements (MMA K, four k-steps of 16)
constexpr int kThreads = 256;         // warps 0-3 select, warps 4-7 stage and issue
constexpr int kTop = 32;              // approximate candidates kept per reference
constexpr int kMaxWt = 16;            // candidate frames per reference on this path
constexpr int kWinHalves = 16384;     // staged window capacity (FP16 values)
constexpr int kTmemCols = 512;        // two accumulators of kN columns
constexpr uint32_t kWaitLimit = 1u << 22;   // mbarrier polls before giving up

// byte offsets of the dynamic shared memory
constexpr int kOffA = 0;                                  // 128 x 64 FP16, core-matrix layout
constexpr int kOffB = kOffA + kRefs * kK * 2;             // 2 x 256 x 64 FP16
constexpr int kOffWin = kOffB + 2 * kN * kK * 2;          // staged window
constexpr int kOffQn = kOffWin + kWinHalves * 2 + 64;     // 2 x 256 candidate norms
// per reference (row of kLs words): the kept 32 (keys and candidates,
// ascending) and up to 32 newcomers waiting for a merge
constexpr int kLs = kTop + 1;                             // row stride: rows start in distinct banks
constexpr int kOffKd = kOffQn + 2 * kN * 4;               // kept keys: 128 x kLs
constexpr int kOffKc = kOffKd + kRefs * kLs * 4;          // kept candidates
constexpr int kOffNd = kOffKc + kRefs * kLs * 4;          // newcomer keys
constexpr int kOffNc = kOffNd + kRefs * kLs * 4;          // newcomer candidates
constexpr int kOffDv = kOffNc + kRefs * kLs * 4;          // 4 warps x 32 lanes x 36 keys (one group)
constexpr int kOffWt = kOffDv + 4 * 32 * 36 * 4;          // windows: kMaxWt x 128 x short4
constexpr int kSmem = kOffWt + kMaxWt * kRefs * 8;

static_assert(kSmem <= 227 * 1024, "shared memory");

// core-matrix layout (umma.cuh): row r, k-block kb (8 elements)
__device__ __forceinline__ int cm_off(int r, int kb) { return (r >> 3) * 1024 + kb * 128 + (r & 7) * 16; }

struct TcArgs {
	const Tile *tiles;
	int ntiles;
	const int *grid;
	const uint32_t *traj;
	int nfm;
	const long long *blocks;    // first group of every 16 x 8 block
	long long nblocks;
	uint32_t *cand;             // [G][32] candidates (qx | qy << 13 | frame << 26)
	float *lb;                  // [G] lower bound on every dropped candidate's distance
	int *status;                // [0]: a wait gave up
	const float *thr0;          // [G] starting threshold (anchor_kernel), distance units
};

struct Union {
	int x0, y0, x1, y1;
};

// Four consecutive FP16 values starting at an even or odd position of a row
// (the window rows are 4-byte aligned).
template <int NW>
__device__ __forceinline__ void row_halves(const __half *row, int x, uint32_t (&out)[NW])
{
	const uint32_t *w = reinterpret_cast<const uint32_t *>(row) + (x >> 1);
	uint32_t v[NW + 1];
#pragma unroll
	for (int i = 0; i <= NW; i++) v[i] = w[i];
	if (x & 1) {
#pragma unroll
		for (int i = 0; i < NW; i++) out[i] = __byte_perm(v[i], v[i + 1], 0x5432);
	} else {
#pragma unroll
		for (int i = 0; i < NW; i++) out[i] = v[i];
	}
}

__device__ __forceinline__ float sq_half2(uint32_t h, float acc)
{
	const float2 f = __half22float2(*reinterpret_cast<const __half2 *>(&h));
	return fmaf(f.y, f.y, fmaf(f.x, f.x, acc));
}

// One lane's 16 patch elements as two 16-byte core-matrix rows: PX = 4
// (PT = 4): patch frame `part`, rows hy 0-1 and 2-3; PX = 8 (PT = 1): rows
// 2*part and 2*part + 1.  `rows(ht, hy)` points at the patch's row start.
template <int PX, class RowFn>
__device__ __forceinline__ float build_rows(RowFn rows, int x, int part, unsigned char *dst, int r)
{
	float s = 0.f;
	if (PX == 4) {
		uint32_t a[2], b[2], c[2], d[2];
		row_halves<2>(rows(part, 0), x, a);
		row_halves<2>(rows(part, 1), x, b);
		row_halves<2>(rows(part, 2), x, c);
		row_halves<2>(rows(part, 3), x, d);
		*reinterpret_cast<uint4 *>(dst + cm_off(r, 2 * part)) = make_uint4(a[0], a[1], b[0], b[1]);
		*reinterpret_cast<uint4 *>(dst + cm_off(r, 2 * part + 1)) = make_uint4(c[0], c[1], d[0], d[1]);
		s = sq_half2(a[0], s); s = sq_half2(a[1], s); s = sq_half2(b[0], s); s = sq_half2(b[1], s);
		s = sq_half2(c[0], s); s = sq_half2(c[1], s); s = sq_half2(d[0], s); s = sq_half2(d[1], s);
	} else {
		uint32_t a[4], b[4];
		row_halves<4>(rows(0, 2 * part), x, a);
		row_halves<4>(rows(0, 2 * part + 1), x, b);
		*reinterpret_cast<uint4 *>(dst + cm_off(r, 2 * part)) = make_uint4(a[0], a[1], a[2], a[3]);
		*reinterpret_cast<uint4 *>(dst + cm_off(r, 2 * part + 1)) = make_uint4(b[0], b[1], b[2], b[3]);
#pragma unroll
		for (int i = 0; i < 4; i++) { s = sq_half2(a[i], s); s = sq_half2(b[i], s); }
	}
	return s;
}

// Lower bound on the reference FP32 distance of every candidate whose
// approximate distance is at least a32 (see the file comment): dp is the
// exact norm of the reference patch's FP16 rounding error, emax the largest
// rounding error of any staged window value (a candidate's error norm is at
// most 8 emax), pn and qmax the patch norms of the split.
__device__ __forceinline__ float drop_bound(float a32, float pn, float qmax, float dp, float emax)
{
	if (a32 != a32 || pn != pn || qmax != qmax || dp != dp || emax != emax) return -1.f;
	if (a32 == __int_as_float(0x7f800000)) return a32;     // fewer than 32 candidates: none dropped
	const float sp = sqrtf(fmaxf(pn, 0.f)), sq = sqrtf(fmaxf(qmax, 0.f));
	// FP32 rounding of the norms (64-term chains), of the tensor-core dot
	// product (64 additions) and of the sums that form the keys
	const float e = 1.0e-5f * (sp + sq) * (sp + sq) + 1e-2f;
	// FP16 rounding of both patches
	const float delta = 1.01f * (dp + 8.f * emax) + 1e-4f;
	const float r = a32 - e;
	if (!(r > 0.f)) return 0.f;
	const float d = sqrtf(r) * 0.99999f - delta;
	if (!(d > 0.f)) return 0.f;
	return d * d * 0.9999f;
}

// Warp-cooperative merge of one reference's newcomers (nd/nc, the first
// `cnt` of its row) into its kept 32 (kd/kc, ascending): the newcomers are
// sorted by a bitonic network across the lanes, the lane-wise minimum of the
// kept list and the reversed newcomers is a bitonic sequence holding the 32
// smallest of both, and a bitonic merge orders it.  Returns the new 32nd
// smallest key (the threshold for newcomers) to every lane.
__device__ __forceinline__ float merge_row(float *kd, uint32_t *kc, const float *nd, const uint32_t *nc, int row,
                                          int cnt)
{
	const int lane = threadIdx.x & 31;
	float x = lane < cnt ? nd[row * kLs + lane] : __int_as_float(0x7f800000);
	uint32_t xc = lane < cnt ? nc[row * kLs + lane] : 0xffffffffu;
#pragma unroll
	for (int k = 2; k <= 32; k <<= 1)
#pragma unroll
		for (int j = k >> 1; j > 0; j >>= 1) {
			const float ox = __shfl_xor_sync(0xffffffffu, x, j);
			const uint32_t oc = __shfl_xor_sync(0xffffffffu, xc, j);
			const bool up = (lane & k) == 0, low = (lane & j) == 0;
			if ((low == up) ? (ox < x) : (x < ox)) { x = ox; xc = oc; }
		}
	float y = kd[row * kLs + lane];
	uint32_t yc = kc[row * kLs + lane];
	const float rx = __shfl_sync(0xffffffffu, x, 31 - lane);
	const uint32_t rc = __shfl_sync(0xffffffffu, xc, 31 - lane);
	if (rx < y) { y = rx; yc = rc; }
#pragma unroll
	for (int j = 16; j > 0; j >>= 1) {
		const float oy = __shfl_xor_sync(0xffffffffu, y, j);
		const uint32_t oc = __shfl_xor_sync(0xffffffffu, yc, j);
		if (((lane & j) == 0) ? (oy < y) : (y < oy)) { y = oy; yc = oc; }
	}
	kd[row * kLs + lane] = y;
	kc[row * kLs + lane] = yc;
	return __shfl_sync(0xffffffffu, y, 31);
}

// Merges every lane's newcomers whose lane is set in `need` (warp-collective).
__device__ __forceinline__ void merge_lanes(float *kd, uint32_t *kc, const float *nd, const uint32_t *nc, int warp,
                                           unsigned need, int &cnt, float &thr, float cap)
{
	const int lane = threadIdx.x & 31;
	while (need) {
		const int L = __ffs(need) - 1;
		need &= need - 1u;
		const int cl = __shfl_sync(0xffffffffu, cnt, L);
		const float t = merge_row(kd, kc, nd, nc, warp * 32 + L, cl);
		if (lane == L) {
			thr = fminf(t, cap);
			cnt = 0;
		}
	}
}

template <int PX, int PT>
__global__ void __launch_bounds__(kThreads, 1) search_tc_kernel(Image src, StepParams sp, TcArgs a)
{
	static_assert(PX * PX * PT == kK, "64-element patches");
	extern __shared__ __align__(1024) unsigned char sm[];
	unsigned char *sA = sm + kOffA;
	unsigned char *sB = sm + kOffB;
	__half *win = reinterpret_cast<__half *>(sm + kOffWin);
	float *qnc = reinterpret_cast<float *>(sm + kOffQn);
	float *kd = reinterpret_cast<float *>(sm + kOffKd);
	uint32_t *kc = reinterpret_cast<uint32_t *>(sm + kOffKc);
	float *nd = reinterpret_cast<float *>(sm + kOffNd);
	uint32_t *nc = reinterpret_cast<uint32_t *>(sm + kOffNc);
	short4 *wt = reinterpret_cast<short4 *>(sm + kOffWt);
	float *dv = reinterpret_cast<float *>(sm + kOffDv);

	// per operand buffer: MMA finished, norms written (staging warps), read out
	// (selection warps)
	__shared__ __align__(8) uint64_t mma_done[2], qn_full[2], epi_done[2];
	__shared__ uint32_t tmem_base;
	__shared__ Union uni[kMaxWt];
	__shared__ int s_nch[kMaxWt];
	__shared__ float s_pn[kRefs], s_dp[kRefs];
	__shared__ long long s_g[kRefs];
	__shared__ int s_x[kRefs], s_y[kRefs];
	__shared__ int s_overflow, s_qmax, s_fail, s_bad, s_emax, s_csum, s_ccnt;

	const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
	const bool selector = warp < 4;
	const int hw = (sp.wx - 1) / 2;

	if (warp == 0) {
		umma::tmem_alloc(&tmem_base, kTmemCols);
		umma::tmem_relinquish();
	}
	if (tid == 0) {
		umma::mbar_init(&mma_done[0], 1);
		umma::mbar_init(&mma_done[1], 1);
		umma::mbar_init(&qn_full[0], 128);
		umma::mbar_init(&qn_full[1], 128);
		umma::mbar_init(&epi_done[0], 4);
		umma::mbar_init(&epi_done[1], 4);
		umma::mbar_init_fence();
		s_fail = 0;
	}
	umma::fence_before_sync();
	__syncthreads();
	umma::fence_after_sync();
	const uint32_t tmem = tmem_base;
	constexpr uint32_t kIdesc = umma::idesc_f16(kRefs, kN, false);
	uint32_t jchunk = 0;   // chunks issued so far (both groups count alike)

	for (long long bi = blockIdx.x; bi < a.nblocks; bi += gridDim.x) {
		// ---- block set-up --------------------------------------------------
		const long long g0 = a.blocks[bi];
		const Tile T = a.tiles[tile_of(a.tiles, a.ntiles, g0)];
		const long long loc = g0 - T.g0;
		const int xi0 = (int)(loc % T.nx), yi0 = (int)((loc / T.nx) % T.ny);
		int xr, yr, tr;
		group_position(T, a.grid, g0, xr, yr, tr);
		int t0, t1;
		temporal_range(sp, tr, t0, t1);
		const int nwt = t1 - t0 + 1;
		if (tid < kRefs) {
			// reference r: warp w covers an 8 x 4 sub-block, lanes along x
			const int dx = (lane & 7) + 8 * (warp & 1), dy = (lane >> 3) + 4 * (warp >> 1);
			const bool ok = xi0 + dx < T.nx && yi0 + dy < T.ny;
			const long long g = g0 + (long long)dy * T.nx + dx;
			int x = 0, y = 0, t = 0;
			if (ok) group_position(T, a.grid, g, x, y, t);
			s_g[tid] = ok ? g : -1;
			s_x[tid] = x;
			s_y[tid] = y;
		}
		if (tid < kMaxWt) uni[tid] = Union{1 << 30, 1 << 30, -1, -1};
		if (tid == 0) {
			s_overflow = 0;
			s_qmax = 0;
			s_bad = 0;
			s_emax = 0;
			s_csum = 0;
			s_ccnt = 0;
		}
		__syncthreads();
		if (tid < kRefs) {
			// the block's centre: the rounded mean of its reference positions'
			// values (integer sums: the same centre on every run)
			int v = 0, n = 0;
			if (s_g[tid] >= 0) {
				const float f = __ldg(src.p + src.at(T.ox + s_x[tid], T.oy + s_y[tid], tr, 0));
				v = __float2int_rn(fminf(fmaxf(f, -30000.f), 30000.f));
				n = 1;
			}
#pragma unroll
			for (int o = 16; o > 0; o >>= 1) {
				v += __shfl_xor_sync(0xffffffffu, v, o);
				n += __shfl_xor_sync(0xffffffffu, n, o);
			}
			if (lane == 0) {
				atomicAdd(&s_csum, v);
				atomicAdd(&s_ccnt, n);
			}
		}
		__syncthreads();
		const float centre = s_ccnt > 0 ? (float)__float2int_rn((float)s_csum / (float)s_ccnt) : 128.f;
		if (selector) {
			// windows of every candidate frame (nldct.cpp:1248-1258) and their union
			const long long g = s_g[tid];
			for (int ii = 0; ii < nwt; ii++) {
				int rx0 = 0, ry0 = 0, nx = 0, ny = 0;
				if (g >= 0) {
					const uint32_t c = a.traj[g * a.nfm + ii];
					const int cx = (int)(c & 0xffffu), cy = (int)(c >> 16);
					const int shx = min(0, cx - hw) + max(0, cx + hw - T.w + PX);
					const int shy = min(0, cy - hw) + max(0, cy + hw - T.h + PX);
					rx0 = max(0, cx - hw - shx);
					ry0 = max(0, cy - hw - shy);
					nx = max(0, min(T.w - PX, cx + hw - shx) - rx0 + 1);
					ny = max(0, min(T.h - PX, cy + hw - shy) - ry0 + 1);
				}
				wt[ii * kRefs + tid] = make_short4((short)rx0, (short)ry0, (short)nx, (short)ny);
				const bool has = nx > 0 && ny > 0;
				int mx0 = has ? rx0 : 1 << 30, my0 = has ? ry0 : 1 << 30;
				int mx1 = has ? rx0 + nx - 1 : -1, my1 = has ? ry0 + ny - 1 : -1;
#pragma unroll
				for (int o = 16; o > 0; o >>= 1) {
					mx0 = min(mx0, __shfl_xor_sync(0xffffffffu, mx0, o));
					my0 = min(my0, __shfl_xor_sync(0xffffffffu, my0, o));
					mx1 = max(mx1, __shfl_xor_sync(0xffffffffu, mx1, o));
					my1 = max(my1, __shfl_xor_sync(0xffffffffu, my1, o));
				}
				if (lane == 0) {
					atomicMin(&uni[ii].x0, mx0);
					atomicMin(&uni[ii].y0, my0);
					atomicMax(&uni[ii].x1, mx1);
					atomicMax(&uni[ii].y1, my1);
				}
			}
			// kept lists: 32 empty slots per reference
			for (int s = 0; s < kTop; s++) {
				kd[tid * kLs + s] = __int_as_float(0x7f800000);
				kc[tid * kLs + s] = 0xffffffffu;
			}
		} else {
			// A operand: the 128 reference patches, centred FP16
			const int pt = tid - 128;
			for (int it = pt; it < kRefs * 4; it += 128) {
				const int r = it >> 2, part = it & 3;
				float s = 0.f, er = 0.f;
				if (s_g[r] >= 0) {
					const int x = T.ox + s_x[r], y = T.oy + s_y[r];
					float v[16];
#pragma unroll
					for (int e = 0; e < 16; e++) {
						int ht, hy, hx;
						if (PX == 4) { ht = part; hy = e >> 2; hx = e & 3; }
						else { ht = 0; hy = 2 * part + (e >> 3); hx = e & 7; }
						v[e] = __ldg(src.p + src.at(x + hx, y + hy, tr + ht, 0)) - centre;
					}
					bool fin = true;
#pragma unroll
					for (int e = 0; e < 16; e++) fin = fin && fabsf(v[e]) < 60000.f;
					if (!fin) s_bad = 1;      // NaN, infinity or beyond FP16: exact search
					uint32_t h[8];
#pragma unroll
					for (int e = 0; e < 8; e++) {
						const __half2 p2 = __floats2half2_rn(v[2 * e], v[2 * e + 1]);
						h[e] = *reinterpret_cast<const uint32_t *>(&p2);
						s = sq_half2(h[e], s);
						const float2 f = __half22float2(p2);
						const float e0 = f.x - v[2 * e], e1 = f.y - v[2 * e + 1];
						er = fmaf(e1, e1, fmaf(e0, e0, er));
					}
					*reinterpret_cast<uint4 *>(sA + cm_off(r, 2 * part)) = make_uint4(h[0], h[1], h[2], h[3]);
					*reinterpret_cast<uint4 *>(sA + cm_off(r, 2 * part + 1)) = make_uint4(h[4], h[5], h[6], h[7]);
				} else {
					*reinterpret_cast<uint4 *>(sA + cm_off(r, 2 * part)) = make_uint4(0, 0, 0, 0);
					*reinterpret_cast<uint4 *>(sA + cm_off(r, 2 * part + 1)) = make_uint4(0, 0, 0, 0);
				}
				// the four parts of a reference are in consecutive threads
				s += __shfl_xor_sync(0xffffffffu, s, 1);
				s += __shfl_xor_sync(0xffffffffu, s, 2);
				er += __shfl_xor_sync(0xffffffffu, er, 1);
				er += __shfl_xor_sync(0xffffffffu, er, 2);
				if (part == 0) {
					s_pn[r] = s;
					s_dp[r] = sqrtf(er);
				}
			}
			umma::fence_proxy_async();
		}
		__syncthreads();
		if (tid < nwt) {
			const Union u = uni[tid];
			const int UW = u.x1 - u.x0 + 1, UH = u.y1 - u.y0 + 1;
			int nch = 0;
			if (UW > 0 && UH > 0) {
				const int pitch = ((UW + PX + 2) + 1) & ~1;
				if ((long long)PT * pitch * (UH + PX - 1) + 8 > kWinHalves) atomicOr(&s_overflow, 1);
				nch = (UW * UH + kN - 1) / kN;
			}
			s_nch[tid] = nch;
		}
		__syncthreads();
		const bool overflow = s_overflow != 0;

		// ---- candidate frames, in chunks of 256 ------------------------------
		if (!overflow) {
			if (selector) {
				const int r = tid;
				const bool valid = s_g[r] >= 0;
				// keys |q'|^2 - 2<p',q'> (the approximate distance less |p'|^2); the
				// anchors' threshold caps the 32nd smallest kept key from the start
				const float cap = valid ? a.thr0[s_g[r]] - s_pn[r] : __int_as_float(0x7f800000);
				float thr = cap < __int_as_float(0x7f800000) ? cap : __int_as_float(0x7f800000);
				int cnt = 0;                               // newcomers waiting for a merge
				const uint32_t tl = tmem + ((uint32_t)(warp * 32) << 16);
				float *mydv = dv + (warp * 32 + lane) * 36;
				for (int ii = 0; ii < nwt; ii++) {
					const Union u = uni[ii];
					const int UW = u.x1 - u.x0 + 1, UH = u.y1 - u.y0 + 1;
					const int nu = UW > 0 && UH > 0 ? UW * UH : 0;
					const short4 w4 = wt[ii * kRefs + r];
					const int lx0 = w4.x - u.x0, ly0 = w4.y - u.y0, wnx = w4.z, wny = w4.w;
					for (int ch = 0; ch < s_nch[ii]; ch++, jchunk++) {
						const int b = jchunk & 1;
						const uint32_t par = (jchunk >> 1) & 1;
						if (!umma::mbar_wait(&qn_full[b], par, kWaitLimit) ||
						    !umma::mbar_wait(&mma_done[b], par, kWaitLimit))
							atomicOr(&s_fail, 1);
						umma::fence_after_sync();
						const float *qn = qnc + b * kN;
						const int n0 = ch * kN;
						for (int grp = 0; grp < kN / 32; grp++) {
							const int g0c = n0 + grp * 32;
							if (g0c >= nu) break;
							const int row0 = g0c / UW, col0 = g0c - row0 * UW;
							uint32_t wmask = 0;
							if (valid && wnx > 0) {
								for (int k = 0;; k++) {
									const int cs = k * UW - col0;
									if (cs >= 32) break;
									if ((unsigned)(row0 + k - ly0) < (unsigned)wny) {
										const int lo = max(0, cs + lx0), hi = min(32, cs + lx0 + wnx);
										if (lo < hi)
											wmask |= (hi >= 32 ? 0xffffffffu : ((1u << hi) - 1u)) & ~((1u << lo) - 1u);
									}
								}
							}
							if (!__any_sync(0xffffffffu, wmask)) continue;
							uint32_t acc[32];
							umma::tmem_ld32(tl + (uint32_t)(b * kN + grp * 32), acc);
							umma::tmem_wait_ld();
							float key[32];
							uint32_t hits = 0;
							const float4 *q4 = reinterpret_cast<const float4 *>(qn + grp * 32);
#pragma unroll
							for (int c4 = 0; c4 < 8; c4++) {
								const float4 q = q4[c4];
								key[4 * c4 + 0] = fmaf(-2.f, __uint_as_float(acc[4 * c4 + 0]), q.x);
								key[4 * c4 + 1] = fmaf(-2.f, __uint_as_float(acc[4 * c4 + 1]), q.y);
								key[4 * c4 + 2] = fmaf(-2.f, __uint_as_float(acc[4 * c4 + 2]), q.z);
								key[4 * c4 + 3] = fmaf(-2.f, __uint_as_float(acc[4 * c4 + 3]), q.w);
							}
#pragma unroll
							for (int c = 0; c < 32; c++)
								if (key[c] < thr) hits |= 1u << c;
							hits &= wmask;
							if (!__any_sync(0xffffffffu, hits)) continue;
							// the hits join the reference's newcomers (candidate = frame << 16 |
							// position in the frame's union), one per lane and round; a full
							// list is merged into the kept 32 by the whole warp
							if (hits) {
#pragma unroll
								for (int c4 = 0; c4 < 8; c4++)
									*reinterpret_cast<float4 *>(mydv + 4 * c4) =
										make_float4(key[4 * c4], key[4 * c4 + 1], key[4 * c4 + 2], key[4 * c4 + 3]);
							}
							const uint32_t cbase = ((uint32_t)ii << 16) | (uint32_t)g0c;
							while (__any_sync(0xffffffffu, hits)) {
								if (hits) {
									const int c = __ffs(hits) - 1;
									hits &= hits - 1u;
									const float d = mydv[c];
									if (d < thr) {
										nd[r * kLs + cnt] = d;
										nc[r * kLs + cnt] = cbase + (uint32_t)c;
										cnt++;
									}
								}
								const unsigned full = __ballot_sync(0xffffffffu, cnt == kTop);
								if (full) merge_lanes(kd, kc, nd, nc, warp, full, cnt, thr, cap);
							}
						}
						umma::fence_before_sync();
						__syncwarp();
						if (lane == 0) umma::mbar_arrive(&epi_done[b]);
					}
				}
				merge_lanes(kd, kc, nd, nc, warp, __ballot_sync(0xffffffffu, cnt > 0), cnt, thr, cap);
			} else {
				// staging warps: window of every candidate frame, then its chunks
				const int pt = tid - 128, pw = pt >> 5;
				for (int ii = 0; ii < nwt; ii++) {
					const Union u = uni[ii];
					const int UW = u.x1 - u.x0 + 1, UH = u.y1 - u.y0 + 1;
					if (s_nch[ii] == 0) continue;
					const int qt = visit_frame(ii, tr, t1);
					const int pitch = ((UW + PX + 2) + 1) & ~1;
					const int wh = UH + PX - 1, ww = UW + PX - 1;
					// the previous frame's chunks are all built: the window can go
					asm volatile("bar.sync 1, 128;" ::: "memory");
					// sixteen rows per warp in flight: loads first, then conversions
					{
						float em = 0.f;
						const int nrow = PT * wh;
						for (int x2 = lane; 2 * x2 < ww; x2 += 32) {
							const bool two = 2 * x2 + 1 < ww;
							for (int r0 = pw; r0 < nrow; r0 += 64) {
								float v0[16], v1[16];
#pragma unroll
								for (int k = 0; k < 16; k++) {
									const int row = r0 + 4 * k;
									v0[k] = v1[k] = 0.f;
									if (row < nrow) {
										const int ht = row / wh, y = row - ht * wh;
										const float *gp = src.p + src.at(T.ox + u.x0 + 2 * x2, T.oy + u.y0 + y, qt + ht, 0);
										v0[k] = __ldg(gp);
										if (two) v1[k] = __ldg(gp + 1);
									}
								}
#pragma unroll
								for (int k = 0; k < 16; k++) {
									const int row = r0 + 4 * k;
									if (row < nrow) {
										const float a0 = v0[k] - centre, a1 = two ? v1[k] - centre : 0.f;
										if (!(fabsf(a0) < 60000.f && fabsf(a1) < 60000.f)) s_bad = 1;
										const __half2 h2 = __floats2half2_rn(a0, a1);
										const float2 f = __half22float2(h2);
										em = fmaxf(em, fmaxf(fabsf(f.x - a0), fabsf(f.y - a1)));
										reinterpret_cast<__half2 *>(win + row * pitch)[x2] = h2;
									}
								}
							}
						}
#pragma unroll
						for (int o = 16; o > 0; o >>= 1) em = fmaxf(em, __shfl_xor_sync(0xffffffffu, em, o));
						if (lane == 0) atomicMax(&s_emax, __float_as_int(em));
					}
					asm volatile("bar.sync 1, 128;" ::: "memory");
					const int nu = UW * UH;
					for (int ch = 0; ch < s_nch[ii]; ch++, jchunk++) {
						const int b = jchunk & 1;
						if (jchunk >= 2 && !umma::mbar_wait(&epi_done[b], ((jchunk >> 1) - 1) & 1, kWaitLimit))
							atomicOr(&s_fail, 1);
						unsigned char *dst = sB + b * (kN * kK * 2);
						float *qn = qnc + b * kN;
						const int n0 = ch * kN;
						// lanes: candidate (lane & 7) of an 8-candidate run, part (lane >> 3)
						const int part = lane >> 3;
						for (int run = pw; run < kN / 8; run += 4) {
							const int n = run * 8 + (lane & 7);
							const int nn = n0 + n;
							float s = 0.f;
							if (nn < nu) {
								const int qy = nn / UW, qx = nn - qy * UW;
								auto rows = [&](int ht, int hy) { return win + (ht * wh + qy + hy) * pitch; };
								s = build_rows<PX>(rows, qx, part, dst, n);
							} else {
								*reinterpret_cast<uint4 *>(dst + cm_off(n, 2 * part)) = make_uint4(0, 0, 0, 0);
								*reinterpret_cast<uint4 *>(dst + cm_off(n, 2 * part + 1)) = make_uint4(0, 0, 0, 0);
							}
							s += __shfl_xor_sync(0xffffffffu, s, 8);
							s += __shfl_xor_sync(0xffffffffu, s, 16);
							if (part == 0) {
								qn[n] = s;
								if (nn < nu) atomicMax(&s_qmax, __float_as_int(s));
							}
						}
						umma::fence_proxy_async();
						umma::mbar_arrive(&qn_full[b]);
						asm volatile("bar.sync 1, 128;" ::: "memory");
						if (pt == 0) {
							umma::fence_after_sync();
							const uint32_t a0 = umma::smem_u32(sA), b0 = umma::smem_u32(dst);
#pragma unroll
							for (int ks = 0; ks < kK / 16; ks++) {
								const uint64_t ad = umma::smem_desc(a0 + ks * 256, 128, 1024);
								const uint64_t bd = umma::smem_desc(b0 + ks * 256, 128, 1024);
								umma::mma_f16(tmem + (uint32_t)(b * kN), ad, bd, kIdesc, ks > 0 ? 1u : 0u);
							}
							umma::mma_commit(&mma_done[b]);
						}
					}
				}
			}
		}
		__syncthreads();
		// ---- results of the block ------------------------------------------
		if (selector) {
			const long long g = s_g[tid];
			if (g >= 0) {
				// every dropped candidate's key was at least min(cap, 32nd kept key)
				const float root = fminf(kd[tid * kLs + kTop - 1], a.thr0[g] - s_pn[tid]);
				const bool skip = overflow || s_bad;
				const float lbv = skip ? -1.f
				                       : drop_bound(root + s_pn[tid], s_pn[tid], __int_as_float(s_qmax), s_dp[tid],
				                                    __int_as_float(s_emax));
				a.lb[g] = lbv;
				// frame << 16 | union position -> qx | qy << 13 | frame << 26
				uint32_t cv[4];
				uint4 *out = reinterpret_cast<uint4 *>(a.cand + g * kTop);
				for (int s = 0; s < kTop; s += 4) {
#pragma unroll
					for (int e = 0; e < 4; e++) {
						const uint32_t v = kc[tid * kLs + s + e];
						uint32_t o = 0xffffffffu;
						if (!skip && v != 0xffffffffu) {
							const int fi = (int)(v >> 16), n = (int)(v & 0xffffu);
							const Union u = uni[fi];
							const int UW = u.x1 - u.x0 + 1;
							const int qy = n / UW, qx = n - qy * UW;
							o = (uint32_t)(u.x0 + qx) | ((uint32_t)(u.y0 + qy) << 13) | ((uint32_t)fi << 26);
						}
						cv[e] = o;
					}
					out[s / 4] = make_uint4(cv[0], cv[1], cv[2], cv[3]);
				}
			}
		}
		__syncthreads();
		if (s_fail) break;
	}
	// a wait that gave up leaves the rest of the work to the exact search:
	// every reference not written keeps the bound the caller set (NaN: not
	// certified); the MMAs still in flight are waited for (bounded) before
	// the tensor memory is released
	if (tid == 0 && s_fail) atomicOr(a.status, 1);
	if (tid == 128 && s_fail) {
		for (uint32_t j = jchunk >= 2 ? jchunk - 2 : 0; j < jchunk; j++)
			umma::mbar_wait(&mma_done[j & 1], (j >> 1) & 1, kWaitLimit);
	}
	umma::fence_before_sync();
	__syncthreads();
	if (warp == 0) {
		umma::fence_after_sync();
		umma::tmem_dealloc(tmem, kTmemCols);
	}
}

// Starting threshold of the pre-screen, per reference: the exact distances
// (FP32, any order: only a threshold) of anchor candidates -- in every frame
// of the temporal range the window's centre (the reference's position moved
// along the flow, or the reference itself) and its four neighbours -- and
// the kAnchorRank-th smallest of them, widened by 5 %.  Candidates above it
// are unlikely to be among the nearest, so the pre-screen lists only those
// below it (or below its 32nd smallest, when lower); the bound on the
// dropped candidates accounts for it.  One warp per reference.
constexpr int kAnchorRank = 20;

struct AnchorArgs {
	const Tile *tiles;
	int ntiles;
	const int *grid;
	const uint32_t *traj;
	int nfm;
	long long G;
	float *thr0;
};

template <int PX, int PT>
__global__ void __launch_bounds__(256) anchor_kernel(Image src, StepParams sp, AnchorArgs a)
{
	constexpr int K = PX * PX * PT;
	const int lane = threadIdx.x & 31;
	const long long nw = (long long)gridDim.x * (blockDim.x >> 5);
	const int hw = (sp.wx - 1) / 2;
	for (long long g = blockIdx.x * (long long)(blockDim.x >> 5) + (threadIdx.x >> 5); g < a.G; g += nw) {
		const Tile T = a.tiles[tile_of(a.tiles, a.ntiles, g)];
		int x, y, t, t0, t1;
		group_position(T, a.grid, g, x, y, t);
		temporal_range(sp, t, t0, t1);
		const int nwt = t1 - t0 + 1;
		float v[2];
#pragma unroll
		for (int rep = 0; rep < 2; rep++) {
			const int ai = lane + 32 * rep;
			v[rep] = __int_as_float(0x7f800000);
			if (ai >= 5 * nwt) continue;
			const int ii = ai / 5, o = ai % 5;
			const uint32_t c = a.traj[g * a.nfm + ii];
			const int cx = (int)(c & 0xffffu), cy = (int)(c >> 16);
			const int shx = min(0, cx - hw) + max(0, cx + hw - T.w + PX);
			const int shy = min(0, cy - hw) + max(0, cy + hw - T.h + PX);
			const int rx0 = max(0, cx - hw - shx), ry0 = max(0, cy - hw - shy);
			const int rx1 = min(T.w - PX, cx + hw - shx), ry1 = min(T.h - PX, cy + hw - shy);
			if (rx1 < rx0 || ry1 < ry0) continue;
			const int qx = min(max(cx + (o == 1) - (o == 2), rx0), rx1);
			const int qy = min(max(cy + (o == 3) - (o == 4), ry0), ry1);
			const int qt = visit_frame(ii, t, t1);
			float acc = 0.f;
#pragma unroll 16
			for (int k = 0; k < K; k++) {
				const int ht = k / (PX * PX), hy = (k / PX) % PX, hx = k % PX;
				const float df = __ldg(src.p + src.at(T.ox + x + hx, T.oy + y + hy, t + ht, 0)) -
				                 __ldg(src.p + src.at(T.ox + qx + hx, T.oy + qy + hy, qt + ht, 0));
				acc = fmaf(df, df, acc);
			}
			v[rep] = acc;
		}
		// the kAnchorRank-th smallest (repeated warp minimum)
		float kth = __int_as_float(0x7f800000);
		for (int k = 0; k < kAnchorRank; k++) {
			const float m = fminf(v[0], v[1]);
			float w = m;
#pragma unroll
			for (int o = 16; o > 0; o >>= 1) w = fminf(w, __shfl_xor_sync(0xffffffffu, w, o));
			kth = w;
			const unsigned holder = __ballot_sync(0xffffffffu, m == w);
			if (lane == __ffs(holder) - 1) {
				if (v[0] == w) v[0] = __int_as_float(0x7f800000);
				else v[1] = __int_as_float(0x7f800000);
			}
		}
		if (lane == 0) a.thr0[g] = kth * 1.05f + 1.f;
	}
}

struct RerankArgs {
	const Tile *tiles;
	int ntiles;
	const int *grid;
	const uint32_t *traj;
	int nfm;
	long long G;
	const uint32_t *cand;
	const float *lb;
	uint8_t *nsimp;
	uint32_t *idx;
	uint32_t *fallback;       // groups left to the exact search
	unsigned *nfallback;
	unsigned *nuncertified;   // groups kept with their uncertified re-rank
	int certified;            // 1: every group not certified goes to the exact search
};

__device__ __forceinline__ bool key_less(float d0, int c0, float d1, int c1)
{
	return d0 < d1 || (d0 == d1 && c0 < c1);
}

// One warp per reference: exact distances of its 32 candidates, sorted;
// certified -> neighbour list and tau rule, else the fallback list.
template <int PX, int PT>
__global__ void __launch_bounds__(256) rerank_kernel(Image src, StepParams sp, RerankArgs a)
{
	constexpr int K = PX * PX * PT;
	const int lane = threadIdx.x & 31;
	const long long nw = (long long)gridDim.x * (blockDim.x >> 5);
	for (long long g = blockIdx.x * (long long)(blockDim.x >> 5) + (threadIdx.x >> 5); g < a.G; g += nw) {
		const Tile T = a.tiles[tile_of(a.tiles, a.ntiles, g)];
		int x, y, t, t0, t1;
		group_position(T, a.grid, g, x, y, t);
		temporal_range(sp, t, t0, t1);
		const int nwt = t1 - t0 + 1;
		const float lbv = a.lb[g];
		// window sizes of every frame (lane = frame), prefix sums = candidate bases
		const int hw = (sp.wx - 1) / 2;
		int rx0 = 0, ry0 = 0, wnx = 0, wny = 0;
		if (lane < nwt) {
			const uint32_t c = a.traj[g * a.nfm + lane];
			const int cx = (int)(c & 0xffffu), cy = (int)(c >> 16);
			const int shx = min(0, cx - hw) + max(0, cx + hw - T.w + PX);
			const int shy = min(0, cy - hw) + max(0, cy + hw - T.h + PX);
			rx0 = max(0, cx - hw - shx);
			ry0 = max(0, cy - hw - shy);
			wnx = max(0, min(T.w - PX, cx + hw - shx) - rx0 + 1);
			wny = max(0, min(T.h - PX, cy + hw - shy) - ry0 + 1);
		}
		const int cnt = wnx * wny;
		int incl = cnt;
#pragma unroll
		for (int o = 1; o < 32; o <<= 1) {
			const int u = __shfl_up_sync(0xffffffffu, incl, o);
			if (lane >= o) incl += u;
		}
		const int ncand = __shfl_sync(0xffffffffu, incl, 31);
		const int base = incl - cnt;
		// this lane's candidate
		const uint32_t c = lbv >= 0.f ? a.cand[g * kTop + lane] : 0xffffffffu;
		const bool has = c != 0xffffffffu;
		const int qx = (int)(c & 0x1fffu), qy = (int)((c >> 13) & 0x1fffu), ii = (int)(c >> 26);
		const int fb = __shfl_sync(0xffffffffu, base, has ? ii : 0);
		const int fx0 = __shfl_sync(0xffffffffu, rx0, has ? ii : 0);
		const int fy0 = __shfl_sync(0xffffffffu, ry0, has ? ii : 0);
		const int fnx = __shfl_sync(0xffffffffu, wnx, has ? ii : 0);
		float d = __int_as_float(0x7f800000);
		int num = 0x7fffffff;
		int qt = 0;
		if (has) {
			qt = visit_frame(ii, t, t1);
			num = fb + (qy - fy0) * fnx + (qx - fx0);
			float acc = 0.f;
#pragma unroll
			for (int k = 0; k < K; k++) {
				const int ht = k / (PX * PX), hy = (k / PX) % PX, hx = k % PX;
				const float rv = __ldg(src.p + src.at(T.ox + x + hx, T.oy + y + hy, t + ht, 0));
				const float qv = __ldg(src.p + src.at(T.ox + qx + hx, T.oy + qy + hy, qt + ht, 0));
				const float df = __fsub_rn(rv, qv);
				acc = __fadd_rn(acc, __fmul_rn(df, df));
			}
			d = acc;
		}
		const bool nan = __any_sync(0xffffffffu, d != d);
		// bitonic sort of (distance, candidate number) with the position
		int px = qx, py = qy, pq = qt;
		for (int k = 2; k <= 32; k <<= 1)
			for (int j = k >> 1; j > 0; j >>= 1) {
				const float od = __shfl_xor_sync(0xffffffffu, d, j);
				const int on = __shfl_xor_sync(0xffffffffu, num, j);
				const int ox = __shfl_xor_sync(0xffffffffu, px, j);
				const int oy = __shfl_xor_sync(0xffffffffu, py, j);
				const int ot = __shfl_xor_sync(0xffffffffu, pq, j);
				const bool up = (lane & k) == 0, low = (lane & j) == 0;
				const bool take = (low == up) ? key_less(od, on, d, num) : key_less(d, num, od, on);
				if (take) { d = od; num = on; px = ox; py = oy; pq = ot; }
			}
		const int Kk = min(sp.np, ncand);
		const float dnext = __shfl_down_sync(0xffffffffu, d, 1);
		// the k nearest pairwise distinct, strictly below the next listed one
		// and below every dropped candidate
		const bool inside = lane < Kk;
		const bool distinct = !inside || lane + 1 >= 32 || dnext > d;
		const float dk = __shfl_sync(0xffffffffu, d, max(Kk - 1, 0));
		const int nlisted = __popc(__ballot_sync(0xffffffffu, has));
		// usable: a finished pre-screen with no NaN; certified: see above
		const bool usable = !nan && lbv >= 0.f && Kk > 0 && nlisted >= Kk;
		const bool ok = usable && __all_sync(0xffffffffu, distinct) && (ncand <= kTop ? nlisted == ncand : dk < lbv);
		if (ok || (usable && !a.certified)) {
			if (!ok && lane == 0) atomicAdd(a.nuncertified, 1u);
			float dn[5];
			dn[0] = __shfl_sync(0xffffffffu, d, 1);
			dn[1] = __shfl_sync(0xffffffffu, d, 2);
			dn[2] = __shfl_sync(0xffffffffu, d, 4);
			dn[3] = __shfl_sync(0xffffffffu, d, 8);
			dn[4] = __shfl_sync(0xffffffffu, d, 16);
			int nS = 1;
			for (int q = 0; q < 5 && 2 * nS <= Kk && dn[q] < sp.tau2; q++) nS *= 2;
			if (lane == 0) a.nsimp[g] = (uint8_t)nS;
			if (lane < nS) a.idx[g * sp.np + lane] = (uint32_t)(((long long)pq * T.h + py) * T.w + px);
		} else if (lane == 0) {
			const unsigned s = atomicAdd(a.nfallback, 1u);
			a.fallback[s] = (uint32_t)g;
		}
	}
}

template <int PX, int PT>
cudaError_t launch_tc_t(const Image &src, const StepParams &sp, const TcArgs &ta, const RerankArgs &ra,
                        const AnchorArgs &aa, int nsm, cudaStream_t st)
{
	long long ab = (aa.G + 7) / 8;   // eight references (warps) per block
	if (ab > (long long)nsm * 16) ab = (long long)nsm * 16;
	if (ab > 0) anchor_kernel<PX, PT><<<(int)ab, 256, 0, st>>>(src, sp, aa);
	cudaError_t e = cudaGetLastError();
	if (e != cudaSuccess) return e;
	e = cudaFuncSetAttribute(search_tc_kernel<PX, PT>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmem);
	if (e != cudaSuccess) return e;
	const long long nb = ta.nblocks < nsm ? ta.nblocks : nsm;
	if (nb > 0) search_tc_kernel<PX, PT><<<(int)nb, kThreads, kSmem, st>>>(src, sp, ta);
	if ((e = cudaGetLastError()) != cudaSuccess) return e;
	long long blocks = (ra.G + 7) / 8;   // eight references (warps) per block
	if (blocks > (long long)nsm * 16) blocks = (long long)nsm * 16;
	if (blocks > 0) rerank_kernel<PX, PT><<<(int)blocks, 256, 0, st>>>(src, sp, ra);
	return cudaGetLastError();
}

// Self-check of the operand layout and descriptors: D = A * B^T for one
// 128 x 256 x 64 FP16 tile, through shared memory, tcgen05.mma and TMEM.
__global__ void __launch_bounds__(kThreads, 1) tc_selftest_kernel(const uint16_t *A, const uint16_t *B, float *D,
                                                                  int *status)
{
	extern __shared__ __align__(1024) unsigned char sm[];
	unsigned char *sA = sm + kOffA;
	unsigned char *sB = sm + kOffB;
	__shared__ __align__(8) uint64_t done;
	__shared__ uint32_t tmem_base;
	const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
	if (warp == 0) {
		umma::tmem_alloc(&tmem_base, 256);
		umma::tmem_relinquish();
	}
	if (tid == 0) {
		umma::mbar_init(&done, 1);
		umma::mbar_init_fence();
	}
	for (int i = tid; i < kRefs * 8; i += kThreads) {
		const int r = i >> 3, kb = i & 7;
		*reinterpret_cast<uint4 *>(sA + cm_off(r, kb)) = *reinterpret_cast<const uint4 *>(A + r * kK + kb * 8);
	}
	for (int i = tid; i < kN * 8; i += kThreads) {
		const int r = i >> 3, kb = i & 7;
		*reinterpret_cast<uint4 *>(sB + cm_off(r, kb)) = *reinterpret_cast<const uint4 *>(B + r * kK + kb * 8);
	}
	umma::fence_proxy_async();
	umma::fence_before_sync();
	__syncthreads();
	umma::fence_after_sync();
	const uint32_t tmem = tmem_base;
	if (tid == 0) {
		const uint32_t a0 = umma::smem_u32(sA), b0 = umma::smem_u32(sB);
		for (int ks = 0; ks < kK / 16; ks++)
			umma::mma_f16(tmem, umma::smem_desc(a0 + ks * 256, 128, 1024), umma::smem_desc(b0 + ks * 256, 128, 1024),
			              umma::idesc_f16(kRefs, kN, false), ks > 0 ? 1u : 0u);
		umma::mma_commit(&done);
	}
	const bool ok = umma::mbar_wait(&done, 0, kWaitLimit);
	umma::fence_after_sync();
	if (!ok && tid == 0) atomicOr(status, 1);
	if (warp < 4 && ok) {
		for (int c = 0; c < kN; c += 32) {
			uint32_t v[32];
			umma::tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c, v);
			umma::tmem_wait_ld();
			for (int j = 0; j < 32; j++) D[(warp * 32 + lane) * kN + c + j] = __uint_as_float(v[j]);
		}
	}
	umma::fence_before_sync();
	__syncthreads();
	if (warp == 0) {
		umma::fence_after_sync();
		umma::tmem_dealloc(tmem, 256);
	}
}

}  // namespace

// First group of every 16 x 8 block of reference positions of one frame.
void tc_blocks(const std::vector<Tile> &tiles, std::vector<long long> &out)
{
	out.clear();
	for (const Tile &T : tiles)
		for (int f = 0; f < T.nf; f++)
			for (int y = 0; y < T.ny; y += kBY)
				for (int x = 0; x < T.nx; x += kBX)
					out.push_back(T.g0 + ((long long)f * T.ny + y) * T.nx + x);
}

bool tc_supported(const StepParams &sp, const std::vector<Tile> &tiles)
{
	if (sp.chn_search != 1 || sp.spc != kK || !((sp.px == 4 && sp.pt == 4) || (sp.px == 8 && sp.pt == 1)))
		return false;
	if (sp.np > kTop || sp.np < 2 || sp.wtf + sp.wtb + 1 > kMaxWt || sp.wx > 64) return false;
	for (const Tile &T : tiles)
		if (T.w >= 8192 || T.h >= 8192) return false;
	return true;
}

size_t tc_smem_bytes() { return (size_t)kSmem; }

cudaError_t launch_search_tc(const Image &src, const Tile *tiles, int ntiles, const int *grid, const uint32_t *traj,
                             const StepParams &sp, const long long *blocks, long long nblocks, long long G,
                             uint32_t *cand, float *lb, float *thr0, int *status, uint8_t *nsimp, uint32_t *idx,
                             uint32_t *fallback, unsigned *nfallback, unsigned *nuncertified, int certified, int nsm,
                             cudaStream_t st)
{
	if (G <= 0) return cudaSuccess;
	TcArgs ta;
	ta.tiles = tiles;
	ta.ntiles = ntiles;
	ta.grid = grid;
	ta.traj = traj;
	ta.nfm = search_frames_max(sp);
	ta.blocks = blocks;
	ta.nblocks = nblocks;
	ta.cand = cand;
	ta.lb = lb;
	ta.status = status;
	ta.thr0 = thr0;
	AnchorArgs aa;
	aa.tiles = tiles;
	aa.ntiles = ntiles;
	aa.grid = grid;
	aa.traj = traj;
	aa.nfm = ta.nfm;
	aa.G = G;
	aa.thr0 = thr0;
	RerankArgs ra;
	ra.tiles = tiles;
	ra.ntiles = ntiles;
	ra.grid = grid;
	ra.traj = traj;
	ra.nfm = ta.nfm;
	ra.G = G;
	ra.cand = cand;
	ra.lb = lb;
	ra.nsimp = nsimp;
	ra.idx = idx;
	ra.fallback = fallback;
	ra.nfallback = nfallback;
	ra.nuncertified = nuncertified;
	ra.certified = certified;
	return sp.px == 4 ? launch_tc_t<4, 4>(src, sp, ta, ra, aa, nsm, st) : launch_tc_t<8, 1>(src, sp, ta, ra, aa, nsm, st);
}

cudaError_t tc_selftest(const uint16_t *A, const uint16_t *B, float *D, int *status, cudaStream_t st)
{
	cudaError_t e = cudaFuncSetAttribute(tc_selftest_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmem);
	if (e != cudaSuccess) return e;
	tc_selftest_kernel<<<1, kThreads, kSmem, st>>>(A, B, D, status);
	return cudaGetLastError();
}

}  // namespace bm4dof
