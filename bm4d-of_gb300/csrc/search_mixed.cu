// search_mixed.cu -- mixed-precision patch search: FP16 tensor-core pre-screen
// of the patch cross terms, exact FP32 re-rank of the best 2k.
//
// Same candidates as VideoNLB::estimateSimilarPatchesStep1/2
// (src/core/nldct.cpp:1143-1348, 1607-1789): flow-chained windows, frames in
// the reference's visiting order.  The squared distance is split as
//     |p - q|^2 = |p'|^2 + |q'|^2 - 2 <p', q'>,   p' = p - 128, q' = q - 128,
// with |q'|^2 in FP32 and <p', q'> on the tensor cores (FP16 operands, FP32
// accumulation).  One CTA serves a 4x4 block of reference patches: each
// candidate frame's union of their windows is converted to FP16 once and fed
// to mma.m16n8k16 as the B operand (16 references x 8 candidates x 16 patch
// elements per instruction).  Every reference keeps its 2k best approximate
// candidates across frames (warp bitonic merges); those are re-ranked with the
// exact FP32 distance in the reference's summation order, the k best kept in
// (distance, candidate order) order and cut by the tau power-of-two rule
// (nldct.cpp:1284-1289).  The selected sets equal the exact path's whenever
// the true k nearest are among the 2k best approximations and no exact
// distance ties occur.
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <cstdint>
#include <vector>

#include "common.cuh"
#include "internal.hpp"

namespace bm4dof {

namespace {

constexpr int kRefs = 16;           // reference patches per CTA (the MMA M)
constexpr int kBX = 4, kBY = 4;     // ... as a 4x4 block of grid positions
constexpr int kThreads = 256;       // 8 warps
constexpr int kTop = 32;            // approximate candidates kept per reference (2k)
constexpr int kCW = 40;             // candidate columns per chunk (multiple of 8): 4 windows at offset 3
constexpr int kCH = 32;             // candidate rows per chunk
constexpr float kShift = 128.f;     // values are centred before the FP16 conversion

struct RefWin {
	int rx0, ry0, nx, ny;
};

__device__ __forceinline__ void group_xyz(const Tile &T, const int *grid, long long g, int &x, int &y, int &t)
{
	const long long local = g - T.g0;
	x = grid[T.gx + (int)(local % T.nx)];
	y = grid[T.gy + (int)((local / T.nx) % T.ny)];
	t = grid[T.gf + (int)(local / ((long long)T.nx * T.ny))];
}

__device__ __forceinline__ void trange(const StepParams &sp, int t, int &t0, int &t1)
{
	const int shift_t = min(0, t - sp.wtb) + max(0, t + sp.wtf - sp.F + sp.pt);
	t0 = max(0, t - sp.wtb - shift_t);
	t1 = min(sp.F - sp.pt, t + sp.wtf - shift_t);
}

__device__ __forceinline__ int visit(int ii, int t, int t1)
{
	return ii == 0 ? t : (ii <= t1 - t ? t + ii : t - (ii - (t1 - t)));
}

__device__ __forceinline__ void mma16816(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1)
{
	asm volatile(
		"mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
		"{%0,%1,%2,%3};"
		: "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
		: "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Keys of the per-reference candidate lists: (approximate distance, candidate
// number in the reference's order).  Smaller is better.
struct Cand {
	float d;
	int c;
};

__device__ __forceinline__ bool better(float d0, int c0, float d1, int c1)
{
	return d0 < d1 || (d0 == d1 && c0 < c1);
}

// Merge 32 new candidates (one per lane) into a sorted 32-list held one per
// lane: bitonic sort of the 64 values, keep the lower half.
__device__ __forceinline__ void merge32(float &ld, int &lc, float nd, int nc)
{
	const int lane = threadIdx.x & 31;
	// sort the new values ascending (bitonic, 32 lanes)
	for (int k = 2; k <= 32; k <<= 1)
		for (int j = k >> 1; j > 0; j >>= 1) {
			const float od = __shfl_xor_sync(0xffffffffu, nd, j);
			const int oc = __shfl_xor_sync(0xffffffffu, nc, j);
			const bool up = (lane & k) == 0, low = (lane & j) == 0;
			const bool take = (low == up) ? better(od, oc, nd, nc) : better(nd, nc, od, oc);
			if (take) { nd = od; nc = oc; }
		}
	// the list is ascending; reverse the new values and keep the lane-wise
	// minimum: the 32 smallest of the union, as a bitonic sequence
	const float rd = __shfl_sync(0xffffffffu, nd, 31 - lane);
	const int rc = __shfl_sync(0xffffffffu, nc, 31 - lane);
	if (better(rd, rc, ld, lc)) { ld = rd; lc = rc; }
	for (int j = 16; j > 0; j >>= 1) {
		const float od = __shfl_xor_sync(0xffffffffu, ld, j);
		const int oc = __shfl_xor_sync(0xffffffffu, lc, j);
		const bool low = (lane & j) == 0;
		const bool take = low ? better(od, oc, ld, lc) : better(ld, lc, od, oc);
		if (take) { ld = od; lc = oc; }
	}
}

// Insert (nd, nc) into the sorted 32-list held one per lane when it beats
// the last entry: lanes after its place shift up by one.
__device__ __forceinline__ void insert32(float &ld, int &lc, float nd, int nc)
{
	const int lane = threadIdx.x & 31;
	const float lastd = __shfl_sync(0xffffffffu, ld, 31);
	const int lastc = __shfl_sync(0xffffffffu, lc, 31);
	if (!better(nd, nc, lastd, lastc)) return;
	const int at = __popc(__ballot_sync(0xffffffffu, better(ld, lc, nd, nc)));
	const float ud = __shfl_up_sync(0xffffffffu, ld, 1);
	const int uc = __shfl_up_sync(0xffffffffu, lc, 1);
	if (lane > at) { ld = ud; lc = uc; }
	else if (lane == at) { ld = nd; lc = nc; }
}

constexpr int kInsertMax = 16;  // newcomers inserted one by one; more: one bitonic merge

struct MixedArgs {
	const Tile *tiles;
	int ntiles;
	const int *grid;
	const uint32_t *traj;
	int nfm;
	const long long *blocks;    // first group of every 16-reference row block
	long long nblocks;
	uint8_t *nsimp;
	uint32_t *idx;
};

template <int PX, int PT>
__global__ void __launch_bounds__(kThreads)
search_mixed_kernel(Image src, StepParams sp, MixedArgs a)
{
	constexpr int K = PX * PX * PT;     // 64: four k-steps of 16
	static_assert(K == 64, "mixed search expects 64-element patches");
	constexpr int WX = kCW + PX - 1, WY = kCH + PX - 1;
	constexpr int WXP = (WX + 1 + 7) / 8 * 8;                   // FP16 row pitch (16-byte rows)
	constexpr int NW = kThreads / 32;
	// dynamic shared memory: the chunk window in centred FP16 ([ht][y][x]),
	// row sums of squares, |q'|^2 of every chunk candidate, per-reference distances
	extern __shared__ __align__(16) unsigned char dsm[];
	__half(*win16)[WY][WXP] = reinterpret_cast<__half(*)[WY][WXP]>(dsm);
	float(*rowsq)[WY][kCW] = reinterpret_cast<float(*)[WY][kCW]>(dsm + sizeof(__half) * PT * WY * WXP);
	float(*qn)[kCW] = reinterpret_cast<float(*)[kCW]>(reinterpret_cast<unsigned char *>(rowsq) + sizeof(float) * PT * WY * kCW);
	float *distb = reinterpret_cast<float *>(reinterpret_cast<unsigned char *>(qn) + sizeof(float) * kCH * kCW);
	const int wmax = sp.wx * sp.wx;
#define dist(r, i) distb[(r) * wmax + (i)]
	__shared__ __align__(16) __half ref16[kRefs][K];
	__shared__ float ref32[kRefs][K];
	__shared__ float pn[kRefs];
	__shared__ RefWin rw[kRefs];
	__shared__ int s_cbase[kRefs];
	__shared__ long long s_g[kRefs];
	__shared__ int s_x[kRefs], s_y[kRefs];
	__shared__ float s_ld[kRefs][kTop];
	__shared__ int s_lc[kRefs][kTop];

	const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
	for (long long bi = blockIdx.x; bi < a.nblocks; bi += gridDim.x) {
		// a 4x4 block of reference positions of one frame
		const long long g0 = a.blocks[bi];
		const Tile T = a.tiles[tile_of(a.tiles, a.ntiles, g0)];
		const long long loc = g0 - T.g0;
		const int xi0 = (int)(loc % T.nx), yi0 = (int)((loc / T.nx) % T.ny);
		const int nbx = min(kBX, T.nx - xi0), nby = min(kBY, T.ny - yi0);
		int xr, yr, tr;
		group_xyz(T, a.grid, g0, xr, yr, tr);
		int t0, t1;
		trange(sp, tr, t0, t1);
		const int nwt = t1 - t0 + 1;
		if (tid < kRefs) {
			const int dx = tid % kBX, dy = tid / kBX;
			const bool ok = dx < nbx && dy < nby;
			const long long g = g0 + (long long)dy * T.nx + dx;
			s_g[tid] = ok ? g : -1;
			int x = 0, y = 0, t;
			if (ok) group_xyz(T, a.grid, g, x, y, t);
			s_x[tid] = x;
			s_y[tid] = y;
			s_cbase[tid] = 0;
		}
		__syncthreads();
		// reference patches: FP32 (re-rank) and centred FP16 (MMA A operand)
		for (int i = tid; i < kRefs * K; i += blockDim.x) {
			const int r = i / K, k = i % K;
			float v = 0.f;
			if (s_g[r] >= 0) {
				const int ht = k / (PX * PX), hy = (k / PX) % PX, hx = k % PX;
				v = src.p[src.at(T.ox + s_x[r] + hx, T.oy + s_y[r] + hy, tr + ht, 0)];
			}
			ref32[r][k] = v;
			ref16[r][k] = __float2half_rn(v - kShift);
		}
		for (int i = tid; i < kRefs * kTop; i += blockDim.x) {
			s_ld[i / kTop][i % kTop] = __int_as_float(0x7f800000);
			s_lc[i / kTop][i % kTop] = 0x7fffffff;
		}
		__syncthreads();
		if (tid < kRefs) {
			float s = 0.f;
			for (int k = 0; k < K; k++) {
				// the rounded values the tensor cores see, so that the split
				// |p'|^2 + |q'|^2 - 2<p',q'> is the distance of the rounded patches
				const float c = __half2float(ref16[tid][k]);
				s = fmaf(c, c, s);
			}
			pn[tid] = s;
		}
		// A fragments (16 references x 64 elements), same in every warp
		uint32_t afr[4][4];
#pragma unroll
		for (int s = 0; s < 4; s++) {
			const int r0 = lane >> 2, c0 = s * 16 + (lane & 3) * 2;
			afr[s][0] = *reinterpret_cast<const uint32_t *>(&ref16[r0][c0]);
			afr[s][1] = *reinterpret_cast<const uint32_t *>(&ref16[r0 + 8][c0]);
			afr[s][2] = *reinterpret_cast<const uint32_t *>(&ref16[r0][c0 + 8]);
			afr[s][3] = *reinterpret_cast<const uint32_t *>(&ref16[r0 + 8][c0 + 8]);
		}

		for (int ii = 0; ii < nwt; ii++) {
			const int qt = visit(ii, tr, t1);
			// own windows of this frame
			if (tid < kRefs) {
				RefWin w = {0, 0, 0, 0};
				if (s_g[tid] >= 0) {
					const uint32_t c = a.traj[(s_g[tid]) * a.nfm + ii];
					const int cx = (int)(c & 0xffffu), cy = (int)(c >> 16);
					const int hw = (sp.wx - 1) / 2;
					const int shx = min(0, cx - hw) + max(0, cx + hw - T.w + PX);
					const int shy = min(0, cy - hw) + max(0, cy + hw - T.h + PX);
					w.rx0 = max(0, cx - hw - shx);
					w.ry0 = max(0, cy - hw - shy);
					w.nx = max(0, min(T.w - PX, cx + hw - shx) - w.rx0 + 1);
					w.ny = max(0, min(T.h - PX, cy + hw - shy) - w.ry0 + 1);
				}
				rw[tid] = w;
			}
			__syncthreads();
			// this lane's two references (MMA rows lane/4 and lane/4 + 8)
			const RefWin wa = rw[lane >> 2], wb = rw[(lane >> 2) + 8];
			const float pna = pn[lane >> 2], pnb = pn[(lane >> 2) + 8];
			int ux0 = 1 << 30, uy0 = 1 << 30, ux1 = -1, uy1 = -1;
			for (int r = 0; r < kRefs; r++)
				if (rw[r].nx > 0 && rw[r].ny > 0) {
					ux0 = min(ux0, rw[r].rx0);
					uy0 = min(uy0, rw[r].ry0);
					ux1 = max(ux1, rw[r].rx0 + rw[r].nx - 1);
					uy1 = max(uy1, rw[r].ry0 + rw[r].ny - 1);
				}
			for (int cy0 = uy0; cy0 <= uy1; cy0 += kCH)
				for (int cx0 = ux0; cx0 <= ux1; cx0 += kCW) {
					const int cw = min(kCW, ux1 - cx0 + 1), ch = min(kCH, uy1 - cy0 + 1);
					const int ww = cw + PX - 1, hh = ch + PX - 1;
					// chunk pixels -> centred FP16: one warp per row, lanes along x
					for (int row = warp; row < PT * hh; row += NW) {
						const int ht = row / hh, y = row - ht * hh;
						const float *gp = src.p + src.at(T.ox + cx0, T.oy + cy0 + y, qt + ht, 0);
						__half *dp = &win16[ht][y][0];
						for (int x = lane; x < ww; x += 32) dp[x] = __float2half_rn(__ldg(gp + x) - kShift);
					}
					__syncthreads();
					// row sums of squares of the rounded values
					for (int row = warp; row < PT * hh; row += NW) {
						const int ht = row / hh, y = row - ht * hh;
						for (int x = lane; x < cw; x += 32) {
							float sq = 0.f;
#pragma unroll
							for (int hx = 0; hx < PX; hx++) {
								const float v = __half2float(win16[ht][y][x + hx]);
								sq = fmaf(v, v, sq);
							}
							rowsq[ht][y][x] = sq;
						}
					}
					__syncthreads();
					for (int y = warp; y < ch; y += NW)
						for (int x = lane; x < cw; x += 32) {
							float sq = 0.f;
#pragma unroll
							for (int ht = 0; ht < PT; ht++)
#pragma unroll
								for (int hy = 0; hy < PX; hy++) sq += rowsq[ht][y + hy][x];
							qn[y][x] = sq;
						}
					__syncthreads();
					// tensor-core cross terms: 8 candidates of one row per n-tile
					const int ntx = (cw + 7) / 8;
					for (int nt = warp; nt < ntx * ch; nt += NW) {
						const int y = nt / ntx, xb = (nt - y * ntx) * 8;
						const int xn = min(xb + (lane >> 2), cw - 1);   // this lane's B column
						const bool odd = xn & 1;
						float acc[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
						for (int s = 0; s < 4; s++) {
							const int k0 = s * 16 + (lane & 3) * 2, k1 = k0 + 8;
							const int ht0 = k0 / (PX * PX), hy0 = (k0 / PX) % PX, hx0 = k0 % PX;
							const int ht1 = k1 / (PX * PX), hy1 = (k1 / PX) % PX, hx1 = k1 % PX;
							uint32_t b0, b1;
							if (!odd) {
								b0 = *reinterpret_cast<const uint32_t *>(&win16[ht0][y + hy0][xn + hx0]);
								b1 = *reinterpret_cast<const uint32_t *>(&win16[ht1][y + hy1][xn + hx1]);
							} else {
								// odd column: pack two 16-bit loads
								const unsigned short *p0 = reinterpret_cast<const unsigned short *>(&win16[ht0][y + hy0][xn + hx0]);
								const unsigned short *p1 = reinterpret_cast<const unsigned short *>(&win16[ht1][y + hy1][xn + hx1]);
								b0 = (uint32_t)p0[0] | ((uint32_t)p0[1] << 16);
								b1 = (uint32_t)p1[0] | ((uint32_t)p1[1] << 16);
							}
							mma16816(acc, afr[s], b0, b1);
						}
						// epilogue: rows lane/4 (wa) and lane/4 + 8 (wb), columns 2*(lane&3), +1
						const int qy = cy0 + y;
#pragma unroll
						for (int e = 0; e < 4; e++) {
							const int cxl = xb + (lane & 3) * 2 + (e & 1);
							if (cxl >= cw) continue;
							const int qx = cx0 + cxl;
							const RefWin &w = e < 2 ? wa : wb;
							const int lx = qx - w.rx0, ly = qy - w.ry0;
							if ((unsigned)lx >= (unsigned)w.nx || (unsigned)ly >= (unsigned)w.ny) continue;
							const int r = (lane >> 2) + (e < 2 ? 0 : 8);
							dist(r, ly * w.nx + lx) = (e < 2 ? pna : pnb) + qn[y][cxl] - 2.f * acc[e];
						}
					}
					__syncthreads();
				}
			// fold this frame into the running 2k lists (one warp per reference)
			for (int r = warp; r < kRefs; r += NW) {
				if (s_g[r] < 0) continue;
				const RefWin w = rw[r];
				const int nw = w.nx * w.ny;
				float ld = s_ld[r][lane];
				int lc = s_lc[r][lane];
				const int base = s_cbase[r];   // candidate numbers continue across frames
				for (int i0 = 0; i0 < nw; i0 += 32) {
					const float th = __shfl_sync(0xffffffffu, ld, 31);
					const int i = i0 + lane;
					const float d = i < nw ? dist(r, i) : __int_as_float(0x7f800000);
					unsigned m = __ballot_sync(0xffffffffu, i < nw && d < th);
					if (m == 0u) continue;
					if (__popc(m) > kInsertMax) {
						merge32(ld, lc, i < nw ? d : __int_as_float(0x7f800000), i < nw ? base + i : 0x7fffffff);
						continue;
					}
					// few newcomers: insert them one at a time (same list)
					while (m) {
						const int j = __ffs(m) - 1;
						m &= m - 1u;
						const float dj = __shfl_sync(0xffffffffu, d, j);
						const int cj = base + i0 + j;
						insert32(ld, lc, dj, cj);
					}
				}
				s_ld[r][lane] = ld;
				s_lc[r][lane] = lc;
			}
			__syncthreads();
			if (tid < kRefs) s_cbase[tid] += rw[tid].nx * rw[tid].ny;
			__syncthreads();
		}
		// exact FP32 re-rank of the 2k candidates, then the k best and tau
		for (int r = warp; r < kRefs; r += NW) {
			if (s_g[r] < 0) continue;
			const int c = s_lc[r][lane];
			float dex = __int_as_float(0x7f800000);
			int qx = 0, qy = 0, qtt = 0;
			if (c != 0x7fffffff) {
				// candidate number -> frame and window position
				int rem = c, jj = 0, rx0 = 0, ry0 = 0, nx = 1;
				for (jj = 0; jj < nwt; jj++) {
					const uint32_t tc = a.traj[s_g[r] * a.nfm + jj];
					const int cx = (int)(tc & 0xffffu), cy = (int)(tc >> 16);
					const int hw = (sp.wx - 1) / 2;
					const int shx = min(0, cx - hw) + max(0, cx + hw - T.w + PX);
					const int shy = min(0, cy - hw) + max(0, cy + hw - T.h + PX);
					rx0 = max(0, cx - hw - shx);
					ry0 = max(0, cy - hw - shy);
					nx = max(0, min(T.w - PX, cx + hw - shx) - rx0 + 1);
					const int ny = max(0, min(T.h - PX, cy + hw - shy) - ry0 + 1);
					if (rem < nx * ny) break;
					rem -= nx * ny;
				}
				qtt = visit(jj, tr, t1);
				qx = rx0 + rem % nx;
				qy = ry0 + rem / nx;
				float v[K];
#pragma unroll
				for (int k = 0; k < K; k++) {
					const int ht = k / (PX * PX), hy = (k / PX) % PX, hx = k % PX;
					v[k] = __ldg(src.p + src.at(T.ox + qx + hx, T.oy + qy + hy, qtt + ht, 0));
				}
				float acc = 0.f;
#pragma unroll
				for (int k = 0; k < K; k++) {
					const float dd = __fsub_rn(ref32[r][k], v[k]);
					acc = __fadd_rn(acc, __fmul_rn(dd, dd));
				}
				dex = acc;
			}
			// sort by (exact distance, candidate number)
			float d = dex;
			int cc = c;
			for (int k = 2; k <= 32; k <<= 1)
				for (int j = k >> 1; j > 0; j >>= 1) {
					const float od = __shfl_xor_sync(0xffffffffu, d, j);
					const int oc = __shfl_xor_sync(0xffffffffu, cc, j);
					const int ox = __shfl_xor_sync(0xffffffffu, qx, j), oy = __shfl_xor_sync(0xffffffffu, qy, j);
					const int ot = __shfl_xor_sync(0xffffffffu, qtt, j);
					const bool up = (lane & k) == 0, low = (lane & j) == 0;
					const bool take = (low == up) ? better(od, oc, d, cc) : better(d, cc, od, oc);
					if (take) { d = od; cc = oc; qx = ox; qy = oy; qtt = ot; }
				}
			const int ncand = s_cbase[r];
			const int Kk = min(sp.np, ncand);
			// tau rule on the sorted exact distances
			float dn[5];
			dn[0] = __shfl_sync(0xffffffffu, d, 1);
			dn[1] = __shfl_sync(0xffffffffu, d, 2);
			dn[2] = __shfl_sync(0xffffffffu, d, 4);
			dn[3] = __shfl_sync(0xffffffffu, d, 8);
			dn[4] = __shfl_sync(0xffffffffu, d, 16);
			int nS = 1;
			for (int q = 0; q < 5 && 2 * nS <= Kk && dn[q] < sp.tau2; q++) nS *= 2;
			const long long g = s_g[r];
			if (lane == 0) a.nsimp[g] = (uint8_t)nS;
			if (lane < nS) a.idx[g * sp.np + lane] = (uint32_t)(((long long)qtt * T.h + qy) * T.w + qx);
		}
		__syncthreads();
	}
#undef dist
}

template <int PX, int PT>
size_t mixed_smem(const StepParams &sp)
{
	constexpr int WX = kCW + PX - 1, WY = kCH + PX - 1;
	constexpr int WXP = (WX + 1 + 7) / 8 * 8;
	return sizeof(__half) * PT * WY * WXP + sizeof(float) * (PT * WY * kCW + kCH * kCW) +
	       sizeof(float) * kRefs * sp.wx * sp.wx;
}

template <int PX, int PT>
cudaError_t launch_mixed_t(const Image &src, const StepParams &sp, const MixedArgs &a, int nsm, cudaStream_t st)
{
	const size_t smem = mixed_smem<PX, PT>(sp);
	cudaError_t e = cudaFuncSetAttribute(search_mixed_kernel<PX, PT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
	if (e != cudaSuccess) return e;
	int per_sm = 0;
	e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, search_mixed_kernel<PX, PT>, kThreads, smem);
	if (e != cudaSuccess) return e;
	long long nb = (long long)nsm * (per_sm < 1 ? 1 : per_sm);
	if (nb > a.nblocks) nb = a.nblocks;
	search_mixed_kernel<PX, PT><<<(int)nb, kThreads, smem, st>>>(src, sp, a);
	return cudaGetLastError();
}

}  // namespace

// First group of every 4x4 block of reference positions of one frame.
void mixed_blocks(const std::vector<Tile> &tiles, std::vector<long long> &out)
{
	out.clear();
	for (const Tile &T : tiles)
		for (int f = 0; f < T.nf; f++)
			for (int y = 0; y < T.ny; y += kBY)
				for (int x = 0; x < T.nx; x += kBX)
					out.push_back(T.g0 + ((long long)f * T.ny + y) * T.nx + x);
}

bool mixed_supported(const StepParams &sp)
{
	return sp.chn_search == 1 && sp.px * sp.px * sp.pt == 64 && sp.wx <= 32 && sp.np <= kTop &&
	       (sp.px == 4 || sp.px == 8);
}

cudaError_t launch_search_mixed(const Image &src, const Tile *tiles, int ntiles, const int *grid,
                                const uint32_t *traj, const StepParams &sp, const long long *blocks,
                                long long nblocks, uint8_t *nsimp, uint32_t *idx, int nsm, cudaStream_t st)
{
	if (nblocks <= 0) return cudaSuccess;
	MixedArgs a;
	a.tiles = tiles;
	a.ntiles = ntiles;
	a.grid = grid;
	a.traj = traj;
	a.nfm = search_frames_max(sp);
	a.blocks = blocks;
	a.nblocks = nblocks;
	a.nsimp = nsimp;
	a.idx = idx;
	return sp.px == 4 ? launch_mixed_t<4, 4>(src, sp, a, nsm, st) : launch_mixed_t<8, 1>(src, sp, a, nsm, st);
}

}  // namespace bm4dof
