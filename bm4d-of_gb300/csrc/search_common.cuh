// search_common.cuh -- device helpers shared by the exhaustive and the
// predictive patch searches (search.cu, search_vbm3d.cu): libstdc++'s heap
// selection, the group's position and temporal range, and the column-strip
// distance loop.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

#include "common.cuh"

namespace bm4dof {

namespace {

constexpr int kR = 7;                  // candidates per thread along y (column strips)

// Packed pair arithmetic (sm_100 and later): sub.rn.f32x2 and mul.rn.f32x2
// round each lane exactly as the scalar instructions do.  The sums stay
// scalar: a packed multiply feeding a packed add is contracted by the
// assembler into a fused multiply-add, which rounds once instead of twice
// (about 30 % of 64-term chains differed in the last bit), while a packed
// multiply whose lanes are added one at a time matched the scalar chain in
// every case.  So the two squared differences are formed packed and added in
// the reference's order.
__device__ __forceinline__ unsigned long long f2pack(float lo, float hi)
{
	unsigned long long r;
	asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
	return r;
}

__device__ __forceinline__ void sqdiff2(float r0, float r1, float v0, float v1, float &m0, float &m1)
{
	unsigned long long d, m;
	asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(f2pack(r0, r1)), "l"(f2pack(v0, v1)));
	asm("mul.rn.f32x2 %0, %1, %1;" : "=l"(m) : "l"(d));
	asm("mov.b64 {%0, %1}, %2;" : "=f"(m0), "=f"(m1) : "l"(m));
}

// libstdc++ __adjust_heap + __push_heap for a max-heap on distance ("less"
// comparator comparaisonFirst, src/utils/utilities.cpp:35-41).
__device__ void adjust_heap(float *hd, int *hi, int hole, int len, float vd, int vi)
{
	const int top = hole;
	int second = hole;
	while (second < (len - 1) / 2) {
		second = 2 * (second + 1);
		if (hd[second] < hd[second - 1]) second--;
		hd[hole] = hd[second];
		hi[hole] = hi[second];
		hole = second;
	}
	if ((len & 1) == 0 && second == (len - 2) / 2) {
		second = 2 * (second + 1);
		hd[hole] = hd[second - 1];
		hi[hole] = hi[second - 1];
		hole = second - 1;
	}
	int parent = (hole - 1) / 2;
	while (hole > top && hd[parent] < vd) {
		hd[hole] = hd[parent];
		hi[hole] = hi[parent];
		hole = parent;
		parent = (hole - 1) / 2;
	}
	hd[hole] = vd;
	hi[hole] = vi;
}

__device__ void make_heap(float *hd, int *hi, int len)
{
	if (len < 2) return;
	for (int parent = (len - 2) / 2;; parent--) {
		adjust_heap(hd, hi, parent, len, hd[parent], hi[parent]);
		if (parent == 0) return;
	}
}

__device__ void sort_heap(float *hd, int *hi, int len)
{
	for (int last = len; last > 1;) {
		--last;
		const float vd = hd[last];
		const int vi = hi[last];
		hd[last] = hd[0];
		hi[last] = hi[0];
		adjust_heap(hd, hi, 0, last, vd, vi);
	}
}

__device__ __forceinline__ void group_position(const Tile &T, const int *grid, long long g, int &x, int &y,
                                               int &t)
{
	const long long local = g - T.g0;
	x = grid[T.gx + (int)(local % T.nx)];
	y = grid[T.gy + (int)((local / T.nx) % T.ny)];
	t = grid[T.gf + (int)(local / ((long long)T.nx * T.ny))];
}

__device__ __forceinline__ void temporal_range(const StepParams &sp, int t, int &t0, int &t1)
{
	const int shift_t = min(0, t - sp.wtb) + max(0, t + sp.wtf - sp.F + sp.pt);
	t0 = max(0, t - sp.wtb - shift_t);
	t1 = min(sp.F - sp.pt, t + sp.wtf - shift_t);
}

__device__ __forceinline__ int visit_frame(int ii, int t, int t1)
{
	// visiting order: t, t+1..t1, t-1..t0 (nldct.cpp:1195-1198)
	return ii == 0 ? t : (ii <= t1 - t ? t + ii : t - (ii - (t1 - t)));
}

// Distances of R vertically adjacent candidates (one column of the window,
// rows r = 0..R-1 below `col`, which points at candidate row 0, patch frame
// 0, channel 0).  Each image row is loaded once and feeds every candidate
// whose patch covers it; per candidate the terms still follow the reference's
// (c, ht, hy, hx) order.  Consecutive lanes take consecutive columns, so each
// warp-wide load touches one or two contiguous row segments.  With the
// reference patch in shared memory (ref_s, 16-byte aligned), small patches
// take one patch frame of it at a time into registers with vector loads.
template <int PX, int PT, bool REFREG, int R>
__device__ __forceinline__ void col_distances(const float *col, size_t rpitch, size_t cpitch, size_t tpitch,
                                              int ymax, int chn, int px_rt, int pt_rt, const float *ref_s,
                                              const float (&ref_r)[(PX > 0 ? PX * PX * PT : 1)], float (&acc)[R])
{
	constexpr int kR = R;   // candidates of the strip
#pragma unroll
	for (int r = 0; r < kR; r++) acc[r] = 0.f;
	if (PX > 0) {
		constexpr int SPC = (PX > 0 ? PX * PX * PT : 1);
		constexpr int Q = PX > 0 ? PX : 1;
		constexpr bool SLICE = !REFREG && Q * Q <= 16;   // one patch frame in registers
		if constexpr (SLICE) {
			// patch frames one at a time (not unrolled: bounded register use)
			for (int c = 0; c < chn; c++)
#pragma unroll 1
				for (int ht = 0; ht < PT; ht++) {
					float rs[Q * Q];
					const float4 *rp = reinterpret_cast<const float4 *>(ref_s + c * SPC + ht * Q * Q);
#pragma unroll
					for (int q = 0; q < Q * Q / 4; q++) {
						const float4 v4 = rp[q];
						rs[4 * q] = v4.x;
						rs[4 * q + 1] = v4.y;
						rs[4 * q + 2] = v4.z;
						rs[4 * q + 3] = v4.w;
					}
					const float *base = col + ht * tpitch + c * cpitch;
#pragma unroll
					for (int yy = 0; yy < kR + Q - 1; yy++) {
						const float *row = base + (size_t)min(yy, ymax) * rpitch;
						float v[Q];
#pragma unroll
						for (int hx = 0; hx < Q; hx++) v[hx] = __ldg(row + hx);
#pragma unroll
						for (int r = 0; r < kR; r++) {
							const int hy = yy - r;
							if (hy >= 0 && hy < Q) {
#pragma unroll
								for (int hx = 0; hx + 1 < Q; hx += 2) {
									float m0, m1;
									sqdiff2(rs[hy * Q + hx], rs[hy * Q + hx + 1], v[hx], v[hx + 1], m0, m1);
									acc[r] = __fadd_rn(__fadd_rn(acc[r], m0), m1);
								}
								if (Q & 1) {
									const float d = __fsub_rn(rs[hy * Q + Q - 1], v[Q - 1]);
									acc[r] = __fadd_rn(acc[r], __fmul_rn(d, d));
								}
							}
						}
					}
				}
		} else {
			for (int c = 0; c < chn; c++)
#pragma unroll
				for (int ht = 0; ht < (PT > 0 ? PT : 1); ht++)
#pragma unroll
					for (int yy = 0; yy < kR + Q - 1; yy++) {
						const float *row = col + ht * tpitch + c * cpitch + (size_t)min(yy, ymax) * rpitch;
						float v[Q];
#pragma unroll
						for (int hx = 0; hx < Q; hx++) v[hx] = __ldg(row + hx);
#pragma unroll
						for (int r = 0; r < kR; r++) {
							const int hy = yy - r;
							if (hy >= 0 && hy < Q) {
#pragma unroll
								for (int hx = 0; hx < Q; hx++) {
									const int kk = (ht * Q + hy) * Q + hx;
									const float rv = REFREG ? ref_r[kk] : ref_s[c * SPC + kk];
									const float d = __fsub_rn(rv, v[hx]);
									acc[r] = __fadd_rn(acc[r], __fmul_rn(d, d));
								}
							}
						}
					}
		}
	} else {
		const int px = px_rt, pt = pt_rt, spc = px * px * pt;
		for (int c = 0; c < chn; c++)
			for (int ht = 0; ht < pt; ht++)
				for (int yy = 0; yy < kR + px - 1; yy++) {
					const float *row = col + ht * tpitch + c * cpitch + (size_t)min(yy, ymax) * rpitch;
#pragma unroll
					for (int r = 0; r < kR; r++) {
						const int hy = yy - r;
						if (hy < 0 || hy >= px) continue;
						for (int hx = 0; hx < px; hx++) {
							const float d = __fsub_rn(ref_s[c * spc + (ht * px + hy) * px + hx], __ldg(row + hx));
							acc[r] = __fadd_rn(acc[r], __fmul_rn(d, d));
						}
					}
				}
	}
}

}  // namespace

}  // namespace bm4dof
