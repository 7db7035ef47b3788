// search_vbm3d.cu -- the predictive patch search of the reference built with
// VBM3D_SEARCH (src/core/nldct.cpp:892-1130 step 1, 1351-1589 step 2), bit
// for bit:
//   * frames visited pt, pt+1 .. t1, then pt-1 .. t0 (nldct.cpp:950-956);
//   * in frame pt one sizeSearchWindow window around the reference patch; in
//     every other frame one sizeSearchWindowPred window around each of the
//     previous frame's nSimilarPatchesPred best matches moved along the flow
//     (rounded half away from zero, clamped), all windows shifted into the
//     frame (975-1028);
//   * the union of those windows in window, then raster order, each position
//     once (the unordered_set of 1031-1035): a position is new when no
//     earlier window of the frame contains it;
//   * distances on channel 0 in the reference's (ht, hy, hx) order with one
//     rounded multiply and one rounded add per term; in step 2 the basic
//     estimate's channel 0 is summed once per channel (1501-1506); minus
//     dsub*dsub*255 at the reference position of every frame (1047);
//   * per frame the nSimilarPatchesPred nearest by libstdc++'s partial_sort,
//     which become the next frame's trajectories and join the pool
//     (1055-1072); the nSimilarPatches nearest of the pool by partial_sort,
//     then the power-of-two truncation by tau (1075-1104).
//
// One warp per group: the frames depend on one another through the
// trajectories, and a frame holds few candidates (21x21 in frame pt, at most
// nSimilarPatchesPred 5x5 windows elsewhere), so the warp walks the frames
// while the other warps of the SM hide its latency.  Frame pt's window is
// computed in column strips (each row of the image loaded once for kR
// vertically adjacent candidates); the predicted windows one candidate per
// lane.  Selections, when the nearest are distinct: repeated warp minima
// (few nearest) or a warp bitonic sort (more nearest, up to 64 candidates);
// else an exact replay of libstdc++'s heap selection by one lane.
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdlib>

#include "common.cuh"
#include "internal.hpp"
#include "search_common.cuh"

namespace bm4dof {

namespace {

constexpr int kWarps = 4;              // groups in flight per CTA, one per warp
constexpr unsigned kFull = 0xffffffffu;

__host__ __device__ __forceinline__ int al4(int n) { return (n + 3) & ~3; }

struct VArgs {
	const Tile *tiles;
	int ntiles;
	const int *grid;
	long long g_begin, g_end;
	uint8_t *nsimp;
	uint32_t *idx;
	int reps;          // passes over channel 0: 1 in step 1, C in step 2
	int cap_win;       // most candidates of one frame (two predicted frames)
	int cap_pred;      // most candidates of one predicted frame
	int cap_pool;      // nSimilarPatchesPred * frames of the temporal range
	int per_warp;      // floats of shared memory per warp
};

// Per-warp shared memory, in floats from the warp's base.
struct Layout {
	int ref, dist, pos, pool_d, pool_i, sel_d, sel_i, hd, hi, total;
	__host__ __device__ Layout(int reps, int spc, int cap_win, int cap_pool)
	{
		ref = 0;
		dist = ref + al4(reps * spc);
		pos = dist + al4(cap_win);
		pool_d = pos + al4(cap_win);
		pool_i = pool_d + al4(cap_pool);
		sel_d = pool_i + al4(cap_pool);
		sel_i = sel_d + kMaxNp;
		hd = sel_i + kMaxNp;
		hi = hd + kMaxNp;
		total = hi + kMaxNp;
	}
};

__device__ __forceinline__ bool lex_less(float a, int ia, float b, int ib)
{
	return a < b || (a == b && ia < ib);
}

// Ascending sort of 64 (distance, position) pairs held two per lane
// (element e = lane + 32*h), ties by position.
__device__ __forceinline__ void warp_sort64(float &d0, int &i0, float &d1, int &i1)
{
	const int lane = threadIdx.x & 31;
	for (int k = 2; k <= 64; k <<= 1)
		for (int j = k >> 1; j > 0; j >>= 1) {
			if (j == 32) {
				// k == 64: the pair (lane, lane + 32), ascending
				if (lex_less(d1, i1, d0, i0)) {
					const float td = d0; d0 = d1; d1 = td;
					const int ti = i0; i0 = i1; i1 = ti;
				}
			} else {
				const float od0 = __shfl_xor_sync(kFull, d0, j), od1 = __shfl_xor_sync(kFull, d1, j);
				const int oi0 = __shfl_xor_sync(kFull, i0, j), oi1 = __shfl_xor_sync(kFull, i1, j);
				const bool low = (lane & j) == 0;
				const bool up0 = (lane & k) == 0, up1 = ((lane + 32) & k) == 0;
				// the lower element of an ascending pair keeps the smaller one
				const bool take0 = (low == up0) ? lex_less(od0, oi0, d0, i0) : lex_less(d0, i0, od0, oi0);
				const bool take1 = (low == up1) ? lex_less(od1, oi1, d1, i1) : lex_less(d1, i1, od1, oi1);
				if (take0) { d0 = od0; i0 = oi0; }
				if (take1) { d1 = od1; i1 = oi1; }
			}
		}
}

// Ascending sort of 32 (distance, position) pairs, one per lane.
__device__ __forceinline__ void warp_sort32(float &d0, int &i0)
{
	const int lane = threadIdx.x & 31;
#pragma unroll
	for (int k = 2; k <= 32; k <<= 1)
#pragma unroll
		for (int j = k >> 1; j > 0; j >>= 1) {
			const float od = __shfl_xor_sync(kFull, d0, j);
			const int oi = __shfl_xor_sync(kFull, i0, j);
			const bool low = (lane & j) == 0, up = (lane & k) == 0;
			const bool take = (low == up) ? lex_less(od, oi, d0, i0) : lex_less(d0, i0, od, oi);
			if (take) { d0 = od; i0 = oi; }
		}
}

constexpr int kRoundsMaxK = 5;   // repeated minima up to this K, else a bitonic sort

// The K nearest of d[0..n) (1 <= K <= min(n, kMaxNp)) in the order
// std::partial_sort(d, d + K, d + n) leaves them: distances to od[0..K),
// positions in d to oi[0..K).  `nan`: this lane saw a NaN among the
// distances.  Called by all 32 lanes of a warp.
__device__ void warp_partial_sort(const float *d, int n, int K, bool nan, float *od, int *oi, float *hd, int *hi)
{
	const int lane = threadIdx.x & 31;
	const float inf = __int_as_float(0x7f800000);
	bool ok = !__any_sync(kFull, nan);
	if (ok && n <= 32 && K > kRoundsMaxK) {
		float d0 = lane < n ? d[lane] : inf;
		int i0 = lane < n ? lane : 0x7fffffff;
		warp_sort32(d0, i0);
		const float next = __shfl_down_sync(kFull, d0, 1);
		ok = !__any_sync(kFull, lane < K && lane + 1 < n && next == d0);
		if (ok && lane < K) { od[lane] = d0; oi[lane] = i0; }
	} else if (ok && n <= 64 && K > kRoundsMaxK) {
		float d0 = lane < n ? d[lane] : inf, d1 = lane + 32 < n ? d[lane + 32] : inf;
		int i0 = lane < n ? lane : 0x7fffffff, i1 = lane + 32 < n ? lane + 32 : 0x7fffffff;
		warp_sort64(d0, i0, d1, i1);
		// distinct among the first K, and the K-th strictly below the next
		const float n0 = __shfl_down_sync(kFull, d0, 1);
		const float f1 = __shfl_sync(kFull, d1, 0);
		const float n1 = __shfl_down_sync(kFull, d1, 1);
		const float next0 = lane == 31 ? f1 : n0;   // element lane + 1
		const bool bad0 = lane < K && lane + 1 < n && next0 == d0;
		const bool bad1 = lane + 32 < K && lane + 33 < n && n1 == d1;
		ok = !__any_sync(kFull, bad0 || bad1);
		if (ok) {
			if (lane < K) { od[lane] = d0; oi[lane] = i0; }
			if (lane + 32 < K) { od[lane + 32] = d1; oi[lane + 32] = i1; }
		}
	} else if (ok) {
		// K + 1 rounds of the warp minimum in (distance, position) order
		float pv = -inf;
		int pi = -1;
		const int rounds = K < n ? K + 1 : K;
		for (int r = 0; r < rounds && ok; r++) {
			float bv = inf;
			int bi = 0x7fffffff;
			for (int i = lane; i < n; i += 32) {
				const float v = d[i];
				if (lex_less(pv, pi, v, i) && lex_less(v, i, bv, bi)) { bv = v; bi = i; }
			}
#pragma unroll
			for (int o = 16; o > 0; o >>= 1) {
				const float ov = __shfl_xor_sync(kFull, bv, o);
				const int oi2 = __shfl_xor_sync(kFull, bi, o);
				if (lex_less(ov, oi2, bv, bi)) { bv = ov; bi = oi2; }
			}
			if (r > 0 && !(bv > pv)) ok = false;   // a tie: the heap order decides
			if (ok && r < K && lane == 0) { od[r] = bv; oi[r] = bi; }
			pv = bv;
			pi = bi;
		}
	}
	if (!ok) {
		// libstdc++: __make_heap(first, middle); __pop_heap for every later
		// element below the top; __sort_heap(first, middle)
		if (lane == 0) {
			for (int i = 0; i < K; i++) { hd[i] = d[i]; hi[i] = i; }
			make_heap(hd, hi, K);
		}
		__syncwarp();
		float top = hd[0];
		for (int base = K; base < n; base += 32) {
			const int i = base + lane;
			const float dv = i < n ? d[i] : 0.f;
			unsigned m = __ballot_sync(kFull, i < n && dv < top);
			while (m) {
				const int j = __ffs(m) - 1;
				if (lane == 0) adjust_heap(hd, hi, 0, K, d[base + j], base + j);
				__syncwarp();
				top = hd[0];
				m &= ~((2u << j) - 1u);
				m &= __ballot_sync(kFull, i < n && dv < top);
			}
		}
		if (lane == 0) {
			sort_heap(hd, hi, K);
			for (int i = 0; i < K; i++) { od[i] = hd[i]; oi[i] = hi[i]; }
		}
	}
	__syncwarp();
}

// One half-warp's selection (lanes 16h .. 16h+15, both halves call it
// together, each on its own frame): the K nearest of d[0..n) by K + 1 rounds
// of the half's minimum over (distance, position), valid when they are
// pairwise distinct and strictly below the rest.  Returns false on the
// half's lanes when a tie or a NaN (`nan`: this lane saw one) leaves the
// order to partial_sort's heap mechanics.
__device__ bool half_select(const float *d, int n, int K, bool nan, float *od, int *oi)
{
	const int hl = threadIdx.x & 15;
	const float inf = __int_as_float(0x7f800000);
	const unsigned nm = __ballot_sync(kFull, nan);
	bool ok = ((nm >> (threadIdx.x & 16)) & 0xffffu) == 0u;
	float pv = -inf;
	int pi = -1;
	for (int r = 0; r <= K; r++) {
		float bv = inf;
		int bi = 0x7fffffff;
		for (int i = hl; i < n; i += 16) {
			const float v = d[i];
			if (lex_less(pv, pi, v, i) && lex_less(v, i, bv, bi)) { bv = v; bi = i; }
		}
#pragma unroll
		for (int o = 8; o > 0; o >>= 1) {
			const float ov = __shfl_xor_sync(kFull, bv, o);
			const int oi2 = __shfl_xor_sync(kFull, bi, o);
			if (lex_less(ov, oi2, bv, bi)) { bv = ov; bi = oi2; }
		}
		if (r > 0 && r < n && !(bv > pv)) ok = false;
		if (ok && r < K && hl == 0) { od[r] = bv; oi[r] = bi; }
		pv = bv;
		pi = bi;
	}
	__syncwarp();
	return ok;
}

// Squared distances of the reference patch (ref, `reps` copies of channel 0
// at stride spc) to the patches at p0 and p1 (channel 0 of each candidate's
// first row and frame), terms in the reference's order; the two sums run
// interleaved so that each hides the other's add latency.
template <int PX, int PT>
__device__ __forceinline__ void patch_distance2(const float *p0, const float *p1, size_t rpitch, size_t tpitch,
                                                const float *ref, int reps, int px_rt, int pt_rt, float &a0,
                                                float &a1)
{
	// compile-time extents when the shape is a template argument (full
	// unrolling of a row), run-time ones otherwise
	const int px = PX > 0 ? PX : px_rt, pt = PX > 0 ? PT : pt_rt, spc = px * px * pt;
	constexpr bool VEC = PX > 0 && PX % 4 == 0;   // reference rows as 16-byte loads
	constexpr int QV = VEC ? PX : 4;
	a0 = 0.f;
	a1 = 0.f;
	for (int r = 0; r < reps; r++) {
		const float *rr = ref + r * spc;
		// one patch frame at a time (bounded register use)
#pragma unroll 1
		for (int tt = 0; tt < pt; tt++) {
#pragma unroll
			for (int yy = 0; yy < (PX > 0 ? PX : px); yy++) {
				const size_t off = tt * tpitch + yy * rpitch;
				const float *rf = rr + (tt * px + yy) * px;
				float rrow[QV];
				if (VEC) {
#pragma unroll
					for (int q = 0; q < QV / 4; q++) {
						const float4 r4 = reinterpret_cast<const float4 *>(rf)[q];
						rrow[4 * q] = r4.x;
						rrow[4 * q + 1] = r4.y;
						rrow[4 * q + 2] = r4.z;
						rrow[4 * q + 3] = r4.w;
					}
				}
#pragma unroll
				for (int xx = 0; xx < (PX > 0 ? PX : px); xx++) {
					const float rv = VEC ? rrow[xx % QV] : rf[xx];
					float m0, m1;
					sqdiff2(rv, rv, __ldg(p0 + off + xx), __ldg(p1 + off + xx), m0, m1);
					a0 = __fadd_rn(a0, m0);
					a1 = __fadd_rn(a1, m1);
				}
			}
		}
	}
}

// Window of one centre, shifted (not clipped) into the frame
// (nldct.cpp:1017-1027): [x0, x0 + nx) x [y0, y0 + ny).
__device__ __forceinline__ void window_box(int cx, int cy, int sw, int tw, int th, int px, int &x0, int &y0,
                                           int &nx, int &ny)
{
	const int hw = (sw - 1) / 2;
	const int shx = min(0, cx - hw) + max(0, cx + hw - tw + px);
	const int shy = min(0, cy - hw) + max(0, cy + hw - th + px);
	x0 = max(0, cx - hw - shx);
	y0 = max(0, cy - hw - shy);
	nx = max(0, min(tw - px, cx + hw - shx) - x0 + 1);
	ny = max(0, min(th - px, cy + hw - shy) - y0 + 1);
}

// The sizeSearchWindowPred window of frame qt around a match `id` (tile
// index) of frame qt - dir, moved along the flow at the match, rounded half
// away from zero and clamped to the tile (nldct.cpp:978-993).
__device__ __forceinline__ void predicted_window(const Image &ffl, const Image &bfl, const Tile &T,
                                                 const StepParams &sp, uint32_t id, int qt, int dir, int &x0,
                                                 int &y0, int &nx, int &ny)
{
	const int cx0 = (int)(id % (uint32_t)T.w);
	const int cy0 = (int)((id / (uint32_t)T.w) % (uint32_t)T.h);
	const int ct0 = qt - dir;
	float ux = 0.f, uy = 0.f;
	if (sp.use_flow) {
		const Image &fl = dir > 0 ? ffl : bfl;
		ux = fl.p[fl.at(T.ox + cx0, T.oy + cy0, ct0, 0)];
		uy = fl.p[fl.at(T.ox + cx0, T.oy + cy0, ct0, 1)];
	}
	const int cx = (int)fmaxf(0.f, fminf(__fsub_rn((float)T.w, 1.f), roundf(__fadd_rn((float)cx0, ux))));
	const int cy = (int)fmaxf(0.f, fminf(__fsub_rn((float)T.h, 1.f), roundf(__fadd_rn((float)cy0, uy))));
	window_box(cx, cy, sp.wxp, T.w, T.h, sp.px, x0, y0, nx, ny);
}

template <int PX, int PT, int MINB>
__global__ void __launch_bounds__(32 * kWarps, MINB)
search_vbm3d_kernel(Image src, Image ffl, Image bfl, StepParams sp, VArgs a)
{
	extern __shared__ __align__(16) float smem_v[];
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	float *ws = smem_v + (size_t)warp * a.per_warp;
	const Layout lo(a.reps, sp.spc, a.cap_win, a.cap_pool);
	float *ref = ws + lo.ref;
	float *dist = ws + lo.dist;
	uint32_t *pos = reinterpret_cast<uint32_t *>(ws + lo.pos);
	float *pool_d = ws + lo.pool_d;
	uint32_t *pool_i = reinterpret_cast<uint32_t *>(ws + lo.pool_i);
	float *sel_d = ws + lo.sel_d;
	int *sel_i = reinterpret_cast<int *>(ws + lo.sel_i);
	float *hd = ws + lo.hd;
	int *hi = reinterpret_cast<int *>(ws + lo.hi);

	const int px = sp.px, spc = sp.spc, npf = sp.npf;
	const size_t rpitch = src.P, tpitch = src.plane() * src.C;
	float ref_r[(PX > 0 ? PX * PX * PT : 1)];   // unused: the reference patch is read from shared memory

	for (long long g = a.g_begin + (long long)blockIdx.x * kWarps + warp; g < a.g_end;
	     g += (long long)gridDim.x * kWarps) {
		const Tile T = a.tiles[tile_of(a.tiles, a.ntiles, g)];
		int x, y, t, t0, t1;
		group_position(T, a.grid, g, x, y, t);
		temporal_range(sp, t, t0, t1);
		const int nwt = t1 - t0 + 1;
		// reference patch, channel 0, `reps` copies
		for (int k = lane; k < spc * a.reps; k += 32) {
			const int r = k % spc;
			const int ht = r / (px * px), hy = (r / px) % px, hx = r % px;
			ref[k] = src.p[src.at(T.ox + x + hx, T.oy + y + hy, t + ht, 0)];
		}
		__syncwarp();
		// with at most 16 matches per frame the forward and backward frames run
		// in pairs, one per half-warp (below); else one frame at a time here
		const bool paired = npf <= 16;
		for (int ii = 0; ii < (paired ? 1 : nwt); ii++) {
			const int qt = visit_frame(ii, t, t1);
			int ncand, fx0 = 0, fy0 = 0, fnx = 1;
			bool nan;
			if (ii == 0) {
				// frame pt: one full window, column strips of kR candidates
				int fny;
				window_box(x, y, sp.wx, T.w, T.h, px, fx0, fy0, fnx, fny);
				ncand = fnx * fny;
				const int nit = fnx * ((fny + kR - 1) / kR);
				nan = false;
				for (int it = lane; it < nit; it += 32) {
					const int rb = it / fnx, cx = it - rb * fnx, qy0 = rb * kR;
					float acc[kR];
					const float *colp = src.p + src.at(T.ox + fx0 + cx, T.oy + fy0 + qy0, qt, 0);
					col_distances<PX, PT, false>(colp, rpitch, 0, tpitch, fny - qy0 + px - 2, a.reps, px, sp.pt,
					                             ref, ref_r, acc);
#pragma unroll
					for (int r = 0; r < kR; r++)
						if (qy0 + r < fny) {
							float dv = acc[r];
							if (fx0 + cx == x && fy0 + qy0 + r == y) dv = __fsub_rn(dv, sp.dsub_bias);
							nan |= dv != dv;
							dist[(qy0 + r) * fnx + cx] = dv;
						}
				}
			} else {
				// centres: the previous frame's matches moved along the flow
				const int dir = qt > t ? 1 : -1;
				const int prev = (qt == t - 1) ? 0 : ii - 1;
				int bx0 = 0, by0 = 0, bnx = 0, bny = 0;
				if (lane < npf)
					predicted_window(ffl, bfl, T, sp, pool_i[prev * npf + lane], qt, dir, bx0, by0, bnx, bny);
				// union of the windows in window, then raster order
				ncand = 0;
				for (int w = 0; w < npf; w++) {
					const int wx0 = __shfl_sync(kFull, bx0, w), wy0 = __shfl_sync(kFull, by0, w);
					const int wnx = __shfl_sync(kFull, bnx, w), wny = __shfl_sync(kFull, bny, w);
					const int nb = wnx * wny;
					for (int base = 0; base < nb; base += 32) {
						const int p = base + lane;
						const int qx = p < nb ? wx0 + p % wnx : 0, qy = p < nb ? wy0 + p / wnx : 0;
						bool fresh = p < nb;
						for (int o = 0; o < w; o++) {
							const int ox0 = __shfl_sync(kFull, bx0, o), oy0 = __shfl_sync(kFull, by0, o);
							const int onx = __shfl_sync(kFull, bnx, o), ony = __shfl_sync(kFull, bny, o);
							if (qx >= ox0 && qx < ox0 + onx && qy >= oy0 && qy < oy0 + ony) fresh = false;
						}
						const unsigned m = __ballot_sync(kFull, fresh);
						if (fresh) pos[ncand + __popc(m & ((1u << lane) - 1u))] = (uint32_t)qx | ((uint32_t)qy << 16);
						ncand += __popc(m);
					}
				}
				__syncwarp();
				nan = false;
				// candidates c and c + 32 of a lane computed together
				for (int c = lane; c < ncand; c += 64) {
					const bool two = c + 32 < ncand;
					const uint32_t q0 = pos[c], q1 = two ? pos[c + 32] : q0;
					const int qx0 = (int)(q0 & 0xffffu), qy0 = (int)(q0 >> 16);
					const int qx1 = (int)(q1 & 0xffffu), qy1 = (int)(q1 >> 16);
					float d0, d1;
					patch_distance2<PX, PT>(src.p + src.at(T.ox + qx0, T.oy + qy0, qt, 0),
					                        src.p + src.at(T.ox + qx1, T.oy + qy1, qt, 0), rpitch, tpitch, ref,
					                        a.reps, px, sp.pt, d0, d1);
					if (qx0 == x && qy0 == y) d0 = __fsub_rn(d0, sp.dsub_bias);
					if (qx1 == x && qy1 == y) d1 = __fsub_rn(d1, sp.dsub_bias);
					nan |= d0 != d0;
					dist[c] = d0;
					if (two) {
						nan |= d1 != d1;
						dist[c + 32] = d1;
					}
				}
			}
			__syncwarp();
			// the npf nearest of this frame join the pool, in partial_sort order
			warp_partial_sort(dist, ncand, npf, nan, sel_d, sel_i, hd, hi);
			if (lane < npf) {
				const int c = sel_i[lane];
				int qx, qy;
				if (ii == 0) {
					qy = fy0 + c / fnx;
					qx = fx0 + c % fnx;
				} else {
					const uint32_t q = pos[c];
					qx = (int)(q & 0xffffu);
					qy = (int)(q >> 16);
				}
				pool_d[ii * npf + lane] = sel_d[lane];
				pool_i[ii * npf + lane] = (uint32_t)(((long long)qt * T.h + qy) * T.w + qx);
			}
			__syncwarp();
		}
		if (paired) {
			// forward frame t + k on lanes 0-15 and backward frame t - k on lanes
			// 16-31: centres, union lists and selections side by side, distances
			// over both lists with the whole warp; pool slots in visiting order
			const int nf = t1 - t, nb = t - t0;
			const int h = lane >> 4, hl = lane & 15;
			const int kmax = nf > nb ? nf : nb;
			uint32_t *hpos = pos + h * a.cap_pred;
			float *hdist = dist + h * a.cap_pred;
			for (int k = 1; k <= kmax; k++) {
				const bool act = h == 0 ? k <= nf : k <= nb;
				const int dir = h == 0 ? 1 : -1;
				const int qt = t + dir * k;
				const int slot = h == 0 ? k : nf + k;
				const int prev = h == 0 ? k - 1 : (k == 1 ? 0 : nf + k - 1);
				int bx0 = 0, by0 = 0, bnx = 0, bny = 0;
				if (act && hl < npf)
					predicted_window(ffl, bfl, T, sp, pool_i[prev * npf + hl], qt, dir, bx0, by0, bnx, bny);
				// each half's union, 16 positions per ballot
				int cnt = 0;
				for (int w = 0; w < npf; w++) {
					const int sl = (h << 4) + w;
					const int wx0 = __shfl_sync(kFull, bx0, sl), wy0 = __shfl_sync(kFull, by0, sl);
					const int wnx = __shfl_sync(kFull, bnx, sl), wny = __shfl_sync(kFull, bny, sl);
					const int nbw = wnx * wny;
					const int nbo = __shfl_xor_sync(kFull, nbw, 16);
					const int nbmax = nbw > nbo ? nbw : nbo;
					for (int base = 0; base < nbmax; base += 16) {
						const int p = base + hl;
						const bool in = p < nbw;
						const int qx = in ? wx0 + p % wnx : 0, qy = in ? wy0 + p / wnx : 0;
						bool fresh = in;
						for (int o = 0; o < w; o++) {
							const int so = (h << 4) + o;
							const int ox0 = __shfl_sync(kFull, bx0, so), oy0 = __shfl_sync(kFull, by0, so);
							const int onx = __shfl_sync(kFull, bnx, so), ony = __shfl_sync(kFull, bny, so);
							if (qx >= ox0 && qx < ox0 + onx && qy >= oy0 && qy < oy0 + ony) fresh = false;
						}
						const unsigned m = (__ballot_sync(kFull, fresh) >> (h << 4)) & 0xffffu;
						if (fresh) hpos[cnt + __popc(m & ((1u << hl) - 1u))] = (uint32_t)qx | ((uint32_t)qy << 16);
						cnt += __popc(m);
					}
				}
				const int nF = __shfl_sync(kFull, cnt, 0), nB = __shfl_sync(kFull, cnt, 16);
				__syncwarp();
				// distances of both lists, candidates c and c + 32 of a lane together
				bool nanF = false, nanB = false;
				const int ntot = nF + nB;
				for (int c = lane; c < ntot; c += 64) {
					const bool two = c + 32 < ntot;
					const int c1 = two ? c + 32 : c;
					const int s0 = c < nF ? 0 : 1, s1 = c1 < nF ? 0 : 1;
					const int j0 = c - s0 * nF, j1 = c1 - s1 * nF;
					const uint32_t q0 = pos[s0 * a.cap_pred + j0], q1 = pos[s1 * a.cap_pred + j1];
					const int qx0 = (int)(q0 & 0xffffu), qy0 = (int)(q0 >> 16);
					const int qx1 = (int)(q1 & 0xffffu), qy1 = (int)(q1 >> 16);
					float d0, d1;
					patch_distance2<PX, PT>(src.p + src.at(T.ox + qx0, T.oy + qy0, s0 ? t - k : t + k, 0),
					                        src.p + src.at(T.ox + qx1, T.oy + qy1, s1 ? t - k : t + k, 0), rpitch,
					                        tpitch, ref, a.reps, px, sp.pt, d0, d1);
					if (qx0 == x && qy0 == y) d0 = __fsub_rn(d0, sp.dsub_bias);
					if (qx1 == x && qy1 == y) d1 = __fsub_rn(d1, sp.dsub_bias);
					dist[s0 * a.cap_pred + j0] = d0;
					if (s0) nanB |= d0 != d0; else nanF |= d0 != d0;
					if (two) {
						dist[s1 * a.cap_pred + j1] = d1;
						if (s1) nanB |= d1 != d1; else nanF |= d1 != d1;
					}
				}
				__syncwarp();
				const int nh = h == 0 ? nF : nB;
				float *hsd = sel_d + (h << 4);
				int *hsi = sel_i + (h << 4);
				const bool fnan = __any_sync(kFull, nanF), bnan = __any_sync(kFull, nanB);
				const bool ok = half_select(hdist, nh, npf, h == 0 ? fnan : bnan, hsd, hsi) || !act;
				// ties or NaN: libstdc++'s heap selection replayed for that frame
				const unsigned bad = __ballot_sync(kFull, !ok);
				if (bad & 0xffffu) warp_partial_sort(dist, nF, npf, true, sel_d, sel_i, hd, hi);
				if (bad & 0xffff0000u)
					warp_partial_sort(dist + a.cap_pred, nB, npf, true, sel_d + 16, sel_i + 16, hd, hi);
				if (act && hl < npf) {
					const uint32_t q = hpos[hsi[hl]];
					const int qx = (int)(q & 0xffffu), qy = (int)(q >> 16);
					pool_d[slot * npf + hl] = hsd[hl];
					pool_i[slot * npf + hl] = (uint32_t)(((long long)qt * T.h + qy) * T.w + qx);
				}
				__syncwarp();
			}
		}
		// the np nearest of the pool, then the tau rule (nldct.cpp:1075-1104)
		const int npool = nwt * npf;
		const int K = min(sp.np, npool);
		bool pnan = false;
		for (int i = lane; i < npool; i += 32) pnan |= pool_d[i] != pool_d[i];
		warp_partial_sort(pool_d, npool, K, pnan, sel_d, sel_i, hd, hi);
		int n = 1;
		while (2 * n <= K && sel_d[n] < sp.tau2) n *= 2;
		if (lane == 0) a.nsimp[g] = (uint8_t)n;
		if (lane < n) a.idx[g * sp.np + lane] = pool_i[sel_i[lane]];
		__syncwarp();
	}
}

template <int PX, int PT, int MINB = 1>
cudaError_t launch_t(const Image &src, const Image &ffl, const Image &bfl, const StepParams &sp, const VArgs &a,
                     int nsm, cudaStream_t st)
{
	auto kern = search_vbm3d_kernel<PX, PT, MINB>;
	const size_t smem = sizeof(float) * (size_t)a.per_warp * kWarps;
	cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
	if (e != cudaSuccess) return e;
	int per_sm = 0;
	e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 32 * kWarps, smem);
	if (e != cudaSuccess) return e;
	const long long n = a.g_end - a.g_begin;
	long long blocks = (long long)nsm * (per_sm < 1 ? 1 : per_sm);
	blocks = blocks < (n + kWarps - 1) / kWarps ? blocks : (n + kWarps - 1) / kWarps;
	kern<<<(int)blocks, 32 * kWarps, smem, st>>>(src, ffl, bfl, sp, a);
	return cudaGetLastError();
}

int window_count(int sw, int extent, int px)
{
	const int full = 2 * ((sw - 1) / 2) + 1;
	const int room = extent - px + 1;
	return full < room ? full : room;
}

}  // namespace

bool vbm3d_check(const StepParams &sp, const std::vector<Tile> &tiles, std::string &why)
{
	if (sp.np <= 1) return true;
	if (sp.npf < 1 || sp.npf > kMaxNp) {
		why = "nSimilarPatchesPred must be between 1 and 32";
		return false;
	}
	for (const Tile &T : tiles) {
		const int first = window_count(sp.wx, T.w, sp.px) * window_count(sp.wx, T.h, sp.px);
		const int pred = window_count(sp.wxp, T.w, sp.px) * window_count(sp.wxp, T.h, sp.px);
		const bool multi = sp.wtf + sp.wtb > 0 && sp.F > sp.pt;
		if (first < sp.npf || (multi && pred < sp.npf)) {
			// the reference reads past its candidate list there
			why = "a search window holds fewer positions than nSimilarPatchesPred";
			return false;
		}
	}
	return true;
}

size_t vbm3d_smem_bytes(const StepParams &sp, int reps)
{
	const int hw = 2 * ((sp.wx - 1) / 2) + 1, hp = 2 * ((sp.wxp - 1) / 2) + 1;
	const int cap_win = hw * hw > 2 * sp.npf * hp * hp ? hw * hw : 2 * sp.npf * hp * hp;
	const Layout lo(reps, sp.spc, cap_win, sp.npf * search_frames_max(sp));
	return sizeof(float) * (size_t)lo.total * kWarps;
}

cudaError_t launch_search_vbm3d(const Image &src, const Image &ffl, const Image &bfl, const Tile *tiles,
                                int ntiles, const int *grid, const StepParams &sp, int reps, long long g_begin,
                                long long g_end, uint8_t *nsimp, uint32_t *idx, int nsm, cudaStream_t st)
{
	if (g_end <= g_begin) return cudaSuccess;
	if (sp.np <= 1) return launch_search(src, tiles, ntiles, grid, nullptr, sp, g_begin, g_end, nsimp, idx,
	                                     nullptr, nsm, st);
	VArgs a;
	a.tiles = tiles;
	a.ntiles = ntiles;
	a.grid = grid;
	a.g_begin = g_begin;
	a.g_end = g_end;
	a.nsimp = nsimp;
	a.idx = idx;
	a.reps = reps;
	const int hw = 2 * ((sp.wx - 1) / 2) + 1, hp = 2 * ((sp.wxp - 1) / 2) + 1;
	a.cap_pred = sp.npf * hp * hp;
	a.cap_win = hw * hw > 2 * a.cap_pred ? hw * hw : 2 * a.cap_pred;
	a.cap_pool = sp.npf * search_frames_max(sp);
	a.per_warp = Layout(reps, sp.spc, a.cap_win, a.cap_pool).total;
	// CTAs per SM for 4x4x4 patches (registers bound the occupancy of this
	// latency-bound kernel); BM4DOF_VBM3D_MINB selects 4, 6 or 8
	static const int minb = [] {
		const char *e = std::getenv("BM4DOF_VBM3D_MINB");
		return e ? std::atoi(e) : 8;
	}();
	if (sp.px == 4 && sp.pt == 4) {
		if (minb == 4) return launch_t<4, 4, 4>(src, ffl, bfl, sp, a, nsm, st);
		if (minb == 6) return launch_t<4, 4, 6>(src, ffl, bfl, sp, a, nsm, st);
		return launch_t<4, 4, 8>(src, ffl, bfl, sp, a, nsm, st);
	}
	if (sp.px == 8 && sp.pt == 1) return launch_t<8, 1, 4>(src, ffl, bfl, sp, a, nsm, st);
	return launch_t<0, 0>(src, ffl, bfl, sp, a, nsm, st);
}

}  // namespace bm4dof
