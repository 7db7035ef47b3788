// search.cu -- flow-guided patch search with exact k-nearest selection.
//
// Restates VideoNLB::estimateSimilarPatchesStep1/2 (src/core/nldct.cpp:1143-1348,
// 1607-1789) on the GPU, bit for bit:
//   * temporal range shifted into the sequence, frames visited pt, pt+1, ..,
//     then pt-1, .. (nldct.cpp:1172-1198);
//   * search centres chained along the flow, rounded half away from zero and
//     clamped (1219-1236); windows shifted, not clipped (1248-1258);
//   * squared L2 distances summed in the reference's order (c, ht, hy, hx) with
//     one rounded multiply and one rounded add per term (1261-1274, 1722-1737);
//   * the k nearest chosen exactly as libstdc++'s std::partial_sort does it
//     (heap select, then sort_heap), so ties keep the reference's order;
//   * the power-of-two truncation by tau (1284-1289).
//
// Kernels:
//   traj_kernel    one thread per group: the flow-chained search centres of
//                  every frame of its temporal range (a short dependent chain
//                  of flow reads, kept out of the distance kernel);
//   search_kernel  one CTA per group at a time: warp 0 lays out the candidate
//                  windows; every thread computes column strips of R (21 or
//                  7) vertically adjacent candidates (lanes on consecutive
//                  columns, window rows read through L1, the reference patch
//                  from shared memory one patch frame at a time into
//                  registers); the distances land in shared memory in the
//                  reference's candidate order; the k nearest are selected by
//                  a bound from the per-thread minima, compaction and a warp
//                  bitonic sort, with an exact replay of the heap selection
//                  when ties make that order ambiguous.
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdlib>
#include <cstring>

#include "common.cuh"
#include "internal.hpp"
#include "search_common.cuh"

namespace bm4dof {

namespace {

constexpr int kThreads = 192;          // 6 warps: the 189 window columns of a 21x21x9 window set in one round

struct FrameWin {
	int qt, rx0, ry0, nx, ny, cbase, ibase;
};

// Search centres of every frame of each group's temporal range, in visiting
// order: traj[g*nfm + ii] = cx | cy << 16 (tile coordinates).
__global__ void traj_kernel(Image ffl, Image bfl, const Tile *__restrict__ tiles, int ntiles,
                            const int *__restrict__ grid, StepParams sp, long long G, int nfm,
                            uint32_t *__restrict__ traj)
{
	for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < G;
	     g += (long long)gridDim.x * blockDim.x) {
		const Tile T = tiles[tile_of(tiles, ntiles, g)];
		int x, y, t, t0, t1;
		group_position(T, grid, g, x, y, t);
		temporal_range(sp, t, t0, t1);
		const int nwt = t1 - t0 + 1;
		int fx = x, fy = y, bx = x, by = y;   // last centres going forward / backward
		for (int ii = 0; ii < nwt; ii++) {
			const int qt = visit_frame(ii, t, t1);
			int cx = x, cy = y;
			if (qt != t) {
				const int dir = qt > t ? 1 : -1;
				const int cx0 = dir > 0 ? fx : bx, cy0 = dir > 0 ? fy : by, ct0 = qt - dir;
				float ux = 0.f, uy = 0.f;
				if (sp.use_flow) {
					const Image &fl = dir > 0 ? ffl : bfl;
					ux = fl.p[fl.at(T.ox + cx0, T.oy + cy0, ct0, 0)];
					uy = fl.p[fl.at(T.ox + cx0, T.oy + cy0, ct0, 1)];
				}
				cx = (int)fmaxf(0.f, fminf(__fsub_rn((float)T.w, 1.f), roundf(__fadd_rn((float)cx0, ux))));
				cy = (int)fmaxf(0.f, fminf(__fsub_rn((float)T.h, 1.f), roundf(__fadd_rn((float)cy0, uy))));
				if (dir > 0) { fx = cx; fy = cy; } else { bx = cx; by = cy; }
			}
			traj[g * nfm + ii] = (uint32_t)cx | ((uint32_t)cy << 16);
		}
	}
}

struct SearchArgs {
	const Tile *tiles;
	int ntiles;
	const int *grid;
	const uint32_t *traj;
	int nfm;
	long long g_begin, g_end;
	const uint32_t *glist;   // when set: the groups glist[0 .. *gcount) instead of [g_begin, g_end)
	const unsigned *gcount;
	uint8_t *nsimp;
	uint32_t *idx;
};

// Window table of one group, one lane per frame of the temporal range
// (warp 0): candidate and column-strip offsets by warp prefix sums.
__device__ void plan_group(const SearchArgs &a, const StepParams &sp, long long g, int R, FrameWin *fw, int &nframes,
                           int &ncand, int &nitems, int &tile, int &gx, int &gy, int &gt)
{
	const int lane = threadIdx.x & 31;
	const int ti = tile_of(a.tiles, a.ntiles, g);
	const Tile T = a.tiles[ti];
	int x, y, t, t0, t1;
	group_position(T, a.grid, g, x, y, t);
	temporal_range(sp, t, t0, t1);
	const int nwt = t1 - t0 + 1;
	const int hw = (sp.wx - 1) / 2;
	FrameWin f = {0, 0, 0, 0, 0, 0, 0};
	int cnt = 0, items = 0;
	if (lane < nwt) {
		const uint32_t c = a.traj[g * a.nfm + lane];
		const int cx = (int)(c & 0xffffu), cy = (int)(c >> 16);
		const int shx = min(0, cx - hw) + max(0, cx + hw - T.w + sp.px);
		const int shy = min(0, cy - hw) + max(0, cy + hw - T.h + sp.px);
		const int rx0 = max(0, cx - hw - shx), ry0 = max(0, cy - hw - shy);
		const int rx1 = min(T.w - sp.px, cx + hw - shx), ry1 = min(T.h - sp.px, cy + hw - shy);
		f.qt = visit_frame(lane, t, t1);
		f.rx0 = rx0;
		f.ry0 = ry0;
		f.nx = max(0, rx1 - rx0 + 1);
		f.ny = max(0, ry1 - ry0 + 1);
		cnt = f.nx * f.ny;
		items = f.nx * ((f.ny + R - 1) / R);
	}
	int ic = cnt, ii = items;
#pragma unroll
	for (int o = 1; o < 32; o <<= 1) {
		const int uc = __shfl_up_sync(0xffffffffu, ic, o), ui = __shfl_up_sync(0xffffffffu, ii, o);
		if (lane >= o) { ic += uc; ii += ui; }
	}
	f.cbase = ic - cnt;
	f.ibase = ii - items;
	if (lane < nwt) fw[lane] = f;
	if (lane == 31) {
		nframes = nwt;
		ncand = ic;
		nitems = ii;
		tile = ti;
		gx = x;
		gy = y;
		gt = t;
	}
}

constexpr int kSelCap = 64;           // candidates the fast selection sorts

struct SelectShared {
	float tmin[kThreads];
	float bound;
	unsigned nsel;
	int has_nan;        // a NaN distance: only the heap replay orders it as the reference does
	float sd[kSelCap];  // candidates under the bound, in no particular order
	int si[kSelCap];
	float od[kMaxNp];   // the K nearest, in partial_sort's order
	int oi[kMaxNp];
	float hd[kMaxNp];
	int hi[kMaxNp];
};

// The k nearest of dist[0..ncand) in std::partial_sort's output order; the
// first K entries of S.od / S.oi receive them, sorted.
//
// Fast path: every thread knows the minimum of the distances it computed; the
// K-th smallest of those minima bounds the K-th smallest distance from above
// (they are K distinct candidates).  All candidates under the bound are
// compacted, and each takes its place in the output from its rank among them
// (ties by candidate index), counted by its own thread.
// When the K smallest are pairwise distinct and strictly below every other
// distance, partial_sort's output is exactly this ascending order.
// Otherwise (exact ties, a NaN, or too many candidates under the bound) warp
// 0 replays libstdc++'s heap selection (__heap_select then __sort_heap) over
// the candidates in order.
__device__ void select_knn(const float *dist, int ncand, int K, float tmin, SelectShared &S)
{
	const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
	S.tmin[tid] = tmin;
	if (tid == 0) {
		S.nsel = 0u;
		S.has_nan = 0;
		S.bound = __int_as_float(0x7f800000);
	}
	__syncthreads();
	if (warp == 0) {
		// K-th smallest of the per-thread minima (repeated warp minimum)
		constexpr int P = kThreads / 32;
		float v[P];
#pragma unroll
		for (int j = 0; j < P; j++) v[j] = S.tmin[lane * P + j];
		float kth = __int_as_float(0x7f800000);
		for (int k = 0; k < K; k++) {
			float m = v[0];
			int mj = 0;
#pragma unroll
			for (int j = 1; j < P; j++)
				if (v[j] < m) { m = v[j]; mj = j; }
			float w = m;
#pragma unroll
			for (int o = 16; o > 0; o >>= 1) w = fminf(w, __shfl_xor_sync(0xffffffffu, w, o));
			kth = w;
			// remove one occurrence of the minimum (lowest lane holding it)
			const unsigned holder = __ballot_sync(0xffffffffu, m == w);
			if (lane == __ffs(holder) - 1) {
#pragma unroll
				for (int j = 0; j < P; j++)
					if (j == mj) v[j] = __int_as_float(0x7f800000);
			}
		}
		if (lane == 0) S.bound = kth;
	}
	__syncthreads();
	const float bound = S.bound;
	int nan = 0;
	for (int i = tid; i < ncand; i += blockDim.x) {
		const float d = dist[i];
		nan |= d != d;
		if (d <= bound) {
			const unsigned s = atomicAdd(&S.nsel, 1u);
			if (s < (unsigned)kSelCap) { S.sd[s] = d; S.si[s] = i; }
		}
	}
	if (__syncthreads_or(nan) && tid == 0) S.has_nan = 1;
	__syncthreads();
	const int n = (int)S.nsel;
	bool ok = n >= K && n <= kSelCap && !S.has_nan;
	if (ok) {
		// each selected candidate's rank among the selected, ties by index
		int bad = 0;
		if (tid < n) {
			const float d = S.sd[tid];
			const int ci = S.si[tid];
			int rank = 0, same = 0;
			for (int j = 0; j < n; j++) {
				const float o = S.sd[j];
				const int oj = S.si[j];
				rank += (o < d || (o == d && oj < ci)) ? 1 : 0;
				same += (o == d && j != tid) ? 1 : 0;
			}
			// one of the K nearest tied with another candidate: the heap decides
			bad = rank < K && same > 0;
			if (rank < K) { S.od[rank] = d; S.oi[rank] = ci; }
		}
		ok = !__syncthreads_or(bad);
	}
	if (!ok) {
		if (warp == 0) {
			// exact replay of libstdc++'s heap selection, candidates in order
			float *hd = S.hd;
			int *hi = S.hi;
			if (lane == 0) {
				for (int i = 0; i < K; i++) { hd[i] = dist[i]; hi[i] = i; }
				make_heap(hd, hi, K);
			}
			__syncwarp();
			float top = hd[0];
			for (int base = K; base < ncand; base += 32) {
				const int i = base + lane;
				const float dv = i < ncand ? dist[i] : 0.f;
				unsigned m = __ballot_sync(0xffffffffu, i < ncand && dv < top);
				while (m) {
					const int j = __ffs(m) - 1;
					if (lane == 0) adjust_heap(hd, hi, 0, K, dist[base + j], base + j);
					__syncwarp();
					top = hd[0];
					m &= ~((2u << j) - 1u);
					m &= __ballot_sync(0xffffffffu, i < ncand && dv < top);
				}
			}
			if (lane == 0) {
				sort_heap(hd, hi, K);
				for (int i = 0; i < K; i++) { S.od[i] = hd[i]; S.oi[i] = hi[i]; }
			}
		}
		__syncthreads();
	}
}

// One CTA handles one group at a time: every thread computes column strips of
// R candidates (window rows read through L1 from the video), then the CTA
// selects the k nearest.  Several CTAs share an SM so that one CTA's
// selection overlaps the others' distance work.
template <int PX, int PT, bool REFREG, int MINB, int R>
__global__ void __launch_bounds__(kThreads, MINB)
search_kernel(Image src, StepParams sp, SearchArgs a)
{
	extern __shared__ __align__(16) float smem_f[];
	float *ref_s = smem_f;                                      // chn * spc, 16-byte aligned
	float *dist = smem_f + ((sp.spc * sp.chn_search + 3) & ~3);
	__shared__ FrameWin fw[kMaxFrames];
	__shared__ int s_nframes, s_ncand, s_nitems, s_tile, s_x, s_y, s_t;
	__shared__ SelectShared S;

	const int tid = threadIdx.x;
	const int chn = sp.chn_search;
	const long long ng = a.glist ? (long long)*a.gcount : a.g_end - a.g_begin;
	for (long long gi = blockIdx.x; gi < ng; gi += gridDim.x) {
		const long long g = a.glist ? (long long)a.glist[gi] : a.g_begin + gi;
		if (tid < 32) plan_group(a, sp, g, R, fw, s_nframes, s_ncand, s_nitems, s_tile, s_x, s_y, s_t);
		__syncthreads();
		const Tile T = a.tiles[s_tile];
		const int nframes = s_nframes;
		float ref_r[(PX > 0 ? PX * PX * PT : 1)];
		if (REFREG) {
#pragma unroll
			for (int k = 0; k < (PX > 0 ? PX * PX * PT : 1); k++) {
				constexpr int Q = PX > 0 ? PX : 1;
				const int ht = k / (Q * Q), hy = (k / Q) % Q, hx = k % Q;
				ref_r[k] = __ldg(src.p + src.at(T.ox + s_x + hx, T.oy + s_y + hy, s_t + ht, 0));
			}
		} else {
			for (int k = tid; k < sp.spc * chn; k += blockDim.x) {
				const int c = k / sp.spc, r = k % sp.spc;
				const int ht = r / (sp.px * sp.px), hy = (r / sp.px) % sp.px, hx = r % sp.px;
				ref_s[k] = src.p[src.at(T.ox + s_x + hx, T.oy + s_y + hy, s_t + ht, c)];
			}
			__syncthreads();
		}
		// distances of every candidate, stored in the reference's candidate order
		const int nit = s_nitems;
		float tmin = __int_as_float(0x7f800000);
		int ii = 0;
		for (int it = tid; it < nit; it += blockDim.x) {
			while (ii + 1 < nframes && fw[ii + 1].ibase <= it) ii++;
			const FrameWin f = fw[ii];
			const int rel = it - f.ibase;
			const int rb = rel / f.nx, cx = rel - rb * f.nx;   // row block, column
			const int qy0 = rb * R;
			float acc[R];
			const float *colp = src.p + src.at(T.ox + f.rx0 + cx, T.oy + f.ry0 + qy0, f.qt, 0);
			col_distances<PX, PT, REFREG, R>(colp, src.P, src.plane(), src.plane() * src.C, f.ny - qy0 + sp.px - 2,
			                              chn, sp.px, sp.pt, ref_s, ref_r, acc);
			float *dd = dist + f.cbase + qy0 * f.nx + cx;
#pragma unroll
			for (int r = 0; r < R; r++)
				if (qy0 + r < f.ny) { dd[r * f.nx] = acc[r]; tmin = fminf(tmin, acc[r]); }
		}
		__syncthreads();
		const int ncand = s_ncand;
		const int K = min(sp.np, ncand);
		select_knn(dist, ncand, K, tmin, S);
		// tau rule (nldct.cpp:1284-1289), then one thread per kept neighbour
		int n = 1;
		while (2 * n <= K && S.od[n] < sp.tau2) n *= 2;
		if (tid == 0) a.nsimp[g] = (uint8_t)n;
		if (tid < n) {
			const int c = S.oi[tid];
			int jj = 0;
			while (jj + 1 < nframes && fw[jj + 1].cbase <= c) jj++;
			const FrameWin &f = fw[jj];
			const int rl = c - f.cbase;
			const int qy = f.ry0 + rl / f.nx, qx = f.rx0 + rl % f.nx;
			a.idx[g * sp.np + tid] = (uint32_t)(((long long)f.qt * T.h + qy) * T.w + qx);
		}
		__syncthreads();
	}
}

// nSimilarPatches == 1: the group is the reference patch alone (nldct.cpp:1326-1327).
__global__ void search_single_kernel(const Tile *__restrict__ tiles, int ntiles, const int *__restrict__ grid,
                                     StepParams sp, long long g_begin, long long g_end,
                                     uint8_t *__restrict__ nsimp_out, uint32_t *__restrict__ idx_out)
{
	for (long long g = g_begin + blockIdx.x * (long long)blockDim.x + threadIdx.x; g < g_end;
	     g += (long long)gridDim.x * blockDim.x) {
		const Tile T = tiles[tile_of(tiles, ntiles, g)];
		int x, y, t;
		group_position(T, grid, g, x, y, t);
		nsimp_out[g] = 1;
		idx_out[g * sp.np] = (uint32_t)(((long long)t * T.h + y) * T.w + x);
	}
}

template <int PX, int PT, bool REFREG, int MINB = 1, int R = kR>
cudaError_t launch_t(const Image &src, const StepParams &sp, const SearchArgs &a, size_t smem, int nsm,
                     long long n, cudaStream_t st)
{
	auto kern = search_kernel<PX, PT, REFREG, MINB, R>;
	cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
	if (e != cudaSuccess) return e;
	int per_sm = 0;
	e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreads, smem);
	if (e != cudaSuccess) return e;
	long long blocks = (long long)nsm * (per_sm < 1 ? 1 : per_sm);
	if (blocks > n) blocks = n;
	kern<<<(int)blocks, kThreads, smem, st>>>(src, sp, a);
	return cudaGetLastError();
}

}  // namespace

int search_frames_max(const StepParams &sp) { return sp.wtf + sp.wtb + 1; }

cudaError_t launch_traj(const Image &ffl, const Image &bfl, const Tile *tiles, int ntiles, const int *grid,
                        const StepParams &sp, long long G, uint32_t *traj, cudaStream_t st)
{
	if (G <= 0) return cudaSuccess;
	long long b = (G + 255) / 256;
	traj_kernel<<<(int)(b < 16384 ? b : 16384), 256, 0, st>>>(ffl, bfl, tiles, ntiles, grid, sp, G,
	                                                           search_frames_max(sp), traj);
	return cudaGetLastError();
}

cudaError_t launch_search(const Image &src, const Tile *tiles, int ntiles, const int *grid,
                          const uint32_t *traj, const StepParams &sp, long long g_begin, long long g_end,
                          uint8_t *nsimp, uint32_t *idx, int *err, int nsm, cudaStream_t st, const uint32_t *glist,
                          const unsigned *gcount)
{
	if (g_end <= g_begin) return cudaSuccess;
	if (sp.np <= 1 && !glist) {
		const long long n = g_end - g_begin;
		const int blocks = (int)((n + 255) / 256 < 65535 ? (n + 255) / 256 : 65535);
		search_single_kernel<<<blocks, 256, 0, st>>>(tiles, ntiles, grid, sp, g_begin, g_end, nsimp, idx);
		return cudaGetLastError();
	}
	SearchArgs a;
	a.tiles = tiles;
	a.ntiles = ntiles;
	a.grid = grid;
	a.traj = traj;
	a.nfm = search_frames_max(sp);
	a.g_begin = g_begin;
	a.g_end = g_end;
	a.glist = glist;
	a.gcount = gcount;
	a.nsimp = nsimp;
	a.idx = idx;
	(void)err;
	const long long n = g_end - g_begin;
	const size_t ncand = (size_t)sp.wx * sp.wx * a.nfm;
	const size_t smem = sizeof(float) * (ncand + (((size_t)sp.spc * sp.chn_search + 3) & ~(size_t)3));
	// The reference patch in shared memory, taken into registers one patch
	// frame at a time, measured faster than the whole patch in registers
	// (two CTAs per SM).  BM4DOF_SEARCH_REFREG=1 selects the register variant.
	static const int refreg_env = [] {
		const char *e = std::getenv("BM4DOF_SEARCH_REFREG");
		return e ? std::atoi(e) : 0;
	}();
	const bool one = sp.chn_search == 1 && refreg_env != 0;
	if (sp.px == 4 && sp.pt == 4) {
		// six CTAs per SM (56 registers, a few spilled) measured faster than
		// four (80 registers) and five (64): 133 vs 137 vs 147 ms on 854x480x20
		if (one) return launch_t<4, 4, true>(src, sp, a, smem, nsm, n, st);
		if (sp.search_ctas == 4) return launch_t<4, 4, false, 4>(src, sp, a, smem, nsm, n, st);
		// whole 21-row window columns per thread (24 rows loaded for 21
		// candidates instead of 30 for three strips of 7): 124.9 -> 112.0 ms on
		// 854x480x20, 2146 -> 1947 ms on 1920x1080x60; windows under 15 rows
		// keep strips of 7 (search_strip: the batched runs' tuning)
		if (sp.search_strip == 21 || (sp.search_strip == 0 && sp.wx >= 15))
			return launch_t<4, 4, false, 6, 21>(src, sp, a, smem, nsm, n, st);
		return launch_t<4, 4, false, 6>(src, sp, a, smem, nsm, n, st);
	}
	if (sp.px == 8 && sp.pt == 1)
		return one ? launch_t<8, 1, true>(src, sp, a, smem, nsm, n, st) : launch_t<8, 1, false>(src, sp, a, smem, nsm, n, st);
	return launch_t<0, 0, false>(src, sp, a, smem, nsm, n, st);
}

}  // namespace bm4dof
