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
// One CTA handles one group at a time: all warps compute distances into shared
// memory (register-tiled strips of SW candidates per thread), then warp 0 runs
// the heap selection with ballots so that only candidates below the current
// heap top are handled one at a time.
#include <cuda_runtime.h>
#include <cstdint>

#include "common.cuh"

namespace bm4dof {

namespace {

constexpr int kSearchThreads = 128;
constexpr int kSW = 4;   // candidates per thread along x

struct FrameWin {
	int qt, rx0, ry0, nx, ny, cbase, ibase;
};

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

// Distances of SW horizontally adjacent candidates starting at (qx0, qy, qt).
template <int PX, int SW>
__device__ __forceinline__ void strip_distances(const Image &src, const Tile &T, int qx0, int qy,
                                                int qt, int px, int pt, int chn,
                                                const float *ref, float acc[SW])
{
	constexpr int NV = (PX > 0 ? PX : 1) + SW - 1;
	const int pxx = PX > 0 ? PX : px;
	const int xmax = T.ox + T.w - 1;
#pragma unroll
	for (int j = 0; j < SW; j++) acc[j] = 0.f;
	int k = 0;
	for (int c = 0; c < chn; c++)
		for (int ht = 0; ht < pt; ht++)
			for (int hy = 0; hy < pxx; hy++) {
				const float *row = src.p + src.at(0, T.oy + qy + hy, qt + ht, c);
				if (PX > 0) {
					float v[NV];
#pragma unroll
					for (int j = 0; j < NV; j++) {
						const int x = min(T.ox + qx0 + j, xmax);
						v[j] = __ldg(row + x);
					}
#pragma unroll
					for (int hx = 0; hx < PX; hx++, k++) {
						const float r = ref[k];
#pragma unroll
						for (int j = 0; j < SW; j++) {
							const float d = __fsub_rn(r, v[j + hx]);
							acc[j] = __fadd_rn(acc[j], __fmul_rn(d, d));
						}
					}
				} else {
					for (int hx = 0; hx < pxx; hx++, k++) {
						const float r = ref[k];
#pragma unroll
						for (int j = 0; j < SW; j++) {
							const int x = min(T.ox + qx0 + j + hx, xmax);
							const float d = __fsub_rn(r, __ldg(row + x));
							acc[j] = __fadd_rn(acc[j], __fmul_rn(d, d));
						}
					}
				}
			}
}

template <int PX>
__global__ void __launch_bounds__(kSearchThreads)
search_exact_kernel(Image src, Image ffl, Image bfl, const Tile *__restrict__ tiles, int ntiles,
                    const int *__restrict__ grid, StepParams sp, long long g_begin,
                    long long g_end, uint8_t *__restrict__ nsimp_out,
                    uint32_t *__restrict__ idx_out)
{
	extern __shared__ float smem[];
	const int spc_c = sp.spc * sp.chn_search;
	float *ref = smem;                       // chn_search * spc
	float *dist = smem + spc_c;              // candidates
	__shared__ FrameWin fw[kMaxFrames];
	__shared__ int s_nframes, s_ncand, s_nitems;
	__shared__ float hd[kMaxNp];
	__shared__ int hi[kMaxNp];
	__shared__ int s_tile, s_x, s_y, s_t;

	const int tid = threadIdx.x;
	const int lane = tid & 31;
	const int warp = tid >> 5;

	for (long long g = g_begin + blockIdx.x; g < g_end; g += gridDim.x) {
		if (tid == 0) {
			const int ti = tile_of(tiles, ntiles, g);
			const Tile T = tiles[ti];
			const long long local = g - T.g0;
			const int xi = (int)(local % T.nx);
			const int yi = (int)((local / T.nx) % T.ny);
			const int fi = (int)(local / ((long long)T.nx * T.ny));
			const int x = grid[T.gx + xi], y = grid[T.gy + yi], t = grid[T.gf + fi];
			s_tile = ti; s_x = x; s_y = y; s_t = t;

			const int W = T.w, H = T.h, F = sp.F, pt = sp.pt, px = sp.px, wx = sp.wx;
			const int shift_t = min(0, t - sp.wtb) + max(0, t + sp.wtf - F + pt);
			const int t0 = max(0, t - sp.wtb - shift_t);
			const int t1 = min(F - pt, t + sp.wtf - shift_t);
			const int nwt = t1 - t0 + 1;
			int cxs[kMaxFrames], cys[kMaxFrames];
			int cb = 0, ib = 0;
			for (int ii = 0; ii < nwt; ii++) {
				// visiting order: t, t+1..t1, t-1..t0 (nldct.cpp:1195-1198)
				const int qt = ii == 0 ? t : (ii <= t1 - t ? t + ii : t - (ii - (t1 - t)));
				const int dt = qt - t0;
				const int dir = qt > t ? 1 : (qt < t ? -1 : 0);
				int cx, cy;
				if (dir != 0) {
					const int cx0 = cxs[dt - dir], cy0 = cys[dt - dir], ct0 = qt - dir;
					float fx = 0.f, fy = 0.f;
					if (sp.use_flow) {
						const Image &fl = dir > 0 ? ffl : bfl;
						fx = fl.p[fl.at(T.ox + cx0, T.oy + cy0, ct0, 0)];
						fy = fl.p[fl.at(T.ox + cx0, T.oy + cy0, ct0, 1)];
					}
					const float cxf = __fadd_rn((float)cx0, fx);
					const float cyf = __fadd_rn((float)cy0, fy);
					cx = (int)fmaxf(0.f, fminf(__fsub_rn((float)W, 1.f), roundf(cxf)));
					cy = (int)fmaxf(0.f, fminf(__fsub_rn((float)H, 1.f), roundf(cyf)));
				} else {
					cx = x; cy = y;
				}
				cxs[dt] = cx; cys[dt] = cy;
				const int hw = (wx - 1) / 2;
				const int shx = min(0, cx - hw) + max(0, cx + hw - W + px);
				const int shy = min(0, cy - hw) + max(0, cy + hw - H + px);
				const int rx0 = max(0, cx - hw - shx), ry0 = max(0, cy - hw - shy);
				const int rx1 = min(W - px, cx + hw - shx), ry1 = min(H - px, cy + hw - shy);
				FrameWin f;
				f.qt = qt; f.rx0 = rx0; f.ry0 = ry0;
				f.nx = max(0, rx1 - rx0 + 1); f.ny = max(0, ry1 - ry0 + 1);
				f.cbase = cb; f.ibase = ib;
				cb += f.nx * f.ny;
				ib += f.ny * ((f.nx + kSW - 1) / kSW);
				fw[ii] = f;
			}
			s_nframes = nwt; s_ncand = cb; s_nitems = ib;
		}
		__syncthreads();

		const Tile T = tiles[s_tile];
		// reference patch, channel-major (c, ht, hy, hx)
		for (int k = tid; k < spc_c; k += blockDim.x) {
			const int c = k / sp.spc, r = k % sp.spc;
			const int ht = r / (sp.px * sp.px), hy = (r / sp.px) % sp.px, hx = r % sp.px;
			ref[k] = src.p[src.at(T.ox + s_x + hx, T.oy + s_y + hy, s_t + ht, c)];
		}
		__syncthreads();

		// distances of all candidates, stored in the reference's candidate order
		const int nitems = s_nitems, nframes = s_nframes;
		for (int it = tid; it < nitems; it += blockDim.x) {
			int ii = 0;
			while (ii + 1 < nframes && fw[ii + 1].ibase <= it) ii++;
			const FrameWin f = fw[ii];
			const int nstrip = (f.nx + kSW - 1) / kSW;
			const int rel = it - f.ibase;
			const int row = rel / nstrip, strip = rel % nstrip;
			const int qx0 = f.rx0 + strip * kSW, qy = f.ry0 + row;
			float acc[kSW];
			strip_distances<PX, kSW>(src, T, qx0, qy, f.qt, sp.px, sp.pt, sp.chn_search, ref, acc);
#pragma unroll
			for (int j = 0; j < kSW; j++)
				if (strip * kSW + j < f.nx) dist[f.cbase + row * f.nx + strip * kSW + j] = acc[j];
		}
		__syncthreads();

		if (warp == 0) {
			const int ncand = s_ncand;
			const int K = min(sp.np, ncand);
			if (lane == 0) {
				for (int i = 0; i < K; i++) { hd[i] = dist[i]; hi[i] = i; }
				make_heap(hd, hi, K);
			}
			__syncwarp();
			float top = hd[0];
			for (int base = K; base < ncand; base += 32) {
				const int i = base + lane;
				const float d = i < ncand ? dist[i] : 0.f;
				unsigned m = __ballot_sync(0xffffffffu, i < ncand && d < top);
				while (m) {
					const int j = __ffs(m) - 1;
					if (lane == 0) adjust_heap(hd, hi, 0, K, dist[base + j], base + j);
					__syncwarp();
					top = hd[0];
					m &= ~((2u << j) - 1u);
					m &= __ballot_sync(0xffffffffu, i < ncand && d < top);
				}
			}
			if (lane == 0) {
				sort_heap(hd, hi, K);
				int n = 1;
				while (2 * n <= K && hd[n] < sp.tau2) n *= 2;
				nsimp_out[g] = (uint8_t)n;
				// candidate number -> tile-linear position (t*h + y)*w + x
				for (int q = 0; q < n; q++) {
					const int c = hi[q];
					int ii = 0;
					while (ii + 1 < nframes && fw[ii + 1].cbase <= c) ii++;
					const FrameWin f = fw[ii];
					const int rel = c - f.cbase;
					const int qy = f.ry0 + rel / f.nx, qx = f.rx0 + rel % f.nx;
					idx_out[g * sp.np + q] = (uint32_t)(((long long)f.qt * T.h + qy) * T.w + qx);
				}
			}
		}
		__syncthreads();
	}
}

// nSimilarPatches == 1: the group is the reference patch alone (nldct.cpp:1326-1327).
__global__ void search_single_kernel(const Tile *__restrict__ tiles, int ntiles,
                                     const int *__restrict__ grid, StepParams sp,
                                     long long g_begin, long long g_end,
                                     uint8_t *__restrict__ nsimp_out, uint32_t *__restrict__ idx_out)
{
	for (long long g = g_begin + blockIdx.x * (long long)blockDim.x + threadIdx.x; g < g_end;
	     g += (long long)gridDim.x * blockDim.x) {
		const Tile T = tiles[tile_of(tiles, ntiles, g)];
		const long long local = g - T.g0;
		const int x = grid[T.gx + (int)(local % T.nx)];
		const int y = grid[T.gy + (int)((local / T.nx) % T.ny)];
		const int t = grid[T.gf + (int)(local / ((long long)T.nx * T.ny))];
		nsimp_out[g] = 1;
		idx_out[g * sp.np] = (uint32_t)(((long long)t * T.h + y) * T.w + x);
	}
}

}  // namespace

size_t search_smem_bytes(const StepParams &sp)
{
	const int ncand = sp.wx * sp.wx * (sp.wtf + sp.wtb + 1);
	return sizeof(float) * ((size_t)sp.spc * sp.chn_search + ncand);
}

cudaError_t launch_search(const Image &src, const Image &ffl, const Image &bfl, const Tile *tiles,
                          int ntiles, const int *grid, const StepParams &sp, long long g_begin,
                          long long g_end, uint8_t *nsimp, uint32_t *idx, int nsm,
                          cudaStream_t st)
{
	if (g_end <= g_begin) return cudaSuccess;
	if (sp.np <= 1) {
		const long long n = g_end - g_begin;
		const int blocks = (int)((n + 255) / 256 < 65535 ? (n + 255) / 256 : 65535);
		search_single_kernel<<<blocks, 256, 0, st>>>(tiles, ntiles, grid, sp, g_begin, g_end, nsimp, idx);
		return cudaGetLastError();
	}
	const size_t smem = search_smem_bytes(sp);
	const long long n = g_end - g_begin;
	const int blocks = (int)(n < (long long)nsm * 16 ? n : (long long)nsm * 16);
	cudaError_t e;
	switch (sp.px) {
	case 4:
		e = cudaFuncSetAttribute(search_exact_kernel<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
		if (e != cudaSuccess) return e;
		search_exact_kernel<4><<<blocks, kSearchThreads, smem, st>>>(src, ffl, bfl, tiles, ntiles, grid, sp,
		                                                               g_begin, g_end, nsimp, idx);
		break;
	case 8:
		e = cudaFuncSetAttribute(search_exact_kernel<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
		if (e != cudaSuccess) return e;
		search_exact_kernel<8><<<blocks, kSearchThreads, smem, st>>>(src, ffl, bfl, tiles, ntiles, grid, sp,
		                                                               g_begin, g_end, nsimp, idx);
		break;
	default:
		e = cudaFuncSetAttribute(search_exact_kernel<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
		if (e != cudaSuccess) return e;
		search_exact_kernel<0><<<blocks, kSearchThreads, smem, st>>>(src, ffl, bfl, tiles, ntiles, grid, sp,
		                                                               g_begin, g_end, nsimp, idx);
		break;
	}
	return cudaGetLastError();
}

}  // namespace bm4dof
