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
//   search_kernel  one CTA per group at a time: each candidate frame's window
//                  (plus patch halo, all patch frames) is copied into shared
//                  memory by a TMA tensor load, double buffered behind an
//                  mbarrier; threads compute register-tiled strips of SW
//                  horizontally adjacent candidates with the reference patch
//                  held in registers; warp 0 then runs the heap selection with
//                  ballots so that only candidates below the current heap top
//                  are handled one at a time.  The next group's first windows
//                  are requested before the selection starts.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>
#include <cstdint>

#include "common.cuh"
#include "internal.hpp"

namespace bm4dof {

namespace {

constexpr int kThreads = 64;
constexpr int kSW = 7;                 // candidates per thread along x
constexpr unsigned kWaitLimit = 1u << 24;

struct FrameWin {
	int qt, rx0, ry0, nx, ny, cbase, ibase, xoff, X0;
};

__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
	return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count)
{
	asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, unsigned bytes)
{
	asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
	             : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, unsigned parity)
{
	uint32_t ok;
	asm volatile(
		"{\n\t.reg .pred p;\n\t"
		"mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
		"selp.u32 %0, 1, 0, p;\n\t}"
		: "=r"(ok)
		: "r"(smem_u32(bar)), "r"(parity)
		: "memory");
	return ok != 0;
}

__device__ __forceinline__ void tma_load_4d(void *dst, const CUtensorMap *map, uint64_t *bar, int x, int y,
                                            int c, int t)
{
	asm volatile(
		"cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
		" [%0], [%1, {%3, %4, %5, %6}], [%2];" ::"r"(smem_u32(dst)),
		"l"(map), "r"(smem_u32(bar)), "r"(x), "r"(y), "r"(c), "r"(t)
		: "memory");
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
	int BX, BY, CB;            // TMA box: x, y, channels (pt frames)
	long long g_begin, g_end;
	uint8_t *nsimp;
	uint32_t *idx;
	int *err;
};

// Window table of one group (thread 0).
__device__ void plan_group(const SearchArgs &a, const StepParams &sp, long long g, FrameWin *fw, int &nframes,
                           int &ncand, int &nitems, int &tile, int &gx, int &gy, int &gt, int nstrip_w)
{
	const int ti = tile_of(a.tiles, a.ntiles, g);
	const Tile T = a.tiles[ti];
	int x, y, t, t0, t1;
	group_position(T, a.grid, g, x, y, t);
	temporal_range(sp, t, t0, t1);
	const int nwt = t1 - t0 + 1;
	const int hw = (sp.wx - 1) / 2;
	int cb = 0, ib = 0;
	for (int ii = 0; ii < nwt; ii++) {
		const uint32_t c = a.traj[g * a.nfm + ii];
		const int cx = (int)(c & 0xffffu), cy = (int)(c >> 16);
		const int shx = min(0, cx - hw) + max(0, cx + hw - T.w + sp.px);
		const int shy = min(0, cy - hw) + max(0, cy + hw - T.h + sp.px);
		const int rx0 = max(0, cx - hw - shx), ry0 = max(0, cy - hw - shy);
		const int rx1 = min(T.w - sp.px, cx + hw - shx), ry1 = min(T.h - sp.px, cy + hw - shy);
		FrameWin f;
		f.qt = visit_frame(ii, t, t1);
		f.rx0 = rx0;
		f.ry0 = ry0;
		f.nx = max(0, rx1 - rx0 + 1);
		f.ny = max(0, ry1 - ry0 + 1);
		f.cbase = cb;
		f.ibase = ib;
		f.X0 = (T.ox + rx0) & ~3;           // TMA x coordinate: 16-byte aligned
		f.xoff = T.ox + rx0 - f.X0;
		cb += f.nx * f.ny;
		ib += f.ny * ((f.nx + kSW - 1) / kSW);
		fw[ii] = f;
	}
	nframes = nwt;
	ncand = cb;
	nitems = ib;
	tile = ti;
	gx = x;
	gy = y;
	gt = t;
	(void)nstrip_w;
}

// Distances of kSW adjacent candidates from a window row block in shared
// memory.  REFREG: reference patch in registers (one channel, PX*PX*PT values).
template <int PX, int PT, bool REFREG>
__device__ __forceinline__ void strip_distances(const float *win, int BX, int BY, int CB, int chn, int xs,
                                                int ys, int px_rt, int pt_rt, const float *ref_s,
                                                const float (&ref_r)[(PX > 0 ? PX * PX * PT : 1)],
                                                float acc[kSW])
{
	const int px = PX > 0 ? PX : px_rt;
	const int pt = PT > 0 ? PT : pt_rt;
#pragma unroll
	for (int j = 0; j < kSW; j++) acc[j] = 0.f;
	if (PX > 0) {
		constexpr int NV = (PX > 0 ? PX : 1) + kSW - 1;
		constexpr int SPC = (PX > 0 ? PX * PX * PT : 1);
		for (int c = 0; c < chn; c++)
#pragma unroll
			for (int ht = 0; ht < (PT > 0 ? PT : 1); ht++)
#pragma unroll
				for (int hy = 0; hy < PX; hy++) {
					const float *row = win + ((ht * CB + c) * BY + ys + hy) * BX;
					float v[NV];
#pragma unroll
					for (int j = 0; j < NV; j++) v[j] = row[min(xs + j, BX - 1)];
#pragma unroll
					for (int hx = 0; hx < PX; hx++) {
						const int kk = (ht * PX + hy) * PX + hx;
						const float r = REFREG ? ref_r[kk] : ref_s[c * SPC + kk];
#pragma unroll
						for (int j = 0; j < kSW; j++) {
							const float d = __fsub_rn(r, v[j + hx]);
							acc[j] = __fadd_rn(acc[j], __fmul_rn(d, d));
						}
					}
				}
	} else {
		int k = 0;
		for (int c = 0; c < chn; c++)
			for (int ht = 0; ht < pt; ht++)
				for (int hy = 0; hy < px; hy++) {
					const float *row = win + ((ht * CB + c) * BY + ys + hy) * BX;
					for (int hx = 0; hx < px; hx++, k++) {
						const float r = ref_s[k];
#pragma unroll
						for (int j = 0; j < kSW; j++) {
							const float d = __fsub_rn(r, row[min(xs + j + hx, BX - 1)]);
							acc[j] = __fadd_rn(acc[j], __fmul_rn(d, d));
						}
					}
				}
	}
}

// Window stream of one CTA: the frames of its groups in processing order,
// each loaded by TMA into one of two buffers (FIFO).  Thread 0 keeps the
// issue cursor; it runs at most one group ahead of the group being computed,
// whose window table lives in the other plan slot.
struct IssueState {
	long long ig;     // group of the next window to request
	int ifr;          // its frame index
	int islot;        // plan slot of that group
	int inflight;     // windows requested and not yet consumed
	unsigned issued;  // windows requested so far
};

template <int PX, int PT, bool REFREG>
__global__ void __launch_bounds__(kThreads)
search_kernel(const __grid_constant__ CUtensorMap map, Image src, StepParams sp, SearchArgs a)
{
	extern __shared__ __align__(128) unsigned char smem_raw[];
	const int box = a.BX * a.BY * a.CB * sp.pt;              // floats per window buffer
	const int boxp = (box + 31) / 32 * 32;
	float *bufs[2] = {reinterpret_cast<float *>(smem_raw), reinterpret_cast<float *>(smem_raw) + boxp};
	float *dist = bufs[1] + boxp;
	const int ncand_max = sp.wx * sp.wx * (sp.wtf + sp.wtb + 1);
	float *ref_s = dist + ncand_max;                           // chn * spc
	__shared__ FrameWin fw[2][kMaxFrames];
	__shared__ int s_nframes[2], s_ncand[2], s_nitems[2], s_tile[2], s_x[2], s_y[2], s_t[2];
	__shared__ float hd[kMaxNp];
	__shared__ int hi[kMaxNp];
	__shared__ __align__(8) uint64_t bars[2];
	__shared__ int s_abort;

	const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
	const int chn = sp.chn_search;
	const unsigned box_bytes = (unsigned)box * 4u;
	IssueState is = {0, 0, 0, 0, 0u};   // meaningful in thread 0 only
	int cur = 0;

	auto issue_more = [&]() {
		while (is.inflight < 2 && is.ig < a.g_end) {
			if (is.ifr >= s_nframes[is.islot]) {
				// next group of this CTA: only into the slot not being computed
				if (is.islot != cur) break;
				is.ig += gridDim.x;
				if (is.ig >= a.g_end) break;
				is.islot ^= 1;
				is.ifr = 0;
				const int sl = is.islot;
				plan_group(a, sp, is.ig, fw[sl], s_nframes[sl], s_ncand[sl], s_nitems[sl], s_tile[sl], s_x[sl],
				           s_y[sl], s_t[sl], 0);
				continue;
			}
			const FrameWin &f = fw[is.islot][is.ifr];
			const int b = is.issued & 1;
			mbar_expect_tx(&bars[b], box_bytes);
			tma_load_4d(bufs[b], &map, &bars[b], f.X0, a.tiles[s_tile[is.islot]].oy + f.ry0, 0, f.qt);
			is.issued++;
			is.ifr++;
			is.inflight++;
		}
	};

	if (tid == 0) {
		mbar_init(&bars[0], 1);
		mbar_init(&bars[1], 1);
		asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
		s_abort = 0;
		is.ig = a.g_begin + blockIdx.x;
		is.ifr = 0;
		is.islot = 0;
		is.inflight = 0;
		is.issued = 0;
		if (is.ig < a.g_end) {
			plan_group(a, sp, is.ig, fw[0], s_nframes[0], s_ncand[0], s_nitems[0], s_tile[0], s_x[0], s_y[0],
			           s_t[0], 0);
			issue_more();
		}
	}
	__syncthreads();

	unsigned consumed = 0;
	for (long long g = a.g_begin + blockIdx.x; g < a.g_end; g += gridDim.x) {
		const Tile T = a.tiles[s_tile[cur]];
		const int nframes = s_nframes[cur];
		// reference patch, channel-major (c, ht, hy, hx)
		float ref_r[(PX > 0 ? PX * PX * PT : 1)];
		if (REFREG) {
#pragma unroll
			for (int k = 0; k < (PX > 0 ? PX * PX * PT : 1); k++) {
				constexpr int Q = PX > 0 ? PX : 1;
				const int ht = k / (Q * Q), hy = (k / Q) % Q, hx = k % Q;
				ref_r[k] = __ldg(src.p + src.at(T.ox + s_x[cur] + hx, T.oy + s_y[cur] + hy, s_t[cur] + ht, 0));
			}
		} else {
			for (int k = tid; k < sp.spc * chn; k += blockDim.x) {
				const int c = k / sp.spc, r = k % sp.spc;
				const int ht = r / (sp.px * sp.px), hy = (r / sp.px) % sp.px, hx = r % sp.px;
				ref_s[k] = src.p[src.at(T.ox + s_x[cur] + hx, T.oy + s_y[cur] + hy, s_t[cur] + ht, c)];
			}
			__syncthreads();
		}

		for (int ii = 0; ii < nframes; ii++, consumed++) {
			const int b = consumed & 1;
			const unsigned parity = (consumed >> 1) & 1u;
			// bounded wait for this frame's window (every thread observes the phase)
			unsigned n = 0;
			while (!mbar_try_wait(&bars[b], parity))
				if (++n > kWaitLimit) { s_abort = 1; atomicExch(a.err, 1); break; }
			__syncthreads();
			if (s_abort) return;
			const FrameWin f = fw[cur][ii];
			const float *win = bufs[b];
			const int nstrip = (f.nx + kSW - 1) / kSW;
			const int nit = f.ny * nstrip;
			for (int it = tid; it < nit; it += blockDim.x) {
				const int row = it / nstrip, strip = it - row * nstrip;
				float acc[kSW];
				strip_distances<PX, PT, REFREG>(win, a.BX, a.BY, a.CB, chn, f.xoff + strip * kSW, row, sp.px, sp.pt,
				                                ref_s, ref_r, acc);
				float *dd = dist + f.cbase + row * f.nx + strip * kSW;
#pragma unroll
				for (int j = 0; j < kSW; j++)
					if (strip * kSW + j < f.nx) dd[j] = acc[j];
			}
			__syncthreads();
			if (tid == 0) {
				// the buffer just read may be refilled by the async proxy
				asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
				is.inflight--;
				issue_more();
			}
		}

		// k nearest with the libstdc++ heap selection (warp 0)
		if (warp == 0) {
			const int ncand = s_ncand[cur];
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
				a.nsimp[g] = (uint8_t)n;
				for (int q = 0; q < n; q++) {
					const int c = hi[q];
					int ii = 0;
					while (ii + 1 < nframes && fw[cur][ii + 1].cbase <= c) ii++;
					const FrameWin &f = fw[cur][ii];
					const int rel = c - f.cbase;
					const int qy = f.ry0 + rel / f.nx, qx = f.rx0 + rel % f.nx;
					a.idx[g * sp.np + q] = (uint32_t)(((long long)f.qt * T.h + qy) * T.w + qx);
				}
			}
		}
		__syncthreads();
		cur ^= 1;
		if (tid == 0) issue_more();
		__syncthreads();
	}
	// every requested window belongs to a group of this CTA and was consumed
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

PFN_cuTensorMapEncodeTiled_v12000 encode_fn()
{
	static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
	if (!fn) {
		void *p = nullptr;
		cudaDriverEntryPointQueryResult q;
		if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
		        cudaSuccess &&
		    q == cudaDriverEntryPointSuccess)
			fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
	}
	return fn;
}

template <int PX, int PT, bool REFREG>
cudaError_t launch_t(const CUtensorMap &map, const Image &src, const StepParams &sp, const SearchArgs &a,
                     size_t smem, int blocks, cudaStream_t st)
{
	cudaError_t e = cudaFuncSetAttribute(search_kernel<PX, PT, REFREG>,
	                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
	if (e != cudaSuccess) return e;
	search_kernel<PX, PT, REFREG><<<blocks, kThreads, smem, st>>>(map, src, sp, a);
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
                          uint8_t *nsimp, uint32_t *idx, int *err, int nsm, cudaStream_t st)
{
	if (g_end <= g_begin) return cudaSuccess;
	if (sp.np <= 1) {
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
	a.BX = (sp.wx + sp.px + 2 + 3) / 4 * 4;     // window + halo + misalignment, multiple of 4
	a.BY = sp.wx + sp.px - 1;
	a.CB = sp.chn_search;
	a.g_begin = g_begin;
	a.g_end = g_end;
	a.nsimp = nsimp;
	a.idx = idx;
	a.err = err;
	if (a.BX > 256 || a.BY > 256 || sp.pt > 256) return cudaErrorInvalidValue;

	PFN_cuTensorMapEncodeTiled_v12000 enc = encode_fn();
	if (!enc) return cudaErrorNotSupported;
	CUtensorMap map;
	const cuuint64_t dims[4] = {(cuuint64_t)src.P, (cuuint64_t)src.H, (cuuint64_t)src.C, (cuuint64_t)src.F};
	const cuuint64_t strides[3] = {(cuuint64_t)src.P * 4, (cuuint64_t)src.P * src.H * 4,
	                               (cuuint64_t)src.P * src.H * src.C * 4};
	const cuuint32_t boxd[4] = {(cuuint32_t)a.BX, (cuuint32_t)a.BY, (cuuint32_t)a.CB, (cuuint32_t)sp.pt};
	const cuuint32_t estr[4] = {1, 1, 1, 1};
	CUresult r = enc(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, src.p, dims, strides, boxd, estr,
	                 CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
	                 CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
	if (r != CUDA_SUCCESS) return cudaErrorInvalidValue;

	const int box = a.BX * a.BY * a.CB * sp.pt;
	const int boxp = (box + 31) / 32 * 32;
	const int ncand = sp.wx * sp.wx * (sp.wtf + sp.wtb + 1);
	const size_t smem = sizeof(float) * (2 * (size_t)boxp + ncand + (size_t)sp.spc * sp.chn_search);
	if (smem > 220 * 1024) return cudaErrorInvalidValue;
	const long long n = g_end - g_begin;
	const int per_sm = (int)((200 * 1024) / (smem + 1024));
	long long blocks = (long long)nsm * (per_sm < 1 ? 1 : (per_sm > 16 ? 16 : per_sm));
	if (blocks > n) blocks = n;
	if (sp.chn_search == 1 && sp.px == 4 && sp.pt == 4) return launch_t<4, 4, true>(map, src, sp, a, smem, (int)blocks, st);
	if (sp.chn_search == 1 && sp.px == 8 && sp.pt == 1) return launch_t<8, 1, true>(map, src, sp, a, smem, (int)blocks, st);
	if (sp.px == 4 && sp.pt == 4) return launch_t<4, 4, false>(map, src, sp, a, smem, (int)blocks, st);
	if (sp.px == 8 && sp.pt == 1) return launch_t<8, 1, false>(map, src, sp, a, smem, (int)blocks, st);
	return launch_t<0, 0, false>(map, src, sp, a, smem, (int)blocks, st);
}

}  // namespace bm4dof
