// aggregate.cu -- deterministic aggregation, reference-grid bookkeeping,
// normalisation, tile rebuild and colour transforms.
//
// The reference adds every group's estimates into a per-tile image and weight
// image one group after another (computeAggregationStep1/2,
// src/core/nldct.cpp:2259-2425), so each pixel's float sum follows the
// processing order (group, then member).  Here the same sums are formed as a
// gather with no float atomics: every member patch ("slot") is listed under
// its origin pixel, the lists are sorted by slot number (= processing order),
// and each pixel walks the slots that cover it in that order.  The result is
// bit-identical to the sequential scatter.
#include <cuda_runtime.h>
#include <cstdint>

#include "common.cuh"

namespace bm4dof {

namespace {

constexpr int kGatherBX = 8, kGatherBY = 8;
constexpr int kGatherThreads = kGatherBX * kGatherBY;
constexpr int kRegionMax = 1024;      // origins feeding one 8x8 pixel block
constexpr int kEntryCap = 4096;       // slots sorted in shared memory per block

__device__ __forceinline__ void group_position(const Tile &T, const int *grid, long long g,
                                               int &x, int &y, int &t)
{
	const long long local = g - T.g0;
	x = grid[T.gx + (int)(local % T.nx)];
	y = grid[T.gy + (int)((local / T.nx) % T.ny)];
	t = grid[T.gf + (int)(local / ((long long)T.nx * T.ny))];
}

// ---------------------------------------------------------------------------
// mask(index[0]) = false (nldct.cpp:2325-2329, 2418-2422).  A group whose best
// match is not itself may switch off a later reference position; those rare
// cases become edges killer -> victim.  The index carries the channel stride
// (t*w*h*C + y*w + x) while the mask has one channel, so for C > 1 the cleared
// position is another frame of the mask; indices past the mask are ignored
// (the reference writes out of bounds there).
// ---------------------------------------------------------------------------
__global__ void kill_edges_kernel(const Tile *__restrict__ tiles, int ntiles,
                                  const int *__restrict__ grid, const int *__restrict__ inv,
                                  StepParams sp, long long G, const uint32_t *__restrict__ idx,
                                  unsigned long long *__restrict__ edges, unsigned *__restrict__ nedges,
                                  unsigned cap)
{
	for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < G;
	     g += (long long)gridDim.x * blockDim.x) {
		const Tile T = tiles[tile_of(tiles, ntiles, g)];
		int x, y, t;
		group_position(T, grid, g, x, y, t);
		const unsigned long long wh = (unsigned long long)T.w * T.h;
		const uint32_t lin = idx[g * sp.np];
		const unsigned long long mt = lin / wh, rem = lin % wh;
		// the reference's index value, interpreted as a one-channel mask index
		const unsigned long long m = mt * wh * sp.C + rem;
		const unsigned long long own = ((unsigned long long)t * T.h + y) * T.w + x;
		if (m >= wh * sp.F || m <= own) continue;
		const int tt = (int)(m / wh), ty = (int)((m % wh) / T.w), tx = (int)(m % T.w);
		const int xi = inv[T.gx + T.nx + tx];
		const int yi = inv[T.gy + T.ny + ty];
		const int fi = inv[T.gf + T.nf + tt];
		if (xi < 0 || yi < 0 || fi < 0) continue;
		const long long victim = T.g0 + ((long long)fi * T.ny + yi) * T.nx + xi;
		const unsigned e = atomicAdd(nedges, 1u);
		if (e < cap) edges[e] = ((unsigned long long)g << 32) | (unsigned long long)victim;
	}
}

__global__ void kill_mark_kernel(const unsigned long long *__restrict__ edges, unsigned n,
                                 const uint8_t *__restrict__ alive, uint8_t *__restrict__ killed,
                                 int clear)
{
	for (unsigned e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
		const unsigned long long v = edges[e];
		const long long u = (long long)(v >> 32), w = (long long)(v & 0xffffffffull);
		if (clear) killed[w] = 0;
		else if (alive[u]) killed[w] = 1;
	}
}

__global__ void kill_apply_kernel(const unsigned long long *__restrict__ edges, unsigned n,
                                  const uint8_t *__restrict__ killed, uint8_t *__restrict__ alive,
                                  unsigned *__restrict__ changed)
{
	for (unsigned e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
		const long long w = (long long)(edges[e] & 0xffffffffull);
		const uint8_t a = killed[w] ? 0 : 1;
		if (alive[w] != a) {
			alive[w] = a;
			*changed = 1u;
		}
	}
}

__global__ void count_alive_kernel(const Tile *__restrict__ tiles, int ntiles, long long G,
                                   const uint8_t *__restrict__ alive, unsigned *__restrict__ counts)
{
	for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < G;
	     g += (long long)gridDim.x * blockDim.x)
		if (alive[g]) atomicAdd(&counts[tile_of(tiles, ntiles, g)], 1u);
}

// ---------------------------------------------------------------------------
// origin lists: for every tile pixel, the slots whose patch starts there,
// sorted by slot number
// ---------------------------------------------------------------------------
__global__ void list_count_kernel(long long ga, long long gb, int np, const uint8_t *__restrict__ nsimp,
                                  const uint32_t *__restrict__ idx, const uint8_t *__restrict__ alive,
                                  unsigned *__restrict__ cnt)
{
	for (long long it = blockIdx.x * (long long)blockDim.x + threadIdx.x; it < (gb - ga) * np;
	     it += (long long)gridDim.x * blockDim.x) {
		const long long g = ga + it / np;
		const int n = (int)(it % np);
		if (!alive[g] || n >= nsimp[g]) continue;
		atomicAdd(&cnt[idx[g * np + n]], 1u);
	}
}

__global__ void list_fill_kernel(long long ga, long long gb, int np, const uint8_t *__restrict__ nsimp,
                                 const uint32_t *__restrict__ idx, const uint8_t *__restrict__ alive,
                                 const unsigned *__restrict__ off, unsigned *__restrict__ cursor,
                                 unsigned *__restrict__ list)
{
	for (long long it = blockIdx.x * (long long)blockDim.x + threadIdx.x; it < (gb - ga) * np;
	     it += (long long)gridDim.x * blockDim.x) {
		const long long g = ga + it / np;
		const int n = (int)(it % np);
		if (!alive[g] || n >= nsimp[g]) continue;
		const uint32_t pos = idx[g * np + n];
		const unsigned k = atomicAdd(&cursor[pos], 1u);
		list[off[pos] + k] = (unsigned)it;     // chunk-relative slot number
	}
}

__global__ void list_sort_kernel(size_t npos, const unsigned *__restrict__ off, unsigned *__restrict__ list)
{
	for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < npos;
	     p += (size_t)gridDim.x * blockDim.x) {
		const unsigned a = off[p], b = off[p + 1];
		for (unsigned i = a + 1; i < b; i++) {
			const unsigned v = list[i];
			unsigned j = i;
			while (j > a && list[j - 1] > v) { list[j] = list[j - 1]; j--; }
			list[j] = v;
		}
	}
}

// ---------------------------------------------------------------------------
// exclusive scan of unsigned counts (three-level, 4096 elements per block)
// ---------------------------------------------------------------------------
constexpr int kScanThreads = 1024, kScanPer = 4, kScanBlock = kScanThreads * kScanPer;

__global__ void scan_block_kernel(unsigned *__restrict__ data, size_t n, unsigned *__restrict__ sums)
{
	__shared__ unsigned s[kScanThreads];
	const size_t base = (size_t)blockIdx.x * kScanBlock + (size_t)threadIdx.x * kScanPer;
	unsigned v[kScanPer], tot = 0;
#pragma unroll
	for (int i = 0; i < kScanPer; i++) {
		v[i] = base + i < n ? data[base + i] : 0u;
		tot += v[i];
	}
	s[threadIdx.x] = tot;
	__syncthreads();
	for (int o = 1; o < kScanThreads; o <<= 1) {
		const unsigned add = threadIdx.x >= (unsigned)o ? s[threadIdx.x - o] : 0u;
		__syncthreads();
		s[threadIdx.x] += add;
		__syncthreads();
	}
	unsigned run = s[threadIdx.x] - tot;
#pragma unroll
	for (int i = 0; i < kScanPer; i++) {
		if (base + i < n) data[base + i] = run;
		run += v[i];
	}
	if (threadIdx.x == kScanThreads - 1) sums[blockIdx.x] = s[threadIdx.x];
}

__global__ void scan_add_kernel(unsigned *__restrict__ data, size_t n, const unsigned *__restrict__ sums)
{
	const size_t base = (size_t)blockIdx.x * kScanBlock;
	const unsigned add = sums[blockIdx.x];
	for (int i = threadIdx.x; i < kScanBlock; i += blockDim.x)
		if (base + i < n) data[base + i] += add;
}

// ---------------------------------------------------------------------------
// ordered gather into one tile's sums (one 8x8 pixel block of one frame)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kGatherThreads)
gather_kernel(Tile T, StepParams sp, int f_lo, const unsigned *__restrict__ off,
              const unsigned *__restrict__ list, const float *__restrict__ vals,
              const float *__restrict__ wslot, const float *__restrict__ win,
              float *__restrict__ acc, float *__restrict__ wacc)
{
	__shared__ unsigned s_start[kRegionMax], s_len[kRegionMax], s_pos[kRegionMax + 1];
	__shared__ unsigned long long s_key[kEntryCap];
	__shared__ float s_win[kMaxSpc];
	const int px = sp.px, pt = sp.pt, spc = sp.spc, C = sp.C;
	const int bx0 = blockIdx.x * kGatherBX, by0 = blockIdx.y * kGatherBY;
	const int t = f_lo + blockIdx.z;
	const int RX = kGatherBX + px - 1, RY = kGatherBY + px - 1, RT = pt;
	const int NR = RX * RY * RT;
	const int tid = threadIdx.x;
	for (int i = tid; i < spc; i += blockDim.x) s_win[i] = win[i];

	// lists of every origin that can cover the block: x in [bx0-px+1, bx0+8) ...
	for (int r = tid; r < NR; r += blockDim.x) {
		const int rx = r % RX, ry = (r / RX) % RY, rt = r / (RX * RY);
		const int ox = bx0 - px + 1 + rx, oy = by0 - px + 1 + ry, ot = t - pt + 1 + rt;
		unsigned st = 0, ln = 0;
		if (ox >= 0 && oy >= 0 && ot >= 0 && ox <= T.w - px && oy <= T.h - px && ot <= sp.F - pt) {
			const size_t lin = ((size_t)ot * T.h + oy) * T.w + ox;
			st = off[lin];
			ln = off[lin + 1] - st;
		}
		s_start[r] = st;
		s_len[r] = ln;
	}
	__syncthreads();
	if (tid == 0) {
		unsigned run = 0;
		for (int r = 0; r < NR; r++) { s_pos[r] = run; run += s_len[r]; }
		s_pos[NR] = run;
	}
	__syncthreads();
	const unsigned E = s_pos[NR];

	const int lx = tid % kGatherBX, ly = tid / kGatherBX;
	const int x = bx0 + lx, y = by0 + ly;
	const bool inside = x < T.w && y < T.h;
	float a[4] = {0.f, 0.f, 0.f, 0.f}, wa = 0.f;
	size_t pix = 0;
	if (inside) {
		pix = ((size_t)t * T.h + y) * T.w + x;
		wa = wacc[pix];
		for (int c = 0; c < C; c++) a[c] = acc[(((size_t)t * C + c) * T.h + y) * T.w + x];
	}

	if (E <= (unsigned)kEntryCap) {
		unsigned P2 = 1;
		while (P2 < E) P2 <<= 1;
		for (int r = tid; r < NR; r += blockDim.x)
			for (unsigned j = 0; j < s_len[r]; j++)
				s_key[s_pos[r] + j] = ((unsigned long long)list[s_start[r] + j] << 32) | (unsigned)r;
		for (unsigned i = E + tid; i < P2; i += blockDim.x) s_key[i] = ~0ull;
		__syncthreads();
		// bitonic sort by slot number
		for (unsigned k = 2; k <= P2; k <<= 1)
			for (unsigned j = k >> 1; j > 0; j >>= 1) {
				for (unsigned i = tid; i < P2; i += blockDim.x) {
					const unsigned l = i ^ j;
					if (l > i) {
						const unsigned long long u = s_key[i], v = s_key[l];
						const bool up = (i & k) == 0;
						if ((u > v) == up) { s_key[i] = v; s_key[l] = u; }
					}
				}
				__syncthreads();
			}
		if (inside) {
			for (unsigned e = 0; e < E; e++) {
				const unsigned long long key = s_key[e];
				const int r = (int)(key & 0xffffffffull);
				const int rx = r % RX, ry = (r / RX) % RY, rt = r / (RX * RY);
				const int dx = lx + px - 1 - rx, dy = ly + px - 1 - ry, dt = pt - 1 - rt;
				if (dx < 0 || dx >= px || dy < 0 || dy >= px) continue;
				const size_t slot = key >> 32;
				const int p = (dt * px + dy) * px + dx;
				const float *v = vals + slot * (size_t)(C * spc);
				for (int c = 0; c < C; c++) a[c] = __fadd_rn(a[c], v[c * spc + p]);
				wa = __fadd_rn(wa, __fmul_rn(wslot[slot], s_win[p]));
			}
		}
	} else if (inside) {
		// too many slots for shared memory: merge this pixel's own lists (one
		// list per patch offset p), smallest slot number first
		const int NL = px * px * pt;
		unsigned cur[kMaxSpc], end[kMaxSpc];
		for (int l = 0; l < NL; l++) {
			const int dx = l % px, dy = (l / px) % px, dt = l / (px * px);
			const int r = ((pt - 1 - dt) * RY + (ly + px - 1 - dy)) * RX + (lx + px - 1 - dx);
			cur[l] = s_start[r];
			end[l] = s_start[r] + s_len[r];
		}
		for (;;) {
			unsigned best = 0xffffffffu;
			int bl = -1;
			for (int l = 0; l < NL; l++)
				if (cur[l] < end[l]) {
					const unsigned s = list[cur[l]];
					if (s < best) { best = s; bl = l; }
				}
			if (bl < 0) break;
			cur[bl]++;
			const float *v = vals + (size_t)best * (C * spc);
			for (int c = 0; c < C; c++) a[c] = __fadd_rn(a[c], v[c * spc + bl]);
			wa = __fadd_rn(wa, __fmul_rn(wslot[best], s_win[bl]));
		}
	}
	if (inside) {
		wacc[pix] = wa;
		for (int c = 0; c < C; c++) acc[(((size_t)t * C + c) * T.h + y) * T.w + x] = a[c];
	}
}

// ---------------------------------------------------------------------------
// colour transforms (src/utils/lib_videot.hpp:727-838), same float expressions
// ---------------------------------------------------------------------------
__device__ __forceinline__ void yuv_forward(float *v, int C)
{
	if (C == 3) {
		const float a = __fdiv_rn(1.f, sqrtf(3.f));
		const float b = __fdiv_rn(1.f, sqrtf(2.f));
		const float c = __fmul_rn(__fmul_rn(2.f, a), sqrtf(2.f));
		const float r = v[0], g = v[1], bl = v[2];
		v[0] = __fmul_rn(a, __fadd_rn(__fadd_rn(r, g), bl));
		v[1] = __fmul_rn(b, __fsub_rn(r, bl));
		v[2] = __fmul_rn(c, __fadd_rn(__fsub_rn(__fmul_rn(0.25f, r), __fmul_rn(0.5f, g)), __fmul_rn(0.25f, bl)));
	} else if (C == 4) {
		const float a = 0.5f;
		const float b = __fdiv_rn(1.f, sqrtf(2.f));
		const float Gr = v[0], R = v[1], B = v[2], Gb = v[3];
		v[0] = __fmul_rn(a, __fadd_rn(__fadd_rn(__fadd_rn(Gr, R), B), Gb));
		v[1] = __fmul_rn(b, __fsub_rn(R, B));
		v[2] = __fmul_rn(a, __fsub_rn(__fadd_rn(__fadd_rn(-Gr, R), B), Gb));
		v[3] = __fmul_rn(b, __fadd_rn(-Gr, Gb));
	}
}

__device__ __forceinline__ void yuv_inverse(float *v, int C)
{
	if (C == 3) {
		const float a = __fdiv_rn(1.f, sqrtf(3.f));
		const float b = __fdiv_rn(1.f, sqrtf(2.f));
		const float c = __fdiv_rn(a, b);
		const float ch = __fmul_rn(c, 0.5f);
		const float y = v[0], u = v[1], w = v[2];
		v[0] = __fadd_rn(__fadd_rn(__fmul_rn(a, y), __fmul_rn(b, u)), __fmul_rn(ch, w));
		v[1] = __fsub_rn(__fmul_rn(a, y), __fmul_rn(c, w));
		v[2] = __fadd_rn(__fsub_rn(__fmul_rn(a, y), __fmul_rn(b, u)), __fmul_rn(ch, w));
	} else if (C == 4) {
		const float a = 0.5f;
		const float b = __fdiv_rn(1.f, sqrtf(2.f));
		const float Gr = v[0], R = v[1], B = v[2], Gb = v[3];
		v[0] = __fsub_rn(__fsub_rn(__fmul_rn(a, Gr), __fmul_rn(a, B)), __fmul_rn(b, Gb));
		v[1] = __fadd_rn(__fadd_rn(__fmul_rn(a, Gr), __fmul_rn(b, R)), __fmul_rn(a, B));
		v[2] = __fadd_rn(__fsub_rn(__fmul_rn(a, Gr), __fmul_rn(b, R)), __fmul_rn(a, B));
		v[3] = __fadd_rn(__fsub_rn(__fmul_rn(a, Gr), __fmul_rn(a, B)), __fmul_rn(b, Gb));
	}
}

__global__ void color_kernel(Image in, Image out, int forward)
{
	const long long n = (long long)in.W * in.H * in.F;
	for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
	     i += (long long)gridDim.x * blockDim.x) {
		const int x = (int)(i % in.W), y = (int)((i / in.W) % in.H), t = (int)(i / ((long long)in.W * in.H));
		float v[4];
		for (int c = 0; c < in.C; c++) v[c] = in.p[in.at(x, y, t, c)];
		if (forward) yuv_forward(v, in.C); else yuv_inverse(v, in.C);
		for (int c = 0; c < in.C; c++) out.p[out.at(x, y, t, c)] = v[c];
	}
}

// computeWeightedAggregation (nldct.cpp:2436-2448) on every tile, then the
// inner-region rebuild of subBuildTight (lib_videot.hpp:1101-1163) and the
// inverse colour transform: one thread per output pixel.
__global__ void finalize_kernel(const Tile *__restrict__ tiles, int nW, int wTmp, int hTmp, StepParams sp,
                                Image noisy, const float *__restrict__ acc, const float *__restrict__ wacc,
                                Image out, int inverse_color)
{
	const long long n = (long long)out.W * out.H * out.F;
	for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
	     i += (long long)gridDim.x * blockDim.x) {
		const int X = (int)(i % out.W), Y = (int)((i / out.W) % out.H);
		const int t = (int)(i / ((long long)out.W * out.H));
		const Tile T = tiles[(Y / hTmp) * nW + X / wTmp];
		const int x = X - T.ox, y = Y - T.oy;
		const size_t pix = ((size_t)t * T.h + y) * T.w + x;
		const float wt = wacc[T.pix0 + pix];
		float v[4];
		for (int c = 0; c < sp.C; c++) {
			const float a = acc[T.pix0 * sp.C + (((size_t)t * sp.C + c) * T.h + y) * T.w + x];
			v[c] = wt > 0.f ? __fdiv_rn(a, wt) : __fdiv_rn(a, noisy.p[noisy.at(X, Y, t, c)]);
		}
		if (inverse_color) yuv_inverse(v, sp.C);
		for (int c = 0; c < sp.C; c++) out.p[out.at(X, Y, t, c)] = v[c];
	}
}

inline int grid_for(long long n, int threads, int cap = 65535)
{
	long long b = (n + threads - 1) / threads;
	if (b < 1) b = 1;
	return (int)(b < cap ? b : cap);
}

}  // namespace

cudaError_t launch_kill_edges(const Tile *tiles, int ntiles, const int *grid, const int *inv,
                              const StepParams &sp, long long G, const uint32_t *idx,
                              unsigned long long *edges, unsigned *nedges, unsigned cap, cudaStream_t st)
{
	kill_edges_kernel<<<grid_for(G, 256, 8192), 256, 0, st>>>(tiles, ntiles, grid, inv, sp, G, idx, edges, nedges, cap);
	return cudaGetLastError();
}

cudaError_t launch_kill_iteration(const unsigned long long *edges, unsigned n, uint8_t *alive, uint8_t *killed,
                                  unsigned *changed, cudaStream_t st)
{
	const int b = grid_for(n, 256, 8192);
	kill_mark_kernel<<<b, 256, 0, st>>>(edges, n, alive, killed, 1);
	kill_mark_kernel<<<b, 256, 0, st>>>(edges, n, alive, killed, 0);
	kill_apply_kernel<<<b, 256, 0, st>>>(edges, n, killed, alive, changed);
	return cudaGetLastError();
}

cudaError_t launch_count_alive(const Tile *tiles, int ntiles, long long G, const uint8_t *alive,
                               unsigned *counts, cudaStream_t st)
{
	count_alive_kernel<<<grid_for(G, 256, 8192), 256, 0, st>>>(tiles, ntiles, G, alive, counts);
	return cudaGetLastError();
}

// Exclusive scan of data[0..n) in place; data[n] receives the total.
cudaError_t exclusive_scan(unsigned *data, size_t n, unsigned *scratch, cudaStream_t st)
{
	// data must hold n+1 entries; scratch needs ceil(n/4096) + ceil(n/4096^2) + 2 entries
	const size_t nb = (n + 1 + kScanBlock - 1) / kScanBlock;
	scan_block_kernel<<<(unsigned)nb, kScanThreads, 0, st>>>(data, n + 1, scratch);
	if (nb > 1) {
		cudaError_t e = exclusive_scan(scratch, nb - 1, scratch + nb + 1, st);
		if (e != cudaSuccess) return e;
		scan_add_kernel<<<(unsigned)nb, 256, 0, st>>>(data, n + 1, scratch);
	}
	return cudaGetLastError();
}

cudaError_t launch_lists(long long ga, long long gb, int np, const uint8_t *nsimp, const uint32_t *idx,
                         const uint8_t *alive, size_t npos, unsigned *cnt, unsigned *off, unsigned *list,
                         unsigned *scratch, cudaStream_t st)
{
	cudaError_t e = cudaMemsetAsync(off, 0, (npos + 1) * sizeof(unsigned), st);
	if (e != cudaSuccess) return e;
	const long long ns = (gb - ga) * np;
	list_count_kernel<<<grid_for(ns, 256, 16384), 256, 0, st>>>(ga, gb, np, nsimp, idx, alive, off);
	e = exclusive_scan(off, npos, scratch, st);
	if (e != cudaSuccess) return e;
	e = cudaMemsetAsync(cnt, 0, npos * sizeof(unsigned), st);
	if (e != cudaSuccess) return e;
	list_fill_kernel<<<grid_for(ns, 256, 16384), 256, 0, st>>>(ga, gb, np, nsimp, idx, alive, off, cnt, list);
	list_sort_kernel<<<grid_for((long long)npos, 256, 16384), 256, 0, st>>>(npos, off, list);
	return cudaGetLastError();
}

cudaError_t launch_gather(const Tile &T, const StepParams &sp, int f_lo, int f_hi, const unsigned *off,
                          const unsigned *list, const float *vals, const float *wslot, const float *win,
                          float *acc, float *wacc, cudaStream_t st)
{
	if (f_hi < f_lo) return cudaSuccess;
	dim3 grid((T.w + kGatherBX - 1) / kGatherBX, (T.h + kGatherBY - 1) / kGatherBY, f_hi - f_lo + 1);
	gather_kernel<<<grid, kGatherThreads, 0, st>>>(T, sp, f_lo, off, list, vals, wslot, win, acc, wacc);
	return cudaGetLastError();
}

int gather_region(const StepParams &sp)
{
	return (kGatherBX + sp.px - 1) * (kGatherBY + sp.px - 1) * sp.pt;
}
int gather_region_max() { return kRegionMax; }

cudaError_t launch_color(const Image &in, const Image &out, int forward, cudaStream_t st)
{
	color_kernel<<<grid_for((long long)in.W * in.H * in.F, 256, 16384), 256, 0, st>>>(in, out, forward);
	return cudaGetLastError();
}

cudaError_t launch_finalize(const Tile *tiles, int nW, int wTmp, int hTmp, const StepParams &sp,
                            const Image &noisy, const float *acc, const float *wacc, const Image &out,
                            int inverse_color, cudaStream_t st)
{
	finalize_kernel<<<grid_for((long long)out.W * out.H * out.F, 256, 16384), 256, 0, st>>>(
		tiles, nW, wTmp, hTmp, sp, noisy, acc, wacc, out, inverse_color);
	return cudaGetLastError();
}

}  // namespace bm4dof
