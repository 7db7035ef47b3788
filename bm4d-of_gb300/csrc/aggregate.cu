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
#include "internal.hpp"

namespace bm4dof {

namespace {


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

// The switch-offs as a fixed point on the device: a victim is dead when a
// live killer points at it; repeat until nothing changes (at most n + 1
// rounds: every round that changes something settles at least one more
// group).  One CTA, so that the rounds need only CTA barriers.
__global__ void __launch_bounds__(1024)
kill_fixpoint_kernel(const unsigned long long *__restrict__ edges, const unsigned *__restrict__ nedges,
                     unsigned cap, uint8_t *__restrict__ alive, uint8_t *__restrict__ killed)
{
	__shared__ int changed;
	const unsigned n = min(*nedges, cap);
	for (unsigned round = 0; round <= n; round++) {
		for (unsigned e = threadIdx.x; e < n; e += blockDim.x) killed[edges[e] & 0xffffffffull] = 0;
		if (threadIdx.x == 0) changed = 0;
		__syncthreads();
		for (unsigned e = threadIdx.x; e < n; e += blockDim.x) {
			const unsigned long long v = edges[e];
			if (alive[v >> 32]) killed[v & 0xffffffffull] = 1;
		}
		__syncthreads();
		for (unsigned e = threadIdx.x; e < n; e += blockDim.x) {
			const long long w = (long long)(edges[e] & 0xffffffffull);
			const uint8_t a = killed[w] ? 0 : 1;
			if (alive[w] != a) {
				alive[w] = a;
				changed = 1;
			}
		}
		__syncthreads();
		if (!changed) break;
		__syncthreads();
	}
}

// Paste trick (doPasteBoost, nldct.cpp:2302-2322 and 2395-2415): a
// processed group switches off every member's position and its four
// neighbours outside the border band of 2*sPx (linear offsets -w, +w, -1, +1,
// so a band wider than the tile crosses rows; unsigned comparisons as the
// reference's).  Only reference positions are ever read from the mask, so a
// switch-off is an edge from a group to a later group of its tile, and a
// group is processed exactly when none of its killers is:
//     alive(g) = no alive k < g with an edge k -> g,
// the reference's sequential order restated as a recursion with one solution.
// It is evaluated by frontier rounds: a group is settled dead as soon as one
// killer is alive, alive once all its killers are dead (a count of pending
// killers per group); each settled group is pushed once and, when popped,
// settles or counts down its victims.  The first rounds run over the whole
// GPU, the tail in one CTA; every round count is fixed on the host side, so
// the sequence is stream ordered and graph capturable.
constexpr unsigned kUndecided = 0u, kAlive = 1u, kDead = 2u;

template <class Fn>
__device__ __forceinline__ void paste_victims(const Tile &T, const int *__restrict__ grid, const StepParams &sp,
                                              long long g, const uint8_t *__restrict__ nsimp,
                                              const uint32_t *__restrict__ idx, Fn fn)
{
	const unsigned w = (unsigned)T.w, h = (unsigned)T.h, band = 2u * (unsigned)sp.px, F = (unsigned)sp.F;
	const int ns = nsimp[g];
	for (int m = 0; m < ns; m++) {
		// member position as the one-channel mask index (t*h + y)*w + x
		const unsigned ind1 = idx[g * sp.np + m];
		const unsigned mx = ind1 % w, my = (ind1 / w) % h, mt = ind1 / (w * h);
#pragma unroll
		for (int q = 0; q < 5; q++) {
			unsigned vx = mx, vy = my, vt = mt;
			if (q == 1) { if (!(my > band)) continue; vy = my - 1; }
			if (q == 2) {
				if (!(my < h - band)) continue;
				if (++vy == h) { vy = 0; vt++; }
			}
			if (q == 3) { if (!(mx > band)) continue; vx = mx - 1; }
			if (q == 4) {
				if (!(mx < w - band)) continue;
				if (++vx == w) { vx = 0; if (++vy == h) { vy = 0; vt++; } }
			}
			if (vt >= F) continue;                          // past the mask
			const int xi = grid[T.gx + T.nx + vx], yi = grid[T.gy + T.ny + vy], fi = grid[T.gf + T.nf + vt];
			if (xi < 0 || yi < 0 || fi < 0) continue;       // not a reference position
			const long long v = T.g0 + ((long long)fi * T.ny + yi) * T.nx + xi;
			if (v > g) fn(v);                               // earlier groups are settled already
		}
	}
}

__global__ void paste_count_kernel(const Tile *__restrict__ tiles, int ntiles, const int *__restrict__ grid,
                                   StepParams sp, long long G, const uint8_t *__restrict__ nsimp,
                                   const uint32_t *__restrict__ idx, unsigned *__restrict__ pending)
{
	for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < G;
	     g += (long long)gridDim.x * blockDim.x) {
		const Tile T = tiles[tile_of(tiles, ntiles, g)];
		paste_victims(T, grid, sp, g, nsimp, idx, [&](long long v) { atomicAdd(&pending[v], 1u); });
	}
}

__global__ void paste_init_kernel(long long G, const unsigned *__restrict__ pending, unsigned *__restrict__ state,
                                  uint32_t *__restrict__ queue, unsigned *__restrict__ count)
{
	for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < G;
	     g += (long long)gridDim.x * blockDim.x) {
		const bool free_ = pending[g] == 0u;
		state[g] = free_ ? kAlive : kUndecided;
		if (free_) queue[atomicAdd(count, 1u)] = (uint32_t)g;
	}
}

// Pops group g: an alive group settles its undecided victims dead, a dead
// one counts them down (the last killer to die settles a victim alive).
__device__ __forceinline__ void paste_settle(const Tile *__restrict__ tiles, int ntiles,
                                             const int *__restrict__ grid, const StepParams &sp, long long g,
                                             const uint8_t *__restrict__ nsimp, const uint32_t *__restrict__ idx,
                                             unsigned *state, unsigned *pending, uint32_t *qout, unsigned *nout)
{
	const Tile T = tiles[tile_of(tiles, ntiles, g)];
	const unsigned sg = state[g];
	paste_victims(T, grid, sp, g, nsimp, idx, [&](long long v) {
		if (sg == kAlive) {
			if (atomicCAS(&state[v], kUndecided, kDead) == kUndecided) qout[atomicAdd(nout, 1u)] = (uint32_t)v;
		} else if (atomicSub(&pending[v], 1u) == 1u) {
			if (atomicCAS(&state[v], kUndecided, kAlive) == kUndecided) qout[atomicAdd(nout, 1u)] = (uint32_t)v;
		}
	});
}

__global__ void paste_round_kernel(const Tile *__restrict__ tiles, int ntiles, const int *__restrict__ grid,
                                   StepParams sp, const uint8_t *__restrict__ nsimp,
                                   const uint32_t *__restrict__ idx, unsigned *state, unsigned *pending,
                                   const uint32_t *__restrict__ qin, const unsigned *__restrict__ nin,
                                   uint32_t *__restrict__ qout, unsigned *nout)
{
	const unsigned n = *nin;
	for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
		paste_settle(tiles, ntiles, grid, sp, qin[i], nsimp, idx, state, pending, qout, nout);
}

// The remaining rounds in one CTA (small frontiers), until the frontier is
// empty: every group is pushed at most once, so at most G + 1 rounds.
__global__ void __launch_bounds__(1024)
paste_finish_kernel(const Tile *__restrict__ tiles, int ntiles, const int *__restrict__ grid, StepParams sp,
                    long long G, const uint8_t *__restrict__ nsimp, const uint32_t *__restrict__ idx,
                    unsigned *state, unsigned *pending, uint32_t *q0, uint32_t *q1, unsigned *n_in,
                    unsigned *n_pair)
{
	uint32_t *qin = q0, *qout = q1;
	unsigned *nin = n_in;
	for (long long r = 0; r <= G; r++) {
		unsigned *nout = n_pair + (r & 1);
		if (threadIdx.x == 0) *nout = 0u;
		__syncthreads();
		const unsigned n = *(volatile unsigned *)nin;
		if (n == 0u) break;
		for (unsigned i = threadIdx.x; i < n; i += blockDim.x)
			paste_settle(tiles, ntiles, grid, sp, qin[i], nsimp, idx, state, pending, qout, nout);
		__syncthreads();
		uint32_t *t = qin;
		qin = qout;
		qout = t;
		nin = nout;
	}
}

__global__ void paste_alive_kernel(long long G, const unsigned *__restrict__ state, uint8_t *__restrict__ alive)
{
	for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < G;
	     g += (long long)gridDim.x * blockDim.x)
		alive[g] = state[g] == kAlive ? 1 : 0;
}

__global__ void count_alive_kernel(const Tile *__restrict__ tiles, int ntiles, long long G,
                                   const uint8_t *__restrict__ alive, unsigned *__restrict__ counts)
{
	// per-thread counts of the current tile, then one atomic per group of
	// lanes holding the same tile (one counter per tile: plain per-group
	// atomics serialise on it)
	int ct = -1;
	unsigned cnt = 0;
	for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < G;
	     g += (long long)gridDim.x * blockDim.x) {
		if (!alive[g]) continue;
		const int t = tile_of(tiles, ntiles, g);
		if (t != ct) {
			if (cnt) atomicAdd(&counts[ct], cnt);
			ct = t;
			cnt = 0;
		}
		cnt++;
	}
	const unsigned same = __match_any_sync(0xffffffffu, ct);
	const unsigned total = __reduce_add_sync(same, cnt);
	if (ct >= 0 && total && (threadIdx.x & 31) == __ffs(same) - 1) atomicAdd(&counts[ct], total);
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
// spatial lists: for every tile position (x, y, t'), the slots whose origin
// lies in frame t' and whose patch covers (x, y), merged into slot order.
// Entry = slot << 6 | dy << 3 | dx (dx, dy < 8 since px <= 8).
// ---------------------------------------------------------------------------
__global__ void slist_count_kernel(int w, int h, int F, int px, int pt, int t_lo, int t_hi,
                                   const unsigned *__restrict__ off, unsigned *__restrict__ cnt)
{
	const size_t npos = (size_t)w * h * F;
	for (size_t pos = blockIdx.x * (size_t)blockDim.x + threadIdx.x; pos < npos;
	     pos += (size_t)gridDim.x * blockDim.x) {
		const int x = (int)(pos % w), y = (int)((pos / w) % h), t = (int)(pos / ((size_t)w * h));
		unsigned c = 0;
		if (t >= t_lo && t <= t_hi && t <= F - pt)
			for (int dy = 0; dy < px; dy++) {
				const int oy = y - dy;
				if (oy < 0 || oy > h - px) continue;
				for (int dx = 0; dx < px; dx++) {
					const int ox = x - dx;
					if (ox < 0 || ox > w - px) continue;
					const size_t o = ((size_t)t * h + oy) * w + ox;
					c += off[o + 1] - off[o];
				}
			}
		cnt[pos] = c;
	}
}

// PX > 0: one list per patch offset (dy, dx), held in registers; PX == 0:
// any patch size, lists compacted in local memory.
template <int PX>
__global__ void slist_build_kernel(int w, int h, int F, int px_rt, int pt, int t_lo, int t_hi,
                                   const unsigned *__restrict__ off, const unsigned *__restrict__ list,
                                   const unsigned *__restrict__ soff, unsigned *__restrict__ sl)
{
	constexpr int L = PX > 0 ? PX * PX : kMaxSpc;
	const int px = PX > 0 ? PX : px_rt;
	const size_t npos = (size_t)w * h * F;
	for (size_t pos = blockIdx.x * (size_t)blockDim.x + threadIdx.x; pos < npos;
	     pos += (size_t)gridDim.x * blockDim.x) {
		unsigned o = soff[pos];
		if (soff[pos + 1] == o) continue;
		const int x = (int)(pos % w), y = (int)((pos / w) % h), t = (int)(pos / ((size_t)w * h));
		unsigned cur[L], end[L], head[L], tag[L];
		int nl = 0;
#pragma unroll
		for (int l = 0; l < L; l++) head[l] = 0xffffffffu;
#pragma unroll
		for (int dy = 0; dy < (PX > 0 ? PX : 8); dy++) {
			if (dy >= px) break;
#pragma unroll
			for (int dx = 0; dx < (PX > 0 ? PX : 8); dx++) {
				if (dx >= px) break;
				const int oy = y - dy, ox = x - dx;
				unsigned a = 0, b = 0;
				if (oy >= 0 && oy <= h - px && ox >= 0 && ox <= w - px) {
					const size_t q = ((size_t)t * h + oy) * w + ox;
					a = off[q];
					b = off[q + 1];
				}
				const int l = PX > 0 ? dy * PX + dx : nl;
				if (PX > 0 || a < b) {
					cur[l] = a; end[l] = b; tag[l] = (unsigned)(dy << 3 | dx);
					head[l] = a < b ? list[a] : 0xffffffffu;
					nl++;
				}
			}
		}
		// merge by slot number (slots are unique across lists)
		for (;;) {
			unsigned best = 0xffffffffu;
			int bl = -1;
#pragma unroll
			for (int l = 0; l < L; l++)
				if ((PX > 0 || l < nl) && head[l] < best) { best = head[l]; bl = l; }
			if (bl < 0) break;
#pragma unroll
			for (int l = 0; l < L; l++)
				if (l == bl) {
					sl[o++] = best << 6 | tag[l];
					head[l] = ++cur[l] < end[l] ? list[cur[l]] : 0xffffffffu;
				}
		}
	}
}

// Ordered gather: each pixel merges the spatial lists of the pt origin frames
// that cover it and adds the terms in slot order -- the order in which the
// reference's scatter loop adds them.  PT > 0 keeps the pt list heads in
// registers; CC is the channel count.  Each list's next entry is fetched one
// step ahead, so that the load of the term being added and the list advance
// overlap instead of forming one dependent chain per term.  A term's C
// estimates and its weight term w * window[p] sit side by side in `vals`
// (term_stride), so each term is one vector load from one 32-byte sector.
template <int PT, int CC>
__global__ void __launch_bounds__(128)
gather_slist_kernel(Tile T, StepParams sp, int f_lo, int f_hi, const unsigned *__restrict__ soff,
                    const unsigned *__restrict__ sl, const float *__restrict__ vals, float *__restrict__ acc,
                    float *__restrict__ wacc)
{
	// any other pt: up to kMaxGatherPt lists (a 64-element patch of px >= 2 has
	// at most 16 frames; runs with more patch frames are refused)
	constexpr int L = PT > 0 ? PT : kMaxGatherPt;
	const int px = sp.px, pt = PT > 0 ? PT : sp.pt, spc = sp.spc;
	const size_t wh = (size_t)T.w * T.h;
	const size_t n = wh * (size_t)(f_hi - f_lo + 1);
	for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
		const int t = f_lo + (int)(i / wh);
		const size_t xy = i % wh;
		unsigned cur[L], end[L], head[L], nxt[L];
		bool any = false;
#pragma unroll
		for (int dt = 0; dt < L; dt++) {
			head[dt] = nxt[dt] = 0xffffffffu;
			cur[dt] = end[dt] = 0;
			const int to = t - dt;
			if (dt < pt && to >= 0 && to <= sp.F - pt) {
				const size_t q = (size_t)to * wh + xy;
				cur[dt] = soff[q];
				end[dt] = soff[q + 1];
				if (cur[dt] < end[dt]) {
					head[dt] = sl[cur[dt]];
					any = true;
					if (cur[dt] + 1 < end[dt]) nxt[dt] = sl[cur[dt] + 1];
				}
			}
		}
		if (!any) continue;
		const size_t pix = (size_t)t * wh + xy;
		float a[CC];
#pragma unroll
		for (int c = 0; c < CC; c++) a[c] = acc[((size_t)t * CC + c) * wh + xy];
		float wa = wacc[pix];
		// the C estimates and the weight term of a term: one vector load
		constexpr int TS = CC == 1 ? 2 : (CC <= 3 ? 4 : 8);
		// terms are fetched D ahead of the one being added (a ring of D
		// register slots, fetched and consumed in the same rotation), so that
		// D loads of this pixel are in flight instead of one
		constexpr int D = TS == 2 ? 8 : (TS == 4 ? 4 : 2);
		auto fetch = [&](float (&x)[TS]) -> bool {
			unsigned best = 0xffffffffu;
			int bl = -1;
#pragma unroll
			for (int l = 0; l < L; l++)
				if (head[l] < best) { best = head[l]; bl = l; }
			if (bl < 0) return false;
			const unsigned slot = best >> 6;
			const int dx = best & 7, dy = (best >> 3) & 7;
			const int p = (bl * px + dy) * px + dx;
			const float *v = vals + ((size_t)slot * spc + p) * TS;
			if (TS == 2) {
				const float2 q = __ldg(reinterpret_cast<const float2 *>(v));
				x[0] = q.x;
				x[1] = q.y;
			} else {
#pragma unroll
				for (int h = 0; h < TS / 4; h++) {
					const float4 q = __ldg(reinterpret_cast<const float4 *>(v) + h);
					x[4 * h] = q.x;
					x[4 * h + 1] = q.y;
					x[4 * h + 2] = q.z;
					x[4 * h + 3] = q.w;
				}
			}
#pragma unroll
			for (int l = 0; l < L; l++)
				if (l == bl) {
					head[l] = nxt[l];
					cur[l]++;
					nxt[l] = cur[l] + 1 < end[l] ? __ldg(sl + cur[l] + 1) : 0xffffffffu;
				}
			return true;
		};
		float x[D][TS];
		bool ok[D];
#pragma unroll
		for (int d = 0; d < D; d++) ok[d] = fetch(x[d]);
		bool live = true;
		while (live) {
#pragma unroll
			for (int d = 0; d < D; d++) {
				if (live && !ok[d]) live = false;
				if (live) {
#pragma unroll
					for (int c = 0; c < CC; c++) a[c] = __fadd_rn(a[c], x[d][c]);
					wa = __fadd_rn(wa, x[d][CC]);   // w * window[p], as the reference forms it
					ok[d] = fetch(x[d]);
				}
			}
		}
		wacc[pix] = wa;
#pragma unroll
		for (int c = 0; c < CC; c++) acc[((size_t)t * CC + c) * wh + xy] = a[c];
	}
}

// ---------------------------------------------------------------------------
// Quad path (4x4 patches): one thread per quad of 4 horizontally adjacent
// pixels.  A member patch whose origin lies in row oy and column ox covers
// quads (ox+3)/4 and ox/4 (one quad when ox is a multiple of 4), so a
// quad's list holds about 7/16 of the entries of its four pixels' lists, and
// the four pixels' terms of one member row sit in one 32-byte sector that a
// single thread reads.  Lists are indexed by quad position
// ((to - t_lo) * h + y) * nq + q over the chunk's origin frames [t_lo, t_hi].
// ---------------------------------------------------------------------------
constexpr int kQuad = 4;

// row lists: for quad q, origin row oy and origin frame to, the slots whose
// origin column lies in [4q-3, 4q+3], merged into slot order.  The origin
// lists of consecutive columns are consecutive in `list`, so the count is one
// difference of offsets.  Entry = slot << 3 | (ox - 4q + 3).
__global__ void rlist_count_kernel(int w, int h, int nq, int t_lo, int nf, const unsigned *__restrict__ off,
                                   unsigned *__restrict__ cnt)
{
	const size_t n = (size_t)nq * h * nf;
	for (size_t pos = blockIdx.x * (size_t)blockDim.x + threadIdx.x; pos < n;
	     pos += (size_t)gridDim.x * blockDim.x) {
		const int q = (int)(pos % nq), oy = (int)((pos / nq) % h), to = t_lo + (int)(pos / ((size_t)nq * h));
		const int lo = max(0, kQuad * q - 3), hi = min(w - kQuad, kQuad * q + 3);
		unsigned c = 0;
		if (oy <= h - kQuad && lo <= hi) {
			const size_t base = ((size_t)to * h + oy) * w;
			c = off[base + hi + 1] - off[base + lo];
		}
		cnt[pos] = c;
	}
}

__global__ void rlist_build_kernel(int w, int h, int nq, int t_lo, int nf, const unsigned *__restrict__ off,
                                   const unsigned *__restrict__ list, const unsigned *__restrict__ roff,
                                   unsigned *__restrict__ rl)
{
	constexpr int L = 2 * kQuad - 1;
	const size_t n = (size_t)nq * h * nf;
	for (size_t pos = blockIdx.x * (size_t)blockDim.x + threadIdx.x; pos < n;
	     pos += (size_t)gridDim.x * blockDim.x) {
		unsigned o = roff[pos];
		if (roff[pos + 1] == o) continue;
		const int q = (int)(pos % nq), oy = (int)((pos / nq) % h), to = t_lo + (int)(pos / ((size_t)nq * h));
		const size_t base = ((size_t)to * h + oy) * w;
		unsigned cur[L], end[L], head[L];
#pragma unroll
		for (int l = 0; l < L; l++) {
			const int ox = kQuad * q - 3 + l;
			cur[l] = end[l] = 0;
			if (ox >= 0 && ox <= w - kQuad) {
				cur[l] = off[base + ox];
				end[l] = off[base + ox + 1];
			}
			head[l] = cur[l] < end[l] ? list[cur[l]] : 0xffffffffu;
		}
		for (;;) {
			unsigned best = 0xffffffffu;
			int bl = -1;
#pragma unroll
			for (int l = 0; l < L; l++)
				if (head[l] < best) { best = head[l]; bl = l; }
			if (bl < 0) break;
			rl[o++] = best << 3 | (unsigned)bl;
#pragma unroll
			for (int l = 0; l < L; l++)
				if (l == bl) head[l] = ++cur[l] < end[l] ? list[cur[l]] : 0xffffffffu;
		}
	}
}

// quad lists: for quad q, pixel row y and origin frame to, the row lists of
// origin rows y-3..y merged into slot order.  Entry = slot << 5 | dy << 3 |
// (ox - 4q + 3), dy = y - oy.
__global__ void qlist_count_kernel(int h, int nq, int nf, const unsigned *__restrict__ roff,
                                   unsigned *__restrict__ cnt)
{
	const size_t n = (size_t)nq * h * nf;
	for (size_t pos = blockIdx.x * (size_t)blockDim.x + threadIdx.x; pos < n;
	     pos += (size_t)gridDim.x * blockDim.x) {
		const int y = (int)((pos / nq) % h);
		unsigned c = 0;
#pragma unroll
		for (int dy = 0; dy < kQuad; dy++) {
			const int oy = y - dy;
			if (oy < 0 || oy > h - kQuad) continue;
			const size_t r = pos - (size_t)dy * nq;
			c += roff[r + 1] - roff[r];
		}
		cnt[pos] = c;
	}
}

__global__ void qlist_build_kernel(int h, int nq, int nf, const unsigned *__restrict__ roff,
                                   const unsigned *__restrict__ rl, const unsigned *__restrict__ qoff,
                                   unsigned *__restrict__ ql)
{
	const size_t n = (size_t)nq * h * nf;
	for (size_t pos = blockIdx.x * (size_t)blockDim.x + threadIdx.x; pos < n;
	     pos += (size_t)gridDim.x * blockDim.x) {
		unsigned o = qoff[pos];
		if (qoff[pos + 1] == o) continue;
		const int y = (int)((pos / nq) % h);
		unsigned cur[kQuad], end[kQuad], head[kQuad];
#pragma unroll
		for (int dy = 0; dy < kQuad; dy++) {
			const int oy = y - dy;
			cur[dy] = end[dy] = 0;
			if (oy >= 0 && oy <= h - kQuad) {
				const size_t r = pos - (size_t)dy * nq;
				cur[dy] = roff[r];
				end[dy] = roff[r + 1];
			}
			head[dy] = cur[dy] < end[dy] ? rl[cur[dy]] : 0xffffffffu;
		}
		for (;;) {
			unsigned best = 0xffffffffu;
			int bl = -1;
#pragma unroll
			for (int l = 0; l < kQuad; l++)
				if (head[l] < best) { best = head[l]; bl = l; }
			if (bl < 0) break;
			ql[o++] = (best >> 3) << 5 | (unsigned)bl << 3 | (best & 7u);
#pragma unroll
			for (int l = 0; l < kQuad; l++)
				if (l == bl) head[l] = ++cur[l] < end[l] ? rl[cur[l]] : 0xffffffffu;
		}
	}
}

// Ordered gather, quad path: each thread merges the quad lists of the pt
// origin frames covering its four pixels and adds each member's terms in
// slot order, the order of the reference's scatter loop for every pixel.  A
// member adds to the pixels j of the quad with 0 <= j - s < 4 (s = ox - 4q),
// from element dx = j - s of its row.  Members are fetched D ahead of the one
// being added (a register ring consumed in fetch order).  One member ahead
// measured best on 1920x1080x60 (aggregation 434 ms per step against 446 ms
// with two and 533 ms with four): fewer registers, more resident warps; the
// batched runs' tuning may choose two (gather_depth).
template <int PT, int CC, int D>
__global__ void __launch_bounds__(128)
gather_quad_kernel(Tile T, StepParams sp, int t_lo, int t_hi, int f_hi, int nq, const unsigned *__restrict__ qoff,
                   const unsigned *__restrict__ ql, const float *__restrict__ vals, float *__restrict__ acc,
                   float *__restrict__ wacc)
{
	constexpr int TS = CC == 1 ? 2 : (CC <= 3 ? 4 : 8);
	const int w = T.w, h = T.h, spc = sp.spc;
	const size_t wh = (size_t)w * h, plane = (size_t)nq * h;
	const size_t n = plane * (size_t)(f_hi - t_lo + 1);
	for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
		const int t = t_lo + (int)(i / plane);
		const size_t r = i % plane;
		const int y = (int)(r / nq), q = (int)(r % nq);
		unsigned cur[PT], end[PT], head[PT], nxt[PT];
		bool any = false;
#pragma unroll
		for (int dt = 0; dt < PT; dt++) {
			head[dt] = nxt[dt] = 0xffffffffu;
			cur[dt] = end[dt] = 0;
			const int to = t - dt;
			if (to >= t_lo && to <= t_hi) {
				const size_t qp = ((size_t)(to - t_lo) * h + y) * nq + q;
				cur[dt] = qoff[qp];
				end[dt] = qoff[qp + 1];
				if (cur[dt] < end[dt]) {
					head[dt] = __ldg(ql + cur[dt]);
					any = true;
					if (cur[dt] + 1 < end[dt]) nxt[dt] = __ldg(ql + cur[dt] + 1);
				}
			}
		}
		if (!any) continue;
		const int x0 = kQuad * q;
		const size_t pix = (size_t)t * wh + (size_t)y * w + x0;
		float a[kQuad][CC], wa[kQuad];
#pragma unroll
		for (int j = 0; j < kQuad; j++) {
			const bool in = x0 + j < w;
#pragma unroll
			for (int c = 0; c < CC; c++) a[j][c] = in ? acc[((size_t)t * CC + c) * wh + (size_t)y * w + x0 + j] : 0.f;
			wa[j] = in ? wacc[pix + j] : 0.f;
		}
		auto fetch = [&](float (&x)[kQuad][TS], unsigned &m) -> bool {
			unsigned best = 0xffffffffu;
			int bl = -1;
#pragma unroll
			for (int l = 0; l < PT; l++)
				if (head[l] < best) { best = head[l]; bl = l; }
			if (bl < 0) return false;
			const unsigned slot = best >> 5;
			const int dy = (best >> 3) & 3, s = (int)(best & 7u) - 3;
			const float *row = vals + ((size_t)slot * spc + (bl * kQuad + dy) * kQuad) * TS;
			m = 0;
#pragma unroll
			for (int j = 0; j < kQuad; j++) {
				const int dx = j - s;
				if ((unsigned)dx < (unsigned)kQuad) {
					m |= 1u << j;
					if (TS == 2) {
						const float2 v = __ldg(reinterpret_cast<const float2 *>(row + dx * TS));
						x[j][0] = v.x;
						x[j][1] = v.y;
					} else {
#pragma unroll
						for (int k = 0; k < TS / 4; k++) {
							const float4 v = __ldg(reinterpret_cast<const float4 *>(row + dx * TS) + k);
							x[j][4 * k] = v.x;
							x[j][4 * k + 1] = v.y;
							x[j][4 * k + 2] = v.z;
							x[j][4 * k + 3] = v.w;
						}
					}
				}
			}
#pragma unroll
			for (int l = 0; l < PT; l++)
				if (l == bl) {
					head[l] = nxt[l];
					cur[l]++;
					nxt[l] = cur[l] + 1 < end[l] ? __ldg(ql + cur[l] + 1) : 0xffffffffu;
				}
			return true;
		};
		float x[D][kQuad][TS];
		unsigned m[D];
		bool ok[D];
#pragma unroll
		for (int d = 0; d < D; d++) ok[d] = fetch(x[d], m[d]);
		bool live = true;
		while (live) {
#pragma unroll
			for (int d = 0; d < D; d++) {
				if (live && !ok[d]) live = false;
				if (live) {
#pragma unroll
					for (int j = 0; j < kQuad; j++)
						if (m[d] >> j & 1u) {
#pragma unroll
							for (int c = 0; c < CC; c++) a[j][c] = __fadd_rn(a[j][c], x[d][j][c]);
							wa[j] = __fadd_rn(wa[j], x[d][j][CC]);   // w * window[p], as the reference forms it
						}
					ok[d] = fetch(x[d], m[d]);
				}
			}
		}
#pragma unroll
		for (int j = 0; j < kQuad; j++)
			if (x0 + j < w) {
#pragma unroll
				for (int c = 0; c < CC; c++) acc[((size_t)t * CC + c) * wh + (size_t)y * w + x0 + j] = a[j][c];
				wacc[pix + j] = wa[j];
			}
	}
}

template <int CC, int D>
void gather_quad_d(int gb, cudaStream_t st, const Tile &T, const StepParams &sp, int t_lo, int t_hi, int f_hi,
                   int nq, const unsigned *qoff, const unsigned *ql, const float *vals, float *acc, float *wacc)
{
	switch (sp.pt) {
	case 1:
		gather_quad_kernel<1, CC, D><<<gb, 128, 0, st>>>(T, sp, t_lo, t_hi, f_hi, nq, qoff, ql, vals, acc, wacc);
		break;
	case 2:
		gather_quad_kernel<2, CC, D><<<gb, 128, 0, st>>>(T, sp, t_lo, t_hi, f_hi, nq, qoff, ql, vals, acc, wacc);
		break;
	default:
		gather_quad_kernel<4, CC, D><<<gb, 128, 0, st>>>(T, sp, t_lo, t_hi, f_hi, nq, qoff, ql, vals, acc, wacc);
		break;
	}
}

template <int CC>
void gather_quad_pt(int gb, cudaStream_t st, const Tile &T, const StepParams &sp, int t_lo, int t_hi, int f_hi,
                    int nq, const unsigned *qoff, const unsigned *ql, const float *vals, float *acc, float *wacc)
{
	if (sp.gather_depth == 2) gather_quad_d<CC, 2>(gb, st, T, sp, t_lo, t_hi, f_hi, nq, qoff, ql, vals, acc, wacc);
	else gather_quad_d<CC, 1>(gb, st, T, sp, t_lo, t_hi, f_hi, nq, qoff, ql, vals, acc, wacc);
}

template <int CC>
void gather_pt(int gb, cudaStream_t st, const Tile &T, const StepParams &sp, int t_lo, int f_hi,
               const unsigned *soff, const unsigned *sl, const float *vals, float *acc, float *wacc)
{
	switch (sp.pt) {
	case 1: gather_slist_kernel<1, CC><<<gb, 128, 0, st>>>(T, sp, t_lo, f_hi, soff, sl, vals, acc, wacc); break;
	case 2: gather_slist_kernel<2, CC><<<gb, 128, 0, st>>>(T, sp, t_lo, f_hi, soff, sl, vals, acc, wacc); break;
	case 4: gather_slist_kernel<4, CC><<<gb, 128, 0, st>>>(T, sp, t_lo, f_hi, soff, sl, vals, acc, wacc); break;
	default: gather_slist_kernel<0, CC><<<gb, 128, 0, st>>>(T, sp, t_lo, f_hi, soff, sl, vals, acc, wacc); break;
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

cudaError_t launch_kill_fixpoint(const unsigned long long *edges, const unsigned *nedges, unsigned cap,
                                 uint8_t *alive, uint8_t *killed, cudaStream_t st)
{
	kill_fixpoint_kernel<<<1, 1024, 0, st>>>(edges, nedges, cap, alive, killed);
	return cudaGetLastError();
}

cudaError_t launch_paste_resolve(const Tile *tiles, int ntiles, const int *grid, const StepParams &sp, long long G,
                                 const uint8_t *nsimp, const uint32_t *idx, PasteScratch w, uint8_t *alive, int nsm,
                                 cudaStream_t st)
{
	if (G <= 0) return cudaSuccess;
	cudaError_t e = cudaMemsetAsync(w.pending, 0, sizeof(unsigned) * (size_t)G, st);
	if (e == cudaSuccess) e = cudaMemsetAsync(w.counts, 0, sizeof(unsigned) * (kPasteRounds + 3), st);
	if (e != cudaSuccess) return e;
	const int b = grid_for(G, 256, 8 * nsm);
	paste_count_kernel<<<b, 256, 0, st>>>(tiles, ntiles, grid, sp, G, nsimp, idx, w.pending);
	paste_init_kernel<<<b, 256, 0, st>>>(G, w.pending, w.state, w.q0, w.counts);
	// the wide rounds: round r reads counts[r] and queue r & 1
	for (int r = 0; r < kPasteRounds; r++)
		paste_round_kernel<<<b, 256, 0, st>>>(tiles, ntiles, grid, sp, nsimp, idx, w.state, w.pending,
		                                      (r & 1) ? w.q1 : w.q0, w.counts + r, (r & 1) ? w.q0 : w.q1,
		                                      w.counts + r + 1);
	const bool odd = (kPasteRounds & 1) != 0;
	paste_finish_kernel<<<1, 1024, 0, st>>>(tiles, ntiles, grid, sp, G, nsimp, idx, w.state, w.pending,
	                                        odd ? w.q1 : w.q0, odd ? w.q0 : w.q1, w.counts + kPasteRounds,
	                                        w.counts + kPasteRounds + 1);
	paste_alive_kernel<<<b, 256, 0, st>>>(G, w.state, alive);
	return cudaGetLastError();
}

cudaError_t launch_count_alive(const Tile *tiles, int ntiles, long long G, const uint8_t *alive,
                               unsigned *counts, cudaStream_t st)
{
	count_alive_kernel<<<grid_for(G, 256, 8192), 256, 0, st>>>(tiles, ntiles, G, alive, counts);
	return cudaGetLastError();
}

// Kernels exclusive_scan launches for n entries.
unsigned scan_kernels(size_t n)
{
	const size_t nb = (n + 1 + kScanBlock - 1) / kScanBlock;
	return nb > 1 ? 2 + scan_kernels(nb - 1) : 1;
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
                         unsigned *scratch, unsigned *launches, cudaStream_t st)
{
	*launches += 3 + scan_kernels(npos);
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

bool quad_path(const StepParams &sp)
{
	return sp.px == kQuad && (sp.pt == 1 || sp.pt == 2 || sp.pt == 4);
}

int list_entries_per_member(const StepParams &sp)
{
	// quad path: at most 2 row-list and 8 quad-list entries per member
	return quad_path(sp) ? 10 : sp.px * sp.px;
}

cudaError_t launch_gather(const Tile &T, const StepParams &sp, int t_lo, int t_hi, const unsigned *off,
                          const unsigned *list, unsigned *cnt, unsigned *soff, unsigned *sl, size_t members,
                          unsigned *scratch, const float *vals, float *acc, float *wacc, unsigned *launches,
                          cudaStream_t st)
{
	// origin frames [t_lo, t_hi] hold the chunk's member patches; pixels of
	// frames [t_lo, t_hi + pt - 1] receive them
	if (t_hi < t_lo) return cudaSuccess;
	const int f_hi = t_hi + sp.pt - 1 < sp.F - 1 ? t_hi + sp.pt - 1 : sp.F - 1;
	if (quad_path(sp)) {
		// row-list offsets in cnt (free once the origin lists are sorted), row
		// lists then quad lists in sl
		const int nq = (T.w + kQuad - 1) / kQuad, nf = t_hi - t_lo + 1;
		const size_t nqp = (size_t)nq * T.h * nf;
		const int b = grid_for((long long)nqp, 256, 16384);
		unsigned *roff = cnt, *rl = sl, *ql = sl + 2 * members;
		*launches += 5 + 2 * scan_kernels(nqp);
		rlist_count_kernel<<<b, 256, 0, st>>>(T.w, T.h, nq, t_lo, nf, off, roff);
		cudaError_t e = exclusive_scan(roff, nqp, scratch, st);
		if (e != cudaSuccess) return e;
		rlist_build_kernel<<<b, 256, 0, st>>>(T.w, T.h, nq, t_lo, nf, off, list, roff, rl);
		qlist_count_kernel<<<b, 256, 0, st>>>(T.h, nq, nf, roff, soff);
		e = exclusive_scan(soff, nqp, scratch, st);
		if (e != cudaSuccess) return e;
		qlist_build_kernel<<<b, 256, 0, st>>>(T.h, nq, nf, roff, rl, soff, ql);
		const long long nthr = (long long)nq * T.h * (f_hi - t_lo + 1);
		const int gb = grid_for(nthr, 128, 65535);
		if (sp.C == 1) gather_quad_pt<1>(gb, st, T, sp, t_lo, t_hi, f_hi, nq, soff, ql, vals, acc, wacc);
		else if (sp.C == 3) gather_quad_pt<3>(gb, st, T, sp, t_lo, t_hi, f_hi, nq, soff, ql, vals, acc, wacc);
		else gather_quad_pt<4>(gb, st, T, sp, t_lo, t_hi, f_hi, nq, soff, ql, vals, acc, wacc);
		return cudaGetLastError();
	}
	const size_t npos = (size_t)T.w * T.h * sp.F;
	const int b = grid_for((long long)npos, 256, 16384);
	*launches += 3 + scan_kernels(npos);
	slist_count_kernel<<<b, 256, 0, st>>>(T.w, T.h, sp.F, sp.px, sp.pt, t_lo, t_hi, off, soff);
	cudaError_t e = exclusive_scan(soff, npos, scratch, st);
	if (e != cudaSuccess) return e;
	if (sp.px == 4)
		slist_build_kernel<4><<<b, 256, 0, st>>>(T.w, T.h, sp.F, sp.px, sp.pt, t_lo, t_hi, off, list, soff, sl);
	else
		slist_build_kernel<0><<<b, 256, 0, st>>>(T.w, T.h, sp.F, sp.px, sp.pt, t_lo, t_hi, off, list, soff, sl);
	const long long npix = (long long)T.w * T.h * (f_hi - t_lo + 1);
	const int gb = grid_for(npix, 128, 65535);
	if (sp.C == 1) gather_pt<1>(gb, st, T, sp, t_lo, f_hi, soff, sl, vals, acc, wacc);
	else if (sp.C == 3) gather_pt<3>(gb, st, T, sp, t_lo, f_hi, soff, sl, vals, acc, wacc);
	else gather_pt<4>(gb, st, T, sp, t_lo, f_hi, soff, sl, vals, acc, wacc);
	return cudaGetLastError();
}

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
