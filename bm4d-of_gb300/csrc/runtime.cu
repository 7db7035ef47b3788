// runtime.cu -- device context and the orchestration of VideoNLB::runNlBayes
// (src/core/nldct.cpp:267-478) on one GPU.
//
// Per step:  colour transform -> reference grid of every tile -> patch search
// of all groups -> resolution of the mask switch-offs -> in chunks of groups:
// group filter, origin lists, ordered gather -> normalisation, tile rebuild
// and inverse colour transform.  Frames, flows, the basic estimate and the
// aggregation buffers stay resident on the device between the two steps.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "../../include/bm4dof.h"
#include "internal.hpp"

using namespace bm4dof;

namespace {

struct DevBuf {
	void *p = nullptr;
	size_t cap = 0;
};

struct KeptGroups {                 // neighbour lists of one tile of one step
	std::vector<unsigned> ref, nsimp, index;
	unsigned stride = 0;
};

}  // namespace

struct bm4dof_ctx {
	int device = 0;
	int nsm = 0;
	cudaStream_t st = nullptr;
	std::map<std::string, DevBuf> bufs;
	std::vector<KeptGroups> kept[2];
	float ms[5] = {0, 0, 0, 0, 0};
	cudaEvent_t t_begin = nullptr, t_end = nullptr;
	unsigned launches = 0;
	std::vector<cudaEvent_t> events;
	size_t next_event = 0;
	// timing marks: (category, begin event, end event)
	std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t> > > marks;
};

namespace {

enum { T_SEARCH = 0, T_FILTER = 1, T_AGG = 2, T_OTHER = 3 };

#define CK(expr)                                                                              \
	do {                                                                                      \
		cudaError_t e_ = (expr);                                                              \
		if (e_ != cudaSuccess) {                                                              \
			set_error(std::string("CUDA error: ") + cudaGetErrorString(e_) + " at " #expr);   \
			return e_ == cudaErrorMemoryAllocation ? BM4DOF_ERR_NO_MEMORY : BM4DOF_ERR_CUDA;  \
		}                                                                                     \
	} while (0)

template <class T>
bm4dof_status dbuf(bm4dof_ctx *ctx, const char *name, size_t count, T **out)
{
	DevBuf &b = ctx->bufs[name];
	const size_t bytes = std::max<size_t>(count, 1) * sizeof(T);
	if (b.cap < bytes) {
		if (b.p) cudaFree(b.p);
		b.p = nullptr;
		b.cap = 0;
		cudaError_t e = cudaMalloc(&b.p, bytes);
		if (e != cudaSuccess) {
			cudaGetLastError();
			set_error(std::string("cudaMalloc of ") + name + " (" + std::to_string(bytes) +
			          " bytes) failed: " + cudaGetErrorString(e));
			return BM4DOF_ERR_NO_MEMORY;
		}
		b.cap = bytes;
	}
	*out = static_cast<T *>(b.p);
	return BM4DOF_OK;
}

#define DBUF(name, count, ptr)                                 \
	do {                                                       \
		bm4dof_status s_ = dbuf(ctx, name, (count), &(ptr));   \
		if (s_ != BM4DOF_OK) return s_;                        \
	} while (0)

cudaEvent_t next_event(bm4dof_ctx *ctx)
{
	if (ctx->next_event == ctx->events.size()) {
		cudaEvent_t e;
		cudaEventCreate(&e);
		ctx->events.push_back(e);
	}
	return ctx->events[ctx->next_event++];
}

struct Mark {
	bm4dof_ctx *ctx;
	int cat;
	cudaEvent_t a;
	Mark(bm4dof_ctx *c, int k) : ctx(c), cat(k) { a = next_event(c); cudaEventRecord(a, c->st); }
	~Mark()
	{
		cudaEvent_t b = next_event(ctx);
		cudaEventRecord(b, ctx->st);
		ctx->marks.push_back(std::make_pair(cat, std::make_pair(a, b)));
	}
};

void determine_factor(unsigned n, unsigned &a, unsigned &b)
{
	// utilities.cpp:137-158: n = a*b with a >= b as balanced as possible
	if (n == 1) { a = 1; b = 1; return; }
	b = 2;
	while (n % b > 0) b++;
	a = n / b;
	if (b > a) { a = b; b = n / a; }
}

struct Plan {
	int nW, nH, wTmp, hTmp;
	std::vector<Tile> tiles;
	std::vector<int> grid;     // per tile: [xs | inverse x] [ys | inverse y] [fs | inverse t]
	long long G = 0;
	size_t pix = 0;            // total tile pixels (one channel)
	size_t maxpos = 0;         // largest tile pixel count
};

// Tiles (subDivideTight, lib_videot.hpp:853-916) and their reference grids
// (processNlBayes, nldct.cpp:520-553).
void make_plan(Plan &pl, unsigned W, unsigned H, unsigned F, unsigned nparts, const bm4dof_params &p)
{
	unsigned a, b;
	determine_factor(nparts, a, b);
	pl.nW = (int)a;
	pl.nH = (int)b;
	pl.wTmp = (int)std::ceil(float(W) / float(pl.nW));
	pl.hTmp = (int)std::ceil(float(H) / float(pl.nH));
	const int N = (int)p.boundary;
	const int sPx = p.sizePatch, sPt = p.sizePatchTime, sWx = p.sizeSearchWindow;
	const int sWt = p.sizeSearchTimeRangeFwd + p.sizeSearchTimeRangeBwd + 1;
	pl.tiles.clear();
	pl.grid.clear();
	pl.G = 0;
	pl.pix = 0;
	pl.maxpos = 0;
	for (int pp = 0; pp < pl.nH; pp++)
		for (int q = 0; q < pl.nW; q++) {
			Tile T;
			std::memset(&T, 0, sizeof(T));
			T.ox = std::max(0, q * pl.wTmp - N);
			T.oy = std::max(0, pp * pl.hTmp - N);
			const int ex = std::min((int)W, (q + 1) * pl.wTmp + N);
			const int ey = std::min((int)H, (pp + 1) * pl.hTmp + N);
			T.w = ex - T.ox;
			T.h = ey - T.oy;
			T.bx0 = T.ox > 0;
			T.by0 = T.oy > 0;
			T.bx1 = ex < (int)W;
			T.by1 = ey < (int)H;
			const int ori_x = T.bx0 ? sPx - 1 + sWx / 2 : 0;
			const int ori_y = T.by0 ? sPx - 1 + sWx / 2 : 0;
			const int end_x = T.w - (T.bx1 ? sPx - 1 + sWx / 2 : sPx - 1);
			const int end_y = T.h - (T.by1 ? sPx - 1 + sWx / 2 : sPx - 1);
			const int end_f = (int)F - (sPt - 1);   // tiles span all frames
			(void)sWt;
			std::vector<int> xs, ys, fs;
			for (int x = ori_x, d = 0; x < end_x; x++, d++)
				if ((unsigned)d % p.offSet == 0 || (!T.bx1 && x == end_x - 1) || (!T.bx0 && x == ori_x))
					xs.push_back(x);
			for (int y = ori_y, d = 0; y < end_y; y++, d++)
				if ((unsigned)d % p.offSet == 0 || (!T.by1 && y == end_y - 1) || (!T.by0 && y == ori_y))
					ys.push_back(y);
			for (int f = 0, d = 0; f < end_f; f++, d++)
				if ((unsigned)d % p.offSetTime == 0 || f == end_f - 1) fs.push_back(f);
			T.nx = (int)xs.size();
			T.ny = (int)ys.size();
			T.nf = (int)fs.size();
			auto push = [&pl](const std::vector<int> &v, int extent) {
				const int off = (int)pl.grid.size();
				pl.grid.insert(pl.grid.end(), v.begin(), v.end());
				const int inv0 = (int)pl.grid.size();
				pl.grid.resize(pl.grid.size() + std::max(extent, 0), -1);
				for (size_t i = 0; i < v.size(); i++) pl.grid[inv0 + v[i]] = (int)i;
				return off;
			};
			T.gx = push(xs, T.w);
			T.gy = push(ys, T.h);
			T.gf = push(fs, (int)F);
			T.g0 = pl.G;
			T.pix0 = (long long)pl.pix;
			T.lin0 = pl.pix;
			pl.G += (long long)T.nx * T.ny * T.nf;
			const size_t np_ = (size_t)T.w * T.h * F;
			pl.pix += np_;
			pl.maxpos = std::max(pl.maxpos, np_);
			pl.tiles.push_back(T);
		}
}

Image image(float *p, unsigned W, unsigned H, unsigned C, unsigned F)
{
	Image im;
	im.p = p;
	im.W = (int)W;
	im.H = (int)H;
	im.P = (int)((W + 7) / 8 * 8);
	im.C = (int)C;
	im.F = (int)F;
	return im;
}

bm4dof_status check_params(const bm4dof_params &p)
{
	if (p.transform == BM4DOF_BIOR1_5 && p.sizePatch != 8) {
		set_error("VideoNLB::processNlBayes: bior1_5 transform is only implemented for patches of size 8 x 8 x pt.");
		return BM4DOF_ERR_BIOR_SIZE;
	}
	const unsigned spc = p.sizePatch * p.sizePatch * p.sizePatchTime;
	std::string why;
	if (p.sizePatchTime == 0 || p.sizePatch == 0) why = "patch sizes must be positive";
	else if (p.offSet == 0 || p.offSetTime == 0) why = "offSet and offSetTime must be positive";
	else if (p.nSimilarPatches == 0 || p.nSimilarPatches > (unsigned)kMaxNp) why = "nSimilarPatches must be in [1, 32]";
	else if (spc > (unsigned)kMaxSpc) why = "sizePatch^2 * sizePatchTime must be at most 64";
	else if (p.sizeSearchWindow == 0) why = "sizeSearchWindow must be positive";
	else if (p.sizeSearchTimeRangeFwd + p.sizeSearchTimeRangeBwd + 1 > (unsigned)kMaxFrames) why = "temporal search range too long";
	else if (p.doPasteBoost) why = "doPasteBoost is not supported";
	else if (p.orderInvariance) why = "orderInvariance is not supported";
	else if (p.sigma <= 0.f) why = "sigma must be positive";
	if (!why.empty()) {
		set_error("bm4dof: unsupported parameters: " + why);
		return BM4DOF_ERR_UNSUPPORTED;
	}
	return BM4DOF_OK;
}

struct RunMode {
	bool mixed = false;   // FP16 pre-screen search (+ BF16 transforms where built)
};

// One step of processNlBayes over all tiles.  out receives the rebuilt video
// (inverse colour transformed when inverse_color).
bm4dof_status run_step(bm4dof_ctx *ctx, int step, const bm4dof_params &p, const Image &noisy,
                       const Image &basic, const Image &ffl, const Image &bfl, bool use_flow,
                       unsigned nparts, const Image &out, bool inverse_color, bool keep,
                       float *ratio, const RunMode &mode)
{
	const unsigned W = noisy.W, H = noisy.H, C = noisy.C, F = noisy.F;
	cudaStream_t st = ctx->st;
	Plan pl;
	make_plan(pl, W, H, F, nparts, p);
	const int ntiles = (int)pl.tiles.size();

	StepParams sp;
	std::memset(&sp, 0, sizeof(sp));
	sp.px = p.sizePatch;
	sp.pt = p.sizePatchTime;
	sp.spc = sp.px * sp.px * sp.pt;
	sp.wx = p.sizeSearchWindow;
	sp.wtf = p.sizeSearchTimeRangeFwd;
	sp.wtb = p.sizeSearchTimeRangeBwd;
	sp.np = p.nSimilarPatches;
	sp.step1 = step == 1;
	sp.C = C;
	sp.F = F;
	sp.chn_search = step == 1 ? 1 : C;
	sp.sigma = p.sigma;
	sp.beta = p.beta;
	sp.tau2 = p.tau * p.tau * sp.px * sp.px * sp.pt;   // nldct.cpp:1158, float
	sp.use_flow = use_flow ? 1 : 0;

	std::vector<float> basis, binv;
	if (!make_basis(p.transform, sp.px, sp.pt, basis, binv)) {
		set_error("VideoNLB::processNlBayes: bior1_5 transform is only implemented for patches of size 8 x 8 x pt.");
		return BM4DOF_ERR_BIOR_SIZE;
	}
	std::vector<float> win = make_window(p.agg_window != 0, sp.px, sp.pt);

	Tile *d_tiles;
	int *d_grid;
	float *d_basis, *d_binv, *d_win;
	DBUF("tiles", pl.tiles.size(), d_tiles);
	DBUF("grid", pl.grid.size(), d_grid);
	DBUF("basis", basis.size(), d_basis);
	DBUF("binv", binv.size(), d_binv);
	DBUF("win", win.size(), d_win);
	CK(cudaMemcpyAsync(d_tiles, pl.tiles.data(), sizeof(Tile) * pl.tiles.size(), cudaMemcpyHostToDevice, st));
	CK(cudaMemcpyAsync(d_grid, pl.grid.data(), sizeof(int) * pl.grid.size(), cudaMemcpyHostToDevice, st));
	CK(cudaMemcpyAsync(d_basis, basis.data(), sizeof(float) * basis.size(), cudaMemcpyHostToDevice, st));
	CK(cudaMemcpyAsync(d_binv, binv.data(), sizeof(float) * binv.size(), cudaMemcpyHostToDevice, st));
	CK(cudaMemcpyAsync(d_win, win.data(), sizeof(float) * win.size(), cudaMemcpyHostToDevice, st));

	const long long G = pl.G;
	uint8_t *d_nsimp, *d_alive, *d_eq, *d_killed;
	uint32_t *d_idx;
	float *d_wgroup;
	unsigned *d_small;
	DBUF("nsimp", G, d_nsimp);
	DBUF("alive", G, d_alive);
	DBUF("eq", G, d_eq);
	DBUF("killed", G, d_killed);
	DBUF("idx", (size_t)G * sp.np, d_idx);
	DBUF("wgroup", G, d_wgroup);
	// [0] edge count, [1] changed flag, [2] search wait-timeout flag,
	// [64 ..] per-tile processed-group counts
	DBUF("small", 64 + ntiles, d_small);
	uint32_t *d_traj;
	DBUF("traj", (size_t)G * search_frames_max(sp), d_traj);
	CK(cudaMemsetAsync(d_small, 0, sizeof(unsigned) * (64 + ntiles), st));

	// ---- patch search of every group -------------------------------------
	{
		Mark m(ctx, T_SEARCH);
		CK(launch_traj(ffl, bfl, d_tiles, ntiles, d_grid, sp, G, d_traj, st));
		if (mode.mixed && mixed_supported(sp)) {
			// FP16 tensor-core pre-screen + exact re-rank of the best 2k
			std::vector<long long> blocks;
			mixed_blocks(pl.tiles, blocks);
			long long *d_blocks;
			DBUF("mixed_blocks", blocks.size(), d_blocks);
			CK(cudaMemcpyAsync(d_blocks, blocks.data(), sizeof(long long) * blocks.size(), cudaMemcpyHostToDevice, st));
			CK(launch_search_mixed(step == 1 ? noisy : basic, d_tiles, ntiles, d_grid, d_traj, sp, d_blocks,
			                       (long long)blocks.size(), d_nsimp, d_idx, ctx->nsm, st));
		} else {
			CK(launch_search(step == 1 ? noisy : basic, d_tiles, ntiles, d_grid, d_traj, sp, 0, G, d_nsimp, d_idx,
			                 reinterpret_cast<int *>(d_small + 2), ctx->nsm, st));
		}
		ctx->launches += 2;
	}

	// ---- mask switch-offs (rare): killer -> victim edges, then fixed point --
	{
		Mark m(ctx, T_OTHER);
		CK(cudaMemsetAsync(d_alive, 1, G, st));
		unsigned timeout = 0;
		CK(cudaMemcpyAsync(&timeout, d_small + 2, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
		CK(cudaStreamSynchronize(st));
		if (timeout) {
			set_error("bm4dof: a shared-memory window load did not complete (bounded wait expired)");
			return BM4DOF_ERR_TIMEOUT;
		}
		unsigned cap = 1u << 16;
		unsigned long long *d_edges;
		DBUF("edges", cap, d_edges);
		CK(launch_kill_edges(d_tiles, ntiles, d_grid, d_grid, sp, G, d_idx, d_edges, d_small, cap, st));
		ctx->launches++;
		unsigned nedges = 0;
		CK(cudaMemcpyAsync(&nedges, d_small, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
		CK(cudaStreamSynchronize(st));
		if (nedges > cap) {
			cap = nedges;
			DBUF("edges", cap, d_edges);
			CK(cudaMemsetAsync(d_small, 0, sizeof(unsigned), st));
			CK(launch_kill_edges(d_tiles, ntiles, d_grid, d_grid, sp, G, d_idx, d_edges, d_small, cap, st));
			ctx->launches++;
		}
		for (unsigned it = 0; nedges > 0 && it <= nedges; it++) {
			unsigned changed = 0;
			CK(cudaMemsetAsync(d_small + 1, 0, sizeof(unsigned), st));
			CK(launch_kill_iteration(d_edges, nedges, d_alive, d_killed, d_small + 1, st));
			ctx->launches += 3;
			CK(cudaMemcpyAsync(&changed, d_small + 1, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
			CK(cudaStreamSynchronize(st));
			if (!changed) break;
		}
		CK(launch_count_alive(d_tiles, ntiles, G, d_alive, d_small + 64, st));
		ctx->launches++;
	}

	// ---- filter + ordered aggregation, in chunks of groups --------------------
	float *d_acc, *d_wacc;
	DBUF("acc", pl.pix * C, d_acc);
	DBUF("wacc", pl.pix, d_wacc);
	CK(cudaMemsetAsync(d_acc, 0, sizeof(float) * pl.pix * C, st));
	CK(cudaMemsetAsync(d_wacc, 0, sizeof(float) * pl.pix, st));
	unsigned *d_cnt, *d_off, *d_soff, *d_scratch;
	DBUF("cnt", pl.maxpos, d_cnt);
	DBUF("off", pl.maxpos + 1, d_off);
	DBUF("soff", pl.maxpos + 1, d_soff);
	DBUF("scratch", pl.maxpos / 4096 + pl.maxpos / (4096ull * 4096ull) + 64, d_scratch);

	// chunk of groups whose slot terms (vals), weights, origin lists and
	// spatial lists fit the slot budget; slot numbers must fit 26 bits
	const size_t per_group = (size_t)sp.np * ((size_t)C * sp.spc + 2 + (size_t)sp.px * sp.px) * sizeof(float);
	size_t budget = (size_t)16384 << 20;
	if (const char *env = std::getenv("BM4DOF_SLOT_MB")) budget = (size_t)std::atoll(env) << 20;
	size_t freeb = 0, totalb = 0;
	if (cudaMemGetInfo(&freeb, &totalb) == cudaSuccess && budget > freeb / 2) budget = freeb / 2;
	long long chunk = std::max<long long>(1, (long long)(budget / per_group));
	chunk = std::min<long long>(chunk, ((1ll << 26) - 1) / sp.np);
	chunk = std::min<long long>(chunk, std::max<long long>(1, G));
	float *d_vals, *d_wslot;
	unsigned *d_list, *d_sl;
	DBUF("vals", (size_t)chunk * sp.np * C * sp.spc, d_vals);
	DBUF("wslot", (size_t)chunk * sp.np, d_wslot);
	DBUF("list", (size_t)chunk * sp.np, d_list);
	DBUF("slist", (size_t)chunk * sp.np * sp.px * sp.px, d_sl);

	for (int ti = 0; ti < ntiles; ti++) {
		const Tile &T = pl.tiles[ti];
		const long long gend = T.g0 + (long long)T.nx * T.ny * T.nf;
		const size_t npos = (size_t)T.w * T.h * F;
		for (long long ga = T.g0; ga < gend; ga += chunk) {
			const long long gb = std::min(gend, ga + chunk);
			{
				Mark m(ctx, T_FILTER);
				CK(launch_filter(noisy, basic, d_tiles, ntiles, sp, d_basis, d_binv, d_win, ga, gb, d_nsimp,
				                 d_idx, d_alive, d_vals, d_wslot, d_wgroup, d_eq, ctx->nsm, st));
				ctx->launches += 2;
			}
			{
				Mark m(ctx, T_AGG);
				const uint32_t *tidx = d_idx;   // tile-local positions
				CK(launch_lists(ga, gb, sp.np, d_nsimp, tidx, d_alive, npos, d_cnt, d_off, d_list,
				                d_scratch, st));
				ctx->launches += 5;
				// origin frames of the chunk's member patches: the temporal search
				// range of a reference frame t lies within t -/+ (wtb + wtf)
				const long long fa = (ga - T.g0) / ((long long)T.nx * T.ny);
				const long long fb = (gb - 1 - T.g0) / ((long long)T.nx * T.ny);
				const int ta = pl.grid[T.gf + (int)fa], tb = pl.grid[T.gf + (int)fb];
				const int reach = sp.wtb + sp.wtf;
				const int t_lo = std::max(0, ta - reach);
				const int t_hi = std::min((int)F - sp.pt, tb + reach);
				CK(launch_gather(T, sp, t_lo, t_hi, d_off, d_list, d_soff, d_sl, d_scratch, d_vals, d_wslot,
				                 d_win, d_acc + T.pix0 * C, d_wacc + T.pix0, st));
				ctx->launches += 4;
			}
		}
	}

	// ---- normalise, rebuild from tile interiors, undo the colour transform --
	{
		Mark m(ctx, T_OTHER);
		CK(launch_finalize(d_tiles, pl.nW, pl.wTmp, pl.hTmp, sp, noisy, d_acc, d_wacc, out,
		                   inverse_color ? 1 : 0, st));
		ctx->launches++;
	}

	std::vector<unsigned> counts(ntiles);
	CK(cudaMemcpyAsync(counts.data(), d_small + 64, sizeof(unsigned) * ntiles, cudaMemcpyDeviceToHost, st));
	CK(cudaStreamSynchronize(st));
	const float whf = (float)(W * H * F);
	for (int n = 0; n < ntiles; n++) *ratio += 100.f * (float)counts[n] / whf;   // nldct.cpp:403-404

	if (keep) {
		std::vector<uint8_t> hn(G), ha(G);
		std::vector<uint32_t> hi((size_t)G * sp.np);
		CK(cudaMemcpy(hn.data(), d_nsimp, G, cudaMemcpyDeviceToHost));
		CK(cudaMemcpy(ha.data(), d_alive, G, cudaMemcpyDeviceToHost));
		CK(cudaMemcpy(hi.data(), d_idx, sizeof(uint32_t) * hi.size(), cudaMemcpyDeviceToHost));
		std::vector<KeptGroups> &kg = ctx->kept[step - 1];
		kg.assign(ntiles, KeptGroups());
		for (int ti = 0; ti < ntiles; ti++) {
			const Tile &T = pl.tiles[ti];
			KeptGroups &k = kg[ti];
			k.stride = sp.np;
			const unsigned wh = (unsigned)T.w * T.h, whc = wh * C;
			const long long n = (long long)T.nx * T.ny * T.nf;
			for (long long l = 0; l < n; l++) {
				const long long g = T.g0 + l;
				if (!ha[g]) continue;
				const int x = pl.grid[T.gx + (int)(l % T.nx)];
				const int y = pl.grid[T.gy + (int)((l / T.nx) % T.ny)];
				const int t = pl.grid[T.gf + (int)(l / ((long long)T.nx * T.ny))];
				k.ref.push_back((unsigned)t * whc + (unsigned)y * T.w + (unsigned)x);
				k.nsimp.push_back(hn[g]);
				for (int q = 0; q < sp.np; q++) {
					const uint32_t lin = hi[(size_t)g * sp.np + q];
					k.index.push_back(q < hn[g] ? (lin / wh) * whc + lin % wh : 0u);
				}
			}
		}
	}
	return BM4DOF_OK;
}

bm4dof_status upload(bm4dof_ctx *ctx, const Image &dst, const float *src)
{
	CK(cudaMemcpy2DAsync(dst.p, sizeof(float) * dst.P, src, sizeof(float) * dst.W, sizeof(float) * dst.W,
	                     (size_t)dst.H * dst.C * dst.F, cudaMemcpyDefault, ctx->st));
	return BM4DOF_OK;
}

bm4dof_status download(bm4dof_ctx *ctx, float *dst, const Image &src)
{
	CK(cudaMemcpy2DAsync(dst, sizeof(float) * src.W, src.p, sizeof(float) * src.P, sizeof(float) * src.W,
	                     (size_t)src.H * src.C * src.F, cudaMemcpyDefault, ctx->st));
	return BM4DOF_OK;
}

}  // namespace

extern "C" {

bm4dof_status bm4dof_create(bm4dof_ctx **out, int device)
{
	clear_error();
	if (!out) { set_error("bm4dof_create: null output"); return BM4DOF_ERR_ARGUMENT; }
	*out = nullptr;
	int n = 0;
	if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
		cudaGetLastError();
		set_error("bm4dof_create: no CUDA device");
		return BM4DOF_ERR_NO_DEVICE;
	}
	if (device < 0 || device >= n) { set_error("bm4dof_create: bad device ordinal"); return BM4DOF_ERR_ARGUMENT; }
	CK(cudaSetDevice(device));
	bm4dof_ctx *ctx = new bm4dof_ctx();
	ctx->device = device;
	cudaDeviceGetAttribute(&ctx->nsm, cudaDevAttrMultiProcessorCount, device);
	if (cudaStreamCreateWithFlags(&ctx->st, cudaStreamNonBlocking) != cudaSuccess) {
		delete ctx;
		set_error("bm4dof_create: stream creation failed");
		return BM4DOF_ERR_CUDA;
	}
	*out = ctx;
	return BM4DOF_OK;
}

void bm4dof_destroy(bm4dof_ctx *ctx)
{
	if (!ctx) return;
	cudaSetDevice(ctx->device);
	cudaStreamSynchronize(ctx->st);
	for (auto &kv : ctx->bufs)
		if (kv.second.p) cudaFree(kv.second.p);
	for (cudaEvent_t e : ctx->events) cudaEventDestroy(e);
	if (ctx->t_begin) cudaEventDestroy(ctx->t_begin);
	if (ctx->t_end) cudaEventDestroy(ctx->t_end);
	cudaStreamDestroy(ctx->st);
	delete ctx;
}

bm4dof_status bm4dof_run(bm4dof_ctx *ctx, const float *noisy, const float *fflow, const float *bflow,
                         unsigned W, unsigned H, unsigned C, unsigned F, float *basic, float *final_,
                         const bm4dof_params *p1, const bm4dof_params *p2, unsigned nparts,
                         unsigned flags, float ratios[2])
{
	clear_error();
	if (!ctx || !noisy || !basic || !p1 || !p2 || W == 0 || H == 0 || F == 0) {
		set_error("bm4dof_run: null pointer or empty video");
		return BM4DOF_ERR_ARGUMENT;
	}
	// nldct.cpp:277-296
	if (!(C == 1 || C == 3 || C == 4)) {
		set_error("VideoNLB::runNlBayes: Wrong number of channels. Must be 1, 3 or 4.");
		return BM4DOF_ERR_CHANNELS;
	}
	const bool use_flow = fflow != nullptr;
	if (use_flow && bflow == nullptr) {
		set_error("VideoNLB::runNlBayes: Wrong size of bwd optical flow.");
		return BM4DOF_ERR_BWD_FLOW;
	}
	// nldct.cpp:329-334
	const int step = p1->sizePatch ? (p2->sizePatch ? 0 : 1) : (p2->sizePatch ? 2 : -1);
	if (step == -1) {
		set_error("VideoNLB::runNlBayes: Both patch sizes are zero.");
		return BM4DOF_ERR_NO_STEP;
	}
	if (step != 1 && !final_) { set_error("bm4dof_run: final output is NULL"); return BM4DOF_ERR_ARGUMENT; }
	if (flags & ~(BM4DOF_DEVICE_POINTERS | BM4DOF_KEEP_GROUPS | BM4DOF_MIXED_PRECISION)) {
		set_error("bm4dof_run: unsupported flags");
		return BM4DOF_ERR_UNSUPPORTED;
	}
	if (nparts == 0) nparts = 2;
	for (int s = 1; s <= 2; s++) {
		if (s == 1 && step == 2) continue;
		if (s == 2 && step == 1) continue;
		bm4dof_status e = check_params(s == 1 ? *p1 : *p2);
		if (e != BM4DOF_OK) return e;
	}
	CK(cudaSetDevice(ctx->device));
	ctx->marks.clear();
	ctx->next_event = 0;
	ctx->launches = 0;
	ctx->kept[0].clear();
	ctx->kept[1].clear();
	const bool keep = (flags & BM4DOF_KEEP_GROUPS) != 0;
	RunMode mode;
	mode.mixed = (flags & BM4DOF_MIXED_PRECISION) != 0;
	if (!ctx->t_begin) {
		CK(cudaEventCreate(&ctx->t_begin));
		CK(cudaEventCreate(&ctx->t_end));
	}
	CK(cudaEventRecord(ctx->t_begin, ctx->st));

	float *d_noisy, *d_noisy_yuv, *d_ff, *d_bf, *d_basic, *d_basic_yuv, *d_final;
	const size_t P = (W + 7) / 8 * 8;
	const size_t nv = P * H * C * F;
	DBUF("noisy", nv, d_noisy);
	DBUF("basic_rgb", nv, d_basic);
	DBUF("final", nv, d_final);
	Image in = image(d_noisy, W, H, C, F);
	Image bas = image(d_basic, W, H, C, F);
	Image fin = image(d_final, W, H, C, F);
	Image ff = image(nullptr, W, H, 2, F), bf = image(nullptr, W, H, 2, F);
	{
		Mark m(ctx, T_OTHER);
		bm4dof_status s = upload(ctx, in, noisy);
		if (s != BM4DOF_OK) return s;
		if (use_flow) {
			DBUF("fflow", P * H * 2 * F, d_ff);
			DBUF("bflow", P * H * 2 * F, d_bf);
			ff.p = d_ff;
			bf.p = d_bf;
			if ((s = upload(ctx, ff, fflow)) != BM4DOF_OK) return s;
			if ((s = upload(ctx, bf, bflow)) != BM4DOF_OK) return s;
		}
		if (step == 2 && (s = upload(ctx, bas, basic)) != BM4DOF_OK) return s;
	}
	const bool color = C > 1;
	Image in_yuv = in;
	if (color && ((step != 2 && p1->colorSpace == BM4DOF_YUV) || (step != 1 && p2->colorSpace == BM4DOF_YUV))) {
		DBUF("noisy_yuv", nv, d_noisy_yuv);
		in_yuv = image(d_noisy_yuv, W, H, C, F);
		Mark m(ctx, T_OTHER);
		CK(launch_color(in, in_yuv, 1, ctx->st));
		ctx->launches++;
	}

	float gr[2] = {0.f, 0.f};
	if (step != 2) {
		const bool yuv = color && p1->colorSpace == BM4DOF_YUV;
		bm4dof_status s = run_step(ctx, 1, *p1, yuv ? in_yuv : in, in, ff, bf, use_flow, nparts, bas,
		                           yuv, keep, &gr[0], mode);
		if (s != BM4DOF_OK) return s;
	}
	if (step != 1) {
		const bool yuv = color && p2->colorSpace == BM4DOF_YUV;
		Image bas_yuv = bas;
		if (yuv) {
			DBUF("basic_yuv", nv, d_basic_yuv);
			bas_yuv = image(d_basic_yuv, W, H, C, F);
			Mark m(ctx, T_OTHER);
			CK(launch_color(bas, bas_yuv, 1, ctx->st));
			ctx->launches++;
		}
		bm4dof_status s = run_step(ctx, 2, *p2, yuv ? in_yuv : in, bas_yuv, ff, bf, use_flow, nparts, fin,
		                           yuv, keep, &gr[1], mode);
		if (s != BM4DOF_OK) return s;
		if (yuv) {
			// the reference returns basic after a forward and inverse transform (nldct.cpp:423, 467)
			Mark m(ctx, T_OTHER);
			CK(launch_color(bas_yuv, bas, 0, ctx->st));
			ctx->launches++;
		}
	}
	{
		Mark m(ctx, T_OTHER);
		bm4dof_status s = download(ctx, basic, bas);
		if (s != BM4DOF_OK) return s;
		if (step != 1 && (s = download(ctx, final_, fin)) != BM4DOF_OK) return s;
	}
	CK(cudaEventRecord(ctx->t_end, ctx->st));
	CK(cudaStreamSynchronize(ctx->st));
	for (int k = 0; k < 5; k++) ctx->ms[k] = 0.f;
	cudaEventElapsedTime(&ctx->ms[4], ctx->t_begin, ctx->t_end);
	for (auto &mk : ctx->marks) {
		float ms = 0.f;
		cudaEventElapsedTime(&ms, mk.second.first, mk.second.second);
		ctx->ms[mk.first] += ms;
	}
	if (ratios) { ratios[0] = gr[0]; ratios[1] = gr[1]; }
	return BM4DOF_OK;
}

bm4dof_status bm4dof_get_groups(bm4dof_ctx *ctx, unsigned step, unsigned tile, unsigned *ref,
                                unsigned *nsimp, unsigned *index, unsigned stride, size_t cap,
                                size_t *count)
{
	clear_error();
	if (!ctx || step < 1 || step > 2 || !count) { set_error("bm4dof_get_groups: bad argument"); return BM4DOF_ERR_ARGUMENT; }
	const std::vector<KeptGroups> &kg = ctx->kept[step - 1];
	if (tile >= kg.size()) { set_error("bm4dof_get_groups: no groups kept for this step/tile"); return BM4DOF_ERR_ARGUMENT; }
	const KeptGroups &k = kg[tile];
	*count = k.ref.size();
	const size_t n = std::min(cap, k.ref.size());
	for (size_t g = 0; g < n; g++) {
		if (ref) ref[g] = k.ref[g];
		if (nsimp) nsimp[g] = k.nsimp[g];
		if (index)
			for (unsigned q = 0; q < stride; q++)
				index[g * stride + q] = q < k.stride ? k.index[g * k.stride + q] : 0u;
	}
	return BM4DOF_OK;
}

bm4dof_status bm4dof_last_timings(bm4dof_ctx *ctx, float ms[5], unsigned *launches)
{
	if (!ctx) return BM4DOF_ERR_ARGUMENT;
	if (ms) for (int k = 0; k < 5; k++) ms[k] = ctx->ms[k];
	if (launches) *launches = ctx->launches;
	return BM4DOF_OK;
}

}  // extern "C"
