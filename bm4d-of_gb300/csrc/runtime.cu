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
#include <cstddef>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
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

struct bm4dof_ctx_ext;

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
	// learned form: gain network (device buffers "gain_master", "gain_wt")
	bool has_gain = false;
	float kappa = 1.5f;
	unsigned long long l_groups = 0, l_fallbacks = 0;
	// mixed form: groups searched through the tensor-core pre-screen, and the
	// ones it left to the exact search, over both steps of the last run
	unsigned long long m_groups = 0, m_exact = 0, m_uncertified = 0;
	size_t slot_budget = 0;   // bytes of per-chunk aggregation terms
	bool fixed_budget = false;   // batched children: slot_budget set by the tuning
	bool no_marks = false;       // inside a graph capture: no timing events
	int search_ctas = 0;         // exact search CTAs per SM (0: default)
	int search_strip = 0;        // exact search candidates per thread along a column (0: default)
	int gather_depth = 0;        // quad gather members in flight per thread (0: 1)
	size_t held = 0;          // device bytes held in bufs
	size_t mem_limit = 0;     // cap on held (0: none), bm4dof_set_memory_limit
	std::recursive_mutex mu;  // calls on one context are serialised (CtxLock)
	float whf = 1.f;          // W*H*F of the current run
	bm4dof_ctx_ext *x = nullptr;
};

namespace {

// Held by every entry point that takes a context, so that calls made on one
// context from several host threads run one after the other.
struct CtxLock {
	std::unique_lock<std::recursive_mutex> l;
	explicit CtxLock(bm4dof_ctx *c)
	{
		if (c) l = std::unique_lock<std::recursive_mutex>(c->mu);
	}
};

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
		if (ctx->mem_limit && ctx->held - b.cap + bytes > ctx->mem_limit) {
			set_error(std::string("device memory limit of ") + std::to_string(ctx->mem_limit) + " bytes reached: " +
			          name + " needs " + std::to_string(bytes) + " bytes beside " +
			          std::to_string(ctx->held - b.cap) + " held");
			return BM4DOF_ERR_NO_MEMORY;
		}
		if (b.p) cudaFree(b.p);
		ctx->held -= b.cap;
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
		ctx->held += bytes;
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
	Mark(bm4dof_ctx *c, int k) : ctx(c), cat(k)
	{
		if (!c->no_marks) {
			a = next_event(c);
			cudaEventRecord(a, c->st);
		}
	}
	~Mark()
	{
		if (ctx->no_marks) return;
		cudaEvent_t b = next_event(ctx);
		cudaEventRecord(b, ctx->st);
		ctx->marks.push_back(std::make_pair(cat, std::make_pair(a, b)));
	}
};

}  // namespace

namespace bm4dof {

void determine_factor(unsigned n, unsigned &a, unsigned &b)
{
	// utilities.cpp:137-158: n = a*b with a >= b as balanced as possible
	if (n == 1) { a = 1; b = 1; return; }
	b = 2;
	while (n % b > 0) b++;
	a = n / b;
	if (b > a) { a = b; b = n / a; }
}

// Tiles (subDivideTight, lib_videot.hpp:853-916) and their reference grids
// (processNlBayes, nldct.cpp:520-553).  With borders (bm4dof_process) the plan
// is one tile over the whole video whose sides {x0, y0, t0, x1, y1, t1} are
// borders as given; the tiles of a run span all frames and have none in time.
void make_plan(Plan &pl, unsigned W, unsigned H, unsigned F, unsigned nparts, const bm4dof_params &p,
               const int *borders)
{
	unsigned a = 1, b = 1;
	if (!borders) determine_factor(nparts, a, b);
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
			bool bt0 = false, bt1 = false;
			if (borders) {
				T.w = (int)W;
				T.h = (int)H;
				T.bx0 = borders[0] != 0;
				T.by0 = borders[1] != 0;
				bt0 = borders[2] != 0;
				T.bx1 = borders[3] != 0;
				T.by1 = borders[4] != 0;
				bt1 = borders[5] != 0;
			} else {
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
			}
			const int ori_x = T.bx0 ? sPx - 1 + sWx / 2 : 0;
			const int ori_y = T.by0 ? sPx - 1 + sWx / 2 : 0;
			const int ori_f = bt0 ? sPt - 1 + sWt / 2 : 0;
			const int end_x = T.w - (T.bx1 ? sPx - 1 + sWx / 2 : sPx - 1);
			const int end_y = T.h - (T.by1 ? sPx - 1 + sWx / 2 : sPx - 1);
			const int end_f = (int)F - (bt1 ? sPt - 1 + sWt / 2 : sPt - 1);
			std::vector<int> xs, ys, fs;
			for (int x = ori_x, d = 0; x < end_x; x++, d++)
				if ((unsigned)d % p.offSet == 0 || (!T.bx1 && x == end_x - 1) || (!T.bx0 && x == ori_x))
					xs.push_back(x);
			for (int y = ori_y, d = 0; y < end_y; y++, d++)
				if ((unsigned)d % p.offSet == 0 || (!T.by1 && y == end_y - 1) || (!T.by0 && y == ori_y))
					ys.push_back(y);
			for (int f = ori_f, d = 0; f < end_f; f++, d++)
				if ((unsigned)d % p.offSetTime == 0 || (!bt1 && f == end_f - 1)) fs.push_back(f);
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

}  // namespace bm4dof

namespace {

// The crop's sides that stop short of its source (nldct.cpp:520-525), in
// make_plan's order {x0, y0, t0, x1, y1, t1}; no crop: no border.
void crop_borders(const bm4dof_crop *crop, int b[6])
{
	for (int k = 0; k < 6; k++) b[k] = 0;
	if (!crop) return;
	b[0] = crop->origin_x > 0;
	b[1] = crop->origin_y > 0;
	b[2] = crop->origin_t > 0;
	b[3] = crop->ending_x < (int)crop->source_sz.width;
	b[4] = crop->ending_y < (int)crop->source_sz.height;
	b[5] = crop->ending_t < (int)crop->source_sz.frames;
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
	else if (p.sizePatchTime > (unsigned)kMaxGatherPt) why = "sizePatchTime must be at most 16";
	else if (p.sizeSearchWindow == 0) why = "sizeSearchWindow must be positive";
	else if (p.sizeSearchTimeRangeFwd + p.sizeSearchTimeRangeBwd + 1 > (unsigned)kMaxFrames) why = "temporal search range too long";
	else if (p.sigma <= 0.f) why = "sigma must be positive";
	if (!why.empty()) {
		set_error("bm4dof: unsupported parameters: " + why);
		return BM4DOF_ERR_UNSUPPORTED;
	}
	return BM4DOF_OK;
}

struct SampleOut {
	float *feat, *target;
	uint8_t *valid;
	size_t cap, *count;
};

struct RunMode {
	bool mixed = false;     // FP16 pre-screen search (+ BF16 transforms where built)
	bool certified = false; // mixed: exact search for every group the re-rank cannot certify
	bool learned = false;   // learned form: groups searched on noisy, gain-network filter
	bool vbm3d = false;     // predictive search of the reference's VBM3D_SEARCH build
	float beta1 = 3.f;      // learned form: hard threshold of the non-mean rows
	const SampleOut *samples = nullptr;   // training pairs instead of filtering
	const int *borders = nullptr;         // bm4dof_process: one tile with these borders
};

// Host staging of one step's tables (pinned, so that the uploads are
// asynchronous and can be recorded into a CUDA graph).
struct HostBuf {
	void *p = nullptr;
	size_t cap = 0;
};

}  // namespace

// Everything one step needs.  prepare_step allocates (and stages) it all
// before the first launch of a run; launch_step then issues the step's work
// on the context's stream with no host round trip.
struct StepState {
	int step = 0;
	bm4dof_params p;
	RunMode mode;
	Plan pl;
	StepParams sp;
	long long G = 0, chunk = 0;
	bool tc_search = false;      // tcgen05 pre-screen + certified re-rank (search_tc.cu)
	size_t nblocks = 0;
	PasteScratch paste = {nullptr, nullptr, nullptr, nullptr, nullptr};   // doPasteBoost only
	Tile *d_tiles = nullptr;
	int *d_grid = nullptr;
	float *d_basis = nullptr, *d_binv = nullptr, *d_win = nullptr;
	uint8_t *d_nsimp = nullptr, *d_alive = nullptr, *d_eq = nullptr, *d_killed = nullptr;
	uint32_t *d_idx = nullptr, *d_traj = nullptr;
	uint32_t *d_cand = nullptr, *d_fb = nullptr;   // tc_search: candidates, exact-search list
	float *d_lb = nullptr, *d_thr0 = nullptr;       // tc_search: bound on the dropped candidates, anchors
	float *d_wgroup = nullptr;
	unsigned *d_small = nullptr;          // [0] edges, [3] fallbacks, [4] exact-search list, [5] tc status,
	                                      // [6] uncertified re-ranks, [64..] per-tile counts
	long long *d_blocks = nullptr;
	unsigned long long *d_edges = nullptr;
	float *d_acc = nullptr, *d_wacc = nullptr, *d_vals = nullptr;
	unsigned *d_cnt = nullptr, *d_off = nullptr, *d_soff = nullptr, *d_scratch = nullptr, *d_list = nullptr,
	         *d_sl = nullptr;
	__nv_bfloat16 *d_lfeat = nullptr;
	float *d_lgain = nullptr, *d_gm = nullptr;
	uint16_t *d_gw = nullptr;
	unsigned char *h_stage = nullptr;     // tiles | grid | basis | binv | win | blocks
	size_t o_grid = 0, o_basis = 0, o_binv = 0, o_win = 0, o_blocks = 0, n_stage = 0;
	unsigned *h_small = nullptr;          // pinned copy of d_small after the step
};

struct bm4dof_ctx_ext {
	std::map<std::string, HostBuf> hbufs;
	StepState steps[2];
	// batched runs: one child context per sequence, on `branches` streams
	// joined into one CUDA graph
	std::vector<bm4dof_ctx *> children;
	std::vector<cudaStream_t> branches;
	std::vector<cudaEvent_t> joins;
	cudaEvent_t fork = nullptr;
	cudaGraphExec_t exec = nullptr;
	std::string exec_key;
};

namespace {

bm4dof_ctx_ext &ext(bm4dof_ctx *ctx) { return *ctx->x; }

bm4dof_status hbuf(bm4dof_ctx *ctx, const std::string &name, size_t bytes, unsigned char **out)
{
	HostBuf &b = ext(ctx).hbufs[name];
	if (b.cap < bytes) {
		if (b.p) cudaFreeHost(b.p);
		b.p = nullptr;
		b.cap = 0;
		if (cudaMallocHost(&b.p, std::max<size_t>(bytes, 64)) != cudaSuccess) {
			cudaGetLastError();
			set_error("cudaMallocHost of " + name + " failed");
			return BM4DOF_ERR_NO_MEMORY;
		}
		b.cap = std::max<size_t>(bytes, 64);
	}
	*out = static_cast<unsigned char *>(b.p);
	return BM4DOF_OK;
}

// Bytes of aggregation terms per chunk: 16 GB, BM4DOF_SLOT_MB when set (a
// decimal number of MiB, fractions allowed), at most half of the device
// memory this context could use.
void set_budget(bm4dof_ctx *ctx)
{
	if (ctx->fixed_budget) return;
	size_t budget = (size_t)16384 << 20;
	if (const char *env = std::getenv("BM4DOF_SLOT_MB")) {
		const double mb = std::atof(env);
		if (mb > 0.0) budget = (size_t)(mb * 1048576.0);
	}
	size_t freeb = 0, totalb = 0;
	if (cudaMemGetInfo(&freeb, &totalb) == cudaSuccess && budget > (freeb + ctx->held) / 2)
		budget = (freeb + ctx->held) / 2;
	if (ctx->mem_limit && budget > ctx->mem_limit / 4) budget = ctx->mem_limit / 4;
	ctx->slot_budget = budget;
}

std::string nm(int slot, const char *base) { return std::string(slot ? "s2_" : "s1_") + base; }

#define SBUF(name, count, ptr)                                                  \
	do {                                                                        \
		bm4dof_status s_ = dbuf(ctx, nm(slot, name).c_str(), (count), &(ptr));  \
		if (s_ != BM4DOF_OK) return s_;                                         \
	} while (0)

// Plan, parameters and every buffer of one step (slot 0: step 1, slot 1:
// step 2 or the learned pass).  Buffers private to a step carry its slot in
// their name; the aggregation work buffers are shared (the steps run one
// after the other on one stream).  Called twice per run for all steps: the
// second call only re-reads the final addresses.
bm4dof_status prepare_step(bm4dof_ctx *ctx, int slot, int step, const bm4dof_params &p, unsigned W, unsigned H,
                           unsigned C, unsigned F, bool use_flow, unsigned nparts, const RunMode &mode)
{
	StepState &S = ext(ctx).steps[slot];
	S.step = step;
	S.p = p;
	S.mode = mode;
	make_plan(S.pl, W, H, F, nparts, p, mode.borders);
	const Plan &pl = S.pl;
	StepParams &sp = S.sp;
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
	const bool on_noisy = step == 1 || mode.learned || mode.samples;   // search source
	sp.chn_search = on_noisy ? 1 : C;
	sp.sigma = p.sigma;
	sp.beta = p.beta;
	sp.tau2 = p.tau * p.tau * sp.px * sp.px * sp.pt;   // nldct.cpp:1158, float
	sp.use_flow = use_flow ? 1 : 0;
	sp.beta1 = mode.beta1;
	sp.search_ctas = ctx->search_ctas;
	sp.search_strip = ctx->search_strip;
	sp.gather_depth = ctx->gather_depth;
	sp.beta_mean = p.betaMean;
	sp.order_inv = p.orderInvariance ? 1 : 0;
	sp.vbm3d = mode.vbm3d ? 1 : 0;
	sp.wxp = (int)p.sizeSearchWindowPred;
	sp.npf = (int)p.nSimilarPatchesPred;
	sp.dsub_bias = p.dsub * p.dsub * 255.f;   // nldct.cpp:921, float
	sp.paste = p.doPasteBoost ? 1 : 0;
	if (sp.vbm3d) {
		std::string why;
		if (!vbm3d_check(sp, pl.tiles, why)) {
			set_error("bm4dof: predictive search: " + why);
			return BM4DOF_ERR_UNSUPPORTED;
		}
		if (vbm3d_smem_bytes(sp, on_noisy ? 1 : (int)C) > (size_t)200 * 1024) {
			set_error("bm4dof: predictive search: search windows too large");
			return BM4DOF_ERR_UNSUPPORTED;
		}
	}
	if ((mode.learned || mode.samples) && !learned_supported(sp)) {
		set_error("bm4dof: the learned form needs grey video and 64-element patches");
		return BM4DOF_ERR_UNSUPPORTED;
	}
	std::vector<float> basis, binv;
	if (!make_basis(p.transform, sp.px, sp.pt, basis, binv)) {
		set_error("VideoNLB::processNlBayes: bior1_5 transform is only implemented for patches of size 8 x 8 x pt.");
		return BM4DOF_ERR_BIOR_SIZE;
	}
	std::vector<float> win = make_window(p.agg_window != 0, sp.px, sp.pt);
	S.tc_search = mode.mixed && tc_supported(sp, pl.tiles);
	std::vector<long long> blocks;
	if (S.tc_search) tc_blocks(pl.tiles, blocks);
	S.nblocks = blocks.size();

	// host staging
	auto al = [](size_t x) { return (x + 15) / 16 * 16; };
	S.o_grid = al(sizeof(Tile) * pl.tiles.size());
	S.o_basis = S.o_grid + al(sizeof(int) * pl.grid.size());
	S.o_binv = S.o_basis + al(sizeof(float) * basis.size());
	S.o_win = S.o_binv + al(sizeof(float) * binv.size());
	S.o_blocks = S.o_win + al(sizeof(float) * win.size());
	S.n_stage = S.o_blocks + al(sizeof(long long) * blocks.size());
	bm4dof_status hs = hbuf(ctx, nm(slot, "stage"), S.n_stage, &S.h_stage);
	if (hs != BM4DOF_OK) return hs;
	unsigned char *hsm;
	const int ntiles = (int)pl.tiles.size();
	if ((hs = hbuf(ctx, nm(slot, "small"), sizeof(unsigned) * (64 + ntiles), &hsm)) != BM4DOF_OK) return hs;
	S.h_small = reinterpret_cast<unsigned *>(hsm);
	std::memcpy(S.h_stage, pl.tiles.data(), sizeof(Tile) * pl.tiles.size());
	std::memcpy(S.h_stage + S.o_grid, pl.grid.data(), sizeof(int) * pl.grid.size());
	std::memcpy(S.h_stage + S.o_basis, basis.data(), sizeof(float) * basis.size());
	std::memcpy(S.h_stage + S.o_binv, binv.data(), sizeof(float) * binv.size());
	std::memcpy(S.h_stage + S.o_win, win.data(), sizeof(float) * win.size());
	if (!blocks.empty()) std::memcpy(S.h_stage + S.o_blocks, blocks.data(), sizeof(long long) * blocks.size());

	// step-private device buffers
	const long long G = pl.G;
	S.G = G;
	SBUF("tiles", pl.tiles.size(), S.d_tiles);
	SBUF("grid", pl.grid.size(), S.d_grid);
	SBUF("basis", basis.size(), S.d_basis);
	SBUF("binv", binv.size(), S.d_binv);
	SBUF("win", win.size(), S.d_win);
	SBUF("nsimp", G, S.d_nsimp);
	SBUF("alive", G, S.d_alive);
	SBUF("eq", G, S.d_eq);
	SBUF("killed", G, S.d_killed);
	SBUF("idx", (size_t)G * sp.np, S.d_idx);
	SBUF("wgroup", G, S.d_wgroup);
	SBUF("small", 64 + ntiles, S.d_small);
	SBUF("traj", (size_t)G * search_frames_max(sp), S.d_traj);
	SBUF("edges", G, S.d_edges);   // a group switches off at most one other
	if (S.tc_search) SBUF("tc_blocks", blocks.size(), S.d_blocks);
	if (S.tc_search) {
		SBUF("tc_cand", (size_t)G * 32, S.d_cand);
		SBUF("tc_lb", G, S.d_lb);
		SBUF("tc_thr0", G, S.d_thr0);
		SBUF("tc_exact", G, S.d_fb);
	}
	if (sp.paste) {
		SBUF("paste_pending", G, S.paste.pending);
		SBUF("paste_state", G, S.paste.state);
		SBUF("paste_q0", G, S.paste.q0);
		SBUF("paste_q1", G, S.paste.q1);
		SBUF("paste_counts", kPasteRounds + 3, S.paste.counts);
	}

	// shared aggregation buffers; chunks of groups whose slot terms (vals),
	// weights, origin lists and spatial lists fit the slot budget; slot
	// numbers must fit 26 bits
	DBUF("acc", pl.pix * C, S.d_acc);
	DBUF("wacc", pl.pix, S.d_wacc);
	DBUF("cnt", pl.maxpos + 1, S.d_cnt);   // also the quad path's row-list offsets: ceil(w/4)*h*F + 1 entries
	DBUF("off", pl.maxpos + 1, S.d_off);
	DBUF("soff", pl.maxpos + 1, S.d_soff);
	DBUF("scratch", pl.maxpos / 4096 + pl.maxpos / (4096ull * 4096ull) + 64, S.d_scratch);
	const size_t per_group = (size_t)sp.np * ((size_t)term_stride(C) * sp.spc + 1 + (size_t)list_entries_per_member(sp)) *
	                             sizeof(float) +
	                         (mode.learned ? (size_t)kMlpInPad * 2 + (size_t)kMlpOutN * 4 : 0);
	size_t budget = ctx->slot_budget;
	long long chunk = std::max<long long>(1, (long long)(budget / per_group));
	chunk = std::min<long long>(chunk, ((1ll << 26) - 1) / sp.np);
	chunk = std::min<long long>(chunk, std::max<long long>(1, G));
	S.chunk = chunk;
	if (!mode.samples) {
		DBUF("vals", (size_t)chunk * sp.np * term_stride(C) * sp.spc, S.d_vals);
		DBUF("list", (size_t)chunk * sp.np, S.d_list);
		DBUF("slist", (size_t)chunk * sp.np * list_entries_per_member(sp), S.d_sl);
	}
	if (mode.learned) {
		DBUF("lfeat", (size_t)chunk * kMlpInPad, S.d_lfeat);
		DBUF("lgain", (size_t)chunk * kMlpOutN, S.d_lgain);
		DBUF("gain_master", kMlpMasterSize, S.d_gm);
		DBUF("gain_wt", kMlpWtSize, S.d_gw);
	}
	return BM4DOF_OK;
}

// One step of processNlBayes over all tiles, all on the context's stream.
// out receives the rebuilt video (inverse colour transformed when
// inverse_color).  The per-tile counts of processed groups (and, for the
// learned form, the fallback count) are copied back asynchronously into
// S.h_small.
bm4dof_status launch_step(bm4dof_ctx *ctx, int slot, const Image &noisy, const Image &basic, const Image &ffl,
                          const Image &bfl, const Image &out, bool inverse_color)
{
	StepState &S = ext(ctx).steps[slot];
	const Plan &pl = S.pl;
	const StepParams &sp = S.sp;
	const RunMode &mode = S.mode;
	const unsigned C = noisy.C, F = noisy.F;
	cudaStream_t st = ctx->st;
	const int ntiles = (int)pl.tiles.size();
	const long long G = S.G;
	const bool on_noisy = S.step == 1 || mode.learned || mode.samples;

	{
		Mark m(ctx, T_OTHER);
		CK(cudaMemcpyAsync(S.d_tiles, S.h_stage, sizeof(Tile) * pl.tiles.size(), cudaMemcpyHostToDevice, st));
		CK(cudaMemcpyAsync(S.d_grid, S.h_stage + S.o_grid, sizeof(int) * pl.grid.size(), cudaMemcpyHostToDevice, st));
		const size_t nbasis = sizeof(float) * sp.spc * sp.spc;   // exact sizes: the staging is padded
		CK(cudaMemcpyAsync(S.d_basis, S.h_stage + S.o_basis, nbasis, cudaMemcpyHostToDevice, st));
		CK(cudaMemcpyAsync(S.d_binv, S.h_stage + S.o_binv, nbasis, cudaMemcpyHostToDevice, st));
		CK(cudaMemcpyAsync(S.d_win, S.h_stage + S.o_win, sizeof(float) * sp.spc, cudaMemcpyHostToDevice, st));
		if (S.tc_search)
			CK(cudaMemcpyAsync(S.d_blocks, S.h_stage + S.o_blocks, sizeof(long long) * S.nblocks,
			                   cudaMemcpyHostToDevice, st));
		CK(cudaMemsetAsync(S.d_small, 0, sizeof(unsigned) * (64 + ntiles), st));
	}

	// ---- patch search of every group -------------------------------------
	{
		Mark m(ctx, T_SEARCH);
		if (sp.vbm3d) {
			// trajectories are chained inside the search (they follow the matches)
			CK(launch_search_vbm3d(on_noisy ? noisy : basic, ffl, bfl, S.d_tiles, ntiles, S.d_grid, sp,
			                       on_noisy ? 1 : (int)C, 0, G, S.d_nsimp, S.d_idx, ctx->nsm, st));
			ctx->launches += 1;
		} else if (S.tc_search) {
			// tensor-core pre-screen and certified re-rank; the groups it cannot
			// certify get the exact search
			const Image &src = on_noisy ? noisy : basic;
			CK(launch_traj(ffl, bfl, S.d_tiles, ntiles, S.d_grid, sp, G, S.d_traj, st));
			CK(cudaMemsetAsync(S.d_lb, 0xff, sizeof(float) * G, st));   // NaN: not certified
			CK(launch_search_tc(src, S.d_tiles, ntiles, S.d_grid, S.d_traj, sp, S.d_blocks, (long long)S.nblocks, G,
			                    S.d_cand, S.d_lb, S.d_thr0, reinterpret_cast<int *>(S.d_small + 5), S.d_nsimp, S.d_idx,
			                    S.d_fb,
			                    S.d_small + 4, S.d_small + 6, mode.certified ? 1 : 0, ctx->nsm, st));
			CK(launch_search(src, S.d_tiles, ntiles, S.d_grid, S.d_traj, sp, 0, G, S.d_nsimp, S.d_idx, nullptr,
			                 ctx->nsm, st, S.d_fb, S.d_small + 4));
			ctx->launches += 5;
		} else {
			CK(launch_traj(ffl, bfl, S.d_tiles, ntiles, S.d_grid, sp, G, S.d_traj, st));
			CK(launch_search(on_noisy ? noisy : basic, S.d_tiles, ntiles, S.d_grid, S.d_traj, sp, 0, G, S.d_nsimp,
			                 S.d_idx, nullptr, ctx->nsm, st));
			ctx->launches += 2;
		}
	}

	// ---- mask switch-offs (rare): killer -> victim edges, then fixed point --
	// (doPasteBoost: every processed group switches off its members' positions
	// and their neighbours, settled tile by tile in processing order)
	if (sp.paste) {
		Mark m(ctx, T_OTHER);
		CK(launch_paste_resolve(S.d_tiles, ntiles, S.d_grid, sp, G, S.d_nsimp, S.d_idx, S.paste, S.d_alive,
		                        ctx->nsm, st));
		CK(launch_count_alive(S.d_tiles, ntiles, G, S.d_alive, S.d_small + 64, st));
		ctx->launches += kPasteRounds + 5;
	} else {
		Mark m(ctx, T_OTHER);
		CK(cudaMemsetAsync(S.d_alive, 1, G, st));
		CK(launch_kill_edges(S.d_tiles, ntiles, S.d_grid, S.d_grid, sp, G, S.d_idx, S.d_edges, S.d_small,
		                     (unsigned)std::min<long long>(G, 0xffffffffll), st));
		CK(launch_kill_fixpoint(S.d_edges, S.d_small, (unsigned)std::min<long long>(G, 0xffffffffll), S.d_alive,
		                        S.d_killed, st));
		CK(launch_count_alive(S.d_tiles, ntiles, G, S.d_alive, S.d_small + 64, st));
		ctx->launches += 3;
	}

	LearnedArgs la;
	std::memset(&la, 0, sizeof(la));
	la.noisy = noisy;
	la.basic = basic;
	la.tiles = S.d_tiles;
	la.ntiles = ntiles;
	la.nsimp = S.d_nsimp;
	la.alive = S.d_alive;
	la.idx = S.d_idx;
	la.basis = S.d_basis;
	la.binv = S.d_binv;
	la.win = S.d_win;
	la.kappa = ctx->kappa;
	la.nfallback = S.d_small + 3;
	if (mode.samples) {
		const SampleOut &so = *mode.samples;
		Mark m(ctx, T_FILTER);
		CK(cudaMemsetAsync(so.valid, 0, (size_t)G, st));
		la.ga = 0;
		la.gb = G;
		la.sfeat = so.feat;
		la.starget = so.target;
		la.svalid = so.valid;
		CK(launch_learned(kLearnedSamples, la, sp, ctx->nsm, st));
		ctx->launches++;
		return BM4DOF_OK;
	}

	// ---- filter + ordered aggregation, in chunks of groups --------------------
	CK(cudaMemsetAsync(S.d_acc, 0, sizeof(float) * pl.pix * C, st));
	CK(cudaMemsetAsync(S.d_wacc, 0, sizeof(float) * pl.pix, st));
	const long long chunk = S.chunk;
	for (int ti = 0; ti < ntiles; ti++) {
		const Tile &T = pl.tiles[ti];
		const long long gend = T.g0 + (long long)T.nx * T.ny * T.nf;
		const size_t npos = (size_t)T.w * T.h * F;
		for (long long ga = T.g0; ga < gend; ga += chunk) {
			const long long gb = std::min(gend, ga + chunk);
			{
				Mark m(ctx, T_FILTER);
				if (mode.learned) {
					la.ga = ga;
					la.gb = gb;
					la.feat = S.d_lfeat;
					la.vals = S.d_vals;
					la.gains = nullptr;
					if (ctx->has_gain) {
						CK(launch_learned(kLearnedFeatures, la, sp, ctx->nsm, st));
						CK(launch_mlp_forward(reinterpret_cast<const uint16_t *>(S.d_lfeat), gb - ga,
						                      mlp_weights(S.d_gw, S.d_gm), S.d_lgain, ctx->nsm, st));
						ctx->launches += 2;
						la.gains = S.d_lgain;
					}
					CK(launch_learned(kLearnedApply, la, sp, ctx->nsm, st));
					ctx->launches++;
				} else {
					CK(launch_filter(noisy, basic, S.d_tiles, ntiles, sp, S.d_basis, S.d_binv, S.d_win, ga, gb,
					                 S.d_nsimp, S.d_idx, S.d_alive, S.d_vals, S.d_wgroup, S.d_eq,
					                 ctx->nsm, st));
					ctx->launches += 2;
				}
			}
			{
				Mark m(ctx, T_AGG);
				CK(launch_lists(ga, gb, sp.np, S.d_nsimp, S.d_idx, S.d_alive, npos, S.d_cnt, S.d_off, S.d_list,
				                S.d_scratch, &ctx->launches, st));
				// origin frames of the chunk's member patches: the temporal search
				// range of a reference frame t lies within t -/+ (wtb + wtf)
				const long long fa = (ga - T.g0) / ((long long)T.nx * T.ny);
				const long long fb = (gb - 1 - T.g0) / ((long long)T.nx * T.ny);
				const int ta = pl.grid[T.gf + (int)fa], tb = pl.grid[T.gf + (int)fb];
				const int reach = sp.wtb + sp.wtf;
				const int t_lo = std::max(0, ta - reach);
				const int t_hi = std::min((int)F - sp.pt, tb + reach);
				CK(launch_gather(T, sp, t_lo, t_hi, S.d_off, S.d_list, S.d_cnt, S.d_soff, S.d_sl,
				                 (size_t)chunk * sp.np, S.d_scratch, S.d_vals, S.d_acc + T.pix0 * C,
				                 S.d_wacc + T.pix0, &ctx->launches, st));
			}
		}
	}

	// ---- normalise, rebuild from tile interiors, undo the colour transform --
	{
		Mark m(ctx, T_OTHER);
		CK(launch_finalize(S.d_tiles, pl.nW, pl.wTmp, pl.hTmp, sp, noisy, S.d_acc, S.d_wacc, out,
		                   inverse_color ? 1 : 0, st));
		ctx->launches++;
		CK(cudaMemcpyAsync(S.h_small, S.d_small, sizeof(unsigned) * (64 + ntiles), cudaMemcpyDeviceToHost, st));
	}
	return BM4DOF_OK;
}

// After the stream has drained: processed-group ratio of a step
// (nldct.cpp:403-404) and the learned-form statistics.
float step_ratio(bm4dof_ctx *ctx, int slot)
{
	const StepState &S = ext(ctx).steps[slot];
	const int ntiles = (int)S.pl.tiles.size();
	float r = 0.f;
	unsigned long long groups = 0;
	for (int n = 0; n < ntiles; n++) groups += S.h_small[64 + n];
	for (int n = 0; n < ntiles; n++) r += 100.f * (float)S.h_small[64 + n] / ctx->whf;
	if (S.mode.learned) {
		ctx->l_groups = groups;
		ctx->l_fallbacks = S.h_small[3];
	}
	if (S.tc_search) {
		ctx->m_groups += (unsigned long long)S.G;
		ctx->m_exact += S.h_small[4];
		ctx->m_uncertified += S.h_small[6];
	}
	return r;
}

// Neighbour lists of a finished step, for bm4dof_get_groups.
bm4dof_status keep_groups(bm4dof_ctx *ctx, int slot, int step)
{
	const StepState &S = ext(ctx).steps[slot];
	const Plan &pl = S.pl;
	const long long G = S.G;
	const int np = S.sp.np, C = S.sp.C, ntiles = (int)pl.tiles.size();
	std::vector<uint8_t> hn(G), ha(G);
	std::vector<uint32_t> hi((size_t)G * np);
	CK(cudaMemcpy(hn.data(), S.d_nsimp, G, cudaMemcpyDeviceToHost));
	CK(cudaMemcpy(ha.data(), S.d_alive, G, cudaMemcpyDeviceToHost));
	CK(cudaMemcpy(hi.data(), S.d_idx, sizeof(uint32_t) * hi.size(), cudaMemcpyDeviceToHost));
	std::vector<KeptGroups> &kg = ctx->kept[step - 1];
	kg.assign(ntiles, KeptGroups());
	for (int ti = 0; ti < ntiles; ti++) {
		const Tile &T = pl.tiles[ti];
		KeptGroups &k = kg[ti];
		k.stride = np;
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
			for (int q = 0; q < np; q++) {
				const uint32_t lin = hi[(size_t)g * np + q];
				k.index.push_back(q < hn[g] ? (lin / wh) * whc + lin % wh : 0u);
			}
		}
	}
	return BM4DOF_OK;
}

bm4dof_ctx *make_child(bm4dof_ctx *parent)
{
	bm4dof_ctx *c = new bm4dof_ctx();
	c->x = new bm4dof_ctx_ext();
	c->device = parent->device;
	c->nsm = parent->nsm;
	c->st = nullptr;        // a branch stream of the parent
	c->no_marks = true;
	c->fixed_budget = true;
	return c;
}

void free_child(bm4dof_ctx *c)
{
	for (auto &kv : c->bufs)
		if (kv.second.p) cudaFree(kv.second.p);
	for (auto &kv : c->x->hbufs)
		if (kv.second.p) cudaFreeHost(kv.second.p);
	for (cudaEvent_t e : c->events) cudaEventDestroy(e);
	delete c->x;
	delete c;
}

// Rows of W floats to or from the padded device pitch P; with no padding the
// video is one contiguous copy (one large DMA instead of H*C*F row copies).
bm4dof_status upload(bm4dof_ctx *ctx, const Image &dst, const float *src)
{
	const size_t rows = (size_t)dst.H * dst.C * dst.F;
	if (dst.P == dst.W)
		CK(cudaMemcpyAsync(dst.p, src, sizeof(float) * dst.W * rows, cudaMemcpyDefault, ctx->st));
	else
		CK(cudaMemcpy2DAsync(dst.p, sizeof(float) * dst.P, src, sizeof(float) * dst.W, sizeof(float) * dst.W, rows,
		                     cudaMemcpyDefault, ctx->st));
	return BM4DOF_OK;
}

bm4dof_status download(bm4dof_ctx *ctx, float *dst, const Image &src)
{
	const size_t rows = (size_t)src.H * src.C * src.F;
	if (src.P == src.W)
		CK(cudaMemcpyAsync(dst, src.p, sizeof(float) * src.W * rows, cudaMemcpyDefault, ctx->st));
	else
		CK(cudaMemcpy2DAsync(dst, sizeof(float) * src.W, src.p, sizeof(float) * src.P, sizeof(float) * src.W, rows,
		                     cudaMemcpyDefault, ctx->st));
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
	ctx->x = new bm4dof_ctx_ext();
	ctx->device = device;
	cudaDeviceGetAttribute(&ctx->nsm, cudaDevAttrMultiProcessorCount, device);
	if (cudaStreamCreateWithFlags(&ctx->st, cudaStreamNonBlocking) != cudaSuccess) {
		delete ctx->x;
		delete ctx;
		set_error("bm4dof_create: stream creation failed");
		return BM4DOF_ERR_CUDA;
	}
	*out = ctx;
	return BM4DOF_OK;
}

bm4dof_status bm4dof_get_stream(bm4dof_ctx *ctx, void **stream)
{
	clear_error();
	if (!ctx || !stream) { set_error("bm4dof_get_stream: null argument"); return BM4DOF_ERR_ARGUMENT; }
	*stream = static_cast<void *>(ctx->st);
	return BM4DOF_OK;
}

void bm4dof_destroy(bm4dof_ctx *ctx)
{
	if (!ctx) return;
	cudaSetDevice(ctx->device);
	cudaStreamSynchronize(ctx->st);
	for (auto &kv : ctx->bufs)
		if (kv.second.p) cudaFree(kv.second.p);
	for (auto &kv : ctx->x->hbufs)
		if (kv.second.p) cudaFreeHost(kv.second.p);
	if (ctx->x->exec) cudaGraphExecDestroy(ctx->x->exec);
	for (bm4dof_ctx *c : ctx->x->children) free_child(c);
	for (cudaStream_t b : ctx->x->branches) cudaStreamDestroy(b);
	for (cudaEvent_t e : ctx->x->joins) cudaEventDestroy(e);
	if (ctx->x->fork) cudaEventDestroy(ctx->x->fork);
	delete ctx->x;
	for (cudaEvent_t e : ctx->events) cudaEventDestroy(e);
	if (ctx->t_begin) cudaEventDestroy(ctx->t_begin);
	if (ctx->t_end) cudaEventDestroy(ctx->t_end);
	cudaStreamDestroy(ctx->st);
	delete ctx;
}

}  // extern "C"

namespace {

// One runNlBayes call: its arguments, what validation derived from them, and
// the device images once prepared.
struct RunArgs {
	const float *noisy, *fflow, *bflow;
	unsigned W, H, C, F;
	float *basic, *final_;
	bm4dof_params p1, p2;
	unsigned nparts, flags;
	int step = 0;
	bool learned = false, use_flow = false, run1 = false, run2 = false, yuv1 = false, yuv2 = false, keep = false;
	RunMode mode;
	float *d_noisy = nullptr, *d_noisy_yuv = nullptr, *d_ff = nullptr, *d_bf = nullptr, *d_basic = nullptr,
	      *d_basic_yuv = nullptr, *d_final = nullptr;
};

bm4dof_status validate_run(RunArgs &r, const char *who)
{
	if (!r.noisy || !r.basic || r.W == 0 || r.H == 0 || r.F == 0) {
		set_error(std::string(who) + ": null pointer or empty video");
		return BM4DOF_ERR_ARGUMENT;
	}
	// nldct.cpp:277-296
	if (!(r.C == 1 || r.C == 3 || r.C == 4)) {
		set_error("VideoNLB::runNlBayes: Wrong number of channels. Must be 1, 3 or 4.");
		return BM4DOF_ERR_CHANNELS;
	}
	r.use_flow = r.fflow != nullptr;
	if (r.use_flow && r.bflow == nullptr) {
		set_error("VideoNLB::runNlBayes: Wrong size of bwd optical flow.");
		return BM4DOF_ERR_BWD_FLOW;
	}
	// nldct.cpp:329-334
	r.step = r.p1.sizePatch ? (r.p2.sizePatch ? 0 : 1) : (r.p2.sizePatch ? 2 : -1);
	if (r.step == -1) {
		set_error("VideoNLB::runNlBayes: Both patch sizes are zero.");
		return BM4DOF_ERR_NO_STEP;
	}
	if (r.step != 1 && !r.final_) { set_error(std::string(who) + ": final output is NULL"); return BM4DOF_ERR_ARGUMENT; }
	if (r.flags & ~(BM4DOF_DEVICE_POINTERS | BM4DOF_KEEP_GROUPS | BM4DOF_MIXED_PRECISION | BM4DOF_LEARNED |
	                BM4DOF_VBM3D_SEARCH | BM4DOF_MIXED_CERTIFIED)) {
		set_error(std::string(who) + ": unsupported flags");
		return BM4DOF_ERR_UNSUPPORTED;
	}
	if ((r.flags & BM4DOF_VBM3D_SEARCH) && (r.flags & (BM4DOF_MIXED_PRECISION | BM4DOF_MIXED_CERTIFIED | BM4DOF_LEARNED))) {
		set_error(std::string(who) + ": the predictive search runs on the plain FP32 path only");
		return BM4DOF_ERR_UNSUPPORTED;
	}
	r.learned = (r.flags & BM4DOF_LEARNED) != 0;
	if (r.learned && (r.step != 0 || r.C != 1)) {
		set_error(std::string(who) + ": the learned form needs both steps' parameters and grey video");
		return BM4DOF_ERR_UNSUPPORTED;
	}
	if (r.nparts == 0) r.nparts = 2;
	for (int s = 1; s <= 2; s++) {
		if (s == 1 && r.step == 2) continue;
		if (s == 2 && r.step == 1) continue;
		bm4dof_status e = check_params(s == 1 ? r.p1 : r.p2);
		if (e != BM4DOF_OK) return e;
	}
	r.keep = (r.flags & BM4DOF_KEEP_GROUPS) != 0;
	r.mode = RunMode();
	r.mode.mixed = (r.flags & (BM4DOF_MIXED_PRECISION | BM4DOF_MIXED_CERTIFIED)) != 0;
	r.mode.certified = (r.flags & BM4DOF_MIXED_CERTIFIED) != 0;
	r.mode.vbm3d = (r.flags & BM4DOF_VBM3D_SEARCH) != 0;
	r.mode.beta1 = r.p1.beta;
	const bool color = r.C > 1;
	r.yuv1 = color && r.p1.colorSpace == BM4DOF_YUV;
	r.yuv2 = color && r.p2.colorSpace == BM4DOF_YUV;
	r.run1 = r.step != 2 && !r.learned;
	r.run2 = r.step != 1 || r.learned;
	return BM4DOF_OK;
}

// Inputs, outputs and both steps allocated before any launch.
bm4dof_status prepare_run(bm4dof_ctx *ctx, RunArgs &r)
{
	const size_t P = (r.W + 7) / 8 * 8;
	const size_t nv = P * r.H * r.C * r.F;
	RunMode m2 = r.mode;
	m2.learned = r.learned;
	for (int pass = 0; pass < 2; pass++) {
		// the second pass allocates nothing: every address is final after it
		DBUF("noisy", nv, r.d_noisy);
		DBUF("basic_rgb", nv, r.d_basic);
		DBUF("final", nv, r.d_final);
		if (r.use_flow) {
			DBUF("fflow", P * r.H * 2 * r.F, r.d_ff);
			DBUF("bflow", P * r.H * 2 * r.F, r.d_bf);
		}
		if ((r.run1 && r.yuv1) || (r.run2 && r.yuv2)) DBUF("noisy_yuv", nv, r.d_noisy_yuv);
		if (r.run2 && r.yuv2 && !r.learned) DBUF("basic_yuv", nv, r.d_basic_yuv);
		bm4dof_status e;
		if (r.run1 && (e = prepare_step(ctx, 0, 1, r.p1, r.W, r.H, r.C, r.F, r.use_flow, r.nparts, r.mode)) != BM4DOF_OK)
			return e;
		if (r.run2 && (e = prepare_step(ctx, 1, 2, r.p2, r.W, r.H, r.C, r.F, r.use_flow, r.nparts, m2)) != BM4DOF_OK)
			return e;
	}
	return BM4DOF_OK;
}

// The whole run on the context's stream: uploads, both steps, downloads.
bm4dof_status launch_run(bm4dof_ctx *ctx, const RunArgs &r)
{
	const unsigned W = r.W, H = r.H, C = r.C, F = r.F;
	const size_t nv = (size_t)(W + 7) / 8 * 8 * H * C * F;
	Image in = image(r.d_noisy, W, H, C, F);
	Image bas = image(r.d_basic, W, H, C, F);
	Image fin = image(r.d_final, W, H, C, F);
	Image ff = image(r.d_ff, W, H, 2, F), bf = image(r.d_bf, W, H, 2, F);
	{
		Mark m(ctx, T_OTHER);
		bm4dof_status s = upload(ctx, in, r.noisy);
		if (s != BM4DOF_OK) return s;
		if (r.use_flow) {
			if ((s = upload(ctx, ff, r.fflow)) != BM4DOF_OK) return s;
			if ((s = upload(ctx, bf, r.bflow)) != BM4DOF_OK) return s;
		}
		if (r.step == 2 && (s = upload(ctx, bas, r.basic)) != BM4DOF_OK) return s;
	}
	Image in_yuv = in;
	if (r.d_noisy_yuv) {
		in_yuv = image(r.d_noisy_yuv, W, H, C, F);
		Mark m(ctx, T_OTHER);
		CK(launch_color(in, in_yuv, 1, ctx->st));
		ctx->launches++;
	}
	if (r.learned) {
		bm4dof_status s = launch_step(ctx, 1, in, in, ff, bf, fin, false);
		if (s != BM4DOF_OK) return s;
		Mark m(ctx, T_OTHER);
		CK(cudaMemcpyAsync(bas.p, fin.p, sizeof(float) * nv, cudaMemcpyDeviceToDevice, ctx->st));
	}
	if (r.run1) {
		bm4dof_status s = launch_step(ctx, 0, r.yuv1 ? in_yuv : in, in, ff, bf, bas, r.yuv1);
		if (s != BM4DOF_OK) return s;
	}
	if (r.run2 && !r.learned) {
		Image bas_yuv = bas;
		if (r.yuv2) {
			bas_yuv = image(r.d_basic_yuv, W, H, C, F);
			Mark m(ctx, T_OTHER);
			CK(launch_color(bas, bas_yuv, 1, ctx->st));
			ctx->launches++;
		}
		bm4dof_status s = launch_step(ctx, 1, r.yuv2 ? in_yuv : in, bas_yuv, ff, bf, fin, r.yuv2);
		if (s != BM4DOF_OK) return s;
		if (r.yuv2) {
			// the reference returns basic after a forward and inverse transform (nldct.cpp:423, 467)
			Mark m(ctx, T_OTHER);
			CK(launch_color(bas_yuv, bas, 0, ctx->st));
			ctx->launches++;
		}
	}
	{
		Mark m(ctx, T_OTHER);
		bm4dof_status s = download(ctx, r.basic, bas);
		if (s != BM4DOF_OK) return s;
		if (r.step != 1 && (s = download(ctx, r.final_, fin)) != BM4DOF_OK) return s;
	}
	return BM4DOF_OK;
}

// After the stream drained: ratios and kept neighbour lists.
bm4dof_status finish_run(bm4dof_ctx *ctx, const RunArgs &r, float ratios[2])
{
	float gr[2] = {0.f, 0.f};
	ctx->m_groups = ctx->m_exact = ctx->m_uncertified = 0;
	if (r.run1) gr[0] = step_ratio(ctx, 0);
	if (r.run2) gr[1] = step_ratio(ctx, 1);
	if (r.keep) {
		bm4dof_status s;
		if (r.run1 && (s = keep_groups(ctx, 0, 1)) != BM4DOF_OK) return s;
		if (r.run2 && (s = keep_groups(ctx, 1, 2)) != BM4DOF_OK) return s;
	}
	if (ratios) { ratios[0] = gr[0]; ratios[1] = gr[1]; }
	return BM4DOF_OK;
}

void begin_call(bm4dof_ctx *ctx)
{
	ctx->marks.clear();
	ctx->next_event = 0;
	ctx->launches = 0;
	ctx->kept[0].clear();
	ctx->kept[1].clear();
}

bm4dof_status collect_times(bm4dof_ctx *ctx)
{
	for (int k = 0; k < 5; k++) ctx->ms[k] = 0.f;
	cudaEventElapsedTime(&ctx->ms[4], ctx->t_begin, ctx->t_end);
	for (auto &mk : ctx->marks) {
		float ms = 0.f;
		cudaEventElapsedTime(&ms, mk.second.first, mk.second.second);
		ctx->ms[mk.first] += ms;
	}
	return BM4DOF_OK;
}

}  // namespace

extern "C" {

bm4dof_status bm4dof_run(bm4dof_ctx *ctx, const float *noisy, const float *fflow, const float *bflow,
                         unsigned W, unsigned H, unsigned C, unsigned F, float *basic, float *final_,
                         const bm4dof_params *p1, const bm4dof_params *p2, unsigned nparts,
                         unsigned flags, float ratios[2])
{
	CtxLock lock_(ctx);
	clear_error();
	if (!ctx || !p1 || !p2) {
		set_error("bm4dof_run: null pointer or empty video");
		return BM4DOF_ERR_ARGUMENT;
	}
	RunArgs r;
	r.noisy = noisy;
	r.fflow = fflow;
	r.bflow = bflow;
	r.W = W;
	r.H = H;
	r.C = C;
	r.F = F;
	r.basic = basic;
	r.final_ = final_;
	r.p1 = *p1;
	r.p2 = *p2;
	r.nparts = nparts;
	r.flags = flags;
	bm4dof_status e = validate_run(r, "bm4dof_run");
	if (e != BM4DOF_OK) return e;
	CK(cudaSetDevice(ctx->device));
	begin_call(ctx);
	if (!ctx->t_begin) {
		CK(cudaEventCreate(&ctx->t_begin));
		CK(cudaEventCreate(&ctx->t_end));
	}
	set_budget(ctx);
	ctx->whf = (float)(W * H * F);
	if ((e = prepare_run(ctx, r)) != BM4DOF_OK) return e;
	CK(cudaEventRecord(ctx->t_begin, ctx->st));
	if ((e = launch_run(ctx, r)) != BM4DOF_OK) return e;
	CK(cudaEventRecord(ctx->t_end, ctx->st));
	CK(cudaStreamSynchronize(ctx->st));
	collect_times(ctx);
	return finish_run(ctx, r, ratios);
}

bm4dof_status bm4dof_plan(unsigned W, unsigned H, unsigned F, unsigned nparts, const bm4dof_params *params,
                          const bm4dof_crop *crop, int process, int *tiles, unsigned tiles_cap, int *coords,
                          size_t coords_cap, unsigned *ntiles, size_t *ncoords)
{
	clear_error();
	if (!params || !ntiles || !ncoords || W == 0 || H == 0 || F == 0 || params->offSet == 0 ||
	    params->offSetTime == 0 || params->sizePatch == 0 || params->sizePatchTime == 0) {
		set_error("bm4dof_plan: bad argument");
		return BM4DOF_ERR_ARGUMENT;
	}
	int borders[6];
	crop_borders(crop, borders);
	Plan pl;
	make_plan(pl, W, H, F, nparts ? nparts : 2, *params, process ? borders : nullptr);
	*ntiles = (unsigned)pl.tiles.size();
	size_t n = 0;
	for (size_t i = 0; i < pl.tiles.size(); i++) {
		const Tile &T = pl.tiles[i];
		if (tiles && i < tiles_cap) {
			const int v[7] = {T.ox, T.oy, T.w, T.h, T.nx, T.ny, T.nf};
			for (int k = 0; k < 7; k++) tiles[7 * i + k] = v[k];
		}
		const int offs[3] = {T.gx, T.gy, T.gf}, cnt[3] = {T.nx, T.ny, T.nf};
		for (int a = 0; a < 3; a++)
			for (int j = 0; j < cnt[a]; j++, n++)
				if (coords && n < coords_cap) coords[n] = pl.grid[offs[a] + j];
	}
	*ncoords = n;
	return BM4DOF_OK;
}

bm4dof_status bm4dof_set_memory_limit(bm4dof_ctx *ctx, size_t bytes)
{
	CtxLock lock_(ctx);
	clear_error();
	if (!ctx) {
		set_error("bm4dof_set_memory_limit: null context");
		return BM4DOF_ERR_ARGUMENT;
	}
	ctx->mem_limit = bytes;
	return BM4DOF_OK;
}

bm4dof_status bm4dof_process(bm4dof_ctx *ctx, const float *noisy, const float *fflow, const float *bflow,
                             unsigned W, unsigned H, unsigned C, unsigned F, float *basic, float *final_,
                             const bm4dof_params *params, const bm4dof_crop *crop, unsigned flags,
                             unsigned *groups)
{
	CtxLock lock_(ctx);
	clear_error();
	if (!ctx || !params) {
		set_error("bm4dof_process: null pointer or empty video");
		return BM4DOF_ERR_ARGUMENT;
	}
	if (flags & BM4DOF_LEARNED) {
		set_error("bm4dof_process: the learned form runs both steps (use bm4dof_run)");
		return BM4DOF_ERR_UNSUPPORTED;
	}
	// processNlBayes runs the step that isFirstStep names (nldct.cpp:502, 740)
	const bool step1 = params->isFirstStep != 0;
	RunArgs r;
	r.noisy = noisy;
	r.fflow = fflow;
	r.bflow = bflow;
	r.W = W;
	r.H = H;
	r.C = C;
	r.F = F;
	r.basic = basic;
	r.final_ = final_;
	r.p1 = *params;
	r.p2 = *params;
	(step1 ? r.p2 : r.p1).sizePatch = 0;
	r.nparts = 1;
	r.flags = flags;
	bm4dof_status e = validate_run(r, "bm4dof_process");
	if (e != BM4DOF_OK) return e;
	int borders[6];
	crop_borders(crop, borders);
	r.mode.borders = borders;
	r.yuv1 = r.yuv2 = false;   // no colour transform of its own
	CK(cudaSetDevice(ctx->device));
	begin_call(ctx);
	if (!ctx->t_begin) {
		CK(cudaEventCreate(&ctx->t_begin));
		CK(cudaEventCreate(&ctx->t_end));
	}
	set_budget(ctx);
	ctx->whf = (float)(W * H * F);
	if ((e = prepare_run(ctx, r)) != BM4DOF_OK) return e;
	CK(cudaEventRecord(ctx->t_begin, ctx->st));
	if ((e = launch_run(ctx, r)) != BM4DOF_OK) return e;
	CK(cudaEventRecord(ctx->t_end, ctx->st));
	CK(cudaStreamSynchronize(ctx->st));
	collect_times(ctx);
	if ((e = finish_run(ctx, r, nullptr)) != BM4DOF_OK) return e;
	if (groups) *groups = ext(ctx).steps[step1 ? 0 : 1].h_small[64];
	return BM4DOF_OK;
}

}  // extern "C"

namespace {

std::string batch_key(const bm4dof_sequence *seqs, unsigned n, unsigned flags, const bm4dof_tuning &t, bool gain)
{
	std::string k;
	auto add = [&k](const void *p, size_t b) { k.append(static_cast<const char *>(p), b); };
	add(&n, sizeof n);
	add(&flags, sizeof flags);
	add(&t, sizeof t);
	add(&gain, sizeof gain);
	for (unsigned i = 0; i < n; i++) add(&seqs[i], offsetof(bm4dof_sequence, ratios));
	return k;
}

bm4dof_status run_batched(bm4dof_ctx *ctx, bm4dof_sequence *seqs, unsigned n, unsigned flags,
                          const bm4dof_tuning &tu)
{
	bm4dof_ctx_ext &X = ext(ctx);
	std::vector<RunArgs> args(n);
	for (unsigned i = 0; i < n; i++) {
		RunArgs &r = args[i];
		const bm4dof_sequence &q = seqs[i];
		r.noisy = q.noisy;
		r.fflow = q.fflow;
		r.bflow = q.bflow;
		r.W = q.width;
		r.H = q.height;
		r.C = q.channels;
		r.F = q.frames;
		r.basic = q.basic;
		r.final_ = q.final_;
		r.p1 = q.params1;
		r.p2 = q.params2;
		r.nparts = q.nparts;
		r.flags = flags | BM4DOF_DEVICE_POINTERS;
		bm4dof_status e = validate_run(r, "bm4dof_run_batched");
		if (e != BM4DOF_OK) {
			set_error(std::string(bm4dof_last_error()) + " (sequence " + std::to_string(i) + ")");
			return e;
		}
	}
	CK(cudaSetDevice(ctx->device));
	begin_call(ctx);
	if (!ctx->t_begin) {
		CK(cudaEventCreate(&ctx->t_begin));
		CK(cudaEventCreate(&ctx->t_end));
	}
	const unsigned nb = std::max(1u, std::min(n, tu.branches ? tu.branches : std::min(n, 16u)));
	const std::string key = batch_key(seqs, n, flags, tu, ctx->has_gain);
	if (!(X.exec && X.exec_key == key)) {
		if (X.exec) {
			cudaGraphExecDestroy(X.exec);
			X.exec = nullptr;
		}
		while (X.branches.size() < nb) {
			cudaStream_t s;
			CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
			X.branches.push_back(s);
			cudaEvent_t e;
			CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
			X.joins.push_back(e);
		}
		if (!X.fork) CK(cudaEventCreateWithFlags(&X.fork, cudaEventDisableTiming));
		while (X.children.size() < n) X.children.push_back(make_child(ctx));
		// every sequence holds its buffers for the whole graph: the chunk
		// budgets of all of them together stay within half the device memory
		size_t per_child = (size_t)(tu.slot_mb ? tu.slot_mb : 1024) << 20;
		{
			size_t freeb = 0, totalb = 0, held = 0;
			for (bm4dof_ctx *c : X.children) held += c->held;
			if (cudaMemGetInfo(&freeb, &totalb) == cudaSuccess) {
				const size_t cap = std::max<size_t>((size_t)64 << 20, (freeb + held) / 2 / n);
				per_child = std::min(per_child, cap);
			}
		}
		// allocation of every sequence's buffers, before the capture
		for (unsigned i = 0; i < n; i++) {
			bm4dof_ctx *c = X.children[i];
			c->st = X.branches[i % nb];
			c->slot_budget = per_child;
			c->search_ctas = tu.search_ctas;
			c->search_strip = tu.search_strip;
			c->gather_depth = tu.gather_depth;
			c->kappa = ctx->kappa;
			c->has_gain = ctx->has_gain;
			c->whf = (float)(args[i].W * args[i].H * args[i].F);
			bm4dof_status e = prepare_run(c, args[i]);
			if (e != BM4DOF_OK) {
				set_error(std::string(bm4dof_last_error()) + " (sequence " + std::to_string(i) + ")");
				return e;
			}
			if (args[i].learned && ctx->has_gain) {
				float *pm, *cm;
				uint16_t *pw, *cw;
				bm4dof_ctx *pc = ctx;
				{
					bm4dof_ctx *ctx = pc;
					DBUF("gain_master", kMlpMasterSize, pm);
					DBUF("gain_wt", kMlpWtSize, pw);
				}
				{
					bm4dof_ctx *ctx = c;
					DBUF("gain_master", kMlpMasterSize, cm);
					DBUF("gain_wt", kMlpWtSize, cw);
				}
				CK(cudaMemcpy(cm, pm, sizeof(float) * kMlpMasterSize, cudaMemcpyDeviceToDevice));
				CK(cudaMemcpy(cw, pw, sizeof(uint16_t) * kMlpWtSize, cudaMemcpyDeviceToDevice));
			}
		}
		CK(cudaDeviceSynchronize());
		// capture: fork the branches off the context's stream, record every
		// sequence on its branch, join
		cudaGraph_t graph = nullptr;
		CK(cudaStreamBeginCapture(ctx->st, cudaStreamCaptureModeRelaxed));
		bool fail = false;
		std::string why;
		bm4dof_status st = BM4DOF_OK;
		if (cudaEventRecord(X.fork, ctx->st) != cudaSuccess) fail = true;
		for (unsigned b = 0; b < nb && !fail; b++)
			if (cudaStreamWaitEvent(X.branches[b], X.fork, 0) != cudaSuccess) fail = true;
		for (unsigned i = 0; i < n && !fail; i++) {
			bm4dof_ctx *c = X.children[i];
			c->launches = 0;
			st = launch_run(c, args[i]);
			if (st != BM4DOF_OK) {
				fail = true;
				why = bm4dof_last_error();
			}
		}
		for (unsigned b = 0; b < nb && !fail; b++) {
			if (cudaEventRecord(X.joins[b], X.branches[b]) != cudaSuccess ||
			    cudaStreamWaitEvent(ctx->st, X.joins[b], 0) != cudaSuccess)
				fail = true;
		}
		cudaError_t ec = cudaStreamEndCapture(ctx->st, &graph);
		if (fail || ec != cudaSuccess || !graph) {
			if (graph) cudaGraphDestroy(graph);
			cudaGetLastError();
			set_error("bm4dof_run_batched: graph capture failed" + (why.empty() ? std::string() : ": " + why) +
			          (ec != cudaSuccess ? std::string(" (") + cudaGetErrorString(ec) + ")" : std::string()));
			return st != BM4DOF_OK ? st : BM4DOF_ERR_CUDA;
		}
		cudaError_t ei = cudaGraphInstantiate(&X.exec, graph, 0);
		cudaGraphDestroy(graph);
		if (ei != cudaSuccess) {
			X.exec = nullptr;
			set_error(std::string("bm4dof_run_batched: graph instantiation failed: ") + cudaGetErrorString(ei));
			return BM4DOF_ERR_CUDA;
		}
		X.exec_key = key;
	}
	CK(cudaEventRecord(ctx->t_begin, ctx->st));
	CK(cudaGraphLaunch(X.exec, ctx->st));
	CK(cudaEventRecord(ctx->t_end, ctx->st));
	CK(cudaStreamSynchronize(ctx->st));
	for (int k = 0; k < 5; k++) ctx->ms[k] = 0.f;
	cudaEventElapsedTime(&ctx->ms[4], ctx->t_begin, ctx->t_end);
	ctx->launches = 0;
	for (unsigned i = 0; i < n; i++) {
		bm4dof_ctx *c = X.children[i];
		ctx->launches += c->launches;
		float r[2] = {0.f, 0.f};
		if (args[i].run1) r[0] = step_ratio(c, 0);
		if (args[i].run2) r[1] = step_ratio(c, 1);
		seqs[i].ratios[0] = r[0];
		seqs[i].ratios[1] = r[1];
	}
	return BM4DOF_OK;
}

}  // namespace

extern "C" {

bm4dof_status bm4dof_run_batched(bm4dof_ctx *ctx, bm4dof_sequence *seqs, unsigned n, unsigned flags,
                                 const bm4dof_tuning *tuning)
{
	CtxLock lock_(ctx);
	clear_error();
	if (!ctx || !seqs || n == 0) {
		set_error("bm4dof_run_batched: null context or no sequences");
		return BM4DOF_ERR_ARGUMENT;
	}
	if (flags & ~(BM4DOF_MIXED_PRECISION | BM4DOF_MIXED_CERTIFIED | BM4DOF_LEARNED | BM4DOF_DEVICE_POINTERS |
	              BM4DOF_VBM3D_SEARCH)) {
		set_error("bm4dof_run_batched: unsupported flags");
		return BM4DOF_ERR_UNSUPPORTED;
	}
	bm4dof_tuning t = tuning ? *tuning : bm4dof_tuning{0, 0, 0, 0, 0};
	if (t.search_ctas != 0 && t.search_ctas != 4 && t.search_ctas != 6) {
		set_error("bm4dof_run_batched: search_ctas must be 0, 4 or 6");
		return BM4DOF_ERR_ARGUMENT;
	}
	if (t.search_strip != 0 && t.search_strip != 7 && t.search_strip != 21) {
		set_error("bm4dof_run_batched: search_strip must be 0, 7 or 21");
		return BM4DOF_ERR_ARGUMENT;
	}
	if (t.gather_depth > 2) {
		set_error("bm4dof_run_batched: gather_depth must be 0, 1 or 2");
		return BM4DOF_ERR_ARGUMENT;
	}
	return run_batched(ctx, seqs, n, flags, t);
}

bm4dof_status bm4dof_autotune(bm4dof_ctx *ctx, bm4dof_sequence *seqs, unsigned n, unsigned sample,
                              unsigned flags, bm4dof_tuning *best, float *table, unsigned cap, unsigned *rows)
{
	CtxLock lock_(ctx);
	clear_error();
	if (!ctx || !seqs || n == 0 || !best) {
		set_error("bm4dof_autotune: bad argument");
		return BM4DOF_ERR_ARGUMENT;
	}
	const unsigned m = std::max(1u, std::min(n, sample ? sample : 16u));
	unsigned nrow = 0;
	auto time_one = [&](const bm4dof_tuning &t, float &ms) -> bm4dof_status {
		bm4dof_status e = run_batched(ctx, seqs, m, flags, t);   // capture + first launch
		if (e != BM4DOF_OK) return e;
		ms = 0.f;
		for (int rep = 0; rep < 2; rep++) {                      // replays
			if ((e = run_batched(ctx, seqs, m, flags, t)) != BM4DOF_OK) return e;
			ms += ctx->ms[4];
		}
		ms *= 0.5f;
		if (table && nrow < cap) {
			float *row = table + 6 * nrow;
			row[0] = (float)t.branches;
			row[1] = (float)t.slot_mb;
			row[2] = (float)t.search_ctas;
			row[3] = (float)t.search_strip;
			row[4] = (float)t.gather_depth;
			row[5] = ms;
		}
		nrow++;
		return BM4DOF_OK;
	};
	bm4dof_tuning cur = {std::min(m, 16u), 1024, 6, 21, 1};
	float best_ms = 0.f;
	bm4dof_status e = time_one(cur, best_ms);
	if (e != BM4DOF_OK) return e;
	const unsigned br[] = {1, 4, 8, 16, 32, 64};
	for (unsigned b : br) {
		if (b > m || b == cur.branches) continue;
		bm4dof_tuning t = cur;
		t.branches = b;
		float ms;
		if ((e = time_one(t, ms)) != BM4DOF_OK) return e;
		if (ms < best_ms) { best_ms = ms; cur = t; }
	}
	const unsigned mbs[] = {256, 4096};
	const bm4dof_tuning base = cur;
	for (unsigned mb : mbs) {
		bm4dof_tuning t = base;
		t.slot_mb = mb;
		float ms;
		if ((e = time_one(t, ms)) != BM4DOF_OK) return e;
		if (ms < best_ms) { best_ms = ms; cur = t; }
	}
	{
		// the exact search's tile shape: 21 or 7 candidates per thread along a
		// window column at 6 CTAs per SM, or strips of 7 at 4 CTAs per SM
		const bm4dof_tuning b2 = cur;
		const unsigned shapes[2][2] = {{6, 7}, {4, 7}};
		for (const auto &sh : shapes) {
			bm4dof_tuning t = b2;
			t.search_ctas = sh[0];
			t.search_strip = sh[1];
			float ms;
			if ((e = time_one(t, ms)) != BM4DOF_OK) return e;
			if (ms < best_ms) { best_ms = ms; cur = t; }
		}
	}
	{
		// the gather's staging depth: members in flight per thread
		bm4dof_tuning t = cur;
		t.gather_depth = 2;
		float ms;
		if ((e = time_one(t, ms)) != BM4DOF_OK) return e;
		if (ms < best_ms) { best_ms = ms; cur = t; }
	}
	// branches scale with the batch: keep the chosen ratio of sequences per branch
	if (m < n && cur.branches == m) cur.branches = std::min(n, 64u);
	*best = cur;
	if (rows) *rows = nrow;
	return BM4DOF_OK;
}

bm4dof_status bm4dof_get_groups(bm4dof_ctx *ctx, unsigned step, unsigned tile, unsigned *ref,
                                unsigned *nsimp, unsigned *index, unsigned stride, size_t cap,
                                size_t *count)
{
	CtxLock lock_(ctx);
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

bm4dof_status bm4dof_set_gain_network(bm4dof_ctx *ctx, const float *params, size_t n, float kappa)
{
	CtxLock lock_(ctx);
	clear_error();
	if (!ctx || (params && n != (size_t)kMlpPublicSize) || kappa < 0.f) {
		set_error("bm4dof_set_gain_network: bad argument (the blob holds " + std::to_string(kMlpPublicSize) +
		          " floats)");
		return BM4DOF_ERR_ARGUMENT;
	}
	CK(cudaSetDevice(ctx->device));
	ctx->kappa = kappa > 0.f ? kappa : 1.5f;
	if (!params) {
		ctx->has_gain = false;
		return BM4DOF_OK;
	}
	std::vector<float> master(kMlpMasterSize);
	mlp_public_to_master(params, master.data());
	float *gm;
	uint16_t *gw;
	DBUF("gain_master", kMlpMasterSize, gm);
	DBUF("gain_wt", kMlpWtSize, gw);
	CK(cudaMemcpyAsync(gm, master.data(), sizeof(float) * kMlpMasterSize, cudaMemcpyHostToDevice, ctx->st));
	CK(launch_pack_weights(gm, gw, ctx->st));
	CK(cudaStreamSynchronize(ctx->st));
	ctx->has_gain = true;
	return BM4DOF_OK;
}

bm4dof_status bm4dof_learned_stats(bm4dof_ctx *ctx, unsigned long long *groups, unsigned long long *fallbacks)
{
	CtxLock lock_(ctx);
	if (!ctx) return BM4DOF_ERR_ARGUMENT;
	if (groups) *groups = ctx->l_groups;
	if (fallbacks) *fallbacks = ctx->l_fallbacks;
	return BM4DOF_OK;
}

bm4dof_status bm4dof_mixed_stats(bm4dof_ctx *ctx, unsigned long long *groups, unsigned long long *exact,
                                 unsigned long long *uncertified)
{
	CtxLock lock_(ctx);
	if (!ctx) return BM4DOF_ERR_ARGUMENT;
	if (groups) *groups = ctx->m_groups;
	if (exact) *exact = ctx->m_exact;
	if (uncertified) *uncertified = ctx->m_uncertified;
	return BM4DOF_OK;
}

bm4dof_status bm4dof_tc_selftest(const void *a, const void *b, float *d, void *stream)
{
	clear_error();
	if (!a || !b || !d) {
		set_error("bm4dof_tc_selftest: null argument");
		return BM4DOF_ERR_ARGUMENT;
	}
	cudaStream_t st = static_cast<cudaStream_t>(stream);
	int *status = nullptr;
	cudaError_t e = cudaMallocAsync(reinterpret_cast<void **>(&status), sizeof(int), st);
	if (e == cudaSuccess) e = cudaMemsetAsync(status, 0, sizeof(int), st);
	if (e == cudaSuccess)
		e = tc_selftest(static_cast<const uint16_t *>(a), static_cast<const uint16_t *>(b), d, status, st);
	int h = 0;
	if (e == cudaSuccess) e = cudaMemcpyAsync(&h, status, sizeof(int), cudaMemcpyDeviceToHost, st);
	if (e == cudaSuccess) e = cudaStreamSynchronize(st);
	if (status) cudaFreeAsync(status, st);
	if (e != cudaSuccess) {
		set_error(std::string("bm4dof_tc_selftest: ") + cudaGetErrorString(e));
		return BM4DOF_ERR_CUDA;
	}
	if (h) {
		set_error("bm4dof_tc_selftest: the MMA completion wait gave up");
		return BM4DOF_ERR_CUDA;
	}
	return BM4DOF_OK;
}

bm4dof_status bm4dof_gain_samples(bm4dof_ctx *ctx, const float *noisy, const float *basic, const float *fflow,
                                  const float *bflow, unsigned W, unsigned H, unsigned F,
                                  const bm4dof_params *p2, unsigned nparts, unsigned flags, float *feat,
                                  float *target, unsigned char *valid, size_t cap, size_t *count)
{
	CtxLock lock_(ctx);
	clear_error();
	if (!ctx || !noisy || !basic || !p2 || !feat || !target || !valid || !count || W == 0 || H == 0 || F == 0 ||
	    (fflow == nullptr) != (bflow == nullptr) || (flags & ~BM4DOF_DEVICE_POINTERS)) {
		set_error("bm4dof_gain_samples: bad argument");
		return BM4DOF_ERR_ARGUMENT;
	}
	bm4dof_status e = check_params(*p2);
	if (e != BM4DOF_OK) return e;
	if (nparts == 0) nparts = 2;
	CK(cudaSetDevice(ctx->device));
	ctx->marks.clear();
	ctx->next_event = 0;
	ctx->launches = 0;
	const size_t P = (W + 7) / 8 * 8, nv = P * H * F;
	float *d_noisy, *d_basic, *d_ff = nullptr, *d_bf = nullptr;
	DBUF("noisy", nv, d_noisy);
	DBUF("basic_rgb", nv, d_basic);
	Image in = image(d_noisy, W, H, 1, F), bas = image(d_basic, W, H, 1, F);
	Image ff = image(nullptr, W, H, 2, F), bf = image(nullptr, W, H, 2, F);
	bm4dof_status s;
	SampleOut so = {feat, target, valid, cap, count};
	RunMode mode;
	mode.samples = &so;
	set_budget(ctx);
	ctx->whf = (float)(W * H * F);
	for (int pass = 0; pass < 2; pass++)
		if ((s = prepare_step(ctx, 1, 2, *p2, W, H, 1, F, fflow != nullptr, nparts, mode)) != BM4DOF_OK) return s;
	const StepState &S = ext(ctx).steps[1];
	*count = (size_t)S.G;
	if ((size_t)S.G > cap) {
		set_error("bm4dof_gain_samples: " + std::to_string(S.G) + " groups do not fit cap = " + std::to_string(cap));
		return BM4DOF_ERR_ARGUMENT;
	}
	// addresses of the inputs after the step's allocations
	DBUF("noisy", nv, d_noisy);
	DBUF("basic_rgb", nv, d_basic);
	in.p = d_noisy;
	bas.p = d_basic;
	if (fflow) {
		DBUF("fflow", P * H * 2 * F, d_ff);
		DBUF("bflow", P * H * 2 * F, d_bf);
		ff.p = d_ff;
		bf.p = d_bf;
	}
	if ((s = upload(ctx, in, noisy)) != BM4DOF_OK || (s = upload(ctx, bas, basic)) != BM4DOF_OK) return s;
	if (fflow && ((s = upload(ctx, ff, fflow)) != BM4DOF_OK || (s = upload(ctx, bf, bflow)) != BM4DOF_OK)) return s;
	if ((s = launch_step(ctx, 1, in, bas, ff, bf, in, false)) != BM4DOF_OK) return s;
	CK(cudaStreamSynchronize(ctx->st));
	return BM4DOF_OK;
}

void bm4dof_tvl1_default_params(bm4dof_tvl1_params *p)
{
	if (!p) return;
	p->tau = 0.25f;
	p->lambda = 0.2f;
	p->theta = 0.3f;
	p->nscales = 100;
	p->fscale = 1;
	p->zfactor = 0.5f;
	p->warps = 5;
	p->epsilon = 0.01f;
}

}  // extern "C"

namespace {

// tvl1flow's parameter checks (main.c:101-140) and the scale cap (147-153)
bm4dof_status tvl1_setup(const bm4dof_tvl1_params *in, unsigned W, unsigned H, Tvl1Params &p)
{
	bm4dof_tvl1_params d;
	bm4dof_tvl1_default_params(&d);
	const bm4dof_tvl1_params q = in ? *in : d;
	p.tau = (q.tau <= 0 || q.tau > 0.25f) ? 0.25f : q.tau;
	p.lambda = q.lambda <= 0 ? 0.15f : q.lambda;
	p.theta = q.theta <= 0 ? 0.3f : q.theta;
	p.nscales = q.nscales <= 0 ? 100 : q.nscales;
	p.zfactor = (q.zfactor <= 0 || q.zfactor >= 1) ? 0.5f : q.zfactor;
	p.warps = q.warps <= 0 ? 5 : q.warps;
	p.epsilon = q.epsilon <= 0 ? 0.01f : q.epsilon;
	p.fscale = q.fscale < 0 ? 0 : q.fscale;
	p.nscales = tvl1_scales((int)W, (int)H, p.nscales, p.zfactor);
	if (p.nscales < 1) p.nscales = 1;
	if (p.nscales < p.fscale) p.fscale = p.nscales;
	return BM4DOF_OK;
}

bm4dof_status tvl1_run(bm4dof_ctx *ctx, const float *dI0, const float *dI1, unsigned W, unsigned H, unsigned n,
                       const Tvl1Params &p, float *du, float *dv)
{
	float *ws;
	int *iws;
	DBUF("tvl1_ws", tvl1_workspace_floats((int)W, (int)H, (int)n, p.nscales, p.zfactor), ws);
	DBUF("tvl1_iws", 2 * (size_t)n + 2, iws);
	std::string why;
	cudaError_t e = tvl1_flow(dI0, dI1, (int)W, (int)H, (int)n, p, du, dv, ws, iws, ctx->nsm, ctx->st, why);
	if (e != cudaSuccess) {
		cudaGetLastError();
		set_error("bm4dof_tvl1: " + (why.empty() ? std::string(cudaGetErrorString(e)) : why));
		return e == cudaErrorInvalidValue ? BM4DOF_ERR_UNSUPPORTED : BM4DOF_ERR_CUDA;
	}
	return BM4DOF_OK;
}

}  // namespace

extern "C" {

bm4dof_status bm4dof_tvl1_pairs(bm4dof_ctx *ctx, const float *I0, const float *I1, unsigned W, unsigned H,
                                unsigned n, const bm4dof_tvl1_params *params, float *uv, unsigned flags)
{
	CtxLock lock_(ctx);
	clear_error();
	if (!ctx || !I0 || !I1 || !uv || W < 2 || H < 2 || n == 0 || (flags & ~BM4DOF_DEVICE_POINTERS)) {
		set_error("bm4dof_tvl1_pairs: bad argument");
		return BM4DOF_ERR_ARGUMENT;
	}
	CK(cudaSetDevice(ctx->device));
	begin_call(ctx);
	Tvl1Params p;
	tvl1_setup(params, W, H, p);
	const size_t plane = (size_t)W * H;
	float *d0, *d1, *du, *dv, *duv;
	DBUF("tvl1_i0", plane * n, d0);
	DBUF("tvl1_i1", plane * n, d1);
	DBUF("tvl1_u", plane * n, du);
	DBUF("tvl1_v", plane * n, dv);
	DBUF("tvl1_uv", plane * 2 * n, duv);
	if (!ctx->t_begin) {
		CK(cudaEventCreate(&ctx->t_begin));
		CK(cudaEventCreate(&ctx->t_end));
	}
	CK(cudaEventRecord(ctx->t_begin, ctx->st));
	CK(cudaMemcpyAsync(d0, I0, sizeof(float) * plane * n, cudaMemcpyDefault, ctx->st));
	CK(cudaMemcpyAsync(d1, I1, sizeof(float) * plane * n, cudaMemcpyDefault, ctx->st));
	bm4dof_status s = tvl1_run(ctx, d0, d1, W, H, n, p, du, dv);
	if (s != BM4DOF_OK) return s;
	// [pair][2][y][x]
	CK(cudaMemcpy2DAsync(duv, sizeof(float) * plane * 2, du, sizeof(float) * plane, sizeof(float) * plane, n,
	                     cudaMemcpyDeviceToDevice, ctx->st));
	CK(cudaMemcpy2DAsync(duv + plane, sizeof(float) * plane * 2, dv, sizeof(float) * plane, sizeof(float) * plane, n,
	                     cudaMemcpyDeviceToDevice, ctx->st));
	CK(cudaMemcpyAsync(uv, duv, sizeof(float) * plane * 2 * n, cudaMemcpyDefault, ctx->st));
	CK(cudaEventRecord(ctx->t_end, ctx->st));
	CK(cudaStreamSynchronize(ctx->st));
	for (int k = 0; k < 5; k++) ctx->ms[k] = 0.f;
	cudaEventElapsedTime(&ctx->ms[4], ctx->t_begin, ctx->t_end);
	return BM4DOF_OK;
}

bm4dof_status bm4dof_tvl1_video(bm4dof_ctx *ctx, const float *video, unsigned W, unsigned H, unsigned F,
                                const bm4dof_tvl1_params *params, float *fflow, float *bflow, unsigned flags)
{
	CtxLock lock_(ctx);
	clear_error();
	if (!ctx || !video || !fflow || !bflow || W < 2 || H < 2 || F < 2 || (flags & ~BM4DOF_DEVICE_POINTERS)) {
		set_error("bm4dof_tvl1_video: bad argument (grey video of at least 2 frames)");
		return BM4DOF_ERR_ARGUMENT;
	}
	CK(cudaSetDevice(ctx->device));
	begin_call(ctx);
	Tvl1Params p;
	tvl1_setup(params, W, H, p);
	const size_t plane = (size_t)W * H;
	const unsigned n = 2 * (F - 1);
	float *dvid, *d0, *d1, *du, *dv, *dff, *dbf;
	DBUF("tvl1_video", plane * F, dvid);
	DBUF("tvl1_i0", plane * n, d0);
	DBUF("tvl1_i1", plane * n, d1);
	DBUF("tvl1_u", plane * n, du);
	DBUF("tvl1_v", plane * n, dv);
	DBUF("tvl1_ff", plane * 2 * F, dff);
	DBUF("tvl1_bf", plane * 2 * F, dbf);
	if (!ctx->t_begin) {
		CK(cudaEventCreate(&ctx->t_begin));
		CK(cudaEventCreate(&ctx->t_end));
	}
	cudaStream_t st = ctx->st;
	CK(cudaEventRecord(ctx->t_begin, st));
	CK(cudaMemcpyAsync(dvid, video, sizeof(float) * plane * F, cudaMemcpyDefault, st));
	// pairs 0..F-2: t -> t+1 (forward); F-1..2F-3: t+1 -> t (backward of t+1)
	const size_t fb = sizeof(float) * plane * (F - 1);
	CK(cudaMemcpyAsync(d0, dvid, fb, cudaMemcpyDeviceToDevice, st));
	CK(cudaMemcpyAsync(d1, dvid + plane, fb, cudaMemcpyDeviceToDevice, st));
	CK(cudaMemcpyAsync(d0 + plane * (F - 1), dvid + plane, fb, cudaMemcpyDeviceToDevice, st));
	CK(cudaMemcpyAsync(d1 + plane * (F - 1), dvid, fb, cudaMemcpyDeviceToDevice, st));
	bm4dof_status s = tvl1_run(ctx, d0, d1, W, H, n, p, du, dv);
	if (s != BM4DOF_OK) return s;
	const size_t pb = sizeof(float) * plane;
	// fflow[t] = pair t (t < F-1), fflow[F-1] = fflow[F-2];
	// bflow[t] = pair F-1 + (t-1) (t >= 1), bflow[0] = bflow[1]  (tvl1flow-seq.sh)
	CK(cudaMemcpy2DAsync(dff, 2 * pb, du, pb, pb, F - 1, cudaMemcpyDeviceToDevice, st));
	CK(cudaMemcpy2DAsync(dff + plane, 2 * pb, dv, pb, pb, F - 1, cudaMemcpyDeviceToDevice, st));
	CK(cudaMemcpyAsync(dff + 2 * plane * (F - 1), dff + 2 * plane * (F - 2), 2 * pb, cudaMemcpyDeviceToDevice, st));
	CK(cudaMemcpy2DAsync(dbf + 2 * plane, 2 * pb, du + plane * (F - 1), pb, pb, F - 1, cudaMemcpyDeviceToDevice, st));
	CK(cudaMemcpy2DAsync(dbf + 3 * plane, 2 * pb, dv + plane * (F - 1), pb, pb, F - 1, cudaMemcpyDeviceToDevice, st));
	CK(cudaMemcpyAsync(dbf, dbf + 2 * plane, 2 * pb, cudaMemcpyDeviceToDevice, st));
	CK(cudaMemcpyAsync(fflow, dff, 2 * pb * F, cudaMemcpyDefault, st));
	CK(cudaMemcpyAsync(bflow, dbf, 2 * pb * F, cudaMemcpyDefault, st));
	CK(cudaEventRecord(ctx->t_end, st));
	CK(cudaStreamSynchronize(st));
	for (int k = 0; k < 5; k++) ctx->ms[k] = 0.f;
	cudaEventElapsedTime(&ctx->ms[4], ctx->t_begin, ctx->t_end);
	return BM4DOF_OK;
}

bm4dof_status bm4dof_last_timings(bm4dof_ctx *ctx, float ms[5], unsigned *launches)
{
	CtxLock lock_(ctx);
	if (!ctx) return BM4DOF_ERR_ARGUMENT;
	if (ms) for (int k = 0; k < 5; k++) ms[k] = ctx->ms[k];
	if (launches) *launches = ctx->launches;
	return BM4DOF_OK;
}

}  // extern "C"
