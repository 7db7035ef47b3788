// noalloc.cu -- the patch search with no device allocation.
//
// Some callers cannot call cudaMalloc: code running inside another
// framework's memory pool or a real-time pipeline that forbids allocation
// after start-up, a plug-in host that owns every device buffer, or a process
// that must not grow its device footprint once a stream is being captured.
// bm4dof_search_groups_noalloc serves them: the caller passes the video, the
// flows and the output arrays (device memory it owns), and every working
// buffer of the search -- tile descriptor, reference grid, flow trajectories,
// neighbour lists -- lives in one file-scope __device__ array of fixed size.
//
// Facts a caller must know:
//   * the array holds kScratchBytes (32 MiB) on every device that loads this
//     library, for the life of the process;
//   * in host code the array's name is only a host-side stand-in: its device
//     address is fetched once per device with cudaGetSymbolAddress (by the
//     first call on that device, with that device current), so make that
//     first call before any stream capture;
//   * every call uses the same array and leaves its contents behind; calls
//     that overlap on the GPU (different streams, or several host threads)
//     race on it and must be serialised by the caller;
//   * the call is asynchronous on the given stream.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <mutex>
#include <string>

#include "../../include/bm4dof.h"
#include "internal.hpp"

namespace bm4dof {

namespace {

constexpr size_t kScratchBytes = (size_t)32 << 20;
constexpr int kMaxDevices = 64;

__device__ __align__(256) unsigned char g_search_scratch[kScratchBytes];

std::mutex g_mu;
void *g_scratch_addr[kMaxDevices];   // device address of g_search_scratch, per device

size_t align256(size_t n) { return (n + 255) / 256 * 256; }

// Grid positions along one axis (nldct.cpp:528-553) in closed form: `base`
// positions ori, ori+step, ..., then, when `extra`, the last position before
// the end of the crop (taken when the crop touches the image border there).
// The setup kernel rebuilds the planner's list and its inverse from it.
struct Axis {
	int ori, step, base, extra, last, n;
};

// The closed form of one of the planner's grid lists (make_plan, shared with
// bm4dof_run); false when the list is not of that form, so that the device
// copy can never differ from the planner's.
bool axis_of(const int *list, int n, int step, Axis &a)
{
	a.ori = n > 0 ? list[0] : 0;
	a.step = step;
	a.n = n;
	a.base = n;
	a.extra = 0;
	a.last = n > 0 ? list[n - 1] : 0;
	if (n >= 2 && (list[n - 1] - a.ori) % step != 0) {
		a.extra = 1;
		a.base = n - 1;
	}
	for (int i = 0; i < a.base; i++)
		if (list[i] != a.ori + i * step) return false;
	return !a.extra || list[n - 1] > list[n - 2];
}

// Writes the tile descriptor and the grid lists (with their inverse maps,
// the layout the search kernels read) into the scratch.
__global__ void setup_kernel(Tile T, Axis ax, Axis ay, Axis af, int F, Tile *tile_out, int *grid)
{
	if (blockIdx.x == 0 && threadIdx.x == 0) *tile_out = T;
	const Axis axes[3] = {ax, ay, af};
	const int offs[3] = {T.gx, T.gy, T.gf};
	const int ext[3] = {T.w, T.h, F};
	for (int k = 0; k < 3; k++) {
		const Axis a = axes[k];
		int *list = grid + offs[k];
		int *inv = list + a.n;
		for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += gridDim.x * blockDim.x)
			list[i] = i < a.base ? a.ori + i * a.step : a.last;
		for (int x = blockIdx.x * blockDim.x + threadIdx.x; x < ext[k]; x += gridDim.x * blockDim.x) {
			int v = -1;
			if (x >= a.ori && (x - a.ori) % a.step == 0 && (x - a.ori) / a.step < a.base) v = (x - a.ori) / a.step;
			else if (a.extra && x == a.last) v = a.n - 1;
			inv[x] = v;
		}
	}
}

// Neighbour lists in the reference's index format (index = t*w*h*C + y*w + x
// of the tile), the layout bm4dof_get_groups returns.
__global__ void export_kernel(Tile T, int C, int np, long long G, const int *grid, const uint8_t *nsimp,
                              const uint32_t *idx, unsigned *ref, unsigned *ns, unsigned *index, unsigned stride)
{
	const unsigned wh = (unsigned)T.w * T.h, whc = wh * C;
	for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < G; g += (long long)gridDim.x * blockDim.x) {
		const int x = grid[T.gx + (int)(g % T.nx)];
		const int y = grid[T.gy + (int)((g / T.nx) % T.ny)];
		const int t = grid[T.gf + (int)(g / ((long long)T.nx * T.ny))];
		ref[g] = (unsigned)t * whc + (unsigned)y * T.w + (unsigned)x;
		const int n = nsimp[g];
		ns[g] = (unsigned)n;
		for (unsigned q = 0; q < stride; q++) {
			unsigned v = 0;
			if ((int)q < n && (int)q < np) {
				const uint32_t lin = idx[g * np + q];
				v = (lin / wh) * whc + lin % wh;
			}
			index[(size_t)g * stride + q] = v;
		}
	}
}

bm4dof_status fail(bm4dof_status s, const std::string &msg)
{
	set_error(msg);
	return s;
}

}  // namespace

}  // namespace bm4dof

using namespace bm4dof;

extern "C" bm4dof_status bm4dof_search_groups_noalloc(const float *video, const float *fflow, const float *bflow,
                                                      unsigned W, unsigned H, unsigned C, unsigned F,
                                                      const bm4dof_params *p, unsigned nparts, unsigned tile,
                                                      unsigned *ref, unsigned *nsimp, unsigned *index,
                                                      unsigned stride, size_t cap, size_t *count, void *stream)
{
	clear_error();
	if (!video || !p || !count || W == 0 || H == 0 || F == 0 || !(C == 1 || C == 3 || C == 4))
		return fail(BM4DOF_ERR_ARGUMENT, "bm4dof_search_groups_noalloc: bad video or null argument");
	if ((fflow == nullptr) != (bflow == nullptr))
		return fail(BM4DOF_ERR_ARGUMENT, "bm4dof_search_groups_noalloc: give both flows or neither");
	const unsigned px = p->sizePatch, pt = p->sizePatchTime, np = p->nSimilarPatches;
	if (px == 0 || pt == 0 || p->offSet == 0 || p->offSetTime == 0 || np == 0 || np > (unsigned)kMaxNp ||
	    px * px * pt > (unsigned)kMaxSpc || p->sizeSearchWindow == 0 ||
	    p->sizeSearchTimeRangeFwd + p->sizeSearchTimeRangeBwd + 1 > (unsigned)kMaxFrames)
		return fail(BM4DOF_ERR_UNSUPPORTED, "bm4dof_search_groups_noalloc: unsupported parameters");
	if (nparts == 0) nparts = 2;

	int dev = 0;
	cudaError_t e = cudaGetDevice(&dev);
	if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices)
		return fail(BM4DOF_ERR_NO_DEVICE, "bm4dof_search_groups_noalloc: no current CUDA device");
	void *base = nullptr;
	{
		// once per device, with that device current: the device address of the
		// static scratch (its host-side name is not a device address)
		std::lock_guard<std::mutex> lock(g_mu);
		if (!g_scratch_addr[dev]) {
			e = cudaGetSymbolAddress(&g_scratch_addr[dev], g_search_scratch);
			if (e != cudaSuccess) {
				g_scratch_addr[dev] = nullptr;
				return fail(BM4DOF_ERR_CUDA, std::string("cudaGetSymbolAddress failed: ") + cudaGetErrorString(e));
			}
		}
		base = g_scratch_addr[dev];
	}

	// the tile (subDivideTight, lib_videot.hpp:853-916) and its grid
	// (processNlBayes, nldct.cpp:520-553), from the planner bm4dof_run uses
	Plan pl;
	make_plan(pl, W, H, F, nparts, *p, nullptr);
	if (tile >= pl.tiles.size()) return fail(BM4DOF_ERR_ARGUMENT, "bm4dof_search_groups_noalloc: tile out of range");
	Tile T = pl.tiles[tile];
	Axis ax, ay, af;
	if (!axis_of(&pl.grid[T.gx], T.nx, (int)p->offSet, ax) || !axis_of(&pl.grid[T.gy], T.ny, (int)p->offSet, ay) ||
	    !axis_of(&pl.grid[T.gf], T.nf, (int)p->offSetTime, af))
		return fail(BM4DOF_ERR_UNSUPPORTED, "bm4dof_search_groups_noalloc: reference grid without a closed form");
	T.gx = 0;
	T.gy = T.gx + T.nx + T.w;
	T.gf = T.gy + T.ny + T.h;
	T.g0 = 0;
	T.pix0 = 0;
	T.lin0 = 0;
	const int sWx = (int)p->sizeSearchWindow;
	const long long G = (long long)T.nx * T.ny * T.nf;
	*count = (size_t)G;

	StepParams sp = {};
	sp.px = (int)px;
	sp.pt = (int)pt;
	sp.spc = (int)(px * px * pt);
	sp.wx = sWx;
	sp.wtf = (int)p->sizeSearchTimeRangeFwd;
	sp.wtb = (int)p->sizeSearchTimeRangeBwd;
	sp.np = (int)np;
	sp.step1 = p->isFirstStep ? 1 : 0;
	sp.C = (int)C;
	sp.F = (int)F;
	sp.chn_search = p->isFirstStep ? 1 : (int)C;
	sp.sigma = p->sigma;
	sp.beta = p->beta;
	sp.tau2 = p->tau * p->tau * sp.px * sp.px * sp.pt;
	sp.use_flow = fflow != nullptr;
	const int nfm = search_frames_max(sp);

	// scratch layout; everything below is rewritten before it is read
	const size_t grid_ints = (size_t)T.nx + T.w + T.ny + T.h + T.nf + F;
	const size_t o_tile = 0;
	const size_t o_grid = o_tile + align256(sizeof(Tile));
	const size_t o_traj = o_grid + align256(grid_ints * sizeof(int));
	const size_t o_nsimp = o_traj + align256((size_t)G * nfm * sizeof(uint32_t));
	const size_t o_idx = o_nsimp + align256((size_t)G);
	const size_t need = o_idx + align256((size_t)G * np * sizeof(uint32_t));
	if (need > kScratchBytes)
		return fail(BM4DOF_ERR_ARGUMENT, "bm4dof_search_groups_noalloc: this tile needs " + std::to_string(need) +
		                                     " bytes of scratch; the static scratch holds " +
		                                     std::to_string(kScratchBytes) + " (" + std::to_string(G) + " groups)");
	// a size query (cap = 0) stops here: it launches nothing and leaves the
	// scratch alone
	if (cap == 0 || G == 0) return BM4DOF_OK;
	if (!ref || !nsimp || !index || stride == 0)
		return fail(BM4DOF_ERR_ARGUMENT, "bm4dof_search_groups_noalloc: null output array");

	unsigned char *s = static_cast<unsigned char *>(base);
	Tile *d_tile = reinterpret_cast<Tile *>(s + o_tile);
	int *d_grid = reinterpret_cast<int *>(s + o_grid);
	uint32_t *d_traj = reinterpret_cast<uint32_t *>(s + o_traj);
	uint8_t *d_nsimp = s + o_nsimp;
	uint32_t *d_idx = reinterpret_cast<uint32_t *>(s + o_idx);
	cudaStream_t st = static_cast<cudaStream_t>(stream);

	int nsm = 0;
	cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
	setup_kernel<<<8, 256, 0, st>>>(T, ax, ay, af, (int)F, d_tile, d_grid);
	Image src;
	src.p = const_cast<float *>(video);
	src.W = (int)W;
	src.H = (int)H;
	src.P = (int)W;                     // the caller's unpadded planar layout
	src.C = (int)C;
	src.F = (int)F;
	Image ff = src, bf = src;
	ff.C = bf.C = 2;
	ff.p = const_cast<float *>(fflow);
	bf.p = const_cast<float *>(bflow);
	if ((e = launch_traj(ff, bf, d_tile, 1, d_grid, sp, G, d_traj, st)) != cudaSuccess ||
	    (e = launch_search(src, d_tile, 1, d_grid, d_traj, sp, 0, G, d_nsimp, d_idx, nullptr, nsm, st)) != cudaSuccess)
		return fail(BM4DOF_ERR_CUDA, std::string("search launch: ") + cudaGetErrorString(e));
	const long long nout = std::min<long long>(G, (long long)cap);
	const long long b = std::min<long long>((nout + 255) / 256, 4096);
	export_kernel<<<(int)b, 256, 0, st>>>(T, (int)C, (int)np, nout, d_grid, d_nsimp, d_idx, ref, nsimp, index,
	                                      stride);
	if ((e = cudaGetLastError()) != cudaSuccess)
		return fail(BM4DOF_ERR_CUDA, std::string("export launch: ") + cudaGetErrorString(e));
	return BM4DOF_OK;
}
