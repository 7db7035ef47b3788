// internal.hpp -- declarations shared by the host runtime and the kernel files.
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "common.cuh"
#include "../../include/bm4dof.h"

namespace bm4dof {

void set_error(const std::string &msg);
void clear_error();

// Dense patch bases, stored basis[k*spc + p] like the reference's
// mat.patch_basis / mat.patch_basis_inv (src/core/nldct.cpp:572-696).
bool make_basis(int transform, unsigned px, unsigned pt, std::vector<float> &basis,
                std::vector<float> &binv);
// Aggregation window (src/core/nldct.cpp:698-737).
std::vector<float> make_window(bool agg, unsigned px, unsigned pt);

// Tiles of a run (subDivideTight, lib_videot.hpp:853-916) and the reference
// grid of each (processNlBayes, nldct.cpp:520-553); runtime.cu.
struct Plan {
	int nW, nH, wTmp, hTmp;
	std::vector<Tile> tiles;
	std::vector<int> grid;     // per tile: [xs | inverse x] [ys | inverse y] [fs | inverse t]
	long long G = 0;
	size_t pix = 0;            // total tile pixels (one channel)
	size_t maxpos = 0;         // largest tile pixel count
};
void determine_factor(unsigned n, unsigned &a, unsigned &b);
// borders: null for the tiles of a run, else the six sides {x0, y0, t0, x1,
// y1, t1} of one crop (bm4dof_process) that stop short of its source.
void make_plan(Plan &pl, unsigned W, unsigned H, unsigned F, unsigned nparts, const bm4dof_params &p,
               const int *borders);

// search.cu
int search_frames_max(const StepParams &sp);
cudaError_t launch_traj(const Image &ffl, const Image &bfl, const Tile *tiles, int ntiles, const int *grid,
                        const StepParams &sp, long long G, uint32_t *traj, cudaStream_t st);
// With glist, the groups glist[0 .. *gcount) (a device-side count, at most
// g_end - g_begin of them) instead of the range [g_begin, g_end).
cudaError_t launch_search(const Image &src, const Tile *tiles, int ntiles, const int *grid,
                          const uint32_t *traj, const StepParams &sp, long long g_begin, long long g_end,
                          uint8_t *nsimp, uint32_t *idx, int *err, int nsm, cudaStream_t st,
                          const uint32_t *glist = nullptr, const unsigned *gcount = nullptr);

// search_vbm3d.cu (the reference's VBM3D_SEARCH build)
bool vbm3d_check(const StepParams &sp, const std::vector<Tile> &tiles, std::string &why);
size_t vbm3d_smem_bytes(const StepParams &sp, int reps);
cudaError_t launch_search_vbm3d(const Image &src, const Image &ffl, const Image &bfl, const Tile *tiles,
                                int ntiles, const int *grid, const StepParams &sp, int reps, long long g_begin,
                                long long g_end, uint8_t *nsimp, uint32_t *idx, int nsm, cudaStream_t st);

// search_tc.cu: tensor-core pre-screen + certified exact re-rank; the groups
// it cannot certify are listed for launch_search (list mode)
void tc_blocks(const std::vector<Tile> &tiles, std::vector<long long> &out);
bool tc_supported(const StepParams &sp, const std::vector<Tile> &tiles);
size_t tc_smem_bytes();
cudaError_t launch_search_tc(const Image &src, const Tile *tiles, int ntiles, const int *grid, const uint32_t *traj,
                             const StepParams &sp, const long long *blocks, long long nblocks, long long G,
                             uint32_t *cand, float *lb, float *thr0, int *status, uint8_t *nsimp, uint32_t *idx,
                             uint32_t *fallback, unsigned *nfallback, unsigned *nuncertified, int certified, int nsm,
                             cudaStream_t st);
cudaError_t tc_selftest(const uint16_t *A, const uint16_t *B, float *D, int *status, cudaStream_t st);

// filter.cu
size_t filter_smem_bytes(const StepParams &sp);
cudaError_t launch_filter(const Image &noisy, const Image &basic, const Tile *tiles, int ntiles,
                          const StepParams &sp, const float *basis, const float *binv,
                          const float *win, long long g_begin, long long g_end,
                          const uint8_t *nsimp, const uint32_t *idx, const uint8_t *alive,
                          float *vals, float *wgroup, uint8_t *eq, int nsm,
                          cudaStream_t st);

// aggregate.cu
cudaError_t launch_kill_edges(const Tile *tiles, int ntiles, const int *grid, const int *inv,
                              const StepParams &sp, long long G, const uint32_t *idx,
                              unsigned long long *edges, unsigned *nedges, unsigned cap,
                              cudaStream_t st);
// Switch-offs resolved on the device in one launch (no host round trip).
cudaError_t launch_kill_fixpoint(const unsigned long long *edges, const unsigned *nedges, unsigned cap,
                                 uint8_t *alive, uint8_t *killed, cudaStream_t st);
// Paste trick (doPasteBoost): the processed groups, settled by frontier
// rounds (kPasteRounds over the whole GPU, the rest in one CTA).
constexpr int kPasteRounds = 24;
struct PasteScratch {
	unsigned *pending, *state;   // G each
	uint32_t *q0, *q1;           // G each
	unsigned *counts;            // kPasteRounds + 3
};
cudaError_t launch_paste_resolve(const Tile *tiles, int ntiles, const int *grid, const StepParams &sp, long long G,
                                 const uint8_t *nsimp, const uint32_t *idx, PasteScratch w, uint8_t *alive, int nsm,
                                 cudaStream_t st);
cudaError_t launch_count_alive(const Tile *tiles, int ntiles, long long G, const uint8_t *alive,
                               unsigned *counts, cudaStream_t st);
cudaError_t exclusive_scan(unsigned *data, size_t n, unsigned *scratch, cudaStream_t st);
unsigned scan_kernels(size_t n);
// launch_lists and launch_gather add the kernels they launch to *launches
cudaError_t launch_lists(long long ga, long long gb, int np, const uint8_t *nsimp,
                         const uint32_t *idx, const uint8_t *alive, size_t npos, unsigned *cnt,
                         unsigned *off, unsigned *list, unsigned *scratch, unsigned *launches, cudaStream_t st);
// Ordered gather of the slots whose origins lie in frames [t_lo, t_hi].  4x4
// patches (quad_path): row lists (offsets in cnt) and quad lists (offsets in
// soff), both in sl, then a merge over origin frames per quad of 4 pixels;
// other patches: spatial lists (soff), then a merge per pixel.  cnt and soff
// hold npos+1 entries, sl list_entries_per_member(sp) entries per slot of a
// chunk of `members` slots.
bool quad_path(const StepParams &sp);
int list_entries_per_member(const StepParams &sp);
cudaError_t launch_gather(const Tile &T, const StepParams &sp, int t_lo, int t_hi,
                          const unsigned *off, const unsigned *list, unsigned *cnt, unsigned *soff, unsigned *sl,
                          size_t members, unsigned *scratch, const float *vals, float *acc, float *wacc,
                          unsigned *launches, cudaStream_t st);
cudaError_t launch_color(const Image &in, const Image &out, int forward, cudaStream_t st);
cudaError_t launch_finalize(const Tile *tiles, int nW, int wTmp, int hTmp, const StepParams &sp,
                            const Image &noisy, const float *acc, const float *wacc,
                            const Image &out, int inverse_color, cudaStream_t st);

// mlp.cu -- gain network 65 -> 256 -> 256 -> 64 (W1 padded to 80 inputs)
constexpr int kMlpIn = 65, kMlpInPad = 80, kMlpHid = 256, kMlpOutN = 64;
constexpr int kMlpOffW1 = 0, kMlpOffB1 = kMlpInPad * kMlpHid, kMlpOffW2 = kMlpOffB1 + kMlpHid,
              kMlpOffB2 = kMlpOffW2 + kMlpHid * kMlpHid, kMlpOffW3 = kMlpOffB2 + kMlpHid,
              kMlpOffB3 = kMlpOffW3 + kMlpHid * kMlpOutN, kMlpMasterSize = kMlpOffB3 + kMlpOutN;
constexpr int kMlpPublicSize = kMlpMasterSize - (kMlpInPad - kMlpIn) * kMlpHid;
constexpr int kMlpWtSize = kMlpHid * kMlpInPad + kMlpHid * kMlpHid + kMlpOutN * kMlpHid;
struct MlpWeights {
	const __nv_bfloat16 *wt1, *wt2, *wt3;   // transposed [out][in]
	const float *b1, *b2, *b3;
};
MlpWeights mlp_weights(const uint16_t *wt, const float *master);
void mlp_public_to_master(const float *pub, float *master);
void mlp_master_to_public(const float *master, float *pub);
cudaError_t launch_pack_weights(const float *master, uint16_t *wt, cudaStream_t st);
cudaError_t launch_mlp_forward(const uint16_t *X, long long n, const MlpWeights &w, float *out, int nsm,
                               cudaStream_t st);

// learned.cu
enum { kLearnedFeatures = 0, kLearnedApply = 1, kLearnedSamples = 2 };
struct LearnedArgs {
	Image noisy, basic;
	const Tile *tiles;
	int ntiles;
	long long ga, gb;                    // group range (rows are g - ga)
	const uint8_t *nsimp, *alive;
	const uint32_t *idx;
	const float *basis, *binv, *win;
	__nv_bfloat16 *feat;                 // features: [rows][80]
	const float *gains;                  // apply: [rows][64], or null (no network)
	float *vals;                         // apply: aggregation terms (estimate, weight term)
	float kappa;                         // apply: residual-variance fallback threshold
	unsigned *nfallback;
	float *sfeat, *starget;              // samples: [G][65], [G][64]
	uint8_t *svalid;                     // samples: [G]
};
bool learned_supported(const StepParams &sp);
cudaError_t launch_learned(int mode, const LearnedArgs &a, const StepParams &sp, int nsm, cudaStream_t st);

// tvl1.cu -- TV-L1 optical flow, batched over frame pairs
struct Tvl1Params {
	float tau, lambda, theta;
	int nscales, fscale;
	float zfactor;
	int warps;
	float epsilon;
};
int tvl1_scales(int nx, int ny, int nscales, float zfactor);
size_t tvl1_workspace_floats(int nx, int ny, int npairs, int nscales, float zfactor);
cudaError_t tvl1_flow(const float *I0, const float *I1, int nx, int ny, int npairs, const Tvl1Params &p, float *u,
                      float *v, float *ws, int *iws, int nsm, cudaStream_t st, std::string &why);

}  // namespace bm4dof
