// internal.hpp -- declarations shared by the host runtime and the kernel files.
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "common.cuh"

namespace bm4dof {

void set_error(const std::string &msg);
void clear_error();

// Dense patch bases, stored basis[k*spc + p] like the reference's
// mat.patch_basis / mat.patch_basis_inv (src/core/nldct.cpp:572-696).
bool make_basis(int transform, unsigned px, unsigned pt, std::vector<float> &basis,
                std::vector<float> &binv);
// Aggregation window (src/core/nldct.cpp:698-737).
std::vector<float> make_window(bool agg, unsigned px, unsigned pt);

// search.cu
int search_frames_max(const StepParams &sp);
cudaError_t launch_traj(const Image &ffl, const Image &bfl, const Tile *tiles, int ntiles, const int *grid,
                        const StepParams &sp, long long G, uint32_t *traj, cudaStream_t st);
cudaError_t launch_search(const Image &src, const Tile *tiles, int ntiles, const int *grid,
                          const uint32_t *traj, const StepParams &sp, long long g_begin, long long g_end,
                          uint8_t *nsimp, uint32_t *idx, int *err, int nsm, cudaStream_t st);

// search_mixed.cu
void mixed_blocks(const std::vector<Tile> &tiles, std::vector<long long> &out);
bool mixed_supported(const StepParams &sp);
cudaError_t launch_search_mixed(const Image &src, const Tile *tiles, int ntiles, const int *grid,
                                const uint32_t *traj, const StepParams &sp, const long long *blocks,
                                long long nblocks, uint8_t *nsimp, uint32_t *idx, int nsm, cudaStream_t st);

// filter.cu
size_t filter_smem_bytes(const StepParams &sp);
cudaError_t launch_filter(const Image &noisy, const Image &basic, const Tile *tiles, int ntiles,
                          const StepParams &sp, const float *basis, const float *binv,
                          const float *win, long long g_begin, long long g_end,
                          const uint8_t *nsimp, const uint32_t *idx, const uint8_t *alive,
                          float *vals, float *wslot, float *wgroup, uint8_t *eq, int nsm,
                          cudaStream_t st);

// aggregate.cu
cudaError_t launch_kill_edges(const Tile *tiles, int ntiles, const int *grid, const int *inv,
                              const StepParams &sp, long long G, const uint32_t *idx,
                              unsigned long long *edges, unsigned *nedges, unsigned cap,
                              cudaStream_t st);
cudaError_t launch_kill_iteration(const unsigned long long *edges, unsigned n, uint8_t *alive,
                                  uint8_t *killed, unsigned *changed, cudaStream_t st);
cudaError_t launch_count_alive(const Tile *tiles, int ntiles, long long G, const uint8_t *alive,
                               unsigned *counts, cudaStream_t st);
cudaError_t exclusive_scan(unsigned *data, size_t n, unsigned *scratch, cudaStream_t st);
cudaError_t launch_lists(long long ga, long long gb, int np, const uint8_t *nsimp,
                         const uint32_t *idx, const uint8_t *alive, size_t npos, unsigned *cnt,
                         unsigned *off, unsigned *list, unsigned *scratch, cudaStream_t st);
// Ordered gather of the slots whose origins lie in frames [t_lo, t_hi]:
// spatial lists (soff: npos+1 entries, sl: px*px entries per slot), then the
// per-pixel merge over origin frames.
cudaError_t launch_gather(const Tile &T, const StepParams &sp, int t_lo, int t_hi,
                          const unsigned *off, const unsigned *list, unsigned *soff, unsigned *sl,
                          unsigned *scratch, const float *vals, const float *wslot, const float *win,
                          float *acc, float *wacc, cudaStream_t st);
cudaError_t launch_color(const Image &in, const Image &out, int forward, cudaStream_t st);
cudaError_t launch_finalize(const Tile *tiles, int nW, int wTmp, int hTmp, const StepParams &sp,
                            const Image &noisy, const float *acc, const float *wacc,
                            const Image &out, int inverse_color, cudaStream_t st);

}  // namespace bm4dof
