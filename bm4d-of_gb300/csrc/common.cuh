// common.cuh -- device-side descriptors shared by the kernels and the runtime.
//
// Data layout in HBM (one context, one GPU):
//   * videos are planar like the reference's Video<float> (t, c, y, x) but
//     with a padded row pitch P (a multiple of 8 floats) so that every row
//     starts on a 32-byte boundary: value(x,y,t,c) = base[((t*C + c)*H + y)*P + x];
//   * the reference's spatial tiles (subDivideTight) are not copied: each tile
//     is a crop box (ox, oy, w, h) into the full-frame buffers; only its
//     aggregation buffers (w*h*F*C sums, w*h*F weights) are private;
//   * a "group" is one reference patch of one tile; groups are numbered in
//     the reference's processing order (tile, then t, y, x raster), which is
//     the order that fixes every floating-point sum downstream.
#pragma once

#include <cstdint>

namespace bm4dof {

constexpr int kMaxNp = 32;        // largest number of similar patches kept
constexpr int kMaxSpc = 64;       // largest patch size px*px*pt on the fast paths
constexpr int kMaxGatherPt = 16;  // largest sizePatchTime (a 64-element patch of px >= 2)
constexpr int kMaxFrames = 32;    // largest temporal search range (wtb+wtf+1)

struct Image {                    // one full-frame planar video on the device
	float *p;
	int W, H, P, C, F;
	__host__ __device__ size_t plane() const { return (size_t)P * H; }
	__host__ __device__ size_t at(int x, int y, int t, int c) const {
		return ((size_t)t * C + c) * plane() + (size_t)y * P + x;
	}
};

struct Tile {                     // one spatial tile (crop) of one step
	int ox, oy, w, h;             // crop box in the full frame
	int nx, ny, nf;               // reference grid sizes along x, y, t
	int gx, gy, gf;               // offsets of the grid coordinate lists
	long long g0;                 // first group id of this tile
	long long pix0;               // first pixel of this tile's aggregation buffers
	unsigned long long lin0;      // first origin-list slot (== pix0)
	int bx0, by0, bx1, by1;       // crop touches an inner border (nldct.cpp:520-525)
};

struct StepParams {               // resolved parameters of one step
	int px, pt, spc;              // patch size, sPC = px*px*pt
	int wx, wtf, wtb;             // search window and temporal range
	int np;                       // nSimilarPatches
	int step1;                    // 1: hard threshold, 2: Wiener
	int C, F;                     // channels, frames
	int chn_search;               // channels compared by the distance
	float sigma, beta, tau2;      // tau2 = tau*tau*px*px*pt (nldct.cpp:1158)
	int use_flow;
	float beta1;                  // learned form: hard threshold of the non-mean Haar rows
	int search_ctas;              // exact search: CTAs per SM (4 or 6; 0 = default)
	int search_strip;             // exact search: candidates per thread along a column (7 or 21; 0 = default)
	int gather_depth;             // quad gather: members in flight per thread (1 or 2; 0 = 1)
	float beta_mean;              // betaMean (order-invariant filtering)
	int order_inv;                // orderInvariance
	int vbm3d;                    // predictive search (the reference's VBM3D_SEARCH build)
	int wxp, npf;                 // sizeSearchWindowPred, nSimilarPatchesPred
	float dsub_bias;              // dsub*dsub*255 (nldct.cpp:921)
	int paste;                    // doPasteBoost
};

// Aggregation terms of a chunk of groups: for slot s (one member of one
// group) and patch element p, the C weighted estimates (w * window[p]) * ghat
// followed by the weight term w * window[p], so that the ordered gather reads
// one aligned vector per term:  vals[(s * spc + p) * term_stride(C) + c],
// c = 0..C (c = C: the weight term).
__host__ __device__ __forceinline__ int term_stride(int C) { return C == 1 ? 2 : (C <= 3 ? 4 : 8); }

// Locate the tile owning global group g (tiles are few: linear scan).
__device__ __forceinline__ int tile_of(const Tile *tiles, int ntiles, long long g)
{
	int t = 0;
	while (t + 1 < ntiles && tiles[t + 1].g0 <= g) t++;
	return t;
}

}  // namespace bm4dof
