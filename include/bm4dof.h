/*
 * bm4dof.h -- C ABI of the GB300 (sm_103a) BM4D-OF / NL-DCT video denoising path.
 *
 * The entry points mirror the reference's C++ interface in namespace VideoNLB
 * (src/core/nldct.h).  Each declaration names the reference function it stands
 * in for.  Plain pointers and sizes only: no C++ or torch types cross this
 * boundary, so the library can be bound from C, ctypes or any FFI.
 *
 * Video layout (the reference's Video<float>, src/utils/lib_videot.hpp:88-92):
 *   planar, value(x, y, t, c) = data[t*W*H*C + c*W*H + y*W + x].
 * Optical flow uses the same layout with C = 2 (channel 0 = x displacement,
 * channel 1 = y displacement).
 *
 * Errors: every call that can fail returns a bm4dof_status; the message of the
 * last failure on the calling thread is available from bm4dof_last_error().
 * The messages of the reference's std::runtime_error throws are kept verbatim
 * (src/core/nldct.cpp:279,289,296,334,341,634).
 */
#ifndef BM4DOF_H_INCLUDED
#define BM4DOF_H_INCLUDED

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum bm4dof_status {
	BM4DOF_OK = 0,
	BM4DOF_ERR_ARGUMENT = 1,      /* null pointer, zero size, bad flag            */
	BM4DOF_ERR_CHANNELS = 2,      /* nldct.cpp:279  channels not 1, 3 or 4         */
	BM4DOF_ERR_FWD_FLOW = 3,      /* nldct.cpp:289  forward flow size mismatch     */
	BM4DOF_ERR_BWD_FLOW = 4,      /* nldct.cpp:296  backward flow size mismatch    */
	BM4DOF_ERR_NO_STEP = 5,       /* nldct.cpp:334  both patch sizes are zero      */
	BM4DOF_ERR_BASIC_SIZE = 6,    /* nldct.cpp:341  basic size differs from noisy  */
	BM4DOF_ERR_BIOR_SIZE = 7,     /* nldct.cpp:634  bior1.5 with patch size != 8   */
	BM4DOF_ERR_UNSUPPORTED = 8,   /* parameter combination the library rejects     */
	BM4DOF_ERR_CUDA = 9,          /* CUDA runtime error (message has the details)  */
	BM4DOF_ERR_NO_MEMORY = 10,    /* device or host allocation failed              */
	BM4DOF_ERR_TIMEOUT = 11,      /* a bounded device-side wait ran out            */
	BM4DOF_ERR_NO_DEVICE = 12     /* no usable CUDA device                          */
} bm4dof_status;

typedef enum bm4dof_color_space { BM4DOF_RGB = 0, BM4DOF_YUV = 1 } bm4dof_color_space;
typedef enum bm4dof_transform  { BM4DOF_DCT = 0, BM4DOF_BIOR1_5 = 1 } bm4dof_transform;

/* Mirror of VideoNLB::nlbParams (src/core/nldct.h:55-82), field for field. */
typedef struct bm4dof_params {
	float    sigma;
	unsigned sizePatch;
	unsigned sizePatchTime;
	unsigned nSimilarPatches;
	unsigned sizeSearchWindow;
	unsigned sizeSearchTimeRangeFwd;
	unsigned sizeSearchTimeRangeBwd;
	unsigned boundary;
	unsigned offSet;
	unsigned offSetTime;
	float    beta;
	float    betaMean;
	float    tau;
	int      orderInvariance;
	int      isFirstStep;
	int      doPasteBoost;
	int      verbose;
	int      colorSpace;            /* bm4dof_color_space */
	int      transform;             /* bm4dof_transform   */
	unsigned sizeSearchWindowPred;
	unsigned nSimilarPatchesPred;
	float    dsub;
	int      agg_window;
} bm4dof_params;

/* Mirror of VideoSize (src/utils/lib_videot.hpp:40-51): the four sizes. */
typedef struct bm4dof_video_size {
	unsigned width;
	unsigned height;
	unsigned frames;
	unsigned channels;
} bm4dof_video_size;

/* ---- parameter resolution (host only, no device needed) ------------------ */

/* VideoNLB::initializeNlbParameters, src/core/nldct.cpp:81-148.
 * betaMean is set to beta here; the reference leaves it uninitialised unless
 * -b1/-bm1 is given (it is read only by the order-invariant filter). */
void bm4dof_initialize_params(bm4dof_params *params, unsigned step, float sigma,
                              const bm4dof_video_size *size, int verbose);

/* VideoNLB::setSizeSearchWindow, src/core/nldct.cpp:160-168. */
void bm4dof_set_size_search_window(bm4dof_params *params, unsigned sizeSearchWindow);

/* VideoNLB::setSizePatch, src/core/nldct.cpp:179-188. */
void bm4dof_set_size_patch(bm4dof_params *params, const bm4dof_video_size *size,
                           unsigned sizePatch);

/* VideoNLB::setNSimilarPatches, src/core/nldct.cpp:199-210. */
void bm4dof_set_n_similar_patches(bm4dof_params *params, unsigned nSimilarPatches);

/* VideoNLB::printNlbParameters, src/core/nldct.cpp:219-249: writes the same
 * text into buf (NUL-terminated, truncated to len) and returns its length. */
int bm4dof_format_params(const bm4dof_params *params, char *buf, size_t len);

/* VideoNLB::printNlbParameters to stdout. */
void bm4dof_print_params(const bm4dof_params *params);

/* Message of the last failed call on this thread ("" if none). */
const char *bm4dof_last_error(void);

/* Library version string. */
const char *bm4dof_version(void);

/* ---- device context ------------------------------------------------------ */

typedef struct bm4dof_ctx bm4dof_ctx;

/* Creates a context bound to one CUDA device with its own stream.  Calls on one
 * context are serialised; distinct contexts may run concurrently. */
bm4dof_status bm4dof_create(bm4dof_ctx **ctx, int device);
void          bm4dof_destroy(bm4dof_ctx *ctx);

/* The context's stream (a cudaStream_t, created non-blocking): every call on
 * the context runs its device work there.  Device inputs written by work on
 * another stream must be ordered before the call by the caller (an event
 * recorded on its stream and cudaStreamWaitEvent on this one), and work of
 * the caller's stream that reads the outputs or reuses the inputs' memory
 * after it (the reverse wait). */
bm4dof_status bm4dof_get_stream(bm4dof_ctx *ctx, void **stream);

/* Caps the device memory the context's buffers may hold (0: no cap, the
 * default).  A call that would need more fails with BM4DOF_ERR_NO_MEMORY and
 * a message naming the buffer; the context stays usable.  The chunk budget of
 * the aggregation terms shrinks with the cap.  Applies to the calls made on
 * this context (not to the private contexts of bm4dof_run_batched). */
bm4dof_status bm4dof_set_memory_limit(bm4dof_ctx *ctx, size_t bytes);

/* Flags for bm4dof_run. */
#define BM4DOF_DEVICE_POINTERS  0x1u  /* all video pointers are device pointers  */
#define BM4DOF_KEEP_GROUPS      0x2u  /* record neighbour lists for inspection   */
/* The patch search as a tensor-core pre-screen (tcgen05, FP16 patches, FP32
 * accumulation) of the 32 best candidates per group, then their exact FP32
 * distances, certified against a bound on every dropped candidate; the group
 * filter stays FP32.  A certified group's neighbour list is the exact path's;
 * see bm4dof_mixed_stats and BM4DOF_MIXED_CERTIFIED. */
#define BM4DOF_MIXED_PRECISION  0x4u
#define BM4DOF_LEARNED          0x8u  /* learned form: no step-1 pass (see below)  */
/* The predictive patch search of the reference built with -DVBM3D_SEARCH
 * (src/core/nldct.cpp:892-1130, 1351-1589) instead of the exhaustive one:
 * the full sizeSearchWindow window in the reference frame only; in every other
 * frame nSimilarPatchesPred windows of sizeSearchWindowPred, one around each
 * of the previous frame's nSimilarPatchesPred best matches moved along the
 * flow; distances on channel 0 (in step 2 summed once per channel, as the
 * reference does), minus dsub^2*255 at the reference position of every frame;
 * the best nSimilarPatchesPred of each frame pooled, the best nSimilarPatches
 * of the pool kept.  Exact: the same neighbours as that build.  Plain FP32
 * path only (not with BM4DOF_MIXED_PRECISION or BM4DOF_LEARNED). */
#define BM4DOF_VBM3D_SEARCH     0x10u
/* BM4DOF_MIXED_PRECISION whose patch search returns the exact path's
 * neighbour lists: every group whose tensor-core pre-screen cannot be
 * certified (near-equal candidates) gets the exact search.  Implies
 * BM4DOF_MIXED_PRECISION. */
#define BM4DOF_MIXED_CERTIFIED  0x20u

/* VideoNLB::runNlBayes, src/core/nldct.cpp:267-478.
 *
 *  noisy        W*H*C*F floats.
 *  fflow,bflow  W*H*2*F floats each, or both NULL for no flow (the reference's
 *               empty Video, nldct.cpp:283).
 *  basic        W*H*C*F floats: output of step 1, or input when
 *               params1->sizePatch == 0 (step 2 only, nldct.cpp:329-342).
 *  final        W*H*C*F floats: output of step 2 (untouched when
 *               params2->sizePatch == 0).
 *  nparts       number of spatial tiles; the reference uses
 *               2*omp_get_max_threads() (nldct.cpp:318-323).  0 means 2.
 *  ratios       out: percentage of processed groups per step (the reference's
 *               return value).  May be NULL.
 */
bm4dof_status bm4dof_run(bm4dof_ctx *ctx,
                         const float *noisy, const float *fflow, const float *bflow,
                         unsigned width, unsigned height, unsigned channels, unsigned frames,
                         float *basic, float *final_,
                         const bm4dof_params *params1, const bm4dof_params *params2,
                         unsigned nparts, unsigned flags, float ratios[2]);

/* The fields of VideoUtils::CropPosition (src/utils/lib_videot.hpp:440-470)
 * that processNlBayes reads: where the processed video was cut from its
 * source.  All zero (the reference's default CropPosition()) means no border. */
typedef struct bm4dof_crop {
	int origin_x, origin_y, origin_t;   /* first column, row and frame of the crop */
	int ending_x, ending_y, ending_t;   /* one past the last                       */
	bm4dof_video_size source_sz;        /* size of the video it was cut from       */
} bm4dof_crop;

/* VideoNLB::processNlBayes, src/core/nldct.cpp:490-890: one step
 * (params->isFirstStep) over one video, typically a tile cut from a larger
 * one, with no tiling and no colour transform of its own.  Reference patches
 * are taken on the grid of nldct.cpp:520-553: on a side where the crop does
 * not reach the source's edge (origin > 0, or ending < the source size), the
 * grid keeps sizePatch-1 + sizeSearchWindow/2 pixels (sizePatchTime-1 +
 * (range)/2 frames) away from it.  Step 1 writes basic, step 2 reads basic and
 * writes final; both aggregate over the whole video (pixels no patch covers
 * are divided by the noisy value, as nldct.cpp:2436-2448 does).
 *  crop    NULL for no border.
 *  groups  out: the number of processed groups (the reference's return value).
 * Flags as bm4dof_run; BM4DOF_LEARNED is rejected (it needs both steps). */
bm4dof_status bm4dof_process(bm4dof_ctx *ctx,
                             const float *noisy, const float *fflow, const float *bflow,
                             unsigned width, unsigned height, unsigned channels, unsigned frames,
                             float *basic, float *final_, const bm4dof_params *params,
                             const bm4dof_crop *crop, unsigned flags, unsigned *groups);

/* The reference-patch grid (host only, no device): the tiles bm4dof_run makes
 * for nparts (process = 0; subDivideTight, lib_videot.hpp:853-916), or the one
 * tile of bm4dof_process with crop (process = 1), and in each the reference
 * patches' positions of nldct.cpp:520-553.  tiles receives 7 ints per tile
 * {ox, oy, w, h, nx, ny, nf} (at most tiles_cap tiles), coords each tile's nx
 * x positions, ny y positions and nf frames in turn (at most coords_cap ints,
 * tile-local); *ntiles and *ncoords receive the full counts.  A tile's groups
 * are all (x, y, t) of its lists. */
bm4dof_status bm4dof_plan(unsigned width, unsigned height, unsigned frames, unsigned nparts,
                          const bm4dof_params *params, const bm4dof_crop *crop, int process, int *tiles,
                          unsigned tiles_cap, int *coords, size_t coords_cap, unsigned *ntiles, size_t *ncoords);

/* Neighbour lists of the last bm4dof_run made with BM4DOF_KEEP_GROUPS, for one
 * step (1 or 2) and tile.  For each processed group in processing order:
 *   ref[g]          reference patch index (tile video index at channel 0, as
 *                   the reference's ij3 = sz.index(px,py,pt,0), nldct.cpp:765),
 *   nsimp[g]        number of similar patches kept (nldct.cpp:1284-1289),
 *   index[g*stride + n]  the reference's index[n] (nldct.cpp:1300-1301).
 * Writes at most cap groups and returns the total count in *count. */
bm4dof_status bm4dof_get_groups(bm4dof_ctx *ctx, unsigned step, unsigned tile,
                                unsigned *ref, unsigned *nsimp, unsigned *index,
                                unsigned stride, size_t cap, size_t *count);

/* Patch search of one tile with no device allocation.  No counterpart in the
 * reference: it exists for callers that cannot call cudaMalloc (code inside
 * another framework's memory pool, plug-in hosts that own every device
 * buffer, pipelines that forbid allocation once running).  The caller passes
 * device pointers for the video to search (the noisy video for step 1, the
 * basic estimate for step 2; already colour transformed when C > 1), the
 * flows (both or neither) and the outputs; all working memory is one static
 * device array of 32 MiB per device, held for the life of the process.
 * Returns BM4DOF_ERR_ARGUMENT with the needed size when a tile does not fit.
 * Outputs, in processing order, for every grid group of tile `tile` of
 * `nparts` tiles: ref[g], nsimp[g] and index[g*stride + n] in the format of
 * bm4dof_get_groups (at most cap groups are written; *count = total).  The
 * tiles and grids are those of bm4dof_run.  Unlike bm4dof_get_groups, every
 * grid group is returned: the mask switch-offs of bm4dof_run are not applied
 * (a group that bm4dof_run skips still appears here), and the search is the
 * reference's default (exhaustive) one.  A size query (cap = 0) only sets
 * *count: it launches nothing and does not touch the scratch.  The first call
 * on a device
 * looks up the scratch's device address, so make it before any stream
 * capture.  Asynchronous on `stream` (a cudaStream_t, NULL for the default
 * stream); calls that overlap on the GPU share the scratch and race. */
bm4dof_status bm4dof_search_groups_noalloc(const float *video, const float *fflow, const float *bflow,
                                           unsigned width, unsigned height, unsigned channels, unsigned frames,
                                           const bm4dof_params *params, unsigned nparts, unsigned tile,
                                           unsigned *ref, unsigned *nsimp, unsigned *index, unsigned stride,
                                           size_t cap, size_t *count, void *stream);

/* Device times (milliseconds, CUDA events on the context's stream) of the
 * last bm4dof_run: ms[0] patch search, ms[1] group filter, ms[2] aggregation,
 * ms[3] everything else (copies, colour, normalisation), ms[4] the whole call
 * from its first to its last event; and the number of kernel launches. */
bm4dof_status bm4dof_last_timings(bm4dof_ctx *ctx, float ms[5], unsigned *launches);

/* ---- batched runs ----------------------------------------------------------
 * No counterpart in the reference (its caller runs one video per process).
 * Many sequences of uneven size, frame count and sigma denoised by one CUDA
 * graph: each sequence's whole runNlBayes (both steps) is recorded on one of
 * `branches` streams, the branches are joined into a single graph, and the
 * graph is launched once.  A call with the same sequences, pointers, flags and
 * tuning as the previous one replays the instantiated graph. */

/* One sequence of a batched run.  All video pointers are device pointers. */
typedef struct bm4dof_sequence {
	const float *noisy, *fflow, *bflow;    /* flows: both or neither          */
	unsigned width, height, channels, frames;
	float *basic, *final_;
	bm4dof_params params1, params2;
	unsigned nparts;                       /* 0 means 2                       */
	float ratios[2];                       /* out, as bm4dof_run              */
} bm4dof_sequence;

/* Launch shape of a batched run (bm4dof_autotune chooses one). */
typedef struct bm4dof_tuning {
	unsigned branches;     /* concurrent streams in the graph; 0: min(n, 16)     */
	unsigned slot_mb;      /* per sequence: MB of aggregation terms per chunk
	                          (the depth of group staging); 0: 1024              */
	unsigned search_ctas;  /* exact search CTAs per SM: 4 or 6; 0: 6             */
	unsigned search_strip; /* exact search candidates per thread along a window
	                          column: 7 or 21; 0: 21 for windows of 15 rows or
	                          more (4x4x4 patches at 6 CTAs per SM; at 4 CTAs
	                          per SM and for other patches the strip is 7)      */
	unsigned gather_depth; /* members in flight per thread of the ordered
	                          gather (4x4 patches): 1 or 2; 0: 1                */
} bm4dof_tuning;

/* Denoises n sequences (flags: BM4DOF_MIXED_PRECISION, BM4DOF_LEARNED,
 * BM4DOF_VBM3D_SEARCH; the pointers are always device pointers).  tuning may
 * be NULL (defaults).  Each sequence's chunk budget is capped so that all the
 * sequences' buffers fit in half the device memory.  bm4dof_last_timings
 * reports the graph launch as ms[4]. */
bm4dof_status bm4dof_run_batched(bm4dof_ctx *ctx, bm4dof_sequence *seqs, unsigned n, unsigned flags,
                                 const bm4dof_tuning *tuning);

/* Times candidate tunings (graph replays of the first `sample` sequences,
 * coordinate descent over branches, slot_mb, search_ctas, search_strip and
 * gather_depth) and returns the fastest in *best.  table (may be NULL)
 * receives up to cap rows of {branches, slot_mb, search_ctas, search_strip,
 * gather_depth, milliseconds} as floats; *rows = count. */
bm4dof_status bm4dof_autotune(bm4dof_ctx *ctx, bm4dof_sequence *seqs, unsigned n, unsigned sample,
                              unsigned flags, bm4dof_tuning *best, float *table, unsigned cap, unsigned *rows);

/* ---- optical flow ------------------------------------------------------------
 * TV-L1 flow (Zach, Pock and Bischof's dual method), the step the reference
 * runs before the denoiser: lib/tvl1flow (Dual_TVL1_optic_flow_multiscale,
 * tvl1flow_lib.c:344-474) as driven by scripts/tvl1flow-seq.sh. */
typedef struct bm4dof_tvl1_params {
	float tau, lambda, theta;   /* time step, data weight, coupling weight      */
	int   nscales, fscale;      /* pyramid levels (capped as main.c:147-153 does),
	                               finest level computed                        */
	float zfactor;              /* pyramid factor                                */
	int   warps;                /* warpings per level                            */
	float epsilon;              /* stopping threshold                            */
} bm4dof_tvl1_params;

/* The values scripts/tvl1flow-seq.sh passes: 0.25 0.2 0.3 100 1 0.5 5 0.01. */
void bm4dof_tvl1_default_params(bm4dof_tvl1_params *p);

/* Flow of npairs grey frame pairs I0[k] -> I1[k] (each width x height,
 * [pair][y][x]) into uv[k] = (u plane, v plane) ([pair][2][y][x]), as
 * tvl1flow writes it for I0 = the first image.  Pointers follow flags
 * (BM4DOF_DEVICE_POINTERS). */
bm4dof_status bm4dof_tvl1_pairs(bm4dof_ctx *ctx, const float *I0, const float *I1, unsigned width,
                                unsigned height, unsigned npairs, const bm4dof_tvl1_params *params,
                                float *uv, unsigned flags);

/* Forward and backward flows of a grey video ([frame][y][x]) in the layout
 * bm4dof_run takes (W*H*2*F each): fflow[t] = flow t -> t+1, bflow[t] = flow
 * t -> t-1, the last forward and the first backward field copied from their
 * neighbours as tvl1flow-seq.sh does.  All 2(F-1) pairs are computed in one
 * batch. */
bm4dof_status bm4dof_tvl1_video(bm4dof_ctx *ctx, const float *video, unsigned width, unsigned height,
                                unsigned frames, const bm4dof_tvl1_params *params, float *fflow, float *bflow,
                                unsigned flags);

/* ---- learned form ----------------------------------------------------------
 * No counterpart in the reference.  With BM4DOF_LEARNED, bm4dof_run skips the
 * step-1 pass: groups are searched on the noisy video with params2's geometry
 * and filtered in the 3-D transform domain of the reference's step 2, with the
 * Wiener gains of the member-mean Haar row predicted by the gain network
 * (65 -> 256 -> 256 -> 64, GELU, sigmoid output, BF16 weights) from the
 * log-variances log(mean_m Z[m][k]^2 / sigma^2) of the 64 patch coefficients
 * across the members and sigma/255; the other Haar rows are hard-thresholded
 * at (params1->beta * sigma)^2.  A group whose residual variance exceeds
 * kappa * sigma^2 is filtered again by the two-step shrinkage of its own
 * coefficients (hard-threshold pilot, then Wiener).  Grey video, 64-element
 * patches.  `basic` receives the same estimate as `final`. */

/* Floats in a gain-network parameter blob: W1[65][256] b1[256] W2[256][256]
 * b2[256] W3[256][64] b3[64], each W[in][out]. */
#define BM4DOF_GAIN_PARAMS 99136u

/* Installs the gain network used by BM4DOF_LEARNED runs (params: host floats,
 * n == BM4DOF_GAIN_PARAMS), or none when params is NULL: the mean-row gains
 * are then the empirical Wiener gains of the noisy coefficients (the method
 * without the network).  kappa: fallback threshold (0 means 1.5). */
bm4dof_status bm4dof_set_gain_network(bm4dof_ctx *ctx, const float *params, size_t n, float kappa);

/* Groups filtered and groups that fell back in the last BM4DOF_LEARNED run. */
bm4dof_status bm4dof_learned_stats(bm4dof_ctx *ctx, unsigned long long *groups,
                                   unsigned long long *fallbacks);

/* No counterpart in the reference.  Over both steps of the last
 * BM4DOF_MIXED_PRECISION run: the groups whose patch search went through the
 * tensor-core pre-screen; of those, the ones that got the exact search
 * instead (pre-screen unusable, or not certified under
 * BM4DOF_MIXED_CERTIFIED); and the ones that kept an uncertified re-rank of
 * their 32 best approximations (only without BM4DOF_MIXED_CERTIFIED).  Every
 * other group's neighbour list is certified to be the exact path's. */
bm4dof_status bm4dof_mixed_stats(bm4dof_ctx *ctx, unsigned long long *groups, unsigned long long *exact,
                                 unsigned long long *uncertified);

/* No counterpart in the reference: the measured FP32 rate of the exact patch
 * search's instruction mix on `device` (per two patch elements one packed
 * subtract, one packed multiply and two scalar adds, the reference's
 * separately rounded operations), in tera-operations per second counting 3
 * per element -- the denominator of that kernel's roofline.  *ms (may be
 * NULL) receives one launch's time.  Allocates a few bytes; synchronises. */
bm4dof_status bm4dof_fp32_mix_rate(int device, float *tops, float *ms);

/* No counterpart in the reference: a self-check of the tensor-core operand
 * layout.  d (128 x 256 floats, row-major) = a (128 x 64 FP16, row-major) times
 * the transpose of b (256 x 64 FP16, row-major), computed through shared
 * memory, tcgen05.mma and tensor memory on the current device.  Device
 * pointers; synchronises `stream`. */
bm4dof_status bm4dof_tc_selftest(const void *a, const void *b, float *d, void *stream);

/* Training pairs for the gain network.  Searches the groups of the learned
 * form on `noisy` (grey, params2's geometry, mask switch-offs applied) and
 * writes, for every grid group g of all tiles in processing order:
 *   feat[g*65 + k]    network inputs,
 *   target[g*64 + k]  the step-2 Wiener gain y^2 / (y^2 + (beta2 sigma)^2) of
 *                     the member-mean Haar coefficient y of patch coefficient
 *                     k of the same members in `basic` (the plain method's
 *                     step-1 output),
 *   valid[g]          1 for groups the filter processes, 0 otherwise.
 * feat/target/valid are device pointers with room for cap groups; the other
 * pointers follow `flags` (BM4DOF_DEVICE_POINTERS).  *count = number of grid
 * groups (BM4DOF_ERR_ARGUMENT when larger than cap). */
bm4dof_status bm4dof_gain_samples(bm4dof_ctx *ctx, const float *noisy, const float *basic,
                                  const float *fflow, const float *bflow,
                                  unsigned width, unsigned height, unsigned frames,
                                  const bm4dof_params *params2, unsigned nparts, unsigned flags,
                                  float *feat, float *target, unsigned char *valid,
                                  size_t cap, size_t *count);

/* Training of the gain network on the GPU: forward, backward (mean squared
 * error of the 64 gains) and AdamW, BF16 operands with FP32 accumulation and
 * FP32 master weights.  feat/target/gains are device pointers of n <= batch
 * rows (feat [n][65], target and gains [n][64]). */
typedef struct bm4dof_trainer bm4dof_trainer;
bm4dof_status bm4dof_trainer_create(bm4dof_trainer **t, int device, unsigned batch, unsigned seed);
void          bm4dof_trainer_destroy(bm4dof_trainer *t);
/* The trainer's own non-blocking stream, ordered against the caller's streams
 * by the caller as for bm4dof_get_stream: bm4dof_trainer_step returns before
 * its kernels have read feat and target unless it reports the loss. */
bm4dof_status bm4dof_trainer_get_stream(bm4dof_trainer *t, void **stream);
/* Reads (set = 0) or writes (set = 1) the FP32 master parameters as a host blob. */
bm4dof_status bm4dof_trainer_params(bm4dof_trainer *t, float *params, size_t n, int set);
/* Reads (set = 0) or writes (set = 1) the AdamW state for a checkpoint: the
 * first and second moments (host blobs laid out like the parameters) and the
 * number of steps taken.  Restored with the parameters, training continues
 * exactly as if it had not stopped. */
bm4dof_status bm4dof_trainer_state(bm4dof_trainer *t, float *moment1, float *moment2, size_t n,
                                   unsigned long long *steps, int set);
/* Loss and gradient (host blob, may be NULL) of one batch, no update. */
bm4dof_status bm4dof_trainer_grad(bm4dof_trainer *t, const float *feat, const float *target, unsigned n,
                                  float *grads, float *loss);
/* One AdamW step (beta1 0.9, beta2 0.999, eps 1e-8; decay on the matrices). */
bm4dof_status bm4dof_trainer_step(bm4dof_trainer *t, const float *feat, const float *target, unsigned n,
                                  float lr, float weight_decay, float *loss);
/* Network outputs for n rows, with the inference kernel bm4dof_run uses. */
bm4dof_status bm4dof_trainer_predict(bm4dof_trainer *t, const float *feat, unsigned n, float *gains);

#ifdef __cplusplus
}
#endif

#endif /* BM4DOF_H_INCLUDED */
