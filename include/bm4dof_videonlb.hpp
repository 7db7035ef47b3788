/* bm4dof_videonlb.hpp -- the reference's C++ entry points over the C ABI.
 *
 * For code written against namespace VideoNLB (src/core/nldct.h): runNlBayes
 * with the reference's parameters and return value (nldct.h:239-247) and its
 * error behaviour (std::runtime_error carrying the messages of
 * nldct.cpp:279-341, which the C ABI keeps verbatim), processNlBayes for one
 * step over one cropped video (nldct.h:270-278), and the parameter
 * functions initializeNlbParameters, setSizeSearchWindow, setSizePatch,
 * setNSimilarPatches and printNlbParameters (nldct.h:149-224).
 * Header-only; link -lbm4dof_gpu.
 *
 * The functions are templates over the caller's types, so this header sits
 * beside the reference's headers without redefining anything:
 *   Params  any struct with nlbParams' fields, by name (nldct.h:55-82);
 *   Size    any struct with VideoSize's width, height, frames, channels;
 *   Video   any type with Video<float>'s members sz (a Size), data (contiguous
 *           float storage with data()) and resize(const Size &);
 *   Crop    any struct with VideoUtils::CropPosition's origin_x/y/t,
 *           ending_x/y/t and source_sz (lib_videot.hpp:440-470).
 * A reference build switches by calling bm4dof_videonlb::runNlBayes where it
 * called VideoNLB::runNlBayes; everything else stays as it is.
 *
 * Tiles: the reference splits the video into 2 x omp_get_max_threads() tiles
 * (nldct.cpp:318-323) and its output depends on that count.  runNlBayes
 * without a tile count uses 2 x T, T = the first number in OMP_NUM_THREADS if
 * it is set, else the host's hardware threads (OpenMP's default); pass nparts
 * explicitly to reproduce a given reference run bit for bit.
 *
 * Contexts: one bm4dof_ctx per calling thread and device, created on first
 * use and destroyed when the thread ends.  The video pointers are host
 * pointers; the library copies them to the GPU and back. */
#pragma once

#include <cstdlib>
#include <memory>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>
#if defined(__linux__)
#include <sched.h>
#endif

#include "bm4dof.h"

namespace bm4dof_videonlb {

/* ---- parameter and size conversion (field for field, same names) -------- */

template <class Params>
bm4dof_params to_c(const Params &s)
{
	bm4dof_params c;
	c.sigma = s.sigma;
	c.sizePatch = s.sizePatch;
	c.sizePatchTime = s.sizePatchTime;
	c.nSimilarPatches = s.nSimilarPatches;
	c.sizeSearchWindow = s.sizeSearchWindow;
	c.sizeSearchTimeRangeFwd = s.sizeSearchTimeRangeFwd;
	c.sizeSearchTimeRangeBwd = s.sizeSearchTimeRangeBwd;
	c.boundary = s.boundary;
	c.offSet = s.offSet;
	c.offSetTime = s.offSetTime;
	c.beta = s.beta;
	c.betaMean = s.betaMean;
	c.tau = s.tau;
	c.orderInvariance = s.orderInvariance ? 1 : 0;
	c.isFirstStep = s.isFirstStep ? 1 : 0;
	c.doPasteBoost = s.doPasteBoost ? 1 : 0;
	c.verbose = s.verbose ? 1 : 0;
	c.colorSpace = (int)s.colorSpace;
	c.transform = (int)s.transform;
	c.sizeSearchWindowPred = s.sizeSearchWindowPred;
	c.nSimilarPatchesPred = s.nSimilarPatchesPred;
	c.dsub = s.dsub;
	c.agg_window = s.agg_window ? 1 : 0;
	return c;
}

template <class Params>
void from_c(const bm4dof_params &c, Params &s)
{
	s.sigma = c.sigma;
	s.sizePatch = c.sizePatch;
	s.sizePatchTime = c.sizePatchTime;
	s.nSimilarPatches = c.nSimilarPatches;
	s.sizeSearchWindow = c.sizeSearchWindow;
	s.sizeSearchTimeRangeFwd = c.sizeSearchTimeRangeFwd;
	s.sizeSearchTimeRangeBwd = c.sizeSearchTimeRangeBwd;
	s.boundary = c.boundary;
	s.offSet = c.offSet;
	s.offSetTime = c.offSetTime;
	s.beta = c.beta;
	s.betaMean = c.betaMean;
	s.tau = c.tau;
	s.orderInvariance = c.orderInvariance != 0;
	s.isFirstStep = c.isFirstStep != 0;
	s.doPasteBoost = c.doPasteBoost != 0;
	s.verbose = c.verbose != 0;
	s.colorSpace = static_cast<decltype(s.colorSpace)>(c.colorSpace);
	s.transform = static_cast<decltype(s.transform)>(c.transform);
	s.sizeSearchWindowPred = c.sizeSearchWindowPred;
	s.nSimilarPatchesPred = c.nSimilarPatchesPred;
	s.dsub = c.dsub;
	s.agg_window = c.agg_window != 0;
}

template <class Size>
bm4dof_video_size to_c_size(const Size &z)
{
	bm4dof_video_size c;
	c.width = z.width;
	c.height = z.height;
	c.frames = z.frames;
	c.channels = z.channels;
	return c;
}

/* ---- parameter functions (nldct.cpp:81-249) ------------------------------ */

template <class Params, class Size>
void initializeNlbParameters(Params &params, const unsigned step, const float sigma, const Size &size,
                             const bool verbose)
{
	bm4dof_params c = to_c(params);
	const bm4dof_video_size z = to_c_size(size);
	bm4dof_initialize_params(&c, step, sigma, &z, verbose ? 1 : 0);
	from_c(c, params);
}

template <class Params>
void setSizeSearchWindow(Params &prms, unsigned sizeSearchWindow)
{
	bm4dof_params c = to_c(prms);
	bm4dof_set_size_search_window(&c, sizeSearchWindow);
	from_c(c, prms);
}

template <class Params, class Size>
void setSizePatch(Params &prms, const Size &size, unsigned sizePatch)
{
	bm4dof_params c = to_c(prms);
	const bm4dof_video_size z = to_c_size(size);
	bm4dof_set_size_patch(&c, &z, sizePatch);
	from_c(c, prms);
}

template <class Params>
void setNSimilarPatches(Params &prms, unsigned nSimilarPatches)
{
	bm4dof_params c = to_c(prms);
	bm4dof_set_n_similar_patches(&c, nSimilarPatches);
	from_c(c, prms);
}

template <class Params>
void printNlbParameters(const Params &params)
{
	const bm4dof_params c = to_c(params);
	bm4dof_print_params(&c);
}

/* ---- the run ------------------------------------------------------------- */

/* 2 x the reference's OpenMP thread count (see the header comment).  Without
 * OMP_NUM_THREADS, libgomp starts one thread per CPU the process may run on
 * (its affinity mask, which taskset or a cpuset narrows), not one per online
 * CPU. */
inline unsigned default_tiles()
{
	const char *e = std::getenv("OMP_NUM_THREADS");
	long t = e ? std::strtol(e, nullptr, 10) : 0;
#if defined(__linux__)
	if (t <= 0) {
		cpu_set_t set;
		CPU_ZERO(&set);
		if (sched_getaffinity(0, sizeof(set), &set) == 0) t = CPU_COUNT(&set);
	}
#endif
	if (t <= 0) t = (long)std::thread::hardware_concurrency();
	return 2u * (unsigned)(t > 0 ? t : 1);
}

namespace detail {

class Context {
public:
	explicit Context(int device)
	{
		if (bm4dof_create(&ctx_, device) != BM4DOF_OK) throw std::runtime_error(bm4dof_last_error());
	}
	~Context() { bm4dof_destroy(ctx_); }
	Context(const Context &) = delete;
	Context &operator=(const Context &) = delete;
	bm4dof_ctx *get() const { return ctx_; }

private:
	bm4dof_ctx *ctx_ = nullptr;
};

inline bm4dof_ctx *context(int device)
{
	thread_local std::vector<std::unique_ptr<Context>> ctxs;
	if (device < 0) throw std::runtime_error("bm4dof_create: bad device ordinal");
	if ((size_t)device >= ctxs.size()) ctxs.resize((size_t)device + 1);
	if (!ctxs[(size_t)device]) ctxs[(size_t)device].reset(new Context(device));
	return ctxs[(size_t)device]->get();
}

template <class SizeA, class SizeB>
bool same_size(const SizeA &a, const SizeB &b)
{
	return a.width == b.width && a.height == b.height && a.frames == b.frames && a.channels == b.channels;
}

}  // namespace detail

/* VideoNLB::runNlBayes (nldct.cpp:267-478) on the GPU: fills basic (step 1)
 * and final (step 2) and returns the percentages of processed patch groups
 * of the two steps.  The checks that need the videos' sizes, which the C ABI
 * does not take, are made here in the reference's order and with its
 * messages (nldct.cpp:276-296, 329-342), before the GPU is touched; the
 * outputs are resized as the reference resizes them.  An empty flow
 * (sz.width == 0) means no flow.  flags: BM4DOF_VBM3D_SEARCH for a reference
 * built with -DVBM3D_SEARCH, or the library's faster forms. */
template <class Video, class Params>
std::vector<float> runNlBayes(Video const &noisy, Video const &fflow, Video const &bflow, Video &basic,
                              Video &final, const Params p_prms1, const Params p_prms2, unsigned nparts,
                              unsigned flags = 0, int device = 0)
{
	const unsigned chnls = noisy.sz.channels;
	if (!(chnls == 1 || chnls == 3 || chnls == 4))
		throw std::runtime_error("VideoNLB::runNlBayes: Wrong number of channels. Must be 1, 3 or 4.");
	const bool use_oflow = fflow.sz.width > 0;
	const auto flow_ok = [&noisy](const Video &f) {
		return f.sz.channels == 2 && f.sz.width == noisy.sz.width && f.sz.height == noisy.sz.height &&
		       f.sz.frames == noisy.sz.frames;
	};
	if (use_oflow && !flow_ok(fflow))
		throw std::runtime_error("VideoNLB::runNlBayes: Wrong size of fwd optical flow.");
	if (use_oflow && !flow_ok(bflow))
		throw std::runtime_error("VideoNLB::runNlBayes: Wrong size of bwd optical flow.");
	const int step = p_prms1.sizePatch ? (p_prms2.sizePatch ? 0 : 1) : (p_prms2.sizePatch ? 2 : -1);
	if (step == -1) throw std::runtime_error("VideoNLB::runNlBayes: Both patch sizes are zero.");
	if (step != 2) basic.resize(noisy.sz);
	if (step != 1) final.resize(noisy.sz);
	if (step == 2 && !detail::same_size(noisy.sz, basic.sz))
		throw std::runtime_error("VideoNLB::runNlBayes: sizes of noisy and basic videos don't match");

	bm4dof_ctx *ctx = detail::context(device);
	const bm4dof_params c1 = to_c(p_prms1), c2 = to_c(p_prms2);
	float ratios[2] = {0.f, 0.f};
	const bm4dof_status s =
	    bm4dof_run(ctx, noisy.data.data(), use_oflow ? fflow.data.data() : nullptr,
	               use_oflow ? bflow.data.data() : nullptr, noisy.sz.width, noisy.sz.height, noisy.sz.channels,
	               noisy.sz.frames, basic.data.data(), step == 1 ? nullptr : final.data.data(), &c1, &c2, nparts,
	               flags, ratios);
	if (s != BM4DOF_OK) throw std::runtime_error(bm4dof_last_error());
	return {ratios[0], ratios[1]};
}

/* VideoNLB::processNlBayes (nldct.cpp:490-890) on the GPU: the step that
 * p.isFirstStep names, over one video cut from a source as crop says; step 1
 * writes basic, step 2 reads it and writes final (each resized to the video,
 * as the reference does).  Returns the number of processed groups.  The
 * reference checks nothing here; the layer refuses flows or a step-2 basic
 * whose size differs from the video's, which the reference would read past. */
template <class Video, class Params, class Crop>
unsigned processNlBayes(Video const &noisy, Video const &fflow, Video const &bflow, Video &basic, Video &final,
                        Params const &p, Crop const &crop, unsigned flags = 0, int device = 0)
{
	const bool use_oflow = fflow.sz.width > 0;
	const auto flow_ok = [&noisy](const Video &f) {
		return f.sz.channels == 2 && f.sz.width == noisy.sz.width && f.sz.height == noisy.sz.height &&
		       f.sz.frames == noisy.sz.frames;
	};
	if (use_oflow && (!flow_ok(fflow) || !flow_ok(bflow)))
		throw std::runtime_error("bm4dof_process: the flows' size differs from the video's");
	if (p.isFirstStep) basic.resize(noisy.sz);
	else if (!detail::same_size(noisy.sz, basic.sz))
		throw std::runtime_error("bm4dof_process: the basic estimate's size differs from the video's");
	else final.resize(noisy.sz);
	bm4dof_crop c;
	c.origin_x = crop.origin_x;
	c.origin_y = crop.origin_y;
	c.origin_t = crop.origin_t;
	c.ending_x = crop.ending_x;
	c.ending_y = crop.ending_y;
	c.ending_t = crop.ending_t;
	c.source_sz = to_c_size(crop.source_sz);
	bm4dof_ctx *ctx = detail::context(device);
	const bm4dof_params cp = to_c(p);
	unsigned groups = 0;
	const bm4dof_status s = bm4dof_process(
	    ctx, noisy.data.data(), use_oflow ? fflow.data.data() : nullptr, use_oflow ? bflow.data.data() : nullptr,
	    noisy.sz.width, noisy.sz.height, noisy.sz.channels, noisy.sz.frames, basic.data.data(),
	    p.isFirstStep ? nullptr : final.data.data(), &cp, &c, flags, &groups);
	if (s != BM4DOF_OK) throw std::runtime_error(bm4dof_last_error());
	return groups;
}

/* processNlBayes with the reference's default crop (no border). */
template <class Video, class Params>
unsigned processNlBayes(Video const &noisy, Video const &fflow, Video const &bflow, Video &basic, Video &final,
                        Params const &p)
{
	struct NoCrop {
		int origin_x = 0, origin_y = 0, origin_t = 0, ending_x = 0, ending_y = 0, ending_t = 0;
		struct {
			unsigned width = 0, height = 0, frames = 0, channels = 0;
		} source_sz;
	};
	return processNlBayes(noisy, fflow, bflow, basic, final, p, NoCrop());
}

/* The reference's own signature: tiles from default_tiles(). */
template <class Video, class Params>
std::vector<float> runNlBayes(Video const &noisy, Video const &fflow, Video const &bflow, Video &basic,
                              Video &final, const Params p_prms1, const Params p_prms2)
{
	return runNlBayes(noisy, fflow, bflow, basic, final, p_prms1, p_prms2, default_tiles());
}

}  // namespace bm4dof_videonlb
