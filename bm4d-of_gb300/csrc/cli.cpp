// cli.cpp -- the bm4d-of command line over the GPU library.
//
// Mirrors the reference's CLI (src/main_vnlb.cpp:31-253): the same flags,
// defaults, checks, messages and parameter overrides, then one bm4dof_run.
// Frame files are addressed by printf patterns with -f/-l/-s exactly as
// Video<float>::loadVideo / saveVideo do (src/utils/lib_videot.cpp:30-126).
//
// Frame files (PFM, TIFF, .flo, PNG) are read and written by frames.cpp.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/bm4dof.h"
#include "frames.hpp"

using bm4dof_frames::load_video;
using bm4dof_frames::save_video;
using bm4dof_frames::Video;

namespace {

// ---- options (the reference's clo_option: "-name value", last one wins) ----
struct Args {
	int argc;
	char **argv;
	bool help = false;
	const char *find(const char *name) const
	{
		const char *v = nullptr;
		for (int i = 1; i + 1 < argc; i++)
			if (!std::strcmp(argv[i], name)) v = argv[i + 1];
		return v;
	}
	std::string str(const char *n, const char *d, const char *use)
	{
		usage(n, d, use);
		const char *v = find(n);
		return v ? v : d;
	}
	int i(const char *n, int d, const char *use)
	{
		usage(n, std::to_string(d).c_str(), use);
		const char *v = find(n);
		return v ? std::atoi(v) : d;
	}
	float f(const char *n, float d, const char *use)
	{
		char b[32];
		std::snprintf(b, sizeof b, "%g", d);
		usage(n, b, use);
		const char *v = find(n);
		if (!v) return d;
		float x = 0.f, y = 1.f;   // "a/b" fractions, as the reference's atof
		std::sscanf(v, "%g/%g", &x, &y);
		return x / y;
	}
	void usage(const char *n, const char *d, const char *use)
	{
		if (help) std::printf("    %-12s = %-16s : %s\n", n, d, use);
	}
};

// printNlbParameters (nldct.cpp:212-248); the predictive search adds three
// lines to the patch-search block, as the reference's VBM3D_SEARCH build does.
void print_params(const bm4dof_params &p, bool vbm3d)
{
	char buf[4096];
	if (bm4dof_format_params(&p, buf, sizeof(buf)) <= 0) return;
	std::string s(buf);
	if (vbm3d) {
		char extra[512];
		const int wp = (int)p.sizeSearchWindowPred;
		std::snprintf(extra, sizeof(extra),
		              "\t\tPred. spatial search window = %dx%d\n"
		              "\t\tPred. distance bias (dsub)  = %g\n"
		              "\t\tSimilar patches per frame   = %d\n",
		              wp, wp, p.dsub, (int)p.nSimilarPatchesPred);
		const size_t at = s.find("\tGroup filtering:");
		if (at != std::string::npos) s.insert(at, extra);
	}
	std::fputs(s.c_str(), stdout);
}

}  // namespace

int main(int argc, char **argv)
{
	Args a{argc, argv};
	for (int i = 1; i < argc; i++)
		if (!std::strcmp(argv[i], "-h") || !std::strcmp(argv[i], "--help")) a.help = true;
	if (a.help) {
		std::printf("%s : BM4D-OF video denoising (GB300)\n", argv[0]);
		std::printf(" NOTE: Input (<) and output (>) sequences are specified by their paths in printf format.\n");
	}
	const std::string input_path = a.str("-i", "", "< input sequence");
	const std::string inbsc_path = a.str("-b", "", "< input basic sequence");
	const std::string final_path = a.str("-deno", "deno_%03d.png", "> denoised sequence");
	const std::string basic_path = a.str("-bsic", "bsic_%03d.png", "> basic denoised sequence");
	const unsigned first_frame = a.i("-f", 0, "first frame");
	const unsigned last_frame = a.i("-l", 0, "last frame");
	const unsigned frame_step = a.i("-s", 1, "frame step");
	const std::string fflow_path = a.str("-fof", "", "< input forward  optical flow");
	const std::string bflow_path = a.str("-bof", "", "< input backward optical flow");
	const float sigma = a.f("-sigma", 0.f, "< standard deviation of the noise");
	const bool verbose = a.i("-verbose", 1, "< verbose output") != 0;
	const bool order_inv = a.i("-order-inv", 0, "< invariance to patch order in stack") != 0;
	const unsigned print_prms = (unsigned)a.i("-print-prms", 0, "< prints parameters for given channels");
	const int time_search1 = a.i("-wt1", 0, "< search window temporal radius, step 1");
	const int time_search2 = a.i("-wt2", 0, "< search window temporal radius, step 2");
	const int space_search1 = a.i("-wx1", -1, "< search window spatial radius, step 1");
	const int space_search2 = a.i("-wx2", -1, "< search window spatial radius, step 2");
	const int patch_sizex1 = a.i("-px1", -1, "< spatial patch size, step 1");
	const int patch_sizex2 = a.i("-px2", -1, "< spatial patch size, step 2");
	const int patch_sizet1 = a.i("-pt1", 1, "< temporal patch size, step 1");
	const int patch_sizet2 = a.i("-pt2", 1, "< temporal patch size, step 2");
	const int num_patches1 = a.i("-np1", -1, "< number of similar patches, step 1");
	const int num_patches2 = a.i("-np2", -1, "< number of similar patches, step 2");
	// -t1/-t2 apply to -print-prms always, to a run only with the predictive search
	const float tau1 = a.f("-t1", -1.f, "< step 1 distance threshold");
	const float tau2 = a.f("-t2", -1.f, "< step 2 distance threshold");
	const float beta1 = a.f("-b1", -1.f, "< noise correction factor beta, step 1");
	const float beta2 = a.f("-b2", -1.f, "< noise correction factor beta, step 2");
	const float beta_mean1 = a.f("-bm1", -1.f, "< noise correction factor beta for mean, step 1");
	const float beta_mean2 = a.f("-bm2", -1.f, "< noise correction factor beta for mean, step 2");
	const bool no_paste1 = a.i("-no-paste1", 0, "< disable paste trick, step 1") != 0;
	const bool no_paste2 = a.i("-no-paste2", 0, "< disable paste trick, step 2") != 0;
	const bool no_step1 = a.i("-no-step1", 0, "< disable patch skipping, step 1") != 0;
	const bool no_step2 = a.i("-no-step2", 0, "< disable patch skipping, step 2") != 0;
	const bool agg_win1 = a.i("-agg-win1", 0, "< aggregation window, step 1") != 0;
	const bool agg_win2 = a.i("-agg-win2", 0, "< aggregation window, step 2") != 0;
	const unsigned nparts = (unsigned)a.i("-nparts", 2, "< spatial tiles (the reference: 2 x OpenMP threads)");
	const int device = a.i("-device", 0, "< CUDA device");
	const bool mixed = a.i("-mixed", 0, "< FP16 tensor-core distance pre-screen") != 0;
	// the reference's VBM3D_SEARCH build as a run-time switch, with its options
	const bool vbm3d = a.i("-vbm3d", 0, "< VBM3D predictive patch search") != 0;
	const int space_search_f1 = a.i("-wxf1", -1, "< search window for predictive search, step 1");
	const int space_search_f2 = a.i("-wxf2", -1, "< search window for predictive search, step 2");
	const int num_patches_f1 = a.i("-npf1", -1, "< number of similar patches per frame, step 1");
	const int num_patches_f2 = a.i("-npf2", -1, "< number of similar patches per frame, step 2");
	const float dsub1 = a.f("-dsub1", -1.f, "< distance bias, step 1");
	const float dsub2 = a.f("-dsub2", -1.f, "< distance bias, step 2");
	(void)time_search1;
	(void)time_search2;
	if (a.help) return EXIT_SUCCESS;

	// checks of main_vnlb.cpp:89-127
	if (input_path.empty())
		return std::fprintf(stderr, "%s: no input sequence.\nTry `%s --help' for more information.\n", argv[0],
		                    argv[0]),
		       EXIT_FAILURE;
	if (patch_sizex1 == 0 && patch_sizex2 > 0 && inbsc_path.empty())
		return std::fprintf(stderr,
		                    "%s: if px1 = 0 and px2 > 0, a basic sequence path must be given.\n"
		                    "Try `%s --help' for more information.\n",
		                    argv[0], argv[0]),
		       EXIT_FAILURE;
	if ((patch_sizex1 < 0 && patch_sizex1 != -1) || (patch_sizex2 < 0 && patch_sizex2 != -1) ||
	    (patch_sizet1 < 0 || patch_sizet2 < 0))
		return std::fprintf(stderr, "%s: px1, px2, pt1 and pt2 cannot be negative.\n"
		                            "Try `%s --help' for more information.\n", argv[0], argv[0]),
		       EXIT_FAILURE;
	if ((num_patches1 < 0 && num_patches1 != -1) || (num_patches2 < 0 && num_patches2 != -1))
		return std::fprintf(stderr, "%s: np1 and np2 cannot be negative.\n"
		                            "Try `%s --help' for more information.\n", argv[0], argv[0]),
		       EXIT_FAILURE;
	if ((space_search1 < 0 && space_search1 != -1) || (space_search2 < 0 && space_search2 != -1) ||
	    (time_search1 < 0 || time_search2 < 0))
		return std::fprintf(stderr, "%s: wx1, wx2, wt1 and wt2 cannot be negative.\n"
		                            "Try `%s --help' for more information.\n", argv[0], argv[0]),
		       EXIT_FAILURE;
	if (patch_sizex1 > 0 && !inbsc_path.empty())
		std::fprintf(stderr, "\x1b[33;1mWarning:\x1b[0m a basic sequence path ignored since px1 > 0.\n");
	if (fflow_path.empty() != bflow_path.empty())
		return std::fprintf(stderr, "Only one oflow path provided.\nTry `%s --help' for more information.\n",
		                    argv[0]),
		       EXIT_FAILURE;
	if (patch_sizex1 == 0 && patch_sizex2 == 0)
		return std::fprintf(stderr, "Given patch sizes for both steps are 0. Nothing to do.\n"), EXIT_FAILURE;

	const bool deno_only = patch_sizex1 == 0 && patch_sizex2 != 0;
	const bool use_oflow = !fflow_path.empty() && (last_frame - first_frame > frame_step);

	Video noisy, basic, fflow, bflow;
	std::string err;
	bm4dof_video_size sz = {0, 0, 0, 0};
	if (print_prms) {
		sz.channels = print_prms;
	} else {
		if (!load_video(input_path, first_frame, last_frame, frame_step, noisy, err))
			return std::fprintf(stderr, "%s\n", err.c_str()), EXIT_FAILURE;
		if (deno_only && !load_video(inbsc_path, first_frame, last_frame, frame_step, basic, err))
			return std::fprintf(stderr, "%s\n", err.c_str()), EXIT_FAILURE;
		if (use_oflow && (!load_video(fflow_path, first_frame, last_frame, frame_step, fflow, err) ||
		                  !load_video(bflow_path, first_frame, last_frame, frame_step, bflow, err)))
			return std::fprintf(stderr, "%s\n", err.c_str()), EXIT_FAILURE;
		sz.width = noisy.w;
		sz.height = noisy.h;
		sz.frames = noisy.f;
		sz.channels = noisy.c;
		if (verbose) std::printf("Running BM4D-OF on the noisy video\n");
	}

	// parameters (main_vnlb.cpp:206-246)
	bm4dof_params p1, p2;
	bm4dof_initialize_params(&p1, 1, sigma, &sz, print_prms ? verbose : verbose);
	bm4dof_initialize_params(&p2, 2, sigma, &sz, verbose);
	if (space_search1 >= 0) bm4dof_set_size_search_window(&p1, (unsigned)space_search1);
	if (space_search2 >= 0) bm4dof_set_size_search_window(&p2, (unsigned)space_search2);
	if (patch_sizex1 >= 0) bm4dof_set_size_patch(&p1, &sz, (unsigned)patch_sizex1);
	if (patch_sizex2 >= 0) bm4dof_set_size_patch(&p2, &sz, (unsigned)patch_sizex2);
	if (num_patches1 >= 0) bm4dof_set_n_similar_patches(&p1, (unsigned)num_patches1);
	if (num_patches2 >= 0) bm4dof_set_n_similar_patches(&p2, (unsigned)num_patches2);
	if (beta1 >= 0) p1.beta = beta1;
	if (beta2 >= 0) p2.beta = beta2;
	if (beta1 >= 0) p1.betaMean = beta1;
	if (beta2 >= 0) p2.betaMean = beta2;
	if (beta_mean1 >= 0) p1.betaMean = beta_mean1;
	if (beta_mean2 >= 0) p2.betaMean = beta_mean2;
	if (patch_sizet1 >= 0) p1.sizePatchTime = patch_sizet1;
	if (patch_sizet2 >= 0) p2.sizePatchTime = patch_sizet2;
	if (agg_win1) p1.agg_window = 1;
	if (agg_win2) p2.agg_window = 1;
	if (no_paste1) p1.doPasteBoost = 0;
	if (no_paste2) p2.doPasteBoost = 0;
	if (no_step1) p1.offSet = 1;
	if (no_step2) p2.offSet = 1;
	if (vbm3d) {
		if (space_search_f1 >= 0) p1.sizeSearchWindowPred = (unsigned)space_search_f1;
		if (space_search_f2 >= 0) p2.sizeSearchWindowPred = (unsigned)space_search_f2;
		if (num_patches_f1 >= 0) p1.nSimilarPatchesPred = (unsigned)num_patches_f1;
		if (num_patches_f2 >= 0) p2.nSimilarPatchesPred = (unsigned)num_patches_f2;
		if (dsub1 >= 0) p1.dsub = dsub1;
		if (dsub2 >= 0) p2.dsub = dsub2;
	}
	if (print_prms || vbm3d) {
		if (tau1 >= 0) p1.tau = tau1;
		if (tau2 >= 0) p2.tau = tau2;
	}
	if (order_inv) p1.orderInvariance = p2.orderInvariance = 1;
	if (print_prms) {
		print_params(p1, vbm3d);
		print_params(p2, vbm3d);
		return EXIT_SUCCESS;
	}

	bm4dof_ctx *ctx = nullptr;
	if (bm4dof_create(&ctx, device) != BM4DOF_OK)
		return std::fprintf(stderr, "%s\n", bm4dof_last_error()), EXIT_FAILURE;
	Video fin = noisy;
	if (!deno_only) basic = noisy;
	float ratios[2] = {0.f, 0.f};
	const bm4dof_status s =
	    bm4dof_run(ctx, noisy.data.data(), use_oflow ? fflow.data.data() : nullptr,
	               use_oflow ? bflow.data.data() : nullptr, noisy.w, noisy.h, noisy.c, noisy.f, basic.data.data(),
	               fin.data.data(), &p1, &p2, nparts,
	               (mixed ? BM4DOF_MIXED_PRECISION : 0u) | (vbm3d ? BM4DOF_VBM3D_SEARCH : 0u), ratios);
	bm4dof_destroy(ctx);
	if (s != BM4DOF_OK) return std::fprintf(stderr, "%s\n", bm4dof_last_error()), EXIT_FAILURE;
	if (verbose)
		std::printf("Done. Processed %5.2f%% of possible patch groups in 1st step, and\n"
		            "%5.2f%% in 2nd step.\n", ratios[0], ratios[1]);
	if (verbose) std::printf("\nSaving output sequences\n");
	if (p2.sizePatch && !save_video(final_path, first_frame, frame_step, fin, err))
		return std::fprintf(stderr, "%s\n", err.c_str()), EXIT_FAILURE;
	if (!save_video(basic_path, first_frame, frame_step, basic, err))
		return std::fprintf(stderr, "%s\n", err.c_str()), EXIT_FAILURE;
	return EXIT_SUCCESS;
}
