// params.cpp -- host-side parameter resolution and error reporting of the C ABI.
//
// Restates the reference's parameter setters (src/core/nldct.cpp:81-249).  The
// resolved values decide the transform, the reference grid offsets and tau,
// so they follow the reference exactly, including its quirks (the temporal
// window printed as [-Bwd, Bwd]; the Fwd+Fwd test in setNSimilarPatches).
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>

#include "../../include/bm4dof.h"
#include "internal.hpp"

namespace {
thread_local std::string g_last_error;
}

namespace bm4dof {

void set_error(const std::string &msg) { g_last_error = msg; }
void clear_error() { g_last_error.clear(); }

}  // namespace bm4dof

extern "C" {

const char *bm4dof_last_error(void) { return g_last_error.c_str(); }

const char *bm4dof_version(void) { return "bm4dof-gb300 0.1 (sm_103a)"; }

void bm4dof_initialize_params(bm4dof_params *p, unsigned step, float sigma,
                              const bm4dof_video_size *size, int verbose)
{
	if (!p || !size) return;
	std::memset(p, 0, sizeof(*p));
	const bool s1 = (step == 1);
	if (size->frames == 1) {
		// image profile (BM3D defaults), nldct.cpp:90-118
		if (sigma <= 40) {
			p->sizePatch = 8;
			p->nSimilarPatches = s1 ? 16 : 32;
			p->offSet = 3;
			p->beta = s1 ? 2.7f : 1.f;
			p->tau = s1 ? 54.8f : 20.f;
		} else {
			p->sizePatch = s1 ? 8 : 11;
			p->nSimilarPatches = 32;
			p->offSet = s1 ? 4 : 6;
			p->beta = s1 ? 2.8f : 1.f;
			p->tau = s1 ? 158.f : 59.2f;
		}
		p->sizePatchTime = 1;
		p->sizeSearchTimeRangeFwd = 0;
		p->sizeSearchTimeRangeBwd = 0;
		p->sizeSearchWindowPred = 0;
		p->offSetTime = 1;
		p->dsub = 0.f;
		p->nSimilarPatchesPred = p->nSimilarPatches;
		p->sizeSearchWindow = 39;
	} else {
		// video profile (VBM3D defaults), nldct.cpp:119-136
		p->sizePatch = (s1 || sigma >= 30) ? 8 : 7;
		p->sizePatchTime = 1;
		p->nSimilarPatches = 8;
		p->sizeSearchWindow = 7;
		p->sizeSearchWindowPred = 5;
		p->sizeSearchTimeRangeFwd = 4;
		p->sizeSearchTimeRangeBwd = 4;
		p->nSimilarPatchesPred = 2;
		p->offSet = s1 ? 6 : 4;
		p->offSetTime = 1;
		p->beta = s1 ? 2.7f : 1.f;
		p->tau = s1 ? 67.1f : 54.8f;
		p->dsub = s1 ? 7.f : 3.f;
	}
	p->betaMean = p->beta;
	p->orderInvariance = 0;
	p->isFirstStep = s1 ? 1 : 0;
	p->sigma = sigma;
	p->verbose = verbose;
	p->colorSpace = BM4DOF_YUV;
	p->doPasteBoost = 0;
	p->agg_window = 1;
	p->boundary = 2 * (p->sizeSearchWindow / 2) + (p->sizePatch - 1);
	p->transform = s1 ? BM4DOF_BIOR1_5 : BM4DOF_DCT;
}

void bm4dof_set_size_search_window(bm4dof_params *p, unsigned wx)
{
	if (!p) return;
	p->sizeSearchWindow = wx;
	p->boundary = 2 * (wx / 2) + (p->sizePatch - 1);
	p->nSimilarPatches = std::min(p->nSimilarPatches,
		wx * wx * (p->sizeSearchTimeRangeFwd + p->sizeSearchTimeRangeBwd + 1));
}

void bm4dof_set_size_patch(bm4dof_params *p, const bm4dof_video_size *size, unsigned px)
{
	if (!p || !size) return;
	p->sizePatch = px;
	p->boundary = 2 * (p->sizeSearchWindow / 2) + (p->sizePatch - 1);
	if (p->sizePatch != 8) p->transform = BM4DOF_DCT;
	if (size->frames > 1)   // (float)px/4.*3. is evaluated in double, then truncated
		p->offSet = p->isFirstStep ? (unsigned)((double)(float)px / 4. * 3.) : px / 2;
}

void bm4dof_set_n_similar_patches(bm4dof_params *p, unsigned np)
{
	if (!p) return;
	p->nSimilarPatches = std::min(np, p->sizeSearchWindow * p->sizeSearchWindow *
		(p->sizeSearchTimeRangeFwd + p->sizeSearchTimeRangeBwd + 1));
	if (p->sizeSearchTimeRangeFwd + p->sizeSearchTimeRangeFwd == 0)
		p->nSimilarPatchesPred = p->nSimilarPatches;
}

int bm4dof_format_params(const bm4dof_params *p, char *buf, size_t len)
{
	if (!p) return -1;
	const int px = p->sizePatch, pt = p->sizePatchTime;
	const int wtb = p->sizeSearchTimeRangeBwd, wtf = p->sizeSearchTimeRangeBwd;
	const int wx = p->sizeSearchWindow;
	return std::snprintf(buf, len,
		"\x1b[37;01mParameters for step %d:\x1b[0m\n"
		"\tPatch search:\n"
		"\t\tPatch size                  = %dx%dx%d\n"
		"\t\tNumber of patches           = %d\n"
		"\t\tSpatial search window       = %dx%d\n"
		"\t\tTemporal search window      = [-%d,%d]\n"
		"\t\tDistance threshold (tau)    = %g\n"
		"\tGroup filtering:\n"
		"\t\tTransform                   = %s\n"
		"\t\tBeta                        = %g\n"
		"\t\tOrder invariance            = %s\n"
		"\tAggregation:\n"
		"\t\tOffset                      = %d\n"
		"\t\tPasteBoost                  = %s\n"
		"\t\tAggregation window          = %s\n"
		"\n",
		p->isFirstStep ? 1 : 2, px, px, pt, (int)p->nSimilarPatches, wx, wx, wtb, wtf,
		(double)p->tau, p->transform == BM4DOF_DCT ? "dct" : "bior1.5", (double)p->beta,
		p->orderInvariance ? "yes" : "no", (int)p->offSet,
		p->doPasteBoost ? "active" : "inactive", p->agg_window ? "yes" : "no");
}

void bm4dof_print_params(const bm4dof_params *p)
{
	char buf[2048];
	if (bm4dof_format_params(p, buf, sizeof(buf)) > 0) std::fputs(buf, stdout);
}

}  // extern "C"
