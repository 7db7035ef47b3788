/*
 * ref_harness.cpp -- TEST INFRASTRUCTURE ONLY.
 *
 * C entry points around the reference's own, unmodified VideoNLB code
 * (src/core/nldct.cpp et al., compiled in place by `make -C oracle ref` into
 * oracle/_ref/libbm4dof_ref.so, and with the reference's VBM3D_SEARCH switch
 * into oracle/_ref/libbm4dof_ref_vbm3d.so).  Videos are built in memory; no
 * file I/O.
 * Used to pin the oracle restatement (oracle/bm4dof_oracle.cpp) and to
 * generate tests/golden fixtures.
 */
#include <ctime>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <string>
#include <unistd.h>

#include "nldct.h"

#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/bm4dof.h"

namespace {

void to_nlb(const bm4dof_params &s, VideoNLB::nlbParams &d)
{
	d.sigma = s.sigma;
	d.sizePatch = s.sizePatch;
	d.sizePatchTime = s.sizePatchTime;
	d.nSimilarPatches = s.nSimilarPatches;
	d.sizeSearchWindow = s.sizeSearchWindow;
	d.sizeSearchTimeRangeFwd = s.sizeSearchTimeRangeFwd;
	d.sizeSearchTimeRangeBwd = s.sizeSearchTimeRangeBwd;
	d.boundary = s.boundary;
	d.offSet = s.offSet;
	d.offSetTime = s.offSetTime;
	d.beta = s.beta;
	d.betaMean = s.betaMean;
	d.tau = s.tau;
	d.orderInvariance = s.orderInvariance != 0;
	d.isFirstStep = s.isFirstStep != 0;
	d.doPasteBoost = s.doPasteBoost != 0;
	d.verbose = s.verbose != 0;
	d.colorSpace = s.colorSpace == BM4DOF_YUV ? VideoNLB::YUV : VideoNLB::RGB;
	d.transform = s.transform == BM4DOF_DCT ? VideoNLB::dct : VideoNLB::bior1_5;
	d.sizeSearchWindowPred = s.sizeSearchWindowPred;
	d.nSimilarPatchesPred = s.nSimilarPatchesPred;
	d.dsub = s.dsub;
	d.agg_window = s.agg_window != 0;
}

void from_nlb(const VideoNLB::nlbParams &s, bm4dof_params &d)
{
	std::memset(&d, 0, sizeof(d));
	d.sigma = s.sigma;
	d.sizePatch = s.sizePatch;
	d.sizePatchTime = s.sizePatchTime;
	d.nSimilarPatches = s.nSimilarPatches;
	d.sizeSearchWindow = s.sizeSearchWindow;
	d.sizeSearchTimeRangeFwd = s.sizeSearchTimeRangeFwd;
	d.sizeSearchTimeRangeBwd = s.sizeSearchTimeRangeBwd;
	d.boundary = s.boundary;
	d.offSet = s.offSet;
	d.offSetTime = s.offSetTime;
	d.beta = s.beta;
	d.betaMean = s.betaMean;
	d.tau = s.tau;
	d.orderInvariance = s.orderInvariance;
	d.isFirstStep = s.isFirstStep;
	d.doPasteBoost = s.doPasteBoost;
	d.verbose = s.verbose;
	d.colorSpace = s.colorSpace == VideoNLB::YUV ? BM4DOF_YUV : BM4DOF_RGB;
	d.transform = s.transform == VideoNLB::dct ? BM4DOF_DCT : BM4DOF_BIOR1_5;
	d.sizeSearchWindowPred = s.sizeSearchWindowPred;
	d.nSimilarPatchesPred = s.nSimilarPatchesPred;
	d.dsub = s.dsub;
	d.agg_window = s.agg_window;
}

void fill(Video<float> &v, const float *src, unsigned W, unsigned H, unsigned F, unsigned C)
{
	v.resize(W, H, F, C);
	std::memcpy(v.data.data(), src, sizeof(float) * (size_t)W * H * F * C);
}

} // namespace

extern "C" {

/* initializeNlbParameters (nldct.cpp:81).  betaMean is left as the caller set
 * it beforehand, since the reference does not initialise it. */
void ref_initialize_params(bm4dof_params *p, unsigned step, float sigma,
                           const bm4dof_video_size *sz, int verbose)
{
	VideoNLB::nlbParams q;
	std::memset(&q, 0, sizeof(q));
	q.betaMean = p->betaMean;
	VideoSize vs(sz->width, sz->height, sz->frames, sz->channels);
	VideoNLB::initializeNlbParameters(q, step, sigma, vs, verbose != 0);
	from_nlb(q, *p);
}

void ref_set_size_search_window(bm4dof_params *p, unsigned wx)
{
	VideoNLB::nlbParams q; to_nlb(*p, q);
	VideoNLB::setSizeSearchWindow(q, wx);
	from_nlb(q, *p);
}

void ref_set_size_patch(bm4dof_params *p, const bm4dof_video_size *sz, unsigned px)
{
	VideoNLB::nlbParams q; to_nlb(*p, q);
	VideoSize vs(sz->width, sz->height, sz->frames, sz->channels);
	VideoNLB::setSizePatch(q, vs, px);
	from_nlb(q, *p);
}

void ref_set_n_similar_patches(bm4dof_params *p, unsigned np)
{
	VideoNLB::nlbParams q; to_nlb(*p, q);
	VideoNLB::setNSimilarPatches(q, np);
	from_nlb(q, *p);
}

/* printNlbParameters (nldct.cpp:219) captured into buf through a temp file. */
int ref_format_params(const bm4dof_params *p, char *buf, size_t len)
{
	VideoNLB::nlbParams q; to_nlb(*p, q);
	fflush(stdout);
	FILE *tmp = tmpfile();
	if (!tmp) return -1;
	const int saved = dup(fileno(stdout));
	dup2(fileno(tmp), fileno(stdout));
	VideoNLB::printNlbParameters(q);
	fflush(stdout);
	dup2(saved, fileno(stdout));
	close(saved);
	rewind(tmp);
	size_t n = fread(buf, 1, len ? len - 1 : 0, tmp);
	if (len) buf[n] = 0;
	fclose(tmp);
	return (int)n;
}

/* runNlBayes (nldct.cpp:267) with OpenMP limited to nthreads, i.e. with
 * 2*nthreads tiles.  Returns 0, or 1 with the exception text in err. */
int ref_run(const float *noisy, const float *fflow, const float *bflow, unsigned W, unsigned H,
            unsigned C, unsigned F, float *basic, float *final_, const bm4dof_params *p1,
            const bm4dof_params *p2, unsigned nthreads, float ratios[2], char *err, size_t errlen)
{
	try {
#ifdef _OPENMP
		omp_set_num_threads(nthreads ? (int)nthreads : 1);
#endif
		Video<float> vn, vf, vb, vbasic, vfinal;
		fill(vn, noisy, W, H, F, C);
		if (fflow) fill(vf, fflow, W, H, F, 2);
		if (bflow) fill(vb, bflow, W, H, F, 2);
		VideoNLB::nlbParams q1, q2;
		to_nlb(*p1, q1);
		to_nlb(*p2, q2);
		if (q1.sizePatch == 0) fill(vbasic, basic, W, H, F, C);
		std::vector<float> r = VideoNLB::runNlBayes(vn, vf, vb, vbasic, vfinal, q1, q2);
		if (vbasic.data.size() == (size_t)W * H * F * C)
			std::memcpy(basic, vbasic.data.data(), sizeof(float) * vbasic.data.size());
		if (q2.sizePatch && vfinal.data.size() == (size_t)W * H * F * C)
			std::memcpy(final_, vfinal.data.data(), sizeof(float) * vfinal.data.size());
		if (ratios) { ratios[0] = r[0]; ratios[1] = r[1]; }
		return 0;
	} catch (const std::exception &e) {
		if (err && errlen) std::snprintf(err, errlen, "%s", e.what());
		return 1;
	}
}

/* processNlBayes (nldct.cpp:490) of one video with the crop position given
 * (NULL: the default CropPosition()).  Step 1 writes basic, step 2 reads it
 * and writes final_.  Returns 0 with the group count in *groups, or 1 with the
 * exception text in err. */
int ref_process(const float *noisy, const float *fflow, const float *bflow, unsigned W, unsigned H,
                unsigned C, unsigned F, float *basic, float *final_, const bm4dof_params *p,
                const bm4dof_crop *crop, unsigned *groups, char *err, size_t errlen)
{
	try {
		Video<float> vn, vf, vb, vbasic, vfinal;
		fill(vn, noisy, W, H, F, C);
		if (fflow) fill(vf, fflow, W, H, F, 2);
		if (bflow) fill(vb, bflow, W, H, F, 2);
		VideoNLB::nlbParams q;
		to_nlb(*p, q);
		if (!q.isFirstStep) fill(vbasic, basic, W, H, F, C);
		VideoUtils::CropPosition cp = VideoUtils::CropPosition();
		if (crop) {
			cp.origin_x = crop->origin_x;
			cp.origin_y = crop->origin_y;
			cp.origin_t = crop->origin_t;
			cp.ending_x = crop->ending_x;
			cp.ending_y = crop->ending_y;
			cp.ending_t = crop->ending_t;
			cp.source_sz = VideoSize(crop->source_sz.width, crop->source_sz.height, crop->source_sz.frames,
			                         crop->source_sz.channels);
		}
		const unsigned n = VideoNLB::processNlBayes(vn, vf, vb, vbasic, vfinal, q, cp);
		const size_t nv = (size_t)W * H * F * C;
		if (q.isFirstStep && vbasic.data.size() == nv)
			std::memcpy(basic, vbasic.data.data(), sizeof(float) * nv);
		if (!q.isFirstStep && vfinal.data.size() == nv)
			std::memcpy(final_, vfinal.data.data(), sizeof(float) * nv);
		if (groups) *groups = n;
		return 0;
	} catch (const std::exception &e) {
		if (err && errlen) std::snprintf(err, errlen, "%s", e.what());
		return 1;
	}
}

/* estimateSimilarPatchesStep1/2 (nldct.cpp:1143, 1607) on one video (a tile):
 * returns nSimP and writes index[0..nSimP). */
unsigned ref_search(unsigned step, const float *noisy, const float *basic, const float *fflow,
                    const float *bflow, unsigned W, unsigned H, unsigned C, unsigned F,
                    const bm4dof_params *p, unsigned pidx, unsigned *index)
{
	Video<float> vn, vbasic, vf, vb;
	fill(vn, noisy, W, H, F, C);
	if (fflow) fill(vf, fflow, W, H, F, 2);
	if (bflow) fill(vb, bflow, W, H, F, 2);
	VideoNLB::nlbParams q; to_nlb(*p, q);
	const unsigned sWt = q.sizeSearchTimeRangeFwd + q.sizeSearchTimeRangeBwd + 1;
	const unsigned patch_num = q.sizeSearchWindow * q.sizeSearchWindow * sWt;
	const unsigned sPC = q.sizePatch * q.sizePatch * q.sizePatchTime;
	std::vector<unsigned> idx(patch_num);
	unsigned n;
	if (step == 1) {
		std::vector<std::vector<float> > group(C, std::vector<float>((size_t)patch_num * sPC));
		n = VideoNLB::estimateSimilarPatchesStep1(vn, vf, vb, group, idx, pidx, q);
	} else {
		fill(vbasic, basic, W, H, F, C);
		std::vector<float> gN((size_t)patch_num * sPC * C), gB((size_t)patch_num * sPC * C);
		n = VideoNLB::estimateSimilarPatchesStep2(vn, vbasic, vf, vb, gN, gB, idx, pidx, q);
	}
	for (unsigned i = 0; i < n; i++) index[i] = idx[i];
	return n;
}

} // extern "C"
