// videonlb_layer.cpp -- TEST DRIVER for include/bm4dof_videonlb.hpp, built by
// tests/test_videonlb_layer.py in two ways:
//   * with stand-in types that have the reference's member names;
//   * with -DWITH_REFERENCE_TYPES, against the reference's own headers
//     (VideoNLB::nlbParams, VideoSize, Video<float>) and linked to the
//     reference's code, so that the layer's parameter functions and errors are
//     compared with the reference's own in the same process.
//
//   videonlb_layer params      parameters resolved through the layer, printed
//   videonlb_layer roundtrip   field-for-field conversion both ways
//   videonlb_layer errors      runNlBayes on inputs the reference rejects
//   videonlb_layer process_errors   processNlBayes on inputs the layer refuses
//   videonlb_layer tiles       the tile count runNlBayes uses without one
//   videonlb_layer run W H C F sigma nparts noisy.raw basic.raw final.raw
//                              one denoising run (needs a GPU), planar floats
//   videonlb_layer process W H C F sigma noisy.raw basic.raw final.raw
//                  ox oy ot ex ey et sw sh sf
//                              processNlBayes step 1 then step 2 on one crop
//                              (needs a GPU); prints the two group counts
#include <ctime>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#ifdef WITH_REFERENCE_TYPES
#include "nldct.h"
typedef VideoNLB::nlbParams Params;
typedef VideoSize Size;
typedef Video<float> Vid;
#else
enum ColorSpace { RGB, YUV };
enum Transform { dct, bior1_5 };
struct Params {
	float sigma;
	unsigned sizePatch, sizePatchTime, nSimilarPatches, sizeSearchWindow, sizeSearchTimeRangeFwd,
	    sizeSearchTimeRangeBwd, boundary, offSet, offSetTime;
	float beta, betaMean, tau;
	bool orderInvariance, isFirstStep, doPasteBoost, verbose;
	ColorSpace colorSpace;
	Transform transform;
	unsigned sizeSearchWindowPred, nSimilarPatchesPred;
	float dsub;
	bool agg_window;
};
struct Size {
	unsigned width, height, frames, channels;
	Size() : width(0), height(0), frames(0), channels(0) {}
	Size(unsigned w, unsigned h, unsigned f, unsigned c) : width(w), height(h), frames(f), channels(c) {}
};
struct Vid {
	Size sz;
	std::vector<float> data;
	Vid() {}
	explicit Vid(const Size &s) { resize(s); }
	void resize(const Size &s)
	{
		sz = s;
		data.assign((size_t)s.width * s.height * s.frames * s.channels, 0.f);
	}
};
#endif

#include "../include/bm4dof_videonlb.hpp"

namespace L = bm4dof_videonlb;

namespace {

// every field but betaMean, which the reference leaves unset
bool same_params(const Params &a, const Params &b)
{
	const bm4dof_params x = L::to_c(a), y = L::to_c(b);
#define SAME(f) (std::memcmp(&x.f, &y.f, sizeof x.f) == 0)
	return SAME(sigma) && SAME(sizePatch) && SAME(sizePatchTime) && SAME(nSimilarPatches) &&
	       SAME(sizeSearchWindow) && SAME(sizeSearchTimeRangeFwd) && SAME(sizeSearchTimeRangeBwd) &&
	       SAME(boundary) && SAME(offSet) && SAME(offSetTime) && SAME(beta) && SAME(tau) &&
	       SAME(orderInvariance) && SAME(isFirstStep) && SAME(doPasteBoost) && SAME(verbose) && SAME(colorSpace) &&
	       SAME(transform) && SAME(sizeSearchWindowPred) && SAME(nSimilarPatchesPred) && SAME(dsub) &&
	       SAME(agg_window);
#undef SAME
}

struct Case {
	unsigned w, h, f, c;
	float sigma;
	unsigned step, wx, px, np;   // 0: setter not called
};
const Case kCases[] = {
    {256, 256, 1, 1, 20.f, 1, 0, 0, 0},   {256, 256, 1, 1, 45.f, 2, 0, 0, 0},  {854, 480, 20, 1, 20.f, 1, 0, 0, 0},
    {854, 480, 20, 1, 20.f, 2, 21, 4, 16}, {64, 48, 8, 3, 30.f, 1, 15, 5, 24},  {64, 48, 8, 3, 10.f, 2, 9, 6, 0},
    {32, 32, 1, 3, 50.f, 1, 0, 8, 8},
};

int cmd_params()
{
	int bad = 0;
	for (const Case &k : kCases) {
		const Size sz(k.w, k.h, k.f, k.c);
		Params p = Params();
		L::initializeNlbParameters(p, k.step, k.sigma, sz, false);
		if (k.wx) L::setSizeSearchWindow(p, k.wx);
		if (k.px) L::setSizePatch(p, sz, k.px);
		if (k.np) L::setNSimilarPatches(p, k.np);
		L::printNlbParameters(p);
#ifdef WITH_REFERENCE_TYPES
		Params q = Params();
		VideoNLB::initializeNlbParameters(q, k.step, k.sigma, sz, false);
		if (k.wx) VideoNLB::setSizeSearchWindow(q, k.wx);
		if (k.px) VideoNLB::setSizePatch(q, sz, k.px);
		if (k.np) VideoNLB::setNSimilarPatches(q, k.np);
		if (!same_params(p, q)) {
			std::fprintf(stderr, "parameters differ from the reference's: %ux%ux%ux%u sigma %g step %u\n", k.w, k.h,
			             k.f, k.c, k.sigma, k.step);
			bad++;
		}
#endif
	}
	std::fflush(stdout);
	return bad ? 1 : 0;
}

int cmd_roundtrip()
{
	Params a = Params();
	a.sigma = 1.5f;
	a.sizePatch = 2;
	a.sizePatchTime = 3;
	a.nSimilarPatches = 4;
	a.sizeSearchWindow = 5;
	a.sizeSearchTimeRangeFwd = 6;
	a.sizeSearchTimeRangeBwd = 7;
	a.boundary = 8;
	a.offSet = 9;
	a.offSetTime = 10;
	a.beta = 11.5f;
	a.betaMean = 12.5f;
	a.tau = 13.5f;
	a.orderInvariance = true;
	a.isFirstStep = false;
	a.doPasteBoost = true;
	a.verbose = false;
	a.colorSpace = (decltype(a.colorSpace))1;
	a.transform = (decltype(a.transform))1;
	a.sizeSearchWindowPred = 14;
	a.nSimilarPatchesPred = 15;
	a.dsub = 16.5f;
	a.agg_window = true;
	const bm4dof_params c = L::to_c(a);
	const bool fields = c.sigma == 1.5f && c.sizePatch == 2 && c.sizePatchTime == 3 && c.nSimilarPatches == 4 &&
	                    c.sizeSearchWindow == 5 && c.sizeSearchTimeRangeFwd == 6 && c.sizeSearchTimeRangeBwd == 7 &&
	                    c.boundary == 8 && c.offSet == 9 && c.offSetTime == 10 && c.beta == 11.5f &&
	                    c.betaMean == 12.5f && c.tau == 13.5f && c.orderInvariance == 1 && c.isFirstStep == 0 &&
	                    c.doPasteBoost == 1 && c.verbose == 0 && c.colorSpace == BM4DOF_YUV &&
	                    c.transform == BM4DOF_BIOR1_5 && c.sizeSearchWindowPred == 14 &&
	                    c.nSimilarPatchesPred == 15 && c.dsub == 16.5f && c.agg_window == 1;
	Params b = Params();
	L::from_c(c, b);
	const bool back = same_params(a, b) && b.betaMean == 12.5f;
	std::printf("roundtrip %s\n", fields && back ? "ok" : "FAILED");
	return fields && back ? 0 : 1;
}

// one call through the layer (and, with the reference's types, the same call
// to the reference): the message it throws, or "" when it throws nothing
template <class Fn>
std::string message(Fn fn)
{
	try {
		fn();
	} catch (const std::exception &e) {
		return e.what();
	}
	return "";
}

int cmd_errors()
{
	const Size sz(16, 12, 3, 1), sz2(16, 12, 3, 2);
	Params p1 = Params(), p2 = Params();
	L::initializeNlbParameters(p1, 1, 20.f, sz, false);
	L::initializeNlbParameters(p2, 2, 20.f, sz, false);
	Params none1 = p1, none2 = p2;
	none1.sizePatch = none2.sizePatch = 0;
	const Vid noisy(sz), noisy2(Size(16, 12, 3, 2)), flow(sz2), bad_flow(Size(16, 12, 2, 2)), empty;
	struct Input {
		const char *what;
		const Vid *noisy, *fflow, *bflow;
		const Params *p1, *p2;
		Size basic;
	};
	const Input inputs[] = {
	    {"two channels", &noisy2, &empty, &empty, &p1, &p2, Size()},
	    {"forward flow of the wrong length", &noisy, &bad_flow, &flow, &p1, &p2, Size()},
	    {"backward flow of the wrong length", &noisy, &flow, &bad_flow, &p1, &p2, Size()},
	    {"forward flow with one channel", &noisy, &noisy, &flow, &p1, &p2, Size()},
	    {"no step", &noisy, &flow, &flow, &none1, &none2, Size()},
	    {"step 2 with a basic of another size", &noisy, &flow, &flow, &none1, &p2, Size(16, 12, 2, 1)},
	};
	int bad = 0;
	for (const Input &in : inputs) {
		Vid basic(in.basic), fin;
		const std::string m = message([&] {
			L::runNlBayes(*in.noisy, *in.fflow, *in.bflow, basic, fin, *in.p1, *in.p2, 2);
		});
		std::printf("%s: %s\n", in.what, m.c_str());
#ifdef WITH_REFERENCE_TYPES
		Vid rbasic(in.basic), rfin;
		const std::string r = message([&] {
			VideoNLB::runNlBayes(*in.noisy, *in.fflow, *in.bflow, rbasic, rfin, *in.p1, *in.p2);
		});
		const bool same = r == m && rbasic.sz == basic.sz && rfin.sz == fin.sz;
		if (!same) {
			std::fprintf(stderr, "%s: the reference says \"%s\"\n", in.what, r.c_str());
			bad++;
		}
#endif
	}
	std::fflush(stdout);
	return bad ? 1 : 0;
}

struct CropArgs {
	int origin_x, origin_y, origin_t, ending_x, ending_y, ending_t;
	Size source_sz;
};

int cmd_process_errors()
{
	const Size sz(16, 12, 3, 1);
	Params p1 = Params(), p2 = Params();
	L::initializeNlbParameters(p1, 1, 20.f, sz, false);
	L::initializeNlbParameters(p2, 2, 20.f, sz, false);
	const Vid noisy(sz), bad_flow(Size(16, 12, 2, 2)), flow(Size(16, 12, 3, 2)), empty;
	Vid basic, fin, small_basic(Size(16, 12, 2, 1));
	std::printf("flows: %s\n", message([&] { L::processNlBayes(noisy, bad_flow, flow, basic, fin, p1); }).c_str());
	std::printf("basic: %s\n",
	            message([&] { L::processNlBayes(noisy, empty, empty, small_basic, fin, p2); }).c_str());
	std::fflush(stdout);
	return 0;
}

bool read_raw(const char *path, std::vector<float> &v)
{
	FILE *f = std::fopen(path, "rb");
	if (!f) return false;
	const bool ok = std::fread(v.data(), sizeof(float), v.size(), f) == v.size();
	std::fclose(f);
	return ok;
}

bool write_raw(const char *path, const std::vector<float> &v)
{
	FILE *f = std::fopen(path, "wb");
	if (!f) return false;
	const bool ok = std::fwrite(v.data(), sizeof(float), v.size(), f) == v.size();
	return std::fclose(f) == 0 && ok;
}

int cmd_run(char **a)
{
	const Size sz((unsigned)std::atoi(a[0]), (unsigned)std::atoi(a[1]), (unsigned)std::atoi(a[3]),
	              (unsigned)std::atoi(a[2]));
	const float sigma = (float)std::atof(a[4]);
	const unsigned nparts = (unsigned)std::atoi(a[5]);
	Vid noisy(sz), basic, fin;
	const Vid empty;
	if (!read_raw(a[6], noisy.data)) return std::fprintf(stderr, "cannot read %s\n", a[6]), 1;
	Params p1 = Params(), p2 = Params();
	L::initializeNlbParameters(p1, 1, sigma, sz, false);
	L::initializeNlbParameters(p2, 2, sigma, sz, false);
	try {
		const std::vector<float> r = L::runNlBayes(noisy, empty, empty, basic, fin, p1, p2, nparts);
		std::printf("%.6f %.6f\n", r[0], r[1]);
	} catch (const std::exception &e) {
		return std::fprintf(stderr, "%s\n", e.what()), 1;
	}
	return write_raw(a[7], basic.data) && write_raw(a[8], fin.data) ? 0 : 1;
}

int cmd_process(char **a)
{
	const Size sz((unsigned)std::atoi(a[0]), (unsigned)std::atoi(a[1]), (unsigned)std::atoi(a[3]),
	              (unsigned)std::atoi(a[2]));
	const float sigma = (float)std::atof(a[4]);
	CropArgs c;
	int *f[6] = {&c.origin_x, &c.origin_y, &c.origin_t, &c.ending_x, &c.ending_y, &c.ending_t};
	for (int k = 0; k < 6; k++) *f[k] = std::atoi(a[8 + k]);
	c.source_sz = Size((unsigned)std::atoi(a[14]), (unsigned)std::atoi(a[15]), (unsigned)std::atoi(a[16]),
	                   sz.channels);
	Vid noisy(sz), basic, fin;
	const Vid empty;
	if (!read_raw(a[5], noisy.data)) return std::fprintf(stderr, "cannot read %s\n", a[5]), 1;
	Params p1 = Params(), p2 = Params();
	L::initializeNlbParameters(p1, 1, sigma, sz, false);
	L::initializeNlbParameters(p2, 2, sigma, sz, false);
	try {
		const unsigned g1 = L::processNlBayes(noisy, empty, empty, basic, fin, p1, c);
		const unsigned g2 = L::processNlBayes(noisy, empty, empty, basic, fin, p2, c);
		std::printf("%u %u\n", g1, g2);
	} catch (const std::exception &e) {
		return std::fprintf(stderr, "%s\n", e.what()), 1;
	}
	return write_raw(a[6], basic.data) && write_raw(a[7], fin.data) ? 0 : 1;
}

}  // namespace

int main(int argc, char **argv)
{
	const std::string c = argc > 1 ? argv[1] : "";
	if (c == "params") return cmd_params();
	if (c == "roundtrip") return cmd_roundtrip();
	if (c == "errors") return cmd_errors();
	if (c == "process_errors") return cmd_process_errors();
	if (c == "tiles") return std::printf("%u\n", L::default_tiles()), 0;
	if (c == "run" && argc == 11) return cmd_run(argv + 2);
	if (c == "process" && argc == 19) return cmd_process(argv + 2);
	std::fprintf(stderr, "usage: videonlb_layer params|roundtrip|errors|process_errors|run|process ...\n");
	return 2;
}
