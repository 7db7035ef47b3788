// tvl1_cli.cpp -- the tvl1flow command line over the GPU library.
//
// Mirrors the reference's lib/tvl1flow/main.c:72-199, which its
// scripts/tvl1flow-seq.sh runs once per frame pair:
//
//   tvl1flow I0 I1 [out nproc tau lambda theta nscales fscale zfactor nwarps
//                   epsilon verbose]
//
// with the same positional arguments, defaults, parameter checks and their
// warnings, scale cap and messages.  The flow of the pair is computed by
// bm4dof_tvl1_pairs on the GPU; nproc (the reference's OpenMP thread count) is
// checked and otherwise unused.  The images are read as iio_read_image_float
// reads them (colour reduced to grey, frames.hpp); the flow is written as
// Middlebury .flo, or as a two-channel float TIFF when out ends in .tif/.tiff.
// The GPU is touched only after both images have been read and checked.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "../../include/bm4dof.h"
#include "frames.hpp"

namespace {

// main.c:24-34
constexpr const char *kOutFlow = "flow.flo";
constexpr int kNproc = 0, kNscales = 100, kFscale = 0, kNwarps = 5, kVerbose = 0;
constexpr float kTau = 0.25f, kLambda = 0.15f, kTheta = 0.3f, kZfactor = 0.5f, kEpsilon = 0.01f;

bool read_image(const char *path, std::vector<float> &img, int &w, int &h)
{
	std::string why;
	if (bm4dof_frames::read_grey(path, img, w, h, why)) return true;
	std::fprintf(stderr, "ERROR: could not read image from file \"%s\" (%s)\n", path, why.c_str());
	return false;
}

}  // namespace

int main(int argc, char *argv[])
{
	if (argc < 3) {
		std::fprintf(stderr,
		             "Usage: %s I0 I1 [out nproc tau lambda theta nscales fscale zfactor nwarps epsilon verbose]\n",
		             *argv);
		return EXIT_FAILURE;
	}
	int i = 1;
	const char *image1 = argv[i++];
	const char *image2 = argv[i++];
	const char *outfile = argc > i ? argv[i] : kOutFlow;              i++;
	int nproc = argc > i ? std::atoi(argv[i]) : kNproc;               i++;
	float tau = argc > i ? (float)std::atof(argv[i]) : kTau;          i++;
	float lambda = argc > i ? (float)std::atof(argv[i]) : kLambda;    i++;
	float theta = argc > i ? (float)std::atof(argv[i]) : kTheta;      i++;
	int nscales = argc > i ? std::atoi(argv[i]) : kNscales;           i++;
	int fscale = argc > i ? std::atoi(argv[i]) : kFscale;             i++;
	float zfactor = argc > i ? (float)std::atof(argv[i]) : kZfactor;  i++;
	int nwarps = argc > i ? std::atoi(argv[i]) : kNwarps;             i++;
	float epsilon = argc > i ? (float)std::atof(argv[i]) : kEpsilon;  i++;
	const int verbose = argc > i ? std::atoi(argv[i]) : kVerbose;     i++;

	// main.c:101-140
	if (nproc < 0) {
		nproc = kNproc;
		if (verbose) std::fprintf(stderr, "warning: nproc changed to %d\n", nproc);
	}
	if (tau <= 0 || tau > 0.25) {
		tau = kTau;
		if (verbose) std::fprintf(stderr, "warning: tau changed to %g\n", tau);
	}
	if (lambda <= 0) {
		lambda = kLambda;
		if (verbose) std::fprintf(stderr, "warning: lambda changed to %g\n", lambda);
	}
	if (theta <= 0) {
		theta = kTheta;
		if (verbose) std::fprintf(stderr, "warning: theta changed to %g\n", theta);
	}
	if (nscales <= 0) {
		nscales = kNscales;
		if (verbose) std::fprintf(stderr, "warning: nscales changed to %d\n", nscales);
	}
	if (zfactor <= 0 || zfactor >= 1) {
		zfactor = kZfactor;
		if (verbose) std::fprintf(stderr, "warning: zfactor changed to %g\n", zfactor);
	}
	if (nwarps <= 0) {
		nwarps = kNwarps;
		if (verbose) std::fprintf(stderr, "warning: nwarps changed to %d\n", nwarps);
	}
	if (epsilon <= 0) {
		epsilon = kEpsilon;
		if (verbose) std::fprintf(stderr, "warning: epsilon changed to %f\n", epsilon);
	}

	int nx = 0, ny = 0, nx2 = 0, ny2 = 0;
	std::vector<float> I0, I1;
	const bool ok0 = read_image(image1, I0, nx, ny);
	const bool ok1 = read_image(image2, I1, nx2, ny2);
	if (!ok0 || !ok1) return EXIT_FAILURE;
	if (nx != nx2 || ny != ny2) {
		std::fprintf(stderr, "ERROR: input images size mismatch %dx%d != %dx%d\n", nx, ny, nx2, ny2);
		return EXIT_FAILURE;
	}
	if (nx < 2 || ny < 2) {
		std::fprintf(stderr, "ERROR: input images are %dx%d, at least 2x2 is needed\n", nx, ny);
		return EXIT_FAILURE;
	}

	// main.c:147-153: the coarsest level stays about 16 pixels across
	const float N = (float)(1 + std::log(std::hypot(nx, ny) / 16.0) / std::log(1 / zfactor));
	if (N < nscales) nscales = (int)N;
	if (nscales < 1) nscales = 1;   // images under about 16 pixels across: one level
	if (nscales < fscale) fscale = nscales;
	if (verbose) {
		std::fprintf(stderr, "nproc=%d tau=%f lambda=%f theta=%f nscales=%d zfactor=%f nwarps=%d epsilon=%g\n",
		             nproc, tau, lambda, theta, nscales, zfactor, nwarps, epsilon);
		// the levels computed, coarsest first (tvl1flow_lib.c:387-413; zoom.c:34-35)
		std::vector<int> wx(1, nx), hy(1, ny);
		for (int s = 1; s < nscales; s++) {
			wx.push_back((int)((float)wx[s - 1] * zfactor + 0.5));
			hy.push_back((int)((float)hy[s - 1] * zfactor + 0.5));
		}
		for (int s = nscales - 1; s >= fscale; s--) std::fprintf(stderr, "Scale %d: %dx%d\n", s, wx[s], hy[s]);
	}

	bm4dof_tvl1_params p;
	bm4dof_tvl1_default_params(&p);
	p.tau = tau;
	p.lambda = lambda;
	p.theta = theta;
	p.nscales = nscales;
	p.fscale = fscale;
	p.zfactor = zfactor;
	p.warps = nwarps;
	p.epsilon = epsilon;
	std::vector<float> uv((size_t)2 * nx * ny);
	bm4dof_ctx *ctx = nullptr;
	if (bm4dof_create(&ctx, 0) != BM4DOF_OK)
		return std::fprintf(stderr, "%s\n", bm4dof_last_error()), EXIT_FAILURE;
	const bm4dof_status s =
	    bm4dof_tvl1_pairs(ctx, I0.data(), I1.data(), (unsigned)nx, (unsigned)ny, 1, &p, uv.data(), 0);
	bm4dof_destroy(ctx);
	if (s != BM4DOF_OK) return std::fprintf(stderr, "%s\n", bm4dof_last_error()), EXIT_FAILURE;

	if (!bm4dof_frames::write_flow(outfile, uv.data(), nx, ny)) {
		std::fprintf(stderr, "ERROR: could not write the flow to \"%s\"\n", outfile);
		return EXIT_FAILURE;
	}
	return EXIT_SUCCESS;
}
