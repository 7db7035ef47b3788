// psnr_cli.cpp -- the psnr command line (host code, no GPU).
//
// Mirrors the reference's src/psnr.cpp:17-75, which scripts/bm4dof-gt.sh runs
// on the denoised and basic sequences:
//
//   psnr input1-path input2-path [first-frame last-frame [output-file]]
//
// Prints the global PSNR and RMSE and, with an output file, appends the global
// and per-frame figures in the reference's format.  RMSE and PSNR follow
// VideoUtils::computePSNR (src/utils/lib_videot.hpp:517-566): squared
// differences summed in double, RMSE = sqrtf(sum / n), PSNR =
// 20 log10f(255 / RMSE), globally and per frame.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "frames.hpp"

namespace {

float rmse_of(const float *a, const float *b, size_t n)
{
	double sum = 0.0;
	for (size_t k = 0; k < n; k++) sum += ((double)a[k] - (double)b[k]) * ((double)a[k] - (double)b[k]);
	return sqrtf((float)(sum / (double)n));
}

float psnr_of(float rmse) { return 20.f * log10f(255.f / rmse); }

}  // namespace

int main(int argc, char **argv)
{
	if (argc != 3 && argc != 5 && argc != 6)
		return std::printf("Compute PSNR and RMSE between two image sequences\n\n"
		                   "USAGE: psnr input1-path input2-path [first-frame last-frame [output-file]]\n\n"
		                   "- Paths for video frames have to be given in printf format\n"
		                   "- First and last frame if not provided are set to zero (for an image)\n"
		                   "- It prints to standard output the global PSNR and RMSE\n"
		                   "- If an output filename is given, it appends to it the global and per-frame PSNR "
		                   "and RMSE\n"),
		       EXIT_FAILURE;
	const std::string p1(argv[1]), p2(argv[2]);
	const int first = argc > 3 ? std::atoi(argv[3]) : 0;
	const int last = argc > 4 ? std::atoi(argv[4]) : 0;
	std::string out_path = argc > 5 ? argv[5] : "";
	if (p1.empty() || p2.empty())
		return std::fprintf(stderr, "%s: input sequence missing.\nTry `%s' for more information.\n", argv[0],
		                    argv[0]),
		       EXIT_FAILURE;

	bm4dof_frames::Video a, b;
	std::string err;
	if (!bm4dof_frames::load_video(p1, (unsigned)first, (unsigned)last, 1, a, err) ||
	    !bm4dof_frames::load_video(p2, (unsigned)first, (unsigned)last, 1, b, err))
		return std::fprintf(stderr, "%s\n", err.c_str()), EXIT_FAILURE;
	if (a.w != b.w || a.h != b.h || a.c != b.c || a.f != b.f)
		return std::fprintf(stderr, "VideoUtils::computePSNR: videos have different sizes\n"), EXIT_FAILURE;

	const float rmse = rmse_of(a.data.data(), b.data.data(), a.data.size());
	const float psnr = psnr_of(rmse);
	const size_t whc = (size_t)a.w * a.h * a.c;
	std::vector<float> frame_psnr(a.f), frame_rmse(a.f);
	for (unsigned t = 0; t < a.f; t++) {
		frame_rmse[t] = rmse_of(a.data.data() + t * whc, b.data.data() + t * whc, whc);
		frame_psnr[t] = psnr_of(frame_rmse[t]);
	}
	std::printf("PSNR %f\nRMSE %f\n", psnr, rmse);

	if (!out_path.empty()) {
		if (out_path == "-") out_path = "stdout";   // a file named stdout, as the reference does
		FILE *f = std::fopen(out_path.c_str(), "a");
		if (!f) return std::fprintf(stderr, "cannot open %s\n", out_path.c_str()), EXIT_FAILURE;
		std::fprintf(f, "Total PSNR %f\nTotal RMSE %f", psnr, rmse);
		if (last > first) {
			std::fprintf(f, "\nFrame PSNR");
			for (float x : frame_psnr) std::fprintf(f, " %f", x);
			std::fprintf(f, "\nFrame RMSE ");
			for (float x : frame_rmse) std::fprintf(f, " %f", x);
		}
		std::fprintf(f, "\n");
		std::fclose(f);
	}
	return EXIT_SUCCESS;
}
