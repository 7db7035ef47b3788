// awgn_cli.cpp -- the awgn command line (host code, no GPU).
//
// Mirrors the reference's src/awgn.cpp:17-48, which scripts/bm4dof-gt.sh runs
// before the denoiser:
//
//   awgn sigma input-path output-path [first-frame last-frame]
//
// Loads the frames, adds white Gaussian noise of standard deviation sigma as
// VideoUtils::addNoise does (src/utils/lib_videot.hpp:481-505) and saves them
// under the output pattern (no clipping).  The generator is MT19937
// (Matsumoto and Nishimura, 1998) with 53-bit uniform doubles, seeded from
// the time and the process id like the reference; each sample is
// sigma * sqrt(-2 ln a) * cos(2 pi b) for two consecutive uniforms a, b, in
// long double.  BM4DOF_AWGN_SEED=<n> seeds the generator with n instead (no
// counterpart in the reference: reproducible noise for tests).
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <ctime>
#include <string>
#include <vector>

#include <unistd.h>

#include "frames.hpp"

namespace {

// MT19937, restated from the published description: 624-word state, the
// linear recurrence with twist matrix constant 0x9908b0df, and the tempering
// shifts and masks of the paper.
class Mt19937 {
public:
	explicit Mt19937(uint32_t seed)
	{
		s_[0] = seed;
		for (int i = 1; i < kN; i++) s_[i] = 1812433253u * (s_[i - 1] ^ (s_[i - 1] >> 30)) + (uint32_t)i;
		i_ = kN;
	}
	uint32_t next()
	{
		if (i_ >= kN) refill();
		uint32_t y = s_[i_++];
		y ^= y >> 11;
		y ^= (y << 7) & 0x9d2c5680u;
		y ^= (y << 15) & 0xefc60000u;
		y ^= y >> 18;
		return y;
	}
	// a uniform double in [0, 1) from 27 + 26 random bits
	double res53()
	{
		const uint32_t a = next() >> 5, b = next() >> 6;
		return ((double)a * 67108864.0 + (double)b) / 9007199254740992.0;
	}

private:
	static const int kN = 624, kM = 397;
	uint32_t s_[kN];
	int i_;
	void refill()
	{
		for (int k = 0; k < kN; k++) {
			const uint32_t y = (s_[k] & 0x80000000u) | (s_[(k + 1) % kN] & 0x7fffffffu);
			s_[k] = s_[(k + kM) % kN] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
		}
		i_ = 0;
	}
};

}  // namespace

int main(int argc, char **argv)
{
	if (argc != 4 && argc != 6)
		return std::printf("Add additive white Gaussian noise to an image sequence\n\n"
		                   "USAGE: awgn sigma input-path output-path [first-frame last-frame]\n\n"
		                   "- Paths for video frames have to be given in printf format.\n"
		                   "- First and last frame if not provided are set to zero (for an image)\n"),
		       EXIT_FAILURE;
	const float sigma = (float)std::atof(argv[1]);
	const std::string input_path(argv[2]), noisy_path(argv[3]);
	const int first = argc > 4 ? std::atoi(argv[4]) : 0;
	const int last = argc > 5 ? std::atoi(argv[5]) : 0;
	if (input_path.empty())
		return std::fprintf(stderr, "%s: no input sequence.\nTry `%s' for more information.\n", argv[0], argv[0]),
		       EXIT_FAILURE;
	if (noisy_path.empty())
		return std::fprintf(stderr, "%s: no output sequence.\nTry `%s' for more information.\n", argv[0], argv[0]),
		       EXIT_FAILURE;

	bm4dof_frames::Video v;
	std::string err;
	if (!bm4dof_frames::load_video(input_path, (unsigned)first, (unsigned)last, 1, v, err))
		return std::fprintf(stderr, "%s\n", err.c_str()), EXIT_FAILURE;
	const char *fixed = std::getenv("BM4DOF_AWGN_SEED");
	const uint32_t seed = fixed ? (uint32_t)std::strtoul(fixed, nullptr, 10)
	                            : (uint32_t)((unsigned long)std::time(nullptr) + (unsigned long)getpid());
	Mt19937 mt(seed);
	for (float &x : v.data) {
		const double a = mt.res53();
		const double b = mt.res53();
		x += (float)(sigma * std::sqrt(-2.0L * std::log(a)) * std::cos(2.0L * M_PI * b));
	}
	if (!bm4dof_frames::save_video(noisy_path, (unsigned)first, 1, v, err))
		return std::fprintf(stderr, "%s\n", err.c_str()), EXIT_FAILURE;
	return EXIT_SUCCESS;
}
