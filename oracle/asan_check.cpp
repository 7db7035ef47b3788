/*
 * asan_check.cpp -- TEST INFRASTRUCTURE ONLY.
 *
 * Runs the oracle restatement (bm4dof_oracle.cpp, linked in) on small seeded
 * videos in every mode it restates -- grey and colour, one to six tiles, with
 * and without flow, order-invariant filtering, the paste trick and the
 * predictive (VBM3D_SEARCH) search -- so that a build with
 * -fsanitize=address,undefined checks its memory accesses.  Exits 0 when every
 * run succeeds.  Built and run by tests/test_oracle_asan.py:
 *     g++ -std=c++17 -O1 -g -fsanitize=address,undefined -ffp-contract=off \
 *         oracle/asan_check.cpp oracle/bm4dof_oracle.cpp -o asan_check
 */
#include <cmath>
#include <cstdio>
#include <cstdint>
#include <vector>

#include "../include/bm4dof.h"

extern "C" {
struct oracle_trace;
void oracle_initialize_params(bm4dof_params *p, unsigned step, float sigma, const bm4dof_video_size *sz,
                              int verbose);
void oracle_set_size_search_window(bm4dof_params *p, unsigned wx);
void oracle_set_size_patch(bm4dof_params *p, const bm4dof_video_size *sz, unsigned px);
void oracle_set_n_similar_patches(bm4dof_params *p, unsigned np);
int oracle_run_ex(const float *noisy, const float *fflow, const float *bflow, unsigned W, unsigned H, unsigned C,
                  unsigned F, float *basic, float *final_, const bm4dof_params *p1, const bm4dof_params *p2,
                  unsigned nparts, unsigned nthreads, unsigned flags, float ratios[2], oracle_trace *trace,
                  char *err, size_t errlen);
}

namespace {

uint32_t lcg(uint32_t &s)
{
	s = s * 1664525u + 1013904223u;
	return s >> 8;
}

struct Case {
	unsigned W, H, F, C, px, pt, wx, np, nparts;
	bool flow, order_inv, paste, vbm3d;
};

int run(const Case &k, uint32_t seed)
{
	const size_t n = (size_t)k.W * k.H * k.F * k.C, nf = (size_t)k.W * k.H * k.F * 2;
	std::vector<float> noisy(n), ff(nf), bf(nf), basic(n), fin(n);
	for (size_t i = 0; i < n; i++) {
		const size_t x = i % k.W, y = (i / k.W) % k.H;
		noisy[i] = 120.f + 60.f * std::sin(0.3f * x + 0.2f * y) + (float)(lcg(seed) % 4000) / 100.f - 20.f;
	}
	for (size_t i = 0; i < nf; i++) {
		ff[i] = (float)(lcg(seed) % 300) / 100.f - 1.5f;
		bf[i] = -ff[i];
	}
	bm4dof_video_size sz = {k.W, k.H, k.F, k.C};
	bm4dof_params p1, p2;
	oracle_initialize_params(&p1, 1, 20.f, &sz, 0);
	oracle_initialize_params(&p2, 2, 20.f, &sz, 0);
	oracle_set_size_search_window(&p1, k.wx);
	oracle_set_size_search_window(&p2, k.wx);
	oracle_set_size_patch(&p1, &sz, k.px);
	oracle_set_size_patch(&p2, &sz, k.px);
	oracle_set_n_similar_patches(&p1, k.np);
	oracle_set_n_similar_patches(&p2, k.np);
	p1.sizePatchTime = p2.sizePatchTime = k.pt;
	p1.beta = p1.betaMean = 3.f;
	p1.orderInvariance = p2.orderInvariance = k.order_inv;
	p1.doPasteBoost = p2.doPasteBoost = k.paste;
	float ratios[2];
	char err[256] = {0};
	const int rc = oracle_run_ex(noisy.data(), k.flow ? ff.data() : nullptr, k.flow ? bf.data() : nullptr, k.W, k.H,
	                             k.C, k.F, basic.data(), fin.data(), &p1, &p2, k.nparts, 1,
	                             k.vbm3d ? BM4DOF_VBM3D_SEARCH : 0u, ratios, nullptr, err, sizeof(err));
	std::printf("%ux%ux%ux%u px%u pt%u wx%u np%u tiles%u flow%d oinv%d paste%d vbm3d%d: rc %d %s ratios %.3f %.3f\n",
	            k.W, k.H, k.F, k.C, k.px, k.pt, k.wx, k.np, k.nparts, k.flow, k.order_inv, k.paste, k.vbm3d, rc,
	            err, ratios[0], ratios[1]);
	return rc;
}

}  // namespace

int main()
{
	const Case cases[] = {
	    {34, 30, 5, 1, 4, 4, 11, 16, 2, true, false, false, false},
	    {34, 30, 5, 1, 4, 4, 11, 16, 2, true, false, false, true},
	    {34, 30, 5, 1, 4, 4, 11, 16, 2, true, false, true, false},
	    {34, 30, 5, 1, 4, 4, 11, 16, 2, true, false, true, true},
	    {34, 30, 5, 1, 4, 4, 11, 16, 2, false, true, false, true},
	    {30, 26, 4, 3, 4, 2, 9, 8, 4, true, false, true, true},
	    {40, 36, 1, 1, 8, 1, 15, 16, 6, false, false, false, true},
	    {40, 36, 6, 1, 8, 1, 7, 8, 2, true, true, true, false},
	};
	int bad = 0;
	uint32_t seed = 12345u;
	for (const Case &k : cases) bad |= run(k, seed++);
	return bad ? 1 : 0;
}
