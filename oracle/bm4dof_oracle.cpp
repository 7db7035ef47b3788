/*
 * bm4dof_oracle.cpp -- TEST INFRASTRUCTURE ONLY.
 *
 * A CPU restatement of the BM4D-OF / NL-DCT denoising path of pariasm/bm4d-of,
 * used as the checker of the GPU library.  Only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline leg load it; the product never calls it.
 *
 * Every function cites the reference file:line it restates (paths relative to
 * the reference project root).  The arithmetic keeps the reference's operation
 * order and its float/double mix so that results are bit-identical to the
 * reference compiled with -ffp-contract=off and the project's sequential
 * sgemm (oracle/ref_sgemm.c).  Parity pinning: tests compare this file's
 * output with the reference itself (oracle/_ref, built from the reference
 * sources by `make -C oracle ref`, also with its VBM3D_SEARCH switch) and
 * with fixtures under tests/golden/.
 *
 * Build: g++ -std=c++17 -O3 -ffp-contract=off -fopenmp -shared -fPIC
 */
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <utility>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/bm4dof.h"

namespace {

/* ------------------------------------------------------------------------ */
/* Video container: planar t*whc + c*wh + y*w + x (lib_videot.hpp:40-181).   */
/* ------------------------------------------------------------------------ */
struct Vid {
	unsigned w = 0, h = 0, f = 0, c = 0;
	std::vector<float> d;
	Vid() {}
	Vid(unsigned W, unsigned H, unsigned F, unsigned C, float v = 0.f)
		: w(W), h(H), f(F), c(C), d((size_t)W * H * F * C, v) {}
	unsigned wh() const { return w * h; }
	unsigned whc() const { return w * h * c; }
	unsigned whf() const { return w * h * f; }
	float &at(unsigned x, unsigned y, unsigned t, unsigned ch = 0) {
		return d[(size_t)t * whc() + (size_t)ch * wh() + (size_t)y * w + x];
	}
	float at(unsigned x, unsigned y, unsigned t, unsigned ch = 0) const {
		return d[(size_t)t * whc() + (size_t)ch * wh() + (size_t)y * w + x];
	}
	bool empty() const { return w == 0; }
};

/* ------------------------------------------------------------------------ */
/* Parameters (nldct.cpp:81-210).                                            */
/* ------------------------------------------------------------------------ */
void init_params(bm4dof_params &p, unsigned step, float sigma, unsigned frames, int verbose)
{
	/* nldct.cpp:81-148 */
	std::memset(&p, 0, sizeof(p));
	const bool s1 = (step == 1);
	if (frames == 1) {
		if (sigma <= 40) {
			p.sizePatch = 8;
			p.nSimilarPatches = s1 ? 16 : 32;
			p.offSet = 3;
			p.beta = s1 ? 2.7f : 1.f;
			p.tau = s1 ? 54.8f : 20.f;
		} else {
			p.sizePatch = s1 ? 8 : 11;
			p.nSimilarPatches = 32;
			p.offSet = s1 ? 4 : 6;
			p.beta = s1 ? 2.8f : 1.f;
			p.tau = s1 ? 158.f : 59.2f;
		}
		p.sizePatchTime = 1;
		p.sizeSearchTimeRangeFwd = 0;
		p.sizeSearchTimeRangeBwd = 0;
		p.sizeSearchWindowPred = 0;
		p.offSetTime = 1;
		p.dsub = 0;
		p.nSimilarPatchesPred = p.nSimilarPatches;
		p.sizeSearchWindow = 39;
	} else {
		p.sizePatch = (s1 || sigma >= 30) ? 8 : 7;
		p.sizePatchTime = 1;
		p.nSimilarPatches = 8;
		p.sizeSearchWindow = 7;
		p.sizeSearchWindowPred = 5;
		p.sizeSearchTimeRangeFwd = 4;
		p.sizeSearchTimeRangeBwd = 4;
		p.nSimilarPatchesPred = 2;
		p.offSet = s1 ? 6 : 4;
		p.offSetTime = 1;
		p.beta = s1 ? 2.7f : 1.f;
		p.tau = s1 ? 67.1f : 54.8f;
		p.dsub = s1 ? 7.f : 3.f;
	}
	p.betaMean = p.beta;
	p.orderInvariance = 0;
	p.isFirstStep = s1;
	p.sigma = sigma;
	p.verbose = verbose;
	p.colorSpace = BM4DOF_YUV;
	p.doPasteBoost = 0;
	p.agg_window = 1;
	p.boundary = 2 * (p.sizeSearchWindow / 2) + (p.sizePatch - 1);
	p.transform = s1 ? BM4DOF_BIOR1_5 : BM4DOF_DCT;
}

void set_search_window(bm4dof_params &p, unsigned wx)
{
	/* nldct.cpp:160-168 */
	p.sizeSearchWindow = wx;
	p.boundary = 2 * (wx / 2) + (p.sizePatch - 1);
	p.nSimilarPatches = std::min(p.nSimilarPatches,
		wx * wx * (p.sizeSearchTimeRangeFwd + p.sizeSearchTimeRangeBwd + 1));
}

void set_patch_size(bm4dof_params &p, unsigned frames, unsigned px)
{
	/* nldct.cpp:179-188; (float)px/4.*3. is a double, truncated to unsigned */
	p.sizePatch = px;
	p.boundary = 2 * (p.sizeSearchWindow / 2) + (p.sizePatch - 1);
	if (p.sizePatch != 8) p.transform = BM4DOF_DCT;
	if (frames > 1)
		p.offSet = p.isFirstStep ? (unsigned)((double)(float)px / 4. * 3.) : px / 2;
}

void set_n_similar(bm4dof_params &p, unsigned np)
{
	/* nldct.cpp:199-210 (the Fwd+Fwd test is the reference's) */
	p.nSimilarPatches = std::min(np, p.sizeSearchWindow * p.sizeSearchWindow *
		(p.sizeSearchTimeRangeFwd + p.sizeSearchTimeRangeBwd + 1));
	if (p.sizeSearchTimeRangeFwd + p.sizeSearchTimeRangeFwd == 0)
		p.nSimilarPatchesPred = p.nSimilarPatches;
}

int format_params(const bm4dof_params &p, char *buf, size_t len)
{
	/* nldct.cpp:219-249: Bwd is printed on both sides of the temporal window */
	const int px = p.sizePatch, pt = p.sizePatchTime;
	const int wtb = p.sizeSearchTimeRangeBwd, wtf = p.sizeSearchTimeRangeBwd;
	const int wx = p.sizeSearchWindow;
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
		p.isFirstStep ? 1 : 2, px, px, pt, (int)p.nSimilarPatches, wx, wx, wtb, wtf,
		(double)p.tau, p.transform == BM4DOF_DCT ? "dct" : "bior1.5", (double)p.beta,
		p.orderInvariance ? "yes" : "no", (int)p.offSet,
		p.doPasteBoost ? "active" : "inactive", p.agg_window ? "yes" : "no");
}

/* ------------------------------------------------------------------------ */
/* Tiling (utilities.cpp:137-158, lib_videot.hpp:853-916, 1101-1163).        */
/* ------------------------------------------------------------------------ */
void determine_factor(unsigned n, unsigned &a, unsigned &b)
{
	if (n == 1) { a = 1; b = 1; return; }
	b = 2;
	while (n % b > 0) b++;
	a = n / b;
	if (b > a) { a = b; b = n / a; }
}

struct Crop {
	int ox, oy, ex, ey;   /* crop box [ox,ex) x [oy,ey), all frames */
	bool bx0, by0, bx1, by1;
	bool bt0 = false, bt1 = false;   /* temporal borders: processNlBayes alone */
};

void tile_grid(unsigned W, unsigned H, unsigned nparts, int &nW, int &nH, int &wTmp, int &hTmp)
{
	unsigned a, b;
	determine_factor(nparts, a, b);
	nW = (int)a; nH = (int)b;
	wTmp = (int)std::ceil(float(W) / float(nW));
	hTmp = (int)std::ceil(float(H) / float(nH));
}

std::vector<Crop> tile_crops(unsigned W, unsigned H, unsigned nparts, int N)
{
	/* lib_videot.hpp:853-916 (subDivideTight) */
	int nW, nH, wTmp, hTmp;
	tile_grid(W, H, nparts, nW, nH, wTmp, hTmp);
	std::vector<Crop> cr;
	for (int p = 0; p < nH; p++)
		for (int q = 0; q < nW; q++) {
			Crop c;
			c.ox = std::max(0, q * wTmp - N);
			c.oy = std::max(0, p * hTmp - N);
			c.ex = std::min((int)W, (q + 1) * wTmp + N);
			c.ey = std::min((int)H, (p + 1) * hTmp + N);
			/* processNlBayes border flags, nldct.cpp:520-525 */
			c.bx0 = c.ox > 0; c.by0 = c.oy > 0;
			c.bx1 = c.ex < (int)W; c.by1 = c.ey < (int)H;
			cr.push_back(c);
		}
	return cr;
}

Vid crop_video(const Vid &v, const Crop &c)
{
	Vid o((unsigned)(c.ex - c.ox), (unsigned)(c.ey - c.oy), v.f, v.c);
	for (unsigned t = 0; t < v.f; t++)
		for (unsigned ch = 0; ch < v.c; ch++)
			for (unsigned y = 0; y < o.h; y++)
				for (unsigned x = 0; x < o.w; x++)
					o.at(x, y, t, ch) = v.at(x + c.ox, y + c.oy, t, ch);
	return o;
}

void build_tight(const std::vector<Vid> &sub, Vid &out, unsigned nparts, int N)
{
	/* lib_videot.hpp:1101-1163 (subBuildTight) */
	int nW, nH, wTmp, hTmp;
	tile_grid(out.w, out.h, nparts, nW, nH, wTmp, hTmp);
	for (int p = 0, n = 0; p < nH; p++)
		for (int q = 0; q < nW; q++, n++) {
			const int cox = std::max(0, q * wTmp - N), coy = std::max(0, p * hTmp - N);
			const int ox = q * wTmp, oy = p * hTmp;
			const int ex = std::min((q + 1) * wTmp, (int)out.w);
			const int ey = std::min((p + 1) * hTmp, (int)out.h);
			for (unsigned t = 0; t < out.f; t++)
				for (unsigned ch = 0; ch < out.c; ch++)
					for (int sy = oy - coy, qy = oy; qy < ey; sy++, qy++)
						for (int sx = ox - cox, qx = ox; qx < ex; sx++, qx++)
							out.at(qx, qy, t, ch) = sub[n].at(sx, sy, t, ch);
		}
}

/* ------------------------------------------------------------------------ */
/* Colour transform (lib_videot.hpp:727-838).                                */
/* ------------------------------------------------------------------------ */
void color_transform(Vid &v, bool forward)
{
	if (v.c == 1) return;
	const unsigned wh = v.wh();
	for (unsigned f = 0; f < v.f; f++) {
		float *base = v.d.data() + (size_t)f * v.whc();
		if (forward) {
			if (v.c == 3) {
				float *r = base, *g = base + wh, *b = base + 2 * wh;
				const float a = 1.f / sqrtf(3.f);
				const float bb = 1.f / sqrtf(2.f);
				const float c = 2.f * a * sqrtf(2.f);
				for (unsigned k = 0; k < wh; k++) {
					const float y0 = a * (r[k] + g[k] + b[k]);
					const float y1 = bb * (r[k] - b[k]);
					const float y2 = c * (0.25f * r[k] - 0.5f * g[k] + 0.25f * b[k]);
					r[k] = y0; g[k] = y1; b[k] = y2;
				}
			} else {
				float *Gr = base, *R = base + wh, *B = base + 2 * wh, *Gb = base + 3 * wh;
				const float a = 0.5f;
				const float bb = 1.f / sqrtf(2.f);
				for (unsigned k = 0; k < wh; k++) {
					const float w0 = a * (Gr[k] + R[k] + B[k] + Gb[k]);
					const float w1 = bb * (R[k] - B[k]);
					const float w2 = a * (-Gr[k] + R[k] + B[k] - Gb[k]);
					const float w3 = bb * (-Gr[k] + Gb[k]);
					Gr[k] = w0; R[k] = w1; B[k] = w2; Gb[k] = w3;
				}
			}
		} else {
			if (v.c == 3) {
				float *r = base, *g = base + wh, *b = base + 2 * wh;
				const float a = 1.f / sqrtf(3.f);
				const float bb = 1.f / sqrtf(2.f);
				const float c = a / bb;
				for (unsigned k = 0; k < wh; k++) {
					const float o0 = a * r[k] + bb * g[k] + c * 0.5f * b[k];
					const float o1 = a * r[k] - c * b[k];
					const float o2 = a * r[k] - bb * g[k] + c * 0.5f * b[k];
					r[k] = o0; g[k] = o1; b[k] = o2;
				}
			} else {
				float *Gr = base, *R = base + wh, *B = base + 2 * wh, *Gb = base + 3 * wh;
				const float a = 0.5f;
				const float bb = 1.f / sqrtf(2.f);
				for (unsigned k = 0; k < wh; k++) {
					const float w0 = a * Gr[k] - a * B[k] - bb * Gb[k];
					const float w1 = a * Gr[k] + bb * R[k] + a * B[k];
					const float w2 = a * Gr[k] - bb * R[k] + a * B[k];
					const float w3 = a * Gr[k] - a * B[k] + bb * Gb[k];
					Gr[k] = w0; R[k] = w1; B[k] = w2; Gb[k] = w3;
				}
			}
		}
	}
}

/* ------------------------------------------------------------------------ */
/* Patch bases and aggregation window (nldct.cpp:572-737).                   */
/* ------------------------------------------------------------------------ */
const double kBior15Fwd[64] = {
	/* nldct.cpp:640-647: 1-D bior1.5 analysis rows for length 8 */
	0.353553390593274, 0.353553390593274, 0.353553390593274, 0.353553390593274,
	0.353553390593274, 0.353553390593274, 0.353553390593274, 0.353553390593274,
	0.219417649252501, 0.449283757993216, 0.449283757993216, 0.219417649252501,
	-0.219417649252501, -0.449283757993216, -0.449283757993216, -0.219417649252501,
	0.569359398342846, 0.402347308162278, -0.402347308162278, -0.569359398342846,
	-0.083506045090284, 0.083506045090284, -0.083506045090284, 0.083506045090284,
	-0.083506045090284, 0.083506045090284, -0.083506045090284, 0.083506045090284,
	0.569359398342846, 0.402347308162278, -0.402347308162278, -0.569359398342846,
	0.707106781186547, -0.707106781186547, 0, 0, 0, 0, 0, 0,
	0, 0, 0.707106781186547, -0.707106781186547, 0, 0, 0, 0,
	0, 0, 0, 0, 0.707106781186547, -0.707106781186547, 0, 0,
	0, 0, 0, 0, 0, 0, 0.707106781186547, -0.707106781186547};

const double kBior15Inv[64] = {
	/* nldct.cpp:670-677: 1-D bior1.5 synthesis table for length 8 */
	0.353553390593274, 0.353553390593274, 0.5, 0.0, 0.707106781186547, -0.121533978016438, -0.000000000000000, 0.121533978016438,
	0.353553390593274, 0.353553390593274, 0.5, -0.0, -0.707106781186547, -0.121533978016438, 0.000000000000000, 0.121533978016438,
	0.353553390593274, 0.353553390593274, -0.5, -0.0, 0.121533978016438, 0.707106781186548, -0.121533978016438, 0.000000000000000,
	0.353553390593274, 0.353553390593274, -0.5, 0.0, 0.121533978016438, -0.707106781186548, -0.121533978016438, 0.000000000000000,
	0.353553390593274, -0.353553390593274, 0.0, 0.5, 0.000000000000000, 0.121533978016438, 0.707106781186547, -0.121533978016438,
	0.353553390593274, -0.353553390593274, 0.0, 0.5, 0.000000000000000, 0.121533978016438, -0.707106781186547, -0.121533978016438,
	0.353553390593274, -0.353553390593274, 0.0, -0.5, -0.121533978016438, -0.000000000000000, 0.121533978016438, 0.707106781186547,
	0.353553390593274, -0.353553390593274, 0.0, -0.5, -0.121533978016438, -0.000000000000000, 0.121533978016438, -0.707106781186547};

const float kKaiser8[64] = {
	/* nldct.cpp:706-713: BM3D Kaiser window, 8x8 */
	0.1924f, 0.2989f, 0.3846f, 0.4325f, 0.4325f, 0.3846f, 0.2989f, 0.1924f,
	0.2989f, 0.4642f, 0.5974f, 0.6717f, 0.6717f, 0.5974f, 0.4642f, 0.2989f,
	0.3846f, 0.5974f, 0.7688f, 0.8644f, 0.8644f, 0.7688f, 0.5974f, 0.3846f,
	0.4325f, 0.6717f, 0.8644f, 0.9718f, 0.9718f, 0.8644f, 0.6717f, 0.4325f,
	0.4325f, 0.6717f, 0.8644f, 0.9718f, 0.9718f, 0.8644f, 0.6717f, 0.4325f,
	0.3846f, 0.5974f, 0.7688f, 0.8644f, 0.8644f, 0.7688f, 0.5974f, 0.3846f,
	0.2989f, 0.4642f, 0.5974f, 0.6717f, 0.6717f, 0.5974f, 0.4642f, 0.2989f,
	0.1924f, 0.2989f, 0.3846f, 0.4325f, 0.4325f, 0.3846f, 0.2989f, 0.1924f};

const float kKaiser10[100] = {
	/* nldct.cpp:722-731: Kaiser window, 10x10 */
	0.1924f, 0.2763f, 0.3503f, 0.4055f, 0.4349f, 0.4349f, 0.4055f, 0.3503f, 0.2763f, 0.1924f,
	0.2763f, 0.3967f, 0.5030f, 0.5822f, 0.6245f, 0.6245f, 0.5822f, 0.5030f, 0.3967f, 0.2763f,
	0.3503f, 0.5030f, 0.6377f, 0.7381f, 0.7917f, 0.7917f, 0.7381f, 0.6377f, 0.5030f, 0.3503f,
	0.4055f, 0.5822f, 0.7381f, 0.8544f, 0.9164f, 0.9164f, 0.8544f, 0.7381f, 0.5822f, 0.4055f,
	0.4349f, 0.6245f, 0.7917f, 0.9164f, 0.9829f, 0.9829f, 0.9164f, 0.7917f, 0.6245f, 0.4349f,
	0.4349f, 0.6245f, 0.7917f, 0.9164f, 0.9829f, 0.9829f, 0.9164f, 0.7917f, 0.6245f, 0.4349f,
	0.4055f, 0.5822f, 0.7381f, 0.8544f, 0.9164f, 0.9164f, 0.8544f, 0.7381f, 0.5822f, 0.4055f,
	0.3503f, 0.5030f, 0.6377f, 0.7381f, 0.7917f, 0.7917f, 0.7381f, 0.6377f, 0.5030f, 0.3503f,
	0.2763f, 0.3967f, 0.5030f, 0.5822f, 0.6245f, 0.6245f, 0.5822f, 0.5030f, 0.3967f, 0.2763f,
	0.1924f, 0.2763f, 0.3503f, 0.4055f, 0.4349f, 0.4349f, 0.4055f, 0.3503f, 0.2763f, 0.1924f};

/* Dense sPC x sPC bases, stored basis[k*sPC + p] exactly as the reference's
 * mat.patch_basis / mat.patch_basis_inv vectors. */
bool make_basis(int transform, unsigned px, unsigned pt, std::vector<float> &basis,
                std::vector<float> &binv)
{
	const unsigned sPC = px * px * pt;
	basis.assign((size_t)sPC * sPC, 0.f);
	binv.assign((size_t)sPC * sPC, 0.f);
	if (transform == BM4DOF_DCT) {
		/* nldct.cpp:582-610; the cosine argument is evaluated in double */
		std::vector<float> cosx(px * px), cost(pt * pt);
		for (unsigned k = 0, i = 0; k < px; k++)
			for (unsigned n = 0; n < px; n++, i++)
				cosx[i] = (float)(cos((0.5 + (float)n) * (float)k * M_PI / (float)px) *
				                  sqrt((k == 0 ? 1. : 2.) / (float)px));
		for (unsigned k = 0, i = 0; k < pt; k++)
			for (unsigned n = 0; n < pt; n++, i++)
				cost[i] = (float)(cos((0.5 + (float)n) * (float)k * M_PI / (float)pt) *
				                  sqrt((k == 0 ? 1. : 2.) / (float)pt));
		size_t i = 0;
		for (unsigned kt = 0; kt < pt; kt++)
			for (unsigned ky = 0; ky < px; ky++)
				for (unsigned kx = 0; kx < px; kx++)
					for (unsigned nt = 0; nt < pt; nt++)
						for (unsigned ny = 0; ny < px; ny++)
							for (unsigned nx = 0; nx < px; nx++, i++)
								basis[i] = cosx[kx * px + nx] * cosx[ky * px + ny] * cost[kt * pt + nt];
		binv = basis;
		return true;
	}
	if (px != 8) return false;
	/* nldct.cpp:637-695 */
	std::vector<float> bx(64), bt(pt * pt);
	for (int i = 0; i < 64; i++) bx[i] = (float)kBior15Fwd[i];
	for (unsigned k = 0, i = 0; k < pt; k++)
		for (unsigned n = 0; n < pt; n++, i++) bt[i] = n == k ? 1.f : 0.f;
	size_t i = 0;
	for (unsigned kt = 0; kt < pt; kt++)
		for (unsigned ky = 0; ky < px; ky++)
			for (unsigned kx = 0; kx < px; kx++)
				for (unsigned nt = 0; nt < pt; nt++)
					for (unsigned ny = 0; ny < px; ny++)
						for (unsigned nx = 0; nx < px; nx++, i++)
							basis[i] = bx[kx * px + nx] * bx[ky * px + ny] * bt[kt * pt + nt];
	for (int j = 0; j < 64; j++) bx[j] = (float)kBior15Inv[j];
	i = 0;
	/* "stored transposed": outer loops run over positions, inner over frequencies */
	for (unsigned nt = 0; nt < pt; nt++)
		for (unsigned ny = 0; ny < px; ny++)
			for (unsigned nx = 0; nx < px; nx++)
				for (unsigned kt = 0; kt < pt; kt++)
					for (unsigned ky = 0; ky < px; ky++)
						for (unsigned kx = 0; kx < px; kx++, i++)
							binv[i] = bx[kx * px + nx] * bx[ky * px + ny] * bt[kt * pt + nt];
	return true;
}

std::vector<float> make_window(bool agg, unsigned px, unsigned pt)
{
	/* nldct.cpp:698-737 */
	std::vector<float> w((size_t)px * px * pt, 1.f);
	if (agg && px == 8)
		for (unsigned t = 0; t < pt; t++) std::copy(kKaiser8, kKaiser8 + 64, w.begin() + t * 64);
	else if (agg && px == 10)
		for (unsigned t = 0; t < pt; t++) std::copy(kKaiser10, kKaiser10 + 100, w.begin() + t * 100);
	return w;
}

/* Column-major C(M x N) = op(A)(M x K) * op(B)(K x N) with one rounded product
 * and one rounded sum per term, the inner index in increasing order: the order
 * of the project's cblas_sgemm (oracle/ref_sgemm.c).  Restates productMatrix,
 * src/core/matrix_funs.cpp:136-164, for alpha = 1, beta = 0. */
void product(float *C, const float *A, const float *B, unsigned M, unsigned N, unsigned K,
             bool transB)
{
	for (unsigned j = 0; j < N; j++)
		for (unsigned i = 0; i < M; i++) {
			float acc = 0.f;
			for (unsigned p = 0; p < K; p++) {
				const float a = A[(size_t)p * M + i];
				const float b = transB ? B[(size_t)p * N + j] : B[(size_t)j * K + p];
				acc = acc + a * b;
			}
			C[(size_t)j * M + i] = acc;
		}
}

void haar_forward(float *z, unsigned nS, unsigned sPC, float isqrt2)
{
	/* nldct.cpp:1846-1860 */
	for (unsigned s = 2, h = 1; s <= nS; s *= 2, h *= 2)
		for (unsigned i = 0; i < sPC; i++)
			for (unsigned n = 0; n < nS; n += s) {
				const float z0 = z[n + i * nS] * isqrt2;
				const float z1 = z[n + h + i * nS] * isqrt2;
				z[n + i * nS] = z0 + z1;
				z[n + h + i * nS] = z0 - z1;
			}
}

void haar_inverse(float *z, unsigned nS, unsigned sPC, float isqrt2)
{
	/* nldct.cpp:1911-1924 */
	for (unsigned s = nS, h = s / 2; s >= 2; s /= 2, h /= 2)
		for (unsigned i = 0; i < sPC; i++)
			for (unsigned n = 0; n < nS; n += s) {
				const float z0 = z[n + i * nS] * isqrt2;
				const float z1 = z[n + h + i * nS] * isqrt2;
				z[n + i * nS] = z0 + z1;
				z[n + h + i * nS] = z0 - z1;
			}
}

bool less_first(const std::pair<float, unsigned> &a, const std::pair<float, unsigned> &b)
{
	/* comparaisonFirst, utilities.cpp:35-41 */
	return a.first < b.first;
}

struct GroupTrace {
	unsigned ref, nsimp;
	std::vector<unsigned> index;
};

/* ------------------------------------------------------------------------ */
/* Patch search (nldct.cpp:1143-1348 step 1, 1607-1789 step 2).              */
/* ------------------------------------------------------------------------ */
unsigned search(const Vid &im, const Vid *basic, const Vid &fflow, const Vid &bflow,
                unsigned pidx, const bm4dof_params &p, std::vector<unsigned> &index,
                std::vector<std::pair<float, unsigned> > &distance)
{
	const bool step1 = basic == nullptr;
	const int sPx = p.sizePatch, sPt = p.sizePatchTime;
	unsigned nSimP = 1;
	if (p.nSimilarPatches <= 1) { index[0] = pidx; return 1; }

	const Vid &src = step1 ? im : *basic;     /* distances: noisy ch0, or basic all ch */
	const int chn = step1 ? 1 : (int)im.c;
	const float tau = p.tau * p.tau * sPx * sPx * sPt;
	const bool use_flow = fflow.w > 0;
	const int W = im.w, H = im.h, F = im.f;
	const int sWx = p.sizeSearchWindow, sWy = p.sizeSearchWindow;
	const int wtf = p.sizeSearchTimeRangeFwd, wtb = p.sizeSearchTimeRangeBwd;

	const int pt = (int)(pidx / im.whc());
	const int py = (int)((pidx % im.wh()) / im.w);
	const int px = (int)(pidx % im.w);

	/* temporal range, shifted to stay inside the sequence: 1172-1186 */
	const int shift_t = std::min(0, pt - wtb) + std::max(0, pt + wtf - F + sPt);
	const int t0 = std::max(0, pt - wtb - shift_t);
	const int t1 = std::min(F - sPt, pt + wtf - shift_t);
	const int sWt = t1 - t0 + 1;

	std::vector<int> order;
	order.push_back(pt);
	for (int qt = pt + 1; qt <= t1; ++qt) order.push_back(qt);
	for (int qt = pt - 1; qt >= t0; --qt) order.push_back(qt);

	const unsigned sPC = sPx * sPx * sPt;
	std::vector<float> ref(sPC * chn);
	for (int c = 0, k = 0; c < chn; c++)
		for (int ht = 0; ht < sPt; ht++)
			for (int hy = 0; hy < sPx; hy++)
				for (int hx = 0; hx < sPx; hx++, k++)
					ref[k] = src.at(px + hx, py + hy, pt + ht, c);

	std::vector<int> cx(sWt, 0), cy(sWt, 0), ct(sWt, 0);
	distance.clear();
	for (int ii = 0; ii < sWt; ++ii) {
		const int qt = order[ii];
		const int dt = qt - t0;
		const int dir = std::max(-1, std::min(1, qt - pt));
		if (dir != 0) {
			/* flow-chained centre, rounded half away from zero and clamped: 1219-1236 */
			const int cx0 = cx[dt - dir], cy0 = cy[dt - dir], ct0 = ct[dt - dir];
			const Vid &fl = dir > 0 ? fflow : bflow;
			const float cxf = cx0 + (use_flow ? fl.at(cx0, cy0, ct0, 0) : 0.f);
			const float cyf = cy0 + (use_flow ? fl.at(cx0, cy0, ct0, 1) : 0.f);
			cx[dt] = (int)std::max(0.f, std::min(W - 1.f, roundf(cxf)));
			cy[dt] = (int)std::max(0.f, std::min(H - 1.f, roundf(cyf)));
			ct[dt] = qt;
		} else {
			cx[dt] = px; cy[dt] = py; ct[dt] = pt;
		}
		/* window shifted (not clipped) to stay inside the frame: 1248-1258 */
		int shx = std::min(0, cx[dt] - (sWx - 1) / 2);
		int shy = std::min(0, cy[dt] - (sWy - 1) / 2);
		shx += std::max(0, cx[dt] + (sWx - 1) / 2 - W + sPx);
		shy += std::max(0, cy[dt] + (sWy - 1) / 2 - H + sPx);
		const int rx0 = std::max(0, cx[dt] - (sWx - 1) / 2 - shx);
		const int ry0 = std::max(0, cy[dt] - (sWy - 1) / 2 - shy);
		const int rx1 = std::min(W - sPx, cx[dt] + (sWx - 1) / 2 - shx);
		const int ry1 = std::min(H - sPx, cy[dt] + (sWy - 1) / 2 - shy);

		for (int qy = ry0; qy <= ry1; qy++)
			for (int qx = rx0; qx <= rx1; qx++) {
				float dist = 0.f;
				for (int c = 0, k = 0; c < chn; c++)
					for (int ht = 0; ht < sPt; ht++)
						for (int hy = 0; hy < sPx; hy++)
							for (int hx = 0; hx < sPx; hx++, k++) {
								const float dif = ref[k] - src.at(qx + hx, qy + hy, qt + ht, c);
								dist = dist + dif * dif;
							}
				distance.push_back(std::make_pair(dist, (unsigned)(qt * im.whc() + qy * im.w + qx)));
			}
	}

	/* k nearest: the reference's std::partial_sort (libstdc++ heap select) */
	nSimP = std::min(p.nSimilarPatches, (unsigned)distance.size());
	std::partial_sort(distance.begin(), distance.begin() + nSimP, distance.end(), less_first);

	/* power-of-two truncation by tau: 1284-1289 */
	{
		unsigned n = 1;
		while (2 * n <= nSimP && distance[n].first < tau) n *= 2;
		nSimP = n;
	}
	for (unsigned n = 0; n < nSimP; n++) index[n] = distance[n].second;
	return nSimP;
}

/* ------------------------------------------------------------------------ */
/* Predictive patch search, the reference built with VBM3D_SEARCH            */
/* (nldct.cpp:892-1130 step 1, 1351-1589 step 2).                            */
/* ------------------------------------------------------------------------ */
unsigned search_vbm3d(const Vid &im, const Vid *basic, const Vid &fflow, const Vid &bflow,
                      unsigned pidx, const bm4dof_params &p, std::vector<unsigned> &index,
                      std::vector<std::pair<float, unsigned> > &distance)
{
	const bool step1 = basic == nullptr;
	const int sPx = p.sizePatch, sPt = p.sizePatchTime;
	unsigned nSimP = 1;
	if (p.nSimilarPatches <= 1) { index[0] = pidx; return 1; }

	/* distances on channel 0 only: the noisy video in step 1; in step 2 the
	 * basic estimate, channel 0 summed once per channel (the loop over c of
	 * nldct.cpp:1501-1506 never indexes the channel) */
	const Vid &src = step1 ? im : *basic;
	const int reps = step1 ? 1 : (int)im.c;
	const unsigned npf = p.nSimilarPatchesPred;
	const float dsub = p.dsub * p.dsub * 255;
	const float tau = p.tau * p.tau * sPx * sPx * sPt;
	const bool use_flow = fflow.w > 0;
	const int W = im.w, H = im.h, F = im.f;
	const int wtf = p.sizeSearchTimeRangeFwd, wtb = p.sizeSearchTimeRangeBwd;

	const int pt = (int)(pidx / im.whc());
	const int py = (int)((pidx % im.wh()) / im.w);
	const int px = (int)(pidx % im.w);

	/* temporal range and visiting order as in the exhaustive search: 934-956 */
	const int shift_t = std::min(0, pt - wtb) + std::max(0, pt + wtf - F + sPt);
	const int t0 = std::max(0, pt - wtb - shift_t);
	const int t1 = std::min(F - sPt, pt + wtf - shift_t);
	const int sWt = t1 - t0 + 1;
	std::vector<int> order;
	order.push_back(pt);
	for (int qt = pt + 1; qt <= t1; ++qt) order.push_back(qt);
	for (int qt = pt - 1; qt >= t0; --qt) order.push_back(qt);

	const unsigned sPC = sPx * sPx * sPt;
	std::vector<float> ref(sPC);
	for (int ht = 0, k = 0; ht < sPt; ht++)
		for (int hy = 0; hy < sPx; hy++)
			for (int hx = 0; hx < sPx; hx++, k++)
				ref[k] = src.at(px + hx, py + hy, pt + ht, 0);

	/* trajectories: the npf best matches of each frame (961-963) */
	std::vector<int> trx((size_t)npf * sWt, 0), try_((size_t)npf * sWt, 0), trt((size_t)npf * sWt, 0);
	distance.clear();
	std::vector<std::pair<float, unsigned> > dframe;
	struct Box { int x0, y0, x1, y1; };
	std::vector<Box> boxes;
	for (int ii = 0; ii < sWt; ++ii) {
		const int qt = order[ii];
		const int dt = qt - t0;
		const int dir = std::max(-1, std::min(1, qt - pt));
		std::vector<int> cx, cy;
		int sW;
		if (dir != 0) {
			/* one small window around each match of the previous frame, moved
			 * along the flow, rounded half away from zero and clamped: 978-993 */
			sW = (int)p.sizeSearchWindowPred;
			for (unsigned i = 0; i < npf; i++) {
				const size_t o = (size_t)i * sWt + (dt - dir);
				const int x0 = trx[o], y0 = try_[o], f0 = trt[o];
				const Vid &fl = dir > 0 ? fflow : bflow;
				const float xf = x0 + (use_flow ? fl.at(x0, y0, f0, 0) : 0.f);
				const float yf = y0 + (use_flow ? fl.at(x0, y0, f0, 1) : 0.f);
				cx.push_back((int)std::max(0.f, std::min(W - 1.f, roundf(xf))));
				cy.push_back((int)std::max(0.f, std::min(H - 1.f, roundf(yf))));
			}
		} else {
			/* one full window around the reference patch: 995-1001 */
			sW = (int)p.sizeSearchWindow;
			cx.push_back(px);
			cy.push_back(py);
		}
		/* windows shifted into the frame (1017-1027); their union in window,
		 * then raster order, each position once (1033-1035) */
		boxes.clear();
		dframe.clear();
		for (size_t i = 0; i < cx.size(); i++) {
			int shx = std::min(0, cx[i] - (sW - 1) / 2);
			int shy = std::min(0, cy[i] - (sW - 1) / 2);
			shx += std::max(0, cx[i] + (sW - 1) / 2 - W + sPx);
			shy += std::max(0, cy[i] + (sW - 1) / 2 - H + sPx);
			Box b;
			b.x0 = std::max(0, cx[i] - (sW - 1) / 2 - shx);
			b.y0 = std::max(0, cy[i] - (sW - 1) / 2 - shy);
			b.x1 = std::min(W - sPx, cx[i] + (sW - 1) / 2 - shx);
			b.y1 = std::min(H - sPx, cy[i] + (sW - 1) / 2 - shy);
			for (int qy = b.y0; qy <= b.y1; qy++)
				for (int qx = b.x0; qx <= b.x1; qx++) {
					bool seen = false;
					for (const Box &o : boxes)
						seen = seen || (qx >= o.x0 && qx <= o.x1 && qy >= o.y0 && qy <= o.y1);
					if (seen) continue;
					float dist = 0.f;
					for (int r = 0; r < reps; r++)
						for (int ht = 0, k = 0; ht < sPt; ht++)
							for (int hy = 0; hy < sPx; hy++)
								for (int hx = 0; hx < sPx; hx++, k++) {
									const float dif = ref[k] - src.at(qx + hx, qy + hy, qt + ht, 0);
									dist = dist + dif * dif;
								}
					/* bias towards the reference position, in every frame: 1047 */
					if (qy == py && qx == px) dist = dist - dsub;
					dframe.push_back(std::make_pair(dist, (unsigned)(qt * im.whc() + qy * im.w + qx)));
				}
			boxes.push_back(b);
		}
		/* the npf best of this frame feed the trajectories and the pool: 1055-1072 */
		std::partial_sort(dframe.begin(), dframe.begin() + npf, dframe.end(), less_first);
		for (unsigned i = 0; i < npf; i++) {
			distance.push_back(dframe[i]);
			const unsigned id = dframe[i].second;
			const size_t o = (size_t)i * sWt + dt;
			trt[o] = (int)(id / im.whc());
			try_[o] = (int)((id % im.wh()) / im.w);
			trx[o] = (int)(id % im.w);
		}
	}

	/* the np best of the pool, then the power-of-two truncation by tau: 1075-1104 */
	nSimP = std::min(p.nSimilarPatches, (unsigned)distance.size());
	std::partial_sort(distance.begin(), distance.begin() + nSimP, distance.end(), less_first);
	{
		unsigned n = 1;
		while (2 * n <= nSimP && distance[n].first < tau) n *= 2;
		nSimP = n;
	}
	for (unsigned n = 0; n < nSimP; n++) index[n] = distance[n].second;
	return nSimP;
}

/* ------------------------------------------------------------------------ */
/* Group filters (nldct.cpp:1799-2006 step 1, 2015-2242 step 2).             */
/* ------------------------------------------------------------------------ */
struct Work {
	std::vector<float> basis, binv, win, Z, Y, tmp;
};

/* returns false when all members are equal (weights left as they are) */
bool filter_step1(std::vector<std::vector<float> > &group, Work &w, const bm4dof_params &p,
                  unsigned nS, std::vector<float> &aggw)
{
	const unsigned sPC = p.sizePatch * p.sizePatch * p.sizePatchTime;
	const unsigned C = group.size();
	if (nS > 1) {
		/* all-equal test, nldct.cpp:1986-1999 */
		bool equal = true;
		for (unsigned c = 0; c < C && equal; c++)
			for (unsigned j = 0; j < sPC && equal; j++) {
				const float v = group[c][j * nS];
				for (unsigned i = 1; i < nS; i++)
					if (v != group[c][j * nS + i]) { equal = false; break; }
			}
		if (equal) return false;
	}
	const float beta_sigma = p.beta * p.sigma;
	const float beta_sigma2 = beta_sigma * beta_sigma;
	const float betaM_sigma = p.betaMean * p.sigma;
	const float betaM_sigma2 = betaM_sigma * betaM_sigma;
	const float sigma2 = p.sigma * p.sigma;
	const float isqrt2 = (float)(1. / sqrt(2.));
	float non_zero = 0;
	for (unsigned c = 0; c < C; c++) {
		float *z = w.Z.data();
		product(z, group[c].data(), w.basis.data(), nS, sPC, sPC, false);
		haar_forward(z, nS, sPC, isqrt2);
		if (p.orderInvariance) {
			/* nldct.cpp:1865-1900 */
			for (unsigned i = 0; i < sPC; i++) {
				float *zi = z + i * nS;
				float var_i = 0.;
				for (unsigned n = 1; n < nS; ++n) var_i += zi[n] * zi[n];
				var_i /= (float)(nS - 1);
				const float var_0 = std::max(zi[0] * zi[0] - sigma2, 0.f);
				const float w_0 = var_0 / (var_0 + betaM_sigma2);
				zi[0] *= w_0;
				var_i = std::max(var_i - sigma2, 0.f);
				const float w_i = var_i / (var_i + beta_sigma2);
				for (unsigned n = 1; n < nS; ++n) zi[n] *= w_i;
				non_zero += w_0 * w_0 + (float)(nS - 1) * w_i * w_i;
			}
		} else {
			/* hard threshold, coefficient (0,0) always kept: 1901-1908 */
			float *zz = z;
			for (unsigned k = 0; k < sPC; ++k)
				for (unsigned i = 0; i < nS; ++i, ++zz)
					if (*zz * *zz > beta_sigma2 || (k == 0 && i == 0)) non_zero += 1;
					else *zz = 0.f;
		}
		haar_inverse(z, nS, sPC, isqrt2);
		product(group[c].data(), z, w.binv.data(), nS, sPC, sPC, true);
	}
	const float variance = 1 / sigma2 / (float)non_zero;   /* 1935 */
	for (unsigned n = 0; n < nS; n++) aggw[n] = variance;
	return true;
}

bool filter_step2(std::vector<float> &gN, std::vector<float> &gB, Work &w,
                  const bm4dof_params &p, unsigned C, unsigned nS, std::vector<float> &aggw)
{
	const unsigned sPC1 = p.sizePatch * p.sizePatch * p.sizePatchTime;
	const unsigned sPCc = sPC1 * C;
	if (nS > 1) {
		/* all-equal test over every channel of the noisy group, 2222-2235 */
		bool equal = true;
		for (unsigned j = 0; j < sPCc && equal; j++) {
			const float v = gN[j * nS];
			for (unsigned i = 1; i < nS; i++)
				if (v != gN[j * nS + i]) { equal = false; break; }
		}
		if (equal) return false;
	}
	const float beta_sigma = p.beta * p.sigma;
	const float beta_sigma2 = beta_sigma * beta_sigma;
	const float betaM_sigma = p.betaMean * p.sigma;
	const float betaM_sigma2 = betaM_sigma * betaM_sigma;
	const float sigma2 = p.sigma * p.sigma;
	const float isqrt2 = (float)(1. / sqrt(2.));
	float variance = 0.;
	for (unsigned c = 0; c < C; c++) {
		float *gn = gN.data() + (size_t)sPC1 * nS * c;
		float *gb = gB.data() + (size_t)sPC1 * nS * c;
		float *z = w.Z.data(), *y = w.Y.data();
		product(z, gn, w.basis.data(), nS, sPC1, sPC1, false);
		product(y, gb, w.basis.data(), nS, sPC1, sPC1, false);
		haar_forward(z, nS, sPC1, isqrt2);
		haar_forward(y, nS, sPC1, isqrt2);
		if (p.orderInvariance) {
			/* nldct.cpp:2101-2122 */
			for (unsigned i = 0; i < sPC1; i++) {
				float *yi = y + i * nS, *zi = z + i * nS;
				const float var_0 = yi[0] * yi[0];
				const float w_0 = var_0 / (var_0 + betaM_sigma2);
				zi[0] *= w_0;
				float var_i = 0.;
				for (unsigned n = 1; n < nS; ++n) var_i += yi[n] * yi[n];
				var_i /= (float)(nS - 1);
				const float w_i = var_i / (var_i + beta_sigma2);
				for (unsigned n = 1; n < nS; ++n) zi[n] *= w_i;
				variance += w_0 * w_0 + (float)(nS - 1) * w_i * w_i;
			}
		} else {
			/* empirical Wiener gain against the basic estimate: 2123-2135 */
			const float *yy = y;
			float *zz = z;
			for (unsigned i = 0; i < sPC1; ++i)
				for (unsigned n = 0; n < nS; ++n, ++yy, ++zz) {
					const float wgt = *yy * *yy / (*yy * *yy + beta_sigma2);
					*zz *= wgt;
					variance += wgt * wgt;
				}
		}
		haar_inverse(z, nS, sPC1, isqrt2);
		product(gn, z, w.binv.data(), nS, sPC1, sPC1, true);
	}
	variance = 1. / sigma2 / variance;                      /* 2167: double arithmetic */
	for (unsigned n = 0; n < nS; n++) aggw[n] = variance;
	return true;
}

/* ------------------------------------------------------------------------ */
/* One tile of one step (processNlBayes, nldct.cpp:490-890).                 */
/* ------------------------------------------------------------------------ */
unsigned process_tile(const Vid &noisy, const Vid &fflow, const Vid &bflow, Vid &basic,
                      Vid &out, const bm4dof_params &p, const Crop &crop,
                      std::vector<GroupTrace> *trace, bool vbm3d)
{
	const bool step1 = p.isFirstStep;
	const unsigned sWx = p.sizeSearchWindow;
	const unsigned sWt = p.sizeSearchTimeRangeFwd + p.sizeSearchTimeRangeBwd + 1;
	const unsigned sPx = p.sizePatch, sPt = p.sizePatchTime;
	const unsigned W = noisy.w, H = noisy.h, F = noisy.f, C = noisy.c;

	Vid weight(W, H, F, 1, 0.f);
	std::vector<char> mask((size_t)W * H * F, 0);

	/* reference-patch grid, nldct.cpp:520-553 (the tiles of a run span all
	 * frames: temporal borders come only from a caller's crop) */
	const bool bx0 = crop.bx0, by0 = crop.by0, bt0 = crop.bt0;
	const bool bx1 = crop.bx1, by1 = crop.by1, bt1 = crop.bt1;
	const int ori_x = bx0 ? sPx - 1 + sWx / 2 : 0;
	const int ori_y = by0 ? sPx - 1 + sWx / 2 : 0;
	const int ori_f = bt0 ? sPt - 1 + sWt / 2 : 0;
	const int end_x = (int)W - (int)(bx1 ? sPx - 1 + sWx / 2 : sPx - 1);
	const int end_y = (int)H - (int)(by1 ? sPx - 1 + sWx / 2 : sPx - 1);
	const int end_f = (int)F - (int)(bt1 ? sPt - 1 + sWt / 2 : sPt - 1);
	const unsigned stepx = p.offSet, stepy = p.offSet, stepf = p.offSetTime;
	for (int f = ori_f, df = 0; f < end_f; f++, df++)
		for (int y = ori_y, dy = 0; y < end_y; y++, dy++)
			for (int x = ori_x, dx = 0; x < end_x; x++, dx++)
				if (((unsigned)df % stepf == 0) || (!bt1 && f == end_f - 1))
					if (((unsigned)dy % stepy == 0) || (!by1 && y == end_y - 1) || (!by0 && y == ori_y))
						if (((unsigned)dx % stepx == 0) || (!bx1 && x == end_x - 1) || (!bx0 && x == ori_x))
							mask[(size_t)f * W * H + y * W + x] = 1;

	const unsigned sPC = sPx * sPx * sPt;
	const unsigned patch_num = sWx * sWx * sWt;
	Work w;
	make_basis(p.transform, sPx, sPt, w.basis, w.binv);
	w.win = make_window(p.agg_window, sPx, sPt);
	w.Z.resize((size_t)patch_num * sPC);
	w.Y.resize((size_t)patch_num * sPC);

	std::vector<unsigned> index(patch_num);
	std::vector<std::pair<float, unsigned> > distance;
	distance.reserve(patch_num);
	unsigned groups = 0;

	if (step1) basic = Vid(W, H, F, C, 0.f); else out = Vid(W, H, F, C, 0.f);
	Vid &acc = step1 ? basic : out;
	std::vector<float> aggw(patch_num, 1.f);             /* stale across groups */
	std::vector<std::vector<float> > group(C, std::vector<float>((size_t)patch_num * sPC));
	std::vector<float> gN((size_t)patch_num * sPC * C), gB((size_t)patch_num * sPC * C);
	const unsigned wh = noisy.wh(), whc = noisy.whc();

	for (unsigned t = 0; t < F; t++)
		for (unsigned y = 0; y < H; y++)
			for (unsigned x = 0; x < W; x++) {
				if (!mask[(size_t)t * wh + y * W + x]) continue;
				groups++;
				const unsigned ij3 = t * whc + y * W + x;
				const unsigned nS = vbm3d
					? search_vbm3d(noisy, step1 ? nullptr : &basic, fflow, bflow, ij3, p, index, distance)
					: search(noisy, step1 ? nullptr : &basic, fflow, bflow, ij3, p, index, distance);
				if (trace) {
					GroupTrace g;
					g.ref = ij3; g.nsimp = nS;
					g.index.assign(index.begin(), index.begin() + nS);
					trace->push_back(g);
				}
				if (step1) {
					/* stack, nldct.cpp:1334-1339 */
					for (unsigned c = 0; c < C; c++)
						for (unsigned ht = 0, k = 0; ht < sPt; ht++)
							for (unsigned hy = 0; hy < sPx; hy++)
								for (unsigned hx = 0; hx < sPx; hx++)
									for (unsigned n = 0; n < nS; n++, k++)
										group[c][k] = noisy.d[c * wh + index[n] + ht * whc + hy * W + hx];
					filter_step1(group, w, p, nS, aggw);
					/* aggregation, nldct.cpp:2284-2300 (channel-0 weight for all channels) */
					for (unsigned n = 0; n < nS; n++) {
						const unsigned ind = index[n];
						const unsigned ind1 = (ind / whc) * wh + ind % wh;
						for (unsigned qt = 0, i = 0; qt < sPt; qt++)
							for (unsigned qy = 0; qy < sPx; qy++)
								for (unsigned qx = 0; qx < sPx; qx++, i++) {
									for (unsigned c = 0; c < C; c++)
										acc.d[ind + c * wh + qt * whc + qy * W + qx] +=
											aggw[n] * w.win[i] * group[c][i * nS + n];
									weight.d[ind1 + qt * wh + qy * W + qx] += aggw[n] * w.win[i];
								}
					}
				} else {
					/* stack noisy and basic, channel-major: 1778-1786 */
					for (unsigned c = 0, k = 0; c < C; c++)
						for (unsigned ht = 0; ht < sPt; ht++)
							for (unsigned hy = 0; hy < sPx; hy++)
								for (unsigned hx = 0; hx < sPx; hx++)
									for (unsigned n = 0; n < nS; n++, k++) {
										const size_t q = c * wh + index[n] + ht * whc + hy * W + hx;
										gN[k] = noisy.d[q];
										gB[k] = basic.d[q];
									}
					filter_step2(gN, gB, w, p, C, nS, aggw);
					/* aggregation, nldct.cpp:2376-2394 */
					for (unsigned n = 0; n < nS; n++) {
						const unsigned ind = index[n];
						for (unsigned c = 0, k = 0; c < C; c++) {
							const unsigned ij = ind + c * wh;
							for (unsigned qt = 0, i = 0; qt < sPt; qt++)
								for (unsigned qy = 0; qy < sPx; qy++)
									for (unsigned qx = 0; qx < sPx; qx++, k++, i++)
										acc.d[ij + qt * whc + qy * W + qx] += aggw[n] * w.win[i] * gN[k * nS + n];
						}
						const unsigned ind1 = (ind / whc) * wh + ind % wh;
						for (unsigned qt = 0, i = 0; qt < sPt; qt++)
							for (unsigned qy = 0; qy < sPx; qy++)
								for (unsigned qx = 0; qx < sPx; qx++, i++)
									weight.d[ind1 + qt * wh + qy * W + qx] += aggw[n] * w.win[i];
					}
				}
				if (p.doPasteBoost) {
					/* paste trick, nldct.cpp:2302-2322 / 2395-2415: every member's
					 * position and its four neighbours away from the border band
					 * of 2*sPx (unsigned comparisons, as the reference's) */
					for (unsigned n = 0; n < nS; n++) {
						const unsigned ind = index[n];
						const unsigned ind1 = (ind / whc) * wh + ind % wh;
						const unsigned mx = ind1 % W, my = (ind1 / W) % H;
						/* linear neighbours, as the reference writes them (a band
						 * wider than the tile lets +1 / +W cross into the next row
						 * or frame); writes past the mask are skipped */
						const size_t msz = mask.size();
						mask[ind1] = 0;
						if (my > 2 * sPx) mask[ind1 - W] = 0;
						if (my < H - 2 * sPx && ind1 + W < msz) mask[ind1 + W] = 0;
						if (mx > 2 * sPx) mask[ind1 - 1] = 0;
						if (mx < W - 2 * sPx && ind1 + 1 < msz) mask[ind1 + 1] = 0;
					}
				} else {
					/* mask(index[0]) = false, nldct.cpp:2325-2329: the index carries
					 * the channel stride, so for C > 1 it addresses another frame of
					 * the one-channel mask; writes past the mask are skipped here
					 * (the reference writes out of bounds there). */
					if ((size_t)index[0] < mask.size()) mask[index[0]] = 0;
				}
			}

	/* computeWeightedAggregation, nldct.cpp:2436-2448 */
	for (unsigned t = 0; t < F; t++)
		for (unsigned c = 0; c < C; c++)
			for (unsigned y = 0; y < H; y++)
				for (unsigned x = 0; x < W; x++) {
					const float wt = weight.at(x, y, t);
					if (wt > 0.f) acc.at(x, y, t, c) /= wt;
					else acc.at(x, y, t, c) /= noisy.at(x, y, t, c);
				}
	return groups;
}

int fail(char *err, size_t len, const char *msg, int code)
{
	if (err && len) std::snprintf(err, len, "%s", msg);
	return code;
}

} // namespace

extern "C" {

struct oracle_trace {
	/* caller-owned arrays; filled for step s in [0,1] and tile in processing order */
	unsigned cap;          /* capacity in groups                                  */
	unsigned stride;       /* index entries per group                             */
	unsigned *step, *tile, *ref, *nsimp, *index;
	unsigned count;        /* groups written (or needed, when above cap)          */
};

void oracle_initialize_params(bm4dof_params *p, unsigned step, float sigma,
                              const bm4dof_video_size *sz, int verbose)
{
	init_params(*p, step, sigma, sz->frames, verbose);
}
void oracle_set_size_search_window(bm4dof_params *p, unsigned wx) { set_search_window(*p, wx); }
void oracle_set_size_patch(bm4dof_params *p, const bm4dof_video_size *sz, unsigned px)
{
	set_patch_size(*p, sz->frames, px);
}
void oracle_set_n_similar_patches(bm4dof_params *p, unsigned np) { set_n_similar(*p, np); }
int oracle_format_params(const bm4dof_params *p, char *buf, size_t len)
{
	return format_params(*p, buf, len);
}
void oracle_determine_factor(unsigned n, unsigned *a, unsigned *b) { determine_factor(n, *a, *b); }

/* crop boxes of subDivideTight: 4 ints per tile (ox, oy, ex, ey) */
int oracle_tile_crops(unsigned W, unsigned H, unsigned nparts, int boundary, int *boxes)
{
	std::vector<Crop> cr = tile_crops(W, H, nparts, boundary);
	for (size_t i = 0; i < cr.size(); i++) {
		boxes[4 * i + 0] = cr[i].ox; boxes[4 * i + 1] = cr[i].oy;
		boxes[4 * i + 2] = cr[i].ex; boxes[4 * i + 3] = cr[i].ey;
	}
	return (int)cr.size();
}

int oracle_basis(int transform, unsigned px, unsigned pt, float *basis, float *binv)
{
	std::vector<float> b, bi;
	if (!make_basis(transform, px, pt, b, bi)) return 1;
	std::copy(b.begin(), b.end(), basis);
	std::copy(bi.begin(), bi.end(), binv);
	return 0;
}

void oracle_window(int agg, unsigned px, unsigned pt, float *win)
{
	std::vector<float> w = make_window(agg != 0, px, pt);
	std::copy(w.begin(), w.end(), win);
}

void oracle_color_transform(float *v, unsigned W, unsigned H, unsigned C, unsigned F, int forward)
{
	Vid x(W, H, F, C);
	std::copy(v, v + x.d.size(), x.d.begin());
	color_transform(x, forward != 0);
	std::copy(x.d.begin(), x.d.end(), v);
}

/* VideoNLB::runNlBayes, nldct.cpp:267-478, with an explicit tile count;
 * flags & BM4DOF_VBM3D_SEARCH selects the predictive search of the
 * reference's VBM3D_SEARCH build. */
int oracle_run_ex(const float *noisy_in, const float *fflow_in, const float *bflow_in,
                  unsigned W, unsigned H, unsigned C, unsigned F, float *basic_io, float *final_out,
                  const bm4dof_params *p1, const bm4dof_params *p2, unsigned nparts,
                  unsigned nthreads, unsigned flags, float ratios[2], oracle_trace *trace,
                  char *err, size_t errlen)
{
	const bool vbm3d = (flags & BM4DOF_VBM3D_SEARCH) != 0;
	if (!(C == 1 || C == 3 || C == 4))
		return fail(err, errlen, "VideoNLB::runNlBayes: Wrong number of channels. Must be 1, 3 or 4.", BM4DOF_ERR_CHANNELS);
	/* an empty forward flow disables flow (nldct.cpp:283); a forward flow
	 * without a backward one fails the size check of nldct.cpp:291-296 */
	const bool use_flow = fflow_in != nullptr;
	if (use_flow && bflow_in == nullptr)
		return fail(err, errlen, "VideoNLB::runNlBayes: Wrong size of bwd optical flow.", BM4DOF_ERR_BWD_FLOW);
	if (nparts == 0) nparts = 2;
#ifdef _OPENMP
	if (nthreads == 0) nthreads = 1;
#endif
	const int step = p1->sizePatch ? (p2->sizePatch ? 0 : 1) : (p2->sizePatch ? 2 : -1);
	if (step == -1)
		return fail(err, errlen, "VideoNLB::runNlBayes: Both patch sizes are zero.", BM4DOF_ERR_NO_STEP);
	for (int s = 0; s < 2; s++) {
		const bm4dof_params *p = s ? p2 : p1;
		if (!p->sizePatch) continue;
		if (p->transform == BM4DOF_BIOR1_5 && p->sizePatch != 8)
			return fail(err, errlen, "VideoNLB::processNlBayes: bior1_5 transform is only implemented for patches of size 8 x 8 x pt.", BM4DOF_ERR_BIOR_SIZE);
		if (p->offSet == 0 || p->offSetTime == 0 || p->sizePatchTime == 0)
			return fail(err, errlen, "oracle: unsupported parameters", BM4DOF_ERR_UNSUPPORTED);
		if (vbm3d && p->nSimilarPatches > 1 && p->nSimilarPatchesPred == 0)
			return fail(err, errlen, "oracle: nSimilarPatchesPred must be positive", BM4DOF_ERR_UNSUPPORTED);
	}

	Vid noisy(W, H, F, C);
	std::copy(noisy_in, noisy_in + noisy.d.size(), noisy.d.begin());
	Vid fflow, bflow;
	if (use_flow) {
		fflow = Vid(W, H, F, 2); bflow = Vid(W, H, F, 2);
		std::copy(fflow_in, fflow_in + fflow.d.size(), fflow.d.begin());
		std::copy(bflow_in, bflow_in + bflow.d.size(), bflow.d.begin());
	}
	Vid basic(W, H, F, C);
	if (step == 2) std::copy(basic_io, basic_io + basic.d.size(), basic.d.begin());
	Vid final_(W, H, F, C);
	float gr[2] = {0.f, 0.f};
	std::vector<std::vector<GroupTrace> > traces[2];
	const unsigned whf = W * H * F;

	for (int s = 0; s < 2; s++) {
		if (s == 0 && step == 2) continue;
		if (s == 1 && step == 1) continue;
		const bm4dof_params &p = s == 0 ? *p1 : *p2;
		Vid im = noisy;
		if (p.colorSpace == BM4DOF_YUV) {
			color_transform(im, true);
			if (s == 1) color_transform(basic, true);
		}
		std::vector<Crop> crops = tile_crops(W, H, nparts, (int)p.boundary);
		const int nt = (int)crops.size();
		std::vector<Vid> nsub(nt), bsub(nt), osub(nt), fsub(nt), bfsub(nt);
		for (int n = 0; n < nt; n++) {
			nsub[n] = crop_video(im, crops[n]);
			if (s == 1) bsub[n] = crop_video(basic, crops[n]);
			if (use_flow) { fsub[n] = crop_video(fflow, crops[n]); bfsub[n] = crop_video(bflow, crops[n]); }
		}
		std::vector<unsigned> cnt(nt, 0);
		traces[s].assign(nt, std::vector<GroupTrace>());
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic) num_threads(nthreads)
#endif
		for (int n = 0; n < nt; n++)
			cnt[n] = process_tile(nsub[n], fsub[n], bfsub[n], bsub[n], osub[n], p, crops[n],
			                      trace ? &traces[s][n] : nullptr, vbm3d);
		if (s == 0) {
			build_tight(bsub, basic, nparts, (int)p.boundary);
			if (p.colorSpace == BM4DOF_YUV) color_transform(basic, false);
		} else {
			build_tight(osub, final_, nparts, (int)p.boundary);
			if (p.colorSpace == BM4DOF_YUV) { color_transform(basic, false); color_transform(final_, false); }
		}
		for (int n = 0; n < nt; n++) gr[s] += 100.f * (float)cnt[n] / (float)whf;
	}

	std::copy(basic.d.begin(), basic.d.end(), basic_io);
	if (step != 1) std::copy(final_.d.begin(), final_.d.end(), final_out);
	if (ratios) { ratios[0] = gr[0]; ratios[1] = gr[1]; }
	if (trace) {
		unsigned k = 0;
		for (int s = 0; s < 2; s++)
			for (size_t n = 0; n < traces[s].size(); n++)
				for (const GroupTrace &g : traces[s][n]) {
					if (k < trace->cap) {
						trace->step[k] = s + 1; trace->tile[k] = (unsigned)n;
						trace->ref[k] = g.ref; trace->nsimp[k] = g.nsimp;
						for (unsigned i = 0; i < trace->stride; i++)
							trace->index[(size_t)k * trace->stride + i] = i < g.nsimp ? g.index[i] : 0u;
					}
					k++;
				}
		trace->count = k;
	}
	return 0;
}

/* VideoNLB::processNlBayes (nldct.cpp:490-890): one step (p->isFirstStep) of
 * one video with the border flags of its crop (nldct.cpp:520-525; crop may be
 * NULL), no tiling, no colour transform.  Step 1 writes basic_io, step 2 reads
 * it and writes final_out.  Returns the processed group count in *groups. */
int oracle_process(const float *noisy_in, const float *fflow_in, const float *bflow_in,
                   unsigned W, unsigned H, unsigned C, unsigned F, float *basic_io, float *final_out,
                   const bm4dof_params *p, const bm4dof_crop *crop, unsigned flags, unsigned *groups,
                   char *err, size_t errlen)
{
	if (p->transform == BM4DOF_BIOR1_5 && p->sizePatch != 8)
		return fail(err, errlen, "VideoNLB::processNlBayes: bior1_5 transform is only implemented for patches of size 8 x 8 x pt.", BM4DOF_ERR_BIOR_SIZE);
	if (p->sizePatch == 0 || p->offSet == 0 || p->offSetTime == 0 || p->sizePatchTime == 0)
		return fail(err, errlen, "oracle: unsupported parameters", BM4DOF_ERR_UNSUPPORTED);
	Crop c;
	c.ox = c.oy = 0;
	c.ex = (int)W;
	c.ey = (int)H;
	c.bx0 = c.by0 = c.bx1 = c.by1 = false;
	if (crop) {
		c.bx0 = crop->origin_x > 0;
		c.by0 = crop->origin_y > 0;
		c.bt0 = crop->origin_t > 0;
		c.bx1 = crop->ending_x < (int)crop->source_sz.width;
		c.by1 = crop->ending_y < (int)crop->source_sz.height;
		c.bt1 = crop->ending_t < (int)crop->source_sz.frames;
	}
	Vid noisy(W, H, F, C);
	std::copy(noisy_in, noisy_in + noisy.d.size(), noisy.d.begin());
	Vid fflow, bflow;
	if (fflow_in) {
		fflow = Vid(W, H, F, 2);
		bflow = Vid(W, H, F, 2);
		std::copy(fflow_in, fflow_in + fflow.d.size(), fflow.d.begin());
		std::copy(bflow_in, bflow_in + bflow.d.size(), bflow.d.begin());
	}
	Vid basic(W, H, F, C), out;
	if (!p->isFirstStep) std::copy(basic_io, basic_io + basic.d.size(), basic.d.begin());
	const unsigned n = process_tile(noisy, fflow, bflow, basic, out, *p, c, nullptr,
	                                (flags & BM4DOF_VBM3D_SEARCH) != 0);
	if (p->isFirstStep) std::copy(basic.d.begin(), basic.d.end(), basic_io);
	else std::copy(out.d.begin(), out.d.end(), final_out);
	if (groups) *groups = n;
	return 0;
}

int oracle_run(const float *noisy_in, const float *fflow_in, const float *bflow_in,
               unsigned W, unsigned H, unsigned C, unsigned F, float *basic_io, float *final_out,
               const bm4dof_params *p1, const bm4dof_params *p2, unsigned nparts,
               unsigned nthreads, float ratios[2], oracle_trace *trace, char *err, size_t errlen)
{
	return oracle_run_ex(noisy_in, fflow_in, bflow_in, W, H, C, F, basic_io, final_out, p1, p2,
	                     nparts, nthreads, 0u, ratios, trace, err, errlen);
}

} // extern "C"
