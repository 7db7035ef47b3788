// basis.cpp -- patch transform bases and aggregation windows (host).
//
// Restates src/core/nldct.cpp:572-737.  The bases are dense sPC x sPC
// matrices stored basis[k*sPC + p] (frequency k, patch position p).  The DCT
// cosines are evaluated in double and rounded to float once, then multiplied
// in float, as the reference does; the bior1.5 tables are the reference's.
#include <cmath>
#include <vector>

#include "../../include/bm4dof.h"
#include "internal.hpp"

namespace bm4dof {

namespace {

// 1-D bior1.5 analysis rows for length 8 (nldct.cpp:640-647)
const double kBiorAnalysis[64] = {
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

// 1-D bior1.5 synthesis table for length 8 (nldct.cpp:670-677)
const double kBiorSynthesis[64] = {
	0.353553390593274, 0.353553390593274, 0.5, 0.0, 0.707106781186547, -0.121533978016438, -0.0, 0.121533978016438,
	0.353553390593274, 0.353553390593274, 0.5, -0.0, -0.707106781186547, -0.121533978016438, 0.0, 0.121533978016438,
	0.353553390593274, 0.353553390593274, -0.5, -0.0, 0.121533978016438, 0.707106781186548, -0.121533978016438, 0.0,
	0.353553390593274, 0.353553390593274, -0.5, 0.0, 0.121533978016438, -0.707106781186548, -0.121533978016438, 0.0,
	0.353553390593274, -0.353553390593274, 0.0, 0.5, 0.0, 0.121533978016438, 0.707106781186547, -0.121533978016438,
	0.353553390593274, -0.353553390593274, 0.0, 0.5, 0.0, 0.121533978016438, -0.707106781186547, -0.121533978016438,
	0.353553390593274, -0.353553390593274, 0.0, -0.5, -0.121533978016438, -0.0, 0.121533978016438, 0.707106781186547,
	0.353553390593274, -0.353553390593274, 0.0, -0.5, -0.121533978016438, -0.0, 0.121533978016438, -0.707106781186547};

// BM3D Kaiser windows (nldct.cpp:706-713, 722-731)
const float kKaiser8Rows[64] = {
	0.1924f, 0.2989f, 0.3846f, 0.4325f, 0.4325f, 0.3846f, 0.2989f, 0.1924f,
	0.2989f, 0.4642f, 0.5974f, 0.6717f, 0.6717f, 0.5974f, 0.4642f, 0.2989f,
	0.3846f, 0.5974f, 0.7688f, 0.8644f, 0.8644f, 0.7688f, 0.5974f, 0.3846f,
	0.4325f, 0.6717f, 0.8644f, 0.9718f, 0.9718f, 0.8644f, 0.6717f, 0.4325f,
	0.4325f, 0.6717f, 0.8644f, 0.9718f, 0.9718f, 0.8644f, 0.6717f, 0.4325f,
	0.3846f, 0.5974f, 0.7688f, 0.8644f, 0.8644f, 0.7688f, 0.5974f, 0.3846f,
	0.2989f, 0.4642f, 0.5974f, 0.6717f, 0.6717f, 0.5974f, 0.4642f, 0.2989f,
	0.1924f, 0.2989f, 0.3846f, 0.4325f, 0.4325f, 0.3846f, 0.2989f, 0.1924f};

const float kKaiser10Rows[100] = {
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

std::vector<float> dct_1d(unsigned n)
{
	std::vector<float> m(n * n);
	for (unsigned k = 0; k < n; k++)
		for (unsigned j = 0; j < n; j++)
			m[k * n + j] = (float)(std::cos((0.5 + (float)j) * (float)k * M_PI / (float)n) *
			                       std::sqrt((k == 0 ? 1. : 2.) / (float)n));
	return m;
}

}  // namespace

bool make_basis(int transform, unsigned px, unsigned pt, std::vector<float> &basis,
                std::vector<float> &binv)
{
	const unsigned spc = px * px * pt;
	basis.assign((size_t)spc * spc, 0.f);
	binv.assign((size_t)spc * spc, 0.f);
	std::vector<float> ax, at, sx;
	if (transform == BM4DOF_DCT) {
		ax = dct_1d(px);
		at = dct_1d(pt);
	} else {
		if (px != 8) return false;
		ax.resize(64);
		sx.resize(64);
		for (int i = 0; i < 64; i++) { ax[i] = (float)kBiorAnalysis[i]; sx[i] = (float)kBiorSynthesis[i]; }
		at.assign((size_t)pt * pt, 0.f);
		for (unsigned i = 0; i < pt; i++) at[i * pt + i] = 1.f;
	}
	// basis[(kt,ky,kx) * spc + (nt,ny,nx)] = a[kx][nx] * a[ky][ny] * at[kt][nt]
	size_t i = 0;
	for (unsigned kt = 0; kt < pt; kt++)
		for (unsigned ky = 0; ky < px; ky++)
			for (unsigned kx = 0; kx < px; kx++)
				for (unsigned nt = 0; nt < pt; nt++)
					for (unsigned ny = 0; ny < px; ny++)
						for (unsigned nx = 0; nx < px; nx++, i++)
							basis[i] = ax[kx * px + nx] * ax[ky * px + ny] * at[kt * pt + nt];
	if (transform == BM4DOF_DCT) {
		binv = basis;   // orthonormal
		return true;
	}
	// bior1.5 synthesis, "stored transposed" (nldct.cpp:684-695): the outer
	// index runs over positions and the inner one over frequencies
	i = 0;
	for (unsigned nt = 0; nt < pt; nt++)
		for (unsigned ny = 0; ny < px; ny++)
			for (unsigned nx = 0; nx < px; nx++)
				for (unsigned kt = 0; kt < pt; kt++)
					for (unsigned ky = 0; ky < px; ky++)
						for (unsigned kx = 0; kx < px; kx++, i++)
							binv[i] = sx[kx * px + nx] * sx[ky * px + ny] * at[kt * pt + nt];
	return true;
}

std::vector<float> make_window(bool agg, unsigned px, unsigned pt)
{
	std::vector<float> w((size_t)px * px * pt, 1.f);
	const float *tab = nullptr;
	if (agg && px == 8) tab = kKaiser8Rows;
	else if (agg && px == 10) tab = kKaiser10Rows;
	if (tab)
		for (unsigned t = 0; t < pt; t++)
			for (unsigned k = 0; k < px * px; k++) w[(size_t)t * px * px + k] = tab[k];
	return w;
}

}  // namespace bm4dof
