// tvl1.cu -- TV-L1 optical flow (Zach, Pock and Bischof's dual method) on the
// GPU, batched over frame pairs.  It produces the flows the denoiser takes as
// input, the step the reference runs before its path (lib/tvl1flow, driven by
// scripts/tvl1flow-seq.sh).
//
// Restates, with the same float/double arithmetic (except |grad u| of the dual
// update, taken in float instead of the reference's double hypot):
//   tvl1flow_lib.c   image_normalization (299-336), Dual_TVL1_optic_flow
//                    (93-263), Dual_TVL1_optic_flow_multiscale (344-474);
//   mask.c           divergence (40-88), forward_gradient (96-139),
//                    centered_gradient (147-203), gaussian (211-333, the
//                    reflecting boundary);
//   zoom.c           zoom_size (24-35), zoom_out (42-77), zoom_in (84-112);
//   bicubic_interpolation.c  bicubic_interpolation_at (141-232, Neumann
//                    boundary, including its use of sx for the row above),
//                    bicubic_interpolation_warp (239-262);
//   main.c           the number of scales (147-153).
//
// Layout: every array is [pair][y][x] at its pyramid level.  Each frame pair
// is one unit of the batch; all pairs of a video go in one call.  The fixed-
// point iterations of one warping run in one cooperative kernel: blocks are
// assigned to pairs, each iteration is two phases separated by grid-wide
// barriers, and the per-pair convergence test (mean squared update below
// epsilon^2, at most 300 iterations) is made identically by every block from
// per-block partial sums read in a fixed order.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <string>
#include <vector>

#include "internal.hpp"

namespace cg = cooperative_groups;

namespace bm4dof {

namespace {

constexpr int kMaxIterations = 300;         // tvl1flow_lib.c:23
constexpr double kPresmoothSigma = 0.8;     // tvl1flow_lib.c:24
constexpr float kGradIsZero = 1e-10f;       // tvl1flow_lib.c:25
constexpr float kZoomSigmaZero = 0.6f;      // zoom.c:16
constexpr int kGaussWindow = 5;             // mask.c:23
constexpr int kMaxGauss = 64;               // kernel taps kept in constant memory

__constant__ double c_gauss[kMaxGauss];

// ---- bicubic interpolation (bicubic_interpolation.c) ---------------------------
__device__ __forceinline__ int neumann(int x, int n, bool &out)
{
	if (x < 0) { out = true; return 0; }
	if (x >= n) { out = true; return n - 1; }
	return x;
}

__device__ __forceinline__ double cubic_cell(const double v[4], double x)
{
	return v[1] + 0.5 * x * (v[2] - v[0] + x * (2.0 * v[0] - 5.0 * v[1] + 4.0 * v[2] - v[3] +
	                                            x * (3.0 * (v[1] - v[2]) + v[3] - v[0])));
}

__device__ float bicubic_at(const float *in, float uu, float vv, int nx, int ny, bool border_out)
{
	const int sx = uu < 0 ? -1 : 1;
	const int sy = vv < 0 ? -1 : 1;
	bool out = false;
	const int x = neumann((int)uu, nx, out);
	const int y = neumann((int)vv, ny, out);
	const int mx = neumann((int)uu - sx, nx, out);
	const int my = neumann((int)vv - sx, ny, out);   // sx, as the reference has it
	const int dx = neumann((int)uu + sx, nx, out);
	const int dy = neumann((int)vv + sy, ny, out);
	const int ddx = neumann((int)uu + 2 * sx, nx, out);
	const int ddy = neumann((int)vv + 2 * sy, ny, out);
	if (out && border_out) return 0.f;
	const int xs[4] = {mx, x, dx, ddx}, ys[4] = {my, y, dy, ddy};
	double v[4];
	for (int a = 0; a < 4; a++) {
		double col[4];
		for (int b = 0; b < 4; b++) col[b] = (double)in[xs[a] + nx * ys[b]];
		v[a] = cubic_cell(col, (double)(vv - y));
	}
	return (float)cubic_cell(v, (double)(uu - x));
}

// ---- per-pixel stencils of mask.c ------------------------------------------------
__device__ __forceinline__ float divergence_at(const float *v1, const float *v2, int i, int j, int nx, int ny)
{
	const int p = i * nx + j;
	const bool top = i == 0, bot = i == ny - 1, lef = j == 0, rig = j == nx - 1;
	if (!top && !bot && !lef && !rig) return (v1[p] - v1[p - 1]) + (v2[p] - v2[p - nx]);
	if (top && lef) return v1[0] + v2[0];
	if (top && rig) return -v1[nx - 2] + v2[nx - 1];
	if (bot && lef) return v1[p] - v2[p - nx];
	if (bot && rig) return -v1[p - 1] - v2[p - nx];
	if (top) return v1[j] - v1[j - 1] + v2[j];
	if (bot) return v1[p] - v1[p - 1] - v2[p - nx];
	if (lef) return v1[p] + v2[p] - v2[p - nx];
	return -v1[p - 1] + v2[p] - v2[p - nx];   // right column
}

__device__ __forceinline__ void forward_gradient_at(const float *f, int i, int j, int nx, int ny, float &fx,
                                                    float &fy)
{
	const int p = i * nx + j;
	fx = j < nx - 1 ? f[p + 1] - f[p] : 0.f;
	fy = i < ny - 1 ? f[p + nx] - f[p] : 0.f;
}

// ---- kernels ---------------------------------------------------------------------
// min and max of both images of every pair, then 255 (I - min) / (max - min)
__global__ void normalize_kernel(const float *__restrict__ I0, const float *__restrict__ I1, int size,
                                 float *__restrict__ O0, float *__restrict__ O1)
{
	const int pair = blockIdx.x;
	const float *a = I0 + (size_t)pair * size, *b = I1 + (size_t)pair * size;
	__shared__ float smin[2][256], smax[2][256];
	float mn0 = a[0], mx0 = a[0], mn1 = b[0], mx1 = b[0];
	for (int i = threadIdx.x; i < size; i += blockDim.x) {
		mn0 = fminf(mn0, a[i]);
		mx0 = fmaxf(mx0, a[i]);
		mn1 = fminf(mn1, b[i]);
		mx1 = fmaxf(mx1, b[i]);
	}
	smin[0][threadIdx.x] = mn0;
	smax[0][threadIdx.x] = mx0;
	smin[1][threadIdx.x] = mn1;
	smax[1][threadIdx.x] = mx1;
	__syncthreads();
	for (int h = blockDim.x / 2; h > 0; h >>= 1) {
		if ((int)threadIdx.x < h)
			for (int k = 0; k < 2; k++) {
				smin[k][threadIdx.x] = fminf(smin[k][threadIdx.x], smin[k][threadIdx.x + h]);
				smax[k][threadIdx.x] = fmaxf(smax[k][threadIdx.x], smax[k][threadIdx.x + h]);
			}
		__syncthreads();
	}
	const float mx = smax[0][0] > smax[1][0] ? smax[0][0] : smax[1][0];
	const float mn = smin[0][0] < smin[1][0] ? smin[0][0] : smin[1][0];
	const float den = mx - mn;
	float *o0 = O0 + (size_t)pair * size, *o1 = O1 + (size_t)pair * size;
	for (int i = threadIdx.x; i < size; i += blockDim.x) {
		if (den > 0) {
			o0[i] = (float)(255.0 * (double)(a[i] - mn) / (double)den);
			o1[i] = (float)(255.0 * (double)(b[i] - mn) / (double)den);
		} else {
			o0[i] = a[i];
			o1[i] = b[i];
		}
	}
}

// one pass of the separable Gaussian with the reflecting boundary of mask.c
// (rows: step 1 along x; columns: along y), double accumulation
__global__ void gauss_pass_kernel(const float *__restrict__ in, float *__restrict__ out, int nx, int ny,
                                  int npairs, int taps, int along_y)
{
	const long long total = (long long)npairs * nx * ny;
	for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total;
	     q += (long long)gridDim.x * blockDim.x) {
		const long long base = q - q % ((long long)nx * ny);
		const int pix = (int)(q % ((long long)nx * ny));
		const int y = pix / nx, x = pix % nx;
		const int n = along_y ? ny : nx, pos = along_y ? y : x;
		auto at = [&](int m) -> double {
			if (m < 0) m = -m;
			else if (m >= n) m = n - (m - n) - 1;
			return (double)(along_y ? in[base + (long long)m * nx + x] : in[base + (long long)y * nx + m]);
		};
		double sum = c_gauss[0] * at(pos);
		for (int j = 1; j < taps; j++) sum += c_gauss[j] * (at(pos - j) + at(pos + j));
		out[q] = (float)sum;
	}
}

// zoom_out's resampling (after the smoothing) and zoom_in, with an optional
// scale of the values (the flow's 1/zfactor)
__global__ void resample_kernel(const float *__restrict__ in, int nx, int ny, float *__restrict__ out, int nxx,
                                int nyy, int npairs, float fx, float fy, int zoom_in, float scale, int use_scale)
{
	const long long total = (long long)npairs * nxx * nyy;
	for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total;
	     q += (long long)gridDim.x * blockDim.x) {
		const int pair = (int)(q / ((long long)nxx * nyy));
		const int pix = (int)(q % ((long long)nxx * nyy));
		const int i1 = pix / nxx, j1 = pix % nxx;
		const float i2 = zoom_in ? (float)i1 / fy : (float)i1 / fy;
		const float j2 = zoom_in ? (float)j1 / fx : (float)j1 / fx;
		float g = bicubic_at(in + (size_t)pair * nx * ny, j2, i2, nx, ny, false);
		if (use_scale) g *= scale;
		out[q] = g;
	}
}

__global__ void centered_gradient_kernel(const float *__restrict__ in, float *__restrict__ dx,
                                         float *__restrict__ dy, int nx, int ny, int npairs)
{
	const long long total = (long long)npairs * nx * ny;
	for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total;
	     q += (long long)gridDim.x * blockDim.x) {
		const long long base = q - q % ((long long)nx * ny);
		const float *f = in + base;
		const int k = (int)(q - base), i = k / nx, j = k % nx;
		const int l = j > 0 ? k - 1 : k, r = j < nx - 1 ? k + 1 : k;
		const int u = i > 0 ? k - nx : k, d = i < ny - 1 ? k + nx : k;
		dx[q] = 0.5f * (f[r] - f[l]);
		dy[q] = 0.5f * (f[d] - f[u]);
	}
}

// the three warps of a warping step and the constant parts of rho
__global__ void warp_kernel(const float *__restrict__ I0, const float *__restrict__ I1,
                            const float *__restrict__ I1x, const float *__restrict__ I1y,
                            const float *__restrict__ u1, const float *__restrict__ u2, float *__restrict__ I1wx,
                            float *__restrict__ I1wy, float *__restrict__ grad, float *__restrict__ rho_c, int nx,
                            int ny, int npairs)
{
	const long long total = (long long)npairs * nx * ny;
	for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total;
	     q += (long long)gridDim.x * blockDim.x) {
		const long long base = q - q % ((long long)nx * ny);
		const int p = (int)(q - base), i = p / nx, j = p % nx;
		const float uu = (float)j + u1[q], vv = (float)i + u2[q];
		const float w = bicubic_at(I1 + base, uu, vv, nx, ny, true);
		const float wx = bicubic_at(I1x + base, uu, vv, nx, ny, true);
		const float wy = bicubic_at(I1y + base, uu, vv, nx, ny, true);
		I1wx[q] = wx;
		I1wy[q] = wy;
		grad[q] = wx * wx + wy * wy;
		rho_c[q] = w - wx * u1[q] - wy * u2[q] - I0[q];
	}
}

struct IterArgs {
	const float *I1wx, *I1wy, *grad, *rho_c;
	float *u1, *u2, *p11, *p12, *p21, *p22;
	float *partial;          // [2][npairs][bpp]
	int *active;             // [npairs]
	int *iters;              // [npairs]
	int nx, ny, npairs, bpp;
	float tau, lambda, theta, eps2;
};

// The fixed-point iterations of one warping step for every pair
// (tvl1flow_lib.c:163-246).  Block b serves pair b / bpp.
__global__ void __launch_bounds__(256) iterate_kernel(IterArgs a)
{
	cg::grid_group grid = cg::this_grid();
	__shared__ float red[256];
	__shared__ int s_any;
	const int pair = blockIdx.x / a.bpp, sub = blockIdx.x % a.bpp;
	const int size = a.nx * a.ny;
	const long long base = (long long)pair * size;
	const float l_t = a.lambda * a.theta;
	const float taut = a.tau / a.theta;
	for (int n = 0; n < kMaxIterations; n++) {
		const bool act = a.active[pair] != 0;
		float err = 0.f;
		if (act) {
			// thresholding, divergence of p, update of u (in place: only the
			// pixel's own u is read)
			for (int p = sub * blockDim.x + threadIdx.x; p < size; p += a.bpp * blockDim.x) {
				const long long q = base + p;
				const int i = p / a.nx, j = p % a.nx;
				const float wx = a.I1wx[q], wy = a.I1wy[q], g = a.grad[q];
				const float u1k = a.u1[q], u2k = a.u2[q];
				const float rho = a.rho_c[q] + (wx * u1k + wy * u2k);
				float d1, d2;
				if (rho < -l_t * g) {
					d1 = l_t * wx;
					d2 = l_t * wy;
				} else if (rho > l_t * g) {
					d1 = -l_t * wx;
					d2 = -l_t * wy;
				} else if (g < kGradIsZero) {
					d1 = d2 = 0.f;
				} else {
					const float fi = -rho / g;
					d1 = fi * wx;
					d2 = fi * wy;
				}
				const float v1 = u1k + d1, v2 = u2k + d2;
				const float dp1 = divergence_at(a.p11 + base, a.p12 + base, i, j, a.nx, a.ny);
				const float dp2 = divergence_at(a.p21 + base, a.p22 + base, i, j, a.nx, a.ny);
				const float n1 = v1 + a.theta * dp1, n2 = v2 + a.theta * dp2;
				a.u1[q] = n1;
				a.u2[q] = n2;
				err += (n1 - u1k) * (n1 - u1k) + (n2 - u2k) * (n2 - u2k);
			}
		}
		red[threadIdx.x] = err;
		__syncthreads();
		for (int h = blockDim.x / 2; h > 0; h >>= 1) {
			if ((int)threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
			__syncthreads();
		}
		float *part = a.partial + (size_t)(n & 1) * a.npairs * a.bpp;
		if (threadIdx.x == 0) part[pair * a.bpp + sub] = red[0];
		grid.sync();
		if (act) {
			// gradient of u, update of the dual variable p
			for (int p = sub * blockDim.x + threadIdx.x; p < size; p += a.bpp * blockDim.x) {
				const long long q = base + p;
				const int i = p / a.nx, j = p % a.nx;
				float u1x, u1y, u2x, u2y;
				forward_gradient_at(a.u1 + base, i, j, a.nx, a.ny, u1x, u1y);
				forward_gradient_at(a.u2 + base, i, j, a.nx, a.ny, u2x, u2y);
				// |grad u| in float (the reference's double hypot rounded to
				// float agrees to the last bit or one unit; FP64 is slow here),
				// and 1.0 + x rounded once to float, as the reference's
				// double sum of two floats is
				const float g1 = sqrtf(u1x * u1x + u1y * u1y);
				const float g2 = sqrtf(u2x * u2x + u2y * u2y);
				const float ng1 = 1.f + taut * g1;
				const float ng2 = 1.f + taut * g2;
				a.p11[q] = (a.p11[q] + taut * u1x) / ng1;
				a.p12[q] = (a.p12[q] + taut * u1y) / ng1;
				a.p21[q] = (a.p21[q] + taut * u2x) / ng2;
				a.p22[q] = (a.p22[q] + taut * u2y) / ng2;
			}
		}
		// every block decides the same way for every pair
		if (threadIdx.x == 0) s_any = 0;
		__syncthreads();
		for (int k = threadIdx.x; k < a.npairs; k += blockDim.x) {
			if (!a.active[k]) continue;
			float e = 0.f;
			for (int b = 0; b < a.bpp; b++) e += part[k * a.bpp + b];
			e /= (float)size;
			if (e > a.eps2 && n + 1 < kMaxIterations) atomicOr(&s_any, 1);
		}
		__syncthreads();
		const int any = s_any;
		grid.sync();   // everyone has read this iteration's active flags
		if (blockIdx.x == 0)
			for (int k = threadIdx.x; k < a.npairs; k += blockDim.x) {
				if (!a.active[k]) continue;
				float e = 0.f;
				for (int b = 0; b < a.bpp; b++) e += part[k * a.bpp + b];
				e /= (float)size;
				a.iters[k] = n + 1;
				if (!(e > a.eps2 && n + 1 < kMaxIterations)) a.active[k] = 0;
			}
		grid.sync();
		if (!any) break;
	}
}

__global__ void set_int_kernel(int *p, int n, int v)
{
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) p[i] = v;
}

int grid_of(long long n, int threads = 256) { return (int)std::max<long long>(1, std::min<long long>((n + threads - 1) / threads, 32768)); }

// Gaussian taps of mask.c:211-237, computed on the host in double
int gauss_taps(double sigma, std::vector<double> &B)
{
	const double den = 2 * sigma * sigma;
	const int size = (int)(kGaussWindow * sigma) + 1;
	B.assign(size, 0.0);
	for (int i = 0; i < size; i++) B[i] = 1 / (sigma * sqrt(2.0 * 3.1415926)) * exp(-i * i / den);
	double norm = 0;
	for (int i = 0; i < size; i++) norm += B[i];
	norm *= 2;
	norm -= B[0];
	for (int i = 0; i < size; i++) B[i] /= norm;
	return size;
}

cudaError_t gaussian(float *img, float *tmp, int nx, int ny, int npairs, double sigma, cudaStream_t st)
{
	std::vector<double> B;
	const int taps = gauss_taps(sigma, B);
	if (taps > kMaxGauss || taps > nx || taps > ny) return cudaErrorInvalidValue;   // "sigma too large"
	cudaError_t e = cudaMemcpyToSymbolAsync(c_gauss, B.data(), sizeof(double) * taps, 0, cudaMemcpyHostToDevice, st);
	if (e != cudaSuccess) return e;
	const long long n = (long long)npairs * nx * ny;
	gauss_pass_kernel<<<grid_of(n), 256, 0, st>>>(img, tmp, nx, ny, npairs, taps, 0);
	gauss_pass_kernel<<<grid_of(n), 256, 0, st>>>(tmp, img, nx, ny, npairs, taps, 1);
	return cudaGetLastError();
}

}  // namespace

int tvl1_scales(int nx, int ny, int nscales, float zfactor)
{
	// main.c:147-153: the smallest level is about 16 pixels across
	const float N = (float)(1 + log(hypot(nx, ny) / 16.0) / log(1 / zfactor));
	if (N < nscales) nscales = (int)N;
	return nscales;
}

// The flow of npairs frame pairs (I0[k] -> I1[k], each nx x ny, device
// memory) into u (x displacement) and v (y displacement), [pair][y][x].
// ws: device workspace of tvl1_workspace_floats(...) floats.
size_t tvl1_workspace_floats(int nx, int ny, int npairs, int nscales, float zfactor)
{
	size_t total = 0;
	int w = nx, h = ny;
	for (int s = 0; s < nscales; s++) {
		total += (size_t)4 * w * h * npairs;   // I0, I1, u1, u2 of the level
		const int nw = (int)((float)w * zfactor + 0.5f), nh = (int)((float)h * zfactor + 0.5f);
		w = nw;
		h = nh;
	}
	total += (size_t)13 * nx * ny * npairs;    // per-level work arrays, sized for level 0
	total += (size_t)2 * npairs * 1024 + 64;   // partial sums
	return total;
}

cudaError_t tvl1_flow(const float *I0, const float *I1, int nx, int ny, int npairs, const Tvl1Params &pr,
                      float *u, float *v, float *ws, int *iws, int nsm, cudaStream_t st, std::string &why)
{
	const int nscales = pr.nscales;
	const int fscale = std::min(pr.fscale, nscales);
	std::vector<int> NX(nscales), NY(nscales);
	std::vector<float *> l0(nscales), l1(nscales), lu(nscales), lv(nscales);
	NX[0] = nx;
	NY[0] = ny;
	for (int s = 1; s < nscales; s++) {   // zoom_size (zoom.c:24-35)
		NX[s] = (int)((float)NX[s - 1] * pr.zfactor + 0.5f);
		NY[s] = (int)((float)NY[s - 1] * pr.zfactor + 0.5f);
	}
	float *w = ws;
	for (int s = 0; s < nscales; s++) {
		const size_t n = (size_t)NX[s] * NY[s] * npairs;
		l0[s] = w; w += n;
		l1[s] = w; w += n;
		lu[s] = w; w += n;
		lv[s] = w; w += n;
	}
	const size_t n0 = (size_t)nx * ny * npairs;
	float *I1x = w, *I1y = w + n0, *I1wx = w + 2 * n0, *I1wy = w + 3 * n0, *grad = w + 4 * n0,
	      *rho_c = w + 5 * n0, *p11 = w + 6 * n0, *p12 = w + 7 * n0, *p21 = w + 8 * n0, *p22 = w + 9 * n0,
	      *tmp = w + 10 * n0;
	float *partial = w + 13 * n0;
	int *active = iws, *iters = iws + npairs;

	// normalisation and pre-smoothing (tvl1flow_lib.c:385-390)
	normalize_kernel<<<npairs, 256, 0, st>>>(I0, I1, nx * ny, l0[0], l1[0]);
	cudaError_t e = gaussian(l0[0], tmp, nx, ny, npairs, kPresmoothSigma, st);
	if (e == cudaSuccess) e = gaussian(l1[0], tmp, nx, ny, npairs, kPresmoothSigma, st);
	if (e != cudaSuccess) { why = "image too small for the Gaussian pre-smoothing"; return e; }
	// pyramid (zoom_out, zoom.c:42-77)
	const float zsig = (float)(kZoomSigmaZero * sqrt(1.0 / (pr.zfactor * pr.zfactor) - 1.0));
	for (int s = 1; s < nscales; s++) {
		for (int k = 0; k < 2; k++) {
			float *src = k ? l1[s - 1] : l0[s - 1], *dst = k ? l1[s] : l0[s];
			const size_t n = (size_t)NX[s - 1] * NY[s - 1] * npairs;
			e = cudaMemcpyAsync(tmp + n0, src, sizeof(float) * n, cudaMemcpyDeviceToDevice, st);   // Is = I
			if (e == cudaSuccess) e = gaussian(tmp + n0, tmp, NX[s - 1], NY[s - 1], npairs, (double)zsig, st);
			if (e != cudaSuccess) { why = "pyramid level too small for the Gaussian"; return e; }
			resample_kernel<<<grid_of((long long)NX[s] * NY[s] * npairs), 256, 0, st>>>(
			    tmp + n0, NX[s - 1], NY[s - 1], dst, NX[s], NY[s], npairs, pr.zfactor, pr.zfactor, 0, 1.f, 0);
		}
	}
	const size_t nc = (size_t)NX[nscales - 1] * NY[nscales - 1] * npairs;
	cudaMemsetAsync(lu[nscales - 1], 0, sizeof(float) * nc, st);
	cudaMemsetAsync(lv[nscales - 1], 0, sizeof(float) * nc, st);

	int per_sm = 0;
	e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, iterate_kernel, 256, 0);
	if (e != cudaSuccess) return e;
	const int maxb = std::max(1, per_sm) * nsm;
	if (npairs > maxb) { why = "too many frame pairs for one cooperative launch"; return cudaErrorInvalidValue; }
	const float scale = (float)1.0 / pr.zfactor;
	for (int s = nscales - 1; s >= fscale; s--) {
		const int sx = NX[s], sy = NY[s];
		const size_t n = (size_t)sx * sy * npairs;
		const long long nn = (long long)n;
		centered_gradient_kernel<<<grid_of(nn), 256, 0, st>>>(l1[s], I1x, I1y, sx, sy, npairs);
		cudaMemsetAsync(p11, 0, sizeof(float) * 4 * n0, st);   // p11, p12, p21, p22 (contiguous)
		const int bpp = std::max(1, std::min(maxb / npairs, (int)((n / npairs + 255) / 256)));
		for (int wp = 0; wp < pr.warps; wp++) {
			warp_kernel<<<grid_of(nn), 256, 0, st>>>(l0[s], l1[s], I1x, I1y, lu[s], lv[s], I1wx, I1wy, grad, rho_c,
			                                         sx, sy, npairs);
			set_int_kernel<<<grid_of(npairs), 256, 0, st>>>(active, npairs, 1);
			IterArgs a;
			a.I1wx = I1wx;
			a.I1wy = I1wy;
			a.grad = grad;
			a.rho_c = rho_c;
			a.u1 = lu[s];
			a.u2 = lv[s];
			a.p11 = p11;
			a.p12 = p12;
			a.p21 = p21;
			a.p22 = p22;
			a.partial = partial;
			a.active = active;
			a.iters = iters;
			a.nx = sx;
			a.ny = sy;
			a.npairs = npairs;
			a.bpp = bpp;
			a.tau = pr.tau;
			a.lambda = pr.lambda;
			a.theta = pr.theta;
			a.eps2 = pr.epsilon * pr.epsilon;
			void *args[] = {&a};
			e = cudaLaunchCooperativeKernel((const void *)iterate_kernel, dim3(npairs * bpp), dim3(256), args, 0, st);
			if (e != cudaSuccess) { why = "cooperative launch failed"; return e; }
		}
		if (s == 0) break;
		// zoom the flow to the next finer level and scale it (tvl1flow_lib.c:429-440)
		const float fx = (float)NX[s - 1] / sx, fy = (float)NY[s - 1] / sy;
		const long long nf = (long long)NX[s - 1] * NY[s - 1] * npairs;
		resample_kernel<<<grid_of(nf), 256, 0, st>>>(lu[s], sx, sy, lu[s - 1], NX[s - 1], NY[s - 1], npairs, fx, fy, 1,
		                                             scale, 1);
		resample_kernel<<<grid_of(nf), 256, 0, st>>>(lv[s], sx, sy, lv[s - 1], NX[s - 1], NY[s - 1], npairs, fx, fy, 1,
		                                             scale, 1);
	}
	// levels below fscale only pass the flow up (tvl1flow_lib.c:443-459)
	for (int s = fscale - 1; s >= 1; s--) {
		const float fx = (float)NX[s - 1] / NX[s], fy = (float)NY[s - 1] / NY[s];
		const long long nf = (long long)NX[s - 1] * NY[s - 1] * npairs;
		resample_kernel<<<grid_of(nf), 256, 0, st>>>(lu[s], NX[s], NY[s], lu[s - 1], NX[s - 1], NY[s - 1], npairs, fx, fy,
		                                             1, scale, 1);
		resample_kernel<<<grid_of(nf), 256, 0, st>>>(lv[s], NX[s], NY[s], lv[s - 1], NX[s - 1], NY[s - 1], npairs, fx, fy,
		                                             1, scale, 1);
	}
	e = cudaMemcpyAsync(u, lu[0], sizeof(float) * n0, cudaMemcpyDeviceToDevice, st);
	if (e == cudaSuccess) e = cudaMemcpyAsync(v, lv[0], sizeof(float) * n0, cudaMemcpyDeviceToDevice, st);
	if (e == cudaSuccess) e = cudaGetLastError();
	return e;
}

}  // namespace bm4dof
