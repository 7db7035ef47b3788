"""TV-L1 optical flow (lib/tvl1flow): the golden fixtures made by the
reference's own code, the GPU restatement against them, the video layout of
bm4dof_tvl1_video (tvl1flow-seq.sh's copy convention) and the denoiser fed
with GPU flow."""
import os

import numpy as np
import pytest

from helpers import psnr, resolve_params, video_case

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
NAMES = ["tvl1_clean_fwd", "tvl1_noisy_bwd", "tvl1_noisy_full"]


def load(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


@pytest.mark.parametrize("name", NAMES)
def test_reference_flow_fixture(name, reference):
    # the fixture is what the reference computes now, and it tracks the true motion
    import importlib.util
    spec = importlib.util.spec_from_file_location("mk", os.path.join(GOLDEN, "make_tvl1_golden.py"))
    mk = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mk)
    g = load(name)
    u, v = mk.ref_tvl1(g["I0"], g["I1"], int(g["fscale"]))
    assert np.array_equal(u, g["u"]) and np.array_equal(v, g["v"])
    # the flow explains the motion: warping I1 back by it cuts the residual
    assert warp_residual(g["I0"], g["I1"], g["u"], g["v"]) < 0.8 * warp_residual(g["I0"], g["I1"], 0 * u, 0 * v)


def warp_residual(I0, I1, u, v):
    """mean |I1(x + u) - I0(x)| (bilinear, clamped), away from the border"""
    H, W = I0.shape
    yy, xx = np.mgrid[0:H, 0:W].astype(np.float64)
    x = np.clip(xx + u, 0, W - 1)
    y = np.clip(yy + v, 0, H - 1)
    x0, y0 = np.floor(x).astype(int), np.floor(y).astype(int)
    x1, y1 = np.minimum(x0 + 1, W - 1), np.minimum(y0 + 1, H - 1)
    fx, fy = x - x0, y - y0
    w = (I1[y0, x0] * (1 - fx) + I1[y0, x1] * fx) * (1 - fy) + (I1[y1, x0] * (1 - fx) + I1[y1, x1] * fx) * fy
    return float(np.abs(w - I0)[4:-4, 4:-4].mean())


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_gpu_tvl1_matches_reference(gpulib, gpuctx, name):
    g = load(name)
    p = gpuctx.tvl1_params(fscale=int(g["fscale"]))
    uv = gpuctx.tvl1_pairs(g["I0"], g["I1"], p)
    epe = np.hypot(uv[0] - g["u"], uv[1] - g["v"])
    print(name, "EPE vs reference: mean", epe.mean(), "max", epe.max())
    assert epe.mean() < 0.02 and np.percentile(epe, 99) < 0.2


@pytest.mark.gpu
def test_gpu_tvl1_video_layout_and_denoising(gpulib, gpuctx):
    W, H, F, sigma = 64, 56, 5, 20.0
    clean, nz, ff_true, bf_true = video_case(W, H, F, sigma=sigma, seed=12)
    ff, bf = gpuctx.tvl1_video(nz)
    pairs_f = gpuctx.tvl1_pairs(nz[:-1, 0], nz[1:, 0])
    pairs_b = gpuctx.tvl1_pairs(nz[1:, 0], nz[:-1, 0])
    assert np.array_equal(ff[:-1], pairs_f) and np.array_equal(ff[-1], ff[-2])
    assert np.array_equal(bf[1:], pairs_b) and np.array_equal(bf[0], bf[1])
    p1, p2 = resolve_params(gpulib, (W, H, F, 1), sigma, px1=4, px2=4, pt1=4, pt2=4, np1=16, np2=16, wx1=21,
                            wx2=21, b1=3.0)
    _, f_tv, _ = gpuctx.runNlBayes(nz, ff, bf, p1, p2)
    _, f_ex, _ = gpuctx.runNlBayes(nz, ff_true, bf_true, p1, p2)
    assert psnr(f_tv, clean) > psnr(nz, clean) + 8.0
    assert abs(psnr(f_tv, clean) - psnr(f_ex, clean)) < 1.0
