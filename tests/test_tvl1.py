"""TV-L1 optical flow (lib/tvl1flow): the golden fixtures made by the
reference's own code, the GPU restatement against them, the video layout of
bm4dof_tvl1_video (tvl1flow-seq.sh's copy convention), the denoiser fed
with GPU flow, and the tvl1flow command line (lib/tvl1flow/main.c): its
checks and messages on the CPU, its flow on the GPU."""
import os
import struct
import subprocess

import numpy as np
import pytest

from helpers import ROOT, psnr, resolve_params, video_case

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
NAMES = ["tvl1_clean_fwd", "tvl1_noisy_bwd", "tvl1_noisy_full"]
TVL1_CLI = os.path.join(ROOT, "bm4d-of_gb300", "lib", "tvl1flow")


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


# ---- the tvl1flow command line -----------------------------------------------
@pytest.fixture(scope="module")
def tvl1_cli(gpulib):
    assert os.path.exists(TVL1_CLI)
    return TVL1_CLI


def write_grey_pfm(path, img):
    h, w = img.shape
    with open(path, "wb") as f:
        f.write(f"Pf\n{w} {h}\n-1.0\n".encode())
        f.write(np.ascontiguousarray(img[::-1], "<f4").tobytes())


def read_flo(path):
    with open(path, "rb") as f:
        magic, w, h = struct.unpack("<fii", f.read(12))
        assert magic == 202021.25
        return np.frombuffer(f.read(), "<f4").reshape(h, w, 2).transpose(2, 0, 1)


def run(exe, *args):
    return subprocess.run([exe, *map(str, args)], capture_output=True, text=True, timeout=120)


def test_tvl1flow_cli_checks(tvl1_cli, tmp_path):
    # every case below ends before the GPU is touched (main.c:74-80, 44-49, 194-197)
    r = run(tvl1_cli, "a.pfm")
    assert r.returncode == 1
    assert "I0 I1 [out nproc tau lambda theta nscales fscale zfactor nwarps epsilon verbose]" in r.stderr
    a, b, c = tmp_path / "a.pfm", tmp_path / "b.pfm", tmp_path / "c.pfm"
    write_grey_pfm(a, np.zeros((4, 5), np.float32))
    write_grey_pfm(b, np.zeros((4, 6), np.float32))
    r = run(tvl1_cli, a, tmp_path / "missing.pfm")
    assert r.returncode == 1 and f'ERROR: could not read image from file "{tmp_path / "missing.pfm"}"' in r.stderr
    r = run(tvl1_cli, a, b)
    assert r.returncode == 1 and "ERROR: input images size mismatch 5x4 != 6x4" in r.stderr
    flo = tmp_path / "f.flo"
    with open(flo, "wb") as f:
        f.write(struct.pack("<fii", 202021.25, 5, 4) + bytes(4 * 2 * 20))
    r = run(tvl1_cli, flo, a)
    assert r.returncode == 1 and "non-scalarizable image" in r.stderr
    write_grey_pfm(c, np.zeros((1, 1), np.float32))
    r = run(tvl1_cli, c, c)
    assert r.returncode == 1 and "at least 2x2" in r.stderr
    # out-of-range parameters are replaced and, with verbose, reported (main.c:101-140)
    r = run(tvl1_cli, a, b, tmp_path / "o.flo", -1, 0.5, 0, -1, 0, 0, 1.5, 0, 0, 1)
    for line in ["warning: nproc changed to 0", "warning: tau changed to 0.25", "warning: lambda changed to 0.15",
                 "warning: theta changed to 0.3", "warning: nscales changed to 100", "warning: zfactor changed to 0.5",
                 "warning: nwarps changed to 5", "warning: epsilon changed to 0.010000"]:
        assert line in r.stderr, line
    assert r.returncode == 1 and "size mismatch" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_gpu_tvl1flow_cli(tvl1_cli, gpuctx, tmp_path, name):
    # tvl1flow-seq.sh's call: nproc 6, then 0.25 0.2 0.3 100 fscale 0.5 5 0.01, here verbose
    g = load(name)
    a, b, out = tmp_path / "a.pfm", tmp_path / "b.pfm", tmp_path / "flow.flo"
    write_grey_pfm(a, g["I0"])
    write_grey_pfm(b, g["I1"])
    fscale = int(g["fscale"])
    r = run(tvl1_cli, a, b, out, 6, 0.25, 0.2, 0.3, 100, fscale, 0.5, 5, 0.01, 1)
    assert r.returncode == 0, r.stderr
    H, W = g["I0"].shape
    assert f"nscales={int(1 + np.log(np.hypot(W, H) / 16.0) / np.log(2.0))}" in r.stderr
    assert f"Scale {fscale}: " in r.stderr
    uv = read_flo(out)
    lib = gpuctx.tvl1_pairs(g["I0"], g["I1"], gpuctx.tvl1_params(fscale=fscale))
    assert np.array_equal(uv, lib)
    epe = np.hypot(uv[0] - g["u"], uv[1] - g["v"])
    assert epe.mean() < 0.02 and np.percentile(epe, 99) < 0.2
