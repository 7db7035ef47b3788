"""The noise and PSNR tools of the reference's evaluation script
(scripts/bm4dof-gt.sh runs awgn, the denoiser, then psnr), built beside the
command line as bm4d-of_gb300/lib/awgn and bm4d-of_gb300/lib/psnr (host code):
their arguments, messages and output formats (src/awgn.cpp, src/psnr.cpp), the
PSNR/RMSE arithmetic of VideoUtils::computePSNR, and the noise of
VideoUtils::addNoise -- the MT19937 stream checked against the reference's own
generator (mt19937ar.c, compiled into oracle/_ref), the Box-Muller transform
restated here in long double."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from helpers import ROOT

LIB = os.path.join(ROOT, "bm4d-of_gb300", "lib")
AWGN = os.path.join(LIB, "awgn")
PSNR = os.path.join(LIB, "psnr")


@pytest.fixture(scope="module")
def tools(gpulib):
    assert os.path.exists(AWGN) and os.path.exists(PSNR)
    return AWGN, PSNR


def write_pfm(path, planar):
    c, h, w = planar.shape
    with open(path, "wb") as f:
        f.write(f"{'PF' if c == 3 else 'Pf'}\n{w} {h}\n-1.0\n".encode())
        f.write(np.ascontiguousarray(planar.transpose(1, 2, 0)[::-1], "<f4").tobytes())


def read_pfm(path):
    with open(path, "rb") as f:
        tag = f.readline().strip()
        w, h = map(int, f.readline().split())
        scale = float(f.readline())
        c = 3 if tag == b"PF" else 1
        a = np.frombuffer(f.read(), "<f4" if scale < 0 else ">f4").reshape(h, w, c)[::-1]
    return np.ascontiguousarray(a.transpose(2, 0, 1))


def run(exe, *args, env=None):
    return subprocess.run([exe, *map(str, args)], capture_output=True, text=True, timeout=60,
                          env=dict(os.environ, **(env or {})))


def test_tool_usage_and_errors(tools, tmp_path):
    awgn, psnr = tools
    r = run(awgn, 10)
    assert r.returncode == 1 and "USAGE: awgn sigma input-path output-path [first-frame last-frame]" in r.stdout
    r = run(psnr, "a")
    assert r.returncode == 1 and "USAGE: psnr input1-path input2-path [first-frame last-frame [output-file]]" \
        in r.stdout
    r = run(awgn, 10, tmp_path / "missing_%03d.pfm", tmp_path / "o_%03d.pfm", 0, 1)
    assert r.returncode == 1 and f"Video<T>::loadVideo: loading of {tmp_path}/missing_000.pfm failed" in r.stderr
    write_pfm(tmp_path / "a_000.pfm", np.zeros((1, 4, 5), np.float32))
    write_pfm(tmp_path / "b_000.pfm", np.zeros((1, 4, 6), np.float32))
    r = run(psnr, tmp_path / "a_%03d.pfm", tmp_path / "b_%03d.pfm")
    assert r.returncode == 1 and "VideoUtils::computePSNR: videos have different sizes" in r.stderr


def close(printed, want):
    return abs(printed - float(want)) <= 1e-6 * abs(float(want)) + 1e-6


def expected_psnr(a, b):
    d = (a.astype(np.float64) - b.astype(np.float64)) ** 2
    rmse = np.sqrt(np.float32(d.sum() / d.size))
    return np.float32(20) * np.log10(np.float32(255) / rmse), rmse


def test_psnr_global_per_frame_and_file(tools, tmp_path):
    _, psnr = tools
    rng = np.random.default_rng(5)
    F = 3
    a = rng.uniform(0, 255, (F, 3, 9, 11)).astype(np.float32)
    b = (a + rng.normal(0, 7, a.shape)).astype(np.float32)
    for t in range(F):
        write_pfm(tmp_path / f"a_{t + 2:03d}.pfm", a[t])
        write_pfm(tmp_path / f"b_{t + 2:03d}.pfm", b[t])
    out = tmp_path / "measures"
    out.write_text("earlier\n")
    r = run(psnr, tmp_path / "a_%03d.pfm", tmp_path / "b_%03d.pfm", 2, 2 + F - 1, out)
    assert r.returncode == 0, r.stderr
    p, e = expected_psnr(a, b)
    lines = r.stdout.splitlines()
    assert lines[0].startswith("PSNR ") and lines[1].startswith("RMSE ")
    # within an ulp or two of float32 (log10f and numpy's float32 log10 may
    # round differently) and the 6 printed decimals
    assert close(float(lines[0].split()[1]), p) and close(float(lines[1].split()[1]), e)
    text = out.read_text().splitlines()
    assert text[0] == "earlier"                                   # appended, as the reference does
    assert text[1] == lines[0].replace("PSNR", "Total PSNR") and text[2] == lines[1].replace("RMSE", "Total RMSE")
    assert text[3].startswith("Frame PSNR ") and text[4].startswith("Frame RMSE  ")
    fp = [float(x) for x in text[3].split()[2:]]
    fr = [float(x) for x in text[4].split()[2:]]
    for t in range(F):
        pt, et = expected_psnr(a[t], b[t])
        assert close(fp[t], pt) and close(fr[t], et)
    # one image: no per-frame lines
    out2 = tmp_path / "m2"
    r = run(psnr, tmp_path / "a_%03d.pfm", tmp_path / "b_%03d.pfm", 2, 2, out2)
    assert r.returncode == 0 and len(out2.read_text().splitlines()) == 2


def reference_mt(seed, n):
    import pyoracle
    if not pyoracle.Reference.available():
        pytest.skip("reference sources not present (oracle/_ref not built)")
    L = C.CDLL(pyoracle.REF_SO)
    L.mt_init_genrand.argtypes = [C.c_ulong]
    L.mt_genrand_res53.restype = C.c_double
    L.mt_init_genrand(seed)
    return np.array([L.mt_genrand_res53() for _ in range(n)])


def test_awgn_noise_follows_the_reference_generator(tools, reference, tmp_path):
    awgn, _ = tools
    rng = np.random.default_rng(6)
    F, sigma, seed = 2, 25.0, 4242
    clean = rng.uniform(0, 255, (F, 1, 7, 13)).astype(np.float32)
    for t in range(F):
        write_pfm(tmp_path / f"c_{t:03d}.pfm", clean[t])
    r = run(awgn, sigma, tmp_path / "c_%03d.pfm", tmp_path / "n_%03d.pfm", 0, F - 1,
            env={"BM4DOF_AWGN_SEED": str(seed)})
    assert r.returncode == 0, r.stderr
    noisy = np.stack([read_pfm(tmp_path / f"n_{t:03d}.pfm") for t in range(F)])
    u = reference_mt(seed, 2 * clean.size)
    a, b = u[0::2], u[1::2]
    ld = np.longdouble
    z = ld(np.float32(sigma)) * np.sqrt(ld(-2.0) * np.log(a).astype(ld)) * np.cos(ld(2.0) * ld(np.pi) * b.astype(ld))
    want = (clean.ravel() + z.astype(np.float32)).astype(np.float32).reshape(clean.shape)
    assert np.array_equal(noisy, want)
    assert abs(float((noisy - clean).std()) - sigma) < 0.15 * sigma


def test_awgn_unseeded_runs_differ(tools, tmp_path):
    awgn, _ = tools
    write_pfm(tmp_path / "c_000.pfm", np.zeros((1, 6, 6), np.float32))
    r1 = run(awgn, 10, tmp_path / "c_%03d.pfm", tmp_path / "x_%03d.pfm")
    r2 = run(awgn, 10, tmp_path / "c_%03d.pfm", tmp_path / "y_%03d.pfm")
    assert r1.returncode == 0 and r2.returncode == 0
    assert not np.array_equal(read_pfm(tmp_path / "x_000.pfm"), read_pfm(tmp_path / "y_000.pfm"))
