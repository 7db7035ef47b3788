"""The bm4dof command line (bm4d-of_gb300/lib/bm4dof): the reference CLI's
flags, checks and parameter printing (src/main_vnlb.cpp), the PFM / .flo frame
files, and -- on the GPU -- the same output as the library call."""
import os
import struct
import subprocess

import numpy as np
import pytest

from helpers import resolve_params, video_case

HERE = os.path.dirname(os.path.abspath(__file__))
CLI = os.path.join(os.path.dirname(HERE), "bm4d-of_gb300", "lib", "bm4dof")


@pytest.fixture(scope="module")
def cli(gpulib):
    assert os.path.exists(CLI)
    return CLI


def write_pfm(path, planar):
    """planar (C, H, W) float32, C in {1, 3}."""
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
    return np.ascontiguousarray(a.transpose(2, 0, 1)).astype(np.float32)


def write_flo(path, planar):
    _, h, w = planar.shape
    with open(path, "wb") as f:
        f.write(struct.pack("<fii", 202021.25, w, h))
        f.write(np.ascontiguousarray(planar.transpose(1, 2, 0), "<f4").tobytes())


def run(cli, *args):
    return subprocess.run([cli, *map(str, args)], capture_output=True, text=True)


def test_cli_checks(cli):
    r = run(cli)
    assert r.returncode == 1 and "no input sequence" in r.stderr
    r = run(cli, "-i", "x_%03d.pfm", "-px1", 0, "-px2", 4)
    assert r.returncode == 1 and "a basic sequence path must be given" in r.stderr
    r = run(cli, "-i", "x_%03d.pfm", "-fof", "f_%03d.flo")
    assert r.returncode == 1 and "Only one oflow path provided" in r.stderr
    r = run(cli, "-i", "x_%03d.pfm", "-px1", 0, "-px2", 0)
    assert r.returncode == 1 and "Nothing to do" in r.stderr
    r = run(cli, "-i", "missing_%03d.pfm")
    assert r.returncode == 1 and "loading of missing_000.pfm failed" in r.stderr


def test_cli_print_params(cli, oracle):
    r = run(cli, "-i", "unused", "-print-prms", 1, "-sigma", 20, "-px1", 4, "-pt1", 4, "-np2", 32, "-b1", 2.5)
    assert r.returncode == 0
    size = (0, 0, 0, 1)
    p1, p2 = resolve_params(oracle, size, 20.0, px1=4, pt1=4, np2=32, b1=2.5)
    assert r.stdout == oracle.formatNlbParameters(p1) + oracle.formatNlbParameters(p2)


def test_cli_under_the_scripts_name(cli):
    # scripts/bm4dof.sh runs "$DIR/bm4d-of"; the build provides that name too
    alias = os.path.join(os.path.dirname(cli), "bm4d-of")
    r = run(alias, "-i", "unused", "-print-prms", 1, "-sigma", 20)
    assert r.returncode == 0 and r.stdout == run(cli, "-i", "unused", "-print-prms", 1, "-sigma", 20).stdout


def test_cli_print_params_tau(cli, oracle):
    # -print-prms takes -t1/-t2 in every build (main_vnlb.cpp:173-174)
    r = run(cli, "-i", "unused", "-print-prms", 1, "-sigma", 20, "-t1", 50, "-t2", 12.5)
    assert r.returncode == 0
    p1, p2 = resolve_params(oracle, (0, 0, 0, 1), 20.0, t1=50.0, t2=12.5)
    assert r.stdout == oracle.formatNlbParameters(p1) + oracle.formatNlbParameters(p2)


def test_cli_print_params_vbm3d(cli):
    # -vbm3d prints what the reference built with VBM3D_SEARCH prints
    import pyoracle
    if not pyoracle.Reference.available(pyoracle.REF_VBM3D_SO):
        pytest.skip("reference sources not present (oracle/_ref not built)")
    ref = pyoracle.Reference(pyoracle.REF_VBM3D_SO)
    r = run(cli, "-i", "unused", "-print-prms", 1, "-vbm3d", 1, "-sigma", 20, "-px1", 4, "-npf1", 3,
            "-wxf2", 7, "-dsub2", 1.5, "-t1", 40)
    assert r.returncode == 0
    p1, p2 = resolve_params(ref, (0, 0, 0, 1), 20.0, px1=4, npf1=3, wxf2=7, dsub2=1.5, t1=40.0)
    assert r.stdout == ref.formatNlbParameters(p1) + ref.formatNlbParameters(p2)


def test_frame_formats_round_trip(tmp_path):
    rng = np.random.default_rng(0)
    a = rng.normal(0, 50, (3, 7, 5)).astype(np.float32)
    write_pfm(tmp_path / "a.pfm", a)
    assert np.array_equal(read_pfm(tmp_path / "a.pfm"), a)


@pytest.mark.gpu
def test_cli_matches_oracle(cli, gpulib, oracle, tmp_path):
    # the CLI is its own process: the test process makes no CUDA context (a
    # GPU in exclusive-process mode admits one), and checks against the oracle
    W, H, F, sigma = 48, 40, 6, 20.0
    clean, nz, ff, bf = video_case(W, H, F, sigma=sigma, seed=31)
    for t in range(F):
        write_pfm(tmp_path / f"n_{t:03d}.pfm", nz[t])
        write_flo(tmp_path / f"f_{t:03d}.flo", ff[t])
        write_flo(tmp_path / f"b_{t:03d}.flo", bf[t])
    r = run(cli, "-i", tmp_path / "n_%03d.pfm", "-fof", tmp_path / "f_%03d.flo", "-bof", tmp_path / "b_%03d.flo",
            "-f", 0, "-l", F - 1, "-sigma", sigma, "-px1", 4, "-px2", 4, "-pt1", 4, "-pt2", 4, "-np1", 16,
            "-np2", 16, "-wx1", 21, "-wx2", 21, "-b1", 3, "-verbose", 0,
            "-deno", tmp_path / "d_%03d.pfm", "-bsic", tmp_path / "s_%03d.pfm")
    assert r.returncode == 0, r.stderr[-2000:]
    p1, p2 = resolve_params(oracle, (W, H, F, 1), sigma, px1=4, px2=4, pt1=4, pt2=4, np1=16, np2=16,
                            wx1=21, wx2=21, b1=3.0)
    basic, final, _ = oracle.runNlBayes(nz, ff, bf, p1, p2, nparts=2)
    got_f = np.stack([read_pfm(tmp_path / f"d_{t:03d}.pfm") for t in range(F)])
    got_b = np.stack([read_pfm(tmp_path / f"s_{t:03d}.pfm") for t in range(F)])
    assert np.array_equal(got_f, final) and np.array_equal(got_b, basic)
    # 8-bit PNG output
    r = run(cli, "-i", tmp_path / "n_%03d.pfm", "-f", 0, "-l", 1, "-sigma", sigma, "-verbose", 0,
            "-deno", tmp_path / "d_%03d.png", "-bsic", tmp_path / "s_%03d.png")
    assert r.returncode == 0, r.stderr[-2000:]
    assert (tmp_path / "d_001.png").read_bytes()[:8] == b"\x89PNG\r\n\x1a\n"


@pytest.mark.gpu
def test_cli_vbm3d_matches_oracle(cli, gpulib, oracle, tmp_path):
    # -vbm3d: the predictive search, with its per-frame options and -t1
    W, H, F, sigma = 44, 36, 6, 20.0
    clean, nz, ff, bf = video_case(W, H, F, sigma=sigma, seed=32)
    for t in range(F):
        write_pfm(tmp_path / f"n_{t:03d}.pfm", nz[t])
        write_flo(tmp_path / f"f_{t:03d}.flo", ff[t])
        write_flo(tmp_path / f"b_{t:03d}.flo", bf[t])
    r = run(cli, "-i", tmp_path / "n_%03d.pfm", "-fof", tmp_path / "f_%03d.flo", "-bof", tmp_path / "b_%03d.flo",
            "-f", 0, "-l", F - 1, "-sigma", sigma, "-px1", 4, "-px2", 4, "-pt1", 2, "-pt2", 2, "-np1", 16,
            "-np2", 16, "-wx1", 15, "-wx2", 15, "-vbm3d", 1, "-npf1", 3, "-wxf2", 7, "-t1", 60, "-verbose", 0,
            "-deno", tmp_path / "d_%03d.pfm", "-bsic", tmp_path / "s_%03d.pfm")
    assert r.returncode == 0, r.stderr[-2000:]
    p1, p2 = resolve_params(oracle, (W, H, F, 1), sigma, px1=4, px2=4, pt1=2, pt2=2, np1=16, np2=16,
                            wx1=15, wx2=15, npf1=3, wxf2=7, t1=60.0)
    basic, final, _ = oracle.runNlBayes(nz, ff, bf, p1, p2, nparts=2, vbm3d=True)
    got_f = np.stack([read_pfm(tmp_path / f"d_{t:03d}.pfm") for t in range(F)])
    got_b = np.stack([read_pfm(tmp_path / f"s_{t:03d}.pfm") for t in range(F)])
    assert np.array_equal(got_f, final) and np.array_equal(got_b, basic)
