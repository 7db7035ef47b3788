"""GPU parity: the plain FP32 path of libbm4dof_gpu.so against the oracle and
the reference's golden outputs.  The bar is bit-identical output (max |diff|
= 0, which is inside the 1e-2 grey-level / 0.01 dB tolerance) and identical
neighbour lists, order included."""
import os

import numpy as np
import pytest

from cases import CASES, CFG_VIDEO
from helpers import ROOT, psnr, resolve_params, video_case

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(ROOT, "tests", "golden")
TOL_GREY = 1e-2      # max |diff| allowed on [0, 255]
TOL_PSNR = 0.01      # dB


def gparams(gpulib, arr):
    p = gpulib.Params()
    for (f, t), v in zip(gpulib.Params._fields_, arr):
        setattr(p, f, float(v) if t.__name__ == "c_float" else int(v))
    return p


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_gpu_matches_golden(gpulib, gpuctx, case):
    g = dict(np.load(os.path.join(GOLDEN, case[0] + ".npz")))
    p1, p2 = gparams(gpulib, g["p1"]), gparams(gpulib, g["p2"])
    nparts = 2 * int(g["nthreads"])
    basic, final, ratios = gpuctx.runNlBayes(g["noisy"], g.get("fflow"), g.get("bflow"), p1, p2, nparts=nparts)
    # NaN where the reference makes NaN (order-invariant filtering of
    # one-member groups divides 0 by 0, nldct.cpp:1872)
    assert np.array_equal(np.isnan(basic), np.isnan(g["basic"]))
    assert np.array_equal(np.isnan(final), np.isnan(g["final"]))
    db = np.nanmax(np.abs(basic.astype(np.float64) - g["basic"]))
    df = np.nanmax(np.abs(final.astype(np.float64) - g["final"]))
    assert db <= TOL_GREY and df <= TOL_GREY, (db, df)
    if not np.isnan(g["final"]).any():
        assert abs(psnr(final, g["clean"]) - psnr(g["final"], g["clean"])) <= TOL_PSNR
    # the exact path is bit-identical
    assert np.array_equal(basic, g["basic"], equal_nan=True), db
    assert np.array_equal(final, g["final"], equal_nan=True), df
    assert ratios == tuple(g["ratios"].tolist())


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_gpu_neighbours_match_oracle(gpulib, gpuctx, oracle, case):
    name, W, H, F, C, sigma, seed, flow, cli, nthreads = case
    clean, nz, ff, bf = video_case(W, H, F, sigma=sigma, seed=seed, channels=C, flow=flow)
    po = resolve_params(oracle, (W, H, F, C), sigma, **cli)
    pg = resolve_params(gpulib, (W, H, F, C), sigma, **cli)
    ob, of, orat, tr = oracle.runNlBayes(nz, ff, bf, *po, nparts=2 * nthreads, trace_cap=100000, trace_stride=32)
    gb, gf, grat = gpuctx.runNlBayes(nz, ff, bf, *pg, nparts=2 * nthreads, keep_groups=True)
    assert np.array_equal(gb, ob, equal_nan=True) and np.array_equal(gf, of, equal_nan=True)
    for step in (1, 2):
        for tile in range(2 * nthreads):
            sel = (tr["step"] == step) & (tr["tile"] == tile)
            gg = gpuctx.groups(step, tile)
            assert np.array_equal(gg["ref"], tr["ref"][sel])
            assert np.array_equal(gg["nsimp"], tr["nsimp"][sel])
            assert np.array_equal(gg["index"], tr["index"][sel])


def test_gpu_exact_ties_follow_partial_sort(gpulib, gpuctx, oracle):
    # piecewise-constant, noise-free frames quantised to integers: many exactly
    # equal distances, so the k-nearest order depends on the heap mechanics of
    # std::partial_sort
    rng = np.random.default_rng(5)
    W, H, F = 32, 28, 5
    base = rng.integers(0, 4, size=(H // 4 + 1, W // 4 + 1)).astype(np.float32) * 40
    fr = np.kron(base, np.ones((4, 4), np.float32))[:H, :W]
    nz = np.stack([np.roll(fr, k, axis=1) for k in range(F)])[:, None].copy()
    nz += rng.integers(0, 3, size=nz.shape).astype(np.float32)
    po = resolve_params(oracle, (W, H, F, 1), 10.0, **CFG_VIDEO)
    pg = resolve_params(gpulib, (W, H, F, 1), 10.0, **CFG_VIDEO)
    ob, of, orat, tr = oracle.runNlBayes(nz, None, None, *po, nparts=2, trace_cap=100000, trace_stride=32)
    gb, gf, grat = gpuctx.runNlBayes(nz, None, None, *pg, nparts=2, keep_groups=True)
    for step in (1, 2):
        for tile in range(2):
            sel = (tr["step"] == step) & (tr["tile"] == tile)
            gg = gpuctx.groups(step, tile)
            assert np.array_equal(gg["index"], tr["index"][sel])
    assert np.array_equal(gb, ob) and np.array_equal(gf, of) and grat == orat


def test_gpu_constant_video_stale_weights(gpulib, gpuctx, oracle):
    # all members equal: the group is left as is with the previous weights
    W, H, F = 24, 20, 4
    nz = np.full((F, 1, H, W), 100.0, np.float32)
    nz[:, :, :, W // 2:] = 50.0
    po = resolve_params(oracle, (W, H, F, 1), 20.0, **CFG_VIDEO)
    pg = resolve_params(gpulib, (W, H, F, 1), 20.0, **CFG_VIDEO)
    ob, of, orat = oracle.runNlBayes(nz, None, None, *po, nparts=2)
    gb, gf, grat = gpuctx.runNlBayes(nz, None, None, *pg, nparts=2)
    # this degenerate input makes the reference itself produce NaNs (zero
    # Wiener energy): they must appear at the same pixels
    assert np.isnan(of).any()
    assert np.array_equal(gb, ob, equal_nan=True) and np.array_equal(gf, of, equal_nan=True)
    assert grat == orat


def test_gpu_patch_longer_than_video(gpulib, gpuctx, oracle):
    # pt > frames: no reference patch fits, every pixel takes 0 / noisy
    # (nldct.cpp:537, 2446)
    W, H, F = 24, 20, 3
    clean, nz, ff, bf = video_case(W, H, F, seed=9)
    po = resolve_params(oracle, (W, H, F, 1), 20.0, **CFG_VIDEO)
    pg = resolve_params(gpulib, (W, H, F, 1), 20.0, **CFG_VIDEO)
    ob, of, orat = oracle.runNlBayes(nz, ff, bf, *po, nparts=2)
    gb, gf, grat = gpuctx.runNlBayes(nz, ff, bf, *pg, nparts=2)
    assert grat == orat == (0.0, 0.0)
    assert np.array_equal(gb, ob, equal_nan=True) and np.array_equal(gf, of, equal_nan=True)


def test_gpu_step2_only_and_step1_only(gpulib, gpuctx, oracle):
    W, H, F = 36, 30, 5
    clean, nz, ff, bf = video_case(W, H, F, sigma=20.0, seed=31)
    po = resolve_params(oracle, (W, H, F, 1), 20.0, **CFG_VIDEO)
    pg = resolve_params(gpulib, (W, H, F, 1), 20.0, **CFG_VIDEO)
    # BSIC_ONLY: px2 = 0
    po2, pg2 = (po[0], type(po[1])()), (pg[0], type(pg[1])())
    ob, _, orat = oracle.runNlBayes(nz, ff, bf, *po2, nparts=2)
    gb, _, grat = gpuctx.runNlBayes(nz, ff, bf, *pg2, nparts=2)
    assert np.array_equal(gb, ob) and grat == orat
    # DENO_ONLY: px1 = 0 with a given basic estimate
    po1, pg1 = (type(po[0])(), po[1]), (type(pg[0])(), pg[1])
    ob2, of2, orat2 = oracle.runNlBayes(nz, ff, bf, *po1, basic=ob, nparts=2)
    gb2, gf2, grat2 = gpuctx.runNlBayes(nz, ff, bf, *pg1, basic=gb, nparts=2)
    assert np.array_equal(gf2, of2) and np.array_equal(gb2, ob2) and grat2 == orat2


def test_gpu_device_pointers_match_host(gpulib, gpuctx):
    import torch
    W, H, F = 36, 30, 5
    clean, nz, ff, bf = video_case(W, H, F, sigma=20.0, seed=41)
    p = resolve_params(gpulib, (W, H, F, 1), 20.0, **CFG_VIDEO)
    hb, hf, hr = gpuctx.runNlBayes(nz, ff, bf, *p, nparts=2)
    t = lambda a: torch.from_numpy(a).cuda()
    db, df, dr = gpuctx.runNlBayes(t(nz), t(ff), t(bf), *p, nparts=2)
    assert np.array_equal(db.cpu().numpy(), hb) and np.array_equal(df.cpu().numpy(), hf) and dr == hr


def test_gpu_errors(gpulib, gpuctx):
    W, H, F = 16, 16, 3
    nz = np.zeros((F, 2, H, W), np.float32)
    p = resolve_params(gpulib, (W, H, F, 2), 20.0, **CFG_VIDEO)
    with pytest.raises(gpulib.BM4DOFError) as e:
        gpuctx.runNlBayes(nz, None, None, *p)
    assert e.value.status == "ERR_CHANNELS"
    assert str(e.value) == "VideoNLB::runNlBayes: Wrong number of channels. Must be 1, 3 or 4."
    nz = np.zeros((F, 1, H, W), np.float32)
    p1, p2 = resolve_params(gpulib, (W, H, F, 1), 20.0, **CFG_VIDEO)
    with pytest.raises(gpulib.BM4DOFError) as e:
        gpuctx.runNlBayes(nz, None, None, type(p1)(), type(p2)())
    assert e.value.status == "ERR_NO_STEP"
    q = resolve_params(gpulib, (W, H, F, 1), 20.0, px1=4, px2=4)
    q[0].transform = 1
    with pytest.raises(gpulib.BM4DOFError) as e:
        gpuctx.runNlBayes(nz, None, None, *q)
    assert e.value.status == "ERR_BIOR_SIZE"
    q = resolve_params(gpulib, (W, H, F, 1), 20.0, **CFG_VIDEO)
    q[1].nSimilarPatches = 64
    with pytest.raises(gpulib.BM4DOFError) as e:
        gpuctx.runNlBayes(nz, None, None, *q)
    assert e.value.status == "ERR_UNSUPPORTED"
    q = resolve_params(gpulib, (W, H, F, 1), 20.0, **CFG_VIDEO)
    q[1].sizePatch, q[1].sizePatchTime = 1, 17   # 17 values, but more patch frames than the gather takes
    with pytest.raises(gpulib.BM4DOFError) as e:
        gpuctx.runNlBayes(nz, None, None, *q)
    assert e.value.status == "ERR_UNSUPPORTED" and "sizePatchTime" in str(e.value)
    # the context stays usable after errors
    clean, nz, ff, bf = video_case(W + 8, H + 8, F + 3, seed=3)
    p = resolve_params(gpulib, (W + 8, H + 8, F + 3, 1), 20.0, **CFG_VIDEO)
    gpuctx.runNlBayes(nz, ff, bf, *p)
