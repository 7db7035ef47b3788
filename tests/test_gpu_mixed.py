"""Mixed-precision form: the patch search on the Blackwell tensor cores
(tcgen05.mma, FP16 operands, FP32 accumulation in tensor memory) as a
pre-screen, then the exact FP32 distances of the 32 best candidates,
certified against a bound on every dropped one.

* BM4DOF_MIXED_CERTIFIED: groups it cannot certify get the exact search, so
  the neighbour lists are the exact search's and (with the FP32 group filter)
  the output is the plain path's, bit for bit.
* BM4DOF_MIXED_PRECISION: an uncertified group keeps the order of its
  re-ranked 32; the bars are neighbour sets that agree with the exact path
  and a PSNR change far inside 0.05 dB."""
import numpy as np
import pytest

from cases import CFG_IMAGE, CFG_VIDEO
from helpers import psnr, resolve_params, video_case

pytestmark = pytest.mark.gpu


def test_tc_selftest_layout(gpulib):
    # the operand layout, descriptors and TMEM read-back of the tensor-core
    # path against a float64 product of the same FP16 values
    import torch
    rng = np.random.default_rng(3)
    a = rng.normal(0, 60, (128, 64)).astype(np.float16)
    b = rng.normal(0, 60, (256, 64)).astype(np.float16)
    d = gpulib.tc_selftest(torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()).cpu().numpy()
    want = a.astype(np.float64) @ b.astype(np.float64).T
    scale = np.abs(a.astype(np.float64)) @ np.abs(b.astype(np.float64)).T
    assert np.all(np.abs(d - want) <= 1e-5 * scale + 1e-3), float(np.max(np.abs(d - want) / (scale + 1)))


def lists(ctx, nparts):
    return [[ctx.groups(s, t) for t in range(nparts)] for s in (1, 2)]


def same_lists(a, b):
    for sa, sb in zip(a, b):
        for ta, tb in zip(sa, sb):
            assert np.array_equal(ta["ref"], tb["ref"])
            assert np.array_equal(ta["nsimp"], tb["nsimp"])
            assert np.array_equal(ta["index"], tb["index"])


@pytest.mark.parametrize("cfg,shape,sigma,nparts", [
    (CFG_VIDEO, (64, 48, 8), 20.0, 2), (CFG_VIDEO, (160, 96, 10), 10.0, 2), (CFG_VIDEO, (120, 88, 12), 40.0, 4),
    (CFG_IMAGE, (96, 80, 1), 20.0, 2), (CFG_VIDEO, (44, 40, 6), 20.0, 2)],
    ids=["video_px4", "video_s10", "video_s40_4tiles", "image_px8", "small"])
def test_mixed_search_is_exact(gpulib, gpuctx, cfg, shape, sigma, nparts):
    W, H, F = shape
    clean, nz, ff, bf = video_case(W, H, F, sigma=sigma, seed=77)
    p = resolve_params(gpulib, (W, H, F, 1), sigma, **cfg)
    pb, pf, pr = gpuctx.runNlBayes(nz, ff, bf, *p, nparts=nparts, keep_groups=True)
    plain = lists(gpuctx, nparts)
    mb, mf, mr = gpuctx.runNlBayes(nz, ff, bf, *p, nparts=nparts, keep_groups=True, mixed="certified")
    groups, exact, uncertified = gpuctx.mixed_stats()
    assert groups > 0 and uncertified == 0
    same_lists(plain, lists(gpuctx, nparts))
    assert np.array_equal(pb, mb) and np.array_equal(pf, mf) and pr == mr
    # the pre-screen certifies most groups (near-equal candidates in the smooth
    # basic estimate are the ones it leaves to the exact search)
    assert exact <= 0.6 * groups, (exact, groups)


def set_agreement(a, b):
    same = total = 0
    for ta, tb in zip(a, b):
        assert np.array_equal(ta["ref"], tb["ref"])
        for i in range(len(ta["ref"])):
            sa = set(ta["index"][i, :ta["nsimp"][i]].tolist())
            sb = set(tb["index"][i, :tb["nsimp"][i]].tolist())
            same += sa == sb
            total += 1
    return same / max(total, 1)


@pytest.mark.parametrize("shape,sigma", [((64, 48, 8), 20.0), ((160, 96, 10), 10.0), ((120, 88, 12), 40.0)],
                         ids=["s20", "s10", "s40"])
def test_mixed_search_default_agrees(gpulib, gpuctx, shape, sigma):
    W, H, F = shape
    clean, nz, ff, bf = video_case(W, H, F, sigma=sigma, seed=78)
    p = resolve_params(gpulib, (W, H, F, 1), sigma, **CFG_VIDEO)
    pb, pf, pr = gpuctx.runNlBayes(nz, ff, bf, *p, nparts=2, keep_groups=True)
    plain = lists(gpuctx, 2)
    mb, mf, mr = gpuctx.runNlBayes(nz, ff, bf, *p, nparts=2, keep_groups=True, mixed=True)
    groups, exact, uncertified = gpuctx.mixed_stats()
    mixed = lists(gpuctx, 2)
    # step 1 searches the same noisy video: its sets agree almost everywhere
    assert set_agreement(plain[0], mixed[0]) >= 0.995
    assert abs(psnr(pf, clean) - psnr(mf, clean)) <= 0.01
    assert exact + uncertified <= groups


def test_mixed_search_ties_fall_back_to_exact(gpulib, gpuctx):
    # noise-free piecewise-constant frames: exact distance ties everywhere, the
    # certification refuses them and the exact search (with its heap replay)
    # decides; the result is still the plain path's
    rng = np.random.default_rng(5)
    W, H, F = 48, 40, 6
    base = rng.integers(0, 4, size=(H // 8 + 1, W // 8 + 1)).astype(np.float32) * 40
    fr = np.kron(base, np.ones((8, 8), np.float32))[:H, :W]
    nz = np.stack([np.roll(fr, k, axis=1) for k in range(F)])[:, None].copy()
    p = resolve_params(gpulib, (W, H, F, 1), 10.0, **CFG_VIDEO)
    a = gpuctx.runNlBayes(nz, None, None, *p, nparts=2, keep_groups=True)
    plain = lists(gpuctx, 2)
    b = gpuctx.runNlBayes(nz, None, None, *p, nparts=2, keep_groups=True, mixed="certified")
    groups, exact, uncertified = gpuctx.mixed_stats()
    assert exact > 0
    same_lists(plain, lists(gpuctx, 2))
    # (constant groups make NaN in places, as the reference does)
    assert np.array_equal(a[0], b[0], equal_nan=True) and np.array_equal(a[1], b[1], equal_nan=True)


def test_mixed_unsupported_falls_back_to_exact(gpulib, gpuctx):
    # RGB step 2 searches three channels: the exact search runs there
    W, H, F = 40, 36, 4
    clean, nz, ff, bf = video_case(W, H, F, sigma=20.0, seed=5, channels=3)
    p = resolve_params(gpulib, (W, H, F, 3), 20.0, **CFG_VIDEO)
    a = gpuctx.runNlBayes(nz, ff, bf, *p, nparts=2)
    b = gpuctx.runNlBayes(nz, ff, bf, *p, nparts=2, mixed=True)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


@pytest.mark.parametrize("sigma", [10.0, 20.0, 40.0])
def test_mixed_rgb_video(gpulib, gpuctx, sigma):
    # RGB video (the mixed-precision colour workload on a crop): step 1 searches
    # the first opponent channel through the tensor-core pre-screen, step 2
    # compares all three channels with the exact search
    W, H, F = 128, 96, 8
    clean, nz, ff, bf = video_case(W, H, F, sigma=sigma, seed=90, channels=3)
    p = resolve_params(gpulib, (W, H, F, 3), sigma, **CFG_VIDEO)
    pb, pf, pr = gpuctx.runNlBayes(nz, ff, bf, *p, nparts=2, keep_groups=True)
    plain = lists(gpuctx, 2)
    cb, cf, cr = gpuctx.runNlBayes(nz, ff, bf, *p, nparts=2, keep_groups=True, mixed="certified")
    same_lists(plain, lists(gpuctx, 2))
    assert np.array_equal(pb, cb) and np.array_equal(pf, cf)
    mb, mf, mr = gpuctx.runNlBayes(nz, ff, bf, *p, nparts=2, keep_groups=True, mixed=True)
    groups, exact, uncertified = gpuctx.mixed_stats()
    assert groups > 0
    assert set_agreement(plain[0], lists(gpuctx, 2)[0]) >= 0.995
    assert abs(psnr(pf, clean) - psnr(mf, clean)) <= 0.01
