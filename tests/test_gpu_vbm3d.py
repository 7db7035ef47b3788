"""GPU parity of the predictive search (BM4DOF_VBM3D_SEARCH) against the
reference built with VBM3D_SEARCH (golden fixtures) and the oracle's
restatement: bit-identical outputs and identical neighbour lists, order
included."""
import os

import numpy as np
import pytest

from cases import CFG_VIDEO, VBM3D_CASES
from helpers import ROOT, resolve_params, video_case

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(ROOT, "tests", "golden")


def gparams(gpulib, arr):
    p = gpulib.Params()
    for (f, t), v in zip(gpulib.Params._fields_, arr):
        setattr(p, f, float(v) if t.__name__ == "c_float" else int(v))
    return p


def same_groups(gpuctx, tr, ntiles, steps=(1, 2)):
    for step in steps:
        for tile in range(ntiles):
            sel = (tr["step"] == step) & (tr["tile"] == tile)
            gg = gpuctx.groups(step, tile)
            assert np.array_equal(gg["ref"], tr["ref"][sel]), (step, tile)
            assert np.array_equal(gg["nsimp"], tr["nsimp"][sel]), (step, tile)
            assert np.array_equal(gg["index"], tr["index"][sel]), (step, tile)


@pytest.mark.parametrize("case", VBM3D_CASES, ids=[c[0] for c in VBM3D_CASES])
def test_gpu_vbm3d_matches_golden(gpulib, gpuctx, case):
    g = dict(np.load(os.path.join(GOLDEN, case[0] + ".npz")))
    p1, p2 = gparams(gpulib, g["p1"]), gparams(gpulib, g["p2"])
    nparts = 2 * int(g["nthreads"])
    basic, final, ratios = gpuctx.runNlBayes(g["noisy"], g.get("fflow"), g.get("bflow"), p1, p2,
                                             nparts=nparts, vbm3d=True)
    assert np.array_equal(basic, g["basic"], equal_nan=True), np.nanmax(np.abs(basic - g["basic"]))
    assert np.array_equal(final, g["final"], equal_nan=True), np.nanmax(np.abs(final - g["final"]))
    assert ratios == tuple(g["ratios"].tolist())


@pytest.mark.parametrize("seed,cfg", [
    (301, dict(CFG_VIDEO)),
    (302, dict(px1=4, px2=4, pt1=1, pt2=2, wx1=11, wx2=9, np1=8, np2=16, npf1=2, npf2=4, wxf2=3)),
    (303, dict(px1=8, px2=8, pt1=1, pt2=1, wx1=15, wx2=15, np1=16, np2=32, npf1=4, npf2=6, wxf1=7)),
])
def test_gpu_vbm3d_neighbours_match_oracle(gpulib, gpuctx, oracle, seed, cfg):
    W, H, F, C = 46, 38, 7, 1
    clean, nz, ff, bf = video_case(W, H, F, sigma=20.0, seed=seed, channels=C)
    po = resolve_params(oracle, (W, H, F, C), 20.0, **cfg)
    pg = resolve_params(gpulib, (W, H, F, C), 20.0, **cfg)
    ob, of, orat, tr = oracle.runNlBayes(nz, ff, bf, *po, nparts=2, trace_cap=100000, trace_stride=32,
                                         vbm3d=True)
    gb, gf, grat = gpuctx.runNlBayes(nz, ff, bf, *pg, nparts=2, keep_groups=True, vbm3d=True)
    same_groups(gpuctx, tr, 2)
    assert np.array_equal(gb, ob) and np.array_equal(gf, of) and grat == orat


def test_gpu_vbm3d_rgb_flow_matches_oracle(gpulib, gpuctx, oracle):
    # step 2 sums the basic estimate's channel 0 once per channel
    W, H, F, C = 34, 30, 6, 3
    clean, nz, ff, bf = video_case(W, H, F, sigma=25.0, seed=304, channels=C)
    po = resolve_params(oracle, (W, H, F, C), 25.0, **CFG_VIDEO)
    pg = resolve_params(gpulib, (W, H, F, C), 25.0, **CFG_VIDEO)
    ob, of, orat, tr = oracle.runNlBayes(nz, ff, bf, *po, nparts=4, trace_cap=100000, trace_stride=32,
                                         vbm3d=True)
    gb, gf, grat = gpuctx.runNlBayes(nz, ff, bf, *pg, nparts=4, keep_groups=True, vbm3d=True)
    same_groups(gpuctx, tr, 4)
    assert np.array_equal(gb, ob) and np.array_equal(gf, of) and grat == orat


def test_gpu_vbm3d_ties_follow_partial_sort(gpulib, gpuctx, oracle):
    # noise-free, piecewise-constant, integer frames: exact distance ties in
    # every frame and in the pool, so the heap mechanics of partial_sort decide
    rng = np.random.default_rng(7)
    W, H, F = 36, 30, 6
    base = rng.integers(0, 4, size=(H // 4 + 1, W // 4 + 1)).astype(np.float32) * 40
    fr = np.kron(base, np.ones((4, 4), np.float32))[:H, :W]
    nz = np.stack([np.roll(fr, k, axis=1) for k in range(F)])[:, None].copy()
    nz += rng.integers(0, 2, size=nz.shape).astype(np.float32)
    cfg = dict(CFG_VIDEO, npf1=3, npf2=3)
    po = resolve_params(oracle, (W, H, F, 1), 10.0, **cfg)
    pg = resolve_params(gpulib, (W, H, F, 1), 10.0, **cfg)
    ob, of, orat, tr = oracle.runNlBayes(nz, None, None, *po, nparts=2, trace_cap=100000, trace_stride=32,
                                         vbm3d=True)
    gb, gf, grat = gpuctx.runNlBayes(nz, None, None, *pg, nparts=2, keep_groups=True, vbm3d=True)
    same_groups(gpuctx, tr, 2)
    assert np.array_equal(gb, ob) and np.array_equal(gf, of)


def test_gpu_vbm3d_nan_distances_follow_partial_sort(gpulib, gpuctx, oracle):
    # NaN pixels make NaN distances, which partial_sort orders by its heap
    # mechanics alone; step 1 only, neighbour lists compared
    W, H, F = 36, 32, 6
    clean, nz, ff, bf = video_case(W, H, F, sigma=20.0, seed=305)
    rng = np.random.default_rng(8)
    for _ in range(6):
        nz[rng.integers(0, F), 0, rng.integers(0, H), rng.integers(0, W)] = np.nan
    po = resolve_params(oracle, (W, H, F, 1), 20.0, **dict(CFG_VIDEO, px2=0))
    pg = resolve_params(gpulib, (W, H, F, 1), 20.0, **dict(CFG_VIDEO, px2=0))
    ob, _, orat, tr = oracle.runNlBayes(nz, ff, bf, *po, nparts=2, trace_cap=100000, trace_stride=32,
                                        vbm3d=True)
    gb, _, grat = gpuctx.runNlBayes(nz, ff, bf, *pg, nparts=2, keep_groups=True, vbm3d=True)
    same_groups(gpuctx, tr, 2, steps=(1,))
    assert np.array_equal(gb, ob, equal_nan=True) and grat == orat


def test_gpu_vbm3d_batched_matches_single(gpulib, gpuctx):
    import torch
    g = dict(np.load(os.path.join(GOLDEN, "vbm3d_video.npz")))
    p1, p2 = gparams(gpulib, g["p1"]), gparams(gpulib, g["p2"])
    dev = torch.device("cuda", 0)
    items = []
    for k in range(3):
        nz = torch.from_numpy(g["noisy"]).to(dev)
        items.append(dict(noisy=nz, fflow=torch.from_numpy(g["fflow"]).to(dev),
                          bflow=torch.from_numpy(g["bflow"]).to(dev), basic=torch.empty_like(nz),
                          final=torch.empty_like(nz), p1=p1, p2=p2, nparts=2))
    ratios = gpuctx.run_batched(items, vbm3d=True)
    for it, r in zip(items, ratios):
        assert np.array_equal(it["basic"].cpu().numpy(), g["basic"])
        assert np.array_equal(it["final"].cpu().numpy(), g["final"])
        assert r == tuple(g["ratios"].tolist())


def test_gpu_vbm3d_rejections(gpulib, gpuctx):
    g = dict(np.load(os.path.join(GOLDEN, "vbm3d_video.npz")))
    p1, p2 = gparams(gpulib, g["p1"]), gparams(gpulib, g["p2"])
    with pytest.raises(gpulib.BM4DOFError, match="plain FP32"):
        gpuctx.runNlBayes(g["noisy"], g["fflow"], g["bflow"], p1, p2, nparts=2, vbm3d=True, mixed=True)
    p1.nSimilarPatchesPred = 0
    with pytest.raises(gpulib.BM4DOFError, match="nSimilarPatchesPred"):
        gpuctx.runNlBayes(g["noisy"], g["fflow"], g["bflow"], p1, p2, nparts=2, vbm3d=True)
    p1.nSimilarPatchesPred = 30   # more than a 5x5 predicted window holds
    with pytest.raises(gpulib.BM4DOFError, match="fewer positions"):
        gpuctx.runNlBayes(g["noisy"], g["fflow"], g["bflow"], p1, p2, nparts=2, vbm3d=True)


@pytest.mark.parametrize("seed,nparts,cfg,vbm3d", [
    (311, 6, dict(CFG_VIDEO, paste_boost=True), False),
    (312, 4, dict(CFG_VIDEO, paste_boost=True), True),
    (313, 2, dict(CFG_VIDEO, order_inv=True), True),
    (314, 2, dict(CFG_VIDEO, paste_boost=True, order_inv=True), False),
])
def test_gpu_paste_and_predictive_combinations(gpulib, gpuctx, oracle, seed, nparts, cfg, vbm3d):
    """The paste trick and the predictive search with more tiles and with
    order-invariant filtering, against the oracle (both pinned to the
    reference separately)."""
    W, H, F = 52, 40, 6
    clean, nz, ff, bf = video_case(W, H, F, sigma=20.0, seed=seed)
    po = resolve_params(oracle, (W, H, F, 1), 20.0, **cfg)
    pg = resolve_params(gpulib, (W, H, F, 1), 20.0, **cfg)
    ob, of, orat, tr = oracle.runNlBayes(nz, ff, bf, *po, nparts=nparts, nthreads=1, trace_cap=100000,
                                         trace_stride=32, vbm3d=vbm3d)
    gb, gf, grat = gpuctx.runNlBayes(nz, ff, bf, *pg, nparts=nparts, keep_groups=True, vbm3d=vbm3d)
    same_groups(gpuctx, tr, nparts)
    assert np.array_equal(gb, ob, equal_nan=True) and np.array_equal(gf, of, equal_nan=True) and grat == orat


def test_gpu_paste_batched_matches_golden(gpulib, gpuctx):
    import torch
    g = dict(np.load(os.path.join(GOLDEN, "video_paste.npz")))
    p1, p2 = gparams(gpulib, g["p1"]), gparams(gpulib, g["p2"])
    dev = torch.device("cuda", 0)
    items = []
    for k in range(2):
        nz = torch.from_numpy(g["noisy"]).to(dev)
        items.append(dict(noisy=nz, fflow=torch.from_numpy(g["fflow"]).to(dev),
                          bflow=torch.from_numpy(g["bflow"]).to(dev), basic=torch.empty_like(nz),
                          final=torch.empty_like(nz), p1=p1, p2=p2, nparts=2))
    ratios = gpuctx.run_batched(items)
    for it, r in zip(items, ratios):
        assert np.array_equal(it["basic"].cpu().numpy(), g["basic"])
        assert np.array_equal(it["final"].cpu().numpy(), g["final"])
        assert r == tuple(g["ratios"].tolist())
