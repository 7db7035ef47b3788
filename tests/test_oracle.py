"""The oracle restatement is pinned to the reference: bit-identical outputs on
the committed golden fixtures (made by the reference itself) and, where the
reference sources are present, on fresh seeded runs."""
import os

import numpy as np
import pytest

from cases import CASES, VBM3D_CASES
from helpers import ROOT, resolve_params, video_case

GOLDEN = os.path.join(ROOT, "tests", "golden")


def load_case(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def params_from(lib, arr):
    import pyoracle
    p = pyoracle.Params()
    for (f, t), v in zip(pyoracle.Params._fields_, arr):
        setattr(p, f, float(v) if t.__name__ == "c_float" else int(v))
    return p


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_oracle_matches_golden(oracle, case):
    name = case[0]
    g = load_case(name)
    p1, p2 = params_from(oracle, g["p1"]), params_from(oracle, g["p2"])
    nthreads = int(g["nthreads"])
    basic, final, ratios = oracle.runNlBayes(g["noisy"], g.get("fflow"), g.get("bflow"), p1, p2,
                                             nparts=2 * nthreads, nthreads=nthreads)
    # NaN where the reference makes NaN (order-invariant filtering of
    # one-member groups divides 0 by 0, nldct.cpp:1872)
    assert np.array_equal(basic, g["basic"], equal_nan=True)
    assert np.array_equal(final, g["final"], equal_nan=True)
    assert ratios == tuple(g["ratios"].tolist())


@pytest.mark.parametrize("case", VBM3D_CASES, ids=[c[0] for c in VBM3D_CASES])
def test_oracle_vbm3d_matches_golden(oracle, case):
    """The predictive search restatement against the reference's VBM3D_SEARCH build."""
    g = load_case(case[0])
    p1, p2 = params_from(oracle, g["p1"]), params_from(oracle, g["p2"])
    nthreads = int(g["nthreads"])
    basic, final, ratios = oracle.runNlBayes(g["noisy"], g.get("fflow"), g.get("bflow"), p1, p2,
                                             nparts=2 * nthreads, nthreads=nthreads, vbm3d=True)
    assert np.array_equal(basic, g["basic"], equal_nan=True)
    assert np.array_equal(final, g["final"], equal_nan=True)
    assert ratios == tuple(g["ratios"].tolist())


def test_vbm3d_golden_differs_from_exhaustive(oracle):
    """The predictive fixtures exercise a different neighbour search."""
    g = load_case("vbm3d_video")
    p1, p2 = params_from(oracle, g["p1"]), params_from(oracle, g["p2"])
    basic, final, _ = oracle.runNlBayes(g["noisy"], g.get("fflow"), g.get("bflow"), p1, p2, nparts=2)
    assert not np.array_equal(basic, g["basic"])


def test_golden_denoises(oracle):
    from helpers import psnr
    for name in ("video_px4", "image_px8", "rgb_video"):
        g = load_case(name)
        assert psnr(g["final"], g["clean"]) > psnr(g["noisy"], g["clean"]) + 5.0


@pytest.mark.parametrize("seed", [101, 102])
def test_oracle_matches_reference_fresh(oracle, reference, seed):
    from cases import CFG_VIDEO
    W, H, F = 36, 30, 5
    clean, nz, ff, bf = video_case(W, H, F, sigma=25.0, seed=seed)
    po = resolve_params(oracle, (W, H, F, 1), 25.0, **CFG_VIDEO)
    pr = resolve_params(reference, (W, H, F, 1), 25.0, **CFG_VIDEO)
    a = oracle.runNlBayes(nz, ff, bf, *po, nparts=2)
    b = reference.runNlBayes(nz, ff, bf, *pr, nthreads=1)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]) and a[2] == b[2]


def test_oracle_neighbours_match_reference_search(oracle, reference):
    # neighbour lists of step 1, tile 0, against estimateSimilarPatchesStep1
    # called on the reference's own tile crop
    from cases import CFG_VIDEO
    W, H, F = 36, 30, 5
    clean, nz, ff, bf = video_case(W, H, F, sigma=20.0, seed=7)
    po = resolve_params(oracle, (W, H, F, 1), 20.0, **CFG_VIDEO)
    pr = resolve_params(reference, (W, H, F, 1), 20.0, **CFG_VIDEO)
    _, _, _, tr = oracle.runNlBayes(nz, ff, bf, *po, nparts=2, trace_cap=20000, trace_stride=16)
    box = oracle.tile_crops(W, H, 2, po[0].boundary)[0]
    ox, oy, ex, ey = box
    tile = lambda v: np.ascontiguousarray(v[:, :, oy:ey, ox:ex])
    sel = np.nonzero((tr["step"] == 1) & (tr["tile"] == 0))[0]
    assert len(sel) > 50
    for k in sel[::7]:
        idx = reference.search(1, tile(nz), None, tile(ff), tile(bf), pr[0], int(tr["ref"][k]))
        n = int(tr["nsimp"][k])
        assert len(idx) == n
        assert np.array_equal(idx, tr["index"][k, :n])


def test_errors_match_reference_messages(oracle, reference):
    from cases import CFG_VIDEO
    nz = np.zeros((3, 2, 16, 16), np.float32)
    po = resolve_params(oracle, (16, 16, 3, 2), 20.0, **CFG_VIDEO)
    pr = resolve_params(reference, (16, 16, 3, 2), 20.0, **CFG_VIDEO)
    with pytest.raises(RuntimeError) as a:
        oracle.runNlBayes(nz, None, None, *po)
    with pytest.raises(RuntimeError) as b:
        reference.runNlBayes(nz, None, None, *pr)
    assert str(a.value) == str(b.value)


@pytest.mark.parametrize("seed", [201, 202])
def test_oracle_vbm3d_matches_reference_fresh(oracle, seed):
    import pyoracle
    if not pyoracle.Reference.available(pyoracle.REF_VBM3D_SO):
        pytest.skip("reference sources not present (oracle/_ref not built)")
    ref = pyoracle.Reference(pyoracle.REF_VBM3D_SO)
    W, H, F = 38, 34, 7
    clean, nz, ff, bf = video_case(W, H, F, sigma=25.0, seed=seed)
    cfg = dict(px1=4, px2=4, pt1=1, pt2=2, wx1=11, wx2=9, np1=8, np2=16, npf1=2, npf2=4, wxf2=3)
    po = resolve_params(oracle, (W, H, F, 1), 25.0, **cfg)
    pr = resolve_params(ref, (W, H, F, 1), 25.0, **cfg)
    a = oracle.runNlBayes(nz, ff, bf, *po, nparts=2, vbm3d=True)
    b = ref.runNlBayes(nz, ff, bf, *pr, nthreads=1)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]) and a[2] == b[2]


@pytest.mark.parametrize("seed", [211, 212])
def test_oracle_paste_boost_matches_reference_fresh(oracle, reference, seed):
    """doPasteBoost (reachable through the API only) against the compiled reference."""
    from cases import CFG_VIDEO
    W, H, F = 42, 34, 6
    clean, nz, ff, bf = video_case(W, H, F, sigma=25.0, seed=seed)
    po = resolve_params(oracle, (W, H, F, 1), 25.0, paste_boost=True, **CFG_VIDEO)
    pr = resolve_params(reference, (W, H, F, 1), 25.0, paste_boost=True, **CFG_VIDEO)
    a = oracle.runNlBayes(nz, ff, bf, *po, nparts=4, nthreads=2)
    b = reference.runNlBayes(nz, ff, bf, *pr, nthreads=2)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]) and a[2] == b[2]
