"""VideoNLB::processNlBayes (nldct.cpp:490-890): one step over one video cut
from a larger source, with the reference-patch grid kept away from the sides
where the crop stops short of its source (nldct.cpp:520-553) -- in x, y and,
for a caller's crop, in time.  The golden fixtures (tests/golden/process_*.npz,
made by tests/golden/make_golden.py from the reference's own processNlBayes)
pin the oracle on the CPU and bm4dof_process on the GPU; the oracle is also
compared live with the reference over every combination of spatial borders."""
import itertools
import os

import numpy as np
import pytest

from cases import PROCESS_CASES
from helpers import video_case

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
IDS = [c[0] for c in PROCESS_CASES]


def load(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def params(mod, arr):
    p = mod.Params()
    for (f, t), v in zip(mod.Params._fields_, arr):
        setattr(p, f, float(v) if t.__name__ == "c_float" else int(v))
    return p


def crop_of(mod, arr):
    arr = [int(v) for v in arr]
    return None if arr[0] < 0 else mod.make_crop(arr[0:3], arr[3:6], arr[6:10])


@pytest.mark.parametrize("case", PROCESS_CASES, ids=IDS)
def test_oracle_process_matches_golden(oracle, case):
    import pyoracle
    g = load(case[0])
    p1, p2 = params(pyoracle, g["p1"]), params(pyoracle, g["p2"])
    crop = crop_of(pyoracle, g["crop"])
    vbm3d = case[-1]
    basic, _, g1 = oracle.processNlBayes(g["noisy"], g.get("fflow"), g.get("bflow"), p1, crop, vbm3d=vbm3d)
    assert g1 == int(g["groups"][0]) and np.array_equal(basic, g["basic"])
    _, final, g2 = oracle.processNlBayes(g["noisy"], g.get("fflow"), g.get("bflow"), p2, crop, basic=g["basic"],
                                         vbm3d=vbm3d)
    assert g2 == int(g["groups"][1]) and np.array_equal(final, g["final"])


def test_golden_crops_cover_every_border():
    # the fixtures exercise each side as a border and as an edge
    seen = set()
    for case in PROCESS_CASES:
        crop = case[10]
        if crop is None:
            continue
        (ox, oy, ot), (ex, ey, et), (sw, sh, sf, _) = crop
        seen |= {k for k, on in zip(("x0", "y0", "t0", "x1", "y1", "t1"),
                                    (ox > 0, oy > 0, ot > 0, ex < sw, ey < sh, et < sf)) if on}
    assert seen == {"x0", "y0", "t0", "x1", "y1", "t1"}


def test_oracle_process_matches_reference_every_spatial_border(oracle, reference):
    import pyoracle
    W, H, F = 28, 24, 3
    clean, nz, ff, bf = video_case(W, H, F, sigma=20.0, seed=49)
    size = (W, H, F, 1)
    p1 = reference.initializeNlbParameters(1, 20.0, size)
    reference.setSizePatch(p1, size, 4)
    reference.setSizeSearchWindow(p1, 9)
    p1.sizePatchTime = 2
    p1.sizeSearchTimeRangeFwd = p1.sizeSearchTimeRangeBwd = 1
    p2 = reference.initializeNlbParameters(2, 20.0, size)
    reference.setSizePatch(p2, size, 4)
    reference.setSizeSearchWindow(p2, 9)
    p2.sizePatchTime = 2
    p2.sizeSearchTimeRangeFwd = p2.sizeSearchTimeRangeBwd = 1
    for bx0, by0, bx1, by1 in itertools.product((0, 1), repeat=4):
        crop = pyoracle.make_crop((5 * bx0, 3 * by0, 0), (5 * bx0 + W, 3 * by0 + H, F),
                                  (5 * bx0 + W + 7 * bx1, 3 * by0 + H + 2 * by1, F, 1))
        rb, _, rg = reference.processNlBayes(nz, ff, bf, p1, crop)
        ob, _, og = oracle.processNlBayes(nz, ff, bf, p1, crop)
        assert og == rg and np.array_equal(ob, rb), (bx0, by0, bx1, by1)
        _, rf, rg2 = reference.processNlBayes(nz, ff, bf, p2, crop, basic=rb)
        _, of, og2 = oracle.processNlBayes(nz, ff, bf, p2, crop, basic=rb)
        assert og2 == rg2 and np.array_equal(of, rf), (bx0, by0, bx1, by1)


def test_oracle_process_without_crop_is_a_one_tile_run(oracle):
    # a crop that touches every edge of its source is the whole video: one tile
    g = load("process_left")
    import pyoracle
    p1, p2 = params(pyoracle, g["p1"]), params(pyoracle, g["p2"])
    noisy, ff, bf = g["noisy"], g["fflow"], g["bflow"]
    basic, _, _ = oracle.processNlBayes(noisy, ff, bf, p1, None)
    _, final, _ = oracle.processNlBayes(noisy, ff, bf, p2, None, basic=basic)
    rb, rf, _ = oracle.runNlBayes(noisy, ff, bf, p1, p2, nparts=1)
    assert np.array_equal(basic, rb) and np.array_equal(final, rf)


@pytest.mark.gpu
@pytest.mark.parametrize("case", PROCESS_CASES, ids=IDS)
def test_gpu_process_matches_golden(gpulib, gpuctx, case):
    g = load(case[0])
    p1, p2 = params(gpulib, g["p1"]), params(gpulib, g["p2"])
    crop = crop_of(gpulib, g["crop"])
    vbm3d = case[-1]
    basic, _, g1 = gpuctx.processNlBayes(g["noisy"], g.get("fflow"), g.get("bflow"), p1, crop, vbm3d=vbm3d)
    assert g1 == int(g["groups"][0]) and np.array_equal(basic, g["basic"])
    _, final, g2 = gpuctx.processNlBayes(g["noisy"], g.get("fflow"), g.get("bflow"), p2, crop, basic=g["basic"],
                                         vbm3d=vbm3d)
    assert g2 == int(g["groups"][1]) and np.array_equal(final, g["final"])


@pytest.mark.gpu
def test_gpu_process_rejects_the_learned_form(gpulib, gpuctx):
    g = load("process_image")
    p1 = params(gpulib, g["p1"])
    with pytest.raises(gpulib.BM4DOFError, match="learned form runs both steps"):
        flags = gpulib.LEARNED
        import ctypes as C
        noisy = np.ascontiguousarray(g["noisy"], np.float32)
        F, Cc, H, W = noisy.shape
        out = np.zeros_like(noisy)
        n = C.c_uint()
        gpulib._check(gpulib.load().bm4dof_process(gpuctx._h, C.c_void_p(noisy.ctypes.data), None, None, W, H, Cc,
                                                   F, C.c_void_p(out.ctypes.data), C.c_void_p(out.ctypes.data),
                                                   C.byref(p1), None, flags, C.byref(n)))


def grid_axis(n, ori, end, step, edge_first, edge_last):
    """One axis of the reference-patch grid, nldct.cpp:536-547: every step-th
    position from ori, plus the last one (end - 1) on a side with no border,
    plus the first one on a side with no border (x and y only)."""
    return [v for d, v in enumerate(range(ori, end))
            if d % step == 0 or (edge_last and v == end - 1) or (edge_first and v == ori)]


def expected_grid(w, h, F, p, b):
    """The grid of one tile w x h x F with borders b = (x0, y0, t0, x1, y1, t1)."""
    sPx, sPt, sWx = p.sizePatch, p.sizePatchTime, p.sizeSearchWindow
    sWt = p.sizeSearchTimeRangeFwd + p.sizeSearchTimeRangeBwd + 1
    ox = sPx - 1 + sWx // 2 if b[0] else 0
    oy = sPx - 1 + sWx // 2 if b[1] else 0
    of = sPt - 1 + sWt // 2 if b[2] else 0
    ex = w - (sPx - 1 + sWx // 2 if b[3] else sPx - 1)
    ey = h - (sPx - 1 + sWx // 2 if b[4] else sPx - 1)
    ef = F - (sPt - 1 + sWt // 2 if b[5] else sPt - 1)
    return (grid_axis(w, ox, ex, p.offSet, not b[0], not b[3]), grid_axis(h, oy, ey, p.offSet, not b[1], not b[4]),
            grid_axis(F, of, ef, p.offSetTime, False, not b[5]))


@pytest.mark.parametrize("case", PROCESS_CASES, ids=IDS)
def test_plan_of_a_crop_is_the_references_grid(gpulib, case):
    # the host plan bm4dof_process runs on (bm4dof_plan, no device needed)
    g = load(case[0])
    F, _, H, W = g["noisy"].shape
    crop_arr = [int(v) for v in g["crop"]]
    crop = crop_of(gpulib, g["crop"])
    if crop is None:
        b = (0,) * 6
    else:
        o, e, s = crop_arr[0:3], crop_arr[3:6], crop_arr[6:9]
        b = (o[0] > 0, o[1] > 0, o[2] > 0, e[0] < s[0], e[1] < s[1], e[2] < s[2])
    for tag in ("p1", "p2"):
        p = params(gpulib, g[tag])
        (t,) = gpulib.plan(W, H, F, p, crop=crop, process=True)
        assert t["box"] == (0, 0, W, H)
        assert (t["xs"], t["ys"], t["fs"]) == expected_grid(W, H, F, p, b), (case[0], tag)


@pytest.mark.parametrize("nparts", [1, 2, 4, 6, 8])
def test_plan_of_a_run_is_the_references_tiling_and_grid(gpulib, oracle, nparts):
    W, H, F = 70, 52, 7
    size = (W, H, F, 1)
    p = gpulib.initializeNlbParameters(2, 20.0, size)
    gpulib.setSizePatch(p, size, 4)
    p.sizePatchTime = 2
    tiles = gpulib.plan(W, H, F, p, nparts=nparts)
    boxes = oracle.tile_crops(W, H, nparts, int(p.boundary))      # subDivideTight, pinned to the reference
    assert len(tiles) == len(boxes)
    for t, (ox, oy, ex, ey) in zip(tiles, boxes.tolist()):
        assert t["box"] == (ox, oy, ex - ox, ey - oy)
        b = (ox > 0, oy > 0, False, ex < W, ey < H, False)
        assert (t["xs"], t["ys"], t["fs"]) == expected_grid(ex - ox, ey - oy, F, p, b)
