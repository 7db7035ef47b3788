"""Parity at the benchmark configurations and on the chunked aggregation path.

* The 854x480x20 grey video of the benchmarks (4x4x4 patches, 21x21 window,
  +-4 frames along the exact flow, sigma 20), run in full on the GPU and by
  the oracle on the host's cores with the same 16 tiles: basic and final
  bit-identical, identical processed-group ratios, and every group's
  neighbour list identical, order included.  (The 256x256 image
  configuration is a golden case, `config1_image` in tests/cases.py, made by
  the reference itself.)
* Every golden case again with a chunk budget so small that each tile of each
  step is filtered and aggregated in three or more chunks of groups: the
  ordered gather then adds a pixel's terms chunk after chunk, and the output
  must stay bit-identical to the reference's.
"""
import os

import numpy as np
import pytest

from cases import CASES, CFG_VIDEO
from helpers import ROOT, resolve_params

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(ROOT, "tests", "golden")


def term_stride(C):
    return 2 if C == 1 else (4 if C <= 3 else 8)


def list_entries(p):
    """List entries per member: 4x4 patches take the quad path (at most 2 row-
    list and 8 quad-list entries), other sizes px*px spatial-list entries."""
    quad = p.sizePatch == 4 and p.sizePatchTime in (1, 2, 4)
    return 10 if quad else p.sizePatch * p.sizePatch


def chunk_bytes(p, C):
    """Bytes one group takes in a chunk (the runtime's per-group budget):
    np x (terms of every patch element, origin list entry, gather lists)."""
    spc = p.sizePatch * p.sizePatch * p.sizePatchTime
    return p.nSimilarPatches * (term_stride(C) * spc + 1 + list_entries(p)) * 4


def gparams(gpulib, arr):
    p = gpulib.Params()
    for (f, t), v in zip(gpulib.Params._fields_, arr):
        setattr(p, f, float(v) if t.__name__ == "c_float" else int(v))
    return p


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_gpu_golden_in_small_chunks(gpulib, gpuctx, case, monkeypatch):
    g = dict(np.load(os.path.join(GOLDEN, case[0] + ".npz")))
    p1, p2 = gparams(gpulib, g["p1"]), gparams(gpulib, g["p2"])
    nparts = 2 * int(g["nthreads"])
    F, C, H, W = g["noisy"].shape
    # the largest budget under which every tile of every step takes >= 3 chunks
    budget, extra = None, 0
    for p in (p1, p2):
        tiles = gpulib.plan(W, H, F, p, nparts=nparts)
        groups = [len(t["xs"]) * len(t["ys"]) * len(t["fs"]) for t in tiles]
        per = chunk_bytes(p, C)
        b = per * max(1, min(groups) // 3)
        budget = b if budget is None else min(budget, b)
    for p in (p1, p2):
        per = chunk_bytes(p, C)
        chunk = max(1, budget // per)
        for t in gpulib.plan(W, H, F, p, nparts=nparts):
            n = len(t["xs"]) * len(t["ys"]) * len(t["fs"])
            assert (n + chunk - 1) // chunk >= 3
            extra += (n + chunk - 1) // chunk - 1
    gpuctx.runNlBayes(g["noisy"], g.get("fflow"), g.get("bflow"), p1, p2, nparts=nparts)
    one_chunk_launches = gpuctx.timings()[1]
    monkeypatch.setenv("BM4DOF_SLOT_MB", repr(budget / 1048576.0))
    basic, final, ratios = gpuctx.runNlBayes(g["noisy"], g.get("fflow"), g.get("bflow"), p1, p2, nparts=nparts)
    launches = gpuctx.timings()[1]
    monkeypatch.delenv("BM4DOF_SLOT_MB")
    # at least 10 launches per chunk (filter 2, origin lists 4, gather 4 or more)
    assert launches >= one_chunk_launches + 10 * extra, (launches, one_chunk_launches, extra)
    assert np.array_equal(basic, g["basic"], equal_nan=True)
    assert np.array_equal(final, g["final"], equal_nan=True)
    assert ratios == tuple(g["ratios"].tolist())


def test_gpu_c2_video_matches_oracle(gpulib, gpuctx, oracle):
    import synthetic
    W, H, F, sigma, seed, nparts = 854, 480, 20, 20.0, 2, 16
    clean, ff, bf = synthetic.video(W, H, F, seed)
    nz = synthetic.noisy(clean, sigma, seed)
    po = resolve_params(oracle, (W, H, F, 1), sigma, **CFG_VIDEO)
    pg = resolve_params(gpulib, (W, H, F, 1), sigma, **CFG_VIDEO)
    cap = sum(len(t["xs"]) * len(t["ys"]) * len(t["fs"])
              for p in pg for t in gpulib.plan(W, H, F, p, nparts=nparts))
    threads = min(nparts, os.cpu_count() or 1)
    ob, of, orat, tr = oracle.runNlBayes(nz, ff, bf, *po, nparts=nparts, nthreads=threads, trace_cap=cap,
                                         trace_stride=16)
    assert tr["count"] <= cap
    gb, gf, grat = gpuctx.runNlBayes(nz, ff, bf, *pg, nparts=nparts, keep_groups=True)
    assert np.array_equal(gb, ob) and np.array_equal(gf, of)
    assert grat == orat
    for step in (1, 2):
        for tile in range(nparts):
            sel = (tr["step"] == step) & (tr["tile"] == tile)
            gg = gpuctx.groups(step, tile, stride=16)
            assert np.array_equal(gg["ref"], tr["ref"][sel])
            assert np.array_equal(gg["nsimp"], tr["nsimp"][sel])
            assert np.array_equal(gg["index"], tr["index"][sel])
