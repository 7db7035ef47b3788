"""Batched runs: many sequences of uneven size, frame count and sigma denoised
by one CUDA graph (bm4dof_run_batched) give, sequence by sequence, exactly the
output of the unbatched call; the instantiated graph is replayed on a repeat
call; the autotuner returns a tuning it measured."""
import numpy as np
import pytest

from helpers import resolve_params, video_case

pytestmark = pytest.mark.gpu

CFG = dict(px1=4, px2=4, pt1=4, pt2=4, wx1=21, wx2=21, np1=16, np2=16, b1=3.0)
SIGMAS = (5.0, 10.0, 20.0, 30.0, 40.0, 50.0)


def batch(gpulib, n=6, seed=3):
    import torch
    rng = np.random.default_rng(seed)
    items = []
    for i in range(n):
        W = int(rng.integers(6, 13)) * 8
        H = int(rng.integers(5, 11)) * 8
        F = int(rng.integers(5, 9))
        sigma = float(SIGMAS[i % len(SIGMAS)])
        clean, nz, ff, bf = video_case(W, H, F, sigma=sigma, seed=100 + i)
        p1, p2 = resolve_params(gpulib, (W, H, F, 1), sigma, **CFG)
        d = [torch.from_numpy(a).cuda() for a in (nz, ff, bf)]
        items.append({"noisy": d[0], "fflow": d[1], "bflow": d[2], "basic": torch.zeros_like(d[0]),
                      "final": torch.zeros_like(d[0]), "p1": p1, "p2": p2, "nparts": 2, "clean": clean})
    return items


def test_batched_matches_unbatched(gpulib, gpuctx):
    items = batch(gpulib)
    ratios = gpuctx.run_batched(items, tuning={"branches": 3, "slot_mb": 64, "search_ctas": 0})
    for it, r in zip(items, ratios):
        b, f, rr = gpuctx.runNlBayes(it["noisy"], it["fflow"], it["bflow"], it["p1"], it["p2"], nparts=2)
        assert np.array_equal(b.cpu().numpy(), it["basic"].cpu().numpy())
        assert np.array_equal(f.cpu().numpy(), it["final"].cpu().numpy())
        assert abs(r[0] - rr[0]) < 1e-4 and abs(r[1] - rr[1]) < 1e-4


def test_batched_replay_and_autotune(gpulib, gpuctx):
    items = batch(gpulib, n=5, seed=8)
    gpuctx.run_batched(items)
    first = [it["final"].clone() for it in items]
    for it in items:
        it["final"].zero_()
    gpuctx.run_batched(items)            # same batch: the graph is replayed
    for a, it in zip(first, items):
        assert bool((a == it["final"]).all())
    best, table = gpuctx.autotune(items, sample=4)
    assert best["branches"] >= 1 and best["slot_mb"] in (256, 1024, 4096) and best["search_ctas"] in (4, 6)
    assert best["search_strip"] in (7, 21) and best["gather_depth"] in (1, 2)
    assert len(table) >= 6 and all(row[5] > 0 for row in table)
    # every tile shape and staging depth was timed
    assert {(r[2], r[3]) for r in table} >= {(6, 21), (6, 7), (4, 7)} and {r[4] for r in table} == {1, 2}
    gpuctx.run_batched(items, tuning=best)
    for a, it in zip(first, items):
        assert bool((a == it["final"]).all())
    # the other shapes and depths give the same outputs
    for tu in ({"search_strip": 7}, {"gather_depth": 2}, {"search_ctas": 4, "search_strip": 7}):
        gpuctx.run_batched(items, tuning=dict(best, **tu))
        for a, it in zip(first, items):
            assert bool((a == it["final"]).all()), tu
    with pytest.raises(gpulib.BM4DOFError):
        gpuctx.run_batched(items, tuning=dict(best, search_strip=9))


def test_batched_learned_matches_unbatched(gpulib, gpuctx):
    items = batch(gpulib, n=3, seed=11)
    gpuctx.set_gain_network(None)
    gpuctx.run_batched(items, learned=True)
    for it in items:
        _, f, _ = gpuctx.runNlBayes(it["noisy"], it["fflow"], it["bflow"], it["p1"], it["p2"], learned=True)
        assert np.array_equal(f.cpu().numpy(), it["final"].cpu().numpy())
