"""Mixed-precision form: FP16 tensor-core pre-screen of the patch distances and
an exact FP32 re-rank of the best 2k candidates.  Not bit-exact by design; the
checks are the bars of the mixed form: neighbour sets that agree with the exact path
(the selected k nearest match whenever the true k nearest are among the 2k
best approximations) and a PSNR loss of at most 0.05 dB against the plain
method."""
import numpy as np
import pytest

from cases import CFG_IMAGE, CFG_VIDEO
from helpers import psnr, resolve_params, video_case

pytestmark = pytest.mark.gpu


def agreement(ctx_groups_a, ctx_groups_b):
    """Fraction of groups whose neighbour sets are equal (order ignored)."""
    same = total = 0
    for a, b in zip(ctx_groups_a, ctx_groups_b):
        assert np.array_equal(a["ref"], b["ref"])
        for i in range(len(a["ref"])):
            n1, n2 = a["nsimp"][i], b["nsimp"][i]
            s1 = set(a["index"][i, :n1].tolist())
            s2 = set(b["index"][i, :n2].tolist())
            same += s1 == s2
            total += 1
    return same / max(total, 1)


@pytest.mark.parametrize("cfg,shape", [(CFG_VIDEO, (64, 48, 8)), (CFG_IMAGE, (96, 80, 1))],
                         ids=["video_px4", "image_px8"])
def test_mixed_search_agrees_with_exact(gpulib, gpuctx, cfg, shape):
    W, H, F = shape
    clean, nz, ff, bf = video_case(W, H, F, sigma=20.0, seed=77)
    p = resolve_params(gpulib, (W, H, F, 1), 20.0, **cfg)
    pb, pf, pr = gpuctx.runNlBayes(nz, ff, bf, *p, nparts=2, keep_groups=True)
    plain1 = [gpuctx.groups(1, t) for t in range(2)]
    mb, mf, mr = gpuctx.runNlBayes(nz, ff, bf, *p, nparts=2, keep_groups=True, mixed=True)
    mixed1 = [gpuctx.groups(1, t) for t in range(2)]
    # step-1 searches run on the same noisy input: compare their neighbour sets
    agree = agreement(plain1, mixed1)
    assert agree >= 0.98, agree
    loss = psnr(pf, clean) - psnr(mf, clean)
    assert loss <= 0.05, loss


def test_mixed_unsupported_falls_back_to_exact(gpulib, gpuctx):
    # RGB step 2 searches three channels: the exact search runs there
    W, H, F = 40, 36, 4
    clean, nz, ff, bf = video_case(W, H, F, sigma=20.0, seed=5, channels=3)
    p = resolve_params(gpulib, (W, H, F, 3), 20.0, **CFG_VIDEO)
    a = gpuctx.runNlBayes(nz, ff, bf, *p, nparts=2)
    b = gpuctx.runNlBayes(nz, ff, bf, *p, nparts=2, mixed=True)
    assert np.isfinite(b[1]).all()
    assert abs(psnr(a[1], clean) - psnr(b[1], clean)) <= 0.05
