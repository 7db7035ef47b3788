"""The allocation-free patch search, for callers that cannot call cudaMalloc.

bm4dof_search_groups_noalloc runs the same search kernels as bm4dof_run but
keeps every working buffer in one static device array; the caller supplies
the video, the flows and the output arrays.  Through the C ABI (ctypes, with
device buffers owned by the test) it must return the same neighbour lists as
bm4dof_run + bm4dof_get_groups -- exact, since indices are integers -- for
every group the run processed, on calls in a row, which also shows that the
contents one call leaves in the shared scratch do not leak into the next.
The run skips the groups its mask switches off; the allocation-free search
returns every grid group, so the comparison matches groups by reference
position, and one case has switch-offs.

This file sorts last so that a run stopping at the first failure has already
run every other test; it also passes alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

from cases import CFG_VIDEO
from helpers import resolve_params, video_case

pytestmark = pytest.mark.gpu


def noalloc_groups(lib, video, ff, bf, prm, nparts, tile, stride=32):
    """Calls the entry point with torch-owned device buffers; returns host arrays."""
    import torch
    F, Cc, H, W = video.shape
    dv = torch.from_numpy(np.ascontiguousarray(video)).cuda()
    df = torch.from_numpy(ff).cuda() if ff is not None else None
    db = torch.from_numpy(bf).cuda() if bf is not None else None
    count = C.c_size_t()
    ptr = lambda t: C.c_void_p(t.data_ptr()) if t is not None else None
    # size query: cap = 0 writes nothing and reports the group count
    rc = lib.bm4dof_search_groups_noalloc(ptr(dv), ptr(df), ptr(db), W, H, Cc, F, C.byref(prm), nparts, tile,
                                          None, None, None, stride, 0, C.byref(count), None)
    assert rc == 0, lib.bm4dof_last_error().decode()
    n = count.value
    ref = torch.empty(n, dtype=torch.int32, device="cuda")
    ns = torch.empty(n, dtype=torch.int32, device="cuda")
    idx = torch.empty(n * stride, dtype=torch.int32, device="cuda")
    rc = lib.bm4dof_search_groups_noalloc(ptr(dv), ptr(df), ptr(db), W, H, Cc, F, C.byref(prm), nparts, tile,
                                          ptr(ref), ptr(ns), ptr(idx), stride, n, C.byref(count), None)
    assert rc == 0, lib.bm4dof_last_error().decode()
    torch.cuda.synchronize()
    u = lambda t: t.cpu().numpy().view(np.uint32)
    return {"ref": u(ref), "nsimp": u(ns), "index": u(idx).reshape(n, stride)}


def plan_groups(gpulib, W, H, F, prm, nparts, tile):
    """Number of grid groups of one tile (bm4dof_plan, host only)."""
    t = gpulib.plan(W, H, F, prm, nparts=nparts)[tile]
    return len(t["xs"]) * len(t["ys"]) * len(t["fs"])


def check_against_run(gpulib, gpuctx, lib, nz, ff, bf, p1, p2, nparts):
    """Every group the run processed has the run's neighbour list in the
    allocation-free output, matched by reference position.  The run skips the
    groups the mask switches off (bm4dof_get_groups returns the processed ones
    only); the allocation-free search returns the whole grid.  Returns the
    number of groups the run switched off."""
    F, _, H, W = nz.shape
    basic, final, ratios = gpuctx.runNlBayes(nz, ff, bf, p1, p2, nparts=nparts, keep_groups=True)
    skipped = 0
    for step, prm, src in ((1, p1, nz), (2, p2, basic)):
        for tile in range(nparts):
            want = gpuctx.groups(step, tile)
            got = noalloc_groups(lib, src, ff, bf, prm, nparts, tile)
            n = plan_groups(gpulib, W, H, F, prm, nparts, tile)
            assert len(got["ref"]) == n
            # grid references are distinct and in processing order
            assert np.all(np.diff(got["ref"].astype(np.int64)) > 0)
            at = np.searchsorted(got["ref"], want["ref"])
            assert np.array_equal(got["ref"][at], want["ref"])
            assert np.array_equal(got["nsimp"][at], want["nsimp"])
            assert np.array_equal(got["index"][at], want["index"])
            skipped += n - len(want["ref"])
    return skipped


def test_noalloc_search_matches_run(gpulib, gpuctx):
    lib = gpulib.load()
    for seed in (61, 62):            # two calls in a row on different inputs
        W, H, F = 44, 38, 6
        clean, nz, ff, bf = video_case(W, H, F, sigma=20.0, seed=seed)
        p1, p2 = resolve_params(gpulib, (W, H, F, 1), 20.0, **CFG_VIDEO)
        check_against_run(gpulib, gpuctx, lib, nz, ff, bf, p1, p2, 2)


def test_noalloc_search_with_switch_offs(gpulib, gpuctx):
    # noise-free piecewise-constant frames: many patches equal the reference
    # patch exactly, the heap selection puts another of them first in some
    # neighbour lists, and the run switches off the groups at those positions
    # (8 per tile in step 1 on this input); the allocation-free search still
    # returns them
    lib = gpulib.load()
    rng = np.random.default_rng(5)
    W, H, F = 32, 28, 5
    base = rng.integers(0, 4, size=(H // 8 + 1, W // 8 + 1)).astype(np.float32) * 40
    fr = np.kron(base, np.ones((8, 8), np.float32))[:H, :W]
    nz = np.stack([np.roll(fr, k, axis=1) for k in range(F)])[:, None].copy()
    p1, p2 = resolve_params(gpulib, (W, H, F, 1), 10.0, **CFG_VIDEO)
    assert check_against_run(gpulib, gpuctx, lib, nz, None, None, p1, p2, 2) > 0


def test_noalloc_rejects_oversized_tile(gpulib, gpuctx):
    lib = gpulib.load()
    import torch
    W, H, F = 1920, 1080, 12
    p1, _ = resolve_params(gpulib, (W, H, F, 1), 20.0, **CFG_VIDEO)
    dv = torch.zeros((F, 1, H, W), dtype=torch.float32, device="cuda")
    count = C.c_size_t()
    rc = lib.bm4dof_search_groups_noalloc(C.c_void_p(dv.data_ptr()), None, None, W, H, 1, F, C.byref(p1), 2, 0,
                                          None, None, None, 32, 0, C.byref(count), None)
    assert rc == 1
    msg = lib.bm4dof_last_error().decode()
    assert "static scratch holds" in msg and "bytes" in msg
