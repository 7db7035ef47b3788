"""The host-core baseline of bench.py counts the groups of a run without the
GPU library (its reference arm loads none of it): the count must equal the
library's own planner (bm4dof_plan, itself checked against the reference's
grid loop) for videos and images, 1 to 32 tiles."""
import sys

import pytest

from helpers import ROOT, resolve_params
from cases import CFG_IMAGE, CFG_VIDEO


@pytest.mark.parametrize("shape,cli", [((1920, 1080, 60), CFG_VIDEO), ((480, 272, 12), CFG_VIDEO),
                                       ((854, 480, 20), CFG_VIDEO), ((256, 256, 1), CFG_IMAGE),
                                       ((101, 77, 9), dict(CFG_VIDEO, wx1=15, px2=5))])
@pytest.mark.parametrize("nparts", [1, 2, 6, 16, 32])
def test_bench_group_count_matches_planner(gpulib, shape, cli, nparts):
    sys.path.insert(0, ROOT)
    import bench
    W, H, F = shape
    for p in resolve_params(gpulib, (W, H, F, 1), 20.0, **cli):
        want = sum(len(t["xs"]) * len(t["ys"]) * len(t["fs"]) for t in gpulib.plan(W, H, F, p, nparts=nparts))
        assert bench.plan_groups(W, H, F, p, nparts) == want
