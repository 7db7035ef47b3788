"""Parameter resolution (src/core/nldct.cpp:81-249, src/main_vnlb.cpp:206-246):
the library, the oracle and the reference resolve identical nlbParams and print
identical text."""
import itertools

import pytest

from helpers import resolve_params

SIZES = [(256, 256, 1, 1), (854, 480, 20, 1), (64, 48, 9, 3), (1920, 1080, 60, 1)]
SIGMAS = [5.0, 20.0, 30.0, 40.0, 50.0]
CLI = [
    {},
    dict(px1=4, px2=4, pt1=4, pt2=4, wx1=21, wx2=21, np1=16, np2=16, b1=3.0),
    dict(px1=8, px2=8, pt1=1, pt2=1, wx1=21, wx2=21, np1=16, np2=16, b1=3.0),
    dict(px1=5, px2=7, pt1=2, pt2=3, wx1=9, wx2=0, np1=100, np2=1, b2=0.5, bm1=1.5, no_step2=True),
    dict(px1=0, px2=6),
]

FIELDS = ["sigma", "sizePatch", "sizePatchTime", "nSimilarPatches", "sizeSearchWindow",
          "sizeSearchTimeRangeFwd", "sizeSearchTimeRangeBwd", "boundary", "offSet", "offSetTime",
          "beta", "tau", "orderInvariance", "isFirstStep", "doPasteBoost", "colorSpace",
          "transform", "sizeSearchWindowPred", "nSimilarPatchesPred", "dsub", "agg_window"]


def _cases():
    return list(itertools.product(SIZES, SIGMAS, range(len(CLI))))


@pytest.mark.parametrize("size,sigma,ci", _cases())
def test_library_matches_oracle(gpulib, oracle, size, sigma, ci):
    a = resolve_params(gpulib, size, sigma, **CLI[ci])
    b = resolve_params(oracle, size, sigma, **CLI[ci])
    for pa, pb in zip(a, b):
        assert pa.as_dict() == pb.as_dict()
        assert gpulib.formatNlbParameters(pa) == oracle.formatNlbParameters(pb)


@pytest.mark.parametrize("size,sigma,ci", _cases()[::3])
def test_oracle_matches_reference(oracle, reference, size, sigma, ci):
    a = resolve_params(oracle, size, sigma, **CLI[ci])
    b = resolve_params(reference, size, sigma, **CLI[ci])
    for pa, pb in zip(a, b):
        da, db = pa.as_dict(), pb.as_dict()
        for f in FIELDS:   # betaMean is left uninitialised by the reference
            assert da[f] == db[f], f
        assert oracle.formatNlbParameters(pa) == reference.formatNlbParameters(pb)


def test_print_prms_quirk_temporal_window(gpulib):
    # printNlbParameters prints the backward range on both sides (nldct.cpp:223)
    p = gpulib.initializeNlbParameters(1, 20.0, (64, 64, 10, 1))
    p.sizeSearchTimeRangeFwd = 2
    p.sizeSearchTimeRangeBwd = 5
    assert "[-5,5]" in gpulib.formatNlbParameters(p)
