"""Generate tests/golden/*.npz by running the reference's own code (built
from its sources into oracle/_ref by oracle/Makefile) on the seeded cases of
tests/cases.py.  Inputs are stored with the outputs, so the fixtures do not
depend on the random generator of the machine that reads them.

    python tests/golden/make_golden.py [case names]   # default: every case
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
from helpers import resolve_params, video_case  # noqa: E402
from cases import CASES, PROCESS_CASES, VBM3D_CASES  # noqa: E402
import pyoracle  # noqa: E402

FIELDS = [f for f, _ in pyoracle.Params._fields_]


def main(names=()):
    pyoracle.build()
    refs = {False: pyoracle.Reference(), True: pyoracle.Reference(pyoracle.REF_VBM3D_SO)}
    for vbm3d, cases in ((False, CASES), (True, VBM3D_CASES)):
        for case in cases:
            if names and case[0] not in names:
                continue
            make_case(refs[vbm3d], case)
    for case in PROCESS_CASES:
        if names and case[0] not in names:
            continue
        make_process_case(refs[case[-1]], case)


def make_case(ref, case):
    (name, W, H, F, C, sigma, seed, flow, cli, nthreads) = case
    if True:
        clean, nz, ff, bf = video_case(W, H, F, sigma=sigma, seed=seed, channels=C, flow=flow)
        p1, p2 = resolve_params(ref, (W, H, F, C), sigma, **cli)
        basic, final, ratios = ref.runNlBayes(nz, ff, bf, p1, p2, nthreads=nthreads)
        out = dict(noisy=nz, clean=clean, basic=basic, final=final, ratios=np.array(ratios, np.float32),
                   nthreads=np.array(nthreads), sigma=np.array(sigma, np.float32))
        if ff is not None:
            out["fflow"], out["bflow"] = ff, bf
        for tag, p in (("p1", p1), ("p2", p2)):
            out[tag] = np.array([float(getattr(p, f)) for f in FIELDS], np.float64)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
        print(name, ratios)


def process_params(lib, case):
    """Both steps' parameters of a processNlBayes case (isFirstStep set as
    initializeNlbParameters sets it; tr overrides the temporal range)."""
    (name, W, H, F, C, sigma, seed, flow, cli, tr, crop, vbm3d) = case
    p1, p2 = resolve_params(lib, (W, H, F, C), sigma, **cli)
    if tr is not None:
        for p in (p1, p2):
            p.sizeSearchTimeRangeFwd = p.sizeSearchTimeRangeBwd = tr
    return p1, p2


def make_process_case(ref, case):
    (name, W, H, F, C, sigma, seed, flow, cli, tr, crop, vbm3d) = case
    clean, nz, ff, bf = video_case(W, H, F, sigma=sigma, seed=seed, channels=C, flow=flow)
    p1, p2 = process_params(ref, case)
    c = None if crop is None else pyoracle.make_crop(*crop)
    basic, _, g1 = ref.processNlBayes(nz, ff, bf, p1, c)
    _, final, g2 = ref.processNlBayes(nz, ff, bf, p2, c, basic=basic)
    out = dict(noisy=nz, basic=basic, final=final, groups=np.array([g1, g2], np.int64),
               crop=np.array([-1] * 10 if crop is None else [*crop[0], *crop[1], *crop[2]], np.int64))
    if ff is not None:
        out["fflow"], out["bflow"] = ff, bf
    for tag, p in (("p1", p1), ("p2", p2)):
        out[tag] = np.array([float(getattr(p, f)) for f in FIELDS], np.float64)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print(name, g1, g2)


if __name__ == "__main__":
    main(tuple(sys.argv[1:]))
