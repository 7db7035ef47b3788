"""Generate tests/golden/tvl1_*.npz with the reference's own TV-L1 code
(lib/tvl1flow, built from its sources into oracle/_ref/libtvl1_ref.so by
oracle/Makefile) on seeded synthetic frame pairs, with the parameters
scripts/tvl1flow-seq.sh passes (tau 0.25, lambda 0.2, theta 0.3, 100 scales
capped by the image size, finest level 1, factor 0.5, 5 warpings, epsilon
0.01).  Inputs are stored with the outputs.

    python tests/golden/make_tvl1_golden.py
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [os.path.dirname(HERE), os.path.join(ROOT, "bm4d-of_gb300"), os.path.join(ROOT, "oracle")]
import pyoracle  # noqa: E402
import synthetic  # noqa: E402

LIB = os.path.join(ROOT, "oracle", "_ref", "libtvl1_ref.so")
PARAMS = dict(tau=0.25, lambda_=0.2, theta=0.3, nscales=100, fscale=1, zfactor=0.5, warps=5, epsilon=0.01)
CASES = [
    # name, W, H, frames of the clip, pair (t0, t1), noise sigma, seed, fscale
    ("tvl1_clean_fwd", 64, 48, 3, (0, 1), 0.0, 41, 1),
    ("tvl1_noisy_bwd", 96, 72, 3, (2, 1), 20.0, 42, 1),
    ("tvl1_noisy_full", 80, 64, 2, (0, 1), 10.0, 43, 0),
]


def ref_tvl1(I0, I1, fscale):
    L = C.CDLL(LIB)
    fp = C.POINTER(C.c_float)
    L.ref_tvl1.argtypes = [fp, fp, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, C.c_int, C.c_int,
                           C.c_float, C.c_int, C.c_float, fp, fp]
    H, W = I0.shape
    a, b = np.ascontiguousarray(I0, np.float32), np.ascontiguousarray(I1, np.float32)
    u, v = np.zeros_like(a), np.zeros_like(a)
    P = PARAMS
    L.ref_tvl1(a.ctypes.data_as(fp), b.ctypes.data_as(fp), W, H, P["tau"], P["lambda_"], P["theta"], P["nscales"],
               fscale, P["zfactor"], P["warps"], P["epsilon"], u.ctypes.data_as(fp), v.ctypes.data_as(fp))
    return u, v


def main():
    pyoracle.build()
    for name, W, H, F, (t0, t1), sigma, seed, fscale in CASES:
        clean, ff, bf = synthetic.video(W, H, F, seed)
        frames = synthetic.noisy(clean, sigma, seed) if sigma > 0 else clean
        I0, I1 = frames[t0, 0], frames[t1, 0]
        u, v = ref_tvl1(I0, I1, fscale)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), I0=I0, I1=I1, u=u, v=v, fscale=np.array(fscale),
                            true_flow=(ff if t1 > t0 else bf)[t0])
        print(name, float(np.abs(u).mean()), float(np.abs(v).mean()))


if __name__ == "__main__":
    main()
