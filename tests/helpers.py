"""Shared helpers of the test-suite: CLI-style parameter resolution and the
small seeded workloads the parity tests run on."""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "bm4d-of_gb300")
for p in (ROOT, PKG, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

import synthetic  # noqa: E402


def resolve_params(lib, size, sigma, px1=-1, px2=-1, pt1=1, pt2=1, wx1=-1, wx2=-1,
                   np1=-1, np2=-1, b1=-1.0, b2=-1.0, bm1=-1.0, bm2=-1.0, no_step1=False,
                   no_step2=False, order_inv=False, verbose=False, wxf1=-1, wxf2=-1, npf1=-1,
                   npf2=-1, dsub1=-1.0, dsub2=-1.0, t1=-1.0, t2=-1.0, paste_boost=False):
    """Parameter resolution of the reference CLI, src/main_vnlb.cpp:206-246
    (the run path: -t1/-t2 only apply under VBM3D_SEARCH, -wt1/-wt2 never).
    wxf*/npf*/dsub*/t* are the VBM3D_SEARCH build's options (main_vnlb.cpp:227-236).
    paste_boost sets nlbParams::doPasteBoost in both steps (no CLI flag enables it)."""
    p1 = lib.initializeNlbParameters(1, sigma, size, verbose)
    p2 = lib.initializeNlbParameters(2, sigma, size, verbose)
    if wx1 >= 0: lib.setSizeSearchWindow(p1, wx1)
    if wx2 >= 0: lib.setSizeSearchWindow(p2, wx2)
    if px1 >= 0: lib.setSizePatch(p1, size, px1)
    if px2 >= 0: lib.setSizePatch(p2, size, px2)
    if np1 >= 0: lib.setNSimilarPatches(p1, np1)
    if np2 >= 0: lib.setNSimilarPatches(p2, np2)
    if b1 >= 0: p1.beta = b1; p1.betaMean = b1
    if b2 >= 0: p2.beta = b2; p2.betaMean = b2
    if bm1 >= 0: p1.betaMean = bm1
    if bm2 >= 0: p2.betaMean = bm2
    if pt1 >= 0: p1.sizePatchTime = pt1
    if pt2 >= 0: p2.sizePatchTime = pt2
    if no_step1: p1.offSet = 1
    if no_step2: p2.offSet = 1
    if wxf1 >= 0: p1.sizeSearchWindowPred = wxf1
    if wxf2 >= 0: p2.sizeSearchWindowPred = wxf2
    if npf1 >= 0: p1.nSimilarPatchesPred = npf1
    if npf2 >= 0: p2.nSimilarPatchesPred = npf2
    if dsub1 >= 0: p1.dsub = dsub1
    if dsub2 >= 0: p2.dsub = dsub2
    if t1 >= 0: p1.tau = t1
    if t2 >= 0: p2.tau = t2
    if order_inv:
        p1.orderInvariance = 1
        p2.orderInvariance = 1
    if paste_boost:
        p1.doPasteBoost = 1
        p2.doPasteBoost = 1
    return p1, p2


def video_case(W, H, F, sigma=20.0, seed=1, channels=1, flow=True):
    """Seeded noisy video (F, C, H, W) with exact flow, and its clean version."""
    clean, ff, bf = synthetic.video(W, H, F, seed, channels=channels)
    nz = synthetic.noisy(clean, sigma, seed)
    if not flow or F == 1:
        ff = bf = None
    return clean, nz, ff, bf


def psnr(a, b):
    mse = np.mean((a.astype(np.float64) - b.astype(np.float64)) ** 2)
    return 10.0 * np.log10(255.0 ** 2 / mse)
