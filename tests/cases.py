"""Seeded parity workloads shared by the oracle, golden and GPU tests.
Each case: (name, W, H, F, C, sigma, seed, flow, cli-params, nthreads)."""
CFG_VIDEO = dict(px1=4, px2=4, pt1=4, pt2=4, wx1=21, wx2=21, np1=16, np2=16, b1=3.0)
CFG_IMAGE = dict(px1=8, px2=8, pt1=1, pt2=1, wx1=21, wx2=21, np1=16, np2=16, b1=3.0)

CASES = [
    ("image_px8", 48, 40, 1, 1, 20.0, 11, False, CFG_IMAGE, 1),
    ("image_defaults", 40, 36, 1, 1, 20.0, 12, False, {}, 1),
    ("image_sigma45", 40, 36, 1, 1, 45.0, 17, False, dict(px2=7), 1),
    ("video_px4", 40, 36, 6, 1, 20.0, 13, True, CFG_VIDEO, 1),
    ("video_px4_4tiles", 44, 40, 6, 1, 20.0, 14, True, CFG_VIDEO, 2),
    ("video_noflow", 36, 32, 5, 1, 20.0, 15, False, CFG_VIDEO, 1),
    ("video_6tiles", 52, 34, 5, 1, 10.0, 18, True, CFG_VIDEO, 3),
    ("video_misc", 40, 36, 5, 1, 30.0, 16, True,
     dict(px1=8, px2=7, pt1=1, pt2=1, wx1=9, wx2=11, np1=8, np2=32), 1),
    ("rgb_image", 40, 36, 1, 3, 20.0, 19, False, CFG_IMAGE, 1),
    ("rgb_video", 30, 28, 4, 3, 20.0, 20, True, CFG_VIDEO, 1),
    # -order-inv: one Wiener gain per coefficient for the mean row and one for the rest
    ("video_order_inv", 40, 36, 6, 1, 20.0, 21, True, dict(CFG_VIDEO, order_inv=True), 1),
    ("image_order_inv", 48, 40, 1, 1, 25.0, 22, False, dict(CFG_IMAGE, order_inv=True), 1),
    # doPasteBoost: every member's position and its 4 neighbours leave the mask
    ("video_paste", 40, 36, 6, 1, 20.0, 23, True, dict(CFG_VIDEO, paste_boost=True), 1),
    ("video_paste_4tiles", 44, 40, 6, 1, 20.0, 24, True, dict(CFG_VIDEO, paste_boost=True), 2),
    ("image_paste", 48, 40, 1, 1, 20.0, 25, False, dict(CFG_IMAGE, paste_boost=True), 1),
    ("rgb_video_paste", 30, 28, 4, 3, 20.0, 26, True, dict(CFG_VIDEO, paste_boost=True), 1),
    # 4x4 image patches (one-frame quad gather) and four-channel video
    ("image_px4", 44, 40, 1, 1, 20.0, 28, False,
     dict(px1=4, px2=4, pt1=1, pt2=1, wx1=21, wx2=21, np1=16, np2=16, b1=3.0), 1),
    ("video_c4", 30, 28, 4, 4, 20.0, 29, True, CFG_VIDEO, 1),
    # 3-frame patches: the generic search, filter and per-pixel gather paths
    ("video_pt3", 36, 32, 6, 1, 20.0, 27, True,
     dict(px1=4, px2=4, pt1=3, pt2=3, wx1=15, wx2=13, np1=16, np2=16, b1=3.0), 1),
    # the plain two-step method on one 256x256 grey image: 8x8 patches, bior1.5
    # in step 1, Kaiser aggregation window (nldct.cpp:637-714), 2 tiles
    ("config1_image", 256, 256, 1, 1, 20.0, 1, False, CFG_IMAGE, 1),
]

# The reference built with its VBM3D_SEARCH switch: predictive search (the
# best nSimilarPatchesPred matches of each frame seed small windows in the
# next), parameters from that build's initializeNlbParameters.
VBM3D_CASES = [
    ("vbm3d_video", 40, 36, 6, 1, 20.0, 31, True, CFG_VIDEO, 1),
    ("vbm3d_video_4tiles", 44, 40, 6, 1, 30.0, 32, True, CFG_VIDEO, 2),
    ("vbm3d_noflow", 36, 32, 5, 1, 20.0, 33, False, CFG_VIDEO, 1),
    ("vbm3d_rgb", 30, 28, 4, 3, 20.0, 34, True, CFG_VIDEO, 1),
    # the video defaults (8x8x1 patches, 7x7 window, 5x5 predicted windows,
    # 2 matches per frame) over a 9-frame temporal range
    ("vbm3d_defaults", 48, 40, 10, 1, 20.0, 35, True, {}, 1),
    # 3 matches per frame, 7x7 predicted windows, no centre bias in step 2
    ("vbm3d_npf3", 44, 36, 8, 1, 25.0, 36, True,
     dict(px1=4, px2=4, pt1=2, pt2=2, wx1=15, wx2=13, np1=16, np2=16, npf1=3, npf2=3,
          wxf1=7, wxf2=7, dsub2=0.0), 1),
    # one frame: the whole search is the reference frame's window
    ("vbm3d_image", 48, 40, 1, 1, 20.0, 37, False, CFG_IMAGE, 1),
    ("vbm3d_paste", 40, 36, 6, 1, 20.0, 38, True, dict(CFG_VIDEO, paste_boost=True), 1),
]

# VideoNLB::processNlBayes on one video cut from a larger source: each case is
# (name, W, H, F, C, sigma, seed, flow, cli-params, temporal range or None,
# crop ((origin x, y, t), (ending x, y, t), (source W, H, F, C)) or None,
# vbm3d).  Step 1 is run on the crop, then step 2 on the crop with that basic.
PROCESS_CASES = [
    ("process_image", 40, 36, 1, 1, 20.0, 41, False, CFG_IMAGE, None, None, False),
    ("process_left", 40, 36, 6, 1, 20.0, 42, True, CFG_VIDEO, None, ((12, 0, 0), (52, 36, 6), (52, 36, 6, 1)), False),
    ("process_inner", 40, 36, 6, 1, 20.0, 43, True, CFG_VIDEO, None, ((10, 8, 0), (50, 44, 6), (70, 60, 6, 1)), False),
    ("process_time", 32, 28, 12, 1, 20.0, 44, True, CFG_VIDEO, 1, ((0, 0, 2), (32, 28, 14), (32, 28, 17, 1)), False),
    ("process_rgb_right", 30, 28, 4, 3, 20.0, 45, True, CFG_VIDEO, None, ((0, 0, 0), (30, 28, 4), (60, 28, 4, 3)), False),
    ("process_paste_top", 40, 36, 6, 1, 20.0, 46, True, dict(CFG_VIDEO, paste_boost=True), None,
     ((0, 6, 0), (40, 42, 6), (40, 42, 6, 1)), False),
    ("process_noflow_bottom", 36, 32, 5, 1, 20.0, 47, False, CFG_VIDEO, None, ((0, 0, 0), (36, 32, 5), (36, 50, 5, 1)),
     False),
    ("process_vbm3d_inner", 40, 36, 6, 1, 20.0, 48, True, CFG_VIDEO, None, ((4, 4, 0), (44, 40, 6), (60, 50, 6, 1)),
     True),
]
