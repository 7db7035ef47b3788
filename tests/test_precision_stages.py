"""Error of the approximate stages against an FP64 restatement, on the CPU.

The GPU kernels of the faster forms round in two places: the mixed form's
distance pre-screen (centred FP16 patch values, cross terms <p', q'> with FP32
accumulation on the tensor cores, |p'|^2 + |q'|^2 - 2<p', q'>), and the BF16
patch transforms of the learned form (BF16 operands, FP32 accumulation).  Here
both are restated in numpy with the same operand rounding and FP32
accumulation and compared with FP64 on patches of the benchmark's synthetic
video, so each stage's error is stated, with its bound written in the test:

* pre-screen: distance error below 0.2 % of max(distance, 2*64*sigma^2)
  (0.09 % measured); the true 16 nearest are among the 32 best approximations
  in every one of the sampled groups of a 21 x 21 window;
* BF16 transform: coefficient error below 1 % of the coefficients' RMS
  (0.6 % measured), and 0.8 % of the pixels' RMS after the BF16 inverse.

The accumulation order on the tensor cores differs from numpy's; FP32
accumulation of 64 terms contributes well under the operand rounding here.
"""
import numpy as np
import pytest

from helpers import video_case

SIGMA = 20.0


def _patches(frame, xs, ys, px=4):
    """(n, px*px) patches with top-left corners (xs, ys) of one frame."""
    return np.stack([frame[y:y + px, x:x + px].ravel() for x, y in zip(xs, ys)])


def _bf16(x):
    a = np.ascontiguousarray(x, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


def _video():
    clean, nz, ff, bf = video_case(96, 80, 4, sigma=SIGMA, seed=41)
    return nz[:, 0].astype(np.float64)   # (F, H, W)


def test_fp16_prescreen_distance_error_and_recall():
    v = _video()
    px, pt, wx, k = 4, 4, 21, 16
    rng = np.random.default_rng(0)
    H, W = v.shape[1:]
    scale = 2.0 * px * px * pt * SIGMA ** 2
    worst, groups = 0.0, 0
    for _ in range(40):
        x = int(rng.integers(10, W - px - 10))
        y = int(rng.integers(10, H - px - 10))
        hw = (wx - 1) // 2
        qs = [(qx, qy) for qy in range(y - hw, y + hw + 1) for qx in range(x - hw, x + hw + 1)
              if 0 <= qx <= W - px and 0 <= qy <= H - px]
        ref = np.concatenate([v[t, y:y + px, x:x + px].ravel() for t in range(pt)])
        cand = np.stack([np.concatenate([v[t, qy:qy + px, qx:qx + px].ravel() for t in range(pt)])
                         for qx, qy in qs])
        exact = ((cand - ref) ** 2).sum(1)                                   # FP64
        p16 = (ref - 128.0).astype(np.float16).astype(np.float32)
        q16 = (cand - 128.0).astype(np.float16).astype(np.float32)
        approx = (p16 * p16).sum(dtype=np.float32) + (q16 * q16).sum(1, dtype=np.float32) \
            - np.float32(2.0) * (q16 * p16).sum(1, dtype=np.float32)
        err = np.abs(approx.astype(np.float64) - exact) / np.maximum(exact, scale)
        worst = max(worst, float(err.max()))
        true_k = set(np.argsort(exact, kind="stable")[:k].tolist())
        top_2k = set(np.argsort(approx, kind="stable")[:2 * k].tolist())
        assert true_k <= top_2k
        groups += 1
    assert groups == 40
    assert worst < 2e-3, worst


@pytest.mark.parametrize("ns", [4, 16])
def test_bf16_transform_error(oracle, ns):
    v = _video()
    B, Bi = oracle.basis(0, 4, 4)            # 64 x 64 DCT, B[k][p]
    rng = np.random.default_rng(1)
    H, W = v.shape[1:]
    xs = rng.integers(0, W - 4, size=ns)
    ys = rng.integers(0, H - 4, size=ns)
    G = np.stack([np.concatenate([v[t, y:y + 4, x:x + 4].ravel() for t in range(4)]) for x, y in zip(xs, ys)])
    Z64 = G @ B.astype(np.float64).T                                         # members x coefficients
    Zbf = (_bf16(G).astype(np.float32) @ _bf16(B.T).astype(np.float32)).astype(np.float64)
    rms = np.sqrt(np.mean(Z64 ** 2))
    err = np.abs(Zbf - Z64).max() / rms
    assert err < 1e-2, err
    # and back: the inverse transform of BF16 coefficients
    back = (_bf16(Zbf).astype(np.float32) @ _bf16(Bi).astype(np.float32)).astype(np.float64)
    assert np.abs(back - G).max() / np.sqrt(np.mean(G ** 2)) < 2e-2
