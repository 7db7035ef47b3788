"""CPU checks of the gain-network oracle (oracle/gain_mlp.py): its analytic
gradient against central finite differences, the BF16 rounding helper, and
the Haar / Wiener-target restatement."""
import numpy as np

import gain_mlp as gm


def small_blob(seed):
    rng = np.random.default_rng(seed)
    parts = []
    for s in gm.SHAPES:
        fan = s[0] if len(s) == 2 else 1
        parts.append(rng.normal(0, 1.0 / np.sqrt(fan), s) if len(s) == 2 else rng.normal(0, 0.1, s))
    return gm.join(parts)


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(1)
    blob = small_blob(2)
    X = rng.normal(0, 1, (5, gm.N_IN))
    T = rng.uniform(0, 1, (5, gm.N_OUT))
    loss, g = gm.loss_and_grad(blob, X, T)
    assert g.shape == blob.shape
    idx = rng.choice(blob.size, 60, replace=False)
    # one index from every tensor as well
    offs = np.cumsum([0] + [int(np.prod(s)) for s in gm.SHAPES])
    idx = np.concatenate([idx, offs[:-1] + 3])
    h = 1e-6
    for i in idx:
        bp, bm = blob.copy(), blob.copy()
        bp[i] += h
        bm[i] -= h
        fd = (gm.loss_and_grad(bp, X, T)[0] - gm.loss_and_grad(bm, X, T)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 + 1e-4 * abs(fd), (i, fd, g[i])


def test_bf16_round():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -2.5, 3.14159265, 0.0], np.float32)
    r = gm.bf16_round(x)
    # ties to even at 1 + 2^-8 (halfway between 1 and 1 + 2^-7) -> 1
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 2 ** -6
    assert r[3] == -2.5 and abs(r[4] - 3.140625) < 1e-12 and r[5] == 0.0


def test_haar_orthonormal_and_target_range():
    rng = np.random.default_rng(3)
    for n in (1, 2, 4, 8, 16, 32):
        Z = rng.normal(0, 10, (n, 64))
        H = gm.haar(Z)
        assert np.allclose((H ** 2).sum(0), (Z ** 2).sum(0))
        assert np.allclose(H[0], Z.sum(0) / np.sqrt(n))
        t = gm.target(Z, 20.0, 1.0)
        assert t.shape == (64,) and np.all((t >= 0) & (t <= 1))
    f = gm.features(rng.normal(0, 20, (16, 64)), 20.0)
    assert f.shape == (65,) and abs(f[64] - 20 / 255) < 1e-12
