"""Known-answer tests derived from the reference source (no golden vectors
ship with it): bases, windows, Haar, tiling, colour transform, tau rule."""
import numpy as np
import pytest


@pytest.mark.parametrize("px,pt", [(4, 4), (8, 1), (7, 1), (4, 1), (2, 3)])
def test_dct_basis_orthonormal(oracle, px, pt):
    # nldct.cpp:582-610: dense 3-D DCT-II, inverse = forward
    B, Bi = oracle.basis(0, px, pt)
    n = px * px * pt
    assert np.array_equal(B, Bi)
    assert np.allclose(B @ B.T, np.eye(n), atol=2e-6)
    # DC basis vector is constant 1/sqrt(n)
    assert np.allclose(B[0], 1.0 / np.sqrt(n), atol=1e-7)


@pytest.mark.parametrize("pt", [1, 2])
def test_bior15_analysis_synthesis_identity(oracle, pt):
    # nldct.cpp:637-695: Z = G.B then G = Z.Binv^T must reproduce G
    B, Bi = oracle.basis(1, 8, pt)
    n = 64 * pt
    # bases stored basis[k*n + p]: forward z_k = sum_p g_p B[k, p] (Z = G B^T),
    # inverse g_p = sum_k z_k Bi[k, p] (G = Z Bi), so B^T Bi is the identity up
    # to the rounding of the reference's tables: within 3e-2 (they are not an
    # exact biorthogonal pair), and far from any other pairing of the factors
    err = np.abs(B.T @ Bi - np.eye(n)).max()
    assert err < 0.035
    assert np.abs(B @ Bi - np.eye(n)).max() > 1.0


def test_bior15_needs_px8(oracle):
    with pytest.raises(ValueError):
        oracle.basis(1, 4, 1)


def test_kaiser_window(oracle):
    w = oracle.window(True, 8, 2).reshape(2, 8, 8)
    assert np.array_equal(w[0], w[1])
    assert w[0, 0, 0] == np.float32(0.1924) and w[0, 3, 3] == np.float32(0.9718)
    assert np.array_equal(w[0], w[0].T) and np.array_equal(w[0], w[0][::-1, ::-1])
    assert np.all(oracle.window(True, 4, 4) == 1.0)
    assert np.all(oracle.window(False, 8, 1) == 1.0)
    w10 = oracle.window(True, 10, 1).reshape(10, 10)
    assert w10[4, 4] == np.float32(0.9829)


def haar(z):
    # nldct.cpp:1846-1860 on one column
    z = np.array(z, np.float32)
    n = len(z)
    is2 = np.float32(1.0 / np.sqrt(2.0))
    s, h = 2, 1
    while s <= n:
        for i in range(0, n, s):
            a, b = z[i] * is2, z[i + h] * is2
            z[i], z[i + h] = a + b, a - b
        s, h = 2 * s, 2 * h
    return z


def ihaar(z):
    z = np.array(z, np.float32)
    n = len(z)
    is2 = np.float32(1.0 / np.sqrt(2.0))
    s, h = n, n // 2
    while s >= 2:
        for i in range(0, n, s):
            a, b = z[i] * is2, z[i + h] * is2
            z[i], z[i + h] = a + b, a - b
        s, h = s // 2, h // 2
    return z


@pytest.mark.parametrize("n", [1, 2, 4, 8, 16])
def test_haar_inverse_and_orthonormal(n):
    rng = np.random.default_rng(n)
    z = rng.normal(size=n).astype(np.float32) * 50
    assert np.allclose(ihaar(haar(z)), z, atol=1e-4)
    assert np.isclose(np.sum(haar(z).astype(np.float64) ** 2), np.sum(z.astype(np.float64) ** 2), rtol=1e-5)


def tau_rule(d, nsim, tau2):
    # nldct.cpp:1284-1289
    n = 1
    while 2 * n <= nsim and d[n] < tau2:
        n *= 2
    return n


def test_tau_power_of_two_rule():
    d = np.arange(16, dtype=np.float32)
    assert tau_rule(d, 16, 100.0) == 16
    assert tau_rule(d, 16, 8.0) == 8       # d[8] = 8 is not < 8
    assert tau_rule(d, 16, 7.5) == 8       # d[4]=4 < 7.5, d[8]=8 stops
    assert tau_rule(d, 16, 1.0) == 1
    assert tau_rule(d, 15, 100.0) == 8     # largest power of two <= 15
    assert tau_rule(d, 1, 100.0) == 1


@pytest.mark.parametrize("n,ab", [(1, (1, 1)), (2, (2, 1)), (4, (2, 2)), (6, (3, 2)), (8, (4, 2)),
                                  (16, (8, 2)), (12, (6, 2)), (9, (3, 3)), (7, (7, 1))])
def test_determine_factor(oracle, n, ab):
    # utilities.cpp:137-158
    assert oracle.determine_factor(n) == ab


def test_tile_boxes(oracle):
    # lib_videot.hpp:853-916: 2 tiles of an 854-wide frame with boundary 23
    b = oracle.tile_crops(854, 480, 2, 23)
    assert b.tolist() == [[0, 0, 450, 480], [404, 0, 854, 480]]
    b = oracle.tile_crops(1920, 1080, 16, 23)
    assert len(b) == 16 and b[0].tolist() == [0, 0, 263, 563]
    assert b[-1].tolist() == [1657, 517, 1920, 1080]


def test_color_transform_roundtrip(oracle):
    rng = np.random.default_rng(0)
    for C in (3, 4):
        v = rng.uniform(0, 255, size=(2, C, 5, 7)).astype(np.float32)
        y = oracle.color_transform(v, True)
        back = oracle.color_transform(y, False)
        assert np.allclose(back, v, atol=1e-3)
        # orthonormal: energy preserved per pixel
        assert np.allclose((y.astype(np.float64) ** 2).sum(1), (v.astype(np.float64) ** 2).sum(1), rtol=1e-5)
    g = rng.uniform(0, 255, size=(2, 1, 5, 7)).astype(np.float32)
    assert np.array_equal(oracle.color_transform(g, True), g)
