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


def _shifted_window(c, sw, extent, px):
    """nldct.cpp:1248-1258: the window is shifted, not clipped, into the frame."""
    hw = (sw - 1) // 2
    sh = min(0, c - hw) + max(0, c + hw - extent + px)
    return max(0, c - hw - sh), min(extent - px, c + hw - sh)


@pytest.mark.parametrize("vbm3d", [False, True])
def test_neighbours_lie_in_the_shifted_window(oracle, vbm3d):
    # one frame, no flow: every neighbour of a reference patch lies in its
    # search window, which keeps its full size at the borders (shifted)
    import pyoracle
    from helpers import resolve_params, video_case
    W, H = 40, 34
    clean, nz, ff, bf = video_case(W, H, 1, sigma=20.0, seed=7)
    cfg = dict(px1=8, px2=8, pt1=1, pt2=1, wx1=21, wx2=21, np1=16, np2=16)
    p1, p2 = resolve_params(oracle, (W, H, 1, 1), 20.0, **cfg)
    _, _, _, tr = oracle.runNlBayes(nz, None, None, p1, p2, nparts=1, trace_cap=100000, trace_stride=32,
                                    vbm3d=vbm3d)
    assert tr["count"] > 0
    for ref, ns, idx in zip(tr["ref"], tr["nsimp"], tr["index"]):
        x, y = int(ref) % W, int(ref) // W
        x0, x1 = _shifted_window(x, 21, W, 8)
        y0, y1 = _shifted_window(y, 21, H, 8)
        assert x1 - x0 + 1 == 21 and y1 - y0 + 1 == 21
        for q in idx[:ns]:
            qx, qy = int(q) % W, int(q) // W
            assert x0 <= qx <= x1 and y0 <= qy <= y1


def test_shifted_window_known_answers():
    # at the left border, in the middle, at the right border (W=40, px=8, 21 wide)
    assert _shifted_window(0, 21, 40, 8) == (0, 20)
    assert _shifted_window(16, 21, 40, 8) == (6, 26)
    assert _shifted_window(39, 21, 40, 8) == (12, 32)
    # a window wider than the frame's positions is clipped to them
    assert _shifted_window(5, 41, 40, 8) == (0, 32)
