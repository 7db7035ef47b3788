"""Learned form: the gain network's GPU kernels against the float64 oracle
(forward outputs and the gradients of the training loss), its training pairs
against a restatement of the step-2 Wiener rule, training on the GPU, and the
learned run itself -- including what the trained network gains over the same
filter without it."""
import os

import numpy as np
import pytest

import gain_mlp as gm
from helpers import psnr, resolve_params, video_case

pytestmark = pytest.mark.gpu

CFG = dict(px1=4, px2=4, pt1=4, pt2=4, wx1=21, wx2=21, np1=16, np2=16, b1=3.0)


def rand_features(rng, n):
    X = np.empty((n, 65), np.float32)
    X[:, :64] = rng.normal(1.0, 2.0, (n, 64))
    X[:, 64] = rng.uniform(5, 50, n) / 255.0
    return X


def rounded_blob(params):
    """The parameters the GPU computes with: matrices rounded to BF16, biases FP32."""
    parts = gm.split(params)
    return gm.join([gm.bf16_round(p) if p.ndim == 2 else p for p in parts])


def test_forward_matches_oracle(gpulib, gpuctx):
    import torch
    rng = np.random.default_rng(11)
    tr = gpulib.Trainer(batch=512, seed=3)
    params = tr.params()
    X = rand_features(rng, 300)
    got = tr.predict(torch.from_numpy(X).cuda()).cpu().numpy()
    want, _ = gm.forward(rounded_blob(params), gm.bf16_round(X))
    # hidden activations are BF16 on the GPU (relative rounding 2^-9)
    assert np.abs(got - want).max() < 1e-2
    assert np.abs(got - want).mean() < 1.5e-3


def test_gradients_match_oracle(gpulib, gpuctx):
    import torch
    rng = np.random.default_rng(12)
    tr = gpulib.Trainer(batch=1024, seed=4)
    params = tr.params()
    X = rand_features(rng, 1000)
    T = rng.uniform(0, 1, (1000, 64)).astype(np.float32)
    g, loss = tr.grad(torch.from_numpy(X).cuda(), torch.from_numpy(T).cuda())
    wl, wg = gm.loss_and_grad(rounded_blob(params), gm.bf16_round(X), T.astype(np.float64))
    assert abs(loss - wl) <= 1e-2 * wl
    for name, a, b in zip(("W1", "b1", "W2", "b2", "W3", "b3"), gm.split(g), gm.split(wg)):
        rel = np.linalg.norm(a - b) / np.linalg.norm(b)
        assert rel < 3e-2, (name, rel)


def samples_case(gpulib, gpuctx, W=64, H=56, F=8, sigma=25.0, seed=21):
    import torch
    clean, nz, ff, bf = video_case(W, H, F, sigma=sigma, seed=seed)
    p1, p2 = resolve_params(gpulib, (W, H, F, 1), sigma, **CFG)
    d = [torch.from_numpy(a).cuda() for a in (nz, ff, bf)]
    basic, _, _ = gpuctx.runNlBayes(*d, p1, p2, nparts=1)
    feat, tgt = gpuctx.gain_samples(d[0], basic, d[1], d[2], p2, nparts=1)
    return nz, basic.cpu().numpy(), d, p1, p2, feat, tgt


def test_gain_samples_match_oracle(gpulib, gpuctx, oracle):
    nz, basic, d, p1, p2, feat, tgt = samples_case(gpulib, gpuctx)
    F, _, H, W = nz.shape
    # the same groups, from a learned run on one tile
    gpuctx.set_gain_network(None)
    gpuctx.runNlBayes(*d, p1, p2, nparts=1, keep_groups=True, learned=True)
    grp = gpuctx.groups(2, 0)
    assert len(grp["ref"]) == feat.shape[0] > 0
    B, _ = oracle.basis(0, 4, 4)
    feat, tgt = feat.cpu().numpy(), tgt.cpu().numpy()
    sigma = p2.sigma
    for i in range(0, len(grp["ref"]), max(1, len(grp["ref"]) // 150)):
        n = grp["nsimp"][i]
        G, Gb = [], []
        for q in grp["index"][i, :n]:
            t, r = divmod(int(q), W * H)
            y, x = divmod(r, W)
            G.append(nz[t:t + 4, 0, y:y + 4, x:x + 4].ravel())
            Gb.append(basic[t:t + 4, 0, y:y + 4, x:x + 4].ravel())
        Z = np.array(G, np.float64) @ B.T.astype(np.float64)
        Zb = np.array(Gb, np.float64) @ B.T.astype(np.float64)
        assert np.allclose(feat[i], gm.features(Z, sigma), atol=1e-3, rtol=1e-4)
        assert np.allclose(tgt[i], gm.target(Zb, sigma, p2.beta), atol=2e-4)


def test_training_reduces_loss(gpulib, gpuctx):
    *_, feat, tgt = samples_case(gpulib, gpuctx, W=96, H=80, F=8, seed=5)
    tr = gpulib.Trainer(batch=1024, seed=9)
    n = feat.shape[0]
    _, first = tr.grad(feat[:1024].contiguous(), tgt[:1024].contiguous())
    import torch
    g = torch.Generator().manual_seed(0)
    for s in range(300):
        idx = torch.randint(0, n, (1024,), generator=g).cuda()
        tr.step(feat[idx].contiguous(), tgt[idx].contiguous(), 2e-3, 1e-4, want_loss=False)
    _, last = tr.grad(feat[:1024].contiguous(), tgt[:1024].contiguous())
    assert last < 0.5 * first, (first, last)


def trained_params():
    import train_gains
    p = train_gains.load_weights()
    if p is None:
        pytest.skip("no trained gain network in the package (bm4d-of_gb300/weights/gain_mlp.npz)")
    return p


def test_learned_run(gpulib, gpuctx):
    """The learned form runs without step 1, falls back on few groups, and the
    trained network beats the same filter without it."""
    import torch
    params = trained_params()
    W, H, F, sigma = 160, 128, 10, 20.0
    clean, nz, ff, bf = video_case(W, H, F, sigma=sigma, seed=99)
    p1, p2 = resolve_params(gpulib, (W, H, F, 1), sigma, **CFG)
    d = [torch.from_numpy(a).cuda() for a in (nz, ff, bf)]
    _, plain, _ = gpuctx.runNlBayes(*d, p1, p2)
    gpuctx.set_gain_network(params)
    basic, learned, _ = gpuctx.runNlBayes(*d, p1, p2, learned=True)
    groups, fallbacks = gpuctx.learned_stats()
    assert groups > 0 and fallbacks < 0.5 * groups
    learned = learned.cpu().numpy()
    assert np.isfinite(learned).all()
    assert np.array_equal(basic.cpu().numpy(), learned)
    gpuctx.set_gain_network(None)
    _, bare, _ = gpuctx.runNlBayes(*d, p1, p2, learned=True)
    p_plain, p_learned, p_bare = psnr(plain.cpu().numpy(), clean), psnr(learned, clean), psnr(bare.cpu().numpy(), clean)
    print(f"PSNR plain {p_plain:.3f}  learned {p_learned:.3f}  without network {p_bare:.3f}  "
          f"fallback {fallbacks}/{groups}")
    assert p_learned > p_bare + 0.1
    assert p_learned > psnr(nz, clean) + 8.0


def test_learned_rejects_color_and_single_step(gpulib, gpuctx):
    W, H, F = 40, 32, 4
    clean, nz, ff, bf = video_case(W, H, F, sigma=20.0, seed=5, channels=3)
    p1, p2 = resolve_params(gpulib, (W, H, F, 3), 20.0, **CFG)
    with pytest.raises(gpulib.BM4DOFError) as e:
        gpuctx.runNlBayes(nz, ff, bf, p1, p2, learned=True)
    assert e.value.status == "ERR_UNSUPPORTED"
