#!/usr/bin/env python
"""Training of the learned form's gain network on the GPU.

    python bm4d-of_gb300/train_gains.py [--clips 2000] [--epochs 12] [--out FILE]
                                        [--checkpoint FILE [--resume]]

Training pairs come from the plain two-step method itself: each seeded
synthetic grey clip (64x64x8, sigma uniform in [5, 50], the cosine+rectangle
texture with global translation, moving rectangles and exact flow) is
denoised by the plain GPU path (bm4dof_run); bm4dof_gain_samples then
searches the learned form's groups on the noisy clip and pairs their network
inputs with the step-2 Wiener gains of the member-mean row computed from that
basic estimate.  The network is trained with the library's BF16 forward,
backward and AdamW kernels (bm4dof_trainer_*), cosine learning-rate decay, and
saved as a float32 blob (BM4DOF_GAIN_PARAMS values, bm4dof.split_params
layout) in an .npz together with its training record.

With --checkpoint the trainer's parameters and AdamW state, the epoch count,
the losses so far and the best validation epoch's parameters are written to
FILE after every epoch, as one file renamed into place (Trainer.checkpoint);
--resume restores them and continues with the next epoch (the shuffles of the
finished epochs are replayed, so the run takes the steps an uninterrupted one
would have taken).  It refuses a checkpoint of a run with other data, batch,
seed or epoch count.

The last 5 % of the clips are held out for the validation loss.  The record
also holds PSNR on a held-out 256x256x12 clip at sigma 20: plain method,
learned form with the network, and learned form without it.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import bm4dof  # noqa: E402
import synthetic  # noqa: E402

WEIGHTS = os.path.join(HERE, "weights", "gain_mlp.npz")
CLI = dict(px1=4, px2=4, pt1=4, pt2=4, wx1=21, wx2=21, np1=16, np2=16, b1=3.0)


def load_weights(path=WEIGHTS):
    """The trained parameter blob, or None when the file is absent."""
    if not os.path.exists(path):
        return None
    with np.load(path) as z:
        return np.array(z["params"], np.float32)


def clip(W, H, F, sigma, seed):
    clean, ff, bf = synthetic.video(W, H, F, seed)
    nz = synthetic.noisy(clean, sigma, seed)
    return clean, nz, ff, bf


def make_dataset(ctx, clips, seed, W=64, H=64, F=8, sig=(5.0, 50.0)):
    import torch
    feats, tgts = [], []
    rng = np.random.default_rng(seed)
    sigmas = rng.uniform(sig[0], sig[1], clips)
    for i in range(clips):
        s = float(sigmas[i])
        _, nz, ff, bf = clip(W, H, F, s, 1_000_003 * seed + i)
        d_nz, d_ff, d_bf = (torch.from_numpy(a).cuda() for a in (nz, ff, bf))
        p1, p2 = bm4dof.cli_params((W, H, F, 1), s, **CLI)
        basic, _, _ = ctx.runNlBayes(d_nz, d_ff, d_bf, p1, p2)
        f, t = ctx.gain_samples(d_nz, basic, d_ff, d_bf, p2)
        feats.append(f)
        tgts.append(t)
    return feats, tgts


def evaluate(ctx, params, W=256, H=256, F=12, sigma=20.0, seed=424242, kappa=0.0):
    """PSNR of plain, learned (network) and learned (no network) on one clip."""
    import torch
    clean, nz, ff, bf = clip(W, H, F, sigma, seed)
    d = [torch.from_numpy(a).cuda() for a in (nz, ff, bf)]
    p1, p2 = bm4dof.cli_params((W, H, F, 1), sigma, **CLI)
    psnr = lambda a: float(10 * np.log10(255.0 ** 2 / np.mean((a.cpu().numpy().astype(np.float64) - clean) ** 2)))
    out = {}
    _, fin, _ = ctx.runNlBayes(*d, p1, p2)
    out["plain_db"] = psnr(fin)
    ctx.set_gain_network(params, kappa)
    _, fin, _ = ctx.runNlBayes(*d, p1, p2, learned=True)
    g, fb = ctx.learned_stats()
    out["learned_db"] = psnr(fin)
    out["learned_fallback_frac"] = fb / max(g, 1)
    ctx.set_gain_network(None, kappa)
    _, fin, _ = ctx.runNlBayes(*d, p1, p2, learned=True)
    out["no_network_db"] = psnr(fin)
    return out


def train(feat, tgt, epochs, batch, lr, wd, seed, val=None, log=print, checkpoint=None, resume=False):
    """AdamW with cosine decay; returns the trainer holding the parameters of
    the epoch with the lowest validation loss (the last epoch without val).
    checkpoint: file written after every epoch (trainer state, run record and
    best-epoch parameters in one atomically replaced file); resume: continue
    from it.  A checkpoint of another run (other sample count, batch, seed or
    epoch count) or one whose AdamW step count disagrees with its epoch count
    is refused."""
    import torch
    tr = bm4dof.Trainer(batch=batch, seed=seed)
    n = feat.shape[0]
    gen = torch.Generator().manual_seed(seed)
    per_epoch = max(1, n // batch)
    total = epochs * per_epoch
    run = {"samples": int(n), "batch": int(batch), "seed": int(seed), "epochs": int(epochs),
           "per_epoch": int(per_epoch)}
    step = 0
    history, vhist = [], []
    best = (float("inf"), None)
    start = 0
    if checkpoint and resume and os.path.exists(checkpoint):
        ck = tr.restore(checkpoint)
        meta = ck["meta"]
        if meta is None or meta.get("run") != run:
            raise ValueError(f"{checkpoint}: written by another training run "
                             f"({None if meta is None else meta.get('run')} vs {run})")
        start, history, vhist = meta["epochs_done"], meta["train_loss"], meta["val_loss_per_epoch"]
        if ck["steps"] != start * per_epoch:
            raise ValueError(f"{checkpoint}: {ck['steps']} AdamW steps after {start} epochs of {per_epoch}")
        if meta.get("best_val") is not None:
            best = (meta["best_val"], ck["best"])
        step = start * per_epoch
        for _ in range(start):
            torch.randperm(n, generator=gen)     # the shuffles of the finished epochs
        log(f"resumed after epoch {start - 1}")
    for e in range(start, epochs):
        perm = torch.randperm(n, generator=gen).cuda()
        losses = []
        for s in range(per_epoch):
            idx = perm[s * batch:(s + 1) * batch]
            lr_t = lr * 0.5 * (1.0 + math.cos(math.pi * step / total))
            want = s % 50 == 0
            l = tr.step(feat[idx].contiguous(), tgt[idx].contiguous(), lr_t, wd, want_loss=want)
            if want:
                losses.append(l)
            step += 1
        history.append(float(np.mean(losses)))
        msg = f"epoch {e}: train loss {history[-1]:.5f}"
        if val is not None:
            vl = val_loss(tr, *val)
            vhist.append(vl)
            msg += f"  validation {vl:.5f}"
            if vl < best[0]:
                best = (vl, tr.params())
        if checkpoint:
            tr.checkpoint(checkpoint, meta={"run": run, "epochs_done": e + 1, "train_loss": history,
                                            "val_loss_per_epoch": vhist,
                                            "best_val": None if best[1] is None else best[0]},
                          best=best[1])
        log(msg)
    if best[1] is not None:
        tr.set_params(best[1])
    return tr, history, vhist


def val_loss(tr, feat, tgt):
    tot, cnt = 0.0, 0
    for s in range(0, feat.shape[0], tr.batch):
        f, t = feat[s:s + tr.batch].contiguous(), tgt[s:s + tr.batch].contiguous()
        _, l = tr.grad(f, t)
        tot += l * f.shape[0]
        cnt += f.shape[0]
    return tot / max(cnt, 1)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--clips", type=int, default=2000)
    ap.add_argument("--epochs", type=int, default=10)
    ap.add_argument("--batch", type=int, default=8192)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--wd", type=float, default=1e-4)
    ap.add_argument("--seed", type=int, default=7)
    ap.add_argument("--out", default=WEIGHTS)
    ap.add_argument("--checkpoint", default=None, help="trainer checkpoint written after every epoch")
    ap.add_argument("--resume", action="store_true", help="continue from --checkpoint")
    args = ap.parse_args()
    import torch
    t0 = time.time()
    ctx = bm4dof.Context(0)
    feats, tgts = make_dataset(ctx, args.clips, args.seed)
    nval = max(1, args.clips // 20)
    ftr, ttr = torch.cat(feats[:-nval]), torch.cat(tgts[:-nval])
    fva, tva = torch.cat(feats[-nval:]), torch.cat(tgts[-nval:])
    t1 = time.time()
    print(f"dataset: {ftr.shape[0]} train / {fva.shape[0]} validation pairs in {t1 - t0:.1f} s", flush=True)
    tr, hist, vhist = train(ftr, ttr, args.epochs, args.batch, args.lr, args.wd, args.seed, val=(fva, tva),
                            checkpoint=args.checkpoint, resume=args.resume)
    t2 = time.time()
    params = tr.params()
    record = {
        "clips": args.clips, "clip": "64x64x8, sigma U[5,50]", "pairs_train": int(ftr.shape[0]),
        "pairs_val": int(fva.shape[0]), "epochs": args.epochs, "batch": args.batch, "lr": args.lr,
        "weight_decay": args.wd, "seed": args.seed, "train_loss": hist, "val_loss_per_epoch": vhist,
        "val_loss": val_loss(tr, fva, tva), "dataset_s": t1 - t0, "train_s": t2 - t1,
    }
    record["eval"] = evaluate(ctx, params)
    os.makedirs(os.path.dirname(os.path.abspath(args.out)), exist_ok=True)
    np.savez(args.out, params=params, record=json.dumps(record))
    print(json.dumps(record), flush=True)


if __name__ == "__main__":
    main()
