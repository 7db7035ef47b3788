"""Checkpoint and resume of the gain network's training (bm4dof_trainer_state,
Trainer.checkpoint / restore): the file format on the CPU, and on the GPU a
run stopped, saved and restored in a new trainer ending with the parameters of
the run that never stopped."""
import numpy as np
import pytest


def test_checkpoint_file_round_trip(gpulib, tmp_path):
    rng = np.random.default_rng(3)
    n = gpulib.GAIN_PARAMS
    p, m1, m2 = (rng.normal(size=n).astype(np.float32) for _ in range(3))
    m2 = np.abs(m2)
    path = tmp_path / "ck.npz"
    gpulib.save_checkpoint(path, p, m1, m2, 1234, batch=512)
    ck = gpulib.load_checkpoint(path)
    assert np.array_equal(ck["params"], p) and np.array_equal(ck["moment1"], m1)
    assert np.array_equal(ck["moment2"], m2) and ck["steps"] == 1234 and ck["batch"] == 512
    assert ck["meta"] is None and ck["best"] is None
    gpulib.save_checkpoint(path, p, m1, m2, 7, batch=8, meta={"epochs_done": 2, "loss": [0.5, 0.25]}, best=m1)
    ck = gpulib.load_checkpoint(path)
    assert ck["meta"] == {"epochs_done": 2, "loss": [0.5, 0.25]} and np.array_equal(ck["best"], m1)
    assert not (tmp_path / "ck.npz.tmp").exists()      # written aside, then renamed into place
    with pytest.raises(ValueError, match="floats each"):
        gpulib.save_checkpoint(path, p[:-1], m1, m2, 1)
    assert gpulib.load_checkpoint(path)["steps"] == 7   # a refused write leaves the last checkpoint
    np.savez(tmp_path / "old.npz", version=np.array(0), params=p, moment1=m1, moment2=m2,
             steps=np.array(1, np.uint64), batch=np.array(0, np.uint64))
    with pytest.raises(ValueError, match="checkpoint version 0"):
        gpulib.load_checkpoint(tmp_path / "old.npz")


@pytest.mark.gpu
def test_gpu_training_resumes_exactly(gpulib, gpuctx, tmp_path):
    import torch
    rng = np.random.default_rng(4)
    batch, steps, stop = 512, 8, 3
    feats = [torch.from_numpy(rng.normal(0, 1, (batch, 65)).astype(np.float32)).cuda() for _ in range(steps)]
    tgts = [torch.from_numpy(rng.uniform(0, 1, (batch, 64)).astype(np.float32)).cuda() for _ in range(steps)]
    lr = lambda s: 2e-3 * (1.0 - s / steps)

    whole = gpulib.Trainer(batch=batch, seed=11)
    for s in range(steps):
        whole.step(feats[s], tgts[s], lr(s), 1e-4, want_loss=False)

    first = gpulib.Trainer(batch=batch, seed=11)
    for s in range(stop):
        first.step(feats[s], tgts[s], lr(s), 1e-4, want_loss=False)
    first.checkpoint(tmp_path / "ck.npz")
    m1, m2, n = first.state()
    assert n == stop and np.any(m1 != 0) and np.all(m2 >= 0)
    first.close()

    second = gpulib.Trainer(batch=batch, seed=99)      # other initial weights, all replaced
    second.restore(tmp_path / "ck.npz")
    for s in range(stop, steps):
        second.step(feats[s], tgts[s], lr(s), 1e-4, want_loss=False)
    assert np.array_equal(second.params(), whole.params())
    assert second.state()[2] == steps


@pytest.mark.gpu
def test_gpu_train_resume_matches_uninterrupted(gpulib, gpuctx, tmp_path):
    # train_gains.train: a run stopped after its second epoch's checkpoint and
    # resumed from it ends with the parameters, losses and best epoch of the
    # run that never stopped; a checkpoint of another run is refused
    import torch
    import train_gains
    rng = np.random.default_rng(8)
    n, batch, epochs = 2048, 512, 3
    feat = torch.from_numpy(rng.normal(0, 1, (n, 65)).astype(np.float32)).cuda()
    tgt = torch.from_numpy(rng.uniform(0, 1, (n, 64)).astype(np.float32)).cuda()
    val = (feat[:512].contiguous(), tgt[:512].contiguous())
    quiet = lambda msg: None
    whole, hist, vhist = train_gains.train(feat, tgt, epochs, batch, 2e-3, 1e-4, 5, val=val, log=quiet)

    class Stop(Exception):
        pass

    def stop_after_second(msg):
        if msg.startswith("epoch 1:"):
            raise Stop()
    ck = str(tmp_path / "train.npz")
    with pytest.raises(Stop):
        train_gains.train(feat, tgt, epochs, batch, 2e-3, 1e-4, 5, val=val, log=stop_after_second, checkpoint=ck)
    assert gpulib.load_checkpoint(ck)["meta"]["epochs_done"] == 2
    again, hist2, vhist2 = train_gains.train(feat, tgt, epochs, batch, 2e-3, 1e-4, 5, val=val, log=quiet,
                                             checkpoint=ck, resume=True)
    assert np.array_equal(again.params(), whole.params())
    assert hist2 == hist and vhist2 == vhist
    with pytest.raises(ValueError, match="another training run"):
        train_gains.train(feat, tgt, epochs + 1, batch, 2e-3, 1e-4, 5, val=val, log=quiet, checkpoint=ck,
                          resume=True)
