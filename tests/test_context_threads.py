"""Calls made on one context from several host threads are serialised by the
library (a lock per context): each thread gets the result of a call made
alone.  ctypes releases the GIL during the calls, so the threads do overlap."""
import threading

import numpy as np
import pytest

from helpers import video_case


@pytest.mark.gpu
def test_gpu_one_context_many_threads(gpulib, gpuctx):
    W, H, F, sigma = 40, 36, 4, 20.0
    cases = [video_case(W, H, F, sigma=sigma, seed=60 + k) for k in range(4)]
    size = (W, H, F, 1)
    p1 = gpulib.initializeNlbParameters(1, sigma, size)
    p2 = gpulib.initializeNlbParameters(2, sigma, size)
    want = [gpuctx.runNlBayes(nz, ff, bf, p1, p2, nparts=2)[1] for _, nz, ff, bf in cases]
    ctx = gpulib.Context(0)
    got, errors = [None] * len(cases), []

    def work(k):
        try:
            _, nz, ff, bf = cases[k]
            for _ in range(3):
                got[k] = ctx.runNlBayes(nz, ff, bf, p1, p2, nparts=2)[1]
        except Exception as e:   # reported below, on the test's thread
            errors.append(e)

    threads = [threading.Thread(target=work, args=(k,)) for k in range(len(cases))]
    for t in threads:
        t.start()
    for t in threads:
        t.join(timeout=300)
    ctx.close()
    assert not errors, errors
    for k in range(len(cases)):
        assert np.array_equal(got[k], want[k]), k
