"""Host-side fault injection of allocation failures (bm4dof_set_memory_limit):
a cap below what a run needs makes it fail with BM4DOF_ERR_NO_MEMORY and a
message naming the buffer, the context stays usable, and under a cap that
leaves room the output is the one without a cap (the smaller chunk budget
changes the chunking, not the ordered sums)."""
import numpy as np
import pytest

from helpers import video_case


@pytest.mark.gpu
def test_gpu_memory_limit_fails_cleanly_and_the_context_recovers(gpulib, gpuctx):
    W, H, F, sigma = 48, 40, 4, 20.0
    clean, nz, ff, bf = video_case(W, H, F, sigma=sigma, seed=29)
    size = (W, H, F, 1)
    p1 = gpulib.initializeNlbParameters(1, sigma, size)
    p2 = gpulib.initializeNlbParameters(2, sigma, size)
    want_b, want_f, _ = gpuctx.runNlBayes(nz, ff, bf, p1, p2, nparts=2)
    ctx = gpulib.Context(0)
    try:
        ctx.set_memory_limit(64 << 10)
        with pytest.raises(gpulib.BM4DOFError, match="device memory limit of 65536 bytes reached") as e:
            ctx.runNlBayes(nz, ff, bf, p1, p2, nparts=2)
        assert e.value.code == 10        # BM4DOF_ERR_NO_MEMORY
        ctx.set_memory_limit(256 << 20)
        b, f, _ = ctx.runNlBayes(nz, ff, bf, p1, p2, nparts=2)
        assert np.array_equal(b, want_b) and np.array_equal(f, want_f)
        ctx.set_memory_limit(0)
        b, f, _ = ctx.runNlBayes(nz, ff, bf, p1, p2, nparts=2)
        assert np.array_equal(b, want_b) and np.array_equal(f, want_f)
    finally:
        ctx.close()
