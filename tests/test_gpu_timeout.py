"""The device-side bounded waits, made to run out on purpose, on the host's
say-so and without a fault.

The tiled forward projector stages image rows in shared memory with bulk
copies tracked by mbarriers; every wait on them gives up after 250 ms,
records the timeout in the kernel error word, drains the copies it issued
and returns, and the host turns the word into UFOIR_ERR_TIMEOUT. Here the
host asks one launch to announce more bytes for one chunk's barrier than its
copy brings (ufoir_ctx_inject_copy_timeout), so the barrier never completes
and every CTA's wait on it runs out. The call
must fail with UFOIR_ERR_TIMEOUT within seconds, and the same context must
then give the oracle's result bit for bit. (The reference only logs OpenCL
errors and continues, src/core/ufo-ir-basic-ops.c:60-64.)
"""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("chunk", [0, 1, 3])
def test_fp_copy_timeout_is_reported_and_context_recovers(ufoir_lib, gpu_ctx, oracle, chunk):
    n, na = 256, 64
    step = np.float32(np.pi / na)
    vol = np.random.default_rng(chunk + 11).random((n, n), dtype=np.float32)
    want = oracle.forward(oracle.projector(n, na, step), vol)
    p = ufoir_lib.ParallelProjector(gpu_ctx, step=float(step), angles_num=na, is_forward=1)
    assert np.array_equal(p.forward(vol, np.zeros((na, n), np.float32)), want)

    assert ufoir_lib.lib().ufoir_ctx_inject_copy_timeout(gpu_ctx.handle, chunk) == ufoir_lib.OK
    t0 = time.perf_counter()
    with pytest.raises(ufoir_lib.UfoirError) as e:
        p.forward(vol, np.zeros((na, n), np.float32))
    elapsed = time.perf_counter() - t0
    assert e.value.status == ufoir_lib.ERR_TIMEOUT, str(e.value)
    assert "gave up waiting" in str(e.value)
    assert 0.2 < elapsed < 10.0, elapsed      # the 250 ms limit ran out, and nothing hung

    # one-shot: the next call runs normally on the same context
    assert np.array_equal(p.forward(vol, np.zeros((na, n), np.float32)), want)
    got = ufoir_lib.sirt(ufoir_lib.ParallelProjector(gpu_ctx, step=float(step), is_forward=0),
                         want, num_iterations=2)
    assert np.array_equal(got, oracle.sirt(oracle.projector(n, na, step), want, 2, 0.25))
    p.close()


def test_inject_copy_timeout_argument_checks(ufoir_lib, gpu_ctx):
    L = ufoir_lib.lib()
    assert L.ufoir_ctx_inject_copy_timeout(None, 0) == ufoir_lib.ERR_INVALID
    assert L.ufoir_ctx_inject_copy_timeout(gpu_ctx.handle, -2) == ufoir_lib.ERR_INVALID
    assert L.ufoir_ctx_inject_copy_timeout(gpu_ctx.handle, 5) == ufoir_lib.OK
    assert L.ufoir_ctx_inject_copy_timeout(gpu_ctx.handle, -1) == ufoir_lib.OK    # cancelled
