"""The allocation-free L1-norm entry point, through the C ABI.

ufoir_l1_norm_fp64_noalloc is for callers that must not allocate device
memory where they need the norm (their GPU memory is owned by another
allocator or held to a hard per-process limit, or they run loops that must
not take the allocator's locks). It keeps its partial sums in a fixed
device array, so these checks run it twice in a row (the second call reuses
the array that the first call filled) and compare each result with the
allocating ufoir_l1_norm in FP64 mode. This file is collected last so that a failure
here comes after every other test has run; it also passes on its own.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_SLICES = 64   # UFOIR_NOALLOC_MAX_SLICES in include/ufoir.h


def _entry(ufoir_lib):
    f = ufoir_lib.lib().ufoir_l1_norm_fp64_noalloc
    f.argtypes = [C.c_void_p, C.c_size_t, C.c_uint, C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    return f


def test_noalloc_l1_matches_allocating_entry_point_twice(ufoir_lib, gpu_ctx):
    f = _entry(ufoir_lib)
    rng = np.random.default_rng(77)
    for call, (slices, h, w) in enumerate([(5, 300, 257), (3, 1448, 1448)]):
        data = (rng.standard_normal((slices, h, w)) * (call + 1)).astype(np.float32)
        d_in = ufoir_lib.DeviceArray.from_numpy(gpu_ctx, data)
        d_out = ufoir_lib.DeviceArray(gpu_ctx, (slices,))
        rc = f(d_in.ptr, h * w, slices, d_out.ptr, gpu_ctx.stream())
        assert rc == ufoir_lib.OK
        gpu_ctx.synchronize()
        got = d_out.download()
        for s in range(slices):
            want = gpu_ctx.l1_norm(data[s], ufoir_lib.NORM_FP64)
            assert abs(float(got[s]) - want) <= 1e-6 * abs(want), (call, s, got[s], want)
            assert np.float32(got[s]) == np.float32(want)
        d_in.close()
        d_out.close()


def test_noalloc_rejects_sizes_beyond_its_scratch(ufoir_lib, gpu_ctx):
    f = _entry(ufoir_lib)
    d_in = ufoir_lib.DeviceArray(gpu_ctx, (MAX_SLICES + 1, 4), zero=True)
    d_out = ufoir_lib.DeviceArray(gpu_ctx, (MAX_SLICES + 1,), zero=True)
    assert f(d_in.ptr, 4, MAX_SLICES + 1, d_out.ptr, gpu_ctx.stream()) == ufoir_lib.ERR_INVALID
    assert f(None, 4, 1, d_out.ptr, gpu_ctx.stream()) == ufoir_lib.ERR_INVALID
    assert f(d_in.ptr, 4, MAX_SLICES, d_out.ptr, gpu_ctx.stream()) == ufoir_lib.OK
    gpu_ctx.synchronize()
    assert np.all(d_out.download()[:MAX_SLICES] == 0.0)
    d_in.close()
    d_out.close()
