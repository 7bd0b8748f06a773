"""GPU parity of the projector (FP / BP / process / subsets) through the C ABI.

Tolerance (the path's stated bar): relative L2 error <= 1e-5 after one application.
The kernels follow the reference's operation order exactly, so the tests
also require bit equality with the oracle and the golden fixtures (made by
the reference's own kernel sources) wherever the inputs are identical.
"""
import glob
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

TOL_ONE = 1e-5


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    den = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (den if den > 0 else 1.0)


def _proj(ufoir, ctx, n, na, step, axis=-1.0, **kw):
    p = ufoir.ParallelProjector(ctx, step=float(step), axis_position=float(axis), **kw)
    p.get_requisition((n, na))
    return p


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLDEN, "proj_*.npz"))),
                         ids=lambda p: os.path.basename(p)[:-4])
def test_golden_fixtures(ufoir_lib, gpu_ctx, path):
    d = np.load(path)
    n, na, step, axis = int(d["n"]), int(d["na"]), np.float32(d["step"]), float(d["axis"])
    p = _proj(ufoir_lib, gpu_ctx, n, na, step, axis)
    s, c = p.host_sin_cos()
    assert np.array_equal(s, d["sin"]) and np.array_equal(c, d["cos"])
    assert p.subsets() == [tuple(x) for x in d["subsets"].tolist()]
    sino = p.forward(d["vol"], np.zeros((na, n), np.float32))
    assert rel_l2(sino, d["fp"]) <= TOL_ONE
    assert np.array_equal(sino, d["fp"])
    vol = p.backward(np.zeros((n, n), np.float32), d["fp"])
    assert rel_l2(vol, d["bp"]) <= TOL_ONE
    assert np.array_equal(vol, d["bp"])
    p.set(is_forward=0)
    x = ufoir_lib.sirt(p, d["fp"], num_iterations=int(d["sirt_iters"]))
    assert rel_l2(x, d["sirt"]) <= 1e-4 and np.array_equal(x, d["sirt"])
    x = ufoir_lib.sart(p, d["fp"], num_iterations=int(d["sart_iters"]))
    assert rel_l2(x, d["sart"]) <= 1e-4 and np.array_equal(x, d["sart"])


# the last two put the axis within half a pixel of an image edge, where the
# backprojector's clamp edges cross (e0 > e1)
CASES = [(7, 5, -1.0), (16, 12, -1.0), (33, 40, 15.3), (33, 40, 17.9), (64, 90, -1.0),
         (100, 180, -1.0), (61, 36, 31.25), (128, 7, -1.0), (24, 30, 0.25), (24, 30, 23.8)]


@pytest.mark.parametrize("n,na,axis", CASES)
def test_fp_bp_match_oracle(ufoir_lib, gpu_ctx, oracle, n, na, axis):
    rng = np.random.default_rng(n + 7 * na)
    step = np.float32(np.pi / na)
    vols = rng.random((3, n, n), dtype=np.float32)
    p = _proj(ufoir_lib, gpu_ctx, n, na, step, axis)
    op = oracle.projector(n, na, step, axis)
    # batched (3 slices) accumulate into a non-zero sinogram
    base = rng.random((3, na, n), dtype=np.float32)
    got = p.forward(vols, base.copy())
    for i in range(3):
        want = oracle.forward(op, vols[i], base[i].copy())
        assert rel_l2(got[i], want) <= TOL_ONE
        assert np.array_equal(got[i], want), (i, np.abs(got[i] - want).max())
    vb = rng.random((3, n, n), dtype=np.float32)
    gotb = p.backward(vb.copy(), got)
    for i in range(3):
        want = oracle.backward(op, got[i], vb[i].copy())
        assert np.array_equal(gotb[i], want), (i, np.abs(gotb[i] - want).max())


def test_properties_scale_and_relaxation(ufoir_lib, gpu_ctx, oracle):
    n, na = 40, 30
    step = np.float32(np.pi / na)
    rng = np.random.default_rng(5)
    vol = rng.random((n, n), dtype=np.float32)
    p = _proj(ufoir_lib, gpu_ctx, n, na, step, correction_scale=-0.75, relaxation=0.3)
    op = oracle.projector(n, na, step, -1.0, 0.3, -0.75)
    b = rng.random((na, n), dtype=np.float32)
    assert np.array_equal(p.forward(vol, b.copy()), oracle.forward(op, vol, b.copy()))
    assert np.array_equal(p.backward(vol.copy(), b), oracle.backward(op, b, vol.copy()))


def test_process_forward_and_backward(ufoir_lib, gpu_ctx, oracle):
    n, na = 48, 33
    step = np.float32(np.pi / na)
    rng = np.random.default_rng(9)
    vol = rng.random((n, n), dtype=np.float32)
    p = ufoir_lib.ParallelProjector(gpu_ctx, step=float(step), angles_num=na, is_forward=1)
    sino = p.process(vol)
    assert sino.shape == (na, n)
    op = oracle.projector(n, na, step)
    want = oracle.projector_process(op, True, vol)
    assert np.array_equal(sino, want)
    q = ufoir_lib.ParallelProjector(gpu_ctx, step=float(step), is_forward=0)
    back = q.process(sino)
    assert back.shape == (n, n)
    assert np.array_equal(back, oracle.backward(op, sino))


def test_subset_fp_bp(ufoir_lib, gpu_ctx, oracle):
    import ctypes
    n, na = 36, 24
    step = np.float32(np.pi / na)
    rng = np.random.default_rng(12)
    vol = rng.random((n, n), dtype=np.float32)
    p = _proj(ufoir_lib, gpu_ctx, n, na, step, correction_scale=-1.0, relaxation=0.5)
    s, c = oracle.lut(na, step)
    k = oracle.kernels().contents
    dims = oracle.Dims(n, n, n, na)
    for (off, cnt, direction) in [(3, 1, 1), (8, 5, 0), (0, 2, 1), (20, 4, 1)]:
        sino = rng.random((na, n), dtype=np.float32)
        want = sino.copy()
        k.fp(oracle.image(vol), oracle.image(want), s.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
             c.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), dims, np.float32(n / 2.0),
             oracle.Subset(off, cnt, direction), np.float32(-1.0))
        got = p.subset_fp(vol, sino.copy(), off, cnt, direction)
        assert np.array_equal(got, want)
        v0 = rng.random((n, n), dtype=np.float32)
        wantv = v0.copy()
        k.bp(oracle.image(wantv), oracle.image(sino), np.float32(0.5),
             s.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), c.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
             dims, np.float32(n / 2.0), oracle.Subset(off, cnt, direction))
        gotv = p.subset_bp(v0.copy(), sino, off, cnt, direction)
        assert np.array_equal(gotv, wantv)


def test_device_pointers_and_host_pointers_agree(ufoir_lib, gpu_ctx):
    n, na = 64, 50
    step = np.float32(np.pi / na)
    rng = np.random.default_rng(2)
    vol = rng.random((2, n, n), dtype=np.float32)
    p = _proj(ufoir_lib, gpu_ctx, n, na, step)
    host = p.forward(vol, np.zeros((2, na, n), np.float32))
    dv = ufoir_lib.DeviceArray.from_numpy(gpu_ctx, vol)
    ds = ufoir_lib.DeviceArray(gpu_ctx, (2, na, n), zero=True)
    p.forward(dv, ds)
    assert np.array_equal(ds.download(), host)
    dv.close()
    ds.close()


def test_full_size_geometry_properties(ufoir_lib, gpu_ctx):
    # 1448 bins, 1200 angles over [0, pi): the configuration of the headline metric.
    n, na = 1448, 1200
    step = np.float32(np.pi / na)
    p = _proj(ufoir_lib, gpu_ctx, n, na, step)
    ones = ufoir_lib.DeviceArray.from_numpy(gpu_ctx, np.ones((n, n), np.float32))
    sino = ufoir_lib.DeviceArray(gpu_ctx, (na, n), zero=True)
    p.forward(ones, sino)
    s = sino.download()
    assert np.all(s[0] == n)                     # theta = 0 samples texel centres only
    rng = np.random.default_rng(4)
    a = rng.random((n, n), dtype=np.float32)
    b = rng.random((n, n), dtype=np.float32)
    fa = p.forward(a, np.zeros((na, n), np.float32))
    fb = p.forward(b, np.zeros((na, n), np.float32))
    fab = p.forward(a + b, np.zeros((na, n), np.float32))
    assert rel_l2(fab, fa + fb) < 1e-6          # linearity up to float rounding
    # a slice computed inside a batch equals the slice computed alone, bit for bit
    batch = p.forward(np.stack([b, a]), np.zeros((2, na, n), np.float32))
    assert np.array_equal(batch[1], fa) and np.array_equal(batch[0], fb)
    back = p.backward(np.zeros((n, n), np.float32), np.ones((na, n), np.float32))
    assert np.allclose(back, na, rtol=0, atol=na * 1e-6)
    ones.close()
    sino.close()


def test_row_kernel_serves_sizes_beyond_the_tiled_kernel(ufoir_lib, gpu_ctx):
    # n = 6200 needs more than 768 threads x 8 detectors: the row kernel
    # (one thread per ray, no shared memory) projects it instead.
    n, na = 6200, 4
    p = _proj(ufoir_lib, gpu_ctx, n, na, np.float32(np.pi / na))
    ones = ufoir_lib.DeviceArray.from_numpy(gpu_ctx, np.ones((n, n), np.float32))
    sino = p.forward(ones, np.zeros((na, n), np.float32))
    assert np.all(sino[0] == n)
    assert np.isfinite(sino).all() and sino[2].max() == n   # theta = pi/2: horizontal rays
    ones.close()


def test_full_size_bp_matches_oracle_on_a_row_band(ufoir_lib, gpu_ctx, oracle):
    # C1 geometry in full (367 bins, 180 angles), compared with the oracle.
    n, na = 367, 180
    step = np.float32(np.pi / na)
    rng = np.random.default_rng(8)
    vol = rng.random((n, n), dtype=np.float32)
    p = _proj(ufoir_lib, gpu_ctx, n, na, step)
    op = oracle.projector(n, na, step)
    got = p.forward(vol, np.zeros((na, n), np.float32))
    want = oracle.forward(op, vol)
    assert rel_l2(got, want) <= TOL_ONE and np.array_equal(got, want)
    gb = p.backward(np.zeros((n, n), np.float32), want)
    wb = oracle.backward(op, want)
    assert rel_l2(gb, wb) <= TOL_ONE and np.array_equal(gb, wb)


@pytest.mark.parametrize("n,na,axis,slices", [(1448, 48, -1.0, 1), (1448, 48, 700.3, 1), (1000, 40, -1.0, 3),
                                               (600, 12, -1.0, 1), (1448, 90, 731.6, 1), (2900, 90, -1.0, 1),
                                               (2900, 37, 1420.25, 1)])
def test_fp_with_few_tiles_splits_detectors(ufoir_lib, gpu_ctx, oracle, n, na, axis, slices):
    # few angles on few slices leave most SMs without an angle tile, so each
    # tile's detectors are spread over several CTAs, each staging only the
    # window of columns its rays reach; results must not change
    step = np.float32(np.pi / na)
    rng = np.random.default_rng(n + na + slices)
    vols = rng.random((slices, n, n), dtype=np.float32)
    p = _proj(ufoir_lib, gpu_ctx, n, na, step, axis)
    got = p.forward(vols, np.zeros((slices, na, n), np.float32))
    op = oracle.projector(n, na, step, axis)
    for i in range(slices):
        want = oracle.forward(op, vols[i])
        assert rel_l2(got[i], want) <= TOL_ONE and np.array_equal(got[i], want)


def test_work_queued_on_a_callers_stream(ufoir_lib, gpu_ctx, oracle):
    # another context's stream stands in for a stream the caller owns
    other = ufoir_lib.Context(0)
    s = other.stream()
    n, na = 64, 90
    step = np.float32(np.pi / na)
    vol = np.random.default_rng(9).random((n, n), dtype=np.float32)
    p = _proj(ufoir_lib, gpu_ctx, n, na, step)
    want = oracle.forward(oracle.projector(n, na, step), vol)
    gpu_ctx.set_stream(s)
    try:
        assert gpu_ctx.stream() == s
        got = p.forward(vol, np.zeros((na, n), np.float32))      # host buffers: staged and waited for
        d_vol = ufoir_lib.DeviceArray.from_numpy(gpu_ctx, vol)
        d_sino = ufoir_lib.DeviceArray(gpu_ctx, (na, n), zero=True)
        p.forward(d_vol, d_sino)
        other.synchronize()                                       # the caller orders on its own stream
        got2 = d_sino.download()
        p.set(is_forward=0)
        rec = ufoir_lib.sirt(p, want, num_iterations=2)           # captured iterations on the caller's stream
        d_vol.close()
        d_sino.close()
    finally:
        gpu_ctx.set_stream(None)
    assert gpu_ctx.stream() != s
    assert np.array_equal(got, want) and np.array_equal(got2, want)
    assert np.array_equal(rec, oracle.sirt(oracle.projector(n, na, step), want, 2, 0.25))
    other.close()


def test_errors_are_reported_not_fatal(ufoir_lib, gpu_ctx):
    with pytest.raises(ufoir_lib.UfoirError) as e:
        ufoir_lib.ParallelProjector(gpu_ctx, model="distance-driven")
    assert e.value.status == ufoir_lib.ERR_UNSUPPORTED
    with pytest.raises(ufoir_lib.UfoirError) as e:
        ufoir_lib.ParallelProjector(gpu_ctx, step=-1.0)
    assert e.value.status == ufoir_lib.ERR_INVALID
    p = ufoir_lib.ParallelProjector(gpu_ctx, step=0.1)
    with pytest.raises(ufoir_lib.UfoirError) as e:
        p.subset_fp(np.zeros((8, 8), np.float32), np.zeros((4, 8), np.float32), 0, 1, 1)
    assert e.value.status == ufoir_lib.ERR_STATE
    p.get_requisition((8, 4))
    with pytest.raises(ufoir_lib.UfoirError) as e:
        p.subset_fp(np.zeros((8, 8), np.float32), np.zeros((4, 8), np.float32), 3, 2, 1)
    assert e.value.status == ufoir_lib.ERR_INVALID
    # the context is still usable
    out = p.forward(np.ones((8, 8), np.float32), np.zeros((4, 8), np.float32))
    assert np.isfinite(out).all()


def test_sample_ceilings_are_measured(gpu_ctx):
    # each projector's per-sample sequence from shared memory: some 1e12
    # samples/s on a GB300, the backprojector's close to the forward one's
    fp = gpu_ctx.sample_ceiling()
    bp = gpu_ctx.sample_ceiling_bp()
    assert 1e11 < fp < 1e14 and 1e11 < bp < 1e14
    assert 0.5 < bp / fp < 2.0



# ---- the "siddon" model: exact line integrals of the pixel image ----

# Tiny and odd sizes (rays mostly at the image border), 4 angles (one at
# exactly 45 degrees, where the walk direction is decided by the float LUT),
# off-centre axes, several slices, and the full C2 width.
@pytest.mark.parametrize("n,na,axis,slices", [(5, 3, -1.0, 1), (7, 4, 2.2, 3), (64, 30, -1.0, 1),
                                               (100, 45, 47.3, 2), (367, 180, -1.0, 1), (1448, 24, 731.6, 1)])
def test_siddon_fp_bp_match_oracle(ufoir_lib, gpu_ctx, oracle, n, na, axis, slices):
    step = np.float32(np.pi / na)
    rng = np.random.default_rng(n * na + slices)
    vols = rng.random((slices, n, n), dtype=np.float32)
    sinos = rng.random((slices, na, n), dtype=np.float32)
    p = _proj(ufoir_lib, gpu_ctx, n, na, step, axis, model="Siddon")
    assert p.params.model == b"siddon"
    got = p.forward(vols, np.zeros((slices, na, n), np.float32))
    back = p.backward(np.zeros((slices, n, n), np.float32), sinos)
    for i in range(slices):
        assert rel_l2(got[i], oracle.siddon_forward(n, na, step, vols[i], axis)) <= TOL_ONE
        assert rel_l2(back[i], oracle.siddon_backward(n, na, step, sinos[i], axis)) <= TOL_ONE
    p.close()


def test_siddon_projection_of_ones_is_the_chord(ufoir_lib, gpu_ctx, oracle):
    n, na = 256, 37
    step = np.float32(np.pi / na)
    p = _proj(ufoir_lib, gpu_ctx, n, na, step, 120.4, model="siddon")
    got = p.forward(np.ones((n, n), np.float32), np.zeros((na, n), np.float32))
    want = oracle.siddon_chords(n, na, step, 120.4)
    assert np.abs(got - want).max() <= 1e-4 * n
    assert rel_l2(got, want) <= TOL_ONE


# <A x, y> = <x, A^T y>: a property of any size, here also the full
# 1448^2 x 1200 geometry with an off-centre axis.
@pytest.mark.parametrize("n,na,axis", [(200, 60, -1.0), (1448, 1200, 731.6)])
def test_siddon_backprojector_is_the_adjoint(ufoir_lib, gpu_ctx, n, na, axis):
    step = np.float32(np.pi / na)
    rng = np.random.default_rng(5)
    x = rng.random((n, n), dtype=np.float32)
    y = rng.random((na, n), dtype=np.float32)
    p = _proj(ufoir_lib, gpu_ctx, n, na, step, axis, model="siddon")
    ax = p.forward(x, np.zeros((na, n), np.float32)).astype(np.float64)
    aty = p.backward(np.zeros((n, n), np.float32), y).astype(np.float64)
    lhs, rhs = float((ax * y).sum()), float((x * aty).sum())
    assert abs(lhs - rhs) <= 1e-5 * abs(lhs)


def test_siddon_subsets_and_scale(ufoir_lib, gpu_ctx, oracle):
    n, na = 80, 20
    step = np.float32(np.pi / na)
    rng = np.random.default_rng(9)
    vol = rng.random((n, n), dtype=np.float32)
    sino0 = rng.random((na, n), dtype=np.float32)
    p = _proj(ufoir_lib, gpu_ctx, n, na, step, model="siddon", correction_scale=-1.0, relaxation=0.5)
    off, cnt, drn = (int(v) for v in p.subsets()[0])
    got = p.subset_fp(vol, sino0.copy(), off, cnt, drn)
    full = oracle.siddon_forward(n, na, step, vol)
    want = sino0.astype(np.float64).copy()
    rows = slice(off, off + cnt)
    want[rows] = sino0[rows] - full[rows]
    assert rel_l2(got, want) <= TOL_ONE
    base = rng.random((n, n), dtype=np.float32)
    only = np.zeros_like(sino0)
    only[rows] = sino0[rows]
    got_b = p.subset_bp(base.copy(), sino0, off, cnt, drn)
    want_b = base + 0.5 * oracle.siddon_backward(n, na, step, only)
    assert rel_l2(got_b, want_b) <= TOL_ONE


def test_methods_need_the_joseph_model(ufoir_lib, gpu_ctx):
    p = ufoir_lib.ParallelProjector(gpu_ctx, step=0.1, is_forward=0, model="siddon")
    with pytest.raises(ufoir_lib.UfoirError) as e:
        ufoir_lib.sirt(p, np.ones((10, 16), np.float32))
    assert e.value.status == ufoir_lib.ERR_UNSUPPORTED and "Joseph" in str(e.value)
