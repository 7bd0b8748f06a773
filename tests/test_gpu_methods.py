"""GPU parity of SART, SIRT, ASD-POCS and split-Bregman TV through the C ABI.

Tolerance (the path's stated bar): relative L2 error <= 1e-4 after the stated number of
iterations. In COMPAT norm mode every operation, including the host-side
float sums, is the reference's, so results are also required to be equal
bit for bit to the oracle and to the golden fixtures.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

TOL_ITER = 1e-4


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    den = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (den if den > 0 else 1.0)


def _method_proj(ufoir, ctx, step, axis=-1.0):
    return ufoir.ParallelProjector(ctx, step=float(step), axis_position=float(axis), is_forward=0)


# ufoir_sirt_process splits the first and last iterations into slice chunks
# where they meet host data (sinograms arriving, volumes leaving on a side
# stream). Every mix of host and device buffers, slice counts that split
# unevenly and iteration counts 1-3 must give the device path's values, and
# the oracle's.
@pytest.mark.parametrize("slices,iters", [(1, 1), (3, 2), (5, 3), (6, 1), (7, 2)])
@pytest.mark.parametrize("sino_on_host,vol_on_host", [(True, True), (True, False), (False, True)])
def test_sirt_host_buffers_split_iterations(ufoir_lib, gpu_ctx, oracle, slices, iters, sino_on_host,
                                            vol_on_host):
    n, na = 72, 45
    step = np.float32(np.pi / na)
    sinos = np.random.default_rng(slices * 10 + iters).random((slices, na, n), dtype=np.float32) * n
    p = _method_proj(ufoir_lib, gpu_ctx, step)
    d_s = ufoir_lib.DeviceArray.from_numpy(gpu_ctx, sinos)
    d_v = ufoir_lib.DeviceArray(gpu_ctx, (slices, n, n), zero=True)
    ufoir_lib.sirt(p, d_s, d_v, num_iterations=iters, relaxation_factor=0.25)
    want_dev = d_v.download()
    s_arg = sinos if sino_on_host else d_s
    v_out = np.full((slices, n, n), np.nan, np.float32)
    v_arg = v_out if vol_on_host else ufoir_lib.DeviceArray(gpu_ctx, (slices, n, n), zero=True)
    ufoir_lib.sirt(p, s_arg, v_arg, num_iterations=iters, relaxation_factor=0.25)
    got = v_out if vol_on_host else v_arg.download()
    assert np.array_equal(got, want_dev)
    for i in range(slices):
        assert np.array_equal(got[i], oracle.sirt(oracle.projector(n, na, step), sinos[i], iters, 0.25)), i
    if not vol_on_host:
        v_arg.close()
    d_s.close()
    d_v.close()
    p.close()


@pytest.mark.parametrize("n,na,axis,iters,slices", [(16, 12, -1.0, 5, 1), (33, 40, 15.3, 4, 3),
                                                     (64, 90, -1.0, 3, 2), (100, 60, 48.75, 3, 1)])
def test_sirt_matches_oracle(ufoir_lib, gpu_ctx, oracle, n, na, axis, iters, slices):
    rng = np.random.default_rng(n * na)
    step = np.float32(np.pi / na)
    sinos = rng.random((slices, na, n), dtype=np.float32) * n
    p = _method_proj(ufoir_lib, gpu_ctx, step, axis)
    got = ufoir_lib.sirt(p, sinos, num_iterations=iters, relaxation_factor=0.25)
    for i in range(slices):
        want = oracle.sirt(oracle.projector(n, na, step, axis), sinos[i], iters, 0.25)
        assert rel_l2(got[i], want) <= TOL_ITER
        assert np.array_equal(got[i], want), (i, np.abs(got[i] - want).max())
    # the reference leaves relaxation = lambda and correction_scale = -1 on the projector
    assert p.params.relaxation == np.float32(0.25) and p.params.correction_scale == -1.0


def _kernels(monkeypatch, kernels):
    """SART's kernels: "auto" (the padded per-angle kernels where they serve
    the geometry, else the general ones) or "general" (always the general
    per-angle kernels)."""
    if kernels == "auto":
        monkeypatch.delenv("UFOIR_SART_KERNELS", raising=False)
    else:
        monkeypatch.setenv("UFOIR_SART_KERNELS", kernels)


@pytest.mark.parametrize("kernels", ["auto", "general"])
@pytest.mark.parametrize("n,na,axis,iters,slices", [(16, 12, -1.0, 2, 1), (33, 40, 15.3, 2, 2),
                                                     (48, 36, -1.0, 1, 1), (100, 60, -1.0, 1, 2),
                                                     (130, 50, 64.7, 2, 1)])
def test_sart_matches_oracle(ufoir_lib, gpu_ctx, oracle, monkeypatch, kernels, n, na, axis, iters, slices):
    _kernels(monkeypatch, kernels)
    rng = np.random.default_rng(3 * n + na)
    step = np.float32(np.pi / na)
    sinos = rng.random((slices, na, n), dtype=np.float32) * n
    p = _method_proj(ufoir_lib, gpu_ctx, step, axis)
    got = ufoir_lib.sart(p, sinos, num_iterations=iters, relaxation_factor=0.3)
    for i in range(slices):
        want = oracle.sart(oracle.projector(n, na, step, axis), sinos[i], iters, 0.3)
        assert rel_l2(got[i], want) <= TOL_ITER
        assert np.array_equal(got[i], want), (i, np.abs(got[i] - want).max())


# Sizes above 512 detectors split a ray's 64-sample blocks over several CTAs
# of the per-angle forward projection (a cluster whose CTA 0 adds the block
# sums), with a launch shape per size: 16-row segments (n <= 1024), one block
# per warp (1111, 1448, 2900), several blocks per warp (2900 x 2 slices,
# 4100); off-centre axes give inactive detectors and clamped tiles.
@pytest.mark.parametrize("kernels,n,na,axis,iters,slices", [
    ("auto", 513, 24, -1.0, 1, 1), ("auto", 600, 40, 290.6, 2, 2), ("general", 600, 40, 290.6, 2, 2),
    ("auto", 1111, 30, -1.0, 1, 1), ("auto", 1448, 36, 700.25, 1, 1), ("auto", 2900, 12, -1.0, 1, 1),
    ("auto", 2900, 6, 1449.5, 1, 2), ("auto", 4100, 6, -1.0, 1, 1)])
def test_sart_chunked_sizes_match_oracle(ufoir_lib, gpu_ctx, oracle, monkeypatch, kernels, n, na, axis, iters,
                                         slices):
    _kernels(monkeypatch, kernels)
    rng = np.random.default_rng(5 * n + na)
    step = np.float32(np.pi / na)
    sinos = rng.random((slices, na, n), dtype=np.float32) * n
    p = _method_proj(ufoir_lib, gpu_ctx, step, axis)
    got = ufoir_lib.sart(p, sinos, num_iterations=iters, relaxation_factor=0.3)
    for i in range(slices):
        want = oracle.sart(oracle.projector(n, na, step, axis), sinos[i], iters, 0.3)
        assert np.array_equal(got[i], want), (i, np.abs(got[i] - want).max())


# An axis within half a pixel of the image edge crosses the backprojection's
# clamp edges; SART then runs the general per-angle kernels.
@pytest.mark.parametrize("axis", [0.25, 23.8])
def test_sart_crossed_clamp_edges_match_oracle(ufoir_lib, gpu_ctx, oracle, axis):
    n, na = 24, 20
    step = np.float32(np.pi / na)
    sino = np.random.default_rng(77).random((na, n), dtype=np.float32) * n
    p = _method_proj(ufoir_lib, gpu_ctx, step, axis)
    got = ufoir_lib.sart(p, sino, num_iterations=2, relaxation_factor=0.25)
    want = oracle.sart(oracle.projector(n, na, step, axis), sino, 2, 0.25)
    assert np.array_equal(got, want), np.abs(got - want).max()


@pytest.mark.parametrize("kernels", ["auto", "general"])
def test_asdpocs_chunked_size_matches_oracle(ufoir_lib, gpu_ctx, oracle, monkeypatch, kernels):
    _kernels(monkeypatch, kernels)
    n, na = 530, 24
    step = np.float32(np.pi / na)
    vol = np.random.default_rng(23).random((n, n), dtype=np.float32)
    sino = oracle.forward(oracle.projector(n, na, step), vol)
    p = _method_proj(ufoir_lib, gpu_ctx, step)
    got = ufoir_lib.asdpocs(p, sino, num_iterations=2, norm_mode=ufoir_lib.NORM_COMPAT,
                            df_minimizer=dict(num_iterations=2, relaxation_factor=0.25))
    prm = oracle.asdpocs_params(num_iterations=2, sart_iterations=2, norm_mode=oracle.NORM_COMPAT)
    want, _ = oracle.asdpocs(oracle.projector(n, na, step), sino, prm)
    assert np.array_equal(got, want), np.abs(got - want).max()


def test_methods_golden_fixture_compat(ufoir_lib, gpu_ctx):
    d = np.load(os.path.join(GOLDEN, "methods_n20_a18.npz"))
    step = np.float32(d["step"])
    p = _method_proj(ufoir_lib, gpu_ctx, step)
    got = ufoir_lib.asdpocs(p, d["sino"], num_iterations=3, norm_mode=ufoir_lib.NORM_COMPAT,
                            df_minimizer=dict(num_iterations=2, relaxation_factor=0.25))
    assert rel_l2(got, d["asdpocs"]) <= TOL_ITER and np.array_equal(got, d["asdpocs"])
    p2 = _method_proj(ufoir_lib, gpu_ctx, step)
    u = ufoir_lib.sbtv(p2, d["sino"], num_iterations=2, norm_mode=ufoir_lib.NORM_COMPAT, mu=1.0,
                       **{"lambda": 0.05})
    assert rel_l2(u, d["sbtv"]) <= TOL_ITER
    assert np.array_equal(u, d["sbtv"]), np.abs(u - d["sbtv"]).max()
    assert np.float32(gpu_ctx.l1_norm(d["a"], ufoir_lib.NORM_COMPAT)) == d["l1"]
    assert np.float32(gpu_ctx.dot_product(d["a"], d["b"], ufoir_lib.NORM_COMPAT)) == d["dot"]


@pytest.mark.parametrize("mode", ["compat", "fp64"])
def test_asdpocs_matches_oracle(ufoir_lib, gpu_ctx, oracle, mode):
    n, na = 40, 30
    rng = np.random.default_rng(21)
    step = np.float32(np.pi / na)
    vol = rng.random((n, n), dtype=np.float32)
    sino = oracle.forward(oracle.projector(n, na, step), vol)
    m = ufoir_lib.NORM_COMPAT if mode == "compat" else ufoir_lib.NORM_FP64
    om = oracle.NORM_COMPAT if mode == "compat" else oracle.NORM_FP64
    p = _method_proj(ufoir_lib, gpu_ctx, step)
    got = ufoir_lib.asdpocs(p, np.stack([sino, sino * 0.5]), num_iterations=3, norm_mode=m,
                            df_minimizer=dict(num_iterations=2, relaxation_factor=0.25))
    prm = oracle.asdpocs_params(num_iterations=3, sart_iterations=2, norm_mode=om)
    want, _ = oracle.asdpocs(oracle.projector(n, na, step), sino, prm)
    want2, _ = oracle.asdpocs(oracle.projector(n, na, step), sino * 0.5, prm)
    assert rel_l2(got[0], want) <= TOL_ITER and rel_l2(got[1], want2) <= TOL_ITER
    assert np.array_equal(got[0], want) and np.array_equal(got[1], want2)
    wd, _ = oracle.asdpocs_d(oracle.projector(n, na, step), sino, prm)
    assert rel_l2(got[0], wd) < 1e-4       # error against the FP64 recomputation


@pytest.mark.parametrize("mode", ["compat", "fp64"])
def test_sbtv_matches_oracle(ufoir_lib, gpu_ctx, oracle, mode):
    n, na = 32, 24
    rng = np.random.default_rng(33)
    step = np.float32(np.pi / na)
    vol = rng.random((n, n), dtype=np.float32)
    sino = oracle.forward(oracle.projector(n, na, step), vol)
    m = ufoir_lib.NORM_COMPAT if mode == "compat" else ufoir_lib.NORM_FP64
    om = oracle.NORM_COMPAT if mode == "compat" else oracle.NORM_FP64
    p = _method_proj(ufoir_lib, gpu_ctx, step)
    keep = sino.copy()
    got = ufoir_lib.sbtv(p, sino, num_iterations=2, norm_mode=m, mu=1.0, **{"lambda": 0.05})
    assert np.array_equal(sino, keep)        # the caller's sinogram is left untouched
    prm = oracle.sbtv_params(num_iterations=2, lambda_=0.05, mu=1.0, norm_mode=om)
    want, _ = oracle.sbtv(oracle.projector(n, na, step), sino, prm)
    assert rel_l2(got, want) <= TOL_ITER
    if mode == "compat":
        assert np.array_equal(got, want), np.abs(got - want).max()
    # Error against the FP64 recomputation, stated rather than bounded tightly:
    # the reference's CGS (with its partNum * i inner product) follows a
    # different trajectory in double precision; the float and double results
    # of the reference algorithm itself differ by about 6 % after 2 outer
    # iterations here (9e-4 after 1).
    wd = oracle.sbtv_d(oracle.projector(n, na, step), sino, prm)
    err64 = rel_l2(got, wd)
    print(f"sbtv {mode}: rel-L2 vs FP64 recomputation {err64:.3e}")
    assert err64 < 0.1


def test_sbtv_batched_slices_match_single_slice_runs(ufoir_lib, gpu_ctx, oracle):
    # 18 slices run as a batch of 16 and a batch of 2; the slices differ in
    # scale and content, so their CGS runs take different branches and exits,
    # and each must equal the oracle's run of that slice alone
    n, na = 24, 20
    rng = np.random.default_rng(44)
    step = np.float32(np.pi / na)
    op = oracle.projector(n, na, step)
    sinos = np.stack([oracle.forward(op, (rng.random((n, n), dtype=np.float32) ** (1 + i % 4)) * (1 + 3 * i))
                      for i in range(18)])
    p = _method_proj(ufoir_lib, gpu_ctx, step)
    got = ufoir_lib.sbtv(p, sinos, num_iterations=2, norm_mode=ufoir_lib.NORM_COMPAT, mu=1.0,
                         **{"lambda": 0.05})
    prm = oracle.sbtv_params(num_iterations=2, lambda_=0.05, mu=1.0, norm_mode=oracle.NORM_COMPAT)
    for i in range(18):
        want, _ = oracle.sbtv(op, sinos[i], prm)
        assert np.array_equal(got[i], want), (i, float(np.abs(got[i] - want).max()))


def test_norms_match_oracle(ufoir_lib, gpu_ctx, oracle):
    rng = np.random.default_rng(5)
    for h, w in [(1, 1), (7, 13), (64, 64), (300, 257)]:
        a = rng.standard_normal((h, w)).astype(np.float32)
        b = rng.standard_normal((h, w)).astype(np.float32)
        assert np.float32(gpu_ctx.l1_norm(a, ufoir_lib.NORM_COMPAT)) == np.float32(oracle.l1_norm(a))
        assert np.float32(gpu_ctx.dot_product(a, b, ufoir_lib.NORM_COMPAT)) == np.float32(oracle.dot_product(a, b))
        assert abs(gpu_ctx.l1_norm(a) - oracle.l1_norm(a, fp64=True)) <= 1e-6 * oracle.l1_norm(a, fp64=True)
        d64 = oracle.dot_product(a, b, fp64=True)
        assert abs(gpu_ctx.dot_product(a, b) - d64) <= 1e-6 * (abs(d64) + 1)


@pytest.mark.parametrize("kernels", ["auto", "general"])
def test_c1_sart_full_size(ufoir_lib, gpu_ctx, oracle, monkeypatch, kernels):
    # SART on the 367-bin, 180-angle geometry with a 256^2 phantom (2 iterations).
    _kernels(monkeypatch, kernels)
    from ufoir import synth
    n, na = 367, 180
    step = np.float32(np.pi / na)
    vol = synth.ellipse_phantom(n, 256, 10, seed=1001)
    sino = oracle.forward(oracle.projector(n, na, step), vol)
    p = _method_proj(ufoir_lib, gpu_ctx, step)
    got = ufoir_lib.sart(p, sino, num_iterations=2, relaxation_factor=0.25)
    want = oracle.sart(oracle.projector(n, na, step), sino, 2, 0.25)
    assert rel_l2(got, want) <= TOL_ITER and np.array_equal(got, want)


def test_method_argument_errors(ufoir_lib, gpu_ctx):
    p = ufoir_lib.ParallelProjector(gpu_ctx, step=0.1)          # is_forward defaults to TRUE
    sino = np.ones((10, 16), np.float32)
    with pytest.raises(ufoir_lib.UfoirError) as e:
        ufoir_lib.sirt(p, sino)
    assert e.value.status == ufoir_lib.ERR_INVALID
    q = _method_proj(ufoir_lib, gpu_ctx, 0.1)
    with pytest.raises(ufoir_lib.UfoirError):
        ufoir_lib.sirt(q, sino, relaxation_factor=1.5)
    with pytest.raises(ufoir_lib.UfoirError):
        ufoir_lib.sart(q, sino, num_iterations=0)
    with pytest.raises(ufoir_lib.UfoirError):
        ufoir_lib.asdpocs(q, sino, ng=5000)
    out = ufoir_lib.sirt(q, sino, num_iterations=1)
    assert np.isfinite(out).all()


def test_c2_full_size_batched_sirt_iteration_matches_oracle(ufoir_lib, gpu_ctx, oracle):
    # The headline configuration (1448 bins, 1200 angles, 1024^2 ellipse
    # phantom) through the batched, graph-captured path that bench.py times:
    # one SIRT iteration, bit for bit against the oracle (about 1e10 oracle
    # samples, OpenMP over the host cores).
    from ufoir import synth
    n, na = 1448, 1200
    step = np.float32(np.pi / na)
    oracle.set_threads(os.cpu_count() or 1)
    op = oracle.projector(n, na, step)
    sino = oracle.forward(op, synth.ellipse_phantom(n, 1024, 10, seed=2000))
    want = oracle.sirt(op, sino, 1, 0.25)
    p = ufoir_lib.ParallelProjector(gpu_ctx, step=float(step), angles_num=na, is_forward=0)
    d_sino = ufoir_lib.DeviceArray.from_numpy(gpu_ctx, sino[None])
    d_vol = ufoir_lib.DeviceArray(gpu_ctx, (1, n, n), zero=True)
    batch = ufoir_lib.SirtBatch(p, d_sino, d_vol, relaxation_factor=0.25)
    batch.run(1)
    got = d_vol.download()[0]
    batch.close()
    assert rel_l2(got, want) <= TOL_ITER and np.array_equal(got, want)
    d_sino.close()
    d_vol.close()
    p.close()
