"""GPU parity of ASD-POCS's TV steepest-descent stage through the C ABI.

The reference copies its output before the TV sub-steps of each outer
iteration (src/tasks/ufo-ir-asdpocs-task.c:468) and SART restarts from zero
(src/tasks/ufo-ir-sart-task.c:207), so ASD-POCS's returned volume never
depends on the TV stage. These tests look at what does: the TV subgradient
kernel l1_grad (src/kernels/ufo-math-tvstd-method.cl:5-57) on its own, and the
iterate after the last outer iteration's 20 TV sub-steps together with the
scalars dp, dd, dg and dtgv (ufoir_asdpocs_process_ex), with enough outer
iterations that the dtgv reduction (:501-503) is both taken and skipped.

Tolerance: bit-exact in COMPAT norm mode (float sequential host sums, the
reference's arithmetic); relative L2 <= 1e-4 in FP64 norm mode, whose sums
are double and so may round differently from the oracle's double sums in the
last float bit of a step size. The error of the FP64 mode against the
oracle's FP64 twin is stated beside the reference arithmetic's own, which it
must not exceed by more than 5 %.
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


def oracle_grad(oracle, a):
    g = np.zeros_like(a)
    oracle.kernels("port").contents.l1_grad(oracle.image(a), oracle.image(g))
    return g


def test_tv_gradient_golden(ufoir_lib, gpu_ctx):
    d = np.load(os.path.join(GOLDEN, "tv_n40_a30.npz"))
    keys = [k[len("g_in_"):] for k in d.files if k.startswith("g_in_")]
    assert {"row_1x57", "col_57x1", "const_40x40", "step_40x40", "rand_1x1"} <= set(keys)
    for k in keys:
        got = ufoir_lib.tv_gradient(gpu_ctx, d["g_in_" + k])
        assert np.array_equal(got, d["g_out_" + k]), (k, np.abs(got - d["g_out_" + k]).max())


@pytest.mark.parametrize("slices,h,w", [(3, 45, 61), (2, 1, 300), (2, 300, 1), (1, 31, 33), (1, 530, 530),
                                        (1, 2900, 2900)])
def test_tv_gradient_matches_oracle(ufoir_lib, gpu_ctx, oracle, slices, h, w):
    rng = np.random.default_rng(slices * 7919 + h * 31 + w)
    a = (rng.standard_normal((slices, h, w)) * 2).astype(np.float32)
    a[0, : h // 2, : w // 3] = 1.25          # a constant patch: zero differences inside it
    got = ufoir_lib.tv_gradient(gpu_ctx, a)
    for s in range(slices):
        want = oracle_grad(oracle, np.ascontiguousarray(a[s]))
        assert np.array_equal(got[s], want), (s, np.abs(got[s] - want).max())


def test_tv_gradient_device_arrays(ufoir_lib, gpu_ctx, oracle):
    a = np.random.default_rng(5).random((2, 64, 96), dtype=np.float32)
    d_in = ufoir_lib.DeviceArray.from_numpy(gpu_ctx, a)
    d_out = ufoir_lib.DeviceArray(gpu_ctx, a.shape, zero=True)
    ufoir_lib.tv_gradient(gpu_ctx, d_in, d_out)
    got = d_out.download()
    for s in range(2):
        assert np.array_equal(got[s], oracle_grad(oracle, np.ascontiguousarray(a[s])))
    d_in.close()
    d_out.close()


def _proj(ufoir, ctx, step):
    return ufoir.ParallelProjector(ctx, step=float(step), is_forward=0)


def test_asdpocs_tv_state_golden(ufoir_lib, gpu_ctx):
    d = np.load(os.path.join(GOLDEN, "tv_n40_a30.npz"))
    p = _proj(ufoir_lib, gpu_ctx, d["step"])
    vol, x_tv, sc = ufoir_lib.asdpocs_state(p, d["sino"], num_iterations=int(d["outer"]),
                                            norm_mode=ufoir_lib.NORM_COMPAT,
                                            df_minimizer=dict(num_iterations=int(d["sart_iterations"]),
                                                              relaxation_factor=0.25))
    assert np.array_equal(vol, d["asdpocs"])
    assert np.array_equal(x_tv, d["asdpocs_x"]), np.abs(x_tv - d["asdpocs_x"]).max()
    got = np.array([sc[0]["dp"], sc[0]["dd"], sc[0]["dg"], sc[0]["dtgv"]], np.float32)
    assert np.array_equal(got, d["scalars"]), (got, d["scalars"])


def _noisy_sino(oracle, n, na, seed):
    from ufoir import synth
    step = np.float32(np.pi / na)
    vol = synth.phantom_for(n, max(8, int(0.7 * n)), "polygons", seed=seed)
    clean = oracle.forward(oracle.projector(n, na, step), vol)
    sino, _ = synth.poisson_noise(clean, 1e4, seed=seed + 1)
    return step, sino


# 40^2 and 530^2 with two slices, 2900^2 x 90 angles (the sparse-view ASD-POCS
# geometry) with one; 4-5 outer iterations, 2 inner SART iterations each
@pytest.mark.parametrize("mode", ["compat", "fp64"])
@pytest.mark.parametrize("n,na,outer,slices", [(40, 30, 5, 2), (530, 24, 4, 2), (2900, 90, 4, 1)])
def test_asdpocs_tv_state_matches_oracle(ufoir_lib, gpu_ctx, oracle, mode, n, na, outer, slices):
    if n == 2900 and mode == "fp64":
        pytest.skip("2900^2 runs in COMPAT mode only (the FP64 twin at that size takes minutes on the host)")
    steps, sinos = zip(*[_noisy_sino(oracle, n, na, 40 + s) for s in range(slices)])
    step = steps[0]
    sinos = np.stack(sinos)
    m = ufoir_lib.NORM_COMPAT if mode == "compat" else ufoir_lib.NORM_FP64
    om = oracle.NORM_COMPAT if mode == "compat" else oracle.NORM_FP64
    p = _proj(ufoir_lib, gpu_ctx, step)
    vol, x_tv, sc = ufoir_lib.asdpocs_state(p, sinos, num_iterations=outer, norm_mode=m,
                                            df_minimizer=dict(num_iterations=2, relaxation_factor=0.25))
    prm = oracle.asdpocs_params(num_iterations=outer, sart_iterations=2, norm_mode=om)
    prm1 = oracle.asdpocs_params(num_iterations=1, sart_iterations=2, norm_mode=om)
    for s in range(slices):
        want_vol, want_x, want_sc = oracle.asdpocs_state(oracle.projector(n, na, step), sinos[s], prm)
        # the dtgv reduction was taken at least once over the outer iterations
        _, _, first = oracle.asdpocs_state(oracle.projector(n, na, step), sinos[s], prm1)
        assert want_sc["dtgv"] < first["dtgv"]
        assert np.array_equal(vol[s], want_vol)
        err = rel_l2(x_tv[s], want_x)
        assert err <= TOL_ITER, err
        for k in ("dp", "dd", "dg", "dtgv"):
            assert abs(sc[s][k] - want_sc[k]) <= TOL_ITER * abs(want_sc[k]), (k, sc[s][k], want_sc[k])
        if mode == "compat":
            assert np.array_equal(x_tv[s], want_x), np.abs(x_tv[s] - want_x).max()
            assert all(np.float32(sc[s][k]) == np.float32(want_sc[k]) for k in want_sc), (sc[s], want_sc)
        elif n <= 530:
            # error of the product (FP64 norm) mode against the FP64 recomputation
            _, xd, _ = oracle.asdpocs_d_state(oracle.projector(n, na, step), sinos[s], prm)
            e64, ref64 = rel_l2(x_tv[s], xd), rel_l2(want_x, xd)
            print(f"\nASD-POCS {n}^2 x {na}, {outer} outer: post-TV x rel-L2 vs the FP64 twin {e64:.2e} "
                  f"(the reference arithmetic's: {ref64:.2e})")
            assert e64 <= max(1.05 * ref64, ref64 + 1e-6), (e64, ref64)
