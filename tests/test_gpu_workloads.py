"""GPU parity at the configured workloads, on noisy inputs, with the error
of each result against the oracle's FP64 twin stated.

Workloads (seeded synthetic stand-ins with the configured shapes):
  C1  SART 367^2 grid (256^2 ellipse phantom), 180 angles, 10 iterations,
      clean sinogram from the Joseph FP (as configured: no noise);
  C2  batched SIRT 1448^2 grid (1024^2 ellipse phantoms), 1200 angles,
      Poisson noise at I0 = 1e5 then log; 4 slices x 10 iterations through the
      resident batch against the oracle, and a 64-slice batch whose slices
      equal single-slice runs;
  C3a ASD-POCS 2900^2 grid (2048^2 polygon phantom), 90 angles, Poisson
      noise at I0 = 1e4; 1 outer iteration with 10 inner SART iterations, in
      COMPAT and FP64 norm modes;
  C4  SBTV 1448^2 grid, 720 angles, lambda 0.05, mu 1.0, I0 = 1e5; 1 outer
      iteration, COMPAT and FP64 norm modes.

Bars: bit-exact against the oracle where every operation is the reference's
(all of the above in COMPAT mode, and SIRT/SART always); relative L2 <= 1e-4
in FP64 norm mode. The error against the FP64 twin is printed (run with -s
to see it) beside the reference arithmetic's own (the oracle's float result
against the same twin): it is the float arithmetic's error, not a parity
figure, and it must not exceed the reference's by more than 5 % (or 1e-6).
The oracle runs OpenMP over every host core; these cases take minutes.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_ITER = 1e-4


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    den = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (den if den > 0 else 1.0)


def _clean(ufoir_lib, gpu_ctx, n, na, vols):
    """Joseph FP of the phantoms on the GPU (bit-equal to the oracle's FP)."""
    step = float(np.float32(np.pi / na))
    p = ufoir_lib.ParallelProjector(gpu_ctx, step=step, angles_num=na, is_forward=1)
    sino = p.forward(vols, np.zeros(vols.shape[:-2] + (na, n), np.float32))
    p.close()
    return sino


def _report(name, got, ref_float, twin):
    """Prints and checks the FP64-twin error of a result (got) against that
    of the reference arithmetic (ref_float, the oracle's float result)."""
    err = rel_l2(got, twin)
    ref_err = rel_l2(ref_float, twin)
    print(f"\n{name}: rel-L2 against the FP64 twin {err:.3e} (the reference arithmetic's: {ref_err:.3e})")
    assert err <= max(1.05 * ref_err, ref_err + 1e-6), (err, ref_err)


@pytest.fixture(scope="module")
def all_cores(oracle):
    oracle.set_threads(os.cpu_count() or 1)


def test_c1_sart_10_iterations(ufoir_lib, gpu_ctx, oracle, all_cores):
    from ufoir import synth
    n, na, iters = 367, 180, 10
    step = np.float32(np.pi / na)
    vol = synth.ellipse_phantom(n, 256, 10, seed=1001)
    sino = oracle.forward(oracle.projector(n, na, step), vol)
    p = ufoir_lib.ParallelProjector(gpu_ctx, step=float(step), is_forward=0)
    got = ufoir_lib.sart(p, sino, num_iterations=iters, relaxation_factor=0.25)
    want = oracle.sart(oracle.projector(n, na, step), sino, iters, 0.25)
    assert np.array_equal(got, want), np.abs(got - want).max()
    _report("C1 SART 367^2 x 180, 10 iterations", got, want,
            oracle.sart_d(oracle.projector(n, na, step), sino, iters, 0.25))
    p.close()


def test_c2_batched_sirt_10_iterations_noisy(ufoir_lib, gpu_ctx, oracle, all_cores):
    from ufoir import synth
    n, na, iters, S = 1448, 1200, 10, 4
    step = np.float32(np.pi / na)
    vols = np.stack([synth.ellipse_phantom(n, 1024, 10, seed=2000 + i) for i in range(S)])
    clean = _clean(ufoir_lib, gpu_ctx, n, na, vols)
    sinos = np.stack([synth.poisson_noise(clean[i], 1e5, seed=3000 + i)[0] for i in range(S)])
    p = ufoir_lib.ParallelProjector(gpu_ctx, step=float(step), angles_num=na, is_forward=0)
    d_sino = ufoir_lib.DeviceArray.from_numpy(gpu_ctx, sinos)
    d_vol = ufoir_lib.DeviceArray(gpu_ctx, (S, n, n), zero=True)
    batch = ufoir_lib.SirtBatch(p, d_sino, d_vol, relaxation_factor=0.25)
    batch.run(iters)
    got = d_vol.download()
    batch.close()
    wants = []
    for i in range(S):
        want = oracle.sirt(oracle.projector(n, na, step), sinos[i], iters, 0.25)
        assert rel_l2(got[i], want) <= TOL_ITER
        assert np.array_equal(got[i], want), (i, np.abs(got[i] - want).max())
        wants.append(want)
    _report("C2 SIRT 1448^2 x 1200, 10 iterations, slice 0", got[0], wants[0],
            oracle.sirt_d(oracle.projector(n, na, step), sinos[0], iters, 0.25))
    d_sino.close()
    d_vol.close()
    p.close()


def test_c2_64_slice_batch_equals_single_slice_runs(ufoir_lib, gpu_ctx):
    # 64 distinct slices (8 phantoms at 8 scales) in one resident batch; a
    # slice's result must not depend on the batch around it
    from ufoir import synth
    n, na, iters, S = 1448, 1200, 10, 64
    step = float(np.float32(np.pi / na))
    base = np.stack([synth.ellipse_phantom(n, 1024, 10, seed=2100 + i) for i in range(8)])
    clean = _clean(ufoir_lib, gpu_ctx, n, na, base)
    sinos = np.empty((S, na, n), np.float32)
    for k in range(S):
        sinos[k], _ = synth.poisson_noise(clean[k % 8] * np.float32(1.0 + k / 64.0), 1e5, seed=3100 + k)
    p = ufoir_lib.ParallelProjector(gpu_ctx, step=step, angles_num=na, is_forward=0)
    d_sino = ufoir_lib.DeviceArray.from_numpy(gpu_ctx, sinos)
    d_vol = ufoir_lib.DeviceArray(gpu_ctx, (S, n, n), zero=True)
    batch = ufoir_lib.SirtBatch(p, d_sino, d_vol, relaxation_factor=0.25)
    batch.run(iters)
    got = d_vol.download()
    batch.close()
    for k in (0, 17, 38, 63):
        alone = ufoir_lib.sirt(p, sinos[k], num_iterations=iters, relaxation_factor=0.25)
        assert np.array_equal(got[k], alone), (k, np.abs(got[k] - alone).max())
    d_sino.close()
    d_vol.close()
    p.close()


@pytest.mark.parametrize("mode", ["compat", "fp64"])
def test_c3a_asdpocs_one_outer_iteration_noisy(ufoir_lib, gpu_ctx, oracle, all_cores, mode):
    from ufoir import synth
    n, na = 2900, 90
    step = np.float32(np.pi / na)
    vol = synth.polygon_phantom(n, 2048, 8, seed=3001)
    sino, _ = synth.poisson_noise(_clean(ufoir_lib, gpu_ctx, n, na, vol), 1e4, seed=3002)
    m = ufoir_lib.NORM_COMPAT if mode == "compat" else ufoir_lib.NORM_FP64
    om = oracle.NORM_COMPAT if mode == "compat" else oracle.NORM_FP64
    p = ufoir_lib.ParallelProjector(gpu_ctx, step=float(step), is_forward=0)
    got, x_tv, sc = ufoir_lib.asdpocs_state(p, sino, num_iterations=1, norm_mode=m,
                                            df_minimizer=dict(num_iterations=10, relaxation_factor=0.25))
    prm = oracle.asdpocs_params(num_iterations=1, sart_iterations=10, norm_mode=om)
    want, want_x, want_sc = oracle.asdpocs_state(oracle.projector(n, na, step), sino, prm)
    assert np.array_equal(got, want), np.abs(got - want).max()
    assert rel_l2(x_tv, want_x) <= TOL_ITER
    if mode == "compat":
        assert np.array_equal(x_tv, want_x), np.abs(x_tv - want_x).max()
        assert all(np.float32(sc[0][k]) == np.float32(want_sc[k]) for k in want_sc), (sc, want_sc)
    else:
        vd, xd, _ = oracle.asdpocs_d_state(oracle.projector(n, na, step), sino, prm)
        _report("C3a ASD-POCS 2900^2 x 90, 1 outer iteration, output", got, want, vd)
        _report("C3a ASD-POCS 2900^2 x 90, 1 outer iteration (FP64 norms), post-TV x", x_tv, want_x, xd)
    p.close()


@pytest.mark.parametrize("mode", ["compat", "fp64"])
def test_c4_sbtv_one_outer_iteration_noisy(ufoir_lib, gpu_ctx, oracle, all_cores, mode):
    from ufoir import synth
    n, na = 1448, 720
    step = np.float32(np.pi / na)
    vol = synth.ellipse_phantom(n, 1024, 10, seed=4001)
    sino, _ = synth.poisson_noise(_clean(ufoir_lib, gpu_ctx, n, na, vol), 1e5, seed=4002)
    m = ufoir_lib.NORM_COMPAT if mode == "compat" else ufoir_lib.NORM_FP64
    om = oracle.NORM_COMPAT if mode == "compat" else oracle.NORM_FP64
    p = ufoir_lib.ParallelProjector(gpu_ctx, step=float(step), is_forward=0)
    got = ufoir_lib.sbtv(p, sino, num_iterations=1, norm_mode=m, mu=1.0, **{"lambda": 0.05})
    want, _ = oracle.sbtv(oracle.projector(n, na, step), sino.copy(),
                          oracle.sbtv_params(num_iterations=1, lambda_=0.05, mu=1.0, norm_mode=om))
    err = rel_l2(got, want)
    print(f"\nC4 SBTV 1448^2 x 720, 1 outer iteration ({mode}): rel-L2 against the oracle {err:.3e}")
    assert err <= TOL_ITER, err
    if mode == "compat":
        assert np.array_equal(got, want), np.abs(got - want).max()
    p.close()
