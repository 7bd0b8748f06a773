"""The projector's fast interpolation arithmetic ("arithmetic": "fast"), an
extension with no counterpart in the reference, through the C ABI.

Tolerance (the path's stated bar): relative L2 <= 1e-5 against the
reference arithmetic after one projection, <= 1e-4 after the stated
iteration count (100 SIRT iterations at the 1448^2 x 1200-angle geometry).
The exact arithmetic is checked bit for bit against the oracle elsewhere;
here fast results are compared with the oracle after one projection and ten
iterations, and with the exact GPU path after 100 iterations.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_ONE = 1e-5
TOL_ITER = 1e-4


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("n,na,axis,slices", [(1448, 1200, -1.0, 2), (367, 180, -1.0, 1), (300, 97, 141.3, 1),
                                              (2900, 90, -1.0, 1), (724, 45, -1.0, 3)])
def test_fast_projections_within_tolerance(ufoir_lib, gpu_ctx, oracle, n, na, axis, slices):
    from ufoir import synth
    step = np.float32(np.pi / na)
    vols = np.stack([synth.ellipse_phantom(n, int(0.7 * n), 10, seed=n + k) for k in range(slices)])
    pf = ufoir_lib.ParallelProjector(gpu_ctx, step=float(step), axis_position=axis, angles_num=na,
                                     arithmetic=ufoir_lib.ARITH_FAST)
    sino = pf.forward(vols, np.zeros((slices, na, n), np.float32))
    back = pf.backward(np.zeros((slices, n, n), np.float32), sino)
    op = oracle.projector(n, na, step, axis)
    differs = False
    for k in range(slices):
        want = oracle.forward(op, vols[k])
        want_bp = oracle.backward(op, want)
        e_fp = rel_l2(sino[k], want)
        e_bp = rel_l2(back[k], want_bp)
        print(f"\nfast {n}^2 x {na}: FP rel-L2 {e_fp:.2e}, BP rel-L2 {e_bp:.2e}")
        assert e_fp <= TOL_ONE and e_bp <= TOL_ONE, (e_fp, e_bp)
        differs = differs or not np.array_equal(sino[k], want) or not np.array_equal(back[k], want_bp)
    assert differs       # the fast kernels ran (their rounding is not the reference's)
    pf.close()


def test_fast_sirt_c2_geometry_within_tolerance(ufoir_lib, gpu_ctx, oracle):
    from ufoir import synth
    import os
    n, na = 1448, 1200
    step = np.float32(np.pi / na)
    oracle.set_threads(os.cpu_count() or 1)
    vol = synth.ellipse_phantom(n, 1024, 10, seed=2000)
    sino, _ = synth.poisson_noise(oracle.forward(oracle.projector(n, na, step), vol), 1e5, seed=3000)
    fast = ufoir_lib.ParallelProjector(gpu_ctx, step=float(step), is_forward=0, arithmetic=ufoir_lib.ARITH_FAST)
    exact = ufoir_lib.ParallelProjector(gpu_ctx, step=float(step), is_forward=0)
    got10 = ufoir_lib.sirt(fast, sino, num_iterations=10)
    e10 = rel_l2(got10, oracle.sirt(oracle.projector(n, na, step), sino, 10, 0.25))
    got100 = ufoir_lib.sirt(fast, sino, num_iterations=100)
    e100 = rel_l2(got100, ufoir_lib.sirt(exact, sino, num_iterations=100))
    print(f"\nfast SIRT 1448^2 x 1200: 10 iterations vs oracle {e10:.2e}, 100 iterations vs exact {e100:.2e}")
    assert e10 <= TOL_ITER and e100 <= TOL_ITER, (e10, e100)
    fast.close()
    exact.close()


def test_fast_batch_members_equal_fast_runs_alone(ufoir_lib, gpu_ctx):
    ufoir = ufoir_lib
    rng = np.random.default_rng(4)
    geo = [(367, 180), (724, 300), (367, 180)]
    mem = []
    for n, na in geo:
        sino = (rng.random((na, n), dtype=np.float32) * np.float32(n / 4)).astype(np.float32)
        mem.append((sino, float(np.float32(np.pi / na))))
    d_s = [ufoir.DeviceArray.from_numpy(gpu_ctx, s) for s, _ in mem]
    d_v = [ufoir.DeviceArray(gpu_ctx, (s.shape[1], s.shape[1]), zero=True) for s, _ in mem]
    arith = [ufoir.ARITH_FAST, ufoir.ARITH_FAST, ufoir.ARITH_EXACT]
    with ufoir.Batch(gpu_ctx, [(d_s[k], d_v[k], dict(step=st, arithmetic=arith[k]))
                               for k, (s, st) in enumerate(mem)]) as b:
        b.run(4)
    for k, (s, st) in enumerate(mem):
        p = ufoir.ParallelProjector(gpu_ctx, step=st, is_forward=0, arithmetic=arith[k])
        alone = ufoir.sirt(p, s, num_iterations=4)
        assert np.array_equal(d_v[k].download(), alone), k
        p.close()
    for a in d_s + d_v:
        a.close()
