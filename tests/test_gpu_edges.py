"""Edge cases of the projector and the methods, through the C ABI.

Degenerate sizes (one detector, one angle, two or three of either), angle
counts either side of the tiled backprojector's threshold (16), odd sizes,
and empty or mis-shaped calls. Results must equal the oracle bit for bit,
and calls that cannot be served must fail with a status, not a fault.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _proj(ufoir, ctx, n, na, step, axis=-1.0, is_forward=1):
    p = ufoir.ParallelProjector(ctx, step=float(step), axis_position=float(axis), is_forward=is_forward)
    p.get_requisition((n, na))
    return p


@pytest.mark.parametrize("n,na", [(1, 1), (1, 5), (2, 3), (3, 16), (4, 1), (5, 17), (9, 15), (2, 64)])
def test_tiny_sizes_fp_bp_match_oracle(ufoir_lib, gpu_ctx, oracle, n, na):
    step = np.float32(np.pi / na)
    rng = np.random.default_rng(100 * n + na)
    vols = rng.random((2, n, n), dtype=np.float32)
    p = _proj(ufoir_lib, gpu_ctx, n, na, step)
    op = oracle.projector(n, na, step)
    got = p.forward(vols, np.zeros((2, na, n), np.float32))
    sinos = rng.random((2, na, n), dtype=np.float32)
    back = p.backward(np.zeros((2, n, n), np.float32), sinos)
    for i in range(2):
        assert np.array_equal(got[i], oracle.forward(op, vols[i])), (n, na, i)
        assert np.array_equal(back[i], oracle.backward(op, sinos[i])), (n, na, i)
    p.close()


@pytest.mark.parametrize("n,na", [(2, 3), (3, 16), (5, 17), (8, 15)])
def test_tiny_sizes_sirt_sart_match_oracle(ufoir_lib, gpu_ctx, oracle, n, na):
    step = np.float32(np.pi / na)
    rng = np.random.default_rng(7 * n + na)
    sino = rng.random((na, n), dtype=np.float32) * n
    p = _proj(ufoir_lib, gpu_ctx, n, na, step, is_forward=0)
    op = oracle.projector(n, na, step)
    assert np.array_equal(ufoir_lib.sirt(p, sino, num_iterations=3), oracle.sirt(op, sino, 3, 0.25))
    assert np.array_equal(ufoir_lib.sart(p, sino, num_iterations=2, relaxation_factor=0.5),
                          oracle.sart(op, sino, 2, 0.5))
    p.close()


def test_zero_angle_step_projects_every_angle_at_theta_zero(ufoir_lib, gpu_ctx, oracle):
    # step = 0 (the property's default): every angle is theta = 0
    n, na = 12, 5
    vol = np.random.default_rng(3).random((n, n), dtype=np.float32)
    p = _proj(ufoir_lib, gpu_ctx, n, na, 0.0)
    got = p.forward(vol, np.zeros((na, n), np.float32))
    assert np.array_equal(got, oracle.forward(oracle.projector(n, na, np.float32(0.0)), vol))
    assert all(np.array_equal(got[0], got[k]) for k in range(1, na))
    p.close()


def test_empty_and_misshaped_calls_fail_with_a_status(ufoir_lib, gpu_ctx):
    u = ufoir_lib
    p = _proj(u, gpu_ctx, 8, 6, 0.5, is_forward=0)
    with pytest.raises(u.UfoirError) as e:            # no slices at all
        u.sirt(p, np.zeros((0, 6, 8), np.float32))
    assert e.value.status == u.ERR_INVALID and "n_slices" in str(e.value)
    with pytest.raises(u.UfoirError) as e:            # angles_num fixed to 6, sinogram has 7 rows
        p.set(angles_num=6)
        u.sart(p, np.zeros((7, 8), np.float32))
    assert e.value.status == u.ERR_INVALID
    with pytest.raises(u.UfoirError) as e:            # num-iterations 0
        u.sirt(p, np.zeros((6, 8), np.float32), num_iterations=0)
    assert e.value.status == u.ERR_INVALID
    # the context is still usable afterwards
    p.set(angles_num=0)
    out = u.sirt(p, np.ones((6, 8), np.float32), num_iterations=1)
    assert out.shape == (8, 8) and np.isfinite(out).all()
    p.close()
