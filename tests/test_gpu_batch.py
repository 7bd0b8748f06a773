"""Mixed SIRT batches (ufoir_batch_*) and the forward projector's autotuner,
through the C ABI.

A batch advances one-slice SIRT jobs of different sizes and angle counts
together; every member must equal ufoir_sirt_process on it alone, bit for
bit, whatever the mix, the order, the launch shapes the autotuner picks,
and with members frozen part-way. The reference advances one slice per
process() call (src/tasks/ufo-ir-sirt-task.c:164-222).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# (n_dets, n_angles, axis) of the members: the four serve sizes with angle
# counts from 90 to 1800, a repeated geometry, an off-centre axis, an odd size
MIX = [(367, 90, -1.0), (724, 611, -1.0), (1448, 1200, -1.0), (2900, 181, -1.0), (367, 90, -1.0),
       (300, 97, 141.3), (1001, 1800, -1.0), (64, 16, -1.0)]


def _members(ufoir, ctx, mix, seed):
    rng = np.random.default_rng(seed)
    out = []
    for k, (n, na, axis) in enumerate(mix):
        step = float(np.float32(np.pi / na))
        sino = (rng.random((na, n), dtype=np.float32) * np.float32(n / 4)).astype(np.float32)
        out.append((sino, step, axis, 0.25 if k % 3 else 0.5))
    return out


def _alone(ufoir, ctx, sino, step, axis, relax, iters):
    p = ufoir.ParallelProjector(ctx, step=step, axis_position=axis, is_forward=0)
    x = ufoir.sirt(p, sino, num_iterations=iters, relaxation_factor=relax)
    p.close()
    return x


@pytest.mark.parametrize("autotune", [False, True])
def test_mixed_batch_equals_each_job_alone(ufoir_lib, gpu_ctx, autotune):
    ufoir = ufoir_lib
    mem = _members(ufoir, gpu_ctx, MIX, 11)
    d_s = [ufoir.DeviceArray.from_numpy(gpu_ctx, s) for s, *_ in mem]
    d_v = [ufoir.DeviceArray(gpu_ctx, (s.shape[1], s.shape[1]), zero=True) for s, *_ in mem]
    gpu_ctx.set_autotune(autotune)
    try:
        with ufoir.Batch(gpu_ctx, [(d_s[k], d_v[k], dict(step=st, axis_position=ax, relaxation_factor=rl))
                                   for k, (s, st, ax, rl) in enumerate(mem)]) as b:
            launches, shapes = b.launches()
            assert launches == 2 + shapes and 1 <= shapes <= len(MIX)
            b.run(3)
            got3 = [v.download() for v in d_v]
            b.set_active(0, False)
            b.set_active(5, False)
            b.run(2)
            got5 = [v.download() for v in d_v]
    finally:
        gpu_ctx.set_autotune(ufoir.AUTOTUNE_AUTO)      # the context default
    for k, (s, st, ax, rl) in enumerate(mem):
        want3 = _alone(ufoir, gpu_ctx, s, st, ax, rl, 3)
        assert np.array_equal(got3[k], want3), (k, MIX[k], float(np.abs(got3[k] - want3).max()))
        if k in (0, 5):
            assert np.array_equal(got5[k], want3), k          # frozen members keep their iterate
        else:
            want5 = _alone(ufoir, gpu_ctx, s, st, ax, rl, 5)
            assert np.array_equal(got5[k], want5), (k, MIX[k])
    for a in d_s + d_v:
        a.close()


def test_batch_member_matches_oracle(ufoir_lib, gpu_ctx, oracle):
    ufoir = ufoir_lib
    mix = [(96, 60, -1.0), (130, 45, 64.7), (96, 60, -1.0)]
    mem = _members(ufoir, gpu_ctx, mix, 5)
    d_s = [ufoir.DeviceArray.from_numpy(gpu_ctx, s) for s, *_ in mem]
    d_v = [ufoir.DeviceArray(gpu_ctx, (s.shape[1], s.shape[1]), zero=True) for s, *_ in mem]
    with ufoir.Batch(gpu_ctx, [(d_s[k], d_v[k], dict(step=st, axis_position=ax, relaxation_factor=rl))
                               for k, (s, st, ax, rl) in enumerate(mem)]) as b:
        b.run(4)
    for k, ((n, na, ax), (s, st, _, rl)) in enumerate(zip(mix, mem)):
        want = oracle.sirt(oracle.projector(n, na, np.float32(st), ax), s, 4, rl)
        assert np.array_equal(d_v[k].download(), want), k
    for a in d_s + d_v:
        a.close()


def test_batch_keep_vol_resumes(ufoir_lib, gpu_ctx):
    ufoir = ufoir_lib
    (s, st, ax, rl), = _members(ufoir, gpu_ctx, [(200, 64, -1.0)], 3)
    d_s = ufoir.DeviceArray.from_numpy(gpu_ctx, s)
    d_v = ufoir.DeviceArray(gpu_ctx, (200, 200), zero=True)
    with ufoir.Batch(gpu_ctx, [(d_s, d_v, dict(step=st, relaxation_factor=rl))]) as b:
        b.run(2)
    with ufoir.Batch(gpu_ctx, [(d_s, d_v, dict(step=st, relaxation_factor=rl, keep_vol=1))]) as b:
        b.run(3)
    assert np.array_equal(d_v.download(), _alone(ufoir, gpu_ctx, s, st, ax, rl, 5))
    d_s.close()
    d_v.close()


def test_batch_rejects_what_it_cannot_serve(ufoir_lib, gpu_ctx):
    ufoir = ufoir_lib
    d_s = ufoir.DeviceArray(gpu_ctx, (8, 64), zero=True)
    d_v = ufoir.DeviceArray(gpu_ctx, (64, 64), zero=True)
    with pytest.raises(ufoir.UfoirError) as e:       # fewer than 16 angles
        ufoir.Batch(gpu_ctx, [(d_s, d_v, dict(step=0.3))])
    assert e.value.status == ufoir.ERR_INVALID
    d_s2 = ufoir.DeviceArray(gpu_ctx, (20, 64), zero=True)
    with pytest.raises(ufoir.UfoirError) as e:       # axis at the image edge
        ufoir.Batch(gpu_ctx, [(d_s2, d_v, dict(step=0.1, axis_position=0.25))])
    assert e.value.status == ufoir.ERR_UNSUPPORTED
    with pytest.raises(ufoir.UfoirError) as e:       # relaxation_factor out of range
        ufoir.Batch(gpu_ctx, [(d_s2, ufoir.DeviceArray(gpu_ctx, (64, 64)), dict(step=0.1, relaxation_factor=2.0))])
    assert e.value.status == ufoir.ERR_INVALID
    for a in (d_s, d_v, d_s2):
        a.close()


@pytest.mark.parametrize("n,na,slices", [(1448, 1200, 8), (367, 90, 1), (2900, 90, 1)])
def test_autotuned_forward_projection_is_unchanged(ufoir_lib, gpu_ctx, oracle, n, na, slices):
    ufoir = ufoir_lib
    step = np.float32(np.pi / na)
    vols = np.random.default_rng(n + na).random((slices, n, n), dtype=np.float32)
    p = ufoir.ParallelProjector(gpu_ctx, step=float(step), angles_num=na, is_forward=1)
    before = p.forward(vols, np.zeros((slices, na, n), np.float32))
    t = p.autotune(slices)
    assert t["tuned"] == 1 and t["candidates"] >= 1 and t["ms_tuned"] <= t["ms_default"] * 1.0001
    after = p.forward(vols, np.zeros((slices, na, n), np.float32))
    assert np.array_equal(before, after)
    assert np.array_equal(after[0], oracle.forward(oracle.projector(n, na, step), vols[0]))
    print(f"\nautotune {n}^2 x {na}, {slices} slices: {t}")
    p.close()


# The default mode (AUTO) searches launch shapes for SIRT calls whose tiles
# cannot fill the GPU (one slice: the fixed rules split detectors there).
# Whatever it picks, the result equals the fixed rules' bit for bit.
@pytest.mark.parametrize("n,na", [(724, 64), (1448, 40), (300, 97)])
def test_auto_search_keeps_results(ufoir_lib, gpu_ctx, n, na):
    ufoir = ufoir_lib
    step = np.float32(np.pi / na)
    sino = np.random.default_rng(n + na).random((na, n), dtype=np.float32) * n
    out = {}
    for mode in (ufoir.AUTOTUNE_OFF, ufoir.AUTOTUNE_AUTO):
        gpu_ctx.set_autotune(mode)
        try:
            p = ufoir.ParallelProjector(gpu_ctx, step=float(step), is_forward=0)
            out[mode] = ufoir.sirt(p, sino, num_iterations=3, relaxation_factor=0.25)
            p.close()
        finally:
            gpu_ctx.set_autotune(ufoir.AUTOTUNE_AUTO)
    assert np.array_equal(out[ufoir.AUTOTUNE_OFF], out[ufoir.AUTOTUNE_AUTO])


def test_autotune_mode_argument_checks(ufoir_lib, gpu_ctx):
    L = ufoir_lib.lib()
    assert L.ufoir_ctx_set_autotune(gpu_ctx.handle, 3) == ufoir_lib.ERR_INVALID
    assert L.ufoir_ctx_set_autotune(gpu_ctx.handle, -1) == ufoir_lib.ERR_INVALID
    assert L.ufoir_ctx_set_autotune(gpu_ctx.handle, ufoir_lib.AUTOTUNE_AUTO) == ufoir_lib.OK
