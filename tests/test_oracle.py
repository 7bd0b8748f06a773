"""CPU tests of the oracle: pinned against the golden fixtures (made by the
reference's own kernel sources through the OpenCL-C shim), against the
shim-compiled reference directly where it is built, and against analytic
known answers derived from the kernel formulas."""
import glob
import os

import numpy as np
import pytest

from conftest import GOLDEN


def _proj_cases():
    return sorted(glob.glob(os.path.join(GOLDEN, "proj_*.npz")))


@pytest.mark.parametrize("path", _proj_cases(), ids=lambda p: os.path.basename(p)[:-4])
def test_oracle_matches_golden_projector(oracle, path):
    d = np.load(path)
    n, na, step, axis = int(d["n"]), int(d["na"]), np.float32(d["step"]), float(d["axis"])
    s, c = oracle.lut(na, step)
    assert np.array_equal(s, d["sin"]) and np.array_equal(c, d["cos"])
    assert oracle.full_subsets(s, c) == [tuple(x) for x in d["subsets"].tolist()]
    p = oracle.projector(n, na, step, axis)
    fp = oracle.forward(p, d["vol"])
    assert np.array_equal(fp, d["fp"])
    bp = oracle.backward(p, d["fp"])
    assert np.array_equal(bp, d["bp"])
    sirt = oracle.sirt(oracle.projector(n, na, step, axis), d["fp"], int(d["sirt_iters"]))
    assert np.array_equal(sirt, d["sirt"])
    sart = oracle.sart(oracle.projector(n, na, step, axis), d["fp"], int(d["sart_iters"]))
    assert np.array_equal(sart, d["sart"])


def test_oracle_matches_golden_methods(oracle):
    d = np.load(os.path.join(GOLDEN, "methods_n20_a18.npz"))
    n, na, step = int(d["n"]), int(d["na"]), np.float32(d["step"])
    prm = oracle.asdpocs_params(num_iterations=3, sart_iterations=2, norm_mode=oracle.NORM_COMPAT)
    vol, x = oracle.asdpocs(oracle.projector(n, na, step), d["sino"], prm)
    assert np.array_equal(vol, d["asdpocs"]) and np.array_equal(x, d["asdpocs_x"])
    sp = oracle.sbtv_params(num_iterations=2, lambda_=0.05, mu=1.0, norm_mode=oracle.NORM_COMPAT)
    u, _ = oracle.sbtv(oracle.projector(n, na, step), d["sino"], sp)
    assert np.array_equal(u, d["sbtv"])
    assert np.float32(oracle.l1_norm(d["a"])) == d["l1"]
    assert np.float32(oracle.dot_product(d["a"], d["b"])) == d["dot"]


def test_oracle_matches_golden_tv(oracle):
    """The port's l1_grad (ufo-math-tvstd-method.cl:5-57) on one-row, one-column,
    constant, step and random images, and ASD-POCS's post-TV iterate and
    scalars dp, dd, dg, dtgv after 5 outer iterations, against the fixture the
    reference kernels produced."""
    d = np.load(os.path.join(GOLDEN, "tv_n40_a30.npz"))
    k = oracle.kernels("port").contents
    for key in [f[len("g_in_"):] for f in d.files if f.startswith("g_in_")]:
        a = d["g_in_" + key]
        g = np.zeros_like(a)
        k.l1_grad(oracle.image(a), oracle.image(g))
        assert np.array_equal(g, d["g_out_" + key]), key
    n, na, step = int(d["n"]), int(d["na"]), np.float32(d["step"])
    prm = oracle.asdpocs_params(num_iterations=int(d["outer"]), sart_iterations=int(d["sart_iterations"]),
                                norm_mode=oracle.NORM_COMPAT)
    vol, x, sc = oracle.asdpocs_state(oracle.projector(n, na, step), d["sino"], prm)
    assert np.array_equal(vol, d["asdpocs"]) and np.array_equal(x, d["asdpocs_x"])
    assert np.array_equal(np.array([sc["dp"], sc["dd"], sc["dg"], sc["dtgv"]], np.float32), d["scalars"])
    # the TV stage changed x, and the dtgv reduction was taken
    assert not np.array_equal(vol, x)
    prm1 = oracle.asdpocs_params(num_iterations=1, sart_iterations=int(d["sart_iterations"]),
                                 norm_mode=oracle.NORM_COMPAT)
    assert sc["dtgv"] < oracle.asdpocs_state(oracle.projector(n, na, step), d["sino"], prm1)[2]["dtgv"]


@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(GOLDEN), "..", "oracle", "_ref",
                                                     "libufoir_ref.so")),
                    reason="reference kernels (oracle/_ref) are built only where the reference tree exists")
@pytest.mark.parametrize("n,na,axis", [(9, 7, -1.0), (32, 45, -1.0), (31, 60, 14.2), (40, 90, 21.7)])
def test_port_equals_reference_kernels(oracle, n, na, axis):
    rng = np.random.default_rng(n * 1000 + na)
    step = np.float32(np.pi / na)
    vol = rng.random((n, n), dtype=np.float32)
    for which in ("port",):
        p = oracle.projector(n, na, step, axis)
        a = oracle.forward(p, vol, which=which)
        b = oracle.forward(p, vol, which="ref")
        assert np.array_equal(a, b)
        assert np.array_equal(oracle.backward(p, a, which=which), oracle.backward(p, a, which="ref"))
        assert np.array_equal(oracle.sirt(oracle.projector(n, na, step, axis), a, 3),
                              oracle.sirt(oracle.projector(n, na, step, axis), a, 3, which="ref"))
    prm = oracle.asdpocs_params(num_iterations=2, sart_iterations=1)
    x1 = oracle.asdpocs(oracle.projector(n, na, step, axis), a, prm)
    x2 = oracle.asdpocs(oracle.projector(n, na, step, axis), a, prm, which="ref")
    assert np.array_equal(x1[0], x2[0]) and np.array_equal(x1[1], x2[1])


def test_kat_fp_of_ones_at_theta0_is_height(oracle):
    # theta = 0: vertical kernel, x = s + 0.5 exactly, every sample a texel centre.
    n = 37
    p = oracle.projector(n, 1, np.float32(0.0))
    sino = oracle.forward(p, np.ones((n, n), np.float32))
    assert np.all(sino == n)


def test_kat_bp_of_ones_is_angle_count(oracle):
    # The edge clamp keeps every sample inside the detector, so each angle adds
    # (1-t)*1 + t*1, i.e. 1 up to one rounding.
    n, na = 21, 30
    p = oracle.projector(n, na, np.float32(np.pi / na))
    vol = oracle.backward(p, np.ones((na, n), np.float32))
    assert np.allclose(vol, na, rtol=0, atol=na * 2e-7)


def test_kat_lut_and_subsets(oracle):
    s, c = oracle.lut(4, np.float32(np.pi / 4))
    assert s[0] == 0.0 and c[0] == 1.0
    # 45 degrees: |sin| == |cos| in float -> vertical (the rule is <=)
    assert oracle.full_subsets(s, c) == [(0, 2, 1), (2, 1, 0), (3, 1, 1)]
    s, c = oracle.lut(180, np.float32(np.pi / 180))
    subs = oracle.full_subsets(s, c)
    assert [x[2] for x in subs] == [1, 0, 1] and sum(x[1] for x in subs) == 180


def test_kat_inv_of_zero_is_zero(oracle):
    k = oracle.kernels("port")
    a = np.array([[0.0, 2.0, -4.0, 0.5]], np.float32)
    k.contents.op_inv(oracle.image(a))
    assert a.tolist() == [[0.0, 0.5, -0.25, 2.0]]


def test_kat_periodic_differences_are_adjoint(oracle):
    k = oracle.kernels("port").contents
    rng = np.random.default_rng(3)
    n = 17
    u = rng.standard_normal((n, n)).astype(np.float32)
    v = rng.standard_normal((n, n)).astype(np.float32)
    for fwd, adj in ((k.dx, k.dxt), (k.dy, k.dyt)):
        du = np.zeros_like(u)
        av = np.zeros_like(v)
        fwd(oracle._f32(u), oracle._f32(du), n, n)
        adj(oracle._f32(v), oracle._f32(av), n, n)
        lhs = np.dot(du.astype(np.float64).ravel(), v.astype(np.float64).ravel())
        rhs = np.dot(u.astype(np.float64).ravel(), av.astype(np.float64).ravel())
        assert abs(lhs - rhs) <= 1e-4 * (abs(lhs) + 1)


def test_fp64_twin_close_to_float(oracle):
    d = np.load(os.path.join(GOLDEN, "proj_n16_a12.npz"))
    n, na, step = int(d["n"]), int(d["na"]), np.float32(d["step"])
    p = oracle.projector(n, na, step)
    fp64 = oracle.forward_d(p, d["vol"])
    rel = np.linalg.norm(fp64 - d["fp"]) / np.linalg.norm(fp64)
    assert rel < 1e-6


def test_fp_bp_adjointness_gap_is_measured_not_assumed(oracle):
    # Joseph FP and pixel-driven BP are not exact adjoints: the reference's FP
    # sums samples at unit spacing along the dominant axis without the
    # 1/max(|cos|, |sin|) path-length factor, and BP clamps to the detector
    # edges. The gap (about 18 % here) is a property of the reference path.
    rng = np.random.default_rng(11)
    n, na = 32, 48
    p = oracle.projector(n, na, np.float32(np.pi / na))
    x = rng.random((n, n), dtype=np.float32)
    y = rng.random((na, n), dtype=np.float32)
    ax = oracle.forward_d(p, x)
    aty = oracle.backward_d(p, y)
    lhs = float(np.sum(ax * y))
    rhs = float(np.sum(x * aty))
    gap = abs(lhs - rhs) / abs(lhs)
    assert 0.05 < gap < 0.3


# ---- the "siddon" model's oracle (no reference counterpart: pinned by an
# analytic known answer and by adjointness) ----

@pytest.mark.parametrize("n,na,axis", [(40, 13, -1.0), (40, 13, 17.3), (65, 7, 30.1), (16, 1, -1.0)])
def test_kat_siddon_fp_of_ones_is_the_chord(oracle, n, na, axis):
    # the projection of a uniform image is each ray's chord through the image square
    step = np.float32(np.pi / na)
    got = oracle.siddon_forward(n, na, step, np.ones((n, n), np.float32), axis)
    want = oracle.siddon_chords(n, na, step, axis)
    assert np.abs(got - want).max() < 1e-10


@pytest.mark.parametrize("n,na,axis", [(40, 13, -1.0), (33, 9, 12.6)])
def test_siddon_oracle_halves_are_adjoint(oracle, n, na, axis):
    step = np.float32(np.pi / na)
    rng = np.random.default_rng(n + na)
    x = rng.random((n, n), dtype=np.float32)
    y = rng.random((na, n), dtype=np.float32)
    ax = oracle.siddon_forward(n, na, step, x, axis)
    aty = oracle.siddon_backward(n, na, step, y, axis)
    lhs, rhs = float((ax * y).sum()), float((x * aty).sum())
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs)
