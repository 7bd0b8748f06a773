"""Generates the golden fixtures in this directory.

The outputs come from the reference's own OpenCL kernel sources compiled on
the CPU through the OpenCL-C shim (oracle/_ref/libufoir_ref.so, built only
where the reference tree is present), driven by the oracle's restatement of
the reference's host loops. Inputs are seeded and stored next to the
outputs, so the fixtures are self-contained.

Run from the repository root:  python tests/golden/make_golden.py [fixture names]
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import pyoracle as O  # noqa: E402


def projector_case(name, n, na, step, axis, seed, sirt_iters, sart_iters):
    rng = np.random.default_rng(seed)
    vol = rng.random((n, n), dtype=np.float32)
    p = O.projector(n, na, np.float32(step), axis)
    sino = O.forward(p, vol, which="ref")
    back = O.backward(p, sino, which="ref")
    sirt = O.sirt(O.projector(n, na, np.float32(step), axis), sino, sirt_iters, 0.25, which="ref")
    sart = O.sart(O.projector(n, na, np.float32(step), axis), sino, sart_iters, 0.25, which="ref")
    s, c = O.lut(na, np.float32(step))
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), n=n, na=na, step=np.float32(step),
                        axis=np.float32(axis), vol=vol, fp=sino, bp=back, sirt=sirt,
                        sirt_iters=sirt_iters, sart=sart, sart_iters=sart_iters, sin=s, cos=c,
                        subsets=np.array(O.full_subsets(s, c), np.int64))


def methods_case(name, n, na, seed):
    rng = np.random.default_rng(seed)
    vol = rng.random((n, n), dtype=np.float32)
    step = np.float32(np.pi / na)
    sino = O.forward(O.projector(n, na, step), vol, which="ref")
    prm = O.asdpocs_params(num_iterations=3, sart_iterations=2, norm_mode=O.NORM_COMPAT)
    asd, asd_x = O.asdpocs(O.projector(n, na, step), sino, prm, which="ref")
    sp = O.sbtv_params(num_iterations=2, lambda_=0.05, mu=1.0, norm_mode=O.NORM_COMPAT)
    sbtv, _ = O.sbtv(O.projector(n, na, step), sino, sp, which="ref")
    a = rng.standard_normal((n, n)).astype(np.float32)
    b = rng.standard_normal((n, n)).astype(np.float32)
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), n=n, na=na, step=step, sino=sino,
                        asdpocs=asd, asdpocs_x=asd_x, sbtv=sbtv, a=a, b=b,
                        l1=np.float32(O.l1_norm(a)), dot=np.float32(O.dot_product(a, b)))


def tv_case(name, n, na, seed, outer):
    """The TV stage of ASD-POCS: l1_grad on images of several shapes (random,
    constant, a step, one row, one column), and ASD-POCS on a noisy sinogram
    with the post-TV iterate and the scalars dp, dd, dg, dtgv after `outer`
    outer iterations, through the reference kernels."""
    rng = np.random.default_rng(seed)
    grads = {}
    shapes = {"rand_33x70": (33, 70), "rand_70x33": (70, 33), "row_1x57": (1, 57), "col_57x1": (57, 1),
              "rand_1x1": (1, 1)}
    for key, (h, w) in shapes.items():
        a = (rng.standard_normal((h, w)) * 3).astype(np.float32)
        grads[key] = a
    grads["const_40x40"] = np.full((40, 40), 2.5, np.float32)
    step_img = np.zeros((40, 40), np.float32)
    step_img[:, 20:] = 1.0
    grads["step_40x40"] = step_img
    out = {}
    k = O.kernels("ref").contents
    for key, a in grads.items():
        g = np.zeros_like(a)
        k.l1_grad(O.image(a), O.image(g))
        out["g_in_" + key] = a
        out["g_out_" + key] = g
    yy, xx = np.mgrid[0:n, 0:n]
    vol = ((xx - n / 2) ** 2 + (yy - n / 2) ** 2 < (0.35 * n) ** 2).astype(np.float32)
    vol += (np.abs(xx - 0.4 * n) + np.abs(yy - 0.55 * n) < 0.12 * n).astype(np.float32) * 0.5
    step = np.float32(np.pi / na)
    clean = O.forward(O.projector(n, na, step), vol, which="ref")
    kappa = 4.0 / float(clean.max())
    counts = rng.poisson(1e4 * np.exp(-kappa * clean.astype(np.float64)))
    sino = (-np.log(np.maximum(counts, 1) / 1e4) / kappa).astype(np.float32)
    prm = O.asdpocs_params(num_iterations=outer, sart_iterations=2, norm_mode=O.NORM_COMPAT)
    asd, asd_x, sc = O.asdpocs_state(O.projector(n, na, step), sino, prm, which="ref")
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), n=n, na=na, step=step, sino=sino, outer=outer,
                        sart_iterations=2, asdpocs=asd, asdpocs_x=asd_x,
                        scalars=np.array([sc["dp"], sc["dd"], sc["dg"], sc["dtgv"]], np.float32), **out)


def main():
    if not O.ref_available():
        O.build()
    if not O.ref_available():
        sys.exit("the reference kernels (oracle/_ref) are not available; cannot generate fixtures")
    only = sys.argv[1:]     # optional fixture names; default: all
    cases = [
        ("proj_n16_a12", lambda: projector_case("proj_n16_a12", 16, 12, np.pi / 12, -1.0, 1, 5, 2)),
        ("proj_n33_a40_offaxis", lambda: projector_case("proj_n33_a40_offaxis", 33, 40, np.pi / 40, 15.3, 2, 3, 2)),
        ("proj_n24_a4_diag", lambda: projector_case("proj_n24_a4_diag", 24, 4, np.pi / 4, -1.0, 3, 3, 2)),
        ("proj_n7_a5", lambda: projector_case("proj_n7_a5", 7, 5, np.pi / 5, -1.0, 4, 2, 2)),
        ("methods_n20_a18", lambda: methods_case("methods_n20_a18", 20, 18, 5)),
        ("tv_n40_a30", lambda: tv_case("tv_n40_a30", 40, 30, 9, 5)),
    ]
    for name, make in cases:
        if not only or name in only:
            make()
    print("fixtures written to", HERE)


if __name__ == "__main__":
    main()
