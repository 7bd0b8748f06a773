"""Generates the golden fixtures in this directory.

The outputs come from the reference's own OpenCL kernel sources compiled on
the CPU through the OpenCL-C shim (oracle/_ref/libufoir_ref.so, built only
where the reference tree is present), driven by the oracle's restatement of
the reference's host loops. Inputs are seeded and stored next to the
outputs, so the fixtures are self-contained.

Run from the repository root:  python tests/golden/make_golden.py
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


def main():
    if not O.ref_available():
        O.build()
    if not O.ref_available():
        sys.exit("the reference kernels (oracle/_ref) are not available; cannot generate fixtures")
    projector_case("proj_n16_a12", 16, 12, np.pi / 12, -1.0, 1, 5, 2)
    projector_case("proj_n33_a40_offaxis", 33, 40, np.pi / 40, 15.3, 2, 3, 2)
    projector_case("proj_n24_a4_diag", 24, 4, np.pi / 4, -1.0, 3, 3, 2)
    projector_case("proj_n7_a5", 7, 5, np.pi / 5, -1.0, 4, 2, 2)
    methods_case("methods_n20_a18", 20, 18, 5)
    print("fixtures written to", HERE)


if __name__ == "__main__":
    main()
