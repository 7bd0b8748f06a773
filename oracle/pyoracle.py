"""ctypes binding of the CPU oracle (oracle/liboracle.so, oracle/_ref/libufoir_ref.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()`` and
by the CPU-baseline leg of ``bench.py``, always as the result compared with. The product
(``ufo-ir_gb300``) never imports this module.

Arrays are numpy, C-contiguous: sinograms ``[n_angles, n_dets]``, volumes
``[n_dets, n_dets]`` (float32 for the reference arithmetic, float64 for the
FP64 twin).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libufoir_ref.so")

NORM_COMPAT = 0
NORM_FP64 = 1


class Dims(C.Structure):
    _fields_ = [("height", C.c_ulong), ("width", C.c_ulong),
                ("n_dets", C.c_ulong), ("n_angles", C.c_ulong)]


class Subset(C.Structure):
    _fields_ = [("offset", C.c_uint), ("n", C.c_uint), ("direction", C.c_int)]


class Image(C.Structure):
    _fields_ = [("data", C.POINTER(C.c_float)), ("width", C.c_long), ("height", C.c_long)]


class Projector(C.Structure):
    _fields_ = [("n_dets", C.c_uint), ("n_angles", C.c_uint), ("step", C.c_float),
                ("axis_position", C.c_float), ("relaxation", C.c_float),
                ("correction_scale", C.c_float)]


class AsdpocsParams(C.Structure):
    _fields_ = [("num_iterations", C.c_uint), ("beta", C.c_float), ("beta_red", C.c_float),
                ("alpha", C.c_float), ("alpha_red", C.c_float), ("r_max", C.c_float),
                ("ng", C.c_uint), ("positive_constraint", C.c_int),
                ("sart_iterations", C.c_uint), ("sart_relaxation", C.c_float),
                ("norm_mode", C.c_int)]


class SbtvParams(C.Structure):
    _fields_ = [("num_iterations", C.c_uint), ("lambda_", C.c_float), ("mu", C.c_float),
                ("norm_mode", C.c_int)]


_FP = C.CFUNCTYPE(None, Image, Image, C.POINTER(C.c_float), C.POINTER(C.c_float), Dims,
                  C.c_float, Subset, C.c_float)
_BP = C.CFUNCTYPE(None, Image, Image, C.c_float, C.POINTER(C.c_float), C.POINTER(C.c_float),
                  Dims, C.c_float, Subset)


class Kernels(C.Structure):
    _fields_ = [("fp", _FP), ("bp", _BP),
                ("op_set", C.CFUNCTYPE(None, Image, C.c_float)),
                ("op_inv", C.CFUNCTYPE(None, Image)),
                ("op_mul", C.CFUNCTYPE(None, Image, Image, Image)),
                ("op_add", C.CFUNCTYPE(None, Image, Image, Image)),
                ("op_deduction", C.CFUNCTYPE(None, Image, Image, Image)),
                ("op_deduction2", C.CFUNCTYPE(None, Image, Image, C.c_float, Image)),
                ("op_add2", C.CFUNCTYPE(None, Image, Image, C.c_float, Image)),
                ("op_mul_rows", C.CFUNCTYPE(None, Image, Image, Image, C.c_uint, C.c_uint)),
                ("op_posc", C.CFUNCTYPE(None, Image, Image)),
                ("l1_grad", C.CFUNCTYPE(None, Image, Image)),
                ("dx", C.CFUNCTYPE(None, C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_long, C.c_long)),
                ("dxt", C.CFUNCTYPE(None, C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_long, C.c_long)),
                ("dy", C.CFUNCTYPE(None, C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_long, C.c_long)),
                ("dyt", C.CFUNCTYPE(None, C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_long, C.c_long))]


# The reference's four OpenCL kernel files, compiled through clshim.hpp into
# _ref/libufoir_ref.so. Where the ufo-ir tree is present they are staged,
# unmodified, into the git-ignored baseline/_ref/kernels so that the build on
# a machine without the tree (the GPU host) compiles the same sources.
REF_TREE_KERNELS = "/root/reference/src/kernels"
STAGED_KERNELS = os.path.join(os.path.dirname(HERE), "baseline", "_ref", "kernels")
REF_KERNEL_FILES = ("projector-parallel-joseph.cl", "ufo-ir-basic-ops.cl", "ufo-math-tvstd-method.cl",
                    "ufo-ir-gradient-processor.cl")


def reference_kernel_dir():
    """Directory of the reference kernel sources: $UFO_IR_REF, else the ufo-ir
    tree (staged into baseline/_ref/kernels on the way), else the staged copy,
    else None."""
    env = os.environ.get("UFO_IR_REF")
    if env:
        return env
    if all(os.path.exists(os.path.join(REF_TREE_KERNELS, f)) for f in REF_KERNEL_FILES):
        import shutil
        os.makedirs(STAGED_KERNELS, exist_ok=True)
        for f in REF_KERNEL_FILES:
            dst = os.path.join(STAGED_KERNELS, f)
            src = os.path.join(REF_TREE_KERNELS, f)
            if not os.path.exists(dst) or open(src, "rb").read() != open(dst, "rb").read():
                shutil.copyfile(src, dst)
        return STAGED_KERNELS
    if all(os.path.exists(os.path.join(STAGED_KERNELS, f)) for f in REF_KERNEL_FILES):
        return STAGED_KERNELS
    return None


def build(quiet: bool = True) -> None:
    """Compile the oracle (and the reference kernels when their sources are available)."""
    cmd = ["make", "-s", "-C", HERE]
    ref_dir = reference_kernel_dir()
    if ref_dir:
        cmd.append("UFO_IR_REF=" + ref_dir)
    out = subprocess.run(cmd, capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    if not quiet:
        print(out.stdout, end="")


_port = None
_ref = None


def port_lib():
    global _port
    if _port is None:
        if not os.path.exists(PORT_SO):
            build()
        lib = C.CDLL(PORT_SO)
        lib.oracle_port_kernels.restype = C.POINTER(Kernels)
        _declare(lib)
        _port = lib
    return _port


def ref_available() -> bool:
    return os.path.exists(REF_SO)


def ref_lib():
    global _ref
    if _ref is None:
        lib = C.CDLL(REF_SO)
        lib.oracle_ref_kernels.restype = C.POINTER(Kernels)
        _ref = lib
    return _ref


def _declare(lib):
    f32p = C.POINTER(C.c_float)
    f64p = C.POINTER(C.c_double)
    kp = C.POINTER(Kernels)
    pp = C.POINTER(Projector)
    lib.oracle_make_lut.argtypes = [C.c_uint, C.c_float, f32p, f32p]
    lib.oracle_make_full_subsets.argtypes = [f32p, f32p, C.c_uint, C.POINTER(Subset)]
    lib.oracle_make_full_subsets.restype = C.c_uint
    lib.oracle_make_angle_subsets.argtypes = [f32p, f32p, C.c_uint, C.POINTER(Subset)]
    lib.oracle_forward.argtypes = [kp, pp, f32p, f32p]
    lib.oracle_backward.argtypes = [kp, pp, f32p, f32p]
    lib.oracle_projector_process.argtypes = [kp, pp, C.c_int, f32p, f32p]
    lib.oracle_sart.argtypes = [kp, pp, C.c_uint, C.c_float, f32p, f32p]
    lib.oracle_sirt.argtypes = [kp, pp, C.c_uint, C.c_float, f32p, f32p]
    lib.oracle_sirt_weights.argtypes = [kp, pp, f32p, f32p]
    lib.oracle_sirt_iterate.argtypes = [kp, pp, C.c_uint, C.c_float, f32p, f32p, f32p, f32p]
    lib.oracle_asdpocs.argtypes = [kp, pp, C.POINTER(AsdpocsParams), f32p, f32p, f32p]
    lib.oracle_asdpocs_state.argtypes = [kp, pp, C.POINTER(AsdpocsParams), f32p, f32p, f32p, f32p]
    lib.oracle_sbtv.argtypes = [kp, pp, C.POINTER(SbtvParams), f32p, f32p]
    for name in ("oracle_l1_norm", "oracle_l1_norm_fp64"):
        getattr(lib, name).argtypes = [f32p, C.c_ulong, C.c_ulong]
        getattr(lib, name).restype = C.c_float
    for name in ("oracle_dot_product", "oracle_dot_product_fp64"):
        getattr(lib, name).argtypes = [f32p, f32p, C.c_ulong, C.c_ulong]
        getattr(lib, name).restype = C.c_float
    lib.oracle_forward_d.argtypes = [pp, f64p, f64p]
    lib.oracle_backward_d.argtypes = [pp, f64p, f64p]
    lib.oracle_sirt_d.argtypes = [pp, C.c_uint, C.c_float, f64p, f64p]
    lib.oracle_sart_d.argtypes = [pp, C.c_uint, C.c_float, f64p, f64p]
    lib.oracle_asdpocs_d.argtypes = [pp, C.POINTER(AsdpocsParams), f64p, f64p, f64p]
    lib.oracle_asdpocs_d_state.argtypes = [pp, C.POINTER(AsdpocsParams), f64p, f64p, f64p, f64p]
    lib.oracle_sbtv_d.argtypes = [pp, C.POINTER(SbtvParams), f64p, f64p]
    lib.oracle_siddon_forward.argtypes = [C.c_uint, C.c_uint, f32p, f32p, C.c_float, f32p, f64p]
    lib.oracle_siddon_backward.argtypes = [C.c_uint, C.c_uint, f32p, f32p, C.c_float, f32p, f64p]
    lib.oracle_siddon_chord.argtypes = [C.c_uint, C.c_float, C.c_float, C.c_float, C.c_uint]
    lib.oracle_siddon_chord.restype = C.c_double
    lib.oracle_set_threads.argtypes = [C.c_int]
    lib.oracle_get_threads.restype = C.c_int


def kernels(which: str = "port"):
    if which == "port":
        return port_lib().oracle_port_kernels()
    if which == "ref":
        return ref_lib().oracle_ref_kernels()
    raise ValueError(which)


def _f32(a):
    assert a.dtype == np.float32 and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_float))


def _f64(a):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_double))


def image(a: np.ndarray) -> Image:
    return Image(_f32(a), a.shape[1], a.shape[0])


def set_threads(n: int) -> None:
    port_lib().oracle_set_threads(int(n))


def get_threads() -> int:
    return int(port_lib().oracle_get_threads())


def projector(n_dets, n_angles, step, axis_position=-1.0, relaxation=1.0, correction_scale=1.0):
    return Projector(n_dets, n_angles, step, axis_position, relaxation, correction_scale)


def lut(n_angles: int, step: float):
    s = np.zeros(n_angles, np.float32)
    c = np.zeros(n_angles, np.float32)
    port_lib().oracle_make_lut(n_angles, step, _f32(s), _f32(c))
    return s, c


def full_subsets(s, c):
    out = (Subset * max(1, len(s)))()
    n = port_lib().oracle_make_full_subsets(_f32(s), _f32(c), len(s), out)
    return [(out[i].offset, out[i].n, out[i].direction) for i in range(n)]


def forward(p: Projector, vol, sino=None, which="port"):
    """Accumulating forward projection over the full subsets (sino += scale * A vol)."""
    if sino is None:
        sino = np.zeros((p.n_angles, p.n_dets), np.float32)
    port_lib().oracle_forward(kernels(which), C.byref(p), _f32(vol), _f32(sino))
    return sino


def backward(p: Projector, sino, vol=None, which="port"):
    """Accumulating backprojection over the full subsets (vol += relax * A^T sino)."""
    if vol is None:
        vol = np.zeros((p.n_dets, p.n_dets), np.float32)
    port_lib().oracle_backward(kernels(which), C.byref(p), _f32(vol), _f32(sino))
    return vol


def projector_process(p: Projector, is_forward: bool, inp, which="port"):
    """State-dependent process: zero the output, then forward or backward."""
    shape = (p.n_angles, p.n_dets) if is_forward else (p.n_dets, p.n_dets)
    out = np.zeros(shape, np.float32)
    port_lib().oracle_projector_process(kernels(which), C.byref(p), int(bool(is_forward)), _f32(inp), _f32(out))
    return out


def sart(p: Projector, sino, iters, relaxation=0.25, which="port"):
    vol = np.zeros((p.n_dets, p.n_dets), np.float32)
    port_lib().oracle_sart(kernels(which), C.byref(p), iters, relaxation, _f32(sino), _f32(vol))
    return vol


def sirt(p: Projector, sino, iters, relaxation=0.25, which="port"):
    vol = np.zeros((p.n_dets, p.n_dets), np.float32)
    port_lib().oracle_sirt(kernels(which), C.byref(p), iters, relaxation, _f32(sino), _f32(vol))
    return vol


def sirt_weights(p: Projector, which="port"):
    R = np.zeros((p.n_angles, p.n_dets), np.float32)
    Cw = np.zeros((p.n_dets, p.n_dets), np.float32)
    port_lib().oracle_sirt_weights(kernels(which), C.byref(p), _f32(R), _f32(Cw))
    return R, Cw


def sirt_iterate(p: Projector, sino, R, Cw, vol, iters=1, relaxation=0.25, which="port"):
    """Continue SIRT from vol (in place) for iters iterations."""
    port_lib().oracle_sirt_iterate(kernels(which), C.byref(p), iters, relaxation, _f32(sino), _f32(R),
                                   _f32(Cw), _f32(vol))
    return vol


def asdpocs_params(**kw) -> AsdpocsParams:
    d = dict(num_iterations=10, beta=1.0, beta_red=0.995, alpha=0.2, alpha_red=0.95,
             r_max=0.95, ng=20, positive_constraint=1, sart_iterations=10,
             sart_relaxation=0.25, norm_mode=NORM_COMPAT)
    d.update(kw)
    return AsdpocsParams(**d)


def asdpocs(p: Projector, sino, prm: AsdpocsParams, which="port"):
    vol = np.zeros((p.n_dets, p.n_dets), np.float32)
    xint = np.zeros_like(vol)
    port_lib().oracle_asdpocs(kernels(which), C.byref(p), C.byref(prm), _f32(sino), _f32(vol), _f32(xint))
    return vol, xint


def asdpocs_state(p: Projector, sino, prm: AsdpocsParams, which="port"):
    """ASD-POCS: (output, post-TV x of the last outer iteration, {dp, dd, dg, dtgv})."""
    vol = np.zeros((p.n_dets, p.n_dets), np.float32)
    xint = np.zeros_like(vol)
    sc = np.zeros(4, np.float32)
    port_lib().oracle_asdpocs_state(kernels(which), C.byref(p), C.byref(prm), _f32(sino), _f32(vol), _f32(xint),
                                    _f32(sc))
    return vol, xint, dict(zip(("dp", "dd", "dg", "dtgv"), (float(v) for v in sc)))


def sbtv_params(**kw) -> SbtvParams:
    d = dict(num_iterations=10, lambda_=0.1, mu=0.5, norm_mode=NORM_COMPAT)
    d.update(kw)
    return SbtvParams(**d)


def sbtv(p: Projector, sino, prm: SbtvParams, which="port"):
    """Returns (volume, normalised sinogram) - the reference normalises its input in place."""
    s = np.array(sino, np.float32, copy=True)
    vol = np.zeros((p.n_dets, p.n_dets), np.float32)
    port_lib().oracle_sbtv(kernels(which), C.byref(p), C.byref(prm), _f32(s), _f32(vol))
    return vol, s


def l1_norm(v, fp64=False):
    f = port_lib().oracle_l1_norm_fp64 if fp64 else port_lib().oracle_l1_norm
    return float(f(_f32(v), v.shape[1], v.shape[0]))


def dot_product(a, b, fp64=False):
    f = port_lib().oracle_dot_product_fp64 if fp64 else port_lib().oracle_dot_product
    return float(f(_f32(a), _f32(b), a.shape[1], a.shape[0]))


# ---- FP64 twin ----

def forward_d(p: Projector, vol):
    sino = np.zeros((p.n_angles, p.n_dets), np.float64)
    port_lib().oracle_forward_d(C.byref(p), _f64(np.ascontiguousarray(vol, np.float64)), _f64(sino))
    return sino


def backward_d(p: Projector, sino):
    vol = np.zeros((p.n_dets, p.n_dets), np.float64)
    port_lib().oracle_backward_d(C.byref(p), _f64(vol), _f64(np.ascontiguousarray(sino, np.float64)))
    return vol


def sirt_d(p: Projector, sino, iters, relaxation=0.25):
    vol = np.zeros((p.n_dets, p.n_dets), np.float64)
    port_lib().oracle_sirt_d(C.byref(p), iters, relaxation,
                             _f64(np.ascontiguousarray(sino, np.float64)), _f64(vol))
    return vol


def sart_d(p: Projector, sino, iters, relaxation=0.25):
    vol = np.zeros((p.n_dets, p.n_dets), np.float64)
    port_lib().oracle_sart_d(C.byref(p), iters, relaxation,
                             _f64(np.ascontiguousarray(sino, np.float64)), _f64(vol))
    return vol


def asdpocs_d(p: Projector, sino, prm: AsdpocsParams):
    vol = np.zeros((p.n_dets, p.n_dets), np.float64)
    xint = np.zeros_like(vol)
    port_lib().oracle_asdpocs_d(C.byref(p), C.byref(prm),
                                _f64(np.ascontiguousarray(sino, np.float64)), _f64(vol), _f64(xint))
    return vol, xint


def asdpocs_d_state(p: Projector, sino, prm: AsdpocsParams):
    vol = np.zeros((p.n_dets, p.n_dets), np.float64)
    xint = np.zeros_like(vol)
    sc = np.zeros(4, np.float64)
    port_lib().oracle_asdpocs_d_state(C.byref(p), C.byref(prm),
                                      _f64(np.ascontiguousarray(sino, np.float64)), _f64(vol), _f64(xint), _f64(sc))
    return vol, xint, dict(zip(("dp", "dd", "dg", "dtgv"), (float(v) for v in sc)))


def sbtv_d(p: Projector, sino, prm: SbtvParams):
    s = np.array(sino, np.float64, copy=True)
    vol = np.zeros((p.n_dets, p.n_dets), np.float64)
    port_lib().oracle_sbtv_d(C.byref(p), C.byref(prm), _f64(s), _f64(vol))
    return vol


# ---- the "siddon" model (siddon.c): double precision, pinned by the
# analytic chord of a uniform image and by adjointness ----

def _siddon_axis(n, axis):
    return np.float32(0.5 * n) if axis < 0 else np.float32(axis)


def siddon_forward(n, n_angles, step, vol, axis=-1.0):
    s, c = lut(n_angles, np.float32(step))
    sino = np.zeros((n_angles, n), np.float64)
    port_lib().oracle_siddon_forward(n, n_angles, _f32(s), _f32(c), _siddon_axis(n, axis),
                                     _f32(np.ascontiguousarray(vol, np.float32)), _f64(sino))
    return sino


def siddon_backward(n, n_angles, step, sino, axis=-1.0):
    s, c = lut(n_angles, np.float32(step))
    vol = np.zeros((n, n), np.float64)
    port_lib().oracle_siddon_backward(n, n_angles, _f32(s), _f32(c), _siddon_axis(n, axis),
                                      _f32(np.ascontiguousarray(sino, np.float32)), _f64(vol))
    return vol


def siddon_chords(n, n_angles, step, axis=-1.0):
    """Projection of an image of ones: each ray's chord through the image square."""
    s, c = lut(n_angles, np.float32(step))
    ax = _siddon_axis(n, axis)
    lib = port_lib()
    return np.array([[lib.oracle_siddon_chord(n, s[a], c[a], ax, k) for k in range(n)]
                     for a in range(n_angles)], np.float64)
