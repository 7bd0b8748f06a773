"""Python binding of libufoir.so (the C ABI declared in include/ufoir.h).

This is the ctypes stub a caller of the library writes; tests and the
benchmark go through it, so every call below crosses the C ABI. There is no
fallback: if the shared library is missing or a call fails, an exception is
raised.

Arrays: numpy float32, C-contiguous. Sinograms are ``[..., n_angles, n_dets]``,
volumes ``[..., n_dets, n_dets]``; a leading axis holds independent slices.
Device-resident data are held in :class:`DeviceArray` (memory owned by a
:class:`Context`); every data argument accepts either.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

PKG_DIR = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG_DIR, "libufoir.so")

OK = 0
ERR_INVALID = -1
ERR_CUDA = -2
ERR_NOMEM = -3
ERR_UNSUPPORTED = -4
ERR_BUDGET = -5
ERR_TIMEOUT = -6
ERR_CANCELLED = -7
ERR_STATE = -8
ERR_NOT_FOUND = -9
ERR_IO = -10

HORIZONTAL = 0
VERTICAL = 1
NORM_COMPAT = 0
NORM_FP64 = 1
ARITH_EXACT = 0
ARITH_FAST = 1
AUTOTUNE_OFF, AUTOTUNE_ON, AUTOTUNE_AUTO = 0, 1, 2


class UfoirError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"ufoir status {status}: {message}")
        self.status = status


class ProjectorParams(C.Structure):
    _fields_ = [("model", C.c_char * 32), ("angles_num", C.c_uint), ("is_forward", C.c_int),
                ("axis_position", C.c_float), ("step", C.c_float), ("relaxation", C.c_float),
                ("correction_scale", C.c_float), ("arithmetic", C.c_int)]


class Subset(C.Structure):
    _fields_ = [("offset", C.c_uint), ("n", C.c_uint), ("direction", C.c_int)]


class SartParams(C.Structure):
    _fields_ = [("num_iterations", C.c_uint), ("relaxation_factor", C.c_float)]


SirtParams = SartParams


class AsdpocsParams(C.Structure):
    _fields_ = [("num_iterations", C.c_uint), ("beta", C.c_float), ("beta_red", C.c_float),
                ("alpha", C.c_float), ("alpha_red", C.c_float), ("r_max", C.c_float),
                ("ng", C.c_uint), ("positive_constraint", C.c_int), ("df_minimizer", SartParams),
                ("norm_mode", C.c_int)]


class AsdpocsScalars(C.Structure):
    _fields_ = [("dp", C.c_float), ("dd", C.c_float), ("dg", C.c_float), ("dtgv", C.c_float)]


class FpTuning(C.Structure):
    _fields_ = [("J", C.c_int), ("A", C.c_int), ("win", C.c_int), ("K", C.c_int), ("dsplit", C.c_int),
                ("threads", C.c_int), ("tuned", C.c_int), ("candidates", C.c_uint), ("ms_default", C.c_float),
                ("ms_tuned", C.c_float)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class BatchJob(C.Structure):
    _fields_ = [("n_dets", C.c_uint), ("n_angles", C.c_uint), ("step", C.c_float), ("axis_position", C.c_float),
                ("relaxation_factor", C.c_float), ("sino", C.c_void_p), ("vol", C.c_void_p), ("keep_vol", C.c_int),
                ("arithmetic", C.c_int)]


class SbtvParams(C.Structure):
    _fields_ = [("num_iterations", C.c_uint), ("lambda_", C.c_float), ("mu", C.c_float),
                ("norm_mode", C.c_int)]


METHOD_SART = 0
METHOD_SIRT = 1
METHOD_ASDPOCS = 2
METHOD_SBTV = 3
PATH_MAX = 1024


class Graph(C.Structure):
    """ufoir_graph: a parsed ufo-core JSON graph (read -> method -> write)."""
    _fields_ = [("method", C.c_int), ("projector", ProjectorParams), ("sart", SartParams),
                ("asdpocs", AsdpocsParams), ("sbtv", SbtvParams), ("read_path", C.c_char * PATH_MAX),
                ("read_raw_width", C.c_uint), ("read_raw_height", C.c_uint), ("read_raw_offset", C.c_uint64),
                ("write_filename", C.c_char * PATH_MAX)]
JOB_QUEUED, JOB_RUNNING, JOB_DONE, JOB_FAILED, JOB_CANCELLED = 0, 1, 2, 3, 4
SERVE_CONTINUOUS = 0
SERVE_ONE_AT_A_TIME = 1
SERVE_SJF_ONE_AT_A_TIME = 2


class JobDesc(C.Structure):
    _fields_ = [("method", C.c_int), ("n_dets", C.c_uint), ("n_angles", C.c_uint), ("step", C.c_float),
                ("axis_position", C.c_float), ("sart", SartParams), ("asdpocs", AsdpocsParams)]


class ServeConfig(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_uint64), ("max_active_jobs", C.c_uint), ("policy", C.c_int),
                ("quantum", C.c_uint), ("fail_allocation_every", C.c_uint), ("max_running", C.c_uint),
                ("admit_age_ms", C.c_uint), ("batch_sirt", C.c_uint)]


class ServeStats(C.Structure):
    _fields_ = [("submitted", C.c_uint64), ("completed", C.c_uint64), ("failed", C.c_uint64),
                ("cancelled", C.c_uint64), ("rejected", C.c_uint64), ("p50_latency_ms", C.c_double),
                ("p99_latency_ms", C.c_double), ("mean_latency_ms", C.c_double), ("max_latency_ms", C.c_double),
                ("p50_queue_ms", C.c_double), ("p99_queue_ms", C.c_double),
                ("throughput_jobs_per_s", C.c_double), ("busy_seconds", C.c_double),
                ("peak_hbm_bytes", C.c_uint64), ("peak_active_jobs", C.c_uint),
                ("batched_iterations", C.c_uint64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_lib = None

# Every symbol include/ufoir.h declares (checked by the CPU test suite).
EXPORTED = (
    "ufoir_ctx_create", "ufoir_ctx_destroy", "ufoir_last_error", "ufoir_ctx_synchronize",
    "ufoir_ctx_stream", "ufoir_ctx_set_stream", "ufoir_device_alloc", "ufoir_device_free", "ufoir_host_alloc",
    "ufoir_host_free", "ufoir_memcpy", "ufoir_ctx_kernel_launches",
    "ufoir_projector_params_init", "ufoir_projector_create", "ufoir_projector_destroy",
    "ufoir_projector_get_params", "ufoir_projector_set_params", "ufoir_projector_get_requisition",
    "ufoir_projector_process", "ufoir_projector_forward", "ufoir_projector_backward",
    "ufoir_projector_subset_fp", "ufoir_projector_subset_bp", "ufoir_projector_get_host_sin_vals",
    "ufoir_projector_get_host_cos_vals", "ufoir_projector_get_subsets",
    "ufoir_sart_params_init", "ufoir_sirt_params_init", "ufoir_asdpocs_params_init",
    "ufoir_sbtv_params_init", "ufoir_sart_process", "ufoir_sirt_process", "ufoir_asdpocs_process",
    "ufoir_sbtv_process", "ufoir_l1_norm", "ufoir_dot_product",
    "ufoir_sirt_batch_create", "ufoir_sirt_batch_run", "ufoir_sirt_batch_reset",
    "ufoir_sirt_batch_profile", "ufoir_sirt_batch_destroy", "ufoir_ctx_timer_begin",
    "ufoir_ctx_timer_end", "ufoir_serve_config_init", "ufoir_job_desc_init", "ufoir_serve_create",
    "ufoir_serve_submit", "ufoir_serve_poll", "ufoir_serve_wait", "ufoir_serve_cancel", "ufoir_serve_drain",
    "ufoir_serve_get_stats", "ufoir_serve_destroy", "ufoir_graph_parse", "ufoir_graph_load",
    "ufoir_graph_job_desc", "ufoir_graph_run", "ufoir_io_last_error", "ufoir_io_tiff_info", "ufoir_io_read_tiff",
    "ufoir_io_write_tiff", "ufoir_io_read_raw", "ufoir_io_write_raw", "ufoir_sample_ceiling", "ufoir_sample_ceiling_bp",
    "ufoir_asdpocs_process_ex", "ufoir_tv_gradient", "ufoir_ctx_inject_copy_timeout",
    "ufoir_ctx_set_autotune", "ufoir_projector_autotune", "ufoir_batch_create", "ufoir_batch_run",
    "ufoir_batch_set_active", "ufoir_batch_launches", "ufoir_batch_destroy", "ufoir_ctx_sm_count",
)


def lib():
    """Load libufoir.so (built by ``make -C ufo-ir_gb300``); raises if absent."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: build it with __graft_entry__.build() "
                              "or `make -C ufo-ir_gb300`")
        L = C.CDLL(LIB_PATH)
        _declare(L)
        _lib = L
    return _lib


def _declare(L):
    vp, f32p, szp = C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_size_t)
    L.ufoir_ctx_create.argtypes = [C.c_int, C.c_uint64, C.POINTER(vp)]
    L.ufoir_ctx_destroy.argtypes = [vp]
    L.ufoir_ctx_destroy.restype = None
    L.ufoir_last_error.argtypes = [vp]
    L.ufoir_last_error.restype = C.c_char_p
    L.ufoir_ctx_synchronize.argtypes = [vp]
    L.ufoir_ctx_stream.argtypes = [vp]
    L.ufoir_ctx_stream.restype = vp
    L.ufoir_ctx_set_stream.argtypes = [vp, vp]
    L.ufoir_device_alloc.argtypes = [vp, C.c_size_t, C.POINTER(vp)]
    L.ufoir_device_free.argtypes = [vp, vp]
    L.ufoir_host_alloc.argtypes = [vp, C.c_size_t, C.POINTER(vp)]
    L.ufoir_host_free.argtypes = [vp, vp]
    L.ufoir_memcpy.argtypes = [vp, vp, vp, C.c_size_t]
    L.ufoir_ctx_kernel_launches.argtypes = [vp]
    L.ufoir_ctx_kernel_launches.restype = C.c_uint64
    L.ufoir_ctx_timer_begin.argtypes = [vp]
    L.ufoir_ctx_timer_end.argtypes = [vp, f32p]
    L.ufoir_projector_params_init.argtypes = [C.POINTER(ProjectorParams)]
    L.ufoir_projector_params_init.restype = None
    L.ufoir_projector_create.argtypes = [vp, C.POINTER(ProjectorParams), C.POINTER(vp)]
    L.ufoir_projector_destroy.argtypes = [vp]
    L.ufoir_projector_destroy.restype = None
    L.ufoir_projector_get_params.argtypes = [vp, C.POINTER(ProjectorParams)]
    L.ufoir_projector_set_params.argtypes = [vp, C.POINTER(ProjectorParams)]
    L.ufoir_projector_get_requisition.argtypes = [vp, szp, szp]
    L.ufoir_projector_process.argtypes = [vp, vp, szp, vp, C.c_size_t]
    L.ufoir_projector_forward.argtypes = [vp, vp, vp, C.c_size_t, C.c_size_t, C.c_size_t]
    L.ufoir_projector_backward.argtypes = [vp, vp, vp, C.c_size_t, C.c_size_t, C.c_size_t]
    L.ufoir_projector_subset_fp.argtypes = [vp, vp, vp, C.POINTER(Subset)]
    L.ufoir_projector_subset_bp.argtypes = [vp, vp, vp, C.POINTER(Subset)]
    L.ufoir_projector_get_host_sin_vals.argtypes = [vp]
    L.ufoir_projector_get_host_sin_vals.restype = f32p
    L.ufoir_projector_get_host_cos_vals.argtypes = [vp]
    L.ufoir_projector_get_host_cos_vals.restype = f32p
    L.ufoir_projector_get_subsets.argtypes = [vp, C.POINTER(C.POINTER(Subset)), C.POINTER(C.c_uint)]
    for name, T in (("sart", SartParams), ("sirt", SartParams), ("asdpocs", AsdpocsParams),
                    ("sbtv", SbtvParams)):
        getattr(L, f"ufoir_{name}_params_init").argtypes = [C.POINTER(T)]
        getattr(L, f"ufoir_{name}_params_init").restype = None
        getattr(L, f"ufoir_{name}_process").argtypes = [vp, C.POINTER(T), vp, szp, vp, C.c_size_t]
    L.ufoir_sirt_batch_create.argtypes = [vp, C.POINTER(SartParams), vp, szp, vp, C.c_size_t, C.POINTER(vp)]
    L.ufoir_sirt_batch_run.argtypes = [vp, C.c_uint]
    L.ufoir_sirt_batch_reset.argtypes = [vp]
    L.ufoir_sirt_batch_profile.argtypes = [vp, f32p]
    L.ufoir_sirt_batch_destroy.argtypes = [vp]
    L.ufoir_sirt_batch_destroy.restype = None
    L.ufoir_serve_config_init.argtypes = [C.POINTER(ServeConfig)]
    L.ufoir_serve_config_init.restype = None
    L.ufoir_job_desc_init.argtypes = [C.POINTER(JobDesc)]
    L.ufoir_job_desc_init.restype = None
    L.ufoir_serve_create.argtypes = [vp, C.POINTER(ServeConfig), C.POINTER(vp)]
    L.ufoir_serve_submit.argtypes = [vp, C.POINTER(JobDesc), vp, vp, C.POINTER(C.c_uint64)]
    L.ufoir_serve_poll.argtypes = [vp, C.c_uint64, C.POINTER(C.c_int)]
    L.ufoir_serve_wait.argtypes = [vp, C.c_uint64, C.c_int]
    L.ufoir_serve_cancel.argtypes = [vp, C.c_uint64]
    L.ufoir_serve_drain.argtypes = [vp, C.c_int]
    L.ufoir_serve_get_stats.argtypes = [vp, C.POINTER(ServeStats)]
    L.ufoir_serve_destroy.argtypes = [vp]
    L.ufoir_serve_destroy.restype = None
    L.ufoir_graph_parse.argtypes = [C.c_char_p, C.c_size_t, C.POINTER(Graph), C.c_char_p, C.c_size_t]
    L.ufoir_graph_load.argtypes = [C.c_char_p, C.POINTER(Graph), C.c_char_p, C.c_size_t]
    L.ufoir_graph_job_desc.argtypes = [C.POINTER(Graph), C.c_uint, C.c_uint, C.POINTER(JobDesc)]
    L.ufoir_graph_run.argtypes = [vp, C.POINTER(Graph), C.POINTER(C.c_uint)]
    L.ufoir_io_last_error.argtypes = []
    L.ufoir_io_last_error.restype = C.c_char_p
    L.ufoir_io_tiff_info.argtypes = [C.c_char_p, C.POINTER(C.c_uint), C.POINTER(C.c_uint), C.POINTER(C.c_uint)]
    L.ufoir_io_read_tiff.argtypes = [C.c_char_p, C.c_uint, vp, C.c_size_t]
    L.ufoir_io_write_tiff.argtypes = [C.c_char_p, vp, C.c_uint, C.c_uint, C.c_uint]
    L.ufoir_io_read_raw.argtypes = [C.c_char_p, C.c_uint64, vp, C.c_size_t]
    L.ufoir_io_write_raw.argtypes = [C.c_char_p, vp, C.c_size_t]
    L.ufoir_sample_ceiling.argtypes = [vp, C.POINTER(C.c_double)]
    L.ufoir_sample_ceiling_bp.argtypes = [vp, C.POINTER(C.c_double)]
    L.ufoir_l1_norm.argtypes = [vp, vp, C.c_size_t, C.c_size_t, C.c_int, f32p]
    L.ufoir_dot_product.argtypes = [vp, vp, vp, C.c_size_t, C.c_size_t, C.c_int, f32p]
    L.ufoir_asdpocs_process_ex.argtypes = [vp, C.POINTER(AsdpocsParams), vp, szp, vp, C.c_size_t, vp,
                                           C.POINTER(AsdpocsScalars)]
    L.ufoir_tv_gradient.argtypes = [vp, vp, C.c_size_t, C.c_size_t, C.c_size_t, vp]
    L.ufoir_ctx_inject_copy_timeout.argtypes = [vp, C.c_int]
    L.ufoir_ctx_set_autotune.argtypes = [vp, C.c_int]
    L.ufoir_ctx_sm_count.argtypes = [vp]
    L.ufoir_projector_autotune.argtypes = [vp, C.c_size_t, C.POINTER(FpTuning)]
    L.ufoir_batch_create.argtypes = [vp, C.POINTER(BatchJob), C.c_size_t, C.POINTER(vp)]
    L.ufoir_batch_run.argtypes = [vp, C.c_uint]
    L.ufoir_batch_set_active.argtypes = [vp, C.c_size_t, C.c_int]
    L.ufoir_batch_launches.argtypes = [vp, C.POINTER(C.c_uint), C.POINTER(C.c_uint)]
    L.ufoir_batch_destroy.argtypes = [vp]
    L.ufoir_batch_destroy.restype = None


class DeviceArray:
    """float32 array in the context's GPU memory (owned; freed on close())."""

    def __init__(self, ctx: "Context", shape, zero: bool = False):
        self.ctx = ctx
        self.shape = tuple(int(s) for s in shape)
        self.size = int(np.prod(self.shape))
        self.nbytes = 4 * self.size
        p = C.c_void_p()
        ctx._check(lib().ufoir_device_alloc(ctx.handle, max(self.nbytes, 16), C.byref(p)))
        self.ptr = p.value
        if zero:
            self.upload(np.zeros(self.shape, np.float32))

    @classmethod
    def from_numpy(cls, ctx: "Context", a: np.ndarray) -> "DeviceArray":
        a = np.ascontiguousarray(a, np.float32)
        d = cls(ctx, a.shape)
        d.upload(a)
        return d

    def upload(self, a: np.ndarray) -> None:
        a = np.ascontiguousarray(a, np.float32)
        assert a.size == self.size
        self.ctx._check(lib().ufoir_memcpy(self.ctx.handle, self.ptr, a.ctypes.data, self.nbytes))

    def download(self) -> np.ndarray:
        out = np.empty(self.shape, np.float32)
        self.ctx._check(lib().ufoir_memcpy(self.ctx.handle, out.ctypes.data, self.ptr, self.nbytes))
        return out

    def slice(self, i: int) -> "DeviceArray":
        """Non-owning view of the i-th entry along the leading axis."""
        v = DeviceArray.__new__(DeviceArray)
        v.ctx = self.ctx
        v.shape = self.shape[1:]
        v.size = int(np.prod(v.shape))
        v.nbytes = 4 * v.size
        v.ptr = self.ptr + i * v.nbytes
        v._view = True
        return v

    def close(self) -> None:
        if self.ptr and not getattr(self, "_view", False):
            lib().ufoir_device_free(self.ctx.handle, self.ptr)
        self.ptr = None


def _ptr(a):
    if isinstance(a, DeviceArray):
        return a.ptr
    assert isinstance(a, np.ndarray) and a.dtype == np.float32 and a.flags.c_contiguous, \
        "host arrays must be C-contiguous float32"
    return a.ctypes.data


def _shape(a):
    return a.shape


class Context:
    """One GPU context (ufoir_ctx)."""

    def __init__(self, device: int = 0, hbm_budget: int = 0):
        h = C.c_void_p()
        rc = lib().ufoir_ctx_create(device, hbm_budget, C.byref(h))
        if rc != OK:
            raise UfoirError(rc, lib().ufoir_last_error(None).decode())
        self.handle = h.value

    def _check(self, rc):
        if rc != OK:
            raise UfoirError(rc, lib().ufoir_last_error(self.handle).decode())
        return rc

    def last_error(self) -> str:
        return lib().ufoir_last_error(self.handle).decode()

    def synchronize(self):
        self._check(lib().ufoir_ctx_synchronize(self.handle))

    def kernel_launches(self) -> int:
        return int(lib().ufoir_ctx_kernel_launches(self.handle))

    def stream(self) -> int:
        return lib().ufoir_ctx_stream(self.handle)

    def timer_begin(self):
        self._check(lib().ufoir_ctx_timer_begin(self.handle))

    def timer_end(self) -> float:
        """Elapsed device milliseconds since timer_begin (CUDA events on the library's stream)."""
        ms = C.c_float()
        self._check(lib().ufoir_ctx_timer_end(self.handle, C.byref(ms)))
        return ms.value

    def set_stream(self, stream):
        """Queue this context's work on `stream` (a cudaStream_t as int; None: its own stream)."""
        self._check(lib().ufoir_ctx_set_stream(self.handle, stream))

    def sample_ceiling(self) -> float:
        """Interpolated samples/s of the forward projector's per-sample sequence, no global traffic."""
        v = C.c_double()
        self._check(lib().ufoir_sample_ceiling(self.handle, C.byref(v)))
        return v.value

    def sample_ceiling_bp(self) -> float:
        """Interpolated samples/s of the backprojector's per-sample sequence, no global traffic."""
        v = C.c_double()
        self._check(lib().ufoir_sample_ceiling_bp(self.handle, C.byref(v)))
        return v.value

    def pinned_empty(self, shape):
        """numpy array backed by page-locked host memory (freed with the context)."""
        n = int(np.prod(shape)) * 4
        p = C.c_void_p()
        self._check(lib().ufoir_host_alloc(self.handle, n, C.byref(p)))
        buf = (C.c_float * (n // 4)).from_address(p.value)
        arr = np.frombuffer(buf, np.float32).reshape(shape)
        self._pinned = getattr(self, "_pinned", []) + [p.value]
        return arr

    def close(self):
        if getattr(self, "handle", None):
            for p in getattr(self, "_pinned", []):
                lib().ufoir_host_free(self.handle, p)
            self._pinned = []
            lib().ufoir_ctx_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def sm_count(self) -> int:
        return int(lib().ufoir_ctx_sm_count(self.handle))

    def set_autotune(self, on):
        """False/True (off/on) or AUTOTUNE_AUTO (the default)."""
        mode = on if isinstance(on, int) and not isinstance(on, bool) else int(bool(on))
        self._check(lib().ufoir_ctx_set_autotune(self.handle, mode))

    def l1_norm(self, v, mode=NORM_FP64) -> float:
        out = C.c_float()
        h, w = _shape(v)[-2:]
        self._check(lib().ufoir_l1_norm(self.handle, _ptr(v), w, h, mode, C.byref(out)))
        return out.value

    def dot_product(self, a, b, mode=NORM_FP64) -> float:
        out = C.c_float()
        h, w = _shape(a)[-2:]
        self._check(lib().ufoir_dot_product(self.handle, _ptr(a), _ptr(b), w, h, mode, C.byref(out)))
        return out.value


def projector_params(**kw) -> ProjectorParams:
    p = ProjectorParams()
    lib().ufoir_projector_params_init(C.byref(p))
    for k, v in kw.items():
        if k == "model":
            v = v.encode()
        setattr(p, k, v)
    return p


class ParallelProjector:
    """The "parallel-projector" plugin: properties mirror the reference's."""

    def __init__(self, ctx: Context, **props):
        self.ctx = ctx
        prm = projector_params(**props)
        h = C.c_void_p()
        ctx._check(lib().ufoir_projector_create(ctx.handle, C.byref(prm), C.byref(h)))
        self.handle = h.value

    def close(self):
        if self.handle:
            lib().ufoir_projector_destroy(self.handle)
            self.handle = None

    @property
    def params(self) -> ProjectorParams:
        p = ProjectorParams()
        self.ctx._check(lib().ufoir_projector_get_params(self.handle, C.byref(p)))
        return p

    def set(self, **props):
        p = self.params
        for k, v in props.items():
            if k == "model":
                v = v.encode()
            setattr(p, k, v)
        self.ctx._check(lib().ufoir_projector_set_params(self.handle, C.byref(p)))

    def get_requisition(self, in_dims):
        i = (C.c_size_t * 2)(*in_dims)
        o = (C.c_size_t * 2)()
        self.ctx._check(lib().ufoir_projector_get_requisition(self.handle, i, o))
        return (o[0], o[1])

    def process(self, inp, out=None):
        """State-dependent process: zero the output, then forward or backward."""
        h, w = _shape(inp)[-2:]
        n_slices = int(np.prod(_shape(inp)[:-2])) if len(_shape(inp)) > 2 else 1
        dims = (C.c_size_t * 2)(w, h)
        od = self.get_requisition((w, h))
        if out is None:
            out = np.zeros(_shape(inp)[:-2] + (od[1], od[0]), np.float32)
        self.ctx._check(lib().ufoir_projector_process(self.handle, _ptr(inp), dims, _ptr(out), n_slices))
        return out

    def forward(self, vol, sino):
        """sino += correction_scale * A vol (accumulating, all subsets)."""
        n_angles, n = _shape(sino)[-2:]
        n_slices = int(np.prod(_shape(sino)[:-2])) if len(_shape(sino)) > 2 else 1
        self.ctx._check(lib().ufoir_projector_forward(self.handle, _ptr(vol), _ptr(sino), n, n_angles, n_slices))
        return sino

    def backward(self, vol, sino):
        """vol += relaxation * A^T sino (accumulating, all subsets)."""
        n_angles, n = _shape(sino)[-2:]
        n_slices = int(np.prod(_shape(sino)[:-2])) if len(_shape(sino)) > 2 else 1
        self.ctx._check(lib().ufoir_projector_backward(self.handle, _ptr(vol), _ptr(sino), n, n_angles, n_slices))
        return vol

    def subset_fp(self, vol, sino, offset, n, direction):
        s = Subset(offset, n, direction)
        self.ctx._check(lib().ufoir_projector_subset_fp(self.handle, _ptr(vol), _ptr(sino), C.byref(s)))
        return sino

    def subset_bp(self, vol, sino, offset, n, direction):
        s = Subset(offset, n, direction)
        self.ctx._check(lib().ufoir_projector_subset_bp(self.handle, _ptr(vol), _ptr(sino), C.byref(s)))
        return vol

    def host_sin_cos(self):
        s = lib().ufoir_projector_get_host_sin_vals(self.handle)
        c = lib().ufoir_projector_get_host_cos_vals(self.handle)
        if not s:
            return None, None
        n = self.params.angles_num
        return (np.ctypeslib.as_array(s, (n,)).copy(), np.ctypeslib.as_array(c, (n,)).copy())

    def autotune(self, n_slices: int = 1) -> dict:
        """Searches the forward projector's launch shapes for this geometry
        (ufoir_projector_autotune); the geometry must be set."""
        t = FpTuning()
        self.ctx._check(lib().ufoir_projector_autotune(self.handle, n_slices, C.byref(t)))
        return t.as_dict()

    def subsets(self):
        p = C.POINTER(Subset)()
        n = C.c_uint()
        rc = lib().ufoir_projector_get_subsets(self.handle, C.byref(p), C.byref(n))
        if rc != OK:
            return []
        return [(p[i].offset, p[i].n, p[i].direction) for i in range(n.value)]


def _method_params(T, init, **kw):
    p = T()
    init(C.byref(p))
    for k, v in kw.items():
        if k == "df_minimizer":
            p.df_minimizer = v if isinstance(v, SartParams) else _method_params(
                SartParams, lib().ufoir_sart_params_init, **v)
        else:
            setattr(p, "lambda_" if k == "lambda" else k, v)
    return p


def sart_params(**kw) -> SartParams:
    return _method_params(SartParams, lib().ufoir_sart_params_init, **kw)


def sirt_params(**kw) -> SartParams:
    return _method_params(SartParams, lib().ufoir_sirt_params_init, **kw)


def asdpocs_params(**kw) -> AsdpocsParams:
    return _method_params(AsdpocsParams, lib().ufoir_asdpocs_params_init, **kw)


def sbtv_params(**kw) -> SbtvParams:
    return _method_params(SbtvParams, lib().ufoir_sbtv_params_init, **kw)


def _run_method(name, proj: ParallelProjector, prm, sino, vol=None):
    n_angles, n = _shape(sino)[-2:]
    lead = _shape(sino)[:-2]
    n_slices = int(np.prod(lead)) if lead else 1
    if vol is None:
        vol = np.zeros(lead + (n, n), np.float32)
    dims = (C.c_size_t * 2)(n, n_angles)
    fn = getattr(lib(), f"ufoir_{name}_process")
    proj.ctx._check(fn(proj.handle, C.byref(prm), _ptr(sino), dims, _ptr(vol), n_slices))
    return vol


class SirtBatch:
    """Resident batched SIRT over device arrays (ufoir_sirt_batch_*)."""

    def __init__(self, proj: ParallelProjector, sino: DeviceArray, vol: DeviceArray, **kw):
        self.proj = proj
        n_angles, n = sino.shape[-2:]
        n_slices = int(np.prod(sino.shape[:-2])) if len(sino.shape) > 2 else 1
        prm = sirt_params(**kw)
        dims = (C.c_size_t * 2)(n, n_angles)
        h = C.c_void_p()
        proj.ctx._check(lib().ufoir_sirt_batch_create(proj.handle, C.byref(prm), sino.ptr, dims, vol.ptr,
                                                      n_slices, C.byref(h)))
        self.handle = h.value

    def run(self, iterations: int = 1):
        self.proj.ctx._check(lib().ufoir_sirt_batch_run(self.handle, iterations))

    def reset(self):
        self.proj.ctx._check(lib().ufoir_sirt_batch_reset(self.handle))

    def profile(self):
        ms = (C.c_float * 3)()
        self.proj.ctx._check(lib().ufoir_sirt_batch_profile(self.handle, ms))
        return {"prepare": ms[0], "fp": ms[1], "bp": ms[2]}

    def close(self):
        if self.handle:
            lib().ufoir_sirt_batch_destroy(self.handle)
            self.handle = None


class Batch:
    """A mixed SIRT batch (ufoir_batch_*): members are (DeviceArray sinogram
    [n_angles, n_dets], DeviceArray volume [n_dets, n_dets], dict(step=...,
    axis_position=-1, relaxation_factor=0.25, keep_vol=0))."""

    def __init__(self, ctx: Context, members):
        self.ctx = ctx
        arr = (BatchJob * len(members))()
        self._keep = []
        for k, (sino, vol, kw) in enumerate(members):
            na, n = sino.shape[-2:]
            arr[k].n_dets = n
            arr[k].n_angles = na
            arr[k].step = float(np.float32(kw["step"]))
            arr[k].axis_position = float(kw.get("axis_position", -1.0))
            arr[k].relaxation_factor = float(kw.get("relaxation_factor", 0.25))
            arr[k].sino = sino.ptr
            arr[k].vol = vol.ptr
            arr[k].keep_vol = int(kw.get("keep_vol", 0))
            arr[k].arithmetic = int(kw.get("arithmetic", ARITH_EXACT))
            self._keep.append((sino, vol))
        h = C.c_void_p()
        ctx._check(lib().ufoir_batch_create(ctx.handle, arr, len(members), C.byref(h)))
        self.handle = h.value

    def run(self, iterations: int = 1):
        self.ctx._check(lib().ufoir_batch_run(self.handle, iterations))

    def set_active(self, member: int, active: bool):
        self.ctx._check(lib().ufoir_batch_set_active(self.handle, member, int(bool(active))))

    def launches(self):
        a, b = C.c_uint(), C.c_uint()
        self.ctx._check(lib().ufoir_batch_launches(self.handle, C.byref(a), C.byref(b)))
        return a.value, b.value

    def close(self):
        if self.handle:
            lib().ufoir_batch_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def sart(proj, sino, vol=None, **kw):
    return _run_method("sart", proj, sart_params(**kw), sino, vol)


def sirt(proj, sino, vol=None, **kw):
    return _run_method("sirt", proj, sirt_params(**kw), sino, vol)


def asdpocs(proj, sino, vol=None, **kw):
    return _run_method("asdpocs", proj, asdpocs_params(**kw), sino, vol)


def asdpocs_state(proj, sino, vol=None, **kw):
    """ASD-POCS returning (output, x after the last outer iteration's TV
    sub-steps, [{dp, dd, dg, dtgv} per slice]) (ufoir_asdpocs_process_ex)."""
    prm = asdpocs_params(**kw)
    n_angles, n = _shape(sino)[-2:]
    lead = _shape(sino)[:-2]
    n_slices = int(np.prod(lead)) if lead else 1
    if vol is None:
        vol = np.zeros(lead + (n, n), np.float32)
    x_tv = np.zeros(lead + (n, n), np.float32)
    sc = (AsdpocsScalars * n_slices)()
    dims = (C.c_size_t * 2)(n, n_angles)
    proj.ctx._check(lib().ufoir_asdpocs_process_ex(proj.handle, C.byref(prm), _ptr(sino), dims, _ptr(vol),
                                                   n_slices, _ptr(x_tv), sc))
    return vol, x_tv, [dict(dp=r.dp, dd=r.dd, dg=r.dg, dtgv=r.dtgv) for r in sc]


def tv_gradient(ctx, v, out=None):
    """l1_grad on one image [h, w] or a stack [s, h, w] (ufoir_tv_gradient)."""
    shp = _shape(v)
    h, w = shp[-2:]
    n_slices = int(np.prod(shp[:-2])) if len(shp) > 2 else 1
    if out is None:
        out = np.zeros(shp, np.float32)
    ctx._check(lib().ufoir_tv_gradient(ctx.handle, _ptr(v), w, h, n_slices, _ptr(out)))
    return out


def sbtv(proj, sino, vol=None, **kw):
    return _run_method("sbtv", proj, sbtv_params(**kw), sino, vol)


def job_desc(method, n_dets, n_angles, step, axis_position=-1.0, **kw) -> JobDesc:
    """A reconstruction job. kw: num_iterations / relaxation_factor (SART, SIRT)
    or asdpocs=dict(...) (ASD-POCS parameters, with df_minimizer=dict(...))."""
    j = JobDesc()
    lib().ufoir_job_desc_init(C.byref(j))
    j.method, j.n_dets, j.n_angles, j.step, j.axis_position = method, n_dets, n_angles, step, axis_position
    if "asdpocs" in kw:
        j.asdpocs = asdpocs_params(**kw.pop("asdpocs"))
    if kw:
        j.sart = sart_params(**kw)
    return j


class Server:
    """The continuous-batching request loop (ufoir_serve_*)."""

    def __init__(self, ctx: Context, hbm_budget: int = 0, max_active_jobs: int = 0,
                 policy: int = SERVE_CONTINUOUS, quantum: int = 1, fail_allocation_every: int = 0,
                 max_running: int = 0, admit_age_ms: int = 0, batch_sirt: bool = False):
        self.ctx = ctx
        cfg = ServeConfig()
        lib().ufoir_serve_config_init(C.byref(cfg))
        if admit_age_ms:
            cfg.admit_age_ms = admit_age_ms
        cfg.batch_sirt = int(bool(batch_sirt))
        cfg.hbm_budget_bytes = hbm_budget
        if max_active_jobs:
            cfg.max_active_jobs = max_active_jobs
        cfg.policy = policy
        cfg.quantum = quantum
        cfg.fail_allocation_every = fail_allocation_every
        if max_running:
            cfg.max_running = max_running
        h = C.c_void_p()
        ctx._check(lib().ufoir_serve_create(ctx.handle, C.byref(cfg), C.byref(h)))
        self.handle = h.value
        self._keep = {}

    def submit(self, job: JobDesc, sino: np.ndarray, vol: np.ndarray = None):
        """Queue a job; returns (job_id, output array). Arrays must stay alive until done."""
        if vol is None:
            vol = np.zeros((job.n_dets, job.n_dets), np.float32)
        assert sino.dtype == np.float32 and sino.flags.c_contiguous and sino.size == job.n_dets * job.n_angles
        jid = C.c_uint64()
        rc = lib().ufoir_serve_submit(self.handle, C.byref(job), sino.ctypes.data, vol.ctypes.data, C.byref(jid))
        if rc != OK:
            raise UfoirError(rc, self.ctx.last_error())
        self._keep[jid.value] = (sino, vol)
        return jid.value, vol

    def poll(self, jid: int) -> int:
        st = C.c_int()
        self.ctx._check(lib().ufoir_serve_poll(self.handle, jid, C.byref(st)))
        return st.value

    def wait(self, jid: int, timeout_ms: int = -1) -> int:
        return lib().ufoir_serve_wait(self.handle, jid, timeout_ms)

    def cancel(self, jid: int) -> int:
        return lib().ufoir_serve_cancel(self.handle, jid)

    def drain(self, timeout_ms: int = -1) -> int:
        return lib().ufoir_serve_drain(self.handle, timeout_ms)

    def stats(self) -> dict:
        s = ServeStats()
        self.ctx._check(lib().ufoir_serve_get_stats(self.handle, C.byref(s)))
        return s.as_dict()

    def close(self):
        if self.handle:
            lib().ufoir_serve_destroy(self.handle)
            self.handle = None
            self._keep.clear()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


# ---------------------------------------------------------------- graphs, I/O

def graph_parse(text: str) -> Graph:
    """Parse a ufo-core JSON graph (read -> ufo-ir method -> write)."""
    g = Graph()
    err = C.create_string_buffer(512)
    b = text.encode()
    rc = lib().ufoir_graph_parse(b, len(b), C.byref(g), err, len(err))
    if rc != OK:
        raise UfoirError(rc, err.value.decode())
    return g


def graph_load(path: str) -> Graph:
    g = Graph()
    err = C.create_string_buffer(512)
    rc = lib().ufoir_graph_load(path.encode(), C.byref(g), err, len(err))
    if rc != OK:
        raise UfoirError(rc, err.value.decode())
    return g


def graph_job_desc(g: Graph, n_dets: int, n_angles: int) -> JobDesc:
    j = JobDesc()
    rc = lib().ufoir_graph_job_desc(C.byref(g), n_dets, n_angles, C.byref(j))
    if rc != OK:
        raise UfoirError(rc, "graph_job_desc")
    return j


def graph_run(ctx: Context, g: Graph) -> int:
    """Read, reconstruct and write every slice of a parsed graph; returns the slice count."""
    n = C.c_uint()
    ctx._check(lib().ufoir_graph_run(ctx.handle, C.byref(g), C.byref(n)))
    return n.value


def _io_check(rc):
    if rc != OK:
        raise UfoirError(rc, lib().ufoir_io_last_error().decode())


def tiff_info(path: str):
    w, h, p = C.c_uint(), C.c_uint(), C.c_uint()
    _io_check(lib().ufoir_io_tiff_info(path.encode(), C.byref(w), C.byref(h), C.byref(p)))
    return w.value, h.value, p.value


def read_tiff(path: str, page: int = 0) -> np.ndarray:
    w, h, _ = tiff_info(path)
    out = np.empty((h, w), np.float32)
    _io_check(lib().ufoir_io_read_tiff(path.encode(), page, out.ctypes.data, out.size))
    return out


def write_tiff(path: str, data: np.ndarray):
    """data: (h, w) or (pages, h, w) float32."""
    a = np.ascontiguousarray(data, np.float32)
    pages = 1 if a.ndim == 2 else a.shape[0]
    _io_check(lib().ufoir_io_write_tiff(path.encode(), a.ctypes.data, a.shape[-1], a.shape[-2], pages))


def read_raw(path: str, shape, offset: int = 0) -> np.ndarray:
    out = np.empty(shape, np.float32)
    _io_check(lib().ufoir_io_read_raw(path.encode(), offset, out.ctypes.data, out.size))
    return out


def write_raw(path: str, data: np.ndarray):
    a = np.ascontiguousarray(data, np.float32)
    _io_check(lib().ufoir_io_write_raw(path.encode(), a.ctypes.data, a.size))
