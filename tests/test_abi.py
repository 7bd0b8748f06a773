"""CPU tests of the C-ABI library: it loads, exports every symbol that
include/*.h declares, and fails loudly (no fallback) where there is no GPU."""
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_symbols():
    names = set()
    for h in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if not h.endswith(".h"):
            continue
        src = open(os.path.join(ROOT, "include", h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names.update(re.findall(r"UFOIR_API[^;(]*?\b(ufoir_\w+)\s*\(", src))
    return names


def test_library_exports_every_declared_symbol(ufoir_lib):
    L = ufoir_lib.lib()
    declared = _declared_symbols()
    assert len(declared) >= 30
    missing = [s for s in sorted(declared) if not hasattr(L, s)]
    assert not missing, missing
    assert set(ufoir_lib.EXPORTED) <= declared


def test_no_internal_symbols_exported(ufoir_lib):
    import subprocess
    out = subprocess.run(["nm", "-D", "--defined-only", ufoir_lib.LIB_PATH], capture_output=True, text=True)
    if out.returncode != 0:
        pytest.skip("nm unavailable")
    syms = [l.split()[-1] for l in out.stdout.splitlines() if " T " in l]
    assert syms and all(s.startswith("ufoir_") for s in syms), [s for s in syms if not s.startswith("ufoir_")]


def test_param_defaults_match_reference(ufoir_lib):
    p = ufoir_lib.projector_params()
    assert p.model == b"joseph" and p.angles_num == 0 and p.is_forward == 1
    assert p.axis_position == -1.0 and p.step == 0.0 and p.relaxation == 1.0 and p.correction_scale == 1.0
    s = ufoir_lib.sart_params()
    assert s.num_iterations == 10 and abs(s.relaxation_factor - 0.25) < 1e-9
    a = ufoir_lib.asdpocs_params()
    assert (a.num_iterations, a.ng, a.positive_constraint) == (10, 20, 1)
    assert np.float32(a.beta) == np.float32(1.0) and np.float32(a.beta_red) == np.float32(0.995)
    assert np.float32(a.alpha) == np.float32(0.2) and np.float32(a.alpha_red) == np.float32(0.95)
    assert np.float32(a.r_max) == np.float32(0.95) and a.df_minimizer.num_iterations == 10
    b = ufoir_lib.sbtv_params()
    assert np.float32(b.lambda_) == np.float32(0.1) and np.float32(b.mu) == np.float32(0.5)
    assert a.norm_mode == ufoir_lib.NORM_FP64 == b.norm_mode


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_has_gpu(), reason="checks the behaviour without a GPU")
def test_context_creation_fails_loudly_without_gpu(ufoir_lib):
    with pytest.raises(ufoir_lib.UfoirError) as e:
        ufoir_lib.Context(0)
    assert e.value.status in (ufoir_lib.ERR_CUDA, ufoir_lib.ERR_INVALID)


def test_null_arguments_are_rejected_without_a_context(ufoir_lib):
    L = ufoir_lib.lib()
    assert L.ufoir_ctx_create(0, 0, None) == ufoir_lib.ERR_INVALID
    assert L.ufoir_sirt_process(None, None, None, None, None, 1) == ufoir_lib.ERR_INVALID
    assert L.ufoir_projector_create(None, None, None) == ufoir_lib.ERR_INVALID
