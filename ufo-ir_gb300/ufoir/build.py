"""Builds libufoir.so in-tree (nvcc for sm_103a + gcc), used by __graft_entry__.build()."""
from __future__ import annotations

import os
import subprocess

PKG_DIR = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def build(jobs: int | None = None, quiet: bool = True) -> str:
    jobs = jobs or max(2, min(16, os.cpu_count() or 2))
    out = subprocess.run(["make", "-C", PKG_DIR, f"-j{jobs}"], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("libufoir build failed:\n" + out.stdout[-4000:] + out.stderr[-4000:])
    if not quiet:
        print(out.stdout[-2000:], end="")
    return os.path.join(PKG_DIR, "libufoir.so")
