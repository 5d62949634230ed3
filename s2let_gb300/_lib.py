"""Locates and loads the in-tree libs2let_gpu.so (built by s2let_gb300/build.py).

There is no CPU fallback: if the library has not been built, loading fails with
an error that says how to build it.
"""
from __future__ import annotations

import ctypes as C
import os

from .capi import FITS_SIGNATURES, GPU_SIGNATURES, SIGNATURES, bind

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "lib", "libs2let_gpu.so")

_lib = None


def load() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it with `python -m s2let_gb300.build` "
                "(nvcc with sm_103a support required)")
        lib = C.CDLL(LIB_PATH, mode=os.RTLD_LOCAL)
        bind(lib, SIGNATURES, required=False)
        bind(lib, GPU_SIGNATURES, required=False)
        bind(lib, FITS_SIGNATURES, required=False)
        _lib = lib
    return _lib


def check(lib: C.CDLL, what: str = "") -> None:
    """Raise if the last call on this thread reported an error."""
    code = lib.s2let_gpu_last_error()
    if code != 0:
        msg = lib.s2let_gpu_last_error_string().decode(errors="replace")
        raise RuntimeError(f"s2let_gpu error {code} {what}: {msg}")
