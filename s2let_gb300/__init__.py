"""GB300-native S2LET: directional and axisymmetric scale-discretised wavelet
transforms on McEwen-Wiaux sampling, computed by hand-written sm_103a kernels
behind a C ABI that mirrors the reference's (include/s2let_gpu.h).

* ``s2let_gb300.capi``     ctypes description of the C ABI (S2letParameters, S2let)
* ``s2let_gb300.pys2let``  pys2let-compatible functions (numpy in, numpy out)
* ``s2let_gb300.torch_ops`` batched torch front-end with exact adjoints for autograd
"""
from __future__ import annotations

from ._lib import LIB_PATH, check, load
from .capi import S2let, S2letParameters, make_parameters

_api = None


def api() -> S2let:
    """numpy front-end bound to the GPU library."""
    global _api
    if _api is None:
        _api = S2let(load())
    return _api


__all__ = ["LIB_PATH", "S2let", "S2letParameters", "api", "check", "load", "make_parameters"]
