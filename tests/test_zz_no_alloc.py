"""The hard threshold that stages through a static device array instead of
allocating: same result as the allocating entry point on two calls in a row
(the second smaller, so stale bytes from the first sit past its request), and
a clear error for requests above its 8 MiB capacity.

Kept in a file of its own, named so that pytest collects it last; it makes no
assumption about what ran before it in the process."""
import ctypes as C

import numpy as np
import pytest

from s2let_gb300.capi import make_parameters, ptr

FN = "s2let_gpu_axisym_wav_hardthreshold_real_noalloc"


def _case(gpu, L, B, J_min, multires, seed):
    p = make_parameters(L, B, J_min, 1, 0, 0)
    nw, _ = gpu.axisym_sizes(p, multires)
    J = gpu.lib.s2let_j_max(C.byref(p))
    rng = np.random.default_rng(seed)
    g0 = rng.normal(scale=3.0, size=nw)
    thr = np.linspace(0.5, 2.5, J - J_min + 1)
    return p, g0, thr


def _allocating(gpu, p, g0, thr, multires):
    g = g0.copy()
    fn = "s2let_transform_axisym_wav_hardthreshold_multires_real" if multires else \
        "s2let_transform_axisym_wav_hardthreshold_real"
    getattr(gpu.lib, fn)(ptr(g), ptr(thr), C.byref(p))
    assert gpu.lib.s2let_gpu_last_error() == 0
    return g


@pytest.mark.gpu
def test_noalloc_threshold_matches_allocating_twice(gpu):
    f = getattr(gpu.lib, FN)
    for L, B, J_min, multires, seed in ((64, 2.0, 1, False, 31), (24, 1.7, 2, True, 32)):
        p, g0, thr = _case(gpu, L, B, J_min, multires, seed)
        want = _allocating(gpu, p, g0, thr, multires)
        got = g0.copy()
        assert f(ptr(got), ptr(thr), C.byref(p), int(multires)) == 0
        np.testing.assert_array_equal(got, want)
        assert np.count_nonzero(got == 0.0) > 0 and np.count_nonzero(got) > 0


@pytest.mark.gpu
def test_noalloc_threshold_rejects_oversize(gpu):
    f = getattr(gpu.lib, FN)
    p, g0, thr = _case(gpu, 512, 2.0, 1, False, 33)
    assert g0.nbytes > 8 << 20
    g = g0.copy()
    st = f(ptr(g), ptr(thr), C.byref(p), 0)
    assert st == 1
    msg = gpu.lib.s2let_gpu_last_error_string().decode()
    assert "8 MiB" in msg and "bytes of scratch" in msg
    np.testing.assert_array_equal(g, g0)
