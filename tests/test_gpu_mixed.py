"""Split-precision (bf16-digit tcgen05) contraction against the FP64 path.

The mixed path must stay within 1e-10 normwise relative max error
(max|a - b| / max|b|) of the FP64 results for every output, and raise no
device fault.  Band-limits >= 128 take the tensor-core kernel; smaller scales
keep the FP64 kernel inside the same call."""
import numpy as np
import pytest

from conftest import random_flm, rel_err
from s2let_gb300.capi import make_parameters

TOL_MIXED = 1e-10

CASES = [
    # L, N, B, J_min, spin, upsample
    (256, 4, 2.0, 2, 0, 0),
    (200, 3, 2.0, 2, 2, 0),
    (160, 4, 2.0, 5, 1, 1),
]


def _both(gpu, fn):
    lib = gpu.lib
    assert lib.s2let_gpu_set_precision(0) == 0
    ref = fn()
    assert lib.s2let_gpu_set_precision(1) == 0
    try:
        got = fn()
    finally:
        lib.s2let_gpu_set_precision(0)
    assert lib.s2let_gpu_device_fault() == 0
    return got, ref


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES, ids=lambda c: "L{}_N{}_s{}_up{}".format(c[0], c[1], c[4], c[5]))
def test_mixed_px2wav_wav2px(gpu, case):
    L, N, B, J_min, spin, up = case
    p = make_parameters(L, B, J_min, N, spin, up)
    rng = np.random.default_rng(40 + L)
    f = gpu.alm2map(random_flm(rng, L, spin), L, spin)
    (w, s), (w0, s0) = _both(gpu, lambda: gpu.px2wav(f, p))
    assert rel_err(w, w0) < TOL_MIXED and rel_err(s, s0) < TOL_MIXED
    r, r0 = _both(gpu, lambda: gpu.wav2px(w0, s0, p))
    assert rel_err(r, r0) < TOL_MIXED
    assert rel_err(r, f) < TOL_MIXED


@pytest.mark.gpu
def test_mixed_real_metric_shape(gpu):
    L = 512
    p = make_parameters(L, 2.0, 2, 4, 0, 0)
    rng = np.random.default_rng(7)
    f = gpu.alm2map(random_flm(rng, L, real=True, power=lambda l: 1.0 / (l + 1)), L, real=True)
    (w, s), (w0, s0) = _both(gpu, lambda: gpu.px2wav(f, p, real=True))
    assert rel_err(w, w0) < TOL_MIXED and rel_err(s, s0) < TOL_MIXED
    r, r0 = _both(gpu, lambda: gpu.wav2px(w0, s0, p, real=True))
    assert rel_err(r, r0) < TOL_MIXED


@pytest.mark.gpu
def test_mixed_sht(gpu):
    L = 300
    rng = np.random.default_rng(9)
    flm = random_flm(rng, L, 0)
    f, f0 = _both(gpu, lambda: gpu.alm2map(flm, L, 0))
    assert rel_err(f, f0) < TOL_MIXED
    a, a0 = _both(gpu, lambda: gpu.map2alm(f0, L, 0))
    assert rel_err(a, a0) < TOL_MIXED


@pytest.mark.gpu
@pytest.mark.parametrize("L,N,nb", [(256, 4, 12), (160, 3, 20), (128, 2, 70)])
def test_mixed_large_batches(gpu, L, N, nb):
    """Batches that need 48-64 coefficient columns per table pass (one 448-column
    TMEM accumulator, MMAs split at N = 256) against the FP64 path; 70 maps at
    two scales per pass make five map groups of 16, run as one launch of four
    interleaved groups and one of the remaining six maps."""
    torch = pytest.importorskip("torch")
    from s2let_gb300 import torch_ops as T

    p = make_parameters(L, 2.0, 2, N, 0, 0)
    s = T.sizes(p)
    g = torch.Generator().manual_seed(nb)
    f = (torch.rand((nb, s["n_px"]), generator=g, dtype=torch.float64) * 2 - 1).cuda()
    w0, s0 = T.px2wav(f, p, precision="fp64")
    w1, s1 = T.px2wav(f, p, precision="mixed")
    assert gpu.lib.s2let_gpu_device_fault() == 0
    rel = lambda a, b: float((a - b).abs().max() / b.abs().max())
    assert rel(w1, w0) < TOL_MIXED and rel(s1, s0) < TOL_MIXED
    r0 = T.wav2px(w0, s0, p, precision="fp64")
    r1 = T.wav2px(w0, s0, p, precision="mixed")
    assert rel(r1, r0) < TOL_MIXED
