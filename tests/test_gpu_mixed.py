"""Split-precision (bf16-digit tcgen05) contraction against the FP64 path.

The mixed path must stay within 1e-10 normwise relative max error
(max|a - b| / max|b|) of the FP64 results for every output, and raise no
device fault.  Band-limits >= 128 take the tensor-core kernel for batches of
more than s2let_gpu_get_df_max_maps() maps (default 1); one-map calls and
smaller scales contract in double-float on the Wigner tables inside the same
call.  The one-map cases cover the double-float kernel; the batch cases both."""
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


@pytest.mark.gpu
@pytest.mark.parametrize("nb,df_max", [(2, 2), (2, 1), (3, 2)])
def test_mixed_host_batch(gpu, nb, df_max):
    """Host batches of two or three maps, contracted in double-float (two
    scales of one band-limit in one pass over each table) when the batch has
    at most df_max maps, else on the tensor cores; each map against its FP64
    single call."""
    import ctypes as C

    from s2let_gb300.capi import ptr

    L = 256
    p = make_parameters(L, 2.0, 2, 4, 0, 0)
    s = gpu.sizes(p)
    rng = np.random.default_rng(11 + nb)
    f = np.ascontiguousarray(np.stack([gpu.alm2map(random_flm(rng, L, 0), L, 0) for _ in range(nb)]))
    w = np.zeros((nb, s["n_wav"]), np.complex128)
    sc = np.zeros((nb, s["n_scal"]), np.complex128)
    r = np.zeros_like(f)
    lib = gpu.lib
    rep = (C.c_double * 36)()
    old = lib.s2let_gpu_get_df_max_maps()
    assert lib.s2let_gpu_set_df_max_maps(df_max) == 0
    assert lib.s2let_gpu_set_precision(1) == 0
    try:
        lib.s2let_gpu_timing_enable(1)
        assert lib.s2let_gpu_analysis_px2wav_host_batch(ptr(w), ptr(sc), ptr(f), nb, C.byref(p)) == 0
        assert lib.s2let_gpu_synthesis_wav2px_host_batch(ptr(r), ptr(w), ptr(sc), nb, C.byref(p)) == 0
        lib.s2let_gpu_timing_report(rep, 9)
        lib.s2let_gpu_timing_enable(0)
    finally:
        lib.s2let_gpu_set_precision(0)
        lib.s2let_gpu_set_df_max_maps(old)
    assert lib.s2let_gpu_device_fault() == 0
    # report row 4: the tensor-core contraction (launch count first)
    assert (rep[4 * 4 + 0] > 0) == (nb > df_max)
    for b in range(nb):
        w0, s0 = gpu.px2wav(f[b], p)
        assert rel_err(w[b], w0) < TOL_MIXED and rel_err(sc[b], s0) < TOL_MIXED, b
        assert rel_err(r[b], gpu.wav2px(w[b], sc[b], p)) < TOL_MIXED, b
        assert rel_err(r[b], f[b]) < TOL_MIXED, b


@pytest.mark.gpu
@pytest.mark.parametrize("L,N,spin,real,ss", [(192, 4, 0, True, 0), (160, 3, 1, False, 1), (320, 4, 0, True, 0)])
def test_df_contraction_table_copies(gpu, L, N, spin, real, ss):
    """One-map calls at split precision contract in double-float on the FP32
    pipe: on double-float copies of the Wigner tables (the default), or
    splitting the FP64 values as they are read.  Both within 1e-11 of the FP64
    path for the four directional operators; the copies count in the plan
    bytes."""
    import ctypes as C

    from s2let_gb300.capi import SAMPLING_MW_SS

    TOL = 1e-11
    lib = gpu.lib
    lib.s2let_gpu_plan_bytes.restype = C.c_size_t
    p = make_parameters(L, 2.0, 2, N, spin, 0, sampling_scheme=SAMPLING_MW_SS if ss else 0)
    s = gpu.sizes(p)
    rng = np.random.default_rng(3 * L + spin)
    f = rng.normal(size=s["n_px"]) if real else rng.normal(size=s["n_px"]) + 1j * rng.normal(size=s["n_px"])
    assert lib.s2let_gpu_set_precision(0) == 0
    w0, s0 = gpu.px2wav(f, p, real=real)
    r0 = gpu.wav2px(w0, s0, p, real=real)
    a0 = gpu.analysis_adjoint_wav2px(w0, s0, p, real=real)
    bw0, bs0 = gpu.synthesis_adjoint_px2wav(f, p, real=real)
    plan_bytes = {}
    try:
        for on in (0, 1):
            lib.s2let_gpu_release_plans()
            assert lib.s2let_gpu_set_split_tables(on) == 0 and lib.s2let_gpu_get_split_tables() == on
            assert lib.s2let_gpu_set_precision(1) == 0
            w, sc = gpu.px2wav(f, p, real=real)
            r = gpu.wav2px(w0, s0, p, real=real)
            a = gpu.analysis_adjoint_wav2px(w0, s0, p, real=real)
            bw, bs = gpu.synthesis_adjoint_px2wav(f, p, real=real)
            assert lib.s2let_gpu_set_precision(0) == 0
            plan_bytes[on] = lib.s2let_gpu_plan_bytes()
            assert rel_err(w, w0) < TOL and rel_err(sc, s0) < TOL, on
            assert rel_err(r, r0) < TOL and rel_err(a, a0) < TOL, on
            assert rel_err(bw, bw0) < TOL and rel_err(bs, bs0) < TOL, on
    finally:
        lib.s2let_gpu_set_precision(0)
        lib.s2let_gpu_set_split_tables(1)
    assert plan_bytes[1] > plan_bytes[0]
    assert lib.s2let_gpu_device_fault() == 0 and lib.s2let_gpu_last_error() == 0
