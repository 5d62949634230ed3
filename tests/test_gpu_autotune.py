"""Autotuned launch shapes (s2let_gpu_autotune): with tuning on, the first call
of each (kernel, band-limit bucket, batch bucket) times the candidate shapes on
the live call and keeps the fastest.  Every candidate computes the same result,
so tuned calls must equal untuned ones bit for bit, in both precisions and on
recomputed tables; the choices are written to the cache file named by
S2LET_GPU_AUTOTUNE_CACHE."""
import ctypes as C

import pytest

from s2let_gb300.capi import make_parameters

torch = pytest.importorskip("torch")


def _batch(lib, p, f, nb):
    from s2let_gb300 import torch_ops as T

    s = T.sizes(p)
    w = torch.zeros((nb, s["n_wav"]), dtype=torch.float64, device="cuda")
    sc = torch.zeros((nb, s["n_scal"]), dtype=torch.float64, device="cuda")
    r = torch.zeros_like(f)
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert lib.s2let_gpu_analysis_px2wav_real_batch(C.c_void_p(w.data_ptr()), C.c_void_p(sc.data_ptr()),
                                                    C.c_void_p(f.data_ptr()), nb, C.byref(p), st) == 0
    assert lib.s2let_gpu_synthesis_wav2px_real_batch(C.c_void_p(r.data_ptr()), C.c_void_p(w.data_ptr()),
                                                     C.c_void_p(sc.data_ptr()), nb, C.byref(p), st) == 0
    torch.cuda.synchronize()
    return w, sc, r


@pytest.mark.gpu
def test_tuned_calls_equal_untuned(gpu, tmp_path, monkeypatch):
    lib = gpu.lib
    cache = tmp_path / "tune.txt"
    monkeypatch.setenv("S2LET_GPU_AUTOTUNE_CACHE", str(cache))
    nb = 12
    cases = [(160, 1, 1), (96, 0, 1), (64, 0, 2)]  # L, precision (1: split), table mode (2: recomputed)
    results = {}
    for tune in (0, 1):
        old = lib.s2let_gpu_autotune(tune)
        try:
            for L, prec, tmode in cases:
                assert lib.s2let_gpu_set_precision(prec) == 0
                assert lib.s2let_gpu_set_table_mode(tmode) == 0
                p = make_parameters(L, 2.0, 2, 4, 0, 0)
                g = torch.Generator().manual_seed(L)
                f = torch.randn((nb, lib.s2let_n_px(C.byref(p))), generator=g, dtype=torch.float64).cuda()
                results[(tune, L)] = _batch(lib, p, f, nb)
        finally:
            lib.s2let_gpu_set_precision(0)
            lib.s2let_gpu_set_table_mode(0)
            lib.s2let_gpu_autotune(old)
    assert lib.s2let_gpu_device_fault() == 0
    for L, _, _ in cases:
        for a, b in zip(results[(0, L)], results[(1, L)]):
            assert torch.equal(a, b), L
    keys = (C.c_int * 500)()
    ms = (C.c_double * 200)()
    n = lib.s2let_gpu_autotune_entries(keys, ms, 100)
    fams = {keys[5 * i] for i in range(min(n, 100))}
    assert {1, 2, 3, 4} <= fams  # FP64, recomputed l->t and t->l, split precision
    lines = cache.read_text().splitlines()
    assert len(lines) >= 4 and all(len(ln.split()) == 8 for ln in lines)
    for i in range(min(n, 100)):
        assert ms[2 * i] <= ms[2 * i + 1] + 1e-9  # the choice is at least as fast as the built-in one
