"""Host-pointer batches (s2let_gpu_*_host_batch): nbatch maps per call in the
drop-in host layout.  Each map must equal the one-map drop-in call (FP64
path, 1e-12): f_wav crosses the bus in pieces (one scale of a group of maps)
on a second stream while the transforms run, device batches hold up to 32
maps (40 maps make two), full-resolution (upsampled) layouts and single maps
included, and the unused tail of f_wav (a scale with N_j < N) stays as the
caller wrote it.  Pageable numpy buffers go through the copy engines;
page-locked buffers (pinned=True) through the copy kernel, as the copy trace
reports."""
import ctypes as C

import numpy as np
import pytest

from conftest import rel_err
from s2let_gb300.capi import SAMPLING_MW_SS, make_parameters, ptr

TOL = 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("L,N,spin,real,nb,ss,up", [(32, 4, 0, True, 3, 0, 0), (24, 5, 2, False, 20, 0, 0),
                                                    (16, 8, 0, True, 17, 0, 0), (16, 3, 0, True, 40, 0, 0),
                                                    (20, 4, 0, True, 6, 1, 0), (18, 3, 1, False, 5, 1, 0),
                                                    (16, 3, 0, True, 9, 0, 1), (12, 2, 2, False, 1, 0, 1)])
@pytest.mark.parametrize("pinned", [False, True], ids=["pageable", "pinned"])
def test_host_batch_equals_single_calls(gpu, L, N, spin, real, nb, ss, up, pinned):
    lib = gpu.lib
    p = make_parameters(L, 2.0, 1, N, 0 if real else spin, up, sampling_scheme=SAMPLING_MW_SS if ss else 0)
    s = gpu.sizes(p)
    rng = np.random.default_rng(L + nb)
    dt = np.float64 if real else np.complex128
    shape = lambda n: (nb, n)
    f = rng.normal(size=shape(s["n_px"])) if real else rng.normal(size=shape(s["n_px"])) + 1j * rng.normal(size=shape(s["n_px"]))
    f = np.ascontiguousarray(f.astype(dt))
    w = np.full(shape(s["n_wav"]), 7.0, dt)  # the unused tail must keep this
    sc = np.zeros(shape(s["n_scal"]), dt)
    r = np.zeros_like(f)
    keep = []
    if pinned:  # the same arrays in page-locked memory
        torch = pytest.importorskip("torch")

        def pin(a):
            t = torch.empty(a.nbytes, dtype=torch.uint8, pin_memory=True)
            keep.append(t)
            v = t.numpy().view(a.dtype).reshape(a.shape)
            v[...] = a
            return v

        f, w, sc, r = pin(f), pin(w), pin(sc), pin(r)
    trace = (C.c_double * 10)()
    lib.s2let_gpu_copy_trace_enable(1)
    fn = lib.s2let_gpu_analysis_px2wav_real_host_batch if real else lib.s2let_gpu_analysis_px2wav_host_batch
    assert fn(ptr(w), ptr(sc), ptr(f), nb, C.byref(p)) == 0
    fn = lib.s2let_gpu_synthesis_wav2px_real_host_batch if real else lib.s2let_gpu_synthesis_wav2px_host_batch
    assert fn(ptr(r), ptr(w), ptr(sc), nb, C.byref(p)) == 0
    assert lib.s2let_gpu_copy_trace_report(trace) == 0
    lib.s2let_gpu_copy_trace_enable(0)
    # trace[5 d + 0] copies, trace[5 d + 4] of them by the copy kernel; d = 0 host to device, 1 device to host
    assert trace[0] > 0 and trace[5] > 0
    assert trace[4] == (trace[0] if pinned else 0) and trace[9] == (trace[5] if pinned else 0)
    for b in range(nb):
        w1 = np.full(s["n_wav"], 7.0, dt)
        s1 = np.zeros(s["n_scal"], dt)
        if real:
            lib.s2let_analysis_px2wav_real(ptr(w1), ptr(s1), ptr(np.ascontiguousarray(f[b])), C.byref(p))
        else:
            lib.s2let_analysis_px2wav(ptr(w1), ptr(s1), ptr(np.ascontiguousarray(f[b])), C.byref(p))
        assert rel_err(w[b], w1) < TOL and rel_err(sc[b], s1) < TOL, b
        r1 = gpu.wav2px(w1, s1, p, real=real)
        assert rel_err(r[b], r1) < TOL, b
    assert lib.s2let_gpu_last_error() == 0
