"""End to end as the reference's denoising demo (src/c/s2let_denoising_demo.c):
a real MW map read from FITS, Gaussian noise added, wavelet analysis, hard
thresholding of the coefficients per scale at 3 sigma of the noise, synthesis,
output written to FITS.  GPU and oracle run the same pipeline on the same
inputs (FP64, normwise relative 1e-12, one threshold mask for both);
denoising must raise the SNR (by more than 1 dB at noise of one signal rms)."""
import ctypes as C

import numpy as np
import pytest

from conftest import random_flm, rel_err
from s2let_gb300.capi import make_parameters, ptr


@pytest.mark.gpu
def test_denoising_pipeline_through_fits(gpu, oracle_port, tmp_path):
    lib = gpu.lib
    L, N, B, J_min = 64, 4, 2.0, 0
    p = make_parameters(L, B, J_min, N, 0, 0, reality=1)
    rng = np.random.default_rng(12)
    f0 = gpu.alm2map(random_flm(rng, L, real=True, power=lambda l: 1.0 / (l + 1) ** 1.5), L, real=True)
    src = str(tmp_path / "signal.fits").encode()
    lib.s2let_fits_mw_write_map(src, ptr(f0), L)
    assert lib.s2let_fits_mw_read_bandlimit(src) == L
    f = np.zeros_like(f0)
    lib.s2let_fits_mw_read_map(ptr(f), src, L)
    np.testing.assert_array_equal(f, f0)
    sigma = np.std(f)
    g = f + gpu.alm2map(random_flm(rng, L, real=True, power=lambda l: sigma * np.sqrt(4 * np.pi) / L), L, real=True)
    J = lib.s2let_j_max(C.byref(p))
    segs, off = [], 0  # the demo's per-scale blocks of N bl (2bl-1) coefficients
    for j in range(J_min, J + 1):
        bl = min(lib.s2let_bandlimit(j, C.byref(p)), L)
        segs.append(slice(off, off + N * bl * (2 * bl - 1)))
        off += N * bl * (2 * bl - 1)
    # thresholds: 3 sigma of the noise's own coefficients, scale by scale
    wn, _ = gpu.px2wav(g - f, p, real=True)
    thr = [3 * np.std(wn[sl]) for sl in segs]
    w, s = gpu.px2wav(g, p, real=True)
    w0, s0 = oracle_port.px2wav(g, p, real=True)
    assert rel_err(w, w0) < 1e-12 and rel_err(s, s0) < 1e-12
    keep = np.ones(w.shape, bool)
    for sl, t in zip(segs, thr):
        keep[sl] = np.abs(w[sl]) >= t
    out = gpu.wav2px(w * keep, s, p, real=True)
    assert rel_err(out, oracle_port.wav2px(w0 * keep, s0, p, real=True)) < 1e-12
    snr_in = 10 * np.log10(np.sum(f ** 2) / np.sum((g - f) ** 2))
    snr_out = 10 * np.log10(np.sum(f ** 2) / np.sum((out - f) ** 2))
    assert snr_out > snr_in + 1.0  # 0.2 dB in, about 2.5 dB out
    dst = str(tmp_path / "denoised.fits").encode()
    lib.s2let_fits_mw_write_map(dst, ptr(out), L)
    back = np.zeros_like(out)
    lib.s2let_fits_mw_read_map(ptr(back), dst, L)
    np.testing.assert_array_equal(back, out)
