"""GPU parity: directional wavelet transforms through the C ABI vs the CPU oracle.

Tolerance: FP64 path, normwise relative max error <= 1e-12
(max|gpu - oracle| / max|oracle|), as the FP64 target of the hot path states.
"""
import numpy as np
import pytest

from conftest import random_flm, rel_err
from s2let_gb300.capi import make_parameters

TOL = 1e-12

CASES = [
    # L, N, B, J_min, spin, upsample
    (8, 1, 2.0, 0, 0, 0),
    (16, 4, 2.0, 2, 0, 0),
    (16, 4, 2.0, 2, 0, 1),
    (16, 4, 2.0, 2, 2, 0),
    (16, 4, 2.0, 2, 2, 1),
    (17, 3, 2.5, 1, 1, 0),
    (12, 5, 2.0, 0, 0, 0),
    (32, 4, 2.0, 2, 0, 0),
]


def ids(c):
    return "L{}N{}B{}J{}s{}u{}".format(*c)


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES, ids=ids)
def test_px2wav_complex(gpu, oracle_port, case):
    L, N, B, J_min, spin, up = case
    p = make_parameters(L, B, J_min, N, spin, up)
    rng = np.random.default_rng(11)
    f = oracle_port.alm2map(random_flm(rng, L, spin), L, spin)
    w_o, s_o = oracle_port.px2wav(f, p)
    w_g, s_g = gpu.px2wav(f, p)
    assert gpu.lib.s2let_gpu_last_error() == 0
    assert rel_err(w_g, w_o) < TOL
    assert rel_err(s_g, s_o) < TOL
    fr_o = oracle_port.wav2px(w_o, s_o, p)
    fr_g = gpu.wav2px(w_o, s_o, p)
    assert rel_err(fr_g, fr_o) < TOL
    assert rel_err(fr_g, f) < 1e-12  # exact round trip on band-limited input


@pytest.mark.gpu
@pytest.mark.parametrize("case", [c for c in CASES if c[4] == 0], ids=ids)
def test_px2wav_real(gpu, oracle_port, case):
    L, N, B, J_min, spin, up = case
    p = make_parameters(L, B, J_min, N, spin, up)
    rng = np.random.default_rng(12)
    f = oracle_port.alm2map(random_flm(rng, L, real=True), L, real=True)
    w_o, s_o = oracle_port.px2wav(f, p, real=True)
    w_g, s_g = gpu.px2wav(f, p, real=True)
    assert rel_err(w_g, w_o) < TOL
    assert rel_err(s_g, s_o) < TOL
    fr_o = oracle_port.wav2px(w_o, s_o, p, real=True)
    fr_g = gpu.wav2px(w_o, s_o, p, real=True)
    assert rel_err(fr_g, fr_o) < TOL
    assert rel_err(fr_g, f) < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES, ids=ids)
def test_adjoints_vs_oracle(gpu, oracle_port, case):
    L, N, B, J_min, spin, up = case
    p = make_parameters(L, B, J_min, N, spin, up)
    rng = np.random.default_rng(13)
    npx = L * (2 * L - 1)
    f = rng.normal(size=npx) + 1j * rng.normal(size=npx)
    w, s = oracle_port.px2wav(f, p)
    a_o = oracle_port.analysis_adjoint_wav2px(w, s, p)
    a_g = gpu.analysis_adjoint_wav2px(w, s, p)
    assert rel_err(a_g, a_o) < TOL
    b_o = oracle_port.synthesis_adjoint_px2wav(f, p)
    b_g = gpu.synthesis_adjoint_px2wav(f, p)
    assert rel_err(b_g[0], b_o[0]) < TOL
    assert rel_err(b_g[1], b_o[1]) < TOL
    if spin == 0:
        fr = rng.normal(size=npx)
        w, s = oracle_port.px2wav(fr, p, real=True)
        assert rel_err(gpu.analysis_adjoint_wav2px(w, s, p, real=True),
                       oracle_port.analysis_adjoint_wav2px(w, s, p, real=True)) < TOL
        bo = oracle_port.synthesis_adjoint_px2wav(fr, p, real=True)
        bg = gpu.synthesis_adjoint_px2wav(fr, p, real=True)
        assert rel_err(bg[0], bo[0]) < TOL and rel_err(bg[1], bo[1]) < TOL


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES[:5], ids=ids)
def test_lm2wav_wav2lm(gpu, oracle_port, case):
    L, N, B, J_min, spin, up = case
    p = make_parameters(L, B, J_min, N, spin, up)
    rng = np.random.default_rng(14)
    flm = random_flm(rng, L, spin)
    w_o, s_o = oracle_port.lm2wav(flm, p)
    w_g, s_g = gpu.lm2wav(flm, p)
    assert rel_err(w_g, w_o) < TOL and rel_err(s_g, s_o) < TOL
    assert rel_err(gpu.wav2lm(w_o, s_o, p), oracle_port.wav2lm(w_o, s_o, p)) < TOL
    assert rel_err(gpu.analysis_adjoint_wav2lm(w_o, s_o, p),
                   oracle_port.analysis_adjoint_wav2lm(w_o, s_o, p)) < TOL
    bo = oracle_port.synthesis_adjoint_lm2wav(flm, p)
    bg = gpu.synthesis_adjoint_lm2wav(flm, p)
    assert rel_err(bg[0], bo[0]) < TOL and rel_err(bg[1], bo[1]) < TOL
    if spin == 0:
        flr = random_flm(rng, L, real=True)
        w_o, s_o = oracle_port.lm2wav(flr, p, real=True)
        w_g, s_g = gpu.lm2wav(flr, p, real=True)
        assert rel_err(w_g, w_o) < TOL and rel_err(s_g, s_o) < TOL
        assert rel_err(gpu.wav2lm(w_o, s_o, p, real=True), oracle_port.wav2lm(w_o, s_o, p, real=True)) < TOL


import glob  # noqa: E402
import os  # noqa: E402

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "dir_*.npz")) +
                glob.glob(os.path.join(os.path.dirname(__file__), "golden", "os_*.npz")))


@pytest.mark.gpu
@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: os.path.basename(p)[:-4])
def test_gpu_matches_reference_golden(gpu, path):
    """GPU outputs against vectors produced by the reference's own S2LET sources
    (os_*: spin-lowered wavelets, original_spin != 0, src/c/s2let_tiling.c:404-423)."""
    from conftest import params_of

    g = np.load(path)
    p = params_of(g)
    w, s = gpu.px2wav(g["f"], p)
    assert rel_err(w, g["px2wav_wav"]) < TOL and rel_err(s, g["px2wav_scal"]) < TOL
    assert rel_err(gpu.wav2px(g["px2wav_wav"], g["px2wav_scal"], p), g["wav2px"]) < TOL
    assert rel_err(gpu.analysis_adjoint_wav2px(g["px2wav_wav"], g["px2wav_scal"], p), g["adj_wav2px"]) < TOL
    a, b = gpu.synthesis_adjoint_px2wav(g["f"], p)
    assert rel_err(a, g["adj_px2wav_wav"]) < TOL and rel_err(b, g["adj_px2wav_scal"]) < TOL
    w, s = gpu.lm2wav(g["flm"], p)
    assert rel_err(w, g["lm2wav_wav"]) < TOL and rel_err(s, g["lm2wav_scal"]) < TOL
    lmn, sc = gpu.lm2lmn(g["flm"], p)
    n = len(g["lm2lmn"])
    assert rel_err(lmn[:n], g["lm2lmn"]) < TOL
    if "f_real" in g.files:
        w, s = gpu.px2wav(g["f_real"], p, real=True)
        assert rel_err(w, g["px2wav_real_wav"]) < TOL and rel_err(s, g["px2wav_real_scal"]) < TOL
        assert rel_err(gpu.wav2px(w, s, p, real=True), g["wav2px_real"]) < TOL


@pytest.mark.gpu
@pytest.mark.parametrize("L", [256, 1024])
def test_full_size_properties(gpu, L):
    """Size-independent checks at the benchmark size: exact round trip on a
    band-limited map, and linearity px2wav(a f + b g) = a px2wav(f) + b px2wav(g)."""
    p = make_parameters(L, 2.0, 2, 4, 0, 0)
    rng = np.random.default_rng(21)
    f = gpu.alm2map(random_flm(rng, L, real=True, power=lambda l: 1.0 / (l + 1)), L, real=True)
    g2 = gpu.alm2map(random_flm(rng, L, real=True, power=lambda l: 1.0 / (l + 1)), L, real=True)
    w, s = gpu.px2wav(f, p, real=True)
    assert rel_err(gpu.wav2px(w, s, p, real=True), f) < 1e-12
    w2, s2 = gpu.px2wav(g2, p, real=True)
    w3, s3 = gpu.px2wav(2.0 * f - 0.5 * g2, p, real=True)
    assert rel_err(w3, 2.0 * w - 0.5 * w2) < 1e-13
