"""McEwen-Wiaux symmetric sampling (MWSS): theta_t = pi t / L for t = 0..L (both
poles), 2L samples per ring; the SO3 wavelet maps use the same (alpha, beta)
grid.  The reference selects it with parameters->sampling_scheme at every SSHT
and SO3 call of the directional transforms (e.g. src/c/s2let_analysis.c:326,
411, 473, 513) and tests it with band-limited round trips
(test/c/test_back_and_forth.c:444-522).

CPU tests pin the oracle's MWSS restatement (direct evaluation of sY_lm at the
MWSS points, round trips, adjoint dot products, the reference's own S2LET code
built in place over it).  GPU tests (marked gpu) compare the C ABI against the
fixtures made by that build (FP64 path: normwise relative max error <= 1e-12)
and check size-independent properties at L = 256 and 512.
"""
import ctypes as C
import glob
import os

import numpy as np
import pytest

from conftest import oracle_sht, params_of, random_flm, rel_err
from oracle import oracle
from s2let_gb300.capi import SAMPLING_MW_SS, make_parameters

TOL = 1e-12
MWSS_GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "mwss_*.npz")))


def mwss(L, N=4, B=2.0, J_min=2, spin=0, up=0):
    return make_parameters(L, B, J_min, N, spin, up, sampling_scheme=SAMPLING_MW_SS)


def n_px(L):
    return (L + 1) * 2 * L


# ---------------------------------------------------------------------------
# oracle (CPU)
# ---------------------------------------------------------------------------


def _direct_inverse(O, flm, L, s):
    """f(theta_t, phi_p) = sum_lm flm sY_lm at theta_t = pi t/L, phi_p = pi p/L,
    with sY_lm = (-1)^s sqrt((2l+1)/4pi) e^{i m phi} d^l_{m,-s}(theta)."""
    fn = O.lib.oracle_wigner_d_column
    fn.restype = None
    fn.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_double]
    f = np.zeros((L + 1, 2 * L), complex)
    phi = np.pi * np.arange(2 * L) / L
    d = np.zeros(L)
    for t in range(L + 1):
        for m in range(-(L - 1), L):
            fn(d.ctypes.data, L, m, -s, np.pi * t / L)
            c = sum((-1) ** s * np.sqrt((2 * l + 1) / (4 * np.pi)) * flm[l * l + l + m] * d[l]
                    for l in range(max(abs(m), abs(s)), L))
            f[t] += c * np.exp(1j * m * phi)
    return f.ravel()


@pytest.mark.parametrize("L,spin", [(8, 0), (9, 2), (7, -3)])
def test_oracle_mwss_inverse_is_the_harmonic_sum(oracle_port, L, spin):
    flm = random_flm(np.random.default_rng(L), L, spin)
    f = oracle_sht(oracle_port, 1, flm, L, spin, ss=1)
    assert rel_err(f, _direct_inverse(oracle_port, flm, L, spin)) < 1e-13


@pytest.mark.parametrize("L,spin", [(8, 0), (12, 1), (11, 2)])
def test_oracle_mwss_round_trip_and_adjoints(oracle_port, L, spin):
    rng = np.random.default_rng(30 + L)
    O = oracle_port
    flm = random_flm(rng, L, spin)
    f = oracle_sht(O, 1, flm, L, spin, ss=1)
    assert np.abs(oracle_sht(O, 0, f, L, spin, ss=1) - flm).max() < 1e-12
    g = rng.normal(size=n_px(L)) + 1j * rng.normal(size=n_px(L))
    # <g, Y flm> = <Y^H g, flm>  and  <F g, flm> = <g, F^H flm>
    lhs, rhs = np.vdot(g, f), np.vdot(oracle_sht(O, 3, g, L, spin, ss=1), flm)
    assert abs(lhs - rhs) < 1e-12 * abs(lhs)
    lhs, rhs = np.vdot(oracle_sht(O, 0, g, L, spin, ss=1), flm), np.vdot(g, oracle_sht(O, 2, flm, L, spin, ss=1))
    assert abs(lhs - rhs) < 1e-12 * abs(lhs)


def test_oracle_mwss_real(oracle_port):
    L, O = 11, oracle_port
    rng = np.random.default_rng(8)
    flm = random_flm(rng, L, real=True)
    f = oracle_sht(O, 1, flm, L, real=True, ss=1)
    np.testing.assert_allclose(f, oracle_sht(O, 1, flm, L, ss=1).real, atol=1e-13)
    assert np.abs(oracle_sht(O, 0, f, L, real=True, ss=1) - flm).max() < 1e-12
    g = rng.normal(size=n_px(L))
    lhs, rhs = np.vdot(g, f), np.vdot(oracle_sht(O, 3, g, L, real=True, ss=1), flm)
    assert abs(lhs - rhs) < 1e-12 * abs(lhs)


@pytest.mark.parametrize("spin,up", [(0, 1), (0, 0), (2, 1), (2, 0)])  # test_back_and_forth.c:593-624
def test_oracle_mwss_wavelet_round_trip(oracle_port, spin, up):
    """test_wav_transform_mwss (test/c/test_back_and_forth.c:444-486; skipped
    there, run here): band-limited MWSS map -> px2wav -> wav2px -> flm."""
    L, O = 16, oracle_port
    p = mwss(L, spin=spin, up=up)
    flm = random_flm(np.random.default_rng(9), L, spin)
    f = oracle_sht(O, 1, flm, L, spin, ss=1)
    w, s = O.px2wav(f, p)
    back = oracle_sht(O, 0, O.wav2px(w, s, p), L, spin, ss=1)
    assert np.abs(back - flm).max() < 1e-12


def test_oracle_mwss_wavelet_round_trip_real(oracle_port):
    """test_wav_transform_mwss_real (test/c/test_back_and_forth.c:488-522)."""
    L, O = 16, oracle_port
    p = mwss(L)
    flm = random_flm(np.random.default_rng(10), L, real=True)
    f = oracle_sht(O, 1, flm, L, real=True, ss=1)
    w, s = O.px2wav(f, p, real=True)
    back = oracle_sht(O, 0, O.wav2px(w, s, p, real=True), L, real=True, ss=1)
    assert np.abs(back - flm).max() < 1e-12


@pytest.mark.parametrize("spin", [0, 2])
def test_oracle_mwss_wavelet_adjoints(oracle_port, spin):
    L, O = 16, oracle_port
    p = mwss(L, spin=spin, up=0)
    rng = np.random.default_rng(11)
    f = rng.normal(size=n_px(L)) + 1j * rng.normal(size=n_px(L))
    wr, sr = O.px2wav(rng.normal(size=n_px(L)) + 1j * rng.normal(size=n_px(L)), p)
    w, s = O.px2wav(f, p)
    a = O.analysis_adjoint_wav2px(wr, sr, p)
    lhs = np.vdot(wr, w) + np.vdot(sr, s)
    assert abs(lhs - np.vdot(a, f)) < 1e-11 * abs(lhs)
    b, c = O.synthesis_adjoint_px2wav(f, p)
    g = O.wav2px(wr, sr, p)
    lhs = np.vdot(b, wr) + np.vdot(c, sr)
    assert abs(lhs - np.vdot(f, g)) < 1e-11 * abs(lhs)


@pytest.mark.skipif(not oracle.ref_available(), reason="in-place reference build not present")
@pytest.mark.parametrize("case", [(12, 3, 2.0, 0, 1, 0), (16, 4, 2.0, 2, 0, 1)])
def test_oracle_mwss_port_equals_reference_build(oracle_port, case):
    R = oracle.ref()
    L, N, B, J_min, spin, up = case
    p = mwss(L, N, B, J_min, spin, up)
    rng = np.random.default_rng(12)
    f = rng.normal(size=n_px(L)) + 1j * rng.normal(size=n_px(L))
    for a, b in zip(oracle_port.px2wav(f, p), R.px2wav(f, p)):
        np.testing.assert_array_equal(a, b)
    w, s = R.px2wav(f, p)
    np.testing.assert_array_equal(oracle_port.wav2px(w, s, p), R.wav2px(w, s, p))
    np.testing.assert_array_equal(oracle_port.analysis_adjoint_wav2px(w, s, p), R.analysis_adjoint_wav2px(w, s, p))


def test_mwss_sizes(oracle_port):
    """n_px, n_scal and n_wav follow the MWSS grid (src/c/s2let_helper.c:5-107)."""
    import s2let_gb300

    host = s2let_gb300.api()  # the size helpers are host code: no GPU needed
    for case in [(16, 4, 2.0, 2, 0, 0), (16, 3, 2.0, 2, 2, 1), (13, 5, 2.0, 1, 1, 0)]:
        L, N, B, J_min, spin, up = case
        p = mwss(L, N, B, J_min, spin, up)
        assert host.sizes(p) == oracle_port.sizes(p)
        assert host.sizes(p)["n_px"] == n_px(L)


# ---------------------------------------------------------------------------
# GPU
# ---------------------------------------------------------------------------


@pytest.mark.gpu
@pytest.mark.parametrize("path", MWSS_GOLDEN, ids=lambda p: os.path.basename(p)[:-4])
def test_gpu_mwss_matches_reference_golden(gpu, path):
    """GPU outputs on MWSS sampling against the reference's own S2LET sources."""
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
    assert rel_err(gpu.wav2lm(g["lm2wav_wav"], g["lm2wav_scal"], p), g["wav2lm"]) < TOL
    if "f_real" in g.files:
        w, s = gpu.px2wav(g["f_real"], p, real=True)
        assert rel_err(w, g["px2wav_real_wav"]) < TOL and rel_err(s, g["px2wav_real_scal"]) < TOL
        assert rel_err(gpu.wav2px(w, s, p, real=True), g["wav2px_real"]) < TOL
        assert rel_err(gpu.analysis_adjoint_wav2px(g["px2wav_real_wav"], g["px2wav_real_scal"], p, real=True),
                       g["adj_wav2px_real"]) < TOL


@pytest.mark.gpu
@pytest.mark.parametrize("L,spin,real,ss", [(17, 0, False, 1), (16, 2, False, 1), (16, 0, True, 1),
                                            (33, -1, False, 1), (16, 2, False, 0)])
def test_gpu_sht_matches_oracle(gpu, oracle_port, L, spin, real, ss):
    """s2let_gpu_sht (all four directions) against the oracle's SSHT restatement."""
    rng = np.random.default_rng(40 + L)
    npx = n_px(L) if ss else L * (2 * L - 1)
    flm = random_flm(rng, L, spin, real=real)
    f = rng.normal(size=npx) if real else rng.normal(size=npx) + 1j * rng.normal(size=npx)
    for d, x in ((0, f), (1, flm), (2, flm), (3, f)):
        got = gpu.sht(d, x, L, spin, real, ss)
        ref = oracle_sht(oracle_port, d, x, L, spin, real, ss)
        assert rel_err(got, ref) < TOL, d
    assert gpu.lib.s2let_gpu_last_error() == 0


@pytest.mark.gpu
@pytest.mark.parametrize("L,N,spin,up", [(256, 4, 0, 0), (200, 3, 2, 0), (130, 4, 1, 1)])
def test_gpu_mwss_round_trip_both_precisions(gpu, L, N, spin, up):
    """Band-limited MWSS round trip (the reference's own MWSS check) at sizes
    that take the tensor-core contraction; the split-precision path agrees
    with the FP64 path to 1e-10 and raises no device fault."""
    p = mwss(L, N, spin=spin, up=up)
    rng = np.random.default_rng(L + N)
    flm = random_flm(rng, L, spin, power=lambda l: 1.0 / (l + 1))
    f = gpu.sht(1, flm, L, spin, False, 1)
    lib = gpu.lib
    out = {}
    for mode in (0, 1):
        assert lib.s2let_gpu_set_precision(mode) == 0
        try:
            w, s = gpu.px2wav(f, p)
            r = gpu.wav2px(w, s, p)
        finally:
            lib.s2let_gpu_set_precision(0)
        out[mode] = (w, s, r)
        assert rel_err(r, f) < (1e-12 if mode == 0 else 1e-10)
    assert lib.s2let_gpu_device_fault() == 0
    (w0, s0, _), (w1, s1, _) = out[0], out[1]
    assert rel_err(w1, w0) < 1e-10 and rel_err(s1, s0) < 1e-10
    back = gpu.sht(0, out[0][2], L, spin, False, 1)
    assert np.abs(back - flm).max() < 1e-12 * max(1.0, np.abs(flm).max())


@pytest.mark.gpu
def test_gpu_mwss_real_batch_and_linearity(gpu):
    """Real MWSS at L = 512 through the device batch entry point: round trip
    and linearity of px2wav, FP64 and split precision."""
    torch = pytest.importorskip("torch")
    from s2let_gb300 import torch_ops as T

    L = 512
    p = mwss(L)
    flms = [random_flm(np.random.default_rng(70 + i), L, real=True, power=lambda l: 1.0 / (l + 1))
            for i in range(2)]
    maps = np.stack([gpu.sht(1, a, L, 0, True, 1) for a in flms])
    x = torch.from_numpy(maps).cuda()
    for prec, tol in (("fp64", 1e-12), ("mixed", 1e-10)):
        w, s = T.px2wav(x, p, precision=prec)
        r = T.wav2px(w, s, p, precision=prec)
        assert float((r - x).abs().max() / x.abs().max()) < tol
        w3, s3 = T.px2wav(2.0 * x[:1] - 0.5 * x[1:], p, precision=prec)
        lin = 2.0 * w[:1] - 0.5 * w[1:]
        assert float((w3 - lin).abs().max() / lin.abs().max()) < tol
    assert gpu.lib.s2let_gpu_device_fault() == 0
    gpu.lib.s2let_gpu_release_plans()
