"""CPU tests of the oracle (test infrastructure): pinned against golden vectors
from the reference's own S2LET sources compiled in place, against the
reference's own identity tests (test/c/test_back_and_forth.c, test_adjoint.c,
test_axisym_vs_directional.c, test_tiling.c), and against closed forms."""
import ctypes as C
import glob
import os
from math import comb, factorial, pi, sqrt

import numpy as np
import pytest

from conftest import params_of, random_flm, rel_err
from oracle import oracle
from s2let_gb300.capi import make_parameters, ptr

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))


@pytest.mark.parametrize("path", [p for p in GOLDEN if os.path.basename(p).startswith(("dir_", "mwss_", "os_"))],
                         ids=lambda p: os.path.basename(p)[:-4])
def test_port_matches_reference_golden_directional(oracle_port, path):
    g = np.load(path)
    p = params_of(g)
    O = oracle_port
    tol = 1e-14
    w, s = O.px2wav(g["f"], p)
    assert rel_err(w, g["px2wav_wav"]) < tol and rel_err(s, g["px2wav_scal"]) < tol
    assert rel_err(O.wav2px(g["px2wav_wav"], g["px2wav_scal"], p), g["wav2px"]) < tol
    assert rel_err(O.analysis_adjoint_wav2px(g["px2wav_wav"], g["px2wav_scal"], p), g["adj_wav2px"]) < tol
    a, b = O.synthesis_adjoint_px2wav(g["f"], p)
    assert rel_err(a, g["adj_px2wav_wav"]) < tol and rel_err(b, g["adj_px2wav_scal"]) < tol
    w, s = O.lm2wav(g["flm"], p)
    assert rel_err(w, g["lm2wav_wav"]) < tol and rel_err(s, g["lm2wav_scal"]) < tol
    assert rel_err(O.wav2lm(g["lm2wav_wav"], g["lm2wav_scal"], p), g["wav2lm"]) < tol
    lmn, sc = O.lm2lmn(g["flm"], p)
    n = len(g["lm2lmn"])
    assert rel_err(lmn[:n], g["lm2lmn"]) < tol
    assert rel_err(O.lmn2lm(g["lm2lmn"], g["lm2lmn_scal"], p), g["lmn2lm"]) < tol
    psi, phi = O.tiling(p)
    np.testing.assert_array_equal(psi, g["psi"])
    np.testing.assert_array_equal(phi, g["phi"])
    if "f_real" in g.files:
        w, s = O.px2wav(g["f_real"], p, real=True)
        assert rel_err(w, g["px2wav_real_wav"]) < tol and rel_err(s, g["px2wav_real_scal"]) < tol
        assert rel_err(O.wav2px(w, s, p, real=True), g["wav2px_real"]) < tol
        assert rel_err(O.analysis_adjoint_wav2px(g["px2wav_real_wav"], g["px2wav_real_scal"], p, real=True),
                       g["adj_wav2px_real"]) < tol


@pytest.mark.parametrize("path", [p for p in GOLDEN if "axi_" in os.path.basename(p)],
                         ids=lambda p: os.path.basename(p)[:-4])
def test_port_matches_reference_golden_axisym(oracle_port, path):
    g = np.load(path)
    L, B, J_min = g["params"]
    p = make_parameters(int(L), B, int(J_min), 1, 0, 0)
    for mr in (0, 1):
        w, s = oracle_port.axisym("analysis", [g["f"]], p, bool(mr), True)
        assert rel_err(w, g[f"ana_mr{mr}_wav"]) < 1e-14 and rel_err(s, g[f"ana_mr{mr}_scal"]) < 1e-14
        assert rel_err(oracle_port.axisym("synthesis", [w, s], p, bool(mr), True), g[f"syn_mr{mr}"]) < 1e-14


@pytest.mark.skipif(not oracle.ref_available(), reason="in-place reference build not present")
@pytest.mark.parametrize("case", [(8, 3, 2.0, 0, 1, 0), (20, 6, 2.0, 1, 0, 0), (16, 2, 3.0, 1, 2, 1)])
def test_port_equals_reference_build(oracle_port, case):
    R = oracle.ref()
    L, N, B, J_min, spin, up = case
    p = make_parameters(L, B, J_min, N, spin, up)
    rng = np.random.default_rng(4)
    f = rng.normal(size=L * (2 * L - 1)) + 1j * rng.normal(size=L * (2 * L - 1))
    for a, b in zip(oracle_port.px2wav(f, p), R.px2wav(f, p)):
        np.testing.assert_array_equal(a, b)
    w, s = R.px2wav(f, p)
    np.testing.assert_array_equal(oracle_port.wav2px(w, s, p), R.wav2px(w, s, p))


# --- identities of the reference's own tests (L=16, N=4, B=2, J_min=2) -----------
STATES = [(0, 1), (0, 0), (2, 1), (2, 0)]  # (spin, upsample), test_back_and_forth.c:593-624


@pytest.mark.parametrize("spin,up", STATES)
def test_round_trip_px2wav(oracle_port, spin, up):
    L = 16
    p = make_parameters(L, 2.0, 2, 4, spin, up)
    flm = random_flm(np.random.default_rng(1), L, spin)
    f = oracle_port.alm2map(flm, L, spin)
    w, s = oracle_port.px2wav(f, p)
    flm2 = oracle_port.map2alm(oracle_port.wav2px(w, s, p), L, spin)
    assert np.abs(flm2 - flm).max() < 1e-12  # test_back_and_forth.c:396-399
    w, s = oracle_port.lm2wav(flm, p)
    assert np.abs(oracle_port.wav2lm(w, s, p) - flm).max() < 1e-12
    lmn, sc = oracle_port.lm2lmn(flm, p)
    assert np.abs(oracle_port.lmn2lm(lmn, sc, p) - flm).max() < 1e-12


def test_round_trip_real(oracle_port):
    L = 16
    p = make_parameters(L, 2.0, 2, 4, 0, 1)
    flm = random_flm(np.random.default_rng(2), L, real=True)
    f = oracle_port.alm2map(flm, L, real=True)
    w, s = oracle_port.px2wav(f, p, real=True)
    flm2 = oracle_port.map2alm(oracle_port.wav2px(w, s, p, real=True), L, real=True)
    assert np.abs(flm2 - flm).max() < 1e-12


def _dot(a, b):
    return np.vdot(a, b)


def _uniform_flm(rng, L, spin):
    """Uniform [-1, 1] real and imaginary parts from l = |spin| on, as
    s2let_lm_random_flm draws them (src/c/s2let_lm.c:31-39)."""
    f = rng.uniform(-1, 1, L * L) + 1j * rng.uniform(-1, 1, L * L)
    f[: spin * spin] = 0
    return f


@pytest.mark.parametrize("spin,up", [(0, 1), (2, 1), (2, 0)])  # test_adjoint.c:461-515
def test_adjoint_dot_products(oracle_port, spin, up):
    L = 16
    p = make_parameters(L, 2.0, 2, 4, spin, up)
    rng = np.random.default_rng(3)
    f = oracle_port.alm2map(_uniform_flm(rng, L, spin), L, spin)
    fr = oracle_port.alm2map(_uniform_flm(rng, L, spin), L, spin)
    w, s = oracle_port.px2wav(f, p)
    wr, sr = oracle_port.px2wav(fr, p)
    a = oracle_port.analysis_adjoint_wav2px(wr, sr, p)
    err = _dot(wr, w) + _dot(sr, s) - _dot(a, f)
    assert abs(err.real) < 1e-11 and abs(err.imag) < 1e-12  # test_adjoint.c:163-164
    b, c = oracle_port.synthesis_adjoint_px2wav(f, p)
    g = oracle_port.wav2px(wr, sr, p)
    err = _dot(b, wr) + _dot(c, sr) - _dot(f, g)
    assert abs(err) < 1e-11


def test_adjoint_dot_products_real(oracle_port):
    L = 16
    p = make_parameters(L, 2.0, 2, 4, 0, 0)
    rng = np.random.default_rng(5)
    f = rng.normal(size=L * (2 * L - 1))
    w2, s2 = oracle_port.px2wav(rng.normal(size=L * (2 * L - 1)), p, real=True)
    w, s = oracle_port.px2wav(f, p, real=True)
    a = oracle_port.analysis_adjoint_wav2px(w2, s2, p, real=True)
    assert abs(np.dot(w2, w) + np.dot(s2, s) - np.dot(a, f)) < 1e-11
    b, c = oracle_port.synthesis_adjoint_px2wav(f, p, real=True)
    g = oracle_port.wav2px(w2, s2, p, real=True)
    assert abs(np.dot(b, w2) + np.dot(c, s2) - np.dot(f, g)) < 1e-11


@pytest.mark.parametrize("multires", [False, True])  # test_axisym_vs_directional.c:13-105
def test_axisym_equals_directional_at_N1(oracle_port, multires):
    L = 16
    p = make_parameters(L, 2.0, 2, 1, 0, 0 if multires else 1)
    rng = np.random.default_rng(6)
    f = oracle_port.alm2map(random_flm(rng, L), L, 0)
    wd, sd = oracle_port.px2wav(f, p)
    wa, sa = oracle_port.axisym("analysis", [f], p, multires, False)
    assert np.abs(wd - wa).max() < 1e-12
    assert np.abs(sd - sa).max() < 1e-12


def test_tiling_identities(oracle_port):  # test_tiling.c:12-101
    p = make_parameters(16, 2.0, 2, 4, 0, 0)
    lib = oracle_port.lib
    J = lib.s2let_j_max(C.byref(p))
    kappa = np.zeros((J + 1) * 16)
    kappa0 = np.zeros(16)
    lib.s2let_tiling_axisym(ptr(kappa), ptr(kappa0), C.byref(p))
    assert lib.s2let_tiling_axisym_check_identity(ptr(kappa), ptr(kappa0), C.byref(p)) < 1e-12
    s_elm = np.zeros(16 * 16, np.complex128)
    lib.s2let_tiling_direction(ptr(s_elm), C.byref(p))
    assert lib.s2let_tiling_direction_check_identity(ptr(s_elm), C.byref(p)) < 1e-12
    psi, phi = oracle_port.tiling(p)
    assert lib.s2let_tiling_wavelet_check_identity(ptr(psi), ptr(phi), C.byref(p)) < 1e-12


def test_binomial_exact():
    lib = oracle.port().lib
    lib.binomial_coefficient.restype = C.c_ulong
    lib.binomial_coefficient.argtypes = [C.c_int, C.c_int, C.c_int]
    for n in range(0, 63):
        for k in range(0, n + 1):
            assert lib.binomial_coefficient(n, k, 1) == comb(n, k)


# --- closed forms: conventions the reference's tests do not pin ---------------------
def test_spherical_harmonics_closed_forms(oracle_port):
    L = 5
    K = 2 * L - 1
    th = np.pi * (2 * np.arange(L) + 1) / K
    ph = 2 * np.pi * np.arange(K) / K
    T, P = np.meshgrid(th, ph, indexing="ij")
    cases = {
        (0, 0, 0): lambda t, p: np.full_like(t, 1 / sqrt(4 * pi)) + 0j,
        (1, 0, 0): lambda t, p: sqrt(3 / (4 * pi)) * np.cos(t) + 0j,
        (1, 1, 0): lambda t, p: -sqrt(3 / (8 * pi)) * np.sin(t) * np.exp(1j * p),  # Condon-Shortley
        (2, -2, 0): lambda t, p: 0.25 * sqrt(15 / (2 * pi)) * np.sin(t) ** 2 * np.exp(-2j * p),
        # spin 2: sY_lm = (-1)^s sqrt((2l+1)/4pi) e^{i m phi} d^l_{m,-s}(theta) with
        # d^2_{2,-2} = sin^4(theta/2):  2Y_22 = (1/8) sqrt(5/pi) (1 - cos t)^2 e^{2ip}
        (2, 2, 2): lambda t, p: 0.125 * sqrt(5 / pi) * (1 - np.cos(t)) ** 2 * np.exp(2j * p),
    }
    for (l, m, s), fn in cases.items():
        flm = np.zeros(L * L, np.complex128)
        flm[l * l + l + m] = 1.0
        f = oracle_port.alm2map(flm, L, s).reshape(L, K)
        assert np.abs(f - fn(T, P)).max() < 1e-14, (l, m, s)


def _d_explicit(l, mp, m, beta):
    tot = 0.0
    for k in range(max(0, m - mp), min(l + m, l - mp) + 1):
        tot += (-1) ** (mp - m + k) / (factorial(l + m - k) * factorial(k) * factorial(mp - m + k) *
                                       factorial(l - mp - k)) * np.cos(beta / 2) ** (2 * l + m - mp - 2 * k) * \
            np.sin(beta / 2) ** (mp - m + 2 * k)
    return sqrt(factorial(l + mp) * factorial(l - mp) * factorial(l + m) * factorial(l - m)) * tot


def test_wigner_d_against_explicit_sum():
    lib = oracle.port().lib
    lib.oracle_delta_quadrant.argtypes = [C.c_void_p, C.c_int]
    lib.oracle_wigner_d_column.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_double]
    for l in range(0, 12):
        D = np.zeros((l + 1) * (l + 1))
        lib.oracle_delta_quadrant(ptr(D), l)
        for mp in range(l + 1):
            for m in range(l + 1):
                assert abs(D[mp * (l + 1) + m] - _d_explicit(l, mp, m, pi / 2)) < 1e-13
    L = 12
    for (m, n) in [(0, 0), (3, 1), (-3, 1), (1, 3), (1, -3), (-2, -4), (4, -2), (2, 2), (-5, 0)]:
        for theta in (0.3, 1.7, 3.0):
            col = np.zeros(L)
            lib.oracle_wigner_d_column(ptr(col), L, m, n, theta)
            for l in range(max(abs(m), abs(n)), L):
                assert abs(col[l] - _d_explicit(l, m, n, theta)) < 1e-12, (l, m, n, theta)


def test_so3_compact_index_is_a_bijection():
    """SO3_STORAGE_COMPACT / NEGATIVE_FIRST index of the restatement covers
    0..flmn_size-1 exactly once (complex and real storage)."""
    from s2let_gb300.capi import S2letParameters  # noqa: F401

    lib = oracle.port().lib
    for (L, N, real) in [(8, 3, 0), (8, 4, 1), (10, 10, 0), (6, 7, 1)]:
        p = make_parameters(L, 2.0, 0, N, 0, 1, reality=real)
        lmn, _ = oracle.port().lm2lmn(np.ones(L * L, np.complex128), p, real=bool(real))
        assert lmn is not None
