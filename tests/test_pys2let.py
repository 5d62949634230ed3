"""pys2let-compatible module (s2let_gb300.pys2let).

CPU tests cover the pure index/tiling helpers (the tilings are the library's
host code, no GPU needed); GPU tests run the transforms and compare them with
the CPU oracle called the way the reference's pys2let calls the C library
(src/pys2let/pys2let.pyx)."""
import ctypes as C

import numpy as np
import pytest

from conftest import rel_err
from s2let_gb300 import pys2let as ps
from s2let_gb300.capi import make_parameters


def test_index_helpers():
    L = 9
    assert ps.mw_size(L) == L * (2 * L - 1)
    assert ps.mw_lm(3, 2) == 3 * 3 + 3 * 2  # the reference's formula, kept as is
    seen = {ps.healpy_lm(el, em, L) for el in range(L) for em in range(el + 1)}
    assert seen == set(range(L * (L + 1) // 2))
    th, ph = ps.mw_sampling(L)
    assert np.allclose(th, np.pi * (2 * np.arange(L) + 1) / (2 * L - 1))
    assert np.allclose(ph, 2 * np.pi * np.arange(2 * L - 1) / (2 * L - 1))


def test_healpy_round_trip_real_field():
    L = 12
    rng = np.random.default_rng(0)
    hp = rng.normal(size=L * (L + 1) // 2) + 1j * rng.normal(size=L * (L + 1) // 2)
    el = np.array([l for l in range(L) for m in range(l + 1)])
    em = np.array([m for l in range(L) for m in range(l + 1)])
    order = np.argsort([ps.healpy_lm(a, b, L) for a, b in zip(el, em)])
    hp[[ps.healpy_lm(a, 0, L) for a in range(L)]] = hp[[ps.healpy_lm(a, 0, L) for a in range(L)]].real
    flm = ps.lm_hp2lm(hp, L)
    for l in range(L):
        for m in range(1, l + 1):
            assert flm[l * l + l - m] == (-1) ** m * np.conj(flm[l * l + l + m])
    np.testing.assert_array_equal(ps.lm2lm_hp(flm, L), hp)
    assert order.size == hp.size


def test_tilings_and_wav_ind(oracle_port):
    B, L, J_min, N = 2.0, 32, 2, 4
    scal, wav = ps.axisym_wav_l(B, L, J_min)
    J = ps.pys2let_j_max(B, L, J_min)
    assert wav.shape == (L, J - J_min + 1)
    # admissibility of the axisymmetric tiling: kappa0^2 + sum_j kappa_j^2 = 1
    assert np.allclose(scal ** 2 + np.sum(wav ** 2, axis=1), 1.0)
    s_l, w_l = ps.wavelet_tiling(B, L, N, J_min, 0)
    p = make_parameters(L, B, J_min, N, 0, 0)
    psi, phi = oracle_port.tiling(p)
    np.testing.assert_array_equal(s_l.real, phi)
    np.testing.assert_array_equal(w_l[:, 0], psi[J_min * L * L:(J_min + 1) * L * L])
    off, bl, size, nel = ps.wav_ind(J_min + 1, 2, B, L, N, J_min, 0)
    assert size == bl * (2 * bl - 1) and off == oracle_port.lib.s2let_n_wav_j(J_min, C.byref(p)) + 2 * size


def test_hybrid_tiling_is_admissible():
    L = 64
    scal, wav, sbl, wbl, J, bounds = ps.construct_hybrid_tiling(L, 2, np.array([2.0, 1.5]), np.array([20]))
    assert wav.shape == (L, J + 1) and bounds[0] == 0 and bounds[-1] == L
    assert np.allclose(scal ** 2 + np.sum(wav ** 2, axis=1), 1.0)


def test_hybrid_tiling_rule():
    """The hybrid tiling against the rule worked out by hand for L = 64,
    J_min = 2, B = (2, 1.5), transition at l = 20.  Band 0 (B = 2) keeps scales
    2..floor(log2 20) = 4 and ends at 2^4 = 16; band 1 (B = 1.5, J_min = 0)
    starts with scale floor(log 16 / log 1.5) + 1 = 7 and keeps up to
    j_max = 11: columns 0, 1 are B=2 scales 2, 3; column 2 is B=2 scale 4 below
    l = 16 and B=1.5 scale 7 above; columns 3..6 are B=1.5 scales 8..11."""
    L = 64
    scal, wav, sbl, wbl, J, bounds = ps.construct_hybrid_tiling(L, 2, np.array([2.0, 1.5]), np.array([20]))
    assert J == 6 and list(bounds) == [0, 16, 64] and sbl == 4.0
    # round(min(B^(j+1), L)); the shared column takes the later band's value
    assert list(wbl) == [8, 16, 26, 38, 58, 64, 64]
    s2, w2 = ps.axisym_wav_l(2.0, L, 2)    # profiles[l, j - 2]
    _, w15 = ps.axisym_wav_l(1.5, L, 0)    # profiles[l, j]
    np.testing.assert_array_equal(scal, s2)
    lo = slice(0, 16)
    hi = slice(16, 64)
    # band 0: scale 2 absorbs "scale 1", which wraps to B=2's last wavelet (zero below 16)
    assert not w2[lo, -1].any()
    np.testing.assert_array_equal(wav[lo, 0], np.sqrt(w2[lo, 0] ** 2 + w2[lo, -1] ** 2))
    np.testing.assert_array_equal(wav[lo, 1], w2[lo, 1])
    # the seam: B=2 scale 4 absorbs scale 5 below 16; B=1.5 scale 7 absorbs scale 6 above
    np.testing.assert_array_equal(wav[lo, 2], np.sqrt(w2[lo, 2] ** 2 + w2[lo, 3] ** 2))
    np.testing.assert_array_equal(wav[hi, 2], np.sqrt(w15[hi, 7] ** 2 + w15[hi, 6] ** 2))
    for col, j in zip(range(3, 7), range(8, 12)):
        np.testing.assert_array_equal(wav[hi, col], w15[hi, j])
        assert not wav[lo, col].any()
    assert not wav[hi, :2].any()
    # admissible in each band
    np.testing.assert_allclose(scal ** 2 + (wav ** 2).sum(axis=1), 1.0, atol=1e-12)


def test_hybrid_single_band_keeps_reference_wrap():
    """With one band the first scale absorbs B's last wavelet (the reference's
    scale -1 wraps), so that wavelet is counted twice and verify_tiling rejects
    the tiling, as the reference does."""
    L = 64
    scal, wav, sbl, wbl, J, bounds = ps.construct_hybrid_tiling(L, 3, np.array([2.0]), np.array([], dtype=int))
    _, w = ps.axisym_wav_l(2.0, L, 3)
    np.testing.assert_array_equal(wav[:, 0], np.sqrt(w[:, 0] ** 2 + w[:, -1] ** 2))
    np.testing.assert_array_equal(wav[:, -1], w[:, -1])
    assert not ps.verify_tiling(L, scal, wav.T.ravel(), sbl, wbl)


def test_verify_tiling(capsys):
    L = 96
    scal, wav, sbl, wbl, J, bounds = ps.construct_hybrid_tiling(L, 0, np.array([3.0, 2.0]), np.array([40]))
    assert ps.verify_tiling(L, scal, wav.T.ravel(), sbl, wbl)
    # a band-limit that is too small is caught and reported
    bad = wbl.copy()
    bad[1] -= 2
    assert not ps.verify_tiling(L, scal, wav.T.ravel(), sbl, bad)
    assert "wavelet 1: band-limit" in capsys.readouterr().out
    # a tiling whose squares do not sum to 1 is not admissible
    assert not ps.verify_tiling(L, scal, 0.5 * wav.T.ravel(), sbl, wbl)
    assert "not admissible" in capsys.readouterr().out


def test_wigner_d_table_against_oracle(oracle_port):
    lib = oracle_port.lib
    lib.oracle_wigner_d_column.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_double]
    L, beta = 8, 1.1
    dl = ps.ssht_dl_beta_risbo(beta, L)
    for m in range(-(L - 1), L):
        for n in range(-(L - 1), L):
            col = np.zeros(L)
            lib.oracle_wigner_d_column(col.ctypes.data, L, m, n, beta)
            lo = max(abs(m), abs(n))
            np.testing.assert_allclose(dl[lo:, m + L - 1, n + L - 1], col[lo:], atol=1e-14)


@pytest.mark.gpu
def test_directional_transforms_match_oracle(gpu, oracle_port):
    B, L, J_min, N, spin, up = 2.0, 16, 2, 3, 0, 0
    rng = np.random.default_rng(3)
    f = rng.normal(size=L * (2 * L - 1)) + 1j * rng.normal(size=L * (2 * L - 1))
    p = make_parameters(L, B, J_min, N, spin, up)
    w, s = ps.analysis_px2wav(f, B, L, J_min, N, spin, up)
    wo, so = oracle_port.px2wav(f, p)
    assert rel_err(w, wo) < 1e-12 and rel_err(s, so) < 1e-12
    assert rel_err(ps.synthesis_wav2px(wo, so, B, L, J_min, N, spin, up), oracle_port.wav2px(wo, so, p)) < 1e-12
    assert rel_err(ps.analysis_adjoint_wav2px(wo, so, B, L, J_min, N, spin, up),
                   oracle_port.analysis_adjoint_wav2px(wo, so, p)) < 1e-12
    a, b = ps.synthesis_adjoint_px2wav(f, B, L, J_min, N, spin, up)
    ao, bo = oracle_port.synthesis_adjoint_px2wav(f, p)
    assert rel_err(a, ao) < 1e-12 and rel_err(b, bo) < 1e-12
    hp = ps.lm2lm_hp(ps.map2alm_mw(f.real.astype(complex), L, 0), L)
    w, s = ps.analysis_lm2wav(hp, B, L, J_min, N, spin, up)
    wo, so = oracle_port.lm2wav(ps.lm_hp2lm(hp, L), p)
    assert rel_err(w, wo) < 1e-12 and rel_err(s, so) < 1e-12
    back = ps.synthesis_wav2lm(w, s, B, L, J_min, N, spin, up)
    assert rel_err(back, hp) < 1e-12


@pytest.mark.gpu
def test_lmn_and_axisym_match_oracle(gpu, oracle_port):
    B, L, J_min, N = 2.0, 16, 1, 4
    rng = np.random.default_rng(4)
    flm = rng.normal(size=L * L) + 1j * rng.normal(size=L * L)
    p = make_parameters(L, B, J_min, N, 0, 0)
    lmn, sc = ps.analysis_lm2lmn(flm, B, L, J_min, N, 0, 0)
    lmno, sco = oracle_port.lm2lmn(flm, p)
    assert rel_err(lmn, lmno[:lmn.size]) < 1e-12 and rel_err(sc, sco[:sc.size]) < 1e-12
    assert rel_err(ps.synthesis_lmn2lm(lmn, sc, B, L, J_min, N, 0, 0), oracle_port.lmn2lm(lmn, sc, p)) < 1e-12
    f = rng.normal(size=L * (2 * L - 1)).astype(complex)
    w, s = ps.analysis_axisym_wav_mw(f, B, L, J_min)
    q = make_parameters(L, B, J_min, 1, 0, 0)
    wo, so = oracle_port.axisym("analysis", [f], q, False, False)
    assert rel_err(w, wo) < 1e-12 and rel_err(s, so) < 1e-12
    assert rel_err(ps.synthesis_axisym_wav_mw(w, s, B, L, J_min), oracle_port.axisym("synthesis", [wo, so], q)) < 1e-12
    hp = ps.lm2lm_hp(flm, L)
    whp, shp = ps.analysis_axisym_lm_wav(hp, B, L, J_min)
    back = ps.synthesis_axisym_lm_wav(whp, shp, B, L, J_min)
    assert rel_err(back, ps.lm2lm_hp(ps.lm_hp2lm(hp, L), L)) < 1e-12
