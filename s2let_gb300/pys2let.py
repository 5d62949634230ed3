"""pys2let-compatible functions backed by the GPU library.

Same names, argument order, argument meaning and return layouts as the
reference's Python binding (src/pys2let/pys2let.pyx), so that
``import s2let_gb300.pys2let as pys2let`` replaces ``import pys2let``:

* healpy-ordered harmonic input/output (m >= 0 only) where the reference uses
  it (analysis_lm2wav, synthesis_wav2lm, the axisymmetric lm transforms);
* complex (``reality = 0``) transforms throughout, parameters built from zero
  like the reference's ``s2let_parameters_t parameters = {}``;
* the reference's quirks: ``mw_lm`` returns el*el + el*em, the manual-tiling
  functions print their band-limits, ``wavelet_tiling`` returns a complex
  scaling array and ignores ``original_spin``.

All transforms run on the GPU (there is no CPU path); the tilings are the
library's host FP64 code, bit-identical to the reference's.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .capi import S2letParameters, ptr

__all__ = [
    "pys2let_j_max", "mw_lm", "healpy_lm", "analysis_axisym_lm_wav", "analysis_axisym_wav_mw",
    "analysis_adjoint_axisym_wav_mw", "synthesis_axisym_lm_wav", "synthesis_axisym_wav_mw",
    "synthesis_adjoint_axisym_wav_mw", "verify_tiling", "analysis_lm2wav_manualtiling",
    "synthesis_wav2lm_manualtiling", "analysis_lm2wav", "synthesis_wav2lm", "analysis_px2wav",
    "analysis_adjoint_wav2px", "synthesis_wav2px", "synthesis_adjoint_px2wav", "analysis_lm2lmn",
    "analysis_adjoint_lmn2lm", "synthesis_lmn2lm", "synthesis_adjoint_lm2lmn", "mw_size", "lm2lm_hp",
    "lm_hp2lm", "wav_ind", "mw_sampling", "alm2map_mw", "map2alm_mw", "wavelet_tiling", "axisym_wav_l",
    "ssht_dl_beta_risbo", "construct_hybrid_tiling",
]


def _lib_():
    return _lib.load()


def _params(B=0.0, L=0, J_min=0, N=0, spin=0, upsample=0, original_spin=0) -> S2letParameters:
    p = S2letParameters()  # all fields zero: reality 0, MW sampling, Risbo
    p.B, p.L, p.J_min, p.N, p.spin = float(B), int(L), int(J_min), int(N), int(spin)
    p.upsample, p.original_spin = int(upsample), int(original_spin)
    return p


# host-side tiling helpers: cannot fail and leave the thread's status alone
_HOST = {"s2let_tiling_wavelet", "s2let_tiling_axisym", "s2let_tiling_direction", "s2let_transform_axisym_lm_wav"}


def _call(name, *args):
    lib = _lib_()
    getattr(lib, name)(*args)
    if name in _HOST:
        return
    code = lib.s2let_gpu_last_error()
    if code != 0:
        raise RuntimeError(f"{name}: {lib.s2let_gpu_last_error_string().decode(errors='replace')}")


def _c128(a):
    return np.ascontiguousarray(a, dtype=np.complex128)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


# ---- index helpers -----------------------------------------------------------

def pys2let_j_max(B, L, J_min):
    return _lib_().s2let_j_max(C.byref(_params(B, L, J_min)))


def mw_lm(el, em):
    # as the reference returns it (not el*el + el + em)
    return el * el + el * em


def healpy_lm(el, em, L):
    return int(em * (2 * L - 1 - em) / 2 + el)


def mw_size(L):
    return L * (2 * L - 1)


def _hp_index(L):
    el, em = np.tril_indices(L)  # el >= em >= 0
    return el, em, (em * (2 * L - 1 - em)) // 2 + el


def lm2lm_hp(f_lm, L):
    """MW-ordered (l^2 + l + m) to healpy-ordered m >= 0 coefficients."""
    f_lm = _c128(f_lm)
    el, em, hp = _hp_index(L)
    out = np.zeros(L * (L + 1) // 2, dtype=complex)
    out[hp] = f_lm[el * el + el + em]
    return out


def lm_hp2lm(flm_hp, L):
    """healpy-ordered m >= 0 to MW-ordered coefficients of a real field:
    f_{l,-m} = (-1)^m conj(f_{lm})."""
    flm_hp = _c128(flm_hp)
    el, em, hp = _hp_index(L)
    out = np.zeros(L * L, dtype=complex)
    v = flm_hp[hp]
    out[el * el + el - em] = np.where(em % 2 == 1, -1.0, 1.0) * v.conj()
    out[el * el + el + em] = v
    return out


def wav_ind(j, n, B, L, N, J_min, upsample):
    """(offset of direction n of scale j in f_wav, band-limit, MW size, elements of scale j)."""
    p = _params(B, L, J_min, N, 0, upsample)
    lib = _lib_()
    offset = sum(lib.s2let_n_wav_j(jp, C.byref(p)) for jp in range(J_min, j))
    bandlimit = L if upsample else min(lib.s2let_bandlimit(j, C.byref(p)), L)
    offset += n * mw_size(bandlimit)
    return offset, bandlimit, mw_size(bandlimit), lib.s2let_n_wav_j(j, C.byref(p))


def mw_sampling(L):
    """MW sample positions theta_t = pi (2t+1)/(2L-1), phi_p = 2 pi p/(2L-1)."""
    K = 2 * L - 1
    return np.pi * (2.0 * np.arange(L) + 1.0) / K, 2.0 * np.pi * np.arange(K) / K


# ---- tilings -----------------------------------------------------------------

def wavelet_tiling(B, L, N, J_min, spin, original_spin=0):
    p = _params(B, L, J_min, N, spin)  # the reference leaves original_spin at 0
    lib = _lib_()
    J = lib.s2let_j_max(C.byref(p))
    psi = np.zeros((J + 1) * L * L, dtype=complex)
    phi = np.zeros(L)
    _call("s2let_tiling_wavelet", ptr(psi), ptr(phi), C.byref(p))
    scal_l = phi.astype(complex)
    wav_l = np.zeros((L * L, J - J_min + 1), dtype=complex)
    lo = spin * spin
    for j in range(J - J_min + 1):
        wav_l[lo:, j] = psi[(j + J_min) * L * L + lo:(j + J_min + 1) * L * L]
    return scal_l, wav_l


def axisym_wav_l(B, L, J_min):
    p = _params(B, L, J_min)
    lib = _lib_()
    J = lib.s2let_j_max(C.byref(p))
    kappa = np.zeros((J + 1) * L)
    kappa0 = np.zeros(L)
    _call("s2let_tiling_axisym", ptr(kappa), ptr(kappa0), C.byref(p))
    return kappa0.copy(), kappa.reshape(J + 1, L)[J_min:].T.copy()


def verify_tiling(L, scal_l, wav_l, scal_bandlimit, wav_bandlimits):
    """Checks a manual axisymmetric tiling before it is used with the *_manual
    transforms (pys2let's verify_tiling, src/pys2let/pys2let.pyx:442-478).

    scal_l (L values) and wav_l ((J+1)*L values, scale-major) are harmonic
    profiles; scal_bandlimit and wav_bandlimits[j] are the band-limits claimed
    for them.  A profile is band-limited at b when its running sum has reached
    its total at l = b - 1 (nothing beyond contributes).  The tiling is
    admissible when scal_l^2 + sum_j wav_l[j]^2 = 1 at every l (np.allclose).
    Prints the measured and the given band-limit of every profile (or the first
    one that is wrong, with the profile) and, when the sum is off, the sum;
    returns True when every band-limit holds and the sum is 1.
    """
    profiles = [("scaling function", np.asarray(scal_l, dtype=np.float64), scal_bandlimit)]
    wav = np.asarray(wav_l, dtype=np.float64).reshape(-1)
    bls = np.asarray(wav_bandlimits)
    for j in range(bls.size):
        profiles.append((f"wavelet {j}", wav[j * L:(j + 1) * L], bls[j]))
    square_sum = np.zeros(L)
    for name, prof, given in profiles:
        square_sum += prof ** 2
        # running sum over l as a fraction of the total; exactly 1 once the
        # profile has ended
        frac = np.cumsum(prof)
        frac = frac / frac[-1]
        measured = int(np.flatnonzero(frac == 1)[0]) + 1
        if frac[int(given - 1)] < 1:
            print(f"{name}: band-limit {given} is too small, the profile reaches l = {measured - 1}")
            if name != "scaling function":
                print("profile:", prof)
            return False
        print(f"{name}: band-limit measured {measured}, given {given}")
    if not np.allclose(square_sum, 1.0):
        print("not admissible: scal_l^2 + sum_j wav_l[j]^2 differs from 1:")
        print(square_sum)
        return False
    return True


def construct_hybrid_tiling(L, J_min0, Bs, L_transitions):
    """Axisymmetric tiling whose dilation factor changes with the multipole
    (pys2let's construct_hybrid_tiling, src/pys2let/pys2let.pyx:1132-1179).

    The multipoles [0, L) are cut into bands, one per factor B_k of Bs.  Band
    k uses the axisymmetric wavelets of B_k (J_min = J_min0 for the first band,
    0 for the others), restricted to the band's multipoles:

    * band k keeps the scales j = first_k .. last_k of B_k, where first_0 =
      J_min0, first_k = floor(log(lo_k) / log(B_k)) + 1 for k > 0 (the first
      scale that ends above the band's start lo_k), last_k = floor(log(T_k) /
      log(B_k)) for the transition multipole T_k = L_transitions[k] (the last
      band keeps every scale up to j_max(B_k));
    * the band ends where its last scale peaks: hi_k = round(B_k^last_k) (= L
      for the last band), and the next band starts there;
    * seams: the first scale of a band absorbs, in quadrature, the scale of
      B_k just below it, and (except in the last band) its last scale absorbs
      the one just above it, so that the squares still sum to 1 inside the band
      (the absorbed profile is used only where the kept one is below 1 at the
      band's first multipole);
    * columns: the scales are numbered across bands; the last scale of band k
      and the first of band k+1 share one column (they live on the two sides of
      the seam), so there are J + 1 = 1 + sum_k (last_k - first_k) columns;
    * band-limits: round(min(B_k^(j+1), L)) per column, the later band's where
      a column is shared; the scaling function is that of B_0 with band-limit
      B_0^J_min0.

    Two behaviours of the reference are kept: in the first band the "scale
    below" of the first scale is B_0's LAST wavelet (the reference indexes
    scale -1, which wraps), which is zero there unless the first band reaches
    that wavelet's support (with a single band it does, and the tiling is then
    not admissible); and band-limits of non-integer powers are rounded, which
    can leave a profile one multipole past its band-limit.

    Returns (scal_l, wav_l of shape (L, J + 1), scal_bandlimit,
    wav_bandlimits, J, band boundaries [lo_0 = 0, lo_1, ..., L]).
    """
    Bs = np.asarray(Bs, dtype=float)
    nband = Bs.size
    # the per-band axisymmetric tilings: (J_min, j_max, profiles[l, j - J_min])
    tilings = []
    for k in range(nband):
        jmin = J_min0 if k == 0 else 0
        _, w = axisym_wav_l(Bs[k], L, jmin)
        tilings.append((jmin, pys2let_j_max(Bs[k], L, jmin), w))
    # band boundaries and the scales each band keeps
    bounds, first, last = [0], [], []
    for k in range(nband):
        jmin, jmax, _ = tilings[k]
        first.append(jmin if k == 0 else int(np.log(bounds[k]) / np.log(Bs[k])) + 1)
        last.append(jmax if k == nband - 1 else int(np.log(L_transitions[k]) / np.log(Bs[k])))
        bounds.append(L if k == nband - 1 else int(np.rint(Bs[k] ** last[k])))
    J = sum(b - a for a, b in zip(first, last))
    wav = np.zeros((L, J + 1))
    wav_bandlimits = np.zeros(J + 1, dtype=np.int32)
    col = 0
    for k in range(nband):
        jmin, _, w = tilings[k]
        lo, hi = bounds[k], bounds[k + 1]
        for j in range(first[k], last[k] + 1):
            c = j - jmin  # column of scale j in B_k's profiles
            prof = w[lo:hi, c]
            below_one = w[lo, c] < 1.0
            if j == first[k] and below_one:
                # c - 1 = -1 in the first band: B_0's last wavelet (see above)
                prof = np.sqrt(prof ** 2 + w[lo:hi, c - 1] ** 2)
            if k < nband - 1 and j == last[k] and below_one:
                prof = np.sqrt(prof ** 2 + w[lo:hi, c + 1] ** 2)
            wav[lo:hi, col] = prof
            wav_bandlimits[col] = np.rint(min(Bs[k] ** (j + 1), L))
            if j < last[k]:
                col += 1
    scal_l, _ = axisym_wav_l(Bs[0], L, J_min0)
    return scal_l, wav, Bs[0] ** J_min0, wav_bandlimits, J, np.asarray(bounds, dtype=np.int32)


# ---- axisymmetric transforms ---------------------------------------------------

def _axisym_kernels(p):
    lib = _lib_()
    J = lib.s2let_j_max(C.byref(p))
    wav_lm = np.zeros((J + 1) * p.L)
    scal_lm = np.zeros(p.L)
    _call("s2let_transform_axisym_lm_wav", ptr(wav_lm), ptr(scal_lm), C.byref(p))
    return J, wav_lm, scal_lm


def analysis_axisym_lm_wav(flm_hp, B, L, J_min, spin_lowered=False):
    p = _params(B, L, J_min, 1)
    J, wav_lm, scal_lm = _axisym_kernels(p)
    f_scal_lm = np.zeros(L * L, dtype=complex)
    f_wav_lm = np.zeros(L * L * (J + 1 - J_min), dtype=complex)
    f_lm = lm_hp2lm(flm_hp, L)
    _call("s2let_transform_axisym_lm_wav_analysis", ptr(f_wav_lm), ptr(f_scal_lm), ptr(f_lm), ptr(wav_lm),
          ptr(scal_lm), C.byref(p))
    wav_hp = np.stack([lm2lm_hp(f_wav_lm[j * L * L:(j + 1) * L * L], L) for j in range(J + 1 - J_min)], axis=1)
    return wav_hp, lm2lm_hp(f_scal_lm, L)


def synthesis_axisym_lm_wav(f_wav_lm_hp, f_scal_lm_hp, B, L, J_min, spin_lowered=False):
    p = _params(B, L, J_min, 1)
    J, wav_lm, scal_lm = _axisym_kernels(p)
    f_wav_lm_hp = _c128(f_wav_lm_hp)
    f_scal_lm = lm_hp2lm(f_scal_lm_hp, L)
    f_wav_lm = np.concatenate([lm_hp2lm(f_wav_lm_hp[:, j], L) for j in range(J + 1 - J_min)])
    f_lm = np.zeros(L * L, dtype=complex)
    _call("s2let_transform_axisym_lm_wav_synthesis", ptr(f_lm), ptr(f_wav_lm), ptr(f_scal_lm), ptr(wav_lm),
          ptr(scal_lm), C.byref(p))
    return lm2lm_hp(f_lm, L)


def _axisym_mw(op, f_in, B, L, J_min):
    p = _params(B, L, J_min, 1)
    J = _lib_().s2let_j_max(C.byref(p))
    n = mw_size(L)
    if op in ("analysis", "synthesis_adjoint"):
        f = _c128(f_in[0])
        f_wav = np.zeros(n * (J - J_min + 1), dtype=complex)
        f_scal = np.zeros(n, dtype=complex)
        _call(f"s2let_transform_axisym_wav_{op}_mw", ptr(f_wav), ptr(f_scal), ptr(f), C.byref(p))
        return f_wav, f_scal
    f_wav, f_scal = _c128(f_in[0]), _c128(f_in[1])
    f = np.zeros(n, dtype=complex)
    _call(f"s2let_transform_axisym_wav_{op}_mw", ptr(f), ptr(f_wav), ptr(f_scal), C.byref(p))
    return f


def analysis_axisym_wav_mw(f, B, L, J_min, spin_lowered=False):
    return _axisym_mw("analysis", (f,), B, L, J_min)


def analysis_adjoint_axisym_wav_mw(f_wav, f_scal, B, L, J_min, spin_lowered=False):
    return _axisym_mw("analysis_adjoint", (f_wav, f_scal), B, L, J_min)


def synthesis_axisym_wav_mw(f_wav, f_scal, B, L, J_min, spin_lowered=False):
    return _axisym_mw("synthesis", (f_wav, f_scal), B, L, J_min)


def synthesis_adjoint_axisym_wav_mw(f, B, L, J_min, spin_lowered=False):
    return _axisym_mw("synthesis_adjoint", (f,), B, L, J_min)


# ---- directional transforms --------------------------------------------------

def _dir_params(B, L, J_min, N, spin, upsample, original_spin):
    return _params(B, L, J_min, N, spin, upsample, original_spin)


def _sizes(p):
    lib = _lib_()
    return lib.s2let_n_wav(C.byref(p)), lib.s2let_n_scal(C.byref(p))


def analysis_lm2wav(flm_hp, B, L, J_min, N, spin, upsample, spin_lowered=False, original_spin=0):
    p = _dir_params(B, L, J_min, N, spin, upsample, original_spin)
    nw, ns = _sizes(p)
    f_wav, f_scal = np.zeros(nw, dtype=complex), np.zeros(ns, dtype=complex)
    f_lm = lm_hp2lm(flm_hp, L)
    _call("s2let_analysis_lm2wav", ptr(f_wav), ptr(f_scal), ptr(f_lm), C.byref(p))
    return f_wav, f_scal


def synthesis_wav2lm(f_wav, f_scal, B, L, J_min, N, spin, upsample, spin_lowered=False, original_spin=0):
    p = _dir_params(B, L, J_min, N, spin, upsample, original_spin)
    f_lm = np.zeros(L * L, dtype=complex)
    _call("s2let_synthesis_wav2lm", ptr(f_lm), ptr(_c128(f_wav)), ptr(_c128(f_scal)), C.byref(p))
    return lm2lm_hp(f_lm, L)


def analysis_px2wav(f, B, L, J_min, N, spin, upsample, spin_lowered=False, original_spin=0):
    p = _dir_params(B, L, J_min, N, spin, upsample, original_spin)
    nw, ns = _sizes(p)
    f_wav, f_scal = np.zeros(nw, dtype=complex), np.zeros(ns, dtype=complex)
    _call("s2let_analysis_px2wav", ptr(f_wav), ptr(f_scal), ptr(_c128(f)), C.byref(p))
    return f_wav, f_scal


def analysis_adjoint_wav2px(f_wav, f_scal, B, L, J_min, N, spin, upsample, spin_lowered=False, original_spin=0):
    p = _dir_params(B, L, J_min, N, spin, upsample, original_spin)
    f = np.zeros(mw_size(L), dtype=complex)
    _call("s2let_analysis_adjoint_wav2px", ptr(f), ptr(_c128(f_wav)), ptr(_c128(f_scal)), C.byref(p))
    return f


def synthesis_wav2px(f_wav, f_scal, B, L, J_min, N, spin, upsample, spin_lowered=False, original_spin=0):
    p = _dir_params(B, L, J_min, N, spin, upsample, original_spin)
    f = np.zeros(mw_size(L), dtype=complex)
    _call("s2let_synthesis_wav2px", ptr(f), ptr(_c128(f_wav)), ptr(_c128(f_scal)), C.byref(p))
    return f


def synthesis_adjoint_px2wav(f, B, L, J_min, N, spin, upsample, spin_lowered=False, original_spin=0):
    p = _dir_params(B, L, J_min, N, spin, upsample, original_spin)
    nw, ns = _sizes(p)
    f_wav, f_scal = np.zeros(nw, dtype=complex), np.zeros(ns, dtype=complex)
    _call("s2let_synthesis_adjoint_px2wav", ptr(f_wav), ptr(f_scal), ptr(_c128(f)), C.byref(p))
    return f_wav, f_scal


def _tiling(p):
    lib = _lib_()
    J = lib.s2let_j_max(C.byref(p))
    wav_lm = np.zeros((J + 1) * p.L * p.L, dtype=complex)
    scal_l = np.zeros(p.L)
    _call("s2let_tiling_wavelet", ptr(wav_lm), ptr(scal_l), C.byref(p))
    return wav_lm, scal_l


def _lmn_split(name, flm, B, L, J_min, N, spin, upsample, original_spin):
    p = _dir_params(B, L, J_min, N, spin, upsample, original_spin)
    wav_lm, scal_l = _tiling(p)
    lib = _lib_()
    f_wav_lmn = np.zeros(lib.s2let_n_lmn_wav(C.byref(p)), dtype=complex)
    f_scal_lm = np.zeros(lib.s2let_n_lm_scal(C.byref(p)), dtype=complex)
    _call(name, ptr(f_wav_lmn), ptr(f_scal_lm), ptr(_c128(flm)), ptr(wav_lm), ptr(scal_l), C.byref(p))
    return f_wav_lmn, f_scal_lm


def _lmn_merge(name, f_wav_lmn, f_scal_lm, B, L, J_min, N, spin, upsample, original_spin):
    p = _dir_params(B, L, J_min, N, spin, upsample, original_spin)
    wav_lm, scal_l = _tiling(p)
    flm = np.zeros(L * L, dtype=complex)
    _call(name, ptr(flm), ptr(_c128(f_wav_lmn)), ptr(_c128(f_scal_lm)), ptr(wav_lm), ptr(scal_l), C.byref(p))
    return flm


def analysis_lm2lmn(flm, B, L, J_min, N, spin, upsample, spin_lowered=False, original_spin=0):
    return _lmn_split("s2let_analysis_lm2lmn", flm, B, L, J_min, N, spin, upsample, original_spin)


def synthesis_adjoint_lm2lmn(flm, B, L, J_min, N, spin, upsample, spin_lowered=False, original_spin=0):
    return _lmn_split("s2let_synthesis_adjoint_lm2lmn", flm, B, L, J_min, N, spin, upsample, original_spin)


def analysis_adjoint_lmn2lm(f_wav_lmn, f_scal_lm, B, L, J_min, N, spin, upsample, spin_lowered=False,
                            original_spin=0):
    return _lmn_merge("s2let_analysis_adjoint_lmn2lm", f_wav_lmn, f_scal_lm, B, L, J_min, N, spin, upsample,
                      original_spin)


def synthesis_lmn2lm(f_wav_lmn, f_scal_lm, B, L, J_min, N, spin, upsample, spin_lowered=False, original_spin=0):
    return _lmn_merge("s2let_synthesis_lmn2lm", f_wav_lmn, f_scal_lm, B, L, J_min, N, spin, upsample,
                      original_spin)


# ---- manual tilings ----------------------------------------------------------

def _manual_wav_lm(L, N, spin, kappa_wav_l, J):
    p = _params(0.0, L, 0, N, spin)
    s_elm = np.zeros(L * L, dtype=complex)
    _call("s2let_tiling_direction", ptr(s_elm), C.byref(p))
    el = np.floor(np.sqrt(np.arange(L * L))).astype(int)
    norm = np.sqrt((2 * el + 1) / (8.0 * np.pi * np.pi))
    kw = _f64(kappa_wav_l).reshape(J + 1, L)
    return np.concatenate([norm * kw[j][el] * s_elm for j in range(J + 1)])


def _manual_scal_l(L, kappa_scal_l):
    el = np.arange(L)
    return np.sqrt((2 * el + 1) / (4.0 * np.pi)) * _f64(kappa_scal_l)


def analysis_lm2wav_manualtiling(flm_hp, L, N, spin, kappa_scal_l, kappa_wav_l, scal_bandlimit, wav_bandlimits):
    wav_bandlimits = np.ascontiguousarray(wav_bandlimits, dtype=np.int32)
    J = wav_bandlimits.size - 1
    scal_l = _manual_scal_l(L, kappa_scal_l)
    wav_lm = _manual_wav_lm(L, N, spin, kappa_wav_l, J)
    n_scal = mw_size(int(scal_bandlimit))
    total = 0
    for j in range(J + 1):
        bl = min(int(wav_bandlimits[j]), L)
        Nj = min(N, bl)
        Nj += (Nj + N) % 2
        total += (2 * Nj - 1) * mw_size(bl)
    f_wav = np.zeros(total, dtype=complex)
    f_scal = np.zeros(n_scal, dtype=complex)
    f_lm = lm_hp2lm(flm_hp, L)
    print('scal_bandlimit =', int(scal_bandlimit))
    print('wav_bandlimits =', wav_bandlimits)
    print('J, L, spin, N =', J, L, spin, N)
    print('Done pre-computing - running s2let_analysis_lm2wav_manual')
    _call("s2let_analysis_lm2wav_manual", ptr(f_wav), ptr(f_scal), ptr(f_lm), ptr(scal_l), ptr(wav_lm),
          int(scal_bandlimit), ptr(wav_bandlimits), J, L, spin, N)
    return f_wav, f_scal


def synthesis_wav2lm_manualtiling(f_wav, f_scal, L, N, spin, kappa_scal_l, kappa_wav_l, scal_bandlimit,
                                  wav_bandlimits):
    wav_bandlimits = np.ascontiguousarray(wav_bandlimits, dtype=np.int32)
    J = wav_bandlimits.size - 1
    scal_l = _manual_scal_l(L, kappa_scal_l)
    wav_lm = _manual_wav_lm(L, N, spin, kappa_wav_l, J)
    f_lm = np.zeros(L * L, dtype=complex)
    print('Done pre-computing - running s2let_synthesis_wav2lm_manual')
    _call("s2let_synthesis_wav2lm_manual", ptr(f_lm), ptr(_c128(f_wav)), ptr(_c128(f_scal)), ptr(scal_l),
          ptr(wav_lm), int(scal_bandlimit), ptr(wav_bandlimits), J, L, spin, N)
    return lm2lm_hp(f_lm, L)


# ---- plain SHT and Wigner d ----------------------------------------------------

def alm2map_mw(f_lm, L, spin):
    f = np.zeros(mw_size(L), dtype=complex)
    _call("s2let_mw_alm2map", ptr(f), ptr(_c128(f_lm)), L, spin)
    return f


def map2alm_mw(f, L, spin):
    f_lm = np.zeros(L * L, dtype=complex)
    _call("s2let_mw_map2alm", ptr(f_lm), ptr(_c128(f)), L, spin)
    return f_lm


def ssht_dl_beta_risbo(beta, L):
    """Wigner d^l_{m,m'}(beta) for all l < L, as dl[l, m + L - 1, m' + L - 1].

    Computed by Risbo's recursion (T. Risbo, J. Geodesy 70, 1996): the
    degree-l matrix is built from degree l - 1/2 by two half-step updates
    with the coefficients p = cos(beta/2), q = sin(beta/2).  The full matrix is
    returned (-l <= m, m' <= l); entries outside |m|, |m'| <= l are zero.
    """
    K = 2 * L - 1
    out = np.zeros((L, K, K))
    p_, q_ = np.cos(beta / 2.0), np.sin(beta / 2.0)
    # d for degree j = twice-degree / 2, indexed [m + j, m' + j] with 2j + 1 rows
    d = np.ones((1, 1))
    sq = np.sqrt(np.arange(2 * L + 2, dtype=float))
    jj = 0  # twice the current degree
    out[0, L - 1, L - 1] = 1.0
    for step in range(1, 2 * (L - 1) + 1):
        n = jj + 1  # new twice-degree
        new = np.zeros((n + 1, n + 1))
        # Risbo half-step: d^{n/2}_{i,k} from d^{(n-1)/2}_{i,k}
        for i in range(jj + 1):
            for k in range(jj + 1):
                v = d[i, k] / n
                a, b = sq[n - i], sq[i + 1]
                c, e = sq[n - k], sq[k + 1]
                new[i, k] += a * c * v * p_
                new[i + 1, k] -= b * c * v * q_
                new[i, k + 1] += a * e * v * q_
                new[i + 1, k + 1] += b * e * v * p_
        d, jj = new, n
        if jj % 2 == 0:
            l = jj // 2
            out[l, L - 1 - l:L + l, L - 1 - l:L + l] = d
    return out
