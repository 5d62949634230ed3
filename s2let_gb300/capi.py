"""ctypes description of the S2LET C ABI declared in include/s2let_gpu.h.

The same table binds any shared library that exports the S2LET API: the GPU
library libs2let_gpu.so built from s2let_gb300/csrc, and (in tests only) CPU
checkers.  `S2letParameters` mirrors ``s2let_parameters_t``
(include/s2let/s2let_types.h:56-137 of the reference) field for field.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

SAMPLING_MW = 0
SAMPLING_MW_SS = 1


class S2letParameters(C.Structure):
    """``s2let_parameters_t``; field order and C types are part of the ABI."""

    _fields_ = [
        ("verbosity", C.c_int),
        ("reality", C.c_int),
        ("upsample", C.c_int),
        ("B", C.c_double),
        ("L", C.c_int),
        ("J_min", C.c_int),
        ("N", C.c_int),
        ("spin", C.c_int),
        ("original_spin", C.c_int),
        ("sampling_scheme", C.c_int),
        ("dl_method", C.c_int),
    ]


def make_parameters(L, B=2.0, J_min=0, N=1, spin=0, upsample=0, reality=0, original_spin=0,
                    sampling_scheme=SAMPLING_MW, dl_method=0, verbosity=0) -> S2letParameters:
    return S2letParameters(verbosity, reality, upsample, float(B), L, J_min, N, spin,
                           original_spin, sampling_scheme, dl_method)


P = C.POINTER(S2letParameters)
V = C.c_void_p
I = C.c_int

# name -> (restype, argtypes)
SIGNATURES = {
    # tiling / helpers
    "s2let_switch_wavtype": (None, [I]),
    "s2let_bandlimit": (I, [I, P]),
    "s2let_L0": (I, [I, P]),
    "s2let_j_max": (I, [P]),
    "s2let_tiling_axisym": (None, [V, V, P]),
    "s2let_tiling_direction": (None, [V, P]),
    "s2let_tiling_wavelet": (None, [V, V, P]),
    "s2let_tiling_axisym_check_identity": (C.c_double, [V, V, P]),
    "s2let_tiling_direction_check_identity": (C.c_double, [V, P]),
    "s2let_tiling_wavelet_check_identity": (C.c_double, [V, V, P]),
    "s2let_n_phi": (I, [P]),
    "s2let_n_theta": (I, [P]),
    "s2let_n_px": (I, [P]),
    "s2let_n_lm": (I, [P]),
    "s2let_n_lm_scal": (I, [P]),
    "s2let_n_lmn_wav": (I, [P]),
    "s2let_n_gamma": (I, [P]),
    "s2let_n_scal": (I, [P]),
    "s2let_n_wav": (I, [P]),
    "s2let_n_wav_j": (I, [I, P]),
    # directional
    "s2let_analysis_lm2lmn": (None, [V, V, V, V, V, P]),
    "s2let_analysis_lm2lmn_real": (None, [V, V, V, V, V, P]),
    "s2let_analysis_lm2wav": (None, [V, V, V, P]),
    "s2let_analysis_lm2wav_real": (None, [V, V, V, P]),
    "s2let_analysis_px2wav": (None, [V, V, V, P]),
    "s2let_analysis_px2wav_real": (None, [V, V, V, P]),
    "s2let_synthesis_lmn2lm": (None, [V, V, V, V, V, P]),
    "s2let_synthesis_lmn2lm_real": (None, [V, V, V, V, V, P]),
    "s2let_synthesis_wav2lm": (None, [V, V, V, P]),
    "s2let_synthesis_wav2lm_real": (None, [V, V, V, P]),
    "s2let_synthesis_wav2px": (None, [V, V, V, P]),
    "s2let_synthesis_wav2px_real": (None, [V, V, V, P]),
    "s2let_analysis_adjoint_lmn2lm": (None, [V, V, V, V, V, P]),
    "s2let_analysis_adjoint_lmn2lm_real": (None, [V, V, V, V, V, P]),
    "s2let_analysis_adjoint_wav2lm": (None, [V, V, V, P]),
    "s2let_analysis_adjoint_wav2lm_real": (None, [V, V, V, P]),
    "s2let_analysis_adjoint_wav2px": (None, [V, V, V, P]),
    "s2let_analysis_adjoint_wav2px_real": (None, [V, V, V, P]),
    "s2let_synthesis_adjoint_lm2lmn": (None, [V, V, V, V, V, P]),
    "s2let_synthesis_adjoint_lm2lmn_real": (None, [V, V, V, V, V, P]),
    "s2let_synthesis_adjoint_lm2wav": (None, [V, V, V, P]),
    "s2let_synthesis_adjoint_lm2wav_real": (None, [V, V, V, P]),
    "s2let_synthesis_adjoint_px2wav": (None, [V, V, V, P]),
    "s2let_synthesis_adjoint_px2wav_real": (None, [V, V, V, P]),
    # manual tiling
    "s2let_analysis_lm2wav_manual": (None, [V, V, V, V, V, I, V, I, I, I, I]),
    "s2let_synthesis_wav2lm_manual": (None, [V, V, V, V, V, I, V, I, I, I, I]),
    "s2let_analysis_adjoint_wav2lm_manual": (None, [V, V, V, V, V, I, V, I, I, I, I]),
    "s2let_synthesis_adjoint_lm2wav_manual": (None, [V, V, V, V, V, I, V, I, I, I, I]),
    # axisymmetric
    "s2let_transform_axisym_lm_wav": (None, [V, V, P]),
    "s2let_transform_axisym_lm_wav_analysis": (None, [V, V, V, V, V, P]),
    "s2let_transform_axisym_lm_wav_synthesis": (None, [V, V, V, V, V, P]),
    "s2let_transform_axisym_lm_wav_analysis_multires": (None, [V, V, V, V, V, P]),
    "s2let_transform_axisym_lm_wav_synthesis_multires": (None, [V, V, V, V, V, P]),
    "s2let_transform_axisym_wav_hardthreshold_real": (None, [V, V, P]),
    "s2let_transform_axisym_wav_hardthreshold_multires_real": (None, [V, V, P]),
    # plain MW SHT
    "s2let_mw_alm2map": (None, [V, V, I, I]),
    "s2let_mw_map2alm": (None, [V, V, I, I]),
    "s2let_mw_alm2map_real": (None, [V, V, I]),
    "s2let_mw_map2alm_real": (None, [V, V, I]),
}
for _op in ("analysis", "analysis_adjoint", "synthesis", "synthesis_adjoint"):
    for _suf in ("", "_multires", "_real", "_multires_real"):
        SIGNATURES[f"s2let_transform_axisym_wav_{_op}_mw{_suf}"] = (None, [V, V, V, P])

# FITS I/O of MW / MWSS maps (host code of libs2let_gpu.so; not in the oracle)
FITS_SIGNATURES = {
    "s2let_fits_mw_read_bandlimit": (I, [C.c_char_p]),
    "s2let_fits_hpx_read_nside": (I, [C.c_char_p]),
    "s2let_fits_mw_read_map": (None, [V, C.c_char_p, I]),
    "s2let_fits_mwss_read_map": (None, [V, C.c_char_p, I]),
    "s2let_fits_mw_write_map": (None, [C.c_char_p, V, I]),
    "s2let_fits_mwss_write_map": (None, [C.c_char_p, V, I]),
    "s2let_fits_mw_read_spin_maps": (None, [V, V, C.c_char_p, I]),
    "s2let_fits_mwss_read_spin_maps": (None, [V, V, C.c_char_p, I]),
    "s2let_fits_mw_write_spin_maps": (None, [C.c_char_p, V, V, I]),
    "s2let_fits_mwss_write_spin_maps": (None, [C.c_char_p, V, V, I]),
}

GPU_SIGNATURES = {
    "s2let_gpu_last_error": (I, []),
    "s2let_gpu_last_error_string": (C.c_char_p, []),
    "s2let_gpu_set_precision": (I, [I]),
    "s2let_gpu_set_split_tables": (I, [I]),
    "s2let_gpu_get_split_tables": (I, []),
    "s2let_gpu_set_df_max_maps": (I, [I]),
    "s2let_gpu_get_df_max_maps": (I, []),
    "s2let_gpu_get_precision": (I, []),
    "s2let_gpu_set_table_mode": (I, [I]),
    "s2let_gpu_get_table_mode": (I, []),
    "s2let_gpu_release_plans": (None, []),
    "s2let_gpu_plan_bytes": (C.c_size_t, []),
    "s2let_gpu_launch_count": (C.c_uint64, []),
    "s2let_gpu_device_fault": (I, []),
    "s2let_gpu_timing_enable": (I, [I]),
    "s2let_gpu_timing_report": (I, [V, I]),
    "s2let_gpu_copy_trace_enable": (I, [I]),
    "s2let_gpu_copy_trace_report": (I, [V]),
    "s2let_gpu_bind_device": (I, [I]),
    "s2let_gpu_fma_rate": (I, [I, I, V]),
    "s2let_gpu_bound_device": (I, []),
    "s2let_gpu_axisym_wav_hardthreshold_real_noalloc": (I, [V, V, P, I]),
    "s2let_gpu_mw_adjoint_map2alm": (None, [V, V, I, I]),
    "s2let_gpu_mw_adjoint_alm2map": (None, [V, V, I, I]),
    "s2let_gpu_sht": (I, [I, I, I, I, I, V, V]),
    "s2let_gpu_analysis_px2wav_real_host_batch": (I, [V, V, V, I, P]),
    "s2let_gpu_synthesis_wav2px_real_host_batch": (I, [V, V, V, I, P]),
    "s2let_gpu_analysis_px2wav_host_batch": (I, [V, V, V, I, P]),
    "s2let_gpu_synthesis_wav2px_host_batch": (I, [V, V, V, I, P]),
    "s2let_gpu_px2wav_multi": (I, [V, V, V, P, V, I, I, V]),
    "s2let_gpu_wav2px_multi": (I, [V, V, V, P, V, I, I, V]),
    "s2let_gpu_analysis_px2wav_real_batch": (I, [V, V, V, I, P, V]),
    "s2let_gpu_synthesis_wav2px_real_batch": (I, [V, V, V, I, P, V]),
    "s2let_gpu_analysis_px2wav_batch": (I, [V, V, V, I, P, V]),
    "s2let_gpu_synthesis_wav2px_batch": (I, [V, V, V, I, P, V]),
    "s2let_gpu_analysis_adjoint_wav2px_real_batch": (I, [V, V, V, I, P, V]),
    "s2let_gpu_synthesis_adjoint_px2wav_real_batch": (I, [V, V, V, I, P, V]),
    "s2let_gpu_analysis_adjoint_wav2px_batch": (I, [V, V, V, I, P, V]),
    "s2let_gpu_synthesis_adjoint_px2wav_batch": (I, [V, V, V, I, P, V]),
    "s2let_gpu_analysis_px2wav_real_batch_f32": (I, [V, V, V, I, P, V]),
    "s2let_gpu_synthesis_wav2px_real_batch_f32": (I, [V, V, V, I, P, V]),
    "s2let_gpu_analysis_px2wav_batch_f32": (I, [V, V, V, I, P, V]),
    "s2let_gpu_synthesis_wav2px_batch_f32": (I, [V, V, V, I, P, V]),
    "s2let_gpu_analysis_adjoint_wav2px_real_batch_f32": (I, [V, V, V, I, P, V]),
    "s2let_gpu_synthesis_adjoint_px2wav_real_batch_f32": (I, [V, V, V, I, P, V]),
    "s2let_gpu_analysis_adjoint_wav2px_batch_f32": (I, [V, V, V, I, P, V]),
    "s2let_gpu_synthesis_adjoint_px2wav_batch_f32": (I, [V, V, V, I, P, V]),
    "s2let_gpu_autotune": (I, [I]),
    "s2let_gpu_autotune_entries": (I, [V, V, I]),
    "s2let_gpu_px2wav_multi_f32": (I, [V, V, V, P, V, I, I, V]),
    "s2let_gpu_wav2px_multi_f32": (I, [V, V, V, P, V, I, I, V]),
}


def bind(lib: C.CDLL, table=SIGNATURES, required=True) -> C.CDLL:
    """Attach restype/argtypes of `table` to the functions `lib` exports."""
    for name, (res, args) in table.items():
        try:
            fn = getattr(lib, name)
        except AttributeError:
            if required:
                raise
            continue
        fn.restype = res
        fn.argtypes = args
    return lib


def ptr(a: np.ndarray) -> C.c_void_p:
    assert a.flags["C_CONTIGUOUS"]
    return C.c_void_p(a.ctypes.data)


class S2let:
    """Thin numpy front-end over a library exporting the S2LET C API.

    Method names drop the ``s2let_`` prefix; arrays are allocated here with the
    sizes the reference helpers report.
    """

    def __init__(self, lib: C.CDLL):
        self.lib = lib

    # sizes -----------------------------------------------------------------
    def sizes(self, p: S2letParameters):
        r = C.byref(p)
        return dict(n_px=self.lib.s2let_n_px(r), n_wav=self.lib.s2let_n_wav(r),
                    n_scal=self.lib.s2let_n_scal(r), n_lm=p.L * p.L,
                    n_lmn=self.lib.s2let_n_lmn_wav(r), n_lm_scal=self.lib.s2let_n_lm_scal(r),
                    J=self.lib.s2let_j_max(r))

    # pixel-space directional transforms -------------------------------------
    def px2wav(self, f, p, real=False):
        s = self.sizes(p)
        dt = np.float64 if real else np.complex128
        f = np.ascontiguousarray(f, dtype=dt)
        w = np.zeros(s["n_wav"], dt)
        sc = np.zeros(s["n_scal"], dt)
        fn = self.lib.s2let_analysis_px2wav_real if real else self.lib.s2let_analysis_px2wav
        fn(ptr(w), ptr(sc), ptr(f), C.byref(p))
        return w, sc

    def wav2px(self, w, sc, p, real=False):
        s = self.sizes(p)
        dt = np.float64 if real else np.complex128
        w = np.ascontiguousarray(w, dtype=dt)
        sc = np.ascontiguousarray(sc, dtype=dt)
        f = np.zeros(s["n_px"], dt)
        fn = self.lib.s2let_synthesis_wav2px_real if real else self.lib.s2let_synthesis_wav2px
        fn(ptr(f), ptr(w), ptr(sc), C.byref(p))
        return f

    def analysis_adjoint_wav2px(self, w, sc, p, real=False):
        s = self.sizes(p)
        dt = np.float64 if real else np.complex128
        w = np.ascontiguousarray(w, dtype=dt)
        sc = np.ascontiguousarray(sc, dtype=dt)
        f = np.zeros(s["n_px"], dt)
        fn = (self.lib.s2let_analysis_adjoint_wav2px_real if real
              else self.lib.s2let_analysis_adjoint_wav2px)
        fn(ptr(f), ptr(w), ptr(sc), C.byref(p))
        return f

    def synthesis_adjoint_px2wav(self, f, p, real=False):
        s = self.sizes(p)
        dt = np.float64 if real else np.complex128
        f = np.ascontiguousarray(f, dtype=dt)
        w = np.zeros(s["n_wav"], dt)
        sc = np.zeros(s["n_scal"], dt)
        fn = (self.lib.s2let_synthesis_adjoint_px2wav_real if real
              else self.lib.s2let_synthesis_adjoint_px2wav)
        fn(ptr(w), ptr(sc), ptr(f), C.byref(p))
        return w, sc

    # harmonic-space directional transforms ----------------------------------
    def lm2wav(self, flm, p, real=False):
        s = self.sizes(p)
        dt = np.float64 if real else np.complex128
        flm = np.ascontiguousarray(flm, dtype=np.complex128)
        w = np.zeros(s["n_wav"], dt)
        sc = np.zeros(s["n_scal"], dt)
        fn = self.lib.s2let_analysis_lm2wav_real if real else self.lib.s2let_analysis_lm2wav
        fn(ptr(w), ptr(sc), ptr(flm), C.byref(p))
        return w, sc

    def wav2lm(self, w, sc, p, real=False):
        dt = np.float64 if real else np.complex128
        w = np.ascontiguousarray(w, dtype=dt)
        sc = np.ascontiguousarray(sc, dtype=dt)
        flm = np.zeros(p.L * p.L, np.complex128)
        fn = self.lib.s2let_synthesis_wav2lm_real if real else self.lib.s2let_synthesis_wav2lm
        fn(ptr(flm), ptr(w), ptr(sc), C.byref(p))
        return flm

    def analysis_adjoint_wav2lm(self, w, sc, p, real=False):
        dt = np.float64 if real else np.complex128
        w = np.ascontiguousarray(w, dtype=dt)
        sc = np.ascontiguousarray(sc, dtype=dt)
        flm = np.zeros(p.L * p.L, np.complex128)
        fn = (self.lib.s2let_analysis_adjoint_wav2lm_real if real
              else self.lib.s2let_analysis_adjoint_wav2lm)
        fn(ptr(flm), ptr(w), ptr(sc), C.byref(p))
        return flm

    def synthesis_adjoint_lm2wav(self, flm, p, real=False):
        s = self.sizes(p)
        dt = np.float64 if real else np.complex128
        flm = np.ascontiguousarray(flm, dtype=np.complex128)
        w = np.zeros(s["n_wav"], dt)
        sc = np.zeros(s["n_scal"], dt)
        fn = (self.lib.s2let_synthesis_adjoint_lm2wav_real if real
              else self.lib.s2let_synthesis_adjoint_lm2wav)
        fn(ptr(w), ptr(sc), ptr(flm), C.byref(p))
        return w, sc

    def tiling(self, p):
        J = self.lib.s2let_j_max(C.byref(p))
        psi = np.zeros((J + 1) * p.L * p.L, np.complex128)
        phi = np.zeros(p.L, np.float64)
        self.lib.s2let_tiling_wavelet(ptr(psi), ptr(phi), C.byref(p))
        return psi, phi

    def lm2lmn(self, flm, p, real=False, adjoint_of_synthesis=False):
        s = self.sizes(p)
        psi, phi = self.tiling(p)
        flm = np.ascontiguousarray(flm, dtype=np.complex128)
        # generous buffers: the reference sizes these with s2let_n_lmn_wav
        lmn = np.zeros(max(s["n_lmn"], 1) * 2, np.complex128)
        sc = np.zeros(max(s["n_lm_scal"], 1), np.complex128)
        name = "s2let_synthesis_adjoint_lm2lmn" if adjoint_of_synthesis else "s2let_analysis_lm2lmn"
        getattr(self.lib, name + ("_real" if real else ""))(
            ptr(lmn), ptr(sc), ptr(flm), ptr(psi), ptr(phi), C.byref(p))
        return lmn, sc

    def lmn2lm(self, lmn, sc, p, real=False, adjoint_of_analysis=False):
        psi, phi = self.tiling(p)
        lmn = np.ascontiguousarray(lmn, dtype=np.complex128)
        sc = np.ascontiguousarray(sc, dtype=np.complex128)
        flm = np.zeros(p.L * p.L, np.complex128)
        name = "s2let_analysis_adjoint_lmn2lm" if adjoint_of_analysis else "s2let_synthesis_lmn2lm"
        getattr(self.lib, name + ("_real" if real else ""))(
            ptr(flm), ptr(lmn), ptr(sc), ptr(psi), ptr(phi), C.byref(p))
        return flm

    # plain SHT --------------------------------------------------------------
    def alm2map(self, flm, L, spin=0, real=False):
        flm = np.ascontiguousarray(flm, dtype=np.complex128)
        if real:
            f = np.zeros(L * (2 * L - 1), np.float64)
            self.lib.s2let_mw_alm2map_real(ptr(f), ptr(flm), L)
        else:
            f = np.zeros(L * (2 * L - 1), np.complex128)
            self.lib.s2let_mw_alm2map(ptr(f), ptr(flm), L, spin)
        return f

    def map2alm(self, f, L, spin=0, real=False):
        flm = np.zeros(L * L, np.complex128)
        if real:
            f = np.ascontiguousarray(f, dtype=np.float64)
            self.lib.s2let_mw_map2alm_real(ptr(flm), ptr(f), L)
        else:
            f = np.ascontiguousarray(f, dtype=np.complex128)
            self.lib.s2let_mw_map2alm(ptr(flm), ptr(f), L, spin)
        return flm

    def sht(self, direction, x, L, spin=0, real=False, sampling=SAMPLING_MW):
        """s2let_gpu_sht: direction 0 forward (map -> flm), 1 inverse, 2 adjoint
        of the forward (flm -> map), 3 adjoint of the inverse (map -> flm), on
        MW or MWSS sampling."""
        npx = (L + 1) * 2 * L if sampling == SAMPLING_MW_SS else L * (2 * L - 1)
        fdt = np.float64 if real else np.complex128
        if direction in (0, 3):
            f = np.ascontiguousarray(x, dtype=fdt)
            flm = np.zeros(L * L, np.complex128)
        else:
            flm = np.ascontiguousarray(x, dtype=np.complex128)
            f = np.zeros(npx, fdt)
        st = self.lib.s2let_gpu_sht(direction, sampling, L, spin, int(real), ptr(f), ptr(flm))
        if st != 0:
            raise RuntimeError(f"s2let_gpu_sht failed with status {st}")
        return flm if direction in (0, 3) else f

    # axisymmetric -------------------------------------------------------------
    def axisym_sizes(self, p, multires):
        J = self.lib.s2let_j_max(C.byref(p))
        L = p.L
        if not multires:
            return (J + 1 - p.J_min) * L * (2 * L - 1), L * (2 * L - 1)
        tot = 0
        for j in range(p.J_min, J + 1):
            bl = min(self.lib.s2let_bandlimit(j, C.byref(p)), L)
            tot += bl * (2 * bl - 1)
        bs = min(self.lib.s2let_bandlimit(p.J_min - 1, C.byref(p)), L)
        return tot, bs * (2 * bs - 1)

    def axisym_lm_kernels(self, p):
        """(wav_lm, scal_lm) of s2let_transform_axisym_lm_wav: rows of L per scale."""
        J = self.lib.s2let_j_max(C.byref(p))
        wav = np.zeros((J + 1) * p.L, np.float64)
        scal = np.zeros(p.L, np.float64)
        self.lib.s2let_transform_axisym_lm_wav(ptr(wav), ptr(scal), C.byref(p))
        return wav, scal

    def axisym_lm_sizes(self, p, multires):
        """Sizes of f_wav_lm and f_scal_lm (s2let_transform_axisym_lm_allocate_f_wav[_multires])."""
        J = self.lib.s2let_j_max(C.byref(p))
        L = p.L
        if not multires:
            return (J + 1 - p.J_min) * L * L, L * L
        tot = sum(min(self.lib.s2let_bandlimit(j, C.byref(p)), L) ** 2 for j in range(p.J_min, J + 1))
        bs = min(self.lib.s2let_bandlimit(p.J_min - 1, C.byref(p)), L)
        return tot, bs * bs

    def axisym_lm_analysis(self, flm, p, multires=False):
        wav, scal = self.axisym_lm_kernels(p)
        nw, ns = self.axisym_lm_sizes(p, multires)
        flm = np.ascontiguousarray(flm, dtype=np.complex128)
        fw = np.zeros(nw, np.complex128)
        fs = np.zeros(ns, np.complex128)
        fn = (self.lib.s2let_transform_axisym_lm_wav_analysis_multires if multires
              else self.lib.s2let_transform_axisym_lm_wav_analysis)
        fn(ptr(fw), ptr(fs), ptr(flm), ptr(wav), ptr(scal), C.byref(p))
        return fw, fs

    def axisym_lm_synthesis(self, fw, fs, p, multires=False):
        wav, scal = self.axisym_lm_kernels(p)
        fw = np.ascontiguousarray(fw, dtype=np.complex128)
        fs = np.ascontiguousarray(fs, dtype=np.complex128)
        flm = np.zeros(p.L * p.L, np.complex128)
        fn = (self.lib.s2let_transform_axisym_lm_wav_synthesis_multires if multires
              else self.lib.s2let_transform_axisym_lm_wav_synthesis)
        fn(ptr(flm), ptr(fw), ptr(fs), ptr(wav), ptr(scal), C.byref(p))
        return flm

    def axisym(self, op, arrays, p, multires=False, real=False):
        """op in {'analysis', 'analysis_adjoint', 'synthesis', 'synthesis_adjoint'}."""
        nw, ns = self.axisym_sizes(p, multires)
        npx = p.L * (2 * p.L - 1)
        dt = np.float64 if real else np.complex128
        name = f"s2let_transform_axisym_wav_{op}_mw" + ("_multires" if multires else "") + \
            ("_real" if real else "")
        fn = getattr(self.lib, name)
        if op in ("analysis", "synthesis_adjoint"):
            f = np.ascontiguousarray(arrays[0], dtype=dt)
            w = np.zeros(nw, dt)
            s = np.zeros(ns, dt)
            fn(ptr(w), ptr(s), ptr(f), C.byref(p))
            return w, s
        w = np.ascontiguousarray(arrays[0], dtype=dt)
        s = np.ascontiguousarray(arrays[1], dtype=dt)
        f = np.zeros(npx, dt)
        fn(ptr(f), ptr(w), ptr(s), C.byref(p))
        return f
