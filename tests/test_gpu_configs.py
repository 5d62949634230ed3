"""GPU parity at the sizes of the benchmark configurations, through the C ABI.

* Axisymmetric, L=128, B=2, J_min=0, one real map (full resolution and
  multiresolution): the four axisym_wav_*_mw operators (real and complex) and
  the harmonic axisym_lm_wav analysis / synthesis (+ multires) element-wise
  against the oracle (src/c/s2let_transform_axisym_lm.c:133-308,
  src/c/s2let_transform_axisym_mw.c:124-1171), plus the reference-generated
  axi_*.npz fixtures run on the GPU.
* Directional, real, L=512, N=4, B=2, J_min=2 (multiresolution), FP64:
  px2wav / wav2px and both adjoints against the oracle.
* Complex spin-2, L=1024, N=5, B=2, J_min=3: FP64 against the oracle on one
  map, and the split-precision path against the FP64 path scale by scale, on
  one map and on a host batch of three.

Inputs follow the benchmark spectra: complex Gaussian flm with C_l = (l+1)^-2
(spin 0, real-field symmetry, f_00 = 0) or l^-2 for l >= 2 (spin 2),
synthesised to MW pixels by the oracle's inverse SHT.

Tolerances (normwise relative max error, max|a - b| / max|b|): FP64 path
1e-12 against the oracle; split precision 1e-10 against the FP64 path for
every output and every scale.  At J_min = 0 the scaling band-limit is 1 (the
l = 0 term only) and f_00 = 0, so the scaling map is rounding noise of the
input's scale on both sides: it is compared relative to max|f| instead.
"""
import glob
import os

import numpy as np
import pytest

from conftest import power_law_flm, rel_err
from s2let_gb300.capi import make_parameters

TOL = 1e-12
TOL_MIXED = 1e-10


def rel_err_to(a, b, scale):
    """max|a - b| relative to the larger of max|b| and `scale`."""
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(b).max(), scale))


def _release(gpu):
    """Drop cached plans so large cases run with the device to themselves."""
    gpu.lib.s2let_gpu_release_plans()
    assert gpu.lib.s2let_gpu_last_error() == 0


# --------------------------------------------------------------------------
# axisymmetric, L = 128, B = 2, J_min = 0
# --------------------------------------------------------------------------
AXI_L, AXI_B, AXI_JMIN = 128, 2.0, 0


@pytest.mark.gpu
@pytest.mark.parametrize("multires", [False, True], ids=["fullres", "multires"])
@pytest.mark.parametrize("real", [True, False], ids=["real", "complex"])
def test_axisym_mw_L128(gpu, oracle_port, multires, real):
    L = AXI_L
    p = make_parameters(L, AXI_B, AXI_JMIN, 1, 0, 1)
    rng = np.random.default_rng(0)
    flm = power_law_flm(rng, L, real=True)
    f = oracle_port.alm2map(flm, L, real=True)
    if not real:  # a complex spin-0 map: the real map plus i times a second one
        f = f + 1j * oracle_port.alm2map(power_law_flm(rng, L, real=True), L, real=True)
    fmax = np.abs(f).max()
    wo, so = oracle_port.axisym("analysis", [f], p, multires, real)
    wg, sg = gpu.axisym("analysis", [f], p, multires, real)
    assert rel_err(wg, wo) < TOL and rel_err_to(sg, so, fmax) < TOL
    for op in ("synthesis", "analysis_adjoint"):
        assert rel_err(gpu.axisym(op, [wo, so], p, multires, real),
                       oracle_port.axisym(op, [wo, so], p, multires, real)) < TOL, op
    ao = oracle_port.axisym("synthesis_adjoint", [f], p, multires, real)
    ag = gpu.axisym("synthesis_adjoint", [f], p, multires, real)
    assert rel_err(ag[0], ao[0]) < TOL and rel_err_to(ag[1], ao[1], fmax) < TOL
    # exact round trip on the band-limited map
    assert rel_err(gpu.axisym("synthesis", [wg, sg], p, multires, real), f) < TOL


@pytest.mark.gpu
@pytest.mark.parametrize("multires", [False, True], ids=["fullres", "multires"])
def test_axisym_lm_wav_L128(gpu, oracle_port, multires):
    """s2let_transform_axisym_lm_wav_{analysis,synthesis}[_multires] element-wise
    against the oracle, with the kernels of s2let_transform_axisym_lm_wav."""
    L = AXI_L
    p = make_parameters(L, AXI_B, AXI_JMIN, 1, 0, 1)
    rng = np.random.default_rng(0)
    flm = power_law_flm(rng, L, real=True)
    wk_g, sk_g = gpu.axisym_lm_kernels(p)
    wk_o, sk_o = oracle_port.axisym_lm_kernels(p)
    assert rel_err(wk_g, wk_o) < 1e-15 and rel_err(sk_g, sk_o) < 1e-15
    fw_o, fs_o = oracle_port.axisym_lm_analysis(flm, p, multires)
    fw_g, fs_g = gpu.axisym_lm_analysis(flm, p, multires)
    assert fw_g.shape == fw_o.shape and fs_g.shape == fs_o.shape
    assert rel_err(fw_g, fw_o) < TOL and rel_err_to(fs_g, fs_o, np.abs(flm).max()) < TOL
    back_o = oracle_port.axisym_lm_synthesis(fw_o, fs_o, p, multires)
    back_g = gpu.axisym_lm_synthesis(fw_o, fs_o, p, multires)
    assert rel_err(back_g, back_o) < TOL
    assert rel_err(back_g, flm) < TOL  # the axisymmetric kernels tile exactly


AXI_GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "axi_*.npz")))


@pytest.mark.gpu
@pytest.mark.parametrize("path", AXI_GOLDEN, ids=lambda p: os.path.basename(p)[:-4])
def test_axisym_reference_golden_on_gpu(gpu, path):
    """The GPU against vectors produced by the reference's own
    s2let_transform_axisym_wav_{analysis,synthesis}_mw[_multires]_real."""
    g = np.load(path)
    L, B, J_min = g["params"]
    p = make_parameters(int(L), B, int(J_min), 1, 0, 0)
    for mr in (0, 1):
        w, s = gpu.axisym("analysis", [g["f"]], p, bool(mr), True)
        assert rel_err(w, g[f"ana_mr{mr}_wav"]) < TOL
        assert rel_err_to(s, g[f"ana_mr{mr}_scal"], np.abs(g["f"]).max()) < TOL
        back = gpu.axisym("synthesis", [g[f"ana_mr{mr}_wav"], g[f"ana_mr{mr}_scal"]], p, bool(mr), True)
        assert rel_err(back, g[f"syn_mr{mr}"]) < TOL


# --------------------------------------------------------------------------
# directional, real, L = 512, N = 4, B = 2, J_min = 2, FP64
# --------------------------------------------------------------------------


@pytest.mark.gpu
def test_directional_real_L512_fp64(gpu, oracle_port):
    _release(gpu)
    L = 512
    p = make_parameters(L, 2.0, 2, 4, 0, 0)
    rng = np.random.default_rng(0)
    f = oracle_port.alm2map(power_law_flm(rng, L, real=True), L, real=True)
    assert gpu.lib.s2let_gpu_get_precision() == 0
    w_o, s_o = oracle_port.px2wav(f, p, real=True)
    w_g, s_g = gpu.px2wav(f, p, real=True)
    assert rel_err(w_g, w_o) < TOL and rel_err(s_g, s_o) < TOL
    fr_o = oracle_port.wav2px(w_o, s_o, p, real=True)
    fr_g = gpu.wav2px(w_o, s_o, p, real=True)
    assert rel_err(fr_g, fr_o) < TOL
    assert rel_err(fr_g, f) < TOL
    # adjoints on inputs that are not in the range of the transforms
    g2 = rng.normal(size=f.size)
    bo = oracle_port.synthesis_adjoint_px2wav(g2, p, real=True)
    bg = gpu.synthesis_adjoint_px2wav(g2, p, real=True)
    assert rel_err(bg[0], bo[0]) < TOL and rel_err(bg[1], bo[1]) < TOL
    wr = rng.normal(size=w_o.size)
    sr = rng.normal(size=s_o.size)
    assert rel_err(gpu.analysis_adjoint_wav2px(wr, sr, p, real=True),
                   oracle_port.analysis_adjoint_wav2px(wr, sr, p, real=True)) < TOL
    _release(gpu)


# --------------------------------------------------------------------------
# complex spin-2, L = 1024, N = 5, B = 2, J_min = 3
# --------------------------------------------------------------------------


def _scales(gpu, p):
    """(j, offset, length) of every scale block inside f_wav, advancing with the
    parity-fixed N_j (src/c/s2let_analysis.c:340-350)."""
    import ctypes as C

    J = gpu.lib.s2let_j_max(C.byref(p))
    out, off = [], 0
    for j in range(p.J_min, J + 1):
        bl = min(gpu.lib.s2let_bandlimit(j, C.byref(p)), p.L)
        Nj = min(p.N, bl)
        Nj += (Nj + p.N) % 2
        n = (2 * Nj - 1) * bl * (2 * bl - 1)
        out.append((j, off, n))
        off += n
    return out


@pytest.mark.gpu
def test_spin2_L1024_N5(gpu, oracle_port):
    _release(gpu)
    L = 1024
    p = make_parameters(L, 2.0, 3, 5, 2, 0)
    rng = np.random.default_rng(0)
    f = oracle_port.alm2map(power_law_flm(rng, L, spin=2), L, 2)
    lib = gpu.lib
    assert lib.s2let_gpu_set_precision(0) == 0
    w64, s64 = gpu.px2wav(f, p)
    fr64 = gpu.wav2px(w64, s64, p)
    # FP64 against the oracle on this map
    w_o, s_o = oracle_port.px2wav(f, p)
    assert rel_err(w64, w_o) < TOL and rel_err(s64, s_o) < TOL
    assert rel_err(fr64, oracle_port.wav2px(w_o, s_o, p)) < TOL
    assert rel_err(fr64, f) < TOL
    # split precision against the FP64 path, scale by scale: one map (double-
    # float contractions on the FP64 tables), then a host batch of three maps
    # (f, -f, f/2), whose contractions the timing report shows on the tensor
    # cores
    import ctypes as C

    from s2let_gb300.capi import ptr

    rep = (C.c_double * 36)()
    s = gpu.sizes(p)
    fb = np.ascontiguousarray(np.stack([f, -f, 0.5 * f]))
    scale = np.array([1.0, -1.0, 0.5])[:, None]
    wb = np.zeros((3, s["n_wav"]), np.complex128)
    sb = np.zeros((3, s["n_scal"]), np.complex128)
    rb = np.zeros_like(fb)
    wb64 = np.ascontiguousarray(w64[None, :] * scale)
    sb64 = np.ascontiguousarray(s64[None, :] * scale)
    assert lib.s2let_gpu_set_precision(1) == 0
    try:
        wmx, smx = gpu.px2wav(f, p)
        frmx = gpu.wav2px(w64, s64, p)
        lib.s2let_gpu_timing_enable(1)
        assert lib.s2let_gpu_analysis_px2wav_host_batch(ptr(wb), ptr(sb), ptr(fb), 3, C.byref(p)) == 0
        assert lib.s2let_gpu_synthesis_wav2px_host_batch(ptr(rb), ptr(wb64), ptr(sb64), 3, C.byref(p)) == 0
        lib.s2let_gpu_timing_report(rep, 9)
        lib.s2let_gpu_timing_enable(0)
    finally:
        lib.s2let_gpu_set_precision(0)
    assert lib.s2let_gpu_device_fault() == 0
    assert rep[4 * 4 + 0] > 0, "the split-precision tensor-core contraction did not run"
    for j, off, n in _scales(gpu, p):
        e = rel_err(wmx[off:off + n], w64[off:off + n])
        assert e < TOL_MIXED, f"scale {j}: {e:.3e}"
        for b in range(3):
            e = rel_err(wb[b, off:off + n], wb64[b, off:off + n])
            assert e < TOL_MIXED, f"map {b} scale {j}: {e:.3e}"
    assert rel_err(smx, s64) < TOL_MIXED
    assert rel_err(frmx, fr64) < TOL_MIXED
    for b in range(3):
        assert rel_err(sb[b], sb64[b]) < TOL_MIXED, b
        assert rel_err(rb[b], fr64 * scale[b, 0]) < TOL_MIXED, b
    _release(gpu)
