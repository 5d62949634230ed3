"""GPU parity for the rest of the drop-in surface: plain MW SHT, axisymmetric
transforms, harmonic tiling multiplies (lm2lmn family), manual tilings, hard
thresholding and the batched device-pointer entry points.  FP64 tolerance 1e-12
(normwise relative max error)."""
import ctypes as C

import numpy as np
import pytest

from conftest import random_flm, rel_err
from s2let_gb300.capi import make_parameters, ptr

TOL = 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("L", [1, 2, 5, 16, 31, 64])
@pytest.mark.parametrize("spin", [0, 1, 2, -3])
def test_mw_sht(gpu, oracle_port, L, spin):
    if abs(spin) >= L:
        pytest.skip("|spin| >= L")
    rng = np.random.default_rng(L * 7 + spin)
    flm = random_flm(rng, L, spin)
    f_o = oracle_port.alm2map(flm, L, spin)
    assert rel_err(gpu.alm2map(flm, L, spin), f_o) < TOL
    assert rel_err(gpu.map2alm(f_o, L, spin), oracle_port.map2alm(f_o, L, spin)) < TOL
    if spin == 0:
        flr = random_flm(rng, L, real=True)
        fr = oracle_port.alm2map(flr, L, real=True)
        assert rel_err(gpu.alm2map(flr, L, real=True), fr) < TOL
        assert rel_err(gpu.map2alm(fr, L, real=True), oracle_port.map2alm(fr, L, real=True)) < TOL


AXI = [(16, 2.0, 0), (16, 2.0, 2), (32, 3.0, 1), (9, 2.0, 1)]


@pytest.mark.gpu
@pytest.mark.parametrize("L,B,J_min", AXI)
@pytest.mark.parametrize("multires", [False, True])
@pytest.mark.parametrize("real", [False, True])
def test_axisym_mw(gpu, oracle_port, L, B, J_min, multires, real):
    p = make_parameters(L, B, J_min, 1, 0, 0)
    rng = np.random.default_rng(5)
    npx = L * (2 * L - 1)
    f = rng.normal(size=npx) if real else rng.normal(size=npx) + 1j * rng.normal(size=npx)
    wo, so = oracle_port.axisym("analysis", [f], p, multires, real)
    wg, sg = gpu.axisym("analysis", [f], p, multires, real)
    assert rel_err(wg, wo) < TOL and rel_err(sg, so) < TOL
    for op in ("synthesis", "analysis_adjoint"):
        assert rel_err(gpu.axisym(op, [wo, so], p, multires, real),
                       oracle_port.axisym(op, [wo, so], p, multires, real)) < TOL, op
    ao = oracle_port.axisym("synthesis_adjoint", [f], p, multires, real)
    ag = gpu.axisym("synthesis_adjoint", [f], p, multires, real)
    assert rel_err(ag[0], ao[0]) < TOL and rel_err(ag[1], ao[1]) < TOL


LMN = [(16, 4, 2.0, 2, 0, 0), (16, 4, 2.0, 2, 2, 1), (12, 5, 2.0, 0, 0, 0), (17, 3, 2.5, 1, 1, 0)]


@pytest.mark.gpu
@pytest.mark.parametrize("case", LMN)
@pytest.mark.parametrize("real", [False, True])
def test_lm2lmn_family(gpu, oracle_port, case, real):
    L, N, B, J_min, spin, up = case
    if real and spin:
        pytest.skip("real signals are spin 0")
    p = make_parameters(L, B, J_min, N, spin, up)
    rng = np.random.default_rng(6)
    flm = random_flm(rng, L, spin, real=real)
    for adj in (False, True):
        lo, so = oracle_port.lm2lmn(flm, p, real=real, adjoint_of_synthesis=adj)
        lg, sg = gpu.lm2lmn(flm, p, real=real, adjoint_of_synthesis=adj)
        assert rel_err(lg, lo) < TOL and rel_err(sg, so) < TOL
        for adj2 in (False, True):
            assert rel_err(gpu.lmn2lm(lo, so, p, real=real, adjoint_of_analysis=adj2),
                           oracle_port.lmn2lm(lo, so, p, real=real, adjoint_of_analysis=adj2)) < TOL


def _manual(lib, name, L, N, spin, flm, wav, scal, psi, phi, sbl, wbl):
    J = len(wbl) - 1
    wb = np.ascontiguousarray(wbl, dtype=np.int32)
    getattr(lib, name)(ptr(wav) if "lm2wav" in name else ptr(flm),
                       ptr(scal) if "lm2wav" in name else ptr(wav),
                       ptr(flm) if "lm2wav" in name else ptr(scal),
                       ptr(phi), ptr(psi), sbl, ptr(wb), J, L, spin, N)


@pytest.mark.gpu
def test_manual_tiling(gpu, oracle_port):
    L, N, spin = 16, 3, 0
    p = make_parameters(L, 2.0, 0, N, spin, 0)
    psi, phi = oracle_port.tiling(p)
    wbl = [min(int(np.ceil(2.0 ** (j + 1))), L) for j in range(0, 5)]
    sbl = 1
    rng = np.random.default_rng(7)
    flm = random_flm(rng, L, spin)
    tot = sum((2 * (min(N, b) + (min(N, b) + N) % 2) - 1) * b * (2 * b - 1) for b in wbl)
    res = {}
    for name, lib in (("o", oracle_port.lib), ("g", gpu.lib)):
        wav = np.zeros(tot, np.complex128)
        scal = np.zeros(sbl * (2 * sbl - 1), np.complex128)
        _manual(lib, "s2let_analysis_lm2wav_manual", L, N, spin, flm, wav, scal, psi, phi, sbl, wbl)
        back = np.zeros(L * L, np.complex128) + 0.5  # these two accumulate into flm
        _manual(lib, "s2let_synthesis_wav2lm_manual", L, N, spin, back, wav, scal, psi, phi, sbl, wbl)
        adj = np.zeros(L * L, np.complex128) + 0.25
        _manual(lib, "s2let_analysis_adjoint_wav2lm_manual", L, N, spin, adj, wav, scal, psi, phi, sbl, wbl)
        wav2 = np.zeros(tot, np.complex128)
        scal2 = np.zeros_like(scal)
        _manual(lib, "s2let_synthesis_adjoint_lm2wav_manual", L, N, spin, flm, wav2, scal2, psi, phi, sbl, wbl)
        res[name] = (wav, scal, back, adj, wav2, scal2)
    for a, b in zip(res["g"], res["o"]):
        assert rel_err(a, b) < TOL


@pytest.mark.gpu
@pytest.mark.parametrize("multires", [False, True])
def test_hard_threshold(gpu, oracle_port, multires):
    L = 16
    p = make_parameters(L, 2.0, 1, 1, 0, 0)
    nw, _ = oracle_port.axisym_sizes(p, multires)
    J = oracle_port.lib.s2let_j_max(C.byref(p))
    rng = np.random.default_rng(8)
    g0 = rng.normal(scale=3.0, size=nw)
    thr = np.linspace(0.5, 2.5, J - p.J_min + 1)
    out = {}
    for name, lib in (("o", oracle_port.lib), ("g", gpu.lib)):
        g = g0.copy()
        fn = "s2let_transform_axisym_wav_hardthreshold_multires_real" if multires else \
            "s2let_transform_axisym_wav_hardthreshold_real"
        getattr(lib, fn)(ptr(g), ptr(thr), C.byref(p))
        out[name] = g
    np.testing.assert_array_equal(out["g"], out["o"])


@pytest.mark.gpu
def test_batch_api_matches_single(gpu):
    torch = pytest.importorskip("torch")
    L, nb = 16, 5
    p = make_parameters(L, 2.0, 2, 4, 0, 0)
    s = gpu.sizes(p)
    rng = np.random.default_rng(9)
    f = rng.normal(size=(nb, s["n_px"]))
    df = torch.tensor(f, device="cuda")
    dw = torch.zeros((nb, s["n_wav"]), dtype=torch.float64, device="cuda")
    ds = torch.zeros((nb, s["n_scal"]), dtype=torch.float64, device="cuda")
    rc = gpu.lib.s2let_gpu_analysis_px2wav_real_batch(
        C.c_void_p(dw.data_ptr()), C.c_void_p(ds.data_ptr()), C.c_void_p(df.data_ptr()), nb, C.byref(p),
        C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0
    torch.cuda.synchronize()
    for b in range(nb):
        w1, s1 = gpu.px2wav(f[b], p, real=True)
        assert rel_err(dw[b].cpu().numpy(), w1) < 1e-14
        assert rel_err(ds[b].cpu().numpy(), s1) < 1e-14
    fr = torch.zeros_like(df)
    rc = gpu.lib.s2let_gpu_synthesis_wav2px_real_batch(
        C.c_void_p(fr.data_ptr()), C.c_void_p(dw.data_ptr()), C.c_void_p(ds.data_ptr()), nb, C.byref(p),
        C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0
    torch.cuda.synchronize()
    for b in range(nb):
        assert rel_err(fr[b].cpu().numpy(), gpu.wav2px(dw[b].cpu().numpy(), ds[b].cpu().numpy(), p, real=True)) < 1e-14
