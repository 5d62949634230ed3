"""Recomputed Wigner tables (s2let_gpu_set_table_mode(2)): the contraction
kernels regenerate d^l_{mn}(theta_t) from double-double checkpoints every 64
degrees and apply the forward quadrature W_eps as a separate operator, instead
of streaming stored D and Q tables.  They must give the stored-table results
(FP64 path, normwise relative max error <= 1e-12) and the reference's, and make
band-limits whose tables do not fit in device memory possible (L = 2048: the
stored D and Q tables of one map at N = 4 would take ~350 GB)."""
import glob
import os

import numpy as np
import pytest

from conftest import params_of, random_flm, rel_err
from s2let_gb300.capi import SAMPLING_MW_SS, make_parameters

TOL = 1e-12
GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))
GOLDEN = [p for p in GOLDEN if os.path.basename(p).startswith(("dir_", "mwss_", "os_"))]


class table_mode:
    def __init__(self, lib, mode):
        self.lib, self.mode = lib, mode

    def __enter__(self):
        self.old = self.lib.s2let_gpu_get_table_mode()
        assert self.lib.s2let_gpu_set_table_mode(self.mode) == 0

    def __exit__(self, *exc):
        self.lib.s2let_gpu_set_table_mode(self.old)


@pytest.mark.gpu
@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: os.path.basename(p)[:-4])
def test_recomputed_tables_match_reference_golden(gpu, path):
    g = np.load(path)
    p = params_of(g)
    with table_mode(gpu.lib, 2):
        w, s = gpu.px2wav(g["f"], p)
        assert rel_err(w, g["px2wav_wav"]) < TOL and rel_err(s, g["px2wav_scal"]) < TOL
        assert rel_err(gpu.wav2px(g["px2wav_wav"], g["px2wav_scal"], p), g["wav2px"]) < TOL
        assert rel_err(gpu.analysis_adjoint_wav2px(g["px2wav_wav"], g["px2wav_scal"], p), g["adj_wav2px"]) < TOL
        a, b = gpu.synthesis_adjoint_px2wav(g["f"], p)
        assert rel_err(a, g["adj_px2wav_wav"]) < TOL and rel_err(b, g["adj_px2wav_scal"]) < TOL
        w, s = gpu.lm2wav(g["flm"], p)
        assert rel_err(w, g["lm2wav_wav"]) < TOL and rel_err(s, g["lm2wav_scal"]) < TOL
        if "f_real" in g.files:
            w, s = gpu.px2wav(g["f_real"], p, real=True)
            assert rel_err(w, g["px2wav_real_wav"]) < TOL and rel_err(s, g["px2wav_real_scal"]) < TOL
            assert rel_err(gpu.wav2px(w, s, p, real=True), g["wav2px_real"]) < TOL
    assert gpu.lib.s2let_gpu_last_error() == 0


@pytest.mark.gpu
@pytest.mark.parametrize("L,N,spin,real,ss", [(1024, 4, 0, True, 0), (300, 3, 2, False, 0),
                                              (256, 5, 1, False, 1), (512, 4, 0, True, 1)])
def test_recomputed_equals_stored(gpu, L, N, spin, real, ss):
    """Both table modes on the same random (not band-limited) inputs, batch of 3,
    analysis, synthesis and both adjoints."""
    torch = pytest.importorskip("torch")
    from s2let_gb300 import torch_ops as T

    p = make_parameters(L, 2.0, 2, N, 0 if real else spin, 0, sampling_scheme=SAMPLING_MW_SS if ss else 0)
    n_px = T.sizes(p)["n_px"]
    gen = torch.Generator().manual_seed(L + N)
    if real:
        x = torch.rand((3, n_px), generator=gen, dtype=torch.float64) * 2 - 1
    else:
        x = torch.complex(torch.rand((3, n_px), generator=gen, dtype=torch.float64) - 0.5,
                          torch.rand((3, n_px), generator=gen, dtype=torch.float64) - 0.5)
    x = x.cuda().requires_grad_(True)
    out = {}
    for mode in (1, 2):
        with table_mode(gpu.lib, mode):
            w, s = T.px2wav(x, p, precision="fp64")
            r = T.wav2px(w, s, p, precision="fp64")
            # backward runs both adjoints (analysis and synthesis)
            loss = (w.abs() ** 2).sum() + (s.abs() ** 2).sum() + (r.abs() ** 2).sum()
            gx = torch.autograd.grad(loss, [x])[0]
            out[mode] = (w.detach(), s.detach(), r.detach(), gx)
    rel = lambda a, b: float((a - b).abs().max() / b.abs().max())
    for a, b in zip(out[2], out[1]):
        assert rel(a, b) < TOL
    gpu.lib.s2let_gpu_release_plans()


@pytest.mark.gpu
def test_L2048_recomputed_round_trip_and_oracle(gpu, oracle_port):
    """One real map at L = 2048, N = 4 (the band-limit of the d-tile
    recomputation case): tables chosen automatically (the top band-limit is
    recomputed), band-limited round trip, and px2wav against the CPU oracle."""
    L = 2048
    p = make_parameters(L, 2.0, 2, 4, 0, 0)
    rng = np.random.default_rng(2048)
    flm = random_flm(rng, L, real=True, power=lambda l: 1.0 / (l + 1))
    with table_mode(gpu.lib, 2):
        f = gpu.sht(1, flm, L, 0, True)
    with table_mode(gpu.lib, 0):
        w, s = gpu.px2wav(f, p, real=True)
        assert gpu.lib.s2let_gpu_last_error() == 0
        r = gpu.wav2px(w, s, p, real=True)
    assert rel_err(r, f) < TOL
    w0, s0 = oracle_port.px2wav(f, p, real=True)
    assert rel_err(w, w0) < TOL and rel_err(s, s0) < TOL
    gpu.lib.s2let_gpu_release_plans()


@pytest.mark.gpu
def test_L2048_adjoint_dot_product_and_gradient(gpu):
    """The differentiable path at L = 2048 (one map, recomputed tables): the
    backward of px2wav is its exact adjoint, <W x, y> = <x, W* y> to 1e-10, and
    a quadratic wavelet-space loss has the gradient W* W x."""
    torch = pytest.importorskip("torch")
    from s2let_gb300 import torch_ops as T

    L = 2048
    p = make_parameters(L, 2.0, 2, 4, 0, 0)
    s = T.sizes(p)
    gen = torch.Generator().manual_seed(7)
    x = (torch.rand((1, s["n_px"]), generator=gen, dtype=torch.float64) - 0.5).cuda().requires_grad_(True)
    yw = (torch.rand((1, s["n_wav"]), generator=gen, dtype=torch.float64) - 0.5).cuda()
    ys = (torch.rand((1, s["n_scal"]), generator=gen, dtype=torch.float64) - 0.5).cuda()
    with table_mode(gpu.lib, 0):
        w, sc = T.px2wav(x, p, precision="fp64")
        lhs = float(((w * yw).sum() + (sc * ys).sum()).detach())
        (g,) = torch.autograd.grad((w * yw).sum() + (sc * ys).sum(), [x])
        rhs = float((x.detach() * g).sum())
        assert abs(lhs - rhs) <= 1e-10 * abs(lhs)
        # gradient of 0.5 ||W x||^2 is W* W x: compare with a central difference along x
        loss = lambda z: 0.5 * sum(float((t ** 2).sum()) for t in T.px2wav(z, p, precision="fp64"))
        w, sc = T.px2wav(x, p, precision="fp64")
        (g2,) = torch.autograd.grad(0.5 * ((w ** 2).sum() + (sc ** 2).sum()), [x])
        d = x.detach()
        h = 1e-3
        fd = (loss(d + h * d) - loss(d - h * d)) / (2 * h)
        assert abs(fd - float((g2 * d).sum())) <= 1e-9 * abs(fd)
    assert gpu.lib.s2let_gpu_device_fault() == 0
    gpu.lib.s2let_gpu_release_plans()
