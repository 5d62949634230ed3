"""Ring DFTs fused with the gamma DFT (split-precision path).

Below band-limit 128 the split-precision path contracts in double-float on
the FP64 tables (no bf16 digits), so at these band-limits precision 1 and
precision 0 differ in double-float arithmetic only: the ring and gamma DFTs
(the fused thread-block-cluster launch, one CTA per n-component, against
separate FP64 launches) and the contractions.  Every directional operator
must agree to 1e-12 normwise relative max error.  The cases cover every
cluster size (2-8 n-components), real signals with and without the n = 0
component, complex signals of spin 0-2, full resolution and multiresolution,
and both samplings (MW, MWSS)."""
import numpy as np
import pytest

from conftest import random_flm, rel_err
from s2let_gb300.capi import make_parameters

TOL = 1e-12

CASES = [
    # L, N, spin, real, upsample, sampling  (n-components per ring in the comment)
    (48, 4, 0, True, 0, 0),   # n = 1, 3
    (48, 5, 0, True, 1, 0),   # n = 0, 2, 4 (Hermitian n = 0)
    (40, 7, 0, True, 0, 0),   # n = 0, 2, 4, 6
    (40, 6, 0, True, 0, 1),   # n = 1, 3, 5 on MWSS
    (48, 2, 1, False, 0, 0),  # n = -1, 1
    (48, 5, 2, False, 0, 0),  # n = -4 .. 4 step 2
    (33, 6, 0, False, 1, 0),  # 6 components
    (40, 7, 1, False, 0, 1),  # 7 components, MWSS
    (32, 8, 2, False, 0, 0),  # 8 components
]


def _both(gpu, fn):
    lib = gpu.lib
    assert lib.s2let_gpu_set_precision(0) == 0
    ref = fn()
    assert lib.s2let_gpu_set_precision(1) == 0
    try:
        got = fn()
    finally:
        lib.s2let_gpu_set_precision(0)
    assert lib.s2let_gpu_last_error() == 0
    return got, ref


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES, ids=lambda c: "L{}_N{}_s{}_{}_up{}_ss{}".format(
    c[0], c[1], c[2], "real" if c[3] else "cplx", c[4], c[5]))
def test_fused_ring_gamma_matches_fp64(gpu, case):
    L, N, spin, real, up, ss = case
    p = make_parameters(L, 2.0, 1, N, spin, up, sampling_scheme=ss)
    s = gpu.sizes(p)
    rng = np.random.default_rng(100 * L + N)
    if real:
        f = rng.normal(size=s["n_px"])
    else:
        f = rng.normal(size=s["n_px"]) + 1j * rng.normal(size=s["n_px"])
    (w, sc), (w0, sc0) = _both(gpu, lambda: gpu.px2wav(f, p, real=real))
    assert rel_err(w, w0) < TOL and rel_err(sc, sc0) < TOL
    r, r0 = _both(gpu, lambda: gpu.wav2px(w0, sc0, p, real=real))
    assert rel_err(r, r0) < TOL
    a, a0 = _both(gpu, lambda: gpu.analysis_adjoint_wav2px(w0, sc0, p, real=real))
    assert rel_err(a, a0) < TOL
    (bw, bs), (bw0, bs0) = _both(gpu, lambda: gpu.synthesis_adjoint_px2wav(f, p, real=real))
    assert rel_err(bw, bw0) < TOL and rel_err(bs, bs0) < TOL


@pytest.mark.gpu
def test_fused_ring_gamma_harmonic_entry_points(gpu):
    """lm2wav / wav2lm through the fused launches (complex spin 2, N = 3)."""
    L = 48
    p = make_parameters(L, 2.0, 1, 3, 2, 0)
    flm = random_flm(np.random.default_rng(9), L, 2)
    (w, sc), (w0, sc0) = _both(gpu, lambda: gpu.lm2wav(flm, p))
    assert rel_err(w, w0) < TOL and rel_err(sc, sc0) < TOL
    g, g0 = _both(gpu, lambda: gpu.wav2lm(w0, sc0, p))
    assert rel_err(g, g0) < TOL
