"""Split precision on recomputed Wigner tables: the recomputed-table
contractions run their recursion and multiply-adds in double-float arithmetic
on the FP32 pipe (k_rc_l2t_df, k_rc_t2l_df).  Every directional operator must
stay within 1e-11 normwise relative max error of the FP64 path on stored
tables (double-float rounding is about 2^-47 per operation; the split-
precision tolerance of the library is 1e-10), at band-limits where the
recomputed tables take every scale (>= 128) and at small ones, for real and
complex signals, multiresolution and full resolution, MW and MWSS."""
import numpy as np
import pytest

from conftest import rel_err
from s2let_gb300.capi import SAMPLING_MW_SS, make_parameters

TOL = 1e-11

CASES = [
    # L, N, spin, real, upsample, sampling
    (192, 4, 0, True, 0, 0),
    (160, 3, 2, False, 0, 0),
    (130, 5, 1, False, 1, 0),
    (128, 4, 0, True, 0, 1),
    (64, 3, 0, True, 1, 0),
]


def _run(gpu, prec, mode, fn):
    lib = gpu.lib
    assert lib.s2let_gpu_set_precision(prec) == 0
    assert lib.s2let_gpu_set_table_mode(mode) == 0
    try:
        return fn()
    finally:
        lib.s2let_gpu_set_precision(0)
        lib.s2let_gpu_set_table_mode(0)


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES, ids=lambda c: "L{}_N{}_s{}_{}_up{}_ss{}".format(
    c[0], c[1], c[2], "real" if c[3] else "cplx", c[4], c[5]))
def test_df_recomputed_matches_fp64_stored(gpu, case):
    L, N, spin, real, up, ss = case
    p = make_parameters(L, 2.0, 2, N, spin, up, sampling_scheme=SAMPLING_MW_SS if ss else 0)
    s = gpu.sizes(p)
    rng = np.random.default_rng(7 * L + N)
    f = rng.normal(size=s["n_px"]) if real else rng.normal(size=s["n_px"]) + 1j * rng.normal(size=s["n_px"])
    ops = {
        "px2wav": lambda: gpu.px2wav(f, p, real=real),
        "adj_px2wav": lambda: gpu.synthesis_adjoint_px2wav(f, p, real=real),
    }
    for name, fn in ops.items():
        (w, sc), (w0, sc0) = _run(gpu, 1, 2, fn), _run(gpu, 0, 1, fn)
        assert rel_err(w, w0) < TOL and rel_err(sc, sc0) < TOL, name
    (w0, sc0) = _run(gpu, 0, 1, ops["px2wav"])
    for name, fn in {"wav2px": lambda: gpu.wav2px(w0, sc0, p, real=real),
                     "adj_wav2px": lambda: gpu.analysis_adjoint_wav2px(w0, sc0, p, real=real)}.items():
        r, r0 = _run(gpu, 1, 2, fn), _run(gpu, 0, 1, fn)
        assert rel_err(r, r0) < TOL, name
    assert gpu.lib.s2let_gpu_last_error() == 0
