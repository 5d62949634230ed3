"""Generates tests/golden/*.npz from the reference's own S2LET C sources compiled
in place (oracle/_ref/libs2let_ref.so, see oracle/Makefile) over the project's
SSHT/SO3 restatement.  Inputs are seeded numpy draws stored with the outputs, so
the fixtures pin the oracle port (oracle/s2let_port.c) without the reference.

Run from the repository root, naming the reference checkout:
  S2LET_REFERENCE_DIR=<checkout> python tests/golden/make_golden.py [name-prefix ...]
(with prefixes, only the fixtures whose names start with one of them are written).
MWSS fixtures (mwss_*) store the sampling scheme as a seventh parameter;
spin-lowered fixtures (os_*, wavelets with original_spin != 0) store the
sampling scheme and the original spin as seventh and eighth parameters.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle  # noqa: E402
from s2let_gb300.capi import make_parameters  # noqa: E402

CASES = {
    # name: (L, N, B, J_min, spin, upsample)
    "dir_L16_N4_s0_multires": (16, 4, 2.0, 2, 0, 0),
    "dir_L16_N4_s0_fullres": (16, 4, 2.0, 2, 0, 1),
    "dir_L16_N4_s2_multires": (16, 4, 2.0, 2, 2, 0),
    "dir_L16_N4_s2_fullres": (16, 4, 2.0, 2, 2, 1),
    "dir_L17_N3_B2.5_s1": (17, 3, 2.5, 1, 1, 0),
    "dir_L12_N5_Jmin0": (12, 5, 2.0, 0, 0, 0),
    "dir_L24_N5_s2_Jmin3": (24, 5, 2.0, 3, 2, 0),
}
AXI = {"axi_L16_J0": (16, 2.0, 0), "axi_L32_B3_J1": (32, 3.0, 1)}
# McEwen-Wiaux symmetric sampling (theta_t = pi t / L, both poles, 2L phi samples)
MWSS = {
    "mwss_L16_N4_s0_multires": (16, 4, 2.0, 2, 0, 0),
    "mwss_L16_N3_s2_fullres": (16, 3, 2.0, 2, 2, 1),
    "mwss_L13_N5_s1_Jmin1": (13, 5, 2.0, 1, 1, 0),
}

# spin-lowered wavelets: the tiling carries the spin normalisation of
# original_spin (src/c/s2let_tiling.c:404-423); MW sampling
ORIG = {
    # name: (L, N, B, J_min, spin, upsample, original_spin)
    "os_L16_N4_s0_os2_multires": (16, 4, 2.0, 2, 0, 0, 2),
    "os_L16_N3_s1_osm3_fullres": (16, 3, 2.0, 1, 1, 1, -3),
}


def main(prefixes=()):
    oracle.build()
    if not oracle.ref_available():
        sys.exit("no in-place reference build: set S2LET_REFERENCE_DIR to the S2LET checkout")
    R = oracle.ref()
    rng = np.random.default_rng(20261203)
    rng_ss = np.random.default_rng(20261204)  # MWSS inputs: a stream of their own
    want = lambda name: not prefixes or any(name.startswith(x) for x in prefixes)
    rng_os = np.random.default_rng(20261205)  # spin-lowered inputs: a stream of their own
    todo = [(k, v + (0,), 0) for k, v in CASES.items()] + [(k, v + (0,), 1) for k, v in MWSS.items()] + \
        [(k, v, 0) for k, v in ORIG.items()]
    written = 0
    for name, (L, N, B, J_min, spin, up, osp), ss in todo:
        p = make_parameters(L, B, J_min, N, spin, up, sampling_scheme=ss, original_spin=osp)
        npx = (L + 1) * 2 * L if ss else L * (2 * L - 1)
        par = [L, N, B, J_min, spin, up] + ([ss] if ss or osp else []) + ([osp] if osp else [])
        out = {"params": np.array(par, dtype=np.float64)}
        rng_case = rng_os if osp else (rng_ss if ss else rng)
        f = rng_case.normal(size=npx) + 1j * rng_case.normal(size=npx)
        flm = rng_case.normal(size=L * L) + 1j * rng_case.normal(size=L * L)
        out["f"] = f
        out["flm"] = flm
        out["px2wav_wav"], out["px2wav_scal"] = R.px2wav(f, p)
        out["wav2px"] = R.wav2px(out["px2wav_wav"], out["px2wav_scal"], p)
        out["adj_wav2px"] = R.analysis_adjoint_wav2px(out["px2wav_wav"], out["px2wav_scal"], p)
        out["adj_px2wav_wav"], out["adj_px2wav_scal"] = R.synthesis_adjoint_px2wav(f, p)
        out["lm2wav_wav"], out["lm2wav_scal"] = R.lm2wav(flm, p)
        out["wav2lm"] = R.wav2lm(out["lm2wav_wav"], out["lm2wav_scal"], p)
        out["lm2lmn"], out["lm2lmn_scal"] = R.lm2lmn(flm, p)
        out["lmn2lm"] = R.lmn2lm(out["lm2lmn"], out["lm2lmn_scal"], p)
        psi, phi = R.tiling(p)
        out["psi"], out["phi"] = psi, phi
        if spin == 0:
            fr = rng_case.normal(size=npx)
            out["f_real"] = fr
            out["px2wav_real_wav"], out["px2wav_real_scal"] = R.px2wav(fr, p, real=True)
            out["wav2px_real"] = R.wav2px(out["px2wav_real_wav"], out["px2wav_real_scal"], p, real=True)
            out["adj_wav2px_real"] = R.analysis_adjoint_wav2px(out["px2wav_real_wav"], out["px2wav_real_scal"], p,
                                                               real=True)
        if want(name):
            np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
            written += 1
    for name, (L, B, J_min) in AXI.items():
        p = make_parameters(L, B, J_min, 1, 0, 0)
        npx = L * (2 * L - 1)
        f = rng.normal(size=npx)
        out = {"params": np.array([L, B, J_min], dtype=np.float64), "f": f}
        for mr in (0, 1):
            w, s = R.axisym("analysis", [f], p, bool(mr), True)
            out[f"ana_mr{mr}_wav"], out[f"ana_mr{mr}_scal"] = w, s
            out[f"syn_mr{mr}"] = R.axisym("synthesis", [w, s], p, bool(mr), True)
        if want(name):
            np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
            written += 1
    print("wrote", written, "fixtures")


if __name__ == "__main__":
    main(tuple(sys.argv[1:]))
