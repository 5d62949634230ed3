import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: longer-running case")


@pytest.fixture(scope="session")
def oracle_port():
    from oracle import oracle

    return oracle.port()


@pytest.fixture(scope="session")
def gpu():
    import s2let_gb300

    lib = s2let_gb300.load()
    return s2let_gb300.api()


def rel_err(a, b):
    """max |a - b| / max |b| (normwise relative max error)."""
    a = np.asarray(a)
    b = np.asarray(b)
    den = np.abs(b).max()
    if den == 0:
        return float(np.abs(a).max())
    return float(np.abs(a - b).max() / den)


def random_flm(rng, L, spin=0, real=False, power=None):
    """Seeded harmonic coefficients; real=True enforces f_{l,-m} = (-1)^m conj(f_lm)."""
    flm = np.zeros(L * L, np.complex128)
    for l in range(L):
        amp = 1.0 if power is None else power(l)
        if real:
            flm[l * l + l] = rng.normal() * amp
            for m in range(1, l + 1):
                v = (rng.normal() + 1j * rng.normal()) * amp / np.sqrt(2)
                flm[l * l + l + m] = v
                flm[l * l + l - m] = (-1) ** m * np.conj(v)
        elif l >= abs(spin):
            flm[l * l:(l + 1) * (l + 1)] = (rng.normal(size=2 * l + 1) + 1j * rng.normal(size=2 * l + 1)) * amp
    return flm


def power_law_flm(rng, L, spin=0, real=False):
    """The benchmark configurations' spectra, vectorised: complex Gaussian flm
    with variance C_l = (l+1)^-2 (spin 0) or l^-2 for l >= |spin| (zero below);
    real=True enforces f_{l,-m} = (-1)^m conj(f_lm) (f_l0 real); f_00 = 0."""
    l = np.repeat(np.arange(L), 2 * np.arange(L) + 1)
    m = np.concatenate([np.arange(-k, k + 1) for k in range(L)]) if L else np.zeros(0, int)
    amp = np.where(l >= abs(spin), 1.0 / np.maximum(l + (1 if spin == 0 else 0), 1), 0.0)
    flm = (rng.normal(size=L * L) + 1j * rng.normal(size=L * L)) * amp / np.sqrt(2)
    if real:
        i0 = l * l + l
        pos = m > 0
        flm[m == 0] = flm[m == 0].real * np.sqrt(2)
        flm[(i0 - m)[pos]] = (-1.0) ** m[pos] * np.conj(flm[pos])
    flm[0] = 0.0
    return flm


def params_of(g):
    """make_parameters from a golden fixture's params (a seventh entry, when
    present, is the sampling scheme; an eighth the original spin)."""
    from s2let_gb300.capi import make_parameters

    v = g["params"]
    ss = int(v[6]) if len(v) > 6 else 0
    osp = int(v[7]) if len(v) > 7 else 0
    return make_parameters(int(v[0]), float(v[2]), int(v[3]), int(v[1]), int(v[4]), int(v[5]),
                           sampling_scheme=ss, original_spin=osp)


_SSHT_NAMES = {
    # direction -> SSHT entry point of the oracle's restatement
    0: "ssht_core_mw_forward_sov_conv_sym",
    1: "ssht_core_mw_inverse_sov_sym",
    2: "ssht_adjoint_mw_forward_sov_sym",
    3: "ssht_adjoint_mw_inverse_sov_sym",
}


def oracle_sht(O, direction, x, L, spin=0, real=False, ss=0):
    """The oracle's SSHT restatement on MW (ss=0) or MWSS (ss=1) sampling;
    directions as s2let_gpu_sht (0 forward, 1 inverse, 2 adjoint of the
    forward, 3 adjoint of the inverse)."""
    import ctypes as C

    name = _SSHT_NAMES[direction] + ("_ss" if ss else "") + ("_real" if real else "")
    fn = getattr(O.lib, name)
    fn.restype = None
    npx = (L + 1) * 2 * L if ss else L * (2 * L - 1)
    fdt = np.float64 if real else np.complex128
    if direction in (0, 3):
        f = np.ascontiguousarray(x, dtype=fdt)
        flm = np.zeros(L * L, np.complex128)
    else:
        flm = np.ascontiguousarray(x, dtype=np.complex128)
        f = np.zeros(npx, fdt)
    first, second = (flm, f) if direction in (0, 3) else (f, flm)
    args = [C.c_void_p(first.ctypes.data), C.c_void_p(second.ctypes.data), C.c_int(L)]
    if not real:
        args.append(C.c_int(spin))
    fn(*args, C.c_int(0), C.c_int(0))
    return flm if direction in (0, 3) else f
