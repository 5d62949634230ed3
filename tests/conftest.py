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
