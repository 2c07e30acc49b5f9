import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


@pytest.fixture(scope="session")
def cfg0():
    from moil_fnrfd_gb300 import systems
    return systems.config0()


@pytest.fixture(scope="session")
def cfg1():
    from moil_fnrfd_gb300 import systems
    return systems.config1()


def rel_rms(a, b):
    """Relative RMS difference of per-atom vectors: |a - b|_2 / |b|_2."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.sqrt(((a - b) ** 2).sum() / (b ** 2).sum()))


ENERGY_TERMS = ("e_vdw", "e_el", "e_vsym", "e_lsym", "e_el14", "e_vdw14", "e_corr", "e_self", "e_ew_receip")


def energy_scale(e):
    """Sum of the magnitudes of the nonbonded energy terms."""
    return sum(abs(e[k]) for k in ENERGY_TERMS)


def energy_report(e, eref):
    """Energy errors against the oracle: each term's error relative to its own size (None
    for a term the oracle gives as exactly zero) and |dE_total| / |E_total|."""
    terms = {k: (abs(e[k] - eref[k]) / abs(eref[k]) if eref[k] != 0 else None) for k in ENERGY_TERMS}
    total = abs(e["e_total"] - eref["e_total"]) / abs(eref["e_total"])
    return terms, total


def format_energy_report(terms, total):
    parts = " ".join(f"{k[2:]} {v:.1e}" for k, v in terms.items() if v is not None)
    return f"|dE_total|/|E_total| {total:.2e}; per term (relative to the term): {parts}"
