"""Edge cases of the GPU path against the oracle: MOIL's geometric LJ rule with tiny-epsilon
hydrogens (the hvdw0 Coulomb-only pairs, pot/nbond.f:115-126), a system without waters, a box
of exactly twice the cutoff (the minimum-image limit), a single water (empty pair lists), and
a batch mixing all of them.  Tolerances as in test_gpu_parity.py."""
import numpy as np
import pytest

from conftest import ENERGY_TERMS, energy_scale, rel_rms
from moil_fnrfd_gb300 import systems as S
from moil_fnrfd_gb300.nb import MOIL_NB_FP64, MOIL_NB_MIXED, Nonbonded
from oracle import oracle as O

pytestmark = pytest.mark.gpu

TOL = {MOIL_NB_MIXED: dict(force=1e-5, energy=1e-6), MOIL_NB_FP64: dict(force=1e-8, energy=1e-10)}


def systems():
    return {
        "geometric_hydrogens": S.config1(seed=11, n_solute=60, n_ions=7, n_waters=300, box=24.0, arith=False,
                                         tiny_h=True),
        "no_water": S.config1(seed=12, n_solute=90, n_ions=7, n_waters=0, box=24.0),
        "box_twice_cutoff": S.water_box(300, 18.0, 5, name="l18", rc=9.0, alpha=0.35, nfft=(18, 18, 18)),
        "single_water": S.water_box(1, 20.0, 6, name="one", rc=9.0, alpha=0.35, nfft=(20, 20, 20)),
    }


@pytest.fixture(scope="module")
def cases():
    return {k: (s, O.eforce(s, mode="parity")) for k, s in systems().items()}


def check(dpot, e, ref, eref, prec, label, cancelling=False):
    scale = energy_scale(eref)
    if cancelling:
        # a lone molecule: its gradient is the small remainder of the reciprocal-space and
        # exclusion-correction terms, each of the energy scale per Å, which cancel; the
        # error is bounded against that scale instead of the remainder
        f = float(np.abs(dpot - ref).max()) / scale
    else:
        f = rel_rms(dpot, ref)
    assert f <= TOL[prec]["force"], f"{label} gradient error {f:.3e}"
    for k in ENERGY_TERMS:
        assert abs(e[k] - eref[k]) <= TOL[prec]["energy"] * scale, f"{label} {k}: {e[k]} vs {eref[k]}"


@pytest.mark.parametrize("name", ["geometric_hydrogens", "no_water", "box_twice_cutoff", "single_water"])
@pytest.mark.parametrize("prec", [MOIL_NB_MIXED, MOIL_NB_FP64])
def test_edge_case(cases, name, prec):
    s, (ref, eref) = cases[name]
    nb = Nonbonded(s, precision=prec)
    dpot, e = nb.eforce(s.coor)
    check(dpot, e, ref, eref, prec, name, cancelling=name == "single_water")
    nb.close()


def test_mixed_batch_of_edge_cases(cases):
    names = list(cases)
    sys_ = [cases[k][0] for k in names]
    nb = Nonbonded(sys_)
    dpots, es = nb.eforce()
    for k, name in enumerate(names):
        ref, eref = cases[name][1]
        check(dpots[k], es[k], ref, eref, MOIL_NB_MIXED, "batch " + name, cancelling=name == "single_water")
    nb.close()
