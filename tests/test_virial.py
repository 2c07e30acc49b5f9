"""LJ virial terms of MOIL's PRESS build (virvdw1..virvdw5, COMMON/ENERGY.BLOCK:94-96).

virvdw = -sum df1 r^2 over the LJ pairs (df1 = (dE_LJ/dr)/r): water-water primary
(pot/watwat_ewald_press.f:146-152) and images (symm/symwat_ewald_press.f:161-168), other
pairs primary (pot/cdie_ewald_press.f:413-419) and images (symm/symcdie_ewald_press.f:164-167),
1-4 (pot/ener14_press.f:51-59).  The oracle's terms are pinned by two independent facts:
scaling every coordinate and the box by l scales every pair distance by l, so
d E_LJ / dl at l = 1 = sum r dE/dr = -sum virvdw (central differences, h = 1e-7); and for
r^-12 / r^-6 pairs sum r dE/dr = -(12 E_r12 - 6 E_r6) = -sum_i sigma_i dE/dsigma_i, the
oracle's parameter derivatives.  The GPU terms are checked against the oracle's.
"""
import numpy as np
import pytest

from moil_fnrfd_gb300 import systems as S
from oracle import oracle as O

LJ = ("e_vdw", "e_vsym", "e_vdw14")


@pytest.fixture(scope="module")
def neutral():
    return S.config1(seed=7, n_solute=60, n_ions=7, n_waters=300, box=24.0)


def scaled(s, l):
    t = s.copy()
    t.coor = s.coor * l
    t.box = tuple(b * l for b in s.box)
    return t


def test_list_path_and_minimum_image_agree(cfg0, neutral):
    for s in (cfg0, neutral):
        vm = np.array(O.eforce(s, mode="mi")[1]["virvdw"])
        for mode in ("parity", "moil"):
            v = np.array(O.eforce(s, mode=mode)[1]["virvdw"])
            assert np.allclose(v, vm, rtol=1e-10, atol=1e-9 * np.abs(vm).sum()), (mode, v, vm)


def test_virial_is_minus_the_scaling_derivative(cfg0, neutral):
    for s in (cfg0, neutral):
        v = O.eforce(s, mode="mi")[1]["virvdw"]
        h = 1e-7

        def elj(l):
            e = O.eforce(scaled(s, l), mode="mi")[1]
            return sum(e[k] for k in LJ)
        fd = (elj(1 + h) - elj(1 - h)) / (2 * h)
        assert -fd == pytest.approx(sum(v), rel=1e-6)


def test_virial_equals_the_sigma_identity(cfg0, neutral):
    for s in (cfg0, neutral):
        v = O.eforce(s, mode="mi")[1]["virvdw"]
        _, _, ds = O.adjoint(s)
        _, sig = S.lj_decode(s)
        assert sum(v) == pytest.approx(float(np.dot(sig, ds)), rel=1e-12)


def test_water_box_has_no_other_terms(cfg0):
    v = O.eforce(cfg0, mode="mi")[1]["virvdw"]
    assert v[0] > 0 and v[1] > 0 and v[2] == v[3] == v[4] == 0.0


# ---- GPU --------------------------------------------------------------------------
def _close(got, want, tol):
    got, want = np.asarray(got), np.asarray(want)
    scale = np.abs(want).sum()
    assert np.all(np.abs(got - want) <= tol * scale), (got, want)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_gpu_virial_matches_oracle(cfg0, neutral, precision):
    from moil_fnrfd_gb300.nb import MOIL_NB_FP64, MOIL_NB_MIXED, Nonbonded
    prec = MOIL_NB_FP64 if precision == "fp64" else MOIL_NB_MIXED
    tol = 1e-10 if precision == "fp64" else 1e-5
    for s in (cfg0, neutral):
        want = O.eforce(s, mode="mi")[1]["virvdw"]
        nb = Nonbonded(s, precision=prec)
        nb.set_virial(True)
        nb.eforce(s.coor)
        _close(nb.virial(), want, tol)
        nb.close()


@pytest.mark.gpu
def test_gpu_water_terms_off_by_default(cfg0):
    from moil_fnrfd_gb300.nb import Nonbonded
    nb = Nonbonded(cfg0)
    nb.eforce(cfg0.coor)
    v = nb.virial()
    assert v[0] == 0.0 and v[1] == 0.0
    nb.set_virial(True)
    d_on, e_on = nb.eforce(cfg0.coor)
    nb.set_virial(False)
    d_off, e_off = nb.eforce(cfg0.coor)
    # the virial accumulators change nothing else
    assert np.array_equal(d_on, d_off) and e_on == e_off


@pytest.mark.gpu
def test_gpu_virial_batch_and_sigma_identity(cfg0, neutral):
    """Per replica of a batch: the oracle's terms, and the GPU's own parameter derivatives
    give the same total."""
    from moil_fnrfd_gb300.nb import Nonbonded
    nb = Nonbonded([cfg0, neutral])
    nb.set_virial(True)
    nb.eforce()
    vir = nb.virial()
    _, _, ds = nb.adjoint()
    for k, s in enumerate((cfg0, neutral)):
        _close(vir[k], O.eforce(s, mode="mi")[1]["virvdw"], 1e-5)
        _, sig = S.lj_decode(s)
        assert sum(vir[k]) == pytest.approx(float(np.dot(sig, ds[k])), rel=1e-5)
