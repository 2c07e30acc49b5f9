"""Parameter derivatives of the nonbonded energy: dE/dq, dE/deps and dE/dsigma per atom.

MOIL computes none of these, so nothing pins them to the reference; the oracle's adjoint
(ora_adjoint_mi) is checked here against central finite differences of the oracle energy
(h = 1e-4 relative, the energy re-encoded and the 1-4 parameters rewritten for every
perturbed parameter), and the GPU adjoint is checked against the oracle's
(tests marked gpu).  LJ parameters are decoded from MOIL's epsgm encoding
(connect/fillpt.f:136-184): geometric epsgm12 = 2 sqrt(eps) sigma^6, epsgm6 = 2 sqrt(eps)
sigma^3; arithmetic epsgm12 = 2 sqrt(eps), epsgm6 = sigma.
"""
import numpy as np
import pytest

from moil_fnrfd_gb300 import systems as S
from oracle import oracle as O

H = 1e-4


ELEC = ("e_el", "e_lsym", "e_el14", "e_corr", "e_self", "e_ew_receip")
LJ = ("e_vdw", "e_vsym", "e_vdw14")


def energy(s, terms):
    """The energy terms that depend on the perturbed parameter (the others only add rounding
    to the difference quotient)."""
    e = O.eforce(s, mode="mi")[1]
    return sum(e[k] for k in terms)


decode = S.lj_decode
encode = S.with_lj


def rewrite_p14(t):
    if len(t.spec1):
        spec = list(zip(t.spec1 - 1, t.spec2 - 1))
        t.p14 = S.np_p14(spec, t.ptchg, t.epsgm6, t.epsgm12, t.arith, eps=t.eps, hvdw0=t.hvdw0)
    return t


def fd(make, h, terms):
    return (energy(make(+h), terms) - energy(make(-h), terms)) / (2.0 * h)


@pytest.fixture(scope="module")
def solute():
    return S.config1(seed=7, n_solute=60, n_ions=2, n_waters=300, box=24.0)


def test_charge_derivatives_match_fd(solute):
    s = solute
    dq, _, _ = O.adjoint(s)
    for i in (0, 17, 59, 60):                 # solute atoms and an ion
        h = H * abs(s.ptchg[i])

        def make(d, i=i):
            t = s.copy()
            t.ptchg = t.ptchg.copy()
            t.ptchg[i] += d
            return rewrite_p14(t)
        assert fd(make, h, ELEC) == pytest.approx(dq[i], rel=1e-6, abs=1e-6)


def test_water_charge_derivative_matches_fd(cfg0):
    """All water charges together (O by +h, H by -h/2: the waters stay identical, as MOIL's
    water kernel assumes)."""
    s = cfg0
    dq, _, _ = O.adjoint(s)
    o = np.zeros(s.npt, dtype=bool)
    o[0::3] = True
    h = H * abs(s.ptchg[0])

    def make(d):
        t = s.copy()
        t.ptchg = t.ptchg + np.where(o, d, -0.5 * d)
        return t
    want = dq[o].sum() - 0.5 * dq[~o].sum()
    assert fd(make, h, ELEC) == pytest.approx(want, rel=1e-6)


@pytest.mark.parametrize("which", ["eps", "sigma"])
def test_lj_derivatives_match_fd(solute, which):
    s = solute
    _, de, ds = O.adjoint(s)
    eps, sig = decode(s)
    for i in (3, 40, 60):
        base = eps[i] if which == "eps" else sig[i]
        # the compact solute's LJ energy (~2e3 kcal/mol) is large next to one atom's share, so
        # the steps are larger than for the charges, where the energy is exactly quadratic:
        # eps enters as sqrt (central-difference error h^2/8), sigma as sigma^12 and sigma^6
        h = (1e-2 if which == "eps" else 1e-3) * base

        def make(d, i=i):
            e, g = eps.copy(), sig.copy()
            if which == "eps":
                e[i] += d
            else:
                g[i] += d
            return encode(s, e, g)
        got = de[i] if which == "eps" else ds[i]
        assert fd(make, h, LJ) == pytest.approx(got, rel=1e-4, abs=1e-7)


def test_water_oxygen_type_derivatives_match_fd(cfg0):
    """The water O type (every oxygen at once) under the geometric encoding."""
    s = cfg0
    _, de, ds = O.adjoint(s)
    eps, sig = decode(s)
    o = np.zeros(s.npt, dtype=bool)
    o[0::3] = True
    for vec, base, got in ((0, eps, de), (1, sig, ds)):
        h = H * base[0]

        def make(d, vec=vec):
            e, g = eps.copy(), sig.copy()
            (e if vec == 0 else g)[o] += d
            return encode(s, e, g)
        assert fd(make, h, LJ) == pytest.approx(got[o].sum(), rel=1e-5)


def test_lj_scaling_identities(solute):
    """Every eps scaled by l scales the LJ energy by l, every sigma by l gives
    dE/dl = 12 E_r12 - 6 E_r6: sum_i eps_i dE/deps_i = E_LJ and sum_i sigma_i dE/dsigma_i =
    12 E_r12 - 6 E_r6, exactly (no finite differences)."""
    s = solute
    _, de, ds = O.adjoint(s)
    eps, sig = decode(s)
    e = O.eforce(s, mode="mi")[1]
    elj = sum(e[k] for k in LJ)
    assert np.dot(eps, de) == pytest.approx(elj, rel=1e-12)
    # 12 E_r12 - 6 E_r6 from two scalings of the repulsive and dispersive parts
    l = 1.0 + 1e-3
    up = encode(s, eps, sig * l)
    dn = encode(s, eps, sig / l)
    want = (energy(up, LJ) - energy(dn, LJ)) / (np.log(l) * 2.0)
    assert np.dot(sig, ds) == pytest.approx(want, rel=1e-4)


# ---- GPU adjoint (moil_nb_adjoint) against the oracle's ---------------------------------
# The mixed path evaluates pair terms in FP32 with fixed-point accumulation, so the per-atom
# derivatives carry FP32 pair rounding; 1e-5 relative RMS is the force tolerance of the path.
ADJ_TOL = 1e-5


@pytest.fixture(scope="module")
def neutral():
    """The small solute with all seven counterions (the GPU library refuses charged systems,
    as MOIL's Ewald setup does)."""
    return S.config1(seed=7, n_solute=60, n_ions=7, n_waters=300, box=24.0)


def _gpu_adjoint_close(got, want, tol=ADJ_TOL):
    from conftest import rel_rms
    for g, w, name in zip(got, want, ("dE/dq", "dE/deps", "dE/dsigma")):
        assert np.all(np.isfinite(g)), name
        assert rel_rms(g, w) < tol, (name, rel_rms(g, w))


@pytest.mark.gpu
def test_gpu_adjoint_water216(cfg0):
    from moil_fnrfd_gb300.nb import Nonbonded
    nb = Nonbonded(cfg0)
    _gpu_adjoint_close(nb.adjoint(cfg0.coor), O.adjoint(cfg0))


@pytest.mark.gpu
def test_gpu_adjoint_solute(neutral):
    from moil_fnrfd_gb300.nb import Nonbonded
    nb = Nonbonded(neutral)
    got = nb.adjoint(neutral.coor)
    _gpu_adjoint_close(got, O.adjoint(neutral))
    again = nb.adjoint(neutral.coor)
    for g, a in zip(got, again):
        assert np.array_equal(g, a)            # deterministic run to run


@pytest.mark.gpu
def test_gpu_adjoint_batch_matches_single(cfg0, neutral):
    from moil_fnrfd_gb300.nb import Nonbonded
    nb = Nonbonded([cfg0, neutral])
    got = nb.adjoint()
    for k, s in enumerate((cfg0, neutral)):
        _gpu_adjoint_close([g[k] for g in got], O.adjoint(s))


@pytest.mark.gpu
@pytest.mark.parametrize("which", ["water216", "solute"])
def test_gpu_adjoint_plain_fp64_path(cfg0, neutral, which):
    """The plain FP64 handle: FP64 pair arithmetic and the PME potential from the FP64 plane
    kernels match the oracle's adjoint to 1e-9 relative RMS."""
    from moil_fnrfd_gb300.nb import MOIL_NB_FP64, Nonbonded
    s = cfg0 if which == "water216" else neutral
    nb = Nonbonded(s, precision=MOIL_NB_FP64)
    _gpu_adjoint_close(nb.adjoint(s.coor), O.adjoint(s), tol=1e-9)
    nb.close()


@pytest.mark.gpu
def test_gpu_adjoint_perturbed_copies_batch(cfg1):
    """The parameter-sensitivity workload: 64 seeded +-1% perturbed copies of the 23,556-atom
    solute system (eps and sigma per LJ type, solute charges per atom) in one batch.  Two
    copies against the oracle's adjoint; every copy against the homogeneity identities of
    the same call's energies: E_elec is quadratic in the charges (sum q dE/dq = 2 E_elec)
    and E_LJ is of degree one in the eps (sum eps dE/deps = E_LJ)."""
    from conftest import energy_scale
    from moil_fnrfd_gb300.nb import Nonbonded
    copies = S.perturbed_copies(cfg1, 64)
    nb = Nonbonded(copies)
    dq, de, ds = nb.adjoint()
    es = nb.energies()
    for k in (0, 63):
        _gpu_adjoint_close([dq[k], de[k], ds[k]], O.adjoint(copies[k]))
    for k, s in enumerate(copies):
        e = es[k]
        scale = energy_scale(e)
        eps, _ = S.lj_decode(s)
        assert abs(np.dot(s.ptchg, dq[k]) - 2.0 * sum(e[t] for t in ELEC)) < 1e-5 * scale, k
        assert abs(np.dot(eps, de[k]) - sum(e[t] for t in LJ)) < 1e-5 * scale, k
        # per-type sums, the quantities a parameter fit consumes, are finite
        assert np.all(np.isfinite(ds[k])), k
