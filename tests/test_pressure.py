"""MOIL's pressure analysis terms (analysis/pressure.f with pressON): the molecular virial
tensor's diagonal split as MOIL prints it -- virXX..ZZ (LJ), V_PIdir (real-space Ewald
Coulomb), V_PIrec (reciprocal) and V_PIrel (PME force times the position relative to the
molecule's centre of mass); pressure.f:235-238 sums vir + dir + rec - rel.

MOIL ships no pressure output to compare with, so the oracle (ora_pressure_mi) is pinned by
its own energy: scaling the box along one axis by (1 + h) and moving every molecule rigidly
with it changes the LJ energy by -h virXX, the real-space Coulomb energy by -h V_PIdirXX
and the reciprocal energy by -h (V_PIrecXX - V_PIrelXX); the intramolecular terms
(exclusion corrections, 1-4, self) do not change.  Central differences with h = 1e-7 (no
pair crosses a cutoff: the pair counts at +h and -h are checked equal).  The GPU pass
(moil_nb_pressure, tests marked gpu) is checked against the oracle."""
import numpy as np
import pytest

from moil_fnrfd_gb300 import systems as S
from oracle import oracle as O

H = 1e-7
LJ = ("e_vdw", "e_vsym")
COUL = ("e_el", "e_lsym")
REC = ("e_ew_receip",)
INTRA = ("e_corr", "e_self", "e_el14", "e_vdw14")


def xrel_np(s, mol, mass):
    """Positions relative to the molecules' centres of mass, each atom placed at the minimum
    image of its displacement from the previous atom of its molecule (the oracle's rule)."""
    L = np.asarray(s.box, dtype=np.float64)
    d = np.zeros_like(s.coor)
    last = {}
    for n in range(s.npt):
        m = int(mol[n])
        if m in last:
            t = s.coor[n] - s.coor[last[m]]
            d[n] = d[last[m]] + t - L * np.round(t / L)
        last[m] = n
    M = np.bincount(mol, weights=mass)
    com = np.stack([np.bincount(mol, weights=mass * d[:, k]) for k in range(3)], 1) / M[:, None]
    return d - com[mol]


def scaled(s, R, ax, f):
    t = s.copy()
    t.coor = s.coor.copy()
    t.coor[:, ax] += (f - 1.0) * R[:, ax]
    box = list(s.box)
    box[ax] *= f
    t.box = tuple(box)
    return t


def solute_system():
    return S.config1(seed=7, n_solute=60, n_ions=7, n_waters=300, box=24.0)


def geometric_system():
    """MOIL's geometric LJ rule with tiny-epsilon hydrogens (the hvdw0 Coulomb-only pairs)."""
    return S.config1(seed=11, n_solute=60, n_ions=7, n_waters=300, box=24.0, arith=False, tiny_h=True)


@pytest.fixture(scope="module", params=["water216", "solute", "geometric_hydrogens"])
def case(request, cfg0):
    s = {"water216": lambda: cfg0, "solute": solute_system, "geometric_hydrogens": geometric_system}[request.param]()
    mol, mass = S.molecules(s)
    return request.param, s, mol, mass


def test_molecules_of_the_synthetic_systems():
    s = solute_system()
    mol, mass = S.molecules(s)
    # the 60-bead chain, 7 ions, 300 waters
    assert mol.max() + 1 == 1 + 7 + 300
    assert np.all(mol[:60] == 0) and len(set(mol[60:67])) == 7
    assert np.all(np.bincount(mol)[8:] == 3)


def test_oracle_pressure_matches_box_scaling(case):
    name, s, mol, mass = case
    _, e0, p = O.pressure(s, mol, mass, mode="mi")
    R = s.coor - xrel_np(s, mol, mass)
    scale = float(np.abs(p).sum())
    for ax in range(3):
        ep = O.eforce(scaled(s, R, ax, 1.0 + H), mode="mi")[1]
        em = O.eforce(scaled(s, R, ax, 1.0 - H), mode="mi")[1]
        assert ep["site_pairs"] == em["site_pairs"] and ep["lj_pairs"] == em["lj_pairs"], (name, ax)

        def d(keys):
            return (sum(ep[k] for k in keys) - sum(em[k] for k in keys)) / (2.0 * H)
        assert -d(LJ) == pytest.approx(p[ax], abs=1e-6 * scale), (name, ax)
        assert -d(COUL) == pytest.approx(p[3 + ax], abs=1e-6 * scale), (name, ax)
        assert -d(REC) == pytest.approx(p[6 + ax] - p[9 + ax], abs=1e-6 * scale), (name, ax)
        assert abs(d(INTRA)) < 1e-6 * scale, (name, ax)


def test_oracle_pressure_evaluation_is_ora_eforce_mi(case):
    """The pressure call returns the same gradient and energies as the plain evaluation."""
    _, s, mol, mass = case
    d0, e0 = O.eforce(s, mode="mi")
    d1, e1, _ = O.pressure(s, mol, mass, mode="mi")
    assert np.array_equal(d0, d1)
    for k in O.ENERGY_KEYS:
        assert e0[k] == e1[k]


def test_oracle_pressure_is_unchanged_by_wrapping(case):
    """Whole water molecules moved by box vectors, and the atoms of the other molecules each
    moved by its own box vector (molecules split across the boundary), give the same
    tensor: centres of mass are formed from molecules made whole."""
    _, s, mol, mass = case
    _, e0, p0 = O.pressure(s, mol, mass, mode="mi")
    t = s.copy()
    t.coor = s.coor.copy()
    rng = np.random.default_rng(5)
    L = np.asarray(s.box)
    shift = rng.integers(-1, 2, size=(s.npt, 3)) * L
    first = 0
    for k in range(s.totmon):
        last = int(s.poipt[k])
        if s.montype[k] == S.MON_WATER:
            shift[first:last] = shift[first]            # waters stay whole (MOIL's group rule)
        first = last
    t.coor += shift
    _, e1, p1 = O.pressure(t, mol, mass, mode="mi")
    assert e1["site_pairs"] == e0["site_pairs"]
    assert np.allclose(p1, p0, rtol=0, atol=1e-9 * np.abs(p0).sum())


# ---- GPU pass (moil_nb_pressure) against the oracle --------------------------------------
# FP32 pair and PME arithmetic with FP64 accumulation: 1e-5 of the tensor's scale.
GPU_TOL = 1e-5


def _close(got, want, label):
    scale = float(np.abs(want).sum())
    for k in range(12):
        assert abs(got[k] - want[k]) <= GPU_TOL * scale, (label, O.PRESS_KEYS[k], got[k], want[k])


@pytest.mark.gpu
def test_gpu_pressure_single(case):
    from moil_fnrfd_gb300.nb import Nonbonded
    name, s, mol, mass = case
    want = O.pressure(s, mol, mass, mode="mi")[2]
    nb = Nonbonded(s)
    nb.set_molecules(mol, mass)
    dpot, e, press = nb.pressure(s.coor)
    _close(press, want, name)
    again = nb.pressure(s.coor)[2]
    assert np.array_equal(press, again)         # deterministic run to run
    nb.close()


@pytest.mark.gpu
def test_gpu_pressure_batch_and_groups(cfg0):
    """A batch (waters, solute, a second water box), grouped and ungrouped: every replica
    matches the oracle and the two groupings agree bit for bit."""
    from moil_fnrfd_gb300.nb import Nonbonded
    reps = [cfg0, solute_system(), S.config3(1, seed=77)[0]]
    mols = [S.molecules(s) for s in reps]
    mol = np.concatenate([m for m, _ in mols])
    mass = np.concatenate([w for _, w in mols])
    out = []
    for groups in (1, 2):
        nb = Nonbonded(reps, groups=groups)
        nb.set_molecules(mol, mass)
        out.append(nb.pressure()[2])
        nb.close()
    for k, s in enumerate(reps):
        _close(out[0][k], O.pressure(s, *mols[k], mode="mi")[2], f"replica {k}")
        assert np.array_equal(out[0][k], out[1][k])


@pytest.mark.gpu
def test_gpu_pressure_plain_fp64_path(case):
    """The plain FP64 handle: the same pass in FP64 arithmetic matches the oracle to 1e-9 of
    the tensor's magnitude sum (the FP64 path's cutoffs are the FP32-rounded squares, so a pair
    within rounding of the cutoff could differ; none does in these systems)."""
    from moil_fnrfd_gb300.nb import MOIL_NB_FP64, Nonbonded
    name, s, mol, mass = case
    want = O.pressure(s, mol, mass, mode="mi")[2]
    nb = Nonbonded(s, precision=MOIL_NB_FP64)
    nb.set_molecules(mol, mass)
    press = nb.pressure(s.coor)[2]
    scale = float(np.abs(want).sum())
    for k in range(12):
        assert abs(press[k] - want[k]) <= 1e-9 * scale, (name, O.PRESS_KEYS[k], press[k], want[k])
    nb.close()


@pytest.mark.gpu
def test_gpu_pressure_needs_molecules(cfg0):
    from moil_fnrfd_gb300.nb import MoilNbError, Nonbonded
    nb = Nonbonded(cfg0)
    with pytest.raises(MoilNbError):
        nb.pressure(cfg0.coor)
    nb.close()
