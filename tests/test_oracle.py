"""CPU tests of the oracle (the FP64 restatement of MOIL's nonbonded path).

MOIL ships no test vectors, so the oracle is pinned by physics known-answer
tests (NaCl Madelung constant, a direct Ewald sum), by central finite
differences of its own energy in the style of MOIL's test_drv
(pot/test_drv.f:357-375), by agreement of the MOIL list path (13 image
translations) with an independent minimum-image evaluator, and by the
committed golden vectors in tests/golden/.
"""
import math
import os

import numpy as np
import pytest

from conftest import ENERGY_TERMS, energy_scale, rel_rms
from moil_fnrfd_gb300 import systems as S
from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
KOF = S.KOFDIE


def ion_system(pos, q, box, rc, alpha, n):
    npt = len(q)
    return S.MoilSystem(name="ions", coor=np.asarray(pos, float), ptchg=np.asarray(q, float),
                        epsgm6=np.zeros(npt), epsgm12=np.zeros(npt), exc1=np.zeros(npt + 1, np.int32),
                        exc2=np.zeros(0, np.int32), spec1=np.zeros(0, np.int32), spec2=np.zeros(0, np.int32),
                        p14=np.zeros((0, 3)), poipt=np.arange(1, npt + 1, dtype=np.int32),
                        montype=np.full(npt, S.MON_ION, np.int32), box=(box, box, box), rvmx=rc, relx=rc,
                        alpha=alpha, nfft=(n, n, n))


def nacl_crystal(m=8, r0=2.82):
    L = m * r0
    g = (np.arange(m) + 0.5) * r0 - L / 2
    X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
    I, J, K = np.meshgrid(np.arange(m), np.arange(m), np.arange(m), indexing="ij")
    pos = np.stack([X.ravel(), Y.ravel(), Z.ravel()], 1)
    q = ((-1.0) ** (I + J + K)).ravel()
    return pos, q, L


# published rock-salt Madelung constant (nearest-neighbour convention)
MADELUNG_NACL = 1.74756459463318219


def test_madelung_nacl():
    pos, q, L = nacl_crystal()
    s = ion_system(pos, q, L, 10.0, 0.5, 96)
    dpot, e = O.eforce(s, mode="parity")
    expected = -(len(q) / 2) * MADELUNG_NACL * KOF / 2.82
    assert abs(e["e_total"] - expected) / abs(expected) < 1e-10
    assert np.abs(dpot).max() < 1e-9     # every ion sits at a centre of symmetry


def direct_ewald(pos, q, L, alpha, rc, kmax=14):
    """Plain Ewald sum: real space over 27 images inside rc, reciprocal over |k| <= kmax (kcal/mol)."""
    n = len(q)
    e_real = 0.0
    grad = np.zeros((n, 3))
    for sx in (-1, 0, 1):
        for sy in (-1, 0, 1):
            for sz in (-1, 0, 1):
                sh = np.array([sx, sy, sz]) * L
                d = pos[:, None, :] - pos[None, :, :] + sh
                r = np.sqrt((d ** 2).sum(-1))
                if sx == sy == sz == 0:
                    np.fill_diagonal(r, np.inf)
                r = np.where(r < rc, r, np.inf)
                qq = q[:, None] * q[None, :]
                from scipy.special import erfc
                e_real += 0.5 * (qq * erfc(alpha * r) / r).sum()
                dedr = -qq * (erfc(alpha * r) / r ** 2 + 2 * alpha / math.sqrt(math.pi) * np.exp(-(alpha * r) ** 2) / r)
                grad += ((dedr / r)[:, :, None] * d).sum(1)
    e_real *= KOF
    grad *= KOF
    ks = np.arange(-kmax, kmax + 1)
    KX, KY, KZ = np.meshgrid(ks, ks, ks, indexing="ij")
    kv = np.stack([KX.ravel(), KY.ravel(), KZ.ravel()], 1).astype(float)
    kv = kv[(kv ** 2).sum(1) > 0]
    m = kv / L
    m2 = (m ** 2).sum(1)
    phase = 2 * np.pi * pos @ m.T
    S_re = (q[:, None] * np.cos(phase)).sum(0)
    S_im = (q[:, None] * np.sin(phase)).sum(0)
    w = np.exp(-np.pi ** 2 * m2 / alpha ** 2) / m2
    V = L ** 3
    e_rec = KOF / (2 * np.pi * V) * (w * (S_re ** 2 + S_im ** 2)).sum()
    # gradient of the reciprocal sum
    g_rec = KOF / (np.pi * V) * (q[:, None] * (w[None, :] * (-np.sin(phase) * S_re + np.cos(phase) * S_im)
                                                * 2 * np.pi))[:, :, None] * m[None, :, :]
    grad += g_rec.sum(1)
    e_self = -alpha / math.sqrt(math.pi) * KOF * (q ** 2).sum()
    return e_real + e_rec + e_self, e_rec, grad


def test_pme_against_direct_ewald():
    rng = np.random.Generator(np.random.PCG64(7))
    L = 20.0
    n = 24
    pos = rng.uniform(-L / 2, L / 2, size=(n, 3))
    q = rng.normal(0, 0.5, size=n)
    q -= q.mean()
    # keep atoms apart so the real-space sum is well conditioned
    s = ion_system(pos, q, L, 10.0, 0.35, 64)
    dpot, e = O.eforce(s, mode="mi")
    e_ref, e_rec_ref, g_ref = direct_ewald(pos, q, L, 0.35, 10.0)
    # PME discretisation (64^3 grid, order 4) against the exact reciprocal sum
    assert abs(e["e_ew_receip"] - e_rec_ref) / abs(e_rec_ref) < 1e-5
    assert abs(e["e_total"] - e_ref) < 1e-5 * energy_scale(e)
    assert rel_rms(dpot, g_ref) < 1e-4


def test_erfc_table_matches_libm():
    alpha, rc = 0.35, 9.0
    tab = O.erfc_table(alpha, rc)
    xs = np.linspace(0.0, alpha * rc * 1.45, 2001)
    err = max(abs(O.erfc_table_eval(tab, x)[0] - math.erfc(x)) for x in xs)
    derr = max(abs(O.erfc_table_eval(tab, x)[1] - 2 / math.sqrt(math.pi) * math.exp(-x * x)) for x in xs)
    assert err < 1e-13 and derr < 1e-10


@pytest.mark.parametrize("alpha,rc", [(0.35, 9.0), (0.32, 10.0)])
def test_find_ewaldcof_inverts_dtol(alpha, rc):
    dtol = math.erfc(alpha * rc) / rc
    assert abs(O.find_ewaldcof(rc, dtol) - alpha) < 1e-12


@pytest.mark.parametrize("n", [7, 20, 25, 27, 36, 45, 64, 100])
def test_fft_matches_numpy(n):
    rng = np.random.default_rng(n)
    x = rng.normal(size=n) + 1j * rng.normal(size=n)
    assert np.abs(O.fft(x, -1) - np.fft.fft(x)).max() < 1e-12 * n
    assert np.abs(O.fft(x, +1) - n * np.fft.ifft(x)).max() < 1e-12 * n


@pytest.mark.parametrize("n", [20, 25, 64])
def test_bspline_moduli(n):
    arr = np.zeros(n)
    arr[1:4] = [1 / 6, 2 / 3, 1 / 6]
    ref = np.abs(np.fft.fft(arr)) ** 2
    assert np.allclose(O.bsp_moduli(n), ref, rtol=1e-12, atol=1e-14)


@pytest.mark.parametrize("which", ["cfg0", "cfg1"])
def test_moil_lists_agree_with_minimum_image(which, request):
    s = request.getfixturevalue(which)
    d1, e1 = O.eforce(s, mode="parity")
    d2, e2 = O.eforce(s, mode="mi")
    assert e1["site_pairs"] == e2["site_pairs"]
    scale = energy_scale(e2)
    for k in ENERGY_TERMS:
        assert abs(e1[k] - e2[k]) <= 1e-12 * scale, k
    assert rel_rms(d1, d2) < 1e-12


def test_erfc_table_and_exact_agree(cfg0):
    """MOIL's spline-table erfc and the exact erfc give the same result (zero buffers)."""
    d1, e1 = O.eforce(cfg0, mode="parity", erfc="table")
    d2, e2 = O.eforce(cfg0, mode="parity", erfc="exact")
    scale = energy_scale(e2)
    assert abs(e1["e_total"] - e2["e_total"]) < 1e-12 * scale
    assert rel_rms(d1, d2) < 1e-11


def test_list_buffers_change_coulomb_semantics(cfg0):
    """With MOIL's default +2 Å buffers, list-1 Coulomb runs without a cutoff test
    (pot/cdie_ewald.f:313-491) and water list-1 pairs beyond the cutoff keep all nine
    site pairs: more pairs than the zero-buffer predicate."""
    _, e_moil = O.eforce(cfg0, mode="moil")
    _, e_par = O.eforce(cfg0, mode="parity")
    assert e_moil["site_pairs"] > e_par["site_pairs"]
    assert e_moil["e_vdw"] == pytest.approx(e_par["e_vdw"], abs=1e-9)


def test_finite_difference_gradient(cfg0):
    """Central differences of the total energy, as MOIL's test_drv does (pot/num_drv.f:71-90)."""
    dpot, e0 = O.eforce(cfg0, mode="parity")
    h = 1e-5
    rng = np.random.default_rng(3)
    for atom in rng.choice(cfg0.npt, size=6, replace=False):
        for k in range(3):
            cp = cfg0.coor.copy(); cp[atom, k] += h
            cm = cfg0.coor.copy(); cm[atom, k] -= h
            ep = O.eforce(cfg0, mode="parity", coor=cp)[1]["e_total"]
            em = O.eforce(cfg0, mode="parity", coor=cm)[1]["e_total"]
            num = (ep - em) / (2 * h)
            assert abs(num - dpot[atom, k]) < 2e-4 * max(1.0, abs(dpot[atom, k])), (atom, k, num, dpot[atom, k])


def test_lj_switch_extension(cfg0):
    s = cfg0.copy()
    s.r_on = 8.0
    d_sw, e_sw = O.eforce(s, mode="mi", lj_switch=True)
    d_no, e_no = O.eforce(s, mode="mi", lj_switch=False)
    assert e_sw["e_el"] == pytest.approx(e_no["e_el"], rel=1e-14)
    assert e_sw["e_vdw"] != e_no["e_vdw"]
    # the switched energy is continuous: FD of the switched LJ is consistent
    dpot, _ = O.eforce(s, mode="mi", lj_switch=True)
    h = 1e-5
    cp = s.coor.copy(); cp[0, 0] += h
    cm = s.coor.copy(); cm[0, 0] -= h
    num = (O.eforce(s, mode="mi", lj_switch=True, coor=cp)[1]["e_total"]
           - O.eforce(s, mode="mi", lj_switch=True, coor=cm)[1]["e_total"]) / (2 * h)
    assert abs(num - dpot[0, 0]) < 2e-4 * max(1.0, abs(dpot[0, 0]))


def test_squeeze_leaves_energy_unchanged(cfg0):
    """Translating whole waters by a box vector changes nothing once squeezed (symm/squeeze.f)."""
    c = cfg0.coor.copy()
    L = cfg0.box[0]
    for w in (3, 50, 101):
        c[3 * w:3 * w + 3, 0] += L
        c[3 * w + 3:3 * w + 6, 2] -= L
    d1, e1 = O.eforce(cfg0, mode="parity")
    d2, e2 = O.eforce(cfg0, mode="parity", coor=c, squeeze=True)
    assert abs(e1["e_total"] - e2["e_total"]) < 1e-9 * energy_scale(e1)
    assert rel_rms(d2, d1) < 1e-10


def test_golden_config0():
    """Regression pin: the oracle reproduces the committed golden vectors bit for bit."""
    g = np.load(os.path.join(GOLDEN, "config0_oracle.npz"))
    s = S.config0()
    assert np.array_equal(s.coor, g["coor"])
    for mode in ("parity", "moil"):
        d, e = O.eforce(s, mode=mode)
        np.testing.assert_allclose(d, g[f"dpot_{mode}"], rtol=0, atol=1e-11)
        for k in ENERGY_TERMS + ("e_total",):
            assert e[k] == pytest.approx(float(g[f"{mode}_{k}"]), rel=1e-12, abs=1e-9), (mode, k)
    mol, mass = S.molecules(s)
    press = O.pressure(s, mol, mass, mode="mi")[2]
    np.testing.assert_allclose(press, g["press_mi"], rtol=1e-12, atol=1e-9)
