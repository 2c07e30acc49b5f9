"""GPU parity tests: the CUDA path through the C ABI against the oracle.

Tolerances (stated per the path's contract):
  mixed precision  relative RMS gradient error <= 1e-5; total energy |dE_total| / |E_total|
                   <= 1e-6; gradients bit-identical run to run.  An additional check holds
                   each term within 1e-6 of the energy-term scale (sum of |term|), and every
                   term's error relative to its own size is printed
  plain FP64       relative RMS gradient error <= 1e-8; |dE_total| / |E_total| <= 1e-9; each
                   term within 1e-10 of the term scale
The oracle reference is MOIL's predicate at the evaluation coordinates ("parity" mode:
MOIL's list path with zero buffers and exact erfc).
"""
import ctypes
import math

import numpy as np
import pytest

from conftest import ENERGY_TERMS, energy_report, energy_scale, format_energy_report, rel_rms
from moil_fnrfd_gb300 import systems as S
from moil_fnrfd_gb300.nb import MOIL_NB_FP64, MOIL_NB_MIXED, MoilNbError, Nonbonded
from oracle import oracle as O

pytestmark = pytest.mark.gpu

TOL = {MOIL_NB_MIXED: dict(force=1e-5, total=1e-6, term=1e-6),
       MOIL_NB_FP64: dict(force=1e-8, total=1e-9, term=1e-10)}


def check(dpot, e, ref, eref, prec, label=""):
    scale = energy_scale(eref)
    f = rel_rms(dpot, ref)
    terms, total = energy_report(e, eref)
    print(f"{label}: rel RMS gradient error {f:.2e}; {format_energy_report(terms, total)}")
    assert f <= TOL[prec]["force"], f"{label} rel RMS gradient error {f:.3e}"
    assert total <= TOL[prec]["total"], f"{label} |dE_total|/|E_total| {total:.3e}"
    for k in ENERGY_TERMS:   # additional: every term against the energy-term scale
        assert abs(e[k] - eref[k]) <= TOL[prec]["term"] * scale, f"{label} {k}: {e[k]} vs {eref[k]}"


@pytest.fixture(scope="module")
def ref0(cfg0):
    return O.eforce(cfg0, mode="parity")


@pytest.fixture(scope="module")
def ref1(cfg1):
    return O.eforce(cfg1, mode="parity")


@pytest.mark.parametrize("prec", [MOIL_NB_MIXED, MOIL_NB_FP64])
def test_water216_parity(cfg0, ref0, prec):
    nb = Nonbonded(cfg0, precision=prec)
    dpot, e = nb.eforce(cfg0.coor)
    check(dpot, e, *ref0, prec, "216 waters")
    assert nb.pair_stats()["site_pairs"] == ref0[1]["site_pairs"]
    nb.close()


@pytest.mark.parametrize("prec", [MOIL_NB_MIXED, MOIL_NB_FP64])
def test_solute_parity(cfg1, ref1, prec):
    """Solute (Lorentz-Berthelot, exclusions, 1-4) + ions + water, 23,556 atoms."""
    nb = Nonbonded(cfg1, precision=prec)
    dpot, e = nb.eforce(cfg1.coor)
    check(dpot, e, *ref1, prec, "solute")
    water = np.arange(cfg1.npt) >= cfg1.npt - 3 * cfg1.nwaters
    assert rel_rms(dpot[water], ref1[0][water]) <= TOL[prec]["force"]
    nb.close()


def test_mixed_is_bit_identical_run_to_run(cfg1):
    nb = Nonbonded(cfg1)
    d1, e1 = nb.eforce(cfg1.coor)
    nb.nblist()
    d2, e2 = nb.eforce(cfg1.coor)
    nb2 = Nonbonded(cfg1)
    d3, e3 = nb2.eforce(cfg1.coor)
    assert np.array_equal(d1, d2) and np.array_equal(d1, d3)
    assert e1 == e2 == e3
    nb.close()
    nb2.close()


def test_graph_replay_matches_kernel_launches(cfg0):
    """Evaluations replayed from the captured CUDA graph equal kernel-by-kernel launches
    bit for bit, across list reuse, rebuilds and a change of the device buffers."""
    torch = pytest.importorskip("torch")
    g, k = Nonbonded(cfg0, skin=1.0), Nonbonded(cfg0, skin=1.0)
    k.set_graph(False)
    rng = np.random.default_rng(5)
    small = cfg0.coor + np.repeat(rng.uniform(-0.2, 0.2, size=(cfg0.nwaters, 3)), 3, axis=0)
    big = cfg0.coor.copy()
    big[:30] += 0.8
    for c in (cfg0.coor, small, small, big, cfg0.coor):
        dg, eg = g.eforce(c)
        dk, ek = k.eforce(c)
        assert np.array_equal(dg, dk) and eg == ek
    for _ in range(2):   # fresh device buffers each round: the graph is captured again
        xc = torch.from_numpy(np.ascontiguousarray(small)).cuda()
        pg, pk = torch.empty_like(xc), torch.empty_like(xc)
        g.eforce_device(xc.data_ptr(), pg.data_ptr())
        k.eforce_device(xc.data_ptr(), pk.data_ptr())
        torch.cuda.synchronize()
        assert torch.equal(pg, pk)
    g.close()
    k.close()


def test_pinned_host_buffers_match_copies(cfg0):
    """Pinned host buffers give the result of pageable ones bit for bit, call after call."""
    torch = pytest.importorskip("torch")
    nb = Nonbonded(cfg0)
    d_page, e_page = nb.eforce(cfg0.coor)
    hc = torch.from_numpy(np.ascontiguousarray(cfg0.coor)).pin_memory()
    hd = torch.zeros_like(hc).pin_memory()
    for _ in range(2):
        e_pin = nb.eforce_into(hc.numpy(), hd.numpy())
        assert np.array_equal(hd.numpy(), d_page)
        assert e_pin[0] == e_page
    nb.close()


def test_batch_matches_single_systems_and_oracle(cfg0):
    sizes = [1503, 2406, 3300]
    reps = [S.water_box(n // 3, (n // 3 / S.WATER_DENSITY) ** (1 / 3), 500 + k, name=f"r{k}")
            for k, n in enumerate(sizes)] + [cfg0]
    nb = Nonbonded(reps)
    dps, es = nb.eforce()
    for k, s in enumerate(reps):
        ref, eref = O.eforce(s, mode="parity")
        check(dps[k], es[k], ref, eref, MOIL_NB_MIXED, f"replica {k}")
        single = Nonbonded(s)
        d1, e1 = single.eforce(s.coor)
        assert np.array_equal(d1, dps[k]), f"replica {k} differs from its single-system run"
        single.close()
    nb.close()


def test_plain_fp64_batch_runs_replicas(cfg0):
    reps = [cfg0, S.water_box(600, (600 / S.WATER_DENSITY) ** (1 / 3), 77)]
    nb = Nonbonded(reps, precision=MOIL_NB_FP64)
    dps, es = nb.eforce()
    for k, s in enumerate(reps):
        ref, eref = O.eforce(s, mode="parity")
        check(dps[k], es[k], ref, eref, MOIL_NB_FP64, f"fp64 replica {k}")
    nb.close()


def test_moved_coordinates_reuse_and_rebuild(cfg0):
    """Small moves reuse the list (skin), large moves rebuild it; both stay exact."""
    nb = Nonbonded(cfg0, skin=1.0, timing=True)
    nb.eforce(cfg0.coor)
    rng = np.random.default_rng(11)
    # whole-molecule moves up to 0.2 Å per axis plus 0.02 Å internal jitter
    shift = np.repeat(rng.uniform(-0.2, 0.2, size=(cfg0.nwaters, 3)), 3, axis=0)
    small = cfg0.coor + shift + rng.uniform(-0.02, 0.02, size=cfg0.coor.shape)
    d, e = nb.eforce(small)
    assert nb.timing()["list_rebuilt"] == 0
    ref, eref = O.eforce(cfg0, mode="parity", coor=small)
    check(d, e, ref, eref, MOIL_NB_MIXED, "small move")
    big = cfg0.coor.copy()
    big[:30] += 0.8            # ten whole waters move 0.8 Å along every axis
    d, e = nb.eforce(big)
    assert nb.timing()["list_rebuilt"] == 1
    ref, eref = O.eforce(cfg0, mode="parity", coor=big)
    check(d, e, ref, eref, MOIL_NB_MIXED, "large move")
    nb.close()


def test_list_period_forces_rebuilds(cfg0):
    nb = Nonbonded(cfg0, list_period=3, timing=True)
    flags = []
    for _ in range(7):
        nb.eforce(cfg0.coor)
        flags.append(nb.timing()["list_rebuilt"])
    assert flags == [1, 0, 0, 1, 0, 0, 1]
    nb.close()


def test_lj_switch_extension_matches_oracle(cfg0):
    s = cfg0.copy()
    s.r_on = 8.0
    nb = Nonbonded(s, lj_switch=True)
    d, e = nb.eforce(s.coor)
    ref, eref = O.eforce(s, mode="parity", lj_switch=True)
    check(d, e, ref, eref, MOIL_NB_MIXED, "switch")
    nb.close()


def test_unsquezed_waters_give_the_same_result(cfg0):
    """A water moved by a box vector is the same periodic system (minimum image)."""
    c = cfg0.coor.copy()
    c[9:12, 0] += cfg0.box[0]
    nb = Nonbonded(cfg0)
    d0, e0 = nb.eforce(cfg0.coor)
    d1, e1 = nb.eforce(c)
    assert rel_rms(d1, d0) < 1e-6
    assert abs(e1["e_total"] - e0["e_total"]) < 1e-6 * energy_scale(e0)
    nb.close()


def test_pme_grid_sizes(cfg0):
    """Odd and mixed-radix grids (25 = 5*5, 27 = 3^3, 36, 45)."""
    for n in (25, 27, 36, 45):
        s = cfg0.copy()
        s.nfft = (n, n, n)
        ref, eref = O.eforce(s, mode="parity")
        nb = Nonbonded(s)
        d, e = nb.eforce(s.coor)
        check(d, e, ref, eref, MOIL_NB_MIXED, f"grid {n}")
        nb.close()


def test_error_statuses(cfg0):
    bad = cfg0.copy()
    bad.ptchg = bad.ptchg.copy()
    bad.ptchg[0] += 0.01
    with pytest.raises(MoilNbError) as ei:
        Nonbonded(bad)
    assert ei.value.status == 3
    g = cfg0.copy()
    g.nfft = (21, 20, 20)        # 21 = 3 * 7 is not 2/3/5-smooth
    with pytest.raises(MoilNbError) as ei:
        Nonbonded(g)
    assert ei.value.status == 4
    b = cfg0.copy()
    b.rvmx = b.relx = 9.5          # > L/2 = 9.31
    with pytest.raises(MoilNbError) as ei:
        Nonbonded(b)
    assert ei.value.status == 5
    nb = Nonbonded(cfg0)
    c = cfg0.coor.copy()
    c[5, 1] = np.nan
    with pytest.raises(MoilNbError) as ei:
        nb.eforce(c)
    assert ei.value.status == 7
    d, e = nb.eforce(cfg0.coor)         # the handle stays usable
    assert np.isfinite(d).all()
    nb.close()


def test_fortran_entry_points_accumulate(cfg0):
    from moil_fnrfd_gb300 import nb as NB
    L = NB.load()
    s = cfg0
    I = lambda v: ctypes.byref(ctypes.c_int(v))
    ip = lambda a: np.ascontiguousarray(a, np.int32).ctypes.data_as(ctypes.POINTER(ctypes.c_int))
    dp = lambda a: np.ascontiguousarray(a, np.float64).ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    keep = [np.ascontiguousarray(x) for x in (s.ptchg, s.epsgm6, s.epsgm12)]
    exc1, exc2 = np.ascontiguousarray(s.exc1, np.int32), np.ascontiguousarray(s.exc2, np.int32)
    poipt, mt = np.ascontiguousarray(s.poipt, np.int32), np.ascontiguousarray(s.montype, np.int32)
    z = np.zeros(1, np.int32)
    p11 = np.array([s.rvmx, s.relx, s.eps, *s.box, 0.0, s.alpha, 0.0, 1.0, 0.0])
    i8 = np.array([*s.nfft, 4, int(s.arith), int(s.hvdw0), 0, 0], np.int32)
    st = ctypes.c_int(-1)
    L.ewald_init_gpu_(I(s.npt), dp(keep[0]), dp(keep[1]), dp(keep[2]), ip(exc1), ip(exc2), I(0), ip(z), ip(z),
                      dp(np.zeros(3)), I(s.totmon), ip(poipt), ip(mt), dp(p11), ip(i8), ctypes.byref(st))
    assert st.value == 0
    coor = np.ascontiguousarray(s.coor)
    dpot = np.ones_like(coor)            # bonded terms already accumulated by the caller
    enb = np.zeros(11)
    L.eforce_nb_gpu_(I(s.npt), dp(coor), dpot.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                     enb.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), ctypes.byref(st))
    assert st.value == 0
    ref, eref = O.eforce(s, mode="parity")
    assert rel_rms(dpot - 1.0, ref) <= 1e-5
    assert abs(enb[9] - eref["e_total"]) <= 1e-6 * abs(eref["e_total"])


def test_alpha_from_dtol_matches_moil_route(cfg0):
    """MOIL takes 'ewald dtol', not alpha (pot/energy.f:226-235), and finds alpha by doubling and
    bisection (symm/ewald_init.f:298-335): through the C API and through ewald_init_gpu_ with
    alpha = 0, the GPU path's alpha equals the oracle's find_ewaldcof to 1e-14 and the
    evaluation passes the 216-water parity check at that alpha."""
    dtol = math.erfc(0.35 * 9.0) / 9.0
    a_ref = O.find_ewaldcof(cfg0.relx, dtol)
    assert abs(a_ref - 0.35) < 1e-12
    s = cfg0.copy()
    s.alpha = a_ref
    ref, eref = O.eforce(s, mode="parity")
    for prec in (MOIL_NB_MIXED, MOIL_NB_FP64):
        nb = Nonbonded(cfg0, precision=prec, dtol=dtol)
        assert abs(nb.alpha() - a_ref) <= 1e-14 * a_ref
        dpot, e = nb.eforce(cfg0.coor)
        check(dpot, e, ref, eref, prec, f"alpha from dtol ({'FP64' if prec else 'mixed'})")
        nb.close()
    # the Fortran entry points, alpha = 0 in params11
    from moil_fnrfd_gb300 import nb as NB
    L = NB.load()
    I = lambda v: ctypes.byref(ctypes.c_int(v))
    ip = lambda a: np.ascontiguousarray(a, np.int32).ctypes.data_as(ctypes.POINTER(ctypes.c_int))
    dp = lambda a: np.ascontiguousarray(a, np.float64).ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    keep = [np.ascontiguousarray(x) for x in (s.ptchg, s.epsgm6, s.epsgm12)]
    ik = [np.ascontiguousarray(x, np.int32) for x in (s.exc1, s.exc2, s.poipt, s.montype)]
    z = np.zeros(1, np.int32)
    p11 = np.array([s.rvmx, s.relx, s.eps, *s.box, dtol, 0.0, 0.0, 1.0, 0.0])
    i8 = np.array([*s.nfft, 4, int(s.arith), int(s.hvdw0), 0, 0], np.int32)
    p14 = np.zeros(3)
    st = ctypes.c_int(-1)
    L.ewald_init_gpu_(I(s.npt), dp(keep[0]), dp(keep[1]), dp(keep[2]), ip(ik[0]), ip(ik[1]), I(0), ip(z), ip(z),
                      dp(p14), I(s.totmon), ip(ik[2]), ip(ik[3]), dp(p11), ip(i8), ctypes.byref(st))
    assert st.value == 0
    coor = np.ascontiguousarray(s.coor)
    dpot = np.zeros_like(coor)
    enb = np.zeros(11)
    L.eforce_nb_gpu_(I(s.npt), dp(coor), dpot.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                     enb.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), ctypes.byref(st))
    assert st.value == 0
    # e_self = -alpha/sqrt(pi) kofdie/eps sum q^2 (FP64 on the host): alpha to 1e-14
    assert abs(enb[7] - eref["e_self"]) <= 1e-14 * abs(eref["e_self"])
    assert rel_rms(dpot, ref) <= 1e-5
    assert abs(enb[9] - eref["e_total"]) <= 1e-6 * abs(eref["e_total"])


def test_device_resident_evaluation(cfg0):
    torch = pytest.importorskip("torch")
    nb = Nonbonded(cfg0)
    dc = torch.tensor(cfg0.coor, dtype=torch.float64, device="cuda")
    dd = torch.empty_like(dc)
    torch.cuda.synchronize()
    e = nb.eforce_device(dc.data_ptr(), dd.data_ptr())[0]
    ref, eref = O.eforce(cfg0, mode="parity")
    check(dd.cpu().numpy(), e, ref, eref, MOIL_NB_MIXED, "device")
    nb.close()


def test_large_water_box_against_fp64_path():
    """96,000 atoms: mixed against the plain FP64 GPU path and the oracle."""
    s = S.config2()
    mixed = Nonbonded(s)
    dm, em = mixed.eforce(s.coor)
    mixed.close()
    plain = Nonbonded(s, precision=MOIL_NB_FP64)
    dp_, ep = plain.eforce(s.coor)
    plain.close()
    ref, eref = O.eforce(s, mode="mi")
    check(dp_, ep, ref, eref, MOIL_NB_FP64, "fp64 96k")
    check(dm, em, ref, eref, MOIL_NB_MIXED, "mixed 96k")


def test_dense_cluster_regrows_lists():
    """Waters packed into part of the box (2.4x the mean density there) overflow the pair-
    list rows sized from the mean density; the evaluation regrows them and stays exact."""
    s = S.water_box(3000, (3000 / S.WATER_DENSITY) ** (1 / 3), 91, name="cluster")
    xyz = s.coor.reshape(-1, 3, 3)
    o = xyz[:, 0, :]                  # the box is centred on the origin: pull molecules in
    s.coor = (xyz - 0.25 * o[:, None, :]).reshape(-1, 3)
    # precondition: the densest rows exceed the capacity sized from the mean density
    # (rows of 4/3 pi (rc + skin)^3 * mean density * 1.4 + 32 entries, rounded up to 32)
    o = s.coor.reshape(-1, 3, 3)[:, 0, :]
    L = np.array(s.box)
    rows = []
    for k in range(0, 3000, 500):
        d = o[k:k + 500, None, :] - o[None, :, :]
        d -= L * np.round(d / L)
        rows.append(((d * d).sum(-1) < 10.0 ** 2).sum(1) - 1)
    assert np.concatenate(rows).max() > 256
    nb = Nonbonded(s)
    d, e = nb.eforce(s.coor)
    ref, eref = O.eforce(s, mode="parity")
    check(d, e, ref, eref, MOIL_NB_MIXED, "dense cluster")
    nb.close()


def test_int32_rows_for_a_box_of_more_than_65535_waters():
    """66,000 waters in one replica: the pair-list rows hold int32 water indices (below 65,536
    waters per replica they hold uint16 offsets); against the oracle (its 128^3 grid is beyond
    the FP64 plane kernels' shared memory)."""
    n = 66000
    s = S.water_box(n, (n / S.WATER_DENSITY) ** (1 / 3), 17, name="w66k", rc=9.0, alpha=0.35)
    mixed = Nonbonded(s)
    dm, em = mixed.eforce(s.coor)
    mixed.close()
    ref, eref = O.eforce(s, mode="mi")
    check(dm, em, ref, eref, MOIL_NB_MIXED, "66k waters")
