"""The allocation-free PME entry point (moil_nb_pme_noalloc) against the handle path and the oracle.

Some callers cannot allocate device memory (their device memory belongs to another
runtime's pool, or they cannot take the synchronisation an allocation may cause), so
the library offers the PME reciprocal sum with all scratch in a static device array.
This file runs last so that, if it fails, every other GPU test has already run.

The comparison system is an ionic lattice whose ions are all farther apart than the
real-space cutoff: the handle path then has no real-space pairs and no exclusions, so
its full gradient is exactly the reciprocal-space gradient the new entry point returns.
"""
import ctypes

import numpy as np
import pytest

from conftest import energy_scale, rel_rms
from moil_fnrfd_gb300 import nb as NB
from moil_fnrfd_gb300 import systems as S

pytestmark = pytest.mark.gpu


def sparse_ion_lattice(seed=5):
    """4x4x4 alternating ions, 12 Å apart (+-0.5 Å jitter) in a 48 Å box; cutoff 10 Å."""
    rng = np.random.Generator(np.random.PCG64(seed))
    m, a = 4, 12.0
    L = m * a
    g = (np.arange(m) + 0.5) * a - L / 2
    X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
    I, J, K = np.meshgrid(np.arange(m), np.arange(m), np.arange(m), indexing="ij")
    pos = np.stack([X.ravel(), Y.ravel(), Z.ravel()], 1) + rng.uniform(-0.5, 0.5, size=(m ** 3, 3))
    q = ((-1.0) ** (I + J + K)).ravel() * 0.8
    n = len(q)
    return S.MoilSystem(name="ions", coor=pos, ptchg=q, epsgm6=np.zeros(n), epsgm12=np.zeros(n),
                        exc1=np.zeros(n + 1, np.int32), exc2=np.zeros(0, np.int32), spec1=np.zeros(0, np.int32),
                        spec2=np.zeros(0, np.int32), p14=np.zeros((0, 3)),
                        poipt=np.arange(1, n + 1, dtype=np.int32), montype=np.full(n, S.MON_ION, np.int32),
                        box=(L, L, L), rvmx=10.0, relx=10.0, alpha=0.35, nfft=(48, 48, 48))


def noalloc_rc(torch, s, natom=None, grid=None):
    """Status of one call with the given (possibly invalid) sizes, and whether the gradient
    buffer was left untouched (still NaN)."""
    L = NB.load()
    fn = L.moil_nb_pme_noalloc
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                   ctypes.POINTER(ctypes.c_int), ctypes.c_double, ctypes.c_double, ctypes.c_void_p,
                   ctypes.POINTER(ctypes.c_double), ctypes.c_void_p]
    n = s.npt if natom is None else natom
    dc = torch.zeros((max(n, s.npt), 3), dtype=torch.float64, device="cuda")
    dc[:s.npt] = torch.tensor(s.coor, dtype=torch.float64)
    dq = torch.zeros(max(n, s.npt), dtype=torch.float64, device="cuda")
    dd = torch.full_like(dc, float("nan"))
    torch.cuda.synchronize()
    box = (ctypes.c_double * 3)(*s.box)
    g = (ctypes.c_int * 3)(*(grid or s.nfft))
    e = ctypes.c_double(float("nan"))
    rc = fn(dc.data_ptr(), dq.data_ptr(), n, box, g, s.alpha, s.eps, dd.data_ptr(), ctypes.byref(e), None)
    torch.cuda.synchronize()
    return rc, bool(torch.isnan(dd).all())


def noalloc(torch, s):
    L = NB.load()
    fn = L.moil_nb_pme_noalloc
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                   ctypes.POINTER(ctypes.c_int), ctypes.c_double, ctypes.c_double, ctypes.c_void_p,
                   ctypes.POINTER(ctypes.c_double), ctypes.c_void_p]
    dc = torch.tensor(s.coor, dtype=torch.float64, device="cuda")
    dq = torch.tensor(s.ptchg, dtype=torch.float64, device="cuda")
    dd = torch.full_like(dc, float("nan"))
    torch.cuda.synchronize()
    box = (ctypes.c_double * 3)(*s.box)
    grid = (ctypes.c_int * 3)(*s.nfft)
    e = ctypes.c_double(float("nan"))
    rc = fn(dc.data_ptr(), dq.data_ptr(), s.npt, box, grid, s.alpha, s.eps, dd.data_ptr(), ctypes.byref(e), None)
    assert rc == 0, L.moil_nb_strerror(rc)
    return dd.cpu().numpy(), e.value


def test_noalloc_pme_matches_handle_path_twice():
    torch = pytest.importorskip("torch")
    s = sparse_ion_lattice()
    h = NB.Nonbonded(s)
    dpot_ref, e_ref = h.eforce(s.coor)
    h.close()
    # no real-space pair and no exclusion: the handle's gradient is purely reciprocal
    assert e_ref["e_el"] == 0.0 and e_ref["e_lsym"] == 0.0 and e_ref["e_corr"] == 0.0
    for _ in range(2):
        dpot, e = noalloc(torch, s)
        assert np.isfinite(dpot).all()
        assert rel_rms(dpot, dpot_ref) <= 1e-5
        assert abs(e - e_ref["e_ew_receip"]) <= 1e-6 * energy_scale(e_ref)


def test_noalloc_pme_energy_matches_handle_path_for_water():
    torch = pytest.importorskip("torch")
    s = S.config0()
    h = NB.Nonbonded(s)
    _, e_ref = h.eforce(s.coor)
    h.close()
    for _ in range(2):
        _, e = noalloc(torch, s)
        assert abs(e - e_ref["e_ew_receip"]) <= 1e-6 * energy_scale(e_ref)


def test_noalloc_pme_matches_the_oracle_twice():
    """The 216-water box against the oracle's reciprocal sum alone (ewald_receip with an exact
    FFT), on two calls in a row: relative RMS gradient error <= 1e-5 and the energy within 1e-6
    relative (the mixed path's tolerances)."""
    torch = pytest.importorskip("torch")
    from oracle import oracle as O
    s = S.config0()
    ref, e_ref = O.pme(s, s.alpha)
    for _ in range(2):
        dpot, e = noalloc(torch, s)
        assert rel_rms(dpot, ref) <= 1e-5
        assert abs(e - e_ref) <= 1e-6 * abs(e_ref)


def test_noalloc_rejects_sizes_beyond_its_array():
    """Sizes the fixed array cannot hold are refused before anything runs: the gradient
    buffer is left as it was."""
    torch = pytest.importorskip("torch")
    s = sparse_ion_lattice()
    ERR_ARG, ERR_GRID = 1, 4          # MOIL_NB_ERR_ARG, MOIL_NB_ERR_GRID (include/moil_nb.h)
    for kw, want in ((dict(natom=65537), ERR_ARG), (dict(grid=(65, 48, 48)), ERR_GRID),
                     (dict(grid=(48, 7, 48)), ERR_GRID), (dict(grid=(48, 48, 3)), ERR_GRID)):
        rc, untouched = noalloc_rc(torch, s, **kw)
        assert rc == want, (kw, rc)
        assert untouched, kw
