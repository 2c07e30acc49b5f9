"""ctypes front end of the oracle (CPU FP64 restatement of MOIL's nonbonded path).

TEST INFRASTRUCTURE ONLY.  The test suite, the smoke check and the
CPU-baseline leg of ``bench.py`` import this module as the checker; the
product library never does.

Modes (the names the tests and the benchmark use):

* ``"moil"``   -- MOIL's own list path: monomer/centroid prefilter
  (``pot/nbondm.f``), atom lists (``pot/nbond.f``), 13 image translations
  (``symm/syminit.f``, ``nbmsym.f``, ``nbsym.f``), erfc from the cubic-spline
  table (``symm/ewald_init.f``), list buffers ``rvbg = rvmx + 2``.
* ``"parity"`` -- the same list path with zero buffers (``rvbg = rvmx``,
  ``rebg = relx``), a lossless monomer prefilter and exact erfc: MOIL's
  predicate evaluated at the given coordinates.  The GPU path is checked
  against this.
* ``"mi"``     -- an independent minimum-image evaluator of the parity
  predicate (cross-checks the image machinery).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libmoil_oracle.so")
_lock = threading.Lock()
_lib = None

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


class OraInput(ctypes.Structure):
    _fields_ = [
        ("npt", ctypes.c_int), ("coor", _dp), ("ptchg", _dp), ("epsgm6", _dp), ("epsgm12", _dp),
        ("exc1", _ip), ("exc2", _ip), ("totspe", ctypes.c_int), ("spec1", _ip), ("spec2", _ip),
        ("p14", _dp), ("totmon", ctypes.c_int), ("poipt", _ip), ("montype", _ip),
        ("arith", ctypes.c_int), ("hvdw0", ctypes.c_int),
        ("a", ctypes.c_double), ("b", ctypes.c_double), ("c", ctypes.c_double),
        ("rvmx", ctypes.c_double), ("rvbg", ctypes.c_double), ("relx", ctypes.c_double),
        ("rebg", ctypes.c_double), ("cutm", ctypes.c_double), ("eps", ctypes.c_double),
        ("ewaldcof", ctypes.c_double), ("dtol", ctypes.c_double),
        ("nfft1", ctypes.c_int), ("nfft2", ctypes.c_int), ("nfft3", ctypes.c_int), ("order", ctypes.c_int),
        ("erfc_mode", ctypes.c_int), ("lj_switch", ctypes.c_int), ("r_on", ctypes.c_double),
        ("squeeze", ctypes.c_int), ("do_pme", ctypes.c_int),
    ]


class OraOutput(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in (
        "e_vdw", "e_el", "e_vsym", "e_lsym", "e_el14", "e_vdw14", "e_corr", "e_self",
        "e_ew_receip", "e_total", "e_dir", "ewaldcof", "fpme")] + [
        ("site_pairs", ctypes.c_longlong), ("lj_pairs", ctypes.c_longlong),
        ("excl_pairs", ctypes.c_longlong), ("n14", ctypes.c_longlong),
        ("list_sizes", ctypes.c_longlong * 8), ("virvdw", ctypes.c_double * 5)]


ENERGY_KEYS = ("e_vdw", "e_el", "e_vsym", "e_lsym", "e_el14", "e_vdw14", "e_corr", "e_self",
               "e_ew_receip", "e_total", "e_dir")


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (gcc, no GPU)."""
    with _lock:
        src = os.path.join(_HERE, "moil_oracle.c")
        if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
            subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        L.ora_eforce.argtypes = [ctypes.POINTER(OraInput), _dp, ctypes.POINTER(OraOutput)]
        L.ora_eforce_mi.argtypes = [ctypes.POINTER(OraInput), _dp, ctypes.POINTER(OraOutput)]
        L.ora_eforce_batch.argtypes = [ctypes.c_int, ctypes.POINTER(OraInput), ctypes.POINTER(_dp),
                                       ctypes.POINTER(OraOutput), ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                       ctypes.c_int]
        L.ora_find_ewaldcof.restype = ctypes.c_double
        L.ora_find_ewaldcof.argtypes = [ctypes.c_double, ctypes.c_double]
        L.ora_erfc_table.argtypes = [ctypes.c_double, ctypes.c_double, _dp, ctypes.c_int]
        L.ora_erfc_table_eval.restype = ctypes.c_double
        L.ora_erfc_table_eval.argtypes = [_dp, ctypes.c_double, ctypes.c_double, _dp]
        L.ora_bsp_moduli.argtypes = [ctypes.c_int, ctypes.c_int, _dp]
        L.ora_fft.argtypes = [_dp, _dp, ctypes.c_int, ctypes.c_int]
        L.ora_pme.argtypes = [ctypes.POINTER(OraInput), ctypes.c_double, _dp, _dp, _dp]
        L.ora_adjoint_mi.argtypes = [ctypes.POINTER(OraInput), _dp, _dp, _dp]
        L.ora_pressure_mi.argtypes = [ctypes.POINTER(OraInput), _ip, _dp, _dp, ctypes.POINTER(OraOutput), _dp]
        _lib = L
    return _lib


def _p(a, t=_dp):
    return a.ctypes.data_as(t)


class _Keep:
    """Holds contiguous copies alive while the C side reads them."""

    def __init__(self):
        self.refs = []

    def d(self, a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        self.refs.append(a)
        return _p(a)

    def i(self, a):
        a = np.ascontiguousarray(a, dtype=np.int32)
        self.refs.append(a)
        return _p(a, _ip)


def make_input(s, mode: str = "parity", keep: _Keep | None = None, coor=None, pme: bool = True,
               lj_switch: bool = False, squeeze: bool = False, alpha: float | None = None,
               erfc: str | None = None) -> OraInput:
    keep = keep if keep is not None else _Keep()
    inp = OraInput()
    c = s.coor if coor is None else coor
    inp.npt = s.npt
    inp.coor = keep.d(c)
    inp.ptchg = keep.d(s.ptchg)
    inp.epsgm6 = keep.d(s.epsgm6)
    inp.epsgm12 = keep.d(s.epsgm12)
    inp.exc1 = keep.i(s.exc1)
    inp.exc2 = keep.i(s.exc2 if len(s.exc2) else np.zeros(1, np.int32))
    inp.totspe = len(s.spec1)
    inp.spec1 = keep.i(s.spec1 if len(s.spec1) else np.zeros(1, np.int32))
    inp.spec2 = keep.i(s.spec2 if len(s.spec2) else np.zeros(1, np.int32))
    inp.p14 = keep.d(s.p14 if len(s.p14) else np.zeros(3))
    inp.totmon = s.totmon
    inp.poipt = keep.i(s.poipt)
    inp.montype = keep.i(s.montype)
    inp.arith = int(s.arith)
    inp.hvdw0 = int(s.hvdw0)
    inp.a, inp.b, inp.c = (float(x) for x in s.box)
    inp.rvmx, inp.relx = float(s.rvmx), float(s.relx)
    if mode == "moil":
        inp.rvbg, inp.rebg, inp.cutm = -1.0, -1.0, -1.0
        inp.erfc_mode = 0
    else:
        inp.rvbg, inp.rebg = float(s.rvmx), float(s.relx)
        inp.cutm = max(s.rvmx, s.relx) + 6.0        # lossless centroid prefilter
        inp.erfc_mode = 1
    if erfc is not None:
        inp.erfc_mode = 0 if erfc == "table" else 1
    inp.eps = float(s.eps)
    inp.ewaldcof = float(s.alpha if alpha is None else alpha)
    inp.dtol = 0.0
    inp.nfft1, inp.nfft2, inp.nfft3 = (int(x) for x in s.nfft)
    inp.order = int(s.order)
    inp.lj_switch = int(lj_switch)
    inp.r_on = float(s.r_on)
    inp.squeeze = int(squeeze)
    inp.do_pme = int(pme)
    inp._keep = keep
    return inp


def output_dict(out: OraOutput) -> dict:
    d = {k: float(getattr(out, k)) for k in ENERGY_KEYS}
    d["ewaldcof"] = out.ewaldcof
    d["fpme"] = out.fpme
    d["site_pairs"] = int(out.site_pairs)
    d["lj_pairs"] = int(out.lj_pairs)
    d["excl_pairs"] = int(out.excl_pairs)
    d["n14"] = int(out.n14)
    d["list_sizes"] = [int(x) for x in out.list_sizes]
    d["virvdw"] = [float(x) for x in out.virvdw]
    return d


def eforce(s, mode: str = "parity", **kw):
    """Nonbonded energies and dpot (= dE/dx, kcal/mol/Å) of one system."""
    keep = _Keep()
    inp = make_input(s, mode=mode, keep=keep, **kw)
    dpot = np.zeros((s.npt, 3), dtype=np.float64)
    out = OraOutput()
    fn = lib().ora_eforce_mi if mode == "mi" else lib().ora_eforce
    rc = fn(ctypes.byref(inp), _p(dpot), ctypes.byref(out))
    if rc != 0:
        raise RuntimeError(f"oracle failed ({rc})")
    return dpot, output_dict(out)


def pme(s, alpha: float, mode: str = "parity", **kw):
    """PME reciprocal energy and gradient alone (moil_oracle.c ora_pme, ewald_receip's
    do_pmesh_kspace with the exact FFT): (dpot, e_recip)."""
    keep = _Keep()
    inp = make_input(s, mode=mode, keep=keep, **kw)
    dpot = np.zeros((s.npt, 3), dtype=np.float64)
    e, f = ctypes.c_double(0.0), ctypes.c_double(0.0)
    if lib().ora_pme(ctypes.byref(inp), float(alpha), _p(dpot), ctypes.byref(e), ctypes.byref(f)) != 0:
        raise RuntimeError("oracle pme failed")
    return dpot, e.value


def adjoint(s, mode: str = "parity", **kw):
    """Parameter derivatives of the energy (moil_oracle.c ora_adjoint_mi): per atom dE/dq,
    dE/deps and dE/dsigma, the LJ parameters decoded from the epsgm encoding."""
    keep = _Keep()
    inp = make_input(s, mode=mode, keep=keep, **kw)
    dq, de, ds = (np.zeros(s.npt, dtype=np.float64) for _ in range(3))
    if lib().ora_adjoint_mi(ctypes.byref(inp), _p(dq), _p(de), _p(ds)) != 0:
        raise RuntimeError("oracle adjoint failed")
    return dq, de, ds


PRESS_KEYS = ("virXX", "virYY", "virZZ", "V_PIdirXX", "V_PIdirYY", "V_PIdirZZ", "V_PIrecXX", "V_PIrecYY",
              "V_PIrecZZ", "V_PIrelXX", "V_PIrelYY", "V_PIrelZZ")


def pressure(s, mol, mass, mode: str = "parity", **kw):
    """MOIL's pressure analysis terms (moil_oracle.c ora_pressure_mi) at the system's
    coordinates: returns (dpot, energies, press) with press the 12 values of PRESS_KEYS.
    mol: molecule index of every atom (0-based), mass: atom masses."""
    keep = _Keep()
    inp = make_input(s, mode=mode, keep=keep, **kw)
    dpot = np.zeros((s.npt, 3), dtype=np.float64)
    press = np.zeros(12, dtype=np.float64)
    out = OraOutput()
    rc = lib().ora_pressure_mi(ctypes.byref(inp), keep.i(mol), keep.d(mass), _p(dpot), ctypes.byref(out),
                               _p(press))
    if rc != 0:
        raise RuntimeError(f"oracle pressure failed ({rc})")
    return dpot, output_dict(out), press


def eforce_batch(systems, mode: str = "parity", nthreads: int = 0, nevals: int = 1, list_period: int = 1, **kw):
    """Independent systems on nthreads host threads (0: OpenMP default); each system is
    evaluated nevals times with its lists rebuilt every list_period evaluations."""
    keep = _Keep()
    n = len(systems)
    ins = (OraInput * n)()
    outs = (OraOutput * n)()
    dp = (_dp * n)()
    res = []
    for k, s in enumerate(systems):
        ins[k] = make_input(s, mode=mode, keep=keep, **kw)
        d = np.zeros((s.npt, 3), dtype=np.float64)
        res.append(d)
        dp[k] = _p(d)
    rc = lib().ora_eforce_batch(n, ins, dp, outs, 1 if mode == "mi" else 0, int(nthreads), int(nevals),
                                int(list_period))
    if rc != 0:
        raise RuntimeError("oracle batch failed")
    return res, [output_dict(outs[k]) for k in range(n)]


def find_ewaldcof(cutoff: float, dtol: float) -> float:
    return lib().ora_find_ewaldcof(cutoff, dtol)


def erfc_table(alpha: float, cutoff: float) -> np.ndarray:
    cap = int(alpha * 5000 * cutoff * 1.5) + 16
    tab = np.zeros(4 * cap, dtype=np.float64)
    n = lib().ora_erfc_table(alpha, cutoff, _p(tab), cap)
    if n <= 0:
        raise RuntimeError("table")
    return tab[:4 * n].reshape(n, 4)


def erfc_table_eval(tab: np.ndarray, x: float):
    t = np.ascontiguousarray(tab.ravel())
    d = ctypes.c_double()
    v = lib().ora_erfc_table_eval(_p(t), 5000.0, x, ctypes.byref(d))
    return v, d.value


def bsp_moduli(n: int, order: int = 4) -> np.ndarray:
    m = np.zeros(n, dtype=np.float64)
    lib().ora_bsp_moduli(n, order, _p(m))
    return m


def fft(x: np.ndarray, sign: int = -1) -> np.ndarray:
    re = np.ascontiguousarray(x.real, dtype=np.float64).copy()
    im = np.ascontiguousarray(x.imag, dtype=np.float64).copy()
    lib().ora_fft(_p(re), _p(im), len(re), sign)
    return re + 1j * im
