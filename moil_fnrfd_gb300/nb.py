"""Python front end of the GPU library, mirroring MOIL's energy-routine interface.

MOIL's callers do ``call ewald_init()`` once, ``call squeeze(); call nbondm();
call syminit()`` when lists are due, then ``call eforce()`` which fills
``dpot`` and the ``/ENERGY/`` scalars (pot/energy.f:410-436,
dynamics/dyna.f:130-144).  :class:`Nonbonded` offers the same steps over the
C ABI of ``include/moil_nb.h``:

    nb = Nonbonded(system)            # ewald_init()
    nb.nblist()                        # nbondm() + syminit() at the next call
    dpot, e = nb.eforce(coor)          # nonbonded block of eforce()

There is no CPU fallback: if the CUDA library cannot be loaded or no GPU is
visible, every call raises.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

TUNE_DEVICE, TUNE_HOST = 0, 1
MOIL_NB_MIXED, MOIL_NB_FP64 = 0, 1
ENERGY_KEYS = ("e_vdw", "e_el", "e_vsym", "e_lsym", "e_el14", "e_vdw14", "e_corr", "e_self",
               "e_ew_receip", "e_total", "e_dir")

EXPORTED = ("moil_nb_create", "moil_nb_destroy", "moil_nb_strerror", "moil_nb_last_error", "moil_nb_init",
            "moil_nb_init_batch", "moil_nb_get_alpha", "moil_nb_eval", "moil_nb_eval_device",
            "moil_nb_eval_device_async", "moil_nb_eval_wait", "moil_nb_adjoint",
            "moil_nb_request_rebuild", "moil_nb_squeeze", "moil_nb_natoms", "moil_nb_stream",
            "moil_nb_set_timing", "moil_nb_get_timing", "moil_nb_pair_stats", "moil_nb_set_graph",
            "moil_nb_get_virial", "moil_nb_set_virial", "moil_nb_set_groups", "moil_nb_groups", "moil_nb_md_step",
            "moil_nb_set_shape", "moil_nb_get_shape", "moil_nb_set_tune_cache", "moil_nb_set_tune_mode",
            "moil_nb_autotune",
            "moil_nb_dcd_write", "moil_nb_set_molecules", "moil_nb_pressure", "ewald_init_gpu_", "nblist_gpu_", "eforce_nb_gpu_", "eforce_nb_press_gpu_")

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


class Params(ctypes.Structure):
    _fields_ = [("rvmx", ctypes.c_double), ("relx", ctypes.c_double), ("eps", ctypes.c_double),
                ("a", ctypes.c_double), ("b", ctypes.c_double), ("c", ctypes.c_double),
                ("dtol", ctypes.c_double), ("alpha", ctypes.c_double),
                ("nfft1", ctypes.c_int), ("nfft2", ctypes.c_int), ("nfft3", ctypes.c_int), ("order", ctypes.c_int),
                ("arith", ctypes.c_int), ("hvdw0", ctypes.c_int), ("lj_switch", ctypes.c_int),
                ("r_on", ctypes.c_double), ("skin", ctypes.c_double), ("list_period", ctypes.c_int),
                ("precision", ctypes.c_int)]


class Topology(ctypes.Structure):
    _fields_ = [("npt", ctypes.c_int), ("ptchg", _dp), ("epsgm6", _dp), ("epsgm12", _dp),
                ("exc1", _ip), ("exc2", _ip), ("totspe", ctypes.c_int), ("spec1", _ip), ("spec2", _ip),
                ("p14", _dp), ("totmon", ctypes.c_int), ("poipt", _ip), ("montype", _ip)]


class Energies(ctypes.Structure):
    _fields_ = [(k, ctypes.c_double) for k in ENERGY_KEYS]


class Replica(ctypes.Structure):
    _fields_ = [("params", ctypes.POINTER(Params)), ("topo", ctypes.POINTER(Topology))]


class Timing(ctypes.Structure):
    _fields_ = [(k, ctypes.c_float) for k in ("prepare_ms", "list_ms", "water_ms", "atom_ms", "excl_ms",
                                               "pme_spread_fft_ms", "pme_conv_ms", "pme_gather_ms",
                                               "finalize_ms", "total_ms")] + [
        ("list_rebuilt", ctypes.c_int), ("launches", ctypes.c_int)]


WATER_AUTO, WATER_FULL, WATER_HALF = 0, 1, 2
TILED_AUTO, TILED_OFF, TILED_ALL = 0, 1, 2
SHAPE_KEYS = ("water_kernel", "half_block", "tiled", "groups")


class Shape(ctypes.Structure):
    _fields_ = [(k, ctypes.c_int) for k in SHAPE_KEYS]


class TuneTrial(ctypes.Structure):
    _fields_ = [("shape", Shape), ("ms_per_eval", ctypes.c_double)]


class MoilNbError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"moil_nb status {status}: {msg}")
        self.status = status


_lib = None


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load ``libmoil_nb.so`` (building it with nvcc when missing or stale)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.build() if build_if_missing else _build.LIB
    if not os.path.exists(path):
        raise MoilNbError(-1, f"CUDA library not built: {path}")
    L = ctypes.CDLL(path)
    L.moil_nb_create.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int]
    L.moil_nb_destroy.argtypes = [ctypes.c_void_p]
    L.moil_nb_destroy.restype = None
    L.moil_nb_strerror.restype = ctypes.c_char_p
    L.moil_nb_strerror.argtypes = [ctypes.c_int]
    L.moil_nb_last_error.restype = ctypes.c_char_p
    L.moil_nb_last_error.argtypes = [ctypes.c_void_p]
    L.moil_nb_init.argtypes = [ctypes.c_void_p, ctypes.POINTER(Params), ctypes.POINTER(Topology)]
    L.moil_nb_init_batch.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(Replica)]
    L.moil_nb_get_alpha.argtypes = [ctypes.c_void_p, ctypes.c_int, _dp]
    L.moil_nb_eval.argtypes = [ctypes.c_void_p, _dp, _dp, ctypes.POINTER(Energies)]
    L.moil_nb_eval_device.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(Energies)]
    L.moil_nb_eval_device_async.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    L.moil_nb_eval_wait.argtypes = [ctypes.c_void_p, ctypes.POINTER(Energies)]
    L.moil_nb_adjoint.argtypes = [ctypes.c_void_p, _dp, _dp, _dp, _dp, ctypes.POINTER(Energies)]
    L.moil_nb_request_rebuild.argtypes = [ctypes.c_void_p]
    L.moil_nb_squeeze.argtypes = [ctypes.POINTER(Params), ctypes.POINTER(Topology), _dp]
    L.moil_nb_natoms.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64)]
    L.moil_nb_stream.restype = ctypes.c_void_p
    L.moil_nb_stream.argtypes = [ctypes.c_void_p]
    L.moil_nb_set_timing.argtypes = [ctypes.c_void_p, ctypes.c_int]
    L.moil_nb_get_timing.argtypes = [ctypes.c_void_p, ctypes.POINTER(Timing)]
    L.moil_nb_pair_stats.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64)]
    L.moil_nb_set_graph.argtypes = [ctypes.c_void_p, ctypes.c_int]
    L.moil_nb_get_virial.argtypes = [ctypes.c_void_p, ctypes.c_int, _dp]
    L.moil_nb_set_virial.argtypes = [ctypes.c_void_p, ctypes.c_int]
    L.moil_nb_set_groups.argtypes = [ctypes.c_void_p, ctypes.c_int]
    L.moil_nb_set_shape.argtypes = [ctypes.c_void_p, ctypes.POINTER(Shape)]
    L.moil_nb_get_shape.argtypes = [ctypes.c_void_p, ctypes.POINTER(Shape)]
    L.moil_nb_set_tune_cache.argtypes = [ctypes.c_void_p, ctypes.c_char_p]
    L.moil_nb_set_tune_mode.argtypes = [ctypes.c_void_p, ctypes.c_int]
    L.moil_nb_autotune.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(Replica), ctypes.c_void_p,
                                   ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(Shape), ctypes.POINTER(TuneTrial),
                                   ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
    L.moil_nb_md_step.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                  ctypes.c_double, ctypes.c_int, _dp, ctypes.POINTER(Energies), _dp]
    L.moil_nb_dcd_write.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, _dp]
    L.moil_nb_groups.argtypes = [ctypes.c_void_p]
    L.moil_nb_set_molecules.argtypes = [ctypes.c_void_p, _ip, _dp]
    L.moil_nb_pressure.argtypes = [ctypes.c_void_p, _dp, _dp, ctypes.POINTER(Energies), _dp]
    _lib = L
    return L


def _check(L, h, rc):
    if rc != 0:
        detail = L.moil_nb_last_error(h).decode() if h else ""
        raise MoilNbError(rc, f"{L.moil_nb_strerror(rc).decode()} {detail}".strip())


class _Keep:
    def __init__(self):
        self.refs = []

    def d(self, a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        self.refs.append(a)
        return a.ctypes.data_as(_dp)

    def i(self, a):
        a = np.ascontiguousarray(a, dtype=np.int32)
        if a.size == 0:
            a = np.zeros(1, dtype=np.int32)
        self.refs.append(a)
        return a.ctypes.data_as(_ip)


def make_params(s, precision=MOIL_NB_MIXED, skin=1.0, list_period=0, lj_switch=False, alpha=None,
                dtol=None) -> Params:
    """moil_nb_params of system s.  dtol (> 0) selects MOIL's route to the Ewald coefficient,
    alpha from erfc(alpha relx) / relx = dtol by bisection (symm/ewald_init.f:298-335);
    otherwise alpha (default s.alpha) is passed as is."""
    p = Params()
    p.rvmx, p.relx, p.eps = float(s.rvmx), float(s.relx), float(s.eps)
    p.a, p.b, p.c = (float(x) for x in s.box)
    if dtol is not None:
        p.dtol, p.alpha = float(dtol), 0.0
    else:
        p.dtol = 0.0
        p.alpha = float(s.alpha if alpha is None else alpha)
    p.nfft1, p.nfft2, p.nfft3 = (int(x) for x in s.nfft)
    p.order = int(s.order)
    p.arith, p.hvdw0 = int(s.arith), int(s.hvdw0)
    p.lj_switch = int(lj_switch)
    p.r_on = float(s.r_on)
    p.skin = float(skin)
    p.list_period = int(list_period)
    p.precision = int(precision)
    return p


def make_topology(s, keep: _Keep) -> Topology:
    t = Topology()
    t.npt = s.npt
    t.ptchg, t.epsgm6, t.epsgm12 = keep.d(s.ptchg), keep.d(s.epsgm6), keep.d(s.epsgm12)
    t.exc1, t.exc2 = keep.i(s.exc1), keep.i(s.exc2)
    t.totspe = len(s.spec1)
    t.spec1, t.spec2 = keep.i(s.spec1), keep.i(s.spec2)
    t.p14 = keep.d(s.p14 if len(s.p14) else np.zeros(3))
    t.totmon = s.totmon
    t.poipt, t.montype = keep.i(s.poipt), keep.i(s.montype)
    return t


class Nonbonded:
    """One device handle over one system or a batch of independent replicas."""

    def __init__(self, systems, precision=MOIL_NB_MIXED, device=0, skin=1.0, list_period=0,
                 lj_switch=False, timing=False, groups=0, dtol=None, shape=None, tune_cache=None,
                 tune_host=False):
        self.L = load()
        h = ctypes.c_void_p()
        _check(self.L, None, self.L.moil_nb_create(ctypes.byref(h), int(device)))
        self.h = h
        _check(self.L, self.h, self.L.moil_nb_set_groups(self.h, int(groups)))
        if shape is not None:
            self.set_shape(**dict(shape, groups=shape.get("groups", groups)))
        if tune_cache is not None:
            _check(self.L, self.h, self.L.moil_nb_set_tune_cache(self.h, str(tune_cache).encode()))
        if tune_host:
            # the tuner (and the cached shape) for callers that pass host buffers (eforce_into)
            _check(self.L, self.h, self.L.moil_nb_set_tune_mode(self.h, TUNE_HOST))
        self.batch = isinstance(systems, (list, tuple))
        self.systems = list(systems) if self.batch else [systems]
        keep = _Keep()
        self._params = [make_params(s, precision, skin, list_period, lj_switch, dtol=dtol) for s in self.systems]
        self._topos = [make_topology(s, keep) for s in self.systems]
        reps = (Replica * len(self.systems))()
        for k in range(len(self.systems)):
            reps[k].params = ctypes.pointer(self._params[k])
            reps[k].topo = ctypes.pointer(self._topos[k])
        _check(self.L, self.h, self.L.moil_nb_init_batch(self.h, len(self.systems), reps))
        # the replica descriptions stay alive: the autotuner rebuilds the handle from them
        self._reps, self._keep = reps, keep
        self.natom = sum(s.npt for s in self.systems)
        self.offsets = np.cumsum([0] + [s.npt for s in self.systems])
        self._e = (Energies * len(self.systems))()
        if timing:
            self.set_timing(True)

    def close(self):
        if getattr(self, "h", None):
            self.L.moil_nb_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def alpha(self, r=0) -> float:
        a = ctypes.c_double()
        _check(self.L, self.h, self.L.moil_nb_get_alpha(self.h, int(r), ctypes.byref(a)))
        return a.value

    def nblist(self):
        """MOIL's nbondm() + syminit(): rebuild the lists at the next evaluation."""
        _check(self.L, self.h, self.L.moil_nb_request_rebuild(self.h))

    def energies(self):
        """Per-replica energies of the last evaluation."""
        return [{k: getattr(self._e[r], k) for k in ENERGY_KEYS} for r in range(len(self.systems))]

    def md_step(self, d_coor_ptr: int, d_vel_ptr: int, d_mass_ptr: int, dt: float, nsteps: int = 1,
                water_geom=None):
        """nsteps device-resident leapfrog steps with rigid waters (moil_nb_md_step) on raw
        CUDA pointers; returns (per-replica energies of the last step, kinetic energy)."""
        ek = ctypes.c_double()
        wg = None
        if water_geom is not None:
            wg = np.ascontiguousarray(water_geom, dtype=np.float64)
        _check(self.L, self.h, self.L.moil_nb_md_step(
            self.h, ctypes.c_void_p(d_coor_ptr), ctypes.c_void_p(d_vel_ptr), ctypes.c_void_p(d_mass_ptr),
            float(dt), int(nsteps), wg.ctypes.data_as(_dp) if wg is not None else None, self._e,
            ctypes.byref(ek)))
        return self.energies(), ek.value

    def groups(self) -> int:
        """Number of concurrently evaluated replica groups (1: none)."""
        return int(self.L.moil_nb_groups(self.h))

    def set_shape(self, water_kernel=WATER_AUTO, half_block=0, tiled=TILED_AUTO, groups=0):
        """Kernel and list shapes (moil_nb_set_shape); the lists are rebuilt at the next call."""
        sh = Shape(int(water_kernel), int(half_block), int(tiled), int(groups))
        _check(self.L, self.h, self.L.moil_nb_set_shape(self.h, ctypes.byref(sh)))

    def shape(self) -> dict:
        """The shapes in use, automatic choices resolved (moil_nb_get_shape)."""
        sh = Shape()
        _check(self.L, self.h, self.L.moil_nb_get_shape(self.h, ctypes.byref(sh)))
        return {k: getattr(sh, k) for k in SHAPE_KEYS}

    def autotune(self, d_coor_ptr: int, d_dpot_ptr: int, evals: int = 0) -> dict:
        """moil_nb_autotune on device buffers of the batch: the chosen shape (applied) and
        every candidate timed, {"best": shape, "trials": [(shape, ms per evaluation), ...]}."""
        best = Shape()
        trials = (TuneTrial * 32)()
        n = ctypes.c_int()
        _check(self.L, self.h, self.L.moil_nb_autotune(
            self.h, len(self.systems), self._reps, ctypes.c_void_p(d_coor_ptr), ctypes.c_void_p(d_dpot_ptr),
            int(evals), ctypes.byref(best), trials, 32, ctypes.byref(n)))
        as_dict = lambda sh: {k: getattr(sh, k) for k in SHAPE_KEYS}
        return {"best": as_dict(best),
                "trials": [{"shape": as_dict(trials[k].shape), "ms_per_eval": trials[k].ms_per_eval}
                           for k in range(min(n.value, 32))]}

    def set_virial(self, on=True):
        """Accumulate the water-water LJ virial terms on the mixed path (off by default)."""
        _check(self.L, self.h, self.L.moil_nb_set_virial(self.h, int(on)))

    def virial(self):
        """MOIL's LJ virial terms virvdw1..virvdw5 of the last evaluation, per replica (a
        (5,) array for a single system)."""
        out = []
        for r in range(len(self.systems)):
            v = np.zeros(5)
            _check(self.L, self.h, self.L.moil_nb_get_virial(self.h, r, v.ctypes.data_as(_dp)))
            out.append(v)
        return out if self.batch else out[0]

    def eforce_into(self, coor: np.ndarray, dpot: np.ndarray, want_energies: bool = True):
        """Evaluate into caller-owned (natom,3) float64 arrays; returns per-replica energies."""
        assert coor.dtype == np.float64 and coor.flags.c_contiguous and coor.size == 3 * self.natom
        assert dpot.dtype == np.float64 and dpot.flags.c_contiguous and dpot.size == 3 * self.natom
        _check(self.L, self.h, self.L.moil_nb_eval(self.h, coor.ctypes.data_as(_dp), dpot.ctypes.data_as(_dp),
                                                   self._e))
        return self.energies() if want_energies else None

    def eforce(self, coor=None):
        """Nonbonded dpot (dE/dx, kcal/mol/Å) and energies.  Single system: (dpot, dict);
        batch: (list of dpot, list of dict)."""
        if coor is None:
            coor = np.concatenate([s.coor for s in self.systems], axis=0)
        elif self.batch and isinstance(coor, (list, tuple)):
            coor = np.concatenate(coor, axis=0)
        coor = np.ascontiguousarray(coor, dtype=np.float64).reshape(self.natom, 3)
        dpot = np.empty_like(coor)
        e = self.eforce_into(coor, dpot)
        if not self.batch:
            return dpot, e[0]
        return [dpot[self.offsets[k]:self.offsets[k + 1]] for k in range(len(self.systems))], e

    def adjoint_into(self, coor: np.ndarray, dq: np.ndarray, de: np.ndarray, ds: np.ndarray):
        """moil_nb_adjoint into caller-owned arrays: coor (natom,3), dq/de/ds (natom,) float64."""
        assert coor.dtype == np.float64 and coor.flags.c_contiguous and coor.size == 3 * self.natom
        for o in (dq, de, ds):
            assert o.dtype == np.float64 and o.flags.c_contiguous and o.size == self.natom
        _check(self.L, self.h, self.L.moil_nb_adjoint(self.h, coor.ctypes.data_as(_dp), dq.ctypes.data_as(_dp),
                                                      de.ctypes.data_as(_dp), ds.ctypes.data_as(_dp), self._e))
        return self.energies()

    def adjoint(self, coor=None):
        """Per-atom dE/dq, dE/deps, dE/dsigma (moil_nb_adjoint).  Single system: three
        (natom,) arrays; batch: three lists of per-replica arrays."""
        if coor is None:
            coor = np.concatenate([s.coor for s in self.systems], axis=0)
        elif self.batch and isinstance(coor, (list, tuple)):
            coor = np.concatenate(coor, axis=0)
        coor = np.ascontiguousarray(coor, dtype=np.float64).reshape(self.natom, 3)
        out = [np.empty(self.natom, dtype=np.float64) for _ in range(3)]
        _check(self.L, self.h, self.L.moil_nb_adjoint(self.h, coor.ctypes.data_as(_dp), *(o.ctypes.data_as(_dp)
                                                                                              for o in out), self._e))
        if not self.batch:
            return tuple(out)
        return tuple([o[self.offsets[k]:self.offsets[k + 1]] for k in range(len(self.systems))] for o in out)

    def set_molecules(self, mol, mass):
        """Molecules and masses of every atom for the pressure analysis
        (moil_nb_set_molecules); None switches it off."""
        if mol is None:
            _check(self.L, self.h, self.L.moil_nb_set_molecules(self.h, None, None))
            return
        self._mol = np.ascontiguousarray(mol, dtype=np.int32).reshape(self.natom)
        self._mass = np.ascontiguousarray(mass, dtype=np.float64).reshape(self.natom)
        _check(self.L, self.h, self.L.moil_nb_set_molecules(self.h, self._mol.ctypes.data_as(_ip),
                                                            self._mass.ctypes.data_as(_dp)))

    def pressure(self, coor=None, with_gradient: bool = True):
        """One evaluation and MOIL's pressure analysis terms (moil_nb_pressure): (dpot,
        energies, press), press the 12 values virXX..ZZ, V_PIdir, V_PIrec, V_PIrel; batch:
        lists per replica.  with_gradient=False skips the gradient copy (dpot is None)."""
        if coor is None:
            coor = np.concatenate([s.coor for s in self.systems], axis=0)
        elif self.batch and isinstance(coor, (list, tuple)):
            coor = np.concatenate(coor, axis=0)
        coor = np.ascontiguousarray(coor, dtype=np.float64).reshape(self.natom, 3)
        dpot = np.empty_like(coor) if with_gradient else None
        press = np.empty((len(self.systems), 12), dtype=np.float64)
        _check(self.L, self.h, self.L.moil_nb_pressure(self.h, coor.ctypes.data_as(_dp),
                                                       dpot.ctypes.data_as(_dp) if with_gradient else None,
                                                       self._e, press.ctypes.data_as(_dp)))
        e = self.energies()
        if not self.batch:
            return dpot, e[0], press[0]
        per = [dpot[self.offsets[k]:self.offsets[k + 1]] for k in range(len(self.systems))] if with_gradient else None
        return per, e, [press[k] for k in range(len(self.systems))]

    def eforce_device(self, d_coor_ptr: int, d_dpot_ptr: int, want_energies: bool = True):
        """Evaluate on device-resident buffers (raw CUDA pointers)."""
        _check(self.L, self.h, self.L.moil_nb_eval_device(self.h, ctypes.c_void_p(d_coor_ptr),
                                                          ctypes.c_void_p(d_dpot_ptr), self._e))
        return self.energies() if want_energies else None

    def eforce_device_async(self, d_coor_ptr: int, d_dpot_ptr: int):
        """Queue an evaluation on device-resident buffers and return at once; ``eval_wait``
        completes it.  The buffers stay untouched until then."""
        _check(self.L, self.h, self.L.moil_nb_eval_device_async(self.h, ctypes.c_void_p(d_coor_ptr),
                                                                ctypes.c_void_p(d_dpot_ptr)))

    def eval_wait(self, want_energies: bool = True):
        """Wait for the evaluation queued by ``eforce_device_async`` (regrowing lists and redoing
        it after an overflow); its energies per replica."""
        _check(self.L, self.h, self.L.moil_nb_eval_wait(self.h, self._e))
        return self.energies() if want_energies else None

    def set_timing(self, on=True):
        _check(self.L, self.h, self.L.moil_nb_set_timing(self.h, int(on)))

    def set_graph(self, on=True):
        """Replay evaluations as a captured CUDA graph (default) or launch kernel by kernel."""
        _check(self.L, self.h, self.L.moil_nb_set_graph(self.h, int(on)))

    def timing(self) -> dict:
        t = Timing()
        _check(self.L, self.h, self.L.moil_nb_get_timing(self.h, ctypes.byref(t)))
        return {k: getattr(t, k) for k, _ in Timing._fields_}

    def pair_stats(self):
        a, b = ctypes.c_int64(), ctypes.c_int64()
        _check(self.L, self.h, self.L.moil_nb_pair_stats(self.h, ctypes.byref(a), ctypes.byref(b)))
        return {"list_entries": a.value, "site_pairs": b.value}

    def stream(self) -> int:
        return self.L.moil_nb_stream(self.h) or 0


def dcd_write(path: str, coor: np.ndarray, first: bool, nframes: int = 1):
    """Append a frame (or start a file) in the binary format of dynamics/wdyncrd.f."""
    L = load()
    c = np.ascontiguousarray(coor, dtype=np.float64).reshape(-1, 3)
    _check(L, None, L.moil_nb_dcd_write(path.encode(), int(first), int(nframes), c.shape[0], c.ctypes.data_as(_dp)))


def squeeze(s, coor: np.ndarray) -> np.ndarray:
    """MOIL's squeeze() on a copy of coor (symm/squeeze.f:66-145) through the C ABI."""
    L = load()
    keep = _Keep()
    p = make_params(s)
    t = make_topology(s, keep)
    out = np.ascontiguousarray(coor, dtype=np.float64).copy()
    _check(L, None, L.moil_nb_squeeze(ctypes.byref(p), ctypes.byref(t), out.ctypes.data_as(_dp)))
    return out
