"""Synthetic MOIL systems laid out exactly as MOIL's COMMON blocks hold them.

MOIL ships no example inputs, so every workload is generated here straight
into the arrays ``eforce()`` reads:

* ``coor(3,npt)``            -> ``coor``  (npt, 3) float64, Å
* ``ptchg/epsgm6/epsgm12``   -> per-atom charge and LJ encodings
  (``connect/fillpt.f:136-184``: geometric ``epsgm12 = 2*sqrt(eps)*sig^6``,
  ``epsgm6 = 2*sqrt(eps)*sig^3``; ``arith``: ``epsgm12 = 2*sqrt(eps)``,
  ``epsgm6 = sig``)
* ``exc1(0:npt)/exc2``       -> exclusion CSR, 1-based atom numbers, every
  pair listed once under its lower atom (``connect/angtor.f:483-567``)
* ``spec1/spec2/p14(3,*)``   -> 1-4 pairs and their parameters
  (``generic/wconn.f:286-325``)
* ``poipt``                  -> last atom (1-based) of every monomer
* monomer kinds: water (``TIP3``/``SPC*``), squeezed ion, other.

Water is TIP3P: O first, then H1 and H2, O-H 0.9572 Å, H-O-H 104.52°,
q_O = -0.834, q_H = +0.417, LJ on O only (eps 0.1521 kcal/mol,
Rmin/2 1.7682 Å).  All randomness is numpy ``PCG64`` with a recorded seed.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

KOFDIE = 332.0716          # COMMON/CONVERT.BLOCK:13
MON_OTHER, MON_WATER, MON_ION = 0, 1, 2

TIP3_QO, TIP3_QH = -0.834, 0.417
TIP3_EPS_O, TIP3_RMIN2_O = 0.1521, 1.7682
TIP3_ROH, TIP3_HOH_DEG = 0.9572, 104.52
WATER_DENSITY = 0.0334     # molecules / Å^3 at 0.997 g/cm^3 (3.3428e-2 to 4 digits)


def rmin2_to_sigma(rmin2: float) -> float:
    """sigma from Rmin/2: Rmin = 2^(1/6) sigma."""
    return 2.0 * rmin2 / 2.0 ** (1.0 / 6.0)


def lj_encode(eps: np.ndarray, sig: np.ndarray, arith: bool):
    """MOIL's per-atom LJ encoding (``connect/fillpt.f:136-184``)."""
    eps = np.asarray(eps, dtype=np.float64)
    sig = np.asarray(sig, dtype=np.float64)
    if arith:
        e12 = np.sqrt(4.0 * eps)
        e6 = sig.copy()
    else:
        s6 = sig ** 6
        e12 = np.sqrt(s6 * 4.0 * s6 * eps)
        e6 = np.sqrt(4.0 * s6 * eps)
    return e6, e12


@dataclasses.dataclass
class MoilSystem:
    """One periodic system in MOIL's COMMON layout plus its run parameters."""
    name: str
    coor: np.ndarray        # (npt,3) float64
    ptchg: np.ndarray       # (npt,)
    epsgm6: np.ndarray
    epsgm12: np.ndarray
    exc1: np.ndarray        # (npt+1,) int32, exc1[0] = 0
    exc2: np.ndarray        # (nexc,) int32, 1-based
    spec1: np.ndarray       # (totspe,) int32, 1-based
    spec2: np.ndarray
    p14: np.ndarray         # (totspe,3)
    poipt: np.ndarray       # (totmon,) int32 last atom of monomer, 1-based
    montype: np.ndarray     # (totmon,) int32 MON_*
    box: tuple              # (a,b,c)
    arith: bool = False
    hvdw0: bool = True
    rvmx: float = 9.0       # LJ cutoff
    relx: float = 9.0       # Coulomb cutoff
    eps: float = 1.0        # dielectric
    alpha: float = 0.35     # Ewald coefficient (Å^-1)
    nfft: tuple = (20, 20, 20)
    order: int = 4
    r_on: float = 0.0       # LJ switch start (extension; used only when switched on)
    seed: int = 0

    @property
    def npt(self) -> int:
        return int(self.coor.shape[0])

    @property
    def totmon(self) -> int:
        return int(self.poipt.shape[0])

    @property
    def nwaters(self) -> int:
        return int(np.count_nonzero(self.montype == MON_WATER))

    def copy(self) -> "MoilSystem":
        return dataclasses.replace(self, **{f.name: (getattr(self, f.name).copy()
                                                      if isinstance(getattr(self, f.name), np.ndarray)
                                                      else getattr(self, f.name))
                                             for f in dataclasses.fields(self)})


# --------------------------------------------------------------------------------------
# geometry helpers


def _water_frame() -> np.ndarray:
    """TIP3P sites (O, H1, H2) in a local frame with O at the origin."""
    half = math.radians(TIP3_HOH_DEG) / 2.0
    h1 = np.array([TIP3_ROH * math.sin(half), TIP3_ROH * math.cos(half), 0.0])
    h2 = np.array([-TIP3_ROH * math.sin(half), TIP3_ROH * math.cos(half), 0.0])
    return np.stack([np.zeros(3), h1, h2])


def _random_rotations(rng: np.random.Generator, n: int) -> np.ndarray:
    """Uniform random rotation matrices from uniform unit quaternions (Shoemake 1992)."""
    u1, u2, u3 = rng.random(n), rng.random(n), rng.random(n)
    q = np.stack([np.sqrt(1 - u1) * np.sin(2 * np.pi * u2),
                  np.sqrt(1 - u1) * np.cos(2 * np.pi * u2),
                  np.sqrt(u1) * np.sin(2 * np.pi * u3),
                  np.sqrt(u1) * np.cos(2 * np.pi * u3)], axis=1)
    x, y, z, w = q.T
    r = np.empty((n, 3, 3))
    r[:, 0, 0] = 1 - 2 * (y * y + z * z); r[:, 0, 1] = 2 * (x * y - z * w); r[:, 0, 2] = 2 * (x * z + y * w)
    r[:, 1, 0] = 2 * (x * y + z * w); r[:, 1, 1] = 1 - 2 * (x * x + z * z); r[:, 1, 2] = 2 * (y * z - x * w)
    r[:, 2, 0] = 2 * (x * z - y * w); r[:, 2, 1] = 2 * (y * z + x * w); r[:, 2, 2] = 1 - 2 * (x * x + y * y)
    return r


def _lattice_sites(m: int, box: float) -> np.ndarray:
    """Cell centres of an m^3 cubic lattice filling a box centred at the origin."""
    s = box / m
    g = (np.arange(m) + 0.5) * s - box / 2.0
    x, y, z = np.meshgrid(g, g, g, indexing="ij")
    return np.stack([x.ravel(), y.ravel(), z.ravel()], axis=1)


def _place_waters(rng, oxy: np.ndarray) -> np.ndarray:
    """Three sites per oxygen site, uniformly random orientation."""
    frame = _water_frame()
    rot = _random_rotations(rng, oxy.shape[0])
    sites = np.einsum("nij,kj->nki", rot, frame) + oxy[:, None, :]
    return sites.reshape(-1, 3)


# --------------------------------------------------------------------------------------
# topology assembly


class _Builder:
    def __init__(self, arith: bool):
        self.arith = arith
        self.coor, self.q, self.eps, self.sig = [], [], [], []
        self.poipt, self.montype = [], []
        self.excl = []      # list of (i,j) 0-based, i<j
        self.pairs14 = []   # (i,j) 0-based
        self.n = 0

    def add_monomer(self, xyz, q, eps, sig, kind, excl_local=(), pairs14_local=()):
        base = self.n
        k = len(q)
        self.coor.append(np.asarray(xyz, dtype=np.float64).reshape(k, 3))
        self.q.extend(q); self.eps.extend(eps); self.sig.extend(sig)
        self.n += k
        self.poipt.append(self.n)
        self.montype.append(kind)
        for (i, j) in excl_local:
            self.excl.append((base + min(i, j), base + max(i, j)))
        for (i, j) in pairs14_local:
            self.pairs14.append((base + min(i, j), base + max(i, j)))
        return base

    def add_waters(self, sites: np.ndarray):
        nw = sites.shape[0] // 3
        sig_o = rmin2_to_sigma(TIP3_RMIN2_O)
        for w in range(nw):
            self.add_monomer(sites[3 * w:3 * w + 3], [TIP3_QO, TIP3_QH, TIP3_QH],
                             [TIP3_EPS_O, 0.0, 0.0], [sig_o, 0.0, 0.0], MON_WATER,
                             excl_local=[(0, 1), (0, 2), (1, 2)])

    def finish(self, name, box, **kw) -> MoilSystem:
        coor = np.concatenate(self.coor, axis=0)
        npt = coor.shape[0]
        q = np.asarray(self.q, dtype=np.float64)
        e6, e12 = lj_encode(np.asarray(self.eps), np.asarray(self.sig), self.arith)
        # exclusion CSR under the lower atom, partners in ascending order
        excl = sorted(set(self.excl))
        exc1 = np.zeros(npt + 1, dtype=np.int32)
        exc2 = np.zeros(len(excl), dtype=np.int32)
        for k, (i, j) in enumerate(excl):
            exc1[i + 1] += 1
            exc2[k] = j + 1
        exc1 = np.cumsum(exc1).astype(np.int32)
        spec = sorted(set(self.pairs14))
        spec1 = np.array([i + 1 for i, _ in spec], dtype=np.int32)
        spec2 = np.array([j + 1 for _, j in spec], dtype=np.int32)
        p14 = np_p14(spec, q, e6, e12, self.arith, eps=kw.get("eps", 1.0))
        return MoilSystem(name=name, coor=coor, ptchg=q, epsgm6=e6, epsgm12=e12,
                          exc1=exc1, exc2=exc2, spec1=spec1, spec2=spec2, p14=p14,
                          poipt=np.asarray(self.poipt, dtype=np.int32),
                          montype=np.asarray(self.montype, dtype=np.int32),
                          box=(box, box, box), arith=self.arith, **kw)


def np_p14(spec, q, e6, e12, arith, eps=1.0, v14=1.0, el14=1.0, hvdw0=True):
    """1-4 parameters as ``generic/wconn.f:286-325`` writes them (scales v14, el14)."""
    p14 = np.zeros((len(spec), 3), dtype=np.float64)
    for k, (j, l) in enumerate(spec):
        if not arith:
            if (e12[j] < 1e-3 or e12[l] < 1e-3) and hvdw0:
                p14[k, 0] = p14[k, 1] = 0.0
            else:
                p14[k, 0] = e12[j] * e12[l] * v14
                p14[k, 1] = e6[j] * e6[l] * v14
        else:
            s6 = (0.5 * (e6[j] + e6[l])) ** 6
            p14[k, 0] = (e12[j] * e12[l]) * s6 * s6 * v14
            p14[k, 1] = (e12[j] * e12[l]) * s6 * v14
        p14[k, 2] = q[j] * q[l] * eps * el14 * KOFDIE
    return p14


# --------------------------------------------------------------------------------------
# the named workloads


def water_box(n_waters: int, box: float, seed: int, name="water", jitter=0.3,
              rc=9.0, alpha=0.35, nfft=None) -> MoilSystem:
    """Periodic TIP3P box: O on a seeded subset of a cubic lattice, jittered, random orientation."""
    rng = np.random.Generator(np.random.PCG64(seed))
    m = int(math.ceil(round(n_waters ** (1.0 / 3.0), 9)))
    sites = _lattice_sites(m, box)
    if sites.shape[0] > n_waters:
        pick = np.sort(rng.choice(sites.shape[0], size=n_waters, replace=False))
        sites = sites[pick]
    oxy = sites + rng.uniform(-jitter, jitter, size=sites.shape)
    b = _Builder(arith=False)
    b.add_waters(_place_waters(rng, oxy))
    if nfft is None:
        n = smooth_grid(box)
        nfft = (n, n, n)
    return b.finish(name, box, rvmx=rc, relx=rc, alpha=alpha, nfft=tuple(nfft), seed=seed)


def smooth_grid(length: float, min_n: int = 1) -> int:
    """Smallest 2/3/5-smooth n >= max(length (1 point / Å), min_n)."""
    n = max(int(math.ceil(length - 1e-9)), min_n)
    while True:
        k = n
        for p in (2, 3, 5):
            while k % p == 0:
                k //= p
        if k == 1:
            return n
        n += 1


def config0(seed: int = 2024) -> MoilSystem:
    """216 TIP3P waters in an 18.62 Å cube, rc 9, alpha 0.35, grid 20^3."""
    return water_box(216, 18.62, seed, name="tip3p_216", rc=9.0, alpha=0.35, nfft=(20, 20, 20))


def config2(seed: int = 2026) -> MoilSystem:
    """32,000 TIP3P waters in a 98.6 Å cube, rc 10, alpha 0.32, grid 100^3."""
    return water_box(32000, 98.6, seed, name="tip3p_96000", rc=10.0, alpha=0.32, nfft=(100, 100, 100))


def config3_sizes(n_rep: int = 512, seed: int = 3000):
    """Replica atom counts: log-uniform in [1500, 12000], rounded to whole molecules."""
    rng = np.random.Generator(np.random.PCG64(seed))
    n = np.exp(rng.uniform(math.log(1500.0), math.log(12000.0), size=n_rep))
    return (3 * np.round(n / 3.0)).astype(np.int64)


def config3(n_rep: int = 512, seed: int = 3000) -> list:
    """Batched uneven water boxes (path-image / milestoning-swarm shape)."""
    out = []
    for r, n_atoms in enumerate(config3_sizes(n_rep, seed)):
        nw = int(n_atoms) // 3
        box = (nw / WATER_DENSITY) ** (1.0 / 3.0)
        n = smooth_grid(box)
        out.append(water_box(nw, box, seed + 1 + r, name=f"rep{r}", rc=9.0, alpha=0.35, nfft=(n, n, n)))
    return out


def _self_avoiding_chain(rng, n, bond, radius, dmin, max_tries=200):
    """Bead chain with fixed bond length confined to a sphere.

    Beads three or more apart along the chain stay at least ``dmin`` apart.
    Steps are drawn uniformly on the sphere; a cell grid keeps the overlap
    test local; a bead that cannot be placed backs the walk up a few beads.
    """
    pos = np.zeros((n, 3))
    cell = dmin
    grid = {}

    def key(p):
        return (int(math.floor(p[0] / cell)), int(math.floor(p[1] / cell)), int(math.floor(p[2] / cell)))

    def ok(p, i):
        if np.dot(p, p) > radius * radius:
            return False
        kx, ky, kz = key(p)
        for dx in (-1, 0, 1):
            for dy in (-1, 0, 1):
                for dz in (-1, 0, 1):
                    for j in grid.get((kx + dx, ky + dy, kz + dz), ()):
                        if j < i - 2 and np.sum((pos[j] - p) ** 2) < dmin * dmin:
                            return False
        return True

    def put(i):
        grid.setdefault(key(pos[i]), []).append(i)

    def drop(i):
        grid[key(pos[i])].remove(i)

    put(0)
    i = 1
    fails = 0
    while i < n:
        placed = False
        for _ in range(max_tries):
            v = rng.normal(size=3)
            v *= bond / np.linalg.norm(v)
            p = pos[i - 1] + v
            if i >= 2:
                # keep a bond angle of at least 80 degrees so 1-3 beads are not on top of each other
                u = pos[i - 2] - pos[i - 1]
                if np.dot(u, v) / (bond * bond) > math.cos(math.radians(80.0)):
                    continue
            if ok(p, i):
                pos[i] = p
                put(i)
                placed = True
                break
        if placed:
            i += 1
            continue
        fails += 1
        back = min(i - 1, 3 + fails // 50)
        for k in range(i - 1, i - 1 - back, -1):
            drop(k)
        i -= back
        if fails > 20000:
            raise RuntimeError("chain generation failed")
    return pos


def config1(seed: int = 2025, n_solute: int = 2489, n_ions: int = 7, n_waters: int = 7020,
            box: float = 62.2, arith: bool = True, tiny_h: bool = False) -> MoilSystem:
    """Protein-like solute + 7 Na+ + TIP3P in a 62.2 Å cube (N = 23,556 with 7,020 waters).

    The stated 23,558 cannot be formed from 2,489 solute atoms, 7 ions and
    whole three-site waters (21,062 is not a multiple of 3); 7,020 waters
    give 23,556 atoms.  arith=False switches to MOIL's geometric encoding; tiny_h makes
    every third solute atom a hydrogen with eps 0.01, Rmin/2 0.2245 (epsgm12 < 1e-3 under
    the geometric rule, so MOIL's hvdw0 rule applies to its pairs, pot/nbond.f:115-126).
    """
    rng = np.random.Generator(np.random.PCG64(seed))
    # solute: compact self-avoiding chain at protein-like density (~0.083 atoms/Å^3)
    radius = (3.0 * (n_solute / 0.083) / (4.0 * math.pi)) ** (1.0 / 3.0)
    chain = _self_avoiding_chain(rng, n_solute, 1.5, radius, 2.0)
    chain -= chain.mean(axis=0)
    q = rng.normal(0.0, 0.35, size=n_solute)
    q += (-7.0 - q.sum()) / n_solute
    eps_t = np.array([0.046, 0.11, 0.155, 0.2])
    rm2_t = np.array([1.2, 1.7, 1.85, 2.0])
    typ = np.arange(n_solute) % 4
    sig = np.array([rmin2_to_sigma(r) for r in rm2_t])[typ]
    eps = eps_t[typ]
    if tiny_h:
        h = np.arange(n_solute) % 3 == 2
        sig[h], eps[h] = rmin2_to_sigma(0.2245), 0.01
    b = _Builder(arith=arith)
    # monomers of three beads; bonded exclusions and 1-4 pairs span monomers
    n_mono = (n_solute + 2) // 3
    for mnum in range(n_mono):
        lo, hi = 3 * mnum, min(3 * mnum + 3, n_solute)
        b.add_monomer(chain[lo:hi], list(q[lo:hi]), list(eps[lo:hi]), list(sig[lo:hi]), MON_OTHER)
    for i in range(n_solute):
        for d in (1, 2, 3):
            if i + d < n_solute:
                b.excl.append((i, i + d))
        if i + 3 < n_solute:
            b.pairs14.append((i, i + 3))
    # ions: random sites at least 3 Å from the solute and from each other
    ions = []
    half = box / 2.0
    while len(ions) < n_ions:
        p = rng.uniform(-half, half, size=3)
        if np.min(np.sum((chain - p) ** 2, axis=1)) < 9.0:
            continue
        if any(np.sum((p - o) ** 2) < 9.0 for o in ions):
            continue
        ions.append(p)
    for p in ions:
        b.add_monomer(p[None, :], [1.0], [0.0469], [rmin2_to_sigma(1.3638)], MON_ION)
    # water: lattice of candidate sites at ~2.96 Å spacing (21 per side of the 62.2 Å box),
    # drop those within 2.4 Å of solute or ions, seeded pick
    m = max(2, int(round(box / 2.962)))
    cand = _lattice_sites(m, box) + rng.uniform(-0.3, 0.3, size=(m ** 3, 3))
    frame_sites = _place_waters(rng, cand).reshape(-1, 3, 3)
    heavy = np.concatenate([chain, np.asarray(ions)], axis=0)
    keep = []
    for w in range(frame_sites.shape[0]):
        d2 = np.sum((heavy[None, :, :] - frame_sites[w][:, None, :]) ** 2, axis=2)
        # minimum-image distance so waters near the faces see solute images too
        dv = heavy[None, :, :] - frame_sites[w][:, None, :]
        dv -= box * np.round(dv / box)
        d2 = np.sum(dv * dv, axis=2)
        if d2.min() >= 2.4 * 2.4:
            keep.append(w)
    keep = np.asarray(keep)
    if keep.shape[0] < n_waters:
        raise RuntimeError(f"only {keep.shape[0]} water sites free, need {n_waters}")
    pick = np.sort(rng.choice(keep.shape[0], size=n_waters, replace=False))
    b.add_waters(frame_sites[keep[pick]].reshape(-1, 3))
    n = smooth_grid(box)  # 64 for 62.2 Å
    return b.finish("solute_23556", box, rvmx=9.0, relx=9.0, alpha=0.35, nfft=(64, 64, 64), seed=seed)


def lj_decode(s: MoilSystem):
    """(eps, sigma) per atom from MOIL's epsgm encoding (connect/fillpt.f:136-184):
    geometric epsgm12 = 2 sqrt(eps) sigma^6, epsgm6 = 2 sqrt(eps) sigma^3; arithmetic
    epsgm12 = 2 sqrt(eps), epsgm6 = sigma.  Atoms without LJ decode to (0, 0)."""
    e12, e6 = s.epsgm12, s.epsgm6
    if s.arith:
        return 0.25 * e12 * e12, e6.copy()
    eps, sig = np.zeros(s.npt), np.zeros(s.npt)
    ok = (e12 > 0) & (e6 > 0)
    sig[ok] = np.cbrt(e12[ok] / e6[ok])
    eps[ok] = (e6[ok] ** 2 / (2.0 * e12[ok])) ** 2
    return eps, sig


def with_lj(s: MoilSystem, eps: np.ndarray, sig: np.ndarray) -> MoilSystem:
    """A copy of s with every atom's LJ parameters set from (eps, sigma) and the 1-4
    parameters re-derived (generic/wconn.f:286-325)."""
    t = s.copy()
    t.epsgm6, t.epsgm12 = lj_encode(eps, sig, s.arith)
    if len(t.spec1):
        spec = list(zip(t.spec1 - 1, t.spec2 - 1))
        t.p14 = np_p14(spec, t.ptchg, t.epsgm6, t.epsgm12, t.arith, eps=t.eps, hvdw0=t.hvdw0)
    return t


def perturbed_copies(base: MoilSystem, n_copies: int = 64, seed: int = 4000, rel: float = 0.01):
    """Copies with seeded relative perturbations in [-rel, rel]: eps and sigma per LJ type
    (atoms sharing one (eps, sigma) pair, the water oxygen among them), charges per solute
    atom.  The charge perturbation is re-centred over the solute so every copy stays
    neutral; waters keep their charges (the water kernel assumes identical waters)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    eps, sig = lj_decode(base)
    types, tid = np.unique(np.round(np.stack([eps, sig], axis=1), 12), axis=0, return_inverse=True)
    tid = tid.reshape(-1)
    solute = np.zeros(base.npt, dtype=bool)
    first = 0
    for m in range(base.totmon):
        last = int(base.poipt[m])
        if base.montype[m] == MON_OTHER:
            solute[first:last] = True
        first = last
    out = []
    for k in range(n_copies):
        fe = 1.0 + rng.uniform(-rel, rel, size=len(types))
        fs = 1.0 + rng.uniform(-rel, rel, size=len(types))
        s = base.copy()
        s.ptchg = base.ptchg.copy()
        if solute.any():
            dq = base.ptchg[solute] * rng.uniform(-rel, rel, size=int(solute.sum()))
            s.ptchg[solute] += dq - dq.mean()
        s = with_lj(s, eps * fe[tid], sig * fs[tid])
        s.name = f"{base.name}_pert{k}"
        out.append(s)
    return out


def make_config(idx: int):
    if idx == 0:
        return config0()
    if idx == 1:
        return config1()
    if idx == 2:
        return config2()
    if idx == 3:
        return config3()
    raise ValueError(idx)


MASS_O, MASS_H, MASS_NA, MASS_BEAD = 15.9994, 1.008, 22.98977, 12.011


def molecules(s: MoilSystem):
    """Covalent molecules and atom masses for the pressure analysis (analysis/pressure.f,
    whose dmolecule groups atoms joined by bonds): here the connected components of the
    exclusion graph (every bond is an exclusion, and every exclusion joins atoms of one
    molecule).  Returns (mol, mass): 0-based molecule index of every atom, numbered in
    order of first atom, and masses (TIP3P O/H, Na+ for ions, a carbon-like bead else)."""
    n = s.npt
    parent = np.arange(n)

    def find(a):
        while parent[a] != a:
            parent[a] = parent[parent[a]]
            a = parent[a]
        return a
    for i in range(n):
        for k in range(int(s.exc1[i]), int(s.exc1[i + 1])):
            a, b = find(i), find(int(s.exc2[k]) - 1)
            if a != b:
                parent[max(a, b)] = min(a, b)
    root = np.array([find(i) for i in range(n)])
    _, mol = np.unique(root, return_inverse=True)   # roots are first atoms: ids in atom order
    mass = np.full(n, MASS_BEAD)
    first = 0
    for k in range(s.totmon):
        last = int(s.poipt[k])
        if s.montype[k] == MON_WATER:
            mass[first:last] = (MASS_O, MASS_H, MASS_H)
        elif s.montype[k] == MON_ION:
            mass[first:last] = MASS_NA
        first = last
    return mol.astype(np.int32), mass
