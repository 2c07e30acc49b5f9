"""Molecular-dynamics harness around the nonbonded evaluation: leapfrog steps with rigid
three-site waters, device-resident coordinates and velocities.

MOIL's own integrator (dynamics/dyna.f:183-330, position SHAKE in shakept.f / mshakpt.f and
velocity SHAKE in shakevl.f / mshakvl.f) stays in the caller; this harness stands in for it
to drive the library through a trajectory: the 32,000-water workload of 1,000 steps at 2 fs
with the pair lists rebuilt every 10 steps.  Every step is one ``moil_nb_eval_device`` on the
step's coordinates followed by

    v(t + dt/2) = v(t - dt/2) - dt * c * dpot / m           (c = 418.4: kcal/mol/Å/amu -> Å/ps^2)
    x(t + dt)   = SETTLE(x(t), x(t) + dt * v(t + dt/2))
    v(t + dt/2) = (x(t + dt) - x(t)) / dt

SETTLE is the analytic rigid-water constraint of Miyamoto and Kollman (J. Comput. Chem. 13,
952 (1992)): the unconstrained molecule is expressed in a frame built from the previous
(rigid) molecule and its centre of mass, and three rotations (phi, psi, theta) place the
rigid molecule so that the centre of mass and the constraint forces' plane are kept.  Atoms
outside waters move unconstrained (the nonbonded forces only; no bonded terms here).

The harness runs in FP64 torch operations on the library's stream; it is not part of the
timed nonbonded evaluation.
"""
from __future__ import annotations

import math

import numpy as np

from moil_fnrfd_gb300.systems import MON_WATER, TIP3_HOH_DEG, TIP3_ROH

ACCEL = 418.4                 # (kcal/mol/Å) / amu in Å/ps^2
MASS_O, MASS_H = 15.9994, 1.008
KB = 0.0019872041             # kcal/mol/K


def _masses(s):
    m = np.full(s.npt, 12.0)
    first = 0
    water = np.zeros(s.npt, dtype=bool)
    for k in range(s.totmon):
        last = int(s.poipt[k])
        if s.montype[k] == MON_WATER:
            m[first:last] = (MASS_O, MASS_H, MASS_H)
            water[first:last] = True
        first = last
    return m, water


# SETTLE geometry (TIP3P): half the H-H distance, O to centre of mass and centre of mass to
# the H-H midpoint along the bisector
_HALF = math.radians(TIP3_HOH_DEG) / 2.0
SETTLE_MT = MASS_O + 2.0 * MASS_H
SETTLE_RC = TIP3_ROH * math.sin(_HALF)
SETTLE_RA = 2.0 * MASS_H * TIP3_ROH * math.cos(_HALF) / SETTLE_MT
SETTLE_RB = TIP3_ROH * math.cos(_HALF) - SETTLE_RA


def settle(x0, x1, widx):
    """Rigid-water positions (torch, FP64, any device) from the previous rigid positions x0
    and the unconstrained positions x1; widx (nwat, 3) holds the O, H1, H2 rows of x."""
    import torch as t
    if widx.numel() == 0:
        return x1
    a0, b0, c0 = (x0[widx[:, k]] for k in range(3))
    a1, b1, c1 = (x1[widx[:, k]] for k in range(3))
    com = (MASS_O * a1 + MASS_H * (b1 + c1)) / SETTLE_MT
    a1, b1, c1 = a1 - com, b1 - com, c1 - com
    ab0, ac0 = b0 - a0, c0 - a0
    # frame: z normal to the previous molecule, x normal to z and the new O offset
    ez = t.linalg.cross(ab0, ac0)
    ex = t.linalg.cross(a1, ez)
    ey = t.linalg.cross(ez, ex)
    ex, ey, ez = (e / t.linalg.vector_norm(e, dim=1, keepdim=True) for e in (ex, ey, ez))

    def loc(v):
        return (v * ex).sum(1), (v * ey).sum(1), (v * ez).sum(1)
    xb0, yb0, _ = loc(ab0)
    xc0, yc0, _ = loc(ac0)
    _, _, za1 = loc(a1)
    xb1, yb1, zb1 = loc(b1)
    xc1, yc1, zc1 = loc(c1)
    # phi and psi: the out-of-plane heights of O and of the H-H axis are kept
    sphi = za1 / SETTLE_RA
    cphi = t.sqrt(t.clamp(1.0 - sphi * sphi, min=0.0))
    spsi = (zb1 - zc1) / (2.0 * SETTLE_RC * cphi)
    cpsi = t.sqrt(t.clamp(1.0 - spsi * spsi, min=0.0))
    ya2 = SETTLE_RA * cphi
    xb2 = -SETTLE_RC * cpsi
    yb2 = -SETTLE_RB * cphi - SETTLE_RC * spsi * sphi
    yc2 = -SETTLE_RB * cphi + SETTLE_RC * spsi * sphi
    # theta: the in-plane rotation for which the constraint forces lie along the old bonds
    al = xb2 * (xb0 - xc0) + yb0 * yb2 + yc0 * yc2
    be = xb2 * (yc0 - yb0) + xb0 * yb2 + xc0 * yc2
    ga = xb0 * yb1 - xb1 * yb0 + xc0 * yc1 - xc1 * yc0
    ab2 = al * al + be * be
    sth = (al * ga - be * t.sqrt(t.clamp(ab2 - ga * ga, min=0.0))) / ab2
    cth = t.sqrt(t.clamp(1.0 - sth * sth, min=0.0))
    a3 = (-ya2 * sth, ya2 * cth, za1)
    b3 = (xb2 * cth - yb2 * sth, xb2 * sth + yb2 * cth, zb1)
    c3 = (-xb2 * cth - yc2 * sth, -xb2 * sth + yc2 * cth, zc1)
    out = x1.clone()
    for k, p in enumerate((a3, b3, c3)):
        out[widx[:, k]] = com + p[0][:, None] * ex + p[1][:, None] * ey + p[2][:, None] * ez
    return out


class RigidWaterDynamics:
    """Leapfrog MD of one system (or a batch handle's concatenated replicas) on the GPU.

    ``nb`` is a :class:`moil_fnrfd_gb300.nb.Nonbonded` handle; ``systems`` the system or the
    list of replicas it was created with.
    """

    def __init__(self, nb, systems, dt=0.002, temperature=0.0, seed=0):
        import torch
        self.torch = torch
        self.nb = nb
        systems = systems if isinstance(systems, (list, tuple)) else [systems]
        self.dt = float(dt)
        m, w = zip(*[_masses(s) for s in systems])
        m, water = np.concatenate(m), np.concatenate(w)
        coor = np.concatenate([s.coor for s in systems], axis=0)
        self.stream = torch.cuda.ExternalStream(nb.stream()) if nb.stream() else torch.cuda.current_stream()
        dev = torch.device("cuda", torch.cuda.current_device())
        with torch.cuda.stream(self.stream):
            self.x = torch.tensor(coor, dtype=torch.float64, device=dev).contiguous()
            self.dpot = torch.zeros_like(self.x)
            self.inv_m = torch.tensor(1.0 / m, dtype=torch.float64, device=dev)[:, None]
            self.m = torch.tensor(m, dtype=torch.float64, device=dev)[:, None]
            widx = np.nonzero(water)[0].reshape(-1, 3)
            self.widx = torch.tensor(widx, dtype=torch.int64, device=dev)
            self.v = torch.zeros_like(self.x)
            if temperature > 0.0:
                rng = np.random.Generator(np.random.PCG64(seed))
                v = rng.normal(size=coor.shape) * np.sqrt(KB * temperature * ACCEL / m)[:, None]
                self.v = torch.tensor(v, dtype=torch.float64, device=dev)
                # project the initial velocities onto the rigid molecules: one constrained drift
                self.v = (self._settle(self.x, self.x + self.dt * self.v) - self.x) / self.dt
        self.steps = 0
        self.energies = None

    def _settle(self, x0, x1):
        return settle(x0, x1, self.widx)

    # ---- stepping -------------------------------------------------------------------
    def evaluate(self):
        """One nonbonded evaluation at the current coordinates (per-replica energies)."""
        self.energies = self.nb.eforce_device(self.x.data_ptr(), self.dpot.data_ptr())
        return self.energies

    def advance(self):
        """The leapfrog update and SETTLE from the gradient of the last evaluation."""
        self.v.sub_(self.dpot * (self.dt * ACCEL) * self.inv_m)
        x1 = self._settle(self.x, self.x + self.dt * self.v)
        # in place: the evaluation's captured graph keeps the coordinate buffer
        self.v.copy_((x1 - self.x) / self.dt)
        self.x.copy_(x1)
        self.steps += 1

    def step(self, n=1):
        """n leapfrog steps; returns the energies of the last evaluation."""
        with self.torch.cuda.stream(self.stream):
            for _ in range(n):
                self.evaluate()
                self.advance()
        return self.energies

    def kinetic(self):
        """Kinetic energy (kcal/mol) of the half-step velocities."""
        return float(0.5 * (self.m * self.v * self.v).sum().item() / ACCEL)

    def constraint_error(self):
        """Largest deviation (Å) of any water's O-H or H-H distance from TIP3P."""
        t = self.torch
        if self.widx.numel() == 0:
            return 0.0
        a, b, c = (self.x[self.widx[:, k]] for k in range(3))
        d = t.stack([t.linalg.vector_norm(b - a, dim=1) - TIP3_ROH, t.linalg.vector_norm(c - a, dim=1) - TIP3_ROH,
                     t.linalg.vector_norm(c - b, dim=1) - 2.0 * SETTLE_RC])
        return float(d.abs().max().item())

    def coordinates(self):
        return self.x.detach().cpu().numpy()
