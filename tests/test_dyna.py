"""Rigid-water leapfrog harness (moil_fnrfd_gb300/dyna.py): SETTLE on the CPU against an
iterative SHAKE solution of the same constraint equations, and a short GPU trajectory
through the library (constraints held, energy conserved, final frame against the oracle)."""
import numpy as np
import pytest
import torch

import dyna as D
from moil_fnrfd_gb300 import systems as S


def shake(x0, x1, m, tol=1e-14, iters=2000):
    """Textbook SHAKE for one water: constraint forces along the previous bond vectors,
    iterated until every distance holds to tol."""
    d = {(0, 1): S.TIP3_ROH, (0, 2): S.TIP3_ROH, (1, 2): 2.0 * D.SETTLE_RC}
    x = x1.copy()
    for _ in range(iters):
        done = True
        for (i, j), l in d.items():
            r = x[i] - x[j]
            diff = r @ r - l * l
            if abs(diff) > tol:
                done = False
                r0 = x0[i] - x0[j]
                g = diff / (2.0 * (r @ r0) * (1.0 / m[i] + 1.0 / m[j]))
                x[i] -= g * r0 / m[i]
                x[j] += g * r0 / m[j]
        if done:
            return x
    raise AssertionError("SHAKE did not converge")


def test_settle_matches_shake():
    s = S.config0()
    rng = np.random.Generator(np.random.PCG64(5))
    x0 = s.coor.copy()
    x1 = x0 + rng.normal(scale=0.02, size=x0.shape)
    widx = torch.arange(s.npt).reshape(-1, 3)
    got = D.settle(torch.tensor(x0), torch.tensor(x1), widx).numpy()
    m = np.array([D.MASS_O, D.MASS_H, D.MASS_H])
    for w in range(0, s.npt // 3, 7):
        sl = slice(3 * w, 3 * w + 3)
        want = shake(x0[sl], x1[sl], m)
        assert np.abs(got[sl] - want).max() < 1e-9
        # centre of mass of the unconstrained molecule is kept
        assert np.allclose(m @ got[sl], m @ x1[sl], atol=1e-12)


def test_settle_keeps_rigid_motion():
    """A rigid rotation plus translation of the previous molecule is left as it is."""
    s = S.config0()
    x0 = s.coor.copy()
    th = 0.01
    R = np.array([[np.cos(th), -np.sin(th), 0], [np.sin(th), np.cos(th), 0], [0, 0, 1]])
    x1 = x0 @ R.T + np.array([0.01, -0.02, 0.005])
    widx = torch.arange(s.npt).reshape(-1, 3)
    got = D.settle(torch.tensor(x0), torch.tensor(x1), widx).numpy()
    assert np.abs(got - x1).max() < 1e-12


@pytest.mark.gpu
def test_trajectory_conserves_energy_and_matches_oracle(cfg0):
    from conftest import energy_scale, rel_rms
    from moil_fnrfd_gb300.nb import Nonbonded
    from oracle import oracle as O
    s = cfg0
    nb = Nonbonded(s, skin=1.5, list_period=10, timing=False)
    md = D.RigidWaterDynamics(nb, s, dt=0.001, temperature=300.0, seed=3)
    total = []
    for _ in range(200):
        e = md.step()[0]
        total.append(e["e_total"] + md.kinetic())
    assert md.constraint_error() < 1e-9
    # leapfrog with half-step kinetic energy: the total fluctuates without drifting (with the
    # oracle's FP64 forces the same trajectory ranges over ~40 kcal/mol, drift -7, while the
    # kinetic energy rises from 400 to 1500 kcal/mol as the lattice start relaxes)
    total = np.array(total)
    scale = energy_scale(e)
    assert total.max() - total.min() < 3e-3 * scale
    assert abs(total[-20:].mean() - total[:20].mean()) < 1e-3 * scale
    # the last frame, far from the start (lists reused and rebuilt on the way), against the oracle
    t = s.copy()
    t.coor = md.coordinates()
    dpot, e = nb.eforce(t.coor)
    ref, eref = O.eforce(t, mode="parity")
    assert rel_rms(dpot, ref) < 1e-5
    assert abs(e["e_total"] - eref["e_total"]) < 1e-6 * abs(eref["e_total"])


# ---- native integrator (moil_nb_md_step) and trajectory writer --------------------
def read_dcd(path):
    """Parse Fortran unformatted records: header, title, atom count, then x/y/z per frame."""
    import struct
    recs = []
    with open(path, "rb") as f:
        data = f.read()
    k = 0
    while k < len(data):
        n = struct.unpack_from("<i", data, k)[0]
        recs.append(data[k + 4:k + 4 + n])
        assert struct.unpack_from("<i", data, k + 4 + n)[0] == n
        k += 8 + n
    assert recs[0][:4] == b"CORD"
    vari = struct.unpack_from("<20i", recs[0], 4)
    natom = struct.unpack("<i", recs[2])[0]
    frames = []
    for f0 in range(3, len(recs), 3):
        frames.append(np.stack([np.frombuffer(recs[f0 + d], dtype="<f4") for d in range(3)], axis=1))
    return vari, natom, frames


def test_dcd_writer_format(tmp_path, cfg0):
    from moil_fnrfd_gb300.nb import dcd_write
    p = str(tmp_path / "t.dcd")
    dcd_write(p, cfg0.coor, first=True, nframes=2)
    dcd_write(p, cfg0.coor + 1.0, first=False)
    vari, natom, frames = read_dcd(p)
    assert vari[0] == 2 and natom == cfg0.npt and len(frames) == 2
    assert np.array_equal(frames[0], cfg0.coor.astype(np.float32))
    assert np.array_equal(frames[1], (cfg0.coor + 1.0).astype(np.float32))


def _masses_of(s):
    return D._masses(s)[0]


@pytest.mark.gpu
def test_native_steps_follow_the_harness(cfg0):
    """The library's leapfrog + SETTLE steps against the torch harness from the same state."""
    from moil_fnrfd_gb300.nb import Nonbonded
    s = cfg0
    nb = Nonbonded(s, skin=1.5, list_period=10)
    md = D.RigidWaterDynamics(nb, s, dt=0.001, temperature=300.0, seed=3)
    x = md.x.clone()
    v = md.v.clone()
    m = torch.tensor(_masses_of(s), dtype=torch.float64, device="cuda")
    nb2 = Nonbonded(s, skin=1.5, list_period=10)
    # one step from the same state: the same forces, two FP64 SETTLE implementations
    md.step(1)
    torch.cuda.synchronize()
    e, ek = nb2.md_step(x.data_ptr(), v.data_ptr(), m.data_ptr(), 0.001, 1)
    assert float((x - md.x).abs().max()) < 1e-12
    assert float((v - md.v).abs().max()) < 1e-9
    assert ek == pytest.approx(md.kinetic(), rel=1e-12)
    # twenty more: a last-bit difference in a position can flip the FP32 rounding of a site,
    # which the dynamics then carries along, so the trajectories separate slowly
    md.step(20)
    e, ek = nb2.md_step(x.data_ptr(), v.data_ptr(), m.data_ptr(), 0.001, 20)
    dx, dv = float((x - md.x).abs().max()), float((v - md.v).abs().max())
    assert dx < 1e-4 and dv < 1e-2, (dx, dv)
    assert ek == pytest.approx(md.kinetic(), rel=1e-5)


@pytest.mark.gpu
def test_native_trajectory_conserves_energy(cfg0):
    from conftest import energy_scale
    from moil_fnrfd_gb300.nb import Nonbonded
    s = cfg0
    nb = Nonbonded(s, skin=1.5, list_period=10)
    md = D.RigidWaterDynamics(nb, s, dt=0.001, temperature=300.0, seed=3)   # initial velocities
    x, v = md.x.clone(), md.v.clone()
    m = torch.tensor(_masses_of(s), dtype=torch.float64, device="cuda")
    total = []
    for _ in range(20):
        e, ek = nb.md_step(x.data_ptr(), v.data_ptr(), m.data_ptr(), 0.001, 10)
        total.append(e[0]["e_total"] + ek)
    total = np.array(total)
    assert total.max() - total.min() < 3e-3 * energy_scale(e[0])
    a, b, c = (x[k::3] for k in range(3))
    assert float((torch.linalg.vector_norm(b - a, dim=1) - S.TIP3_ROH).abs().max()) < 1e-9


@pytest.mark.gpu
def test_native_steps_grouped_batch_is_bit_identical():
    from moil_fnrfd_gb300.nb import Nonbonded
    reps = S.config3(6, seed=77)
    coor = torch.tensor(np.concatenate([r.coor for r in reps]), dtype=torch.float64, device="cuda")
    m = torch.tensor(np.concatenate([_masses_of(r) for r in reps]), dtype=torch.float64, device="cuda")
    out = []
    for groups in (1, 3):
        nb = Nonbonded(reps, skin=1.5, list_period=10, groups=groups)
        x, v = coor.clone(), torch.zeros_like(coor)
        torch.cuda.synchronize()
        e, ek = nb.md_step(x.data_ptr(), v.data_ptr(), m.data_ptr(), 0.002, 15)
        out.append((x, v, e, ek))
    assert torch.equal(out[0][0], out[1][0]) and torch.equal(out[0][1], out[1][1])
    assert out[0][2] == out[1][2] and out[0][3] == out[1][3]


@pytest.mark.gpu
def test_device_step_loop_matches_the_per_step_path():
    """moil_nb_md_step(n) replays a captured graph of whole steps n times on the device (one
    wait per call); n calls of one step run the per-step path (an evaluation and the
    integrator per call).  Both apply the same kernels and the same list schedule, so the
    trajectories are bit-identical -- over 25 steps with thermal velocities, list rebuilds by
    the list period and by the skin on the way, on a three-replica batch."""
    from moil_fnrfd_gb300.nb import Nonbonded
    reps = S.config3(3, seed=91)
    m = torch.tensor(np.concatenate([_masses_of(r) for r in reps]), dtype=torch.float64, device="cuda")
    loop = Nonbonded(reps, skin=1.0, list_period=10)
    md = D.RigidWaterDynamics(loop, reps, dt=0.002, temperature=300.0, seed=4)
    x0, v0 = md.x.clone(), md.v.clone()
    torch.cuda.synchronize()
    xa, va = x0.clone(), v0.clone()
    ea, ka = loop.md_step(xa.data_ptr(), va.data_ptr(), m.data_ptr(), 0.002, 25)
    step = Nonbonded(reps, skin=1.0, list_period=10)
    xb, vb = x0.clone(), v0.clone()
    for _ in range(25):
        eb, kb = step.md_step(xb.data_ptr(), vb.data_ptr(), m.data_ptr(), 0.002, 1)
    assert torch.equal(xa, xb) and torch.equal(va, vb)
    assert ea == eb and ka == kb
    loop.close()
    step.close()
