"""The two batched callers of the nonbonded path, restated as test harnesses.

Chain of images (chain/sds.f:60-105): MOIL loops over the interior images j = 2..igrid-1,
copies image j out of the chain array r into coor, rebuilds the lists (squeeze, nbondm,
syminit), calls eforce, stores e0(j) = e_total, adds it to sener and copies dpot into the
chain gradient dv.  Here the loop is one batched call over all interior images (each a
replica of the same topology); e0, sener and dv per image are checked against the oracle
(parity mode), and the end images' gradient rows stay zero as in MOIL.

Swarm of trajectories (dim/dim_sample_MD.f:113-264 runs many short trajectories from one
milestone): one batch handle steps six uneven water boxes together on the device
(moil_nb_md_step: evaluation, leapfrog, SETTLE); every replica's final frame is evaluated
and checked against the oracle, the constraints are held, and a replica stepped alone follows
the same trajectory (to 1e-3 Å over 30 steps: only the list-rebuild steps, decided per handle,
differ).

Tolerances: the mixed path's (relative RMS gradient error <= 1e-5, |dE_total|/|E_total|
<= 1e-6, each term within 1e-6 of the energy-term scale).
"""
import numpy as np
import pytest

import dyna as D
from moil_fnrfd_gb300 import systems as S
from moil_fnrfd_gb300.nb import Nonbonded
from oracle import oracle as O
from test_gpu_parity import check

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def chain_images(s, igrid, seed=3, step=0.25):
    """igrid images of s along a path: every water translated rigidly by j times its own
    random step (at most `step` Å per axis), so each image keeps the water geometry."""
    rng = np.random.Generator(np.random.PCG64(seed))
    d = np.repeat(rng.uniform(-step, step, size=(s.nwaters, 3)), 3, axis=0)
    return np.concatenate([s.coor + j * d for j in range(igrid)])   # r(3, igrid*npt)


def sds_batched(nb, r, npt, igrid):
    """The energy part of chain/sds.f:60-105, the image loop as one call over the interior
    images: e0(j), sener and dv(3, igrid*npt) (end images' rows zero)."""
    dv = np.zeros_like(r)
    e0 = np.zeros(igrid)
    dps, es = nb.eforce(r[npt:(igrid - 1) * npt])
    for j in range(1, igrid - 1):
        e0[j] = es[j - 1]["e_total"]
        dv[j * npt:(j + 1) * npt] = dps[j - 1]
    return e0, e0.sum(), dv


def test_chain_image_loop_as_one_batched_call(cfg0):
    igrid, npt = 6, cfg0.npt
    r = chain_images(cfg0, igrid)
    nb = Nonbonded([cfg0] * (igrid - 2), skin=1.0)
    e0, sener, dv = sds_batched(nb, r, npt, igrid)
    ref_sum = 0.0
    for j in range(1, igrid - 1):
        img = cfg0.copy()
        img.coor = r[j * npt:(j + 1) * npt].copy()
        ref, eref = O.eforce(img, mode="parity")
        ref_sum += eref["e_total"]
        e = nb.energies()[j - 1]
        assert e["e_total"] == e0[j]
        check(dv[j * npt:(j + 1) * npt], e, ref, eref, 0, f"image {j + 1}")
    assert abs(sener - ref_sum) <= 1e-6 * abs(ref_sum)
    assert not dv[:npt].any() and not dv[(igrid - 1) * npt:].any()
    # the next sweep over moved images reuses the handle: the lists follow the coordinates
    r2 = chain_images(cfg0, igrid, seed=4)
    _, _, dv2 = sds_batched(nb, r2, npt, igrid)
    img = cfg0.copy()
    img.coor = r2[2 * npt:3 * npt].copy()
    ref, eref = O.eforce(img, mode="parity")
    check(dv2[2 * npt:3 * npt], nb.energies()[1], ref, eref, 0, "image 3, second sweep")
    nb.close()


def test_swarm_final_frames_match_oracle():
    reps = S.config3(6, seed=77)
    offs = np.cumsum([0] + [s.npt for s in reps])
    nb = Nonbonded(reps, skin=1.5, list_period=10)
    md = D.RigidWaterDynamics(nb, reps, dt=0.002, temperature=300.0, seed=9)   # thermal velocities
    x0, v0 = md.x.clone(), md.v.clone()
    m = torch.tensor(np.concatenate([D._masses(s)[0] for s in reps]), dtype=torch.float64, device="cuda")
    x, v = x0.clone(), v0.clone()
    torch.cuda.synchronize()
    nb.md_step(x.data_ptr(), v.data_ptr(), m.data_ptr(), 0.002, 30)   # lists rebuilt on the way
    xf = x.cpu().numpy()
    assert np.abs(xf - x0.cpu().numpy()).max() > 0.05                 # the replicas moved
    dps, es = nb.eforce(xf)
    for r, s in enumerate(reps):
        t = s.copy()
        t.coor = xf[offs[r]:offs[r + 1]].copy()
        ref, eref = O.eforce(t, mode="parity")
        check(dps[r], es[r], ref, eref, 0, f"swarm replica {r} ({s.npt} atoms) after 30 steps")
        oh = np.linalg.norm(t.coor[1::3] - t.coor[0::3], axis=1)
        assert np.abs(oh - S.TIP3_ROH).max() < 1e-9
    nb.close()
    # replica 3 stepped alone from the same state ends where it ended in the swarm.  Not bit
    # for bit: a handle rebuilds all its replicas' lists when any site moved more than half
    # the skin, so the swarm rebuilds at other steps than the lone replica; the pair set is
    # the same, the FP32 summation order is not
    k = 3
    one = Nonbonded(reps[k], skin=1.5, list_period=10)
    xs = x0[offs[k]:offs[k + 1]].clone()
    vs = v0[offs[k]:offs[k + 1]].clone()
    ms = m[offs[k]:offs[k + 1]].clone()
    torch.cuda.synchronize()
    one.md_step(xs.data_ptr(), vs.data_ptr(), ms.data_ptr(), 0.002, 30)
    assert float((xs - x[offs[k]:offs[k + 1]]).abs().max()) < 1e-3
    one.close()
