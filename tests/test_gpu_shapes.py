"""Kernel and list shapes (moil_nb_set_shape) against the oracle.

Every shape evaluates MOIL's pair set: the full-list water kernel (one water per thread over
both directions), the half-list kernel (each water pair once, the partner's share summed per
block in int32 shared-memory accumulators at 2^17, 2^16 or 2^15 units per kcal/mol/Å) with blocks
of 128, 256 and 512 waters, and the water rows built by cell search or by all-pairs tiles.  Each is
held to the mixed path's tolerances against the oracle in parity mode (relative RMS gradient
error <= 1e-5, |dE_total|/|E_total| <= 1e-6, each term within 1e-6 of the energy-term scale),
gives the oracle's site-pair count, and is bit-identical run to run.
"""
import numpy as np
import pytest

from conftest import rel_rms
from moil_fnrfd_gb300 import systems as S
from moil_fnrfd_gb300.nb import TILED_ALL, TILED_OFF, WATER_FULL, WATER_HALF, Nonbonded
from oracle import oracle as O
from test_gpu_parity import check

pytestmark = pytest.mark.gpu

SHAPES = [dict(water_kernel=WATER_FULL), dict(water_kernel=WATER_HALF, half_block=128),
          dict(water_kernel=WATER_HALF, half_block=256), dict(water_kernel=WATER_HALF, half_block=512)]


def _ids(shapes):
    return [f"{'half' if s['water_kernel'] == WATER_HALF else 'full'}{s.get('half_block', '')}" for s in shapes]


@pytest.fixture(scope="module")
def batch3():
    # the smallest, a middle and the largest of the first 24 batch replicas
    reps = S.config3(24)
    n = [r.npt for r in reps]
    pick = sorted({int(np.argmin(n)), 11, int(np.argmax(n))})
    return [reps[k] for k in pick]


@pytest.fixture(scope="module")
def refs3(batch3):
    return [O.eforce(s, mode="parity") for s in batch3]


@pytest.mark.parametrize("shape", SHAPES, ids=_ids(SHAPES))
def test_water_kernels_match_oracle(cfg0, shape):
    ref, eref = O.eforce(cfg0, mode="parity")
    nb = Nonbonded(cfg0, shape=shape)
    assert nb.shape()["water_kernel"] == shape["water_kernel"]
    dpot, e = nb.eforce(cfg0.coor)
    check(dpot, e, ref, eref, 0, f"216 waters {_ids([shape])[0]}")
    assert nb.pair_stats()["site_pairs"] == eref["site_pairs"]
    nb.close()


@pytest.mark.parametrize("shape", SHAPES, ids=_ids(SHAPES))
def test_water_kernels_on_a_batch(batch3, refs3, shape):
    """Replicas of 1.5k to 12k atoms in one handle: each against its oracle evaluation."""
    nb = Nonbonded(batch3, shape=shape)
    dps, es = nb.eforce()
    for r, (s, (ref, eref)) in enumerate(zip(batch3, refs3)):
        check(dps[r], es[r], ref, eref, 0, f"replica {r} ({s.npt} atoms) {_ids([shape])[0]}")
    n_pairs = sum(eref["site_pairs"] for _, eref in refs3)
    assert nb.pair_stats()["site_pairs"] == n_pairs
    d2, e2 = nb.eforce()
    assert all(np.array_equal(a, b) for a, b in zip(dps, d2)) and es == e2
    nb.close()


def test_half_lists_on_the_solute_system(cfg1):
    """Waters beside a solute: water-water pairs on half lists, water-solute pairs on the
    water's full W2 list and the solute's X list."""
    ref, eref = O.eforce(cfg1, mode="parity")
    nb = Nonbonded(cfg1, shape=dict(water_kernel=WATER_HALF))
    dpot, e = nb.eforce(cfg1.coor)
    check(dpot, e, ref, eref, 0, "solute, half lists")
    nb.close()


def test_shape_switch_on_a_live_handle(cfg0):
    """Switching shapes on one handle gives what a fresh handle with that shape gives."""
    rng = np.random.default_rng(11)
    coor = cfg0.coor + np.repeat(rng.uniform(-0.3, 0.3, size=(cfg0.nwaters, 3)), 3, axis=0)
    live = Nonbonded(cfg0)
    for shape in SHAPES + [dict(water_kernel=WATER_FULL, tiled=TILED_OFF),
                           dict(water_kernel=WATER_HALF, tiled=TILED_ALL)]:
        live.set_shape(**shape)
        dl, el = live.eforce(coor)
        fresh = Nonbonded(cfg0, shape=shape)
        df, ef = fresh.eforce(coor)
        assert np.array_equal(dl, df) and el == ef, shape
        fresh.close()
    live.close()


def test_list_build_methods_agree(batch3, refs3):
    """Cell search and all-pairs tiles give the same rows up to order: the same pair count
    and results within the mixed path's tolerances."""
    out = {}
    for tiled in (TILED_OFF, TILED_ALL):
        nb = Nonbonded(batch3, shape=dict(tiled=tiled))
        out[tiled] = nb.eforce() + (nb.pair_stats()["site_pairs"],)
        nb.close()
    assert out[TILED_OFF][2] == out[TILED_ALL][2]
    for r, (ref, eref) in enumerate(refs3):
        assert rel_rms(out[TILED_OFF][0][r], out[TILED_ALL][0][r]) < 1e-6
        for tiled in out:
            check(out[tiled][0][r], out[tiled][1][r], ref, eref, 0, f"replica {r} tiled={tiled}")
