"""The autotuner (moil_nb_autotune) and its cache.

The tuner times every candidate shape on the handle's own batch and leaves the fastest
applied; whatever it picks, the evaluation stays within the mixed path's tolerances against
the oracle (parity mode).  Its cache file holds one line per (GPU, precision, replica count,
replica-size histogram): a new handle over the same batch starts with the cached shape, one
over another batch does not.  The host-buffer objective (MOIL_NB_TUNE_HOST) has a cache line
of its own.
"""
import numpy as np
import pytest

from moil_fnrfd_gb300 import systems as S
from moil_fnrfd_gb300.nb import Nonbonded
from oracle import oracle as O
from test_gpu_parity import check

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def batch():
    return S.config3(10)


def test_autotune_picks_a_timed_shape_that_matches_the_oracle(batch, tmp_path):
    cache = tmp_path / "tune.tsv"
    nb = Nonbonded(batch, skin=1.0, list_period=10, tune_cache=cache)
    coor = np.concatenate([s.coor for s in batch])
    dc = torch.from_numpy(coor).cuda()
    dd = torch.empty_like(dc)
    res = nb.autotune(dc.data_ptr(), dd.data_ptr(), evals=4)
    best, trials = res["best"], res["trials"]
    # groups 1..4, then the water kernels, then the row builds, duplicates timed once
    assert 6 <= len(trials) <= 11
    assert all(t["ms_per_eval"] > 0 for t in trials)
    assert best in [t["shape"] for t in trials]
    assert min(trials, key=lambda t: t["ms_per_eval"])["shape"] == best
    assert nb.shape() == best and nb.groups() == best["groups"]
    dps, es = nb.eforce()
    for r in (0, len(batch) - 1):
        ref, eref = O.eforce(batch[r], mode="parity")
        check(dps[r], es[r], ref, eref, 0, f"tuned replica {r}")
    nb.close()
    # the cache: one line for this batch; a new handle over the batch starts with its shape
    lines = cache.read_text().strip().splitlines()
    assert len(lines) == 1 and lines[0].split("\t")[1] == " ".join(
        str(best[k]) for k in ("water_kernel", "half_block", "tiled", "groups"))
    again = Nonbonded(batch, skin=1.0, list_period=10, tune_cache=cache)
    assert again.shape() == best
    again.close()
    other = Nonbonded(batch[:3], skin=1.0, list_period=10, tune_cache=cache)
    assert other.groups() == 1           # no entry for a 3-replica batch: the automatic choice
    other.close()


def test_host_objective_has_its_own_cache_line(batch, tmp_path):
    """MOIL_NB_TUNE_HOST times moil_nb_eval on page-locked copies of the batch; its result is
    stored under its own key, which device-mode handles do not read."""
    cache = tmp_path / "tune.tsv"
    nb = Nonbonded(batch, skin=1.0, list_period=10, tune_cache=cache, tune_host=True)
    coor = np.concatenate([s.coor for s in batch])
    dc = torch.from_numpy(coor).cuda()
    dd = torch.empty_like(dc)
    res = nb.autotune(dc.data_ptr(), dd.data_ptr(), evals=4)
    best = res["best"]
    assert nb.shape() == best
    hd = np.zeros_like(coor)
    es = nb.eforce_into(coor, hd)
    ref, eref = O.eforce(batch[0], mode="parity")
    check(hd[:batch[0].npt], es[0], ref, eref, 0, "host-tuned replica 0")
    nb.close()
    lines = cache.read_text().strip().splitlines()
    assert len(lines) == 1 and lines[0].split("\t")[0].endswith("|host")
    again = Nonbonded(batch, skin=1.0, list_period=10, tune_cache=cache, tune_host=True)
    assert again.shape() == best
    again.close()
    dev = Nonbonded(batch, skin=1.0, list_period=10, tune_cache=cache)
    assert dev.groups() == 1            # no device-mode entry: the automatic choice (1 for 10 replicas)
    dev.close()
