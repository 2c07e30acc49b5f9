"""Replica groups (moil_nb_set_groups): a batch evaluated as concurrent contiguous replica
ranges gives every replica the bit-identical result of the ungrouped evaluation, through
host buffers and device buffers, with list overflows regrown inside a group, and for the
parameter derivatives and virial terms."""
import numpy as np
import pytest

from moil_fnrfd_gb300 import systems as S
from moil_fnrfd_gb300.nb import Nonbonded

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def batch():
    reps = S.config3(10, seed=4321)
    reps.insert(3, S.config1(seed=7, n_solute=60, n_ions=7, n_waters=300, box=24.0))
    return reps


def _pair(batch, groups, **kw):
    a = Nonbonded(batch, groups=1, **kw)
    b = Nonbonded(batch, groups=groups, **kw)
    assert a.groups() == 1 and b.groups() == groups
    return a, b


@pytest.mark.parametrize("groups", [2, 3])
def test_grouped_host_evaluation_is_bit_identical(batch, groups):
    a, b = _pair(batch, groups)
    for _ in range(3):                      # first build, then list reuse
        da, ea = a.eforce()
        db, eb = b.eforce()
        for x, y in zip(da, db):
            assert np.array_equal(x, y)
        assert ea == eb
    assert a.pair_stats()["site_pairs"] == b.pair_stats()["site_pairs"]


def test_grouped_device_evaluation_is_bit_identical(batch):
    import torch
    a, b = _pair(batch, 3)
    coor = torch.from_numpy(np.concatenate([s.coor for s in batch])).cuda()
    da, db = torch.empty_like(coor), torch.empty_like(coor)
    torch.cuda.synchronize()
    ea = a.eforce_device(coor.data_ptr(), da.data_ptr())
    eb = b.eforce_device(coor.data_ptr(), db.data_ptr())
    assert torch.equal(da, db)
    assert ea == eb


def test_grouped_adjoint_and_virial(batch):
    a, b = _pair(batch, 2)
    a.set_virial(True)
    b.set_virial(True)
    a.eforce()
    b.eforce()
    for x, y in zip(a.virial(), b.virial()):
        assert np.array_equal(x, y)
    for x, y in zip(a.adjoint(), b.adjoint()):
        for u, v in zip(x, y):
            assert np.array_equal(u, v)


def test_group_overflow_regrows_within_the_group():
    """A densely packed replica in the second group overflows its rows; that group is redone
    with larger lists and the batch still matches the ungrouped evaluation."""
    reps = S.config3(6, seed=99)
    s = S.water_box(3000, (3000 / S.WATER_DENSITY) ** (1 / 3), 91, name="cluster")
    xyz = s.coor.reshape(-1, 3, 3)
    s.coor = (xyz - 0.25 * xyz[:, 0, :][:, None, :]).reshape(-1, 3)
    reps.append(s)
    a, b = _pair(reps, 2)
    da, ea = a.eforce()
    db, eb = b.eforce()
    for x, y in zip(da, db):
        assert np.array_equal(x, y)
    assert ea == eb


def test_automatic_groups_for_large_batches():
    small = Nonbonded(S.config3(4, seed=5))
    assert small.groups() == 1
