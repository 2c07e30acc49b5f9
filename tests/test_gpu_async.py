"""Asynchronous device-resident evaluation (moil_nb_eval_device_async + moil_nb_eval_wait).

The queued evaluation equals the synchronous one bit for bit (same kernels, same graph), over a
list rebuild and with replica groups; the caller's host work runs while the GPU evaluates; a
second queue before the wait, a wait without a queue, and other calls on the handle while an
evaluation is pending are refused with MOIL_NB_ERR_STATE and leave the pending evaluation intact.
"""
import numpy as np
import pytest

from moil_fnrfd_gb300 import systems as S
from moil_fnrfd_gb300.nb import MoilNbError, Nonbonded

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

STATE = 11      # MOIL_NB_ERR_STATE ("call order")


@pytest.mark.parametrize("groups", [1, 3])
def test_async_equals_sync(groups):
    reps = S.config3(6, seed=41)
    coor = np.concatenate([s.coor for s in reps])
    a = Nonbonded(reps, skin=1.0, list_period=4, groups=groups)
    b = Nonbonded(reps, skin=1.0, list_period=4, groups=groups)
    assert a.groups() == groups and b.groups() == groups
    rng = np.random.default_rng(5)
    dc = torch.from_numpy(coor).cuda()
    da, db = torch.empty_like(dc), torch.empty_like(dc)
    nw = len(coor) // 3                             # config-3 replicas are water boxes
    for step in range(6):                          # a rebuild every 4 evaluations
        # every water translated rigidly (its geometry kept)
        step_d = np.repeat(rng.uniform(-0.05, 0.05, size=(nw, 3)), 3, axis=0)
        dc += torch.from_numpy(step_d).cuda()
        torch.cuda.synchronize()
        ea = a.eforce_device(dc.data_ptr(), da.data_ptr())
        b.eforce_device_async(dc.data_ptr(), db.data_ptr())
        work = sum(k * k for k in range(20000))    # host work while the GPU evaluates
        eb = b.eval_wait()
        assert work > 0
        assert torch.equal(da, db), f"step {step}"
        for r in range(len(reps)):
            assert ea[r] == eb[r], (step, r)
    a.close()
    b.close()


def test_async_state_rules():
    s = S.config0()
    nbh = Nonbonded(s, skin=1.0)
    dc = torch.from_numpy(s.coor.copy()).cuda()
    dd = torch.empty_like(dc)
    ref = nbh.eforce_device(dc.data_ptr(), dd.data_ptr())[0]
    with pytest.raises(MoilNbError) as ex:
        nbh.eval_wait()                                            # nothing queued
    assert ex.value.status == STATE
    nbh.eforce_device_async(dc.data_ptr(), dd.data_ptr())
    for call in (lambda: nbh.eforce_device_async(dc.data_ptr(), dd.data_ptr()),   # one pending
                 lambda: nbh.eforce_device(dc.data_ptr(), dd.data_ptr()),         # the handle is busy
                 lambda: nbh.set_shape(groups=1)):
        with pytest.raises(MoilNbError) as ex:
            call()
        assert ex.value.status == STATE
    e = nbh.eval_wait()[0]
    assert e == ref
    nbh.close()
