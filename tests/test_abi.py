"""CPU checks of the C ABI library: it builds for sm_103a, loads, and exports every
function include/moil_nb.h declares.  No compute call runs without a GPU."""
import ctypes
import os
import re

import numpy as np

from moil_fnrfd_gb300 import build as B
from moil_fnrfd_gb300 import nb
from moil_fnrfd_gb300 import systems as S

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "moil_nb.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\**\s*([a-z_][a-z0-9_]*)\s*\(", text, flags=re.M)
    return sorted(set(n for n in names if n not in ("if", "return", "sizeof")))


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(B.build())
    names = declared_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert set(nb.EXPORTED) <= set(names)


def test_status_strings():
    L = nb.load()
    assert L.moil_nb_strerror(0) == b"ok"
    assert L.moil_nb_strerror(3) == b"system not neutral"
    assert L.moil_nb_strerror(999) == b"unknown status"


def test_async_evaluation_rejects_bad_arguments():
    """The asynchronous evaluation pair checks its arguments before any CUDA call."""
    L = nb.load()
    assert L.moil_nb_eval_device_async(None, None, None) == 1       # MOIL_NB_ERR_ARG
    assert L.moil_nb_eval_wait(None, None) == 1


def test_create_without_gpu_fails_cleanly():
    """With no visible GPU the handle constructor reports a CUDA error instead of aborting."""
    L = nb.load()
    h = ctypes.c_void_p()
    rc = L.moil_nb_create(ctypes.byref(h), 0)
    if rc == 0:          # a GPU is visible: just release it
        L.moil_nb_destroy(h)
    else:
        assert rc == 2 and not h.value


def test_squeeze_matches_moil_rule():
    """moil_nb_squeeze moves water/ion monomers by one box length when the first atom is
    outside [-L/2, L/2] (symm/squeeze.f:66-145), and never touches solute monomers."""
    s = S.config0()
    L = s.box[0]
    c = s.coor.copy()
    c[0:3, 0] += L          # water 0 pushed out along +x
    c[6:9, 1] -= L          # water 2 out along -y
    out = nb.squeeze(s, c)
    np.testing.assert_allclose(out, s.coor, atol=1e-12)
