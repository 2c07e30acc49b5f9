"""Generate the committed golden vectors for the 216-water configuration.

MOIL cannot be compiled here (no Fortran compiler) and ships no test
vectors, so these fixtures are the oracle's own output, pinned by the
known-answer tests in tests/test_oracle.py.  They guard the oracle and the
synthetic-system generator against silent changes.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from moil_fnrfd_gb300 import systems  # noqa: E402
from oracle import oracle  # noqa: E402


def main():
    s = systems.config0()
    out = {"coor": s.coor, "ptchg": s.ptchg}
    for mode in ("parity", "moil"):
        d, e = oracle.eforce(s, mode=mode)
        out[f"dpot_{mode}"] = d
        for k, v in e.items():
            if k.startswith("e_"):
                out[f"{mode}_{k}"] = np.float64(v)
        out[f"{mode}_site_pairs"] = np.int64(e["site_pairs"])
    # pressure analysis terms (molecules: the waters), minimum-image evaluator
    mol, mass = systems.molecules(s)
    out["press_mi"] = oracle.pressure(s, mol, mass, mode="mi")[2]
    np.savez_compressed(os.path.join(HERE, "config0_oracle.npz"), **out)
    print("wrote config0_oracle.npz")


if __name__ == "__main__":
    main()
