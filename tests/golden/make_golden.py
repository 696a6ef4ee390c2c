"""Generates the committed golden fixtures of tests/golden/ with the oracle.

The reference ships no test data and cannot be compiled here (no Fortran
compiler), so these fixtures pin the oracle against its own earlier output:
residual history, forces and final state of two small seeded cases.
Run:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from tests import oracle_binding as ob  # noqa: E402
from turns2d_urans_git_gb300 import api  # noqa: E402

CASES = {
    "c1_small": ("c1", dict(jmax=97, kmax=25), 120),
    "c2_small": ("c2", dict(jmax=97, kmax=33, ds_wall=1e-4), 80),
}


def case(kind, kw):
    return (api.config_c1 if kind == "c1" else api.config_c2)(**kw)


def main():
    ob.build()
    for name, (kind, kw, nsteps) in CASES.items():
        _, prm, xv, yv = case(kind, kw)
        n, hist, forces, q = ob.solve(prm, xv.ravel(), yv.ravel(), nsteps)
        assert n == nsteps, (name, n)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), nsteps=nsteps,
                            hist=hist[:, 0], forces=forces[0][:4], q=q)
        print(name, "rsum", hist[0, 0], hist[-1, 0], "cl cd cm", forces[0][:3])


if __name__ == "__main__":
    main()
