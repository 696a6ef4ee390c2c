"""Generates the full-size golden fixtures of tests/golden/ with the oracle.

The three single-grid configurations of the benchmark at their full sizes:

  c1_full  inviscid NACA 0012, C-mesh 257x65, M 0.80, alpha 1.25, MUSCL +
           Roe, LU-SGS at local CFL 10: the configuration's 2000 iterations
           (Turns_overset.f:360-505 with nsteps = 2000)
  c2_full  RANS-SA NACA 0012, C-mesh 513x129 with 1e-6 wall spacing, M 0.15,
           alpha 10, Re 6e6, MUSCL + Roe, LU-SGS at CFL 50: 2000 iterations
           (the solve needs far more than that to converge in FP64; the
           fixture pins the first 2000)
  c3_full  k-omega SST on a NACA 2412 C-mesh 769x193 with 5e-7 wall spacing,
           M 0.73, alpha 2.8, Re 6.5e6, WENO5 + Roe, ADI (ilhs 2): 400
           iterations at local CFL 0.25 (larger CFLs, and LU-SGS, blow up on
           this mesh in the oracle and on the GPU alike)

Each fixture keeps the per-iteration L2 norm rsum (step.f:86-93), the final
CL, CD, CM and cpower (forces.f), and checksums of the final state q
(jd,kd,nspec,nq): per variable the sum, the sum of squares and a sum with
seeded weights, plus 1024 seeded sample cells with all their variables.  The
full state would be megabytes; a difference in any cell above 1e-12 relative
shows in the weighted sums.

The reference cannot be compiled here (no Fortran compiler), so the
fixtures are the oracle's output, committed so that the GPU path can be
compared with it without running the oracle for minutes.
Run:  python tests/golden/make_full_golden.py   (about four minutes)
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from tests import oracle_binding as ob  # noqa: E402
from turns2d_urans_git_gb300 import api  # noqa: E402

CASES = {
    "c1_full": ("c1", 2000),
    "c2_full": ("c2", 2000),
    "c3_full": ("c3", 400),
}
NSAMPLE = 1024


def case(kind):
    if kind == "c1":
        return api.config_c1()
    if kind == "c2":
        return api.config_c2()
    return api.config_c3(dt=0.25)


def checksums(q, prm):
    """Per-variable sums, sums of squares and seeded-weight sums of q, and
    the values of NSAMPLE seeded cells (all variables)."""
    n = prm.jd * prm.kd * prm.nspec
    qv = q.reshape(prm.nq, n)
    w = np.random.default_rng(2024).uniform(0.5, 1.5, n)
    cells = np.sort(np.random.default_rng(7).choice(n, size=min(NSAMPLE, n), replace=False))
    return dict(qsum=qv.sum(axis=1), qsq=(qv * qv).sum(axis=1), qw=(qv * w).sum(axis=1), cells=cells,
                qcells=qv[:, cells])


def main(names=None):
    ob.build()
    for name, (kind, nsteps) in CASES.items():
        if names and name not in names:
            continue
        _, prm, xv, yv = case(kind)
        t0 = time.time()
        n, hist, forces, q = ob.solve(prm, xv.ravel(), yv.ravel(), nsteps)
        assert n == nsteps, (name, n)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), nsteps=nsteps, hist=hist[:, 0], forces=forces[0][:4],
                            **checksums(q, prm))
        print(name, "%.0f s" % (time.time() - t0), "rsum", hist[0, 0], hist[-1, 0], "cl cd cm", forces[0][:3],
              flush=True)


if __name__ == "__main__":
    main(sys.argv[1:])
