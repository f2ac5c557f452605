"""Golden vectors of the FP64 oracle for one short evolution.

A 32^3 periodic OTC grid (h = 1 A), an N = 200 Woods-Saxon droplet (seed 3)
with a Morse impurity (De = 10 K, re = 4.5 A, alpha = 1.2 / A, capped at
1000 K) fixed at (0.5, -0.25, 1.0) A: start (potenimp, poten), the first
energy balance, 3 Runge-Kutta-Gill steps and 10 imaginary-time
predictor-corrector steps at dt = 2.5e-4, then poten + energy again.  The
energies, mu, errHe and density checksums are written to
oracle_otc_32.json; the tests check that the oracle still reproduces them
and that the FP64 GPU path matches them.

    python tests/golden/make_oracle_fixture.py
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

N, XMAX, N4, DT, RIMP = 32, 16.0, 200.0, 2.5e-4, (0.5, -0.25, 1.0)
KEYS = ("etot", "etot4", "ekin4", "elj4", "ecor4", "ealphas", "esolid", "eHeX")


def scenario(solver_cls):
    import eff_pot_gb300 as ep
    from eff_pot_gb300 import _abi
    cfg = ep.make_config(nx=N, ny=N, nz=N, xmax=XMAX, ymax=XMAX, zmax=XMAX, icon=_abi.EP_ICON_PERIODIC,
                         core="OTC", n4=N4, impurity=_abi.EP_IMPURITY_FIXED)
    psi = ep.woods_saxon_psi(N, N, N, XMAX, XMAX, XMAX, N4, seed=3)
    with solver_cls(cfg) as s:
        m = ep.morse(10.0, 4.5, 1.2, r_cutoff=0.0, umax=1000.0)
        s.set_impurity_potentials(m, m, ep.null_potential())
        s.set_impurity(rimp=RIMP, invar=np.zeros(10, dtype=np.complex128))
        s.start(psi)
        e0 = s.energy()
        for _ in range(3):
            s.steprk(DT)
        st = s.run(10, DT)
        s.poten()
        e1 = s.energy()
        den = s.field("den")
    x = (np.arange(N) * (2 * XMAX / N) - XMAX)
    return {
        "start": {k: e0[k] for k in KEYS},
        "after": {k: e1[k] for k in KEYS},
        "mu": st["mu"], "errHe": st["errHe"], "norm": st["norm"],
        "den_sum": float(den.sum()), "den_sq": float((den ** 2).sum()),
        "den_xmom": float((den.sum(axis=(1, 2)) * x).sum()),
        "den_samples": [float(den[i, j, k]) for i, j, k in ((16, 16, 16), (8, 20, 12), (0, 0, 0), (31, 5, 17))],
    }


if __name__ == "__main__":
    from oracle import pyoracle
    out = scenario(pyoracle.OracleSolver)
    out["note"] = __doc__.strip().splitlines()[0]
    json.dump(out, open(os.path.join(HERE, "oracle_otc_32.json"), "w"), indent=1)
    print(json.dumps(out)[:300])
