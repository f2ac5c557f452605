"""A short run of one instance of the benchmark workload, for profilers.

One N=1000 droplet with a Morse impurity at the centre on a periodic 128^3
grid (h = 0.4 A, OTC, imaginary time, dt = 1e-4): start-up, three
Runge-Kutta-Gill steps, then --steps predictor-corrector steps.  It spawns
no other process and holds about 0.4 GB (FP32) or 0.8 GB (FP64) on the GPU.

    python -m eff_pot_gb300.profile_case --precision fp32 --steps 6
"""
import argparse

import numpy as np

from . import _abi
from .build import build
from .config import make_config, morse
from .initial import woods_saxon_psi
from .solver import Solver


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64", "dfloat"])
    ap.add_argument("--steps", type=int, default=6)
    ap.add_argument("--n", type=int, default=128)
    a = ap.parse_args(argv)
    build()
    n, xmax = a.n, 0.2 * a.n
    cfg = make_config(nx=n, ny=n, nz=n, xmax=xmax, ymax=xmax, zmax=xmax, icon=_abi.EP_ICON_PERIODIC,
                      core="OTC", n4=1000.0, impurity=_abi.EP_IMPURITY_FIXED,
                      precision={"fp32": _abi.EP_FP32, "fp64": _abi.EP_FP64, "dfloat": _abi.EP_DFLOAT}[a.precision])
    with Solver(cfg) as s:
        pot = morse(10.0, 4.5, 1.2)
        s.set_impurity_potentials(pot, pot, pot)
        s.set_impurity(rimp=(0.0, 0.0, 0.0), invar=np.zeros(10, dtype=np.complex128))
        s.start(woods_saxon_psi(n, n, n, xmax, xmax, xmax, 1000.0, seed=1))
        for _ in range(3):
            s.steprk(1e-4)
        st = s.run(a.steps, 1e-4)
        print(f"profile_case {a.precision} {n}^3: {a.steps} steps, mu = {st['mu']:.8f}, "
              f"{s.kernel_launches()} kernel launches")


if __name__ == "__main__":
    main()
