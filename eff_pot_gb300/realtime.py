"""Real-time evolution of a droplet with a kicked impurity: energy and norm drift.

The large real-time workload: an N=10000 droplet with a Morse He-X impurity
(De = 10 K, re = 4.5 A, alpha = 1.2/A) on a periodic 256 x 256 x 320 grid at
h = 0.4 A.  The ground state comes from imaginary time (FP32 steps, then FP64
refinement sweeps); the impurity is then given a 50 m/s kick along z and the
complex order parameter evolves in real time (steprk.f90 / steppc.f90 with
timec = i, the impurity a classical particle moved by forceimp): 4
Runge-Kutta-Gill start steps, then predictor-corrector steps at dt = 0.5 fs.
Every `sample` steps the fields are refreshed (poten) and the energy and the
norm are reduced in FP64 (energy.f90).  The same evolution on the plain FP64
path gives the reference the FP32 path's drift is measured against.

    python -m eff_pot_gb300.realtime [--fp32-steps 20000] [--fp64-steps 2000]
"""
import argparse
import json
import time

import numpy as np

from . import _abi
from .config import KTOPS, make_config, morse
from .initial import woods_saxon_psi
from .solver import Solver

DIMS, H, N4, SEED = (256, 256, 320), 0.4, 10000.0, 4
DT_FS = 0.5
MIMPUR = 40.0          # amu
KICK_M_PER_S = 50.0


def config(precision, time_mode, impurity, dims=DIMS, h=H, n4=N4):
    nx, ny, nz = dims
    return make_config(nx=nx, ny=ny, nz=nz, xmax=nx * h / 2, ymax=ny * h / 2, zmax=nz * h / 2,
                       icon=_abi.EP_ICON_PERIODIC, core="OTC", n4=n4, impurity=impurity, time_mode=time_mode,
                       renormalize=1 if time_mode == _abi.EP_IMAGINARY_TIME else 0, precision=precision,
                       mimpur=MIMPUR, fix_lambda=1)


def _attach(s, rimp, vimp=None):
    pot = morse(10.0, 4.5, 1.2)
    s.set_impurity_potentials(pot, pot, pot)
    s.set_impurity(rimp=rimp, vimp=vimp, invar=np.zeros(10, dtype=np.complex128))


def ground_state(steps32=2000, steps64=300, dt=1e-4, dims=DIMS, h=H, n4=N4, seed=SEED):
    """Imaginary-time ground state with the impurity fixed at the centre:
    steps32 FP32 steps, then steps64 FP64 refinement sweeps; psi on the host."""
    s = Solver(config(_abi.EP_FP32, _abi.EP_IMAGINARY_TIME, _abi.EP_IMPURITY_FIXED, dims, h, n4))
    try:
        _attach(s, (0.0, 0.0, 0.0))
        s.start(woods_saxon_psi(*dims, dims[0] * h / 2, dims[1] * h / 2, dims[2] * h / 2, n4, seed=seed))
        for _ in range(3):
            s.steprk(dt)
        s.run(steps32, dt)
        s.set_precision("fp64")
        s.run(steps64, dt)
        return s.psi()
    finally:
        s.close()


def kicked_run(psi, precision, nsteps, sample=100, dims=DIMS, h=H, n4=N4, dt_fs=DT_FS, kick=KICK_M_PER_S):
    """Real-time evolution after the kick; one sample (time in ps, total
    energy, norm, impurity z) before the start steps and every `sample` steps.
    Returns the samples and the wall time of the evolution."""
    dt = dt_fs * 1e-3 / KTOPS                      # fs -> ps -> hbar/k_B units
    v = kick * 1e10 / 1e12 * KTOPS                 # m/s -> A/ps -> A per hbar/k_B
    prec = {"fp32": _abi.EP_FP32, "fp64": _abi.EP_FP64, "dfloat": _abi.EP_DFLOAT}[precision]
    s = Solver(config(prec, _abi.EP_REAL_TIME, _abi.EP_IMPURITY_MOVING, dims, h, n4))
    out = []
    try:
        _attach(s, (0.0, 0.0, 0.0), (0.0, 0.0, v))
        s.start(psi)

        def record(step):
            s.poten()
            e = s.energy()
            out.append({"step": step, "t_ps": step * dt_fs * 1e-3, "etot": e["etot"], "n4": e["n4"],
                        "z": float(s.impurity()["rimp"][2])})

        record(0)
        t0 = time.perf_counter()
        for _ in range(4):
            s.steprk(dt)
        done = 4
        while done < nsteps:
            k = min(sample - done % sample, nsteps - done)
            s.run(k, dt)
            done += k
            if done % sample == 0 or done == nsteps:
                record(done)
        s.synchronize()
        return out, time.perf_counter() - t0
    finally:
        s.close()


def drift_report(fp32, fp64):
    """Drift of the energy and the norm over each run, and the FP32 run's
    distance from the FP64 run at the common sample steps."""
    e0, n0 = fp32[0]["etot"], fp32[0]["n4"]
    rep = {"fp32_energy_drift_K": fp32[-1]["etot"] - e0, "fp32_norm_drift_rel": (fp32[-1]["n4"] - n0) / n0,
           "fp32_max_abs_energy_drift_K": max(abs(r["etot"] - e0) for r in fp32),
           "fp32_max_norm_drift_rel": max(abs(r["n4"] - n0) / n0 for r in fp32)}
    if fp64:
        f64 = {r["step"]: r for r in fp64}
        common = [r for r in fp32 if r["step"] in f64]
        rep.update(
            fp64_energy_drift_K=fp64[-1]["etot"] - fp64[0]["etot"],
            fp64_norm_drift_rel=(fp64[-1]["n4"] - fp64[0]["n4"]) / fp64[0]["n4"],
            common_steps=common[-1]["step"],
            max_abs_energy_diff_fp32_vs_fp64_K=max(abs(r["etot"] - f64[r["step"]]["etot"]) for r in common),
            max_rel_norm_diff_fp32_vs_fp64=max(abs(r["n4"] - f64[r["step"]]["n4"]) / f64[r["step"]]["n4"]
                                               for r in common),
            max_abs_z_diff_fp32_vs_fp64_A=max(abs(r["z"] - f64[r["step"]]["z"]) for r in common))
    return rep


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--fp32-steps", type=int, default=20000)
    ap.add_argument("--fp64-steps", type=int, default=2000)
    ap.add_argument("--dfloat-steps", type=int, default=0, help="also the double-float path")
    ap.add_argument("--ground-fp32", type=int, default=2000)
    ap.add_argument("--ground-fp64", type=int, default=300)
    ap.add_argument("--sample", type=int, default=100)
    a = ap.parse_args(argv)
    from .build import build
    build()
    t0 = time.perf_counter()
    psi = ground_state(a.ground_fp32, a.ground_fp64)
    t_gs = time.perf_counter() - t0
    r32, w32 = kicked_run(psi, "fp32", a.fp32_steps, a.sample)
    r64, w64 = kicked_run(psi, "fp64", a.fp64_steps, a.sample) if a.fp64_steps else ([], 0.0)
    rdd, wdd = kicked_run(psi, "dfloat", a.dfloat_steps, a.sample) if a.dfloat_steps else ([], 0.0)
    print(json.dumps({"workload": "N=10000 droplet + Morse impurity kicked at 50 m/s along z, 256x256x320, "
                                  "h=0.4 A, OTC, real time, dt=0.5 fs, impurity mass 40 u",
                      "ground_state": {"fp32_steps": a.ground_fp32, "fp64_steps": a.ground_fp64, "wall_s": t_gs},
                      "fp32": {"steps": a.fp32_steps, "wall_s": w32, "steps_per_s": a.fp32_steps / w32},
                      "fp64": {"steps": a.fp64_steps, "wall_s": w64,
                               "steps_per_s": a.fp64_steps / w64 if w64 else None},
                      "dfloat": {"steps": a.dfloat_steps, "wall_s": wdd,
                                 "steps_per_s": a.dfloat_steps / wdd if wdd else None},
                      "drift": drift_report(r32, r64),
                      "drift_dfloat": drift_report(rdd, r64) if rdd else None,
                      "samples_fp32": r32, "samples_fp64": r64, "samples_dfloat": rdd}))


if __name__ == "__main__":
    main()
