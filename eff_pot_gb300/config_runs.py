"""Short timed runs of the five benchmark configurations, for the results table.

Each configuration is run for a bounded number of steps (the full step counts of
the configurations are minutes to hours of work): device-timed steps/s of the
plain FP64 path and of the FP32 path (batched where the configuration is a
batch), the HBM fraction of the algorithmic step bytes, and the CPU oracle on a
bounded sample with all host threads.  Configuration 0 also checks the FP64 GPU
path against the oracle on its own geometry.

    python -m eff_pot_gb300.config_runs [--only 0,1,3,4] [--no-cpu]

Prints one JSON object per configuration.
"""
import argparse
import json
import os
import time

import numpy as np

from . import _abi
from .build import build
from .config import make_config, morse, null_potential
from .initial import woods_saxon_psi
from .roofline import step_bytes
from .solver import Batch, Solver

HBM_GBS = 6796.2
DT = 1e-4


def _peak():
    try:
        here = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
        return float(json.load(open(os.path.join(here, "MEASURED_PEAKS.json")))["hbm_gbs"])
    except Exception:
        return HBM_GBS


def _cfg(n, h, n4, impurity, precision, time_mode=_abi.EP_IMAGINARY_TIME, dims=None):
    nx, ny, nz = dims or (n, n, n)
    return make_config(nx=nx, ny=ny, nz=nz, xmax=nx * h / 2, ymax=ny * h / 2, zmax=nz * h / 2,
                       icon=_abi.EP_ICON_PERIODIC, core="OTC", n4=n4, impurity=impurity,
                       time_mode=time_mode, renormalize=1 if time_mode == _abi.EP_IMAGINARY_TIME else 0,
                       precision=precision)


def _prepare(s, psi, rimp, pot=None, vimp=None):
    p = pot if pot is not None else null_potential()
    s.set_impurity_potentials(p, p, p)
    s.set_impurity(rimp=rimp, vimp=vimp, invar=np.zeros(10, dtype=np.complex128))
    s.start(psi)


def _timed(obj, steps, dt):
    """Device time of obj.run(steps) between two events on obj's stream."""
    f, h = obj._f, obj._h
    batch = isinstance(obj, Batch)
    rec = f["batch_event_record"] if batch else f["event_record"]
    ela = f["batch_event_elapsed"] if batch else f["event_elapsed"]
    import ctypes as C
    rec(h, 0)
    obj.run(steps, dt, wait=False)
    rec(h, 1)
    ms = C.c_double()
    ela(h, 0, 1, C.byref(ms))
    return ms.value


def _single(cfg, psi, rimp, pot, steps, warmup, dt=DT, rk=3, vimp=None):
    with Solver(cfg) as s:
        _prepare(s, psi, rimp, pot, vimp)
        s.autotune()
        for _ in range(rk):
            s.steprk(dt)
        s.run(warmup, dt)
        s.synchronize()
        ms = _timed(s, steps, dt)
    return steps / (ms / 1e3)


def _cpu(cfg, psi, rimp, pot, steps, dt=DT, rk=3, vimp=None):
    from oracle import pyoracle  # the CPU baseline is the oracle
    threads = os.cpu_count() or 1
    pyoracle.set_threads(threads)
    s = pyoracle.OracleSolver(cfg)
    _prepare(s, psi, rimp, pot, vimp)
    for _ in range(rk):
        s.steprk(dt)
    s.steppc(dt)
    t0 = time.perf_counter()
    for _ in range(steps):
        s.steppc(dt, wait=False)
        if cfg.time_mode == _abi.EP_IMAGINARY_TIME:
            s.renormalize()
    el = time.perf_counter() - t0
    s.close()
    return {"steps_per_s": steps / el, "cores": threads, "sample_steps": steps}


def _frac(cfg, steps_per_s, s):
    b = sum(step_bytes(cfg.nx, cfg.ny, cfg.nz, otc=True, grad=True, s=s, renorm=False).values())
    return b * steps_per_s / 1e9 / _peak()


def config0(args):
    """Pure N=500 droplet, 64^3, h = 0.8 A, FP64 (CPU-runnable)."""
    n, h, n4 = 64, 0.8, 500.0
    c64 = _cfg(n, h, n4, _abi.EP_IMPURITY_NONE, _abi.EP_FP64)
    c32 = _cfg(n, h, n4, _abi.EP_IMPURITY_NONE, _abi.EP_FP32)
    psi = woods_saxon_psi(n, n, n, c64.xmax, c64.ymax, c64.zmax, n4, seed=0)
    z = (0.0, 0.0, 0.0)
    out = {"config": 0, "workload": "pure N=500 droplet, 64^3, h=0.8 A, OTC, imaginary time, dt=1e-4"}
    out["gpu_fp64_steps_per_s"] = _single(c64, psi, z, None, 200, 5)
    out["gpu_fp32_steps_per_s"] = _single(c32, psi, z, None, 400, 5)
    out["hbm_frac_fp64"] = _frac(c64, out["gpu_fp64_steps_per_s"], 8)
    out["hbm_frac_fp32"] = _frac(c32, out["gpu_fp32_steps_per_s"], 4)
    if not args.no_cpu:
        out["cpu"] = _cpu(c64, psi, z, None, 40)
        # parity on this geometry: 3 RK-Gill + 50 PC steps, FP64 GPU vs oracle
        from oracle import pyoracle
        with Solver(c64) as s:
            _prepare(s, psi, z)
            for _ in range(3):
                s.steprk(DT)
            s.run(50, DT)
            s.poten()
            eg, dg = s.energy(), s.field("den")
        o = pyoracle.OracleSolver(c64)
        _prepare(o, psi, z)
        for _ in range(3):
            o.steprk(DT)
        for _ in range(50):
            o.steppc(DT, wait=False)
            o.renormalize()
        o.poten()
        eo, do = o.energy(), o.field("den")
        o.close()
        out["parity_vs_oracle"] = {"steps": "3 RK-Gill + 50 PC", "etot_rel": abs(eg["etot"] - eo["etot"]) / abs(eo["etot"]),
                                   "den_maxabs": float(np.max(np.abs(dg - do)))}
    return out


def config1(args):
    """N=1000 droplet + Morse impurity at the centre, 128^3, h = 0.4 A."""
    n, h, n4 = 128, 0.4, 1000.0
    c64 = _cfg(n, h, n4, _abi.EP_IMPURITY_FIXED, _abi.EP_FP64)
    c32 = _cfg(n, h, n4, _abi.EP_IMPURITY_FIXED, _abi.EP_FP32)
    psi = woods_saxon_psi(n, n, n, c64.xmax, c64.ymax, c64.zmax, n4, seed=1)
    z, pot = (0.0, 0.0, 0.0), morse(10.0, 4.5, 1.2)
    out = {"config": 1, "workload": "N=1000 droplet + Morse impurity at the centre, 128^3, h=0.4 A, OTC"}
    out["gpu_fp64_steps_per_s"] = _single(c64, psi, z, pot, 100, 5)
    out["gpu_fp32_steps_per_s"] = _single(c32, psi, z, pot, 400, 5)
    r = 200.0 / 5000.0
    out["gpu_fp32_refine_steps_per_s"] = 1.0 / ((1 - r) / out["gpu_fp32_steps_per_s"] + r / out["gpu_fp64_steps_per_s"])
    out["hbm_frac_fp64"] = _frac(c64, out["gpu_fp64_steps_per_s"], 8)
    out["hbm_frac_fp32"] = _frac(c32, out["gpu_fp32_steps_per_s"], 4)
    if not args.no_cpu:
        out["cpu"] = _cpu(c64, psi, z, pot, 20)
    return out


def config3(args):
    """Uneven batch: 64 droplets, N and grid drawn by seed 2, half with the impurity."""
    rng = np.random.default_rng(2)
    ns = rng.choice([300, 1000, 2000, 5000], size=64)
    grid_of = {300: 96, 1000: 128, 2000: 160, 5000: 192}
    cfgs, psis, rimps, has = [], [], [], []
    for i, nn in enumerate(ns):
        g = grid_of[int(nn)]
        imp = i % 2 == 0
        c = _cfg(g, 0.4, float(nn), _abi.EP_IMPURITY_FIXED if imp else _abi.EP_IMPURITY_NONE, _abi.EP_FP32)
        R = 2.22 * float(nn) ** (1.0 / 3.0)
        rr = rng.uniform(0.0, R) if imp else 0.0
        cfgs.append(c)
        psis.append(woods_saxon_psi(g, g, g, c.xmax, c.ymax, c.zmax, float(nn), seed=100 + i))
        rimps.append((0.0, 0.0, rr))
        has.append(imp)
    steps, warm = 20, 3
    k64 = 1
    with Batch(cfgs) as b:
        for s, psi, r, imp in zip(b, psis, rimps, has):
            _prepare(s, psi, r, morse(10.0, 4.5, 1.2) if imp else None)
        b.autotune()
        for _ in range(3):
            b.steprk(DT)
        b.run(warm, DT)
        b.set_precision("fp64")
        b.run(1, DT)
        b.set_precision("fp32")
        b.synchronize()
        ms32 = _timed(b, steps - k64, DT)
        b.set_precision("fp64")
        ms64 = _timed(b, k64, DT)
    pts = sum(c.nx * c.ny * c.nz for c in cfgs)
    total_ms = ms32 + ms64
    out = {"config": 3, "workload": "64 droplets, N in {300,1000,2000,5000} (seed 2), grids 96..192^3 at h=0.4 A, "
                                     "half with the Morse impurity",
           "instances": 64, "grid_points_total": pts,
           "batch_fp32_instance_steps_per_s": 64 * (steps - k64) / (ms32 / 1e3),
           "batch_fp64_instance_steps_per_s": 64 * k64 / (ms64 / 1e3),
           "batch_fp32_refine_instance_steps_per_s": 64 * steps / (total_ms / 1e3),
           "refine_steps_in_sample": f"{steps - k64} FP32 + {k64} FP64"}
    b32 = sum(sum(step_bytes(c.nx, c.ny, c.nz, s=4, renorm=False).values()) for c in cfgs)
    out["hbm_frac_fp32"] = b32 * (steps - k64) / (ms32 / 1e3) / 1e9 / _peak()
    return out


def config4(args):
    """Large real-time run: N=10000 + moving Morse impurity, 256x256x320, h = 0.4 A."""
    dims, h, n4 = (256, 256, 320), 0.4, 10000.0
    c32 = _cfg(0, h, n4, _abi.EP_IMPURITY_MOVING, _abi.EP_FP32, _abi.EP_REAL_TIME, dims)
    c64 = _cfg(0, h, n4, _abi.EP_IMPURITY_MOVING, _abi.EP_FP64, _abi.EP_REAL_TIME, dims)
    c32.mimpur = c64.mimpur = 40.0
    c32.fix_lambda = c64.fix_lambda = 1
    psi = woods_saxon_psi(*dims, c32.xmax, c32.ymax, c32.zmax, n4, seed=4)
    dt = 0.5e-15 / 7.6382e-12  # 0.5 fs in units of hbar / k_B
    v = (0.0, 0.0, 50.0 * 1e10 / 1e12 * 7.6382)  # 50 m/s in A per (hbar / k_B)
    pot = morse(10.0, 4.5, 1.2)
    out = {"config": 4, "workload": "N=10000 + Morse impurity kicked at 50 m/s, 256x256x320, h=0.4 A, real time, "
                                     "dt=0.5 fs", "dt_reduced": dt}
    out["gpu_fp32_steps_per_s"] = _single(c32, psi, (0.0, 0.0, 0.0), pot, 30, 3, dt=dt, rk=4, vimp=v)
    out["gpu_fp64_steps_per_s"] = _single(c64, psi, (0.0, 0.0, 0.0), pot, 10, 2, dt=dt, rk=4, vimp=v)
    out["hbm_frac_fp32"] = _frac(c32, out["gpu_fp32_steps_per_s"], 4)
    out["hbm_frac_fp64"] = _frac(c64, out["gpu_fp64_steps_per_s"], 8)
    if not args.no_cpu:
        out["cpu"] = _cpu(c64, psi, (0.0, 0.0, 0.0), pot, 3, dt=dt, rk=4, vimp=v)
    return out


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--only", default="0,1,3,4")
    ap.add_argument("--no-cpu", action="store_true")
    a = ap.parse_args(argv)
    build()
    runs = {"0": config0, "1": config1, "3": config3, "4": config4}
    for k in a.only.split(","):
        t0 = time.perf_counter()
        r = runs[k.strip()](a)
        r["wall_s"] = time.perf_counter() - t0
        print(json.dumps(r), flush=True)


if __name__ == "__main__":
    main()
