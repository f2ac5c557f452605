"""Benchmark of the helium order-parameter time evolution on GB300.

Workload (one "step" = one predictor-corrector step, steppc): a single
N=1000 helium droplet with a Morse He-X impurity fixed at the centre on a
periodic 128^3 grid, h = 0.4 A, Orsay-Trento functional with the alpha_s
term ('OTC'), imaginary time, dt = 1e-4 1/K, renormalised to N after each
step; seeded Woods-Saxon start (seed 1).  The working set (~0.8 GB in FP64)
is far larger than L2, so no flush is needed between steps.

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                [--precision fp64|fp32]
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_GRID, XMAX, N4, DT, SEED = 128, 25.6, 1000.0, 1e-4, 1
METRIC = "time-steps/s at 128^3 (OTC droplet N=1000 + Morse impurity, imaginary-time steppc)"
UNIT = "steps/s"


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def dist_init(world):
    if world <= 1:
        return None
    import torch.distributed as dist
    dist.init_process_group("gloo")
    return dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, v):
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = os.path.join(ROOT, "gpurun_out", f"clocks_bench_{device}.csv")

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            time.sleep(0.3)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        try:
            rows = [l.split(",") for l in open(self.path).read().splitlines() if l.strip()]
        except Exception:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
                for n, v in zip(names, r[5:9]):
                    if v.strip().lower() == "active":
                        reasons.add(n)
            except Exception:
                continue
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def workload_config(precision, device=0):
    import eff_pot_gb300 as ep
    from eff_pot_gb300 import _abi
    return ep.make_config(nx=N_GRID, ny=N_GRID, nz=N_GRID, xmax=XMAX, ymax=XMAX, zmax=XMAX,
                          icon=_abi.EP_ICON_PERIODIC, core="OTC", n4=N4, impurity=_abi.EP_IMPURITY_FIXED,
                          time_mode=_abi.EP_IMAGINARY_TIME, renormalize=1,
                          precision=_abi.EP_FP32 if precision == "fp32" else _abi.EP_FP64, device=device)


def setup_solver(solver_cls, cfg, psi):
    import numpy as np
    import eff_pot_gb300 as ep
    s = solver_cls(cfg)
    pot = ep.morse(10.0, 4.5, 1.2)
    s.set_impurity_potentials(pot, pot, pot)
    s.set_impurity(rimp=(0.0, 0.0, 0.0), invar=np.zeros(10, dtype=np.complex128))
    s.start(psi)
    for _ in range(3):
        s.steprk(DT)
    return s


def cpu_sample(psi, steps=2):
    """Oracle (FP64, OpenMP, all host threads) on the same workload."""
    from oracle import pyoracle
    threads = os.cpu_count() or 1
    pyoracle.set_threads(threads)
    cfg = workload_config("fp64")
    t0 = time.perf_counter()
    s = setup_solver(pyoracle.OracleSolver, cfg, psi)
    t_setup = time.perf_counter() - t0
    s.steppc(DT)
    t0 = time.perf_counter()
    for _ in range(steps):
        s.steppc(DT, wait=False)
        s.renormalize()
    dt = time.perf_counter() - t0
    s.close()
    return {"value": steps / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{steps} steppc steps of the 128^3 workload after start-up ({t_setup:.1f} s), "
                      f"C++ FP64 oracle with {threads} OpenMP threads"}


def run_reference(args):
    rank, world, local = dist_env()
    if rank != 0:
        return 0
    import eff_pot_gb300 as ep
    psi = ep.woods_saxon_psi(N_GRID, N_GRID, N_GRID, XMAX, XMAX, XMAX, N4, seed=SEED)
    from oracle import pyoracle
    threads = os.cpu_count() or 1
    pyoracle.set_threads(threads)
    cfg = workload_config("fp64")
    s = setup_solver(pyoracle.OracleSolver, cfg, psi)
    for _ in range(args.warmup):
        s.steppc(DT)
        s.renormalize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        s.steppc(DT, wait=False)
        s.renormalize()
    el = time.perf_counter() - t0
    s.close()
    v = args.steps / el
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded Woods-Saxon droplet)",
            "config": {"workload": "single droplet N=1000 + Morse impurity, 128^3, h=0.4 A, OTC",
                       "grid": [N_GRID] * 3, "parallelism": "host OpenMP"},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{args.steps} steppc steps after {args.warmup} warm-up steps, "
                                       f"C++ FP64 oracle (the reference Fortran does not build here)"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def run_ours(args):
    rank, world, local = dist_env()
    dist = dist_init(world)
    import numpy as np
    import eff_pot_gb300 as ep
    from eff_pot_gb300.build import build
    from eff_pot_gb300.roofline import step_bytes
    if rank == 0 or world > 1:
        build()
    barrier(dist)
    psi = ep.woods_saxon_psi(N_GRID, N_GRID, N_GRID, XMAX, XMAX, XMAX, N4, seed=SEED)
    cfg = workload_config(args.precision, device=local)
    s = setup_solver(ep.Solver, cfg, psi)
    s.run(args.warmup, DT)
    s.synchronize()
    barrier(dist)
    l0 = s.kernel_launches()
    with ClockSampler(local) as clk:
        s.profile(True)
        s.synchronize()
        s._f["event_record"](s._h, 0)
        s.run(args.steps, DT, wait=False)
        s._f["event_record"](s._h, 1)
        import ctypes as C
        ms = C.c_double()
        s._f["event_elapsed"](s._h, 0, 1, C.byref(ms))
        s.synchronize()
    launches = s.kernel_launches() - l0
    prof = s.profile_read()
    s.profile(False)
    el_ms = max_over_ranks(dist, ms.value)
    value = world * args.steps / (el_ms / 1e3)
    # end-to-end through the C ABI with host buffers: upload, start-up,
    # K steps each returning its errors to the host, download
    host = np.asfortranarray(psi)
    out = np.empty_like(host)
    barrier(dist)
    t0 = time.perf_counter()
    s.upload_psi(host)
    s.potenimp()
    s.poten()
    for _ in range(3):
        s.steprk(DT)
    for _ in range(args.steps):
        s.steppc(DT)
        if cfg.renormalize:
            s._f["renormalize"](s._h, None)
    out[...] = s.psi()
    e2e_s = max_over_ranks(dist, time.perf_counter() - t0)
    e2e = world * args.steps / e2e_s
    st = s.run(1, DT)
    s.close()
    if rank != 0:
        return 0
    sz = 4 if args.precision == "fp32" else 8
    bytes_cls = step_bytes(N_GRID, N_GRID, N_GRID, otc=True, grad=True, s=sz, renorm=True)
    per_step_ms = {k: v[0] / args.steps for k, v in prof.items()}
    dom = max((k for k in per_step_ms if k in bytes_cls), key=lambda k: per_step_ms[k])
    launches_dom = prof[dom][1]
    avg_launch_ms = prof[dom][0] / launches_dom
    bytes_launch = bytes_cls[dom] / (launches_dom / args.steps)
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    peak = peaks.get("hbm_gbs", 6800.0)
    achieved = bytes_launch / (avg_launch_ms / 1e3) / 1e9
    traffic = None
    try:
        tr = json.load(open(os.path.join(ROOT, "profiles", "ncu_traffic.json")))
        traffic = tr.get(args.precision, {}).get(dom)
    except Exception:
        pass
    total_bytes = sum(bytes_cls.values())
    cpu = None
    if not args.no_cpu:
        try:
            cpu = cpu_sample(psi, steps=2)
        except Exception as exc:
            cpu = {"value": None, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                   "sample": f"failed: {exc}"}
    h2d = 16 * N_GRID ** 3 / args.steps
    d2h = (16 * N_GRID ** 3 + 32 * args.steps) / args.steps
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": el_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f32" if args.precision == "fp32" else "f64",
        "data": "synthetic (seeded Woods-Saxon droplet, seed 1)",
        "config": {"workload": "single droplet N=1000 + Morse impurity (De=10 K, re=4.5 A, a=1.2/A) "
                               "fixed at the centre, 128^3, h=0.4 A, OTC, imaginary time",
                   "grid": [N_GRID] * 3, "precision": args.precision, "dt": DT,
                   "parallelism": "replicas" if world > 1 else "single GPU",
                   "l2": "inputs larger than L2 (working set %.2f GB)" % (total_bytes / 1e9)},
        "hbm_gbs_step": total_bytes / (el_ms / args.steps / 1e3) / 1e9,
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs" if "hbm_gbs" in peaks else "fallback"},
        "kernels_ms_per_step": {k: round(v, 4) for k, v in sorted(per_step_ms.items(), key=lambda t: -t[1])},
        "gpu_launches": launches,
        "clocks": clk.summary(),
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "cpu_baseline": cpu,
        "mu": st["mu"],
    }
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="fp64", choices=["fp64", "fp32"])
    ap.add_argument("--no-cpu", action="store_true")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
