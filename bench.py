"""Benchmark of the helium order-parameter time evolution on one GB300.

Headline workload (the effective-potential scan): 32 instances, each an
N=1000 helium droplet on a periodic 128^3 grid (h = 0.4 A, Orsay-Trento with
the alpha_s term, 'OTC') with a Morse He-X impurity (De=10 K, re=4.5 A,
alpha=1.2/A) fixed at z = 0, 1.25, ..., 38.75 A on the x=y=0 axis, advanced
together in imaginary time (dt = 1e-4 1/K, renormalised after every step):
FP32 bulk steps then FP64-class refinement sweeps in the scan's 4000:200
ratio -- by default in double-float arithmetic (pairs of FP32 values, the
engine that matches the FP64 oracle to the FP64 gates on the FP32 pipes;
--refine fp64 for native FP64), with the other arithmetic timed beside it.
A "step" is one steppc of every instance; value = instance-steps/s.
Beside it: the plain FP64, double-float and FP32 paths on one instance (the
configuration of a single droplet + impurity at 128^3), the per-kernel
roofline of the FP32 instance, the end-to-end rate through the C ABI with
host buffers, and the C++ FP64 oracle on the host cores.  Inputs are seeded
Woods-Saxon droplets; every working set is far larger than L2.

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                [--batch B] [--no-cpu] [--refine dfloat|fp64] [--step-graphs 0|1|2]
                [--workload scan|pure64|impurity128|uneven|realtime]
"""
import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import tempfile
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_GRID, XMAX, N4, DT, SEED = 128, 25.6, 1000.0, 1e-4, 1
REFINE_RATIO = 200.0 / 4200.0
METRIC = ("time-steps/s at 128^3: batched (32 droplets + Morse impurity scan) FP32 + FP64-class refine, "
          "instance-steps/s")
UNIT = "instance-steps/s"


def dist_env():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


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
    """nvidia-smi clocks and throttle reasons sampled during a timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device, tag, directory=None):
        self.device = device
        self.proc = None
        self.path = os.path.join(directory or tempfile.gettempdir(), f"clocks_{tag}_{device}.csv")

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
            time.sleep(0.25)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            time.sleep(0.25)
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
        sm, mx, pw, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
                pw.append(float(r[3]))
                for n, v in zip(names, r[5:9]):
                    if v.strip().lower() == "active":
                        reasons.add(n)
            except Exception:
                continue
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "power_w_max": max(pw), "samples": len(sm)}


def make_cfg(precision, z=0.0, device=0):
    import eff_pot_gb300 as ep
    from eff_pot_gb300 import _abi
    return ep.make_config(nx=N_GRID, ny=N_GRID, nz=N_GRID, xmax=XMAX, ymax=XMAX, zmax=XMAX,
                          icon=_abi.EP_ICON_PERIODIC, core="OTC", n4=N4, impurity=_abi.EP_IMPURITY_FIXED,
                          time_mode=_abi.EP_IMAGINARY_TIME, renormalize=1,
                          precision={"fp32": _abi.EP_FP32, "fp64": _abi.EP_FP64, "dfloat": _abi.EP_DFLOAT}[precision],
                          device=device)


def prepare(s, psi, z):
    import numpy as np
    import eff_pot_gb300 as ep
    pot = ep.morse(10.0, 4.5, 1.2)
    s.set_impurity_potentials(pot, pot, pot)
    s.set_impurity(rimp=(0.0, 0.0, z), invar=np.zeros(10, dtype=np.complex128))
    s.start(psi)


def time_single(precision, psi, steps, warmup, device, profile=False):
    """One instance: device-timed steppc steps (replayed from the step graph),
    then, if asked, the same number of steps again with per-kernel events
    (direct launches) for the per-kernel table."""
    import eff_pot_gb300 as ep
    s = ep.Solver(make_cfg(precision, device=device))
    prepare(s, psi, 0.0)
    tuned = s.autotune()
    for _ in range(3):
        s.steprk(DT)
    s.run(warmup, DT)
    s.synchronize()
    l0 = s.kernel_launches()
    s._f["event_record"](s._h, 0)
    s.run(steps, DT, wait=False)
    s._f["event_record"](s._h, 1)
    ms = C.c_double()
    s._f["event_elapsed"](s._h, 0, 1, C.byref(ms))
    launches = s.kernel_launches() - l0
    prof = {}
    if profile:
        s.profile(True)
        s.run(steps, DT, wait=False)
        prof = s.profile_read()
    s.close()
    return ms.value, launches, prof, tuned


def run_reference(args):
    rank, world, local = dist_env()
    if rank != 0:
        return 0
    import eff_pot_gb300 as ep
    from oracle import pyoracle
    threads = os.cpu_count() or 1
    pyoracle.set_threads(threads)
    psi = ep.woods_saxon_psi(N_GRID, N_GRID, N_GRID, XMAX, XMAX, XMAX, N4, seed=SEED)
    s = pyoracle.OracleSolver(make_cfg("fp64"))
    prepare(s, psi, 0.0)
    for _ in range(3):
        s.steprk(DT)
    for _ in range(args.warmup):
        s.steppc(DT, wait=False)
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
            "data": "synthetic (seeded Woods-Saxon droplets)",
            "config": {"workload": "droplet N=1000 + Morse impurity, 128^3, h=0.4 A, OTC, imaginary time "
                                   "(one instance of the scan per step)",
                       "grid": [N_GRID] * 3, "parallelism": "host OpenMP"},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{args.steps} steppc steps of one scan instance after {args.warmup} "
                                       "warm-up steps; C++ FP64 oracle (the reference Fortran needs ifort/"
                                       "gfortran + FFTW/MKL, absent here)"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def cpu_sample(psi, steps=2):
    from oracle import pyoracle
    threads = os.cpu_count() or 1
    pyoracle.set_threads(threads)
    t0 = time.perf_counter()
    s = pyoracle.OracleSolver(make_cfg("fp64"))
    prepare(s, psi, 0.0)
    for _ in range(3):
        s.steprk(DT)
    s.steppc(DT)
    t_setup = time.perf_counter() - t0
    t0 = time.perf_counter()
    for _ in range(steps):
        s.steppc(DT, wait=False)
        s.renormalize()
    el = time.perf_counter() - t0
    s.close()
    return {"value": steps / el, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{steps} steppc steps of one 128^3 instance after start-up ({t_setup:.0f} s); "
                      f"C++ FP64 oracle, {threads} OpenMP threads"}


def fp64_flop_roofline(steps_per_s):
    """The FP64 path is bound by the FP64 pipe, not HBM: algorithmic FLOP/s of
    the plain FP64 single instance against the measured FMA peak."""
    from eff_pot_gb300.roofline import step_flops
    achieved = step_flops(N_GRID, N_GRID, N_GRID, otc=True) * steps_per_s / 1e12
    peak = 1.25
    return {"bound": "fp64 alu", "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
            "peak_source": "nominal GB300 FP64 rate (no measured FP64 peak in MEASURED_PEAKS.json)"}


def run_ours(args):
    rank, world, local = dist_env()
    dist = dist_init(world)
    import numpy as np
    import eff_pot_gb300 as ep
    from eff_pot_gb300.build import build
    from eff_pot_gb300.roofline import step_bytes
    build()
    barrier(dist)
    psi = ep.woods_saxon_psi(N_GRID, N_GRID, N_GRID, XMAX, XMAX, XMAX, N4, seed=SEED)
    K = args.steps
    k64 = max(1, int(round(K * REFINE_RATIO)))
    k32 = K - k64

    # --- single instance: plain FP64 path, FP32 path with per-kernel events
    ms64, _, prof64, tuned64 = time_single("fp64", psi, K, args.warmup, local, profile=True)
    ms32, l32, prof, tuned32 = time_single("fp32", psi, K, args.warmup, local, profile=True)
    msdd, _, profdd, tuneddd = time_single("dfloat", psi, K, args.warmup, local, profile=True)

    # --- the batched scan, FP32 then FP64 refinement
    # N ranks scan the same z range N times more finely: rank r takes every
    # N-th point of the 32N-point scan (its own batch of 32; no data-path
    # collective between ranks)
    zs = [1.25 * (rank + world * k) / world for k in range(args.batch)]
    cfgs = [make_cfg("fp32", z, device=local) for z in zs]
    b = ep.Batch(cfgs)
    b.step_graphs(args.step_graphs)
    for s, z in zip(b, zs):
        prepare(s, psi, z)
    b.autotune()
    b.steprk(DT)
    b.steprk(DT)
    b.steprk(DT)
    # warm-up, including one precision round trip (allocates the FP64 buffers,
    # whose launch shapes are tuned too)
    b.run(args.warmup, DT)
    b.set_precision(args.refine)
    b.autotune()
    b.run(1, DT)
    b.set_precision("fp32")
    b.run(1, DT)
    b.synchronize()
    barrier(dist)
    l0 = b.kernel_launches()
    with ClockSampler(local, "batch", args.clocks_dir) as clk:
        b.event_record(0)
        b.run(k32, DT, wait=False)
        b.set_precision(args.refine)
        b.run(k64, DT, wait=False)
        b.event_record(1)
        ms_b = b.event_elapsed(0, 1)
    launches = b.kernel_launches() - l0
    stats = b.run(1, DT)
    # the same K steps with the other refinement arithmetic, for comparison
    other = "fp64" if args.refine == "dfloat" else "dfloat"
    b.set_precision(other)
    b.autotune()
    b.run(1, DT)
    b.set_precision("fp32")
    b.run(1, DT)
    b.synchronize()
    b.event_record(2)
    b.run(k32, DT, wait=False)
    b.set_precision(other)
    b.run(k64, DT, wait=False)
    b.event_record(3)
    ms_other = max_over_ranks(dist, b.event_elapsed(2, 3))
    b.close()
    ms_b = max_over_ranks(dist, ms_b)
    value = world * args.batch * K / (ms_b / 1e3)

    # --- end to end through the C ABI with host buffers (pinned where torch
    # can provide it): upload every psi, start-up, the FP32+refine steps,
    # energies and psi back to the host.
    try:
        import torch
        host = torch.empty((N_GRID ** 3, 2), dtype=torch.float64, pin_memory=True).numpy()
        pinned = True
    except Exception:
        host = np.empty((N_GRID ** 3, 2))
        pinned = False
    host[...] = np.asfortranarray(psi).ravel(order="F").view(np.float64).reshape(-1, 2)
    psi_host = host.view(np.complex128).reshape((N_GRID,) * 3, order="F")
    b = ep.Batch(cfgs)
    b.step_graphs(args.step_graphs)
    for s, z in zip(b, zs):
        pot = ep.morse(10.0, 4.5, 1.2)
        s.set_impurity_potentials(pot, pot, pot)
        s.set_impurity(rimp=(0.0, 0.0, z), invar=np.zeros(10, dtype=np.complex128))
    b.set_precision(args.refine)
    b.set_precision("fp32")
    b.synchronize()
    barrier(dist)
    t0 = time.perf_counter()
    for s in b:
        s.upload_psi(psi_host)
        s.potenimp()
        s.poten()
    b.steprk(DT)
    b.steprk(DT)
    b.steprk(DT)
    b.run(k32, DT, wait=False)
    b.set_precision(args.refine)
    b.run(k64, DT)
    # the final fields of every instance first (their kernels overlap on the
    # instance streams), then energies and psi into page-locked memory
    for s in b:
        s.poten()
    energies = [s.energy()["etot"] for s in b]
    for s in b:
        s.psi(out=psi_host)
    e2e_s = max_over_ranks(dist, time.perf_counter() - t0)
    b.close()
    e2e = world * args.batch * K / e2e_s
    e2e_fixed = max(0.0, e2e_s - ms_b / 1e3)
    if rank != 0:
        return 0

    bytes32 = step_bytes(N_GRID, N_GRID, N_GRID, otc=True, grad=True, s=4, renorm=False)
    per_step = {k: v[0] / K for k, v in prof.items()}
    dom = max((k for k in per_step if k in bytes32), key=lambda k: per_step[k])
    n_dom = prof[dom][1]
    achieved = (bytes32[dom] / (n_dom / K)) / (prof[dom][0] / n_dom / 1e3) / 1e9
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    peak = peaks.get("hbm_gbs", 6800.0)
    traffic = None
    try:
        traffic = json.load(open(os.path.join(ROOT, "profiles", "ncu_traffic.json")))["fp32"].get(dom)
    except Exception:
        pass
    b32 = sum(bytes32.values())
    b64 = sum(step_bytes(N_GRID, N_GRID, N_GRID, otc=True, grad=True, s=8, renorm=False).values())
    batch_bytes = args.batch * (k32 * b32 + k64 * b64)
    cpu = None
    if not args.no_cpu:
        try:
            cpu = cpu_sample(psi, steps=40)
        except Exception as exc:
            cpu = {"value": None, "unit": UNIT, "cores": os.cpu_count(), "kind": "port", "sample": f"failed: {exc}"}
    n3 = N_GRID ** 3
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K, "warmup": args.warmup,
        "ms_per_step": ms_b / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64" if args.refine == "fp64" else "f32+dfloat", "data": "synthetic (seeded Woods-Saxon droplets, seed 1)",
        "config": {"workload": f"{args.batch} droplets N=1000 + Morse impurity at z=0..{zs[-1]} A, 128^3, h=0.4 A, "
                               "OTC, imaginary time, dt=1e-4",
                   "instances": args.batch, "grid": [N_GRID] * 3, "fp32_steps": k32, "fp64_refine_steps": k64,
                   "parallelism": "one stream per instance" + (f", {world} GPUs x {args.batch}" if world > 1 else ""),
                   "step_graphs": args.step_graphs, "refine": args.refine,
                   "l2": "inputs larger than L2 (%.1f GB of state)" % (args.batch * 0.39 + args.batch * 0.77)},
        "fp64_single_steps_per_s": K / (ms64 / 1e3),
        "dfloat_single_steps_per_s": K / (msdd / 1e3),
        "fp32_single_steps_per_s": K / (ms32 / 1e3),
        "speedup_vs_fp64_single": value / (world * K / (ms64 / 1e3)),
        f"batch_{other}_refine_instance_steps_per_s": world * args.batch * K / (ms_other / 1e3),
        "hbm_gbs_batch": batch_bytes / (ms_b / 1e3) / 1e9,
        "fp64_flop_roofline": fp64_flop_roofline(K / (ms64 / 1e3)),
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "measured_on": "single FP32 instance, kernels timed alone (burst peak)",
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if "hbm_gbs" in peaks else "fallback"},
        "kernels_ms_per_step_fp32_single": {k: round(v, 4) for k, v in sorted(per_step.items(), key=lambda t: -t[1])},
        "kernels_ms_per_step_dfloat_single": {k: round(v[0] / K, 4)
                                              for k, v in sorted(profdd.items(), key=lambda t: -t[1][0])},
        "kernels_ms_per_step_fp64_single": {k: round(v[0] / K, 4)
                                            for k, v in sorted(prof64.items(), key=lambda t: -t[1][0])},
        "autotune": {"fp32": tuned32, "fp64": tuned64},
        "gpu_launches": launches,
        "clocks": clk.summary(),
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": args.batch * 16 * n3 / K,
                "d2h_bytes_per_step": args.batch * (16 * n3 + 8) / K, "pinned": pinned,
                # the job's fixed part (uploads, start-up, Runge-Kutta start, final
                # fields, energies, read-back): e2e wall time minus the device time
                # of its K steps; and the e2e rate of the scan's 4200-step job
                "fixed_s": e2e_fixed, "per_step_ms": ms_b / K,
                "value_at_4200_steps": world * args.batch * 4200 / (e2e_fixed + 4200 * ms_b / K / 1e3)},
        "cpu_baseline": cpu,
        "mu": stats[0]["mu"],
        "etot_first_instance": energies[0],
    }
    print(json.dumps(line))
    return 0


# ---------------------------------------------------------------------------
# The other workloads of the benchmark configurations, one JSON line each
# (--workload): bounded samples of their step counts, device-timed steps/s
# of every engine, the HBM fraction of the algorithmic step bytes, and the
# C++ FP64 oracle on the host cores for the CPU column.

def _wl_cfg(dims, h, n4, impurity, precision, real_time=False, device=0):
    import eff_pot_gb300 as ep
    from eff_pot_gb300 import _abi
    nx, ny, nz = dims
    kw = dict(nx=nx, ny=ny, nz=nz, xmax=nx * h / 2, ymax=ny * h / 2, zmax=nz * h / 2, icon=_abi.EP_ICON_PERIODIC,
              core="OTC", n4=n4, impurity=impurity, device=device,
              time_mode=_abi.EP_REAL_TIME if real_time else _abi.EP_IMAGINARY_TIME, renormalize=0 if real_time else 1,
              precision={"fp32": _abi.EP_FP32, "fp64": _abi.EP_FP64, "dfloat": _abi.EP_DFLOAT}[precision])
    if impurity == _abi.EP_IMPURITY_MOVING:
        kw.update(mimpur=40.0, fix_lambda=1)
    return ep.make_config(**kw)


def _wl_prepare(s, psi, rimp, pot, vimp=None):
    import numpy as np
    import eff_pot_gb300 as ep
    p = pot if pot is not None else ep.null_potential()
    s.set_impurity_potentials(p, p, p)
    s.set_impurity(rimp=rimp, vimp=vimp, invar=np.zeros(10, dtype=np.complex128))
    s.start(psi)


def _wl_timed(obj, steps, dt, batch=False):
    f, h = obj._f, obj._h
    rec = f["batch_event_record"] if batch else f["event_record"]
    ela = f["batch_event_elapsed"] if batch else f["event_elapsed"]
    rec(h, 0)
    obj.run(steps, dt, wait=False)
    rec(h, 1)
    ms = C.c_double()
    ela(h, 0, 1, C.byref(ms))
    return ms.value


def _wl_single(cfg, psi, rimp, pot, steps, warmup, dt, rk=3, vimp=None):
    import eff_pot_gb300 as ep
    with ep.Solver(cfg) as s:
        _wl_prepare(s, psi, rimp, pot, vimp)
        s.autotune()
        for _ in range(rk):
            s.steprk(dt)
        s.run(warmup, dt)
        s.synchronize()
        ms = _wl_timed(s, steps, dt)
    return steps / (ms / 1e3)


def _wl_cpu(cfg, psi, rimp, pot, steps, dt, rk=3, vimp=None):
    from oracle import pyoracle
    threads = os.cpu_count() or 1
    pyoracle.set_threads(threads)
    s = pyoracle.OracleSolver(cfg)
    _wl_prepare(s, psi, rimp, pot, vimp)
    for _ in range(rk):
        s.steprk(dt)
    s.steppc(dt)
    t0 = time.perf_counter()
    for _ in range(steps):
        s.steppc(dt, wait=False)
        if cfg.time_mode == 0:
            s.renormalize()
    el = time.perf_counter() - t0
    s.close()
    return {"value": steps / el, "unit": "steps/s", "cores": threads, "kind": "port",
            "sample": f"{steps} steppc steps after start-up; C++ FP64 oracle, {threads} OpenMP threads"}


def _peak_gbs():
    try:
        return float(json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"])
    except Exception:
        return 6800.0


def _wl_frac(dims, steps_per_s, s):
    from eff_pot_gb300.roofline import step_bytes
    b = sum(step_bytes(*dims, otc=True, grad=True, s=s, renorm=False).values())
    return b * steps_per_s / 1e9 / _peak_gbs()


def run_workload(args):
    """One of the benchmark configurations other than the scan."""
    import numpy as np
    import eff_pot_gb300 as ep
    from eff_pot_gb300 import _abi
    from eff_pot_gb300.build import build
    build()
    wl = args.workload
    line = {"workload": wl, "unit": "steps/s", "data": "synthetic (seeded Woods-Saxon droplets)"}
    if wl in ("pure64", "impurity128"):
        if wl == "pure64":
            dims, h, n4, seed, imp, pot = (64,) * 3, 0.8, 500.0, 0, _abi.EP_IMPURITY_NONE, None
            line["config"] = "pure N=500 droplet, 64^3, h=0.8 A, OTC, imaginary time, dt=1e-4"
            n64, n32, ncpu = 200, 400, 40
        else:
            dims, h, n4, seed, imp, pot = (128,) * 3, 0.4, 1000.0, 1, _abi.EP_IMPURITY_FIXED, ep.morse(10.0, 4.5, 1.2)
            line["config"] = "N=1000 droplet + Morse impurity at the centre, 128^3, h=0.4 A, OTC, imaginary time"
            n64, n32, ncpu = 100, 400, 20
        psi = ep.woods_saxon_psi(*dims, dims[0] * h / 2, dims[1] * h / 2, dims[2] * h / 2, n4, seed=seed)
        z = (0.0, 0.0, 0.0)
        for prec, n in (("fp64", n64), ("dfloat", n64 * 2), ("fp32", n32)):
            v = _wl_single(_wl_cfg(dims, h, n4, imp, prec), psi, z, pot, n, 5, 1e-4)
            line[f"gpu_{prec}_steps_per_s"] = v
            line[f"hbm_frac_{prec}"] = _wl_frac(dims, v, 4 if prec == "fp32" else 8)
        r = 200.0 / 5000.0
        line["gpu_fp32_dfloat_refine_steps_per_s"] = 1.0 / ((1 - r) / line["gpu_fp32_steps_per_s"] +
                                                          r / line["gpu_dfloat_steps_per_s"])
        if not args.no_cpu:
            line["cpu_baseline"] = _wl_cpu(_wl_cfg(dims, h, n4, imp, "fp64"), psi, z, pot, ncpu, 1e-4)
    elif wl == "uneven":
        rng = np.random.default_rng(2)
        ns = rng.choice([300, 1000, 2000, 5000], size=64)
        grid_of = {300: 96, 1000: 128, 2000: 160, 5000: 192}
        cfgs, psis, rimps, has = [], [], [], []
        for i, nn in enumerate(ns):
            g = grid_of[int(nn)]
            imp = i % 2 == 0
            c = _wl_cfg((g,) * 3, 0.4, float(nn), _abi.EP_IMPURITY_FIXED if imp else _abi.EP_IMPURITY_NONE, "fp32")
            R = 2.22 * float(nn) ** (1.0 / 3.0)
            cfgs.append(c)
            psis.append(ep.woods_saxon_psi(g, g, g, c.xmax, c.ymax, c.zmax, float(nn), seed=100 + i))
            rimps.append((0.0, 0.0, rng.uniform(0.0, R) if imp else 0.0))
            has.append(imp)
        steps, k64 = 20, 1
        with ep.Batch(cfgs) as b:
            for s, psi, r, imp in zip(b, psis, rimps, has):
                _wl_prepare(s, psi, r, ep.morse(10.0, 4.5, 1.2) if imp else None)
            b.autotune()
            for _ in range(3):
                b.steprk(1e-4)
            b.run(3, 1e-4)
            for prec in ("fp64", "dfloat"):
                b.set_precision(prec)
                b.autotune()
                b.run(1, 1e-4)
            b.set_precision("fp32")
            b.synchronize()
            ms32 = _wl_timed(b, steps - k64, 1e-4, batch=True)
            out = {}
            for prec in ("dfloat", "fp64"):
                b.set_precision(prec)
                out[prec] = _wl_timed(b, k64, 1e-4, batch=True)
                b.set_precision("fp32")
        from eff_pot_gb300.roofline import step_bytes
        pts = sum(c.nx * c.ny * c.nz for c in cfgs)
        b32 = sum(sum(step_bytes(c.nx, c.ny, c.nz, s=4, renorm=False).values()) for c in cfgs)
        line.update(config="64 droplets, N in {300,1000,2000,5000} (seed 2), grids 96..192^3 at h=0.4 A, "
                           "half with the Morse impurity", unit="instance-steps/s", grid_points_total=pts,
                    batch_fp32_instance_steps_per_s=64 * (steps - k64) / (ms32 / 1e3),
                    batch_dfloat_instance_steps_per_s=64 * k64 / (out["dfloat"] / 1e3),
                    batch_fp64_instance_steps_per_s=64 * k64 / (out["fp64"] / 1e3),
                    batch_fp32_dfloat_refine_instance_steps_per_s=64 * steps / ((ms32 + out["dfloat"]) / 1e3),
                    hbm_frac_fp32=b32 * (steps - k64) / (ms32 / 1e3) / 1e9 / _peak_gbs(),
                    sample=f"{steps - k64} FP32 steps, then one refinement step in each FP64-class arithmetic")
    elif wl == "realtime":
        dims, h, n4 = (256, 256, 320), 0.4, 10000.0
        psi = ep.woods_saxon_psi(*dims, dims[0] * h / 2, dims[1] * h / 2, dims[2] * h / 2, n4, seed=4)
        dt = 0.5e-3 / ep.KTOPS
        v = (0.0, 0.0, 50.0 * 1e10 / 1e12 * ep.KTOPS)
        pot = ep.morse(10.0, 4.5, 1.2)
        line["config"] = ("N=10000 + Morse impurity kicked at 50 m/s, 256x256x320, h=0.4 A, real time, dt=0.5 fs "
                          "(steady-state steps; the drift run is eff_pot_gb300.realtime)")
        for prec, n in (("fp32", 30), ("dfloat", 10), ("fp64", 6)):
            r = _wl_single(_wl_cfg(dims, h, n4, _abi.EP_IMPURITY_MOVING, prec, real_time=True), psi, (0.0, 0.0, 0.0),
                           pot, n, 2, dt, rk=4, vimp=v)
            line[f"gpu_{prec}_steps_per_s"] = r
            line[f"hbm_frac_{prec}"] = _wl_frac(dims, r, 4 if prec == "fp32" else 8)
        if not args.no_cpu:
            line["cpu_baseline"] = _wl_cpu(_wl_cfg(dims, h, n4, _abi.EP_IMPURITY_MOVING, "fp64", real_time=True),
                                           psi, (0.0, 0.0, 0.0), pot, 3, dt, rk=4, vimp=v)
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=42)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--batch", type=int, default=32)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--workload", default="scan", choices=["scan", "pure64", "impurity128", "uneven", "realtime"],
                    help="scan (default): the headline batch; the others: one line per benchmark configuration")
    ap.add_argument("--refine", default="dfloat", choices=["fp64", "dfloat"],
                    help="arithmetic of the refinement sweeps: FP64, or double-float (FP64-class on the FP32 pipes)")
    ap.add_argument("--step-graphs", type=int, default=1, choices=[0, 1, 2],
                    help="batch steps: 0 direct launches, 1 one replayed graph per step (default), "
                         "2 one graph per 10-step rotation period")
    ap.add_argument("--clocks-dir", default=None, help="where the nvidia-smi samples of the timed region go "
                                                      "(default: the temporary directory)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        return run_reference(args)
    if args.workload != "scan":
        return run_workload(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
