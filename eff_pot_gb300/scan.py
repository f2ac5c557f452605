"""The effective-potential scan as one GPU job: V_eff(z) = E(z) - E(pure).

The reference computes the effective potential of an impurity in a droplet
by running the solver once per impurity position and once without the
impurity, then subtracting the total energies printed by energy.f90
(energy.f90:146-165, collected by loop.sh / get_impurity_energy.sh).  Here
every instance -- the pure droplet and the droplet with the impurity fixed
at each z on the x = y = 0 axis -- advances together in one Batch: FP32
steps, then FP64-class refinement sweeps (double-float by default, or FP64),
then poten + energy of each instance.  With reference=True the same instances are also run on the plain FP64
path to the same imaginary time, and every V_eff(z) carries its difference
from the FP64 result.

Across ranks (one process per GPU) the instance list is partitioned: rank r
takes instances r, r + world, ...; each rank runs its share as one Batch,
and the per-instance energies are gathered on rank 0 (host scalars, no
collective on the data path).

    python -m eff_pot_gb300.scan [--points 32] [--fp32-steps 4000]
                                 [--fp64-steps 200] [--reference]
"""
import argparse
import json
import time

import numpy as np

from . import _abi
from .config import make_config, morse
from .initial import woods_saxon_psi
from .solver import Batch

PURE = "pure"


def instance_list(zs):
    """The scan's instances: the pure droplet, then one per impurity position."""
    return [(PURE, None)] + [(f"z={z:g}", float(z)) for z in zs]


def partition(instances, rank, world):
    """Rank r's share of the instance list (strided: r, r + world, ...)."""
    return instances[rank::world]


def scan_config(z, precision, n=128, h=0.4, n4=1000.0, device=0):
    return make_config(nx=n, ny=n, nz=n, xmax=n * h / 2, ymax=n * h / 2, zmax=n * h / 2, icon=_abi.EP_ICON_PERIODIC,
                       core="OTC", n4=n4, impurity=_abi.EP_IMPURITY_NONE if z is None else _abi.EP_IMPURITY_FIXED,
                       time_mode=_abi.EP_IMAGINARY_TIME, renormalize=1, precision=precision, device=device)


def _prepare(s, psi, z, pot):
    s.set_impurity_potentials(pot, pot, pot)
    s.set_impurity(rimp=(0.0, 0.0, 0.0 if z is None else z), invar=np.zeros(10, dtype=np.complex128))
    s.start(psi)


def run_instances(mine, psi, *, precision, steps32, steps64, dt, pot, make_batch, cfg_of, rk_steps=3, tune=True,
                  refine="fp64"):
    """Advance this rank's instances as one batch and return {key: energies}.

    precision 'fp32': steps32 FP32 steps, then steps64 refinement sweeps in
    `refine` arithmetic ('fp64', or 'dfloat': the double-float engine);
    'fp64': steps32 + steps64 plain FP64 steps (the same imaginary time).
    Start: density, potenimp, poten, rk_steps Runge-Kutta-Gill steps."""
    if not mine:
        return {}
    prec = _abi.EP_FP32 if precision == "fp32" else _abi.EP_FP64
    b = make_batch([cfg_of(z, prec) for _, z in mine])
    try:
        for s, (_, z) in zip(b, mine):
            _prepare(s, psi, z, pot)
        if tune and hasattr(b, "autotune"):
            b.autotune()
        for _ in range(rk_steps):
            b.steprk(dt)
        if precision == "fp32":
            if steps32:
                b.run(steps32, dt, wait=False)
            b.set_precision(refine)
            if steps64:
                b.run(steps64, dt, wait=False)
        else:
            b.run(steps32 + steps64, dt, wait=False)
        out = {}
        for s in b:
            s.poten()
        for s, (key, _) in zip(b, mine):
            e = s.energy()
            out[key] = {"etot": e["etot"], "eHeX": e["eHeX"], "n4": e["n4"]}
        return out
    finally:
        b.close()


def gather(dist, part):
    """Rank 0 receives every rank's {key: energies}; other ranks get None."""
    if dist is None:
        return dict(part)
    allparts = [None] * dist.get_world_size()
    dist.all_gather_object(allparts, part)
    if dist.get_rank() != 0:
        return None
    out = {}
    for p in allparts:
        out.update(p)
    return out


def veff_table(zs, e32, e64=None):
    """V_eff(z) = E(z) - E(pure) per point, with the FP64 path's value and the
    difference when e64 is given."""
    rows = []
    for key, z in instance_list(zs)[1:]:
        row = {"z": z, "E": e32[key]["etot"], "Veff": e32[key]["etot"] - e32[PURE]["etot"],
               "Ustar": e32[key]["eHeX"]}
        if e64 is not None:
            v64 = e64[key]["etot"] - e64[PURE]["etot"]
            row.update(E_fp64=e64[key]["etot"], Veff_fp64=v64, Veff_err=row["Veff"] - v64,
                       E_rel_err=(row["E"] - e64[key]["etot"]) / abs(e64[key]["etot"]))
        rows.append(row)
    return rows


def veff_scan(zs, *, steps32=4000, steps64=200, dt=1e-4, n=128, h=0.4, n4=1000.0, seed=1, reference=False,
              pot=None, rank=0, world=1, dist=None, device=0, make_batch=Batch, tune=True, refine="dfloat"):
    """V_eff(z) for the impurity positions zs (A, on the x = y = 0 axis).

    Returns (on rank 0) a dict with the pure droplet's energy and one row
    per z; other ranks return None.  make_batch builds the batch of this
    rank's instances (the library's Batch)."""
    pot = pot if pot is not None else morse(10.0, 4.5, 1.2)
    psi = woods_saxon_psi(n, n, n, n * h / 2, n * h / 2, n * h / 2, n4, seed=seed)
    mine = partition(instance_list(zs), rank, world)

    def cfg_of(z, prec):
        return scan_config(z, prec, n=n, h=h, n4=n4, device=device)

    kw = dict(steps32=steps32, steps64=steps64, dt=dt, pot=pot, make_batch=make_batch, cfg_of=cfg_of, tune=tune)
    t0 = time.perf_counter()
    e32 = gather(dist, run_instances(mine, psi, precision="fp32", refine=refine, **kw))
    t32 = time.perf_counter() - t0
    e64, t64 = None, None
    if reference:
        t0 = time.perf_counter()
        e64 = gather(dist, run_instances(mine, psi, precision="fp64", **kw))
        t64 = time.perf_counter() - t0
    if e32 is None:
        return None
    res = {"E_pure": e32[PURE]["etot"], "rows": veff_table(zs, e32, e64), "wall_s_fp32_refine": t32,
           "steps": {"fp32": steps32, "refine": steps64, "refine_arithmetic": refine, "dt": dt},
           "instances": len(zs) + 1,
           "ranks": world}
    if e64 is not None:
        res["E_pure_fp64"] = e64[PURE]["etot"]
        res["wall_s_fp64_reference"] = t64
        res["max_abs_Veff_err_K"] = max(abs(r["Veff_err"]) for r in res["rows"])
        res["max_E_rel_err"] = max(abs(r["E_rel_err"]) for r in res["rows"])
    return res


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--points", type=int, default=32)
    ap.add_argument("--dz", type=float, default=1.25)
    ap.add_argument("--fp32-steps", type=int, default=4000)
    ap.add_argument("--fp64-steps", type=int, default=200)
    ap.add_argument("--reference", action="store_true", help="also run the plain FP64 path (per-point error)")
    ap.add_argument("--refine", default="dfloat", choices=["dfloat", "fp64"],
                    help="arithmetic of the refinement sweeps (default: double-float)")
    a = ap.parse_args(argv)
    import os
    from .build import build
    rank, world = int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    if rank == 0:
        build()
    if dist is not None:
        dist.barrier()
    zs = [a.dz * k for k in range(a.points)]
    res = veff_scan(zs, steps32=a.fp32_steps, steps64=a.fp64_steps, reference=a.reference, rank=rank,
                    world=world, dist=dist, device=local, refine=a.refine)
    if rank == 0:
        print(json.dumps(res))
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
