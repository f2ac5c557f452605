"""The CUDA path against the CPU FP64 oracle at the benchmark geometries.

Each case runs the same seeded input through the GPU engine and the oracle:
the poten fields and the energies of the start-up density, then Runge-Kutta-
Gill start steps and predictor-corrector steps (steprk.f90, steppc.f90),
then the fields and energies again.  The grids are the workloads' own, so
every transform length they run is checked against the oracle:

* 64^3, h = 0.8 A, pure N=500 droplet (the CPU-runnable configuration):
  X half-lines of 32, Y/Z lines of 64;
* 128^3, h = 0.4 A, N=1000 + Morse impurity at the centre (the single
  droplet and every instance of the effective-potential scan): X half-lines
  of 64, Y/Z lines of 128;
* 96 x 160 x 192, h = 0.4 A, N=2000 + an off-centre impurity: the lengths of
  the uneven batch (X half-lines of 48, Y lines of 160, Z lines of 192 --
  mixed-radix register transforms in FP32, the shared-memory engine in FP64);
* 256 x 256 x 320, h = 0.4 A, N=10000 + a Morse impurity kicked at 50 m/s in
  real time (the large real-time configuration, on its full grid): X
  half-lines of 128, Y lines of 256, Z lines of 320.

Gates: FP64 and double-float -- the drop-in bar, 1e-10 relative in the
total energy and the chemical potential and 1e-9 A^-3 max-abs in the
density, fields 1e-11 relative, psi 1e-10 relative; FP32 -- 2e-5 relative
in fields and energies, 1e-4 relative in psi, 1e-6 A^-3 max-abs in the
density.
"""
import numpy as np
import pytest

import eff_pot_gb300 as ep
from eff_pot_gb300 import _abi
from eff_pot_gb300.build import build

pytestmark = pytest.mark.gpu

FIELDS_OTC = ["den", "pot4", "dencg", "delj4", "dxden", "dyden", "dzden", "falfs",
              "intxalf", "intyalf", "intzalf", "ualphas", "uimp"]
ENERGIES = ("etot", "etot4", "ekin4", "elj4", "ecor4", "ealphas", "eHeX", "n4")
KTOPS = 7.63822291  # ps K (DFT4He3d.f90:55)

CASES = {
    "64cubed_pure_N500": dict(dims=(64, 64, 64), h=0.8, n4=500.0, seed=0, impurity=_abi.EP_IMPURITY_NONE,
                              rimp=(0.0, 0.0, 0.0), nrk=3, npc=20, dt=1e-4),
    "128cubed_N1000_morse": dict(dims=(128, 128, 128), h=0.4, n4=1000.0, seed=1, impurity=_abi.EP_IMPURITY_FIXED,
                                 rimp=(0.0, 0.0, 0.0), nrk=3, npc=4, dt=1e-4),
    "96x160x192_N2000_morse": dict(dims=(96, 160, 192), h=0.4, n4=2000.0, seed=2,
                                   impurity=_abi.EP_IMPURITY_FIXED, rimp=(0.0, 0.0, 5.3), nrk=3, npc=4, dt=1e-4),
    "256x256x320_N10000_realtime": dict(dims=(256, 256, 320), h=0.4, n4=10000.0, seed=4,
                                        impurity=_abi.EP_IMPURITY_MOVING, rimp=(0.0, 0.0, 0.0),
                                        vimp=(0.0, 0.0, 0.5 * KTOPS), real_time=True, nrk=4, npc=2,
                                        dt=0.5e-3 / KTOPS),
}


@pytest.fixture(scope="module", autouse=True)
def _lib():
    build()
    ep.load_library()


def make_cfg(case, precision):
    nx, ny, nz = case["dims"]
    h = case["h"]
    rt = case.get("real_time", False)
    kw = dict(nx=nx, ny=ny, nz=nz, xmax=nx * h / 2, ymax=ny * h / 2, zmax=nz * h / 2,
              icon=_abi.EP_ICON_PERIODIC, core="OTC", n4=case["n4"], impurity=case["impurity"],
              time_mode=_abi.EP_REAL_TIME if rt else _abi.EP_IMAGINARY_TIME, renormalize=0 if rt else 1,
              precision=precision)
    if case["impurity"] == _abi.EP_IMPURITY_MOVING:
        kw.update(mimpur=40.0, fix_lambda=1)
    return ep.make_config(**kw)


def evolve(solver_cls, case, precision):
    """Start-up fields and energies, then nrk RK-Gill + npc PC steps."""
    cfg = make_cfg(case, precision)
    psi = ep.woods_saxon_psi(cfg.nx, cfg.ny, cfg.nz, cfg.xmax, cfg.ymax, cfg.zmax, case["n4"], seed=case["seed"])
    out = {}
    with solver_cls(cfg) as s:
        pot = ep.morse(10.0, 4.5, 1.2, r_cutoff=0.0, umax=1000.0)
        s.set_impurity_potentials(pot, pot, ep.morse(12.0, 4.0, 1.1))
        s.set_impurity(rimp=case["rimp"], vimp=case.get("vimp"), invar=np.zeros(10, dtype=np.complex128))
        s.start(psi)
        out["fields0"] = {f: s.field(f) for f in FIELDS_OTC}
        out["e0"] = s.energy()
        for _ in range(case["nrk"]):
            s.steprk(case["dt"])
        out["stats"] = s.run(case["npc"], case["dt"])
        out["psi"] = s.psi()
        out["den"] = s.field("den")
        if case["impurity"] == _abi.EP_IMPURITY_MOVING:
            out["imp"] = s.impurity()
        s.poten()
        out["e1"] = s.energy()
        out["pot4"] = s.field("pot4")
    return out


def rel(a, b):
    d = np.max(np.abs(np.asarray(a) - np.asarray(b)))
    s = np.max(np.abs(np.asarray(b)))
    return d / s if s > 0 else d


_ORACLE = {}


def oracle_result(oracle, name):
    if name not in _ORACLE:
        _ORACLE.clear()  # one case's fields at a time (the largest is ~4 GB on the host)
        _ORACLE[name] = evolve(oracle.OracleSolver, CASES[name], _abi.EP_FP64)
    return _ORACLE[name]


@pytest.mark.parametrize("prec", [_abi.EP_FP64, _abi.EP_FP32, _abi.EP_DFLOAT], ids=["fp64", "fp32", "dfloat"])
@pytest.mark.parametrize("name", list(CASES))
def test_benchmark_geometry_matches_oracle(oracle, name, prec):
    case = CASES[name]
    o = oracle_result(oracle, name)
    g = evolve(ep.Solver, case, prec)
    # the double-float path is gated like FP64 (the drop-in bar)
    fp64 = prec in (_abi.EP_FP64, _abi.EP_DFLOAT)
    ftol, etol, ptol, dtol = (1e-11, 1e-10, 1e-10, 1e-9) if fp64 else (2e-5, 2e-5, 1e-4, 1e-6)
    report = {}
    for f in FIELDS_OTC:
        if f == "uimp" and case["impurity"] == _abi.EP_IMPURITY_NONE:
            continue
        report[f] = rel(g["fields0"][f], o["fields0"][f])
    for part in ("e0", "e1"):
        for k in ENERGIES:
            scale = abs(o[part]["etot"]) if not fp64 else max(1.0, abs(o[part][k]))
            report[f"{part}.{k}"] = abs(g[part][k] - o[part][k]) / scale
    report["psi"] = rel(g["psi"], o["psi"])
    report["den_maxabs"] = float(np.max(np.abs(g["den"] - o["den"])))
    report["pot4_after"] = rel(g["pot4"], o["pot4"])
    if not case.get("real_time"):
        report["mu"] = abs(g["stats"]["mu"] - o["stats"]["mu"]) / abs(o["stats"]["mu"])
    if "imp" in o:
        for k in ("rimp", "vimp", "aimp"):
            report[f"imp.{k}"] = float(np.max(np.abs(g["imp"][k] - o["imp"][k]))) / max(
                1.0, float(np.max(np.abs(o["imp"][k]))))
    print(f"PARITY {name} {({_abi.EP_FP64: 'fp64', _abi.EP_FP32: 'fp32', _abi.EP_DFLOAT: 'dfloat'})[prec]} " +
          " ".join(f"{k}={v:.2e}" for k, v in report.items()))
    for f in FIELDS_OTC:
        if f in report:
            assert report[f] < ftol, (f, report[f])
    for k, v in report.items():
        if k.startswith(("e0.", "e1.")):
            assert v < etol, (k, v)
    assert report["psi"] < ptol
    assert report["pot4_after"] < ftol * 10
    assert report["den_maxabs"] < dtol
    if "mu" in report:
        assert report["mu"] < etol
    for k in ("imp.rimp", "imp.vimp", "imp.aimp"):
        if k in report:
            assert report[k] < (1e-9 if fp64 else 1e-4), (k, report[k])
