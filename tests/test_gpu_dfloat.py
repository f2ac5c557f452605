"""The double-float engine (EP_DFLOAT) against the FP64 oracle.

Each real of the double-float fields is an unevaluated sum of two FP32
values (about 48 significant bits) and every operation runs on the FP32
pipes (eff_pot_gb300/csrc/ep_dd.cuh).  It is held to the FP64 drop-in gates:
fields 1e-11 relative, energies and the chemical potential 1e-10 relative,
psi 1e-10 relative, density 1e-9 A^-3 max-abs -- on poten (OT and OTC, both
boundary modes), Runge-Kutta-Gill + predictor-corrector steps in imaginary
time, and a moving impurity in real time.  The benchmark geometries are in
test_gpu_parity_configs.py.
"""
import numpy as np
import pytest

import eff_pot_gb300 as ep
from eff_pot_gb300 import _abi
from eff_pot_gb300.build import build

from test_gpu_parity import FIELDS_ALL, droplet_case, rel

pytestmark = pytest.mark.gpu
D = _abi.EP_DFLOAT


@pytest.fixture(scope="module", autouse=True)
def _lib():
    build()
    ep.load_library()


def pair(cfg_gpu, cfg_ref, psi, oracle, rimp=(0.3, -0.2, 0.7), vimp=(0.0, 0.0, 0.0)):
    g = ep.Solver(cfg_gpu)
    o = oracle.OracleSolver(cfg_ref)
    pot = ep.morse(10.0, 4.5, 1.2, r_cutoff=0.0, umax=1000.0)
    inv = np.zeros(10, dtype=np.complex128)
    inv[0] = 1.0
    for s in (g, o):
        s.set_impurity_potentials(pot, pot, ep.morse(12.0, 4.0, 1.1))
        s.set_impurity(rimp=rimp, vimp=vimp, invar=inv)
        s.start(psi)
    return g, o


@pytest.mark.parametrize("core,icon", [("OTC", 8), ("OT ", 8), ("OTC", 13)])
def test_dfloat_poten_fields_and_energies_match_oracle(oracle, core, icon):
    cfg, psi = droplet_case(core=core, icon=icon, precision=D)
    ref, _ = droplet_case(core=core, icon=icon)
    g, o = pair(cfg, ref, psi, oracle)
    with g, o:
        assert g.precision() == "dfloat"
        names = FIELDS_ALL if core == "OTC" else ["den", "pot4", "dencg", "delj4", "uimp"]
        for f in names:
            assert rel(g.field(f), o.field(f)) < 1e-11, (f, rel(g.field(f), o.field(f)))
        eg, eo = g.energy(), o.energy()
        for k in eo:
            assert abs(eg[k] - eo[k]) <= 1e-10 * max(1.0, abs(eo[k])), (k, eg[k], eo[k])


@pytest.mark.parametrize("icon", [8, 13])
def test_dfloat_rk_then_pc_match_oracle(oracle, icon):
    cfg, psi = droplet_case(icon=icon, precision=D)
    ref, _ = droplet_case(icon=icon)
    g, o = pair(cfg, ref, psi, oracle)
    dt = 5e-4
    with g, o:
        for _ in range(3):
            g.steprk(dt)
            o.steprk(dt)
        assert rel(g.psi(), o.psi()) < 1e-11
        sg = g.run(12, dt)
        so = o.run(12, dt)
        err = {"psi": rel(g.psi(), o.psi()), "den": float(np.max(np.abs(g.field("den") - o.field("den")))),
               "mu": abs(sg["mu"] - so["mu"]) / abs(so["mu"]),
               "errHe": abs(sg["errHe"] - so["errHe"]) / abs(so["errHe"])}
        g.poten()
        o.poten()
        err["etot"] = abs(g.energy()["etot"] - o.energy()["etot"]) / abs(o.energy()["etot"])
        print("DFLOAT rk+pc", icon, " ".join(f"{k}={v:.2e}" for k, v in err.items()))
        assert err["psi"] < 1e-10 and err["den"] < 1e-9 and err["mu"] < 1e-10 and err["etot"] < 1e-10
        assert err["errHe"] < 1e-8


def test_dfloat_real_time_moving_impurity_matches_oracle(oracle):
    kw = dict(time_mode=_abi.EP_REAL_TIME, impurity=_abi.EP_IMPURITY_MOVING, mimpur=85.4678, renormalize=0,
              fix_lambda=1)
    cfg, psi = droplet_case(precision=D, **kw)
    ref, _ = droplet_case(**kw)
    g, o = pair(cfg, ref, psi, oracle, rimp=(0.4, 0.1, -0.3), vimp=(0.0, 0.0, 0.5 * ep.KTOPS))
    dt = 6.546e-5 * 10
    with g, o:
        for _ in range(3):
            g.steprk(dt)
            o.steprk(dt)
        for _ in range(6):
            g.steppc(dt)
            o.steppc(dt)
        assert rel(g.psi(), o.psi()) < 1e-10
        ig, io = g.impurity(), o.impurity()
        for k in ("rimp", "vimp", "aimp"):
            assert np.max(np.abs(ig[k] - io[k])) < 1e-9 * max(1.0, np.max(np.abs(io[k]))), k


def test_precision_switches_through_dfloat_keep_the_state(oracle):
    """FP64 -> double-float -> FP64 keeps psi to double-float rounding (the
    conversion splits each double into two floats, ~1e-14 relative), and the
    steps after the switches still track the oracle."""
    cfg, psi = droplet_case()
    ref, _ = droplet_case()
    g, o = pair(cfg, ref, psi, oracle)
    dt = 5e-4
    with g, o:
        for _ in range(3):
            g.steprk(dt)
            o.steprk(dt)
        before = g.psi()
        g.set_precision("dfloat")
        assert g.precision() == "dfloat"
        assert rel(g.psi(), before) < 1e-13
        g.run(5, dt)
        g.set_precision("fp32")
        g.set_precision("dfloat")
        g.set_precision("fp64")
        g.run(5, dt)
        o.run(10, dt)
        assert rel(g.psi(), o.psi()) < 1e-5  # one FP32 rounding of the state on the way


def test_dfloat_builds_the_13_point_stencils_only():
    cfg, _ = droplet_case(precision=D, npd=9)
    with pytest.raises(ep.EffPotError) as ei:
        ep.Solver(cfg)
    assert ei.value.status == _abi.EP_ERR_UNSUPPORTED


def test_dfloat_batch_and_step_graphs_equal_independent_direct_launches():
    """The refinement sweeps of the batched scan run in double-float: a
    batch that switches FP32 -> double-float gives every instance the bits
    of the same instance run alone with every kernel launched directly."""
    cfgs = [ep.make_config(nx=n, ny=n, nz=n, xmax=0.5 * n, ymax=0.5 * n, zmax=0.5 * n, icon=_abi.EP_ICON_PERIODIC,
                           core="OTC", n4=200.0, impurity=_abi.EP_IMPURITY_FIXED, precision=_abi.EP_FP32)
            for n in (32, 24)]
    psis = [ep.woods_saxon_psi(c.nx, c.ny, c.nz, c.xmax, c.ymax, c.zmax, c.n4, seed=30 + i) for i, c in enumerate(cfgs)]
    zs = (0.0, 0.6)

    def prep(s, psi, z):
        pot = ep.morse()
        s.set_impurity_potentials(pot, pot, pot)
        s.set_impurity(rimp=(0.0, 0.0, z), invar=np.zeros(10, dtype=np.complex128))
        s.start(psi)

    with ep.Batch(cfgs) as b:
        for s, psi, z in zip(b, psis, zs):
            prep(s, psi, z)
        for _ in range(3):
            b.steprk(5e-4)
        b.run(12, 5e-4)
        b.set_precision("dfloat")
        stats = b.run(13, 5e-4)
        got = [s.psi() for s in b]
    for cfg, psi, z, g, st in zip(cfgs, psis, zs, got, stats):
        with ep.Solver(cfg) as s:
            s.step_graphs(False)
            prep(s, psi, z)
            for _ in range(3):
                s.steprk(5e-4)
            s.run(12, 5e-4)
            s.set_precision("dfloat")
            ref = s.run(13, 5e-4)
            assert np.array_equal(g, s.psi())
            assert st["mu"] == ref["mu"]
