"""The two-points-per-thread FP32 predictor / corrector against the one-point form.

The FP32 engine marches the predictor and the corrector (steppc.f90:53-64,
135-151) with two x-neighbouring points per thread whenever the stencil radius
and nx are even, staging its planes and inputs with TMA boxes when the grid
is made of whole 64 x 16 tiles and with per-thread cp.async copies otherwise;
EP_MARCH_TMA=0 at context creation keeps the cp.async staging,
EP_MARCH_PAIRS=0 the one-point form.  Each point's Laplacian and update are
summed in the same order in every form, so the fields they write must agree
bit for bit; only the order in which the block reductions meet differs (the
norm, errHe and mu agree to the FP32 reductions' compensated accuracy).  The
runs do not renormalise, so no reduction feeds back into the fields.  The
cases cover both boundary modes, tiles that the grid fills only partly
(nx = 30, 96: cp.async staging), the 5- and 9-point stencils, real time with
a moving impurity, the benchmark grid, and grids whose tiles all touch the
periodic wrap (nx = 64, ny = 16) for the TMA boxes.
"""
import os

import numpy as np
import pytest

import eff_pot_gb300 as ep
from eff_pot_gb300 import _abi
from eff_pot_gb300.build import build

pytestmark = pytest.mark.gpu

CASES = {
    "128cubed_periodic": dict(dims=(128, 128, 128), h=0.4, n4=1000.0, icon=_abi.EP_ICON_PERIODIC, npd=13),
    "30x36x40_periodic": dict(dims=(30, 36, 40), h=0.8, n4=300.0, icon=_abi.EP_ICON_PERIODIC, npd=13),
    "30x36x40_zero_outside": dict(dims=(30, 36, 40), h=0.8, n4=300.0, icon=_abi.EP_ICON_ZERO_OUTSIDE, npd=13),
    "96x40x48_zero_outside_9pt": dict(dims=(96, 40, 48), h=0.6, n4=400.0, icon=_abi.EP_ICON_ZERO_OUTSIDE, npd=9),
    "64x24x32_periodic_5pt": dict(dims=(64, 24, 32), h=0.8, n4=200.0, icon=_abi.EP_ICON_PERIODIC, npd=5),
    "64cubed_realtime_moving": dict(dims=(64, 64, 64), h=0.6, n4=500.0, icon=_abi.EP_ICON_PERIODIC, npd=13,
                                    real_time=True),
    "64x16x24_periodic": dict(dims=(64, 16, 24), h=0.8, n4=100.0, icon=_abi.EP_ICON_PERIODIC, npd=13),
    "64x16x24_zero_outside": dict(dims=(64, 16, 24), h=0.8, n4=100.0, icon=_abi.EP_ICON_ZERO_OUTSIDE, npd=13),
    "192x32x24_zero_outside_9pt": dict(dims=(192, 32, 24), h=0.6, n4=300.0, icon=_abi.EP_ICON_ZERO_OUTSIDE,
                                       npd=9),
    "128x16x20_periodic_5pt": dict(dims=(128, 16, 20), h=0.8, n4=100.0, icon=_abi.EP_ICON_PERIODIC, npd=5),
}
FORMS = {"tma": {}, "pairs": {"EP_MARCH_TMA": "0"}, "one": {"EP_MARCH_PAIRS": "0"}}


@pytest.fixture(scope="module", autouse=True)
def _lib():
    build()
    ep.load_library()


def run(case, form):
    nx, ny, nz = case["dims"]
    h = case["h"]
    rt = case.get("real_time", False)
    kw = dict(nx=nx, ny=ny, nz=nz, xmax=nx * h / 2, ymax=ny * h / 2, zmax=nz * h / 2, icon=case["icon"],
              npd=case["npd"], core="OTC", n4=case["n4"], precision=_abi.EP_FP32,
              impurity=_abi.EP_IMPURITY_MOVING if rt else _abi.EP_IMPURITY_FIXED,
              time_mode=_abi.EP_REAL_TIME if rt else _abi.EP_IMAGINARY_TIME, renormalize=0)
    if rt:
        kw.update(mimpur=40.0, fix_lambda=1)
    cfg = ep.make_config(**kw)
    psi = ep.woods_saxon_psi(nx, ny, nz, cfg.xmax, cfg.ymax, cfg.zmax, case["n4"], seed=7)
    keys = ("EP_MARCH_PAIRS", "EP_MARCH_TMA")
    old = {k: os.environ.pop(k, None) for k in keys}
    os.environ.update(FORMS[form])
    try:
        s = ep.Solver(cfg)
    finally:
        for k in keys:
            os.environ.pop(k, None)
            if old[k] is not None:
                os.environ[k] = old[k]
    with s:
        pot = ep.morse(10.0, 4.5, 1.2, r_cutoff=0.0, umax=1000.0)
        s.set_impurity_potentials(pot, pot, pot)
        s.set_impurity(rimp=(0.3, -0.2, 0.5), vimp=(0.0, 0.0, 3.0) if rt else None,
                       invar=np.zeros(10, dtype=np.complex128))
        s.start(psi)
        dt = 2e-4 if rt else 1e-4
        for _ in range(4 if rt else 3):
            s.steprk(dt)
        stats = s.run(6, dt)
        out = {"psi": s.psi(), "den": s.field("den"), "pc": s.cfield("pc"), "stats": stats}
        for k in ("psiold1", "psiold2", "psiold3", "hpsiold1", "hpsiold2"):
            out[k] = s.cfield(k)
    return out


@pytest.mark.parametrize("form", ["tma", "pairs"])
@pytest.mark.parametrize("name", list(CASES))
def test_pair_march_gives_the_one_point_bits(name, form):
    a = run(CASES[name], form)
    b = run(CASES[name], "one")
    for k in ("psi", "den", "pc", "psiold1", "psiold2", "psiold3", "hpsiold1", "hpsiold2"):
        assert np.array_equal(a[k], b[k]), (name, form, k, float(np.max(np.abs(a[k] - b[k]))))
    for k in ("norm", "mu", "errHe"):
        ref = b["stats"][k]
        assert abs(a["stats"][k] - ref) <= 1e-6 * max(1.0, abs(ref)), (name, form, k, a["stats"][k], ref)


def test_tma_wait_that_runs_out_reports_timeout():
    """Failure detection of the TMA march: with EP_TEST_TMA_TIMEOUT=1 the
    predictor and corrector announce each plane's bytes on the mbarrier but
    issue no copy, so every bounded wait runs out (4096 polls); the blocks
    end their march, raise EP_FLAG_TIMEOUT, and ep_run returns
    EP_ERR_TIMEOUT.  Nothing is in flight and the context stays usable; a
    context made afterwards without the switch runs normally."""
    case = CASES["64x16x24_periodic"]
    nx, ny, nz = case["dims"]
    h = case["h"]
    cfg = ep.make_config(nx=nx, ny=ny, nz=nz, xmax=nx * h / 2, ymax=ny * h / 2, zmax=nz * h / 2,
                         icon=case["icon"], core="OTC", n4=case["n4"], precision=_abi.EP_FP32,
                         impurity=_abi.EP_IMPURITY_NONE, renormalize=0)
    psi = ep.woods_saxon_psi(nx, ny, nz, cfg.xmax, cfg.ymax, cfg.zmax, case["n4"], seed=7)
    old = os.environ.pop("EP_TEST_TMA_TIMEOUT", None)
    os.environ["EP_TEST_TMA_TIMEOUT"] = "1"
    try:
        s = ep.Solver(cfg)
    finally:
        os.environ.pop("EP_TEST_TMA_TIMEOUT", None)
        if old is not None:
            os.environ["EP_TEST_TMA_TIMEOUT"] = old
    with s:
        s.start(psi)
        for _ in range(3):
            s.steprk(1e-4)
        with pytest.raises(ep.EffPotError) as ei:
            s.run(2, 1e-4)
        assert ei.value.status == _abi.EP_ERR_TIMEOUT, ei.value
        s.synchronize()
    out = run(case, "tma")
    assert np.all(np.isfinite(out["psi"]))
