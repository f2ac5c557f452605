"""Batched instances and the FP32 + FP64-refinement path.

* A batch advances each instance exactly as an independent context does
  (same kernels, deterministic reductions): results agree bit for bit.
* FP32 bulk steps followed by FP64 refinement sweeps reach the FP64 ground
  state: total energy within 1e-8 relative of the plain FP64 path run to the
  same imaginary time, and the impurity energy U* evaluated on that density
  within 1e-6 relative.
"""
import numpy as np
import pytest

import eff_pot_gb300 as ep
from eff_pot_gb300 import _abi
from eff_pot_gb300.build import build

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib():
    build()
    ep.load_library()


def cfg_of(n=32, xmax=16.0, n4=200.0, **kw):
    base = dict(nx=n, ny=n, nz=n, xmax=xmax, ymax=xmax, zmax=xmax, icon=_abi.EP_ICON_PERIODIC,
                core="OTC", n4=n4, impurity=_abi.EP_IMPURITY_FIXED)
    base.update(kw)
    return ep.make_config(**base)


def prepare(s, psi, rimp):
    pot = ep.morse()
    s.set_impurity_potentials(pot, pot, pot)
    s.set_impurity(rimp=rimp, invar=np.zeros(10, dtype=np.complex128))
    s.start(psi)


def test_batch_equals_independent_contexts():
    rimps = [(0.0, 0.0, z) for z in (0.0, 1.25, 2.5)]
    grids = [32, 24, 32]
    cfgs = [cfg_of(n=n, xmax=0.5 * n) for n in grids]
    psis = [ep.woods_saxon_psi(c.nx, c.ny, c.nz, c.xmax, c.ymax, c.zmax, c.n4, seed=i)
            for i, c in enumerate(cfgs)]
    dt = 5e-4
    with ep.Batch(cfgs) as b:
        for s, psi, r in zip(b, psis, rimps):
            prepare(s, psi, r)
        b.steprk(dt)
        b.steprk(dt)
        b.steprk(dt)
        stats = b.run(15, dt)
        got = [s.psi() for s in b]
        launches = b.kernel_launches()
    assert launches > 0
    for cfg, psi, r, g, st in zip(cfgs, psis, rimps, got, stats):
        with ep.Solver(cfg) as s:
            prepare(s, psi, r)
            for _ in range(3):
                s.steprk(dt)
            ref = s.run(15, dt)
            assert np.array_equal(g, s.psi())
            assert st["mu"] == ref["mu"] and st["errHe"] == ref["errHe"]


def _converge(cfg, psi, dt, nbulk, nref, refine, pot=None):
    """Imaginary-time ground state (FP64, or FP32 then FP64 sweeps); with
    pot=None the impurity slot holds the null potential and U* = int rho u of
    a Morse impurity at the centre is evaluated on the converged density, as
    the reference's scan does for saved densities (energy.f90:146-165)."""
    with ep.Solver(cfg) as s:
        p = pot if pot is not None else ep.null_potential()
        s.set_impurity_potentials(p, p, p)
        s.set_impurity(rimp=(0.0, 0.0, 0.0), invar=np.zeros(10, dtype=np.complex128))
        s.start(psi)
        for _ in range(3):
            s.steprk(dt)
        s.run(nbulk, dt)
        if refine:
            assert s.precision() == "fp32"
            s.set_precision("fp64")
            assert s.precision() == "fp64"
        st = s.run(nref, dt)
        s.poten()
        e = s.energy()
        if pot is None:
            m = ep.morse(10.0, 4.5, 1.2)
            s.set_impurity_potentials(m, m, m)
            s.potenimp()
            e["ustar"] = s.energy()["eHeX"]
        return e, st


N_, XMAX_, N4_, DT_, NBULK_, NREF_ = 24, 14.4, 100.0, 2.5e-4, 22000, 2000


def _pair(pot=None, dt=DT_, nbulk=NBULK_, nref=NREF_):
    psi = ep.woods_saxon_psi(N_, N_, N_, XMAX_, XMAX_, XMAX_, N4_, seed=5)
    e64, _ = _converge(cfg_of(n=N_, xmax=XMAX_, n4=N4_), psi, dt, nbulk, nref, False, pot)
    e32, st = _converge(cfg_of(n=N_, xmax=XMAX_, n4=N4_, precision=_abi.EP_FP32), psi, dt, nbulk, nref,
                        True, pot)
    assert st["errHe"] < 1e-9
    return e64, e32


def test_fp32_then_fp64_refinement_reaches_the_fp64_ground_state():
    # A stable ground state: an N=100 droplet (R = 10.3 A) in a 28.8 A
    # periodic box at h = 1.2 A (imaginary time converges it to 12 digits).
    # A droplet that fills its box merges with its periodic images instead.
    e64, e32 = _pair()
    assert abs(e32["etot"] - e64["etot"]) < 1e-8 * abs(e64["etot"]), (e32["etot"], e64["etot"])
    # U* is linear in the density, so it keeps the first-order FP32 residual
    # of the slow modes that the FP64 sweeps leave: gate it at 1e-6 relative.
    assert abs(e64["ustar"]) > 1.0
    assert abs(e32["ustar"] - e64["ustar"]) < 1e-6 * abs(e64["ustar"]), (e32["ustar"], e64["ustar"])


@pytest.mark.parametrize("prec", [_abi.EP_FP64, _abi.EP_FP32])
def test_autotune_keeps_results_bit_identical(prec):
    """Launch shapes only change the thread-to-work mapping, never the
    arithmetic: poten fields agree bit for bit before and after tuning."""
    cfg = cfg_of(n=48, xmax=24.0, precision=prec)
    psi = ep.woods_saxon_psi(48, 48, 48, 24.0, 24.0, 24.0, 200.0, seed=7)
    with ep.Solver(cfg) as s:
        prepare(s, psi, (0.3, 0.0, -0.2))
        before = {f: s.field(f) for f in ("pot4", "dencg", "delj4", "ualphas", "intxalf")}
        rep = s.autotune()
        assert "poten" in rep
        sh = s.launch_shapes()
        s.set_launch_shapes([2, 64, 4, 64, 4, 64])
        s.poten()
        odd = {f: s.field(f) for f in before}
        s.set_launch_shapes(sh)
        s.poten()
        for f in before:
            assert np.array_equal(before[f], s.field(f)), f
            assert np.array_equal(before[f], odd[f]), f


@pytest.mark.parametrize("prec", [_abi.EP_FP64, _abi.EP_FP32])
def test_step_graphs_match_direct_launches(prec):
    """run() replays a captured step graph (only the predictor / corrector
    nodes are updated to the rotated history buffers): same bits, same kernel
    count as launching every kernel, also after the launch shapes change."""
    cfg = cfg_of(n=32, xmax=16.0, precision=prec)
    psi = ep.woods_saxon_psi(32, 32, 32, 16.0, 16.0, 16.0, 200.0, seed=3)
    out = []
    for graphs in (False, True):
        with ep.Solver(cfg) as s:
            s.step_graphs(graphs)
            prepare(s, psi, (0.0, 0.0, 0.5))
            for _ in range(3):
                s.steprk(5e-4)
            st1 = s.run(7, 5e-4)
            s.set_launch_shapes([2, 64, 4, 64, 4, 64])
            st2 = s.run(9, 5e-4)
            s.run(4, 5e-4)
            out.append((s.psi(), st1, st2, s.kernel_launches()))
    assert np.array_equal(out[0][0], out[1][0])
    assert out[0][1] == out[1][1] and out[0][2] == out[1][2]
    assert out[0][3] == out[1][3]


def test_batch_step_graphs_match_direct_launches():
    grids = [32, 24, 32]
    cfgs = [cfg_of(n=n, xmax=0.5 * n, precision=_abi.EP_FP32) for n in grids]
    psis = [ep.woods_saxon_psi(c.nx, c.ny, c.nz, c.xmax, c.ymax, c.zmax, c.n4, seed=10 + i)
            for i, c in enumerate(cfgs)]
    res = []
    for graphs in (False, True):
        with ep.Batch(cfgs) as b:
            b.step_graphs(graphs)
            for s, psi, z in zip(b, psis, (0.0, 0.7, 1.4)):
                prepare(s, psi, (0.0, 0.0, z))
            for _ in range(3):
                b.steprk(5e-4)
            b.run(8, 5e-4)
            b.set_precision("fp64")
            b.run(5, 5e-4)
            b.set_precision("fp32")
            stats = b.run(6, 5e-4)
            res.append(([s.psi() for s in b], stats, b.kernel_launches()))
    for a, c in zip(res[0][0], res[1][0]):
        assert np.array_equal(a, c)
    assert res[0][1] == res[1][1]
    assert res[0][2] == res[1][2]


@pytest.mark.parametrize("n", [64, 128])
def test_fp32_fields_track_fp64_at_production_sizes(n):
    """At the grids of the benchmark configurations the FP32 path (register
    FFTs in every direction) gives the mean-field potential and the energies
    of the FP64 path to FP32 accuracy."""
    xmax = 0.2 * n
    psi = ep.woods_saxon_psi(n, n, n, xmax, xmax, xmax, 1000.0, seed=11)
    fields = ("pot4", "dencg", "delj4", "ualphas", "intxalf")
    res = {}
    for prec in (_abi.EP_FP64, _abi.EP_FP32):
        cfg = cfg_of(n=n, xmax=xmax, n4=1000.0, precision=prec)
        with ep.Solver(cfg) as s:
            prepare(s, psi, (0.0, 0.0, 1.0))
            e = s.energy()
            res[prec] = ({f: s.field(f) for f in fields}, e)
    f64, e64 = res[_abi.EP_FP64]
    f32, e32 = res[_abi.EP_FP32]
    for f in fields:
        scale = np.abs(f64[f]).max()
        assert np.abs(f32[f] - f64[f]).max() < 2e-5 * scale, f
    for k in ("etot", "ekin4", "elj4", "ecor4", "ealphas", "eHeX"):
        assert abs(e32[k] - e64[k]) < 2e-5 * abs(e64["etot"]), k


@pytest.mark.parametrize("prec", [_abi.EP_FP64, _abi.EP_FP32])
def test_multi_step_graphs_match_direct_launches(prec):
    """Runs long enough for whole rotation periods (10 steps) replay a
    captured multi-step graph with no node updates; runs of other lengths
    realign the phase with single replayed steps.  Same bits, same kernel
    count as launching every kernel, for one context and for a batch."""
    cfgs = [cfg_of(n=n, xmax=0.5 * n, precision=prec) for n in (32, 24)]
    psis = [ep.woods_saxon_psi(c.nx, c.ny, c.nz, c.xmax, c.ymax, c.zmax, c.n4, seed=20 + i)
            for i, c in enumerate(cfgs)]
    runs = (25, 13, 31, 3, 10)
    res = []
    for graphs in (0, 2):
        with ep.Batch(cfgs) as b, ep.Solver(cfgs[0]) as s:
            b.step_graphs(graphs)
            s.step_graphs(graphs)
            for inst, psi, z in zip(list(b) + [s], psis + [psis[0]], (0.0, 0.7, 0.3)):
                prepare(inst, psi, (0.0, 0.0, z))
            for _ in range(3):
                b.steprk(5e-4)
                s.steprk(5e-4)
            stats = [b.run(k, 5e-4) for k in runs] + [s.run(k, 5e-4) for k in runs]
            res.append(([x.psi() for x in b] + [s.psi()], stats, b.kernel_launches(), s.kernel_launches()))
    for a, c in zip(res[0][0], res[1][0]):
        assert np.array_equal(a, c)
    assert res[0][1] == res[1][1]
    assert res[0][2] == res[1][2] and res[0][3] == res[1][3]
