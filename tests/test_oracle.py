"""The CPU oracle pinned against the reference's table, published functions
and analytic known answers (no GPU needed)."""
import json
import os
from decimal import Decimal

import numpy as np
import pytest

from eff_pot_gb300 import make_config, woods_saxon_psi
from eff_pot_gb300 import _abi

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def ulp_diff(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    ia = a.view(np.int64).astype(object)
    ib = b.view(np.int64).astype(object)
    return max(abs(int(x) - int(y)) for x, y in zip(ia.ravel(), ib.ravel()))


def test_fd_weights_match_bickley_table(oracle):
    """Central rows of mates.f BLKDS (NEWDER ICON=1) == closed forms."""
    rows = json.load(open(os.path.join(GOLD, "bickley_central_rows.json")))["rows"]
    assert len(rows) == 23
    for key, vals in rows.items():
        M, K = (int(t[1:]) for t in key.split("_"))
        ref = np.array([float(Decimal(v)) for v in vals])
        got = oracle.fd_weights(M, K)
        d = ulp_diff(got, ref)
        assert d <= 1, (key, d, got, ref)


def test_sinint_matches_mpmath(oracle):
    vals = json.load(open(os.path.join(GOLD, "si_values.json")))["values"]
    for xs, ref in vals.items():
        x = float(xs)
        r = float(Decimal(ref))
        assert abs(oracle.sinint(x) - r) <= 5e-16 * max(1.0, abs(r)), (x, oracle.sinint(x), r)
        assert oracle.sinint(-x) == -oracle.sinint(x)


@pytest.mark.parametrize("shape", [(16, 12, 10), (8, 16, 30), (20, 18, 24), (6, 5, 9)])
def test_rfft3_matches_numpy(oracle, shape):
    rng = np.random.default_rng(7)
    a = np.asfortranarray(rng.standard_normal(shape))
    got = oracle.rfft3(a)
    ref = np.fft.rfftn(a, axes=(2, 1, 0))
    assert got.shape == ref.shape
    assert np.max(np.abs(got - ref)) <= 1e-13 * np.max(np.abs(ref))
    back = oracle.irfft3(got, shape[0]) / a.size
    assert np.max(np.abs(back - a)) <= 1e-14 * np.max(np.abs(a))


def test_bforce_is_b4(oracle):
    # fforma.f90:256-280 integrates the OT-cored LJ potential; modules.f90:195
    # quotes the rounded value b4 = -718.99 K A^3.
    b = oracle.bforce(_abi.EP_CORE_OT, 10.22, 2.556, 2.190323)
    assert abs(b - (-718.99)) < 0.01


def small_cfg(**kw):
    base = dict(nx=16, ny=16, nz=16, xmax=8.0, ymax=8.0, zmax=8.0, icon=_abi.EP_ICON_PERIODIC)
    base.update(kw)
    return make_config(**base)


def test_form_factor_values_at_p0(oracle):
    with oracle.OracleSolver(small_cfg(core="OTC")) as s:
        fv, wc, ka = s.form_factors()
        b = oracle.bforce(_abi.EP_CORE_OT, 10.22, 2.556, 2.190323)
        assert fv[0, 0, 0] == b
        assert wc[0, 0, 0] == 1.0 and ka[0, 0, 0] == 1.0
        assert np.all(np.isfinite(fv)) and np.all(np.abs(wc) <= 1.0)


@pytest.mark.parametrize("core", ["OT ", "OTC"])
def test_uniform_bulk_energy_and_field(oracle, core):
    """Uniform density: E/N = b rho/2 + c2 rho^2/2 + c3 rho^3/3 and
    pot4 = b rho + 3/2 c2 rho^2 + 4/3 c3 rho^3 + penalty(rho)."""
    rho0 = 0.021836
    cfg = small_cfg(core=core)
    with oracle.OracleSolver(cfg) as s:
        psi = np.full(s.shape, np.sqrt(rho0), dtype=np.complex128, order="F")
        s.upload_psi(psi)
        s.potenimp()
        s.poten()
        e = s.energy()
        b = oracle.bforce(_abi.EP_CORE_OT, cfg.eps4, cfg.sigma4, cfg.h4ot)
        c2, c3 = cfg.cp4, cfg.cpp4
        rho = float(np.abs(psi[0, 0, 0]) ** 2)
        epn = b * rho / 2 + c2 * rho ** 2 / 2 + c3 * rho ** 3 / 3
        assert abs(e["etot4"] / e["n4"] - epn) < 1e-12 * abs(epn)
        assert abs(epn - (-7.15)) < 0.01
        t = np.tanh(cfg.beta * (rho - cfg.den_m))
        pen = cfg.C * (1 + t + cfg.beta * rho * (1 - t * t))
        mu = b * rho + 1.5 * c2 * rho ** 2 + 4.0 / 3.0 * c3 * rho ** 3 + pen
        pot4 = s.field("pot4")
        assert np.max(np.abs(pot4 - mu)) < 1e-12 * abs(mu)
        assert abs(e["ekin4"]) < 1e-20 and abs(e["ealphas"]) < 1e-12


@pytest.mark.parametrize("icon", [_abi.EP_ICON_PERIODIC, _abi.EP_ICON_ZERO_OUTSIDE])
def test_derivative_symbol_of_plane_waves(oracle, icon):
    """Periodic: derivative of exp(i theta j) is the FD symbol times it."""
    cfg = small_cfg(nx=32, ny=20, nz=24, icon=icon)
    with oracle.OracleSolver(cfg) as s:
        x, y, z = s.axes()
        n = {0: 32, 1: 20, 2: 24}
        hh = {0: s.hx, 1: s.hy, 2: s.hz}
        for axis, coord in enumerate((x, y, z)):
            m = 3
            th = 2 * np.pi * m / n[axis]
            j = np.arange(n[axis])
            f1 = np.exp(1j * th * j)
            shp = [1, 1, 1]
            shp[axis] = n[axis]
            f = np.broadcast_to(f1.reshape(shp), s.shape).copy(order="F")
            w1, w2 = oracle.fd_weights(13, 1), oracle.fd_weights(13, 2)
            k = np.arange(-6, 7)
            s1 = np.sum(w1 * np.exp(1j * th * k)) / hh[axis]
            s2 = np.sum(w2 * np.exp(1j * th * k)) / hh[axis] ** 2
            d1 = s.deriv(f, 1, axis)
            d2 = s.deriv(f, 2, axis)
            sl = [slice(None)] * 3
            if icon == _abi.EP_ICON_ZERO_OUTSIDE:
                sl[axis] = slice(6, n[axis] - 6)
            sl = tuple(sl)
            assert np.max(np.abs(d1[sl] - s1 * f[sl])) < 1e-12 * abs(s1)
            assert np.max(np.abs(d2[sl] - s2 * f[sl])) < 1e-12 * abs(s2)
            # real input path equals the real part
            dr = s.deriv(np.ascontiguousarray(f.real).copy(order="F"), 2, axis)
            assert np.max(np.abs(dr - d2.real)) < 1e-12 * abs(s2)


def free_config(time_mode):
    # zero functional: pot4 == 0 so the step is the linear free equation
    return small_cfg(nx=24, ny=16, nz=16, xmax=12.0, cp4=0.0, cpp4=0.0, eps4=0.0, C=0.0,
                     time_mode=time_mode, renormalize=0)


@pytest.mark.parametrize("time_mode", [_abi.EP_IMAGINARY_TIME, _abi.EP_REAL_TIME])
def test_rk_and_pc_on_the_free_equation(oracle, time_mode):
    """psi = plane wave: exact evolution exp(lam t) (imaginary) or
    exp(i lam t) (real), lam = h2o2m4 * FD symbol."""
    cfg = free_config(time_mode)
    with oracle.OracleSolver(cfg) as s:
        x, y, z = s.axes()
        m = 2
        th = 2 * np.pi * m / cfg.nx
        psi0 = np.exp(1j * th * np.arange(cfg.nx))[:, None, None] * np.ones(s.shape)
        psi0 = np.asfortranarray(psi0 * 0.1)
        s.upload_psi(psi0)
        s.poten()
        assert np.max(np.abs(s.field("pot4"))) == 0.0
        w2 = oracle.fd_weights(13, 2)
        k = np.arange(-6, 7)
        lam = cfg.h2o2m4 * np.real(np.sum(w2 * np.exp(1j * th * k))) / s.hx ** 2
        dt = 0.02 / abs(lam)
        rate = lam if time_mode == _abi.EP_IMAGINARY_TIME else 1j * lam
        for _ in range(3):
            s.steprk(dt)
        got = s.psi()
        exact = psi0 * np.exp(rate * 3 * dt)
        assert np.max(np.abs(got - exact)) < 1e-9 * np.max(np.abs(exact))
        for _ in range(20):
            err = s.steppc(dt)
        got = s.psi()
        exact = psi0 * np.exp(rate * 23 * dt)
        assert np.max(np.abs(got - exact)) < 1e-8 * np.max(np.abs(exact))
        assert err["errHe"] < 1e-9


def test_imaginary_time_lowers_the_energy(oracle):
    cfg = make_config(nx=24, ny=24, nz=24, xmax=14.4, ymax=14.4, zmax=14.4, icon=_abi.EP_ICON_PERIODIC,
                      core="OTC", n4=100.0)
    psi = woods_saxon_psi(24, 24, 24, 14.4, 14.4, 14.4, 100.0, seed=0)
    with oracle.OracleSolver(cfg) as s:
        s.start(psi)
        e0 = s.energy()["etot"]
        for _ in range(3):
            s.steprk(1e-3)
        energies = []
        for _ in range(4):
            s.run(5, 1e-3)
            s.poten()
            energies.append(s.energy()["etot"])
        assert energies[0] < e0
        assert all(b < a for a, b in zip(energies, energies[1:]))


@pytest.mark.parametrize("core", ["OT ", "OTC"])
def test_real_time_conserves_norm_and_energy(oracle, core):
    """Real time without an impurity: 3 Runge-Kutta-Gill and 60 Hamming
    steps of a 24^3 droplet keep the norm to 1e-12 and the total energy to
    2e-5 relative (the method's truncation error at dt = 2e-4 K^-1)."""
    n, xmax, n4 = 24, 12.0, 100.0
    cfg = make_config(nx=n, ny=n, nz=n, xmax=xmax, ymax=xmax, zmax=xmax, icon=_abi.EP_ICON_PERIODIC, core=core,
                      n4=n4, time_mode=_abi.EP_REAL_TIME, renormalize=0)
    psi = woods_saxon_psi(n, n, n, xmax, xmax, xmax, n4, seed=5)
    h3 = (2 * xmax / n) ** 3
    with oracle.OracleSolver(cfg) as s:
        s.start(psi)
        e0 = s.energy()["etot"]
        n0 = np.sum(np.abs(s.psi()) ** 2) * h3
        for _ in range(3):
            s.steprk(2e-4)
        for _ in range(60):
            s.steppc(2e-4)
        moved = np.max(np.abs(s.psi() - psi))
        s.poten()
        e1 = s.energy()["etot"]
        n1 = np.sum(np.abs(s.psi()) ** 2) * h3
    assert moved > 1e-3 * np.max(np.abs(psi))  # the state did evolve
    assert abs(n1 - n0) < 1e-12 * n0
    assert abs(e1 - e0) < 2e-5 * abs(e0)


def test_oracle_reproduces_its_golden_vectors(oracle):
    """The committed golden vectors of a short OTC evolution
    (tests/golden/make_oracle_fixture.py) pin the oracle against regressions."""
    import importlib.util
    import json
    import os
    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    spec = importlib.util.spec_from_file_location("mk", os.path.join(here, "make_oracle_fixture.py"))
    mk = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mk)
    want = json.load(open(os.path.join(here, "oracle_otc_32.json")))
    got = mk.scenario(oracle.OracleSolver)
    for part in ("start", "after"):
        for k, v in want[part].items():
            assert abs(got[part][k] - v) <= 1e-11 * max(1.0, abs(v)), (part, k, got[part][k], v)
    for k in ("mu", "norm", "den_sum", "den_sq", "den_xmom"):
        assert abs(got[k] - want[k]) <= 1e-11 * max(1e-12, abs(want[k])), k
    assert abs(got["errHe"] - want["errHe"]) <= 1e-9 * abs(want["errHe"])
    assert np.allclose(got["den_samples"], want["den_samples"], rtol=1e-11, atol=1e-18)
