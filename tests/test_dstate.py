"""D-state impurity (Lstate = 'D'): oracle known answers on the CPU, GPU parity.

The reference has no test vectors for this branch either, so the oracle's
restatement of potenimp/potinvar/energy/steppc (D state) is pinned by what
the algebra must satisfy:
  * at every grid point the 5x5 field matrix M = Delta 1 + Pi_Del d d^T +
    Sig_Del P(x) (potenimp.f90:68-131) is the spectral sum of three
    projectors: eigenvalues Delta (twice), Delta + Pi_Del r^4 (once) and
    Delta + Sig_Del r^4 (twice) -- this pins all 15 polynomial entries;
  * SOD (potenimp.f90:429-451) is 2 L.S for l = 2, s = 1/2: eigenvalues 2
    (six) and -3 (four);
  * <iv| i Hinvar + Ev0 iv> = eHeX + eso (potinvar against potenimp+energy);
  * with V_Pi = V_Sigma = V_Delta the field is that pair potential, equal to
    the P state's;
  * in real time the internal variables evolve unitarily, all ten of them.
The GPU path is then checked against the oracle on the same inputs (FP64:
fields 1e-12, matrix and potinvar 1e-11, energies and the evolution 1e-10).
"""
import numpy as np
import pytest

import eff_pot_gb300 as ep
from eff_pot_gb300 import _abi

N, XMAX, N4 = 16, 12.0, 60.0
RIMP = (0.37, -0.55, 0.81)
# Morse channels small enough that no grid point reaches the 1000 K cap
PI = dict(De=5.0, re=4.0, alpha=0.5)
SIGMA = dict(De=4.0, re=4.5, alpha=0.5)
DELTA = dict(De=3.0, re=3.5, alpha=0.7)


def morse(p, umax=1000.0):
    return ep.morse(p["De"], p["re"], p["alpha"], r_cutoff=0.0, umax=umax)


def d_config(n=N, xmax=XMAX, **kw):
    base = dict(nx=n, ny=n, nz=n, xmax=xmax, ymax=xmax, zmax=xmax, icon=_abi.EP_ICON_PERIODIC, core="OTC",
                n4=N4, impurity=_abi.EP_IMPURITY_FIXED, state=_abi.EP_STATE_D, als_d=2.0)
    base.update(kw)
    return ep.make_config(**base)


def d_solver(S, cfg, psi, invar, rimp=RIMP, vimp=(0.0, 0.0, 0.0)):
    s = S(cfg)
    s.set_impurity_potentials_d(morse(PI), morse(SIGMA), morse(DELTA), ep.morse(12.0, 4.0, 1.1))
    s.set_impurity(rimp=rimp, vimp=vimp, invar=invar)
    s.upload_psi(psi)
    s.potenimp()
    return s


def random_invar(seed):
    rng = np.random.default_rng(seed)
    v = rng.normal(size=10) + 1j * rng.normal(size=10)
    return v / np.linalg.norm(v)


def droplet(cfg, seed=4):
    return ep.woods_saxon_psi(cfg.nx, cfg.ny, cfg.nz, cfg.xmax, cfg.ymax, cfg.zmax, cfg.n4, seed=seed)


def rel(a, b):
    d = np.max(np.abs(np.asarray(a) - np.asarray(b)))
    s = np.max(np.abs(np.asarray(b)))
    return d / s if s > 0 else d


# ---------------------------------------------------------------- oracle (CPU)

def test_field_matrix_is_the_sum_of_three_projectors(oracle):
    cfg = d_config()
    psi = droplet(cfg)
    with d_solver(oracle.OracleSolver, cfg, psi, np.zeros(10, complex)) as s:
        # M_ij from the field of unit internal variables: a = e_i gives M_ii,
        # a = e_i + e_j gives M_ii + M_jj + 2 M_ij
        def field(i, j=None):
            iv = np.zeros(10, complex)
            iv[2 * i] = 1.0
            if j is not None:
                iv[2 * j] = 1.0
            s.set_impurity(invar=iv)
            s.potenimp()
            return s.field("uimp").ravel(order="F")
        d = [field(i) for i in range(5)]
        M = np.zeros((cfg.nx * cfg.ny * cfg.nz, 5, 5))
        for i in range(5):
            M[:, i, i] = d[i]
            for j in range(i + 1, 5):
                M[:, i, j] = M[:, j, i] = 0.5 * (field(i, j) - d[i] - d[j])
        dl = s.field("delta").ravel(order="F")
        pd = s.field("vpi").ravel(order="F")
        sd = s.field("sigdel").ravel(order="F")
        x, y, z = s.axes()
        X, Y, Z = np.meshgrid(x - RIMP[0], y - RIMP[1], z - RIMP[2], indexing="ij")
        r4 = ((X ** 2 + Y ** 2 + Z ** 2) ** 2).ravel(order="F")
    w = np.linalg.eigvalsh(M)
    want = np.sort(np.stack([dl, dl, dl + pd * r4, dl + sd * r4, dl + sd * r4], axis=1), axis=1)
    scale = np.max(np.abs(want), axis=1) + 1.0
    assert np.max(np.abs(w - want) / scale[:, None]) < 1e-12
    # the three channels differ, so the test sees every projector
    assert np.min(np.abs(pd - sd) * r4) < np.max(np.abs(pd - sd) * r4)


def test_spin_orbit_matrix_is_two_l_dot_s(oracle):
    cfg = d_config(als_d=2.0, impurity=_abi.EP_IMPURITY_MOVING, mimpur=40.0)
    with d_solver(oracle.OracleSolver, cfg, np.zeros((N, N, N), complex), np.zeros(10, complex)) as s:
        S = np.zeros((10, 10), complex)
        for j in range(10):  # no helium: i Hinvar = (Als_D / 2) SOD iv
            iv = np.zeros(10, complex)
            iv[j] = 1.0
            s.set_impurity(invar=iv)
            S[:, j] = 1j * s.potinvar()
    assert np.allclose(S, S.conj().T, atol=1e-15)
    assert np.allclose(np.linalg.eigvalsh(S), [-3.0] * 4 + [2.0] * 6, atol=1e-13)


def test_potinvar_agrees_with_the_field_and_spin_orbit_energies(oracle):
    cfg = d_config(als_d=3.0, ev0=0.0, impurity=_abi.EP_IMPURITY_MOVING, mimpur=40.0)
    iv = random_invar(11)
    with d_solver(oracle.OracleSolver, cfg, droplet(cfg), iv) as s:
        assert s.field("uimp").max() < 999.0  # no point capped
        s.poten()
        e = s.energy()
        h = s.potinvar()
    expect = e["eHeX"] + e["eso"]
    got = np.vdot(iv, 1j * h).real
    assert abs(got - expect) < 1e-11 * abs(expect)
    # the spin-orbit energy itself: Als_D/2 <iv|SOD|iv> within the 2 L.S range
    assert -4.5 - 1e-12 <= e["eso"] <= 3.0 + 1e-12


def test_isotropic_channels_give_the_pair_potential(oracle):
    iv = random_invar(12)
    res = {}
    for state in (_abi.EP_STATE_P, _abi.EP_STATE_D):
        cfg = d_config(state=state)
        with oracle.OracleSolver(cfg) as s:
            m = morse(PI)
            if state == _abi.EP_STATE_D:
                s.set_impurity_potentials_d(m, m, m)
                s.set_impurity(rimp=RIMP, invar=iv)
            else:  # P field = V_Pi whatever invar when V_Sigma = V_Pi
                s.set_impurity_potentials(m, m)
                s.set_impurity(rimp=RIMP, invar=iv)
            s.upload_psi(droplet(cfg))
            s.potenimp()
            res[state] = s.field("uimp")
    assert rel(res[_abi.EP_STATE_D], res[_abi.EP_STATE_P]) < 1e-14


def test_real_time_evolves_all_ten_internal_variables_unitarily(oracle):
    cfg = d_config(time_mode=_abi.EP_REAL_TIME, impurity=_abi.EP_IMPURITY_MOVING, mimpur=40.0, renormalize=0,
                   als_d=2.0)
    psi = droplet(cfg)
    iv0 = random_invar(13)
    with d_solver(oracle.OracleSolver, cfg, psi, iv0, vimp=(0.0, 0.0, 0.3 * ep.KTOPS)) as s:
        s.poten()
        e = s.energy()
    # Ev0 = eHeX + eso removes the common phase (DFT4He3d.f90:446)
    cfg.ev0 = e["eHeX"] + e["eso"]
    with d_solver(oracle.OracleSolver, cfg, psi, iv0, vimp=(0.0, 0.0, 0.3 * ep.KTOPS)) as s:
        s.poten()
        dt = 2e-4
        for _ in range(3):
            s.steprk(dt)
        for _ in range(8):
            err = s.steppc(dt)
        iv = s.impurity()["invar"]
    assert np.all(np.abs(iv[6:]) > 1e-3)  # the P state would zero components 7-10
    assert abs(np.linalg.norm(iv) - 1.0) < 1e-6
    assert err["erriv"] > 0.0


# ---------------------------------------------------------------- GPU parity

@pytest.mark.gpu
def test_gpu_d_state_fields_and_moments_match_oracle(oracle):
    from eff_pot_gb300.build import build
    build()
    cfg = d_config(n=32, xmax=16.0, n4=200.0, impurity=_abi.EP_IMPURITY_MOVING, mimpur=40.0, als_d=4.0, ev0=-3.0)
    psi = droplet(cfg, seed=5)
    iv = random_invar(21)
    g = d_solver(ep.Solver, cfg, psi, iv)
    o = d_solver(oracle.OracleSolver, cfg, psi, iv)
    with g, o:
        for f in ("uimp", "delta", "vpi", "sigdel"):
            assert rel(g.field(f), o.field(f)) < 1e-12, f
        assert rel(g.impurity_matrix_d(), o.impurity_matrix_d()) < 1e-11
        assert rel(g.forceimp(), o.forceimp()) < 1e-10
        assert rel(g.potinvar(), o.potinvar()) < 1e-11
        g.poten()
        o.poten()
        eg, eo = g.energy(), o.energy()
        for k in ("eHeX", "eso", "eimpu", "etot"):
            assert abs(eg[k] - eo[k]) <= 1e-10 * max(1.0, abs(eo[k])), (k, eg[k], eo[k])
        assert eo["eso"] != 0.0


@pytest.mark.gpu
def test_gpu_d_state_real_time_evolution_matches_oracle(oracle):
    from eff_pot_gb300.build import build
    build()
    cfg = d_config(n=32, xmax=16.0, n4=200.0, time_mode=_abi.EP_REAL_TIME, impurity=_abi.EP_IMPURITY_MOVING,
                   mimpur=40.0, renormalize=0, als_d=2.0, ev0=-2.0)
    psi = droplet(cfg, seed=6)
    iv = random_invar(22)
    v = (0.0, 0.1 * ep.KTOPS, 0.3 * ep.KTOPS)
    g = d_solver(ep.Solver, cfg, psi, iv, vimp=v)
    o = d_solver(oracle.OracleSolver, cfg, psi, iv, vimp=v)
    dt = 2e-4
    with g, o:
        g.poten()
        o.poten()
        for _ in range(3):
            g.steprk(dt)
            o.steprk(dt)
        for _ in range(6):
            eg = g.steppc(dt)
            eo = o.steppc(dt)
        assert rel(g.psi(), o.psi()) < 1e-10
        ig, io = g.impurity(), o.impurity()
        for k in ("rimp", "vimp", "invar"):
            assert np.max(np.abs(ig[k] - io[k])) < 1e-10 * max(1.0, np.max(np.abs(io[k]))), k
        assert eo["erriv"] > 0.0
        assert abs(eg["erriv"] - eo["erriv"]) < 1e-8 * eo["erriv"]


@pytest.mark.gpu
def test_gpu_d_state_fp32_tracks_fp64():
    from eff_pot_gb300.build import build
    build()
    psi = None
    out = {}
    for prec in (_abi.EP_FP64, _abi.EP_FP32):
        cfg = d_config(n=32, xmax=16.0, n4=200.0, precision=prec, als_d=2.0)
        psi = droplet(cfg, seed=7) if psi is None else psi
        with d_solver(ep.Solver, cfg, psi, random_invar(23)) as s:
            out[prec] = (s.field("uimp"), s.field("sigdel"))
    for a, b in zip(out[_abi.EP_FP32], out[_abi.EP_FP64]):
        assert rel(a, b) < 1e-6
