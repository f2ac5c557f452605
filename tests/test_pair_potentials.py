"""He-M+ pair potentials of Koutselos et al. (Select_Pot 'Na_plus_Koutselos'
... 'Cs_plus_Koutselos', V_impur.f90:232-290,1704-1883): the U+ integral of the
reference's post-processing scan (prep.sh sets selec_plus='Rb_plus_Koutselos').

CPU: the oracle's U+ against a numpy quadrature of the same density with the
potential restated here from the published form, and the long-range tail of
every ion against the He polarisability alone, -(alpha_d / 2) / x^4 (the
exchange term is gone and the C6, C8 terms are below 1e-3 of it at 100 A).  GPU: the
library's U+ equals the oracle's to 1e-10, cutoff rule included.
"""
import numpy as np
import pytest

import eff_pot_gb300 as ep
from eff_pot_gb300 import _abi

HARTREE_K = 27.2114 * 11604.448
A_BOHR = 0.529177
# v0, rho, R_m, C6, C8 (atomic units) per ion
IONS = {"Na": (0.2063, 0.7640, 4.55, 1.424, 13.17), "K": (0.2690, 0.8589, 5.49, 5.83, 72.05),
        "Rb": (0.3474, 0.8868, 5.85, 8.8, 126.2), "Cs": (0.5092, 0.9241, 6.38, 13.69, 236.4)}


def v_koutselos(ion, r):
    v0, rho, rm, c6, c8 = IONS[ion]
    x = np.asarray(r, dtype=np.float64) / A_BOHR
    vex = v0 * (146.98 * np.exp(-1.5024 * x / rho) - 70.198 * np.exp(-1.4041 * x / rho))
    aux = 1.28 * rm
    with np.errstate(divide="ignore", invalid="ignore"):
        h = np.where(x >= aux, 1.0, np.exp(-(aux / x - 1.0) ** 2))
        disp = -(1.3831 / 2) / x ** 4 - (c6 + 2.4434 / 2) / x ** 6 - (c8 + 10.614 / 2) / x ** 8
    return (vex + np.where(x > 0, disp * h, 0.0)) * HARTREE_K


def case(n=24, xmax=12.0, n4=100.0):
    cfg = ep.make_config(nx=n, ny=n, nz=n, xmax=xmax, ymax=xmax, zmax=xmax, icon=_abi.EP_ICON_PERIODIC,
                         core="OT ", n4=n4, impurity=_abi.EP_IMPURITY_FIXED)
    psi = ep.woods_saxon_psi(n, n, n, xmax, xmax, xmax, n4, seed=9)
    return cfg, psi


def uplus(S, cfg, psi, plus, rimp=(0.3, -0.1, 0.45)):
    with S(cfg) as s:
        m = ep.morse(10.0, 4.5, 1.2, umax=1000.0)
        s.set_impurity_potentials(m, m, plus)
        s.set_impurity(rimp=rimp, invar=np.zeros(10, complex))
        s.start(psi)
        return s.energy()["uplus"], s


@pytest.mark.parametrize("ion", ["Na", "K", "Rb", "Cs"])
def test_long_range_tail_is_the_helium_polarisability(ion, oracle):
    cfg, psi = case()
    r = np.array([100.0, 150.0])
    tail = -(1.3831 / 2) / (r / A_BOHR) ** 4 * HARTREE_K
    assert np.allclose(v_koutselos(ion, r), tail, rtol=1e-3)


def test_oracle_uplus_matches_the_published_form(oracle):
    cfg, psi = case()
    rimp = (0.3, -0.1, 0.45)
    for ion in IONS:
        rc, umax = 2.0, 6.1105922888e3  # prep.sh's r_cutoff_plus, umax_plus
        got, s = uplus(oracle.OracleSolver, cfg, psi, ep.koutselos(ion, r_cutoff=rc, umax=umax), rimp)
        x, y, z = (np.arange(n) * 2 * cfg.xmax / n - cfg.xmax for n in (cfg.nx, cfg.ny, cfg.nz))
        X, Y, Z = np.meshgrid(x - rimp[0], y - rimp[1], z - rimp[2], indexing="ij")
        rr = np.sqrt(X ** 2 + Y ** 2 + Z ** 2)
        v = np.where(rr < rc, umax, v_koutselos(ion, rr))
        h = 2 * cfg.xmax / cfg.nx
        want = np.sum(np.abs(psi) ** 2 * v) * h ** 3
        assert abs(got - want) < 1e-11 * abs(want), (ion, got, want)


@pytest.mark.gpu
def test_gpu_uplus_matches_oracle(oracle):
    from eff_pot_gb300.build import build
    build()
    cfg, psi = case(n=32, xmax=16.0, n4=200.0)
    for ion in IONS:
        plus = ep.koutselos(ion, r_cutoff=2.0, umax=6.1105922888e3)
        ug, _ = uplus(ep.Solver, cfg, psi, plus)
        uo, _ = uplus(oracle.OracleSolver, cfg, psi, plus)
        assert abs(ug - uo) < 1e-10 * abs(uo), (ion, ug, uo)
