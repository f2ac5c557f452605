"""forceimp with Lfilter_exciplex_force (potenimp.f90:211-248): the z
component of the force sums only the planes beyond z_exciplex_exclusion on
the far side of the impurity (iz >= iz0 when the impurity sits below z = 0,
iz <= nz0 otherwise, both truncated as Fortran's integer assignment does);
the x and y components are unchanged.  CPU: the oracle against a numpy sum
of its own fields; GPU: the library against the oracle."""
import numpy as np
import pytest

import eff_pot_gb300 as ep
from eff_pot_gb300 import _abi

N, XMAX, N4 = 24, 12.0, 100.0


def cfg_of(filt, **kw):
    return ep.make_config(nx=N, ny=N, nz=N, xmax=XMAX, ymax=XMAX, zmax=XMAX, icon=_abi.EP_ICON_PERIODIC,
                          core="OTC", n4=N4, impurity=_abi.EP_IMPURITY_MOVING, mimpur=40.0, fix_lambda=1,
                          z_exciplex_exclusion=2.3, filter_exciplex_force=filt, **kw)


def started(S, cfg, rimp):
    s = S(cfg)
    m = ep.morse(10.0, 4.5, 1.2, r_cutoff=0.0, umax=1000.0)
    s.set_impurity_potentials(m, m, ep.null_potential())
    s.set_impurity(rimp=rimp, invar=np.zeros(10, dtype=np.complex128))
    s.start(ep.woods_saxon_psi(N, N, N, XMAX, XMAX, XMAX, N4, seed=13))
    return s


def planes(rz, hz, zexc):
    z1 = -XMAX
    if rz < 0.0:
        return max(1, int((rz - z1 + zexc) / hz + 1.5)), N
    return 1, min(N, int((rz - z1 - zexc) / hz + 1.5))


@pytest.mark.parametrize("rz", [-1.7, 0.9])
def test_oracle_filtered_force_sums_the_far_planes(oracle, rz):
    rimp = (0.3, -0.2, rz)
    with started(oracle.OracleSolver, cfg_of(1), rimp) as s, started(oracle.OracleSolver, cfg_of(0), rimp) as u:
        F, Fu = s.forceimp(), u.forceimp()
        dz, uimp = s.field("dzden"), s.field("uimp")
        h = 2 * XMAX / N
        lo, hi = planes(rz, h, 2.3)
        want = -np.sum((dz * uimp)[:, :, lo - 1:hi]) * h ** 3
    assert np.allclose(F[:2], Fu[:2], rtol=0, atol=0)
    assert abs(F[2] - want) < 1e-12 * max(1.0, abs(want))
    assert abs(F[2] - Fu[2]) > 1e-6 * abs(Fu[2])  # the filter removed planes that matter


@pytest.mark.gpu
@pytest.mark.parametrize("rz", [-1.7, 0.9])
@pytest.mark.parametrize("prec", [_abi.EP_FP64, _abi.EP_FP32])
def test_gpu_filtered_force_matches_oracle(oracle, rz, prec):
    from eff_pot_gb300.build import build
    build()
    rimp = (0.3, -0.2, rz)
    with started(ep.Solver, cfg_of(1, precision=prec), rimp) as g, \
            started(oracle.OracleSolver, cfg_of(1), rimp) as o:
        Fg, Fo = g.forceimp(), o.forceimp()
    tol = 1e-10 if prec == _abi.EP_FP64 else 5e-4
    assert np.max(np.abs(Fg - Fo)) < tol * np.max(np.abs(Fo)), (Fg, Fo)
