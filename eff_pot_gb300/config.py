"""Solver configuration: the reference's module defaults and namelist keys.

Defaults follow modules.f90 (deriva :15,19; grid :75-84; he4 :124-133;
lenard4 :191-196), V_impur.f90:1-16 and DFT4He3d.f90:78 (n4=300).
"""
import ctypes as C

from . import _abi

DEFAULTS = dict(
    nx=64, ny=64, nz=64, xmax=64.0, ymax=64.0, zmax=64.0,
    npd=13, icon=_abi.EP_ICON_ZERO_OUTSIDE, core=_abi.EP_CORE_OT,
    cp4=-2.41186e4, cpp4=1.85850e6, den4c=0.062, alphas=54.31, l=1.0,
    den0s=0.04, h2o2m4=6.05969638298, C=3.1577504e4, beta=40.0, den_m=0.37,
    h4ot=2.190323, h4op=2.359665, eps4=10.22, sigma4=2.556, b4=-718.99,
    time_mode=_abi.EP_IMAGINARY_TIME, renormalize=1, n4=300.0,
    impurity=_abi.EP_IMPURITY_NONE, mimpur=0.0, fix_lambda=0, als_p=0.0,
    ev0=0.0, z_exciplex_exclusion=0.0, precision=_abi.EP_FP64, device=0,
    state=_abi.EP_STATE_P, als_d=0.0, filter_exciplex_force=0,
)

CORES = {"OT": _abi.EP_CORE_OT, "OT ": _abi.EP_CORE_OT, "OTC": _abi.EP_CORE_OTC,
         "OP": _abi.EP_CORE_OP, "OP ": _abi.EP_CORE_OP}

# Ktops: picoseconds per kelvin^-1 (DFT4He3d.f90:55).
KTOPS = 7.63822291
# proton mass in A^-2 K^-1 (modules.f90:333).
MP_U = 0.0207569277


def make_config(**kw):
    """An EpConfig with the reference defaults overridden by kw.

    ``core`` may be given as the namelist string ('OT ', 'OTC', 'OP ').
    """
    vals = dict(DEFAULTS)
    for k, v in kw.items():
        if k not in vals:
            raise KeyError(f"unknown configuration key {k!r}")
        if k == "core" and isinstance(v, str):
            v = CORES[v.upper() if len(v) == 3 else v.upper()]
        vals[k] = v
    cfg = _abi.EpConfig()
    for k, v in vals.items():
        setattr(cfg, k, v)
    return cfg


def config_dict(cfg):
    return {name: getattr(cfg, name) for name, _ in cfg._fields_}


def morse(De=10.0, re=4.5, alpha=1.2, r_cutoff=0.0, umax=1000.0):
    """The He-X Morse pair potential V = De*(exp(-2a(r-re)) - 2exp(-a(r-re)))."""
    p = _abi.EpPotential()
    p.kind = _abi.EP_POT_MORSE
    p.r_cutoff = r_cutoff
    p.umax = umax
    p.par[0], p.par[1], p.par[2], p.par[3] = De, re, alpha, 0.0
    return p


KOUTSELOS_IONS = {"Na": 0, "K": 1, "Rb": 2, "Cs": 3}


def koutselos(ion="Rb", r_cutoff=0.0, umax=0.0):
    """He-M+ of Koutselos et al. (selec = 'Na_plus_Koutselos' ... 'Cs_plus_Koutselos')."""
    p = _abi.EpPotential()
    p.kind = _abi.EP_POT_KOUTSELOS
    p.r_cutoff = r_cutoff
    p.umax = umax
    p.par[0], p.par[1], p.par[2], p.par[3] = float(KOUTSELOS_IONS[ion]), 0.0, 0.0, 0.0
    return p


def null_potential():
    p = _abi.EpPotential()
    p.kind = _abi.EP_POT_NULL
    return p


PATIL_ATOMS = {"LI": 0, "NA": 1, "K": 2, "RB": 3, "CS": 4}
TANG_TOENNIES_ATOMS = {"Ar": 0, "Xe": 1}


def _closed(kind, atom=0.0, r_cutoff=0.0, umax=0.0):
    p = _abi.EpPotential()
    p.kind = kind
    p.r_cutoff = r_cutoff
    p.umax = umax
    p.par[0] = float(atom)
    return p


def patil(atom="RB", r_cutoff=0.0, umax=0.0):
    """Patil's alkali-He potential (selec = 'LI', 'NA', 'K', 'RB', 'CS')."""
    return _closed(_abi.EP_POT_PATIL, PATIL_ATOMS[atom], r_cutoff, umax)


def aziz_he(r_cutoff=0.0, umax=0.0):
    """The He-He potential of Aziz et al. (selec = 'Aziz_He')."""
    return _closed(_abi.EP_POT_AZIZ, 0, r_cutoff, umax)


def tang_toennies(atom="Xe", r_cutoff=0.0, umax=0.0):
    """Tang-Toennies rare-gas-He potentials (selec = 'Ar_He', 'Xe_He')."""
    return _closed(_abi.EP_POT_TANG_TOENNIES, TANG_TOENNIES_ATOMS[atom], r_cutoff, umax)


def series_potential(coef, k0, r_core, f_core, r0, aa, bb, cc, quad=True, r_cutoff=0.0, umax=0.0):
    """An inverse-power fit with a parabolic core (the Param_LJ_* form of
    V_impur.f90): f_core for x <= r_core, |aa x^2 + bb x + cc| for x <= r0,
    sum_k coef[k-1] x^-(k+k0) beyond.  coef entries are floats or (hi, lo)
    pairs (a double-double coefficient); quad sums in double-double.  The
    returned EpPotential holds a reference to its EpSeries."""
    if not 1 <= len(coef) <= _abi.EP_SERIES_MAX:
        raise ValueError(f"1 <= len(coef) <= {_abi.EP_SERIES_MAX}")
    s = _abi.EpSeries()
    s.r_core, s.f_core, s.r0, s.aa, s.bb, s.cc = r_core, f_core, r0, aa, bb, cc
    s.k0, s.n, s.quad = int(k0), len(coef), 1 if quad else 0
    for k, c in enumerate(coef):
        hi, lo = (c, 0.0) if not isinstance(c, (tuple, list)) else c
        s.c_hi[k], s.c_lo[k] = float(hi), float(lo)
    p = _abi.EpPotential()
    p.kind = _abi.EP_POT_SERIES
    p.r_cutoff, p.umax = r_cutoff, umax
    p.series = C.pointer(s)
    p._series = s
    return p
