"""Select_Pot beyond Morse and Koutselos (V_impur.f90:87-932): Patil's
alkali-He potentials ('LI' .. 'CS'), Aziz's He-He ('Aziz_He'), the
Tang-Toennies rare-gas-He pair ('Ar_He', 'Xe_He') and the inverse-power fits
with a parabolic core (the Param_LJ_* family: 'Rb_gs_Fausto', 'Ba_plus_gs',
'He2S_fci', 'LJ_OT', ...), read by ep_select_pot from the reference's own
V_impur.f90.

CPU: the library's host evaluator against the oracle's restatement; known
answers of the closed forms (the dispersion tails, the He-He well); every
inverse-power fit of the reference source (when it is present) against an
exact rational evaluation of its series from the decimal literals, parsed
here independently, with each literal's Fortran kind (Q: Real*16, D: double,
none or E: default REAL, rounded to binary32); the double-double sum of the
Real*16 fits against the same sum in double.  GPU: U+ and the impurity
field of these potentials equal the oracle's.
"""
import math
import os
import re
from fractions import Fraction

import numpy as np
import pytest

import eff_pot_gb300 as ep
from eff_pot_gb300 import _abi

# The reference checkout: $EP_REFERENCE_ROOT, else a "reference" directory
# beside this repository.  Tests that read its V_impur.f90 skip without it.
REFERENCE_ROOT = os.environ.get("EP_REFERENCE_ROOT") or os.path.join(
    os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))), "reference")
SOURCE = os.path.join(REFERENCE_ROOT, "src", "V_impur.f90")
BOHR_PATIL, K_PATIL = 0.529177249, 11604.448 * 27.211608


@pytest.fixture(scope="module")
def lib():
    pytest.importorskip("ctypes")
    try:
        ep.load_library()
    except Exception as e:  # the library is built by the session fixture
        pytest.skip(f"libeffpot.so not loadable: {e}")


SURFACES = ["Grafeno", "Grafeno_sin_dispersion", "TiO2", "Au", "Au_TiO2", "dAu_TiO2", "Ag_Graphene",
            "dz_Ag_Graphene", "Au_Graphene", "dz_Au_Graphene"]


def closed_forms():
    out = [(f"patil-{a}", ep.patil(a)) for a in ep.config.PATIL_ATOMS]
    out += [("aziz", ep.aziz_he()), ("tt-Ar", ep.tang_toennies("Ar")), ("tt-Xe", ep.tang_toennies("Xe"))]
    for name, kind, par in [("Ag_gs", _abi.EP_POT_AG, 0), ("Ag_Pi", _abi.EP_POT_AG, 1),
                            ("Ag_Sig", _abi.EP_POT_AG, 2), ("Ba_gs", _abi.EP_POT_BA_GS, 0)] + \
            [(f"CH3I_{l}", _abi.EP_POT_CH3I, l) for l in range(5)] + \
            [(n, _abi.EP_POT_SURFACE, i) for i, n in enumerate(SURFACES)]:
        p = _abi.EpPotential()
        p.kind, p.par[0] = kind, float(par)
        out.append((name, p))
    return out


@pytest.mark.parametrize("name,pot", closed_forms())
def test_library_and_oracle_agree_on_the_closed_forms(lib, oracle, name, pot):
    r = np.linspace(1.0, 40.0, 3001)
    a = ep.potential_values(pot, r)
    b = oracle.potential_values(pot, r)
    assert np.all(np.isfinite(a))
    assert np.all(np.abs(a - b) <= 1e-12 * np.maximum(np.abs(b), 100.0)), name


@pytest.mark.parametrize("atom", list(ep.config.PATIL_ATOMS))
def test_patil_tail_is_the_dispersion_series(lib, atom):
    """Beyond 60 A the exchange term and the damping are below e^-100: V is
    -(c6/d^6 + c8/d^8) in hartree (the published c6, c8 per alkali)."""
    c6, c8 = {"LI": (22.5, 1.06e3), "NA": (24.7, 1.29e3), "K": (38.9, 2.66e3), "RB": (44.6, 3.18e3),
              "CS": (51.2, 4.34e3)}[atom]
    r = np.array([60.0, 80.0, 120.0])
    d = r / BOHR_PATIL
    want = -(c6 / d ** 6 + c8 / d ** 8) * K_PATIL
    assert np.allclose(ep.potential_values(ep.patil(atom), r), want, rtol=1e-12, atol=0)


def test_aziz_well(lib):
    """The He-He well of the HFD form: minimum at r_m = 2.963 A within the
    fit's accuracy, depth -eps (10.948 K) times A e^(beta-alpha)/eps-scaled
    balance, about 0.999 eps."""
    r = np.linspace(2.8, 3.2, 40001)
    v = ep.potential_values(ep.aziz_he(), r)
    i = int(np.argmin(v))
    assert abs(r[i] - 2.963) < 0.01
    F = math.exp(-(1.4826 - 1.0) ** 2)
    v_rm = (1.8443101e5 * math.exp(-10.43329537 - 2.27965105) - F * (1.36745214 + 0.42123807 + 0.17473318)) * 10.948
    assert abs(ep.potential_values(ep.aziz_he(), np.array([2.963]))[0] - v_rm) < 1e-12 * abs(v_rm)
    assert -11.0 < v[i] < -10.8


@pytest.mark.parametrize("atom,consts", [("Ar", (9.7697, 152.8468, 3249.728)),
                                         ("Xe", (21.5674, 430.148, 10610.21))])
def test_tang_toennies_tail(lib, atom, consts):
    """At 40 A the Born-Mayer term and the damping are below e^-130: V is
    -sum_{n=3..9} C_2n / x^2n with C_12.. from the recursion C_2n =
    (C_2n-2 / C_2n-4)^3 C_2n-6 (Tang and Toennies' extrapolation)."""
    C = list(consts)
    for i in range(3, 7):
        C.append((C[i - 1] / C[i - 2]) ** 3 * C[i - 3])
    r = np.array([40.0, 60.0])
    x = r / 0.5292
    want = -sum(C[i] / x ** (2 * i + 6) for i in range(7)) * 27.21 * 11604.0
    assert np.allclose(ep.potential_values(ep.tang_toennies(atom), r), want, rtol=1e-12, atol=0)


# ------------------------------------------- closed forms vs the reference source
def _function_body(text, name):
    m = re.search(r"(?is)function\s+" + name + r"\s*\((.*?)\n\s*end(?:\s*function)?\b", text)
    assert m, name
    return m.group(1)


def _decl(body):
    """name -> value of the `name = literal` initialisations and assignments
    of a function body, each literal with its Fortran kind."""
    out = {}
    for name, lit in re.findall(r"(?i)\b(\w+)\s*=\s*([-+]?(?:\d+\.?\d*|\.\d+)(?:[edq][-+]?\d+)?)(?![\w.])", body):
        out.setdefault(name.lower(), float(literal(lit)[0]))
    return out


@pytest.fixture(scope="module")
def source_text():
    if not os.path.exists(SOURCE):
        pytest.skip("the reference's V_impur.f90 is not present here")
    with open(SOURCE, encoding="latin-1") as f:
        return re.sub(r"![^\n]*", "", f.read())


def test_ag_ba_ch3i_constants_and_forms_match_the_reference_source(lib, source_text):
    """The He-Ag HFD forms, Lovallo's He-Ba and the He-CH3I Morse components
    restated here in numpy with the constants read from V_impur.f90 (each
    literal with its kind) equal the library's evaluator."""
    r = np.linspace(0.5, 30.0, 600)
    for i, (fn, suf) in enumerate((("V_Ag_gs", "gs"), ("V_Ag_Pi", "pi"), ("V_Ag_Sig", "si"))):
        k = _decl(_function_body(source_text, fn))
        A, al, be, D = (k[n + suf] for n in ("a", "alpha", "beta", "d"))
        C = [k[f"c{j}{suf}"] for j in (6, 8, 10, 12)]
        ff = np.where(r <= D, np.exp(-(D / r - 1.0) ** 2), 1.0)
        want = A * np.exp(-al * r - be * r ** 2) - ff * sum(c / r ** p for c, p in zip(C, (6, 8, 10, 12)))
        got = ep.potential_values(ep.select_pot(fn[2:]), r)
        assert np.allclose(got, want, rtol=1e-13, atol=1e-13 * np.max(np.abs(want))), fn
    body = _function_body(source_text, "V_Ba_gs")
    terms = re.findall(r"([-+]?\s*\d+\.\d*d\d+)\s*/\s*x\*\*(\d+)", body.replace("&\n", " "))
    assert len(terms) == 7
    x = r[r > 3.7]
    want = sum(float(literal(c.replace(" ", ""))[0]) / x ** int(p) for c, p in terms)
    got = ep.potential_values(ep.select_pot("Ba_gs"), x)
    assert np.allclose(got, want, rtol=1e-12, atol=1e-12 * np.max(np.abs(want)))
    assert np.all(ep.potential_values(ep.select_pot("Ba_gs"), r[r <= 3.7]) == 1297.1)
    rad = _function_body(source_text, "radpot")
    cases = re.split(r"(?i)case\s*\(", rad)[2:7]
    for l in range(5):
        k = _decl(cases[l])
        kf = _decl(_function_body(source_text, f"V_CH3I_{l}"))
        xa = r / kf["a_bohr"]
        want = (k["d"] * (1.0 - np.exp(-k["b"] * (xa - k["c"]))) ** 2 - k["d"]) * kf["hartree"] * kf["ev_k"]
        want = np.where(r <= kf["r_cutoff"], kf["umax"], want)
        got = ep.potential_values(ep.select_pot(f"CH3I_{l}"), r)
        assert np.allclose(got, want, rtol=1e-13, atol=1e-15), l


def _data(body):
    """name -> value of the DATA statements of a function body."""
    out = {}
    for stmt in re.findall(r"(?i)\bdata\b([^\n]*)", body):
        for name, lit in re.findall(r"(\w+)\s*/\s*([^/,]+?)\s*/", stmt):
            out[name.lower()] = float(literal(lit)[0])
    return out


def test_surface_potentials_match_the_reference_source(lib, source_text):
    """The ten surface and adatom entries restated in numpy with the
    constants read from V_impur.f90 equal the library's evaluator."""
    z = np.linspace(1.0, 20.0, 500)
    k = _data(_function_body(source_text, "V_grafeno"))
    want = {"Grafeno": (k["a"] * np.exp(-k["alpha"] * z) - k["c4"] / z ** 4 - k["c6"] / z ** 6) * k["c_mev_to_k"]}
    k = _data(_function_body(source_text, "V_grafeno_sin_dispersion"))
    want["Grafeno_sin_dispersion"] = (k["d"] * (1 - np.exp(-k["alpha"] * (z - k["ze"]))) ** 2 - k["d"]) * k["c_mev_to_k"]
    k = _data(_function_body(source_text, "V_TiO2"))
    vz = k["de"] * (1 - np.exp(-k["alpha"] * (z - k["ze"]))) ** 2 - k["de"]
    vzd = -0.5 * (1 + np.tanh((z - k["z0"]) / k["aa"]) * k["c3"] * (k["c3"] / z) ** 3)
    want["TiO2"] = (vz + vzd) * k["cmm1tok"]
    k = _data(_function_body(source_text, "V_Au"))
    r = z - k["re"]
    poly = 1.0 + sum(k[f"a{j}"] * r ** j for j in range(1, 10))
    want["Au"] = -k["de"] * poly * np.exp(-k["a1"] * r)
    k = _decl(_function_body(source_text, "V_Au_TiO2"))
    a2 = 1.0 / z ** 2
    v = sum(k[f"c{n}"] * a2 ** (n // 2) for n in (6, 8, 10, 12, 14)) * k["cmev_to_k"]
    want["Au_TiO2"] = np.where(z > 2, v, 1821.44287109375 * k["cmev_to_k"])
    dv = sum(-n * k[f"c{n}"] * a2 ** (n // 2) / z for n in (6, 8, 10, 12, 14)) * k["cmev_to_k"]
    want["dAu_TiO2"] = np.where(z > 2, dv, -5415.35400390625 * k["cmev_to_k"])
    for name, fn, unit in (("Ag_Graphene", "Ag_Graphene", "ckcal_to_k"), ("Au_Graphene", "Au_Graphene", "xmev_to_k")):
        k = _data(_function_body(source_text, fn))
        want[name] = (k["a"] * np.exp(-k["beta"] * z) - k["c4"] / z ** 4) * k[unit]
        want["dz_" + name] = (-k["a"] * k["beta"] * np.exp(-k["beta"] * z) + 4 * k["c4"] / z ** 5) * k[unit]
    for name in SURFACES:
        got = ep.potential_values(ep.select_pot(name), z)
        assert np.allclose(got, want[name], rtol=1e-12, atol=1e-10), name


def test_patil_aziz_tang_toennies_constants_match_the_reference_source(lib, source_text):
    """The constants of V_alka, V_Aziz_He, V_Ar_He and V_Xe_He as read from
    the source give the library's values through numpy restatements."""
    r = np.linspace(1.0, 30.0, 400)
    k = _decl(_function_body(source_text, "V_Aziz_He"))
    x = r / k["rm"]
    ff = np.where(x <= k["d"], np.exp(-(k["d"] / x - 1.0) ** 2), 1.0)
    want = (k["a"] * np.exp(-k["alpha"] * x + k["beta"] * x ** 2) -
            ff * (k["c6"] / x ** 6 + k["c8"] / x ** 8 + k["c10"] / x ** 10)) * k["eps"]
    assert np.allclose(ep.potential_values(ep.aziz_he(), r), want, rtol=1e-13, atol=1e-12)
    for atom, fn in (("Ar", "V_Ar_He"), ("Xe", "V_Xe_He")):
        k = _decl(_function_body(source_text, fn))
        B = [k["bb"]]
        for i in range(2, 19):
            B.append(B[-1] * k["bb"] / i)
        C = [k["c6"], k["c8"], k["c10"]]
        for i in range(3, 7):
            C.append((C[i - 1] / C[i - 2]) ** 3 * C[i - 3])
        rr = r / k["rbohr"]
        e = np.exp(-k["bb"] * rr)
        S = np.cumsum([B[i] * rr ** (i + 1) for i in range(18)], axis=0)
        v = k["aa"] * e + sum(((S[2 * i + 5] + 1.0) * e - 1.0) * C[i] / rr ** (2 * i + 6) for i in range(7))
        assert np.allclose(ep.potential_values(ep.tang_toennies(atom), r), v * 27.21 * 11604.0, rtol=1e-11,
                           atol=1e-9), atom
    body = _function_body(source_text, "V_alka")
    data = {n.lower(): [float(literal(v)[0]) for v in vals.split(",")]
            for n, vals in re.findall(r"(?i)data\s+(\w+)\s*/([^/]*)/", body) if n.lower() != "celem"}
    d = r / 0.529177249
    for i, atom in enumerate(("LI", "NA", "K", "RB", "CS")):
        a, b, c6, c8 = data["av"][i], data["bv"][i], data["c6v"][i], data["c8v"][i]
        r2, r4, r6, ag = data["r2v"][i], data["r4v"][i], data["r6v"][i], data["agranv"][i]
        abar, u = (a + b) / 4.0, a - 1.0
        v = -0.5 * a ** 2 * u
        roa = ag * d ** (2.0 * u) * (1.0 + v / d) ** 2 * np.exp(-2.0 * d / a)
        f = [1.0 - np.exp(-d / abar) * sum((d / abar) ** n / math.factorial(n) for n in range(2 * l + 8))
             for l in (1, 2)]
        want = (4.0 * math.pi / 3.0 * roa * (r2 + 37.0 / 90.0 * r4 / a ** 2 + 28.0 / 525.0 * r6 / a ** 4) -
                c6 * f[0] / d ** 6 - c8 * f[1] / d ** 8) * 11604.448 * 27.211608
        assert np.allclose(ep.potential_values(ep.patil(atom), r), want, rtol=1e-12, atol=1e-9), atom


# --------------------------------------------------------------- series fits
def rn32(fr):
    """Fraction rounded to the nearest binary32 (ties to even)."""
    if fr == 0:
        return Fraction(0)
    s = -1 if fr < 0 else 1
    a = abs(fr)
    e = math.floor(math.log2(a.numerator) - math.log2(a.denominator))
    while Fraction(2) ** e > a:
        e -= 1
    while Fraction(2) ** (e + 1) <= a:
        e += 1
    m = a / Fraction(2) ** (e - 23)
    q, rem = divmod(m.numerator, m.denominator)
    if 2 * rem > m.denominator or (2 * rem == m.denominator and q % 2):
        q += 1
    return s * Fraction(q) * Fraction(2) ** (e - 23)


def literal(tok):
    """(value, kind) of a Fortran real literal: kind 16 (Q), 8 (D), 4 (none/E)."""
    t = tok.strip().lower()
    m = re.fullmatch(r"([+-]?)(\d*)\.?(\d*)(?:([edq])([+-]?\d+))?", t)
    assert m, tok
    sign, ip, fp, letter, ex = m.groups()
    v = Fraction(int((ip or "0") + fp), 10 ** len(fp)) * Fraction(10) ** int(ex or 0)
    v = -v if sign == "-" else v
    if letter == "q":
        return v, 16
    if letter == "d":
        return Fraction(float(v)), 8
    return rn32(v), 4


def parse_fits(text):
    """name -> (Fraction coefficients, k0, quad, core constants) of every
    Select_Pot name whose function is an inverse-power fit."""
    text = re.sub(r"![^\n]*", "", text)
    text = re.sub(r"&\s*\n\s*&?", " ", text)
    sel = text[re.search(r"(?i)function\s+select_pot", text).start():]
    names, pending = {}, []
    for m in re.finditer(r"(?is)if\s*\(\s*(trim\(selec\).*?)\)\s*then|select_pot\s*=\s*(\w+)\s*\(", sel):
        if m.group(1):
            pending = re.findall(r"'([^']+)'", m.group(1))
        else:
            for n in pending:
                names.setdefault(n, m.group(2).lower())
            pending = []
        if re.match(r"(?i)end\s*function\s*select_pot", sel[m.end():m.end() + 30]):
            break
    funcs = {}
    for m in re.finditer(r"(?is)\n\s*double precision\s+function\s+(\w+)\s*\(x\)(.*?)\n\s*end\b", text):
        body = m.group(2).lower().replace(" ", "")
        if "abs(aa*x**2+bb*x+cc)" not in body or "sto=sto+pg(k)" not in body:
            continue
        com = re.search(r"common/(\w+)/", body).group(1)
        lit = re.search(r"x\*\*\(k\+(\d+)\)", body)
        funcs[m.group(1).lower()] = (com, "real*16pg,sto" in body, int(lit.group(1)) if lit else None)
    blocks = {}
    for m in re.finditer(r"(?is)\n\s*block\s*data\s+\w+(.*?)\n\s*end\b", text):
        b = m.group(1)
        com = re.search(r"(?i)common/(\w+)/", b).group(1).lower()
        data = {k.lower(): [v for v in vals.split(",") if v.strip()]
                for k, vals in re.findall(r"(?i)data\s+(\w+)\s*/([^/]*)/", b)}
        pg16 = re.search(r"(?i)real\*16\s+pg", b) is not None
        blocks[com] = (data, pg16)
    fits = {}
    for name, fn in names.items():
        if fn not in funcs:
            continue
        com, quad, k0lit = funcs[fn]
        data, pg16 = blocks[com]
        coef = []
        for tok in data["pg"]:
            v, kind = literal(tok)
            if not pg16 and kind == 16:
                v = Fraction(float(v))
            coef.append(v)
        k0 = k0lit if k0lit is not None else int(data["k0"][0])
        core = {k: float(literal(data[k][0])[0]) for k in ("rcutoff", "fcutoff", "r0", "aa", "bb", "cc")}
        fits[name] = (coef, k0, quad, core)
    return fits


def exact(coef, k0, x):
    xq = 1 / Fraction(x)
    return sum(c * xq ** (k + 1 + k0) for k, c in enumerate(coef))


@pytest.fixture(scope="module")
def reference_fits():
    if not os.path.exists(SOURCE):
        pytest.skip("the reference's V_impur.f90 is not present here")
    with open(SOURCE, encoding="latin-1") as f:
        fits = parse_fits(f.read())
    assert len(fits) >= 25, sorted(fits)
    return fits


def test_every_reference_fit_matches_exact_arithmetic(lib, oracle, reference_fits):
    for name, (coef, k0, quad, core) in sorted(reference_fits.items()):
        p = ep.select_pot(name, 0.0, 0.0, SOURCE)
        assert p.kind == _abi.EP_POT_SERIES, name
        s = p.series.contents
        assert (s.k0, s.n, s.quad) == (k0, len(coef), int(quad)), name
        for k, c in enumerate(coef):  # hi + lo is c to 2^-104 (exactly c for D and default-REAL literals)
            assert abs(Fraction(s.c_hi[k]) + Fraction(s.c_lo[k]) - c) <= abs(c) * Fraction(1, 2 ** 104), (name, k)
        assert (s.r_core, s.f_core, s.r0, s.aa, s.bb, s.cc) == tuple(
            core[k] for k in ("rcutoff", "fcutoff", "r0", "aa", "bb", "cc")), name
        r = np.linspace(0.5 * core["rcutoff"], 25.0, 60)
        if core["r0"] > core["rcutoff"]:
            r = np.unique(np.concatenate([r, [core["r0"] - 1e-3, core["r0"] + 1e-3]]))
        got = ep.potential_values(p, r)
        ora = oracle.potential_values(p, r)
        if quad:  # both correctly rounded double-double sums
            assert np.array_equal(got, ora), name
        else:  # the oracle raises 1/x to each power, the library multiplies up
            assert np.all(np.abs(got - ora) <= 1e-13 * np.maximum(np.abs(ora), 1.0)), name
        for x, g in zip(r, got):
            if x <= core["rcutoff"]:
                assert g == core["fcutoff"]
                continue
            if x <= core["r0"]:
                want = abs(Fraction(core["aa"]) * Fraction(x) ** 2 + Fraction(core["bb"]) * Fraction(x) +
                           Fraction(core["cc"]))
                scale = abs(core["aa"]) * x * x + abs(core["bb"]) * x + abs(core["cc"])
                assert abs(g - float(want)) <= 4e-16 * scale, (name, x)
                continue
            want = exact(coef, k0, x)
            if quad:  # correctly rounded but for the last bit
                assert abs(g - float(want)) <= 2 * np.spacing(abs(float(want))), (name, x, g, float(want))
            else:
                scale = float(sum(abs(c) / Fraction(x) ** (k + 1 + k0) for k, c in enumerate(coef)))
                assert abs(g - float(want)) <= 1e-14 * scale, (name, x)


def _block(text, common):
    """The DATA of the BLOCK DATA holding COMMON /common/ (name -> literals)."""
    t = re.sub(r"&\s*\n\s*&?", " ", text)
    for m in re.finditer(r"(?is)\n\s*block\s*data\s+\w+(.*?)\n\s*end\b", t):
        if re.search(r"(?i)common/" + common + "/", m.group(1)):
            return {k.lower(): [v for v in vals.split(",") if v.strip()]
                    for k, vals in re.findall(r"(?i)data\s+(\w+)\s*/([^/]*)/", m.group(1))}
    raise AssertionError(common)


def test_old_ba_plus_and_cs_7s_fits(lib, oracle, source_text):
    """'Ba_plus_old_gs' (through Func_Ba_plus_gs: a plain parabola, then even
    inverse powers 6..36) against exact rational arithmetic, and 'Cs_7s' (x
    clamped at 2.5 A, a parabola, then Pg(1) e^(-Ps(1) x)/x + sum Pg(k)
    x^(k-1) e^(-Ps(k) x)) against a numpy restatement, both with the
    coefficients read here from the BLOCK DATA."""
    d = _block(source_text, "Param_LJ_Ba_plus_gs")
    pg = [literal(v)[0] for v in d["pg"]]
    r0, aa, bb, cc = (literal(d[k][0])[0] for k in ("r0", "aa", "bb", "cc"))
    p = ep.select_pot("Ba_plus_old_gs", 0.0, 0.0, SOURCE)
    assert p.kind == _abi.EP_POT_EVENPOW
    x = np.linspace(1.0, 25.0, 300)
    got = ep.potential_values(p, x)
    for v, g in zip(x, got):
        X = Fraction(v)
        if X <= r0:
            want = aa * X * X + bb * X + cc
            scale = abs(aa) * X * X + abs(bb) * X + abs(cc)
        else:
            want = sum(c / X ** (2 * k + 6) for k, c in enumerate(pg))
            scale = sum(abs(c) / X ** (2 * k + 6) for k, c in enumerate(pg))
        assert abs(g - float(want)) <= 1e-14 * float(scale), v
    assert np.allclose(oracle.potential_values(p, x), got, rtol=0, atol=1e-13 * np.max(np.abs(got)))
    d = _block(source_text, "Param_AP_Fit_APG_Cs_7s0")
    pg = [float(literal(v)[0]) for v in d["pg"]]
    ps = [float(literal(v)[0]) for v in d["ps"]]
    r0, aa, bb, cc = (float(literal(d[k][0])[0]) for k in ("r0", "aa", "bb", "cc"))
    p = ep.select_pot("Cs_7s", 0.0, 0.0, SOURCE)
    assert p.kind == _abi.EP_POT_EXPFIT and p.series.contents.r_core == 2.5
    xc = np.maximum(x, 2.5)
    series = pg[0] * np.exp(-ps[0] * xc) / xc + sum(pg[k] * xc ** k * np.exp(-ps[k] * xc) for k in range(1, 12))
    want = np.where(xc <= r0, aa * xc ** 2 + bb * xc + cc, series)
    scale = np.abs(pg[0] * np.exp(-ps[0] * xc) / xc) + sum(np.abs(pg[k] * xc ** k * np.exp(-ps[k] * xc))
                                                           for k in range(1, 12))
    assert np.all(np.abs(ep.potential_values(p, x) - want) <= 1e-13 * scale)
    assert np.all(np.abs(oracle.potential_values(p, x) - want) <= 1e-13 * scale)


def test_real16_fits_need_the_double_double_sum(lib, reference_fits):
    """Near the core the terms of the Fausto fits cancel by ten orders of
    magnitude: the same coefficients summed in double miss the exact value by
    far more than the double-double sum does."""
    coef, k0, quad, core = reference_fits["Rb_gs_Fausto"]
    assert quad
    p = ep.select_pot("Rb_gs_Fausto", 0.0, 0.0, SOURCE)
    s = p.series.contents
    d = ep.series_potential([(s.c_hi[k], s.c_lo[k]) for k in range(s.n)], s.k0, s.r_core, s.f_core, s.r0, s.aa,
                            s.bb, s.cc, quad=False)
    x0 = max(core["r0"], core["rcutoff"])
    x = np.linspace(x0 + 0.01, x0 + 1.0, 25)
    want = np.array([float(exact(coef, k0, v)) for v in x])
    err_dd = np.max(np.abs(ep.potential_values(p, x) - want))
    err_d = np.max(np.abs(ep.potential_values(d, x) - want))
    assert err_dd <= 2 * np.max(np.spacing(np.abs(want)))
    assert err_d > 100 * max(err_dd, 1e-13), (err_d, err_dd)


def test_default_real_literals_are_binary32(lib, reference_fits):
    """V_Rb_6s, V_Cs_sigma and V_Cs_pi write their Pg without an exponent
    letter: default REAL constants, rounded to binary32 before DATA widens
    them to Real*16 -- kept, so the fit is the one the reference computes."""
    for name in ("Rb_6s", "Cs_sigma", "Cs_pi"):
        p = ep.select_pot(name, 0.0, 0.0, SOURCE)
        s = p.series.contents
        assert all(float(np.float32(s.c_hi[k])) == s.c_hi[k] and s.c_lo[k] == 0.0 for k in range(s.n)), name


def test_synthetic_series_in_double_double(lib, oracle):
    """A fit built by the caller (no source): 1e4 (1 - 2/x)^12 x^-6 expanded
    in powers of 1/x cancels by up to 28 orders of magnitude near x = 2: the
    double-double sum is within 2 ulp plus 1e-30 of the terms' magnitude
    (106-bit arithmetic), the double sum only within 1e-16 of it; the oracle's
    restatement agrees to the same bound."""
    coef = [1e4 * math.comb(12, j) * (-2.0) ** j for j in range(13)]
    p = ep.series_potential(coef, 5, 1.0, 500.0, 1.5, 0.0, -10.0, 400.0, quad=True)
    d = ep.series_potential(coef, 5, 1.0, 500.0, 1.5, 0.0, -10.0, 400.0, quad=False)
    x = np.linspace(1.6, 12.0, 300)
    got = ep.potential_values(p, x)
    want = np.array([float(exact([Fraction(c) for c in coef], 5, v)) for v in x])
    scale = np.array([sum(abs(c) * v ** -(k + 6) for k, c in enumerate(coef)) for v in x])
    assert np.all(np.abs(got - want) <= 2 * np.spacing(np.abs(want)) + 1e-30 * scale)
    err_d = np.abs(ep.potential_values(d, x) - want)
    assert np.max(err_d / scale) > 1e-18 and np.all(err_d <= 1e-15 * scale)
    ora = oracle.potential_values(p, x)
    assert np.all(np.abs(got - ora) <= 2 * np.spacing(np.abs(want)) + 2e-30 * scale)
    core = ep.potential_values(p, np.array([0.9, 1.0, 1.2]))
    assert core[0] == 500.0 and core[1] == 500.0 and core[2] == abs(-10.0 * 1.2 + 400.0)


SYNTHETIC = os.path.join(os.path.dirname(__file__), "golden", "synthetic_fit.f90")


def synthetic_fit():
    """The fit of tests/golden/synthetic_fit.f90 built through the API."""
    c0 = Fraction(-25000000000000000000000000000001, 10 ** 27)  # -2.5...1Q4 to 106 bits
    hi = float(c0)
    coef = [(hi, float(c0 - Fraction(hi))), 1.0e6, float(np.float32(-0.1)), 3.0e6]
    return ep.series_potential(coef, 3, 1.5, 4.0e3, 2.0, -1.0e3, 0.0, 8.0e3, quad=True), c0


def test_reader_on_a_synthetic_source(lib):
    """Both names of the .Or. branch give the fit; its default-REAL literal
    -0.1 is binary32; the Q literal keeps its 32nd digit in c_lo."""
    want, c0 = synthetic_fit()
    w = want.series.contents
    for name in ("Test_fit", "Test_fit_alias"):
        p = ep.select_pot(name, 0.0, 0.0, SYNTHETIC)
        s = p.series.contents
        assert (s.k0, s.n, s.quad, s.r_core, s.f_core, s.r0, s.aa, s.bb, s.cc) == (
            3, 4, 1, 1.5, 4.0e3, 2.0, -1.0e3, 0.0, 8.0e3)
        assert list(s.c_hi[:4]) == list(w.c_hi[:4]) and s.c_lo[0] == w.c_lo[0] != 0.0
        assert s.c_hi[2] == float(np.float32(-0.1)) != -0.1
        x = np.linspace(1.0, 20.0, 200)
        assert np.array_equal(ep.potential_values(p, x), ep.potential_values(want, x))
    with pytest.raises(ep.EffPotError, match="inverse-power"):
        ep.select_pot("Other", 0.0, 0.0, SYNTHETIC)


def test_reader_on_the_other_two_forms(lib, oracle):
    """The synthetic file's even-power fit behind a forwarding function and
    its exponential fit with the x0 clamp (the forms of 'Ba_plus_old_gs' and
    'Cs_7s'), against their formulas."""
    p = ep.select_pot("Test_even", 0.0, 0.0, SYNTHETIC)
    assert p.kind == _abi.EP_POT_EVENPOW and p.series.contents.n == 3
    x = np.linspace(1.0, 12.0, 200)
    pg = [-2.0e3, 5.0e4, -1.0e5]
    want = np.where(x <= 2.0, 10.0 * x ** 2 - 5.0 * x + 100.0, sum(c / x ** (2 * k + 6) for k, c in enumerate(pg)))
    assert np.allclose(ep.potential_values(p, x), want, rtol=1e-14, atol=1e-13)
    assert np.allclose(oracle.potential_values(p, x), want, rtol=1e-14, atol=1e-13)
    p = ep.select_pot("Test_exp", 0.0, 0.0, SYNTHETIC)
    assert p.kind == _abi.EP_POT_EXPFIT and p.series.contents.r_core == 2.0
    xc = np.maximum(x, 2.0)
    ser = 3.0e3 * np.exp(-1.5 * xc) / xc - 10.0 * xc * np.exp(-0.5 * xc) + 0.2 * xc ** 2 * np.exp(-0.25 * xc)
    want = np.where(xc <= 2.5, xc ** 2 + 50.0, ser)
    assert np.allclose(ep.potential_values(p, x), want, rtol=1e-13, atol=1e-12)
    assert np.allclose(oracle.potential_values(p, x), want, rtol=1e-13, atol=1e-12)


def test_reader_survives_damaged_sources(lib, tmp_path):
    """Cut or gapped copies of a source (the synthetic one, and the
    reference's where present) give a potential or EP_ERR_INVALID_ARG, never
    a crash: every index the reader takes is checked against its statement."""
    import random
    rng = random.Random(7)
    texts = [(open(SYNTHETIC).read(), ["Test_fit", "Other"])]
    if os.path.exists(SOURCE):
        texts.append((open(SOURCE, encoding="latin-1").read(), ["Rb_gs_Fausto", "Cs_7s", "Ba_plus_old_gs"]))
    f = tmp_path / "v.f90"
    for text, names in texts:
        for trial in range(40):
            i = rng.randrange(len(text))
            j = min(len(text), i + rng.randrange(1, 400))
            cut = (text[:i], text[i:], text[:i] + text[j:])[trial % 3]
            f.write_text(cut, encoding="latin-1")
            for n in names:
                try:
                    p = ep.select_pot(n, 0.0, 0.0, str(f))
                    assert p.kind in (_abi.EP_POT_SERIES, _abi.EP_POT_EVENPOW, _abi.EP_POT_EXPFIT)
                    assert 1 <= p.series.contents.n <= _abi.EP_SERIES_MAX
                except ep.EffPotError as e:
                    assert e.status == 1


def test_select_pot_errors(lib):
    with pytest.raises(ep.EffPotError):
        ep.select_pot("No_such_potential", 0.0, 0.0, None)
    with pytest.raises(ep.EffPotError):
        ep.select_pot("Rb_gs_Fausto", 0.0, 0.0, None)  # a fit needs its source
    if os.path.exists(SOURCE):
        with pytest.raises(ep.EffPotError, match="not in the Select_Pot chain"):
            ep.select_pot("Cs_8s", 0.0, 0.0, SOURCE)
    p = ep.select_pot("Xe_He", 2.0, 21450.4867067095, None)
    assert p.kind == _abi.EP_POT_TANG_TOENNIES and p.r_cutoff == 2.0
    assert ep.potential_values(p, np.array([1.0]))[0] == 21450.4867067095


# ------------------------------------------------------------------- GPU
def _case(n=32, xmax=16.0, n4=200.0):
    cfg = ep.make_config(nx=n, ny=n, nz=n, xmax=xmax, ymax=xmax, zmax=xmax, icon=_abi.EP_ICON_PERIODIC,
                         core="OT ", n4=n4, impurity=_abi.EP_IMPURITY_FIXED)
    return cfg, ep.woods_saxon_psi(n, n, n, xmax, xmax, xmax, n4, seed=17)


def _fit():
    coef = [1e4 * math.comb(12, j) * (-2.0) ** j for j in range(13)]
    return ep.series_potential(coef, 5, 1.0, 500.0, 1.5, 0.0, -10.0, 400.0, quad=True)


@pytest.mark.gpu
def test_gpu_uplus_of_the_new_forms_matches_oracle(oracle):
    from eff_pot_gb300.build import build
    build()
    cfg, psi = _case()
    pluses = {"patil": ep.patil("RB", r_cutoff=2.0, umax=5000.0), "aziz": ep.aziz_he(r_cutoff=1.5, umax=2000.0),
              "tt": ep.tang_toennies("Xe", r_cutoff=2.0, umax=21450.4867067095), "series": _fit(),
              "ag": ep.select_pot("Ag_Pi", 1.0, 3000.0), "ba": ep.select_pot("Ba_gs"),
              "ch3i": ep.select_pot("CH3I_2"), "tio2": ep.select_pot("TiO2", 2.5, 1.887964e4),
              "au": ep.select_pot("Au", 1.0, 6.645232e4)}
    for name, plus in pluses.items():
        res = []
        for S in (ep.Solver, oracle.OracleSolver):
            with S(cfg) as s:
                m = ep.morse(10.0, 4.5, 1.2, umax=1000.0)
                s.set_impurity_potentials(m, m, plus)
                s.set_impurity(rimp=(0.3, -0.1, 0.45), invar=np.zeros(10, complex))
                s.start(psi)
                res.append(s.energy()["uplus"])
        assert abs(res[0] - res[1]) < 1e-10 * abs(res[1]), (name, res)


@pytest.mark.gpu
def test_gpu_series_channels_give_the_oracle_field(oracle):
    from eff_pot_gb300.build import build
    build()
    cfg, psi = _case()
    inv = np.zeros(10, complex)
    inv[0], inv[2] = 0.6, 0.8
    f = []
    for S in (ep.Solver, oracle.OracleSolver):
        with S(cfg) as s:
            s.set_impurity_potentials(_fit(), ep.patil("NA", r_cutoff=2.5, umax=3000.0), ep.null_potential())
            s.set_impurity(rimp=(0.4, 0.2, -0.3), invar=inv)
            s.start(psi)
            f.append((s.field("uimp"), s.energy()["eimpu"]))
    assert np.max(np.abs(f[0][0] - f[1][0])) < 1e-12 * np.max(np.abs(f[1][0]))
    assert abs(f[0][1] - f[1][1]) < 1e-10 * abs(f[1][1])
