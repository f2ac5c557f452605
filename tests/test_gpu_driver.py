"""The DFT4He3d driver on the GPU: namelist + readenc files in, the reference's
first energy balance out, equal to the same calls made through the Python
host mirror; evolution writes a printoutc file that reads back in mode 2."""
import os
import re
import subprocess

import numpy as np
import pytest

import eff_pot_gb300 as ep
from eff_pot_gb300 import _abi
from eff_pot_gb300.build import build, DRIVER

pytestmark = pytest.mark.gpu

N, XMAX, N4, DT = 32, 16.0, 200.0, 2.5e-4


@pytest.fixture(scope="module", autouse=True)
def _lib():
    build()
    ep.load_library()


def fmt(v):
    return f"{v:.17E}"


def write_density(path, den, rimp):
    """readenc mode 0: comment lines, header (limp, impurity position), den."""
    h = 2 * XMAX / N
    flat = np.asarray(den).ravel(order="F")
    with open(path, "w") as f:
        f.write("#  Density written for a test\n#  second comment line\n")
        f.write(" ".join(fmt(v) for v in (XMAX, XMAX, XMAX, h, h, h)) + f" {N} {N} {N} T "
                + " ".join(fmt(v) for v in rimp) + "\n")
        # a repeat count and both separators, as list-directed writers produce
        f.write(f" 2*{fmt(flat[0])}," if flat[0] == flat[1] else f" {fmt(flat[0])}, {fmt(flat[1])}")
        for i in range(2, flat.size):
            f.write((" " if i % 4 else "\n ") + fmt(flat[i]))
        f.write("\n")


def write_wavefunction(path, psi, rimp, vimp, invar):
    """readenc mode 2 (the printoutc layout)."""
    h = 2 * XMAX / N
    with open(path, "w") as f:
        f.write("#  Density after 0 iterations.\n#  Backup copy.\n")
        f.write(" ".join(fmt(v) for v in (XMAX, XMAX, XMAX, h, h, h)) + f" {N} {N} {N}\n")
        f.write(" ".join(fmt(v) for v in rimp) + "\n" + " ".join(fmt(v) for v in vimp) + "\n 10\n")
        f.write(" ".join(f"({fmt(z.real)},{fmt(z.imag)})" for z in invar) + "\n")
        for i, z in enumerate(np.asarray(psi).ravel(order="F")):
            f.write(f" ({fmt(z.real)},{fmt(z.imag)})" + ("\n" if i % 2 else ""))
        f.write("\n")


def namelist(mode, extra=""):
    return (f"&input\n title='driver test', n4={int(N4)}, mode={mode},\n"
            f" nx={N}, ny={N}, nz={N}, xmax={XMAX}, ymax={XMAX}, zmax={XMAX},\n"
            " core4='OTC', npd=13, icon=8, deltat=2.5d-4, mimpur=40.d0, Lfix_lambda=.true.,\n"
            " selec_pi='Morse', selec_sigma='Morse', selec_plus='null', umax_pi=1000.d0, umax_sigma=1000.d0,\n"
            " r_cutoff_pi=0.d0, r_cutoff_sigma=0.d0, morse_de=10.d0, morse_re=4.5d0, morse_alpha=1.2d0,\n"
            f" filedenin='in.dat', filedenout='out.dat' {extra}\n/\n")


def run_driver(cwd, text):
    r = subprocess.run([DRIVER], input=text, cwd=cwd, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout


LABELS = {"etot4": "TOTAL   energy (He)", "ekin4": "Kinetic energy (He)", "elj4": "Lennard-Jones energy (He)",
          "ealphas": "Alpha_s term  energy (He)", "esolid": "Solid energy (He)", "ecor4": "Correlation energy   (He)",
          "eHeX": "Interaction energy (X*-He)", "etot": "TOTAL ENERGY (He+X)"}


def balance(out):
    vals = {}
    for k, lab in LABELS.items():
        m = re.search(re.escape(lab) + r" +\.*: +(-?\d+\.\d+) K", out)
        assert m, (k, out)
        vals[k] = m.group(1)
    return vals


def solver(rimp, invar, vimp=(0.0, 0.0, 0.0)):
    cfg = ep.make_config(nx=N, ny=N, nz=N, xmax=XMAX, ymax=XMAX, zmax=XMAX, icon=_abi.EP_ICON_PERIODIC, core="OTC",
                         n4=N4, impurity=_abi.EP_IMPURITY_MOVING, mimpur=40.0, fix_lambda=1)
    s = ep.Solver(cfg)
    m = ep.morse(10.0, 4.5, 1.2, r_cutoff=0.0, umax=1000.0)
    s.set_impurity_potentials(m, m, ep.null_potential())
    s.set_impurity(rimp=rimp, vimp=vimp, invar=invar)
    return s


def test_first_energy_balance_mode0(tmp_path):
    psi = ep.woods_saxon_psi(N, N, N, XMAX, XMAX, XMAX, N4, seed=3)
    den = np.abs(psi) ** 2
    rimp = (0.5, -0.25, 1.0)
    write_density(tmp_path / "in.dat", den, rimp)
    (tmp_path / "invar.dat").write_text("\n".join(["(0.d0,0.d0)"] * 10) + "\n")
    got = balance(run_driver(tmp_path, namelist(0, ", instate=5")))
    with solver(rimp, np.zeros(10, dtype=np.complex128)) as s:
        s.upload_psi(np.sqrt(den).astype(np.complex128))
        s.potenimp()
        s.poten()
        e = s.energy()
    for k, v in got.items():
        assert v == f"{e[k]:.6f}", (k, v, e[k])
    # the namelist echo
    assert "core4 = OTC" in (tmp_path / "DFT4He3d.namelist.read").read_text()


def test_mode2_evolution_writes_a_file_that_reads_back(tmp_path):
    psi = ep.woods_saxon_psi(N, N, N, XMAX, XMAX, XMAX, N4, seed=4)
    rimp = (0.0, 0.0, 0.75)
    invar = np.zeros(10, dtype=np.complex128)
    write_wavefunction(tmp_path / "in.dat", psi, rimp, (0.0, 0.0, 0.0), invar)
    out = run_driver(tmp_path, namelist(2, ", niter=10, pener=4"))
    rows = [ln.split() for ln in out.splitlines() if re.match(r"^\s+\d+ +-?\d+\.\d+ +-?\d+\.\d+ ", ln)]
    assert [int(r[0]) for r in rows] == [7, 10]
    with solver(rimp, invar) as s:
        s.upload_psi(psi)
        s.potenimp()
        s.poten()
        s.energy()
        s.forceimp()  # as the driver does after the first balance
        for _ in range(3):
            s.steprk(DT)
        s.run(4, DT)
        s.poten()  # the driver prints the energy after every pener steps
        s.energy()
        st = s.run(3, DT)
        s.poten()
        e = s.energy()
        final = s.psi()
        imp = s.impurity()
    assert rows[-1][1] == f"{st['mu']:.10f}" and rows[-1][2] == f"{e['etot']:.10f}"
    # the printoutc file of the run is a valid mode-2 input holding the final state
    text = (tmp_path / "out.dat").read_text()
    assert re.match(r"#  Density after +10 iterations\.\n#  Actual delatatps", text)
    os.replace(tmp_path / "out.dat", tmp_path / "in.dat")
    got = balance(run_driver(tmp_path, namelist(2)))
    with solver(tuple(imp["rimp"]), imp["invar"], tuple(imp["vimp"])) as s:
        s.upload_psi(final)
        s.potenimp()
        s.poten()
        e2 = s.energy()
    assert got["etot"] == f"{e2['etot']:.6f}"


def per_file_line(cwd, path):
    """get_impurity_energy.sh with this driver: run on one file, pick the awk
    fields it picks, print them with its printf."""
    out = run_driver(cwd, namelist(2).replace("filedenin='in.dat'", f"filedenin='{path}'"))
    with open(path) as f:
        head = [next(f) for _ in range(3)]
    t = float([ln.split()[4] for ln in head if "Total evolution time" in ln][0].replace("D", "E"))

    def field(pat, k):
        return float([ln.split()[k - 1] for ln in out.splitlines() if re.search(pat, ln)][0])
    vals = (field(r"X-HE CoM distance", 4), field(r"Kinetic energy \(X", 5), field(r"Interaction energy \(X\*", 5),
            field(r"Interaction energy \(X\+", 5), field(r"Spin-Orbit energy", 5))
    return "%.1f\t\t%f\t%f\t%f\t%f\t%f" % ((t,) + vals)


def test_scan_matches_per_file_runs(tmp_path):
    files = []
    for k, z in enumerate((0.0, 1.5, 3.0)):
        psi = ep.woods_saxon_psi(N, N, N, XMAX, XMAX, XMAX, N4, seed=20 + k)
        p = tmp_path / f"density.{k}.out"
        write_wavefunction(p, psi, (0.0, 0.0, z), (0.0, 0.0, 0.1 * k), np.zeros(10, dtype=np.complex128))
        # the evolution time loop.sh reads from the third line
        lines = p.read_text().splitlines(True)
        lines.insert(2, f"#  Total evolution time(ps)...:  {2.5 * k:.12E}\n")
        p.write_text("".join(lines))
        files.append(str(p))
    r = subprocess.run([DRIVER, "--scan", *files], input=namelist(2), cwd=tmp_path, capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    table = [ln for ln in r.stdout.splitlines() if ln and not ln.startswith("#") and "\t" in ln]
    assert r.stdout.splitlines()[1].startswith("# time (ps)")
    assert len(table) == 3
    for line, f in zip(table, files):
        assert line == per_file_line(tmp_path, f)


def test_impurity_moments_match_the_oracle():
    from oracle import pyoracle
    psi = ep.woods_saxon_psi(N, N, N, XMAX, XMAX, XMAX, N4, seed=6)
    rimp = (0.7, -0.4, 1.1)
    cfg = ep.make_config(nx=N, ny=N, nz=N, xmax=XMAX, ymax=XMAX, zmax=XMAX, icon=_abi.EP_ICON_PERIODIC, core="OTC",
                         n4=N4, impurity=_abi.EP_IMPURITY_MOVING, mimpur=40.0, fix_lambda=1)
    m1 = ep.morse(10.0, 4.5, 1.2, r_cutoff=0.0, umax=1000.0)
    m2 = ep.morse(25.0, 4.0, 1.1, r_cutoff=0.0, umax=1000.0)  # sigma != pi: an anisotropic field
    res = []
    for S in (ep.Solver, pyoracle.OracleSolver):
        with S(cfg) as s:
            s.set_impurity_potentials(m1, m2, ep.null_potential())
            s.set_impurity(rimp=rimp, invar=np.zeros(10, dtype=np.complex128))
            s.upload_psi(psi)
            s.potenimp()
            res.append(s.impurity_moments())
    assert np.allclose(res[0], res[1], rtol=1e-11, atol=1e-11 * np.abs(res[1]).max())
    assert abs(res[1][3]) > 0  # off-diagonal moments are exercised


def test_p_state_instate_matches_the_api(tmp_path):
    psi = ep.woods_saxon_psi(N, N, N, XMAX, XMAX, XMAX, N4, seed=7)
    den = np.abs(psi) ** 2
    rimp = (0.3, 0.2, -0.6)
    write_density(tmp_path / "in.dat", den, rimp)
    for instate in (0, 1):
        out = run_driver(tmp_path, namelist(0, f", instate={instate}, Als_P=5.d0"))
        got = balance(out)
        eso = float(re.search(r"Spin-Orbit energy \(X\) \.*: +(-?\d+\.\d+) K", out).group(1))
        cfg = ep.make_config(nx=N, ny=N, nz=N, xmax=XMAX, ymax=XMAX, zmax=XMAX, icon=_abi.EP_ICON_PERIODIC,
                             core="OTC", n4=N4, impurity=_abi.EP_IMPURITY_MOVING, mimpur=40.0, fix_lambda=1,
                             als_p=5.0)
        with ep.Solver(cfg) as s:
            m = ep.morse(10.0, 4.5, 1.2, r_cutoff=0.0, umax=1000.0)
            s.set_impurity_potentials(m, m, ep.null_potential())
            s.set_impurity(rimp=rimp, invar=np.zeros(10, dtype=np.complex128))
            s.upload_psi(np.sqrt(den).astype(np.complex128))
            s.potenimp()
            vx, vy, vz, vxy, vxz, vyz = s.impurity_moments()
            M = np.zeros((6, 6), complex)
            for (i, j), v in {(0, 0): vx, (1, 1): vx, (2, 2): vy, (3, 3): vy, (4, 4): vz, (5, 5): vz,
                              (0, 2): vxy, (1, 3): vxy, (0, 4): vxz, (1, 5): vxz, (2, 4): vyz, (3, 5): vyz}.items():
                M[i, j] = M[j, i] = v
            so = {(0, 2): -1j, (1, 3): 1j, (1, 4): -1, (0, 5): 1, (3, 4): -1j, (2, 5): -1j}
            for (i, j), v in so.items():
                M[i, j] += 2.5 * v
                M[j, i] += 2.5 * np.conj(v)
            w, V = np.linalg.eigh(M)
            iv = np.zeros(10, complex)
            iv[:6] = (V[:, 2 * instate] + V[:, 2 * instate + 1]) / np.sqrt(2)
            s.set_impurity(rimp=rimp, invar=iv)
            s.potenimp()
            s.poten()
            e = s.energy()
        # energies do not depend on the basis inside the Kramers pair
        for k, v in got.items():
            assert abs(float(v) - e[k]) < 2e-6, (instate, k, v, e[k])
        assert abs(eso - e["eso"]) < 2e-6
        assert abs(e["eso"] - 5.0 * (-1.0 if instate == 0 else 0.5)) < 0.3  # j = 1/2 vs 3/2 level


def test_tabulated_pair_potentials_equal_the_formula(tmp_path):
    """selec_* = 'table' with (r, V) files on potenimpini's knots gives the
    energies of the same potential selected by name."""
    psi = ep.woods_saxon_psi(N, N, N, XMAX, XMAX, XMAX, N4, seed=8)
    write_density(tmp_path / "in.dat", np.abs(psi) ** 2, (0.2, 0.1, 0.4))
    (tmp_path / "invar.dat").write_text("\n".join(["(0.d0,0.d0)"] * 10) + "\n")
    npot = 100 * N + 1
    dr = 4.0 * XMAX / (npot - 1)
    r = np.arange(npot) * dr
    v = 10.0 * (1.0 - np.exp(-1.2 * (r - 4.5))) ** 2 - 10.0
    with open(tmp_path / "morse.tab", "w") as f:
        f.write("# r (A)  V (K)\n")
        for a, b in zip(r, v):
            f.write(f"{a:.17E} {b:.17E}\n")
    by_name = balance(run_driver(tmp_path, namelist(0, ", instate=5")))
    tab = namelist(0, ", instate=5, selec_pi='table', selec_sigma='table', table_pi='morse.tab', "
                      "table_sigma='morse.tab'")
    by_table = balance(run_driver(tmp_path, tab))
    for k in by_name:
        assert abs(float(by_name[k]) - float(by_table[k])) <= 2e-6, (k, by_name[k], by_table[k])
    assert abs(float(by_table["eHeX"])) > 1.0  # the impurity field is not trivial


def _sod():
    """SOD of potenimp.f90:429-451, restated: the listed upper triangle plus
    its conjugate transpose."""
    S = np.zeros((10, 10), complex)
    s3 = np.sqrt(3.0)
    for (i, j), v in {(1, 4): 1, (1, 8): -1j, (1, 9): 2j, (2, 3): -1, (2, 7): -1j, (2, 10): -2j,
                      (3, 6): -1j * s3, (3, 7): 1j, (3, 10): -1j, (4, 5): -1j * s3, (4, 8): -1j, (4, 9): -1j,
                      (5, 8): -s3, (6, 7): s3, (7, 10): -1, (8, 9): 1}.items():
        S[i - 1, j - 1] = v
    return S + S.conj().T


def test_d_state_instate_matches_the_api(tmp_path):
    """Lstate='D': the driver builds invar from the field matrix and SOD
    (instates.f90:440-647, default branch) as the host mirror does with
    numpy; three different tabulated channels make the field anisotropic."""
    psi = ep.woods_saxon_psi(N, N, N, XMAX, XMAX, XMAX, N4, seed=9)
    den = np.abs(psi) ** 2
    rimp = (0.4, -0.3, 0.9)
    write_density(tmp_path / "in.dat", den, rimp)
    npot = 100 * N + 1
    r = np.arange(npot) * (4.0 * XMAX / (npot - 1))
    chans = {"pi": (10.0, 4.5, 1.2), "sigma": (25.0, 4.0, 1.1), "delta": (6.0, 5.0, 1.0)}
    for name, (de, re_, al) in chans.items():
        e = np.exp(-al * (r - re_))
        with open(tmp_path / f"{name}.tab", "w") as f:
            for a, b in zip(r, de * (e * e - 2.0 * e)):
                f.write(f"{a:.17E} {b:.17E}\n")
    als = 4.0
    extra = (", Lstate='D', Als_D=4.d0, selec_pi='table', selec_sigma='table', selec_delta='table', "
             "table_pi='pi.tab', table_sigma='sigma.tab', table_delta='delta.tab', umax_delta=1000.d0")
    for instate in (0, 2):
        out = run_driver(tmp_path, namelist(0, f", instate={instate}" + extra))
        got = balance(out)
        eso = float(re.search(r"Spin-Orbit energy \(X\) \.*: +(-?\d+\.\d+) K", out).group(1))
        cfg = ep.make_config(nx=N, ny=N, nz=N, xmax=XMAX, ymax=XMAX, zmax=XMAX, icon=_abi.EP_ICON_PERIODIC,
                             core="OTC", n4=N4, impurity=_abi.EP_IMPURITY_MOVING, mimpur=40.0, fix_lambda=1,
                             state=_abi.EP_STATE_D, als_d=als)
        with ep.Solver(cfg) as s:
            pots = [ep.morse(*chans[c], r_cutoff=0.0, umax=1000.0) for c in ("pi", "sigma", "delta")]
            s.set_impurity_potentials_d(*pots, ep.null_potential())
            s.set_impurity(rimp=rimp, invar=np.zeros(10, dtype=np.complex128))
            s.upload_psi(np.sqrt(den).astype(np.complex128))
            s.potenimp()
            M = s.impurity_matrix_d()
            w, V = np.linalg.eigh(np.kron(M, np.eye(2)) + 0.5 * als * _sod())
            iv = (V[:, 2 * instate] + V[:, 2 * instate + 1]) / np.sqrt(2)
            s.set_impurity(rimp=rimp, invar=iv)
            s.potenimp()
            s.poten()
            e = s.energy()
        assert abs(w[2 * instate] - w[2 * instate + 1]) < 1e-9 * max(1.0, abs(w).max())  # a Kramers pair
        for k, v in got.items():
            assert abs(float(v) - e[k]) < 2e-6, (instate, k, v, e[k])
        assert abs(eso - e["eso"]) < 2e-6
        assert abs(float(got["eHeX"])) > 1.0


def test_scan_settings_of_prep_sh_give_the_api_uplus(tmp_path):
    """selec_plus='Rb_plus_Koutselos', r_cutoff_plus=2, umax_plus=6110.59...
    (the settings prep.sh writes) give the U+ the ABI computes."""
    psi = ep.woods_saxon_psi(N, N, N, XMAX, XMAX, XMAX, N4, seed=10)
    den = np.abs(psi) ** 2
    rimp = (0.6, 0.2, -0.8)
    write_density(tmp_path / "in.dat", den, rimp)
    (tmp_path / "invar.dat").write_text("\n".join(["(0.d0,0.d0)"] * 10) + "\n")
    text = namelist(0, ", instate=5").replace(
        "selec_plus='null'", "selec_plus='Rb_plus_Koutselos', r_cutoff_plus=2.d0, umax_plus=6.1105922888E+03")
    out = run_driver(tmp_path, text)
    m = re.search(r"Interaction energy \(X\+-He\) \.*: +(-?\d+\.\d+) K", out)
    assert m, out
    s = solver(rimp, np.zeros(10, dtype=np.complex128))
    with s:
        m_ = ep.morse(10.0, 4.5, 1.2, r_cutoff=0.0, umax=1000.0)
        s.set_impurity_potentials(m_, m_, ep.koutselos("Rb", r_cutoff=2.0, umax=6.1105922888e3))
        s.upload_psi(np.sqrt(den).astype(np.complex128))
        s.potenimp()
        s.poten()
        e = s.energy()
    assert abs(float(m.group(1)) - e["uplus"]) < 2e-6
    assert abs(e["uplus"]) > 1.0


def test_named_potentials_through_the_namelist(tmp_path):
    """selec_pi='Xe_He', selec_sigma='RB' (closed forms built into the
    library) and selec_plus='Test_fit', an inverse-power fit read from the
    file named by potentials_source: the driver's eHeX and U+ equal the ABI's
    with the same potentials built through the Python API."""
    from test_select_pot import SYNTHETIC, synthetic_fit
    psi = ep.woods_saxon_psi(N, N, N, XMAX, XMAX, XMAX, N4, seed=12)
    den = np.abs(psi) ** 2
    rimp = (0.4, -0.3, 0.6)
    write_density(tmp_path / "in.dat", den, rimp)
    (tmp_path / "invar.dat").write_text("\n".join(["(0.d0,0.d0)"] * 10) + "\n")
    text = namelist(0, f", instate=5, potentials_source='{SYNTHETIC}'").replace(
        "selec_pi='Morse', selec_sigma='Morse', selec_plus='null', umax_pi=1000.d0, umax_sigma=1000.d0,\n"
        " r_cutoff_pi=0.d0, r_cutoff_sigma=0.d0,",
        "selec_pi='Xe_He', selec_sigma='RB', selec_plus='Test_fit', umax_pi=2.1450E+04, umax_sigma=5.d3,\n"
        " r_cutoff_pi=2.d0, r_cutoff_sigma=2.5d0, r_cutoff_plus=0.d0, umax_plus=0.d0,")
    out = run_driver(tmp_path, text)
    m = re.search(r"Interaction energy \(X\+-He\) \.*: +(-?\d+\.\d+) K", out)
    assert m, out
    got = balance(out)
    s = solver(rimp, np.zeros(10, dtype=np.complex128))
    with s:
        s.set_impurity_potentials(ep.tang_toennies("Xe", r_cutoff=2.0, umax=2.1450e4),
                                  ep.patil("RB", r_cutoff=2.5, umax=5.0e3), synthetic_fit()[0])
        s.upload_psi(np.sqrt(den).astype(np.complex128))
        s.potenimp()
        s.poten()
        e = s.energy()
    assert abs(float(m.group(1)) - e["uplus"]) < 2e-6 and abs(e["uplus"]) > 1e-3
    assert abs(float(got["eHeX"]) - e["eHeX"]) < 2e-6 and abs(e["eHeX"]) > 1e-3


def test_ldiag_jz_namelist_selects_the_jz_state(tmp_path):
    """Ldiag_jz=.true., Ljz='+3/2' in an isotropic field (V_Sigma = V_Pi):
    the internal variables the driver writes (printoutc, frozen by
    Lfix_lambda) are the Jz = +3/2 member of the j = 3/2 level."""
    psi = ep.woods_saxon_psi(N, N, N, XMAX, XMAX, XMAX, N4, seed=11)
    write_density(tmp_path / "in.dat", np.abs(psi) ** 2, (0.3, -0.2, 0.5))
    run_driver(tmp_path, namelist(0, ", instate=1, Als_P=4.d0, Ldiag_jz=.true., Ljz='+3/2', niter=1"))
    text = (tmp_path / "out.dat").read_text()
    z = re.findall(r"\(([-+0-9.E]+),([-+0-9.E]+)\)", text)[:10]
    iv = np.array([complex(float(a), float(b)) for a, b in z])
    J = np.zeros((6, 6), complex)
    for (i, j), v in {(1, 1): .5, (1, 3): -1j, (2, 2): -.5, (2, 4): -1j, (3, 1): 1j, (3, 3): .5, (4, 2): 1j,
                      (4, 4): -.5, (5, 5): .5, (6, 6): -.5}.items():
        J[i - 1, j - 1] = v
    assert abs(np.vdot(iv, iv) - 1.0) < 1e-10 and np.all(iv[6:] == 0)
    assert np.allclose(J @ iv[:6], 1.5 * iv[:6], atol=1e-9)
