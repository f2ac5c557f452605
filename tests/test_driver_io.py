"""The Fortran I/O of the DFT4He3d driver (namelist, list-directed text,
unformatted records) and its input checks that stop before any GPU call.

The I/O module is compiled here with a small harness; the driver itself is
built by build() and run on inputs that it must reject the way the reference
does (DFT4He3d.f90:176-196, readenc.f90:170-245).
"""
import os
import struct
import subprocess
import textwrap

import numpy as np

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DRV = os.path.join(ROOT, "eff_pot_gb300", "csrc", "driver")

HARNESS = r"""
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <sstream>
#include "ep_fortran_io.h"
#include "ep_instates.h"
int main(int argc, char** argv) {
  std::string what = argv[1];
  if (what == "nml") {
    fio::Namelist n; std::string err;
    std::ifstream f(argv[2]);
    if (!fio::parse_namelist(f, "input", n, err)) { std::printf("ERR %s\n", err.c_str()); return 0; }
    for (auto& k : n.order) {
      std::printf("%s", k.c_str());
      for (auto& v : n.vars[k]) std::printf("|%s", v.c_str());
      std::printf("\n");
    }
    std::printf("real=%.17g int=%ld log=%d\n", fio::to_real(n.vars["a"][0]), fio::to_int(n.vars["n"][0]),
                (int)fio::to_logical(n.vars["flag"][0]));
  } else if (what == "list") {
    std::ifstream f(argv[2]);
    fio::ListReader r(f);
    r.skip_comments('#');
    double h[3]; long n; bool l; double c[6];
    r.reals(h, 3); r.integer(n); r.logical(l); r.end_statement();
    r.complexes(c, 3); r.end_statement();
    double tail[4]; r.reals(tail, 4);
    std::printf("%.17g %.17g %.17g %ld %d\n", h[0], h[1], h[2], n, (int)l);
    for (double v : c) std::printf("%.17g ", v);
    std::printf("\n");
    for (double v : tail) std::printf("%.17g ", v);
    std::printf("\n");
  } else if (what == "eig") {
    // moments and Als from the command line; prints the P matrix, eigenvalues,
    // eigenvectors (column-major re im) and the invar of instate 0, 1, 2
    double m[6]; for (int i = 0; i < 6; ++i) m[i] = std::atof(argv[2 + i]);
    const double als = std::atof(argv[8]);
    auto M = instates::p_matrix(m, als);
    for (auto z : M) std::printf("%.17g %.17g ", z.real(), z.imag());
    std::printf("\n");
    std::vector<double> w; std::vector<std::complex<double>> v;
    instates::hermitian_eigen(6, M, w, v);
    for (double x : w) std::printf("%.17g ", x);
    std::printf("\n");
    for (int k = 0; k < 6; ++k) for (int i = 0; i < 6; ++i) std::printf("%.17g %.17g ", v[i * 6 + k].real(), v[i * 6 + k].imag());
    std::printf("\n");
    for (int st = 0; st < 3; ++st) {
      double iv[20]; instates::p_state(m, als, st, iv);
      for (double x : iv) std::printf("%.17g ", x);
      std::printf("\n");
    }
  } else if (what == "jz") {
    // argv: state (P|D), Als, instate, Ljz ('-' for the default), then the 6
    // P moments or the 25 entries of the D field matrix; prints invar
    const bool d = std::string(argv[2]) == "D";
    const double als = std::atof(argv[3]);
    const int st = std::atoi(argv[4]);
    const std::string ljz = std::string(argv[5]) == "-" ? "" : argv[5];
    int ki, njz, il;
    instates::jz_selection(d, st, ljz, ki, njz, il);
    if (il < 0) { std::printf("BAD\n"); return 0; }
    double m[25]; for (int i = 0; i < (d ? 25 : 6); ++i) m[i] = std::atof(argv[6 + i]);
    double iv[20];
    if (d) instates::d_state(m, als, st, iv, ki, njz, il);
    else instates::p_state(m, als, st, iv, ki, njz, il);
    for (double x : iv) std::printf("%.17g ", x);
    std::printf("\n");
  } else if (what == "rec") {
    std::ofstream o(argv[2], std::ios::binary);
    double v[3] = {1.5, -2.25, 3.0}; int k = 7;
    fio::write_record(o, v, sizeof v); fio::write_record(o, &k, sizeof k);
    o.close();
    std::ifstream i(argv[2], std::ios::binary);
    std::vector<char> a, b;
    const int ra = fio::read_record(i, a);
    const int rb = fio::read_record(i, b);
    std::printf("%d %d %zu %zu\n", ra, rb, a.size(), b.size());
  }
  return 0;
}
"""


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    d = tmp_path_factory.mktemp("fio")
    src = d / "h.cpp"
    src.write_text(HARNESS)
    exe = d / "h"
    subprocess.check_call(["g++", "-O1", "-std=c++17", "-I" + DRV, str(src), os.path.join(DRV, "ep_fortran_io.cpp"),
                           "-o", str(exe)])
    return str(exe)


def run(exe, *a):
    return subprocess.run([exe, *map(str, a)], check=True, capture_output=True, text=True).stdout


def test_namelist_forms(harness, tmp_path):
    f = tmp_path / "in.nml"
    f.write_text(textwrap.dedent("""\
        ! comment before the group
        &INPUT  title='He droplet, ''test''' , N=300
           a = 1.5d-3   flag = .True.   core4 = 'OTC'   ! trailing comment
           xs = 3*2.0, 1.0E2  , vals=2*'ab'
           z = (1.0, -2.0)
        /
        """))
    out = run(harness, "nml", f).splitlines()
    assert out[0] == "title|He droplet, 'test'"
    assert out[1] == "n|300"
    assert "core4|OTC" in out
    assert "xs|2.0|2.0|2.0|1.0E2" in out
    assert "vals|ab|ab" in out
    assert "z|(1.0,-2.0)" in out
    assert out[-1] == "real=0.0015 int=300 log=1"


def test_namelist_end_forms_and_errors(harness, tmp_path):
    f = tmp_path / "a.nml"
    f.write_text("$input n = 2, a = 1, flag = F $end\n")
    assert run(harness, "nml", f).splitlines()[-1] == "real=1 int=2 log=0"
    f.write_text("&other x=1 /\n")
    assert run(harness, "nml", f).startswith("ERR namelist group &input not found")
    f.write_text("&input n = 2\n")
    assert "not terminated" in run(harness, "nml", f)


def test_list_directed_reader(harness, tmp_path):
    f = tmp_path / "d.txt"
    f.write_text("# header line\n#  another\n 25.6D0, 25.6 ,0.4 64 T extra values ignored\n"
                 " (1.0,2.0) 2*( 3.5 ,\n -4.0 )\n 3*0.25 7.0\n")
    out = run(harness, "list", f).splitlines()
    assert out[0] == "25.600000000000001 25.600000000000001 0.40000000000000002 64 1"
    assert out[1].split() == ["1", "2", "3.5", "-4", "3.5", "-4"]
    assert out[2].split() == ["0.25", "0.25", "0.25", "7"]


def test_unformatted_records(harness, tmp_path):
    f = tmp_path / "r.bin"
    assert run(harness, "rec", f).split() == ["1", "1", "24", "4"]
    raw = f.read_bytes()
    assert struct.unpack("<i", raw[:4])[0] == 24 and struct.unpack("<i", raw[28:32])[0] == 24
    assert struct.unpack("<3d", raw[4:28]) == (1.5, -2.25, 3.0)


@pytest.fixture(scope="module")
def driver():
    from eff_pot_gb300.build import build, DRIVER
    build()
    return DRIVER


def drive(driver, cwd, text):
    return subprocess.run([driver], input=text, cwd=cwd, capture_output=True, text=True, timeout=120)


def test_driver_time_step_checks(driver, tmp_path):
    r = drive(driver, tmp_path, "&input nx=32, ny=32, nz=32 /\n")
    assert r.returncode == 1
    assert "You must specify either Deltat (in kelvin) or Deltatps (in picosecond)" in r.stdout
    echo = (tmp_path / "DFT4He3d.namelist.read").read_text()
    assert "nx = 32" in echo and echo.startswith("&INPUT")
    r = drive(driver, tmp_path, "&input deltat=1.d-4, deltatps=1.0 /\n")
    assert r.returncode == 1 and "Inconsistent deltat - deltatps" in r.stdout


def test_driver_rejects_unknown_core_and_bad_namelist(driver, tmp_path):
    r = drive(driver, tmp_path, "&input deltat=1.d-4, core4='XYZ' /\n")
    assert r.returncode == 1 and "I do not know how to work with the core: XYZ" in r.stdout
    r = drive(driver, tmp_path, "&input deltat=1.d-4, nx = 'abc' /\n")
    assert r.returncode == 1 and "Error in input master file" in r.stdout
    r = drive(driver, tmp_path, "no namelist here\n")
    assert r.returncode == 1 and "Error in input master file" in r.stdout


def test_driver_resolves_pair_potentials_before_the_gpu(driver, tmp_path):
    """selec_* names go through Select_Pot's registry before any device
    work: unknown names, fits without potentials_source and unknown names in
    a given source stop the run with the registry's message."""
    base = "&input deltat=1.d-4, selec_pi='Morse', selec_sigma='Morse', selec_plus='null', {} /\n"
    r = drive(driver, tmp_path, base.format("selec_plus='No_such_pot'"))
    assert r.returncode == 1 and "selec_plus='No_such_pot'" in r.stdout and "built in:" in r.stdout
    r = drive(driver, tmp_path, base.format("selec_pi='Rb_gs_Fausto'"))
    assert r.returncode == 1 and "give the V_impur.f90 source" in r.stdout
    src = os.path.join(os.path.dirname(__file__), "golden", "synthetic_fit.f90")
    r = drive(driver, tmp_path, base.format(f"selec_sigma='Other', potentials_source='{src}'"))
    assert r.returncode == 1 and "is not an inverse-power fit" in r.stdout
    r = drive(driver, tmp_path, base.format("potentials_source='/nonexistent/V_impur.f90', selec_pi='Test_fit'"))
    assert r.returncode == 1 and "cannot read" in r.stdout


def test_p_state_eigenvectors(harness):
    """The Jacobi eigen-solver of the P-state matrix V + (Als/2) SO
    (instates.f90:150-193): eigenpairs of the Hermitian matrix, Kramers
    pairs, and the j = 1/2 / 3/2 levels V0 - Als, V0 + Als/2 of an
    isotropic field; invar = (v_2k + v_2k+1)/sqrt(2) lies in the pair."""
    import numpy as np
    for m, als in (([-3.0, -2.5, -2.0, 0.3, -0.2, 0.1], 4.0), ([-5.0, -5.0, -5.0, 0.0, 0.0, 0.0], 6.0)):
        out = run(harness, "eig", *m, als).splitlines()
        M = np.array([float(x) for x in out[0].split()]).view(np.complex128).reshape(6, 6)
        assert np.allclose(M, M.conj().T)
        w = np.array([float(x) for x in out[1].split()])
        V = np.array([float(x) for x in out[2].split()]).view(np.complex128).reshape(6, 6).T
        assert np.allclose(w, np.linalg.eigvalsh(M), atol=1e-13)
        assert np.allclose(M @ V, V * w, atol=1e-12)
        assert np.allclose(V.conj().T @ V, np.eye(6), atol=1e-13)
        assert np.allclose(w[0::2], w[1::2], atol=1e-12)  # Kramers pairs
        for st in range(3):
            iv = np.array([float(x) for x in out[3 + st].split()]).view(np.complex128)
            assert abs(np.vdot(iv, iv) - 1.0) < 1e-13 and np.all(iv[6:] == 0)
            assert np.allclose(M @ iv[:6], w[2 * st] * iv[:6], atol=1e-12)
        if m[3] == 0.0:
            assert np.allclose(w, [m[0] - als] * 2 + [m[0] + als / 2] * 4, atol=1e-12)


def _jz(nd):
    """Jz = Lz + Sz over the internal variables, restated from the matrix
    elements instates.f90 writes (P :246-258, D :632-651)."""
    J = np.zeros((nd, nd), complex)
    ent = ({(1, 1): .5, (1, 3): -1j, (2, 2): -.5, (2, 4): -1j, (3, 1): 1j, (3, 3): .5, (4, 2): 1j, (4, 4): -.5,
            (5, 5): .5, (6, 6): -.5} if nd == 6 else
           {(9, 9): .5, (9, 1): -2j, (10, 10): -.5, (10, 2): -2j, (3, 3): .5, (3, 7): 1j, (4, 4): -.5, (4, 8): 1j,
            (5, 5): .5, (6, 6): -.5, (7, 3): -1j, (7, 7): .5, (8, 4): -1j, (8, 8): -.5, (1, 9): 2j, (1, 1): .5,
            (2, 10): 2j, (2, 2): -.5})
    for (i, j), v in ent.items():
        J[i - 1, j - 1] = v
    return J


def _state_matrix(d, m, als):
    """P: V + (Als/2) SO (instates.f90:150-193); D: M (x) 1_2 + (Als/2) SOD."""
    if not d:
        vx, vy, vz, vxy, vxz, vyz = m
        M = np.zeros((6, 6), complex)
        for (i, j), v in {(0, 0): vx, (1, 1): vx, (2, 2): vy, (3, 3): vy, (4, 4): vz, (5, 5): vz, (0, 2): vxy,
                          (1, 3): vxy, (0, 4): vxz, (1, 5): vxz, (2, 4): vyz, (3, 5): vyz}.items():
            M[i, j] = M[j, i] = v
        for (i, j), v in {(0, 2): -1j, (1, 3): 1j, (1, 4): -1, (0, 5): 1, (3, 4): -1j, (2, 5): -1j}.items():
            M[i, j] += 0.5 * als * v
            M[j, i] += 0.5 * als * np.conj(v)
        return M
    S = np.zeros((10, 10), complex)
    s3 = np.sqrt(3.0)
    for (i, j), v in {(1, 4): 1, (1, 8): -1j, (1, 9): 2j, (2, 3): -1, (2, 7): -1j, (2, 10): -2j, (3, 6): -1j * s3,
                      (3, 7): 1j, (3, 10): -1j, (4, 5): -1j * s3, (4, 8): -1j, (4, 9): -1j, (5, 8): -s3,
                      (6, 7): s3, (7, 10): -1, (8, 9): 1}.items():
        S[i - 1, j - 1] = v
    S = S + S.conj().T
    return np.kron(np.asarray(m).reshape(5, 5), np.eye(2)) + 0.5 * als * S


@pytest.mark.parametrize("d", [False, True])
def test_ldiag_jz_picks_the_requested_jz_state(harness, d):
    """Ldiag_jz (instates.f90:228-300, :613-690): the state is the eigenvector
    of Jz restricted to the selected j manifold of the state matrix with the
    requested <Jz>; in an isotropic field it is an exact Jz eigenstate with
    <Jz> = m_j.  Checked against numpy for both states, isotropic and
    anisotropic fields, every Ljz and the reference's defaults."""
    rng = np.random.default_rng(3)
    nd = 10 if d else 6
    if d:
        A = rng.normal(size=(5, 5))
        fields = [list(np.diag([-4.0] * 5).ravel()), list((np.diag([-4.0] * 5) + 0.3 * (A + A.T)).ravel())]
        cases = [(0, "-"), (1, "-"), (0, "+3/2"), (2, "-"), (3, "-"), (4, "+5/2"), (4, "-1/2")]
        names = {0: ["-3/2", "-1/2", "+1/2", "+3/2"], 1: ["-5/2", "-3/2", "-1/2", "+1/2", "+3/2", "+5/2"]}
        dflt = {0: "-3/2", 1: "-1/2", 2: "-5/2", 3: "-3/2", 4: "-1/2"}
    else:
        fields = [[-3.0, -3.0, -3.0, 0.0, 0.0, 0.0], [-3.0, -2.5, -2.0, 0.3, -0.2, 0.1]]
        cases = [(0, "-"), (0, "+1/2"), (1, "-"), (2, "-"), (1, "+3/2"), (2, "+1/2")]
        names = {0: ["-1/2", "+1/2"], 1: ["-3/2", "-1/2", "+1/2", "+3/2"]}
        dflt = {0: "-1/2", 1: "-3/2", 2: "-1/2"}
    J = _jz(nd)
    als = 3.0
    for iso, m in enumerate(fields):
        H = _state_matrix(d, m, als)
        w, V = np.linalg.eigh(H)
        for st, ljz in cases:
            out = run(harness, "jz", "D" if d else "P", als, st, ljz, *m).split()
            iv = np.array([float(x) for x in out]).view(np.complex128)[:nd]
            man = (0 if st <= 1 else 1) if d else (0 if st == 0 else 1)
            ki, njz = ((0, 4) if man == 0 else (4, 6)) if d else ((0, 2) if man == 0 else (2, 4))
            want_name = dflt[st] if ljz == "-" else ljz
            il = names[man].index(want_name)
            Vm = V[:, ki:ki + njz]
            jw, Z = np.linalg.eigh(Vm.conj().T @ J @ Vm)
            expect = Vm @ Z[:, il]
            assert abs(np.vdot(iv, iv) - 1.0) < 1e-12
            assert abs(abs(np.vdot(expect, iv)) - 1.0) < 1e-10, (d, iso, st, ljz)
            if iso == 0:  # exact Jz eigenstate with m_j = the requested value
                mj = float(want_name.replace("/2", "")) / 2.0
                assert np.allclose(J @ iv, mj * iv, atol=1e-10), (d, st, ljz)
    assert run(harness, "jz", "D" if d else "P", als, 1, "+9/2", *fields[0]).strip() == "BAD"
