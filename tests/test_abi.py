"""The C-ABI library loads, exports every declared symbol and validates its
configuration on the host (no GPU work is issued here)."""
import ctypes as C
import os
import re

import pytest

import eff_pot_gb300 as ep
from eff_pot_gb300 import _abi
from eff_pot_gb300.build import build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    build()
    return ep.load_library()


def header_symbols():
    src = open(os.path.join(ROOT, "include", "eff_pot.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(ep_[a-z_0-9]+)\s*\(", src)))


def test_header_and_binding_agree():
    assert header_symbols() == _abi.HEADER_SYMBOLS


def test_header_enums_and_struct_sizes_match_the_binding():
    """Every EP_* enumerator and #define of the header has the binding's
    value, and the ctypes structs have the C layout's size (a C compile of
    the header reports sizeof)."""
    src = open(os.path.join(ROOT, "include", "eff_pot.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    vals = {}
    for body in re.findall(r"enum\s*\{([^}]*)\}", src):
        for name, v in re.findall(r"\b(EP_[A-Z0-9_]+)\s*=\s*(-?\d+)", body):
            vals[name] = int(v)
    for name, v in re.findall(r"#define\s+(EP_[A-Z0-9_]+)\s+(\d+)", src):
        vals[name] = int(v)
    checked = 0
    for name, v in vals.items():
        if hasattr(_abi, name):
            assert getattr(_abi, name) == v, name
            checked += 1
    assert checked >= 25
    import shutil
    import subprocess
    import tempfile
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "s.c")
        open(c, "w").write('#include <stdio.h>\n#include "eff_pot.h"\nint main(void){printf("%zu %zu %zu %zu\\n",'
                           " sizeof(ep_config), sizeof(ep_potential), sizeof(ep_series), sizeof(ep_energies));"
                           "return 0;}\n")
        exe = os.path.join(d, "s")
        subprocess.run([cc, "-I", os.path.join(ROOT, "include"), c, "-o", exe], check=True)
        sizes = [int(x) for x in subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()]
    assert sizes == [C.sizeof(_abi.EpConfig), C.sizeof(_abi.EpPotential), C.sizeof(_abi.EpSeries),
                     C.sizeof(_abi.EpEnergies)]


def test_library_exports_every_declared_symbol(lib):
    cdll, _ = lib
    missing = [s for s in header_symbols() if not hasattr(cdll, s)]
    assert not missing, missing


def test_config_defaults_match_reference_modules(lib):
    d = ep.library_config_defaults()
    for k, v in ep.DEFAULTS.items():
        assert d[k] == pytest.approx(v, rel=0, abs=0), k


@pytest.mark.parametrize("kw,status", [
    (dict(nx=14), _abi.STATUS_NAMES and 2),            # 7 is not a factor 2,3,5
    (dict(nx=75), 2),                                   # odd
    (dict(npd=15), 8),                                  # wider stencils not built
    (dict(npd=4), 1),
    (dict(icon=0), 8),
    (dict(impurity=_abi.EP_IMPURITY_MOVING, mimpur=0.0), 1),
])
def test_create_rejects_bad_configurations(lib, kw, status):
    with pytest.raises(ep.EffPotError) as ei:
        ep.Solver(**kw)
    assert ei.value.status == status


def test_widened_grid_validator_accepts_320(lib):
    # tstgrid.f90:8-12 rejects 320; the build accepts every even 2^a 3^b 5^c.
    from eff_pot_gb300.solver import _abi as a
    cfg = ep.make_config(nx=320, ny=256, nz=256)
    h = C.c_void_p()
    _, f = lib
    st = f["create"](C.byref(cfg), C.byref(h))
    if st == a.EP_OK:
        f["destroy"](h)
    assert st in (a.EP_OK, 7)  # 7: no device on this host


def test_noalloc_grid_checks_come_before_any_device_work(lib):
    """ep_convolve_noalloc refuses grids on the host: sizes past its fixed
    scratch (a half spectrum above 33*64*64, an axis above 320) with
    EP_ERR_UNSUPPORTED, odd nx or prime factors other than 2, 3, 5 with
    EP_ERR_BAD_GRID, null buffers with EP_ERR_INVALID_ARG.  The pointers are
    never dereferenced on these paths."""
    _, f = lib
    p = 4096  # a dummy address: refused calls touch no memory
    assert f["convolve_noalloc"](p, p, p, 128, 128, 128, None) == _abi.EP_ERR_UNSUPPORTED
    assert f["convolve_noalloc"](p, p, p, 32, 384, 8, None) == _abi.EP_ERR_UNSUPPORTED
    assert f["convolve_noalloc"](p, p, p, 640, 2, 2, None) == _abi.EP_ERR_UNSUPPORTED
    assert f["convolve_noalloc"](p, p, p, 33, 24, 40, None) == _abi.EP_ERR_BAD_GRID
    assert f["convolve_noalloc"](p, p, p, 32, 28, 40, None) == _abi.EP_ERR_BAD_GRID
    assert f["convolve_noalloc"](p, p, p, 32, 24, 0, None) == _abi.EP_ERR_BAD_GRID
    assert f["convolve_noalloc"](None, p, p, 32, 24, 40, None) == _abi.EP_ERR_INVALID_ARG
