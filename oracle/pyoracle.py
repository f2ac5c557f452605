"""ctypes loader of the CPU FP64 oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline use this
module, as the parity checker and the timed CPU reference.  It builds
oracle/_build/liboracle.so on first use if it is missing.
"""
import ctypes as C
import os
import subprocess

import numpy as np

from eff_pot_gb300 import _abi
from eff_pot_gb300.solver import Solver, EffPotError

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
_lib = None
_funcs = None


def build(force=False):
    src = [os.path.join(HERE, f) for f in ("oracle.cpp", "oracle.h", "Makefile")]
    if force or not os.path.exists(LIB) or any(os.path.getmtime(s) > os.path.getmtime(LIB) for s in src):
        subprocess.run(["make", "-s", "-C", HERE] + (["-B"] if force else []), check=True)
    return LIB


def load():
    global _lib, _funcs
    if _lib is None:
        build()
        _lib = C.CDLL(LIB)
        _funcs = _abi.bind(_lib, "oc_", product=False)
        _lib.oc_set_threads.restype = C.c_int
        _lib.oc_set_threads.argtypes = [C.c_int]
        _lib.oc_rfft3.argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
        _lib.oc_irfft3.argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
        _lib.oc_fd_weights.argtypes = [C.c_int, C.c_int, C.c_void_p]
        _lib.oc_deriv.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
        _lib.oc_sinint.restype = C.c_double
        _lib.oc_sinint.argtypes = [C.c_double]
        _lib.oc_bforce.restype = C.c_double
        _lib.oc_bforce.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double]
        _lib.oc_form_factors.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        _lib.oc_get_impurity_tables.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    return _lib, _funcs


def set_threads(n):
    return load()[0].oc_set_threads(n)


def rfft3(a):
    """Oracle r2c of a real (nx,ny,nz) Fortran-order array."""
    lib, _ = load()
    a = np.asfortranarray(a, dtype=np.float64)
    nx, ny, nz = a.shape
    out = np.empty((nx // 2 + 1, ny, nz), dtype=np.complex128, order="F")
    st = lib.oc_rfft3(nx, ny, nz, a.ctypes.data, out.ctypes.data)
    if st:
        raise EffPotError(st, "oc_rfft3")
    return out


def irfft3(c, nx):
    lib, _ = load()
    c = np.asfortranarray(c, dtype=np.complex128)
    _, ny, nz = c.shape
    out = np.empty((nx, ny, nz), dtype=np.float64, order="F")
    st = lib.oc_irfft3(nx, ny, nz, c.ctypes.data, out.ctypes.data)
    if st:
        raise EffPotError(st, "oc_irfft3")
    return out


def fd_weights(npd, order):
    lib, _ = load()
    w = np.zeros(npd)
    st = lib.oc_fd_weights(npd, order, w.ctypes.data)
    if st:
        raise EffPotError(st, "oc_fd_weights")
    return w


def potential_values(pot, r):
    """The oracle's Select_Pot restatement at the radii r (oc_potential_values)."""
    _, f = load()
    r = np.ascontiguousarray(r, dtype=np.float64)
    v = np.empty_like(r)
    st = f["potential_values"](C.byref(pot), _abi.dptr(r), _abi.dptr(v), r.size)
    if st != 0:
        raise EffPotError(st, "oc_potential_values")
    return v


def sinint(x):
    return load()[0].oc_sinint(float(x))


def bforce(core, eps, sigma, hc):
    return load()[0].oc_bforce(core, eps, sigma, hc)


class OracleSolver(Solver):
    """The oracle behind the Solver interface (same methods, CPU FP64)."""

    prefix = "oc_"

    def _bind(self):
        return load()[1]

    def _create_error(self):
        return "oracle rejected the configuration"

    def deriv(self, f, order, axis):
        lib, _ = load()
        cplx = np.iscomplexobj(f)
        f = np.asfortranarray(f, dtype=np.complex128 if cplx else np.float64)
        out = np.empty_like(f)
        st = lib.oc_deriv(self._h, order, axis, 1 if cplx else 0, f.ctypes.data, out.ctypes.data)
        if st:
            raise EffPotError(st, "oc_deriv")
        return out

    def form_factors(self):
        lib, _ = load()
        nx, ny, nz = self.shape
        sh = (nx // 2 + 1, ny, nz)
        fv, wc, ka = (np.empty(sh, order="F") for _ in range(3))
        lib.oc_form_factors(self._h, fv.ctypes.data, wc.ctypes.data, ka.ctypes.data)
        return fv, wc, ka

    def impurity_tables(self):
        lib, _ = load()
        n = C.c_int()
        d = C.c_double()
        lib.oc_get_impurity_tables(self._h, None, None, C.byref(n), C.byref(d))
        tp, td = np.empty(n.value + 2), np.empty(n.value + 2)
        lib.oc_get_impurity_tables(self._h, tp.ctypes.data, td.ctypes.data, None, None)
        return tp, td, d.value

    # product-only services do not exist on the CPU checker
    def synchronize(self):
        return None

    def kernel_launches(self):
        return 0
