"""Host-side mirror of the reference's hot-path subroutines over the C ABI.

The reference calls argument-light Fortran subroutines over module globals
(potenimp, poten, energy, forceimp, potinvar, steprk, steppc).  Solver keeps
one solver context in HBM and exposes the same operations, in the same
order and with the same meaning; arrays cross the boundary as numpy arrays
shaped (nx, ny, nz) in Fortran order (x fastest), exactly the module layout.

Errors come back as EffPotError carrying the C status code where the
reference would STOP.
"""
import ctypes as C
import os

import numpy as np

from . import _abi
from .config import make_config, config_dict, MP_U

_HERE = os.path.dirname(os.path.abspath(__file__))
PRECISIONS = {"fp64": _abi.EP_FP64, "fp32": _abi.EP_FP32, "dfloat": _abi.EP_DFLOAT}
PRECISION_NAMES = {v: k for k, v in PRECISIONS.items()}
LIBPATH = os.path.join(_HERE, "_build", "libeffpot.so")
_lib = None
_funcs = None


class EffPotError(RuntimeError):
    def __init__(self, status, message):
        self.status = status
        super().__init__(f"{_abi.STATUS_NAMES.get(status, status)}: {message}")


def load_library(path=None):
    """Load libeffpot.so (built by eff_pot_gb300.build).  No fallback."""
    global _lib, _funcs
    if _lib is not None and path is None:
        return _lib, _funcs
    p = path or LIBPATH
    if not os.path.exists(p):
        raise EffPotError(_abi.EP_ERR_UNSUPPORTED if hasattr(_abi, "EP_ERR_UNSUPPORTED") else 8,
                          f"{p} is missing: run eff_pot_gb300.build.build() first")
    lib = C.CDLL(p)
    funcs = _abi.bind(lib, "ep_", product=True)
    if path is None:
        _lib, _funcs = lib, funcs
    return lib, funcs


def select_pot(selec, r_cutoff=0.0, umax=0.0, source=None):
    """Select_Pot by name (V_impur.f90:87-932) through ep_select_pot: the
    closed forms built into the library, or an inverse-power fit read from
    the reference's V_impur.f90 at `source`.  Host only (no GPU)."""
    _, f = load_library()
    p, s = _abi.EpPotential(), _abi.EpSeries()
    err = C.create_string_buffer(512)
    st = f["select_pot"](selec.encode(), float(r_cutoff), float(umax),
                         None if source is None else os.fsencode(source), C.byref(p), C.byref(s), err, 512)
    if st != _abi.EP_OK:
        raise EffPotError(st, err.value.decode())
    if p.kind in (_abi.EP_POT_SERIES, _abi.EP_POT_EVENPOW, _abi.EP_POT_EXPFIT):
        p.series = C.pointer(s)
        p._series = s
    return p


def potential_values(pot, r):
    """V(r) of an EpPotential in the library's host arithmetic (ep_potential_values)."""
    _, f = load_library()
    r = np.ascontiguousarray(r, dtype=np.float64)
    v = np.empty_like(r)
    st = f["potential_values"](C.byref(pot), _abi.dptr(r), _abi.dptr(v), r.size)
    if st != _abi.EP_OK:
        raise EffPotError(st, "ep_potential_values")
    return v


def library_config_defaults():
    """ep_config_init() of the library, as a dict."""
    _, f = load_library()
    cfg = _abi.EpConfig()
    f["config_init"](C.byref(cfg))
    return config_dict(cfg)


class Solver:
    """One solver instance (one ep_ctx) on one GPU."""

    prefix = "ep_"

    def __init__(self, cfg=None, **kw):
        self._f = self._bind()
        self.cfg = cfg if cfg is not None else make_config(**kw)
        h = C.c_void_p()
        st = self._f["create"](C.byref(self.cfg), C.byref(h))
        if st != _abi.EP_OK:
            raise EffPotError(st, self._create_error())
        self._h = h
        self._owned = True
        self._init_geometry()

    @classmethod
    def _view(cls, cfg, handle):
        """A Solver over a context owned by someone else (a batch)."""
        self = cls.__new__(cls)
        self._f = self._bind()
        self.cfg = cfg
        self._h = C.c_void_p(handle)
        self._owned = False
        self._init_geometry()
        return self

    def _init_geometry(self):
        c = self.cfg
        self.shape = (c.nx, c.ny, c.nz)
        self.N = c.nx * c.ny * c.nz
        self.hx = 2.0 * abs(c.xmax) / c.nx
        self.hy = 2.0 * abs(c.ymax) / c.ny
        self.hz = 2.0 * abs(c.zmax) / c.nz
        self.dxyz = self.hx * self.hy * self.hz

    # -- plumbing ------------------------------------------------------------
    def _bind(self):
        return load_library()[1]

    def _create_error(self):
        return self._f["create_error"]().decode()

    def _check(self, st, what):
        if st != _abi.EP_OK:
            msg = self._f["last_error"](self._h)
            raise EffPotError(st, f"{what}: {msg.decode() if msg else ''}")

    def close(self):
        if getattr(self, "_h", None):
            if getattr(self, "_owned", True):
                self._f["destroy"](self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- grid ----------------------------------------------------------------
    def axes(self):
        """x, y, z of DFT4He3d.f90:248-256."""
        c = self.cfg
        x = -c.xmax + self.hx * np.arange(c.nx)
        y = -c.ymax + self.hy * np.arange(c.ny)
        z = -c.zmax + self.hz * np.arange(c.nz)
        return x, y, z

    # -- impurity ------------------------------------------------------------
    def set_impurity_potentials(self, pi, sigma=None, plus=None):
        sigma = pi if sigma is None else sigma
        st = self._f["set_impurity_potentials"](self._h, C.byref(pi), C.byref(sigma),
                                                C.byref(plus) if plus is not None else None)
        self._check(st, "set_impurity_potentials")

    def set_impurity_tables(self, potpi, potdel, delinter, umax_sigma):
        potpi = np.ascontiguousarray(potpi, dtype=np.float64)
        potdel = np.ascontiguousarray(potdel, dtype=np.float64)
        st = self._f["set_impurity_tables"](self._h, _abi.dptr(potpi), _abi.dptr(potdel),
                                            len(potpi) - 2, delinter, umax_sigma)
        self._check(st, "set_impurity_tables")

    def set_impurity_potentials_d(self, pi, sigma, delta, plus=None):
        """D state (Lstate='D'): potenimpini's three tables from V_Pi, V_Sigma, V_Delta."""
        st = self._f["set_impurity_potentials_d"](self._h, C.byref(pi), C.byref(sigma), C.byref(delta),
                                                  C.byref(plus) if plus is not None else None)
        self._check(st, "set_impurity_potentials_d")

    def set_impurity_tables_d(self, potdel, potpidel, potsigdel, delinter, umax_pi, umax_sigma):
        t = [np.ascontiguousarray(a, dtype=np.float64) for a in (potdel, potpidel, potsigdel)]
        st = self._f["set_impurity_tables_d"](self._h, *(_abi.dptr(a) for a in t), len(t[0]) - 2, delinter,
                                              umax_pi, umax_sigma)
        self._check(st, "set_impurity_tables_d")

    def impurity_matrix_d(self):
        """The D-state 5x5 density-weighted field matrix (potinvar / instates)."""
        m = np.zeros(25)
        self._check(self._f["impurity_matrix_d"](self._h, _abi.dptr(m)), "impurity_matrix_d")
        return m.reshape(5, 5)

    def set_impurity(self, rimp=None, vimp=None, invar=None):
        def arr(a, n):
            if a is None:
                return None
            a = np.ascontiguousarray(a)
            if np.iscomplexobj(a):
                a = a.astype(np.complex128).view(np.float64)
            a = np.ascontiguousarray(a, dtype=np.float64)
            assert a.size == n
            self._keep = getattr(self, "_keep", []) + [a]
            return _abi.dptr(a)
        st = self._f["set_impurity_state"](self._h, arr(rimp, 3), arr(vimp, 3), arr(invar, 20))
        self._check(st, "set_impurity_state")

    def impurity(self):
        r, v, a, iv = (np.zeros(3), np.zeros(3), np.zeros(3), np.zeros(20))
        st = self._f["get_impurity_state"](self._h, _abi.dptr(r), _abi.dptr(v), _abi.dptr(a), _abi.dptr(iv))
        self._check(st, "get_impurity_state")
        return dict(rimp=r, vimp=v, aimp=a, invar=iv.view(np.complex128))

    # -- fields --------------------------------------------------------------
    def upload_psi(self, psi):
        psi = np.asarray(psi, dtype=np.complex128)
        assert psi.shape == self.shape, psi.shape
        buf = np.asfortranarray(psi)
        st = self._f["upload_psi"](self._h, buf.ctypes.data_as(C.POINTER(C.c_double)))
        self._check(st, "upload_psi")

    def psi(self, out=None):
        """psi as a (nx, ny, nz) complex array in Fortran order.  out: an array
        of that shape and layout to fill (e.g. in page-locked memory, which
        the device copies into at full link speed) instead of a new one."""
        if out is None:
            out = np.empty(self.shape, dtype=np.complex128, order="F")
        elif out.shape != self.shape or out.dtype != np.complex128 or not out.flags.f_contiguous:
            raise ValueError("out must be a Fortran-ordered complex128 array of the grid's shape")
        self._check(self._f["download_psi"](self._h, out.ctypes.data_as(C.POINTER(C.c_double))), "download_psi")
        return out

    def cfield(self, name):
        out = np.empty(self.shape, dtype=np.complex128, order="F")
        st = self._f["download_cfield"](self._h, _abi.CFIELDS[name], out.ctypes.data_as(C.POINTER(C.c_double)))
        self._check(st, f"download_cfield({name})")
        return out

    def field(self, name):
        out = np.empty(self.shape, dtype=np.float64, order="F")
        st = self._f["download_field"](self._h, _abi.FIELDS[name], out.ctypes.data_as(C.POINTER(C.c_double)))
        self._check(st, f"download_field({name})")
        return out

    # -- the hot-path subroutines -------------------------------------------
    def potenimp(self):
        self._check(self._f["potenimp"](self._h), "potenimp")

    def poten(self):
        self._check(self._f["poten"](self._h), "poten")

    def energy(self):
        e = _abi.EpEnergies()
        self._check(self._f["energy"](self._h, C.byref(e)), "energy")
        return e.as_dict()

    def forceimp(self):
        F = np.zeros(3)
        self._check(self._f["forceimp"](self._h, _abi.dptr(F)), "forceimp")
        return F

    def impurity_moments(self):
        """(Vx, Vy, Vz, Vxy, Vxz, Vyz): the P-state matrix of instates."""
        v = np.zeros(6)
        self._check(self._f["impurity_moments"](self._h, _abi.dptr(v)), "impurity_moments")
        return v

    def potinvar(self):
        H = np.zeros(20)
        self._check(self._f["potinvar"](self._h, _abi.dptr(H)), "potinvar")
        return H.view(np.complex128)

    def steprk(self, deltat):
        self._check(self._f["steprk"](self._h, deltat), "steprk")

    def steppc(self, deltat, wait=True):
        if not wait:
            self._check(self._f["steppc"](self._h, deltat, None), "steppc")
            return None
        e = _abi.EpStepErrors()
        self._check(self._f["steppc"](self._h, deltat, C.byref(e)), "steppc")
        return dict(errHe=e.errHe, errimp=e.errimp, errvimp=e.errvimp, erriv=e.erriv)

    def run(self, nsteps, deltat, wait=True):
        if not wait:
            self._check(self._f["run"](self._h, nsteps, deltat, None), "run")
            return None
        s = _abi.EpRunStats()
        self._check(self._f["run"](self._h, nsteps, deltat, C.byref(s)), "run")
        return dict(errHe=s.errHe, mu=s.mu, norm=s.norm, steps_done=s.steps_done)

    def renormalize(self):
        n = C.c_double()
        self._check(self._f["renormalize"](self._h, C.byref(n)), "renormalize")
        return n.value

    def set_precision(self, precision):
        """'fp32' / 'fp64' / 'dfloat' (or EP_FP32 / EP_FP64 / EP_DFLOAT):
        convert the state and go on in that arithmetic."""
        self._check(self._f["set_precision"](self._h, PRECISIONS.get(precision, precision)), "set_precision")

    def precision(self):
        return PRECISION_NAMES[self._f["get_precision"](self._h)]

    def autotune(self):
        """Pick the FFT-pass launch shapes for this grid (needs a density)."""
        buf = C.create_string_buffer(256)
        self._check(self._f["autotune"](self._h, buf, 256), "autotune")
        return buf.value.decode()

    def launch_shapes(self):
        a = (C.c_int * 6)()
        self._check(self._f["get_launch_shapes"](self._h, a), "get_launch_shapes")
        return list(a)

    def set_launch_shapes(self, shapes):
        a = (C.c_int * 6)(*shapes)
        self._check(self._f["set_launch_shapes"](self._h, a), "set_launch_shapes")

    # -- product-only services ----------------------------------------------
    def synchronize(self):
        self._check(self._f["synchronize"](self._h), "synchronize")

    def stream(self):
        return self._f["stream"](self._h)

    def kernel_launches(self):
        return int(self._f["kernel_launches"](self._h))

    def device_bytes(self):
        return int(self._f["device_bytes"](self._h))

    def profile(self, on=True):
        self._check(self._f["profile_enable"](self._h, 1 if on else 0), "profile_enable")

    def step_graphs(self, on=True):
        """Replay run() steps from a captured CUDA graph (True or 1, the
        default), whole rotation periods of steps from one graph (2), or
        launch every kernel directly (False or 0)."""
        self._check(self._f["set_step_graphs"](self._h, int(on)), "set_step_graphs")

    def profile_read(self):
        cap, maxn = 4096, 64
        names = C.create_string_buffer(cap)
        ms = np.zeros(maxn)
        cnt = (C.c_longlong * maxn)()
        n = C.c_int()
        st = self._f["profile_read"](self._h, names, cap, _abi.dptr(ms), cnt, maxn, C.byref(n))
        self._check(st, "profile_read")
        parts = names.raw.split(b"\0")
        return {parts[i].decode(): (float(ms[i]), int(cnt[i])) for i in range(min(n.value, maxn))}

    # -- convenience: the reference's start-up sequence ---------------------
    def start(self, psi):
        """den=|psi|^2, potenimp, poten (DFT4He3d.f90:436-438)."""
        self.upload_psi(psi)
        self.potenimp()
        self.poten()


def mass_units(mimpur):
    """mAg_u of DFT4He3d.f90:203."""
    return mimpur * MP_U


class Batch:
    """Many independent instances advanced together (ep_batch_*)."""

    def __init__(self, cfgs):
        _, self._f = load_library()
        self.cfgs = list(cfgs)
        n = len(self.cfgs)
        arr = (_abi.EpConfig * n)(*self.cfgs)
        h = C.c_void_p()
        st = self._f["batch_create"](arr, n, C.byref(h))
        if st != _abi.EP_OK:
            raise EffPotError(st, self._f["create_error"]().decode())
        self._h = h
        self.solvers = [Solver._view(self.cfgs[i], self._f["batch_ctx"](h, i)) for i in range(n)]

    def __len__(self):
        return len(self.solvers)

    def __getitem__(self, i):
        return self.solvers[i]

    def _check(self, st, what):
        if st != _abi.EP_OK:
            raise EffPotError(st, what)

    def steprk(self, deltat):
        self._check(self._f["batch_steprk"](self._h, deltat), "batch_steprk")

    def run(self, nsteps, deltat, wait=True):
        if not wait:
            self._check(self._f["batch_run"](self._h, nsteps, deltat, None), "batch_run")
            return None
        stats = (_abi.EpRunStats * len(self))()
        self._check(self._f["batch_run"](self._h, nsteps, deltat, stats), "batch_run")
        return [dict(errHe=s.errHe, mu=s.mu, norm=s.norm, steps_done=s.steps_done) for s in stats]

    def set_precision(self, precision):
        self._check(self._f["batch_set_precision"](self._h, PRECISIONS.get(precision, precision)),
                    "batch_set_precision")

    def autotune(self):
        self._check(self._f["batch_autotune"](self._h), "batch_autotune")

    def synchronize(self):
        self._check(self._f["batch_synchronize"](self._h), "batch_synchronize")

    def event_record(self, slot):
        self._check(self._f["batch_event_record"](self._h, slot), "batch_event_record")

    def event_elapsed(self, a, b):
        ms = C.c_double()
        self._check(self._f["batch_event_elapsed"](self._h, a, b, C.byref(ms)), "batch_event_elapsed")
        return ms.value

    def kernel_launches(self):
        return int(self._f["batch_kernel_launches"](self._h))

    def step_graphs(self, on=True):
        """As Solver.step_graphs, for every instance of the batch."""
        self._check(self._f["batch_set_step_graphs"](self._h, int(on)), "batch_set_step_graphs")

    def close(self):
        if getattr(self, "_h", None):
            for s in self.solvers:
                s._h = None
            self._f["batch_destroy"](self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
