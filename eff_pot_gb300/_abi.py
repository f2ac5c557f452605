"""ctypes mirror of include/eff_pot.h (structs, enums, prototypes).

The same prototypes describe any library that exports the eff_pot ABI under
a name prefix, so one binding routine serves libeffpot.so ("ep_").
"""
import ctypes as C

# ---- status codes -----------------------------------------------------------
EP_OK = 0
STATUS_NAMES = {
    0: "EP_OK", 1: "EP_ERR_INVALID_ARG", 2: "EP_ERR_BAD_GRID", 3: "EP_ERR_CUDA",
    4: "EP_ERR_OOM", 5: "EP_ERR_NONFINITE", 6: "EP_ERR_STATE",
    7: "EP_ERR_NO_DEVICE", 8: "EP_ERR_UNSUPPORTED", 9: "EP_ERR_TIMEOUT",
}
(EP_ERR_INVALID_ARG, EP_ERR_BAD_GRID, EP_ERR_CUDA, EP_ERR_OOM, EP_ERR_NONFINITE, EP_ERR_STATE,
 EP_ERR_NO_DEVICE, EP_ERR_UNSUPPORTED, EP_ERR_TIMEOUT) = range(1, 10)
EP_CORE_OT, EP_CORE_OTC, EP_CORE_OP = 0, 1, 2
EP_IMAGINARY_TIME, EP_REAL_TIME = 0, 1
EP_IMPURITY_NONE, EP_IMPURITY_FIXED, EP_IMPURITY_MOVING = 0, 1, 2
EP_FP64, EP_FP32, EP_DFLOAT = 0, 1, 2
EP_ICON_PERIODIC, EP_ICON_ZERO_OUTSIDE = 8, 13
EP_STATE_P, EP_STATE_D = 0, 1
EP_POT_NULL, EP_POT_MORSE, EP_POT_KOUTSELOS = 0, 1, 2
EP_POT_PATIL, EP_POT_AZIZ, EP_POT_TANG_TOENNIES, EP_POT_SERIES = 3, 4, 5, 6
EP_POT_AG, EP_POT_BA_GS, EP_POT_CH3I, EP_POT_SURFACE = 7, 8, 9, 10
EP_POT_EVENPOW, EP_POT_EXPFIT = 11, 12
EP_SERIES_MAX = 24

FIELDS = {
    "den": 0, "pot4": 1, "uimp": 2, "dencg": 3, "delj4": 4, "dxden": 5,
    "dyden": 6, "dzden": 7, "falfs": 8, "intxalf": 9, "intyalf": 10,
    "intzalf": 11, "ualphas": 12, "vpi": 13, "delta": 14, "sigdel": 15,
}
CFIELDS = {
    "psi": 0, "psiold1": 1, "psiold2": 2, "psiold3": 3, "hpsiold1": 4,
    "hpsiold2": 5, "pc": 6, "q": 7,
}


class EpConfig(C.Structure):
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
        ("xmax", C.c_double), ("ymax", C.c_double), ("zmax", C.c_double),
        ("npd", C.c_int), ("icon", C.c_int), ("core", C.c_int),
        ("cp4", C.c_double), ("cpp4", C.c_double), ("den4c", C.c_double),
        ("alphas", C.c_double), ("l", C.c_double), ("den0s", C.c_double),
        ("h2o2m4", C.c_double),
        ("C", C.c_double), ("beta", C.c_double), ("den_m", C.c_double),
        ("h4ot", C.c_double), ("h4op", C.c_double), ("eps4", C.c_double),
        ("sigma4", C.c_double), ("b4", C.c_double),
        ("time_mode", C.c_int), ("renormalize", C.c_int), ("n4", C.c_double),
        ("impurity", C.c_int), ("mimpur", C.c_double), ("fix_lambda", C.c_int),
        ("als_p", C.c_double), ("ev0", C.c_double),
        ("z_exciplex_exclusion", C.c_double),
        ("precision", C.c_int), ("device", C.c_int),
        ("state", C.c_int), ("als_d", C.c_double), ("filter_exciplex_force", C.c_int),
    ]


class EpSeries(C.Structure):
    _fields_ = [("r_core", C.c_double), ("f_core", C.c_double), ("r0", C.c_double),
                ("aa", C.c_double), ("bb", C.c_double), ("cc", C.c_double),
                ("k0", C.c_int), ("n", C.c_int), ("quad", C.c_int),
                ("c_hi", C.c_double * EP_SERIES_MAX), ("c_lo", C.c_double * EP_SERIES_MAX)]


class EpPotential(C.Structure):
    _fields_ = [("kind", C.c_int), ("r_cutoff", C.c_double),
                ("umax", C.c_double), ("par", C.c_double * 4),
                ("series", C.POINTER(EpSeries))]


class EpEnergies(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "etot", "etot4", "ekin4", "elj4", "ecor4", "ealphas", "esolid",
        "eimpu", "ekinx", "eHeX", "uplus", "eso", "n4")]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


class EpStepErrors(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("errHe", "errimp", "errvimp", "erriv")]


class EpRunStats(C.Structure):
    _fields_ = [("errHe", C.c_double), ("mu", C.c_double),
                ("norm", C.c_double), ("steps_done", C.c_int)]


_P = C.c_void_p
_D = C.POINTER(C.c_double)
_I = C.c_int
_prototypes = {
    "config_init": (_I, [C.POINTER(EpConfig)]),
    "create": (_I, [C.POINTER(EpConfig), C.POINTER(_P)]),
    "destroy": (_I, [_P]),
    "last_error": (C.c_char_p, [_P]),
    "set_impurity_potentials": (_I, [_P, C.POINTER(EpPotential), C.POINTER(EpPotential), C.POINTER(EpPotential)]),
    "set_impurity_tables": (_I, [_P, _D, _D, _I, C.c_double, C.c_double]),
    "set_impurity_potentials_d": (_I, [_P, C.POINTER(EpPotential), C.POINTER(EpPotential),
                                       C.POINTER(EpPotential), C.POINTER(EpPotential)]),
    "set_impurity_tables_d": (_I, [_P, _D, _D, _D, _I, C.c_double, C.c_double, C.c_double]),
    "impurity_matrix_d": (_I, [_P, _D]),
    "set_impurity_state": (_I, [_P, _D, _D, _D]),
    "get_impurity_state": (_I, [_P, _D, _D, _D, _D]),
    "upload_psi": (_I, [_P, _D]),
    "download_psi": (_I, [_P, _D]),
    "download_cfield": (_I, [_P, _I, _D]),
    "download_field": (_I, [_P, _I, _D]),
    "potenimp": (_I, [_P]),
    "poten": (_I, [_P]),
    "energy": (_I, [_P, C.POINTER(EpEnergies)]),
    "forceimp": (_I, [_P, _D]),
    "potinvar": (_I, [_P, _D]),
    "impurity_moments": (_I, [_P, _D]),
    "steprk": (_I, [_P, C.c_double]),
    "steppc": (_I, [_P, C.c_double, C.POINTER(EpStepErrors)]),
    "run": (_I, [_P, _I, C.c_double, C.POINTER(EpRunStats)]),
    "renormalize": (_I, [_P, _D]),
    "potential_values": (_I, [C.POINTER(EpPotential), _D, _D, _I]),
}
_product_only = {
    "select_pot": (_I, [C.c_char_p, C.c_double, C.c_double, C.c_char_p, C.POINTER(EpPotential),
                        C.POINTER(EpSeries), C.c_char_p, _I]),
    "create_error": (C.c_char_p, []),
    "synchronize": (_I, [_P]),
    "stream": (_P, [_P]),
    "kernel_launches": (C.c_longlong, [_P]),
    "event_record": (_I, [_P, _I]),
    "event_elapsed": (_I, [_P, _I, _I, _D]),
    "profile_enable": (_I, [_P, _I]),
    "profile_read": (_I, [_P, C.c_char_p, _I, _D, C.POINTER(C.c_longlong), _I, C.POINTER(_I)]),
    "device_bytes": (C.c_longlong, [_P]),
    "convolve_noalloc": (_I, [_P, _P, _P, _I, _I, _I, _P]),
    "set_precision": (_I, [_P, _I]),
    "get_precision": (_I, [_P]),
    "batch_create": (_I, [C.POINTER(EpConfig), _I, C.POINTER(_P)]),
    "batch_destroy": (_I, [_P]),
    "batch_size": (_I, [_P]),
    "batch_ctx": (_P, [_P, _I]),
    "batch_run": (_I, [_P, _I, C.c_double, C.POINTER(EpRunStats)]),
    "batch_steprk": (_I, [_P, C.c_double]),
    "batch_set_precision": (_I, [_P, _I]),
    "batch_synchronize": (_I, [_P]),
    "batch_event_record": (_I, [_P, _I]),
    "batch_event_elapsed": (_I, [_P, _I, _I, _D]),
    "batch_kernel_launches": (C.c_longlong, [_P]),
    "autotune": (_I, [_P, C.c_char_p, _I]),
    "get_launch_shapes": (_I, [_P, C.POINTER(_I)]),
    "set_launch_shapes": (_I, [_P, C.POINTER(_I)]),
    "batch_autotune": (_I, [_P]),
    "set_step_graphs": (_I, [_P, _I]),
    "batch_set_step_graphs": (_I, [_P, _I]),
}

# Every symbol include/eff_pot.h declares.
HEADER_SYMBOLS = sorted("ep_" + n for n in list(_prototypes) + list(_product_only))


def bind(lib, prefix, product=True):
    """Attach restype/argtypes to lib's functions named prefix+name."""
    table = dict(_prototypes)
    if product:
        table.update(_product_only)
    funcs = {}
    for name, (res, args) in table.items():
        if not product and name == "config_init":
            continue
        f = getattr(lib, prefix + name)
        f.restype = res
        f.argtypes = args
        funcs[name] = f
    return funcs


def dptr(a):
    """double* of a contiguous numpy array (float64 or complex128)."""
    return a.ctypes.data_as(_D)
