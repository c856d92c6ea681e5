"""ctypes binding of libmgbf's C-ABI (include/mgbf.h).

Loads the in-tree standalone_mgbf_loc_gb300/_lib/libmgbf.so.  There is no
CPU fallback: if the library is missing, loading fails loudly.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libmgbf.so")

MGBF_MAX_GEN = 16

MGBF_OK = 0
MGBF_ERR_ARG = -1
MGBF_ERR_CONFIG = -2
MGBF_ERR_REACH = -3
MGBF_ERR_DIVISIBILITY = -4
MGBF_ERR_UNSUPPORTED = -5
MGBF_ERR_CUDA = -6
MGBF_ERR_NAMELIST = -7
MGBF_ERR_IO = -8
MGBF_ERR_TIMEOUT = -9
MGBF_ERR_NOMEM = -10

MGBF_F64, MGBF_F32, MGBF_BF16 = 0, 1, 2
MGBF_MEM_DEVICE, MGBF_MEM_HOST = 0, 1
MGBF_LAYOUT_HALO, MGBF_LAYOUT_COMPACT = 0, 1

_I = ctypes.c_int
_D = ctypes.c_double


class MgbfConfig(ctypes.Structure):
    """Mirror of `mgbf_config` (namelist &PARAMETERS_MGBETA + extensions)."""
    _fields_ = [
        ("mg_ampl01", _D), ("mg_ampl02", _D), ("mg_ampl03", _D),
        ("mg_weig1", _D), ("mg_weig2", _D), ("mg_weig3", _D), ("mg_weig4", _D), ("mg_weig5", _D),
        ("hx", _I), ("hy", _I), ("hz", _I), ("p", _I),
        ("mgbf_line", _I), ("mgbf_proc", _I), ("n_ens", _I),
        ("lm_a", _I), ("lm", _I), ("km2", _I), ("km3", _I),
        ("l_loc", _I), ("l_loc_vertical", _I), ("l_filt_g1", _I), ("l_lin_vertical", _I),
        ("l_lin_horizontal", _I),
        ("l_quad_horizontal", _I), ("l_new_map", _I), ("l_vertical_filter", _I),
        ("ldelta", _I), ("lquart", _I), ("lhelm", _I),
        ("gm_max", _I),
        ("nm0", _I), ("mm0", _I), ("nxPE", _I), ("nyPE", _I), ("im_filt", _I), ("jm_filt", _I),
        ("gm_uncapped", _I), ("n_weig_ext", _I),
        ("weig_ext", _D * MGBF_MAX_GEN), ("helm_b", _D * MGBF_MAX_GEN),
        ("layout", _I),
    ]


class MgbfDims(ctypes.Structure):
    _fields_ = [
        ("im", _I), ("jm", _I), ("km_all", _I), ("km", _I), ("km3_all", _I), ("gm", _I),
        ("hx", _I), ("hy", _I), ("hz", _I), ("reach_h", _I), ("reach_z", _I), ("layout", _I),
        ("field_elems", ctypes.c_size_t), ("hbeta_kernel", _I), ("reach_line", _I),
        ("nm0", _I), ("mm0", _I), ("km_a_all", _I), ("anal_elems", ctypes.c_size_t),
    ]


class MgbfGroupDesc(ctypes.Structure):
    _fields_ = [
        ("nk", _I), ("lm", _I), ("nzcol", _I), ("hx", _I), ("hy", _I), ("hz", _I), ("p", _I),
        ("mg_ampl01", _D), ("mg_ampl02", _D),
    ]


class MgbfTimerStat(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char * 16), ("count", ctypes.c_longlong), ("total_ms", _D), ("points", _D)]


# Every symbol include/mgbf.h declares, with its ctypes signature.
_VP = ctypes.c_void_p
_HP = ctypes.c_void_p
SIGNATURES = {
    "mgbf_config_init": (_I, [ctypes.POINTER(MgbfConfig)]),
    "mgbf_config_read_namelist": (_I, [ctypes.c_char_p, ctypes.POINTER(MgbfConfig), ctypes.c_char_p, ctypes.c_size_t]),
    "mgbf_create": (_I, [ctypes.POINTER(MgbfConfig), ctypes.POINTER(_HP)]),
    "mgbf_create_from_namelist": (_I, [ctypes.c_char_p, ctypes.POINTER(_HP)]),
    "mgbf_get_dims": (_I, [_HP, ctypes.POINTER(MgbfDims)]),
    "mgbf_get_line_filters": (_I, [_HP, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                                   ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]),
    "mgbf_filtering_procedure": (_I, [_HP, _I, _VP, _I, _I, _VP]),
    "mgbf_filtering_procedure_adjoint": (_I, [_HP, _I, _VP, _I, _I, _VP]),
    "mgbf_apply_with_weight_grads": (_I, [_HP, _I, _VP, _VP, _VP, ctypes.POINTER(_D), _I, _I, _VP]),
    "mgbf_set_weights": (_I, [_HP, ctypes.POINTER(_D), _I]),
    "mgbf_destroy": (_I, [_HP]),
    "mgbf_strerror": (ctypes.c_char_p, [_I]),
    "mgbf_last_error": (ctypes.c_char_p, []),
    "mgbf_batch_create": (_I, [_I, _I, _I, ctypes.POINTER(_D), _I, _I, ctypes.POINTER(MgbfGroupDesc), _I,
                               ctypes.POINTER(_HP)]),
    "mgbf_batch_apply": (_I, [_HP, ctypes.POINTER(_VP), _I, _I, _VP]),
    "mgbf_batch_destroy": (_I, [_HP]),
    "mgbf_status": (_I, [_HP]),
    "mgbf_batch_status": (_I, [_HP]),
    "mgbf_batch_use_graphs": (_I, [_HP, _I]),
    "mgbf_batch_set_procedure": (_I, [_HP, _I]),
    "mgbf_autotune": (_I, [_HP, _I, _VP]),
    "mgbf_anal_to_filt": (_I, [_HP, _VP, _VP, _I, _I, _VP]),
    "mgbf_filt_to_anal": (_I, [_HP, _VP, _VP, _I, _I, _VP]),
    "mgbf_set_tuning": (_I, [_HP, _I, _I, _I]),
    "mgbf_batch_autotune": (_I, [_HP, _I, _VP]),
    "mgbf_batch_get_tuning": (_I, [_HP, _I, _I, _I, _I, ctypes.POINTER(_I), ctypes.POINTER(_I)]),
    "mgbf_batch_use_persistent": (_I, [_HP, _I]),
    "mgbf_batch_set_priorities": (_I, [_HP, _I]),
    "mgbf_set_wait_limit": (_I, [_HP, _I]),
    "mgbf_batch_set_wait_limit": (_I, [_HP, _I]),
    "mgbf_set_vertical_passes": (_I, [_HP, _I]),
    "mgbf_batch_set_vertical_passes": (_I, [_HP, _I]),
    "mgbf_batch_set_tuning": (_I, [_HP, _I, _I, _I, _I, _I, _I]),
    "mgbf_batch_set_weights": (_I, [_HP, ctypes.POINTER(_D), _I]),
    "mgbf_radial_filter_noalloc": (_I, [_VP, _VP, _I, _I, _I, _I, _D, _I, _I, _D, _VP]),
    "mgbf_timers_enable": (_I, [_I]),
    "mgbf_timers_read": (_I, [ctypes.POINTER(MgbfTimerStat), _I, ctypes.POINTER(_I)]),
}


def timers_enable(on: bool = True) -> None:
    check(load().mgbf_timers_enable(int(on)), "mgbf_timers_enable")


def timers_read() -> dict:
    """{stage: (launches, total_ms, points)} accumulated since timers_enable()."""
    arr = (MgbfTimerStat * 16)()
    n = _I()
    check(load().mgbf_timers_read(arr, 16, ctypes.byref(n)), "mgbf_timers_read")
    return {arr[i].name.decode(): (arr[i].count, arr[i].total_ms, arr[i].points) for i in range(n.value)}

_lib = None


class MGBFError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


def load(path: str = LIB_PATH) -> ctypes.CDLL:
    """Load libmgbf.so and attach signatures; raise if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise MGBFError(MGBF_ERR_ARG, f"libmgbf.so not found at {path}; run __graft_entry__.build() first")
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def check(rc: int, what: str = "") -> None:
    if rc != MGBF_OK:
        lib = load()
        msg = lib.mgbf_last_error().decode() or lib.mgbf_strerror(rc).decode()
        raise MGBFError(rc, f"{what}: {msg}" if what else msg)
