"""Python host interface of the GB300 MGBF filtering path.

Mirrors the reference's operator interface for this path:
  mg_initialize (mg_entrymod.f90:36)         -> MGBF(config) / MGBF.from_namelist(path)
  filtering_procedure(mg_filt) (mg_filtering.f90:67)
                                             -> MGBF.filtering_procedure(mg_filt, vall)
  mg_finalize (mg_entrymod.f90:222)          -> MGBF.close()
with the same namelist fields, the same argument meaning and the same error
cases (the reference's `stop` becomes an MGBFError).  Fields are torch
tensors (device or host) or numpy arrays (host), laid out in C order as
(jm+2hy, im+2hx, km_all) -- which is the memory order of the reference's
VALL(km_all, 1-hx:im+hx, 1-hy:jm+hy) -- or (jm, im, km_all) with the
compact layout.  Every call goes through libmgbf's C-ABI; nothing here
computes the filter.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field, fields
from typing import Dict, List, Optional, Sequence

import numpy as np

from . import _abi
from ._abi import MGBFError

try:  # torch is optional for numpy callers
    import torch
except Exception:  # pragma: no cover
    torch = None


@dataclass
class MGBFConfig:
    """Namelist &PARAMETERS_MGBETA (mg_parameter.f90:190-208) plus extensions."""
    mg_ampl01: float = 1.0
    mg_ampl02: float = 1.0
    mg_ampl03: float = 1.0
    mg_weig1: float = 1.0
    mg_weig2: float = 1.0
    mg_weig3: float = 1.0
    mg_weig4: float = 1.0
    mg_weig5: float = 1.0
    hx: int = 6
    hy: int = 6
    hz: int = 3
    p: int = 2
    mgbf_line: bool = False
    mgbf_proc: int = 1
    n_ens: int = 1
    lm_a: int = 1
    lm: int = 1
    km2: int = 0
    km3: int = 1
    l_loc: bool = False
    l_loc_vertical: bool = False
    l_filt_g1: bool = True
    l_lin_vertical: bool = False
    l_lin_horizontal: bool = False
    l_quad_horizontal: bool = False
    l_new_map: bool = True
    l_vertical_filter: bool = True
    ldelta: bool = False
    lquart: bool = False
    lhelm: bool = False
    gm_max: int = 4
    nm0: int = 0
    mm0: int = 0
    nxPE: int = 1
    nyPE: int = 1
    im_filt: int = 0
    jm_filt: int = 0
    # extensions
    gm_uncapped: bool = False
    weig_ext: List[float] = field(default_factory=list)
    helm_b: List[float] = field(default_factory=list)
    layout: int = _abi.MGBF_LAYOUT_HALO

    def to_c(self) -> _abi.MgbfConfig:
        c = _abi.MgbfConfig()
        _abi.load().mgbf_config_init(ctypes.byref(c))
        for f in fields(self):
            v = getattr(self, f.name)
            if f.name == "weig_ext":
                c.n_weig_ext = len(v)
                for i, x in enumerate(v):
                    c.weig_ext[i] = float(x)
            elif f.name == "helm_b":
                for i, x in enumerate(v):
                    c.helm_b[i] = float(x)
            elif isinstance(v, bool):
                setattr(c, f.name, int(v))
            else:
                setattr(c, f.name, v)
        return c

    @classmethod
    def from_c(cls, c: _abi.MgbfConfig) -> "MGBFConfig":
        kw = {}
        for f in fields(cls):
            if f.name == "weig_ext":
                kw[f.name] = [c.weig_ext[i] for i in range(c.n_weig_ext)]
            elif f.name == "helm_b":
                kw[f.name] = [c.helm_b[i] for i in range(_abi.MGBF_MAX_GEN) if c.helm_b[i] != 0.0]
            elif f.type in ("bool", bool):
                kw[f.name] = bool(getattr(c, f.name))
            else:
                kw[f.name] = getattr(c, f.name)
        return cls(**kw)

    @classmethod
    def from_namelist(cls, path: str) -> "MGBFConfig":
        lib = _abi.load()
        c = _abi.MgbfConfig()
        lib.mgbf_config_init(ctypes.byref(c))
        err = ctypes.create_string_buffer(512)
        _abi.check(lib.mgbf_config_read_namelist(path.encode(), ctypes.byref(c), err, 512),
                   f"reading namelist {path}")
        return cls.from_c(c)


@dataclass
class MGBFDims:
    im: int
    jm: int
    km_all: int
    km: int
    km3_all: int
    gm: int
    hx: int
    hy: int
    hz: int
    reach_h: int
    reach_z: int
    layout: int
    field_elems: int
    hbeta_kernel: int
    reach_line: int
    nm0: int
    mm0: int
    km_a_all: int
    anal_elems: int

    def analysis_shape(self):
        """WORKA(km_a_all, nm0, mm0) in C order."""
        return (self.mm0, self.nm0, self.km_a_all)

    def field_shape(self):
        if self.layout == _abi.MGBF_LAYOUT_HALO:
            return (self.jm + 2 * self.hy, self.im + 2 * self.hx, self.km_all)
        return (self.jm, self.im, self.km_all)


def _dtype_code(dt) -> int:
    if torch is not None and isinstance(dt, torch.dtype):
        m = {torch.float64: _abi.MGBF_F64, torch.float32: _abi.MGBF_F32, torch.bfloat16: _abi.MGBF_BF16}
    else:
        dt = np.dtype(dt)
        m = {np.dtype(np.float64): _abi.MGBF_F64, np.dtype(np.float32): _abi.MGBF_F32}
    if dt not in m:
        raise MGBFError(_abi.MGBF_ERR_ARG, f"unsupported dtype {dt}")
    return m[dt]


def _field_args(arr):
    """(pointer, dtype code, memory space, stream) of a tensor / ndarray."""
    if torch is not None and isinstance(arr, torch.Tensor):
        if not arr.is_contiguous():
            raise MGBFError(_abi.MGBF_ERR_ARG, "field must be contiguous")
        if arr.is_cuda:
            stream = torch.cuda.current_stream(arr.device).cuda_stream
            return arr.data_ptr(), _dtype_code(arr.dtype), _abi.MGBF_MEM_DEVICE, stream
        return arr.data_ptr(), _dtype_code(arr.dtype), _abi.MGBF_MEM_HOST, None
    if isinstance(arr, np.ndarray):
        if not arr.flags.c_contiguous or not arr.flags.writeable:
            raise MGBFError(_abi.MGBF_ERR_ARG, "field must be a writeable C-contiguous array")
        return arr.ctypes.data, _dtype_code(arr.dtype), _abi.MGBF_MEM_HOST, None
    raise MGBFError(_abi.MGBF_ERR_ARG, f"unsupported field type {type(arr)}")


class MGBF:
    """One configured filter (the reference's initialised module state)."""

    def __init__(self, config: MGBFConfig):
        self._lib = _abi.load()
        self.config = config
        self._c = config.to_c()
        h = ctypes.c_void_p()
        _abi.check(self._lib.mgbf_create(ctypes.byref(self._c), ctypes.byref(h)), "mgbf_create")
        self._h = h
        d = _abi.MgbfDims()
        _abi.check(self._lib.mgbf_get_dims(self._h, ctypes.byref(d)), "mgbf_get_dims")
        self.dims = MGBFDims(**{n: getattr(d, n) for n, _ in _abi.MgbfDims._fields_})

    @classmethod
    def from_namelist(cls, path: str) -> "MGBF":
        return cls(MGBFConfig.from_namelist(path))

    # -- reference operator interface ------------------------------------
    def filtering_procedure(self, mg_filt: int, vall) -> None:
        """filtering_procedure(mg_filt) in place on VALL."""
        self._check_shape(vall)
        p, dt, mem, st = _field_args(vall)
        _abi.check(self._lib.mgbf_filtering_procedure(self._h, int(mg_filt), p, dt, mem, st),
                   f"filtering_procedure({mg_filt})")

    def filtering_procedure_adjoint(self, mg_filt: int, vall) -> None:
        self._check_shape(vall)
        p, dt, mem, st = _field_args(vall)
        _abi.check(self._lib.mgbf_filtering_procedure_adjoint(self._h, int(mg_filt), p, dt, mem, st),
                   f"filtering_procedure_adjoint({mg_filt})")

    def apply_with_weight_grads(self, mg_filt: int, x, gy, gx=None):
        """gx = L^T gy and d<gy, L x>/d a_g for every generation."""
        self._check_shape(x)
        self._check_shape(gy)
        if gx is None:
            gx = gy.clone() if (torch is not None and isinstance(gy, torch.Tensor)) else np.array(gy, copy=True)
        px, dt, mem, st = _field_args(x)
        pg, dt2, mem2, _ = _field_args(gy)
        po, dt3, mem3, _ = _field_args(gx)
        if len({dt, dt2, dt3}) != 1 or len({mem, mem2, mem3}) != 1:
            raise MGBFError(_abi.MGBF_ERR_ARG, "x, gy, gx must share dtype and memory space")
        ga = (ctypes.c_double * self.dims.gm)()
        _abi.check(self._lib.mgbf_apply_with_weight_grads(self._h, int(mg_filt), px, pg, po, ga, dt, mem, st),
                   "apply_with_weight_grads")
        return gx, np.array(list(ga))

    def status(self) -> None:
        """Raise if a bounded device wait ran out since the last check."""
        _abi.check(self._lib.mgbf_status(self._h), "mgbf_status")

    def set_wait_limit(self, polls: int) -> None:
        """mbarrier polls per row before a TMA-fed radial kernel gives up and
        reports MGBF_ERR_TIMEOUT (polls < 0: the default)."""
        _abi.check(self._lib.mgbf_set_wait_limit(self._h, int(polls)), "mgbf_set_wait_limit")

    def set_vertical_passes(self, passes: int) -> None:
        """2 (default): Bz^T first and Bz last, as the reference; 1: M = Bz Bz^T
        once, in the last prolongation (same operator, one field write less
        per call where it applies)."""
        _abi.check(self._lib.mgbf_set_vertical_passes(self._h, int(passes)), "mgbf_set_vertical_passes")

    def line_filters(self) -> list:
        """Procedures 2 and 7's three line filters (colors 1..3): dicts with
        the generator d, half-span h, formal half-span hs and weights fil[0..h]."""
        gen = (ctypes.c_int * 6)()
        hspan = (ctypes.c_int * 3)()
        hs = (ctypes.c_double * 3)()
        fil = (ctypes.c_double * 27)()
        _abi.check(self._lib.mgbf_get_line_filters(self._h, gen, hspan, hs, fil), "mgbf_get_line_filters")
        return [{"d": (gen[2 * q], gen[2 * q + 1]), "h": hspan[q], "hs": hs[q],
                 "fil": np.array(fil[9 * q:9 * q + hspan[q] + 1])} for q in range(3)]

    def autotune(self, dtype=None) -> None:
        """Choose radial-kernel variants and tile heights by measurement."""
        dt = _dtype_code(dtype if dtype is not None else torch.float32)
        stream = torch.cuda.current_stream().cuda_stream if torch is not None else None
        _abi.check(self._lib.mgbf_autotune(self._h, dt, stream), "mgbf_autotune")

    def analysis_shape(self):
        return self.dims.analysis_shape()

    def anal_to_filt(self, worka, vall) -> None:
        """anal_to_filt_all2: WORKA (analysis grid) -> VALL (overwritten)."""
        if tuple(worka.shape) != self.analysis_shape():
            raise MGBFError(_abi.MGBF_ERR_ARG, f"WORKA shape {tuple(worka.shape)} != {self.analysis_shape()}")
        self._check_shape(vall)
        pa, dt, mem, st = _field_args(worka)
        pv, dt2, mem2, _ = _field_args(vall)
        if dt != dt2 or mem != mem2:
            raise MGBFError(_abi.MGBF_ERR_ARG, "WORKA and VALL must share dtype and memory space")
        _abi.check(self._lib.mgbf_anal_to_filt(self._h, pa, pv, dt, mem, st), "mgbf_anal_to_filt")

    def filt_to_anal(self, vall, worka) -> None:
        """filt_to_anal_all2: VALL -> WORKA (VALL's interpolation halo is
        filled in place, as in the reference)."""
        if tuple(worka.shape) != self.analysis_shape():
            raise MGBFError(_abi.MGBF_ERR_ARG, f"WORKA shape {tuple(worka.shape)} != {self.analysis_shape()}")
        self._check_shape(vall)
        pv, dt, mem, st = _field_args(vall)
        pa, dt2, mem2, _ = _field_args(worka)
        if dt != dt2 or mem != mem2:
            raise MGBFError(_abi.MGBF_ERR_ARG, "WORKA and VALL must share dtype and memory space")
        _abi.check(self._lib.mgbf_filt_to_anal(self._h, pv, pa, dt, mem, st), "mgbf_filt_to_anal")

    def set_tuning(self, variant: int, rows: int = 0, dtype=None) -> None:
        """Pin the radial-kernel variant and rows per block (variant < 0: defaults)."""
        dt = _dtype_code(dtype if dtype is not None else torch.float32)
        _abi.check(self._lib.mgbf_set_tuning(self._h, dt, int(variant), int(rows)), "mgbf_set_tuning")

    def set_weights(self, a: Sequence[float]) -> None:
        arr = (ctypes.c_double * len(a))(*[float(v) for v in a])
        _abi.check(self._lib.mgbf_set_weights(self._h, arr, len(a)), "set_weights")

    # -- helpers ------------------------------------------------------------
    def field_shape(self):
        return self.dims.field_shape()

    def _check_shape(self, arr):
        if tuple(arr.shape) != tuple(self.field_shape()):
            raise MGBFError(_abi.MGBF_ERR_ARG,
                            f"field shape {tuple(arr.shape)} != expected {tuple(self.field_shape())}")

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.mgbf_destroy(self._h)
            self._h = None

    def __del__(self):  # pragma: no cover
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


@dataclass
class GroupDesc:
    """One variable group of a batched ensemble (extension)."""
    nk: int
    lm: int
    nzcol: int
    hx: int
    hy: int
    hz: int
    p: int
    mg_ampl01: float
    mg_ampl02: float


class MGBFBatch:
    """Variable groups with their own reach and levels, filtered by one call."""

    def __init__(self, im: int, jm: int, gm: int, weights: Sequence[float], groups: Sequence[GroupDesc],
                 lquart: bool = False, l_filt_g1: bool = True):
        self._lib = _abi.load()
        self.im, self.jm, self.gm = im, jm, gm
        self.groups = list(groups)
        descs = (_abi.MgbfGroupDesc * len(groups))()
        for i, g in enumerate(groups):
            for n, _ in _abi.MgbfGroupDesc._fields_:
                setattr(descs[i], n, getattr(g, n))
        w = (ctypes.c_double * gm)(*[float(x) for x in weights])
        h = ctypes.c_void_p()
        _abi.check(self._lib.mgbf_batch_create(im, jm, gm, w, int(lquart), int(l_filt_g1), descs, len(groups),
                                               ctypes.byref(h)), "mgbf_batch_create")
        self._h = h

    def field_shape(self, q: int):
        return (self.jm, self.im, self.groups[q].nk)

    def apply(self, fields_, adjoint: bool = False) -> None:
        if len(fields_) != len(self.groups):
            raise MGBFError(_abi.MGBF_ERR_ARG, "one field per group")
        ptrs = (ctypes.c_void_p * len(fields_))()
        dts = set()
        stream = None
        for i, f in enumerate(fields_):
            if tuple(f.shape) != self.field_shape(i):
                raise MGBFError(_abi.MGBF_ERR_ARG, f"group {i}: shape {tuple(f.shape)} != {self.field_shape(i)}")
            p, dt, mem, st = _field_args(f)
            if mem != _abi.MGBF_MEM_DEVICE:
                raise MGBFError(_abi.MGBF_ERR_ARG, "batched fields must be device tensors")
            ptrs[i] = p
            dts.add(dt)
            stream = st
        if len(dts) != 1:
            raise MGBFError(_abi.MGBF_ERR_ARG, "all groups must share a dtype")
        _abi.check(self._lib.mgbf_batch_apply(self._h, ptrs, dts.pop(), int(adjoint), stream), "mgbf_batch_apply")

    def status(self) -> None:
        _abi.check(self._lib.mgbf_batch_status(self._h), "mgbf_batch_status")

    def autotune(self, dtype=None) -> None:
        """Choose radial-kernel variants and tile heights by measurement."""
        dt = _dtype_code(dtype if dtype is not None else torch.float32)
        stream = torch.cuda.current_stream().cuda_stream if torch is not None else None
        _abi.check(self._lib.mgbf_batch_autotune(self._h, dt, stream), "mgbf_batch_autotune")

    def use_persistent(self, blocks_per_sm: int = 8) -> None:
        """Run each radial side of every group as one persistent launch over
        all generations (FP32/BF16), with up to blocks_per_sm resident
        blocks per SM; 0 (or False) returns to one launch per generation."""
        _abi.check(self._lib.mgbf_batch_use_persistent(self._h, int(blocks_per_sm)), "mgbf_batch_use_persistent")

    def set_priorities(self, mode: int) -> None:
        """Graph-node scheduling priorities: 0 none (the default), 1 the
        memory-bound kernels first, 2 the radial kernels first."""
        _abi.check(self._lib.mgbf_batch_set_priorities(self._h, int(mode)), "mgbf_batch_set_priorities")

    def tuning(self, dtype=None):
        """The radial-kernel choice per group, generation and pass: a list
        (one entry per group) of lists (per generation) of two
        (variant, rows) pairs; variant -1 means the default."""
        dt = _dtype_code(dtype if dtype is not None else torch.float32)
        v, r = ctypes.c_int(), ctypes.c_int()
        out = []
        for q in range(len(self.groups)):
            gens = []
            for g in range(self.gm):
                pair = []
                for ps in range(2):
                    _abi.check(self._lib.mgbf_batch_get_tuning(self._h, dt, q, g, ps, ctypes.byref(v), ctypes.byref(r)),
                               "mgbf_batch_get_tuning")
                    pair.append((v.value, r.value))
                gens.append(pair)
            out.append(gens)
        return out

    def set_weights(self, a: Sequence[float]) -> None:
        """Replace the generation weights a_1..a_n (n <= gm)."""
        arr = (ctypes.c_double * len(a))(*[float(v) for v in a])
        _abi.check(self._lib.mgbf_batch_set_weights(self._h, arr, len(a)), "mgbf_batch_set_weights")

    def set_wait_limit(self, polls: int) -> None:
        """As MGBF.set_wait_limit, for every group of the batch."""
        _abi.check(self._lib.mgbf_batch_set_wait_limit(self._h, int(polls)), "mgbf_batch_set_wait_limit")

    def set_tuning(self, group: int, gen: int, pass_: int, variant: int, rows: int = 0, dtype=None) -> None:
        """Pin the radial kernel of one group, generation and pass (variant
        -1: back to the default; rows 0: the default)."""
        dt = _dtype_code(dtype if dtype is not None else torch.float32)
        _abi.check(self._lib.mgbf_batch_set_tuning(self._h, dt, int(group), int(gen), int(pass_), int(variant), int(rows)),
                   "mgbf_batch_set_tuning")

    def set_vertical_passes(self, passes: int) -> None:
        """As MGBF.set_vertical_passes, for every group of the batch."""
        _abi.check(self._lib.mgbf_batch_set_vertical_passes(self._h, int(passes)), "mgbf_batch_set_vertical_passes")

    def set_procedure(self, mg_filt: int) -> None:
        """6: radial filters (default); 8: the fast 1D+1D line filters."""
        _abi.check(self._lib.mgbf_batch_set_procedure(self._h, int(mg_filt)), "mgbf_batch_set_procedure")

    def use_graphs(self, enable: bool = True) -> None:
        """Replay repeated calls on the same fields as captured CUDA graphs."""
        _abi.check(self._lib.mgbf_batch_use_graphs(self._h, int(enable)), "mgbf_batch_use_graphs")

    def close(self):
        if getattr(self, "_h", None):
            self._lib.mgbf_batch_destroy(self._h)
            self._h = None

    def __del__(self):  # pragma: no cover
        try:
            self.close()
        except Exception:
            pass
