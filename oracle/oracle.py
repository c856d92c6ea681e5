"""ctypes wrapper around the FP64 C oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module.  It restates the reference's CPU algorithm for
filtering_procedure(1|2|3|4|6|8) and the analysis<->filter transfers; it is
the checker, never the thing measured or
shipped.  Parity with the reference itself is unpinned (see mgbf_oracle.h).
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

from . import build as _build

MAX_GEN = 16


class _Cfg(ctypes.Structure):
    _fields_ = [
        ("I", ctypes.c_int), ("J", ctypes.c_int), ("nk", ctypes.c_int),
        ("hx", ctypes.c_int), ("hy", ctypes.c_int), ("hz", ctypes.c_int),
        ("p", ctypes.c_int),
        ("ampl01", ctypes.c_double), ("ampl02", ctypes.c_double),
        ("gm", ctypes.c_int),
        ("a", ctypes.c_double * MAX_GEN), ("b", ctypes.c_double * MAX_GEN),
        ("lhelm", ctypes.c_int), ("proc", ctypes.c_int),
        ("l_vertical_filter", ctypes.c_int), ("l_filt_g1", ctypes.c_int),
        ("lquart", ctypes.c_int), ("lm", ctypes.c_int), ("nzcol", ctypes.c_int),
        ("nthreads", ctypes.c_int), ("ampl03", ctypes.c_double), ("mgbf_line", ctypes.c_int),
    ]


_lib = None


def _load():
    global _lib
    if _lib is None:
        path = _build.build()
        lib = ctypes.CDLL(path)
        dp = ctypes.POINTER(ctypes.c_double)
        cp = ctypes.POINTER(_Cfg)
        lib.orc_filtering_procedure.argtypes = [cp, dp]
        lib.orc_filter_compact.argtypes = [cp, dp, dp]
        lib.orc_weight_grads.argtypes = [cp, dp, dp, dp]
        lib.orc_stage.argtypes = [cp, ctypes.c_int, ctypes.c_int, dp, dp]
        lib.orc_setup_values.argtypes = [cp, dp]
        ip = ctypes.POINTER(ctypes.c_int)
        lib.orc_dibeta_values.argtypes = [cp, ip, ip, dp, dp]
        lib.orc_triad.argtypes = [dp, ip, dp]
        lib.orc_dibeta_values.restype = ctypes.c_int
        lib.orc_triad.restype = ctypes.c_int
        lib.orc_hexad.argtypes = [dp, ip, dp]
        lib.orc_hexad.restype = ctypes.c_int
        xp = ctypes.POINTER(_CXfer)
        lib.orc_anal_to_filt.argtypes = [xp, dp, dp]
        lib.orc_filt_to_anal.argtypes = [xp, dp, dp]
        for f in (lib.orc_filtering_procedure, lib.orc_filter_compact, lib.orc_weight_grads,
                  lib.orc_stage, lib.orc_setup_values, lib.orc_anal_to_filt, lib.orc_filt_to_anal):
            f.restype = ctypes.c_int
        _lib = lib
    return _lib


class OracleError(RuntimeError):
    pass


@dataclass
class OracleConfig:
    """Global-grid form of the reference's parameters (mg_parameter.f90)."""
    I: int
    J: int
    nk: int
    hx: int
    hy: int
    hz: int
    p: int
    ampl01: float
    ampl02: float
    gm: int
    weights: List[float]
    proc: int = 1
    lm: int = 1
    nzcol: int = 0
    l_vertical_filter: bool = True
    l_filt_g1: bool = True
    lquart: bool = False
    lhelm: bool = False
    helm_b: Optional[List[float]] = None
    nthreads: int = 0
    ampl03: float = 1.0
    mgbf_line: bool = True

    def to_c(self) -> _Cfg:
        c = _Cfg()
        c.I, c.J, c.nk = self.I, self.J, self.nk
        c.hx, c.hy, c.hz, c.p = self.hx, self.hy, self.hz, self.p
        c.ampl01, c.ampl02 = float(self.ampl01), float(self.ampl02)
        c.gm = self.gm
        for g in range(self.gm):
            c.a[g] = float(self.weights[g])
            c.b[g] = float(self.helm_b[g]) if self.helm_b else 0.0
        c.lhelm = int(self.lhelm)
        c.proc = self.proc
        c.l_vertical_filter = int(self.l_vertical_filter)
        c.l_filt_g1 = int(self.l_filt_g1)
        c.lquart = int(self.lquart)
        c.lm = self.lm
        c.nzcol = self.nzcol
        c.nthreads = self.nthreads
        c.ampl03 = float(self.ampl03)
        c.mgbf_line = int(self.mgbf_line)
        return c

    def gen_shape(self, g: int):
        return (self.J >> (g - 1), self.I >> (g - 1), self.nk)


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _check(rc: int, what: str):
    if rc != 0:
        raise OracleError(f"{what} failed with code {rc}")


def filter_compact(cfg: OracleConfig, x: np.ndarray) -> np.ndarray:
    """y = L x on a compact array shaped (J, I, nk) (C order == Fortran (nk,I,J))."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    assert x.shape == (cfg.J, cfg.I, cfg.nk), x.shape
    y = np.empty_like(x)
    c = cfg.to_c()
    _check(_load().orc_filter_compact(ctypes.byref(c), _ptr(x), _ptr(y)), "orc_filter_compact")
    return y


def filtering_procedure(cfg: OracleConfig, vall: np.ndarray) -> None:
    """In place on VALL laid out (J+2hy, I+2hx, nk) in C order."""
    assert vall.dtype == np.float64 and vall.flags.c_contiguous
    assert vall.shape == (cfg.J + 2 * cfg.hy, cfg.I + 2 * cfg.hx, cfg.nk)
    c = cfg.to_c()
    _check(_load().orc_filtering_procedure(ctypes.byref(c), _ptr(vall)), "orc_filtering_procedure")


def weight_grads(cfg: OracleConfig, x: np.ndarray, gy: np.ndarray) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float64)
    gy = np.ascontiguousarray(gy, dtype=np.float64)
    ga = np.zeros(cfg.gm, dtype=np.float64)
    c = cfg.to_c()
    _check(_load().orc_weight_grads(ctypes.byref(c), _ptr(x), _ptr(gy), _ptr(ga)), "orc_weight_grads")
    return ga


(STAGE_Z_FWD, STAGE_Z_ADJ, STAGE_H_FWD, STAGE_H_ADJ, STAGE_RESTRICT, STAGE_PROLONG, STAGE_FAST_FWD,
 STAGE_FAST_ADJ, STAGE_LIN2_FWD, STAGE_LIN2_ADJ, STAGE_LIN3_GEN) = range(11)
DIB_NH = 6
DIB_NFIL = DIB_NH + 2


def stage(cfg: OracleConfig, which: int, gen: int, x: np.ndarray) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float64)
    J, I, nk = cfg.gen_shape(gen)
    if which == STAGE_RESTRICT:
        out_shape = (J // 2, I // 2, nk)
    elif which == STAGE_PROLONG:
        out_shape = (J, I, nk)
    else:
        out_shape = (J, I, nk)
    y = np.zeros(out_shape, dtype=np.float64)
    c = cfg.to_c()
    _check(_load().orc_stage(ctypes.byref(c), which, gen, _ptr(x), _ptr(y)), f"orc_stage({which})")
    return y


def contributions(cfg: OracleConfig, x: np.ndarray) -> list:
    """Per-generation terms of the radial procedures 1 and 6:
    y_g = Bz P_{1<-g} B_g a_g B_g R_{g<-1} Bz^T x for g = 1..gm, composed from
    the oracle's stages in the order of orc_filtering_procedure (vertical
    adjoint, restrictions, per generation vrbeta2t + fold, weight, fill +
    vrbeta2, prolongations, vertical forward).  Without l_filt_g1 (proc 6)
    generation 1 is neither filtered nor weighted.  sum_g y_g equals
    filter_compact(cfg, x) up to rounding."""
    assert cfg.proc in (1, 6), "radial procedures only"
    z = bool(cfg.l_vertical_filter and cfg.nzcol > 0)
    x = np.ascontiguousarray(x, dtype=np.float64)
    h = [stage(cfg, STAGE_Z_ADJ, 1, x) if z else x.copy()]
    for g in range(1, cfg.gm):
        h.append(stage(cfg, STAGE_RESTRICT, g, h[-1]))
    filt1 = cfg.proc == 1 or cfg.l_filt_g1
    out = []
    for g in range(cfg.gm):
        if g == 0 and not filt1:
            u = h[0]
        else:
            u = stage(cfg, STAGE_H_FWD, g + 1, cfg.weights[g] * stage(cfg, STAGE_H_ADJ, g + 1, h[g]))
        for fine in range(g, 0, -1):  # generation fine+1 -> fine
            u = stage(cfg, STAGE_PROLONG, fine, u)
        out.append(stage(cfg, STAGE_Z_FWD, 1, u) if z else u)
    return out


def setup_values(cfg: OracleConfig) -> dict:
    out = np.zeros(11, dtype=np.float64)
    c = cfg.to_c()
    _check(_load().orc_setup_values(ctypes.byref(c), _ptr(out)), "orc_setup_values")
    keys = ["rmom2_1", "rmom2_2", "exx1", "exx2", "ss1", "ss2", "reach_z", "reach_h", "exx_line", "ss_line",
            "reach_line"]
    return dict(zip(keys, out.tolist()))


def dibeta_values(cfg: OracleConfig) -> list:
    """Proc 2's three line filters (colors 1..3): dicts with the generator
    (dx, dy), integer half-span h, formal half-span hs and weights fil[0..h]."""
    gen = (ctypes.c_int * 6)()
    h = (ctypes.c_int * 3)()
    hs = np.zeros(3)
    fil = np.zeros(3 * (DIB_NFIL + 1))
    c = cfg.to_c()
    _check(_load().orc_dibeta_values(ctypes.byref(c), gen, h, _ptr(hs), _ptr(fil)), "orc_dibeta_values")
    return [{"d": (gen[2 * q], gen[2 * q + 1]), "h": h[q], "hs": float(hs[q]),
             "fil": fil[q * (DIB_NFIL + 1):q * (DIB_NFIL + 1) + h[q] + 1].copy()} for q in range(3)]


def hexad(aspect) -> tuple:
    """The hexad decomposition of (A11, A22, A33, A23, A31, A12): (generators
    7x3 for colors 1..7, weights 7)."""
    a = np.ascontiguousarray(aspect, dtype=np.float64)
    lh = (ctypes.c_int * 21)()
    w = np.zeros(7)
    _check(_load().orc_hexad(_ptr(a), lh, _ptr(w)), "orc_hexad")
    return np.array(list(lh)).reshape(7, 3), w


def triad(aspect) -> tuple:
    """The triad decomposition of (A11, A22, A12): (generators 3x2, weights 3)."""
    a = np.ascontiguousarray(aspect, dtype=np.float64)
    lt = (ctypes.c_int * 6)()
    w = np.zeros(3)
    _check(_load().orc_triad(_ptr(a), lt, _ptr(w)), "orc_triad")
    return np.array(list(lt)).reshape(3, 2), w


# ------------------------------------------------ analysis <-> filter grid


class _CXfer(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int) for n in ("nm0", "mm0", "nxpe", "nype", "im", "jm", "hx", "hy", "nkf", "nka",
                                            "lm", "lm_a", "en", "order")]


@dataclass
class XferConfig:
    """Transfer geometry (mg_parameter.f90:357-358, 515-541): nm0 x mm0
    analysis points and nxpe*im x nype*jm filter points; order 3 = lsqr,
    2 = quadratic (l_quad_horizontal), 1 = linear (l_lin_horizontal)."""
    nm0: int
    mm0: int
    nxpe: int
    nype: int
    im: int
    jm: int
    hx: int
    hy: int
    nkf: int
    nka: int = 0
    lm: int = 1
    lm_a: int = 1
    en: int = 0
    order: int = 3

    def to_c(self):
        c = _CXfer()
        for n, _ in _CXfer._fields_:
            setattr(c, n, int(getattr(self, n)))
        if not self.nka:
            c.nka = self.nkf
        return c

    @property
    def I(self):
        return self.nxpe * self.im

    @property
    def J(self):
        return self.nype * self.jm

    def vall_shape(self):
        return (self.J + 2 * self.hy, self.I + 2 * self.hx, self.nkf)

    def worka_shape(self):
        return (self.mm0, self.nm0, self.nka or self.nkf)


def filt_to_anal(cfg: XferConfig, vall: np.ndarray) -> np.ndarray:
    """filt_to_anal_all2: VALL (halo layout; its interpolation halo is filled
    in place, as in the reference) -> WORKA."""
    assert vall.shape == cfg.vall_shape() and vall.dtype == np.float64 and vall.flags.c_contiguous
    w = np.zeros(cfg.worka_shape(), dtype=np.float64)
    c = cfg.to_c()
    _check(_load().orc_filt_to_anal(ctypes.byref(c), _ptr(vall), _ptr(w)), "orc_filt_to_anal")
    return w


def anal_to_filt(cfg: XferConfig, worka: np.ndarray) -> np.ndarray:
    """anal_to_filt_all2: WORKA -> VALL (halo layout)."""
    worka = np.ascontiguousarray(worka, dtype=np.float64)
    assert worka.shape == cfg.worka_shape()
    v = np.zeros(cfg.vall_shape(), dtype=np.float64)
    c = cfg.to_c()
    _check(_load().orc_anal_to_filt(ctypes.byref(c), _ptr(worka), _ptr(v)), "orc_anal_to_filt")
    return v
