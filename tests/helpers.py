"""Shared test helpers: namelist config -> oracle config, error norms."""
from __future__ import annotations

import numpy as np

from oracle import oracle as O
from standalone_mgbf_loc_gb300.mgbf import MGBFConfig


def def_maxgen(nxm: int, nym: int) -> int:
    """mg_parameter.f90:578-611."""
    def one(n):
        g = 1
        while True:
            n = (n + 1) // 2
            g += 1
            if n == 1:
                return g
    return min(one(nxm), one(nym))


def gens(c: MGBFConfig) -> int:
    return c.gm_max if c.gm_uncapped else min(c.gm_max, def_maxgen(c.nxPE, c.nyPE))


def gen_weights(c: MGBFConfig, gm: int):
    if c.weig_ext:
        return [c.weig_ext[min(g, len(c.weig_ext) - 1)] for g in range(gm)]
    w = [c.mg_weig1, c.mg_weig2, c.mg_weig3, c.mg_weig4]
    return [w[g] if g < 4 else c.mg_weig5 for g in range(gm)]


def oracle_cfg(c: MGBFConfig, proc: int, nthreads: int = 0) -> O.OracleConfig:
    gm = gens(c)
    km = c.km2 + c.lm * c.km3
    return O.OracleConfig(
        I=c.nxPE * c.im_filt, J=c.nyPE * c.jm_filt, nk=km * c.n_ens,
        hx=c.hx, hy=c.hy, hz=c.hz, p=c.p, ampl01=c.mg_ampl01, ampl02=c.mg_ampl02, gm=gm,
        weights=gen_weights(c, gm), proc=proc, lm=c.lm,
        nzcol=(c.km3 if proc in (4, 5) else
               ((c.km3 if proc in (1, 2, 3) else c.km3 * c.n_ens) if (c.l_vertical_filter and c.lm > 1) else 0)),
        l_vertical_filter=bool(c.l_vertical_filter and c.lm > 1), l_filt_g1=bool(c.l_filt_g1),
        lquart=bool(c.lquart), lhelm=bool(c.lhelm), nthreads=nthreads, ampl03=c.mg_ampl03,
        mgbf_line=bool(c.mgbf_line))


def rel_l2(a, b) -> float:
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (den if den > 0 else 1.0))


def canonical(h: int, p: int = 2) -> float:
    """mg_ampl02 giving a radial disk of radius h + 1/2 (reach h)."""
    return (h + 0.5) ** 2 / (2 * p + 4)


def canonical_z(hz: int, p: int = 2) -> float:
    """mg_ampl01 giving a vertical reach hz."""
    return (hz + 0.5) ** 2 / (2 * p + 3)


def small_config(**kw) -> MGBFConfig:
    d = dict(nxPE=4, nyPE=4, im_filt=16, jm_filt=12, lm=8, km3=2, km2=0, n_ens=1, gm_max=3,
             hx=4, hy=4, hz=2, p=2, mg_ampl02=canonical(4), mg_ampl01=canonical_z(2),
             mg_weig1=1.0, mg_weig2=0.5, mg_weig3=0.25, mg_weig4=0.125, mg_weig5=0.0625,
             layout=1)
    d.update(kw)
    return MGBFConfig(**d)
