"""Definitions of the golden cases (shared by the generator and the tests)."""
import numpy as np

from oracle import oracle as O
from tests.helpers import canonical, canonical_z, oracle_cfg
from standalone_mgbf_loc_gb300.mgbf import MGBFConfig

# name -> (namelist-style config, procedure, input kind, seed)
CASES = {
    "proc1_impulse": (dict(lm=4, km3=1, km2=0, n_ens=1, lquart=False), 1, "impulse", 0),
    "proc1_lquart_noise": (dict(lm=4, km3=1, km2=0, n_ens=1, lquart=True), 1, "noise", 1),
    "proc6_nofilt1_noise": (dict(lm=4, km3=1, km2=0, n_ens=2, l_filt_g1=False), 6, "noise", 2),
    "proc1_2d_var_noise": (dict(lm=4, km3=1, km2=1, n_ens=1), 1, "noise", 3),
}


def case_config(name) -> MGBFConfig:
    kw, _, _, _ = CASES[name]
    d = dict(nxPE=4, nyPE=4, im_filt=8, jm_filt=8, gm_max=3, hx=4, hy=4, hz=1, p=2,
             mg_ampl02=canonical(4), mg_ampl01=canonical_z(1), mg_ampl03=0.3,
             mg_weig1=1.0, mg_weig2=0.5, mg_weig3=0.25, layout=1)
    d.update(kw)
    return MGBFConfig(**d)


def case_oracle_cfg(name) -> O.OracleConfig:
    return oracle_cfg(case_config(name), CASES[name][1])


def case_input(name) -> np.ndarray:
    c = case_config(name)
    nk = (c.km2 + c.lm * c.km3) * c.n_ens
    shape = (c.nyPE * c.jm_filt, c.nxPE * c.im_filt, nk)
    _, _, kind, seed = CASES[name]
    if kind == "impulse":
        x = np.zeros(shape)
        x[shape[0] // 2 - 1, shape[1] // 2 - 1, 1] = 1.0
        return x
    return np.random.default_rng(seed).standard_normal(shape)
