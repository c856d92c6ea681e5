"""CPU tests of the C-ABI library: it loads, exports every symbol that
include/mgbf.h declares, and its host-side logic (namelist, validation,
error codes) works without a GPU.  No compute call is made here."""
import ctypes
import os
import re

import numpy as np
import pytest

from standalone_mgbf_loc_gb300 import MGBF, MGBFConfig, MGBFError, _abi
from oracle import oracle as O
from tests.helpers import canonical, canonical_z, oracle_cfg, small_config

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    text = open(os.path.join(ROOT, "include", "mgbf.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(mgbf_[a-z_0-9]+)\s*\(", text)))


def test_every_declared_symbol_is_exported(lib):
    names = header_functions()
    assert len(names) >= 15
    for n in names:
        assert hasattr(lib, n), n
        assert n in _abi.SIGNATURES, n


def test_strerror_codes(lib):
    for code in range(0, -11, -1):
        assert lib.mgbf_strerror(code)
    assert lib.mgbf_strerror(-99) == b"unknown error"


NML = """
&PARAMETERS_MGBETA
! comment line
  mg_ampl01=2.0, mg_ampl02=5.28125, mg_ampl03=1.,
  mg_weig1=10.,mg_weig2=50.,mg_weig3=100.,mg_weig4=200.,mg_weig5=0.,
  hx=6,hy=6,hz=3,p=2,
  mgbf_line=.false., mgbf_proc=6, n_ens=20,
  lm_a = 65, lm = 65,
  km2=0,km3=6,
  l_loc=.false.
  l_filt_g1 =.true.,
  l_vertical_filter=.true.,
  ldelta=.true.,
  lquart=.false., lhelm=.false.,
  gm_max=4,
  nm0 = 1440, mm0 = 960,
  nxPE=20,nyPE=20,im_filt=64,jm_filt=32,
/
"""


def write(tmp_path, text, name="mgbeta.nml"):
    p = tmp_path / name
    p.write_text(text)
    return str(p)


def test_namelist_parse(lib, tmp_path):
    c = MGBFConfig.from_namelist(write(tmp_path, NML))
    assert c.mgbf_proc == 6 and c.n_ens == 20 and c.lm == 65 and c.km3 == 6
    assert c.mg_weig4 == 200.0 and c.mg_ampl02 == 5.28125
    assert c.l_filt_g1 and c.l_vertical_filter and not c.lquart and c.ldelta
    assert (c.nxPE, c.nyPE, c.im_filt, c.jm_filt) == (20, 20, 64, 32)


def test_namelist_mgbf_line_reaches_the_line_filter_setup(lib, tmp_path):
    """mgbf_line from the namelist decides whether procs 2/5/7 get the triad
    line filters (init_mg_line) or copies, as mg_entrymod.f90:155-157 does."""
    text = NML.replace("mgbf_line=.false., mgbf_proc=6, n_ens=20", "mgbf_line=.true., mgbf_proc=2, n_ens=1")
    c = MGBFConfig.from_namelist(write(tmp_path, text))
    assert c.mgbf_line and c.mgbf_proc == 2
    cols = MGBF(c).line_filters()
    assert [col["d"] for col in cols] == [(1, 0), (0, 1), (-1, -1)]
    assert cols[0]["h"] >= 1 and abs(cols[0]["fil"][0] + 2 * cols[0]["fil"][1:].sum() - 1.0) < 1e-14
    c_off = MGBFConfig.from_namelist(write(tmp_path, NML, "off.nml"))
    assert all(col["h"] == 0 for col in MGBF(c_off).line_filters())


def test_namelist_case_and_fortran_exponents(lib, tmp_path):
    text = NML.replace("&PARAMETERS_MGBETA", "&parameters_mgbeta").replace("mg_ampl01=2.0", "MG_AMPL01=2.0D0")
    c = MGBFConfig.from_namelist(write(tmp_path, text))
    assert c.mg_ampl01 == 2.0


def test_namelist_real_for_integer_p_is_rejected(lib, tmp_path):
    # the shipped RUN/mgbf.nml says p=1.3 while p is an integer (mg_parameter.f90:110)
    with pytest.raises(MGBFError) as e:
        MGBFConfig.from_namelist(write(tmp_path, NML.replace("p=2", "p=1.3")))
    assert e.value.code == _abi.MGBF_ERR_NAMELIST


def test_namelist_unknown_item(lib, tmp_path):
    with pytest.raises(MGBFError) as e:
        MGBFConfig.from_namelist(write(tmp_path, NML.replace("hx=6", "hxx=6")))
    assert e.value.code == _abi.MGBF_ERR_NAMELIST


def test_namelist_missing_file(lib):
    with pytest.raises(MGBFError) as e:
        MGBFConfig.from_namelist("/nonexistent/mgbeta.nml")
    assert e.value.code == _abi.MGBF_ERR_IO


def test_namelist_extensions(lib, tmp_path):
    text = NML.replace("gm_max=4,", "gm_max=6, gm_uncapped=.true., weig_ext=1.0,0.5,0.25, layout=1,")
    c = MGBFConfig.from_namelist(write(tmp_path, text))
    assert c.gm_uncapped and c.weig_ext == [1.0, 0.5, 0.25] and c.layout == 1


def test_create_from_namelist_and_dims(lib, tmp_path):
    op = MGBF.from_namelist(write(tmp_path, NML))
    d = op.dims
    assert (d.im, d.jm) == (1280, 640)
    assert d.km_all == 20 * 65 * 6 and d.km3_all == 120
    assert d.gm == 4  # min(gm_max, def_maxgen(20, 20) = 6)
    assert d.reach_h == 6 and d.hbeta_kernel == 1
    assert op.field_shape() == (640 + 12, 1280 + 12, 20 * 65 * 6)
    op.close()


def test_generation_cap_follows_rank_layout(lib):
    c = small_config(nxPE=2, nyPE=2, im_filt=32, jm_filt=32, gm_max=4, hx=4, hy=4)
    assert MGBF(c).dims.gm == 2  # def_maxgen(2,2) = 2
    c.gm_uncapped = True
    assert MGBF(c).dims.gm == 4


@pytest.mark.parametrize("change,code", [
    (dict(hx=3), _abi.MGBF_ERR_REACH),                       # getlinesum2 stop
    (dict(hz=1), _abi.MGBF_ERR_REACH),                       # getlinesum1 stop
    (dict(nxPE=1, im_filt=66, gm_uncapped=True), _abi.MGBF_ERR_DIVISIBILITY),  # 66 % 4
    (dict(nm0=10), _abi.MGBF_ERR_CONFIG),                    # nm0 not divisible by nxm
    (dict(mg_ampl03=100.0), _abi.MGBF_ERR_REACH),            # getlinesum3 on pasp3
    (dict(helm_b=[0.1]), _abi.MGBF_ERR_UNSUPPORTED),
    (dict(p=-1), _abi.MGBF_ERR_CONFIG),
])
def test_create_validation(lib, change, code):
    with pytest.raises(MGBFError) as e:
        MGBF(small_config(**change))
    assert e.value.code == code


def test_reach_larger_than_coarsest_generation(lib):
    c = small_config(nxPE=1, nyPE=1, im_filt=16, jm_filt=16, gm_max=3, gm_uncapped=True,
                     hx=6, hy=6, mg_ampl02=canonical(6))
    with pytest.raises(MGBFError) as e:
        MGBF(c)
    assert e.value.code == _abi.MGBF_ERR_DIVISIBILITY


def test_unsupported_and_unknown_procedures(lib):
    op = MGBF(small_config())
    x = np.zeros(op.field_shape())
    # filtering_lin3 (5) is not self-adjoint: adjoint and weight gradients are refused
    with pytest.raises(MGBFError) as e:
        op.filtering_procedure_adjoint(5, x)
    assert e.value.code == _abi.MGBF_ERR_UNSUPPORTED
    with pytest.raises(MGBFError) as e:
        op.apply_with_weight_grads(5, x, x.copy())
    assert e.value.code == _abi.MGBF_ERR_UNSUPPORTED
    # proc 5 with several members is refused like the other background procedures
    with pytest.raises(MGBFError) as e:
        MGBF(small_config(n_ens=2)).filtering_procedure(5, np.zeros(MGBF(small_config(n_ens=2)).field_shape()))
    assert e.value.code == _abi.MGBF_ERR_CONFIG
    # no case default in the reference's select: other values do nothing
    x[...] = 1.0
    op.filtering_procedure(0, x)
    op.filtering_procedure(9, x)
    assert (x == 1.0).all()


def test_line_filter_procedure_validation(lib):
    """filtering_lin2_bckg (proc 2): a spread beyond the moment table or a
    line reach beyond the halo is refused before any device work."""
    # spread^2 1/sqrt(0.035) = 5.3 lies beyond the table's largest (half-span
    # 6: 5.14); the fast filters' line reach 75 that every handle checks
    # (def_mg_weights) needs the 80-point halo
    op = MGBF(small_config(mg_ampl02=0.035, hx=80, hy=80, im_filt=32, jm_filt=32, gm_max=1, mgbf_line=True))
    with pytest.raises(MGBFError) as e:
        op.filtering_procedure(2, np.zeros(op.field_shape()))
    assert e.value.code == _abi.MGBF_ERR_REACH
    with pytest.raises(MGBFError) as e:  # proc 2 is a single-member procedure
        MGBF(small_config(n_ens=2)).filtering_procedure(2, np.zeros(MGBF(small_config(n_ens=2)).field_shape()))
    assert e.value.code == _abi.MGBF_ERR_CONFIG


@pytest.mark.parametrize("p", [1, 2, 3, 4])
@pytest.mark.parametrize("ampl02", [3.0, 1.2, 0.6, 0.3, 0.15])
def test_line_filter_setup_matches_oracle(lib, p, ampl02):
    """The library's own setup of procedure 2's line filters (triad,
    half-span transform, two-beta weights) equals the oracle's."""
    # every handle checks the fast filters' line reach and the radial disk's
    line = int(np.floor(np.sqrt(2 * p + 3) / ampl02 - 1e-12))
    disk = int(np.floor(np.sqrt((2 * p + 4) * ampl02) - 1e-12))
    h = max(4, line, disk)
    c = small_config(p=p, mg_ampl02=ampl02, hx=h, hy=h, nxPE=1, nyPE=1, im_filt=64, jm_filt=64, gm_max=2,
                     mg_ampl01=canonical_z(2, p), mg_ampl03=0.3, mgbf_line=True)
    got = MGBF(c).line_filters()
    ref = O.dibeta_values(oracle_cfg(c, 2))
    for g, r in zip(got, ref):
        assert g["d"] == r["d"] and g["h"] == r["h"]
        assert abs(g["hs"] - r["hs"]) < 1e-13
        assert np.abs(g["fil"] - r["fil"]).max() < 1e-15


def test_line_filter_setup_error_is_reported(lib):
    op = MGBF(small_config(mg_ampl02=0.035, hx=80, hy=80, im_filt=32, jm_filt=32, gm_max=1, mgbf_line=True))
    with pytest.raises(MGBFError) as e:
        op.line_filters()
    assert e.value.code == _abi.MGBF_ERR_REACH


def test_line_filters_are_identities_without_mgbf_line(lib):
    """mgbf_line off: init_mg_line does not run (mg_entrymod.f90:155-157),
    so no table limit applies and every color is a copy."""
    op = MGBF(small_config(mg_ampl02=0.035, hx=80, hy=80, im_filt=32, jm_filt=32, gm_max=1, mgbf_line=False))
    for col in op.line_filters():
        assert col["h"] == 0 and col["fil"].tolist() == [1.0]


def test_adjoint_of_rad3_is_refused(lib):
    op = MGBF(small_config(lm=6, km3=2, km2=2, hz=2, mg_ampl03=1.0, layout=_abi.MGBF_LAYOUT_COMPACT))
    with pytest.raises(MGBFError) as e:
        op.filtering_procedure_adjoint(4, np.zeros(op.field_shape()))
    assert e.value.code == _abi.MGBF_ERR_UNSUPPORTED


def test_lin2_ens_not_self_adjoint_calls_refused(lib):
    """filtering_lin2_ens (proc 7) ends with the adjoint vertical filter:
    neither its adjoint nor its weight gradients are the symmetric chain."""
    op = MGBF(small_config(n_ens=2, layout=_abi.MGBF_LAYOUT_COMPACT))
    x = np.zeros(op.field_shape())
    with pytest.raises(MGBFError) as e:
        op.filtering_procedure_adjoint(7, x)
    assert e.value.code == _abi.MGBF_ERR_UNSUPPORTED
    with pytest.raises(MGBFError) as e:
        op.apply_with_weight_grads(7, x, x.copy())
    assert e.value.code == _abi.MGBF_ERR_UNSUPPORTED


def test_proc1_requires_single_member(lib):
    op = MGBF(small_config(n_ens=2))
    with pytest.raises(MGBFError) as e:
        op.filtering_procedure(1, np.zeros(op.field_shape()))
    assert e.value.code == _abi.MGBF_ERR_CONFIG


def test_proc6_vertical_requires_km2_zero(lib):
    op = MGBF(small_config(km2=1, n_ens=2))
    with pytest.raises(MGBFError) as e:
        op.filtering_procedure(6, np.zeros(op.field_shape()))
    assert e.value.code == _abi.MGBF_ERR_CONFIG


def test_shape_and_dtype_checks(lib):
    op = MGBF(small_config())
    with pytest.raises(MGBFError):
        op.filtering_procedure(1, np.zeros((3, 3, 3)))
    with pytest.raises(MGBFError):
        op.filtering_procedure(1, np.zeros(op.field_shape(), dtype=np.int32))


def test_null_arguments_rejected(lib):
    assert lib.mgbf_filtering_procedure(None, 1, None, 0, 0, None) == _abi.MGBF_ERR_ARG
    assert lib.mgbf_create(None, None) == _abi.MGBF_ERR_ARG
    assert lib.mgbf_destroy(None) == _abi.MGBF_OK


def test_set_tuning_validation(lib):
    """Pinning a radial-kernel variant is host-side bookkeeping: unknown
    variants and dtypes are rejected, valid ones and the reset are accepted."""
    op = MGBF(small_config())
    op.set_tuning(0)
    op.set_tuning(2, 5)
    op.set_tuning(-1)
    with pytest.raises(MGBFError):
        op.set_tuning(4)
    assert lib.mgbf_set_tuning(None, 1, 0, 0) == _abi.MGBF_ERR_ARG
    assert lib.mgbf_set_tuning(op._h, 7, 0, 0) == _abi.MGBF_ERR_ARG


def test_fast_line_reach_beyond_coarsest_generation(lib):
    """Procs 3/8 need the line reach within the coarsest generation (one
    mirror image); the handle still serves procs 1/6.  Checked before any
    device work, so no GPU is needed."""
    c = small_config(nxPE=4, nyPE=4, im_filt=16, jm_filt=16, gm_max=4, gm_uncapped=True, hx=13, hy=13,
                     mg_ampl02=0.2)
    op = MGBF(c)
    assert op.dims.gm == 4 and op.dims.reach_line == -1
    with pytest.raises(MGBFError) as e:
        op.filtering_procedure(3, np.zeros(op.field_shape()))
    assert e.value.code == _abi.MGBF_ERR_DIVISIBILITY
    assert "coarsest generation" in str(e.value)


def test_batch_set_procedure_validation(lib):
    from standalone_mgbf_loc_gb300 import GroupDesc, MGBFBatch
    ok = GroupDesc(nk=8, lm=8, nzcol=1, hx=6, hy=6, hz=2, p=2, mg_ampl01=canonical_z(2), mg_ampl02=0.4)
    b = MGBFBatch(64, 64, 3, [1.0, 0.5, 0.25], [ok])
    b.set_procedure(8)
    b.set_procedure(6)
    for bad in (1, 3, 7):
        with pytest.raises(MGBFError) as e:
            b.set_procedure(bad)
        assert e.value.code == _abi.MGBF_ERR_UNSUPPORTED
    # line reach 6 > hx = 4: the radial procedure still works, 8 is refused
    short = GroupDesc(nk=8, lm=8, nzcol=1, hx=4, hy=4, hz=2, p=2, mg_ampl01=canonical_z(2), mg_ampl02=0.4)
    b2 = MGBFBatch(64, 64, 3, [1.0, 0.5, 0.25], [short])
    with pytest.raises(MGBFError) as e:
        b2.set_procedure(8)
    assert e.value.code == _abi.MGBF_ERR_DIVISIBILITY


@pytest.mark.parametrize("change,code", [
    (dict(nm0=0, mm0=0), _abi.MGBF_ERR_CONFIG),
    (dict(l_new_map=False), _abi.MGBF_ERR_UNSUPPORTED),
    (dict(lm_a=5), _abi.MGBF_ERR_CONFIG),                       # neither lm nor 2*lm-1
    (dict(lm_a=15, km2=1), _abi.MGBF_ERR_UNSUPPORTED),          # spec2 blocks break with 2D variables
    (dict(hx=2, layout=_abi.MGBF_LAYOUT_HALO), _abi.MGBF_ERR_CONFIG),  # lsqr needs a halo of 3
])
def test_transfer_validation(lib, change, code):
    """Checked before any device work."""
    d = dict(nm0=72, mm0=48, lm=8, lm_a=8, km3=2, hx=4, hy=4, mg_ampl02=1.0)  # every reach 2
    d.update(change)
    op = MGBF(small_config(**d))
    with pytest.raises(MGBFError) as e:
        op.filt_to_anal(np.zeros(op.field_shape()), np.zeros(op.analysis_shape()))
    assert e.value.code == code


def test_rad3_validation(lib):
    """filtering_rad3: weight gradients are refused (its adjoint side is not
    the transpose of its forward side); a ball reach beyond hz is refused when
    the handle is created (getlinesum3 in def_mg_weights)."""
    op = MGBF(small_config(lm=6, km3=2, hz=2, hx=3, hy=3, mg_ampl02=canonical(3), mg_ampl03=1.0))
    x = np.zeros(op.field_shape())
    with pytest.raises(MGBFError) as e:
        op.apply_with_weight_grads(4, x, x)
    assert e.value.code == _abi.MGBF_ERR_UNSUPPORTED
    with pytest.raises(MGBFError) as e:
        MGBF(small_config(lm=6, km3=2, hz=2, hx=3, hy=3, mg_ampl02=canonical(3), mg_ampl03=1.5))
    assert e.value.code == _abi.MGBF_ERR_REACH
