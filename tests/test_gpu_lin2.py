"""GPU parity of filtering_procedure(2), filtering_lin2_bckg, against the FP64
oracle: per generation the three dibeta line filters of the triad
(colors 3, 2, 1 as dibetat + bocoT_2d, then colors 1, 2, 3 as boco_2d +
dibeta), between the vertical filter, the restriction and the
prolongation of procedure 1."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import oracle as O
from standalone_mgbf_loc_gb300 import MGBF, _abi
from tests.helpers import canonical, oracle_cfg, rel_l2, small_config

pytestmark = pytest.mark.gpu

TOL = {torch.float64: 1e-12, torch.float32: 1e-5, torch.bfloat16: 2e-2}


def lin2_config(**kw):
    # mgbf_line on (init_mg_line runs): colors along x and y with half-span 2
    # (spread^2 0.63), identity diagonal
    d = dict(layout=_abi.MGBF_LAYOUT_COMPACT, mgbf_line=True)
    d.update(kw)
    return small_config(**d)


def run(op, x, dtype, proc=2, adjoint=False):
    t = torch.from_numpy(x).to(torch.device("cuda"), dtype).contiguous()
    if adjoint:
        op.filtering_procedure_adjoint(proc, t)
    else:
        op.filtering_procedure(proc, t)
    torch.cuda.synchronize()
    op.status()
    return t.double().cpu().numpy()


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32, torch.bfloat16])
@pytest.mark.parametrize("lquart", [False, True])
@pytest.mark.parametrize("km2", [0, 2])
def test_lin2_parity_compact(lib, cuda, dtype, lquart, km2):
    c = lin2_config(lquart=lquart, km2=km2)
    op = MGBF(c)
    x = np.random.default_rng(50 + km2).standard_normal(op.field_shape())
    assert rel_l2(run(op, x, dtype), O.filter_compact(oracle_cfg(c, 2), x)) < TOL[dtype]


@pytest.mark.parametrize("ampl02", [0.5, 0.3])
def test_lin2_longer_lines(lib, cuda, ampl02):
    """Half-span 3 (mg_ampl02 0.5: spread^2 1.41) and 3 with a wider
    fraction (0.3: spread^2 1.83) along x and y; the fast filters' line
    reach that every handle checks (5 and 8) sets the halo."""
    c = lin2_config(mg_ampl02=ampl02, hx=8, hy=8)
    op = MGBF(c)
    x = np.random.default_rng(51).standard_normal(op.field_shape())
    assert rel_l2(run(op, x, torch.float64), O.filter_compact(oracle_cfg(c, 2), x)) < 1e-12


def test_lin2_small_coarse_generations(lib, cuda):
    """Generation 3 is 4x3 points with a fold width of 3: a cell receives
    from both halo bands on the adjoint side."""
    c = lin2_config(nxPE=1, nyPE=1, im_filt=16, jm_filt=12, gm_max=3, hx=3, hy=3, mg_ampl02=canonical(3),
                    gm_uncapped=True)
    op = MGBF(c)
    x = np.random.default_rng(52).standard_normal(op.field_shape())
    assert rel_l2(run(op, x, torch.float64), O.filter_compact(oracle_cfg(c, 2), x)) < 1e-12


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_lin2_parity_halo_layout(lib, cuda, dtype):
    c = lin2_config(layout=_abi.MGBF_LAYOUT_HALO)
    op = MGBF(c)
    v = np.random.default_rng(53).standard_normal(op.field_shape())
    ref = v.copy()
    O.filtering_procedure(oracle_cfg(c, 2), ref)
    assert rel_l2(run(op, v, dtype), ref) < TOL[dtype]


def test_lin2_self_adjoint(lib, cuda):
    c = lin2_config()
    op = MGBF(c)
    rng = np.random.default_rng(54)
    a, b = rng.standard_normal(op.field_shape()), rng.standard_normal(op.field_shape())
    la = run(op, a, torch.float64)
    ltb = run(op, b, torch.float64, adjoint=True)
    assert abs((la * b).sum() - (a * ltb).sum()) < 1e-11 * np.abs(la * b).sum()


def test_lin2_weight_grads(lib, cuda):
    c = lin2_config()
    op = MGBF(c)
    rng = np.random.default_rng(55)
    x, gy = rng.standard_normal(op.field_shape()), rng.standard_normal(op.field_shape())
    tx = torch.from_numpy(x).to(cuda)
    tg = torch.from_numpy(gy).to(cuda)
    gx, ga = op.apply_with_weight_grads(2, tx, tg)
    torch.cuda.synchronize()
    oc = oracle_cfg(c, 2)
    assert np.allclose(ga, O.weight_grads(oc, x, gy), rtol=1e-10, atol=1e-10)
    assert rel_l2(gx.cpu().numpy(), O.filter_compact(oc, gy)) < 1e-12


@pytest.mark.parametrize("proc", [2, 7])
def test_lin2_without_mgbf_line_is_identity_filtering(lib, cuda, proc):
    """mgbf_line off: init_mg_line never runs, the generators stay zero and
    every color copies (vdibeta2's zero-generator branch)."""
    c = lin2_config(mgbf_line=False, n_ens=2 if proc == 7 else 1)
    op = MGBF(c)
    x = np.random.default_rng(57).standard_normal(op.field_shape())
    assert rel_l2(run(op, x, torch.float64, proc=proc), O.filter_compact(oracle_cfg(c, proc), x)) < 1e-12


def test_lin2_host_memory(lib, cuda):
    c = lin2_config()
    op = MGBF(c)
    x = np.random.default_rng(56).standard_normal(op.field_shape())
    y = x.copy()
    op.filtering_procedure(2, y)
    assert rel_l2(y, O.filter_compact(oracle_cfg(c, 2), x)) < 1e-12


# ------------------------------------------- proc 7: filtering_lin2_ens

@pytest.mark.parametrize("dtype", [torch.float64, torch.float32, torch.bfloat16])
@pytest.mark.parametrize("lquart", [False, True])
@pytest.mark.parametrize("filt_g1", [True, False])
def test_lin2_ens_parity_compact(lib, cuda, dtype, lquart, filt_g1):
    """Proc 7: two members stacked, ending with the adjoint vertical filter."""
    c = lin2_config(n_ens=2, lquart=lquart, l_filt_g1=filt_g1)
    op = MGBF(c)
    x = np.random.default_rng(60).standard_normal(op.field_shape())
    assert rel_l2(run(op, x, dtype, proc=7), O.filter_compact(oracle_cfg(c, 7), x)) < TOL[dtype]


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_lin2_ens_parity_halo_layout(lib, cuda, dtype):
    c = lin2_config(n_ens=2, layout=_abi.MGBF_LAYOUT_HALO)
    op = MGBF(c)
    v = np.random.default_rng(61).standard_normal(op.field_shape())
    ref = v.copy()
    O.filtering_procedure(oracle_cfg(c, 7), ref)
    assert rel_l2(run(op, v, dtype, proc=7), ref) < TOL[dtype]
