"""GPU parity of filtering_procedure(5), filtering_lin3, against the FP64
oracle: per generation the 2D variables through procedure 2's triad line
filters, the 3D variables through the seven colors of the hexad (adjoint
side: vdibetax3t + bocoT_3d per color, then the weight; forward side: the
z mirror once, then boco_3d + vdibetax3 per color), with the generation-1
halo forms of the reference (east edge mirrored about the last column, east
column and north row folded onto themselves); restriction and
prolongation as procedure 1, no separate vertical filter."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import oracle as O
from standalone_mgbf_loc_gb300 import MGBF, _abi
from tests.helpers import canonical, oracle_cfg, rel_l2, small_config

pytestmark = pytest.mark.gpu

TOL = {torch.float64: 1e-12, torch.float32: 1e-5, torch.bfloat16: 2e-2}


def lin3_config(**kw):
    # mgbf_line on: x, y and z lines of spread^2 1/sqrt(mg_ampl03) (half-span
    # 2 at 0.6), three identity diagonals, color 7 null; 2D variables with
    # proc 2's lines
    d = dict(layout=_abi.MGBF_LAYOUT_COMPACT, mgbf_line=True, mg_ampl03=0.6, lm=8, km3=2, hz=3)
    d.update(kw)
    return small_config(**d)


def run(op, x, dtype):
    t = torch.from_numpy(x).to(torch.device("cuda"), dtype).contiguous()
    op.filtering_procedure(5, t)
    torch.cuda.synchronize()
    op.status()
    return t.double().cpu().numpy()


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32, torch.bfloat16])
@pytest.mark.parametrize("lquart", [False, True])
@pytest.mark.parametrize("km2", [0, 2])
def test_lin3_parity_compact(lib, cuda, dtype, lquart, km2):
    c = lin3_config(lquart=lquart, km2=km2)
    op = MGBF(c)
    x = np.random.default_rng(70 + km2).standard_normal(op.field_shape())
    assert rel_l2(run(op, x, dtype), O.filter_compact(oracle_cfg(c, 5), x)) < TOL[dtype]


@pytest.mark.parametrize("ampl03,hz", [(0.6, 3), (0.35, 4), (1.5, 3)])
def test_lin3_spans(lib, cuda, ampl03, hz):
    """Other 3D spans (half-span 3 at mg_ampl03 0.35, 2 at 1.5) and z halos
    (def_mg_weights' reach check of the 3D ball on mg_ampl03 sets the
    smallest hz a handle accepts)."""
    c = lin3_config(mg_ampl03=ampl03, hz=hz, hx=6, hy=6, mg_ampl02=canonical(4))
    op = MGBF(c)
    x = np.random.default_rng(71).standard_normal(op.field_shape())
    assert rel_l2(run(op, x, torch.float64), O.filter_compact(oracle_cfg(c, 5), x)) < 1e-12


def test_lin3_east_edge_and_north_row(lib, cuda):
    """An impulse in the east column and one in the north row at
    generation 1: the bocoT_3d_g1 fold adds those lines to themselves once
    per adjoint color; GPU and oracle agree there too."""
    c = lin3_config(gm_max=1)
    op = MGBF(c)
    J, I, nk = op.field_shape()
    x = np.zeros((J, I, nk))
    x[J // 2, I - 1, 3] = 1.0
    x[J - 1, I // 3, 9] = 1.0
    assert rel_l2(run(op, x, torch.float64), O.filter_compact(oracle_cfg(c, 5), x)) < 1e-12


def test_lin3_small_coarse_generations(lib, cuda):
    """Generation 3 of 4x3 points with halos of 3: fills and folds read
    and write across both halo bands."""
    c = lin3_config(nxPE=1, nyPE=1, im_filt=16, jm_filt=12, gm_max=3, hx=3, hy=3, mg_ampl02=canonical(3),
                    gm_uncapped=True)
    op = MGBF(c)
    x = np.random.default_rng(72).standard_normal(op.field_shape())
    assert rel_l2(run(op, x, torch.float64), O.filter_compact(oracle_cfg(c, 5), x)) < 1e-12


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_lin3_parity_halo_layout(lib, cuda, dtype):
    c = lin3_config(layout=_abi.MGBF_LAYOUT_HALO, km2=1)
    op = MGBF(c)
    v = np.random.default_rng(73).standard_normal(op.field_shape())
    ref = v.copy()
    O.filtering_procedure(oracle_cfg(c, 5), ref)
    assert rel_l2(run(op, v, dtype), ref) < TOL[dtype]


def test_lin3_without_mgbf_line_copies(lib, cuda):
    """Without mgbf_line every color copies: the 3D part is the identity
    between the halo routines, as in the oracle."""
    c = lin3_config(mgbf_line=False)
    op = MGBF(c)
    x = np.random.default_rng(74).standard_normal(op.field_shape())
    assert rel_l2(run(op, x, torch.float64), O.filter_compact(oracle_cfg(c, 5), x)) < 1e-12


def test_lin3_repeated_calls_and_host_memory(lib, cuda):
    """The work arrays carry state from the adjoint to the forward side of a
    generation; a second call and a host-memory call give the same result."""
    c = lin3_config()
    op = MGBF(c)
    x = np.random.default_rng(75).standard_normal(op.field_shape())
    a = run(op, x, torch.float64)
    b = run(op, x, torch.float64)
    h = x.copy()
    op.filtering_procedure(5, h)
    assert np.array_equal(a, b) and np.array_equal(a, h)
