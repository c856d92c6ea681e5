"""GPU parity of filtering_procedure(4), filtering_rad3, against the FP64
oracle: the 3D ball on the 3D variables, the 2D radial filter on the 2D
ones, the reference's halo behaviour included."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import oracle as O
from standalone_mgbf_loc_gb300 import MGBF, _abi
from tests.helpers import canonical, oracle_cfg, rel_l2, small_config

pytestmark = pytest.mark.gpu

TOL = {torch.float64: 1e-12, torch.float32: 1e-5, torch.bfloat16: 2e-2}


def rad3_config(**kw):
    # 2 3D variables of 6 levels + km2 2D ones; ball reach 2 (mg_ampl03 = 1),
    # disk reach 3
    d = dict(nxPE=4, nyPE=4, im_filt=16, jm_filt=16, lm=6, km3=2, km2=2, gm_max=3, hx=3, hy=3, hz=2,
             mg_ampl02=canonical(3), mg_ampl03=1.0)
    d.update(kw)
    return small_config(**d)


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32, torch.bfloat16])
@pytest.mark.parametrize("lquart", [False, True])
@pytest.mark.parametrize("km2", [0, 2])
def test_rad3_parity_compact(lib, cuda, dtype, lquart, km2):
    c = rad3_config(lquart=lquart, km2=km2, layout=_abi.MGBF_LAYOUT_COMPACT)
    op = MGBF(c)
    x = np.random.default_rng(40 + km2).standard_normal(op.field_shape())
    t = torch.from_numpy(x).to(cuda, dtype).contiguous()
    op.filtering_procedure(4, t)
    torch.cuda.synchronize()
    op.status()
    assert rel_l2(t.double().cpu().numpy(), O.filter_compact(oracle_cfg(c, 4), x)) < TOL[dtype]


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("gm", [1, 3])
def test_rad3_parity_halo_layout(lib, cuda, dtype, gm):
    """VALL with a random halo: the adjoint side folds the caller's halo into
    the 3D variables, and the result's halo holds the mirror fill (3D) and
    zero (2D), as in the reference."""
    c = rad3_config(layout=_abi.MGBF_LAYOUT_HALO, gm_max=gm)
    op = MGBF(c)
    v = np.random.default_rng(41).standard_normal(op.field_shape())
    ref = v.copy()
    O.filtering_procedure(oracle_cfg(c, 4), ref)
    t = torch.from_numpy(v).to(cuda, dtype).contiguous()
    op.filtering_procedure(4, t)
    torch.cuda.synchronize()
    assert rel_l2(t.double().cpu().numpy(), ref) < TOL[dtype]


def test_rad3_ball_reaches(lib, cuda):
    """Ball reach 1 (mg_ampl03 = 0.3), 3 (1.5), 4 (2.0, the widest row
    kernel) and 5 (3.0, beyond the row kernels: the per-tap kernel)."""
    for a3, hz, h in ((0.3, 2, 3), (1.5, 3, 3), (2.0, 4, 4), (3.0, 5, 5)):
        c = rad3_config(mg_ampl03=a3, hz=hz, hx=h, hy=h, layout=_abi.MGBF_LAYOUT_COMPACT)
        op = MGBF(c)
        x = np.random.default_rng(42).standard_normal(op.field_shape())
        t = torch.from_numpy(x).to(cuda).contiguous()
        op.filtering_procedure(4, t)
        torch.cuda.synchronize()
        assert rel_l2(t.cpu().numpy(), O.filter_compact(oracle_cfg(c, 4), x)) < 1e-12
