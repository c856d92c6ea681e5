"""GPU parity of the analysis <-> filter transfers (anal_to_filt_all2 /
filt_to_anal_all2) against the FP64 oracle."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import oracle as O
from standalone_mgbf_loc_gb300 import MGBF, _abi
from tests.helpers import canonical, rel_l2, small_config

pytestmark = pytest.mark.gpu

TOL = {torch.float64: 1e-12, torch.float32: 1e-5, torch.bfloat16: 2e-2}
# (nm0, mm0, nxPE, nyPE, im_filt, jm_filt): per-rank ratios 1.125 x 1.5 (the
# shipped namelist's), 2 x 1 and 1 x 1.25
GEOMS = [(36, 24, 4, 2, 8, 8), (32, 16, 2, 2, 8, 8), (16, 20, 2, 2, 8, 8)]


def setup(geom, order, layout, lm=8, lm_a=None, km2=0, n_ens=1):
    nm0, mm0, nx, ny, im, jm = geom
    c = small_config(nxPE=nx, nyPE=ny, im_filt=im, jm_filt=jm, nm0=nm0, mm0=mm0, lm=lm, lm_a=lm_a or lm, km3=2,
                     km2=km2, n_ens=n_ens, hx=4, hy=4, mg_ampl02=canonical(2), layout=layout,
                     l_lin_horizontal=order == 1, l_quad_horizontal=order == 2)
    op = MGBF(c)
    xc = O.XferConfig(nm0=nm0, mm0=mm0, nxpe=nx, nype=ny, im=im, jm=jm, hx=4, hy=4, nkf=op.dims.km_all,
                      nka=op.dims.km_a_all, lm=lm, lm_a=lm_a or lm, en=2 * n_ens, order=order)
    return c, op, xc


def to_halo(xc, v):
    """A compact (J, I, nk) field inside a zero halo (J+2hy, I+2hx, nk)."""
    out = np.zeros(xc.vall_shape())
    out[xc.hy:xc.hy + xc.J, xc.hx:xc.hx + xc.I] = v
    return out


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32, torch.bfloat16])
@pytest.mark.parametrize("order", [1, 2, 3])
@pytest.mark.parametrize("layout", [_abi.MGBF_LAYOUT_HALO, _abi.MGBF_LAYOUT_COMPACT])
@pytest.mark.parametrize("geom", GEOMS)
def test_filt_to_anal(lib, cuda, dtype, order, layout, geom):
    c, op, xc = setup(geom, order, layout)
    v = np.random.default_rng(1).standard_normal(op.field_shape())
    vh = v.copy() if layout == _abi.MGBF_LAYOUT_HALO else to_halo(xc, v)
    ref = O.filt_to_anal(xc, vh)  # fills vh's interpolation halo
    tv = torch.from_numpy(v).to(cuda, dtype).contiguous()
    tw = torch.zeros(op.analysis_shape(), device=cuda, dtype=dtype)
    op.filt_to_anal(tv, tw)
    torch.cuda.synchronize()
    assert rel_l2(tw.double().cpu().numpy(), ref) < TOL[dtype]
    if layout == _abi.MGBF_LAYOUT_HALO:
        assert rel_l2(tv.double().cpu().numpy(), vh) < TOL[dtype]


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32, torch.bfloat16])
@pytest.mark.parametrize("order", [1, 2, 3])
@pytest.mark.parametrize("layout", [_abi.MGBF_LAYOUT_HALO, _abi.MGBF_LAYOUT_COMPACT])
@pytest.mark.parametrize("geom", GEOMS)
def test_anal_to_filt(lib, cuda, dtype, order, layout, geom):
    c, op, xc = setup(geom, order, layout)
    w = np.random.default_rng(2).standard_normal(op.analysis_shape())
    ref = O.anal_to_filt(xc, w)
    if layout == _abi.MGBF_LAYOUT_COMPACT:
        ref = ref[xc.hy:xc.hy + xc.J, xc.hx:xc.hx + xc.I]
    tw = torch.from_numpy(w).to(cuda, dtype).contiguous()
    tv = torch.full(op.field_shape(), 7.0, device=cuda, dtype=dtype)  # overwritten everywhere
    op.anal_to_filt(tw, tv)
    torch.cuda.synchronize()
    assert rel_l2(tv.double().cpu().numpy(), ref) < TOL[dtype]


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("n_ens", [1, 3])
def test_vertical_spec2_transfers(lib, cuda, dtype, n_ens):
    """lm_a = 2*lm-1: the vertical map in both directions."""
    c, op, xc = setup(GEOMS[0], 3, _abi.MGBF_LAYOUT_HALO, lm=6, lm_a=11, n_ens=n_ens)
    assert op.dims.km_a_all == 2 * 11 * n_ens
    rng = np.random.default_rng(3)
    v = rng.standard_normal(op.field_shape())
    w = rng.standard_normal(op.analysis_shape())
    tv = torch.from_numpy(v).to(cuda, dtype).contiguous()
    tw = torch.zeros(op.analysis_shape(), device=cuda, dtype=dtype)
    op.filt_to_anal(tv, tw)
    vh = v.copy()
    assert rel_l2(tw.double().cpu().numpy(), O.filt_to_anal(xc, vh)) < TOL[dtype]
    tw2 = torch.from_numpy(w).to(cuda, dtype).contiguous()
    op.anal_to_filt(tw2, tv)
    torch.cuda.synchronize()
    assert rel_l2(tv.double().cpu().numpy(), O.anal_to_filt(xc, w)) < TOL[dtype]


def test_host_memory_transfers(lib, cuda):
    c, op, xc = setup(GEOMS[0], 3, _abi.MGBF_LAYOUT_HALO)
    rng = np.random.default_rng(4)
    v = rng.standard_normal(op.field_shape())
    w = np.zeros(op.analysis_shape())
    vh = v.copy()
    op.filt_to_anal(v, w)  # host arrays: copied in and out, VALL's halo filled
    assert rel_l2(w, O.filt_to_anal(xc, vh)) < 1e-12
    assert rel_l2(v, vh) < 1e-12
    w2 = rng.standard_normal(op.analysis_shape())
    op.anal_to_filt(w2, v)
    assert rel_l2(v, O.anal_to_filt(xc, w2)) < 1e-12


def test_transfer_filter_chain_is_self_adjoint(lib, cuda):
    """The driver's chain a2f -> filtering_procedure(1) -> f2a, on the
    analysis grid: <C w, u> = <w, C u> (the transfers are an adjoint pair
    and the filter is self-adjoint)."""
    c, op, xc = setup(GEOMS[0], 3, _abi.MGBF_LAYOUT_COMPACT)
    rng = np.random.default_rng(5)

    def chain(w):
        tw = torch.from_numpy(w).to(cuda).contiguous()
        tv = torch.zeros(op.field_shape(), device=cuda, dtype=torch.float64)
        op.anal_to_filt(tw, tv)
        op.filtering_procedure(1, tv)
        out = torch.zeros_like(tw)
        op.filt_to_anal(tv, out)
        torch.cuda.synchronize()
        return out.cpu().numpy()

    w, u = rng.standard_normal(op.analysis_shape()), rng.standard_normal(op.analysis_shape())
    cw, cu = chain(w), chain(u)
    assert abs((cw * u).sum() - (w * cu).sum()) < 1e-12 * np.linalg.norm(cw) * np.linalg.norm(u)
