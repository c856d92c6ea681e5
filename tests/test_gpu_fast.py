"""GPU parity of the fast 1D+1D filters, filtering_procedure(3) and (8)
(filtering_fast_bckg / filtering_fast_ens), against the FP64 oracle."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import oracle as O
from standalone_mgbf_loc_gb300 import MGBF, _abi
from tests.helpers import canonical_z, oracle_cfg, rel_l2, small_config

pytestmark = pytest.mark.gpu

TOL = {torch.float64: 1e-12, torch.float32: 1e-5, torch.bfloat16: 2e-2}


def fast_config(**kw):
    # mg_ampl02 = 0.4: line reach floor(sqrt(7)/0.4) = 6 (the radial reach is 1)
    d = dict(nxPE=4, nyPE=4, im_filt=16, jm_filt=16, lm=8, km3=2, gm_max=3, hx=6, hy=6, hz=2,
             mg_ampl02=0.4, mg_ampl01=canonical_z(2))
    d.update(kw)
    return small_config(**d)


def run_gpu(op, proc, x, dtype, cuda, adjoint=False):
    t = torch.from_numpy(x).to(device=cuda, dtype=dtype).contiguous()
    if adjoint:
        op.filtering_procedure_adjoint(proc, t)
    else:
        op.filtering_procedure(proc, t)
    torch.cuda.synchronize()
    op.status()
    return t.double().cpu().numpy()


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32, torch.bfloat16])
@pytest.mark.parametrize("proc", [3, 8])
@pytest.mark.parametrize("lquart", [False, True])
def test_fast_parity(lib, cuda, dtype, proc, lquart):
    c = fast_config(lquart=lquart, n_ens=1 if proc == 3 else 2)
    op = MGBF(c)
    assert op.dims.reach_line == 6
    x = np.random.default_rng(31 + proc).standard_normal(op.field_shape())
    y = run_gpu(op, proc, x, dtype, cuda)
    assert rel_l2(y, O.filter_compact(oracle_cfg(c, proc), x)) < TOL[dtype]


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("ampl02", [0.9, 0.2, 0.12])
def test_fast_reaches(lib, cuda, dtype, ampl02):
    """Line reaches 2 (window kernel, reach <= 4), 13 (<= 16; the FP64
    path's generic kernel) and 22 (generic kernel for every type)."""
    reach = int(np.floor(np.sqrt(7) / ampl02 - 1e-12))
    h = max(reach, 2)
    c = fast_config(im_filt=32, jm_filt=32, gm_max=2, hx=h, hy=h, mg_ampl02=ampl02)
    op = MGBF(c)
    assert op.dims.reach_line == reach
    x = np.random.default_rng(7).standard_normal(op.field_shape())
    y = run_gpu(op, 3, x, dtype, cuda)
    assert rel_l2(y, O.filter_compact(oracle_cfg(c, 3), x)) < TOL[dtype]


def test_fast_unaligned_levels(lib, cuda):
    """nk = 5 levels: the one-level-per-thread line kernel."""
    c = fast_config(lm=5, km3=1)
    op = MGBF(c)
    assert op.dims.km_all == 5
    x = np.random.default_rng(8).standard_normal(op.field_shape())
    y = run_gpu(op, 3, x, torch.float32, cuda)
    assert rel_l2(y, O.filter_compact(oracle_cfg(c, 3), x)) < TOL[torch.float32]


@pytest.mark.parametrize("proc", [3, 8])
def test_fast_halo_layout_keeps_corners(lib, cuda, proc):
    """VALL with halos in place: the line filters zero the x halo of the
    interior rows and the y halo of the interior columns and leave the
    corners as they were."""
    c = fast_config(layout=_abi.MGBF_LAYOUT_HALO, n_ens=1 if proc == 3 else 2)
    op = MGBF(c)
    v = np.random.default_rng(9).standard_normal(op.field_shape())
    ref = v.copy()
    O.filtering_procedure(oracle_cfg(c, proc), ref)
    y = run_gpu(op, proc, v, torch.float64, cuda)
    assert rel_l2(y, ref) < 1e-12
    hx, hy = c.hx, c.hy
    assert np.array_equal(y[:hy, :hx], v[:hy, :hx]) and np.array_equal(y[-hy:, -hx:], v[-hy:, -hx:])
    assert np.abs(y[hy:-hy, :hx]).max() == 0.0 and np.abs(y[:hy, hx:-hx]).max() == 0.0


@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-14), (torch.float32, 1e-6)])
@pytest.mark.parametrize("proc", [3, 8])
def test_fast_adjoint_dot_product(lib, cuda, dtype, tol, proc):
    c = fast_config(n_ens=1 if proc == 3 else 2)
    op = MGBF(c)
    rng = np.random.default_rng(10)
    x, w = rng.standard_normal(op.field_shape()), rng.standard_normal(op.field_shape())
    lx = run_gpu(op, proc, x, dtype, cuda)
    ltw = run_gpu(op, proc, w, dtype, cuda, adjoint=True)
    assert abs(np.vdot(lx, w) - np.vdot(x, ltw)) <= tol * np.linalg.norm(lx) * np.linalg.norm(w)


def test_fast_weight_gradients(lib, cuda):
    c = fast_config(n_ens=2)
    op = MGBF(c)
    rng = np.random.default_rng(11)
    x, gy = rng.standard_normal(op.field_shape()), rng.standard_normal(op.field_shape())
    tx = torch.from_numpy(x).to(cuda)
    tg = torch.from_numpy(gy).to(cuda)
    gx, ga = op.apply_with_weight_grads(8, tx, tg)
    torch.cuda.synchronize()
    oc = oracle_cfg(c, 8)
    assert np.allclose(ga, O.weight_grads(oc, x, gy), rtol=1e-10, atol=1e-10)
    assert rel_l2(gx.cpu().numpy(), O.filter_compact(oc, gy)) < 1e-12


@pytest.mark.parametrize("graphs", [False, True])
def test_fast_batch_groups(lib, cuda, graphs):
    """A batch switched to procedure 8: every group == its own oracle run."""
    from standalone_mgbf_loc_gb300 import GroupDesc, MGBFBatch
    I = J = 64
    gm = 3
    w = [1.0, 0.5, 0.25]
    groups = [
        GroupDesc(nk=3 * 8, lm=8, nzcol=3, hx=6, hy=6, hz=2, p=2, mg_ampl01=canonical_z(2), mg_ampl02=0.4),
        GroupDesc(nk=5, lm=1, nzcol=0, hx=9, hy=9, hz=2, p=2, mg_ampl01=canonical_z(2), mg_ampl02=0.3),
    ]
    b = MGBFBatch(I, J, gm, w, groups)
    b.set_procedure(8)
    b.use_graphs(graphs)
    rng = np.random.default_rng(12)
    xs = [rng.standard_normal((J, I, g.nk)) for g in groups]
    ts = [torch.empty((J, I, g.nk), device=cuda, dtype=torch.float32) for g in groups]
    for _ in range(3 if graphs else 1):  # with graphs: direct, capture, replay (same pointers)
        for t, x in zip(ts, xs):
            t.copy_(torch.from_numpy(x))
        b.apply(ts)
    torch.cuda.synchronize()
    b.status()
    for g, x, t in zip(groups, xs, ts):
        oc = O.OracleConfig(I=I, J=J, nk=g.nk, hx=g.hx, hy=g.hy, hz=g.hz, p=g.p, ampl01=g.mg_ampl01,
                            ampl02=g.mg_ampl02, gm=gm, weights=w, proc=8, lm=g.lm, nzcol=g.nzcol,
                            l_vertical_filter=g.nzcol > 0)
        assert rel_l2(t.double().cpu().numpy(), O.filter_compact(oc, x)) < 1e-5
