"""GPU parity of libmgbf against the FP64 oracle, through the C-ABI.

Tolerances (relative L2 against the FP64 oracle):
  FP64 storage/arithmetic      1e-12
  FP32 storage/arithmetic      1e-5
  BF16 storage, FP32 arithmetic 2e-2  (2^-8 rounding at every stored stage)
"""
import numpy as np
import pytest

from oracle import oracle as O
from standalone_mgbf_loc_gb300 import MGBF, MGBFBatch, GroupDesc, _abi
from tests.helpers import canonical, canonical_z, oracle_cfg, rel_l2, small_config

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = {torch.float64: 1e-12, torch.float32: 1e-5, torch.bfloat16: 2e-2}


def run_gpu(op, proc, x, dtype, cuda, adjoint=False):
    t = torch.from_numpy(x).to(device=cuda, dtype=dtype).contiguous()
    if adjoint:
        op.filtering_procedure_adjoint(proc, t)
    else:
        op.filtering_procedure(proc, t)
    torch.cuda.synchronize()
    op.status()  # no bounded device wait ran out
    return t.double().cpu().numpy()


def compact_input(op, seed=0):
    return np.random.default_rng(seed).standard_normal(op.field_shape())


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32, torch.bfloat16])
@pytest.mark.parametrize("proc", [1, 6])
@pytest.mark.parametrize("lquart", [False, True])
def test_parity_moment_kernel(lib, cuda, dtype, proc, lquart):
    c = small_config(lquart=lquart, n_ens=1 if proc == 1 else 2)
    op = MGBF(c)
    assert op.dims.hbeta_kernel == 1
    x = compact_input(op)
    y = run_gpu(op, proc, x, dtype, cuda)
    ref = O.filter_compact(oracle_cfg(c, proc), x)
    assert rel_l2(y, ref) < TOL[dtype]


@pytest.mark.parametrize("h", [5, 8, 10, 12, 16, 24])
@pytest.mark.parametrize("dtype", [torch.float64, torch.float32, torch.bfloat16])
def test_parity_moment_kernel_reaches(lib, cuda, h, dtype):
    """Every compiled reach (the larger ones use > 48 KB of shared memory)."""
    c = small_config(nxPE=4, nyPE=4, im_filt=48 if h < 24 else 96, jm_filt=48 if h < 24 else 96, lm=8, km3=1,
                     gm_max=3, hx=h, hy=h, hz=2, mg_ampl02=canonical(h), mg_ampl01=canonical_z(2))
    op = MGBF(c)
    assert op.dims.hbeta_kernel == 1 and op.dims.reach_h == h
    x = compact_input(op, h)
    y = run_gpu(op, 1, x, dtype, cuda)
    assert rel_l2(y, O.filter_compact(oracle_cfg(c, 1), x)) < TOL[dtype]


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("ampl02", [2.0, 2.5, 1.3])
def test_parity_direct_kernel(lib, cuda, dtype, ampl02):
    c = small_config(mg_ampl02=ampl02)
    op = MGBF(c)
    assert op.dims.hbeta_kernel == 0
    x = compact_input(op, 1)
    y = run_gpu(op, 1, x, dtype, cuda)
    ref = O.filter_compact(oracle_cfg(c, 1), x)
    assert rel_l2(y, ref) < TOL[dtype]


@pytest.mark.parametrize("p", [1, 3])
def test_parity_other_powers(lib, cuda, p):
    c = small_config(p=p, mg_ampl02=canonical(4, p), mg_ampl01=canonical_z(2, p), mg_ampl03=0.5)
    op = MGBF(c)
    x = compact_input(op, 2)
    y = run_gpu(op, 1, x, torch.float64, cuda)
    assert rel_l2(y, O.filter_compact(oracle_cfg(c, 1), x)) < 1e-12


def test_proc6_without_generation1_filter(lib, cuda):
    c = small_config(n_ens=3, l_filt_g1=False)
    op = MGBF(c)
    x = compact_input(op, 3)
    y = run_gpu(op, 6, x, torch.float64, cuda)
    assert rel_l2(y, O.filter_compact(oracle_cfg(c, 6), x)) < 1e-12


def test_2d_variables_and_no_vertical_filter(lib, cuda):
    c = small_config(km2=3, km3=2)
    op = MGBF(c)
    x = compact_input(op, 4)
    y = run_gpu(op, 1, x, torch.float64, cuda)
    assert rel_l2(y, O.filter_compact(oracle_cfg(c, 1), x)) < 1e-12
    c2 = small_config(l_vertical_filter=False)
    op2 = MGBF(c2)
    y2 = run_gpu(op2, 1, x[..., :op2.dims.km_all], torch.float64, cuda)
    assert rel_l2(y2, O.filter_compact(oracle_cfg(c2, 1), x[..., :op2.dims.km_all])) < 1e-12


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_halo_layout_in_place(lib, cuda, dtype):
    """VALL(km_all, 1-hx:im+hx, 1-hy:jm+hy) in place; halos end up zero."""
    c = small_config(layout=_abi.MGBF_LAYOUT_HALO)
    op = MGBF(c)
    v = np.random.default_rng(5).standard_normal(op.field_shape())
    ref = v.copy()
    O.filtering_procedure(oracle_cfg(c, 1), ref)
    y = run_gpu(op, 1, v, dtype, cuda)
    assert rel_l2(y, ref) < TOL[dtype]
    hx, hy = c.hx, c.hy
    inner = np.zeros(y.shape, bool)
    inner[hy:-hy, hx:-hx, :] = True
    assert np.abs(y[~inner]).max() == 0.0


def test_host_memory_path(lib, cuda):
    c = small_config()
    op = MGBF(c)
    x = compact_input(op, 6)
    h64 = x.copy()
    op.filtering_procedure(1, h64)
    h32 = x.astype(np.float32)
    op.filtering_procedure(1, h32)
    ref = O.filter_compact(oracle_cfg(c, 1), x)
    assert rel_l2(h64, ref) < 1e-12
    assert rel_l2(h32, ref) < 1e-5


@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-14), (torch.float32, 1e-6)])
@pytest.mark.parametrize("proc", [1, 6])
def test_adjoint_dot_product(lib, cuda, dtype, tol, proc):
    """Dot-product test: |<Lx,y> - <x,L^T y>| / (||Lx|| ||y||) <= tol."""
    c = small_config(n_ens=1 if proc == 1 else 2)
    op = MGBF(c)
    rng = np.random.default_rng(7)
    x, y = rng.standard_normal(op.field_shape()), rng.standard_normal(op.field_shape())
    lx = run_gpu(op, proc, x, dtype, cuda)
    lty = run_gpu(op, proc, y, dtype, cuda, adjoint=True)
    a, b = (lx * y).sum(), (x * lty).sum()
    assert abs(a - b) / (np.linalg.norm(lx) * np.linalg.norm(y)) < tol


@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-11), (torch.float32, 1e-4)])
@pytest.mark.parametrize("proc", [1, 6])
def test_weight_gradients(lib, cuda, dtype, tol, proc):
    c = small_config(n_ens=1 if proc == 1 else 2)
    op = MGBF(c)
    rng = np.random.default_rng(8)
    x, gy = rng.standard_normal(op.field_shape()), rng.standard_normal(op.field_shape())
    tx = torch.from_numpy(x).to(cuda, dtype)
    tg = torch.from_numpy(gy).to(cuda, dtype)
    gx, ga = op.apply_with_weight_grads(proc, tx, tg)
    oc = oracle_cfg(c, proc)
    ga_ref = O.weight_grads(oc, x, gy)
    gx_ref = O.filter_compact(oc, gy)
    assert np.abs(ga - ga_ref).max() / np.abs(ga_ref).max() < tol
    assert rel_l2(gx.double().cpu().numpy(), gx_ref) < max(tol, TOL[dtype])


def test_autograd_function_finite_differences(lib, cuda):
    from standalone_mgbf_loc_gb300.autograd import mgbf_apply
    c = small_config()
    op = MGBF(c)
    rng = np.random.default_rng(9)
    x = torch.from_numpy(rng.standard_normal(op.field_shape())).to(cuda).requires_grad_(True)
    w = torch.tensor([1.0, 0.5, 0.25], dtype=torch.float64, device=cuda, requires_grad=True)
    r = torch.from_numpy(rng.standard_normal(op.field_shape())).to(cuda)
    loss = (mgbf_apply(op, x, w, 1) * r).sum()
    loss.backward()
    h = 1e-3
    for g in range(3):
        wp, wm = w.detach().clone(), w.detach().clone()
        wp[g] += h
        wm[g] -= h
        fd = ((mgbf_apply(op, x.detach(), wp, 1) * r).sum() - (mgbf_apply(op, x.detach(), wm, 1) * r).sum()) / (2 * h)
        assert float(w.grad[g]) == pytest.approx(float(fd), rel=1e-8, abs=1e-8)
    d = torch.from_numpy(rng.standard_normal(op.field_shape())).to(cuda)
    fd = ((mgbf_apply(op, x.detach() + h * d, w.detach(), 1) * r).sum()
          - (mgbf_apply(op, x.detach() - h * d, w.detach(), 1) * r).sum()) / (2 * h)
    assert float((x.grad * d).sum()) == pytest.approx(float(fd), rel=1e-8)


def test_config1_impulse_and_noise(lib, cuda):
    """256x256x32, 4 generations (8x8 ranks), h=6, hz=3, weights 1,.5,.25,.125."""
    c = small_config(nxPE=8, nyPE=8, im_filt=32, jm_filt=32, lm=32, km3=1, gm_max=4, hx=6, hy=6, hz=3,
                     mg_ampl02=canonical(6), mg_ampl01=canonical_z(3))
    op = MGBF(c)
    imp = np.zeros(op.field_shape())
    imp[127, 127, 15] = 1.0  # Fortran (128,128,16)
    noise = np.random.default_rng(0).standard_normal(op.field_shape())
    oc = oracle_cfg(c, 1)
    for x in (imp, noise):
        ref = O.filter_compact(oc, x)
        for dtype in (torch.float64, torch.float32):
            assert rel_l2(run_gpu(op, 1, x, dtype, cuda), ref) < TOL[dtype]


def test_batched_groups(lib, cuda):
    """Groups with their own reach and levels in one call == per-group oracle runs."""
    I = J = 64
    gm = 3
    w = [1.0, 0.5, 0.25]
    groups = [
        GroupDesc(nk=3 * 8, lm=8, nzcol=3, hx=4, hy=4, hz=2, p=2, mg_ampl01=canonical_z(2), mg_ampl02=canonical(4)),
        GroupDesc(nk=2 * 6, lm=6, nzcol=2, hx=6, hy=6, hz=2, p=2, mg_ampl01=canonical_z(2), mg_ampl02=canonical(6)),
        GroupDesc(nk=5, lm=1, nzcol=0, hx=5, hy=5, hz=2, p=2, mg_ampl01=canonical_z(2), mg_ampl02=canonical(5) * 0.9),
    ]
    b = MGBFBatch(I, J, gm, w, groups)
    rng = np.random.default_rng(10)
    xs = [rng.standard_normal((J, I, g.nk)) for g in groups]
    ts = [torch.from_numpy(x).to(cuda, torch.float32).contiguous() for x in xs]
    b.apply(ts)
    torch.cuda.synchronize()
    b.status()
    for g, x, t in zip(groups, xs, ts):
        oc = O.OracleConfig(I=I, J=J, nk=g.nk, hx=g.hx, hy=g.hy, hz=g.hz, p=g.p, ampl01=g.mg_ampl01,
                            ampl02=g.mg_ampl02, gm=gm, weights=w, proc=6, lm=g.lm, nzcol=g.nzcol,
                            l_vertical_filter=g.nzcol > 0)
        assert rel_l2(t.double().cpu().numpy(), O.filter_compact(oc, x)) < 1e-5


def test_batch_set_tuning_pins_variant(lib, cuda):
    """mgbf_batch_set_tuning pins one group's kernel for one generation and
    pass (read back by mgbf_batch_get_tuning; -1 returns to the default);
    the result still matches the oracle."""
    I = J = 64
    groups = [GroupDesc(nk=2 * 8, lm=8, nzcol=2, hx=4, hy=4, hz=2, p=2, mg_ampl01=canonical_z(2),
                        mg_ampl02=canonical(4))]
    w = [1.0, 0.5, 0.25]
    b = MGBFBatch(I, J, 3, w, groups)
    b.use_graphs(True)
    x = np.random.default_rng(14).standard_normal((J, I, 16))
    oc = O.OracleConfig(I=I, J=J, nk=16, hx=4, hy=4, hz=2, p=2, ampl01=canonical_z(2), ampl02=canonical(4), gm=3,
                        weights=w, proc=6, lm=8, nzcol=2, l_vertical_filter=True)
    ref = O.filter_compact(oc, x)
    for variant in (1, 2, 3, 0):
        b.set_tuning(0, 0, 0, variant, 16)
        b.set_tuning(0, 0, 1, variant, 32)
        assert b.tuning()[0][0] == [(variant, 16), (variant, 32)]
        t = torch.from_numpy(x).to(cuda, torch.float32)
        b.apply([t])
        torch.cuda.synchronize()
        b.status()
        assert rel_l2(t.double().cpu().numpy(), ref) < 1e-5
    b.set_tuning(0, 0, 0, -1)
    assert b.tuning()[0][0][0] == (-1, 0)
    with pytest.raises(_abi.MGBFError):
        b.set_tuning(0, 5, 0, 1)
    b.close()


def test_batch_one_vertical_pass(lib, cuda):
    """A batch with one vertical pass (M = Bz Bz^T in the last prolongation),
    replayed as a graph: against the oracle and against the two-pass chain
    (rounding only)."""
    I = J = 64
    groups = [GroupDesc(nk=3 * 8, lm=8, nzcol=3, hx=4, hy=4, hz=3, p=2, mg_ampl01=canonical_z(3),
                        mg_ampl02=canonical(4)),
              GroupDesc(nk=6, lm=1, nzcol=0, hx=6, hy=6, hz=2, p=2, mg_ampl01=canonical_z(2),
                        mg_ampl02=canonical(6))]
    w = [1.0, 0.5, 0.25]
    rng = np.random.default_rng(13)
    xs = [rng.standard_normal((J, I, g.nk)) for g in groups]
    outs = {}
    for passes in (2, 1):
        b = MGBFBatch(I, J, 3, w, groups)
        b.use_graphs(True)
        b.set_vertical_passes(passes)
        ts = [torch.from_numpy(x).to(cuda, torch.float32) for x in xs]
        for _ in range(3):  # direct, capture, replay: each call starts from x again
            for t, x in zip(ts, xs):
                t.copy_(torch.from_numpy(x))
            b.apply(ts)
        torch.cuda.synchronize()
        b.status()
        outs[passes] = [t.double().cpu().numpy() for t in ts]
        b.close()
    for g, x, y1, y2 in zip(groups, xs, outs[1], outs[2]):
        oc = O.OracleConfig(I=I, J=J, nk=g.nk, hx=g.hx, hy=g.hy, hz=g.hz, p=g.p, ampl01=g.mg_ampl01,
                            ampl02=g.mg_ampl02, gm=3, weights=w, proc=6, lm=g.lm, nzcol=g.nzcol,
                            l_vertical_filter=g.nzcol > 0)
        assert rel_l2(y1, O.filter_compact(oc, x)) < 1e-5
        assert rel_l2(y1, y2) < 1e-6


@pytest.mark.parametrize("mode", [1, 2])
def test_batch_graph_node_priorities(lib, cuda, mode):
    """Graph-node priorities change only the order in which the SMs take
    blocks of the concurrent group branches: results equal the graph
    without priorities bit for bit."""
    I = J = 64
    groups = [GroupDesc(nk=2 * 8, lm=8, nzcol=2, hx=4, hy=4, hz=2, p=2, mg_ampl01=canonical_z(2),
                        mg_ampl02=canonical(4)),
              GroupDesc(nk=6, lm=1, nzcol=0, hx=6, hy=6, hz=2, p=2, mg_ampl01=canonical_z(2),
                        mg_ampl02=canonical(6))]
    rng = np.random.default_rng(12)
    xs = [torch.from_numpy(rng.standard_normal((J, I, g.nk))).to(cuda, torch.float32) for g in groups]
    plain = MGBFBatch(I, J, 3, [1.0, 0.5, 0.25], groups)
    prio = MGBFBatch(I, J, 3, [1.0, 0.5, 0.25], groups)
    for b in (plain, prio):
        b.use_graphs(True)
    prio.set_priorities(mode)
    a = [x.clone() for x in xs]
    p = [x.clone() for x in xs]
    for _ in range(3):  # first call direct, second captures, third replays
        plain.apply(a)
        plain.apply(a, adjoint=True)
        prio.apply(p)
        prio.apply(p, adjoint=True)
    torch.cuda.synchronize()
    prio.status()
    for u, v in zip(a, p):
        assert torch.equal(u, v)
    with pytest.raises(_abi.MGBFError):
        prio.set_priorities(3)
    plain.close()
    prio.close()


def test_batch_graph_replay_matches_direct(lib, cuda):
    """Graph replay (captured launch sequence) gives bit-identical results."""
    I = J = 64
    groups = [GroupDesc(nk=2 * 8, lm=8, nzcol=2, hx=4, hy=4, hz=2, p=2, mg_ampl01=canonical_z(2),
                        mg_ampl02=canonical(4))]
    x = torch.from_numpy(np.random.default_rng(11).standard_normal((J, I, 16))).to(cuda, torch.float32)
    direct = MGBFBatch(I, J, 3, [1.0, 0.5, 0.25], groups)
    graphed = MGBFBatch(I, J, 3, [1.0, 0.5, 0.25], groups)
    graphed.use_graphs(True)
    a, g = x.clone(), x.clone()
    for _ in range(3):  # first call direct, second captures, third replays
        direct.apply([a])
        direct.apply([a], adjoint=True)
        graphed.apply([g])
        graphed.apply([g], adjoint=True)
    torch.cuda.synchronize()
    graphed.status()
    assert torch.equal(a, g)


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_autotuned_choice_keeps_parity(lib, cuda, dtype):
    c = small_config(nxPE=4, nyPE=4, im_filt=32, jm_filt=32, lm=8, km3=2, gm_max=3, hx=8, hy=8, hz=2,
                     mg_ampl02=canonical(8))
    op = MGBF(c)
    op.autotune(dtype)
    op.status()
    x = compact_input(op, 12)
    y = run_gpu(op, 1, x, dtype, cuda)
    assert rel_l2(y, O.filter_compact(oracle_cfg(c, 1), x)) < TOL[dtype]


@pytest.mark.parametrize("dtype", [torch.float32, torch.bfloat16])
@pytest.mark.parametrize("variant", [0, 1, 2, 3])
@pytest.mark.parametrize("rows", [0, 7])
@pytest.mark.parametrize("h", [5, 8, 10, 12, 16])
def test_parity_each_radial_variant(lib, cuda, dtype, variant, rows, h):
    """Every kernel variant the autotuner may choose, with the default row
    blocking and with short, uneven row blocks."""
    c = small_config(nxPE=4, nyPE=4, im_filt=48, jm_filt=48, lm=8, km3=1, gm_max=3, hx=h, hy=h, hz=2,
                     mg_ampl02=canonical(h), mg_ampl01=canonical_z(2))
    op = MGBF(c)
    op.set_tuning(variant, rows, dtype)
    x = compact_input(op, 100 + h)
    y = run_gpu(op, 1, x, dtype, cuda)
    op.status()
    assert rel_l2(y, O.filter_compact(oracle_cfg(c, 1), x)) < TOL[dtype]
    # the adjoint passes run the same variant: dot-product test
    w = compact_input(op, 200 + h)
    ltw = run_gpu(op, 1, w, dtype, cuda, adjoint=True)
    lhs, rhs = float(np.vdot(y, w)), float(np.vdot(x, ltw))
    assert abs(lhs - rhs) <= (1e-6 if dtype == torch.float32 else 2e-2) * np.linalg.norm(y) * np.linalg.norm(w)


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32, torch.bfloat16])
@pytest.mark.parametrize("nk_levels", [(7, 2), (5, 2), (9, 1)])
def test_level_counts_not_multiple_of_four(lib, cuda, dtype, nk_levels):
    """Leading dimensions 14, 10, 9 (2 or 1 mod 4) through every generation:
    the vectorised kernels take 4 levels per lane and must not be chosen."""
    lm, km3 = nk_levels
    c = small_config(lm=lm, km3=km3, gm_max=3, hz=2)
    op = MGBF(c)
    x = compact_input(op, 60 + lm)
    y = run_gpu(op, 1, x, dtype, cuda)
    assert rel_l2(y, O.filter_compact(oracle_cfg(c, 1), x)) < TOL[dtype]


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32, torch.bfloat16])
@pytest.mark.parametrize("lm,km3,km2", [(8, 2, 0), (12, 2, 0), (48, 2, 0), (40, 1, 0), (16, 1, 4)])
def test_fused_vertical_adjoint_and_restriction(lib, cuda, dtype, lm, km3, km2):
    """Generation 1's Bz^T and restriction run as one kernel when the z
    columns fit its 128- or 96-level blocks (lm 8, 12, 48, 16 with 2D levels
    after them) and apart otherwise (lm 40): both against the oracle."""
    c = small_config(lm=lm, km3=km3, km2=km2, n_ens=1, hz=3, mg_ampl01=canonical_z(3))
    op = MGBF(c)
    x = compact_input(op, 300 + lm)
    y = run_gpu(op, 1, x, dtype, cuda)
    assert rel_l2(y, O.filter_compact(oracle_cfg(c, 1), x)) < TOL[dtype]


@pytest.mark.parametrize("dtype", [torch.float32, torch.bfloat16])
@pytest.mark.parametrize("layout", ["compact", "halo"])
@pytest.mark.parametrize("hz,hx,grid", [(2, 4, (4, 4)), (4, 8, (4, 4)), (3, 4, (1, 1))])
def test_one_vertical_pass_and_direct_first_pass(lib, cuda, dtype, layout, hz, hx, grid):
    """Vertical reach <= 4 (FP32/BF16, radial moment kernel): the filter runs
    as M H x with M = Bz Bz^T applied once in the last prolongation;
    generation 1's first radial pass reads the caller's field itself, its
    edge tiles mirrored in shared memory (grid (1, 1): a 16 x 12 field whose
    tiles reach past both edges).  No vertical stage runs before the
    radial passes; forward against the oracle, adjoint by the dot-product
    test."""
    c = small_config(nxPE=grid[0], nyPE=grid[1], lm=8, km3=2, n_ens=1, hz=hz, mg_ampl01=canonical_z(hz), hx=hx, hy=hx,
                     mg_ampl02=canonical(hx),
                     layout=_abi.MGBF_LAYOUT_COMPACT if layout == "compact" else _abi.MGBF_LAYOUT_HALO)
    op = MGBF(c)
    op.set_vertical_passes(1)
    rng = np.random.default_rng(500 + hz + hx + grid[0])
    x, yv = rng.standard_normal(op.field_shape()), rng.standard_normal(op.field_shape())
    if layout == "compact":
        ref = O.filter_compact(oracle_cfg(c, 1), x)
    else:
        ref = x.copy()
        O.filtering_procedure(oracle_cfg(c, 1), ref)
    _abi.timers_enable(True)
    lx = run_gpu(op, 1, x, dtype, cuda)
    stages = _abi.timers_read()
    _abi.timers_enable(False)
    assert "upsend" in stages and "dnsend+vfilt" in stages
    assert "vfiltT" not in stages and "vfiltT+upsend" not in stages
    assert rel_l2(lx, ref) < TOL[dtype]
    if dtype == torch.float32:
        lty = run_gpu(op, 1, yv, dtype, cuda, adjoint=True)
        a, b = (lx * yv).sum(), (x * lty).sum()
        assert abs(a - b) / (np.linalg.norm(lx) * np.linalg.norm(yv)) < 1e-6
        # the reference's two passes on the same handle: the same operator
        op.set_vertical_passes(2)
        _abi.timers_enable(True)
        l2 = run_gpu(op, 1, x, dtype, cuda)
        stages = _abi.timers_read()
        _abi.timers_enable(False)
        assert "vfiltT+upsend" in stages
        assert rel_l2(l2, lx) < 1e-6
    with pytest.raises(_abi.MGBFError):
        op.set_vertical_passes(3)
    op.close()


@pytest.mark.parametrize("dtype", [torch.float32, torch.bfloat16])
@pytest.mark.parametrize("lm", [16, 48])
@pytest.mark.parametrize("hz", [5, 6, 7, 8])
def test_fused_z_kernels_vertical_reach_above_four(lib, cuda, dtype, lm, hz):
    """Vertical reach 5..8: generation 1's fused Bz^T + restriction and the
    fused last prolongation + Bz run their wide-window form (20-level
    window, 8 padding levels; reaches 5, 6 and 8 compiled, 7 runs as 8;
    128-level blocks for lm 16, 96 for lm 48).
    Stage timers show the fused stages ran; forward against the oracle and
    the adjoint by the dot-product test."""
    c = small_config(lm=lm, km3=2, n_ens=1, hz=hz, mg_ampl01=canonical_z(hz))
    op = MGBF(c)
    rng = np.random.default_rng(400 + lm + hz)
    x, yv = rng.standard_normal(op.field_shape()), rng.standard_normal(op.field_shape())
    _abi.timers_enable(True)
    lx = run_gpu(op, 1, x, dtype, cuda)
    stages = _abi.timers_read()
    _abi.timers_enable(False)
    assert "vfiltT+upsend" in stages and "dnsend+vfilt" in stages and "vfiltT" not in stages
    assert rel_l2(lx, O.filter_compact(oracle_cfg(c, 1), x)) < TOL[dtype]
    if dtype == torch.float32:
        lty = run_gpu(op, 1, yv, dtype, cuda, adjoint=True)
        a, b = (lx * yv).sum(), (x * lty).sum()
        assert abs(a - b) / (np.linalg.norm(lx) * np.linalg.norm(yv)) < 1e-6
