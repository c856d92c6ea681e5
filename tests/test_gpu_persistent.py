"""Persistent radial sides: each variable group's radial pass over all its
generations as one launch of k_hmom_persist (blocks take tiles from a device
counter), checked against the FP64 oracle, against the per-generation
launches, under graph replay, and through its bounded waits."""
import numpy as np
import pytest

from oracle import oracle as O
from standalone_mgbf_loc_gb300 import GroupDesc, MGBFBatch, _abi
from standalone_mgbf_loc_gb300._abi import MGBFError
from tests.helpers import canonical, canonical_z, rel_l2

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

I = J = 64
GM = 4
W = [1.0, 0.5, 0.25, 0.125]
GROUPS = [
    GroupDesc(nk=3 * 8, lm=8, nzcol=3, hx=4, hy=4, hz=2, p=2, mg_ampl01=canonical_z(2), mg_ampl02=canonical(4)),
    GroupDesc(nk=2 * 6, lm=6, nzcol=2, hx=8, hy=8, hz=2, p=2, mg_ampl01=canonical_z(2), mg_ampl02=canonical(8)),
    GroupDesc(nk=6, lm=1, nzcol=0, hx=5, hy=5, hz=2, p=2, mg_ampl01=canonical_z(2), mg_ampl02=canonical(5)),
]
TOL = {torch.float32: 1e-5, torch.bfloat16: 2e-2}


def _inputs(seed):
    rng = np.random.default_rng(seed)
    return [rng.standard_normal((J, I, g.nk)) for g in GROUPS]


def _oracle(g, x, adjoint=False, l_filt_g1=True):
    oc = O.OracleConfig(I=I, J=J, nk=g.nk, hx=g.hx, hy=g.hy, hz=g.hz, p=g.p, ampl01=g.mg_ampl01,
                        ampl02=g.mg_ampl02, gm=GM, weights=W, proc=6, lm=g.lm, nzcol=g.nzcol,
                        l_vertical_filter=g.nzcol > 0, l_filt_g1=l_filt_g1)
    return O.filter_compact(oc, x)


@pytest.mark.parametrize("dtype", [torch.float32, torch.bfloat16])
@pytest.mark.parametrize("tuned", [False, True])
def test_persistent_sides_match_oracle(lib, cuda, dtype, tuned):
    b = MGBFBatch(I, J, GM, W, GROUPS)
    if tuned:
        b.autotune(dtype)  # rows per block of every generation from the autotuner
    b.use_persistent(True)
    xs = _inputs(20)
    ts = [torch.from_numpy(x).to(cuda, dtype).contiguous() for x in xs]
    b.apply(ts)
    torch.cuda.synchronize()
    b.status()
    for g, x, t in zip(GROUPS, xs, ts):
        assert rel_l2(t.double().cpu().numpy(), _oracle(g, x)) < TOL[dtype]
    b.close()


def test_persistent_matches_per_generation_launches(lib, cuda):
    """The same operator either way: per-generation launches (default kernel
    variants) and persistent sides agree to FP32 rounding, forward and
    adjoint."""
    xs = _inputs(21)
    outs = []
    for persistent in (0, 2):
        b = MGBFBatch(I, J, GM, W, GROUPS)
        b.use_persistent(persistent)
        ts = [torch.from_numpy(x).to(cuda, torch.float32).contiguous() for x in xs]
        b.apply(ts)
        b.apply(ts, adjoint=True)
        torch.cuda.synchronize()
        b.status()
        outs.append([t.double().cpu().numpy() for t in ts])
        b.close()
    for a, p in zip(*outs):
        assert rel_l2(p, a) < 1e-6


def test_persistent_without_generation_one(lib, cuda):
    """l_filt_g1 = .false.: generation 1 is neither filtered nor weighted, the
    persistent sides cover generations 2..gm only."""
    b = MGBFBatch(I, J, GM, W, GROUPS, l_filt_g1=False)
    b.use_persistent(True)
    xs = _inputs(22)
    ts = [torch.from_numpy(x).to(cuda, torch.float32).contiguous() for x in xs]
    b.apply(ts)
    torch.cuda.synchronize()
    b.status()
    for g, x, t in zip(GROUPS, xs, ts):
        assert rel_l2(t.double().cpu().numpy(), _oracle(g, x, l_filt_g1=False)) < 1e-5
    b.close()


def test_persistent_graph_replay(lib, cuda):
    """Captured into the batch's CUDA graph (the tile counters are zeroed by
    a memset node before each persistent launch): replays equal direct calls."""
    xs = _inputs(23)
    direct = MGBFBatch(I, J, GM, W, GROUPS)
    graphed = MGBFBatch(I, J, GM, W, GROUPS)
    for b in (direct, graphed):
        b.use_persistent(True)
    graphed.use_graphs(True)
    a = [torch.from_numpy(x).to(cuda, torch.float32).contiguous() for x in xs]
    g = [t.clone() for t in a]
    for _ in range(3):  # first call direct, second captures, third replays
        direct.apply(a)
        graphed.apply(g)
    torch.cuda.synchronize()
    graphed.status()
    for u, v in zip(a, g):
        assert rel_l2(v.double().cpu().numpy(), u.double().cpu().numpy()) < 1e-6
    direct.close()
    graphed.close()


def test_persistent_wait_runs_out_and_recovers(lib, cuda):
    """Poll limit 0: every tile's first row wait gives up, the block records
    it, drains its copies and stops taking tiles; the call returns and the
    status reports MGBF_ERR_TIMEOUT.  With the limit restored the next call
    is correct."""
    b = MGBFBatch(I, J, GM, W, GROUPS)
    b.use_persistent(True)
    xs = _inputs(24)
    ts = [torch.from_numpy(x).to(cuda, torch.float32).contiguous() for x in xs]
    b.status()
    b.set_wait_limit(0)
    b.apply(ts)
    torch.cuda.synchronize()
    with pytest.raises(MGBFError) as e:
        b.status()
    assert e.value.code == _abi.MGBF_ERR_TIMEOUT
    b.set_wait_limit(-1)
    ts = [torch.from_numpy(x).to(cuda, torch.float32).contiguous() for x in xs]
    b.apply(ts)
    torch.cuda.synchronize()
    b.status()
    for g, x, t in zip(GROUPS, xs, ts):
        assert rel_l2(t.double().cpu().numpy(), _oracle(g, x)) < 1e-5
    b.close()
