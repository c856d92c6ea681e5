"""The bounded mbarrier wait of the TMA-fed radial kernels, made to run out.

With a poll limit of 0 every row wait of k_hmom_tma / k_hmom_tma1 gives up
at once on a healthy GPU: each block records the failure in the handle's
status word, waits (with the default bound) for its own copies in flight and
returns.  Nothing faults or hangs; the call returns, mgbf_status reports
MGBF_ERR_TIMEOUT once, and after the limit is restored the next call is
correct against the oracle.
"""
import numpy as np
import pytest

from oracle import oracle as O
from standalone_mgbf_loc_gb300 import MGBF, MGBFBatch, GroupDesc, _abi
from standalone_mgbf_loc_gb300._abi import MGBFError
from tests.helpers import canonical, canonical_z, oracle_cfg, rel_l2, small_config

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("variant", [0, 1, 3])  # the TMA variants
def test_wait_runs_out_and_recovers(lib, cuda, variant):
    c = small_config()
    op = MGBF(c)
    assert op.dims.hbeta_kernel == 1
    op.set_tuning(variant, dtype=torch.float32)
    x = np.random.default_rng(5).standard_normal(op.field_shape())
    t = torch.from_numpy(x).to(device=cuda, dtype=torch.float32)
    op.status()  # clean before
    op.set_wait_limit(0)
    op.filtering_procedure(1, t)  # the radial kernels give up on their first row
    torch.cuda.synchronize()
    with pytest.raises(MGBFError) as e:
        op.status()
    assert e.value.code == _abi.MGBF_ERR_TIMEOUT
    op.status()  # reading the status cleared it
    op.set_wait_limit(-1)
    t = torch.from_numpy(x).to(device=cuda, dtype=torch.float32)
    op.filtering_procedure(1, t)
    torch.cuda.synchronize()
    op.status()
    ref = O.filter_compact(oracle_cfg(c, 1), x)
    assert rel_l2(t.double().cpu().numpy(), ref) < 1e-5
    op.close()


def test_batch_wait_runs_out_and_recovers(lib, cuda):
    h = 6
    gd = [GroupDesc(nk=2 * 16, lm=16, nzcol=2, hx=h, hy=h, hz=2, p=2, mg_ampl01=canonical_z(2),
                    mg_ampl02=canonical(h))]
    w = [1.0, 0.5, 0.25]
    b = MGBFBatch(64, 48, 3, w, gd)
    b.use_graphs(True)
    x = np.random.default_rng(6).standard_normal((48, 64, 32))
    f = [torch.from_numpy(x).to(device=cuda, dtype=torch.float32)]
    b.apply(f)  # first call of the dtype runs directly and sets up buffers
    torch.cuda.synchronize()
    b.status()
    b.set_wait_limit(0)
    f = [torch.from_numpy(x).to(device=cuda, dtype=torch.float32)]
    b.apply(f)
    torch.cuda.synchronize()
    with pytest.raises(MGBFError) as e:
        b.status()
    assert e.value.code == _abi.MGBF_ERR_TIMEOUT
    b.set_wait_limit(-1)
    f = [torch.from_numpy(x).to(device=cuda, dtype=torch.float32)]
    b.apply(f)
    torch.cuda.synchronize()
    b.status()
    cfg = O.OracleConfig(I=64, J=48, nk=16, hx=h, hy=h, hz=2, p=2, ampl01=canonical_z(2), ampl02=canonical(h),
                         gm=3, weights=w, proc=6, lm=16, nzcol=1, l_vertical_filter=True)
    got = f[0].double().cpu().numpy()
    for m in range(2):
        ref = O.filter_compact(cfg, np.ascontiguousarray(x[:, :, 16 * m:16 * (m + 1)]))
        assert rel_l2(got[:, :, 16 * m:16 * (m + 1)], ref) < 1e-5
    b.close()
