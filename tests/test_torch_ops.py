"""torch.ops.mgbf.*: the PyTorch operators over the C-ABI call the same entry
points as the MGBF / MGBFBatch classes."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from standalone_mgbf_loc_gb300 import MGBF, GroupDesc, MGBFBatch, torch_ops  # noqa: E402
from tests.helpers import canonical, canonical_z, small_config  # noqa: E402


def test_operators_are_registered():
    for name in ("filtering_procedure_", "filtering_procedure_adjoint_", "batch_apply_"):
        assert hasattr(torch.ops.mgbf, name)


def test_unknown_id_is_refused_before_any_library_call():
    x = torch.zeros(4)
    with pytest.raises(ValueError):
        torch.ops.mgbf.filtering_procedure_(x, 987654, 1)
    with pytest.raises(TypeError):
        torch_ops.register(object())


@pytest.mark.gpu
def test_filtering_procedure_op_equals_method(lib, cuda):
    op = MGBF(small_config())
    hid = torch_ops.register(op)
    x = torch.from_numpy(np.random.default_rng(31).standard_normal(op.field_shape())).to(cuda, torch.float32)
    a, b = x.clone(), x.clone()
    op.filtering_procedure(1, a)
    torch.ops.mgbf.filtering_procedure_(b, hid, 1)
    op.filtering_procedure_adjoint(1, a)
    torch.ops.mgbf.filtering_procedure_adjoint_(b, hid, 1)
    torch.cuda.synchronize()
    op.status()
    assert torch.equal(a, b)
    torch_ops.unregister(hid)
    op.close()


@pytest.mark.gpu
def test_batch_apply_op_equals_method(lib, cuda):
    groups = [GroupDesc(nk=2 * 8, lm=8, nzcol=2, hx=4, hy=4, hz=2, p=2, mg_ampl01=canonical_z(2),
                        mg_ampl02=canonical(4)),
              GroupDesc(nk=4, lm=1, nzcol=0, hx=6, hy=6, hz=2, p=2, mg_ampl01=canonical_z(2),
                        mg_ampl02=canonical(6))]
    b = MGBFBatch(64, 64, 3, [1.0, 0.5, 0.25], groups)
    bid = torch_ops.register(b)
    rng = np.random.default_rng(32)
    xs = [torch.from_numpy(rng.standard_normal((64, 64, g.nk))).to(cuda, torch.float32) for g in groups]
    u = [x.clone() for x in xs]
    v = [x.clone() for x in xs]
    b.apply(u)
    torch.ops.mgbf.batch_apply_(v, bid, False)
    b.apply(u, adjoint=True)
    torch.ops.mgbf.batch_apply_(v, bid, True)
    torch.cuda.synchronize()
    b.status()
    for p, q in zip(u, v):
        assert torch.equal(p, q)
    torch_ops.unregister(bid)
    b.close()
