"""The host-streaming pipeline returns, for every step, the same result as
filtering the step's fields directly (GPU)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("nsets", [2, 3])
def test_host_stream_matches_direct(lib, cuda, nsets):
    from standalone_mgbf_loc_gb300 import GroupDesc, MGBFBatch
    from standalone_mgbf_loc_gb300.pipeline import HostStream
    from tests.helpers import canonical, canonical_z
    I = J = 64
    groups = [GroupDesc(nk=4 * 8, lm=8, nzcol=4, hx=4, hy=4, hz=2, p=2, mg_ampl01=canonical_z(2),
                        mg_ampl02=canonical(4)),
              GroupDesc(nk=4, lm=1, nzcol=0, hx=6, hy=6, hz=2, p=2, mg_ampl01=canonical_z(2),
                        mg_ampl02=canonical(6))]
    b = MGBFBatch(I, J, 3, [1.0, 0.5, 0.25], groups)
    hs = HostStream(b, torch.float32, cuda, nsets=nsets)
    steps = 7
    ins = [[torch.randn((J, I, g.nk), generator=torch.Generator().manual_seed(10 * s + q)).pin_memory()
            for q, g in enumerate(groups)] for s in range(steps)]
    outs = [[torch.empty_like(x).pin_memory() for x in step] for step in ins]
    for s in range(steps):
        hs.submit(ins[s], outs[s])
    hs.finish()
    for s in range(steps):
        ref = [x.to(cuda) for x in ins[s]]
        b.apply(ref)
        b.apply(ref, adjoint=True)
        torch.cuda.synchronize()
        for r, o in zip(ref, outs[s]):
            assert torch.equal(r.cpu(), o)
