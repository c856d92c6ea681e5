"""Golden fixtures (tests/golden/golden.npz, made by make_golden.py from the
FP64 oracle): the oracle reproduces them (CPU), and libmgbf matches them on
the GPU through the C-ABI."""
import os

import numpy as np
import pytest

from oracle import oracle as O
from tests.golden.cases import CASES, case_config, case_input, case_oracle_cfg
from tests.helpers import rel_l2

GOLDEN = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "golden.npz"))


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_reproduces_golden(name):
    y = O.filter_compact(case_oracle_cfg(name), case_input(name))
    ref = GOLDEN[name]
    assert np.abs(y - ref).max() <= 1e-14 * np.abs(ref).max()


def test_golden_impulse_properties():
    """Impulse response: peak at the impulse, positive centre, symmetric in x<->y."""
    y = GOLDEN["proc1_impulse"]
    lev = y[:, :, 1]
    assert np.unravel_index(np.abs(lev).argmax(), lev.shape) == (15, 15)
    assert np.abs(lev - lev.T).max() < 1e-15


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(CASES))
def test_gpu_matches_golden(lib, cuda, name):
    torch = pytest.importorskip("torch")
    from standalone_mgbf_loc_gb300 import MGBF
    op = MGBF(case_config(name))
    x = case_input(name)
    proc = CASES[name][1]
    for dtype, tol in ((torch.float64, 1e-12), (torch.float32, 1e-5)):
        t = torch.from_numpy(x).to(cuda, dtype).contiguous()
        op.filtering_procedure(proc, t)
        torch.cuda.synchronize()
        op.status()
        assert rel_l2(t.double().cpu().numpy(), GOLDEN[name]) < tol
