"""The allocation-free entry point, mgbf_radial_filter_noalloc, called through
the C-ABI.  It exists for callers that cannot allocate device memory (work
captured into a CUDA graph, applications that own all device memory through
their own pool, fixed memory budgets); its intermediate fields live in a
static device array instead of cudaMalloc'd scratch.  It must give the same
result as the allocating entry point, filtering_procedure with one
generation and no vertical filter, on consecutive calls that reuse the
shared array.  This file is collected last on purpose."""
import ctypes

import numpy as np
import pytest

from standalone_mgbf_loc_gb300 import MGBF, MGBFConfig, _abi
from tests.helpers import canonical, rel_l2

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _noalloc(lib, x, y, nk, im, jm, h, weight, stream):
    return lib.mgbf_radial_filter_noalloc(ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y.data_ptr()), nk, im, jm,
                                          2, canonical(h), h, h, weight, ctypes.c_void_p(stream))


def _allocating(nk, im, jm, h, weight):
    """filtering_procedure(1) with one generation and no vertical filter."""
    cfg = MGBFConfig(nxPE=1, nyPE=1, im_filt=im, jm_filt=jm, lm=1, km2=nk, km3=0, gm_max=1, hx=h, hy=h, hz=3,
                     mg_ampl01=1.0, mg_ampl02=canonical(h), mg_ampl03=0.3, mg_weig1=weight,
                     l_vertical_filter=False, layout=_abi.MGBF_LAYOUT_COMPACT)
    return MGBF(cfg)


# (nk, im, jm, h); the last case fills the static array exactly:
# 32 * (992 + 2 * (8 + 8)) * 256 == MGBF_NOALLOC_MAX_ELEMS
CASES = [(16, 96, 64, 6), (6, 64, 80, 8), (8, 64, 48, 16), (32, 992, 256, 8)]


@pytest.mark.parametrize("nk,im,jm,h", CASES)
@pytest.mark.parametrize("in_place", [False, True])
def test_noalloc_matches_allocating_entry_point(lib, cuda, nk, im, jm, h, in_place):
    weight = 0.7
    op = _allocating(nk, im, jm, h, weight)
    stream = torch.cuda.current_stream(cuda).cuda_stream
    gen = torch.Generator(device=cuda)
    for seed in (0, 1):  # two calls in a row share the static array
        gen.manual_seed(seed)
        x = torch.randn((jm, im, nk), generator=gen, device=cuda, dtype=torch.float32)
        ref = x.clone()
        op.filtering_procedure(1, ref)
        y = x if in_place else torch.full_like(x, float("nan"))
        rc = _noalloc(lib, x, y, nk, im, jm, h, weight, stream)
        assert rc == _abi.MGBF_OK, lib.mgbf_last_error().decode()
        torch.cuda.synchronize()
        assert rel_l2(y.double().cpu().numpy(), ref.double().cpu().numpy()) < 1e-6
    op.close()


def test_noalloc_rejects_one_element_over_the_limit(lib, cuda):
    nk, im, jm, h = 32, 993, 256, 8  # 32 * (993 + 32) * 256 = MGBF_NOALLOC_MAX_ELEMS + 8192
    x = torch.zeros((jm, im, nk), device=cuda, dtype=torch.float32)
    rc = _noalloc(lib, x, x, nk, im, jm, h, 1.0, torch.cuda.current_stream(cuda).cuda_stream)
    assert rc == _abi.MGBF_ERR_ARG
    assert "MGBF_NOALLOC_MAX_ELEMS" in lib.mgbf_last_error().decode()


def test_noalloc_rejects_grid_narrower_than_reach(lib, cuda):
    nk, im, jm, h = 4, 6, 32, 8
    x = torch.zeros((jm, im, nk), device=cuda, dtype=torch.float32)
    rc = _noalloc(lib, x, x, nk, im, jm, h, 1.0, torch.cuda.current_stream(cuda).cuda_stream)
    assert rc == _abi.MGBF_ERR_DIVISIBILITY


def test_noalloc_rejects_oversize_field(lib, cuda):
    nk, im, jm, h = 64, 512, 512, 8  # 64 * (512 + 32) * 512 > MGBF_NOALLOC_MAX_ELEMS
    x = torch.zeros((jm, im, nk), device=cuda, dtype=torch.float32)
    rc = _noalloc(lib, x, x, nk, im, jm, h, 1.0, torch.cuda.current_stream(cuda).cuda_stream)
    assert rc == _abi.MGBF_ERR_ARG
    assert "MGBF_NOALLOC_MAX_ELEMS" in lib.mgbf_last_error().decode()
