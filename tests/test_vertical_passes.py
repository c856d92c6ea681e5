"""The identity behind the one-vertical-pass form (mgbf_set_vertical_passes):
the vertical filter acts on every column alike and the horizontal chain
(restrictions, radial filters, weights, prolongations) on every level alike,
so Bz H Bz^T x = H (Bz Bz^T x) = Bz Bz^T (H x).  Checked on the FP64 oracle,
on the CPU."""
import dataclasses

import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import canonical, canonical_z, oracle_cfg, rel_l2, small_config


@pytest.mark.parametrize("proc,hz,lquart", [(1, 2, False), (1, 4, True), (6, 3, False)])
def test_vertical_filter_commutes_with_the_horizontal_chain(proc, hz, lquart):
    c = small_config(lm=8, km3=2, km2=1, n_ens=2, hz=hz, mg_ampl01=canonical_z(hz), hx=4, hy=4,
                     mg_ampl02=canonical(4), lquart=lquart)
    oc = oracle_cfg(c, proc)
    assert oc.l_vertical_filter and oc.nzcol > 0
    horiz = dataclasses.replace(oc, l_vertical_filter=False, nzcol=0)
    x = np.random.default_rng(600 + hz).standard_normal((oc.J, oc.I, oc.nk))

    def m(v):  # Bz Bz^T on every column (the levels past the z columns copied)
        return O.stage(oc, O.STAGE_Z_FWD, 1, O.stage(oc, O.STAGE_Z_ADJ, 1, v))

    y = O.filter_compact(oc, x)                    # Bz H Bz^T x, as the reference runs it
    assert rel_l2(O.filter_compact(horiz, m(x)), y) < 1e-13
    assert rel_l2(m(O.filter_compact(horiz, x)), y) < 1e-13
