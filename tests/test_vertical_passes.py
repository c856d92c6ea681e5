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


def test_option_setters_validate_arguments():
    """The pass-form, priority and tuning setters refuse bad values with
    MGBF_ERR_ARG and take good ones; none needs a GPU."""
    from standalone_mgbf_loc_gb300 import MGBF, GroupDesc, MGBFBatch, _abi
    op = MGBF(small_config())
    op.set_vertical_passes(1)
    op.set_vertical_passes(2)
    for bad in (0, 3):
        with pytest.raises(_abi.MGBFError) as e:
            op.set_vertical_passes(bad)
        assert e.value.code == _abi.MGBF_ERR_ARG
    op.close()
    b = MGBFBatch(64, 64, 3, [1.0, 0.5, 0.25],
                  [GroupDesc(nk=16, lm=8, nzcol=2, hx=4, hy=4, hz=2, p=2, mg_ampl01=canonical_z(2),
                             mg_ampl02=canonical(4))])
    b.set_vertical_passes(1)
    b.set_priorities(2)
    b.set_tuning(0, 0, 0, 1, 16)
    b.set_tuning(0, 0, 0, -1)
    for call in (lambda: b.set_vertical_passes(3), lambda: b.set_priorities(5), lambda: b.set_tuning(0, 9, 0, 1),
                 lambda: b.set_tuning(1, 0, 0, 1), lambda: b.set_tuning(0, 0, 2, 1), lambda: b.set_tuning(0, 0, 0, 7)):
        with pytest.raises(_abi.MGBFError) as e:
            call()
        assert e.value.code == _abi.MGBF_ERR_ARG
    b.close()
