"""The global-grid oracle equals a literal emulation of the reference's MPI
tiling (oracle/virtual_ranks.py): rank tiles with halo exchange in the
reference's order, quadrant upsend/downsend between generations.  This is
what justifies collapsing the decomposition into one array on one GPU."""
import numpy as np
import pytest

from oracle import oracle as O
from oracle import virtual_ranks as VR
from tests.helpers import canonical, canonical_z

CASES = [
    # nxPE, nyPE, tile, hx, proc, lquart, l_filt_g1
    (2, 2, 8, 3, 1, False, True),
    (4, 4, 6, 3, 1, False, True),
    (4, 2, 8, 4, 6, False, False),
    (4, 4, 8, 3, 6, True, True),
    (8, 8, 4, 2, 1, False, True),
    # line filters (procs 2 and 7): half-span 2 along x and y, identity diagonal
    (2, 2, 8, 3, 2, False, True),
    (4, 4, 6, 3, 2, True, True),
    (4, 2, 8, 4, 7, False, False),
    (4, 4, 8, 3, 7, True, True),
]


@pytest.mark.parametrize("nxPE,nyPE,tile,hx,proc,lquart,filt1", CASES)
def test_virtual_ranks_match_global_oracle(nxPE, nyPE, tile, hx, proc, lquart, filt1):
    gm = VR.def_maxgen(nxPE, nyPE)
    # generations are capped by the rank layout exactly as in the reference
    gm = min(gm, 4)
    I, J = nxPE * tile, nyPE * tile
    lm, nzcol = 4, 2
    nk = lm * nzcol
    w = [1.0, 0.5, 0.25, 0.125][:gm]
    ampl02 = canonical(hx)
    ampl01 = canonical_z(1)
    x = np.random.default_rng(nxPE * 100 + tile).standard_normal((J, I, nk))
    y_vr = VR.filtering(x, nxPE=nxPE, nyPE=nyPE, im=tile, jm=tile, hx=hx, p=2, ampl01=ampl01, ampl02=ampl02,
                        weights=w, gm=gm, proc=proc, lm=lm, nzcol=nzcol, lquart=lquart, l_filt_g1=filt1)
    oc = O.OracleConfig(I=I, J=J, nk=nk, hx=hx, hy=hx, hz=1, p=2, ampl01=ampl01, ampl02=ampl02, gm=gm,
                        weights=w, proc=proc, lm=lm, nzcol=nzcol, lquart=lquart, l_filt_g1=filt1)
    y_or = O.filter_compact(oc, x)
    assert np.abs(y_vr - y_or).max() <= 1e-13 * np.abs(y_or).max()


def test_stencil_setup_matches_oracle():
    st = VR.radial_stencil(2, canonical(6))
    assert max(abs(g) for g, _, _ in st) == 6
    assert abs(sum(w for _, _, w in st) - 1.0) < 1e-14
    oc = O.OracleConfig(I=64, J=64, nk=1, hx=6, hy=6, hz=1, p=2, ampl01=canonical_z(1), ampl02=canonical(6),
                        gm=1, weights=[1.0], lm=1, nzcol=0, l_vertical_filter=False)
    v = O.setup_values(oc)
    s_vr = [w for g, gy, w in st if g == 0 and gy == 0][0]
    assert s_vr == pytest.approx(v["ss2"], rel=1e-14)


@pytest.mark.parametrize("nxPE,nyPE,tile,hx,lquart", [(2, 2, 8, 4, False), (4, 2, 8, 4, True), (4, 4, 8, 3, False)])
def test_virtual_ranks_match_global_oracle_lin3(nxPE, nyPE, tile, hx, lquart):
    """Proc 5: the 3D halo routines' generation-1 index forms act at the
    physical east and north edges only; rank boundaries exchange exactly."""
    gm = min(VR.def_maxgen(nxPE, nyPE), 3)
    I, J = nxPE * tile, nyPE * tile
    lm, nzcol, km2, hz = 4, 2, 1, 3
    nk = lm * nzcol + km2
    w = [1.0, 0.5, 0.25][:gm]
    ampl02 = canonical(hx)
    x = np.random.default_rng(nxPE * 10 + tile).standard_normal((J, I, nk))
    y_vr = VR.filtering(x, nxPE=nxPE, nyPE=nyPE, im=tile, jm=tile, hx=hx, p=2, ampl01=1.0, ampl02=ampl02,
                        weights=w, gm=gm, proc=5, lm=lm, nzcol=nzcol, lquart=lquart, ampl03=0.6, hz=hz)
    oc = O.OracleConfig(I=I, J=J, nk=nk, hx=hx, hy=hx, hz=hz, p=2, ampl01=1.0, ampl02=ampl02, gm=gm,
                        weights=w, proc=5, lm=lm, nzcol=nzcol, lquart=lquart, ampl03=0.6,
                        l_vertical_filter=False)
    y_or = O.filter_compact(oc, x)
    assert np.abs(y_vr - y_or).max() <= 1e-12 * np.abs(y_or).max()
