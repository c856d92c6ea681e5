"""CPU tests of the oracle's fast 1D+1D filters, filtering_procedure(3) and (8)
(filtering_fast_bckg / filtering_fast_ens, mg_filtering.f90:825-997 and
1316-1506).  Their horizontal filter is vrbeta1 along x and along y with
paspx = paspy = mg_ampl02 taken without cholaspect (mg_intstate.f90:370-375),
so exx = mg_ampl02 / sqrt(2p+3) and the reach is floor(sqrt(2p+3)/mg_ampl02)."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import canonical_z, oracle_cfg, small_config

rng = np.random.default_rng(4321)
AMPL = 0.4  # line reach floor(sqrt(7)/0.4) = 6


def cfg(**kw):
    d = dict(I=32, J=24, nk=10, hx=6, hy=6, hz=2, p=2, ampl01=canonical_z(2), ampl02=AMPL,
             gm=3, weights=[1.0, 0.5, 0.25], proc=3, lm=5, nzcol=2)
    d.update(kw)
    return O.OracleConfig(**d)


def line_weights(ampl02=AMPL, p=2):
    exx = ampl02 / np.sqrt(2 * p + 3)
    r = int(np.floor(1.0 / exx - 1e-12))
    g = np.arange(-r, r + 1)
    w = (1.0 - (g * exx) ** 2) ** p
    return w / w.sum(), r


def numpy_fast_forward(x, ampl02=AMPL):
    """Independent restatement: half-sample mirror padding (numpy 'symmetric')
    and the normalised 1D beta along y, then along x."""
    w, r = line_weights(ampl02)
    J, I, _ = x.shape
    xp = np.pad(x, ((r, r), (0, 0), (0, 0)), mode="symmetric")
    y = sum(w[t] * xp[t:t + J] for t in range(2 * r + 1))
    yp = np.pad(y, ((0, 0), (r, r), (0, 0)), mode="symmetric")
    return sum(w[t] * yp[:, t:t + I] for t in range(2 * r + 1))


def test_line_setup_values():
    v = O.setup_values(cfg())
    w, r = line_weights()
    assert v["exx_line"] == pytest.approx(AMPL / np.sqrt(7))
    assert v["reach_line"] == r == 6
    exx = AMPL / np.sqrt(7)
    g = np.arange(-6, 7)
    assert v["ss_line"] == pytest.approx(1.0 / ((1 - (g * exx) ** 2) ** 2).sum())


@pytest.mark.parametrize("gen", [1, 2, 3])
def test_fast_forward_matches_independent_numpy(gen):
    c = cfg()
    J, I, nk = c.gen_shape(gen)
    x = rng.standard_normal((J, I, nk))
    assert np.abs(O.stage(c, O.STAGE_FAST_FWD, gen, x) - numpy_fast_forward(x)).max() < 1e-13


@pytest.mark.parametrize("gen", [1, 2, 3])
def test_fast_forward_preserves_constants(gen):
    c = cfg()
    J, I, nk = c.gen_shape(gen)
    y = O.stage(c, O.STAGE_FAST_FWD, gen, np.ones((J, I, nk)))
    assert np.abs(y - 1).max() < 1e-13


@pytest.mark.parametrize("gen", [1, 2])
def test_fast_adjoint_pair_and_symmetry(gen):
    c = cfg()
    J, I, nk = c.gen_shape(gen)
    a, b = rng.standard_normal((J, I, nk)), rng.standard_normal((J, I, nk))
    fa = O.stage(c, O.STAGE_FAST_FWD, gen, a)
    atb = O.stage(c, O.STAGE_FAST_ADJ, gen, b)
    assert abs((fa * b).sum() - (a * atb).sum()) < 1e-11 * np.abs(fa * b).sum()
    # symmetric stencil + half-sample mirror: the scatter form equals the gather form
    assert np.abs(O.stage(c, O.STAGE_FAST_ADJ, gen, a) - fa).max() < 1e-13


def test_fast_generation_filter_is_separable():
    """An impulse through one generation's forward filter gives the outer
    product of the 1D responses."""
    c = cfg(nk=1, lm=1, nzcol=0, l_vertical_filter=False)
    x = np.zeros((24, 32, 1))
    x[10, 13, 0] = 1.0
    y = O.stage(c, O.STAGE_FAST_FWD, 1, x)[..., 0]
    u, s, vt = np.linalg.svd(y)
    assert s[1] < 1e-14 * s[0]


@pytest.mark.parametrize("proc", [3, 8])
@pytest.mark.parametrize("lquart", [False, True])
def test_fast_operator_self_adjoint(proc, lquart):
    c = cfg(proc=proc, lquart=lquart)
    a, b = rng.standard_normal((c.J, c.I, c.nk)), rng.standard_normal((c.J, c.I, c.nk))
    la, lb = O.filter_compact(c, a), O.filter_compact(c, b)
    assert abs((la * b).sum() - (a * lb).sum()) < 1e-12 * np.abs(la * b).sum()


@pytest.mark.parametrize("proc", [3, 8])
def test_fast_weight_gradients_are_exact_derivatives(proc):
    c = cfg(proc=proc)
    x, gy = rng.standard_normal((c.J, c.I, c.nk)), rng.standard_normal((c.J, c.I, c.nk))
    ga = O.weight_grads(c, x, gy)
    base = (O.filter_compact(c, x) * gy).sum()
    for g in range(c.gm):
        w = list(c.weights)
        w[g] += 1.0
        d = (O.filter_compact(cfg(proc=proc, weights=w), x) * gy).sum() - base
        assert ga[g] == pytest.approx(d, rel=1e-10, abs=1e-10)


def test_fast_single_generation_no_z_is_weighted_square():
    """G = 1, no vertical filter: L = a_1 F F with F the separable filter."""
    c = cfg(gm=1, weights=[0.7], nzcol=0, l_vertical_filter=False)
    x = rng.standard_normal((c.J, c.I, c.nk))
    ref = 0.7 * numpy_fast_forward(numpy_fast_forward(x))
    assert np.abs(O.filter_compact(c, x) - ref).max() < 1e-13


def test_proc8_without_g1_filter_keeps_identity_term():
    c = cfg(proc=8, l_filt_g1=False, gm=1, nzcol=0, l_vertical_filter=False)
    x = rng.standard_normal((c.J, c.I, c.nk))
    assert np.abs(O.filter_compact(c, x) - x).max() == 0.0


def test_fast_differs_from_radial():
    x = rng.standard_normal((24, 32, 10))
    y3 = O.filter_compact(cfg(proc=3), x)
    y1 = O.filter_compact(cfg(proc=1), x)
    assert np.abs(y3 - y1).max() > 1e-3


def test_line_reach_exceeding_halo_is_an_error():
    with pytest.raises(O.OracleError):
        O.filter_compact(cfg(hx=5), np.zeros((24, 32, 10)))
    with pytest.raises(O.OracleError):
        O.filter_compact(cfg(hy=5), np.zeros((24, 32, 10)))


def test_helper_maps_proc3_like_proc1():
    c = small_config()
    assert oracle_cfg(c, 3).nzcol == oracle_cfg(c, 1).nzcol
