"""CPU tests of the FP64 oracle's invariants (the oracle is the checker of
the CUDA path; these tests pin it without a GPU)."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import canonical, canonical_z, oracle_cfg, small_config

rng = np.random.default_rng(1234)


def cfg(**kw):
    d = dict(I=32, J=24, nk=10, hx=4, hy=4, hz=2, p=2, ampl01=canonical_z(2), ampl02=canonical(4),
             gm=3, weights=[1.0, 0.5, 0.25], proc=1, lm=5, nzcol=2)
    d.update(kw)
    return O.OracleConfig(**d)


def test_setup_values_match_reference_formulas():
    c = cfg()
    v = O.setup_values(c)
    assert v["rmom2_1"] == pytest.approx(1 / np.sqrt(7))
    assert v["rmom2_2"] == pytest.approx(1 / np.sqrt(8))
    # canonical aspect gives e = 1/(h+1/2) and reach h
    assert v["exx2"] == pytest.approx(1 / 4.5)
    assert v["reach_h"] == 4 and v["reach_z"] == 2


@pytest.mark.parametrize("gen", [1, 2, 3])
def test_horizontal_filter_preserves_constants(gen):
    c = cfg()
    J, I, nk = c.gen_shape(gen)
    y = O.stage(c, O.STAGE_H_FWD, gen, np.ones((J, I, nk)))
    assert np.abs(y - 1).max() < 1e-13


def test_vertical_filter_preserves_constants():
    c = cfg()
    y = O.stage(c, O.STAGE_Z_FWD, 1, np.ones((c.J, c.I, c.nk)))
    assert np.abs(y[..., :10] - 1).max() < 1e-13


@pytest.mark.parametrize("which", [(O.STAGE_H_FWD, O.STAGE_H_ADJ), (O.STAGE_Z_FWD, O.STAGE_Z_ADJ)])
@pytest.mark.parametrize("gen", [1, 2])
def test_adjoint_pairs(which, gen):
    c = cfg()
    J, I, nk = c.gen_shape(gen)
    a, b = rng.standard_normal((J, I, nk)), rng.standard_normal((J, I, nk))
    fa = O.stage(c, which[0], gen, a)
    atb = O.stage(c, which[1], gen, b)
    assert abs((fa * b).sum() - (a * atb).sum()) < 1e-11 * np.abs(fa * b).sum()


@pytest.mark.parametrize("lquart", [False, True])
def test_restriction_is_transpose_of_prolongation(lquart):
    c = cfg(lquart=lquart)
    a = rng.standard_normal((c.J, c.I, c.nk))
    b = rng.standard_normal((c.J // 2, c.I // 2, c.nk))
    ra = O.stage(c, O.STAGE_RESTRICT, 1, a)
    pb = O.stage(c, O.STAGE_PROLONG, 1, b)
    assert abs((ra * b).sum() - (a * pb).sum()) < 1e-11 * np.abs(ra * b).sum()


def test_horizontal_scatter_equals_gather():
    """vrbeta2t+fold (scatter) == fill+vrbeta2 (gather): B is symmetric."""
    c = cfg()
    a = rng.standard_normal((c.J, c.I, c.nk))
    assert np.abs(O.stage(c, O.STAGE_H_FWD, 1, a) - O.stage(c, O.STAGE_H_ADJ, 1, a)).max() < 1e-14


def test_vertical_filter_is_not_symmetric():
    """Whole-sample mirror: Bz^T != Bz (the adjoint needs its own kernel)."""
    c = cfg()
    a = rng.standard_normal((c.J, c.I, c.nk))
    assert np.abs(O.stage(c, O.STAGE_Z_FWD, 1, a) - O.stage(c, O.STAGE_Z_ADJ, 1, a)).max() > 1e-3


@pytest.mark.parametrize("proc", [1, 6])
@pytest.mark.parametrize("lquart", [False, True])
def test_full_operator_self_adjoint(proc, lquart):
    c = cfg(proc=proc, lquart=lquart)
    a, b = rng.standard_normal((c.J, c.I, c.nk)), rng.standard_normal((c.J, c.I, c.nk))
    la, lb = O.filter_compact(c, a), O.filter_compact(c, b)
    assert abs((la * b).sum() - (a * lb).sum()) < 1e-12 * np.abs(la * b).sum()


def test_weight_gradients_are_exact_derivatives():
    c = cfg()
    x, gy = rng.standard_normal((c.J, c.I, c.nk)), rng.standard_normal((c.J, c.I, c.nk))
    ga = O.weight_grads(c, x, gy)
    base = (O.filter_compact(c, x) * gy).sum()
    for g in range(c.gm):
        w = list(c.weights)
        w[g] += 1.0
        d = (O.filter_compact(cfg(weights=w), x) * gy).sum() - base
        assert ga[g] == pytest.approx(d, rel=1e-10, abs=1e-10)


def test_impulse_response_symmetric():
    """Centred impulse on a square grid: response symmetric under i<->I+1-i."""
    c = cfg(I=32, J=32, nzcol=0, l_vertical_filter=False, nk=1, lm=1)
    x = np.zeros((32, 32, 1))
    x[15, 15, 0] = x[16, 16, 0] = x[15, 16, 0] = x[16, 15, 0] = 1.0
    y = O.filter_compact(c, x)
    assert np.abs(y - y[::-1, :, :]).max() < 1e-14
    assert np.abs(y - y[:, ::-1, :]).max() < 1e-14
    assert np.abs(y - y.transpose(1, 0, 2)).max() < 1e-14


def test_proc6_without_g1_filter_keeps_identity_term():
    """l_filt_g1 = false: generation 1 contributes x unweighted (weighting_ens)."""
    c = cfg(proc=6, l_filt_g1=False, gm=1, nzcol=0, l_vertical_filter=False)
    x = rng.standard_normal((c.J, c.I, c.nk))
    assert np.abs(O.filter_compact(c, x) - x).max() == 0.0


def test_reach_exceeding_halo_is_an_error():
    with pytest.raises(O.OracleError):
        O.filter_compact(cfg(hx=3), np.zeros((24, 32, 10)))


def test_helper_maps_namelist_config():
    c = small_config()
    oc = oracle_cfg(c, 1)
    assert (oc.I, oc.J, oc.nk, oc.gm, oc.nzcol) == (64, 48, 16, 3, 2)


@pytest.mark.parametrize("proc,l_filt_g1,lquart", [(1, True, False), (6, True, True), (6, False, False)])
def test_per_generation_contributions_sum_to_the_operator(proc, l_filt_g1, lquart):
    """oracle.contributions (the per-generation terms y_g reported against the
    GPU) adds up to filtering_procedure's output."""
    c = cfg(I=48, J=32, nk=12, lm=6, nzcol=2, proc=proc, l_filt_g1=l_filt_g1, lquart=lquart, gm=3)
    x = rng.standard_normal((c.J, c.I, c.nk))
    ys = O.contributions(c, x)
    y = O.filter_compact(c, x)
    assert len(ys) == c.gm
    assert np.linalg.norm(sum(ys) - y) <= 1e-14 * np.linalg.norm(y)
    # a generation's term equals the operator with only that weight kept
    # (without l_filt_g1 the unfiltered generation-1 term stays in every run)
    for g in range(c.gm):
        w = [c.weights[q] if q == g else 0.0 for q in range(c.gm)]
        yg = O.filter_compact(O.OracleConfig(**{**c.__dict__, "weights": w}), x)
        ref = ys[g] if (l_filt_g1 or proc == 1 or g == 0) else ys[g] + ys[0]
        assert np.linalg.norm(ref - yg) <= 1e-14 * np.linalg.norm(yg)


@pytest.mark.parametrize("proc", [1, 6])
def test_row_parallel_and_level_split_runs_are_bit_identical(proc):
    """With few levels per thread the radial pipeline splits rows instead of
    levels over the threads (and runs the scatters in target-row form); the
    results must not change by a single bit."""
    c = cfg(I=64, J=48, nk=32, lm=8, nzcol=4, proc=proc, gm=3, hx=5, hy=5, ampl02=canonical(5))
    x = rng.standard_normal((c.J, c.I, c.nk))
    gy = rng.standard_normal((c.J, c.I, c.nk))
    ys = [O.filter_compact(O.OracleConfig(**{**c.__dict__, "nthreads": n}), x) for n in (1, 2, 4, 8)]
    gs = [O.weight_grads(O.OracleConfig(**{**c.__dict__, "nthreads": n}), x, gy) for n in (1, 2, 4, 8)]
    for y, g in zip(ys[1:], gs[1:]):
        assert np.array_equal(y, ys[0])
        assert np.array_equal(g, gs[0])
