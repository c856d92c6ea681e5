"""CPU tests of the oracle's filtering_procedure(2), filtering_lin2_bckg
(mg_filtering.f90:683-822): per generation, the three "dibeta" line filters
of the triad decomposition (jp_pbfil3.f90:573-624) applied as dibetat +
bocoT_2d for colors 3, 2, 1, weighting, then boco_2d + dibeta for colors
1, 2, 3 (jp_pbfil3.f90:1801-1837, 2345-2382).  The setup follows
init_mg_line (mg_intstate.f90:436-480), which sees the Cholesky factor of the
inverse aspect, (c, c, 0) with c = 1/sqrt(mg_ampl02)."""
import numpy as np
import pytest

from oracle import oracle as O

rng = np.random.default_rng(202)
P = 2


def cfg(**kw):
    d = dict(I=24, J=20, nk=5, hx=4, hy=4, hz=2, p=P, ampl01=1.0, ampl02=0.5, gm=1, weights=[0.7], proc=2,
             lm=5, nzcol=0, l_vertical_filter=False)
    d.update(kw)
    return O.OracleConfig(**d)


def moments(p, nh=O.DIB_NH):
    """Normalisation and spread^2 of the beta filters of half-span 1..nh."""
    bnorm, bsprd = np.zeros(nh + 1), np.zeros(nh + 1)
    for h in range(1, nh + 1):
        i = np.arange(-h, h + 1)
        w = (1.0 - (i / h) ** 2) ** p
        bnorm[h], bsprd[h] = 1.0 / w.sum(), (i * i * w).sum() / w.sum()
    return bnorm, bsprd


def numpy_colors(c):
    """The three colors for the isotropic aspect: generators (1,0), (0,1),
    (-1,-1) with spread^2 (el, el, 0), el = 1/sqrt(ampl02), each through the
    half-span transform and the two-beta weights."""
    bnorm, bsprd = moments(c.p)
    el = np.sqrt(1.0 / c.ampl02)
    out = []
    for d, s2 in (((1, 0), el), ((0, 1), el), ((-1, -1), 0.0)):
        h2 = next(h for h in range(2, O.DIB_NH + 1) if bsprd[h] >= s2)
        hs = h2 - (bsprd[h2] - s2) / (bsprd[h2] - bsprd[h2 - 1])
        h = int(hs)
        hp = h + 1
        fil = np.zeros(h + 1)
        i = np.arange(h + 1)
        fil += (hs - h) * bnorm[hp] * (1.0 - (i / hp) ** 2) ** c.p
        fil[:h] += (hp - hs) * bnorm[h] * (1.0 - (i[:h] / h) ** 2) ** c.p
        out.append((d, h, hs, fil))
    return out


def test_triad_reconstructs_positive_definite_aspects():
    for asp in ([1.4, 1.4, 0.0], [2.0, 1.0, 0.9], [1.0, 3.0, -1.2], [5.0, 0.6, 1.5], [1.0, 1.0, 0.99],
                [0.3, 7.0, 1.1]):
        lt, w = O.triad(asp)
        A = sum(w[q] * np.outer(lt[q], lt[q]) for q in range(3))
        assert np.abs(A - [[asp[0], asp[2]], [asp[2], asp[1]]]).max() < 1e-13
        assert w.min() >= -1e-14
        # the three generators pairwise span the integer lattice
        for a, b in ((0, 1), (1, 2), (2, 0)):
            assert abs(lt[a][0] * lt[b][1] - lt[a][1] * lt[b][0]) == 1
    with pytest.raises(O.OracleError):  # not positive definite: no triad
        O.triad([1.0, 2.0, -1.5])


@pytest.mark.parametrize("ampl02", [0.5, 0.3, 1.0, 3.0])
@pytest.mark.parametrize("p", [1, 2, 3])
def test_setup_matches_numpy(ampl02, p):
    c = cfg(ampl02=ampl02, p=p, hx=6, hy=6)
    got = O.dibeta_values(c)
    for g, (d, h, hs, fil) in zip(got, numpy_colors(c)):
        assert g["d"] == d and g["h"] == h
        assert abs(g["hs"] - hs) < 1e-13
        assert np.abs(g["fil"] - fil).max() < 1e-15


@pytest.mark.parametrize("ampl02", [0.5, 0.3, 1.0])
def test_weights_normalised_with_the_prescribed_spread(ampl02):
    """Each dibeta sums to one and its second moment is the spread^2 the
    triad assigned: el along x and y, 0 on the diagonal."""
    c = cfg(ampl02=ampl02, hx=6, hy=6)
    el = np.sqrt(1.0 / ampl02)
    for g, s2 in zip(O.dibeta_values(c), (el, el, 0.0)):
        f = g["fil"]
        t = np.arange(len(f))
        assert abs(f[0] + 2 * f[1:].sum() - 1.0) < 1e-14
        assert abs(2 * (t * t * f).sum() - s2) < 1e-13


def fill_h(U, hx, hy):
    U = U.copy()
    J, I = U.shape[0] - 2 * hy, U.shape[1] - 2 * hx
    for t in range(1, hy + 1):
        U[hy - t, hx:hx + I] = U[hy + t - 1, hx:hx + I]
        U[hy + J + t - 1, hx:hx + I] = U[hy + J - t, hx:hx + I]
    for t in range(1, hx + 1):
        U[:, hx - t] = U[:, hx + t - 1]
        U[:, hx + I + t - 1] = U[:, hx + I - t]
    return U


def fold_h(U, hx, hy):
    U = U.copy()
    J, I = U.shape[0] - 2 * hy, U.shape[1] - 2 * hx
    for t in range(1, hx + 1):
        U[:, hx + t - 1] += U[:, hx - t]
        U[:, hx + I - t] += U[:, hx + I + t - 1]
    for t in range(1, hy + 1):
        U[hy + t - 1, hx:hx + I] += U[hy - t, hx:hx + I]
        U[hy + J - t, hx:hx + I] += U[hy + J + t - 1, hx:hx + I]
    return U


def dibeta(U, d, fil, hx, hy, adj):
    J, I = U.shape[0] - 2 * hy, U.shape[1] - 2 * hx
    B = np.zeros_like(U)
    dx, dy = d
    inner = (slice(hy, hy + J), slice(hx, hx + I))

    def shifted(t):
        return (slice(hy + t * dy, hy + t * dy + J), slice(hx + t * dx, hx + t * dx + I))

    if not adj:
        B[inner] = fil[0] * U[inner]
        for t in range(1, len(fil)):
            B[inner] += fil[t] * (U[shifted(t)] + U[shifted(-t)])
    else:
        B[inner] += fil[0] * U[inner]
        for t in range(1, len(fil)):
            B[shifted(t)] += fil[t] * U[inner]
            B[shifted(-t)] += fil[t] * U[inner]
    return B


def numpy_lin2_g1(c, V):
    colors = numpy_colors(c)
    U = V.copy()
    for d, _, _, fil in reversed(colors):
        U = fold_h(dibeta(U, d, fil, c.hx, c.hy, True), c.hx, c.hy)
    U[c.hy:c.hy + c.J, c.hx:c.hx + c.I] *= c.weights[0]
    for d, _, _, fil in colors:
        U = dibeta(fill_h(U, c.hx, c.hy), d, fil, c.hx, c.hy, False)
    return U


@pytest.mark.parametrize("ampl02", [0.5, 1.0])
@pytest.mark.parametrize("p", [1, 2, 3])
def test_one_generation_matches_numpy(ampl02, p):
    c = cfg(ampl02=ampl02, p=p)
    V = rng.standard_normal((c.J + 2 * c.hy, c.I + 2 * c.hx, c.nk))
    ref = numpy_lin2_g1(c, V)
    got = V.copy()
    O.filtering_procedure(c, got)
    assert np.abs(got - ref).max() < 1e-13


def test_stages_are_an_adjoint_pair():
    c = cfg(gm=2, weights=[1.0, 0.5])
    x, y = rng.standard_normal((c.J, c.I, c.nk)), rng.standard_normal((c.J, c.I, c.nk))
    fx = O.stage(c, O.STAGE_LIN2_FWD, 1, x)
    aty = O.stage(c, O.STAGE_LIN2_ADJ, 1, y)
    assert abs((fx * y).sum() - (x * aty).sum()) < 1e-12 * np.abs(fx * y).sum()


@pytest.mark.parametrize("lquart", [False, True])
def test_operator_is_symmetric(lquart):
    """The adjoint side is the exact transpose of the forward side, so the
    whole operator is self-adjoint (the diagonal color alone is not
    symmetric near the edges: the transpose is needed)."""
    c = cfg(I=32, J=32, nk=6, gm=3, weights=[1.0, 0.5, 0.25], lquart=lquart, lm=3, nzcol=2,
            l_vertical_filter=True, ampl01=0.8, hz=2)
    a, b = rng.standard_normal((32, 32, 6)), rng.standard_normal((32, 32, 6))
    la, lb = O.filter_compact(c, a), O.filter_compact(c, b)
    assert abs((la * b).sum() - (a * lb).sum()) < 1e-12 * np.abs(la * b).sum()


def test_constant_field_is_kept_by_one_generation():
    c = cfg(weights=[1.0])
    x = np.full((c.J, c.I, c.nk), 2.5)
    assert np.abs(O.filter_compact(c, x) - 2.5).max() < 1e-13


def test_weight_grads_match_finite_differences():
    c = cfg(I=16, J=16, gm=2, weights=[1.0, 0.5])
    x, gy = rng.standard_normal((16, 16, c.nk)), rng.standard_normal((16, 16, c.nk))
    ga = O.weight_grads(c, x, gy)
    for g in range(2):
        w = list(c.weights)
        w[g] += 1.0
        c2 = cfg(I=16, J=16, gm=2, weights=w)
        # L is linear in the weights: L(w + e_g) - L(w) is the derivative
        d = ((O.filter_compact(c2, x) - O.filter_compact(c, x)) * gy).sum()
        assert abs(d - ga[g]) < 1e-10 * max(1.0, abs(d))


def test_errors():
    with pytest.raises(O.OracleError):  # half-span 3 along x needs hx >= 3
        O.filter_compact(cfg(hx=2), np.zeros((20, 24, 5)))
    with pytest.raises(O.OracleError):  # spread^2 beyond the moment table
        O.filter_compact(cfg(ampl02=0.02, hx=8, hy=8), np.zeros((20, 24, 5)))


# ------------------------------------------- proc 7: filtering_lin2_ens

@pytest.mark.parametrize("lquart", [False, True])
def test_proc7_is_proc2_between_two_adjoint_vertical_filters(lquart):
    """filtering_lin2_ens (mg_filtering.f90:1150-1313) runs proc 2's
    horizontal part (generation 1 filtered: l_filt_g1) and ends with the
    adjoint vertical filter sup_vrbeta1T_ens (:1304), so L7 = Bz^T M Bz^T."""
    kw = dict(I=32, J=32, nk=6, gm=3, weights=[1.0, 0.5, 0.25], lquart=lquart, lm=3, nzcol=2, ampl01=0.8, hz=2)
    c7 = cfg(proc=7, l_vertical_filter=True, l_filt_g1=True, **kw)
    c2 = cfg(proc=2, l_vertical_filter=False, **kw)
    cz = cfg(proc=7, l_vertical_filter=True, **kw)
    x = rng.standard_normal((32, 32, 6))
    ref = O.stage(cz, O.STAGE_Z_ADJ, 1, O.filter_compact(c2, O.stage(cz, O.STAGE_Z_ADJ, 1, x)))
    assert np.abs(O.filter_compact(c7, x) - ref).max() < 1e-13
    # not self-adjoint
    a, b = rng.standard_normal((32, 32, 6)), rng.standard_normal((32, 32, 6))
    la, lb = O.filter_compact(c7, a), O.filter_compact(c7, b)
    assert abs((la * b).sum() - (a * lb).sum()) > 1e-6 * np.abs(la * b).sum()


def test_proc7_generation1_unfiltered_without_filt_g1():
    """With l_filt_g1 false, generation 1 is neither filtered nor weighted
    (weighting_ens, mg_generations.f90:1012-1052): one generation and no
    vertical filter leave the field unchanged."""
    c = cfg(proc=7, l_filt_g1=False, weights=[0.3])
    x = rng.standard_normal((c.J, c.I, c.nk))
    assert np.abs(O.filter_compact(c, x) - x).max() == 0.0


def test_proc7_weight_grads_refused():
    c = cfg(proc=7)
    with pytest.raises(O.OracleError):
        O.weight_grads(c, np.zeros((c.J, c.I, c.nk)), np.zeros((c.J, c.I, c.nk)))


@pytest.mark.parametrize("proc", [2, 7])
def test_identity_filters_without_mgbf_line(proc):
    """mgbf_line off: zero generators, every color copies, so one
    generation without a vertical filter is the weight alone."""
    c = cfg(proc=proc, mgbf_line=False, weights=[0.7], ampl02=0.02)  # no table limit applies
    x = rng.standard_normal((c.J, c.I, c.nk))
    assert np.abs(O.filter_compact(c, x) - 0.7 * x).max() < 1e-15
    assert all(d["h"] == 0 and d["fil"].tolist() == [1.0] for d in O.dibeta_values(c))
