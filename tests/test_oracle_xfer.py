"""CPU tests of the oracle's analysis <-> filter transfers (anal_to_filt_all2 /
filt_to_anal_all2, mg_transfer.f90:154-203, 339-464; offset interpolations
mg_interpolate.f90:89-298, 634-960; l_vertical_*_spec2, :963-1044)."""
import numpy as np
import pytest

from oracle import oracle as O

rng = np.random.default_rng(77)
# (nm0, mm0, nxpe, nype, im, jm): per-rank ratios 1.125 x 1.5 (the shipped
# namelist's 72/64 and 48/32), 1 x 2, and 1.5 x 1.125
GEOMS = [(36, 24, 4, 2, 8, 8), (16, 32, 2, 2, 8, 8), (24, 18, 2, 2, 8, 8)]


def cfg(geom=GEOMS[0], order=3, nk=3, **kw):
    nm0, mm0, nx, ny, im, jm = geom
    return O.XferConfig(nm0=nm0, mm0=mm0, nxpe=nx, nype=ny, im=im, jm=jm, hx=4, hy=4, nkf=nk, order=order, **kw)


def numpy_axis(na, nf, order):
    """The per-rank tables written independently: first tap and weights of
    the blend of two quadratic Lagrange interpolants (order 3), quadratic (2)
    or linear (1) interpolation at x = n - 1/2 from nodes (i - 1/2) na/nf."""
    df = na / nf
    refs, ws = [], []
    for n in range(1, na + 1):
        x = 0.5 + (n - 1)
        i = next(i for i in range(-5, nf + 6) if x < df * 0.5 + df * (i - 1))
        first = i - 2 if order == 3 else i - 1
        nodes = [df * 0.5 + df * (first + t - 1) for t in range(order + 1)]

        def lag(pts, t):
            return np.prod([(x - pts[u]) / (pts[t] - pts[u]) for u in range(len(pts)) if u != t])

        if order == 3:
            left, right = nodes[:3], nodes[1:]
            wl = (nodes[2] - x) / (nodes[2] - nodes[1])
            wr = 1.0 - wl
            w = [wl * lag(left, 0), wl * lag(left, 1) + wr * lag(right, 0),
                 wl * lag(left, 2) + wr * lag(right, 1), wr * lag(right, 2)]
        else:
            w = [lag(nodes, t) for t in range(order + 1)]
        refs.append(first)
        ws.append(w)
    return np.array(refs), np.array(ws)


def numpy_direct(c, vall):
    """Mirror-fill the interior (half-sample, numpy 'symmetric') and gather."""
    ib = c.order
    inner = vall[c.hy:c.hy + c.J, c.hx:c.hx + c.I]
    pad = np.pad(inner, ((ib, ib), (ib, ib), (0, 0)), mode="symmetric")
    nm, mm = c.nm0 // c.nxpe, c.mm0 // c.nype
    rx, wx = numpy_axis(nm, c.im, c.order)
    ry, wy = numpy_axis(mm, c.jm, c.order)
    out = np.zeros(c.worka_shape())
    for M in range(c.mm0):
        rj, m = divmod(M, mm)
        j0 = rj * c.jm + ry[m] - 1 + ib  # 0-based row in the padded array
        for N in range(c.nm0):
            ri, n = divmod(N, nm)
            i0 = ri * c.im + rx[n] - 1 + ib
            blk = pad[j0:j0 + c.order + 1, i0:i0 + c.order + 1]
            out[M, N] = np.einsum("s,t,stk->k", wy[m], wx[n], blk)
    return out


@pytest.mark.parametrize("geom", GEOMS)
@pytest.mark.parametrize("order", [1, 2, 3])
def test_direct_matches_independent_numpy(geom, order):
    c = cfg(geom, order)
    v = rng.standard_normal(c.vall_shape())
    assert np.abs(O.filt_to_anal(c, v.copy()) - numpy_direct(c, v)).max() < 1e-13


@pytest.mark.parametrize("order", [1, 2, 3])
def test_direct_reproduces_polynomials_inside(order):
    """Away from the edges the interpolation is exact for polynomials of its
    degree (quadratic for the lsqr blend)."""
    c = cfg(GEOMS[0], order, nk=1)
    deg = 1 if order == 1 else 2
    dfx, dfy = (c.nm0 // c.nxpe) / c.im, (c.mm0 // c.nype) / c.jm
    xf = (np.arange(1, c.I + 1) - 0.5) * dfx
    yf = (np.arange(1, c.J + 1) - 0.5) * dfy
    f = lambda x, y: 0.3 + 0.7 * x - 0.2 * y + (0.05 * x * x - 0.03 * x * y if deg == 2 else 0.0)
    v = np.zeros(c.vall_shape())
    v[c.hy:c.hy + c.J, c.hx:c.hx + c.I, 0] = f(xf[None, :], yf[:, None])
    w = O.filt_to_anal(c, v)[..., 0]
    xa, ya = np.arange(1, c.nm0 + 1) - 0.5, np.arange(1, c.mm0 + 1) - 0.5
    exact = f(xa[None, :], ya[:, None])
    sx = slice(3, c.nm0 - 3)
    sy = slice(4, c.mm0 - 4)
    assert np.abs(w[sy, sx] - exact[sy, sx]).max() < 1e-11


@pytest.mark.parametrize("order", [1, 2, 3])
def test_constants_and_halo_fill(order):
    c = cfg(GEOMS[1], order)
    v = np.zeros(c.vall_shape())
    v[c.hy:c.hy + c.J, c.hx:c.hx + c.I] = 2.5
    w = O.filt_to_anal(c, v)
    assert np.abs(w - 2.5).max() < 1e-13
    # boco_2d filled the interpolation halo (width = order) in place
    ib = order
    assert np.all(v[c.hy - ib:c.hy + c.J + ib, c.hx - ib:c.hx + c.I + ib] == 2.5)


@pytest.mark.parametrize("geom", GEOMS)
@pytest.mark.parametrize("order", [1, 2, 3])
def test_adjoint_pair(geom, order):
    """<D fill v, w> = <v, (fold D^T w)> on the filter interior."""
    c = cfg(geom, order)
    v = np.zeros(c.vall_shape())
    v[c.hy:c.hy + c.J, c.hx:c.hx + c.I] = rng.standard_normal((c.J, c.I, c.nkf))
    w = rng.standard_normal(c.worka_shape())
    dv = O.filt_to_anal(c, v.copy())
    atw = O.anal_to_filt(c, w)
    inner = (slice(c.hy, c.hy + c.J), slice(c.hx, c.hx + c.I))
    lhs, rhs = (dv * w).sum(), (v[inner] * atw[inner]).sum()
    assert abs(lhs - rhs) < 1e-12 * np.abs(dv * w).sum()


def test_anal_to_filt_halo():
    """The scatter's halo part stays in VALL's interpolation halo (bocoT_2d
    does not clear it); VALL beyond that halo is zero."""
    c = cfg(GEOMS[0], 3)
    a = O.anal_to_filt(c, rng.standard_normal(c.worka_shape()))
    ib, hx, hy = 3, c.hx, c.hy
    assert np.abs(a[hy - ib:hy, hx:hx + c.I]).max() > 0
    assert np.abs(a[:hy - ib]).max() == 0 and np.abs(a[:, :hx - ib]).max() == 0


def test_vertical_spec2():
    """lm_a = 2 lm - 1: odd analysis levels copy the filter levels, even ones
    average their neighbours, applied to every block of lm_a levels; and the
    adjoint pair holds with the vertical step included."""
    lm, lm_a, en = 4, 7, 2
    c1 = cfg(GEOMS[1], 3, nk=lm * en)
    c2 = cfg(GEOMS[1], 3, nk=lm * en, nka=lm_a * en, lm=lm, lm_a=lm_a, en=en)
    v = np.zeros(c1.vall_shape())
    v[c1.hy:c1.hy + c1.J, c1.hx:c1.hx + c1.I] = rng.standard_normal((c1.J, c1.I, c1.nkf))
    h = O.filt_to_anal(c1, v.copy())
    w = O.filt_to_anal(c2, v.copy())
    for e in range(en):
        f = h[..., e * lm:(e + 1) * lm]
        a = w[..., e * lm_a:(e + 1) * lm_a]
        assert np.array_equal(a[..., 0::2], f)
        assert np.array_equal(a[..., 1::2], 0.5 * (f[..., :-1] + f[..., 1:]))
    ww = rng.standard_normal(c2.worka_shape())
    atw = O.anal_to_filt(c2, ww)
    inner = (slice(c2.hy, c2.hy + c2.J), slice(c2.hx, c2.hx + c2.I))
    assert abs((w * ww).sum() - (v[inner] * atw[inner]).sum()) < 1e-12 * np.abs(w * ww).sum()


def test_invalid_geometry_is_an_error():
    """VALL's halo narrower than the interpolation halo, and lm_a neither lm
    nor 2 lm - 1, are errors."""
    narrow = O.XferConfig(nm0=36, mm0=24, nxpe=4, nype=2, im=8, jm=8, hx=2, hy=4, nkf=1, order=3)
    with pytest.raises(O.OracleError):
        O.filt_to_anal(narrow, np.zeros(narrow.vall_shape()))
    bad_v = cfg(GEOMS[1], 3, nk=4, nka=5, lm=4, lm_a=5, en=1)
    with pytest.raises(O.OracleError):
        O.anal_to_filt(bad_v, np.zeros(bad_v.worka_shape()))
