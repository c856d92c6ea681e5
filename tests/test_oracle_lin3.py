"""CPU tests of the oracle's filtering_procedure(5), filtering_lin3
(mg_filtering.f90:260-557): the 2D variables through the triad line
filters of procedure 2, the 3D variables through the seven colors of the
hexad (jp_pbfil3.f90:798-904) with the 3D halo routines boco_3d / bocoT_3d
(mg_bocos.f90:1425-2908: the generation-1 forms have the reference's
east-edge and north-fold index forms), no separate vertical filter."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.test_oracle_lin2 import dibeta, fill_h, fold_h, moments, numpy_colors

rng = np.random.default_rng(505)


def cfg(**kw):
    d = dict(I=16, J=12, nk=9, hx=4, hy=4, hz=3, p=2, ampl01=1.0, ampl02=0.5, ampl03=0.6, gm=1, weights=[0.7],
             proc=5, lm=4, nzcol=2, l_vertical_filter=False)
    d.update(kw)
    return O.OracleConfig(**d)


def spread_weights(p, s2):
    """Half-span transform and two-beta weights of a spread^2."""
    bnorm, bsprd = moments(p)
    h2 = next(h for h in range(2, O.DIB_NH + 1) if bsprd[h] >= s2)
    hs = h2 - (bsprd[h2] - s2) / (bsprd[h2] - bsprd[h2 - 1])
    h = int(hs)
    hp = h + 1
    i = np.arange(h + 1)
    fil = (hs - h) * bnorm[hp] * (1.0 - (i / hp) ** 2) ** p
    fil[:h] += (hp - hs) * bnorm[h] * (1.0 - (i[:h] / h) ** 2) ** p
    return fil


def hexad_colors(c):
    """Colors 1..7 for the isotropic aspect (c3, c3, c3, 0, 0, 0),
    c3 = 1/sqrt(ampl03): x, y, z with spread^2 c3, three diagonals with
    spread 0 (identity), color 7 null (copy)."""
    c3 = np.sqrt(1.0 / c.ampl03)
    out = {1: ((1, 0, 0), spread_weights(c.p, c3)), 2: ((0, 1, 0), spread_weights(c.p, c3)),
           3: ((0, 0, 1), spread_weights(c.p, c3))}
    for col, d in ((4, (1, -1, 0)), (5, (-1, 0, 1)), (6, (0, 1, -1))):
        out[col] = (d, spread_weights(c.p, 0.0))
    out[7] = None
    return out


class W3:
    """W(L, j, i, v) with halos hz, hy, hx (numpy order: z, y, x, variable)."""

    def __init__(self, c, I, J):
        self.c, self.I, self.J = c, I, J
        self.a = np.zeros((c.lm + 2 * c.hz, J + 2 * c.hy, I + 2 * c.hx, c.nzcol))

    def L(self, L):  # 1-based level -> index
        return L - 1 + self.c.hz

    def from_stack(self, U):
        c = self.c
        for L in range(1, c.lm + 1):
            self.a[self.L(L)] = U[:, :, [v * c.lm + L - 1 for v in range(c.nzcol)]]

    def to_stack(self, U):
        c = self.c
        for L in range(1, c.lm + 1):
            U[:, :, [v * c.lm + L - 1 for v in range(c.nzcol)]] = self.a[self.L(L)]

    def zmirror(self):
        for L in range(1, self.c.hz + 1):
            self.a[self.L(1 - L)] = self.a[self.L(1 + L)]
            self.a[self.L(self.c.lm + L)] = self.a[self.L(self.c.lm - L)]

    def boco(self, gh):
        c, I, J, a = self.c, self.I, self.J, self.a
        hx, hy = c.hx, c.hy
        z = slice(c.hz, c.hz + c.lm)
        xi = slice(hx, hx + I)
        for j in range(1, hy + 1):  # north, then south, interior columns
            a[z, hy + J + j - 1, xi] = a[z, hy + J - j, xi]
        for j in range(1, hy + 1):
            a[z, j - 1, xi] = a[z, 2 * hy - j, xi]
        for i in range(1, hx + 1):  # west, then east, every row
            a[z, :, i - 1] = a[z, :, 2 * hx - i]
        for i in range(1, hx + 1):
            src = I + 1 - i if gh else I - i
            a[z, :, hx + I + i - 1] = a[z, :, hx + src - 1]
        if gh:
            self.zmirror()

    def bocoT(self, gh):
        c, I, J, a = self.c, self.I, self.J, self.a
        hx, hy, o = c.hx, c.hy, 1 if gh else 0
        z = slice(c.hz, c.hz + c.lm)
        xi = slice(hx, hx + I)
        for i in range(1, hx + 1):
            a[z, :, hx + i - 1] += a[z, :, hx - i]
        for i in range(1, hx + 1):
            a[z, :, hx + I - hx + i - 1] += a[z, :, hx + I + o + hx - i - 1]
        for j in range(1, hy + 1):
            a[z, hy + j - 1, xi] += a[z, hy - j, xi]
        for j in range(1, hy + 1):
            a[z, hy + J - hy + j - 1, xi] += a[z, hy + J + o + hy - j - 1, xi]
        for L in range(1, c.hz + 1):
            a[self.L(1 + L)] += a[self.L(1 - L)]
            a[self.L(c.lm - L)] += a[self.L(c.lm + L)]

    def dib(self, colors, col, adj):
        c, I, J = self.c, self.I, self.J
        B = np.zeros_like(self.a)
        inner = (slice(c.hz, c.hz + c.lm), slice(c.hy, c.hy + J), slice(c.hx, c.hx + I))
        if colors[col] is None:
            B[inner] = self.a[inner]
        else:
            (dx, dy, dz), fil = colors[col]

            def sh(t):
                return (slice(c.hz + t * dz, c.hz + t * dz + c.lm), slice(c.hy + t * dy, c.hy + t * dy + J),
                        slice(c.hx + t * dx, c.hx + t * dx + I))

            if not adj:
                B[inner] = fil[0] * self.a[inner]
                for t in range(1, len(fil)):
                    B[inner] += fil[t] * (self.a[sh(t)] + self.a[sh(-t)])
            else:
                B[inner] += fil[0] * self.a[inner]
                for t in range(1, len(fil)):
                    B[sh(t)] += fil[t] * self.a[inner]
                    B[sh(-t)] += fil[t] * self.a[inner]
        self.a = B


def numpy_lin3_generation(c, V, I, J, a, gh):
    """One generation on V (J+2hy, I+2hx, nk) with halo."""
    n3 = c.nzcol * c.lm
    cols2 = numpy_colors(c)
    cols3 = hexad_colors(c)
    U = V.copy()
    U2 = U[..., n3:]
    for d, _, _, fil in reversed(cols2):
        U2 = fold_h(dibeta(U2, d, fil, c.hx, c.hy, True), c.hx, c.hy)
    U[..., n3:] = U2
    w = W3(c, I, J)
    w.from_stack(U)
    for col in range(7, 0, -1):
        w.zmirror()
        w.dib(cols3, col, True)
        w.bocoT(gh)
    w.to_stack(U)
    U[c.hy:c.hy + J, c.hx:c.hx + I] *= a
    U2 = U[..., n3:]
    for d, _, _, fil in cols2:
        U2 = dibeta(fill_h(U2, c.hx, c.hy), d, fil, c.hx, c.hy, False)
    U[..., n3:] = U2
    w.from_stack(U)
    w.zmirror()
    for col in range(1, 8):
        w.boco(gh)
        w.dib(cols3, col, False)
    w.to_stack(U)
    return U


def test_hexad_reconstructs_positive_definite_aspects():
    lh, w = O.hexad([1.2, 1.2, 1.2, 0, 0, 0])
    assert lh.tolist() == [[1, 0, 0], [0, 1, 0], [0, 0, 1], [1, -1, 0], [-1, 0, 1], [0, 1, -1], [0, 0, 0]]
    r = np.random.default_rng(7)
    for _ in range(20):
        B = r.standard_normal((3, 3))
        A = B @ B.T + 0.2 * np.eye(3)
        lh, w = O.hexad([A[0, 0], A[1, 1], A[2, 2], A[1, 2], A[2, 0], A[0, 1]])
        R = sum(w[q] * np.outer(lh[q], lh[q]) for q in range(7))
        assert np.abs(R - A).max() < 1e-12 * np.abs(A).max()
        assert w.min() >= -1e-12
        assert (np.abs(lh).sum(1) == 0).sum() == 1  # one null color


@pytest.mark.parametrize("gen", [1, 2])
@pytest.mark.parametrize("p,ampl03,hz", [(2, 0.6, 3), (1, 1.5, 2), (3, 0.35, 4)])
def test_one_generation_matches_numpy(gen, p, ampl03, hz):
    """Generation 1 uses boco_3d_g1 / bocoT_3d_g1, generation 2 the _gh forms;
    z-line half-spans 2 to 4."""
    c = cfg(gm=2, weights=[0.7, 0.4], p=p, ampl03=ampl03, hz=hz, lm=max(4, hz + 1), nk=2 * max(4, hz + 1) + 1)
    J, I = c.J >> (gen - 1), c.I >> (gen - 1)
    V = np.zeros((J + 2 * c.hy, I + 2 * c.hx, c.nk))
    V[c.hy:c.hy + J, c.hx:c.hx + I] = rng.standard_normal((J, I, c.nk))
    ref = numpy_lin3_generation(c, V, I, J, c.weights[gen - 1], gen > 1)
    got = O.stage(c, O.STAGE_LIN3_GEN, gen, V[c.hy:c.hy + J, c.hx:c.hx + I].copy())
    assert np.abs(got - ref[c.hy:c.hy + J, c.hx:c.hx + I]).max() < 1e-13


def test_whole_procedure_is_one_generation_when_gm_is_one():
    c = cfg()
    x = rng.standard_normal((c.J, c.I, c.nk))
    assert np.abs(O.filter_compact(c, x) - O.stage(c, O.STAGE_LIN3_GEN, 1, x)).max() < 1e-14


def test_generation1_east_edge_quirk():
    """At generation 1 the reference's 3D fold adds the east edge column to
    itself and its fill mirrors about it: the operator is not symmetric
    there, while the _gh forms at coarser generations are transposes."""
    c = cfg(nk=8, nzcol=2, weights=[1.0])
    a, b = rng.standard_normal((c.J, c.I, c.nk)), rng.standard_normal((c.J, c.I, c.nk))
    la, lb = O.filter_compact(c, a), O.filter_compact(c, b)
    assert abs((la * b).sum() - (a * lb).sum()) > 1e-6 * np.abs(la * b).sum()


def test_lin3_setup_errors():
    with pytest.raises(O.OracleError):  # z line half-span beyond hz
        O.filter_compact(cfg(hz=1, lm=4), np.zeros((12, 16, 9)))
    with pytest.raises(O.OracleError):  # weight gradients: not self-adjoint
        O.weight_grads(cfg(), np.zeros((12, 16, 9)), np.zeros((12, 16, 9)))


def test_identity_filters_without_mgbf_line():
    """mgbf_line off: every color copies, so only the halo routines act.
    bocoT_3d_g1's east and north folds add the edge column and row to
    themselves once per adjoint color: seven colors scale the 3D variables'
    east column and north row by 2^7 and their north-east corner by 4^7,
    as the reference does; the 2D variables and the rest are the weight."""
    c = cfg(mgbf_line=False, weights=[0.7])
    x = rng.standard_normal((c.J, c.I, c.nk))
    n3 = c.nzcol * c.lm
    m = np.ones((c.J, c.I, c.nk))
    m[:, -1, :n3] *= 2.0 ** 7
    m[-1, :, :n3] *= 2.0 ** 7
    assert np.abs(O.filter_compact(c, x) - 0.7 * m * x).max() < 1e-12 * np.abs(0.7 * m * x).max()
