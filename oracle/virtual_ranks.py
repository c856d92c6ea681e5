"""Literal emulation of the reference's MPI-decomposed filtering -- TEST
INFRASTRUCTURE ONLY.

A second, independent restatement of filtering_procedure(1|2|5|6|7) that keeps the
reference's structure: every rank (nx, my) owns an im x jm tile with halos;
halos are filled and folded by emulated point-to-point exchange in the
reference's order; restriction output of 2x2 finer tiles is assembled into the
quadrants of one coarser tile (upsend_all) and scattered back (downsend_all).
It exists to show that the global-grid oracle (mgbf_oracle.c), which
collapses the tiling into one array, computes the same operator.  Only tests
import it.

Followed routines (reference paths):
  boco_2d_g1/gh      mg_bocos.f90:89-784    (N/S rows first, then E/W columns
                                             including the halo rows; mirror at
                                             physical edges)
  bocoT_2d_g1/gh     mg_bocos.f90:787-1422  (E/W first over all rows, then N/S)
  upsend_all         mg_bocos.f90:2911-3492 (quadrants SW, SE, NW, NE)
  downsend_all       mg_bocos.f90:3495-4041
  adjoint/direct1    mg_generations.f90:1117-1250, adjoint2/direct2 1253-1374
  upsending/downsending[_ens] mg_generations.f90:158-267, 382-494
  vrbeta2/vrbeta2t   jp_pbfil.f90:888-928, 1011-1050
  sup_vrbeta1[T]_*   mg_filtering.f90:2042-2262
  filtering_rad2_bckg / _ens  mg_filtering.f90:560-680, 1000-1147
  filtering_lin2_bckg / _ens  mg_filtering.f90:683-822, 1150-1313
  vdibeta2/vdibeta2t jp_pbfil3.f90:1801-1837, 2345-2382 (as gather/scatter
                     stencils over each color's generator)
Arrays are numpy (J_ext, I_ext, nk) per tile: Fortran element (k, i, j) with
i in 1-h..im+h sits at [j-1+h, i-1+h, k-1].
"""
from __future__ import annotations

import math
from typing import Dict, List, Tuple

import numpy as np

EPS = 1e-12
PC = np.array([-9.0, 111.0, 29.0, -3.0]) / 128.0
QC = np.array([-3.0, 29.0, 111.0, -9.0]) / 128.0
AC = np.array([5.0, 30.0, -3.0]) / 32.0
BC = np.array([-3.0, 30.0, 5.0]) / 32.0


def def_maxgen(nxm: int, nym: int) -> int:
    def one(n):
        g = 1
        while True:
            n = (n + 1) // 2
            g += 1
            if n == 1:
                return g
    return min(one(nxm), one(nym))


def radial_stencil(p: int, ampl02: float):
    """(gx, gy, w) of vrbeta2 with its normalisation (getlinesum2)."""
    rmom2_2 = 1.0 / math.sqrt(2 * p + 4)
    e = math.sqrt(1.0 / ampl02) * rmom2_2
    out = []
    y = 1.0 / e
    for gy in range(math.ceil(-y + EPS), math.floor(y - EPS) + 1):
        rrx = (gy * e) ** 2
        x = math.sqrt(1.0 - rrx)
        for gx in range(math.ceil(-x / e + EPS), math.floor(x / e - EPS) + 1):
            out.append((gx, gy, (1.0 - (rrx + (gx * e) ** 2)) ** p))
    s = 1.0 / sum(w for _, _, w in out)
    return [(gx, gy, s * w) for gx, gy, w in out]


def line_stencil(p: int, ampl01: float):
    rmom2_1 = 1.0 / math.sqrt(2 * p + 3)
    e = (1.0 / math.sqrt(ampl01)) * rmom2_1
    x = 1.0 / e
    g = list(range(math.ceil(-x + EPS), math.floor(x - EPS) + 1))
    w = [(1.0 - (t * e) ** 2) ** p for t in g]
    s = 1.0 / sum(w)
    return [(t, s * v) for t, v in zip(g, w)]


class Tile:
    """One rank's array with halo h (same in x and y)."""

    def __init__(self, nk, im, jm, h):
        self.im, self.jm, self.h = im, jm, h
        self.a = np.zeros((jm + 2 * h, im + 2 * h, nk))

    def interior(self):
        h = self.h
        return self.a[h:h + self.jm, h:h + self.im, :]


class Layout:
    """Tiles of one generation: ntx x nty tiles of im x jm."""

    def __init__(self, ntx, nty, nk, im, jm, h):
        self.ntx, self.nty = ntx, nty
        self.t = {(x, y): Tile(nk, im, jm, h) for x in range(ntx) for y in range(nty)}

    def __getitem__(self, k):
        return self.t[k]

    def keys(self):
        return self.t.keys()

    # -------------------------------------------------------------- boco_2d
    def fill(self, nb):
        """boco_2d: N/S halo rows on interior columns, then E/W halo columns on
        all rows (incl. halo rows); mirror at the physical edges."""
        ny, nx = self.nty, self.ntx
        snap = {k: v.a.copy() for k, v in self.t.items()}
        for (x, y), T in self.t.items():
            h, im, jm = T.h, T.im, T.jm
            ci = slice(h, h + im)
            for j in range(1, nb + 1):  # south halo row 1-j (j = 1..nb)
                if y == 0:
                    T.a[h - j, ci] = snap[(x, y)][h + j - 1, ci]
                else:
                    T.a[h - j, ci] = snap[(x, y - 1)][h + jm - j, ci]
                if y == ny - 1:
                    T.a[h + jm - 1 + j, ci] = snap[(x, y)][h + jm - j, ci]
                else:
                    T.a[h + jm - 1 + j, ci] = snap[(x, y + 1)][h + j - 1, ci]
        snap = {k: v.a.copy() for k, v in self.t.items()}
        for (x, y), T in self.t.items():
            h, im, jm = T.h, T.im, T.jm
            rj = slice(h - nb, h + jm + nb)
            for i in range(1, nb + 1):
                if x == 0:
                    T.a[rj, h - i] = snap[(x, y)][rj, h + i - 1]
                else:
                    T.a[rj, h - i] = snap[(x - 1, y)][rj, h + im - i]
                if x == nx - 1:
                    T.a[rj, h + im - 1 + i] = snap[(x, y)][rj, h + im - i]
                else:
                    T.a[rj, h + im - 1 + i] = snap[(x + 1, y)][rj, h + i - 1]

    # ------------------------------------------------------------- bocoT_2d
    def fold(self, nb):
        """bocoT_2d: E/W halo columns (all rows) added to the neighbour's (or
        the mirrored own) interior, then N/S halo rows (interior columns)."""
        ny, nx = self.nty, self.ntx
        snap = {k: v.a.copy() for k, v in self.t.items()}
        for (x, y), T in self.t.items():
            h, im, jm = T.h, T.im, T.jm
            rj = slice(h - nb, h + jm + nb)
            for i in range(1, nb + 1):
                # from west: own west halo (mirror) or the west neighbour's east halo
                if x == 0:
                    T.a[rj, h + i - 1] += snap[(x, y)][rj, h - i]
                else:
                    T.a[rj, h + i - 1] += snap[(x - 1, y)][rj, h + im - 1 + i]
                if x == nx - 1:
                    T.a[rj, h + im - i] += snap[(x, y)][rj, h + im - 1 + i]
                else:
                    T.a[rj, h + im - i] += snap[(x + 1, y)][rj, h - i]
        snap = {k: v.a.copy() for k, v in self.t.items()}
        for (x, y), T in self.t.items():
            h, im, jm = T.h, T.im, T.jm
            ci = slice(h, h + im)
            for j in range(1, nb + 1):
                if y == 0:
                    T.a[h + j - 1, ci] += snap[(x, y)][h - j, ci]
                else:
                    T.a[h + j - 1, ci] += snap[(x, y - 1)][h + jm - 1 + j, ci]
                if y == ny - 1:
                    T.a[h + jm - j, ci] += snap[(x, y)][h + jm - 1 + j, ci]
                else:
                    T.a[h + jm - j, ci] += snap[(x, y + 1)][h - j, ci]


def vrbeta2(T: Tile, st):
    h, im, jm = T.h, T.im, T.jm
    b = np.zeros_like(T.a)
    for gx, gy, w in st:
        b[h:h + jm, h:h + im] += w * T.a[h + gy:h + gy + jm, h + gx:h + gx + im]
    T.a = b


def vrbeta2t(T: Tile, st):
    h, im, jm = T.h, T.im, T.jm
    b = np.zeros_like(T.a)
    src = T.a[h:h + jm, h:h + im]
    for gx, gy, w in st:
        b[h + gy:h + gy + jm, h + gx:h + gx + im] += w * src
    T.a = b


def adjoint(F: np.ndarray, quart: bool) -> np.ndarray:
    """P^T of one tile interior F (jm, im, nk) into the coarse transfer
    array with halo 2 (1 if quart): returns (jmL+2hb, imL+2hb, nk)."""
    jm, im, nk = F.shape
    hb = 1 if quart else 2
    imL, jmL = im // 2, jm // 2
    W = np.zeros((jmL + 2 * hb, imL + 2 * hb, nk))
    P1 = prolong_matrix(im, quart)  # (im, imL+2hb): fine x coarse-with-halo
    P2 = prolong_matrix(jm, quart)
    # W = P2^T F P1 (y pass then x pass; same operator as the loops)
    W += np.einsum("ja,jik,ib->abk", P2, F, P1)
    return W


def prolong_matrix(n: int, quart: bool) -> np.ndarray:
    """direct1/direct2 coefficients: fine (n) from coarse with halo."""
    hb = 1 if quart else 2
    nL = n // 2
    M = np.zeros((n, nL + 2 * hb))
    for i in range(1, n + 1):
        if not quart:
            iL = i // 2
            cf = QC if i % 2 else PC
            for t in range(4):
                M[i - 1, iL - 1 + t + hb - 1] += cf[t]
        else:
            if i % 2:
                iL, cf = (i + 1) // 2, AC
            else:
                iL, cf = i // 2, BC
            for t in range(3):
                M[i - 1, iL - 1 + t + hb - 1] += cf[t]
    return M


def direct(W: np.ndarray, im: int, jm: int, quart: bool) -> np.ndarray:
    P1 = prolong_matrix(im, quart)
    P2 = prolong_matrix(jm, quart)
    return np.einsum("ja,abk,ib->jik", P2, W, P1)


def vfilter(V: np.ndarray, lm: int, nzcol: int, zst, adj: bool):
    """sup_vrbeta1[T]_*: columns of lm levels at offsets (c-1)*lm."""
    hz = max(abs(g) for g, _ in zst)
    for c in range(nzcol):
        col = V[..., c * lm:(c + 1) * lm]
        W = np.zeros(col.shape[:2] + (lm + 2 * hz,))
        W[..., hz:hz + lm] = col
        for L in range(1, hz + 1):
            W[..., hz - L] = W[..., hz + L]
            W[..., hz + lm - 1 + L] = W[..., hz + lm - 1 - L]
        B = np.zeros_like(W)
        if not adj:
            for g, w in zst:
                B[..., hz:hz + lm] += w * W[..., hz + g:hz + g + lm]
        else:
            for g, w in zst:
                B[..., hz + g:hz + g + lm] += w * W[..., hz:hz + lm]
            for L in range(1, hz + 1):
                B[..., hz + L] += B[..., hz - L]
                B[..., hz + lm - 1 - L] += B[..., hz + lm - 1 + L]
        V[..., c * lm:(c + 1) * lm] = B[..., hz:hz + lm]


def line_colors(p: int, ampl02: float, nh: int = 6):
    """Procs 2/7 (init_mg_line, mg_intstate.f90:436-480): the triad of the
    Cholesky factor of the inverse aspect, (c, c, 0) with c = 1/sqrt(ampl02),
    gives generators (1,0), (0,1), (-1,-1) with spreads^2 (c, c, 0); each
    through hstform and blinfil (jp_pbfil3.f90:1399-1501).  Returned as
    gather stencils (gx, gy, w) per color."""
    bnorm, bsprd = np.zeros(nh + 1), np.zeros(nh + 1)
    for h in range(1, nh + 1):
        i = np.arange(-h, h + 1)
        w = (1.0 - (i / h) ** 2) ** p
        bnorm[h], bsprd[h] = 1.0 / w.sum(), (i * i * w).sum() / w.sum()
    c = math.sqrt(1.0 / ampl02)
    out = []
    for (dx, dy), s2 in (((1, 0), c), ((0, 1), c), ((-1, -1), 0.0)):
        m = next(m for m in range(2, nh + 1) if bsprd[m] >= s2)
        hs = m - (bsprd[m] - s2) / (bsprd[m] - bsprd[m - 1])
        h = int(hs)
        hp = h + 1
        fil = np.array([(hs - h) * bnorm[hp] * (1.0 - (t / hp) ** 2) ** p for t in range(h + 1)])
        fil[:h] += np.array([(hp - hs) * bnorm[h] * (1.0 - (t / h) ** 2) ** p for t in range(h)])
        st = [(0, 0, fil[0])]
        for t in range(1, h + 1):
            st += [(t * dx, t * dy, fil[t]), (-t * dx, -t * dy, fil[t])]
        out.append(st)
    return out


def dibeta_weights(p: int, s2: float, nh: int = 6) -> np.ndarray:
    """hstform + blinfil (jp_pbfil3.f90:1399-1501) of one spread^2."""
    bnorm, bsprd = np.zeros(nh + 1), np.zeros(nh + 1)
    for h in range(1, nh + 1):
        i = np.arange(-h, h + 1)
        w = (1.0 - (i / h) ** 2) ** p
        bnorm[h], bsprd[h] = 1.0 / w.sum(), (i * i * w).sum() / w.sum()
    m = next(m for m in range(2, nh + 1) if bsprd[m] >= s2)
    hs = m - (bsprd[m] - s2) / (bsprd[m] - bsprd[m - 1])
    h = int(hs)
    hp = h + 1
    fil = np.array([(hs - h) * bnorm[hp] * (1.0 - (t / hp) ** 2) ** p for t in range(h + 1)])
    fil[:h] += np.array([(hp - hs) * bnorm[h] * (1.0 - (t / h) ** 2) ** p for t in range(h)])
    return fil


class Layout3:
    """Proc 5's 3D variables on every tile of a generation: arrays
    (jm+2h, im+2h, (lm+2hz)*nv), last axis (L+hz-1)*nv + v."""

    def __init__(self, L2: "Layout", nv: int, lm: int, hz: int):
        self.L2, self.nv, self.lm, self.hz = L2, nv, lm, hz
        self.t = {}
        for k, T in L2.t.items():
            a = np.zeros(T.a.shape[:2] + ((lm + 2 * hz) * nv,))
            for L in range(1, lm + 1):
                a[..., (L + hz - 1) * nv:(L + hz) * nv] = T.a[..., [v * lm + L - 1 for v in range(nv)]]
            self.t[k] = a

    def back(self):
        for k, T in self.L2.t.items():
            a = self.t[k]
            for L in range(1, self.lm + 1):
                T.a[..., [v * self.lm + L - 1 for v in range(self.nv)]] = a[..., (L + self.hz - 1) * self.nv:
                                                                             (L + self.hz) * self.nv]

    def zl(self, L):
        return slice((L + self.hz - 1) * self.nv, (L + self.hz) * self.nv)

    def zmirror(self):
        for a in self.t.values():
            for L in range(1, self.hz + 1):
                a[..., self.zl(1 - L)] = a[..., self.zl(1 + L)]
                a[..., self.zl(self.lm + L)] = a[..., self.zl(self.lm - L)]

    def fill(self, nb, gh):
        """boco_3d (mg_bocos.f90:1425-2170) on levels 1..lm: N/S rows, then
        E/W columns; physical east edge W(I+i) = W(I-i) at generation 1
        (_g1), W(I+1-i) at coarser ones (_gh, which then mirrors z)."""
        L2, ks = self.L2, slice(self.hz * self.nv, (self.hz + self.lm) * self.nv)
        ny, nx = L2.nty, L2.ntx
        snap = {k: a.copy() for k, a in self.t.items()}
        for (x, y), a in self.t.items():
            T = L2[(x, y)]
            h, im, jm = T.h, T.im, T.jm
            ci = slice(h, h + im)
            for j in range(1, nb + 1):
                a[h + jm - 1 + j, ci, ks] = (snap[(x, y)][h + jm - j, ci, ks] if y == ny - 1
                                             else snap[(x, y + 1)][h + j - 1, ci, ks])
                a[h - j, ci, ks] = (snap[(x, y)][h + j - 1, ci, ks] if y == 0
                                    else snap[(x, y - 1)][h + jm - j, ci, ks])
        snap = {k: a.copy() for k, a in self.t.items()}
        for (x, y), a in self.t.items():
            T = L2[(x, y)]
            h, im, jm = T.h, T.im, T.jm
            rj = slice(h - nb, h + jm + nb)
            for i in range(1, nb + 1):
                a[rj, h - i, ks] = (snap[(x, y)][rj, h + i - 1, ks] if x == 0
                                    else snap[(x - 1, y)][rj, h + im - i, ks])
                src = h + im - i if gh else h + im - i - 1
                a[rj, h + im - 1 + i, ks] = (snap[(x, y)][rj, src, ks] if x == nx - 1
                                             else snap[(x + 1, y)][rj, h + i - 1, ks])
        if gh:
            self.zmirror()

    def fold(self, nb, gh):
        """bocoT_3d (mg_bocos.f90:2173-2908): E/W columns on every row, N/S
        rows on the interior columns (levels 1..lm), then the z halo.  At
        generation 1 the physical east and north folds read one cell
        inward: W(I+hx-i), W(J+hy-j)."""
        L2, ks = self.L2, slice(self.hz * self.nv, (self.hz + self.lm) * self.nv)
        ny, nx = L2.nty, L2.ntx
        o = 0 if gh else 1
        snap = {k: a.copy() for k, a in self.t.items()}
        for (x, y), a in self.t.items():
            T = L2[(x, y)]
            h, im, jm = T.h, T.im, T.jm
            rj = slice(h - nb, h + jm + nb)
            for i in range(1, nb + 1):
                a[rj, h + i - 1, ks] += (snap[(x, y)][rj, h - i, ks] if x == 0
                                         else snap[(x - 1, y)][rj, h + im - 1 + i, ks])
                a[rj, h + im - i, ks] += (snap[(x, y)][rj, h + im - 1 + i - o, ks] if x == nx - 1
                                          else snap[(x + 1, y)][rj, h - i, ks])
        snap = {k: a.copy() for k, a in self.t.items()}
        for (x, y), a in self.t.items():
            T = L2[(x, y)]
            h, im, jm = T.h, T.im, T.jm
            ci = slice(h, h + im)
            for j in range(1, nb + 1):
                a[h + j - 1, ci, ks] += (snap[(x, y)][h - j, ci, ks] if y == 0
                                         else snap[(x, y - 1)][h + jm - 1 + j, ci, ks])
                a[h + jm - j, ci, ks] += (snap[(x, y)][h + jm - 1 + j - o, ci, ks] if y == ny - 1
                                          else snap[(x, y + 1)][h - j, ci, ks])
        for a in self.t.values():
            for L in range(1, self.hz + 1):
                a[..., self.zl(1 + L)] += a[..., self.zl(1 - L)]
                a[..., self.zl(self.lm - L)] += a[..., self.zl(self.lm + L)]

    def dib(self, color, adj):
        """vdibetax3 / vdibetax3t of one color on every tile (None: copy)."""
        nv, hz, lm = self.nv, self.hz, self.lm
        for k, a in self.t.items():
            T = self.L2[k]
            h, im, jm = T.h, T.im, T.jm
            b = np.zeros_like(a)
            inner = (slice(h, h + jm), slice(h, h + im), slice(hz * nv, (hz + lm) * nv))

            def sh(t, d):
                dx, dy, dz = d
                return (slice(h + t * dy, h + t * dy + jm), slice(h + t * dx, h + t * dx + im),
                        slice((hz + t * dz) * nv, (hz + t * dz + lm) * nv))

            if color is None:
                b[inner] = a[inner]
            else:
                d, fil = color
                if not adj:
                    b[inner] = fil[0] * a[inner]
                    for t in range(1, len(fil)):
                        b[inner] += fil[t] * (a[sh(t, d)] + a[sh(-t, d)])
                else:
                    b[inner] += fil[0] * a[inner]
                    for t in range(1, len(fil)):
                        b[sh(t, d)] += fil[t] * a[inner]
                        b[sh(-t, d)] += fil[t] * a[inner]
            self.t[k] = b


def sub_layout(L: "Layout", k0: int, k1: int) -> "Layout":
    """The levels [k0, k1) of every tile as a Layout of copies."""
    S = Layout(L.ntx, L.nty, k1 - k0, next(iter(L.t.values())).im, next(iter(L.t.values())).jm,
               next(iter(L.t.values())).h)
    for k, T in L.t.items():
        S[k].a = T.a[..., k0:k1].copy()
    return S


def filtering(x: np.ndarray, *, nxPE, nyPE, im, jm, hx, p, ampl01, ampl02, weights, gm, proc=1, lm=1,
              nzcol=0, lquart=False, l_filt_g1=True, ampl03=1.0, hz=1) -> np.ndarray:
    """Apply filtering_procedure(proc) to the global compact field x
    (J, I, nk) through the emulated rank tiles; returns the global result."""
    J, I, nk = x.shape
    assert I == nxPE * im and J == nyPE * jm
    h = hx
    st = radial_stencil(p, ampl02)
    colors = line_colors(p, ampl02) if proc in (2, 5, 7) else None  # filtering_lin2_* / lin3
    if proc == 5:  # the hexad of (c3, c3, c3, 0, 0, 0): x, y, z lines, identity diagonals, color 7 null
        c3 = math.sqrt(1.0 / ampl03)
        hexcols = {1: ((1, 0, 0), dibeta_weights(p, c3)), 2: ((0, 1, 0), dibeta_weights(p, c3)),
                   3: ((0, 0, 1), dibeta_weights(p, c3)), 4: ((1, -1, 0), dibeta_weights(p, 0.0)),
                   5: ((-1, 0, 1), dibeta_weights(p, 0.0)), 6: ((0, 1, -1), dibeta_weights(p, 0.0)), 7: None}
    filt1 = proc in (1, 2, 5) or l_filt_g1
    zfilt = nzcol and proc != 5  # filtering_lin3 has no separate vertical filter
    hb = 1 if lquart else 2
    V = x.copy()
    if zfilt:
        vfilter(V, lm, nzcol, line_stencil(p, ampl01), adj=True)
    # generation layouts: gen g has (nxPE >> (g-1)) x (nyPE >> (g-1)) full tiles
    gens: List[Layout] = []
    for g in range(gm):
        ntx, nty = nxPE >> g, nyPE >> g
        assert ntx >= 1 and nty >= 1 and (ntx << g) == nxPE and (nty << g) == nyPE, "power-of-2 rank layout"
        gens.append(Layout(ntx, nty, nk, im, jm, h))
    for (tx, ty) in gens[0].keys():
        gens[0][(tx, ty)].interior()[...] = V[ty * jm:(ty + 1) * jm, tx * im:(tx + 1) * im]
    # upsending: adjoint, bocoT with halo 2 on the finer layout, upsend into quadrants
    for g in range(gm - 1):
        fine = gens[g]
        tr = Layout(fine.ntx, fine.nty, nk, im // 2, jm // 2, hb)
        for k in fine.keys():
            tr[k].a = adjoint(fine[k].interior(), lquart)
        tr.fold(hb)
        coarse = gens[g + 1]
        for (tx, ty) in fine.keys():
            q = coarse[(tx // 2, ty // 2)]
            ox, oy = (tx % 2) * (im // 2), (ty % 2) * (jm // 2)
            q.interior()[oy:oy + jm // 2, ox:ox + im // 2] = tr[(tx, ty)].interior()
    # filters at all generations
    for g in range(gm):
        if g == 0 and not filt1:
            continue
        L = gens[g]
        if proc == 5:
            # filtering_lin3 (mg_filtering.f90:285-535): 2D variables as
            # proc 2, 3D variables through the seven colors; _g1 halo
            # routines at generation 1, _gh at coarser ones
            n3 = nzcol * lm
            S2 = sub_layout(L, n3, nk)
            for cst in reversed(colors):
                for k in S2.keys():
                    vrbeta2t(S2[k], cst)
                S2.fold(h)
            L3 = Layout3(L, nzcol, lm, hz)
            for col in range(7, 0, -1):
                L3.zmirror()
                L3.dib(hexcols[col], True)
                L3.fold(h, g > 0)
            L3.back()
            for k in L.keys():
                L[k].a[..., n3:] = S2[k].a
                L[k].interior()[...] *= weights[g]
            S2 = sub_layout(L, n3, nk)
            for cst in colors:
                S2.fill(h)
                for k in S2.keys():
                    vrbeta2(S2[k], cst)
            L3 = Layout3(L, nzcol, lm, hz)
            L3.zmirror()
            for col in range(1, 8):
                L3.fill(h, g > 0)
                L3.dib(hexcols[col], False)
            L3.back()
            for k in L.keys():
                L[k].a[..., n3:] = S2[k].a
            continue
        if colors is not None:
            # colors 3, 2, 1: dibetat + bocoT_2d; weighting; colors 1, 2, 3:
            # boco_2d + dibeta (mg_filtering.f90:725-797, 1180-1290)
            for cst in reversed(colors):
                for k in L.keys():
                    vrbeta2t(L[k], cst)
                L.fold(h)
            for k in L.keys():
                L[k].interior()[...] *= weights[g]
            for cst in colors:
                L.fill(h)
                for k in L.keys():
                    vrbeta2(L[k], cst)
            continue
        for k in L.keys():
            vrbeta2t(L[k], st)
        L.fold(h)
        for k in L.keys():
            L[k].interior()[...] *= weights[g]
        L.fill(h)
        for k in L.keys():
            vrbeta2(L[k], st)
    # downsending: coarse quadrants to the finer tiles' transfer arrays, fill halo 2, direct, add
    for g in range(gm - 1, 0, -1):
        fine, coarse = gens[g - 1], gens[g]
        tr = Layout(fine.ntx, fine.nty, nk, im // 2, jm // 2, hb)
        for (tx, ty) in fine.keys():
            q = coarse[(tx // 2, ty // 2)]
            ox, oy = (tx % 2) * (im // 2), (ty % 2) * (jm // 2)
            tr[(tx, ty)].interior()[...] = q.interior()[oy:oy + jm // 2, ox:ox + im // 2]
        tr.fill(hb)
        for k in fine.keys():
            fine[k].interior()[...] += direct(tr[k].a, im, jm, lquart)
    out = np.empty_like(V)
    for (tx, ty) in gens[0].keys():
        out[ty * jm:(ty + 1) * jm, tx * im:(tx + 1) * im] = gens[0][(tx, ty)].interior()
    if zfilt:
        # filtering_lin2_ens (proc 7) ends with the adjoint vertical filter
        vfilter(out, lm, nzcol, line_stencil(p, ampl01), adj=proc == 7)
    return out
