"""The adjoint line filter as a gather (the form the library's k_dibeta
adjoint uses) equals the reference's scatter + fold (vdibeta2t then
bocoT_2d, jp_pbfil3.f90:2345-2382, mg_bocos.f90:787-1422) for any integer
generator: target s collects, for every extended point q that the fold maps
onto s (s and its mirror images within the fold widths, up to three per axis
when the grid is narrower than twice the halo), the weight of every interior
source q - t d.  The reachable setups only give zero weights on the
diagonal; this checks the form for diagonal and knight-move generators with
nonzero weights too."""
import numpy as np
import pytest

from tests.test_oracle_lin2 import dibeta, fold_h

rng = np.random.default_rng(77)


def gather_adjoint(x, d, fil, hx, hy):
    J, I, nk = x.shape
    dx, dy = d
    h = len(fil) - 1
    out = np.zeros_like(x)
    for j in range(J):
        qy = [j] + ([-1 - j] if j < hy else []) + ([2 * J - 1 - j] if j >= J - hy else [])
        for i in range(I):
            qx = [i] + ([-1 - i] if i < hx else []) + ([2 * I - 1 - i] if i >= I - hx else [])
            acc = np.zeros(nk)
            for a in qx:
                for b in qy:
                    for t in range(-h, h + 1):
                        sx, sy = a - t * dx, b - t * dy
                        if 0 <= sx < I and 0 <= sy < J:
                            acc += fil[abs(t)] * x[sy, sx]
            out[j, i] = acc
    return out


@pytest.mark.parametrize("d", [(1, 0), (0, 1), (1, 1), (-1, 1), (2, 1), (1, -2)])
@pytest.mark.parametrize("I,J,hx,hy", [(12, 10, 4, 4), (5, 4, 4, 4), (3, 7, 2, 3)])
def test_gather_equals_scatter_and_fold(d, I, J, hx, hy):
    dx, dy = d
    h = min(hx // max(abs(dx), 1), hy // max(abs(dy), 1))  # reach within the halo
    fil = rng.random(h + 1)
    x = rng.standard_normal((J, I, 3))
    V = np.zeros((J + 2 * hy, I + 2 * hx, 3))
    V[hy:hy + J, hx:hx + I] = x
    ref = fold_h(dibeta(V, d, fil, hx, hy, True), hx, hy)[hy:hy + J, hx:hx + I]
    assert np.abs(gather_adjoint(x, d, fil, hx, hy) - ref).max() < 1e-13
