"""CPU tests of the oracle's filtering_procedure(4), filtering_rad3
(mg_filtering.f90:123-257): the 2D variables through the 2D radial filter,
the 3D variables through the 3D ball filter vrbeta3 (jp_pbfil.f90:930-977)
with a whole-sample mirror in the level index.  As in the reference, the 3D
adjoint keeps only the interior of its scatter (sup_vrbeta3T copies the
interior back, mg_filtering.f90:1983-2039) and bocoT_2d then folds whatever
halo the generation held: the caller's VALL halo at generation 1."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import canonical

rng = np.random.default_rng(404)
P = 2


def cfg(**kw):
    # 2 3D variables of 6 levels + 2 2D variables; ball reach 2 (ampl03 = 1),
    # disk reach 3
    d = dict(I=20, J=16, nk=14, hx=3, hy=3, hz=2, p=P, ampl01=1.0, ampl02=canonical(3), gm=1, weights=[0.8],
             proc=4, lm=6, nzcol=2, ampl03=1.0)
    d.update(kw)
    return O.OracleConfig(**d)


def ball(ampl03, p=P, eps=1e-12):
    e = np.sqrt(1.0 / ampl03) / np.sqrt(2 * p + 5)
    out = []
    z = 1.0 / e
    for gz in range(int(np.ceil(-z + eps)), int(np.floor(z - eps)) + 1):
        rry = (gz * e) ** 2
        y = np.sqrt(1.0 - rry)
        for gy in range(int(np.ceil(-y / e + eps)), int(np.floor(y / e - eps)) + 1):
            rrx = rry + (gy * e) ** 2
            x = np.sqrt(1.0 - rrx)
            for gx in range(int(np.ceil(-x / e + eps)), int(np.floor(x / e - eps)) + 1):
                out.append((gx, gy, gz, (1.0 - rrx - (gx * e) ** 2) ** p))
    s = 1.0 / sum(w for *_, w in out)
    return [(gx, gy, gz, s * w) for gx, gy, gz, w in out]


def disk(ampl02, p=P, eps=1e-12):
    e = np.sqrt(1.0 / ampl02) / np.sqrt(2 * p + 4)
    out = []
    y = 1.0 / e
    for gy in range(int(np.ceil(-y + eps)), int(np.floor(y - eps)) + 1):
        rrx = (gy * e) ** 2
        x = np.sqrt(1.0 - rrx)
        for gx in range(int(np.ceil(-x / e + eps)), int(np.floor(x / e - eps)) + 1):
            out.append((gx, gy, (1.0 - rrx - (gx * e) ** 2) ** p))
    s = 1.0 / sum(w for *_, w in out)
    return [(gx, gy, s * w) for gx, gy, w in out]


def fold_xy(U, hx, hy):
    """bocoT_2d at the physical edges: x on every row, then y on the
    interior columns; the halo keeps its values."""
    U = U.copy()
    J, I = U.shape[0] - 2 * hy, U.shape[1] - 2 * hx
    for t in range(1, hx + 1):
        U[:, hx + t - 1] += U[:, hx - t]
        U[:, hx + I - t] += U[:, hx + I + t - 1]
    for t in range(1, hy + 1):
        U[hy + t - 1, hx:hx + I] += U[hy - t, hx:hx + I]
        U[hy + J - t, hx:hx + I] += U[hy + J + t - 1, hx:hx + I]
    return U


def fill_xy(U, hx, hy):
    """boco_2d: y on the interior columns, then x on every row."""
    U = U.copy()
    J, I = U.shape[0] - 2 * hy, U.shape[1] - 2 * hx
    for t in range(1, hy + 1):
        U[hy - t, hx:hx + I] = U[hy + t - 1, hx:hx + I]
        U[hy + J + t - 1, hx:hx + I] = U[hy + J - t, hx:hx + I]
    for t in range(1, hx + 1):
        U[:, hx - t] = U[:, hx + t - 1]
        U[:, hx + I + t - 1] = U[:, hx + I - t]
    return U


def numpy_rad3_g1(c, V):
    """One generation of filtering_rad3 on a VALL with halo, restated."""
    hx, hy, hz, lm = c.hx, c.hy, c.hz, c.lm
    J, I = c.J, c.I
    n3 = c.nzcol * lm
    U = V.copy()
    # adjoint, 2D variables: scatter into the extended domain (halo included)
    for k in range(n3, c.nk):
        E = np.zeros(U.shape[:2])
        for gx, gy, w in disk(c.ampl02):
            E[hy + gy:hy + gy + J, hx + gx:hx + gx + I] += w * V[hy:hy + J, hx:hx + I, k]
        U[..., k] = E
    # adjoint, 3D variables: scatter, level fold, interior only
    bl = ball(c.ampl03)
    for v in range(c.nzcol):
        col = V[hy:hy + J, hx:hx + I, v * lm:(v + 1) * lm]
        E = np.zeros((J + 2 * hy, I + 2 * hx, lm + 2 * hz))
        for gx, gy, gz, w in bl:
            E[hy + gy:hy + gy + J, hx + gx:hx + gx + I, hz + gz:hz + gz + lm] += w * col
        for t in range(1, hz + 1):
            E[..., hz + t] += E[..., hz - t]
            E[..., hz + lm - 1 - t] += E[..., hz + lm - 1 + t]
        U[hy:hy + J, hx:hx + I, v * lm:(v + 1) * lm] = E[hy:hy + J, hx:hx + I, hz:hz + lm]
    U = fold_xy(U, hx, hy)
    U[hy:hy + J, hx:hx + I] *= c.weights[0]
    U = fill_xy(U, hx, hy)
    out = U.copy()
    for k in range(n3, c.nk):  # forward 2D: gather, halo zeroed
        acc = np.zeros((J, I))
        for gx, gy, w in disk(c.ampl02):
            acc += w * U[hy + gy:hy + gy + J, hx + gx:hx + gx + I, k]
        out[..., k] = 0.0
        out[hy:hy + J, hx:hx + I, k] = acc
    for v in range(c.nzcol):  # forward 3D: gather with the level mirror, interior only
        col = np.pad(U[..., v * lm:(v + 1) * lm], ((0, 0), (0, 0), (hz, hz)), mode="reflect")
        acc = np.zeros((J, I, lm))
        for gx, gy, gz, w in bl:
            acc += w * col[hy + gy:hy + gy + J, hx + gx:hx + gx + I, hz + gz:hz + gz + lm]
        out[hy:hy + J, hx:hx + I, v * lm:(v + 1) * lm] = acc
    return out


def test_one_generation_matches_numpy_with_halo():
    c = cfg()
    V = rng.standard_normal((c.J + 2 * c.hy, c.I + 2 * c.hx, c.nk))
    ref = numpy_rad3_g1(c, V)
    got = V.copy()
    O.filtering_procedure(c, got)
    assert np.abs(got - ref).max() < 1e-13


def test_input_halo_of_3d_variables_enters_the_result():
    """The caller's halo reaches the result through the 3D variables only."""
    c = cfg()
    V = rng.standard_normal((c.J + 2 * c.hy, c.I + 2 * c.hx, c.nk))
    W = V.copy()
    W[:c.hy] += 1.0  # change the halo only
    a, b = V.copy(), W.copy()
    O.filtering_procedure(c, a)
    O.filtering_procedure(c, b)
    inner = (slice(c.hy, c.hy + c.J), slice(c.hx, c.hx + c.I))
    n3 = c.nzcol * c.lm
    assert np.abs(a[inner][..., :n3] - b[inner][..., :n3]).max() > 1e-3
    assert np.abs(a[inner][..., n3:] - b[inner][..., n3:]).max() == 0.0


@pytest.mark.parametrize("lquart", [False, True])
def test_interior_impulse_is_symmetric(lquart):
    """Away from the edges the truncation does not act: a centred impulse
    gives a response symmetric under the grid's reflections."""
    c = cfg(I=32, J=32, gm=3, weights=[1.0, 0.5, 0.25], lquart=lquart, nk=6, nzcol=1, lm=6)
    x = np.zeros((32, 32, 6))
    x[15:17, 15:17, 2:4] = 1.0
    y = O.filter_compact(c, x)
    assert np.abs(y - y[::-1]).max() < 1e-14
    assert np.abs(y - y[:, ::-1]).max() < 1e-14
    assert np.abs(y - y.transpose(1, 0, 2)).max() < 1e-14


def test_not_self_adjoint_near_the_edges():
    """The dropped halo scatter makes the reference's proc 4 operator
    non-symmetric (procs 1, 3, 6, 8 are symmetric)."""
    c = cfg(gm=2, weights=[1.0, 0.5])
    a, b = rng.standard_normal((c.J, c.I, c.nk)), rng.standard_normal((c.J, c.I, c.nk))
    la, lb = O.filter_compact(c, a), O.filter_compact(c, b)
    assert abs((la * b).sum() - (a * lb).sum()) > 1e-6 * np.abs(la * b).sum()


def test_rad3_errors():
    with pytest.raises(O.OracleError):  # ball reach 3 (ampl03 = 1.5) > hz = 2
        O.filter_compact(cfg(ampl03=1.5), np.zeros((16, 20, 14)))
    with pytest.raises(O.OracleError):  # weight gradients are not defined for proc 4
        O.weight_grads(cfg(), np.zeros((16, 20, 14)), np.zeros((16, 20, 14)))
