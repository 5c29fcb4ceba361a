"""The Dirichlet solve with its face values entering in DST space, as the
padded block's boundary-value solve and the inner box's final solve run it
(csrc/block_solve.cu: k_extract_faces / k_extract_box_faces, k_thomas_faces),
restated in numpy on small boxes.  It is checked against a direct sparse
solve of the same 7-point system (the reference's solve_eq_3d,
source/pmsolve.f90:284-365, solves that system with MKL's Helmholtz solver).

The fold under test: along an axis of m interior nodes the last layer's sine
is (-1)^p times the first's, sin(pi m (p+1)/(m+1)) = (-1)^p sin(pi (p+1)/(m+1)),
so a pair of opposite faces enters mode p as its sum (p even) or its
difference (p odd) times the first layer's sine.  CPU only.
"""
import numpy as np
import pytest

scipy_sparse = pytest.importorskip("scipy.sparse")
from scipy.sparse.linalg import spsolve  # noqa: E402


def _lap1(m, h):
    e = np.ones(m)
    return scipy_sparse.diags([e[:-1], -2.0 * e, e[:-1]], [-1, 0, 1]) / (h * h)


def _direct(r, faces, h):
    """Interior solution of the 7-point Laplacian = r with Dirichlet faces;
    arrays indexed [k][j][i] (z slowest)."""
    m2, m1, m0 = r.shape
    fx0, fxN, fy0, fyN, fz0, fzN = faces
    Ix, Iy, Iz = (scipy_sparse.identity(m) for m in (m0, m1, m2))
    L = (scipy_sparse.kron(Iz, scipy_sparse.kron(Iy, _lap1(m0, h[0])))
         + scipy_sparse.kron(Iz, scipy_sparse.kron(_lap1(m1, h[1]), Ix))
         + scipy_sparse.kron(_lap1(m2, h[2]), scipy_sparse.kron(Iy, Ix)))
    b = r.copy()
    b[:, :, 0] -= fx0 / h[0] ** 2
    b[:, :, -1] -= fxN / h[0] ** 2
    b[:, 0, :] -= fy0 / h[1] ** 2
    b[:, -1, :] -= fyN / h[1] ** 2
    b[0, :, :] -= fz0 / h[2] ** 2
    b[-1, :, :] -= fzN / h[2] ** 2
    return spsolve(L.tocsc(), b.ravel()).reshape(r.shape)


def _sines(m):
    n = np.arange(1, m + 1)
    return np.sin(np.pi * np.outer(n, n) / (m + 1))  # [p][i]


def _dst_space(r, faces, h, fold=True):
    """Forward x/y sine transforms of the RHS alone; the faces transformed
    along their own axes and added per mode; a Thomas sweep along z per
    (p, q) with the z faces at its ends; inverse transforms."""
    m2, m1, m0 = r.shape
    fx0, fxN, fy0, fyN, fz0, fzN = faces
    Sx, Sy = _sines(m0), _sines(m1)
    g = np.einsum("pi,qj,kji->kqp", Sx, Sy, r)
    ex1, ey1 = Sx[:, 0], Sy[:, 0]
    if fold:
        # the x pair as (sum, difference), chosen by the parity of p; the y
        # pair by the parity of q (k_extract_faces, k_thomas_faces)
        xs, xd = (fx0 + fxN) @ Sy.T, (fx0 - fxN) @ Sy.T  # [k][q]
        ys, yd = (fy0 + fyN) @ Sx.T, (fy0 - fyN) @ Sx.T  # [k][p]
        podd = (np.arange(m0) % 2 == 1)[None, None, :]
        qodd = (np.arange(m1) % 2 == 1)[None, :, None]
        fx = np.where(podd, xd[:, :, None], xs[:, :, None])
        fy = np.where(qodd, yd[:, None, :], ys[:, None, :])
        g = g - ex1[None, None, :] * fx / h[0] ** 2 - ey1[None, :, None] * fy / h[1] ** 2
    else:
        exN, eyN = Sx[:, -1], Sy[:, -1]
        g = g - (ex1[None, None, :] * (fx0 @ Sy.T)[:, :, None] + exN[None, None, :] * (fxN @ Sy.T)[:, :, None]) / h[0] ** 2
        g = g - (ey1[None, :, None] * (fy0 @ Sx.T)[:, None, :] + eyN[None, :, None] * (fyN @ Sx.T)[:, None, :]) / h[1] ** 2
    g[0] -= (Sy @ fz0 @ Sx.T) / h[2] ** 2
    g[-1] -= (Sy @ fzN @ Sx.T) / h[2] ** 2
    lx = -4.0 / h[0] ** 2 * np.sin(np.pi * np.arange(1, m0 + 1) / (2 * (m0 + 1))) ** 2
    ly = -4.0 / h[1] ** 2 * np.sin(np.pi * np.arange(1, m1 + 1) / (2 * (m1 + 1))) ** 2
    u = np.empty_like(g)
    off = np.ones(m2 - 1) / h[2] ** 2
    for q in range(m1):
        for p in range(m0):
            d = np.full(m2, -2.0 / h[2] ** 2 + lx[p] + ly[q])
            A = np.diag(d) + np.diag(off, 1) + np.diag(off, -1)
            u[:, q, p] = np.linalg.solve(A, g[:, q, p])
    return (2.0 / (m0 + 1)) * (2.0 / (m1 + 1)) * np.einsum("pi,qj,kqp->kji", Sx, Sy, u)


@pytest.mark.parametrize("m", [1, 2, 7, 8, 143, 271, 272])
def test_last_layer_sine_is_signed_first(m):
    p = np.arange(m)
    last = np.sin(np.pi * m * (p + 1) / (m + 1))
    first = np.sin(np.pi * (p + 1) / (m + 1))
    assert np.abs(last - (-1.0) ** p * first).max() <= 4e-13


@pytest.mark.parametrize("shape,h", [((5, 6, 7), (0.1, 0.1, 0.1)),
                                     ((7, 8, 9), (0.05, 0.07, 0.03)),
                                     ((6, 5, 4), (0.2, 0.11, 0.13))])
def test_folded_face_terms_match_direct_solve(shape, h):
    rng = np.random.default_rng(sum(shape))
    m2, m1, m0 = shape
    r = rng.standard_normal(shape)
    faces = (rng.standard_normal((m2, m1)), rng.standard_normal((m2, m1)),
             rng.standard_normal((m2, m0)), rng.standard_normal((m2, m0)),
             rng.standard_normal((m1, m0)), rng.standard_normal((m1, m0)))
    ref = _direct(r, faces, h)
    folded = _dst_space(r, faces, h, fold=True)
    unfolded = _dst_space(r, faces, h, fold=False)
    scale = np.abs(ref).max()
    assert np.abs(folded - ref).max() <= 1e-12 * scale
    assert np.abs(unfolded - ref).max() <= 1e-12 * scale
    assert np.abs(folded - unfolded).max() <= 1e-13 * scale
