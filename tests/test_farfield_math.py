"""The coarsest tree level of the boundary operator as FFT convolutions on
the face lattices (csrc/farfield.cu), restated in numpy and checked against
the direct sum it replaces (tree_calc_3d's coarsest level,
source/pmbound.f90:1135-1249: each boundary node sums dS/r times the source
of every coarsest cell it does not open).

With each face side a multiple of istep = 2^levmax panels, the coarsest
cell centres (a * istep + istep/2 along each in-plane axis) and the boundary
nodes are points of one node lattice, and dS/r depends only on index
offsets:
- between parallel faces the sum over a face's cells is a 2-D convolution
  over the in-plane offsets, at the fixed distance between the planes;
- between perpendicular faces it is a 1-D convolution along the axis the
  two faces share.  For each frequency it is a dense sum over the target's
  index along the source face's normal and the cell's index along the
  target face's normal.
Opened cells (closer than the opening radius) are summed by the FFTs too and
then subtracted; the dense block's zero slots are exactly those cells.  A
cell centre on a target node (r = 0) contributes 0 in both.  CPU only.
"""
import numpy as np
import pytest


def _ax_u(f):  # in-plane axes of face f (normal f // 2): X faces (y, z), Y (x, z), Z (x, y)
    return 1 if f // 2 == 0 else 0


def _ax_v(f):
    return 1 if f // 2 == 2 else 2


def _cells(N, istep):
    """Per face: the coarsest cells' centres as lattice coordinates (3 ints each)."""
    out = []
    for f in range(6):
        n, u, v = f // 2, _ax_u(f), _ax_v(f)
        ma, mb = (N[u] - 1) // istep, (N[v] - 1) // istep
        c = np.zeros((ma * mb, 3), dtype=np.int64)
        c[:, n] = 0 if f % 2 == 0 else N[n] - 1
        c[:, u] = np.tile(np.arange(ma) * istep + istep // 2, mb)
        c[:, v] = np.repeat(np.arange(mb) * istep + istep // 2, ma)
        out.append(c)
    return out


def _targets(N, f):
    """Face f's nodes as lattice coordinates, u fastest."""
    n, u, v = f // 2, _ax_u(f), _ax_v(f)
    t = np.zeros((N[u] * N[v], 3), dtype=np.int64)
    t[:, n] = 0 if f % 2 == 0 else N[n] - 1
    t[:, u] = np.tile(np.arange(N[u]), N[v])
    t[:, v] = np.repeat(np.arange(N[v]), N[u])
    return t


def _kern(dS, d):
    """dS / r for offset vectors d (already scaled by the spacings); 0 at r = 0."""
    r = np.sqrt((d * d).sum(-1))
    with np.errstate(divide="ignore"):
        return np.where(r > 0, dS / np.where(r > 0, r, 1.0), 0.0)


def _direct(N, h, istep, sig, opened=None):
    """Every face's nodes summing every (accepted) cell of every face."""
    cells = _cells(N, istep)
    out = []
    for T in range(6):
        t = _targets(N, T)
        acc = np.zeros(len(t))
        for G in range(6):
            dS = istep * h[_ax_u(G)] * istep * h[_ax_v(G)]
            d = (t[:, None, :] - cells[G][None, :, :]) * np.asarray(h)
            w = _kern(dS, d)
            if opened is not None:
                w = np.where(opened(d, dS), 0.0, w)
            acc += w @ sig[G]
        out.append(acc)
    return out


def _fft(N, h, istep, sig):
    """The same sums (every cell) by FFT convolutions on the face lattices."""
    h = np.asarray(h)
    cells = _cells(N, istep)
    out = [np.zeros(N[_ax_u(T)] * N[_ax_v(T)]) for T in range(6)]
    for T in range(6):
        nT, uT, vT = T // 2, _ax_u(T), _ax_v(T)
        sT = 0 if T % 2 == 0 else N[nT] - 1
        res = np.zeros((N[vT], N[uT]))
        for G in range(6):
            nG, uG, vG = G // 2, _ax_u(G), _ax_v(G)
            sG = 0 if G % 2 == 0 else N[nG] - 1
            dS = istep * h[uG] * istep * h[vG]
            if nG == nT:
                # parallel: 2-D linear convolution over (u, v) offsets
                Pu, Pv = 2 * N[uT], 2 * N[vT]
                src = np.zeros((Pv, Pu))
                src[cells[G][:, vG], cells[G][:, uG]] = sig[G]
                du = np.fft.fftfreq(Pu, 1.0 / Pu)  # signed circular offsets
                dv = np.fft.fftfreq(Pv, 1.0 / Pv)
                D = (sT - sG) * h[nT]
                d = np.stack(np.broadcast_arrays(du[None, :] * h[uT], dv[:, None] * h[vT],
                                                 np.full((Pv, Pu), D)), axis=-1)
                K = _kern(dS, d)
                conv = np.real(np.fft.ifft2(np.fft.fft2(src) * np.fft.fft2(K)))
                res += conv[:N[vT], :N[uT]]
            else:
                # perpendicular: 1-D convolution along the shared axis w,
                # dense over (target index along nG, cell index along nT)
                w = 3 - nT - nG
                Pw = 2 * N[w]
                ct = np.unique(cells[G][:, nT])           # cells' coordinates along nT
                S = np.zeros((len(ct), Pw))
                row = np.searchsorted(ct, cells[G][:, nT])
                np.add.at(S, (row, cells[G][:, w]), sig[G])
                Shat = np.fft.fft(S, axis=1)               # [cell row][omega]
                ig = np.arange(N[nG])                       # target index along nG
                dw = np.fft.fftfreq(Pw, 1.0 / Pw)
                d = np.stack(np.broadcast_arrays(
                    ((ig - sG) * h[nG])[:, None, None],
                    ((ct - sT) * h[nT])[None, :, None],
                    (dw * h[w])[None, None, :]), axis=-1)
                Khat = np.fft.fft(_kern(dS, d), axis=2)     # [ig][cell row][omega]
                Ohat = np.einsum("gcw,cw->gw", Khat, Shat)  # the dense sum per frequency
                o = np.real(np.fft.ifft(Ohat, axis=1))[:, :N[w]]  # [ig][iw]
                # place on T's (v, u) grid: T's in-plane axes are nG and w
                res += o.T if uT == nG else o
        out[T] = res.ravel()
    return out


CASES = [((17, 13, 21), (0.1, 0.07, 0.05), 4),
         ((9, 17, 13), (0.06, 0.05, 0.08), 4),
         ((13, 9, 9), (0.05, 0.05, 0.05), 2)]


@pytest.mark.parametrize("N,h,istep", CASES)
def test_fft_sum_equals_direct_sum(N, h, istep):
    rng = np.random.default_rng(sum(N))
    cells = _cells(N, istep)
    sig = [rng.standard_normal(len(c)) for c in cells]
    ref = _direct(N, h, istep, sig)
    got = _fft(N, h, istep, sig)
    for T in range(6):
        scale = np.abs(ref[T]).max()
        assert np.abs(got[T] - ref[T]).max() <= 1e-12 * scale, T


@pytest.mark.parametrize("N,h,istep", CASES[:2])
def test_opened_cells_subtracted(N, h, istep):
    """FFT sum over every cell minus the opened cells' terms = the direct sum
    over the accepted cells.  The tree walk opens cells closer than
    10 sqrt(dS); on these small lattices that would open all of them, so the
    radius here is 2 sqrt(dS), which splits them."""
    rng = np.random.default_rng(7 + sum(N))
    cells = _cells(N, istep)
    sig = [rng.standard_normal(len(c)) for c in cells]

    def opened(d, dS):
        return np.sqrt((d * d).sum(-1)) < 2.0 * np.sqrt(dS)

    accepted = _direct(N, h, istep, sig, opened)
    every = _fft(N, h, istep, sig)
    n_open = n_all = 0
    for T in range(6):
        t = _targets(N, T)
        corr = np.zeros(len(t))
        for G in range(6):
            dS = istep * h[_ax_u(G)] * istep * h[_ax_v(G)]
            d = (t[:, None, :] - cells[G][None, :, :]) * np.asarray(h)
            op = opened(d, dS)
            n_open += int(op.sum())
            n_all += op.size
            corr += np.where(op, _kern(dS, d), 0.0) @ sig[G]
        scale = np.abs(every[T]).max()
        assert np.abs((every[T] - corr) - accepted[T]).max() <= 1e-12 * scale, T
    assert 0 < n_open < n_all  # both opened and accepted cells occur
