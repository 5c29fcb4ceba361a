"""CPU checks of the oracle: pins against the reference's known answers.

The reference (Fortran + MPI + Intel MKL) cannot be built here, and it ships
no numeric fixtures.  The oracle is pinned by (1) the MKL Dirichlet-solver
semantics it restates (discrete residual, scipy.fft.dstn), (2) Hill's
spherical vortex (source/test_applic.f90:2-179), (3) the untreed boundary
sum, (4) the reference's sizing rules (source/pmlib.f90:216-432,
source/vpm.f90:477-660) and (5) its own committed regression fixtures.
"""
import os

import numpy as np
import pytest
import scipy.fft as sf

from helpers import rel_l2

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _lap(u, d):
    return ((u[1:-1, 1:-1, 2:] - 2 * u[1:-1, 1:-1, 1:-1] + u[1:-1, 1:-1, :-2]) / d[0] ** 2 +
            (u[1:-1, 2:, 1:-1] - 2 * u[1:-1, 1:-1, 1:-1] + u[1:-1, :-2, 1:-1]) / d[1] ** 2 +
            (u[2:, 1:-1, 1:-1] - 2 * u[1:-1, 1:-1, 1:-1] + u[:-2, 1:-1, 1:-1]) / d[2] ** 2)


@pytest.mark.parametrize("shape", [(13, 11, 17), (9, 34, 19), (18, 18, 18)])
def test_dirichlet_residual_and_boundary(oracle, shape):
    rng = np.random.default_rng(0)
    d = (0.1, 0.13, 0.07)
    rhs = rng.standard_normal(shape)
    sol = rng.standard_normal(shape)
    s0 = sol.copy()
    oracle.dirichlet(rhs, sol, d)
    scale = np.abs(rhs).max() + np.abs(sol).max() / min(d) ** 2
    assert np.abs(_lap(sol, d) - rhs[1:-1, 1:-1, 1:-1]).max() <= 1e-12 * scale
    for sl in (np.s_[0], np.s_[-1], np.s_[:, 0], np.s_[:, -1], np.s_[:, :, 0], np.s_[:, :, -1]):
        assert np.array_equal(sol[sl], s0[sl])


def test_dirichlet_zero_bc_matches_scipy_dstn(oracle):
    rng = np.random.default_rng(1)
    nz, ny, nx = 15, 12, 19
    d = (0.2, 0.1, 0.15)
    rhs = rng.standard_normal((nz, ny, nx))
    out = np.full_like(rhs, 7.0)
    oracle.dirichlet(rhs, out, d, zero_bc=True)
    f = rhs[1:-1, 1:-1, 1:-1]
    lam = [-(2 - 2 * np.cos(np.pi * np.arange(1, n - 1) / (n - 1))) / h ** 2 for n, h in ((nx, d[0]), (ny, d[1]), (nz, d[2]))]
    L = lam[2][:, None, None] + lam[1][None, :, None] + lam[0][None, None, :]
    u = sf.idstn(sf.dstn(f, type=1) / L, type=1)
    assert rel_l2(out[1:-1, 1:-1, 1:-1], u) <= 1e-13
    assert np.all(out[0] == 0) and np.all(out[:, :, -1] == 0)


def test_hill_vortex_known_answer(oracle):
    """Infinite-domain solve of Hill's vortex: max |u| error shrinks with h
    (first order at the vorticity jump of the sphere)."""
    from golden.make_golden import hill
    errs = []
    for h in (0.1, 0.05):
        L = 1.6
        n = int(round(2 * L / h)) + 1
        x = -L + h * np.arange(n)
        Z, Y, X = np.meshgrid(x, x, x, indexing="ij")
        U, Wv = hill(X, Y, Z)
        rhs = [np.ascontiguousarray(-w) for w in Wv]
        sol = [np.zeros_like(rhs[0]) for _ in range(3)]
        oracle.pmesh(sol, rhs, (-L, -L, -L, L, L, L), (h, h, h), iynbc=1, itree=1, levmax=3)

        def d(f, ax):
            g = np.zeros_like(f)
            sp = [slice(1, -1)] * 3
            sm = [slice(1, -1)] * 3
            sp[ax], sm[ax] = slice(2, None), slice(0, -2)
            g[1:-1, 1:-1, 1:-1] = (f[tuple(sp)] - f[tuple(sm)]) / (2 * h)
            return g
        ux = d(sol[2], 1) - d(sol[1], 0)
        uy = -(d(sol[2], 2) - d(sol[0], 0))
        uz = d(sol[1], 2) - d(sol[0], 1)
        I = (slice(1, -1),) * 3
        vm = np.sqrt(ux ** 2 + uy ** 2 + uz ** 2)[I]
        am = np.sqrt(U[0] ** 2 + U[1] ** 2 + U[2] ** 2)[I]
        errs.append(np.abs(vm - am).max())
    assert errs[0] < 0.07 and errs[1] < 0.04 and errs[1] < 0.65 * errs[0]


def test_hill_golden_fixture():
    from golden.make_golden import hill
    g = np.load(os.path.join(GOLD, "hill_vortex.npz"))
    p = g["points"]
    u, w = hill(p[:, 0], p[:, 1], p[:, 2])
    assert np.allclose(u, g["u"], rtol=0, atol=1e-15) and np.allclose(w, g["omega"], rtol=0, atol=1e-15)


def test_tree_close_to_direct_sum_and_levmax0_equals_direct(oracle):
    n, h = 33, 0.1
    L = (n - 1) * h / 2
    x = -L + h * np.arange(n)
    Z, Y, X = np.meshgrid(x, x, x, indexing="ij")
    blob = np.exp(-(X ** 2 + Y ** 2 + Z ** 2) / (0.2 * L * L))
    sol0 = [np.zeros_like(blob) for _ in range(3)]
    for c in range(3):
        oracle.dirichlet(-blob * (c + 1), sol0[c], (h, h, h), zero_bc=True)
    xb = (-L, -L, -L, L, L, L)
    direct, nd = oracle.boundary_values(sol0, xb, (h, h, h), 0, direct=True)
    tree, nt = oracle.boundary_values(sol0, xb, (h, h, h), 3)
    flat, nf = oracle.boundary_values(sol0, xb, (h, h, h), 0)
    face = np.zeros(blob.shape, bool)
    face[0] = face[-1] = True
    face[:, 0] = face[:, -1] = True
    face[:, :, 0] = face[:, :, -1] = True
    for c in range(3):
        assert rel_l2(flat[c][face], direct[c][face]) <= 1e-13   # untreed walk == direct sum
        assert rel_l2(tree[c][face], direct[c][face]) <= 2e-3    # monopole tree error bound
    assert nt < nd and nf == nd


def test_fsour_a4_is_the_constant_source_panel_potential(oracle):
    """FSOUR_A4 (source/pmbound.f90:1540-1620) against the integral
    -1/(4 pi) ∫∫ dS / |x - y| over the panel, by adaptive quadrature, for
    points above, beside (in the panel's plane) and below the panel, in
    the frame of every target plane; far points take the monopole branch."""
    from scipy import integrate
    d = (0.1, 0.07, 0.05)
    frames = {1: ((1, 0, 0), (0, 0, 1), (0, -1, 0), 0.1, 0.05), 2: ((0, 0, 1), (0, -1, 0), (-1, 0, 0), 0.07, 0.05),
              3: ((1, 0, 0), (0, -1, 0), (0, 0, -1), 0.1, 0.07)}
    rg = np.array([0.3, -0.2, 0.1])
    for iplane in (1, -1, 2, -2, 3, -3):
        e1, e2, e3, a, b = frames[abs(iplane)]
        si = 1 if iplane > 0 else -1
        E1, E2, E3 = np.array(e1, float), np.array(e2, float), np.array(e3, float)
        if abs(iplane) == 1:
            E1, E3 = E1 * si, E3 * si
        else:
            E2, E3 = E2 * si, E3 * si
        for off in ((0.03, 0.02, 0.04), (0.0, 0.0, 0.01), (0.2, -0.1, 0.03), (0.05, 0.035, 1e-4),
                    (0.01, 0.01, -0.02), (0.09, 0.0, 0.0), (0.0, -0.06, 0.0)):
            xo = rg + off[0] * E1 + off[1] * E2 + off[2] * E3
            got = oracle.fsour_a4(xo, rg, iplane, d, a * b)
            val, _ = integrate.dblquad(lambda t, s: 1.0 / np.linalg.norm(xo - (rg + s * E1 + t * E2)),
                                       -a / 2, a / 2, -b / 2, b / 2, epsabs=1e-14, epsrel=1e-12)
            assert abs(got + val / (4 * np.pi)) <= 1e-12 * abs(val), (iplane, off)
        far = rg + 3.0 * E3
        assert oracle.fsour_a4(far, rg, iplane, d, a * b) == -(a * b / (4 * np.pi)) / 3.0


def test_constant_panel_boundary_values(oracle):
    """ibctyp = 3: the untreed panel sum (calc_boundinf_3d_s) is close to
    the point-source sum of ibctyp = 2 (the two differ only in the near
    field of each node); the tree walk of ibctyp = 3 (tree_calc_3d_s) runs
    with its start-cell source at the coarsest level, as written."""
    n, h = 25, 0.1
    L = (n - 1) * h / 2
    x = -L + h * np.arange(n)
    Z, Y, X = np.meshgrid(x, x, x, indexing="ij")
    blob = np.exp(-(X ** 2 + Y ** 2 + Z ** 2) / (0.2 * L * L))
    sol0 = [np.zeros_like(blob) for _ in range(3)]
    for c in range(3):
        oracle.dirichlet(-blob * (c + 1), sol0[c], (h, h, h), zero_bc=True)
    xb = (-L, -L, -L, L, L, L)
    face = np.zeros(blob.shape, bool)
    face[0] = face[-1] = True
    face[:, 0] = face[:, -1] = True
    face[:, :, 0] = face[:, :, -1] = True
    p2, n2 = oracle.boundary_values(sol0, xb, (h, h, h), 0, direct=True, ibctyp=2)
    p3, n3 = oracle.boundary_values(sol0, xb, (h, h, h), 0, direct=True, ibctyp=3)
    t3, nt = oracle.boundary_values(sol0, xb, (h, h, h), 3, ibctyp=3)
    assert n2 == n3 and nt < n3
    for c in range(3):
        assert 0 < rel_l2(p3[c][face], p2[c][face]) <= 3e-2
        assert np.all(np.isfinite(t3[c][face])) and np.all(t3[c][~face] == 0)


@pytest.mark.parametrize("nb,nc,ncell", [((2, 1, 1), 4, 32), ((1, 1, 2), 4, 32), ((2, 2, 2), 4, 32),
                                         ((3, 2, 1), 4, 48), ((3, 3, 3), 8, 48)])
def test_multiblock_seams_agree(oracle, nb, nc, ncell):
    """NBI x NBJ x NBK YAPS blocks (yaps3d.f90 with mapnodes_bl's neighbour
    transfers): every node that lies on the inner faces of several blocks
    (shared planes, edges, corners) gets the same boundary value from each
    of them, because the same terms reach it through the neighbours'
    transfers.  A wrong transfer shows as a seam of the size of the field."""
    from vpm_free_gb300 import workloads as W
    xp, qp, w = W.scaled_ring(ncell)
    cfg = oracle.make_config(dpm=w["dpm"], box=w["box"], nb=nb, ncoarse=nc)
    s = oracle.define_sizes(cfg, xp)
    oracle.step_fields(cfg, s, xp, qp, nthreads=4)
    assert oracle.lib().vpmo_yaps_seam() <= 1e-14


def test_multiblock_close_to_one_block(oracle):
    """The block decomposition changes the YAPS approximation, not the
    problem: psi of 2 x 2 x 2 blocks stays within the coarse-correction
    error (a few 1e-2 with ncoarse = 4 on 32^3) of the one-block psi."""
    from vpm_free_gb300 import workloads as W
    xp, qp, w = W.scaled_ring(32)
    out = []
    for nb in ((1, 1, 1), (2, 2, 2)):
        cfg = oracle.make_config(dpm=w["dpm"], box=w["box"], nb=nb, ncoarse=4)
        s = oracle.define_sizes(cfg, xp)
        up, _ = oracle.step_fields(cfg, s, xp, qp, nthreads=4)
        out.append((oracle.get_field(oracle.F_SOL).copy(), up))
    assert 1e-4 < rel_l2(out[1][0], out[0][0]) < 3e-2
    assert rel_l2(out[1][1], out[0][1]) < 3e-2


def test_sizes_known_answers(oracle):
    from vpm_free_gb300 import workloads as W
    for gen, nn, nnbl, nnc in ((W.ring64, 65, 81, 17), (W.leapfrog256, 257, 273, 41)):
        xp, qp, w = gen() if gen is W.ring64 else (np.zeros((1, 3)), None, W.LEAPFROG256)
        cfg = oracle.make_config(dpm=w["dpm"], box=w["box"])
        s = oracle.define_sizes(cfg, xp)
        assert list(s.nn) == [nn] * 3 and list(s.nnbl) == [nnbl] * 3 and list(s.nn_coarse) == [nnc] * 3
        assert list(s.nnbl_bl) == [9, 9, 9, nnbl - 8, nnbl - 8, nnbl - 8] and s.ilevmax == 3
    # shrink-wrap sizing (definepm itype 3): box = particle extent +- 4 cells,
    # padded so that cells divide by NBI*ncoarse, odd remainder on the min side
    xp = np.array([[0.0, 0.0, 0.0], [1.03, 0.5, 0.26]])
    cfg = oracle.make_config(dpm=(0.1, 0.1, 0.1))
    s = oracle.define_sizes(cfg, xp)
    for d in range(3):
        assert (s.nn[d] - 1) % 8 == 0
    # x: extent 1.03 + 0.8 -> 18.3 cells -> nint 18, pad 8 - 2 = 6 (3 each side)
    assert s.nn[0] == 25 and np.isclose(s.xbound[0], -0.4 - 0.3) and np.isclose(s.xbound[3], 1.43 + 0.3)
    # y: 13 cells, pad 8 - 5 = 3 (odd): 2 on the min side, 1 on the max side
    assert s.nn[1] == 17 and np.isclose(s.xbound[1], -0.4 - 0.2) and np.isclose(s.xbound[4], 0.9 + 0.1)


def test_projection_function_partition_of_unity(oracle):
    L = oracle.lib()
    for itype, lo, hi in ((4, -1, 3), (3, -1, 3), (2, 0, 2)):
        for x in np.linspace(0.0, 0.999, 37):
            s = sum(L.vpmo_projection_fun(itype, x - k) for k in range(lo, hi))
            assert abs(s - 1.0) < 1e-13, (itype, x)


def test_ring16_regression_fixture(oracle):
    g = np.load(os.path.join(GOLD, "ring16_oracle.npz"))
    from vpm_free_gb300 import workloads as W
    xp, qp, w = W.scaled_ring(16)
    assert np.array_equal(xp, g["xp"]) and np.array_equal(qp, g["qp"])
    cfg = oracle.make_config(dpm=w["dpm"], box=w["box"])
    s = oracle.define_sizes(cfg, xp)
    up, gp = oracle.step_fields(cfg, s, xp, qp, nthreads=2)
    assert rel_l2(up, g["up"]) <= 1e-12 and rel_l2(gp, g["gp"]) <= 1e-12


def test_remesh_threshold_is_single_precision_literal(oracle):
    """vpm_remesh.f90:184 compares with 1e-09 written as a default REAL."""
    from vpm_free_gb300 import workloads as W
    xp, qp, w = W.scaled_ring(16)
    cfg = oracle.make_config(dpm=w["dpm"], box=w["box"])
    s = oracle.define_sizes(cfg, xp)
    xr, qr = oracle.remesh(cfg, s, xp, qp)
    wm = np.linalg.norm(qr[:, :3], axis=1) / qr[:, 3]
    assert wm.min() >= np.float64(np.float32(1e-9)) * (1 - 1e-12)
    assert np.allclose(qr[:, 3], np.prod(w["dpm"]))
