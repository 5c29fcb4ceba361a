"""GPU Dirichlet and infinite-domain Poisson solves vs the oracle.

pmesh (source/pmlib.f90:69-192) is called through the C-ABI on random
right-hand sides; the oracle restates MKL's 7-point Dirichlet semantics
(source/pmsolve.f90:284-432) and the tree boundary values.
Tolerance: relative L2 <= 1e-10 (fields), as the spec parity bar.
"""
import os

import numpy as np
import pytest

from helpers import rel_l2

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("shape", [(17, 13, 11), (33, 33, 33), (41, 29, 35), (23, 59, 24)])
def test_dirichlet_matches_oracle(gpulib, oracle, shape):
    """(23, 59, 24): lines of 57 (N = 58 = 2 x 29) and 22 points (N = 23, odd
    extension of length 46 = 2 x 23), primes above the specialised radices."""
    V = gpulib
    rng = np.random.default_rng(11)
    nz, ny, nx = shape
    d = (0.07, 0.05, 0.09)
    rhs = [rng.standard_normal(shape) for _ in range(3)]
    sol = [rng.standard_normal(shape) for _ in range(3)]
    ref = [s.copy() for s in sol]
    for c in range(3):
        oracle.dirichlet(rhs[c], ref[c], d)
    cfg = V.VPMConfig.make(dpm=d, box=(0, 0, 0, 0.07 * 8, 0.05 * 8, 0.09 * 8))
    with V.VPM(cfg) as h:
        out = [s.copy() for s in sol]
        h.pmesh(out, rhs, (0.0, 0.0, 0.0, 1.0, 1.0, 1.0), d, iynbc=0, NN_bl=(1, 1, 1, nx, ny, nz))
    for c in range(3):
        assert rel_l2(out[c], ref[c]) <= 1e-12
        # boundary values untouched
        assert np.array_equal(out[c][0], sol[c][0]) and np.array_equal(out[c][:, :, -1], sol[c][:, :, -1])


@pytest.mark.parametrize("n,levmax", [(33, 2), (49, 3), (41, 3)])
def test_infinite_domain_matches_oracle(gpulib, oracle, n, levmax):
    V = gpulib
    rng = np.random.default_rng(5)
    h = 0.1
    L = (n - 1) * h / 2
    xb = (-L, -L, -L, L, L, L)
    x = -L + h * np.arange(n)
    Z, Y, X = np.meshgrid(x, x, x, indexing="ij")
    blob = np.exp(-(X ** 2 + Y ** 2 + Z ** 2) / (0.25 * L * L))
    rhs = [blob * rng.uniform(0.5, 1.5) + 0.01 * rng.standard_normal(blob.shape) * blob for _ in range(3)]
    ref = [np.zeros_like(blob) for _ in range(3)]
    oracle.pmesh(ref, rhs, xb, (h, h, h), iynbc=1, itree=1, levmax=levmax)
    cfg = V.VPMConfig.make(dpm=(h, h, h), box=(0, 0, 0, 0.8, 0.8, 0.8))
    with V.VPM(cfg) as hd:
        out = [np.zeros_like(blob) for _ in range(3)]
        hd.pmesh(out, rhs, xb, (h, h, h), iynbc=1, itree=1, levmax=levmax)
    for c in range(3):
        assert rel_l2(out[c], ref[c]) <= 1e-10, c


@pytest.mark.parametrize("n,levmax,itree,d", [(33, 2, 1, (0.1, 0.1, 0.1)), (37, 3, 1, (0.1, 0.08, 0.12)),
                                               (29, 0, 1, (0.1, 0.1, 0.1)), (21, 0, 0, (0.1, 0.09, 0.11))])
def test_constant_panel_boundary_matches_oracle(gpulib, oracle, n, levmax, itree, d):
    """ibctyp = 3 (constant-source panels, FSOUR_A4): the tree walk
    tree_calc_3d_s (37: dummy cells at level 3, anisotropic spacing;
    levmax 0: every cell at the coarsest level) and the untreed
    calc_boundinf_3d_s, through pmesh(iynbc = 1)."""
    V = gpulib
    rng = np.random.default_rng(9)
    xb = tuple(-(n - 1) * d[k] / 2 for k in range(3)) + tuple((n - 1) * d[k] / 2 for k in range(3))
    ax = [xb[k] + d[k] * np.arange(n) for k in range(3)]
    Z, Y, X = np.meshgrid(ax[2], ax[1], ax[0], indexing="ij")
    blob = np.exp(-(X ** 2 + Y ** 2 + Z ** 2) / (0.25 * xb[3] ** 2))
    rhs = [blob * rng.uniform(0.5, 1.5) + 0.01 * rng.standard_normal(blob.shape) * blob for _ in range(3)]
    ref = [np.zeros_like(blob) for _ in range(3)]
    oracle.pmesh(ref, rhs, xb, d, iynbc=1, itree=itree, levmax=levmax, ibctyp=3)
    cfg = V.VPMConfig.make(dpm=d, box=(0, 0, 0, 0.8, 0.8, 0.8), ibctyp=3)
    with V.VPM(cfg) as hd:
        out = [np.zeros_like(blob) for _ in range(3)]
        hd.pmesh(out, rhs, xb, d, iynbc=1, itree=itree, levmax=levmax)
    for c in range(3):
        assert rel_l2(out[c], ref[c]) <= 1e-10, c


def test_dst_tile_shape_does_not_change_results(gpulib):
    """The autotuned tile (line pairs per CTA) must not change a single bit:
    the same Dirichlet solve with each tile forced through VPMG_DST_PAIRS,
    in separate processes (the choice is read once per process).  Lines of
    18, 20, 34 and 40 points take the real-symmetric form (34 = 2 x 17),
    81 and 85 the odd extension."""
    import hashlib
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    code = (
        "import hashlib, numpy as np, vpm_free_gb300 as V\n"
        "rng = np.random.default_rng(5)\n"
        "for nz, ny, nx in ((23, 21, 19), (30, 41, 35), (20, 86, 82)):\n"
        "    R = [rng.normal(size=(nz, ny, nx)) for _ in range(3)]\n"
        "    S = [np.zeros_like(R[0]) for _ in range(3)]\n"
        "    S[0][0] = 1.0\n"
        f"    with V.VPM(V.VPMConfig.make(), arith='{gpulib.arith}') as h:\n"
        "        h.pmesh(S, R, [0, 0, 0, 1, 1, 1], [0.1, 0.11, 0.09], 0)\n"
        "    print(hashlib.sha256(b''.join(s.tobytes() for s in S)).hexdigest())\n")
    outs = []
    for pairs in ("2", "4", "8"):
        env = dict(os.environ, VPMG_DST_PAIRS=pairs)
        r = subprocess.run([sys.executable, "-c", code], cwd=root, env=env, capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stderr[-2000:]
        outs.append(r.stdout.split())
    assert outs[0] == outs[1] == outs[2] and len(outs[0]) == 3
