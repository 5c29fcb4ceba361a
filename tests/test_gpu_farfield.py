"""The coarsest tree level of the boundary operator by FFT convolutions
(csrc/farfield.cu) against the recorded dense block it replaces and the
oracle's tree walk (source/pmbound.f90:980-1249).

In FP64 handles whose coarsest cells form a uniform lattice on every face,
the library sums every coarsest cell by FFTs (2-D between parallel faces,
1-D along the shared axis between perpendicular ones) and subtracts the
cells each node opened.  VPMG_FARFIELD=0 at set-up keeps the dense block.
The two must agree to rounding (1e-13), and both with the oracle to the
field tolerance.  Float-float handles keep the dense block.
"""
import numpy as np
import pytest

from helpers import configs_for, rel_l2

pytestmark = pytest.mark.gpu

SAME = 1e-13
FIELD_TOL = 1e-10


def _solve(V, arith, shape, d, levmax, seed):
    """vpmg_pmesh(iynbc = 1, tree) of seeded random RHS on a box of shape (nz, ny, nx)."""
    rng = np.random.default_rng(seed)
    rhs = [rng.standard_normal(shape) for _ in range(3)]
    sol = [np.zeros(shape) for _ in range(3)]
    nz, ny, nx = shape
    xb = (0.0, 0.0, 0.0, (nx - 1) * d[0], (ny - 1) * d[1], (nz - 1) * d[2])
    with V.VPM(V.VPMConfig.make(dpm=d), arith=arith) as h:
        h.pmesh(sol, rhs, xb, d, iynbc=1, itree=1, levmax=levmax)
    return rhs, sol, xb


# (nz, ny, nx), spacings, levmax: cubic, anisotropic with three different
# sides (lengths 96 / 64 / 108 transforms, radix 3 included), and two
# levels; all face sides multiples of 2^levmax panels
CASES = [((33, 33, 33), (0.05, 0.05, 0.05), 3),
         ((57, 33, 41), (0.03, 0.04, 0.025), 3),
         ((29, 37, 25), (0.06, 0.05, 0.07), 2)]


@pytest.mark.parametrize("case", range(len(CASES)))
def test_fft_far_field_equals_dense_block_and_oracle(gpulib, oracle, monkeypatch, case):
    V, O = gpulib, oracle
    shape, d, levmax = CASES[case]
    monkeypatch.delenv("VPMG_FARFIELD", raising=False)
    rhs, fast, xb = _solve(V, gpulib.arith, shape, d, levmax, 11 + case)
    monkeypatch.setenv("VPMG_FARFIELD", "0")
    _, dense, _ = _solve(V, gpulib.arith, shape, d, levmax, 11 + case)
    for c in range(3):
        assert rel_l2(fast[c], dense[c]) <= SAME, (c, rel_l2(fast[c], dense[c]))
    ref = [np.zeros(shape) for _ in range(3)]
    O.pmesh(ref, rhs, xb, d, iynbc=1, itree=1, levmax=levmax)
    for c in range(3):
        assert rel_l2(fast[c], ref[c]) <= FIELD_TOL, c


def test_fft_far_field_in_the_step(gpulib, oracle, monkeypatch):
    """A whole field step of the 64^3 ring (81^3 padded block, coarsest
    cells 8 x 8 panels): on in FP64, off in float-float; every mesh field
    equal to the dense block's to rounding and to the oracle's to 1e-10."""
    from vpm_free_gb300 import workloads as W
    V, O = gpulib, oracle
    xp, qp, w = W.ring64()
    ocfg, gcfg = configs_for(w)
    s = O.define_sizes(ocfg, xp)
    O.step_fields(ocfg, s, xp, qp)
    names = ("rhs", "sol", "vel", "def")
    ref = {nm: O.get_field(fid) for nm, fid in zip(names, (O.F_RHS, O.F_SOL, O.F_VEL, O.F_DEF))}
    out = {}
    for ff in ("on", "off"):
        if ff == "on":
            monkeypatch.delenv("VPMG_FARFIELD", raising=False)
        else:
            monkeypatch.setenv("VPMG_FARFIELD", "0")
        n = xp.shape[0]
        with V.VPM(gcfg) as h:
            h.vpm(xp, qp, None, None, n, WhatToDo=0)
            up, gp = np.zeros((n, 3)), np.zeros((n, 3))
            h.vpm(np.ascontiguousarray(xp), np.ascontiguousarray(qp), up, gp, n, WhatToDo=2)
            st = h.farfield_stats()
            out[ff] = {nm: h.field(nm).ravel() for nm in names}
            out[ff]["up"], out[ff]["gp"] = up, gp
        if ff == "on":
            assert st["on"] == (gpulib.arith == "fp64")
            if st["on"]:
                assert st["corrections"] > 0 and st["flops"] > 0
        else:
            assert not st["on"]
    for nm in names:
        assert rel_l2(out["on"][nm], out["off"][nm]) <= 1e-12, nm
        assert rel_l2(out["on"][nm], ref[nm]) <= FIELD_TOL, nm
    assert rel_l2(out["on"]["up"], out["off"]["up"]) <= 1e-12
    assert rel_l2(out["on"]["gp"], out["off"]["gp"]) <= 1e-12


def test_fft_far_field_declines_irregular_lattices(gpulib, oracle, monkeypatch):
    """A face side that is not a multiple of 2^levmax panels puts dummy cells
    at the coarsest level: the dense block stays, results still match."""
    V, O = gpulib, oracle
    monkeypatch.delenv("VPMG_FARFIELD", raising=False)
    shape, d, levmax = (27, 35, 30), (0.05, 0.04, 0.06), 3
    rhs, fast, xb = _solve(V, gpulib.arith, shape, d, levmax, 5)
    ref = [np.zeros(shape) for _ in range(3)]
    O.pmesh(ref, rhs, xb, d, iynbc=1, itree=1, levmax=levmax)
    for c in range(3):
        assert rel_l2(fast[c], ref[c]) <= FIELD_TOL, c


def test_fft_operators_are_not_grouped(gpulib, monkeypatch):
    """Problems whose coarsest level goes by FFT keep their own operators in
    a batch (the group apply would use the dense block); with the dense
    block (float-float, or VPMG_FARFIELD=0) the two ring32 problems share
    one."""
    from vpm_free_gb300 import workloads as W
    V = gpulib
    probs = [p for p in W.batched_rings(64) if p[2]["name"] == "ring32"][:2]

    def handles():
        out = []
        for xp, qp, w in probs:
            h = V.VPM(V.VPMConfig.make(dpm=w["dpm"], box=w["box"]))
            h.define_sizes(xp)
            xr, qr = h.remesh_particles_3d(1, xp, qp)
            h.set_particles(xr, qr)
            out.append(h)
        return out
    monkeypatch.delenv("VPMG_FARFIELD", raising=False)
    hs = handles()
    fft = hs[0].farfield_stats()["on"]
    assert fft == (gpulib.arith == "fp64")
    with V.Batch(hs) as b:
        assert b.info() == ((2, 0) if fft else (1, 2))
        b.run(1, 0.01)
    for h in hs:
        h.close()
    monkeypatch.setenv("VPMG_FARFIELD", "0")
    hs = handles()
    assert not hs[0].farfield_stats()["on"]
    with V.Batch(hs) as b:
        assert b.info() == (1, 2)
    for h in hs:
        h.close()
