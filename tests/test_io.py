"""The reference's particle file (particles.bin, source/test.f90:24-37) and
the pm.inp write windows, through the C-ABI, on CPU (no GPU needed)."""
import os
import struct

import numpy as np
import pytest

from helpers import fortran_records

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden")


def test_read_particles_bin_fixture(gpulib):
    """The fixture was written with struct, independently of the library."""
    xp, qp, vref = gpulib.read_particles_bin(os.path.join(GOLD, "particles_ring16.bin"))
    recs = fortran_records(os.path.join(GOLD, "particles_ring16.bin"))
    (n,) = struct.unpack("<i", recs[0])
    (v,) = struct.unpack("<d", recs[1])
    rows = np.array([struct.unpack("<6d", r) for r in recs[2:]])
    assert xp.shape == (n, 3) and qp.shape == (n, 4) and vref == v
    assert np.array_equal(xp, rows[:, :3])
    assert np.array_equal(qp[:, :3], -rows[:, 3:] * v)  # QPR(1:3) = -QPR(1:3)*Vref
    assert np.all(qp[:, 3] == v)                         # QPR(neq+1) = Vref
    # the fixture holds the 16^3 ring of the workloads
    from vpm_free_gb300 import workloads as W
    x16, q16, _ = W.scaled_ring(16)
    assert np.array_equal(xp, x16)
    assert np.allclose(qp, q16, rtol=1e-15, atol=0)


def test_particles_bin_round_trip(gpulib, tmp_path):
    rng = np.random.default_rng(4)
    xp = rng.normal(size=(257, 3))
    qp = np.empty((257, 4))
    qp[:, :3] = rng.normal(size=(257, 3))
    vref = 0.125  # a power of two: -(-q / v) * v == q exactly
    qp[:, 3] = vref
    p = str(tmp_path / "particles.bin")
    gpulib.write_particles_bin(p, xp, qp, vref)
    x2, q2, v2 = gpulib.read_particles_bin(p)
    assert v2 == vref and np.array_equal(x2, xp) and np.array_equal(q2, qp)
    # empty file of zero particles
    gpulib.write_particles_bin(p, xp[:0], qp[:0], vref)
    x3, q3, v3 = gpulib.read_particles_bin(p)
    assert x3.shape == (0, 3) and v3 == vref


def test_particles_bin_errors(gpulib, tmp_path):
    V = gpulib
    with pytest.raises(V.VPMError):
        V.read_particles_bin(str(tmp_path / "missing.bin"))
    p = tmp_path / "trunc.bin"
    good = open(os.path.join(GOLD, "particles_ring16.bin"), "rb").read()
    p.write_bytes(good[:len(good) - 20])  # last record cut
    with pytest.raises(V.VPMError):
        V.read_particles_bin(str(p))
    p.write_bytes(good[:6])  # broken first record
    with pytest.raises(V.VPMError):
        V.read_particles_bin(str(p))


def test_pm_inp_write_windows(gpulib):
    cfg = gpulib.read_pm_inp(os.path.join(GOLD, "pm.inp"))
    assert cfg.ipmwrite == 7
    assert list(cfg.ipmwstart)[:7] == [100, 180, 360, 760, 1120, 3600, 7200]
    assert list(cfg.ipmwsteps)[:7] == [1] * 7
