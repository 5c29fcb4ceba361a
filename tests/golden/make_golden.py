"""Generates the committed golden fixtures of tests/golden/.

hill_vortex.npz: velocity and vorticity of Hill's spherical vortex
(radius a = 1, us = -1) at seeded points, from the closed-form solution
that the reference implements in source/test_applic.f90:2-77
(fUi_HillsVortex_1); the restatement is ``hill`` below.

ring16_oracle.npz: one oracle field step on a 16^3 ring case (regression
snapshot of the checker itself: particle velocities, stretching and field
norms).

particles_ring16.bin: the 16^3 ring particles in the particles.bin format
that source/test.f90:24-33 reads (Fortran sequential unformatted: NVR as a
4-byte integer, Vref, then one record X Y Z w1 w2 w3 per particle), written
here with ``struct`` -- independently of the library -- with Vref = the
particle volume and w = -QP(1:3) / Vref.

Regenerate with ``python tests/golden/make_golden.py``.
"""
import struct
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def hill(X, Y, Z, a=1.0, us=-1.0):
    """Hill's vortex: returns (u, omega) as (3, ...) arrays."""
    rho = np.sqrt(X ** 2 + Y ** 2)
    r3 = np.sqrt(X ** 2 + Y ** 2 + Z ** 2)
    small = rho / a < 1e-12
    with np.errstate(divide="ignore", invalid="ignore"):
        ephx = np.where(small, 0.0, -Y / rho)
        ephy = np.where(small, 0.0, X / rho)
        erx = np.where(small, 0.0, X / rho)
        ery = np.where(small, 0.0, Y / rho)
        q = (a ** 2 / (Z ** 2 + rho ** 2)) ** 2.5
        inside = r3 < a
        uz = np.where(inside, 3 / 5 * us * (1 - (2 * rho ** 2 + Z ** 2) / a ** 2) + us * 2 / 5,
                      2 / 5 * us * q * (2 * Z ** 2 - rho ** 2) / (2 * a ** 2))
        ur = np.where(inside, 3 / 5 * us * rho * Z / a ** 2, 3 / 5 * us * rho * Z / a ** 2 * q)
    om = np.where(inside, 3 * us * rho / a ** 2, 0.0)
    return np.stack([ur * erx, ur * ery, uz]), np.stack([om * ephx, om * ephy, 0 * om])


def fortran_records(path, records):
    """Sequential unformatted records, each framed by its 4-byte length."""
    with open(path, "wb") as f:
        for r in records:
            f.write(struct.pack("<i", len(r)) + r + struct.pack("<i", len(r)))


def particles_bin(path, xp, w, vref):
    recs = [struct.pack("<i", xp.shape[0]), struct.pack("<d", vref)]
    recs += [struct.pack("<6d", *xp[i], *w[i]) for i in range(xp.shape[0])]
    fortran_records(path, recs)


def main():
    rng = np.random.default_rng(31)
    pts = rng.uniform(-1.6, 1.6, (256, 3))
    u, w = hill(pts[:, 0], pts[:, 1], pts[:, 2])
    np.savez(os.path.join(HERE, "hill_vortex.npz"), points=pts, u=u, omega=w)
    from oracle import oracle as O
    from vpm_free_gb300 import workloads as W
    xp, qp, wk = W.scaled_ring(16)
    vref = float(qp[0, 3])
    particles_bin(os.path.join(HERE, "particles_ring16.bin"), xp, -qp[:, :3] / vref, vref)
    cfg = O.make_config(dpm=wk["dpm"], box=wk["box"])
    s = O.define_sizes(cfg, xp)
    up, gp = O.step_fields(cfg, s, xp, qp, nthreads=1)
    norms = {k: np.linalg.norm(O.get_field(f)) for k, f in
             (("rhs", O.F_RHS), ("sol", O.F_SOL), ("vel", O.F_VEL), ("def", O.F_DEF))}
    np.savez(os.path.join(HERE, "ring16_oracle.npz"), xp=xp, qp=qp, up=up, gp=gp,
             norms=np.array([norms["rhs"], norms["sol"], norms["vel"], norms["def"]]))


if __name__ == "__main__":
    main()
