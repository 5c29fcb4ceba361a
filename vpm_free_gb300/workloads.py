"""Seeded synthetic vortex inputs (the reference ships no particle files).

Each generator returns particle arrays in the reference's layout, C-order
(nvr, 3) positions = Fortran XP(3,NVR) and (nvr, 4) strengths = QP(4,NVR),
with QP(1:3) = -omega * volume and QP(4) = volume (source/test.f90:34,
source/main_pm.f90:29-36), plus the pm.inp settings and explicit mesh box
of the workload.
"""
import numpy as np

RING64 = dict(name="ring64", box=(-1.6, -1.6, -1.6, 1.6, 1.6, 1.6), dpm=(0.05, 0.05, 0.05), steps=10, dt=0.01)
LEAPFROG256 = dict(name="leapfrog256", box=(-1.5, -1.5, -1.0, 1.5, 1.5, 2.5),
                   dpm=(3.0 / 256, 3.0 / 256, 3.5 / 256), steps=100, dt=0.005)
SCATTER384 = dict(name="scatter384", box=(-1.0 - 8 * 2.0 / 384, -1.0 - 8 * 2.0 / 384, -1.0 - 8 * 2.0 / 384,
                                          1.0 + 8 * 2.0 / 384, 1.0 + 8 * 2.0 / 384, 1.0 + 8 * 2.0 / 384),
                  dpm=(2.0 / 384,) * 3, steps=5, dt=0.002)


def _ring_particles(R, sigma, gamma, center, axis, h, keep, jitter=0.0, rng=None):
    """Lattice points of spacing h inside the torus tube radius <= keep, with a
    Gaussian core omega_theta = gamma/(pi sigma^2) exp(-rho^2/sigma^2)."""
    h = np.asarray(h, dtype=np.float64)
    axis = np.asarray(axis, dtype=np.float64)
    axis = axis / np.linalg.norm(axis)
    ext = R + keep
    # lattice in a local frame aligned with the axis
    tmp = np.array([1.0, 0.0, 0.0]) if abs(axis[0]) < 0.9 else np.array([0.0, 1.0, 0.0])
    e1 = np.cross(axis, tmp)
    e1 /= np.linalg.norm(e1)
    e2 = np.cross(axis, e1)
    if np.allclose(axis, [0, 0, 1]):
        e1, e2 = np.array([1.0, 0, 0]), np.array([0, 1.0, 0])
    nx = int(np.ceil(ext / h[0])) + 1
    ny = int(np.ceil(ext / h[1])) + 1
    nz = int(np.ceil(keep / h[2])) + 1
    a = (np.arange(-nx, nx + 1) + 0.5) * h[0]
    b = (np.arange(-ny, ny + 1) + 0.5) * h[1]
    c = (np.arange(-nz, nz + 1) + 0.5) * h[2]
    A, B, Cc = np.meshgrid(a, b, c, indexing="ij")
    A, B, Cc = A.ravel(), B.ravel(), Cc.ravel()
    if jitter > 0:
        A = A + rng.uniform(-jitter, jitter, A.shape) * h[0]
        B = B + rng.uniform(-jitter, jitter, B.shape) * h[1]
        Cc = Cc + rng.uniform(-jitter, jitter, Cc.shape) * h[2]
    rr = np.sqrt(A * A + B * B)
    rho = np.sqrt((rr - R) ** 2 + Cc * Cc)
    m = rho <= keep
    A, B, Cc, rr, rho = A[m], B[m], Cc[m], rr[m], rho[m]
    w = gamma / (np.pi * sigma * sigma) * np.exp(-(rho * rho) / (sigma * sigma))
    tx, ty = -B / rr, A / rr  # tangent in the local frame
    pos = (np.asarray(center)[None, :] + A[:, None] * e1[None, :] + B[:, None] * e2[None, :]
           + Cc[:, None] * axis[None, :])
    tang = tx[:, None] * e1[None, :] + ty[:, None] * e2[None, :]
    vol = float(np.prod(h))
    qp = np.empty((pos.shape[0], 4))
    qp[:, :3] = -(w[:, None] * tang) * vol
    qp[:, 3] = vol
    return np.ascontiguousarray(pos), qp


def ring64():
    """Single thick ring: R=1, sigma=0.1, circulation 1, axis z, lattice 0.05,
    tube radius <= 3.5 sigma (about 2e4 particles); 64^3 mesh on [-1.6,1.6]^3."""
    xp, qp = _ring_particles(1.0, 0.1, 1.0, (0.0, 0.0, 0.0), (0, 0, 1), (0.05,) * 3, 0.35)
    return xp, qp, RING64


def leapfrog256(seed=1234):
    """Two coaxial rings R=1 and R=0.7 at z=0 and z=0.5, sigma=0.08, circulation 1,
    lattice of the mesh spacing jittered by U(-0.25h, 0.25h); 256^3 mesh."""
    rng = np.random.default_rng(seed)
    h = LEAPFROG256["dpm"]
    x1, q1 = _ring_particles(1.0, 0.08, 1.0, (0.0, 0.0, 0.0), (0, 0, 1), h, 3.5 * 0.08, 0.25, rng)
    x2, q2 = _ring_particles(0.7, 0.08, 1.0, (0.0, 0.0, 0.5), (0, 0, 1), h, 3.5 * 0.08, 0.25, rng)
    return np.concatenate([x1, x2]), np.concatenate([q1, q2]), LEAPFROG256


def scatter384(n=8_000_000, seed=42):
    """n particles uniform in [-1,1]^3, strengths N(0, 1e-3), volume h^3; 384^3 mesh + 8-cell pad."""
    rng = np.random.default_rng(seed)
    h = SCATTER384["dpm"]
    xp = rng.uniform(-1.0, 1.0, (n, 3))
    qp = np.empty((n, 4))
    qp[:, :3] = rng.normal(0.0, 1e-3, (n, 3))
    qp[:, 3] = float(np.prod(h))
    return xp, qp, SCATTER384


def scatter_scaled(cells=96, seed=42):
    """The scatter stress case at a smaller mesh with the same particle
    density (8e6 particles on 384^3): uniform in [-1,1]^3, strengths
    N(0, 1e-3), volume h^3, cells^3 mesh plus the 8-cell pad, dt 0.002."""
    rng = np.random.default_rng(seed)
    h = 2.0 / cells
    n = int(round(8_000_000 * (cells / 384.0) ** 3))
    xp = rng.uniform(-1.0, 1.0, (n, 3))
    qp = np.empty((n, 4))
    qp[:, :3] = rng.normal(0.0, 1e-3, (n, 3))
    qp[:, 3] = h ** 3
    L = 1.0 + 8 * h
    return xp, qp, dict(name=f"scatter{cells}", box=(-L, -L, -L, L, L, L), dpm=(h, h, h), steps=5, dt=0.002)


def scaled_ring(n_cells, seed=7):
    """Small ring case on an n_cells^3 mesh (parity tests at oracle-friendly sizes)."""
    L = 1.6
    h = 2 * L / n_cells
    xp, qp = _ring_particles(1.0, 0.15, 1.0, (0.0, 0.0, 0.0), (0, 0, 1), (h,) * 3, 0.45)
    return xp, qp, dict(name=f"ring{n_cells}", box=(-L, -L, -L, L, L, L), dpm=(h, h, h), steps=2, dt=0.01)


BATCH_MESHES = (32, 48, 64, 96, 128)


def batched_rings(n=64, seed=2025):
    """Independent problems: one ring each, radius U(0.5,1.5), random unit
    axis, sigma = 0.1 R, circulation U(0.5,2), mesh edge drawn from
    {32,48,64,96,128} cells on a cube of half-width 2.5 R around the ring
    (room for about 20 steps of self-advection at the largest Gamma / R).
    Returns a list of (xp, qp, workload dict)."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        R = rng.uniform(0.5, 1.5)
        axis = rng.normal(size=3)
        axis /= np.linalg.norm(axis)
        gamma = rng.uniform(0.5, 2.0)
        cells = int(rng.choice(BATCH_MESHES))
        L = 2.5 * R
        h = 2 * L / cells
        xp, qp = _ring_particles(R, 0.1 * R, gamma, (0.0, 0.0, 0.0), axis, (h, h, h), 0.35 * R)
        out.append((xp, qp, dict(name=f"ring{cells}", box=(-L, -L, -L, L, L, L), dpm=(h, h, h), steps=20, dt=0.01)))
    return out


def two_level_128():
    """128^3 ring problem solved with ncoarse = 2: the fine block and a
    2x-coarser grid of the two-level YAPS coupling."""
    xp, qp, w = scaled_ring(128)
    w = dict(w, name="ring128_nc2", ncoarse=2)
    return xp, qp, w
