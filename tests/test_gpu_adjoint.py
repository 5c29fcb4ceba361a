"""Whole-step reverse mode: vpmg_apply_poisson / vpmg_adjoint_poisson /
vpmg_adjoint_loss / vpmg_adjoint_run and the torch.autograd bridge.

* the transposed vector-potential solve satisfies <L r, p> = <r, L^T p>
  to rounding (single-level and two-level YAPS, quadtree with dummy cells);
* the gradient of a 10-step loss (64^3 ring, 1024 probes in a shell around
  the ring plus a kinetic-energy term) matches central differences of the
  GPU forward and of the oracle's forward (h = 1e-6, 64 random directions
  each);
* the GPU loss equals the oracle's loss on the same particles.
"""
import itertools

import numpy as np
import pytest

from helpers import configs_for, rel_l2

pytestmark = pytest.mark.gpu

FD_H = 1e-6
FD_TOL = 1e-6     # relative L2 over the probed directional derivatives
DOT_TOL = 1e-12   # |<Lr,p> - <r,L^T p>| / (|Lr| |p|)
KE = 0.1


def _m4(t):
    a = np.abs(t)
    return np.where(a > 2.0, 0.0, np.where(a >= 1.0, 0.5 * (2.0 - a) ** 2 * (1.0 - a), 1.0 - 2.5 * a * a + 1.5 * a ** 3))


def interp_m4(field, xmin, d, pts):
    """M4' interpolation of a (3, NZ, NY, NX) node field at points (n, 3)."""
    xmin, d = np.asarray(xmin, dtype=np.float64), np.asarray(d, dtype=np.float64)
    c = np.floor((pts - xmin) / d).astype(np.int64)
    out = np.zeros((pts.shape[0], 3))
    for a, b, e in itertools.product(range(4), repeat=3):
        ix, iy, iz = c[:, 0] - 1 + a, c[:, 1] - 1 + b, c[:, 2] - 1 + e
        w = (_m4((pts[:, 0] - xmin[0] - ix * d[0]) / d[0]) * _m4((pts[:, 1] - xmin[1] - iy * d[1]) / d[1])
             * _m4((pts[:, 2] - xmin[2] - iz * d[2]) / d[2]))
        out += w[:, None] * field[:, iz, iy, ix].T
    return out


def shell_probes(n, r0, r1, seed=11):
    rng = np.random.default_rng(seed)
    v = rng.normal(size=(n, 3))
    v /= np.linalg.norm(v, axis=1)[:, None]
    return v * rng.uniform(r0, r1, size=n)[:, None]


def field_loss(vel, xmin, d, probes, ke):
    up = interp_m4(vel, xmin, d, probes)
    return float(np.sum(up * up) + ke * 0.5 * np.prod(d) * np.sum(vel * vel))


def _ring64_state(V, jitter=True):
    """Remeshed 64^3 ring particles.  With jitter, each coordinate moves off
    its node by 0.25-0.75 of a cell: at a node the M4' weights have
    second-derivative jumps, which central differences resolve only to
    O(h) (about 1e-5 here); off the nodes they are O(h^2)."""
    from vpm_free_gb300 import workloads as W
    xp, qp, w = W.ring64()
    _, gcfg = configs_for(w)
    h = V.VPM(gcfg)
    h.define_sizes(xp)
    x0, q0 = h.remesh_particles_3d(1, xp, qp)
    if jitter:
        rng = np.random.default_rng(21)
        x0 = x0 + np.asarray(w["dpm"]) * rng.uniform(0.25, 0.75, size=x0.shape) * rng.choice([-1.0, 1.0], size=x0.shape)
    return h, x0, q0, w


def _directions(x0, q0, n, seed=5):
    rng = np.random.default_rng(seed)
    qs = np.sqrt(np.mean(q0[:, :3] ** 2))
    out = []
    for _ in range(n):
        dq = np.zeros_like(q0)
        dq[:, :3] = rng.normal(size=(q0.shape[0], 3)) * qs
        out.append((rng.normal(size=x0.shape), dq))
    return out


@pytest.mark.parametrize("case", ["ring32", "ring64", "ring32_nc2", "ring32_panels"])
def test_poisson_transpose_identity(gpulib, case):
    from vpm_free_gb300 import workloads as W
    V = gpulib
    if case == "ring32":
        xp, qp, w = W.scaled_ring(32)
        _, gcfg = configs_for(w)
    elif case == "ring64":
        xp, qp, w = W.ring64()
        _, gcfg = configs_for(w)
    elif case == "ring32_panels":  # ibctyp = 3: constant-source panel boundary
        xp, qp, w = W.scaled_ring(32)
        _, gcfg = configs_for(w, ibctyp=3)
    else:  # ncoarse = 2: dummy quadtree cells on the padded block
        xp, qp, w = W.scaled_ring(32)
        _, gcfg = configs_for(w, ncoarse=2)
    rng = np.random.default_rng(3)
    with V.VPM(gcfg) as h:
        h.define_sizes(xp)
        shp = h._mesh_shape()
        for _ in range(2):
            r = rng.normal(size=shp)
            p = rng.normal(size=shp)
            Lr = h.apply_poisson(r)
            LTp = h.adjoint_poisson(p)
            lhs, rhs = float(np.vdot(Lr, p)), float(np.vdot(r, LTp))
            scale = np.linalg.norm(Lr) * np.linalg.norm(p)
            assert abs(lhs - rhs) <= DOT_TOL * scale, (lhs, rhs, scale)
            # linearity of the transpose
            p2 = rng.normal(size=shp)
            assert rel_l2(h.adjoint_poisson(p + 2.0 * p2), LTp + 2.0 * h.adjoint_poisson(p2)) <= 1e-12


def _dirs_mixed(x0, q0, seed, relative_q=False):
    """Position-only, strength-only and mixed directions.  relative_q scales
    each particle's strength direction by its own |q| instead of the rms."""
    out = []
    qs = np.sqrt(np.mean(q0[:, :3] ** 2))
    for i, (dx, dq) in enumerate(_directions(x0, q0, 6, seed=seed)):
        if relative_q:
            dq[:, :3] *= np.abs(q0[:, :3]) / qs
        if i % 3 == 0:
            dq = np.zeros_like(dq)
        elif i % 3 == 1:
            dx = np.zeros_like(dx)
        out.append((dx, dq))
    return out


def test_fields_vjp_matches_central_differences(gpulib):
    """VJP of vpm(WhatToDo = 2): (XP, QP) -> (UP, GP)."""
    V = gpulib
    h, x0, q0, w = _ring64_state(V)
    rng = np.random.default_rng(8)
    n = x0.shape[0]
    upbar, gpbar = rng.normal(size=(n, 3)), rng.normal(size=(n, 3)) * 1e3
    with h:
        xb, qb = h.vjp_fields(x0, q0, upbar, gpbar)

        def F(x, q):
            up, gp = np.zeros((n, 3)), np.zeros((n, 3))
            h.vpm(np.ascontiguousarray(x), np.ascontiguousarray(q), up, gp, n, WhatToDo=2)
            return float(np.sum(upbar * up) + np.sum(gpbar * gp))
        g_adj, g_fd = [], []
        for dx, dq in _dirs_mixed(x0, q0, 31):
            g_fd.append((F(x0 + FD_H * dx, q0 + FD_H * dq) - F(x0 - FD_H * dx, q0 - FD_H * dq)) / (2 * FD_H))
            g_adj.append(float(np.sum(xb * dx) + np.sum(qb * dq[:, :3])))
        assert rel_l2(g_adj, g_fd) <= FD_TOL, (g_adj, g_fd)


def _smooth_field(x):
    return np.stack([np.sin(2.0 * x[:, 0] + x[:, 1]), np.cos(3.0 * x[:, 1] - x[:, 2]),
                     np.sin(x[:, 0] * x[:, 2] + 1.0)], axis=1)


def test_remesh_vjp_matches_central_differences(gpulib):
    """VJP of remesh_particles_3d(1), |w| cut held fixed.  The probed
    functional J = sum_s f(X''_s) . Q''_s weighs each emitted particle by a
    smooth field of its node, so a node crossing the 1e-9 cut under the
    perturbation changes J by O(1e-9 DV) only; strength directions are
    relative to each particle's |q|, so the many particles of the outer
    shell (|q| ~ 1e-13) do not push hundreds of nodes across the cut."""
    V = gpulib
    h, x0, q0, w = _ring64_state(V)
    with h:
        xr, qr = h.remesh_particles_3d(1, x0, q0)
        xb, qb = h.vjp_remesh(x0, q0, _smooth_field(xr))
        with pytest.raises(V.VPMError):
            h.vjp_remesh(x0, q0, _smooth_field(xr)[:-1])

        def J(x, q):
            xn, qn = h.remesh_particles_3d(1, x, q)
            return float(np.sum(_smooth_field(xn) * qn[:, :3]))
        g_adj, g_fd = [], []
        for dx, dq in _dirs_mixed(x0, q0, 32, relative_q=True):
            g_fd.append((J(x0 + FD_H * dx, q0 + FD_H * dq) - J(x0 - FD_H * dx, q0 - FD_H * dq)) / (2 * FD_H))
            g_adj.append(float(np.sum(xb * dx) + np.sum(qb * dq[:, :3])))
        assert rel_l2(g_adj, g_fd) <= FD_TOL, (g_adj, g_fd)


def test_adjoint_gradient_matches_gpu_central_differences(gpulib):
    V = gpulib
    h, x0, q0, w = _ring64_state(V)
    probes = shell_probes(1024, 1.2, 1.4)
    nsteps, dt = w["steps"], w["dt"]
    with h:
        h.set_particles(x0, q0)
        loss, xbar, qbar, ms_f, ms_b = h.adjoint_run(nsteps, dt, probes, KE)
        assert np.isfinite(loss) and loss > 0
        # the particles are left as they were
        x1, q1 = h.get_particles()
        assert np.array_equal(x1, x0) and np.array_equal(q1, q0)
        # the device-resident particles are those given
        assert x1.shape == x0.shape
        # the loss-only entry point agrees bitwise with the gradient run, with
        # the reference's remesh cut and with the masks that run recorded
        assert h.adjoint_loss(nsteps, dt, probes, KE) == loss
        assert h.adjoint_loss(nsteps, dt, probes, KE, mask_mode=2) == loss
        # central differences of the fixed-mask map (the reference's cut
        # flips nodes with |w| ~ 1e-9 under a 1e-6 perturbation: each flip
        # moves the loss by ~1e-10, i.e. ~1e-4 in a difference quotient)
        g_adj, g_fd = [], []
        for dx, dq in _directions(x0, q0, 64):
            h.set_particles(x0 + FD_H * dx, q0 + FD_H * dq)
            lp = h.adjoint_loss(nsteps, dt, probes, KE, mask_mode=2)
            h.set_particles(x0 - FD_H * dx, q0 - FD_H * dq)
            lm = h.adjoint_loss(nsteps, dt, probes, KE, mask_mode=2)
            g_fd.append((lp - lm) / (2 * FD_H))
            g_adj.append(float(np.sum(xbar * dx) + np.sum(qbar * dq[:, :3])))
        g_adj, g_fd = np.array(g_adj), np.array(g_fd)
        assert rel_l2(g_adj, g_fd) <= FD_TOL, (g_adj[:4], g_fd[:4])


_ORACLE_FD = {}  # the oracle's difference quotients, shared by both arithmetics' runs


def _oracle_steps_loss(O, ocfg, s, x, q, masks, mode, nsteps, dt, probes, nthreads=0):
    """The oracle's loss after nsteps steps; mode 1: the reference's remesh
    cut, recording the masks; 2: replaying them."""
    nn = list(s.nn)
    x, q = x.copy(), q.copy()
    for k in range(nsteps):
        up, gp = O.step_fields(ocfg, s, x, q, nthreads=nthreads)
        O.euler(x, q, up, gp, dt)
        x, q = O.remesh_masked(ocfg, s, x, q, masks[k], mode, nthreads=nthreads)
    O.step_fields(ocfg, s, x, q, nthreads=nthreads)
    vel = O.get_field(O.F_VEL).reshape(3, nn[2], nn[1], nn[0])
    return field_loss(vel, list(s.xbound)[:3], list(s.dpm), probes, KE)


def _oracle_fd_worker(job):
    """Central differences of the oracle's loss along some directions, in a
    spawned process that loads the oracle itself."""
    x0, q0, dirs, masks, nsteps, dt, probes, nthreads = job
    from oracle import oracle as O
    from vpm_free_gb300 import workloads as W
    xp, _, w = W.ring64()
    ocfg, _ = configs_for(w)
    s = O.define_sizes(ocfg, xp)
    out = []
    for dx, dq in dirs:
        lp = _oracle_steps_loss(O, ocfg, s, x0 + FD_H * dx, q0 + FD_H * dq, masks, 2, nsteps, dt, probes, nthreads)
        lm = _oracle_steps_loss(O, ocfg, s, x0 - FD_H * dx, q0 - FD_H * dq, masks, 2, nsteps, dt, probes, nthreads)
        out.append((lp - lm) / (2 * FD_H))
    return out


def test_adjoint_gradient_matches_oracle_central_differences(gpulib, oracle):
    """The GPU gradient of the 10-step loss against central differences of
    the oracle's forward (the C++ restatement of the reference's step) on
    64 random directions: 128 oracle runs of 10 steps, computed once per
    process, spread over a few spawned processes."""
    import multiprocessing as mp
    import os
    V, O = gpulib, oracle
    from vpm_free_gb300 import workloads as W
    xp, qp, w = W.ring64()
    ocfg, _ = configs_for(w)
    s = O.define_sizes(ocfg, xp)
    h, x0, q0, _ = _ring64_state(V)
    probes = shell_probes(1024, 1.2, 1.4)
    nsteps, dt = w["steps"], w["dt"]
    masks = [np.zeros(int(np.prod(list(s.nn))), dtype=np.int32) for _ in range(nsteps)]
    dirs = _directions(x0, q0, 64, seed=9)
    with h:
        h.set_particles(x0, q0)
        loss, xbar, qbar, _, _ = h.adjoint_run(nsteps, dt, probes, KE)
        assert abs(loss - _oracle_steps_loss(O, ocfg, s, x0, q0, masks, 1, nsteps, dt, probes)) <= 1e-10 * abs(loss)
        if "fd" not in _ORACLE_FD:
            nproc = max(1, min(4, (os.cpu_count() or 1) // 4))
            threads = max(1, (os.cpu_count() or 1) // nproc)
            jobs = [(x0, q0, dirs[i::nproc], masks, nsteps, dt, probes, threads) for i in range(nproc)]
            with mp.get_context("spawn").Pool(nproc) as pool:
                parts = pool.map(_oracle_fd_worker, jobs)
            g = np.empty(len(dirs))
            for i, part in enumerate(parts):
                g[i::nproc] = part
            _ORACLE_FD["fd"] = g
        g_fd = _ORACLE_FD["fd"]
        g_adj = np.array([float(np.sum(xbar * dx) + np.sum(qbar * dq[:, :3])) for dx, dq in dirs])
        assert rel_l2(g_adj, g_fd) <= FD_TOL, (g_adj[:4], g_fd[:4])


def test_torch_autograd_bridge(gpulib):
    torch = pytest.importorskip("torch")
    from vpm_free_gb300.autograd import StepLoss
    V = gpulib
    h, x0, q0, w = _ring64_state(V)
    probes = shell_probes(128, 1.2, 1.4, seed=4)
    with h:
        h.set_particles(x0, q0)
        loss_ref, xbar, qbar, _, _ = h.adjoint_run(2, w["dt"], probes, KE)
        xt = torch.tensor(x0, requires_grad=True)
        qt = torch.tensor(q0, requires_grad=True)
        loss = StepLoss.apply(xt, qt, h, 2, w["dt"], probes, KE)
        (3.0 * loss).backward()
        assert float(loss.detach()) == loss_ref
        # the two gradient runs differ only in the order of atomic additions
        assert rel_l2(xt.grad.numpy(), 3.0 * xbar) <= 1e-10
        assert rel_l2(qt.grad.numpy()[:, :3], 3.0 * qbar) <= 1e-10
        assert np.all(qt.grad.numpy()[:, 3] == 0.0)
