"""Whole-step parity (vpm WhatToDo = 2, Euler, remesh) vs the oracle.

Fields: relative L2 <= 1e-10 (vorticity/RHS, vector potential, velocity,
stretching); particles: relative L2 <= 1e-9 (positions, strengths).
"""
import numpy as np
import pytest

from helpers import configs_for, rel_l2

pytestmark = pytest.mark.gpu

FIELD_TOL = 1e-10
PART_TOL = 1e-9


def _pairs(V, O):
    return [("rhs", O.F_RHS), ("sol", O.F_SOL), ("vel", O.F_VEL), ("def", O.F_DEF)]


@pytest.mark.parametrize("ncell", [32, 48])
def test_step_fields_match_oracle(gpulib, oracle, ncell):
    from vpm_free_gb300 import workloads as W
    V, O = gpulib, oracle
    xp, qp, w = W.scaled_ring(ncell)
    ocfg, gcfg = configs_for(w)
    s = O.define_sizes(ocfg, xp)
    up_o, gp_o = O.step_fields(ocfg, s, xp, qp)
    with V.VPM(gcfg) as h:
        h.vpm(xp, qp, None, None, xp.shape[0], WhatToDo=0)
        up = np.zeros_like(up_o)
        gp = np.zeros_like(gp_o)
        h.vpm(np.ascontiguousarray(xp), np.ascontiguousarray(qp), up, gp, xp.shape[0], WhatToDo=2)
        for name, fid in _pairs(V, O):
            ref = O.get_field(fid)
            got = h.field(name).ravel()
            assert rel_l2(got, ref) <= FIELD_TOL, name
    assert rel_l2(up, up_o) <= PART_TOL
    assert rel_l2(gp, gp_o) <= PART_TOL


def test_ring64_ten_steps_match_oracle(gpulib, oracle):
    """The 64^3 single-ring case: remesh, then 10 x (step, Euler, remesh)."""
    from vpm_free_gb300 import workloads as W
    V, O = gpulib, oracle
    xp, qp, w = W.ring64()
    ocfg, gcfg = configs_for(w)
    s = O.define_sizes(ocfg, xp)
    xo, qo = O.remesh(ocfg, s, xp, qp)
    with V.VPM(gcfg) as h:
        h.define_sizes(xp)
        xg, qg = h.remesh_particles_3d(1, xp, qp)
        assert xg.shape == xo.shape
        h.set_particles(xg, qg)
        for step in range(w["steps"]):
            up, gp = O.step_fields(ocfg, s, xo, qo)
            O.euler(xo, qo, up, gp, w["dt"])
            xo, qo = O.remesh(ocfg, s, xo, qo)
            h.step(w["dt"])
            xg, qg = h.get_particles()
            assert xg.shape[0] == xo.shape[0], step
            assert rel_l2(xg, xo) <= PART_TOL, step
            assert rel_l2(qg, qo) <= PART_TOL, step


def test_deposition_deterministic(gpulib):
    from vpm_free_gb300 import workloads as W
    V = gpulib
    xp, qp, w = W.scaled_ring(32)
    _, gcfg = configs_for(w)
    with V.VPM(gcfg) as h:
        h.define_sizes(xp)
        a = h.project_particles_3D(xp, qp)
        perm = np.random.default_rng(3).permutation(xp.shape[0])
        b = h.project_particles_3D(xp[perm], qp[perm])
        c = h.project_particles_3D(xp, qp)
    for x, y in zip(a, c):
        assert np.array_equal(x, y)          # run to run: bitwise
    for x, y in zip(a, b):
        assert rel_l2(x, y) <= 1e-14         # input order only changes rounding


def test_deposition_matches_oracle(gpulib, oracle):
    from vpm_free_gb300 import workloads as W
    V, O = gpulib, oracle
    xp, qp, w = W.scaled_ring(48)
    ocfg, gcfg = configs_for(w)
    s = O.define_sizes(ocfg, xp)
    nx, ny, nz = list(s.nn)
    ref = [np.zeros(nx * ny * nz) for _ in range(3)]
    O.lib().vpmo_project_particles(s, 4, np.ascontiguousarray(xp), np.ascontiguousarray(qp), xp.shape[0], *ref, 0)
    with V.VPM(gcfg) as h:
        h.define_sizes(xp)
        got = h.project_particles_3D(xp, qp)
    for c in range(3):
        assert rel_l2(got[c], ref[c]) <= 1e-13


@pytest.mark.parametrize("ncell", [32, 64])
def test_partial_block_solves_equal_full_solves(gpulib, ncell):
    """The block solves evaluated only where the step reads them give the
    same step as solving the whole padded block (the reference's way)."""
    from vpm_free_gb300 import workloads as W
    V = gpulib
    xp, qp, w = W.scaled_ring(ncell)
    _, gcfg = configs_for(w)
    out = {}
    for mode in (0, 3):
        with V.VPM(gcfg) as h:
            h.set_profiling(mode)
            h.define_sizes(xp)
            up = np.zeros((xp.shape[0], 3))
            gp = np.zeros((xp.shape[0], 3))
            h.vpm(xp, qp, up, gp, xp.shape[0], WhatToDo=2)
            out[mode] = (up, gp, h.field("sol"), h.field("vel"), h.field("coarse_sol"))
    for a, b in zip(out[0], out[3]):
        assert rel_l2(a, b) <= 1e-12


def _ring_handle(V, ncell, **kw):
    from vpm_free_gb300 import workloads as W
    xp, qp, w = W.scaled_ring(ncell)
    _, gcfg = configs_for(w, **kw)
    h = V.VPM(gcfg)
    h.define_sizes(xp)
    xr, qr = h.remesh_particles_3d(1, xp, qp)
    h.set_particles(xr, qr)
    return h, w


def test_zero_particles(gpulib):
    """NVR = 0 on a sized handle: vpm(WhatToDo = 2) returns at once and
    leaves the resident fields as they were (vpm.f90:171, `if (NVR.eq.0)
    return`); remesh_particles_3d emits no particle.  No error either way."""
    V = gpulib
    h, _ = _ring_handle(V, 32)
    before = {name: h.field(name).copy() for name in ("rhs", "sol", "vel", "def")}
    xp, qp = np.zeros((0, 3)), np.zeros((0, 4))
    up, gp = np.zeros((0, 3)), np.zeros((0, 3))
    assert h.vpm(xp, qp, up, gp, 0, WhatToDo=2) == 0
    for name, f in before.items():
        assert np.array_equal(h.field(name), f), name
    x2, q2 = h.remesh_particles_3d(1, xp, qp)
    assert x2.shape[0] == 0 and q2.shape[0] == 0
    h.close()


def test_graph_replay_equals_uncaptured_steps(gpulib):
    """vpmg_run replays one captured step graph; it must reproduce the
    uncaptured vpmg_step loop bit for bit (deterministic kernels)."""
    V = gpulib
    a, w = _ring_handle(V, 48)
    b, _ = _ring_handle(V, 48)
    for _ in range(4):
        a.step(w["dt"])
    ms, ps = b.run(4, w["dt"])
    xa, qa = a.get_particles()
    xb, qb = b.get_particles()
    assert np.array_equal(xa, xb) and np.array_equal(qa, qb)
    assert ms > 0 and ps > 0
    a.close()
    b.close()


def test_batched_problems_equal_individual_runs(gpulib):
    V = gpulib
    sizes = (32, 48, 64)
    solo = []
    for n in sizes:
        h, w = _ring_handle(V, n)
        h.run(3, w["dt"])
        solo.append(h.get_particles())
        h.close()
    hs = [_ring_handle(V, n)[0] for n in sizes]
    ms, solves, ps = V.VPM.batch_run(hs, 3, 0.01)
    assert solves == 3 * len(sizes) and ms > 0 and ps > 0
    for h, (x0, q0) in zip(hs, solo):
        x1, q1 = h.get_particles()
        assert np.array_equal(x0, x1) and np.array_equal(q0, q1)
        h.close()


def _batch_problems(V, names):
    """Ring problems of the uneven batch (mesh edge 32..128 cells, the box
    scaled with the ring radius), remeshed and resident."""
    from vpm_free_gb300 import workloads as W
    probs = W.batched_rings(64)
    used = []
    for n in names:
        used.append([i for i, p in enumerate(probs) if p[2]["name"] == n and i not in used][0])
    out = []
    for xp, qp, w in (probs[i] for i in used):
        h = V.VPM(V.VPMConfig.make(dpm=w["dpm"], box=w["box"]))
        h.define_sizes(xp)
        xr, qr = h.remesh_particles_3d(1, xp, qp)
        h.set_particles(xr, qr)
        out.append((h, xr, qr, w))
    return out


def test_shared_operator_batch_equals_individual_runs(gpulib, monkeypatch):
    """Three 32^3 problems with different spacings share one recorded
    boundary operator (weights scaled by the spacing ratio, one apply for
    the group); a 48^3 problem runs its own graph.  Each must reproduce its
    individual run: the grouped ones to rounding (another summation order,
    scaled weights), the single one bit for bit.  The operators keep their
    dense coarsest level (VPMG_FARFIELD=0): FFT-evaluated ones are not
    grouped."""
    monkeypatch.setenv("VPMG_FARFIELD", "0")
    V = gpulib
    names = ["ring32", "ring32", "ring32", "ring48"]
    solo = []
    for h, _, _, w in _batch_problems(V, names):
        h.run(3, 0.01)
        solo.append(h.get_particles())
        h.close()
    hp = _batch_problems(V, names)
    hs = [t[0] for t in hp]
    assert len({t[3]["dpm"][0] for t in hp[:3]}) == 3  # three spacings
    with V.Batch(hs) as b:
        assert b.info() == (2, 3)
        ms, solves, ps = b.run(3, 0.01)
    assert solves == 12 and ms > 0 and ps > 0
    for i, (h, (x0, q0)) in enumerate(zip(hs, solo)):
        x1, q1 = h.get_particles()
        assert x1.shape == x0.shape
        if i == 3:
            assert np.array_equal(x0, x1) and np.array_equal(q0, q1)
        else:
            assert rel_l2(x1, x0) <= 1e-12 and rel_l2(q1, q0) <= 1e-11
        h.close()


@pytest.mark.parametrize("count", [6, 9])
def test_large_batch_groups_equal_individual_runs(gpulib, count, monkeypatch):
    """Groups of 6 and 9 problems: two and three problem quads per warp set
    in the dense-block kernel, 5 and 3 lane sets in the row kernel (2 and 5
    idle lanes); every member reproduces its individual run."""
    monkeypatch.setenv("VPMG_FARFIELD", "0")
    V = gpulib
    names = ["ring32"] * count
    solo = []
    for h, _, _, w in _batch_problems(V, names):
        h.run(2, 0.01)
        solo.append(h.get_particles())
        h.close()
    hp = _batch_problems(V, names)
    hs = [t[0] for t in hp]
    with V.Batch(hs, release_shared=True) as b:
        assert b.info() == (1, count)
        b.run(2, 0.01)
    for h, (x0, q0) in zip(hs, solo):
        x1, q1 = h.get_particles()
        assert x1.shape == x0.shape
        assert rel_l2(x1, x0) <= 1e-12 and rel_l2(q1, q0) <= 1e-11
        h.close()


def test_shared_operator_batch_fields_match_oracle(gpulib, oracle, monkeypatch):
    """One batched step of a two-problem group: the resident vector
    potential and velocity of each member against the oracle's step on the
    same particles.  The follower's own operator is released; afterwards it
    steps alone by walking the tree."""
    monkeypatch.setenv("VPMG_FARFIELD", "0")
    V, O = gpulib, oracle
    hp = _batch_problems(V, ["ring32", "ring32"])
    with V.Batch([t[0] for t in hp], release_shared=True) as b:
        assert b.info() == (1, 2)
        b.run(1, 0.01)
    assert hp[1][0].tree_stats()["precomputed"] is False
    for h, xr, qr, w in hp:
        ocfg, _ = configs_for(w)
        s = O.define_sizes(ocfg, xr)
        O.step_fields(ocfg, s, xr, qr)
        assert rel_l2(h.field("sol").ravel(), O.get_field(O.F_SOL)) <= FIELD_TOL
        assert rel_l2(h.field("vel").ravel(), O.get_field(O.F_VEL)) <= FIELD_TOL
    h = hp[1][0]
    h.set_particles(hp[1][1], hp[1][2])
    h.step(0.01)
    ocfg, _ = configs_for(hp[1][3])
    s = O.define_sizes(ocfg, hp[1][1])
    O.step_fields(ocfg, s, hp[1][1], hp[1][2])
    assert rel_l2(h.field("sol").ravel(), O.get_field(O.F_SOL)) <= FIELD_TOL
    for t in hp:
        t[0].close()


def test_two_level_ncoarse2_matches_oracle(gpulib, oracle):
    """YAPS with ncoarse = 2: the padded block (cells = 4 mod 8) has dummy
    quadtree cells at levels 2 and 3 (build_level_nbound_3d)."""
    from vpm_free_gb300 import workloads as W
    V, O = gpulib, oracle
    xp, qp, w = W.scaled_ring(32)  # padded block of 36 cells: 36 = 4 mod 8
    ocfg, gcfg = configs_for(w, ncoarse=2)
    s = O.define_sizes(ocfg, xp)
    assert (s.nnbl[0] - 1) % 8 != 0
    up_o, gp_o = O.step_fields(ocfg, s, xp, qp)
    with V.VPM(gcfg) as h:
        h.define_sizes(xp)
        up = np.zeros_like(up_o)
        gp = np.zeros_like(gp_o)
        h.vpm(xp, qp, up, gp, xp.shape[0], WhatToDo=2)
        for name, fid in (("sol", O.F_SOL), ("vel", O.F_VEL)):
            assert rel_l2(h.field(name).ravel(), O.get_field(fid)) <= FIELD_TOL, name
    assert rel_l2(up, up_o) <= PART_TOL and rel_l2(gp, gp_o) <= PART_TOL


@pytest.mark.parametrize("iyntree", [1, 0])
def test_constant_panel_step_matches_oracle(gpulib, oracle, iyntree):
    """A whole WhatToDo = 2 step with ibctyp = 3 on the fine block and the
    coarse YAPS grid, treed and untreed."""
    from vpm_free_gb300 import workloads as W
    V, O = gpulib, oracle
    xp, qp, w = W.scaled_ring(32)
    ocfg, gcfg = configs_for(w, ibctyp=3, iyntree=iyntree)
    s = O.define_sizes(ocfg, xp)
    up_o, gp_o = O.step_fields(ocfg, s, xp, qp)
    with V.VPM(gcfg) as h:
        h.define_sizes(xp)
        up = np.zeros_like(up_o)
        gp = np.zeros_like(gp_o)
        h.vpm(xp, qp, up, gp, xp.shape[0], WhatToDo=2)
        for name, fid in _pairs(V, O):
            assert rel_l2(h.field(name).ravel(), O.get_field(fid)) <= FIELD_TOL, name
    assert rel_l2(up, up_o) <= PART_TOL and rel_l2(gp, gp_o) <= PART_TOL


@pytest.mark.parametrize("nb,nc,ncell,extra", [((2, 1, 1), 8, 32, {}), ((2, 2, 2), 4, 32, {}),
                                               ((3, 2, 1), 4, 48, {}), ((2, 2, 1), 4, 32, {"ibctyp": 3}),
                                               ((1, 2, 2), 4, 32, {"iyntree": 0})])
def test_multiblock_step_matches_oracle(gpulib, oracle, nb, nc, ncell, extra):
    """YAPS on NBI x NBJ x NBK blocks of one GPU (rhsscat, per-block
    infinite-domain solves, neighbour transfers as gathers, solget) against
    the oracle's block-by-block restatement: every mesh field and the
    particle velocities and stretching of one WhatToDo = 2 step."""
    from vpm_free_gb300 import workloads as W
    V, O = gpulib, oracle
    xp, qp, w = W.scaled_ring(ncell)
    ocfg, gcfg = configs_for(w, nb=nb, ncoarse=nc, **extra)
    s = O.define_sizes(ocfg, xp)
    up_o, gp_o = O.step_fields(ocfg, s, xp, qp)
    with V.VPM(gcfg) as h:
        h.define_sizes(xp)
        up = np.zeros_like(up_o)
        gp = np.zeros_like(gp_o)
        h.vpm(xp, qp, up, gp, xp.shape[0], WhatToDo=2)
        for name, fid in _pairs(V, O):
            assert rel_l2(h.field(name).ravel(), O.get_field(fid)) <= FIELD_TOL, name
    assert rel_l2(up, up_o) <= PART_TOL and rel_l2(gp, gp_o) <= PART_TOL


def test_multiblock_steps_on_device_match_oracle(gpulib, oracle):
    """2 x 2 x 2 blocks through the device-resident loop (graph replay,
    Euler, remesh) for three steps against the oracle's steps."""
    from vpm_free_gb300 import workloads as W
    V, O = gpulib, oracle
    xp, qp, w = W.scaled_ring(32)
    ocfg, gcfg = configs_for(w, nb=(2, 2, 2), ncoarse=4)
    s = O.define_sizes(ocfg, xp)
    xo, qo = O.remesh(ocfg, s, xp, qp)
    with V.VPM(gcfg) as h:
        h.define_sizes(xp)
        xg, qg = h.remesh_particles_3d(1, xp, qp)
        h.set_particles(xg, qg)
        for step in range(3):
            up, gp = O.step_fields(ocfg, s, xo, qo)
            O.euler(xo, qo, up, gp, w["dt"])
            xo, qo = O.remesh(ocfg, s, xo, qo)
            h.step(w["dt"])
            xg, qg = h.get_particles()
            assert xg.shape[0] == xo.shape[0], step
            assert rel_l2(xg, xo) <= PART_TOL and rel_l2(qg, qo) <= PART_TOL, step


def test_viscous_diffusion_matches_oracle(gpulib, oracle):
    """vpm(WhatToDo = 5): deposition, diffuse_vort_3d and the GP gather of
    back_to_particles_3D(itype = 2) (source/vpm.f90:345-372)."""
    from vpm_free_gb300 import workloads as W
    V, O = gpulib, oracle
    xp, qp, w = W.scaled_ring(32)
    ocfg, gcfg = configs_for(w)
    s = O.define_sizes(ocfg, xp)
    ni = -0.1  # NI_in of source/test.f90:17
    gp_o = O.diffuse(ocfg, s, xp, qp, ni)
    with V.VPM(gcfg) as h:
        h.vpm(xp, qp, None, None, xp.shape[0], WhatToDo=0)
        up = np.full((xp.shape[0], 3), 7.0)
        gp = np.zeros((xp.shape[0], 3))
        h.vpm(np.ascontiguousarray(xp), np.ascontiguousarray(qp), up, gp, xp.shape[0], WhatToDo=5, NI=ni)
        assert np.all(up == 7.0)  # itype 2 leaves UP alone
        assert rel_l2(h.field("rhs").ravel(), O.get_field(O.F_RHS)) <= FIELD_TOL
        assert rel_l2(h.field("sol").ravel(), O.get_field(O.F_SOL)) <= FIELD_TOL
    assert rel_l2(gp, gp_o) <= PART_TOL
    assert np.abs(gp).max() > 0


def test_whattodo_1_and_4(gpulib):
    """WhatToDo 1 (solve + velocity field only) and 4 (stretching from the
    resident velocity, then UP/GP) reproduce the pieces of WhatToDo 2."""
    from vpm_free_gb300 import workloads as W
    V = gpulib
    xp, qp, w = W.scaled_ring(32)
    _, gcfg = configs_for(w)
    n = xp.shape[0]
    x, q = np.ascontiguousarray(xp), np.ascontiguousarray(qp)
    with V.VPM(gcfg) as h:
        h.vpm(xp, qp, None, None, n, WhatToDo=0)
        up2, gp2 = np.zeros((n, 3)), np.zeros((n, 3))
        h.vpm(x, q, up2, gp2, n, WhatToDo=2)
        vel2 = h.field("vel")
        up1, gp1 = np.full((n, 3), 3.0), np.full((n, 3), 3.0)
        h.vpm(x, q, up1, gp1, n, WhatToDo=1)
        assert np.array_equal(h.field("vel"), vel2)
        assert np.all(up1 == 3.0) and np.all(gp1 == 3.0)
        up4, gp4 = np.zeros((n, 3)), np.zeros((n, 3))
        h.vpm(x, q, up4, gp4, n, WhatToDo=4)
        assert np.array_equal(up4, up2) and np.array_equal(gp4, gp2)
        # new particles: GP from their own deposition and the kept velocity
        x2 = x + 0.3 * np.asarray(w["dpm"])
        h.vpm(np.ascontiguousarray(x2), q, up4, gp4, n, WhatToDo=4)
        assert np.array_equal(h.field("vel"), vel2)
        assert not np.array_equal(gp4, gp2)


def test_leapfrog256_step_matches_oracle(gpulib, oracle):
    """The headline configuration itself (two rings on the 256^3 mesh,
    ~2e6 particles): initial remesh, one field step on identical particles
    (every mesh field and UP/GP), then one full step (field step, Euler,
    remesh) against the oracle."""
    from vpm_free_gb300 import workloads as W
    V, O = gpulib, oracle
    xp, qp, w = W.leapfrog256()
    ocfg, gcfg = configs_for(w)
    s = O.define_sizes(ocfg, xp)
    xo, qo = O.remesh(ocfg, s, xp, qp)
    with V.VPM(gcfg) as h:
        h.define_sizes(xp)
        xg, qg = h.remesh_particles_3d(1, xp, qp)
        assert xg.shape == xo.shape
        assert rel_l2(xg, xo) <= PART_TOL and rel_l2(qg, qo) <= PART_TOL
        n = xo.shape[0]
        up_o, gp_o = O.step_fields(ocfg, s, xo, qo)
        up, gp = np.zeros((n, 3)), np.zeros((n, 3))
        h.vpm(np.ascontiguousarray(xo), np.ascontiguousarray(qo), up, gp, n, WhatToDo=2)
        for name, fid in _pairs(V, O):
            assert rel_l2(h.field(name).ravel(), O.get_field(fid)) <= FIELD_TOL, name
        assert rel_l2(up, up_o) <= PART_TOL and rel_l2(gp, gp_o) <= PART_TOL
        O.euler(xo, qo, up_o, gp_o, w["dt"])
        xo2, qo2 = O.remesh(ocfg, s, xo, qo)
        h.set_particles(xg, qg)
        h.step(w["dt"])
        xg2, qg2 = h.get_particles()
        assert xg2.shape[0] == xo2.shape[0]
        assert rel_l2(xg2, xo2) <= PART_TOL and rel_l2(qg2, qo2) <= PART_TOL


def test_scatter_stress_matches_oracle(gpulib, oracle):
    """The scatter stress configuration at 96^3 (+ the 8-cell pad), same
    particle density: uniform random particles with N(0, 1e-3) strengths,
    remesh then 3 full steps; counts equal, particles to 1e-9; and the
    sort-based deposition of the 125k unsorted particles is bitwise
    repeatable."""
    from vpm_free_gb300 import workloads as W
    V, O = gpulib, oracle
    xp, qp, w = W.scatter_scaled(96)
    ocfg, gcfg = configs_for(w)
    s = O.define_sizes(ocfg, xp)
    xo, qo = O.remesh(ocfg, s, xp, qp)
    with V.VPM(gcfg) as h:
        h.define_sizes(xp)
        a = h.project_particles_3D(xp, qp)
        b = h.project_particles_3D(xp, qp)
        for x, y in zip(a, b):
            assert np.array_equal(x, y)
        xg, qg = h.remesh_particles_3d(1, xp, qp)
        assert xg.shape == xo.shape
        assert rel_l2(xg, xo) <= PART_TOL and rel_l2(qg, qo) <= PART_TOL
        h.set_particles(xg, qg)
        for step in range(3):
            up, gp = O.step_fields(ocfg, s, xo, qo)
            O.euler(xo, qo, up, gp, w["dt"])
            xo, qo = O.remesh(ocfg, s, xo, qo)
            h.step(w["dt"])
            xg, qg = h.get_particles()
            assert xg.shape[0] == xo.shape[0], step
            assert rel_l2(xg, xo) <= PART_TOL and rel_l2(qg, qo) <= PART_TOL, step
