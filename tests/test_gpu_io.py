"""The reference's solution and line files (writesol, writeline:
source/vpm.f90:662-709, 789-833) written from the GPU fields, through the
direct calls and through vpm(WhatToDo = 2) with the pm.inp windows."""
import os
import struct

import numpy as np
import pytest

from helpers import configs_for, fortran_records, rel_l2

pytestmark = pytest.mark.gpu


def _solution(path):
    recs = fortran_records(path)
    head = recs[0].decode()
    zone = recs[1]
    ni, nj, nk = struct.unpack_from("<i", zone, 7)[0], struct.unpack_from("<i", zone, 14)[0], \
        struct.unpack_from("<i", zone, 21)[0]
    rows = np.array([struct.unpack("<9d", r) for r in recs[2:]])
    return head, zone, (ni, nj, nk), rows


def test_solution_file_matches_fields_and_oracle(gpulib, oracle, tmp_path):
    from vpm_free_gb300 import workloads as W
    V, O = gpulib, oracle
    xp, qp, w = W.scaled_ring(32)
    ocfg, gcfg = configs_for(w)
    s = O.define_sizes(ocfg, xp)
    O.step_fields(ocfg, s, xp, qp)
    with V.VPM(gcfg) as h:
        h.vpm(xp, qp, None, None, xp.shape[0], WhatToDo=0)
        up, gp = np.zeros((xp.shape[0], 3)), np.zeros((xp.shape[0], 3))
        h.vpm(np.ascontiguousarray(xp), np.ascontiguousarray(qp), up, gp, xp.shape[0], WhatToDo=2, NTIME=7)
        h.write_solution(7, str(tmp_path))
        sz = h.sizes()
        vel, rhs = h.field("vel"), h.field("rhs")
    head, zone, (ni, nj, nk), rows = _solution(str(tmp_path / "00007solution.bin"))
    assert head == 'VARIABLES = "X" "Y" "Z" "U" "V" "W" "VORTX" "VORTY" "VORTZ"'
    assert zone[:7] == b"ZONE I=" and zone[11:14] == b" J=" and zone[18:21] == b" K=" and zone[25:] == b" F=POINT"
    nb = list(sz.nn_bl)
    assert (ni, nj, nk) == (nb[3] - nb[0] + 1, nb[4] - nb[1] + 1, nb[5] - nb[2] + 1)
    assert rows.shape == (ni * nj * nk, 9)
    # node order k, j, i (i fastest), coordinates XMIN + (I-1) DX
    i = np.arange(nb[0], nb[3] + 1)
    j = np.arange(nb[1], nb[4] + 1)
    k = np.arange(nb[2], nb[5] + 1)
    K, J, I = np.meshgrid(k, j, i, indexing="ij")
    xb, d = list(sz.xbound), list(sz.dpm)
    assert np.array_equal(rows[:, 0], (xb[0] + (I - 1) * d[0]).ravel())
    assert np.array_equal(rows[:, 2], (xb[2] + (K - 1) * d[2]).ravel())
    sel = (slice(None), K - 1, J - 1, I - 1)
    for c in range(3):
        assert np.array_equal(rows[:, 3 + c], vel[c][K - 1, J - 1, I - 1].ravel())
        assert np.array_equal(rows[:, 6 + c], -rhs[c][K - 1, J - 1, I - 1].ravel())
    nn = list(s.nn)
    ov = O.get_field(O.F_VEL).reshape(3, nn[2], nn[1], nn[0])[sel].reshape(3, -1).T
    orr = O.get_field(O.F_RHS).reshape(3, nn[2], nn[1], nn[0])[sel].reshape(3, -1).T
    assert rel_l2(rows[:, 3:6], ov) <= 1e-10
    assert rel_l2(rows[:, 6:9], -orr) <= 1e-10


def test_vpm_writers_follow_pm_inp_windows(gpulib, tmp_path):
    from vpm_free_gb300 import workloads as W
    V = gpulib
    xp, qp, w = W.scaled_ring(32)
    _, gcfg = configs_for(w)
    gcfg.ipmwrite = 2
    gcfg.ipmwstart[0], gcfg.ipmwsteps[0] = 2, 0   # NTIME 2
    gcfg.ipmwstart[1], gcfg.ipmwsteps[1] = 4, 1   # NTIME 4, 5
    with V.VPM(gcfg) as h:
        h.set_output(str(tmp_path), solution=True, hist=True)
        h.vpm(xp, qp, None, None, xp.shape[0], WhatToDo=0)
        lines = []
        for nt in range(1, 7):
            up, gp = np.zeros((xp.shape[0], 3)), np.zeros((xp.shape[0], 3))
            h.vpm(np.ascontiguousarray(xp), np.ascontiguousarray(qp), up, gp, xp.shape[0], WhatToDo=2, NTIME=nt)
            vel = h.field("vel")
            lines.append(vel)
        sz = h.sizes()
    got = sorted(f for f in os.listdir(tmp_path) if f.endswith("solution.bin"))
    assert got == ["00002solution.bin", "00004solution.bin", "00005solution.bin"]
    nb = list(sz.nn_bl)
    NNJ, NNK = nb[4] - nb[1] + 1, nb[5] - nb[2] + 1
    fj = [0.5, 0.25, 0.25, 0.75, 0.75, 0.5, 0.5, 0.25, 0.75]
    fk = [0.5, 0.25, 0.75, 0.25, 0.75, 0.25, 0.75, 0.5, 0.5]
    for l in range(9):
        recs = fortran_records(str(tmp_path / ("%02dhist.bin" % (l + 1))))
        assert len(recs) == 3 + 6  # header (NTIME = 1) + one record per field step
        assert struct.unpack("<3d", recs[0]) == tuple(list(sz.xbound)[:3])
        assert struct.unpack("<3d", recs[1]) == tuple(list(sz.dpm))
        i0, i1, j, k = struct.unpack("<4i", recs[2])
        assert (i0, i1) == (nb[0], nb[3])
        assert j == int(np.float32(fj[l]) * np.float32(NNJ)) and k == int(np.float32(fk[l]) * np.float32(NNK))
        nl = i1 - i0 + 1
        for t, r in enumerate(recs[3:]):
            (nt,) = struct.unpack_from("<i", r, 0)
            vals = np.frombuffer(r[4:], dtype="<f8").reshape(3, nl)
            assert nt == t + 1
            assert np.array_equal(vals, lines[t][:, k - 1, j - 1, i0 - 1:i1])
