"""World-size-2 gloo test of bench.py's multi-rank bookkeeping (replicas:
barrier, max of per-rank time, sum of per-rank particle-steps)."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, ws, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(ws), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    import bench
    d = bench.Dist(ws, rank, rank, "gloo")
    d.barrier()
    t = d.reduce(10.0 + rank, "max")
    ps = d.reduce(1000 * (rank + 1), "sum")
    out.put((rank, t, ps))
    d.close()


def test_two_rank_reductions():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res == [(0, 11.0, 3000.0), (1, 11.0, 3000.0)]


def test_clock_parser(tmp_path):
    import bench
    c = bench.Clocks(0)
    c.path = str(tmp_path / "c.csv")
    with open(c.path, "w") as f:
        f.write("0, 1965, 2070, 900.1, 0x0, Not Active, Not Active, Not Active, Active\n")
        f.write("0, 2070, 2070, 950.3, 0x0, Not Active, Not Active, Not Active, Not Active\n")

    class P:
        def terminate(self):
            pass

        def wait(self, timeout=None):
            return 0
    c.proc = P()
    c.fh = open(os.devnull, "w")
    r = c.stop()
    assert r["sm_mhz"] == 2017.5 and r["sm_max_mhz"] == 2070 and r["reasons"] == ["sw_power_cap"]
