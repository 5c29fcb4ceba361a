#!/usr/bin/env python
"""Particle-steps/s of vpm_free's particle-mesh time step, FP64, on GB300.

Workload: two coaxial leapfrogging vortex rings (R = 1 and 0.7, 0.5 apart,
sigma = 0.08, circulation 1, seeded jittered lattice) on a 256^3 mesh over
[-1.5,1.5]^2 x [-1,2.5], M4' projection, infinite-domain quadtree
boundary values, one YAPS block (ncoarse = 8, 3 tree levels), remesh every
step, dt = 0.005.  One step = field step (vpm WhatToDo = 2) + forward Euler
+ remesh_particles_3d(1), as source/test.f90:83-150.  Unit of work: a
particle-step = particles at the start of a step x 1 step.

  value : device-resident steps timed with CUDA events on the library's
          stream (vpmg_run), inputs resident in HBM, every kernel in IEEE
          FP64 (--arith fp64, the default and the reference's arithmetic).
  ff48  : the same loop with the heavy kernels in float-float (about 48
          significant bits), reported beside the FP64 figures, never as the
          headline.
  e2e   : the same loop through the reference-facing C-ABI calls with host
          arrays (vpm(...,2,...), host Euler, vpm(...,0,...),
          remesh_particles_3d(1)), host<->device copies inside, host clock.
  --impl reference : the oracle (C++ restatement of the reference's CPU
          path; the Fortran/MPI/MKL original cannot be built on this
          hardware) on all host cores.

Multi-GPU: the path runs one YAPS block per GPU; N GPUs run N independent
replicas (torchrun, one process per GPU); value = total particle-steps /
max time over ranks.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s at 256^3 FP64"
UNIT = "particle-steps/s"


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Dist:
    """Barrier and max/sum reductions across ranks (torch.distributed when N > 1)."""

    def __init__(self, ws, rank, local, backend):
        self.ws, self.rank = ws, rank
        self.td = None
        if ws > 1:
            import torch
            import torch.distributed as td
            if backend == "nccl":
                torch.cuda.set_device(local)
            td.init_process_group(backend=backend)
            self.td, self.torch = td, torch
            self.dev = torch.device("cuda", local) if backend == "nccl" else torch.device("cpu")

    def barrier(self):
        if self.td:
            self.td.barrier()

    def reduce(self, v, op):
        if not self.td:
            return v
        t = self.torch.tensor([float(v)], dtype=self.torch.float64, device=self.dev)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX if op == "max" else self.td.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.td:
            self.td.destroy_process_group()


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during a region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.fh,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        if not self.proc:
            return out
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                p = [x.strip() for x in line.split(",")]
                if len(p) < 9:
                    continue
                try:
                    sm.append(float(p[1]))
                    mx.append(float(p[2]))
                except ValueError:
                    continue
                for n, v in zip(names, p[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(n)
        os.unlink(self.path)
        if sm:
            out = {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                   "samples": len(sm)}
        return out


WORKLOADS = {"leapfrog256": "leapfrog256", "ring64": "ring64", "ring128": "ring128", "dirichlet273": "dirichlet273"}


def _workload(name="leapfrog256"):
    """Headline workload (leapfrog256); ring64 / ring128 are the small cases
    used for profiler captures."""
    from vpm_free_gb300 import workloads as W
    if name == "ring64":
        return W.ring64()
    if name == "ring128":
        return W.scaled_ring(128)
    return W.leapfrog256()


def workload_config(name, nn, nnbl, blocks):
    """The `config` object both arms print: the workload and its sizes
    (define_sizes' mesh and padded block), nothing about how it runs."""
    desc = ("leapfrog256 (two coaxial rings, 256^3 mesh, M4', tree levels 3, ncoarse 8, remesh every step, "
            "dt 0.005)") if name == "leapfrog256" else name
    field_mb = float(np.prod(nn)) * 8 / 1e6
    return {"workload": desc, "mesh": [int(n) - 1 for n in nn], "block": [int(n) for n in nnbl],
            "yaps_blocks": [int(b) for b in blocks],
            "l2": f"inputs larger than L2 (each field component {field_mb:.0f} MB, and the recorded boundary operator)"}


def _measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except Exception:
        return {}


def _traffic_table():
    """Per-launch DRAM bytes of the profiled kernels (summaries of ncu captures)."""
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            return json.load(f)
    except Exception:
        return {}


def cpu_step_sample(xp, qp, w, steps, threads):
    """The oracle's step (field step + Euler + remesh) on `steps` steps of the
    workload; returns (particle-steps/s, seconds, particle-steps)."""
    from oracle import oracle as O
    O.build()
    cfg = O.make_config(dpm=w["dpm"], box=w["box"], ompthreads=threads)
    s = O.define_sizes(cfg, xp)
    xr, qr = O.remesh(cfg, s, xp, qp, nthreads=threads)
    ps = 0
    t0 = time.perf_counter()
    for _ in range(steps):
        ps += xr.shape[0]
        up, gp = O.step_fields(cfg, s, xr, qr, nthreads=threads)
        O.euler(xr, qr, up, gp, w["dt"])
        xr, qr = O.remesh(cfg, s, xr, qr, nthreads=threads)
    t = time.perf_counter() - t0
    return ps / t, t, ps


def run_batched(args, local):
    """Batched solves/s: 64 independent ring problems on meshes drawn from
    {32,48,64,96,128}^3 plus the 128^3 two-level (ncoarse = 2) case,
    advanced together (problems of one mesh edge share one recorded
    boundary operator and one apply per step; each group and each other
    problem is one captured graph, replayed concurrently), against looping
    the plain path (one problem after the other, vpmg_step with its host
    sync per step)."""
    import vpm_free_gb300 as V
    from vpm_free_gb300 import workloads as W
    probs = W.batched_rings(64)
    xp2, qp2, w2 = W.two_level_128()
    probs.append((xp2, qp2, w2))
    hs, init = [], []
    t0 = time.perf_counter()
    for xp, qp, w in probs:
        cfg = V.VPMConfig.make(dpm=w["dpm"], box=w["box"], ncoarse=w.get("ncoarse", 8))
        h = V.VPM(cfg, device=local)
        h.set_operator_budget(args.batch_operator_budget)
        h.define_sizes(xp)
        xr, qr = h.remesh_particles_3d(1, xp, qp)
        init.append((xr, qr))
        hs.append(h)
    setup_s = time.perf_counter() - t0
    dt = 0.01
    k = max(1, args.batch_steps)

    def reset():  # every phase starts from the same remeshed particles
        for h, (xr, qr) in zip(hs, init):
            h.set_particles(xr, qr)
    reset()
    V.VPM.batch_run(hs, 1, dt)                       # warm-up, captures the graphs
    reset()
    ms_c, solves_c, _ = V.VPM.batch_run(hs, k, dt)   # one graph per problem, concurrent
    t0 = time.perf_counter()
    batch = V.Batch(hs)                              # groups problems that share an operator
    group_s = time.perf_counter() - t0
    units, shared, corr_rows = batch.details()
    reset()
    batch.run(2, dt)                                 # warm-up: captures the group graphs, tunes the schedule
    sched, sched_ms = batch.schedule()
    reset()
    ms_b, solves, ps_b = batch.run(k, dt)
    batch.close()
    reset()
    for h in hs:                                     # plain loop: problem after problem
        h.step(dt)
    reset()
    t1 = time.perf_counter()
    for h in hs:
        for _ in range(k):
            h.step(dt)
    loop_s = time.perf_counter() - t1
    reset()
    t2 = time.perf_counter()
    for h in hs:                                     # looped graph replays, one problem at a time
        h.run(k, dt)
    graph_loop_s = time.perf_counter() - t2
    # the loop of a drop-in host (source/test.f90:83-150) over the problems:
    # per problem and step vpm(WhatToDo = 2) with host arrays, host Euler,
    # remesh_particles_3d(1) -- copies in and out inside the calls
    t3 = time.perf_counter()
    for h, (xr, qr) in zip(hs, init):
        XP, QP = xr.copy(), qr.copy()
        for it in range(k):
            n = XP.shape[0]
            UP, GP = np.zeros((n, 3)), np.zeros((n, 3))
            h.vpm(XP, QP, UP, GP, n, WhatToDo=2, NTIME=it + 1)
            np.multiply(UP, dt, out=UP)
            XP += UP
            np.multiply(GP, dt, out=GP)
            QP[:, :3] -= GP
            XP, QP = h.remesh_particles_3d(1, XP, QP)
    ref_loop_s = time.perf_counter() - t3
    precomputed = sum(1 for h in hs if h.tree_stats()["precomputed"])
    for h in hs:
        h.close()
    return {"problems": len(hs), "steps": k, "solves_per_s": solves / (ms_b * 1e-3),
            "particle_steps_per_s": ps_b / (ms_b * 1e-3), "ms": ms_b,
            "loop_plain_solves_per_s": len(hs) * k / loop_s, "loop_graph_solves_per_s": len(hs) * k / graph_loop_s,
            "loop_reference_calls_solves_per_s": len(hs) * k / ref_loop_s,
            "speedup_vs_plain_loop": (solves / (ms_b * 1e-3)) / (len(hs) * k / loop_s),
            "speedup_vs_reference_call_loop": (solves / (ms_b * 1e-3)) / (len(hs) * k / ref_loop_s),
            "graphs_per_step": units, "problems_sharing_an_operator": shared, "grouping_s": group_s,
            "corrected_rows": corr_rows,
            "schedule": {"chosen": ["concurrent", "in sequence"][sched], "tuning_step_ms": sched_ms},
            "concurrent_graphs_solves_per_s": solves_c / (ms_c * 1e-3),
            "batched": "vpmg_batch_step: problems with the same index geometry share one recorded boundary "
                       "operator (one apply per group and step); each group and each other problem is one graph, "
                       "replayed concurrently",
            "concurrent_graphs": "vpmg_batch_run: one graph per problem, replayed concurrently",
            "loops": {"plain": "vpmg_step per problem and step (device-resident particles, host sync per step)",
                      "graph": "vpmg_run per problem (one captured step graph, problems one after another)",
                      "reference_calls": "vpm(WhatToDo=2) + host Euler + remesh_particles_3d per problem and step, "
                                         "host arrays (what a drop-in Fortran host runs)"},
            "setup_s": setup_s, "precomputed_operators": precomputed,
            "timing": "batched: CUDA events over all streams; loops: host clock (each step synchronous)"}


def run_batch_group(args, local):
    """One shared-operator group of the batched workload: the problems of
    one mesh class (`--batch-group ring64` or `ring64:8` for the first 8),
    their followers' own operators released, `--steps` batched steps.  A
    small profiling case for k_apply_group; prints one JSON line."""
    import vpm_free_gb300 as V
    from vpm_free_gb300 import workloads as W
    from vpm_free_gb300 import build as B
    B.build()
    name, _, cnt = args.batch_group.partition(":")
    probs = [p for p in W.batched_rings(64) if p[2]["name"] == name]
    if cnt:
        probs = probs[:int(cnt)]
    if not probs:
        raise SystemExit(f"no problem of class {name!r} in the batched workload")
    hs = []
    try:
        for xp, qp, w in probs:
            h = V.VPM(V.VPMConfig.make(dpm=w["dpm"], box=w["box"]), device=local, arith=args.arith)
            hs.append(h)
            h.define_sizes(xp)
            xr, qr = h.remesh_particles_3d(1, xp, qp)
            h.set_particles(xr, qr)
        with V.Batch(hs, release_shared=True) as b:
            b.set_schedule(0)
            ms, solves, ps = b.run(max(1, args.steps), 0.01)
            units, shared, rows = b.details()
    finally:
        for h in hs:
            h.close()
    print(json.dumps({"workload": f"batch group {name} x {len(probs)}", "arith": args.arith, "steps": max(1, args.steps),
                      "ms": ms,
                      "solves_per_s": solves / (ms * 1e-3), "graphs_per_step": units,
                      "problems_sharing_an_operator": shared, "corrected_rows": rows}))
    return 0


def run_adjoint(args, local, reps=3):
    """Adjoint:forward time ratio on the 64^3 ring: 10 steps (dt 0.01) and a
    loss on 1024 probes in the shell 1.2 <= r <= 1.4 plus 0.1 x the mesh
    kinetic energy; gradient with respect to every particle position and
    strength (checkpointed forward, recomputed step by step backward)."""
    import vpm_free_gb300 as V
    from vpm_free_gb300 import workloads as W
    xp, qp, w = W.ring64()
    cfg = V.VPMConfig.make(dpm=w["dpm"], box=w["box"])
    rng = np.random.default_rng(11)
    v = rng.normal(size=(1024, 3))
    probes = v / np.linalg.norm(v, axis=1)[:, None] * rng.uniform(1.2, 1.4, size=1024)[:, None]
    with V.VPM(cfg, device=local) as h:
        h.define_sizes(xp)
        xr, qr = h.remesh_particles_3d(1, xp, qp)
        h.set_particles(xr, qr)
        h.adjoint_run(w["steps"], w["dt"], probes, 0.1)       # warm-up (allocations, graph capture)
        fw, bw = [], []
        for _ in range(reps):
            loss, xbar, qbar, f, b = h.adjoint_run(w["steps"], w["dt"], probes, 0.1)
            fw.append(f)
            bw.append(b)
        h.run(1, w["dt"])                                      # plain forward of the same steps
        h.set_particles(xr, qr)
        plain = []
        for _ in range(reps):
            ms, _ = h.run(w["steps"], w["dt"])
            plain.append(ms)
            h.set_particles(xr, qr)
    f, b, p = float(np.median(fw)), float(np.median(bw)), float(np.median(plain))
    return {"workload": "ring64 (64^3, 10 steps, dt 0.01, 1024 probes, ke 0.1)", "particles": int(xr.shape[0]),
            "ms_forward": f, "ms_backward": b, "ratio": b / f, "ms_plain_forward": p, "ratio_vs_plain": b / p,
            "loss": loss, "timing": "CUDA events on the library stream, median of %d" % reps,
            "forward": "checkpointed steps (step graph) + final field + loss",
            "backward": "per step: recompute + remesh/Euler/M2P/stretching/curl/Poisson/deposition transposes"}


def run_reference(args, dist):
    if dist.rank != 0:
        return 0
    threads = os.cpu_count() or 1
    xp, qp, w = _workload()
    warm = min(args.warmup, 1)
    steps = max(1, min(args.steps, 3))
    if warm:
        cpu_step_sample(xp, qp, w, warm, threads)
    v, t, ps = cpu_step_sample(xp, qp, w, steps, threads)
    from oracle import oracle as O
    sz = O.define_sizes(O.make_config(dpm=w["dpm"], box=w["box"], ompthreads=threads), xp)
    sample = (f"{steps} full steps (field step + Euler + remesh) of the 256^3 leapfrog workload after {warm} warm-up "
              f"step(s); oracle = C++ restatement of the reference's CPU path (Fortran/MPI/MKL original not buildable)")
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": steps,
        "warmup": warm, "ms_per_step": 1e3 * t / steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded leapfrogging rings)",
        "config": workload_config("leapfrog256", list(sz.nn), list(sz.nnbl), (1, 1, 1)),
        "parallelism": "host threads",
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_dirichlet(args, local):
    """Profiling case for the DST solver alone: pmesh(iynbc = 0), three
    component Dirichlet solves on a 273^3 box (the padded block of the
    headline mesh; interior 271^3, so each line is a 272-point DST-I),
    about 1.3 GB on the device.  Prints ms per 3-component solve."""
    import vpm_free_gb300 as V
    n = args.dirichlet_nodes
    rng = np.random.default_rng(0)
    R = [rng.normal(size=(n, n, n)) for _ in range(3)]
    S = [np.zeros((n, n, n)) for _ in range(3)]
    with V.VPM(V.VPMConfig.make(), device=local, arith=args.arith) as h:
        t = []
        for _ in range(max(1, args.steps)):
            t0 = time.perf_counter()
            h.pmesh(S, R, [0.0, 0.0, 0.0, 1.0, 1.0, 1.0], [1.0 / (n - 1)] * 3, 0)
            t.append(time.perf_counter() - t0)
    print(json.dumps({"workload": f"dirichlet{n}", "arith": args.arith,
                      "unit": "s per pmesh(iynbc=0) call, host clock incl. copies",
                      "s": t}))
    return 0


KERNELS = (  # vpmg_bench_kernel ids: (id, name, launches per step); the first word keys profiles/traffic.json
    (0, "boundary (the fine block's operator: coarsest level by FFT k_ff_* or the dense block k_apply_dense, "
        "finer levels and corrections k_apply_csr)", 1),
    (1, "inner-box Dirichlet solve (k_dst_x_fwd, k_dst_y x2, k_thomas, k_dst_x_inv)", 3),
    (6, "padded-block zero-BC solve where read (k_dst_x_fwd, k_dst_y, k_thomas_faces, k_partial_x/y, "
        "partial inverses)", 3),
    (2, "k_deposit (M4' gather deposition; field step and remesh)", 2),
    (5, "k_m2p (mesh-to-particle gather + Euler)", 1),
    (4, "k_deformation (stretching)", 1),
    (3, "k_velocity (curl)", 1),
    (7, "k_remesh_flags + scan", 1),
    (8, "k_records64 + sort by cell (k_keys, scan, k_scatter, k_cell_order)", 2),
)


def kernel_rooflines(h, fp64_tflops, hbm_gbs, traffic):
    """Per-kernel figures replayed on the resident state: the algorithmic
    FP64 flops (FMA = 2) and HBM bytes per launch against the measured FP64
    peak and HBM bandwidth; the bound is the resource whose time at peak is
    longer, and frac = that time / the measured time."""
    out = []
    for which, name, per_step in KERNELS:
        try:
            kms, fl, by = h.bench_kernel(which, reps=3)
        except Exception as e:  # not available on this handle (several YAPS blocks)
            out.append({"kernel": name, "error": str(e)})
            continue
        t = kms * 1e-3
        tf, gbs = fl / t / 1e12, by / t / 1e9
        t_fp, t_hbm = fl / (fp64_tflops * 1e12), by / (hbm_gbs * 1e9)
        if t_fp >= t_hbm:
            r = {"bound": "fp64", "achieved": tf, "peak": fp64_tflops, "unit": "TFLOP/s", "frac": t_fp / t}
        else:
            r = {"bound": "hbm", "achieved": gbs, "peak": hbm_gbs, "unit": "GB/s", "frac": t_hbm / t}
        r.update({"kernel": name, "ms_per_launch": kms, "launches_per_step": per_step,
                  "ms_per_step": kms * per_step, "fp64_tflops": tf, "fp64_frac": t_fp / t, "hbm_gbs": gbs,
                  "hbm_frac": t_hbm / t, "flops": fl, "bytes": by,
                  "traffic": traffic.get(name.split(" ")[0])})
        out.append(r)
    return out


def device_resident(V, cfg, xp, qp, w, args, local, dist, arith, clocks=None):
    """Set-up (sizes, plans, recorded operator, first remesh) and the timed
    device-resident loop in one arithmetic."""
    import torch
    torch.cuda.set_device(local)
    free0 = torch.cuda.mem_get_info(local)[0]
    t0 = time.perf_counter()
    h = V.VPM(cfg, device=local, arith=arith)
    if args.operator_budget >= 0:
        h.set_operator_budget(args.operator_budget)
    h.define_sizes(xp)
    xr, qr = h.remesh_particles_3d(1, xp, qp)
    h.set_particles(xr, qr)
    setup_s = time.perf_counter() - t0
    hbm_bytes = free0 - torch.cuda.mem_get_info(local)[0]
    dt = w["dt"]
    if args.warmup:
        h.run(args.warmup, dt)
    dist.barrier()
    if clocks:
        clocks.start()
    l0 = h.kernel_launches()
    ms, ps = h.run(args.steps, dt)
    launches = h.kernel_launches() - l0
    clk = clocks.stop() if clocks else {}
    dist.barrier()
    return h, xr, ms, ps, launches, clk, setup_s, hbm_bytes


def run_ours(args, dist):
    import vpm_free_gb300 as V
    from vpm_free_gb300 import build as B
    B.build()
    ws, rank, local = _dist()
    if args.workload == "dirichlet273":
        return run_dirichlet(args, local)
    xp, qp, w = _workload(args.workload)
    blocks = tuple(int(v) for v in args.blocks.split(","))
    cfg = V.VPMConfig.make(dpm=w["dpm"], box=w["box"], nb=blocks)
    h, xr, ms, ps, launches, clk, setup_s, hbm_bytes = device_resident(
        V, cfg, xp, qp, w, args, local, dist, args.arith, Clocks(local) if rank == 0 else None)
    dt = w["dt"]
    t_max = dist.reduce(ms, "max")
    ps_all = dist.reduce(ps, "sum")
    value = ps_all / (t_max * 1e-3)
    # ---- per-kernel roofline figures (replays on the resident state) -------
    fp64 = h.fp64_peak()
    peaks = _measured_peaks()
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    roofs = kernel_rooflines(h, fp64, hbm, _traffic_table())
    timed = [r for r in roofs if "error" not in r]
    dom = max(timed, key=lambda r: r["ms_per_step"])
    roof = {k: dom[k] for k in ("bound", "achieved", "peak", "unit", "frac", "kernel", "ms_per_launch", "traffic")}
    roof["peak_source"] = ("FP64: DFMA-loop TFLOP/s measured in this run (MEASURED_PEAKS.json has no FP64 entry); "
                           "HBM: MEASURED_PEAKS.json hbm_gbs (of measured)")
    roof["hbm_frac"] = dom["hbm_frac"]
    tree = h.tree_stats()
    tiles = h.dst_tiles()
    sizes_bl = list(h.sizes().nnbl)
    sizes_nn = list(h.sizes().nn)
    np_end = h.num_particles()
    phases = None
    if args.workload == "leapfrog256":
        h.set_profiling(1)
        h.step(dt)
        phases = dict(zip(["deposit", "fine_zero_bc", "boundary", "fine_bc", "coarse", "final", "fd", "m2p+euler",
                           "remesh"], [round(v, 3) for v in h.phase_times()]))
        h.set_profiling(0)
    h.close()
    # ---- end to end through the reference-facing calls, host arrays -------
    ke = max(1, min(args.steps, args.e2e_steps))
    he = V.VPM(cfg, device=local, arith=args.arith)
    if args.operator_budget >= 0:
        he.set_operator_budget(args.operator_budget)
    he.vpm(xp, qp, None, None, xp.shape[0], WhatToDo=0, NTIME=0)
    # the host's particle arrays hold NVRM = mesh nodes rows, the most a
    # remesh can emit; UP / GP likewise (test.f90 keeps XPR/QPR/UPR/GPR)
    nvrm = int(np.prod(sizes_nn))

    def host_array(rows, cols):  # pinned host memory (page-locked), numpy view
        try:
            import torch
            return torch.empty((rows, cols), dtype=torch.float64).pin_memory().numpy()
        except Exception:
            return np.empty((rows, cols))
    XP, QP = host_array(nvrm, 3), host_array(nvrm, 4)
    UP, GP = host_array(nvrm, 3), host_array(nvrm, 3)
    XP[:xp.shape[0]], QP[:qp.shape[0]] = xp, qp
    n = he.remesh_in_place(XP, QP, xp.shape[0])
    for _ in range(min(args.warmup, 1)):
        UP[:n] = 0.0; GP[:n] = 0.0
        he.vpm(XP[:n], QP[:n], UP[:n], GP[:n], n, WhatToDo=2, NTIME=1)
    dist.barrier()
    h2d = d2h = eps = 0
    t0 = time.perf_counter()
    for it in range(ke):
        eps += n
        up, gp = UP[:n], GP[:n]
        ctypes.memset(up.ctypes.data, 0, up.nbytes)   # the caller zeroes UP/GP (test.f90:90-91)
        ctypes.memset(gp.ctypes.data, 0, gp.nbytes)
        he.vpm(XP[:n], QP[:n], up, gp, n, WhatToDo=2, NTIME=it + 1)
        V.VPM.host_euler(XP, QP, UP, GP, n, dt)       # test.f90:104-117, one compiled pass, UINF = 0
        he.vpm(XP[:n], QP[:n], None, None, n, WhatToDo=0, NTIME=it + 1)
        n_old = n
        n = he.remesh_in_place(XP, QP, n)
        # vpm(2): XP, QP and UP in, UP and GP out; remesh: XP, QP in, the new set out
        h2d += n_old * (3 + 4 + 3) * 8 + n_old * 7 * 8
        d2h += n_old * 6 * 8 + n * 7 * 8
    te = time.perf_counter() - t0
    te_max = dist.reduce(te, "max")
    he.close()
    e2e = {"value": dist.reduce(eps, "sum") / te_max, "unit": UNIT, "h2d_bytes_per_step": h2d // ke,
           "d2h_bytes_per_step": d2h // ke, "steps": ke,
           "timing": "host clock around synchronous vpm()/remesh_particles_3d() C-ABI calls on pinned host arrays "
                     "of NVRM rows; between them the host zeroes UP/GP (memset) and runs the Euler update in one "
                     "compiled single-threaded pass (vpmg_host_euler), as the reference's test.f90 loop does"}
    # ---- the float-float arithmetic, labelled separately --------------------
    ff = None
    if args.arith == "fp64" and not args.no_ff48 and ws == 1:
        hf, _, ms_f, ps_f, _, clk_f, setup_f, hbm_f = device_resident(V, cfg, xp, qp, w, args, local, dist, "ff48",
                                                                     Clocks(local))
        roofs_f = kernel_rooflines(hf, fp64, hbm, {})
        timed_f = [r for r in roofs_f if "error" not in r]
        dom_f = max(timed_f, key=lambda r: r["ms_per_step"])
        hf.close()
        ff = {"dtype": "ff48", "value": ps_f / (ms_f * 1e-3), "unit": UNIT, "ms_per_step": ms_f / args.steps,
              "steps": args.steps, "setup_s": setup_f, "hbm_bytes": hbm_f, "clocks": clk_f,
              "arithmetic": ("float-float (hi + lo floats, about 48 significant bits, magnitudes 1e-38..3e38) in the "
                             "boundary operator, DST solves, projection weights, deposition, stretching and "
                             "mesh-to-particle kernels on the FP32 pipes; the rest FP64; parity with the FP64 oracle "
                             "<= 1e-10 (fields), <= 1e-9 (particles)"),
              "dominant_kernel": {k: dom_f[k] for k in ("kernel", "ms_per_launch", "fp64_tflops", "hbm_gbs",
                                                        "hbm_frac")},
              "kernels": [{k: r[k] for k in ("kernel", "ms_per_launch", "hbm_gbs", "hbm_frac")} for r in timed_f]}
    # ---- CPU baseline (rank 0, N = 1, bounded sample) -----------------------
    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu and args.workload == "leapfrog256" and blocks == (1, 1, 1):
        threads = os.cpu_count() or 1
        v, t, _ = cpu_step_sample(xp, qp, w, 1, threads)
        cpu = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"1 full step (field step + Euler + remesh) of this workload, {t:.1f} s on {threads} threads"}
        if args.cpu_1thread:  # the same step on one host thread (about 16x longer)
            v1, t1, _ = cpu_step_sample(xp, qp, w, 1, 1)
            cpu["one_thread"] = {"value": v1, "cores": 1, "sample": f"1 full step, {t1:.1f} s on 1 thread"}
    batched = None
    if not args.no_batched and args.workload == "leapfrog256":
        batched = run_batched(args, local)
    adjoint = None
    if not args.no_adjoint and args.workload == "leapfrog256":
        adjoint = run_adjoint(args, local)
    arith_text = ("IEEE FP64 in every kernel (the reference's REAL(8)); no tensor cores: no step is a dense "
                  "contraction" if args.arith == "fp64" else ff["arithmetic"] if ff else "float-float heavy kernels")
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t_max / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if args.arith == "fp64" else "ff48", "data": "synthetic (seeded leapfrogging rings)",
        "arithmetic": arith_text,
        "config": workload_config(args.workload, sizes_nn, sizes_bl, blocks),
        "parallelism": "replicas" if ws > 1 else "single GPU",
        "particles": {"start": int(xr.shape[0]), "end": np_end},
        "clocks": clk if rank == 0 else None,
        "setup_s": setup_s, "hbm_bytes": hbm_bytes,
        "setup": "define_sizes (plans, DST tile autotuning, tree geometry, recorded boundary operator) and the "
                 "initial remesh, host clock; hbm_bytes = device memory the handle holds after it",
        "e2e": e2e, "gpu_launches": launches, "roofline": roof, "roofline_kernels": roofs, "phase_ms": phases,
        "tree": tree, "dst_tiles_autotuned": tiles, "cpu_baseline": cpu, "ff48": ff, "batched": batched,
        "adjoint": adjoint,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--cpu-1thread", action="store_true",
                    help="also time the CPU baseline step on one host thread (adds about two minutes)")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="leapfrog256",
                    help="leapfrog256 is the benchmark; the rings are small profiling cases")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched-problems measurement")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the adjoint:forward measurement")
    ap.add_argument("--arith", choices=["fp64", "ff48"], default="fp64",
                    help="arithmetic of the headline run (fp64, the reference's, is the default)")
    ap.add_argument("--no-ff48", action="store_true", help="skip the float-float run reported beside the FP64 one")
    ap.add_argument("--batch-steps", type=int, default=20, help="steps of the batched workload (20, its stated length)")
    ap.add_argument("--batch-operator-budget", type=int, default=12 << 30,
                    help="bytes of recorded boundary operator per batched problem")
    ap.add_argument("--dirichlet-nodes", type=int, default=273,
                    help="nodes per axis of the dirichlet273 profiling workload (257: the inner box)")
    ap.add_argument("--blocks", default="1,1,1",
                    help="YAPS blocks NBI,NBJ,NBK on the one GPU (pm.inp line 7); the headline is 1,1,1")
    ap.add_argument("--operator-budget", type=int, default=-1,
                    help="bytes for the precomputed boundary operator (0: walk the tree each step)")
    ap.add_argument("--batch-group", default="",
                    help="profiling case: one shared-operator group of the batched workload, e.g. ring64 or ring64:8")
    args = ap.parse_args()
    if args.batch_group:
        return run_batch_group(args, _dist()[2])
    ws, rank, local = _dist()
    if args.impl == "reference":
        # rank 0 alone times the host-CPU path; other ranks exit without work
        dist = Dist(1, rank, local, "gloo")
    else:
        dist = Dist(ws, rank, local, "nccl")
    try:
        rc = run_reference(args, dist) if args.impl == "reference" else run_ours(args, dist)
    finally:
        dist.close()
    return rc


if __name__ == "__main__":
    sys.exit(main())
