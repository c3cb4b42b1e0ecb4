#!/usr/bin/env python
"""Throughput of the FVDBM step (MCUPS and fraction of the HBM roofline).

Workload (default): the porous square, 400 seeded circular obstacles at
porosity 0.70, ~1M triangles, D2Q9, tau=0.6, dt=0.5*min edge, upwind,
inlet rho=1.001 / outlet rho=1.0 density nodes, no-slip walls and obstacles,
float32.  Inputs are synthetic (seeded mesh generator; Triangle is not
available).

A bench step is one FVDBM time step over the whole mesh.  Between timed steps
L2 is flushed by writing a buffer of 2x L2 size on the step's stream and then
reading it back (so the lines left in L2 are clean and the timed step pays no
write-back of the flush data): each timed step reads its inputs from HBM.  Each step is bracketed by CUDA events
on the library's stream; the cell kernel (the dominant one) is timed on its
own for the roofline.

The timed family is ``--kernel`` (default ``fast``: the single-launch step
with contracted float32 arithmetic, bitwise reproducible run to run and as
close to the float64 step as the reference's own float32 step); the
bit-exact default family of ``Environment`` is timed beside it on the same
mesh under ``bitexact``.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Under torchrun (N>1) every rank runs an independent replica (a differently
seeded mesh of the same size): units processed over all ranks / max time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "MCUPS at 1M tris (% HBM roofline); time-to-steady @1e-6 resid, warm vs plain"
L2_BYTES = 129 * 1024 * 1024


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=200)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="porous1m",
                    choices=["porous1m", "porous2m", "porous4m", "cavity", "channel", "batch", "warmstart",
                             "mpnn_epoch"])
    ap.add_argument("--flux", default="upwind", choices=["upwind", "lax_wendroff"])
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-above-l2", action="store_true",
                    help="skip the ~4M-triangle point whose per-step traffic is well above L2")
    ap.add_argument("--e2e-steps", type=int, default=100)
    ap.add_argument("--kernel", default=None,
                    choices=["auto", "one", "fused", "fused_nodes", "fast", "persist", "staged", "tile", "tile_split"],
                    help="kernel family timed (default: fast for the porous workloads, auto otherwise: on "
                         "the small cavity and channel meshes the two-launch family is the faster one)")
    # --workload batch: time-to-steady of many independent cases, batched vs one at a time
    ap.add_argument("--cases", type=int, default=256)
    ap.add_argument("--units", default="lattice", choices=["lattice", "unit"],
                    help="--workload batch: lattice units (mesh spacing ~1, the reference's update and "
                         "tau = 3UL/Re + 1/2) or the unit square (finite-volume update, tau = 3UL/Re)")
    ap.add_argument("--threshold", type=float, default=1e-6)
    ap.add_argument("--check-every", type=int, default=100)
    ap.add_argument("--check-time", type=float, default=None,
                    help="residual window in each case's own time units (default: 100 for the batch in "
                         "lattice units, 5 otherwise)")
    ap.add_argument("--step-cap", type=int, default=None,
                    help="per-case step cap (default: 20000 for batch, 100000 for warmstart)")
    # --workload warmstart: learned warm start against the uniform start
    ap.add_argument("--train-cases", type=int, default=400)
    ap.add_argument("--eval-cases", type=int, default=64)
    ap.add_argument("--group-cases", type=int, default=200,
                    help="warmstart: training cases meshed, solved and turned into samples per group "
                         "(bounds the host memory the cases take)")
    ap.add_argument("--epochs", type=int, default=300)
    ap.add_argument("--ws-cells", type=str, default="50000,200000",
                    help="warmstart: cell-count range of the porous geometries")
    ap.add_argument("--batch-cells", type=int, default=6_000_000,
                    help="warmstart: cells per training minibatch")
    ap.add_argument("--graph-cells", type=int, default=1_500_000,
                    help="mpnn_epoch: cells of the synthetic graph")
    args = ap.parse_args()
    if args.kernel is None:
        args.kernel = "fast" if args.workload.startswith("porous") else "auto"
    return args


def workload(name, flux, seed):
    from fvdbm_jax_gb300 import D2Q9, Mesher, meshgen
    t0 = time.perf_counter()
    if name.startswith("porous"):
        target = {"porous1m": 1_000_000, "porous2m": 2_000_000, "porous4m": 4_000_000}[name]
        raw = meshgen.porous(n_obstacles=400, n_target=target, porosity=0.70, seed=seed)
        tau = 0.6
    elif name == "channel":
        raw = meshgen.channel_cylinder(seed=seed)
        tau = 0.55
    else:
        raw = meshgen.cavity(seed=seed)
        tau = 0.6
    m = Mesher().import_meshpy(raw)
    m.calc_mesh_properties()
    dyn = D2Q9(tau, 0.5 * float(m.face_lengths.min()))
    c, f, n = m.to_env(dyn, flux)
    if name.startswith("porous"):
        for mk in (1, 3, 5):
            n = m.set_vel_node(n, mk, (0.0, 0.0))
        n = m.set_rho_node(n, 4, 1.001)
        n = m.set_rho_node(n, 2, 1.0)
    elif name == "channel":
        import numpy as np
        for mk in (1, 3, 5):
            n = m.set_vel_node(n, mk, (0.0, 0.0))
        n = m.set_vel_node(n, 4, (0.0, 0.0))
        sel = m.point_markers == 4
        y = m.points[sel, 1]
        v = np.array(n.vel)
        v[sel, 0] = 4 * 0.1 * y * (0.41 - y) / 0.41 ** 2
        n.vel = v
        n = m.set_rho_node(n, 2, 1.0)
    else:
        for mk in (1, 2, 4):
            n = m.set_vel_node(n, mk, (0.0, 0.0))
        n = m.set_vel_node(n, 3, (0.1, 0.0))
    desc = {"workload": {"porous1m": "porous square, 400 obstacles, ~1M triangles",
                         "porous2m": "porous square, 400 obstacles, ~2M triangles",
                         "porous4m": "porous square, 400 obstacles, ~4M triangles",
                         "channel": "channel 2.2x0.41 with cylinder, ~60k triangles",
                         "cavity": "lid-driven cavity 41x41 grid, 3,200 triangles"}[name],
            "cells": int(c.pdf.shape[0]), "faces": int(f.pdf.shape[0]), "nodes": int(n.pdf.shape[0]),
            "lattice": "D2Q9", "flux": flux, "tau": tau, "delta_t": float(dyn.delta_t),
            "porosity": float(raw.info.get("porosity", 1.0)) if name.startswith("porous") else None,
            "seed": seed, "setup_s": round(time.perf_counter() - t0, 2)}
    return m, dyn, c, f, n, desc


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            pk = json.load(fh)
        return float(pk["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profiled_traffic(kernel, desc):
    """DRAM bytes per launch of a kernel on this workload from the committed
    ncu summary, if one was captured for it."""
    try:
        with open(os.path.join(ROOT, "profiles", "ncu_traffic.json")) as fh:
            rec = json.load(fh).get(kernel, {})
    except Exception:
        return None
    if rec.get("workload") != desc.get("workload") or rec.get("flux") != desc.get("flux"):
        return None
    return rec.get("bytes_per_launch")


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.lines = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 6:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[2:6]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    return ws, rank, local


def max_over_ranks(x, ws, device):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=f"cuda:{device}")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(x, ws, device):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=f"cuda:{device}")
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def cpu_oracle_rate(c, f, n, dyn, seconds, threads=0):
    """C restatement of the step on the host cores: MCUPS over a bounded
    sample (whole steps of the same mesh until ``seconds`` elapse)."""
    import oracle_c as OC
    import oracle_np as O
    geo = O.geo_from_containers(c, f, n)
    st = O.state_from_containers(c, n)
    pr = OC.Prepared(geo, dyn.inv_tau, dyn.dt32)
    threads = threads or OC.max_threads()
    OC.step(geo, st, dyn.inv_tau, dyn.dt32, n_steps=1, threads=threads, prepared=pr)  # warm
    done, t0 = 0, time.perf_counter()
    while True:
        st = OC.step(geo, st, dyn.inv_tau, dyn.dt32, n_steps=1, threads=threads, prepared=pr)
        done += 1
        el = time.perf_counter() - t0
        if el >= seconds or done >= 10_000:
            break
    N = int(c.pdf.shape[0])
    return N * done / el / 1e6, threads, done, el


def numpy_oracle_rate(c, f, n, dyn, seconds):
    """The vectorised numpy restatement (gathers and folds over whole arrays,
    like the reference's XLA program on the CPU): MCUPS over whole steps of
    the same mesh until ``seconds`` elapse (at least one)."""
    import numpy as np
    import oracle_np as O
    geo = O.geo_from_containers(c, f, n)
    st = O.state_from_containers(c, n)
    done, t0 = 0, time.perf_counter()
    with np.errstate(all="ignore"):
        while True:
            st = O.step(geo, st, dyn.inv_tau, dyn.dt32)
            done += 1
            el = time.perf_counter() - t0
            if el >= seconds:
                break
    return int(c.pdf.shape[0]) * done / el / 1e6, done, el


def above_l2_point(args, local, flush_l2_on):
    """The same step on the ~4M-triangle porous square (same generator,
    parameters and boundary conditions): about 460 MB of algorithmic traffic
    per step against the 129 MB L2, so consecutive steps read their inputs
    from HBM without any flush.  Times K flushed single steps (as the main
    line) and 512 consecutive graph-replayed steps; each with its roofline
    fraction of the same measured peak."""
    import torch

    from fvdbm_jax_gb300 import Environment
    from fvdbm_jax_gb300 import _native as nat
    m, dyn, c, f, n, desc = workload("porous4m", args.flux, seed=0)
    env = Environment(c, f, n, device=local, kernel=args.kernel)
    env.init()
    info = env.info()
    L = nat.lib()
    h = env.handle
    stream = torch.cuda.ExternalStream(env.stream_ptr, device=f"cuda:{local}")
    env.step(max(args.warmup, 3))
    env.sync()
    K = max(3, min(args.steps, 50))
    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(2)] for _ in range(K)]
    for k in range(K):
        with torch.cuda.stream(stream):
            flush_l2_on(k)
        ev[k][0].record(stream)
        nat.check(L.fvdbm_step(h, 1), h)
        ev[k][1].record(stream)
    env.sync()
    flushed_us = statistics.mean(e[0].elapsed_time(e[1]) for e in ev) * 1e3
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    steps = 512
    env.step(64)
    e0.record(stream)
    env.step(steps)
    e1.record(stream)
    env.sync()
    cons_us = e0.elapsed_time(e1) * 1e3 / steps
    peak, peak_kind = measured_peaks()
    B = info["bytes_per_step"]
    N = info["n_cells"]
    env.close()
    return {"workload": desc["workload"], "cells": N, "faces": info["n_faces"], "bytes_per_step": B,
            "l2_bytes": L2_BYTES, "kernel": {7: "k_fused_nodes", 9: "k_fused_nodes_fast"}.get(info["kernel"], str(info["kernel"])),
            "flushed": {"us_per_step": round(flushed_us, 3), "mcups": round(N / flushed_us, 1),
                        "frac": round(B / flushed_us / 1e3 / peak, 4), "steps": K},
            "consecutive": {"us_per_step": round(cons_us, 3), "mcups": round(N / cons_us, 1),
                            "frac": round(B / cons_us / 1e3 / peak, 4), "steps": steps,
                            "note": "graph replay without a flush; the step's inputs are 3.6x the L2"},
            "peak": peak, "peak_kind": peak_kind}


def bitexact_point(args, local, flush_l2, c, f, n, K, desc):
    """The bit-exact default family (what ``Environment`` runs unless told
    otherwise) on the same mesh and protocol: K single steps, L2 flushed
    before each, each bracketed by CUDA events on the library's stream."""
    import torch

    from fvdbm_jax_gb300 import Environment
    from fvdbm_jax_gb300 import _native as nat
    env = Environment(c, f, n, device=local, kernel="auto")
    env.init()
    info = env.info()
    L = nat.lib()
    h = env.handle
    stream = torch.cuda.ExternalStream(env.stream_ptr, device=f"cuda:{local}")
    env.step(max(args.warmup, 3))
    env.sync()
    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(2)] for _ in range(K)]
    for k in range(K):
        with torch.cuda.stream(stream):
            flush_l2(k)
        ev[k][0].record(stream)
        nat.check(L.fvdbm_step(h, 1), h)
        ev[k][1].record(stream)
    env.sync()
    us = statistics.mean(e[0].elapsed_time(e[1]) for e in ev) * 1e3
    peak, peak_kind = measured_peaks()
    N, B = info["n_cells"], info["bytes_per_step"]
    env.close()
    # the whole step: one launch for the single-launch family (meshes of 2^18
    # cells or more), else the two-launch family's pair
    return {"kernel": {7: "k_fused_nodes", 2: "k_nodes_cp + k_fused"}.get(info["kernel"], str(info["kernel"])),
            "launches_per_step": info["launches_per_step"],
            "note": "bit for bit with the reference's step; the same flushed protocol",
            "avg_launch_us": round(us, 3), "mcups": round(N / us, 1),
            "frac": round(B / us / 1e3 / peak, 4), "traffic": profiled_traffic("k_fused_nodes", desc), "steps": K}


def run_reference(args):
    ws, rank, local = dist_setup()
    if rank != 0:
        return
    m, dyn, c, f, n, desc = workload(args.workload, args.flux, seed=0)
    budget = max(5.0, min(150.0, 0.05 * args.steps + 10.0))
    rate, threads, done, el = cpu_oracle_rate(c, f, n, dyn, budget)
    N = int(c.pdf.shape[0])
    line = {"impl": "reference", "metric": METRIC, "value": round(rate, 3), "unit": "MCUPS",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(el / done * 1e3, 3), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": desc,
            "cpu_baseline": {"value": round(rate, 3), "unit": "MCUPS", "cores": threads, "kind": "port",
                             "sample": f"{done} whole steps of the {N}-cell mesh ({el:.1f}s), "
                                       f"C restatement of the reference step, OpenMP"},
            "e2e": {"value": round(rate, 3), "unit": "MCUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_gb300(args):
    import numpy as np
    import torch

    from fvdbm_jax_gb300 import Environment
    from fvdbm_jax_gb300 import _native as nat

    ws, rank, local = dist_setup()
    torch.cuda.set_device(local)
    m, dyn, c, f, n, desc = workload(args.workload, args.flux, seed=rank)
    env = Environment(c, f, n, device=local, kernel=args.kernel)
    env.init()
    info = env.info()
    L = nat.lib()
    h = env.handle
    N = info["n_cells"]
    stream = torch.cuda.ExternalStream(env.stream_ptr, device=f"cuda:{local}")
    flush = torch.empty(2 * L2_BYTES, dtype=torch.uint8, device=f"cuda:{local}")
    flush_sum = torch.zeros((), dtype=torch.int64, device=f"cuda:{local}")

    def flush_l2(k):
        # write 2x L2, then read it: L2 holds only clean, unrelated lines
        flush.fill_(k & 0xFF)
        flush_sum.add_(flush.view(torch.int64).sum())

    # warm-up (graph replay, as a long run would)
    env.step(max(args.warmup, 3))
    env.sync()

    K = args.steps
    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(2)] for _ in range(K)]
    barrier(ws)
    torch.cuda.synchronize(local)
    env.sync()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    # timed region: K steps through the library's step call, L2 flushed
    # before each (the flush is outside the events)
    t_wall = time.perf_counter()
    for k in range(K):
        with torch.cuda.stream(stream):
            flush_l2(k)
        ev[k][0].record(stream)
        nat.check(L.fvdbm_step(h, 1), h)
        ev[k][1].record(stream)
    env.sync()
    torch.cuda.synchronize(local)
    t_wall = time.perf_counter() - t_wall
    barrier(ws)
    clk = clocks.stop()
    step_ms = [e[0].elapsed_time(e[1]) for e in ev]
    total_ms = sum(step_ms)

    # per-kernel durations for the roofline: the same flushed steps with the
    # node and cell kernels bracketed separately (no overlap between them)
    Kp = min(K, 200)
    evp = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(Kp)]
    for k in range(Kp):
        with torch.cuda.stream(stream):
            flush_l2(k)
        evp[k][0].record(stream)
        nat.check(L.fvdbm_step_phase(h, 1), h)
        evp[k][1].record(stream)
        nat.check(L.fvdbm_step_phase(h, 2), h)
        evp[k][2].record(stream)
    env.sync()
    node_ms = [e[0].elapsed_time(e[1]) for e in evp]
    cell_ms = [e[1].elapsed_time(e[2]) for e in evp]
    total_ms_max = max_over_ranks(total_ms, ws, local)
    cells_all = sum_over_ranks(float(N), ws, local)
    value = cells_all * K / (total_ms_max / 1e3) / 1e6

    # the dominant kernel's algorithmic bytes per launch: pdf read + write,
    # cell->face slots, face geometry, boundary-node pdf traffic.  The tile
    # kernel does the whole step in one launch.
    F = info["n_faces"]
    K3 = int(np.asarray(c.face_indices).shape[1])
    if info["kernel"] in (3, 5, 7, 8, 9):
        cell_bytes = info["bytes_per_step"]
    elif info["kernel"] == 4:
        cell_bytes = info["bytes_per_step"] - 36.0 * info["n_bc_nodes"]
    else:
        cell_bytes = 72.0 * N + 4.0 * K3 * N + 20.0 * F + \
            (8.0 * F if args.flux == "lax_wendroff" else 0.0) + 36.0 * info["n_bc_nodes"]
    cell_avg_s = statistics.mean(cell_ms) / 1e3
    peak, peak_kind = measured_peaks()
    achieved = cell_bytes / cell_avg_s / 1e9
    step_achieved = info["bytes_per_step"] / (statistics.mean(step_ms) / 1e3) / 1e9

    # the same steps back to back from the captured CUDA graph, no flush (the
    # state then partly stays in L2, as in a long run)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    resident_steps = 1024
    env.step(64)
    e0.record(stream)
    env.step(resident_steps)
    e1.record(stream)
    env.sync()
    res_ms = e0.elapsed_time(e1) / resident_steps

    # end to end through the C ABI with host buffers: per step the pdf is
    # copied in from pinned memory, one step runs, rho and vel are read back
    pdf_h = torch.empty((N, 9), dtype=torch.float32, pin_memory=True).numpy()
    rho_h = torch.empty((N,), dtype=torch.float32, pin_memory=True).numpy()
    vel_h = torch.empty((N, 2), dtype=torch.float32, pin_memory=True).numpy()
    nat.check(L.fvdbm_get_cells(h, nat.fptr(pdf_h), None, None, None), h)
    E = max(3, min(args.e2e_steps, K))
    for _ in range(2):
        nat.check(L.fvdbm_set_state(h, nat.fptr(pdf_h), None, None, None), h)
        nat.check(L.fvdbm_step(h, 1), h)
        nat.check(L.fvdbm_get_cells(h, None, nat.fptr(rho_h), nat.fptr(vel_h), None), h)
    barrier(ws)
    t0 = time.perf_counter()
    for _ in range(E):
        nat.check(L.fvdbm_set_state(h, nat.fptr(pdf_h), None, None, None), h)
        nat.check(L.fvdbm_step(h, 1), h)
        nat.check(L.fvdbm_get_cells(h, None, nat.fptr(rho_h), nat.fptr(vel_h), None), h)
    e2e_s = max_over_ranks(time.perf_counter() - t0, ws, local)
    e2e_value = cells_all * E / e2e_s / 1e6

    above = None
    if rank == 0 and args.workload == "porous1m" and not args.no_above_l2:
        above = above_l2_point(args, local, flush_l2)
    exact = None
    if rank == 0 and info["kernel"] == nat.KERNEL_FAST:
        exact = bitexact_point(args, local, flush_l2, c, f, n, Kp, desc)

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        rate, threads, done, el = cpu_oracle_rate(c, f, n, dyn, args.cpu_seconds)
        nrate, ndone, nel = numpy_oracle_rate(c, f, n, dyn, 8.0)
        cpu = {"value": round(rate, 3), "unit": "MCUPS", "cores": threads, "kind": "port",
               "sample": f"{done} whole steps of the same {N}-cell mesh ({el:.1f}s), C restatement "
                         f"of the reference step with OpenMP",
               "numpy": {"value": round(nrate, 3), "unit": "MCUPS",
                         "sample": f"{ndone} whole steps ({nel:.1f}s) of the vectorised numpy restatement, "
                                   f"whole-array gathers and folds as the reference's XLA CPU program does"}}

    kname = {1: "k_gather", 2: "k_fused", 3: "k_tile", 4: "k_tile", 5: "k_step",
             7: "k_fused_nodes", 8: "k_persist", 9: "k_fused_nodes_fast"}[info["kernel"]]
    if rank == 0:
        desc.update({"global_cells": int(cells_all), "parallelism": f"replicas x{ws}" if ws > 1 else "single GPU",
                     "l2": "flushed between timed steps (2x L2 written, then read back, on the step's stream)",
                     "kernel": {1: "staged", 2: "fused", 3: "tile", 4: "tile_split", 5: "one",
                                7: "fused_nodes", 8: "persist", 9: "fast"}[info["kernel"]],
                     "launches_per_step": info["launches_per_step"],
                     "ctas_per_sm": info["ctas_per_sm"]})
        if info["kernel"] == nat.KERNEL_FAST:
            desc["arithmetic"] = ("contracted float32 (multiply-adds, reciprocals of the lattice constants, "
                                  "compact face slots): bitwise reproducible run to run, as close to the float64 "
                                  "step as the reference's float32 step (tests/test_gpu_fast.py); the bit-exact "
                                  "default family is timed beside it under 'bitexact'")
        line = {
            "metric": METRIC, "value": round(value, 3), "unit": "MCUPS", "n_gpus": ws, "steps": K,
            "warmup": args.warmup, "ms_per_step": round(total_ms_max / K, 5), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": desc,
            "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                         "frac": round(achieved / peak, 4), "traffic": profiled_traffic(kname, desc),
                         "kernel": kname,
                         "bytes_per_launch": cell_bytes, "avg_launch_us": round(cell_avg_s * 1e6, 3),
                         "peak_kind": peak_kind,
                         "step_frac": round(step_achieved / peak, 4),
                         "node_kernel_avg_us": round(statistics.mean(node_ms) * 1e3, 3),
                         "timed_launches": Kp},
            "cpu_baseline": cpu,
            "e2e": {"value": round(e2e_value, 3), "unit": "MCUPS", "h2d_bytes_per_step": 36 * N,
                    "d2h_bytes_per_step": 12 * N, "steps": E},
            "gpu_launches": K * info["launches_per_step"],
            "clocks": clk,
            "l2_resident": {"mcups": round(N / (res_ms / 1e3) / 1e6, 3), "ms_per_step": round(res_ms, 5),
                            "steps": resident_steps,
                            "frac": round(info["bytes_per_step"] / (res_ms / 1e3) / 1e9 / peak, 4),
                            "note": "graph replay of consecutive steps, no flush (a long run's steady state); "
                                    "frac: the step's algorithmic bytes per step time over the same peak"},
            "wall_s": round(t_wall, 3),
        }
        if above is not None:
            line["above_l2"] = above
        if exact is not None:
            line["bitexact"] = exact
        print(json.dumps(line), flush=True)
    env.close()
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def run_batch(args):
    """Time to steady state (residual < threshold, or the per-case step cap)
    of a suite of independent cases: all of them in one packed Batch (one
    launch per kernel per step, cases retiring independently) against the
    plain solver running each case alone, one after the other, with the same
    per-case check windows.  Set-up (meshing, plans, autotuning) is outside
    both timings.

    Regime (``--units lattice``, the default): every case meshed at a
    spacing of about 1, the reference's own update (no division by the cell
    area), tau = 3 U L / Re + 1/2 with U = 0.1 and L the case's side in those
    units (the notebooks' convention, tests/flow_over_cyl.ipynb:216),
    dt = 0.5 min edge; porous inlet / outlet densities 1.05 / 0.95
    (tests/porous_flow.ipynb:470-474).  ``--units unit``: the unit square,
    the finite-volume scaled update, tau = 3 U L / Re with L = 1 and
    dt = min(area / perimeter, tau).  A case's residual is taken over at
    least ``--check-time`` units of its own time, which keeps float32
    rounding noise below the threshold."""
    import numpy as np
    import torch

    from fvdbm_jax_gb300 import Batch, Environment
    from fvdbm_jax_gb300 import cases as CS

    ws, rank, local = dist_setup()
    t0 = time.perf_counter()
    n_cav = args.cases // 2
    # several GPUs: the cases are split (greedy by size), no exchange at all
    lattice = args.units == "lattice"
    fv = not lattice
    suite, desc = CS.batch_suite(seed=0, n_cavity=n_cav, n_porous=args.cases - n_cav, flux=args.flux,
                                 workers=min(16, os.cpu_count() or 1), rank=rank, n_ranks=ws,
                                 fv_dt=None if lattice else 1.0, rho_in=1.05, rho_out=0.95,
                                 tau_rule="notebook" if lattice else "dbm", units=args.units)
    torch.cuda.set_device(local)
    setup_s = time.perf_counter() - t0
    cells = np.array([d["cells"] for d in desc], np.int64)
    thr, every, cap = args.threshold, args.check_every, args.step_cap or 1_000_000
    # per-case window in whole chunks, as the batch loop takes it
    ct = args.check_time if args.check_time is not None else (100.0 if lattice else 5.0)
    window = np.array([int(np.ceil(max(1, int(np.ceil(ct / d["dt"]))) / every)) * every
                       for d in desc], np.int64)

    b = Batch([(c, f, n) for _, c, f, n in suite], device=local, finite_volume=fv)
    b.init()
    tune = b.autotune(steps=32)
    b.sync()
    torch.cuda.synchronize()
    barrier(ws)
    t = time.perf_counter()
    steps_b, res_b, st_b = b.run_to_steady(thr, every, cap, check_time=ct)
    b.sync()
    batched_s = max_over_ranks(time.perf_counter() - t, ws, local)
    b.close()

    steps_p, plain_s = [], 0.0
    for (_, c, f, n), w in zip(suite, window):
        env = Environment(c, f, n, device=local, finite_volume=fv)
        env.init()
        env.sync()
        t = time.perf_counter()
        s, _ = env.run_to_steady(thr, int(w), cap)
        env.sync()
        plain_s += time.perf_counter() - t
        steps_p.append(s)
        env.close()
    plain_s = max_over_ranks(plain_s, ws, local)
    steps_p = np.array(steps_p, np.int64)
    work = sum_over_ranks(float(np.sum(cells * steps_b)), ws, local)
    work_p = sum_over_ranks(float(np.sum(cells * steps_p)), ws, local)
    same = sum_over_ranks(float(not np.array_equal(steps_b[st_b != 4], steps_p[st_b != 4])), ws, local) == 0
    counts = [sum_over_ranks(float(np.sum(st_b == k)), ws, local) for k in (1, 0, 2, 3, 4)]
    all_cells = sum_over_ranks(float(cells.sum()), ws, local)
    if rank != 0:
        return
    kinds = np.array([d["kind"] for d in desc])
    line = {"metric": f"time-to-steady @{thr:g} resid (or {cap}-step cap), batched vs plain",
            "value": round(batched_s, 3), "unit": "s", "higher_is_better": False,
            "plain_s": round(plain_s, 3), "speedup": round(plain_s / batched_s, 2),
            "batched_mcups": round(work / batched_s / 1e6, 1),
            "plain_mcups": round(work_p / plain_s / 1e6, 1),
            "same_steps": bool(same),
            "converged": int(counts[0]), "capped": int(counts[1]), "nonfinite": int(counts[2]),
            "frozen": int(counts[3]), "stalled": int(counts[4]),
            "steps_median": int(np.median(steps_b)), "steps_max": int(steps_b.max()),
            "steps_median_cavity": int(np.median(steps_b[kinds == "cavity"])) if (kinds == "cavity").any() else None,
            "steps_median_porous": int(np.median(steps_b[kinds == "porous"])) if (kinds == "porous").any() else None,
            "res_max_converged": float(res_b[st_b == 1].max()) if (st_b == 1).any() else None,
            "converged_at_exact_fixed_point": int(np.sum((st_b == 1) & (res_b == 0.0))),
            "status_by_kind": {k: {name: int(np.sum((kinds == k) & (st_b == code)))
                                   for name, code in (("converged", 1), ("capped", 0), ("nonfinite", 2),
                                                      ("frozen", 3), ("stalled", 4))}
                               for k in ("cavity", "porous")},
            "stalled_cases": [{"kind": str(kinds[i]), "cells": int(cells[i]), "re": round(float(desc[i]["re"]), 1),
                               "tau": round(float(desc[i]["tau"]), 4), "steps": int(steps_b[i]),
                               "res": float(res_b[i])} for i in np.nonzero(st_b == 4)[0]],
            "n_gpus": ws, "scaling": "strong", "dtype": "f32", "data": "synthetic",
            "autotune": tune,
            "config": {"workload": f"{args.cases} independent cases: {n_cav} lid cavities (2k-60k cells, lid 0.1), "
                                   f"{args.cases - n_cav} porous squares (10k-120k cells, 20-200 obstacles, "
                                   "rho 1.05 / 0.95), Re 50-400; " + (
                                       "lattice units (mesh spacing ~1), tau = 3UL/Re + 1/2 with L the side "
                                       "in cells, the reference's update, dt = 0.5 min edge" if lattice else
                                       "unit square, tau = 3UL/Re, finite-volume update, "
                                       "dt = min(area/perimeter, tau)"),
                       "units": args.units, "cells": int(all_cells), "flux": args.flux,
                       "check_every": every, "check_time": ct, "step_cap": cap,
                       "setup_s": round(setup_s, 1)}}
    print(json.dumps(line), flush=True)


def _ws_case(spec):
    from fvdbm_jax_gb300 import cases as CS
    return CS.porous_square(spec["obstacles"], spec["n_target"], spec["tau"], rho_in=spec["rho_in"],
                            rho_out=spec["rho_out"], porosity=spec["porosity"], fv_dt=spec["fv_dt"],
                            seed=spec["seed"], mesher=True, scale=spec["scale"])


def _ws_sample(job):
    """Network input of one case (features and aggregation stages), with
    targets when rho/vel are given; the potential-flow system is left for
    one GPU solve over all cases (warmstart.solve_potentials)."""
    from fvdbm_jax_gb300 import warmstart as WS
    case, rho_in, rho_out, rho, vel = job
    return WS.sample(case, rho_in, rho_out, rho, vel, defer_potential=True)


def run_warmstart(args):
    """Learned warm start: solver-generated steady states of seeded porous
    squares train the network (on the GPU, by the library's kernels); on
    held-out geometries the solver runs to the residual threshold from the
    uniform start and from f = feq(predicted rho, u), with the stall fallback,
    both as one Batch with the same loop; and the plain solver runs each case
    alone from the uniform start.  Reports steps and seconds.

    Regime (``--units lattice``, the default): the mesh spacing about 1,
    the reference's update, tau = 3 U L / Re + 1/2 with Re 100, U = 0.1 and L
    the side in cells, dt = 0.5 min edge.  ``--units unit``: the unit square,
    the finite-volume scaled update, tau = 0.003 (Re 100 with U = 0.1, L = 1
    by nu = c_s^2 tau), dt = min(area / perimeter, tau).  Inlet density
    1.01-1.05, outlet 0.95-0.99; residual windows of ``--check-time`` time
    units per case (default 100 in lattice units, else 5)."""
    import concurrent.futures as cf
    import multiprocessing as mp

    import numpy as np
    import torch

    from fvdbm_jax_gb300 import Batch
    from fvdbm_jax_gb300 import warmstart as WS

    rng = np.random.default_rng(2024)
    lo_cells, hi_cells = (int(v) for v in args.ws_cells.split(","))

    from fvdbm_jax_gb300 import cases as CS
    lattice = args.units == "lattice"
    fv = not lattice

    def spec(i):
        s = {"obstacles": int(rng.integers(20, 201)), "n_target": int(rng.uniform(lo_cells, hi_cells)),
             "tau": 0.003, "rho_in": float(rng.uniform(1.01, 1.05)), "rho_out": float(rng.uniform(0.95, 0.99)),
             "porosity": float(rng.uniform(0.75, 0.85)), "seed": 50_000 + i, "scale": 1.0, "fv_dt": 1.0}
        if lattice:
            s["scale"] = CS.porous_lattice_scale(s["n_target"], s["porosity"])
            s["tau"] = CS.tau_from_re(100.0, length=s["scale"], rule="notebook")
            s["fv_dt"] = None
        return s
    specs = [spec(i) for i in range(args.train_cases + args.eval_cases)]
    t0 = time.perf_counter()
    # one pool of host workers, started before the first GPU call, builds the
    # cases and later the per-case network inputs
    ex = cf.ProcessPoolExecutor(min(16, os.cpu_count() or 1), mp_context=mp.get_context("spawn"))
    tspec, espec = specs[:args.train_cases], specs[args.train_cases:]
    evalc = list(ex.map(_ws_case, espec, chunksize=2))
    setup_s = time.perf_counter() - t0
    thr, every, cap = args.threshold, args.check_every, args.step_cap or 1_000_000
    ct = args.check_time if args.check_time is not None else (100.0 if lattice else 5.0)

    # training data: the solver's own steady states, a group of cases at a
    # time (meshed by the workers, solved as one batch, turned into samples;
    # only the samples are kept)
    data_s, samples, steps_t, st_t, train_cells = 0.0, [], [], [], 0
    G = max(1, args.group_cases)
    for g0 in range(0, len(tspec), G):
        gspec = tspec[g0:g0 + G]
        t = time.perf_counter()
        train = list(ex.map(_ws_case, gspec, chunksize=2))
        setup_s += time.perf_counter() - t
        t = time.perf_counter()
        b = Batch([c[1:4] for c in train], finite_volume=fv)
        b.init()
        stp, _, sts = b.run_to_steady(thr, every, cap, check_time=ct)
        state = b.state()
        data_s += time.perf_counter() - t
        steps_t += list(stp)
        st_t += list(sts)
        # converged and frozen states alike: an update below half an ulp
        # rounds away, so either way the float32 iteration has stopped inside
        # a band around the discrete steady state whose width grows like 1/dt
        jobs = []
        for s, (case, sp) in enumerate(zip(train, gspec)):
            train_cells += int(case[1].pdf.shape[0])
            if sts[s] not in (1, 3):
                continue
            rho, vel = WS.macros(b.case_state(s, state)["pdf"])
            jobs.append((case, sp["rho_in"], sp["rho_out"], rho, vel))
        b.close()
        del state, train
        grp = list(ex.map(_ws_sample, jobs, chunksize=2))
        del jobs
        WS.solve_potentials(grp)
        samples += grp
    steps_t, st_t = np.array(steps_t), np.array(st_t)
    t = time.perf_counter()
    net = WS.MPNN(seed=0)
    hist = net.fit(samples, epochs=args.epochs, lr=3e-3, log_every=max(args.epochs // 10, 1),
                   batch_cells=args.batch_cells)
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t

    # held-out: uniform start against the predicted start
    def timed(init):
        bb = Batch([c[1:4] for c in evalc], finite_volume=fv)
        bb.init()
        bb.sync()
        t1 = time.perf_counter()
        out = WS.run_cases(bb, thr, every, cap, init=init, check_time=ct)
        bb.sync()
        el = time.perf_counter() - t1
        fin = bb.state()
        bb.close()
        return out, el, fin
    (sp_, stp, _), plain_s, fin_p = timed(None)
    rho, vel = [], []
    # the prediction: features, stages and the network, all built and run on
    # the GPU (warmstart.predict_cases)
    torch.cuda.synchronize()
    t = time.perf_counter()
    preds, pcg_iters, pcg_rel = WS.predict_cases(net, evalc, [sp["rho_in"] for sp in espec],
                                                 [sp["rho_out"] for sp in espec])
    for y, sp in zip(preds, espec):
        r, v = WS.untarget(y, sp["rho_in"], sp["rho_out"])
        rho.append(r)
        vel.append(v)
    torch.cuda.synchronize()
    infer_s = time.perf_counter() - t
    ex.shutdown()
    (sw, stw, restarted), warm_s, fin_w = timed((np.concatenate(rho), np.concatenate(vel)))
    # the plain solver as a user runs it: each case alone from the uniform start
    from fvdbm_jax_gb300 import Environment
    seq_s, seq_steps = 0.0, 0
    for case in evalc:
        env = Environment(*case[1:4], finite_volume=fv)
        env.init()
        env.sync()
        w = int(np.ceil(max(1, int(np.ceil(ct / float(case[0].delta_t)))) / every)) * every
        t1 = time.perf_counter()
        n_s, _ = env.run_to_steady(thr, w, cap)
        env.sync()
        seq_s += time.perf_counter() - t1
        seq_steps += n_s
        env.close()
    # accuracy of the prediction against the plain run's steady state
    rho_p, vel_p = WS.macros(fin_p["pdf"])
    pr, pv = np.concatenate(rho), np.concatenate(vel)
    drho = np.concatenate([np.full(c[1].pdf.shape[0], s["rho_in"] - s["rho_out"]) for c, s in zip(evalc, espec)])
    total_s = warm_s + infer_s  # the prediction is part of the warm start's cost
    ecells = np.array([c[1].pdf.shape[0] for c in evalc])
    line = {"metric": f"time-to-steady @{thr:g} resid, warm vs plain (held-out porous squares)",
            "value": round(total_s, 3), "unit": "s", "higher_is_better": False,
            "warm_solve_s": round(warm_s, 3),
            "plain_s": round(plain_s, 3), "speedup_time": round(plain_s / total_s, 2),
            "speedup_solve_only": round(plain_s / warm_s, 2),
            "plain_one_at_a_time_s": round(seq_s, 3), "plain_one_at_a_time_steps": int(seq_steps),
            "speedup_batched_warm_vs_plain_one_at_a_time": round(seq_s / total_s, 2),
            "steps_plain": int(sp_.sum()), "steps_warm": int(sw.sum()),
            "speedup_steps": round(float(sp_.sum()) / max(float(sw.sum()), 1.0), 2),
            "converged_plain": int(np.sum(stp == 1)), "converged_warm": int(np.sum(stw == 1)),
            "frozen_plain": int(np.sum(stp == 3)), "frozen_warm": int(np.sum(stw == 3)),
            "restarts": int(restarted.sum()), "inference_s": round(infer_s, 3),
            "inference_pcg": {"iterations": pcg_iters, "rel_residual": pcg_rel},
            "pred_rel_err_rho": round(float(np.sqrt(np.mean(((pr - rho_p) / drho) ** 2))), 4),
            "pred_rel_err_u": round(float(np.linalg.norm(pv - vel_p) / np.linalg.norm(vel_p)), 4),
            "train": {"cases": len(samples), "cells": int(sum(s.n for s in samples)), "epochs": args.epochs,
                      "batch_cells": args.batch_cells, "loss": hist, "train_s": round(train_s, 2),
                      "data_s": round(data_s, 2), "data_converged": int(np.sum(st_t == 1)),
                      "data_frozen": int(np.sum(st_t == 3)),
                      "data_steps_median": int(np.median(steps_t))},
            "eval_cells": int(ecells.sum()),
            "n_gpus": 1, "dtype": "f32 solver; bf16 weights / f32 accumulate network (TF32 tensor cores)",
            "data": "synthetic",
            "config": {"workload": f"porous squares, 20-200 obstacles, porosity 0.75-0.85, {lo_cells}-{hi_cells} "
                                   f"cells, rho_in 1.01-1.05 / rho_out 0.95-0.99, Re 100, " + (
                                       "lattice units (mesh spacing ~1), tau = 3UL/Re + 1/2 with L the side in "
                                       "cells, the reference's update, dt = 0.5 min edge" if lattice else
                                       "unit square, tau 0.003, finite-volume update, dt = min(area/perimeter, tau)")
                                   + f", upwind; {args.train_cases} training + {args.eval_cases} held-out geometries",
                       "units": args.units, "check_every": every, "check_time": ct, "step_cap": cap,
                       "setup_s": round(setup_s, 1)}}
    print(json.dumps(line), flush=True)


def run_mpnn_epoch(args):
    """Training speed of the warm-start network: Adam epochs (forward, loss,
    backward, update) on one synthetic graph of --graph-cells cells with the
    network's four aggregation stages (a ring plus random chords, row-mean
    weights; count-aware 16x16 bins; 4x4 bin means), random features and
    targets.  Reports milliseconds per epoch (CUDA-synchronised wall time)."""
    import numpy as np
    import scipy.sparse as sp
    import torch

    from fvdbm_jax_gb300.warmstart import MPNN, NFEAT, Sample, _stage, grid_mean
    n = args.graph_cells
    rng = np.random.default_rng(1)
    i = np.arange(n)
    j1, j2 = (i + 1) % n, rng.integers(0, n, n)
    rows, cols = np.concatenate([i, j1, i, j2]), np.concatenate([j1, i, j2, i])
    M = sp.csr_matrix((np.ones(rows.size), (rows, cols)), shape=(n, n))
    M.data[:] = 1.0
    deg = np.asarray(M.sum(1)).reshape(-1)
    A = (sp.diags(1.0 / deg) @ M).tocsr().astype(np.float32)
    xy = rng.uniform(0, 1, (n, 2))
    P16, U16 = grid_mean(xy, 16, counted=True)
    P4, U4 = grid_mean(xy, 4)
    aggs = [[_stage(A)], [_stage(A)], [_stage(P16), _stage(U16)], [_stage(P4), _stage(U4)]]
    smp = Sample(rng.standard_normal((n, NFEAT)).astype(np.float32), aggs,
                 rng.standard_normal((n, 3)).astype(np.float32))
    net = MPNN(seed=0, scales=("mesh", "mesh", 16, 4))
    net.fit([smp], epochs=max(args.warmup, 1), lr=1e-3, log_every=1)
    torch.cuda.synchronize()
    E = args.steps
    t = time.perf_counter()
    net.fit([smp], epochs=E, lr=1e-3, log_every=E)
    torch.cuda.synchronize()
    el = time.perf_counter() - t
    print(json.dumps({"metric": "warm-start network training epoch", "value": round(el / E * 1e3, 3),
                      "unit": "ms/epoch", "higher_is_better": False, "epochs": E, "cells": n,
                      "dtype": "bf16 weights, tf32 tensor-core products, f32 accumulation", "data": "synthetic",
                      "config": {"workload": f"synthetic graph of {n} cells, 4 message-passing layers, hidden 64"}}),
          flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "batch":
        run_batch(args)
    elif args.workload == "warmstart":
        run_warmstart(args)
    elif args.workload == "mpnn_epoch":
        run_mpnn_epoch(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
