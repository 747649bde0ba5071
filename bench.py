#!/usr/bin/env python3
"""Benchmark of the irregular reduction on GB300: edges/s and the HBM roofline.

Workload (one "step" = one IrregularStart, i.e. one reduction over all edges):
the large moldyn-style Lennard-Jones reduction -- 4,194,304 nodes with float32
positions uniform-random in a periodic cube at the density that gives ~64
neighbours within the cutoff 2.5 (~134.2M half-list edges, float32 forces).
Inputs are synthetic and seeded; the edge list is built on the GPU by the
library's own neighbour builder.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Our arm prints one JSON line with
  value        edges/s with node data already resident in HBM (CUDA events on
               the launching stream over K steps);
  e2e          the same metric through the public C ABI with host buffers:
               every step copies float xyz positions from pinned host memory,
               reduces, and reads the float xyz forces back, steps pipelined
               (irr_step_pipelined: copies overlap the neighbouring steps'
               reductions); e2e_sequential makes the same calls one after
               another (irr_set_nodes, irr_step, irr_get_result);
  roofline     algorithmic bytes per step 8*E + 24*N (int32 endpoint pair per
               edge; float xyz read and force write per node) over the
               measured step time, against the measured HBM copy bandwidth;
  cpu_baseline the reference's CPU executor (ported, oracle/) on all host
               cores over a bounded sample of the same edge list;
  clocks       nvidia-smi samples taken during the timed region;
  force_err    a seeded sample of 2,000 nodes recomputed in FP64 by this
               file's own FP64 recomputation (fp64_forces): normwise, per node against
               the terms' magnitudes, and per result (p50 / p99 / max);
  md, batched, served
               the other configurations of the metric, measured in the same
               run (N = 1): the 1,048,576-atom MD loop, 512 batched instances
               in one graph-captured persistent launch per step against the
               same instances run one by one, and the served stream (p50 /
               p99 latency, throughput against serial execution, capacity);
  plugin       the same workload through the irregular.h plugin: the LJ law
               as an application's FP64 user map, compiled at run time.
`--impl reference` times that CPU executor alone (rank 0; other ranks exit).
With N > 1 (torchrun) the workload is split into N shards of the node order,
one per rank, with the halo positions exchanged over NCCL every step (strong
scaling, `--mode sharded`, the default), or every rank reduces its own
replica (`--mode replicas`, weak scaling); times are maxed over ranks.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "ipdps15-pattern_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

N_NODES = 4194304
FORCE_SAMPLE = 2000   # nodes whose results the FP64 recomputation covers
LAYOUTS = {"auto": 0, "csr": 1, "sliced": 2, "staged": 3}  # enum irr_layout
CUTOFF = 2.5
DENSITY = 64.0 / (4.0 / 3.0 * math.pi * CUTOFF ** 3)
SEED = 20260002
WORKLOAD = ("moldyn-style LJ irregular reduction: 4,194,304 nodes, float32 positions "
            "uniform-random in a periodic cube, ~64 neighbours within cutoff 2.5 "
            "(~134.2M half-list edges), float32 forces")
METRIC = "edges/s"


def workload_name(n: int) -> str:
    return WORKLOAD if n == N_NODES else WORKLOAD.replace("4,194,304", f"{n:,}") + \
        " (reduced size)"


def positions(n: int, seed: int = SEED):
    rng = np.random.Generator(np.random.PCG64(seed))
    side = np.float32((n / DENSITY) ** (1.0 / 3.0))
    pos = (rng.random((n, 3), dtype=np.float32) * side).astype(np.float32)
    pos[pos >= side] = 0.0
    return pos, side


def measured_hbm_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def ncu_traffic(key: str):
    """Bytes per launch from the committed ncu summary (profiles/ncu_traffic.txt)."""
    path = os.path.join(ROOT, "profiles", "ncu_traffic.txt")
    try:
        for line in open(path):
            parts = line.split()
            if len(parts) >= 2 and parts[0] == key:
                return float(parts[1])
    except OSError:
        pass
    return None


def fp64_forces(pos32, edges, side: float, cutoff: float, periodic: bool = True):
    """FP64 recomputation for the force-error fields: the LJ law d (r^-14 - r^-8/2) of
    the reference's `map` (moldyn/irregular.h:47-78) on the float positions
    widened to double, minimum image in a cube of side `side`, applied when
    r^2 < cutoff^2, +f to idx0 and -f to idx1.  Returns per node the forces,
    the per-component sum of the terms' magnitudes |d_c| (r^-14 + r^-8/2), and
    the sum of each term's largest component."""
    n = pos32.shape[0]
    p = np.asarray(pos32, np.float64)
    i, j = edges[:, 0].astype(np.int64), edges[:, 1].astype(np.int64)
    d = p[i] - p[j]
    if periodic:
        half = 0.5 * side
        d = np.where(d < -half, d + side, d)
        d = np.where(d > half, d - side, d)
    rd = (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]
    inside = rd < cutoff * cutoff
    with np.errstate(divide="ignore", invalid="ignore"):
        r = np.where(inside, 1.0 / np.where(inside, rd, 1.0), 0.0)
    r4 = (r * r) * (r * r)
    s = r4 * (r * r * r) - 0.5 * r4
    sa = r4 * (r * r * r) + 0.5 * r4
    fe = d * s[:, None]
    ae = np.abs(d) * sa[:, None]
    f = np.zeros((n, 3))
    sabs = np.zeros((n, 3))
    sinf = np.zeros(n)
    np.add.at(f, i, fe)
    np.add.at(f, j, -fe)
    np.add.at(sabs, i, ae)
    np.add.at(sabs, j, ae)
    m = np.abs(fe).max(axis=1)
    np.add.at(sinf, i, m)
    np.add.at(sinf, j, m)
    return f, sabs, sinf


def incident(edges, n: int, sample):
    sel = np.zeros(n, bool)
    sel[sample] = True
    return edges[sel[edges[:, 0]] | sel[edges[:, 1]]]


def force_err(f, f64, sabs, sinf) -> dict:
    """Errors of results f against the FP64 recomputation, on the nodes given:
    normwise max|df| / max|f64|; per node and component |df| / sabs (sabs: the
    terms' magnitudes); and per result |df|inf / max(|f64|inf, 2^-10 sinf) at
    the median, 99th percentile and worst node."""
    f = np.asarray(f, np.float64).reshape(-1, 3)
    g = np.asarray(f64, np.float64).reshape(-1, 3)
    d = np.abs(f - g)
    with np.errstate(divide="ignore", invalid="ignore"):
        pern = np.where(sabs > 0, d / np.where(sabs > 0, sabs, 1.0), np.where(d > 0, np.inf, 0.0))
        den = np.maximum(np.abs(g).max(axis=1), np.asarray(sinf) / 1024.0)
        res = np.where(den > 0, d.max(axis=1) / np.where(den > 0, den, 1.0), 0.0)
    return {"normwise": float(d.max() / max(np.abs(g).max(), 1e-300)),
            "per_node_S": float(pern.max()),
            "per_result": {"p50": float(np.percentile(res, 50)), "p99": float(np.percentile(res, 99)),
                           "max": float(res.max())},
            "nodes": int(g.shape[0]),
            "metric_note": "per_result = |df|inf / max(|f64|inf, 2^-10 sum_e |f_e|inf)"}


def merge_err(errs):
    """The worst of several force_err results."""
    if not errs:
        return None
    return {"normwise": max(e["normwise"] for e in errs),
            "per_node_S": max(e["per_node_S"] for e in errs),
            "per_result": {k: max(e["per_result"][k] for e in errs) for k in ("p50", "p99", "max")},
            "nodes": sum(e["nodes"] for e in errs), "metric_note": errs[0]["metric_note"]}


class ClockSampler:
    """nvidia-smi clock/throttle samples while the timed region runs."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def dist_init(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    return rank, world, local


def max_over_ranks(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world: int):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


# Edges per mutex grab of the CPU executor: CPU_BLOCK_SIZE of the reference's
# miniMD copy (miniMD/irregular/parameters.h:7); the moldyn copy's 1,000,000
# would leave most cores idle on a bounded sample of a few million edges.
CPU_CHUNK = 100000


def cpu_port_rate(pos, edges_sample, side, seconds: float, threads: int):
    """Times the ported reference executor (oracle/) over a bounded edge sample."""
    from oracle import oracle as O

    p = O.lj_param(CUTOFF * CUTOFF, float(side), True)
    ex = O.Executor(pos.shape[0], threads)
    ex.run(pos, edges_sample, p, chunk=CPU_CHUNK)  # warm-up pass (untimed)
    total, passes = 0.0, 0
    while total < seconds or passes < 1:
        total += ex.run(pos, edges_sample, p, chunk=CPU_CHUNK)
        passes += 1
    ex.close()
    return edges_sample.shape[0] * passes / total, passes


def run_reference(args, rank, world):
    """The reference arm: its CPU executor (ported) on all host cores."""
    if rank != 0:
        return 0
    from oracle import oracle as O

    threads = os.cpu_count() or 1
    pos, side = positions(args.nodes)
    rows = 131072  # rows [0, 131072) of the half list: ~4.2M edges per step
    sample = O.neighbor_half_list_rows(pos, float(side), np.float32(CUTOFF * CUTOFF), 0, rows)
    p = O.lj_param(CUTOFF * CUTOFF, float(side), True)
    ex = O.Executor(pos.shape[0], threads)
    for _ in range(args.warmup):
        ex.run(pos, sample, p, chunk=CPU_CHUNK)
    total = 0.0
    for _ in range(args.steps):
        total += ex.run(pos, sample, p, chunk=CPU_CHUNK)
    ex.close()
    rate = sample.shape[0] * args.steps / total
    desc = (f"edges of rows [0, {rows}) of the workload's half list ({sample.shape[0]} edges) "
            f"per step, {threads} threads, {CPU_CHUNK}-edge chunks, table re-initialisation "
            f"excluded")
    line = {
        "impl": "reference", "metric": METRIC, "value": rate, "unit": "edges/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64 per edge, f32 accumulate", "data": "synthetic",
        "config": {"workload": workload_name(args.nodes), "nodes": args.nodes,
                   "edges_per_step": int(sample.shape[0]),
                   "sample": f"rows [0, {rows}) of the workload's half list, every step; the "
                             f"rate is the metric (edges/s), so the sample stands for the "
                             f"whole list",
                   "chunk_edges": CPU_CHUNK,
                   "chunk_source": "CPU_BLOCK_SIZE of the reference's miniMD copy "
                                   "(miniMD/irregular/parameters.h:7); the moldyn copy's "
                                   "1,000,000 would leave most threads idle on the sample",
                   "kind": "port",
                   "why_port": "the reference's CPU code, compiled from its own sources, needs "
                               "the reference tree at run time, which a deployment of this repository does not "
                               "include, and its "
                               "1,048,577-bucket table overflows (its insert then spins) at "
                               "4,194,304 nodes",
                   "threads": threads,
                   "executor": "reference CPU executor (port of compute_cpu + Cobject)"},
        "cpu_baseline": {"value": rate, "unit": "edges/s", "cores": threads, "kind": "port",
                         "sample": desc},
        "e2e": {"value": rate, "unit": "edges/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def time_steps(h, stream, steps: int):
    import torch
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        h.step()
    e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1)


def run_ours(args, rank, world, local):
    import torch

    import irregular_gb300 as irr

    torch.cuda.set_device(local)
    dev = local
    stream = torch.cuda.Stream(device=dev)
    pos, side = positions(args.nodes)
    n = pos.shape[0]
    edges = irr.neighbor_build(pos, float(side), CUTOFF * CUTOFF, device=dev,
                               stream=stream.cuda_stream)
    E = edges.count

    def handle(**cfg):
        h = irr.Handle(irr.default_config(device=dev, map_idx=irr.IRR_MAP_LJ_MOLDYN, **cfg))
        h.set_stream(stream.cuda_stream)
        h.set_params(irr.moldyn_params(float(side), CUTOFF))
        h.set_edges(edges)
        h.set_nodes(pos, 12)
        h.init()
        return h

    h = handle(exec=irr.IRR_EXEC_PARTITIONED, layout=LAYOUTS[args.layout])
    for _ in range(args.warmup):
        h.step()
    h.sync()
    barrier(world)
    torch.cuda.synchronize()
    clocks = ClockSampler(dev)
    clocks.start()
    ms = time_steps(h, stream, args.steps)
    clk = clocks.stop()
    h.sync()
    barrier(world)
    ms = max_over_ranks(ms, world)
    step_s = ms / 1e3 / args.steps
    value = E * args.steps * world / (ms / 1e3)
    if args.legs == "value":
        h.close()
        edges.close()
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": "edges/s",
                              "legs": "value only", "nodes": n, "edges": E,
                              "layout": args.layout, "ms_per_step": ms / args.steps}), flush=True)
        return 0

    # force error of the timed configuration on a seeded node sample (FP64 recomputation)
    err = None
    if rank == 0:
        f_gpu = h.get_result(elm_size=12)
        host_edges = edges.to_host()
        smp = np.sort(np.random.Generator(np.random.PCG64(SEED + 1)).choice(
            n, min(n, FORCE_SAMPLE), replace=False))
        g, sabs, sinf = fp64_forces(pos, incident(host_edges, n, smp), float(side), CUTOFF)
        err = force_err(f_gpu[smp], g[smp], sabs[smp], sinf[smp])
        del host_edges

    # e2e through the public API with host buffers (pinned)
    pin_in = torch.empty((n, 3), dtype=torch.float32, pin_memory=True)
    pin_in.numpy()[:] = pos
    pin_out = torch.empty((n, 3), dtype=torch.float32, pin_memory=True)
    out_np = pin_out.numpy()
    e2e_steps = max(1, min(args.steps, 200))
    for _ in range(3):
        h.set_nodes(pin_in.numpy(), 12)
        h.step()
        h.get_result(out_np, 12)
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        h.set_nodes(pin_in.numpy(), 12)
        h.step()
        h.get_result(out_np, 12)
    e2e_s = max_over_ranks(time.perf_counter() - t0, world)
    e2e_seq = E * e2e_steps * world / e2e_s
    # the same, pipelined (irr_step_pipelined): the upload of step k+1 and the
    # read-back of step k-1 overlap the reduction of step k
    for _ in range(3):
        h.step_pipelined(pin_in.numpy(), out_np, 12, 12)
    h.pipeline_sync()
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        h.step_pipelined(pin_in.numpy(), out_np, 12, 12)
    h.pipeline_sync()
    e2e_s = max_over_ranks(time.perf_counter() - t0, world)
    e2e = E * e2e_steps * world / e2e_s

    # the same reduction in the caller's random node order, for comparison
    variants = {}
    vsteps = max(3, min(args.steps, 50))
    for name, cfg in (("plain_atomics_random_order", dict(exec=irr.IRR_EXEC_PLAIN)),
                      ("partitioned_random_order", dict(exec=irr.IRR_EXEC_PARTITIONED, reorder=0))):
        hv = handle(**cfg)
        for _ in range(3):
            hv.step()
        hv.sync()
        vms = max_over_ranks(time_steps(hv, stream, vsteps), world)
        variants[name] = E * vsteps * world / (vms / 1e3)
        hv.close()

    info = h.info()
    alg_bytes = 8.0 * E + 24.0 * n
    achieved = alg_bytes / step_s / 1e9
    peak, peak_kind = measured_hbm_peak()
    kernel = "halo_kernel" if info.layout == LAYOUTS["staged"] else "tiled_kernel"
    traffic = ncu_traffic(f"{kernel}_moldyn_4M") if n == N_NODES else None
    roofline = {"bound": "hbm", "kernel": kernel, "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": traffic,
                "peak_source": f"{peak_kind} (hbm_gbs, MEASURED_PEAKS.json)",
                "algorithmic_bytes_per_step": alg_bytes}

    cpu = None
    if rank == 0 and world == 1:
        threads = os.cpu_count() or 1
        sample = edges.to_host(count=min(E, 8 * 1024 * 1024))
        rate, passes = cpu_port_rate(pos, sample, side, args.cpu_seconds, threads)
        cpu = {"value": rate, "unit": "edges/s", "cores": threads, "kind": "port",
               "sample": f"first {sample.shape[0]} edges of the workload's half list, "
                         f"{passes} timed passes, {CPU_CHUNK}-edge chunks, table "
                         f"re-initialisation excluded"}
    edges.close()

    line = {
        "metric": METRIC, "value": value, "unit": "edges/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded uniform-random positions; edge list built on the GPU)",
        "config": {"workload": workload_name(n), "nodes": n, "edges": E,
                   "exec": "partitioned: Hilbert-ordered nodes, " + {0: "plain", 1: "CSR", 2: "sliced",
                                                                      3: "staged (halo)"}[info.layout]
                           + " layout, owner-computes kernel",
                   "lanes_per_row": info.lanes_per_row, "stage_smem": info.stage_smem,
                   "l2": "inputs larger than L2 (1.07 GB entry stream read every step)",
                   "parallelism": f"replicas x{world}"},
        "roofline": roofline,
        "e2e": {"value": e2e, "unit": "edges/s", "h2d_bytes_per_step": 12 * n,
                "d2h_bytes_per_step": 12 * n, "steps": e2e_steps,
                "mode": "pipelined (irr_step_pipelined): every step uploads float xyz positions "
                        "from pinned host memory, reduces and reads float xyz forces back; the "
                        "upload of step k+1 and the read-back of step k-1 overlap the reduction "
                        "of step k (independent inputs: a served stream, a sweep)"},
        "e2e_sequential": {"value": e2e_seq, "unit": "edges/s", "h2d_bytes_per_step": 12 * n,
                           "d2h_bytes_per_step": 12 * n, "steps": e2e_steps,
                           "mode": "irr_set_nodes, irr_step, irr_get_result one after another "
                                   "(a dependent loop such as MD: nothing to overlap)"},
        "clocks": clk,
        "gpu_launches": args.steps,
        "variants_edges_per_s": variants,
    }
    if err is not None:
        line["force_err"] = err
    if cpu is not None:
        line["cpu_baseline"] = cpu
    h.close()
    if rank == 0 and world == 1 and args.legs == "all":
        # the other configurations of the metric, measured in the same run
        line["md"] = run_md(args)
        line["batched"] = run_batched(args)
        line["served"] = run_served(args)
        line["plugin"] = run_plugin(args, pos, side)
    elif args.legs == "all":
        line["legs"] = "md / batched / served run at N = 1 only"
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def run_sharded(args, rank, world, local):
    """Strong scaling: the one workload split into `world` shards of the
    partition's execution order (sharding.plan: equal entry counts), one per
    rank, each reduced by a shard handle (irr_set_shard) after a per-step halo
    exchange of float4 positions over NCCL point-to-point (sharding.
    HaloExchange) -- the reference's per-rank view and its halo exchange
    (moldyn/irregular/partition_view.cpp:44-282, 285-435).  value = all edges
    / the slowest rank's time for the step (exchange + reduction)."""
    import torch

    import irregular_gb300 as irr
    import sharding

    torch.cuda.set_device(local)
    dev = local
    stream = torch.cuda.Stream(device=dev)
    pos, side = positions(args.nodes)
    n = pos.shape[0]
    edges = irr.neighbor_build(pos, float(side), CUTOFF * CUTOFF, device=dev,
                               stream=stream.cuda_stream)
    E = edges.count
    params = irr.moldyn_params(float(side), CUTOFF)
    # the whole problem's partition (every rank computes the same one)
    hw = irr.Handle(irr.default_config(device=dev, map_idx=irr.IRR_MAP_LJ_MOLDYN,
                                       exec=irr.IRR_EXEC_PARTITIONED))
    hw.set_stream(stream.cuda_stream)
    hw.set_params(params)
    hw.set_edges(edges)
    hw.set_nodes(pos, 12)
    hw.init()
    perm, row_off, col = hw.partition()
    hw.close()
    edges.close()
    shards = sharding.plan(row_off, col, world)
    lp = sharding.local_problem(shards[rank], row_off, col)
    pos4 = np.zeros((n, 4), np.float32)
    pos4[:, :3] = pos[perm]
    del pos
    n_local = lp.nodes.shape[0]
    loc_np = np.ascontiguousarray(pos4[lp.nodes])
    h = irr.Handle(irr.default_config(device=dev, map_idx=irr.IRR_MAP_LJ_MOLDYN,
                                      exec=irr.IRR_EXEC_PARTITIONED, reorder=0,
                                      layout=LAYOUTS[args.layout]))
    h.set_stream(stream.cuda_stream)
    h.set_params(params)
    h.set_shard(lp.own_lo, lp.own_hi)
    h.set_edges(lp.edges)
    h.set_nodes(loc_np, 16)
    h.init()
    loc = torch.from_numpy(loc_np).to(f"cuda:{dev}")
    hx = sharding.HaloExchange(lp, f"cuda:{dev}")
    # a collective first, so that the exchange's batched point-to-point calls
    # are not the group's first NCCL operation (which every rank must join)
    barrier(world)
    below = loc[:lp.own_lo]
    above = loc[lp.own_hi:]

    def one_step():
        hx.run(loc)
        if lp.own_lo > 0:
            h.set_nodes_range(below, 0, 16)
        if lp.own_hi < n_local:
            h.set_nodes_range(above, lp.own_hi, 16)
        h.step()

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            one_step()
        h.sync()
        barrier(world)
        torch.cuda.synchronize()
        clocks = ClockSampler(dev)
        clocks.start()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            one_step()
        e1.record(stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        clk = clocks.stop()
        h.sync()
    barrier(world)
    ms = max_over_ranks(ms, world)
    value = E * args.steps / (ms / 1e3)
    # force error of this rank's owned rows on a seeded sample (FP64 recomputation)
    err = None
    if rank == 0:
        f_own = h.get_result(elm_size=12)
        own = np.arange(lp.lo, lp.hi)
        smp = np.sort(np.random.Generator(np.random.PCG64(SEED + 3)).choice(
            own, min(own.shape[0], FORCE_SAMPLE), replace=False))
        rows = np.repeat(smp, (row_off[smp + 1] - row_off[smp]).astype(np.int64))
        cols = np.concatenate([col[row_off[r]:row_off[r + 1]] for r in smp])
        insmp = np.zeros(n, bool)
        insmp[smp] = True
        keep = ~insmp[cols] | (rows < cols)  # a pair of two sampled rows once
        inc = np.stack([rows[keep], cols[keep]], axis=1)
        g, sabs, sinf = fp64_forces(pos4[:, :3], inc, float(side), CUTOFF)
        err = force_err(f_own[smp - lp.lo], g[smp], sabs[smp], sinf[smp])
    halo = max_over_ranks(float(n_local - (lp.hi - lp.lo)), world)
    h.close()
    line = {
        "metric": METRIC, "value": value, "unit": "edges/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "strong", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded uniform-random positions; edge list built on the GPU)",
        "config": {"workload": workload_name(n), "nodes": n, "edges": E,
                   "exec": "sharded: equal-entry ranges of the Hilbert order, one shard handle "
                           "per rank, halo positions exchanged every step (NCCL send/recv)",
                   "max_halo_nodes_per_rank": int(halo),
                   "l2": "inputs larger than L2 (1.07 GB entry stream read every step)",
                   "parallelism": f"shards x{world}"},
        "clocks": clk,
        "gpu_launches": args.steps,
    }
    if err is not None:
        line["force_err"] = err
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def run_plugin(args, pos, side):
    """The irregular.h plugin path on the same workload: the LJ law written
    as an application's FP64 user map (tests/plugin/lj/irregular.h, the
    reference's irregular.h form), compiled through the compat shim
    (compat/irregular/irr_user_map.cu, one map inlined, compensated float
    sums) and run by a partitioned handle (irr_set_user_map).  Returns the
    leg's JSON object, or its reason for being unavailable."""
    import ctypes as C

    import irregular_gb300 as irr
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from plugin_build import build_plugins

    out = {"leg": "plugin", "map": "LJ as an FP64 user map (irregular.h form), IRR_PLUGIN_INLINE_MAP, "
                                   "IRR_PLUGIN_COMPENSATED"}
    lib_path = os.path.join(tempfile.mkdtemp(), "libplugin_lj.so")
    try:
        build_plugins({"lj": (os.path.join(ROOT, "tests", "plugin", "lj"), lib_path, True,
                              ("IRR_PLUGIN_INLINE_MAP=lj_box", "IRR_PLUGIN_COMPENSATED"), True)})
    except Exception as e:  # no nvcc on the host running the bench
        out["unavailable"] = str(e).splitlines()[0][:200]
        return out
    lib = C.CDLL(lib_path)
    fn = C.cast(lib.irr_compat_user_launch, C.c_void_p).value
    n = pos.shape[0]
    edges = irr.neighbor_build(pos, float(side), CUTOFF * CUTOFF)
    E = edges.count
    h = irr.Handle(irr.default_config(exec=irr.IRR_EXEC_PARTITIONED))
    h.set_user_map(fn, 12, 1)
    h.set_params(np.array([float(side), CUTOFF], np.float64))
    h.set_edges(edges)
    h.set_nodes(pos.astype(np.float64), 24)
    h.init()
    for _ in range(3):
        h.step()
    h.sync()
    steps = 20
    t0 = time.perf_counter()
    for _ in range(steps):
        h.step()
    h.sync()
    dt = (time.perf_counter() - t0) / steps
    f = h.get_result(elm_size=12)
    host_edges = edges.to_host()
    smp = np.sort(np.random.Generator(np.random.PCG64(SEED + 1)).choice(n, min(n, FORCE_SAMPLE),
                                                                        replace=False))
    g, sabs, sinf = fp64_forces(pos, incident(host_edges, n, smp), float(side), CUTOFF)
    out.update({"ms_per_step": 1e3 * dt, "edges_per_s": E / dt, "steps": steps,
                "timing": "host wall clock around synchronised steps",
                "force_err": force_err(f[smp], g[smp], sabs[smp], sinf[smp]),
                "note": "FP64-pipe bound: two FP64 law evaluations per edge; the built-in FP32 law "
                        "is the fast path"})
    h.close()
    edges.close()
    return out


def run_batched(args):
    """Config 4: 512 instances, sizes log-uniform in [1,024, 262,144] atoms, each
    uniform-random in its own periodic box at density 0.8442, cutoff 2.5; one
    persistent launch per step (CUDA graph, autotuned shape) vs the same
    instances one by one through the single-instance paths.  Returns the leg's
    JSON object."""
    import torch

    import irregular_gb300 as irr
    import workloads as W

    dev = 0
    torch.cuda.set_device(dev)
    stream = torch.cuda.Stream(device=dev)
    rng = np.random.Generator(np.random.PCG64(SEED + 2))
    count = args.instances
    sizes = np.floor(np.exp(rng.uniform(math.log(1024), math.log(262144), count))).astype(int)
    checked = {int(np.argmax(sizes))}
    checked |= set(int(k) for k in np.random.Generator(np.random.PCG64(SEED + 3)).choice(
        count, min(3, count), replace=False))
    t_setup = time.perf_counter()
    part, plain, keep = [], [], {}
    E = 0
    for k, n in enumerate(sizes):
        pos, side = W.random_box(int(n), 0.8442, SEED + 100 + k)
        edges = irr.neighbor_build(pos, side, CUTOFF * CUTOFF, device=dev, stream=stream.cuda_stream)
        E += edges.count
        if k in checked:
            keep[k] = (pos, side, edges.to_host())
        for mode, bucket in ((irr.IRR_EXEC_PARTITIONED, part), (irr.IRR_EXEC_PLAIN, plain)):
            h = irr.Handle(irr.default_config(device=dev, map_idx=irr.IRR_MAP_LJ_MOLDYN, exec=mode))
            h.set_stream(stream.cuda_stream)
            h.set_params(irr.moldyn_params(side, CUTOFF))
            h.set_edges(edges)
            h.set_nodes(pos, 12)
            h.init()
            bucket.append(h)
        edges.close()
    b = irr.Batch(dev)
    b.set_stream(stream.cuda_stream)
    for h in part:
        b.add(h)
    b.finalize(autotune=True)
    b.capture()
    setup_s = time.perf_counter() - t_setup
    for _ in range(args.warmup):
        b.step()
    b.sync()
    ms_batch = time_steps(b, stream, args.batch_steps)
    b.sync()
    errs = []
    for k, (pos, side, host_edges) in sorted(keep.items()):
        f_gpu = part[k].get_result(elm_size=12)
        nk = pos.shape[0]
        smp = np.sort(np.random.Generator(np.random.PCG64(SEED + 1000 + k)).choice(
            nk, min(nk, 1000), replace=False))
        g, sabs, sinf = fp64_forces(pos, incident(host_edges, nk, smp), side, CUTOFF)
        errs.append(force_err(f_gpu[smp], g[smp], sabs[smp], sinf[smp]))

    class Serial:
        def __init__(self, hs):
            self.hs = hs

        def step(self):
            for h in self.hs:
                h.step()

    for _ in range(2):
        Serial(part).step()
    ms_part = time_steps(Serial(part), stream, args.batch_steps)
    ser_steps = max(3, args.batch_steps // 10)
    Serial(plain).step()
    ms_plain = time_steps(Serial(plain), stream, ser_steps)
    torch.cuda.synchronize()
    inf = b.info()
    batched = E * args.batch_steps / (ms_batch / 1e3)
    serial_part = E * args.batch_steps / (ms_part / 1e3)
    serial_plain = E * ser_steps / (ms_plain / 1e3)
    alg = 8.0 * E + 24.0 * float(sizes.sum())
    peak = measured_hbm_peak()[0]
    achieved = alg / (ms_batch / 1e3 / args.batch_steps) / 1e9
    line = {"leg": "batched", "metric": "aggregate edges/s", "unit": "edges/s",
            "instances": int(count), "nodes": int(sizes.sum()), "edges_per_step": int(E),
            "steps": args.batch_steps, "batched": batched,
            "serial_partitioned": serial_part, "serial_plain": serial_plain,
            "speedup_vs_serial_partitioned": batched / serial_part,
            "speedup_vs_serial_plain": batched / serial_plain,
            "ms_per_step": {"batched": ms_batch / args.batch_steps,
                            "serial_partitioned": ms_part / args.batch_steps,
                            "serial_plain": ms_plain / ser_steps},
            "shape": {"lanes_per_row": inf.lanes_per_row, "rows_per_item": inf.block_nodes,
                      "work_items": int(inf.num_items), "cuda_graph": bool(inf.graph)},
            "setup_s": setup_s,
            "roofline": {"algorithmic_bytes_per_step": alg, "achieved_GBs": achieved,
                         "peak_GBs": peak, "frac": achieved / peak},
            "force_err": merge_err(errs),
            "force_err_instances": sorted(int(k) for k in keep),
            "data": "synthetic (seeded sizes and positions; lists built on the GPU)"}
    b.close()
    for h in part + plain:
        h.close()
    return line


def run_md(args):
    """Config 3: miniMD-style LJ MD, FCC 4 x 64^3 = 1,048,576 atoms at density
    0.8442, Maxwell velocities at T = 1.44, cutoff 2.5, skin 0.3, rebuild every
    20 steps, velocity Verlet dt = 0.005, 1000 steps; FP32 forces, FP64
    integration and energies.  Returns the leg's JSON object."""
    import torch

    import irregular_gb300 as irr
    import workloads as W

    torch.cuda.set_device(0)
    stream = torch.cuda.Stream()
    pos, side = W.fcc_lattice(64, 64, 64, 0.8442)
    vel = W.maxwell_velocities(pos.shape[0], 1.44, SEED + 3)
    md = irr.MD(pos, vel, side, dt=0.005, cutforce=2.5, skin=0.3, rebuild_every=20)
    md.set_stream(stream.cuda_stream)
    ke0, pe0, vir0 = md.energy()
    md.run(20)  # warm-up (includes one rebuild)
    ke_w, pe_w, _ = md.energy()
    steps = args.md_steps
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    md.run(steps)
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    ke1, pe1, vir1 = md.energy()
    n = pos.shape[0]
    info = md.info()
    # forces at the end against the FP64 recomputation (x48: the MD's force units)
    gp, _ = md.state()
    f_gpu = md.forces()
    p32 = gp.astype(np.float32)
    lst = irr.neighbor_build(p32, float(np.float32(side)), 2.8 ** 2)
    host_edges = lst.to_host()
    lst.close()
    smp = np.sort(np.random.Generator(np.random.PCG64(SEED + 4)).choice(n, FORCE_SAMPLE,
                                                                      replace=False))
    g, sabs, sinf = fp64_forces(p32, incident(host_edges, n, smp), side, 2.5)
    err = force_err(f_gpu[smp], 48.0 * g[smp], 48.0 * sabs[smp], 48.0 * sinf[smp])
    line = {"leg": "md", "metric": "ms per MD step", "unit": "ms", "atoms": n,
            "steps": steps, "ms_per_step": ms / steps, "atom_steps_per_s": n * steps / (ms / 1e3),
            "pairs_in_list": int(info.num_edges), "rebuilds": int(info.rebuilds),
            "energy_per_atom": {"start": (ke0 + pe0) / n, "after_warmup": (ke_w + pe_w) / n,
                                "end": (ke1 + pe1) / n},
            "energy_drift_rel": abs((ke1 + pe1) - (ke_w + pe_w)) / abs(ke_w + pe_w),
            "temperature_end": 2.0 * ke1 / (3 * n - 3),
            "pressure_end": (2.0 * ke1 / 3.0 + vir1 / 3.0) / side ** 3,
            "force_err": err,
            "precision": "FP32 per-edge forces (compensated sums), FP64 integration and energies",
            "data": "synthetic (miniMD FCC lattice, seeded Maxwell velocities)"}
    md.close()
    return line


# Served capacity: the p99 job latency a rate must keep to count as sustained.
P99_BOUND_S = 1.0
CAPACITY_RATES = (200.0, 400.0, 800.0, 1600.0, 3200.0, 1e9)


def run_served(args):
    """Config 5: Poisson arrivals at 200 jobs/s, sizes log-uniform in
    [2,048, 2,097,152] atoms, density 0.8442, cutoff 2.5, 50 velocity-Verlet
    steps each, 120 GB admission budget; continuous batching vs serial
    execution (one job at a time through the partitioned force kernel) and
    serial plain execution (one job at a time, every force by the plain
    edge-parallel kernel), all admitting in arrival order, and continuous
    batching admitting the smallest waiting job first.  Then the capacity: the
    same stream offered at rising rates (1e9/s: every job waiting at t = 0),
    the highest rate whose p99 latency stays within P99_BOUND_S, and the
    throughput there against serial plain execution's at the same rate.
    Returns the leg's JSON object."""
    import irregular_gb300 as irr

    out = {"leg": "served", "jobs": args.jobs, "arrival_rate_per_s": 200.0,
           "steps_per_job": 50, "budget_GB": 120.0,
           "data": "synthetic (seeded arrivals and sizes; FCC + jitter, Maxwell velocities)"}
    # untimed warm-up: a long-running server has its memory pool grown and its
    # kernels loaded; without it the first measured schedule would pay for both
    irr.serve(num_jobs=max(1, args.jobs // 4), mode=irr.IRR_SERVE_CONTINUOUS, arrival_rate=200.0,
              steps_per_job=50, budget_bytes=120e9, seed=SEED + 6)

    def one(mode, policy, rate):
        st, _ = irr.serve(num_jobs=args.jobs, mode=mode, policy=policy, arrival_rate=rate,
                          steps_per_job=50, budget_bytes=120e9, seed=SEED + 5)
        return {"p50_ms": st.p50_ms, "p99_ms": st.p99_ms, "mean_ms": st.mean_ms,
                "max_ms": st.max_ms, "makespan_s": st.makespan_s,
                "edges_per_s": st.edges_per_s, "jobs_done": int(st.jobs_done),
                "max_resident": int(st.max_resident)}

    runs = ((irr.IRR_SERVE_CONTINUOUS, irr.IRR_SERVE_FIFO, "continuous"),
            (irr.IRR_SERVE_SERIAL, irr.IRR_SERVE_FIFO, "serial"),
            (irr.IRR_SERVE_SERIAL_PLAIN, irr.IRR_SERVE_FIFO, "serial_plain"),
            (irr.IRR_SERVE_CONTINUOUS, irr.IRR_SERVE_SJF, "continuous_sjf"))
    for mode, policy, name in runs:
        out[name] = one(mode, policy, 200.0)
    out["speedup_edges_per_s"] = out["continuous"]["edges_per_s"] / out["serial"]["edges_per_s"]
    out["speedup_vs_serial_plain"] = out["continuous"]["edges_per_s"] / out["serial_plain"]["edges_per_s"]
    if args.capacity:
        sweep = []
        for rate in CAPACITY_RATES:
            r = one(irr.IRR_SERVE_CONTINUOUS, irr.IRR_SERVE_FIFO, rate)
            r["rate_per_s"] = rate
            sweep.append(r)
        ok = [r for r in sweep if r["p99_ms"] <= 1e3 * P99_BOUND_S]
        best = max(ok, key=lambda r: r["rate_per_s"]) if ok else None
        cap = {"p99_bound_s": P99_BOUND_S, "sweep": sweep,
               "sustained_rate_per_s": best["rate_per_s"] if best else None}
        if best:
            plain = one(irr.IRR_SERVE_SERIAL_PLAIN, irr.IRR_SERVE_FIFO, best["rate_per_s"])
            cap["at_sustained_rate"] = {"continuous_edges_per_s": best["edges_per_s"],
                                        "continuous_p99_ms": best["p99_ms"],
                                        "serial_plain_edges_per_s": plain["edges_per_s"],
                                        "serial_plain_p99_ms": plain["p99_ms"],
                                        "speedup_vs_serial_plain": best["edges_per_s"] / plain["edges_per_s"]}
        out["capacity"] = cap
    return out


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--nodes", type=int, default=N_NODES,
                    help="workload size (default: the full 4,194,304-node workload; "
                         "smaller sizes are for profiling captures)")
    ap.add_argument("--legs", choices=["all", "value", "batched", "md", "served"], default="all",
                    help="'value': only the device-resident timed leg (profiling); "
                         "'batched' / 'md' / 'served': the other configurations' measurements")
    ap.add_argument("--instances", type=int, default=512)
    ap.add_argument("--md-steps", type=int, default=1000)
    ap.add_argument("--jobs", type=int, default=200)
    ap.add_argument("--batch-steps", type=int, default=200)
    ap.add_argument("--layout", choices=sorted(LAYOUTS), default="auto",
                    help="entry layout of the timed partitioned handle (irr_config.layout)")
    ap.add_argument("--capacity", type=int, default=1,
                    help="1: the served leg also sweeps the arrival rate for its capacity")
    ap.add_argument("--mode", choices=["auto", "replicas", "sharded"], default="auto",
                    help="N > 1: 'sharded' (default) splits the one workload across the ranks "
                         "with a halo exchange per step (strong scaling); 'replicas' runs one "
                         "workload per rank (weak scaling).  N = 1: 'sharded' runs the shard "
                         "path with one shard")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        world = int(os.environ.get("WORLD_SIZE", "1"))
        rank = int(os.environ.get("RANK", "0"))
        return run_reference(args, rank, world)
    if args.legs in ("batched", "md", "served"):
        leg = {"batched": run_batched, "md": run_md, "served": run_served}[args.legs](args)
        print(json.dumps(leg), flush=True)
        return 0
    rank, world, local = dist_init(args)
    sharded = args.mode == "sharded" or (args.mode == "auto" and world > 1)
    rc = (run_sharded if sharded else run_ours)(args, rank, world, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return rc


if __name__ == "__main__":
    sys.exit(main())
