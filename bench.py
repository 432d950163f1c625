#!/usr/bin/env python
"""PageRank GTEPS of GraphMP's shard-wise gather-apply on one GB300.

Workload (default): seeded R-MAT, scale 24, edge factor 16 (a,b,c,d =
.57/.19/.19/.05, self-loops and duplicates removed), 256 edge-balanced
destination-range shards; one step = one PageRank run of 20 supersteps with
the reference's semantics (comp_pagerank<float>, GraphMP/app/pagerank.cpp).
value = 20 * E / step time, in GTEPS, inputs resident in HBM; e2e = the same
metric through the C ABI with host buffers (load + run + read-back per step).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gx|reference]

Under torchrun (N > 1) every rank runs an independent replica on its own GPU
(the path is single-GPU; no collective on the data path): weak scaling.
`--impl reference` times the reference's CPU algorithm (the oracle's
restatement of GraphMP's OpenMP engine) on this host's cores instead.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

SEED = 20240601
SHARDS = 256


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gx", choices=["gx", "reference"])
    ap.add_argument("--scale", type=int, default=24)
    ap.add_argument("--edge-factor", type=int, default=16)
    ap.add_argument("--iters", type=int, default=20)
    ap.add_argument("--cpu-iters", type=int, default=2, help="PageRank supersteps in the CPU-baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=2)
    return ap.parse_args()


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("LOCAL_RANK", 0)), int(os.environ.get("WORLD_SIZE", 1))


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.path = Path(tempfile.mkstemp(suffix=".csv")[1])

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if self.proc is None or not self.path.exists():
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        self.path.unlink(missing_ok=True)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peak_hbm():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except (KeyError, ValueError):
            pass
    return 6800.0, "fallback"


def ncu_traffic(workload: str):
    """DRAM bytes per pull launch from the committed ncu summary, if any."""
    p = ROOT / "profiles" / f"pull_kernel_pagerank_ref_{workload}.md"
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        if line.startswith("traffic_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].strip())
            except ValueError:
                return None
    return None


def build_graph(args):
    import graphee_gb300 as gx
    t0 = time.time()
    g = gx.rmat_graph(args.scale, args.edge_factor, seed=SEED, P=SHARDS)
    return g, time.time() - t0


def cpu_pagerank(g, iters):
    """The reference's CPU algorithm (oracle restatement of GraphPS::run +
    comp_pagerank, OpenMP over shards) on this host's cores."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import gx_oracle as O
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    _, _, ms = O.run(O.PAGERANK_REF, g.V, g.P, g.bounds, g.off, g.col, g.outdeg, iters, threads=threads)
    wall = time.perf_counter() - t0
    return float(sum(ms)) / 1000.0, wall, threads


def workload_name(args):
    return f"rmat{args.scale}"


def base_config(args, g):
    return {"workload": f"R-MAT scale {args.scale} edge factor {args.edge_factor} (a,b,c=.57,.19,.19), "
                        f"{args.iters} PageRank supersteps (reference semantics), {SHARDS} shards",
            "vertices": g.V, "edges": g.E, "shards": SHARDS, "supersteps": args.iters, "seed": SEED,
            "l2": "inputs larger than L2 (column indices 4E bytes); no flush"}


def run_reference(args, rank, world):
    if rank != 0:
        return 0
    g, build_s = build_graph(args)
    for _ in range(args.warmup):
        cpu_pagerank(g, args.cpu_iters)
    secs = []
    for _ in range(args.steps):
        s, _, threads = cpu_pagerank(g, args.cpu_iters)
        secs.append(s)
    total = sum(secs)
    value = args.cpu_iters * g.E * args.steps / total / 1e9
    line = {"metric": "pagerank_gteps", "value": value, "unit": "GTEPS", "impl": "reference",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": total / args.steps * 1000, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded R-MAT)",
            "config": base_config(args, g),
            "cpu_baseline": {"value": value, "unit": "GTEPS", "cores": threads, "kind": "port",
                             "sample": f"{args.cpu_iters} of {args.iters} supersteps per step, same graph"},
            "e2e": {"value": value, "unit": "GTEPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def run_gx(args, rank, local_rank, world):
    import torch
    import graphee_gb300 as gx
    if not gx.LIB_PATH.exists():
        import __graft_entry__
        __graft_entry__.build()
    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    g, build_s = build_graph(args)
    eng = gx.Engine(device=local_rank)
    eng.load(g)
    for _ in range(args.warmup):
        eng.run(gx.APP_PAGERANK_REF, args.iters)

    barrier()
    with ClockSampler(local_rank) as clk:
        t0 = time.perf_counter()
        dev_ms = 0.0
        launches = 0
        iters_done = 0
        for _ in range(args.steps):
            st = eng.run(gx.APP_PAGERANK_REF, args.iters)
            dev_ms += st["ms_total"]
            launches += st["kernel_launches"]
            iters_done += st["iterations"]
        barrier()
        wall = time.perf_counter() - t0
    clocks = clk.summary()
    ms_step = dev_ms / args.steps
    if dist is not None:
        t = torch.tensor([ms_step], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms_step = float(t.item())
    edges_per_step = g.E * args.iters
    value = world * edges_per_step / (ms_step / 1000) / 1e9

    # Dominant kernel, timed live with CUDA events on the engine's stream.
    prof = gx.Engine(device=local_rank, profile=1)
    prof.load(g)
    prof.run(gx.APP_PAGERANK_REF, args.iters)
    ps = prof.run(gx.APP_PAGERANK_REF, args.iters)
    prof.close()
    pull_ms = ps["ms_pull"] / max(ps["pull_launches"], 1)
    alg_bytes = 8 * g.E + 24 * g.V
    peak, peak_kind = measured_peak_hbm()
    achieved = alg_bytes / (pull_ms / 1000) / 1e9
    traffic = ncu_traffic(workload_name(args))

    # End to end through the C ABI: host buffers in, values out, every step.
    e2e_s = []
    for i in range(args.e2e_steps + 1):
        barrier()
        t1 = time.perf_counter()
        with gx.Engine(device=local_rank) as e2:
            e2.load(g)
            e2.run(gx.APP_PAGERANK_REF, args.iters)
            vals = e2.values()
        torch.cuda.synchronize()
        if i > 0:
            e2e_s.append(time.perf_counter() - t1)
    e2e_step = sum(e2e_s) / len(e2e_s)
    if dist is not None:
        t = torch.tensor([e2e_step], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_step = float(t.item())
    h2d = 4 * g.E + 8 * (g.V + 1) + 4 * g.V
    d2h = 4 * g.V
    assert np.isfinite(vals).all()

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        s, wall_cpu, threads = cpu_pagerank(g, args.cpu_iters)
        cpu = {"value": args.cpu_iters * g.E / s / 1e9, "unit": "GTEPS", "cores": threads, "kind": "port",
               "sample": f"{args.cpu_iters} of {args.iters} PageRank supersteps on the same graph "
                         f"({s:.2f} s of superstep time, {wall_cpu:.2f} s wall)"}

    if rank == 0:
        cfg = base_config(args, g)
        cfg.update({"parallelism": f"replicas{world}", "graph_build_s": round(build_s, 2)})
        line = {"metric": "pagerank_gteps", "value": value, "unit": "GTEPS", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded R-MAT)",
                "config": cfg,
                "e2e": {"value": world * edges_per_step / e2e_step / 1e9, "unit": "GTEPS",
                        "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h, "s_per_step": e2e_step},
                "gpu_launches": launches,
                "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                             "frac": achieved / peak, "traffic": traffic, "peak_source": peak_kind,
                             "kernel": "pull_kernel<PAGERANK_REF>", "kernel_ms": pull_ms,
                             "algorithmic_bytes_per_launch": alg_bytes},
                "cpu_baseline": cpu, "clocks": clocks, "wall_s_timed": wall,
                "iterations_per_step": iters_done / args.steps}
        print(json.dumps(line), flush=True)
    eng.close()
    if dist is not None:
        dist.destroy_process_group()
    return 0


def main():
    args = parse()
    rank, local_rank, world = dist_env()
    if args.impl == "reference":
        return run_reference(args, rank, world)
    return run_gx(args, rank, local_rank, world)


if __name__ == "__main__":
    sys.exit(main())
