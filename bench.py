#!/usr/bin/env python
"""PageRank GTEPS of GraphMP's shard-wise gather-apply on one GB300.

Workload (default): seeded R-MAT, scale 26, edge factor 16 (a,b,c,d =
.57/.19/.19/.05, self-loops and duplicates removed), 256 edge-balanced
destination-range shards; one step = one PageRank run of 20 supersteps with
the reference's semantics (comp_pagerank<float>, GraphMP/app/pagerank.cpp).
value = 20 * E / step time, in GTEPS, inputs resident in HBM; e2e = the same
metric through the C ABI with host buffers: one engine, and per step a load
of the graph from the caller's arrays, the run, and the read-back of the
ranks into the caller's buffer.  The line also carries weighted SSSP on the
same graph and the scale-24 PageRank figures.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gx|reference]

Under torchrun (N > 1) every rank runs an independent replica on its own GPU
(the path is single-GPU; no collective on the data path): weak scaling.
`--impl reference` times the reference's CPU PageRank on this host's cores
instead: its own app, compiled from the reference sources, where that binary
was built for this host, else the oracle's restatement of GraphMP's OpenMP
engine.  That arm builds its graph with the oracle's restatement of the
generator and never loads this package's library.
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
from contextlib import nullcontext as _nullcontext
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

SEED = 20240601
SHARDS = 256


def aggregate(ms_step: float, units_per_rank: float, dist=None, device=None):
    """Replicas: the step time is the max over ranks, the work the sum.
    Returns (max ms per step, total units per second)."""
    if dist is None:
        return ms_step, units_per_rank / (ms_step / 1000)
    import torch
    t = torch.tensor([ms_step, units_per_rank], dtype=torch.float64, device=device)
    mx = t.clone()
    dist.all_reduce(mx, op=dist.ReduceOp.MAX)
    tot = t.clone()
    dist.all_reduce(tot, op=dist.ReduceOp.SUM)
    return float(mx[0]), float(tot[1]) / (float(mx[0]) / 1000)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gx", choices=["gx", "reference"])
    ap.add_argument("--scale", type=int, default=26)
    ap.add_argument("--edge-factor", type=int, default=16)
    ap.add_argument("--iters", type=int, default=20)
    ap.add_argument("--cpu-iters", type=int, default=2, help="PageRank supersteps in the CPU-baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--no-sssp", action="store_true", help="skip the SSSP keys of the default run")
    ap.add_argument("--no-scale24", action="store_true", help="skip the scale-24 keys of the default run")
    ap.add_argument("--layout", default="relabel", choices=["relabel", "plain"],
                    help="the headline engine's vertex layout: relabel = config.relabel (per-shard renumbering "
                         "by in-degree at load), plain = the caller's numbering")
    ap.add_argument("--no-other-layout", action="store_true", help="skip the keys of the other layout")
    ap.add_argument("--workload", default="pagerank",
                    choices=["pagerank", "cc_tc", "stream", "batch", "ppr", "warm"],
                    help="pagerank = the headline run; the others measure the remaining configurations")
    return ap.parse_args()


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("LOCAL_RANK", 0)), int(os.environ.get("WORLD_SIZE", 1))


class ClockSampler:
    """nvidia-smi clocks / throttle reasons, sampled every 100 ms from before
    the warm-up to the end of the timed regions.  Each sample carries
    nvidia-smi's own timestamp; the summary keeps the samples taken inside the
    timed regions (marked with window())."""

    FIELDS = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    REASONS = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.windows = []
        fd, name = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        self.path = Path(name)

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
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

    class _Window:
        def __init__(self, owner):
            self.owner = owner

        def __enter__(self):
            self.t0 = time.time()

        def __exit__(self, *exc):
            self.owner.windows.append((self.t0, time.time()))

    def window(self):
        return ClockSampler._Window(self)

    def _samples(self):
        from datetime import datetime
        out = []
        for line in self.path.read_text().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 10:
                continue
            try:
                ts = datetime.strptime(parts[0], "%Y/%m/%d %H:%M:%S.%f").timestamp()
                sm, smax = float(parts[2]), float(parts[3])
            except ValueError:
                continue
            active = {n for n, v in zip(self.REASONS, parts[6:10]) if v.lower() == "active"}
            out.append((ts, sm, smax, active))
        return out

    def summary(self):
        samples = self._samples() if self.proc is not None and self.path.exists() else []
        self.path.unlink(missing_ok=True)
        inside = [x for x in samples if any(a <= x[0] <= b for a, b in self.windows)]
        where = "timed regions"
        if not inside and self.windows:
            # Timed regions shorter than the sampling period: the samples
            # from the warm-up on (the GPU under the same load) stand in.
            inside = [x for x in samples if x[0] >= self.windows[0][0] - 2.0]
            where = "warm-up and timed regions (timed regions shorter than the 100 ms period)"
        if not inside:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        reasons = set().union(*(x[3] for x in inside))
        return {"sm_mhz": statistics.median(x[1] for x in inside), "sm_max_mhz": max(x[2] for x in inside),
                "reasons": sorted(reasons), "samples": len(inside), "sampled": where}


def measured_peak_hbm():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except (KeyError, ValueError):
            pass
    return 6800.0, "fallback"


def layout_cfg(layout: str) -> dict:
    return {"relabel": 1} if layout == "relabel" else {}


def ncu_traffic(workload: str, layout: str = "plain"):
    """DRAM bytes per pull launch from the committed ncu summary, if any."""
    tag = "relabel_" if layout == "relabel" else ""
    p = ROOT / "profiles" / f"pull_kernel_pagerank_ref_{tag}{workload}.md"
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        if line.startswith("traffic_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].strip())
            except ValueError:
                return None
    return None


def build_graph(args, device=None):
    """The R-MAT graph: built on GPU `device` (gx_rmat_csc_gpu), or on the
    host when device is None; both give the same graph."""
    import graphee_gb300 as gx
    t0 = time.time()
    g = gx.rmat_graph(args.scale, args.edge_factor, seed=SEED, P=SHARDS, gpu=device is not None,
                      device=device or 0)
    return g, time.time() - t0


REF_BIN = ROOT / "oracle" / "_ref" / "ref_pagerank_cached"
REF_CMPNUM = 24            # per-thread buffers the reference allocates (GraphMP/system/Global.h:58)
_ref_dirs = {}


def _reference_pagerank(g, iters):
    """The reference's own PageRank app (oracle/_ref, compiled from the
    reference sources with the in-RAM edge cache on) run on a shard directory
    of this graph.  It runs iters + 1 iterations, the first of which reads the
    shard files into the cache; the time is the sum of the other iterations'
    COMP_TIME (GraphMP/system/GraphPS.h:376-377).  None where the binary is
    absent or does not run on this host."""
    import re
    if not (REF_BIN.exists() and os.access(REF_BIN, os.X_OK)):
        return None
    O = _oracle()
    key = id(g)
    if key not in _ref_dirs:
        d = tempfile.TemporaryDirectory(prefix="gx_ref_shards_")
        O.write_shards(g, d.name + "/")
        _ref_dirs[key] = d
    d = _ref_dirs[key].name + "/"
    threads = min(os.cpu_count() or 1, REF_CMPNUM)
    with tempfile.NamedTemporaryFile(suffix=".bin") as out:
        t0 = time.perf_counter()
        try:
            r = subprocess.run([str(REF_BIN), d, str(g.V), str(g.P), str(iters + 1), out.name, str(threads)],
                               capture_output=True, text=True, timeout=1800)
        except OSError:
            return None
        wall = time.perf_counter() - t0
    if r.returncode != 0:
        return None
    ms = [int(m) for m in re.findall(r"Iteration: \d+, uses (\d+) ms", r.stderr)]
    # Whole milliseconds: a graph whose supersteps round to 0 ms is timed by the port.
    if len(ms) != iters + 1 or sum(ms[1:]) == 0:
        return None
    return sum(ms[1:]) / 1000.0, wall, threads, "reference"


def _oracle():
    sys.path.insert(0, str(ROOT / "oracle"))
    import gx_oracle as O
    return O


CPU_SAMPLE = {"reference": "the reference's own PageRank app (in-RAM edge cache on; "
                           "its first, file-reading iteration not timed)",
              "port": "the oracle's restatement of the reference's OpenMP loop"}


def cpu_pagerank(g, iters):
    """The reference's CPU PageRank on this host's cores: its own app binary
    where that was built for this host, else the oracle's restatement of
    GraphPS::run + comp_pagerank (OpenMP over shards).  Returns (superstep
    seconds, wall seconds, threads, kind)."""
    got = _reference_pagerank(g, iters)
    if got is not None:
        return got
    O = _oracle()
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    _, _, ms = O.run(O.PAGERANK_REF, g.V, g.P, g.bounds, g.off, g.col, g.outdeg, iters, threads=threads)
    wall = time.perf_counter() - t0
    return float(sum(ms)) / 1000.0, wall, threads, "port"


def workload_name(args):
    return f"rmat{args.scale}"


def base_config(args, g, world):
    """The workload, the same dict in both arms."""
    return {"workload": f"R-MAT scale {args.scale} edge factor {args.edge_factor} (a,b,c=.57,.19,.19), "
                        f"{args.iters} PageRank supersteps (reference semantics), {SHARDS} shards",
            "vertices": g.V, "edges": g.E, "shards": SHARDS, "supersteps": args.iters, "seed": SEED,
            "l2": "inputs larger than L2 (column indices 4E bytes); no flush",
            "parallelism": f"replicas{world}"}


def run_reference(args, rank, world):
    if rank != 0:
        return 0
    O = _oracle()
    t0 = time.time()
    g = O.rmat_graph(args.scale, args.edge_factor, seed=SEED, P=SHARDS)
    build_s = time.time() - t0
    for _ in range(args.warmup):
        cpu_pagerank(g, args.cpu_iters)
    secs = []
    for _ in range(args.steps):
        s, _, threads, kind = cpu_pagerank(g, args.cpu_iters)
        secs.append(s)
    total = sum(secs)
    value = args.cpu_iters * g.E * args.steps / total / 1e9
    line = {"metric": "pagerank_gteps", "value": value, "unit": "GTEPS", "impl": "reference",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": total / args.steps * 1000, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded R-MAT)",
            "config": base_config(args, g, world),
            "graph_build": {"s": round(build_s, 1), "by": "the oracle's restatement of the generator, on the host"},
            "cpu_baseline": {"value": value, "unit": "GTEPS", "cores": threads, "kind": kind,
                             "sample": f"{args.cpu_iters} of {args.iters} supersteps per step, same graph; "
                                       f"{CPU_SAMPLE[kind]}"},
            "e2e": {"value": value, "unit": "GTEPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def pull_kernel_ms(gx, g, device, iters, **cfg):
    """Average pull-kernel launch time of a PageRank run (CUDA events on the
    engine's stream, one engine with per-launch timing)."""
    with gx.Engine(device=device, profile=1, **cfg) as prof:
        prof.load(g)
        prof.run(gx.APP_PAGERANK_REF, iters)
        ps = prof.run(gx.APP_PAGERANK_REF, iters)
    return ps["ms_pull"] / max(ps["pull_launches"], 1)


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

    g, build_s = build_graph(args, device=local_rank)
    lcfg = layout_cfg(args.layout)
    eng = gx.Engine(device=local_rank, **lcfg)
    eng.load(g)
    clk = ClockSampler(local_rank).__enter__()
    for _ in range(args.warmup):
        eng.run(gx.APP_PAGERANK_REF, args.iters)

    barrier()
    with clk.window():
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
    edges_per_step = g.E * args.iters
    ms_step, eps = aggregate(dev_ms / args.steps, float(edges_per_step), dist, "cuda")
    value = eps / 1e9

    # Dominant kernel, timed live with CUDA events on the engine's stream.
    pull_ms = pull_kernel_ms(gx, g, local_rank, args.iters, **lcfg)
    alg_bytes = 8 * g.E + 24 * g.V
    peak, peak_kind = measured_peak_hbm()
    achieved = alg_bytes / (pull_ms / 1000) / 1e9
    traffic = ncu_traffic(workload_name(args), args.layout)

    # End to end through the C ABI: host buffers in, values out, every step.
    # One engine serves every step (created before the timed steps); each step
    # loads the graph from the caller's host arrays, runs the supersteps and
    # reads the ranks back into the caller's result buffer.
    e2e_s = []
    result = np.empty(g.V, np.float32)
    e2 = gx.Engine(device=local_rank, **lcfg)
    for i in range(args.e2e_steps + 1):
        barrier()
        with clk.window() if i > 0 else _nullcontext():
            t1 = time.perf_counter()
            e2.load(g)
            e2.run(gx.APP_PAGERANK_REF, args.iters)
            vals = e2.values(out=result)
            torch.cuda.synchronize()
            if i > 0:
                e2e_s.append(time.perf_counter() - t1)
    e2.close()
    clk.__exit__(None, None, None)
    clocks = clk.summary()
    e2e_step, e2e_eps = aggregate(sum(e2e_s) / len(e2e_s) * 1000, float(edges_per_step), dist, "cuda")
    e2e_step /= 1000
    h2d = 4 * g.E + 8 * (g.V + 1) + 4 * g.V
    d2h = 4 * g.V
    assert np.isfinite(vals).all()

    # The other vertex layout (config.relabel on or off): device steps, the
    # pull kernel and the same end-to-end step (a relabelling load includes
    # the renumbering).
    other = None
    other_name = "plain" if args.layout == "relabel" else "relabel"
    if not args.no_other_layout:
        ocfg = layout_cfg(other_name)
        with gx.Engine(device=local_rank, **ocfg) as eo:
            eo.load(g)
            for _ in range(args.warmup):
                eo.run(gx.APP_PAGERANK_REF, args.iters)
            runs_o = [eo.run(gx.APP_PAGERANK_REF, args.iters) for _ in range(args.steps)]
            launches += sum(r["kernel_launches"] for r in runs_o)
            ms_o = sum(r["ms_total"] for r in runs_o) / len(runs_o)
            e2e_o = []
            for i in range(args.e2e_steps + 1):
                torch.cuda.synchronize()
                t1 = time.perf_counter()
                eo.load(g)
                eo.run(gx.APP_PAGERANK_REF, args.iters)
                eo.values(out=result)
                torch.cuda.synchronize()
                if i > 0:
                    e2e_o.append(time.perf_counter() - t1)
            assert np.isfinite(result).all()
        ko = pull_kernel_ms(gx, g, local_rank, args.iters, **ocfg)
        other = {"value": g.E * args.iters / (ms_o / 1000) / 1e9, "unit": "GTEPS", "ms_per_step": ms_o,
                 "kernel_ms": ko, "achieved_gbs": alg_bytes / (ko / 1000) / 1e9,
                 "frac": alg_bytes / (ko / 1000) / 1e9 / peak,
                 "traffic": ncu_traffic(workload_name(args), other_name),
                 "e2e": {"value": edges_per_step / (sum(e2e_o) / len(e2e_o)) / 1e9, "unit": "GTEPS",
                         "s_per_step": sum(e2e_o) / len(e2e_o), "steps": len(e2e_o)}}

    sssp = None
    if not args.no_sssp:
        g.weights = gx.edge_weights(7, g)
        eng.set_weights(g.weights)
        for _ in range(2):
            eng.run(gx.APP_SSSP, 10000, source=0, weighted=True)
        runs = [eng.run(gx.APP_SSSP, 10000, source=0, weighted=True) for _ in range(3)]
        ms_s = sum(r["ms_total"] for r in runs) / len(runs)
        scanned = runs[-1]["edges_scanned"]
        launches += sum(r["kernel_launches"] for r in runs)
        sssp = {"metric": "sssp_gteps", "value": g.E / (ms_s / 1000) / 1e9, "unit": "GTEPS (input edges / run)",
                "scanned_gteps": scanned / (ms_s / 1000) / 1e9, "ms_per_run": ms_s,
                "supersteps": runs[-1]["iterations"], "push_supersteps": runs[-1]["push_iterations"],
                "weights": "uint32 in [1,255], seeded", "source": 0}
        # Per pull superstep: the pull kernel timed with CUDA events on the
        # engine's stream (profiling engine), over the edges its pull steps
        # scanned; algorithmic bytes 12 per edge (index, weight, distance
        # gather) + 16 per vertex of the swept shards (offsets, old and new
        # distance), the latter prorated by the edges a selective step swept.
        pe = gx.Engine(device=local_rank, profile=1, **lcfg)
        pe.load(g)
        pe.set_weights(g.weights)
        pe.run(gx.APP_SSSP, 10000, source=0, weighted=True)
        pst = pe.run(gx.APP_SSSP, 10000, source=0, weighted=True)
        steps = [pe.iter_stats(i) for i in range(pst["iterations"])]
        pe.close()
        pulled = [s for s in steps if s["mode"] in (0, 1)]
        e_pull = sum(s["edges_scanned"] for s in pulled)
        if pulled and pst["ms_pull"] > 0:
            bytes_pull = 12 * e_pull + 16 * g.V * (e_pull / g.E)
            ach = bytes_pull / (pst["ms_pull"] / 1000) / 1e9
            sssp["pull_supersteps"] = {"count": len(pulled), "edges": e_pull, "ms_pull_kernels": pst["ms_pull"],
                                       "gteps": e_pull / (pst["ms_pull"] / 1000) / 1e9, "achieved_gbs": ach,
                                       "frac_of_measured_hbm": ach / measured_peak_hbm()[0]}

    # The scale-24 graph of the earlier headline: PageRank GTEPS and the pull
    # kernel's fraction of measured HBM bandwidth.
    rmat24 = None
    if args.scale == 26 and not args.no_scale24:
        g24 = gx.rmat_graph(24, args.edge_factor, seed=SEED, P=SHARDS, gpu=True, device=local_rank)
        with gx.Engine(device=local_rank, **lcfg) as e24:
            e24.load(g24)
            for _ in range(args.warmup):
                e24.run(gx.APP_PAGERANK_REF, args.iters)
            runs24 = [e24.run(gx.APP_PAGERANK_REF, args.iters) for _ in range(args.steps)]
        launches += sum(r["kernel_launches"] for r in runs24)
        ms24 = sum(r["ms_total"] for r in runs24) / len(runs24)
        k24 = pull_kernel_ms(gx, g24, local_rank, args.iters, **lcfg)
        b24 = 8 * g24.E + 24 * g24.V
        rmat24 = {"value": g24.E * args.iters / (ms24 / 1000) / 1e9, "unit": "GTEPS", "ms_per_step": ms24,
                  "vertices": g24.V, "edges": g24.E, "kernel_ms": k24,
                  "achieved_gbs": b24 / (k24 / 1000) / 1e9, "frac": b24 / (k24 / 1000) / 1e9 / peak}
        del g24

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        s, wall_cpu, threads, kind = cpu_pagerank(g, args.cpu_iters)
        cpu = {"value": args.cpu_iters * g.E / s / 1e9, "unit": "GTEPS", "cores": threads, "kind": kind,
               "sample": f"{args.cpu_iters} of {args.iters} PageRank supersteps on the same graph, "
                         f"{CPU_SAMPLE[kind]} "
                         f"({s:.2f} s of superstep time, {wall_cpu:.2f} s wall)"}

    if rank == 0:
        line = {"metric": "pagerank_gteps", "value": value, "unit": "GTEPS", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded R-MAT)",
                "config": base_config(args, g, world),
                "graph_build": {"s": round(build_s, 2), "by": "on the GPU (gx_rmat_csc_gpu), identical to the "
                                                              "host build and to the oracle's"},
                "e2e": {"value": e2e_eps / 1e9, "unit": "GTEPS",
                        "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h, "s_per_step": e2e_step,
                        "step": "gx_load_csc from host arrays + gx_run (20 supersteps) + gx_get_values into a "
                                "reused host buffer, one engine" +
                                (" with config.relabel = 1 (the renumbering is part of every load)"
                                 if args.layout == "relabel" else "")},
                "gpu_launches": launches,
                "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                             "frac": achieved / peak, "traffic": traffic, "peak_source": peak_kind,
                             "kernel": "pull_kernel<PAGERANK_REF>", "kernel_ms": pull_ms,
                             "algorithmic_bytes_per_launch": alg_bytes},
                "cpu_baseline": cpu, "clocks": clocks, "wall_s_timed": wall, "sssp": sssp,
                "rmat24": rmat24, "layout": args.layout, other_name: other,
                "iterations_per_step": iters_done / args.steps}
        print(json.dumps(line), flush=True)
    eng.close()
    if dist is not None:
        dist.destroy_process_group()
    return 0


# ---------------------------------------------------------------------------
# The other configurations (opt-in with --workload; one JSON line each).
# ---------------------------------------------------------------------------

def _line(metric, value, unit, args, config, **extra):
    d = {"metric": metric, "value": value, "unit": unit, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
         "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "data": "synthetic (seeded R-MAT)",
         "config": config}
    d.update(extra)
    print(json.dumps(d), flush=True)


def run_cc_tc(args):
    """Configuration 2's CC and TC: symmetrised R-MAT scale 24 unless
    --scale names another."""
    import graphee_gb300 as gx
    sys.path.insert(0, str(ROOT / "oracle"))
    import gx_oracle as O
    if args.scale == 26:
        args.scale = 24
    t0 = time.time()
    g = gx.rmat_graph(args.scale, args.edge_factor, seed=SEED, P=SHARDS, symmetric=True, gpu=True)
    build_s = time.time() - t0
    with gx.Engine(**layout_cfg(args.layout)) as e:
        e.load(g)
        for _ in range(args.warmup):
            e.run(gx.APP_CC, 10000)
        runs = [e.run(gx.APP_CC, 10000) for _ in range(args.steps)]
        cc = e.values()
        ms_cc = sum(r["ms_total"] for r in runs) / len(runs)
        tri, st = e.triangle_count()
        tri2, st2 = e.triangle_count()
    t1 = time.perf_counter()
    ref, ch, _ = O.run(O.CC, g.V, g.P, g.bounds, g.off, g.col, g.outdeg, 10000, threads=os.cpu_count())
    cpu_s = time.perf_counter() - t1
    cfg = {"workload": f"R-MAT scale {args.scale} edge factor {args.edge_factor}, symmetrised, deduplicated",
           "vertices": g.V, "directed_entries": g.E, "graph_build_s": round(build_s, 1)}
    _line("cc_gteps", g.E / (ms_cc / 1000) / 1e9, "GTEPS (input entries / run)", args, cfg, dtype="int32",
          ms_per_run=ms_cc, supersteps=runs[-1]["iterations"], push_supersteps=runs[-1]["push_iterations"],
          scanned_gteps=runs[-1]["edges_scanned"] / (ms_cc / 1000) / 1e9,
          bit_exact_vs_oracle=bool(np.array_equal(cc, ref)), oracle_supersteps=len(ch),
          cpu_baseline={"value": g.E * len(ch) / cpu_s / 1e9, "unit": "GTEPS (entries x supersteps / s)",
                        "cores": os.cpu_count(), "kind": "port", "sample": "full CC run, same graph"},
          triangles=tri, tc_ms=min(st["ms_total"], st2["ms_total"]), tc_repeatable=tri == tri2,
          tc_work_edges=st["edges_scanned"], layout=args.layout)


def pinned_h2d_gbs(nbytes=2 << 30, repeats=7):
    """The host link's rate for the streaming ring's kind of copy: one
    cudaMemcpyAsync of pinned host memory to the device (torch's copy_ of a
    pinned tensor), timed with CUDA events; the median of the repeats."""
    import torch
    h = torch.empty(nbytes, dtype=torch.uint8).pin_memory()
    d = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    rates = []
    for i in range(repeats + 1):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        d.copy_(h, non_blocking=True)
        e1.record()
        e1.synchronize()
        if i:
            rates.append(nbytes / (e0.elapsed_time(e1) / 1000) / 1e9)
    del h, d
    return statistics.median(rates)


def run_stream(args):
    import graphee_gb300 as gx
    scale = args.scale if args.scale not in (24, 26) else 28
    t0 = time.time()
    g = gx.rmat_graph(scale, args.edge_factor, seed=SEED, P=256, gpu=True)
    build_s = time.time() - t0
    budget = 8 << 30
    t1 = time.time()
    e = gx.Engine(cache_budget_bytes=budget)
    e.load(g)
    load_s = time.time() - t1
    e.run(gx.APP_PAGERANK_REF, 2)
    pr = e.run(gx.APP_PAGERANK_REF, 10)
    cfg = {"workload": f"R-MAT scale {scale} edge factor {args.edge_factor}, 256 shards, HBM shard cache 8 GiB, "
                       "10 PageRank supersteps then weighted SSSP", "vertices": g.V, "edges": g.E,
           "graph_build_s": round(build_s, 1), "load_s": round(load_s, 1)}
    w = gx.edge_weights(7, g)
    e.set_weights(w)
    del w
    ss = e.run(gx.APP_SSSP, 10000, source=0, weighted=True)
    ss_steps = [e.iter_stats(i) for i in range(ss["iterations"])]
    e.close()
    link = pinned_h2d_gbs()
    pr_gbs = pr["h2d_bytes"] / (pr["ms_copy"] / 1000) / 1e9 if pr["ms_copy"] > 0 else None
    _line("pagerank_gteps_streamed", 10 * g.E / (pr["ms_total"] / 1000) / 1e9, "GTEPS", args, cfg, dtype="f32",
          ms_per_superstep=pr["ms_total"] / 10, shards_resident=pr["shards_resident"],
          h2d_gb_per_superstep=pr["h2d_bytes"] / 10 / 1e9, copy_ms=pr["ms_copy"], compute_ms=pr["ms_compute"],
          overlap=pr["overlap"],
          roofline={"bound": "host link", "achieved": pr_gbs, "peak": link, "unit": "GB/s",
                    "frac": pr_gbs / link if pr_gbs else None,
                    "peak_source": "measured here: pinned host-to-device cudaMemcpyAsync of 2 GiB, median of 7"},
          link_frac=pr_gbs / link if pr_gbs else None,
          sssp={"gteps": g.E / (ss["ms_total"] / 1000) / 1e9, "ms": ss["ms_total"], "supersteps": ss["iterations"],
                "h2d_gb": ss["h2d_bytes"] / 1e9, "overlap": ss["overlap"], "shard_visits_streamed": ss["shards_streamed"],
                "shards_swept_per_step": [s["shards_active"] for s in ss_steps],
                "modes": [s["mode"] for s in ss_steps]})


def run_batch(args):
    import graphee_gb300 as gx
    t0 = time.time()
    g, vb = gx.batch_graph(2048, scales=(10, 17), edge_factors=(8, 32), seed=SEED)
    build_s = time.time() - t0
    n = len(vb) - 1
    with gx.Engine() as e:
        e.load(g)
        # Every candidate schedule's time, beside the run's other outputs.
        table = Path(os.environ.get("GX_AUTOTUNE_TABLE", tempfile.gettempdir())) / "gx_batch_autotune_table.jsonl"
        best, best_ms = e.batch_autotune(vb, pr_iters=30, cc_max_iter=1000, table_path=str(table))
        for _ in range(args.warmup):
            e.batch_run(vb, 30, 1000, tuning=best)
        runs = [e.batch_run(vb, 30, 1000, tuning=best)[4] for _ in range(args.steps)]
        ms_b = sum(r["ms_total"] for r in runs) / len(runs)
        edges_b = runs[-1]["edges_scanned"]
    # One engine launch sequence per instance (load excluded from the timing).
    ms_sep = 0.0
    edges_sep = 0
    for i in range(n):
        b, en = int(vb[i]), int(vb[i + 1])
        sub = gx.Graph(en - b, g.off[b:en + 1] - g.off[b], g.col[g.off[b]:g.off[en]] - b, g.outdeg[b:en], 1)
        with gx.Engine() as e1:
            e1.load(sub)
            a = e1.run(gx.APP_PAGERANK_REF, 30)
            c = e1.run(gx.APP_CC, 1000)
            ms_sep += a["ms_total"] + c["ms_total"]
            edges_sep += a["edges_scanned"] + c["edges_scanned"]
    cfg = {"workload": "2048 R-MAT instances, scale U{10..17}, edge factor U{8..32}, per-instance seeds; "
                       "PageRank (reference semantics, 30 supersteps) then CC per instance",
           "vertices": g.V, "edges": g.E, "graph_build_s": round(build_s, 1), "tuning": best}
    _line("batch_instances_per_s", n / (ms_b / 1000), "instances/s", args, cfg, dtype="f32+int32",
          ms_per_batch=ms_b, gteps=edges_b / (ms_b / 1000) / 1e9, gpu_launches=1,
          separate={"instances_per_s": n / (ms_sep / 1000), "gteps": edges_sep / (ms_sep / 1000) / 1e9,
                    "ms": ms_sep, "note": "one engine run (graph replay of its superstep kernels) per instance"},
          speedup_vs_separate=ms_sep / ms_b)


def run_ppr(args):
    """Configuration 4b: 64-source personalized PageRank on R-MAT (scale 24
    by default) as one persistent launch per call, against 64 calls of one
    source each (the one-launch-per-instance baseline)."""
    import graphee_gb300 as gx
    scale = 24 if args.scale == 26 else args.scale
    args.scale = scale
    g, build_s = build_graph(args, device=0)
    rng = np.random.default_rng(SEED)
    src = rng.integers(0, g.V, size=64).astype(np.int32)
    with gx.Engine(**layout_cfg(args.layout)) as e:
        e.load(g)
        e.ppr(src, 2, fetch=False)
        runs = [e.ppr(src, args.iters, fetch=False)[1] for _ in range(args.steps)]
        e.ppr(src[:1], 2, fetch=False)
        single = [e.ppr(src[j:j + 1], args.iters, fetch=False)[1] for j in range(len(src))]
    ms = sum(r["ms_total"] for r in runs) / len(runs)
    ms_sep = sum(r["ms_total"] for r in single)
    per_it = ms / args.iters
    W = 64
    alg = 4 * g.E + 4 * W * g.E + 2 * 4 * W * g.V
    peak, kind = measured_peak_hbm()
    cfg = {"workload": f"personalized PageRank, 64 sources U[0,V), restart 0.15, R-MAT scale {scale}, "
                       f"{args.iters} steps", "vertices": g.V, "edges": g.E}
    _line("ppr_gteps", 64 * g.E * args.iters / (ms / 1000) / 1e9, "GTEPS (edges x steps x sources / s)", args,
          cfg, dtype="f32", ms_per_call=ms, ms_per_step=per_it, gpu_launches_per_call=runs[-1]["kernel_launches"],
          roofline={"bound": "hbm", "achieved": alg / (per_it / 1000) / 1e9, "peak": peak, "unit": "GB/s",
                    "frac": alg / (per_it / 1000) / 1e9 / peak, "peak_source": kind,
                    "algorithmic_bytes_per_step": alg},
          separate={"ms": ms_sep, "gteps": 64 * g.E * args.iters / (ms_sep / 1000) / 1e9,
                    "note": "64 calls of one source each (rows of 8 columns), one persistent launch per call"},
          speedup_vs_separate=ms_sep / ms, layout=args.layout)


def run_warm(args):
    import graphee_gb300 as gx
    rng = np.random.default_rng(SEED)
    t0 = time.time()
    m = gx.MLP(seed=SEED)
    for i in range(256):
        s = int(rng.integers(16, 21))
        ja, jb, jc = rng.uniform(-0.05, 0.05, size=3)
        while 0.57 + ja + 0.19 + jb + 0.19 + jc > 0.99:   # keep d = 1 - a - b - c >= 0.01
            ja, jb, jc = rng.uniform(-0.05, 0.05, size=3)
        g = gx.rmat_graph(s, 16, seed=SEED + 17 * i, P=16, a=0.57 + ja, b=0.19 + jb, c=0.19 + jc, gpu=True)
        with gx.Engine() as e:
            e.load(g)
            m.add_graph(e, max_samples=65536, max_iter=500, tolerance=1e-9)
    prep_s = time.time() - t0
    t1 = time.time()
    loss = m.train(20, batch=8192, lr=2e-3)
    train_s = time.time() - t1
    evals = {}
    for scale in (24, 26):
        g = gx.rmat_graph(scale, 16, seed=SEED + 99991 + scale, P=256, gpu=True)
        with gx.Engine() as e:
            e.load(g)
            e.run(gx.APP_PAGERANK_STD, 3)
            uni = e.run(gx.APP_PAGERANK_STD, 1000, tolerance=1e-6)
            e.pagerank_warm(m, 1000, tolerance=1e-6)
            ws = e.pagerank_warm(m, 1000, tolerance=1e-6)
        warm_ms = ws["ms_features"] + ws["ms_mlp"] + ws["ms_pagerank"]
        evals[f"rmat{scale}"] = {"uniform_iters": uni["iterations"], "uniform_ms": uni["ms_total"],
                                 "warm_iters": ws["iterations"], "warm_ms": warm_ms, "used_warm": ws["used_warm"],
                                 "features_ms": ws["ms_features"], "mlp_ms": ws["ms_mlp"],
                                 "resid_first_uniform": ws["resid_uniform_first"],
                                 "resid_first_warm": ws["resid_warm_first"],
                                 "time_ratio_uniform_over_warm": uni["ms_total"] / warm_ms}
    cfg = {"workload": "warm start: 256 R-MAT training graphs (scale U{16..20}, a,b,c jittered +-0.05, 65536 "
                       "sampled vertices each), standard PageRank to L1 < 1e-6 on held-out scale 24 and 26",
           "train_prep_s": round(prep_s, 1), "train_s": round(train_s, 1), "final_loss": loss}
    r24 = evals["rmat24"]
    _line("warm_start_time_ratio", r24["time_ratio_uniform_over_warm"], "x (uniform time / warm time, scale 24)",
          args, cfg, dtype="bf16 weights, f32 accumulate", evals=evals)


def main():
    args = parse()
    rank, local_rank, world = dist_env()
    if args.impl == "reference":
        return run_reference(args, rank, world)
    if args.workload != "pagerank":
        return {"cc_tc": run_cc_tc, "stream": run_stream, "batch": run_batch, "ppr": run_ppr,
                "warm": run_warm}[args.workload](args) or 0
    return run_gx(args, rank, local_rank, world)


if __name__ == "__main__":
    sys.exit(main())
