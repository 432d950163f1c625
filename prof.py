"""Runs one workload of the engine and nothing else, so a profiler sees only
its kernels:  python prof.py --app pagerank --scale 22 --iters 3

Graph: seeded R-MAT (a,b,c=.57,.19,.19), edge factor 16, 256 shards, the
same generator and seed as bench.py.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

import graphee_gb300 as gx

APPS = {"pagerank": gx.APP_PAGERANK_REF, "pagerank_std": gx.APP_PAGERANK_STD, "sssp": gx.APP_SSSP, "cc": gx.APP_CC}
OTHER = ["tc", "ppr", "batch", "warm", "build"]


def run_other(a):
    """Workloads beside the superstep loop, one each, for a profiler."""
    t0 = time.perf_counter()
    if a.app == "build":
        g = gx.rmat_graph(a.scale, a.edge_factor, seed=20240601, gpu=True)
        print(json.dumps({"V": g.V, "E": g.E, "wall_s": time.perf_counter() - t0}))
        return
    if a.app == "batch":
        g, vb = gx.batch_graph(256, scales=(10, 15), edge_factors=(8, 32), seed=20240601)
        with gx.Engine() as e:
            e.load(g)
            out = e.batch_run(vb, 30, 1000)
        print(json.dumps({"V": g.V, "E": g.E, "stats": out[-1]}, default=str))
        return
    sym = a.app == "tc"
    g = gx.rmat_graph(a.scale, a.edge_factor, seed=20240601, P=256, symmetric=sym, gpu=True)
    with gx.Engine() as e:
        e.load(g)
        if a.app == "tc":
            n, st = e.triangle_count()
            st["triangles"] = n
        elif a.app == "ppr":
            src = np.random.default_rng(1).integers(0, g.V, size=64).astype(np.int32)
            st = e.ppr(src, a.iters, fetch=False)[1]
        else:
            m = gx.MLP(seed=1)
            st = e.pagerank_warm(m, max_iter=a.iters)
        st.update({"V": g.V, "E": g.E, "wall_s": time.perf_counter() - t0})
        print(json.dumps(st))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--app", default="pagerank", choices=sorted(APPS) + OTHER)
    ap.add_argument("--scale", type=int, default=22)
    ap.add_argument("--edge-factor", type=int, default=16)
    ap.add_argument("--iters", type=int, default=3)
    ap.add_argument("--runs", type=int, default=1)
    ap.add_argument("--graph", type=int, default=0, help="replay supersteps as a CUDA graph")
    ap.add_argument("--heavy-degree", type=int, default=None)
    ap.add_argument("--tile-edges", type=int, default=None)
    ap.add_argument("--profile-kernels", type=int, default=0, help="time each pull launch with CUDA events")
    ap.add_argument("--relabel", type=int, default=0, help="config.relabel: per-shard renumbering at load")
    a = ap.parse_args()
    if a.app in OTHER:
        run_other(a)
        return
    sym = a.app == "cc"
    g = gx.rmat_graph(a.scale, a.edge_factor, seed=20240601, P=256, symmetric=sym,
                      weight_seed=7 if a.app == "sssp" else None, gpu=True)
    cfg = {"use_graph": a.graph, "profile": a.profile_kernels, "relabel": a.relabel}
    if a.heavy_degree is not None:
        cfg["heavy_degree"] = a.heavy_degree
    if a.tile_edges is not None:
        cfg["tile_edges"] = a.tile_edges
    with gx.Engine(**cfg) as e:
        e.load(g)
        kw = {"source": 0, "weighted": True} if a.app == "sssp" else {}
        for _ in range(a.runs):
            t0 = time.perf_counter()
            st = e.run(APPS[a.app], a.iters, **kw)
            st["wall_s"] = time.perf_counter() - t0
        st.update({"V": g.V, "E": g.E})
        if st["pull_launches"] and st["ms_pull"]:
            st["pull_ms_avg"] = st["ms_pull"] / st["pull_launches"]
            st["pull_alg_GBps"] = (8 * g.E + 24 * g.V) / (st["pull_ms_avg"] / 1e3) / 1e9
        print(json.dumps(st))


if __name__ == "__main__":
    main()
