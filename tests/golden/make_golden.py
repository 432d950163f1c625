"""Generates the golden fixtures in this directory from the REFERENCE's own
GraphMP apps.

The reference ships no tests, fixtures or expected outputs, so its apps are
compiled from the reference tree against single-rank stubs (oracle/Makefile,
target `ref`) and run here on small graphs written in the reference's shard
format.  Each fixture stores the input graph (global CSC + shard bounds) and
the reference's final _VertexMsg plus its per-iteration `Update` counts
(GraphMP/system/GraphPS.h:375-382) for PageRank (20 iterations), SSSP from
vertex 1 (the reference's hard-coded source) and from vertex 0, and CC.

Run from the repository root, where the reference tree is available:
    make -C oracle ref && python tests/golden/make_golden.py
"""
from __future__ import annotations

import re
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
import graphee_gb300 as gx  # noqa: E402

REF = ROOT / "oracle" / "_ref"
OUT = Path(__file__).resolve().parent
ITER_RE = re.compile(r"Iteration: (\d+), uses \S+ ms, Update (-?\d+)")


def run_ref(app: str, d: str, V: int, P: int, iters: int, dtype, source: int | None = None):
    with tempfile.NamedTemporaryFile(suffix=".bin") as f:
        cmd = [str(REF / f"ref_{app}"), d, str(V), str(P), str(iters), f.name, "2"]
        if source is not None:
            cmd.append(str(source))
        r = subprocess.run(cmd, capture_output=True, text=True, timeout=600)
        if r.returncode != 0:
            raise RuntimeError(f"{cmd} failed ({r.returncode}):\n{r.stderr[-2000:]}")
        vals = np.fromfile(f.name, dtype=dtype)
    steps = [(int(a), int(b)) for a, b in ITER_RE.findall(r.stderr)]
    changed = np.array([b for _, b in steps], np.int64)
    assert [a for a, _ in steps] == list(range(len(steps))), steps
    return vals, changed


def graph_from_edges(V, edges, P, flags=gx.BUILD_DROP_SELF | gx.BUILD_DEDUP):
    e = np.asarray(edges, np.int32).reshape(-1, 2)
    off, col = gx.build_csc(V, e[:, 0], e[:, 1], flags)
    return gx.Graph(V, off, col, None, P)


def cases():
    rng = np.random.default_rng(7)
    yield "rmat10_p4", gx.rmat_graph(10, 8, seed=1, P=4)
    yield "rmat12_sym_p8", gx.rmat_graph(12, 8, seed=2, P=8, symmetric=True)
    yield "rmat11_p1", gx.rmat_graph(11, 16, seed=3, P=1)
    # path 0->1->...->49 plus the reverse of every third edge
    path = [(i, i + 1) for i in range(49)] + [(i + 1, i) for i in range(0, 49, 3)]
    yield "path50_p3", graph_from_edges(50, path, 3)
    # a hub with 3000 in-neighbours (above the heavy-vertex threshold) and a
    # ring through the leaves
    hub = [(i, 0) for i in range(1, 3001)] + [(0, 1), (0, 2)] + [(i, i % 3000 + 1) for i in range(1, 3001, 7)]
    yield "hub3000_p2", graph_from_edges(3001, hub, 2)
    # two components, isolated vertices, dangling vertices, self-loops kept
    e = [(1, 2), (2, 3), (3, 1), (3, 4), (4, 4), (6, 7), (7, 8), (8, 6), (9, 9), (8, 10), (12, 11)]
    yield "twocomp_selfloop_p5", graph_from_edges(16, e, 5, flags=gx.BUILD_DEDUP)
    # more shards than edge mass: several shards are empty ranges
    e = [(int(a), int(b)) for a, b in rng.integers(0, 8, size=(12, 2))] + [(40, 41), (41, 40)]
    yield "sparse_emptyshards_p16", graph_from_edges(64, e, 16)


def main():
    for name, g in cases():
        with tempfile.TemporaryDirectory() as td:
            d = gx.write_shards(g, td)
            out = {"V": g.V, "P": g.P, "bounds": g.bounds, "off": g.off, "col": g.col, "outdeg": g.outdeg}
            out["pr"], out["pr_changed"] = run_ref("pagerank", d, g.V, g.P, 20, np.float32)
            out["sssp1"], out["sssp1_changed"] = run_ref("sssp", d, g.V, g.P, 200, np.int32, 1)
            out["sssp0"], out["sssp0_changed"] = run_ref("sssp", d, g.V, g.P, 200, np.int32, 0)
            out["cc"], out["cc_changed"] = run_ref("cc", d, g.V, g.P, 200, np.int32)
        np.savez_compressed(OUT / f"{name}.npz", **out)
        print(name, "V", g.V, "E", g.E, "P", g.P, "pr iters", len(out["pr_changed"]),
              "sssp1 iters", len(out["sssp1_changed"]), "cc iters", len(out["cc_changed"]))


if __name__ == "__main__":
    main()
