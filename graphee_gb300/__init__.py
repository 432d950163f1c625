"""graphee_gb300 — GraphMP's shard-wise gather-apply hot path on one GB300.

Python side of the C ABI in ``include/gx.h`` (libgx.so, built in-tree by
``graphee_gb300._build``).  It mirrors the reference's operator interface,
``GraphPS<T>`` (GraphMP/system/GraphPS.h:22-63): ``init(path, V, P,
max_iteration)`` then ``run()``, with the vertex program chosen by the app
class (PagerankPS / SsspPS / CcPS, GraphMP/app/*.cpp) and ``init_vertex``
overridable.  There is no CPU fallback: every compute call goes through
libgx.so and fails loudly when it is missing or no GPU is visible.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "libgx.so"

GX_OK, GX_ERR_INVALID, GX_ERR_IO, GX_ERR_FORMAT, GX_ERR_OOM, GX_ERR_CUDA, GX_ERR_TIMEOUT, \
    GX_ERR_NODEVICE, GX_ERR_STATE = range(9)
STATUS_NAMES = ["OK", "INVALID", "IO", "FORMAT", "OOM", "CUDA", "TIMEOUT", "NODEVICE", "STATE"]

APP_PAGERANK_REF, APP_PAGERANK_STD, APP_SSSP, APP_CC, APP_INDEGREE = range(5)
BUILD_DROP_SELF, BUILD_DEDUP, BUILD_SYMMETRIZE = 1, 2, 4
GPS_INF = 10000          # GraphMP/system/Global.h:50
INF_WEIGHTED = 0xFFFFFFFF


class GxError(RuntimeError):
    """A gx_status other than GX_OK, with gx_last_error()'s message."""

    def __init__(self, status: int, where: str, msg: str):
        self.status = status
        name = STATUS_NAMES[status] if 0 <= status < len(STATUS_NAMES) else str(status)
        super().__init__(f"{where}: GX_ERR_{name}: {msg}")


class Config(C.Structure):
    _fields_ = [("device", C.c_int32), ("cache_budget_bytes", C.c_int64), ("stream_slots", C.c_int32),
                ("copy_streams", C.c_int32),
                ("selective_threshold", C.c_double), ("heavy_degree", C.c_int32), ("tile_edges", C.c_int32),
                ("exact_order", C.c_int32),
                ("push_sparse", C.c_int32), ("use_graph", C.c_int32), ("wait_limit", C.c_uint32),
                ("verbose", C.c_int32), ("profile", C.c_int32),
                ("compress_cache", C.c_int32), ("push_edge_fraction", C.c_double), ("hot_vertices", C.c_int32),
                ("relabel", C.c_int32)]


class RunParams(C.Structure):
    _fields_ = [("app", C.c_int), ("max_iter", C.c_int32), ("damping", C.c_double), ("source", C.c_int32),
                ("weighted", C.c_int32), ("tolerance", C.c_double), ("use_init", C.c_int32),
                ("first_step", C.c_int32), ("async_mode", C.c_int32), ("checkpoint_every", C.c_int32),
                ("checkpoint_prefix", C.c_char_p)]


class RunStats(C.Structure):
    _fields_ = [("iterations", C.c_int32), ("push_iterations", C.c_int32), ("changed_last", C.c_int64),
                ("residual_l1_last", C.c_double), ("edges_scanned", C.c_int64), ("ms_total", C.c_double),
                ("ms_copy", C.c_double), ("ms_compute", C.c_double), ("overlap", C.c_double),
                ("h2d_bytes", C.c_int64), ("shards_resident", C.c_int32), ("shards_streamed", C.c_int32),
                ("kernel_launches", C.c_int32), ("pull_launches", C.c_int32), ("ms_pull", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class BatchTuning(C.Structure):
    _fields_ = [("threads", C.c_int32), ("lane_max", C.c_int32), ("ctas_per_sm", C.c_int32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class WarmStats(C.Structure):
    _fields_ = [("used_warm", C.c_int32), ("iterations", C.c_int32), ("resid_uniform_first", C.c_double),
                ("resid_warm_first", C.c_double), ("resid_last", C.c_double), ("ms_features", C.c_double),
                ("ms_mlp", C.c_double), ("ms_pagerank", C.c_double), ("ms_total", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class IterStats(C.Structure):
    _fields_ = [("changed", C.c_int64), ("active", C.c_int64), ("shards_active", C.c_int32),
                ("mode", C.c_int32), ("residual_l1", C.c_double), ("dangling", C.c_double),
                ("edges_scanned", C.c_int64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_lib = None


def lib() -> C.CDLL:
    """Loads libgx.so (raises if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RuntimeError(f"{LIB_PATH} is missing: run `python -c 'import __graft_entry__ as g; g.build()'`")
    L = C.CDLL(str(LIB_PATH))
    P, I32, I64, U64, D = C.c_void_p, C.c_int32, C.c_int64, C.c_uint64, C.c_double
    sig = {
        "gx_config_default": (None, [P]),
        "gx_run_params_default": (None, [P, C.c_int]),
        "gx_last_error": (C.c_char_p, []),
        "gx_create": (C.c_int, [P, P]),
        "gx_destroy": (C.c_int, [P]),
        "gx_set_wait_limit": (C.c_int, [P, C.c_uint32]),
        "gx_release_cached_memory": (C.c_int, [I32]),
        "gx_build_csc_gpu": (C.c_int, [I32, I32, I64, P, P, I32, P, P, P]),
        "gx_rmat_csc_gpu": (C.c_int, [I32, I32, I64, D, D, D, U64, I32, P, P, P]),
        "gx_write_values_npy": (C.c_int, [P, C.c_char_p]),
        "gx_read_values_npy": (C.c_int, [C.c_char_p, I64, P]),
        "gx_load_shards": (C.c_int, [P, C.c_char_p, I32, I32]),
        "gx_load_csc": (C.c_int, [P, I32, I32, P, P, P, P]),
        "gx_set_weights": (C.c_int, [P, P]),
        "gx_set_init": (C.c_int, [P, P]),
        "gx_run": (C.c_int, [P, P, P]),
        "gx_get_values": (C.c_int, [P, P]),
        "gx_get_iter_stats": (C.c_int, [P, I32, P]),
        "gx_rmat_edges": (C.c_int, [I32, I64, D, D, D, U64, I64, P, P]),
        "gx_build_csc": (C.c_int, [I32, I64, P, P, I32, P, P, P]),
        "gx_partition_bounds": (C.c_int, [I32, P, I32, P]),
        "gx_out_degree": (C.c_int, [I32, P, P, P]),
        "gx_write_shards": (C.c_int, [C.c_char_p, I32, I32, P, P, P, P]),
        "gx_read_shards": (C.c_int, [C.c_char_p, I32, I32, P, P, P, P, P]),
        "gx_edge_weights": (C.c_int, [U64, I32, P, P, P]),
        "gx_convert_edge_list": (C.c_int, [C.c_char_p, I32, I32, I32, C.c_char_p, P]),
        "gx_pagerank_noalloc": (C.c_int, [P, P, I64, I64, P, I32, I32, D, P, P, P]),
        "gx_triangle_count": (C.c_int, [P, P, P]),
        "gx_ppr": (C.c_int, [P, I32, P, I32, D, P, P]),
        "gx_batch_tuning_default": (None, [P]),
        "gx_mlp_num_params": (C.c_int32, []),
        "gx_mlp_create": (C.c_int, [I32, U64, P]),
        "gx_mlp_destroy": (C.c_int, [P]),
        "gx_mlp_get_params": (C.c_int, [P, P, P]),
        "gx_mlp_set_params": (C.c_int, [P, P, P]),
        "gx_mlp_add_graph": (C.c_int, [P, P, I32, I32, D]),
        "gx_mlp_train": (C.c_int, [P, I32, I32, D, P]),
        "gx_mlp_grad": (C.c_int, [P, P, P, I32, P, P]),
        "gx_mlp_predict": (C.c_int, [P, P, D, P, P, P]),
        "gx_pagerank_warm": (C.c_int, [P, P, I32, D, D, P]),
        "gx_batch_run": (C.c_int, [P, I32, P, I32, I32, D, P, P, P, P, P, P]),
        "gx_batch_autotune": (C.c_int, [P, I32, P, I32, I32, C.c_char_p, P, P]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def _check(st: int, where: str) -> None:
    if st != GX_OK:
        raise GxError(st, where, lib().gx_last_error().decode(errors="replace"))


def _ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


# ---------------------------------------------------------------- graphs ----

class Graph:
    """A graph in the reference's shard layout, held as one global CSC:
    bounds[P+1] destination ranges, off[V+1] in-edge offsets, col[E] source
    ids (ascending per destination), outdeg[V]."""

    def __init__(self, V, off, col, outdeg=None, P=1, bounds=None, weights=None):
        self.V = int(V)
        self.off = np.ascontiguousarray(off, dtype=np.int64)
        self.col = np.ascontiguousarray(col, dtype=np.int32)
        if outdeg is None:
            outdeg = out_degree(self.V, self.off, self.col)
        self.outdeg = np.ascontiguousarray(outdeg, dtype=np.int32)
        self.P = int(P)
        self.bounds = partition_bounds(self.V, self.off, self.P) if bounds is None else \
            np.ascontiguousarray(bounds, dtype=np.int32)
        self.weights = weights

    @property
    def E(self) -> int:
        return int(self.off[-1])

    def with_partitions(self, P: int) -> "Graph":
        return Graph(self.V, self.off, self.col, self.outdeg, P, None, self.weights)


def rmat_edges(scale: int, n: int, seed: int, a=0.57, b=0.19, c=0.19, first: int = 0):
    src = np.empty(n, np.int32)
    dst = np.empty(n, np.int32)
    _check(lib().gx_rmat_edges(scale, n, a, b, c, seed & 0xFFFFFFFFFFFFFFFF, first, _ptr(src), _ptr(dst)),
           "gx_rmat_edges")
    return src, dst


def build_csc(V: int, src, dst, flags=BUILD_DROP_SELF | BUILD_DEDUP):
    src = np.ascontiguousarray(src, np.int32)
    dst = np.ascontiguousarray(dst, np.int32)
    n = len(src)
    cap = 2 * n if flags & BUILD_SYMMETRIZE else n
    off = np.empty(V + 1, np.int64)
    col = np.empty(max(cap, 1), np.int32)
    nout = C.c_int64(0)
    _check(lib().gx_build_csc(V, n, _ptr(src), _ptr(dst), flags, _ptr(off), _ptr(col), C.byref(nout)),
           "gx_build_csc")
    return off, col[:nout.value].copy()


def build_csc_gpu(V: int, src, dst, flags=BUILD_DROP_SELF | BUILD_DEDUP, device: int = 0):
    """build_csc computed on the GPU (same output)."""
    src = np.ascontiguousarray(src, np.int32)
    dst = np.ascontiguousarray(dst, np.int32)
    n = len(src)
    cap = 2 * n if flags & BUILD_SYMMETRIZE else n
    off = np.empty(V + 1, np.int64)
    col = np.empty(max(cap, 1), np.int32)
    nout = C.c_int64(0)
    _check(lib().gx_build_csc_gpu(device, V, n, _ptr(src), _ptr(dst), flags, _ptr(off), _ptr(col), C.byref(nout)),
           "gx_build_csc_gpu")
    return off, col[:nout.value].copy()


def rmat_csc_gpu(scale: int, n: int, seed: int, a=0.57, b=0.19, c=0.19, flags=BUILD_DROP_SELF | BUILD_DEDUP,
                 device: int = 0):
    """The CSC of rmat_edges(scale, n, seed, a, b, c) built with `flags`,
    generated and built on the GPU."""
    cap = 2 * n if flags & BUILD_SYMMETRIZE else n
    off = np.empty((1 << scale) + 1, np.int64)
    col = np.empty(max(cap, 1), np.int32)
    nout = C.c_int64(0)
    _check(lib().gx_rmat_csc_gpu(device, scale, n, a, b, c, seed & 0xFFFFFFFFFFFFFFFF, flags, _ptr(off), _ptr(col),
                                 C.byref(nout)), "gx_rmat_csc_gpu")
    return off, col[:nout.value].copy()


def rmat_graph(scale: int, edge_factor: int, seed: int, P: int = 1, symmetric=False, a=0.57, b=0.19, c=0.19,
               weight_seed: int | None = None, gpu: bool = False, device: int = 0) -> Graph:
    """Seeded R-MAT graph, self-loops and duplicates removed (optionally
    symmetrised), as a Graph with P edge-balanced shards.  gpu=True
    generates and builds it on GPU `device` (the same graph)."""
    V = 1 << scale
    flags = BUILD_DROP_SELF | BUILD_DEDUP | (BUILD_SYMMETRIZE if symmetric else 0)
    if gpu:
        off, col = rmat_csc_gpu(scale, edge_factor * V, seed, a, b, c, flags, device)
    else:
        src, dst = rmat_edges(scale, edge_factor * V, seed, a, b, c)
        off, col = build_csc(V, src, dst, flags)
        del src, dst
    g = Graph(V, off, col, None, P)
    if weight_seed is not None:
        g.weights = edge_weights(weight_seed, g)
    return g


def partition_bounds(V: int, off: np.ndarray, P: int) -> np.ndarray:
    bounds = np.empty(P + 1, np.int32)
    _check(lib().gx_partition_bounds(V, _ptr(np.ascontiguousarray(off, np.int64)), P, _ptr(bounds)),
           "gx_partition_bounds")
    return bounds


def out_degree(V: int, off: np.ndarray, col: np.ndarray) -> np.ndarray:
    od = np.empty(V, np.int32)
    _check(lib().gx_out_degree(V, _ptr(off), _ptr(col), _ptr(od)), "gx_out_degree")
    return od


def edge_weights(seed: int, g: Graph) -> np.ndarray:
    w = np.empty(max(g.E, 1), np.uint32)
    _check(lib().gx_edge_weights(seed & 0xFFFFFFFFFFFFFFFF, g.V, _ptr(g.off), _ptr(g.col), _ptr(w)),
           "gx_edge_weights")
    return w[:g.E]


def write_shards(g: Graph, directory: str) -> str:
    d = str(directory)
    if not d.endswith("/"):
        d += "/"
    os.makedirs(d, exist_ok=True)
    _check(lib().gx_write_shards(d.encode(), g.V, g.P, _ptr(g.bounds), _ptr(g.off), _ptr(g.col), _ptr(g.outdeg)),
           "gx_write_shards")
    return d


def convert_edge_list(path: str, V: int, P: int, directory: str, flags=BUILD_DROP_SELF | BUILD_DEDUP) -> int:
    """Text edge list ("src dst" lines) -> the reference's shard directory."""
    d = str(directory)
    if not d.endswith("/"):
        d += "/"
    os.makedirs(d, exist_ok=True)
    n = C.c_int64(0)
    _check(lib().gx_convert_edge_list(str(path).encode(), V, P, flags, d.encode(), C.byref(n)),
           "gx_convert_edge_list")
    return n.value


def read_shards(directory: str, V: int, P: int) -> Graph:
    d = str(directory)
    if not d.endswith("/"):
        d += "/"
    E = C.c_int64(0)
    _check(lib().gx_read_shards(d.encode(), V, P, None, None, None, None, C.byref(E)), "gx_read_shards")
    bounds = np.empty(P + 1, np.int32)
    off = np.empty(V + 1, np.int64)
    col = np.empty(max(E.value, 1), np.int32)
    od = np.empty(V, np.int32)
    _check(lib().gx_read_shards(d.encode(), V, P, _ptr(bounds), _ptr(off), _ptr(col), _ptr(od), C.byref(E)),
           "gx_read_shards")
    return Graph(V, off, col[:E.value].copy(), od, P, bounds)


def batch_graph(n: int, scales=(10, 17), edge_factors=(8, 32), seed: int = 1, a=0.57, b=0.19, c=0.19):
    """n independent seeded R-MAT graphs (scale and edge factor drawn
    uniformly from the inclusive ranges, per-graph seeds), packed side by
    side into one Graph.  Returns (graph, inst_vbegin int32[n+1])."""
    rng = np.random.default_rng(seed)
    sc = rng.integers(scales[0], scales[1] + 1, size=n)
    ef = rng.integers(edge_factors[0], edge_factors[1] + 1, size=n)
    offs, cols, vbeg, ebase = [], [], [0], 0
    for i in range(n):
        V = 1 << int(sc[i])
        src, dst = rmat_edges(int(sc[i]), int(ef[i]) * V, seed * 1000003 + i, a, b, c)
        off, col = build_csc(V, src, dst)
        offs.append(off[:-1] + ebase)
        cols.append(col + vbeg[-1])
        ebase += int(off[-1])
        vbeg.append(vbeg[-1] + V)
    off = np.concatenate(offs + [np.array([ebase], np.int64)])
    col = np.concatenate(cols) if cols else np.zeros(0, np.int32)
    return Graph(vbeg[-1], off, col, None, 1), np.array(vbeg, np.int32)


# ---------------------------------------------------------------- engine ----

def read_values(path: str, n: int) -> np.ndarray:
    """A checkpoint written by Engine.write_values or gx_run (4-byte elements)."""
    out = np.empty(n, np.uint32)
    _check(lib().gx_read_values_npy(str(path).encode(), n, _ptr(out)), "gx_read_values_npy")
    return out


def release_cached_memory(device: int = 0) -> None:
    """Returns the device memory engines keep cached after close()."""
    _check(lib().gx_release_cached_memory(device), "gx_release_cached_memory")


def default_config(**kw) -> Config:
    cfg = Config()
    lib().gx_config_default(C.byref(cfg))
    for k, v in kw.items():
        setattr(cfg, k, v)
    return cfg


class Engine:
    """One gx_engine (one GPU, one host thread)."""

    def __init__(self, **config):
        self.cfg = default_config(**config)
        self._h = C.c_void_p()
        _check(lib().gx_create(C.byref(self.cfg), C.byref(self._h)), "gx_create")
        self.V = 0
        self.app = None

    def close(self):
        if self._h:
            lib().gx_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_wait_limit(self, polls: int) -> None:
        """Polls a device-side wait makes before the call gives up with
        GX_ERR_TIMEOUT (config.wait_limit)."""
        _check(lib().gx_set_wait_limit(self._h, polls), "gx_set_wait_limit")

    def load(self, g: Graph) -> "Engine":
        _check(lib().gx_load_csc(self._h, g.V, g.P, _ptr(g.bounds), _ptr(g.off), _ptr(g.col), _ptr(g.outdeg)),
               "gx_load_csc")
        self.V = g.V
        if g.weights is not None:
            self.set_weights(g.weights)
        return self

    def load_shards(self, directory: str, V: int, P: int) -> "Engine":
        d = str(directory)
        if not d.endswith("/"):
            d += "/"
        _check(lib().gx_load_shards(self._h, d.encode(), V, P), "gx_load_shards")
        self.V = V
        return self

    def set_weights(self, w: np.ndarray) -> None:
        w = np.ascontiguousarray(w, np.uint32)
        _check(lib().gx_set_weights(self._h, _ptr(w)), "gx_set_weights")

    def set_init(self, vals: np.ndarray) -> None:
        vals = np.ascontiguousarray(vals)
        if vals.itemsize != 4 or vals.size != self.V:
            raise ValueError("initial values must be V 4-byte elements")
        _check(lib().gx_set_init(self._h, _ptr(vals)), "gx_set_init")

    def run(self, app: int, max_iter: int, damping=0.85, source=None, weighted=False, tolerance=0.0,
            use_init=False, first_step=0, async_mode=False, checkpoint_every=0, checkpoint_prefix=None) -> dict:
        p = RunParams()
        lib().gx_run_params_default(C.byref(p), app)
        p.max_iter = max_iter
        p.damping = damping
        if source is not None:
            p.source = source
        p.weighted = int(weighted)
        p.tolerance = tolerance
        p.use_init = int(use_init)
        p.first_step = first_step
        p.async_mode = int(async_mode)
        p.checkpoint_every = checkpoint_every
        prefix = None if checkpoint_prefix is None else str(checkpoint_prefix).encode()
        p.checkpoint_prefix = prefix
        st = RunStats()
        _check(lib().gx_run(self._h, C.byref(p), C.byref(st)), "gx_run")
        self.app = app
        self._weighted = weighted
        return st.as_dict()

    def values(self, out: np.ndarray | None = None) -> np.ndarray:
        """The current values; `out` (V 4-byte elements, C-contiguous) is
        filled and reused instead of a new array."""
        if out is None:
            out = np.empty(self.V, np.uint32)
        elif out.dtype.itemsize != 4 or out.size != self.V or not out.flags.c_contiguous:
            raise ValueError("values(out=...): need a C-contiguous array of V 4-byte elements")
        out = out.view(np.uint32)
        _check(lib().gx_get_values(self._h, _ptr(out)), "gx_get_values")
        if self.app in (APP_PAGERANK_REF, APP_PAGERANK_STD):
            return out.view(np.float32)
        if self.app == APP_SSSP and self._weighted:
            return out
        return out.view(np.int32)

    def triangle_count(self) -> tuple[int, dict]:
        """Exact triangle count of the loaded (symmetric) graph."""
        tot = C.c_uint64(0)
        st = RunStats()
        _check(lib().gx_triangle_count(self._h, C.byref(tot), C.byref(st)), "gx_triangle_count")
        return int(tot.value), st.as_dict()

    def ppr(self, sources, iters: int, restart: float = 0.15, fetch: bool = True):
        """Personalized PageRank for len(sources) <= 64 columns; returns
        (R float32[V, k] or None, stats)."""
        src = np.ascontiguousarray(sources, np.int32)
        out = np.empty((self.V, len(src)), np.float32) if fetch else None
        st = RunStats()
        _check(lib().gx_ppr(self._h, len(src), _ptr(src), iters, restart, _ptr(out), C.byref(st)), "gx_ppr")
        return out, st.as_dict()

    def batch_run(self, inst_vbegin, pr_iters=30, cc_max_iter=1000, damping=0.85, tuning: dict | None = None):
        """Batched PageRank + CC over the packed instances (one persistent
        launch).  Returns (pr float32[V], cc int32[V], pr_steps, cc_steps, stats)."""
        vb = np.ascontiguousarray(inst_vbegin, np.int32)
        n = len(vb) - 1
        t = None
        if tuning is not None:
            t = BatchTuning()
            lib().gx_batch_tuning_default(C.byref(t))
            for k, v in tuning.items():
                setattr(t, k, v)
        pr = np.empty(self.V, np.float32)
        cc = np.empty(self.V, np.int32)
        ps = np.empty(n, np.int32)
        cs = np.empty(n, np.int32)
        st = RunStats()
        _check(lib().gx_batch_run(self._h, n, _ptr(vb), pr_iters, cc_max_iter, damping,
                                  None if t is None else C.byref(t), _ptr(pr), _ptr(cc), _ptr(ps), _ptr(cs),
                                  C.byref(st)), "gx_batch_run")
        return pr, cc, ps, cs, st.as_dict()

    def batch_autotune(self, inst_vbegin, pr_iters=30, cc_max_iter=1000, table_path: str | None = None):
        vb = np.ascontiguousarray(inst_vbegin, np.int32)
        best = BatchTuning()
        ms = C.c_double(0)
        _check(lib().gx_batch_autotune(self._h, len(vb) - 1, _ptr(vb), pr_iters, cc_max_iter,
                                       None if table_path is None else str(table_path).encode(), C.byref(best),
                                       C.byref(ms)), "gx_batch_autotune")
        return best.as_dict(), ms.value

    def pagerank_warm(self, mlp: "MLP", max_iter=500, tolerance=1e-6, damping=0.85) -> dict:
        """Standard PageRank to the L1 tolerance from the MLP's predicted start
        (uniform start when the prediction's first step is worse)."""
        ws = WarmStats()
        _check(lib().gx_pagerank_warm(self._h, mlp._h, max_iter, tolerance, damping, C.byref(ws)),
               "gx_pagerank_warm")
        self.app = APP_PAGERANK_STD
        return ws.as_dict()

    def write_values(self, path: str) -> None:
        """Checkpoint: the current values as a 1-D .npy file."""
        _check(lib().gx_write_values_npy(self._h, str(path).encode()), "gx_write_values_npy")

    def iter_stats(self, step: int) -> dict:
        s = IterStats()
        _check(lib().gx_get_iter_stats(self._h, step, C.byref(s)), "gx_get_iter_stats")
        return s.as_dict()


class MLP:
    """The warm-start network (gx_mlp): 6 -> 64 -> 64 -> 1, BF16 weights."""

    def __init__(self, device: int = 0, seed: int = 0):
        self._h = C.c_void_p()
        _check(lib().gx_mlp_create(device, seed & 0xFFFFFFFFFFFFFFFF, C.byref(self._h)), "gx_mlp_create")
        self.n_params = int(lib().gx_mlp_num_params())

    def close(self):
        if self._h:
            lib().gx_mlp_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self):
        p = np.empty(self.n_params, np.float32)
        nrm = np.empty(12, np.float32)
        _check(lib().gx_mlp_get_params(self._h, _ptr(p), _ptr(nrm)), "gx_mlp_get_params")
        return p, nrm

    def set_params(self, p=None, norm=None):
        p = None if p is None else np.ascontiguousarray(p, np.float32)
        norm = None if norm is None else np.ascontiguousarray(norm, np.float32)
        _check(lib().gx_mlp_set_params(self._h, _ptr(p), _ptr(norm)), "gx_mlp_set_params")

    def add_graph(self, engine: Engine, max_samples=65536, max_iter=300, tolerance=1e-9):
        _check(lib().gx_mlp_add_graph(self._h, engine._h, max_samples, max_iter, tolerance), "gx_mlp_add_graph")

    def train(self, epochs: int, batch: int = 4096, lr: float = 1e-3) -> float:
        loss = C.c_double(0)
        _check(lib().gx_mlp_train(self._h, epochs, batch, lr, C.byref(loss)), "gx_mlp_train")
        return loss.value

    def grad(self, x, t):
        x = np.ascontiguousarray(x, np.float32)
        t = np.ascontiguousarray(t, np.float32)
        g = np.empty(self.n_params, np.float32)
        loss = C.c_double(0)
        _check(lib().gx_mlp_grad(self._h, _ptr(x), _ptr(t), len(t), _ptr(g), C.byref(loss)), "gx_mlp_grad")
        return g, loss.value

    def predict(self, engine: Engine, damping=0.85):
        out = np.empty(engine.V, np.float32)
        mf, mm = C.c_double(0), C.c_double(0)
        _check(lib().gx_mlp_predict(self._h, engine._h, damping, _ptr(out), C.byref(mf), C.byref(mm)),
               "gx_mlp_predict")
        return out, {"ms_features": mf.value, "ms_mlp": mm.value}


# ------------------------------------------- the reference's app interface ----

class GraphPS:
    """Mirror of GraphPS<T> (GraphMP/system/GraphPS.h:22-63).

    ``init(data_path, vertex_num, partition_num, max_iteration=10)`` loads
    the shard directory (GraphPS.h:77); ``run()`` runs the superstep loop
    (GraphPS.h:171) on the GPU; after it ``vertex_msg`` holds _VertexMsg.
    Subclasses choose the vertex program (``app``) and may override
    ``init_vertex()`` to return initial values (GraphPS.h:60)."""

    app = APP_PAGERANK_REF

    def __init__(self, **config):
        self._engine = Engine(**config)
        self._DataPath = ""
        self._VertexNum = 0
        self._PartitionNum = 0
        self._MaxIteration = 0
        self.vertex_msg = None
        self.stats = None

    def init(self, data_path: str, vertex_num: int, partition_num: int, max_iteration: int = 10):
        self._DataPath = data_path
        self._VertexNum = vertex_num
        self._PartitionNum = partition_num
        self._MaxIteration = max_iteration
        self._engine.load_shards(data_path, vertex_num, partition_num)

    def init_vertex(self):
        """Return initial vertex values, or None for the app's own init."""
        return None

    def run_params(self) -> dict:
        return {}

    def run(self):
        init = self.init_vertex()
        if init is not None:
            self._engine.set_init(init)
        self.stats = self._engine.run(self.app, self._MaxIteration, use_init=init is not None, **self.run_params())
        self.vertex_msg = self._engine.values()
        return self.stats


class PagerankPS(GraphPS):
    """GraphMP/app/pagerank.cpp: PagerankPS<float>."""
    app = APP_PAGERANK_REF


class SsspPS(GraphPS):
    """GraphMP/app/sssp.cpp: unit-weight SSSP from vertex 1 (``source`` moves it)."""
    app = APP_SSSP
    source = 1

    def run_params(self):
        return {"source": self.source}


class CcPS(GraphPS):
    """GraphMP/app/cc.cpp: min-label connected components."""
    app = APP_CC
