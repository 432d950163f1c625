"""Child process of tests/test_host_sanitizers.py (not a test module).

Drives the host graph code (graphee_gb300/csrc/gx_graph.cpp: R-MAT edges,
CSC build, partition, out-degree, weights, shard and .npy I/O, the edge-list
converter) and the oracle (oracle/gx_oracle.cpp: the engine loop and every
vertex program, triangles, PPR), both compiled with AddressSanitizer and
UBSan, through their C ABI, including the error paths for malformed input.
A sanitizer report ends the process with a non-zero status; a wrong result
fails an assert.

usage: python sanitized_host_run.py <libgx_host_san.so> <libgxoracle_san.so> <scratch dir>
"""
import ctypes as C
import os
import sys

import numpy as np

host = C.CDLL(sys.argv[1])
orc = C.CDLL(sys.argv[2])
tmp = sys.argv[3]
P, I32, I64, U64, D = C.c_void_p, C.c_int32, C.c_int64, C.c_uint64, C.c_double


def bind(lib, name, res, args):
    f = getattr(lib, name)
    f.restype = res
    f.argtypes = args
    return f


rmat = bind(host, "gx_rmat_edges", C.c_int, [I32, I64, D, D, D, U64, I64, P, P])
build = bind(host, "gx_build_csc", C.c_int, [I32, I64, P, P, I32, P, P, P])
bounds_of = bind(host, "gx_partition_bounds", C.c_int, [I32, P, I32, P])
out_degree = bind(host, "gx_out_degree", C.c_int, [I32, P, P, P])
weights_of = bind(host, "gx_edge_weights", C.c_int, [U64, I32, P, P, P])
write_shards = bind(host, "gx_write_shards", C.c_int, [C.c_char_p, I32, I32, P, P, P, P])
read_shards = bind(host, "gx_read_shards", C.c_int, [C.c_char_p, I32, I32, P, P, P, P, P])
convert = bind(host, "gx_convert_edge_list", C.c_int, [C.c_char_p, I32, I32, I32, C.c_char_p, P])
read_npy = bind(host, "gx_read_values_npy", C.c_int, [C.c_char_p, I64, P])
gxo_run = bind(orc, "gxo_run", C.c_int, [C.c_int, I32, I32, P, P, P, P, P, I32, D, I32, D, C.c_int,
                                          P, P, P, P, P])
gxo_tri = bind(orc, "gxo_triangles", C.c_uint64, [I32, P, P, C.c_int])
gxo_ppr = bind(orc, "gxo_ppr", C.c_int, [I32, P, P, P, I32, P, I32, D, C.c_int, P])
DROP_SELF, DEDUP, SYM = 1, 2, 4


def ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def graph(scale, ef, flags, seed=5):
    V, n = 1 << scale, ef << scale
    src, dst = np.empty(n, np.int32), np.empty(n, np.int32)
    assert rmat(scale, n, 0.57, 0.19, 0.19, seed, 0, ptr(src), ptr(dst)) == 0
    off = np.empty(V + 1, np.int64)
    col = np.empty(2 * n if flags & SYM else n, np.int32)
    ne = C.c_int64(0)
    assert build(V, n, ptr(src), ptr(dst), flags, ptr(off), ptr(col), C.byref(ne)) == 0
    col = col[:ne.value].copy()
    assert off[0] == 0 and off[-1] == ne.value and (np.diff(off) >= 0).all()
    return V, off, col, src, dst


# CSC build against numpy: dedup, no self-loops, sources ascending per destination.
V, off, col, src, dst = graph(12, 16, DROP_SELF | DEDUP)
keep = src != dst
pairs = np.unique(np.stack([dst[keep], src[keep]], 1), axis=0)
assert np.array_equal(col, pairs[:, 1]) and np.array_equal(np.diff(off), np.bincount(pairs[:, 0], minlength=V))

P_ = 8
bounds = np.empty(P_ + 1, np.int32)
assert bounds_of(V, ptr(off), P_, ptr(bounds)) == 0 and bounds[0] == 0 and bounds[-1] == V
outdeg = np.empty(V, np.int32)
assert out_degree(V, ptr(off), ptr(col), ptr(outdeg)) == 0
assert np.array_equal(outdeg, np.bincount(col, minlength=V))
w = np.empty(len(col), np.uint32)
assert weights_of(7, V, ptr(off), ptr(col), ptr(w)) == 0 and w.min() >= 1 and w.max() <= 255

# Shard files in the reference layout: round trip, then malformed files.
d = os.path.join(tmp, "shards") + "/"
os.makedirs(d)
assert write_shards(d.encode(), V, P_, ptr(bounds), ptr(off), ptr(col), ptr(outdeg)) == 0
b2, e_out = np.empty(P_ + 1, np.int32), C.c_int64(0)
assert read_shards(d.encode(), V, P_, ptr(b2), None, None, None, C.byref(e_out)) == 0 and e_out.value == len(col)
off2, col2, od2 = np.empty(V + 1, np.int64), np.empty(len(col), np.int32), np.empty(V, np.int32)
assert read_shards(d.encode(), V, P_, ptr(b2), ptr(off2), ptr(col2), ptr(od2), C.byref(e_out)) == 0
assert np.array_equal(b2, bounds) and np.array_equal(off2, off) and np.array_equal(col2, col)


def read_all():
    """Size query (headers only), then the full read; the first error status."""
    st = read_shards(d.encode(), V, P_, ptr(b2), None, None, None, C.byref(e_out))
    if st != 0:
        return st
    n = max(e_out.value, 1)
    return read_shards(d.encode(), V, P_, ptr(b2), ptr(np.empty(V + 1, np.int64)), ptr(np.empty(n, np.int32)),
                       ptr(np.empty(V, np.int32)), C.byref(e_out))


shard3 = d + "3.edge.npy"
raw = open(shard3, "rb").read()
open(shard3, "wb").write(raw[: len(raw) // 2])                      # truncated payload
assert read_all() != 0
open(shard3, "wb").write(raw[:60])                                  # header cut short
assert read_all() != 0
open(shard3, "wb").write(b"")                                       # empty file
assert read_all() != 0
os.remove(shard3)                                                   # missing file
assert read_all() != 0
open(shard3, "wb").write(raw)                                       # intact again
assert read_all() == 0

# .npy values: short and garbage files are errors, not reads past the end.
vals = np.arange(100, dtype=np.float32)
np.save(os.path.join(tmp, "v.npy"), vals)
out = np.empty(100, np.float32)
assert read_npy(os.path.join(tmp, "v.npy").encode(), 100, ptr(out)) == 0 and np.array_equal(out, vals)
assert read_npy(os.path.join(tmp, "v.npy").encode(), 101, ptr(np.empty(101, np.float32))) != 0
blob = open(os.path.join(tmp, "v.npy"), "rb").read()
open(os.path.join(tmp, "short.npy"), "wb").write(blob[:200])
assert read_npy(os.path.join(tmp, "short.npy").encode(), 100, ptr(out)) != 0
open(os.path.join(tmp, "junk.npy"), "wb").write(b"\x93NUMPY\x01\x00\xff\xff{'descr'")
assert read_npy(os.path.join(tmp, "junk.npy").encode(), 100, ptr(out)) != 0

# Bad ids are rejected.
bad = np.array([0, V], np.int32)
assert build(V, 1, ptr(bad[:1]), ptr(bad[1:]), DEDUP, ptr(np.empty(V + 1, np.int64)),
             ptr(np.empty(1, np.int32)), C.byref(C.c_int64(0))) != 0

# Edge-list converter: comments, blank lines, self-loops, duplicates.
el = os.path.join(tmp, "edges.tsv")
with open(el, "w") as f:
    f.write("# comment\n% other comment\n\n0 1\n1 2\n2 0\n2 2\n0 1\n3\t4\n")
n_kept = C.c_int64(0)
cd = os.path.join(tmp, "conv") + "/"
os.makedirs(cd)
assert convert(el.encode(), 5, 2, DROP_SELF | DEDUP, cd.encode(), C.byref(n_kept)) == 0 and n_kept.value == 4
with open(el, "a") as f:
    f.write("5 x\n")                                                # malformed line
assert convert(el.encode(), 5, 2, DROP_SELF | DEDUP, cd.encode(), C.byref(n_kept)) != 0

# Oracle: every vertex program on the directed graph, CC and triangles on the
# symmetric one, PPR.
it = C.c_int32(0)
for app, dt, wts, src_v in ((0, np.float32, None, 1), (1, np.float64, None, 1), (5, np.float64, None, 1),
                            (2, np.int32, None, 1), (2, np.uint32, w, 0), (4, np.int32, None, 1)):
    res = np.empty(V, dt)
    ch, ms = np.zeros(60, np.int64), np.zeros(60)
    assert gxo_run(app, V, P_, ptr(bounds), ptr(off), ptr(col), ptr(outdeg), ptr(wts), 60, 0.85, src_v, 0.0, 4,
                   None, ptr(res), ptr(ch), ptr(ms), C.byref(it)) == 0
    assert 1 <= it.value <= 60
Vs, offs, cols, _, _ = graph(11, 8, DROP_SELF | DEDUP | SYM, seed=9)
bs = np.empty(P_ + 1, np.int32)
assert bounds_of(Vs, ptr(offs), P_, ptr(bs)) == 0
ods = np.empty(Vs, np.int32)
assert out_degree(Vs, ptr(offs), ptr(cols), ptr(ods)) == 0
lab = np.empty(Vs, np.int32)
ch, ms = np.zeros(200, np.int64), np.zeros(200)
assert gxo_run(3, Vs, P_, ptr(bs), ptr(offs), ptr(cols), ptr(ods), None, 200, 0.85, 1, 0.0, 4, None, ptr(lab),
               ptr(ch), ptr(ms), C.byref(it)) == 0
assert (lab <= np.arange(Vs)).all()
assert gxo_tri(Vs, ptr(offs), ptr(cols), 4) > 0
srcs = np.array([0, 5, 17], np.int32)
R = np.empty((V, 3), np.float64)
assert gxo_ppr(V, ptr(off), ptr(col), ptr(outdeg), 3, ptr(srcs), 10, 0.15, 4, ptr(R)) == 0
assert np.isfinite(R).all() and (R.sum(0) <= 1 + 1e-9).all()
print("sanitized host run ok")
