"""Host graph construction and the reference's shard format (no GPU)."""
import numpy as np
import pytest

import graphee_gb300 as gx


def test_rmat_is_counter_based():
    s1, d1 = gx.rmat_edges(12, 5000, seed=3)
    s2, d2 = gx.rmat_edges(12, 5000, seed=3)
    assert np.array_equal(s1, s2) and np.array_equal(d1, d2)
    a, b = gx.rmat_edges(12, 2000, seed=3, first=3000)
    assert np.array_equal(a, s1[3000:]) and np.array_equal(b, d1[3000:])
    s3, _ = gx.rmat_edges(12, 5000, seed=4)
    assert not np.array_equal(s1, s3)
    assert s1.min() >= 0 and s1.max() < 4096 and d1.max() < 4096


def test_rmat_quadrant_frequencies():
    src, dst = gx.rmat_edges(16, 200000, seed=1)
    top_s, top_d = src >> 15, dst >> 15   # first level's quadrant
    q = np.bincount(top_s * 2 + top_d, minlength=4) / len(src)
    assert np.allclose(q, [0.57, 0.19, 0.19, 0.05], atol=0.005)


def test_build_csc_matches_numpy():
    src, dst = gx.rmat_edges(10, 20000, seed=5)
    V = 1024
    off, col = gx.build_csc(V, src, dst, gx.BUILD_DROP_SELF | gx.BUILD_DEDUP)
    keep = src != dst
    pairs = np.unique(np.stack([dst[keep], src[keep]], 1), axis=0)   # sorted by (dst, src)
    assert np.array_equal(col, pairs[:, 1])
    assert np.array_equal(off, np.concatenate([[0], np.cumsum(np.bincount(pairs[:, 0], minlength=V))]))
    # without dedup / self-loop removal every edge survives
    off2, col2 = gx.build_csc(V, src, dst, 0)
    assert off2[-1] == len(src)


def test_build_csc_symmetric():
    src, dst = gx.rmat_edges(9, 4000, seed=8)
    off, col = gx.build_csc(512, src, dst, gx.BUILD_DROP_SELF | gx.BUILD_DEDUP | gx.BUILD_SYMMETRIZE)
    dst_of = np.repeat(np.arange(512), np.diff(off))
    e = set(zip(col.tolist(), dst_of.tolist()))
    assert all((v, u) in e for u, v in e)
    assert all(u != v for u, v in e)


def test_build_csc_rejects_bad_ids():
    with pytest.raises(gx.GxError):
        gx.build_csc(4, np.array([0, 5], np.int32), np.array([1, 2], np.int32))


def format_spark_bounds(off, P):
    """format_spark.py:91-108 restated: per = ceil(E/P); bound_i = argmax(cum >= per*i)."""
    E = int(off[-1])
    per = -(-E // P)
    b = [0]
    for i in range(1, P):
        hit = np.nonzero(off >= per * i)[0]
        b.append(int(hit[0]) if len(hit) else len(off) - 1)
    b.append(len(off) - 1)
    return np.maximum.accumulate(np.array(b))


@pytest.mark.parametrize("P", [1, 2, 7, 64])
def test_partition_bounds_rule(P):
    g = gx.rmat_graph(11, 8, seed=2)
    assert np.array_equal(gx.partition_bounds(g.V, g.off, P), format_spark_bounds(g.off, P))


def test_shard_roundtrip_and_layout(tmp_path):
    g = gx.rmat_graph(10, 8, seed=6, P=5)
    d = gx.write_shards(g, tmp_path / "s")
    # the reference's layout: [E, len(indices), len(indptr), start, end, indices..., indptr...]
    for p in range(g.P):
        a = np.load(tmp_path / "s" / f"{p}.edge.npy")
        assert a.dtype == np.int32 and a.ndim == 1
        s, e = g.bounds[p], g.bounds[p + 1]
        ni, npt = a[1], a[2]
        assert a[3] == s and a[4] == e and npt == e - s + 1 and len(a) == 5 + ni + npt
        assert np.array_equal(a[5:5 + ni], g.col[g.off[s]:g.off[e]])
        assert np.array_equal(a[5 + ni:], g.off[s:e + 1] - g.off[s])
    assert np.array_equal(np.load(tmp_path / "s" / "vertexout.npy"), g.outdeg)
    assert np.array_equal(np.load(tmp_path / "s" / "vertexin.npy"), np.diff(g.off).astype(np.int32))
    h = gx.read_shards(d, g.V, g.P)
    assert np.array_equal(h.off, g.off) and np.array_equal(h.col, g.col)
    assert np.array_equal(h.bounds, g.bounds) and np.array_equal(h.outdeg, g.outdeg)


def test_read_shards_errors(tmp_path):
    g = gx.rmat_graph(8, 4, seed=1, P=3)
    d = gx.write_shards(g, tmp_path / "s")
    with pytest.raises(gx.GxError) as ei:
        gx.read_shards(d, g.V, 4)          # shard 3 missing
    assert ei.value.status == gx.GX_ERR_IO
    with pytest.raises(gx.GxError) as ei:
        gx.read_shards(d, g.V + 5, 3)      # last shard does not end at V
    assert ei.value.status == gx.GX_ERR_FORMAT
    a = np.load(tmp_path / "s" / "1.edge.npy")
    a[1] += 1                               # header length mismatch
    np.save(tmp_path / "s" / "1.edge.npy", a)
    with pytest.raises(gx.GxError) as ei:
        gx.read_shards(d, g.V, 3)
    assert ei.value.status == gx.GX_ERR_FORMAT


def test_edge_weights():
    g = gx.rmat_graph(9, 8, seed=3)
    w = gx.edge_weights(77, g)
    assert w.min() >= 1 and w.max() <= 255
    assert np.array_equal(w, gx.edge_weights(77, g))
    assert not np.array_equal(w, gx.edge_weights(78, g))
    h = g.with_partitions(3)
    assert np.array_equal(gx.edge_weights(77, h), w)   # a function of (u, v), not of the layout


def test_convert_edge_list(tmp_path):
    src, dst = gx.rmat_edges(10, 6000, seed=12)
    lines = ["# comment", "% another"] + [f"{a}\t{b}" for a, b in zip(src.tolist(), dst.tolist())]
    (tmp_path / "g.tsv").write_text("\n".join(lines) + "\n")
    E = gx.convert_edge_list(tmp_path / "g.tsv", 1024, 5, tmp_path / "s")
    h = gx.read_shards(tmp_path / "s", 1024, 5)
    off, col = gx.build_csc(1024, src, dst)
    assert E == off[-1] == h.E
    assert np.array_equal(h.off, off) and np.array_equal(h.col, col)
    assert np.array_equal(h.bounds, gx.partition_bounds(1024, off, 5))
    (tmp_path / "bad.tsv").write_text("1 2\n3 x\n")
    with pytest.raises(gx.GxError) as ei:
        gx.convert_edge_list(tmp_path / "bad.tsv", 1024, 2, tmp_path / "t")
    assert ei.value.status == gx.GX_ERR_FORMAT


def test_values_npy_roundtrip_and_errors(tmp_path):
    for dt in (np.float32, np.int32, np.uint32):
        a = (np.arange(1000) * 7 % 113).astype(dt)
        p = tmp_path / f"v_{np.dtype(dt).str[1:]}.npy"
        np.save(p, a)
        back = gx.read_values(p, a.size)
        assert np.array_equal(back.view(dt), a)
    p = tmp_path / "v.npy"
    np.save(p, np.zeros(10, np.float32))
    with pytest.raises(gx.GxError):
        gx.read_values(p, 11)                       # wrong length
    np.save(tmp_path / "d.npy", np.zeros(10, np.float64))
    with pytest.raises(gx.GxError):
        gx.read_values(tmp_path / "d.npy", 10)      # 8-byte elements
    with pytest.raises(gx.GxError):
        gx.read_values(tmp_path / "missing.npy", 10)
