"""The oracle's restatement of the graph construction (seeded R-MAT, CSC
build, partition rule, out-degree, SSSP weights) against the library's, on
CPU: the benchmark's reference arm builds its input with the former, the
GPU arm with the latter, so both measure the same graph."""
import numpy as np
import pytest

import graphee_gb300 as gx
import gx_oracle as O


@pytest.mark.parametrize("scale,ef,sym,P", [(10, 8, False, 1), (12, 16, False, 8), (13, 16, True, 16),
                                            (16, 16, False, 256)])
def test_oracle_rmat_graph_equals_library(scale, ef, sym, P):
    a = O.rmat_graph(scale, ef, seed=20240601, P=P, symmetric=sym, weight_seed=7)
    b = gx.rmat_graph(scale, ef, seed=20240601, P=P, symmetric=sym, weight_seed=7)
    assert a.V == b.V and a.E == b.E
    for name in ("off", "col", "outdeg", "bounds", "weights"):
        assert np.array_equal(getattr(a, name), getattr(b, name)), name


def test_oracle_rmat_jittered_quadrants():
    a = O.rmat_graph(11, 16, seed=5, a=0.55, b=0.22, c=0.16)
    b = gx.rmat_graph(11, 16, seed=5, a=0.55, b=0.22, c=0.16)
    assert np.array_equal(a.off, b.off) and np.array_equal(a.col, b.col)


def test_oracle_shard_files_equal_library(tmp_path):
    a = O.rmat_graph(12, 16, seed=3, P=8)
    b = gx.rmat_graph(12, 16, seed=3, P=8)
    da, db = tmp_path / "a", tmp_path / "b"
    O.write_shards(a, str(da))
    gx.write_shards(b, str(db))
    names = sorted(p.name for p in da.iterdir())
    assert names == sorted(p.name for p in db.iterdir())
    for n in names:
        assert (da / n).read_bytes() == (db / n).read_bytes(), n
