"""GPU graph construction (gx_build_csc_gpu, gx_rmat_csc_gpu) against the
host build, bit for bit: offsets and source order, every flag combination,
empty and ragged inputs, vertex counts that are not powers of two."""
import time

import numpy as np
import pytest

import graphee_gb300 as gx

pytestmark = pytest.mark.gpu

FLAGS = [0, gx.BUILD_DROP_SELF, gx.BUILD_DEDUP, gx.BUILD_SYMMETRIZE,
         gx.BUILD_DROP_SELF | gx.BUILD_DEDUP, gx.BUILD_DROP_SELF | gx.BUILD_DEDUP | gx.BUILD_SYMMETRIZE,
         gx.BUILD_DEDUP | gx.BUILD_SYMMETRIZE]


@pytest.mark.parametrize("flags", FLAGS)
@pytest.mark.parametrize("V,n", [(1, 0), (1, 5), (7, 40), (1000, 20000), (100003, 300000)])
def test_build_matches_host(V, n, flags):
    rng = np.random.default_rng(V * 31 + n + flags)
    src = rng.integers(0, V, n, dtype=np.int32)
    dst = rng.integers(0, max(1, V // 3), n, dtype=np.int32)   # a zero-degree tail of destinations
    k = n // 10
    src[:k] = dst[:k]                                            # self-loops
    src[k:2 * k] = src[:k]                                       # duplicates
    dst[k:2 * k] = dst[:k]
    off_h, col_h = gx.build_csc(V, src, dst, flags)
    off_g, col_g = gx.build_csc_gpu(V, src, dst, flags)
    assert np.array_equal(off_h, off_g)
    assert np.array_equal(col_h, col_g)


def test_build_rejects_bad_ids():
    with pytest.raises(gx.GxError):
        gx.build_csc_gpu(10, np.array([1, 10], np.int32), np.array([0, 1], np.int32))
    with pytest.raises(gx.GxError):
        gx.build_csc_gpu(10, np.array([1, 2], np.int32), np.array([-1, 1], np.int32))


@pytest.mark.parametrize("symmetric", [False, True])
@pytest.mark.parametrize("scale", [10, 16, 20])
def test_rmat_gpu_matches_host(scale, symmetric):
    t0 = time.perf_counter()
    g_h = gx.rmat_graph(scale, 16, seed=20240601, symmetric=symmetric)
    t1 = time.perf_counter()
    g_g = gx.rmat_graph(scale, 16, seed=20240601, symmetric=symmetric, gpu=True)
    t2 = time.perf_counter()
    assert np.array_equal(g_h.off, g_g.off)
    assert np.array_equal(g_h.col, g_g.col)
    print(f"scale {scale} sym {symmetric}: host {t1 - t0:.3f} s, gpu {t2 - t1:.3f} s")
