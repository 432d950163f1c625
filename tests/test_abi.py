"""The C-ABI library loads on a machine without a GPU and exports every
function include/gx.h declares; host-only entry points work; engine entry
points report errors instead of crashing when no device is visible."""
import ctypes as C
import re
from pathlib import Path

import pytest

import graphee_gb300 as gx

ROOT = Path(__file__).resolve().parents[1]


def declared_functions():
    names = set()
    for h in sorted((ROOT / "include").glob("*.h")):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"^\s*(?:const\s+)?\w+\**\s+\**(gx_\w+)\s*\(", text, flags=re.M))
    return sorted(names)


def test_header_declares_functions():
    names = declared_functions()
    assert "gx_run" in names and "gx_load_shards" in names and len(names) >= 15


def test_library_exports_every_declared_symbol():
    L = gx.lib()
    missing = [n for n in declared_functions() if not hasattr(L, n)]
    assert not missing, missing


def test_config_defaults():
    cfg = gx.default_config()
    assert cfg.cache_budget_bytes == -1
    assert cfg.selective_threshold == pytest.approx(0.001)   # BF_THRE
    assert cfg.stream_slots >= 2
    p = gx.RunParams()
    gx.lib().gx_run_params_default(C.byref(p), gx.APP_SSSP)
    assert p.source == 1 and p.damping == pytest.approx(0.85)


def test_python_structs_match_the_header():
    """The ctypes mirrors of the ABI's structs have the C structs' size and
    field offsets (a field added on one side only would shift every later
    one)."""
    import subprocess
    import tempfile
    structs = {"gx_config": gx.Config, "gx_run_params": gx.RunParams, "gx_run_stats": gx.RunStats,
               "gx_iter_stats": gx.IterStats, "gx_batch_tuning": gx.BatchTuning, "gx_warm_stats": gx.WarmStats}
    lines = ["#include <stddef.h>", "#include <stdio.h>", "#include \"gx.h\"", "int main(void) {"]
    for cname, py in structs.items():
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for f, _ in py._fields_:
            lines.append(f'  printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines += ["  return 0;", "}"]
    with tempfile.TemporaryDirectory() as d:
        src, exe = Path(d) / "layout.c", Path(d) / "layout"
        src.write_text("\n".join(lines) + "\n")
        r = subprocess.run(["gcc", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], capture_output=True,
                           text=True)
        assert r.returncode == 0, r.stderr
        out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    got = {tuple(x.split()[:2]): int(x.split()[2]) for x in out if x}
    for cname, py in structs.items():
        assert got[(cname, "size")] == C.sizeof(py), cname
        for f, _ in py._fields_:
            assert got[(cname, f)] == getattr(py, f).offset, (cname, f)


def test_null_arguments_are_errors():
    L = gx.lib()
    assert L.gx_create(None, None) == gx.GX_ERR_INVALID
    assert L.gx_run(None, None, None) == gx.GX_ERR_INVALID
    assert L.gx_get_values(None, None) == gx.GX_ERR_INVALID
    assert "bad arguments" in L.gx_last_error().decode()
    assert L.gx_destroy(None) == gx.GX_OK


def test_cpp_header_compiles():
    import subprocess
    src = "#include \"gx_graphps.hpp\"\nint main(){ gx::PagerankPS<float>* p = nullptr; (void)p; return 0; }\n"
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-I", str(ROOT / "include"), "-x", "c++", "-"],
                       input=src, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_app_driver_reports_missing_device(tmp_path):
    """Without a GPU the driver fails with an error status, not a crash."""
    import subprocess
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    g = gx.rmat_graph(8, 4, seed=1, P=2)
    d = gx.write_shards(g, tmp_path / "s")
    app = gx.LIB_PATH.parent / "gx_app"
    if not app.exists():
        from graphee_gb300 import _build
        _build.build_apps()
    r = subprocess.run([str(app), "pagerank", d, str(g.V), "2", "5"], capture_output=True, text=True)
    assert r.returncode == 1 and "no CUDA device" in r.stderr, r.stderr
