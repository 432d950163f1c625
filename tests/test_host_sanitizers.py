"""Host code under AddressSanitizer and UBSan, on CPU.

The host half of the library (graphee_gb300/csrc/gx_graph.cpp: graph
construction, partitioning and the reference's file formats) and the oracle
(oracle/gx_oracle.cpp) are plain C++/OpenMP.  They are compiled here with
-fsanitize=address,undefined into a scratch directory and driven through
their C ABI by tests/sanitized_host_run.py in a child process, which loads
the sanitizer runtime first.  Out-of-bounds accesses, use-after-free and
undefined behaviour (overflow, misaligned or null accesses, bad shifts) end
that process with a report; the malformed-file paths are part of the run.
Device code is not covered: a GPU sanitizer is not used on this hardware."""
import os
import shutil
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
FLAGS = ["-std=c++17", "-O1", "-g", "-fsanitize=address,undefined", "-fno-sanitize-recover=undefined",
         "-fno-omit-frame-pointer", "-fopenmp", "-shared", "-fPIC"]


def _asan_runtime():
    cxx = shutil.which("g++")
    if not cxx:
        return None
    p = subprocess.run([cxx, "-print-file-name=libasan.so"], capture_output=True, text=True).stdout.strip()
    return p if os.path.isabs(p) and os.path.exists(p) else None


def test_host_code_under_address_and_ub_sanitizers(tmp_path):
    asan = _asan_runtime()
    if asan is None:
        pytest.skip("g++ with the AddressSanitizer runtime is not available")
    host = tmp_path / "libgx_host_san.so"
    orc = tmp_path / "libgxoracle_san.so"
    subprocess.run(["g++", *FLAGS, f"-I{ROOT / 'include'}", str(ROOT / "graphee_gb300" / "csrc" / "gx_graph.cpp"),
                    "-o", str(host)], check=True)
    subprocess.run(["g++", *FLAGS, "-ffp-contract=off", str(ROOT / "oracle" / "gx_oracle.cpp"), "-o", str(orc)],
                   check=True)
    env = dict(os.environ, LD_PRELOAD=asan, OMP_NUM_THREADS="4",
               ASAN_OPTIONS="detect_leaks=0:halt_on_error=1:exitcode=23",
               UBSAN_OPTIONS="halt_on_error=1:print_stacktrace=1")
    r = subprocess.run([sys.executable, str(ROOT / "tests" / "sanitized_host_run.py"), str(host), str(orc),
                        str(tmp_path)], env=env, capture_output=True, text=True, timeout=900)
    report = (r.stdout + r.stderr)[-6000:]
    assert r.returncode == 0, report
    assert "AddressSanitizer" not in r.stderr and "runtime error" not in r.stderr, report
    assert "sanitized host run ok" in r.stdout
