"""Builds libgx.so (CUDA kernels for sm_103a + the C ABI + host graph code)
in-tree, and the oracle's CPU libraries under oracle/.

Everything is compiled with nvcc / g++ directly (no cmake).  Objects go to
graphee_gb300/_build/, the shared library to graphee_gb300/libgx.so.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OBJ = PKG / "_build"
LIB = PKG / "libgx.so"
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
if not Path(NVCC).exists():
    NVCC = shutil.which("nvcc") or NVCC
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
                     "-Xcompiler", "-fPIC,-fopenmp,-O3", "-Xptxas", "-v"] + os.environ.get("GX_NVCC_FLAGS", "").split()
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-fopenmp", "-Wall", "-Wno-unused-function"]


def _sources():
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))


def _headers():
    return sorted(list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list((ROOT / "include").glob("*.h")))


def _compile(src: Path) -> Path:
    obj = OBJ / (src.name + ".o")
    dep_mtime = max([src.stat().st_mtime] + [h.stat().st_mtime for h in _headers()])
    if obj.exists() and obj.stat().st_mtime >= dep_mtime:
        return obj
    if src.suffix == ".cu":
        cmd = [NVCC] + NVCC_FLAGS + ["-I", str(ROOT / "include"), "-c", str(src), "-o", str(obj)]
    else:
        cmd = ["g++"] + CXX_FLAGS + ["-I", str(ROOT / "include"), "-I", "/usr/local/cuda/include",
                                     "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if src.suffix == ".cu":
        (OBJ / (src.name + ".ptxas.txt")).write_text(r.stderr)
    return obj


def build_lib(force: bool = False) -> Path:
    OBJ.mkdir(exist_ok=True)
    if force:
        for o in OBJ.glob("*.o"):
            o.unlink()
    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 2)) as ex:
        objs = list(ex.map(_compile, srcs))
    newest = max(o.stat().st_mtime for o in objs)
    if LIB.exists() and LIB.stat().st_mtime >= newest and not force:
        return LIB
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [NVCC] + ARCH + ["-shared", "-o", str(tmp)] + [str(o) for o in objs] + \
        ["-Xcompiler", "-fopenmp", "-lgomp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


APP = PKG / "gx_app"


def build_apps() -> Path:
    """The C++ app drivers (apps/gx_app.cpp over include/gx_graphps.hpp),
    linked against libgx.so with an rpath to it."""
    src = PKG / "apps" / "gx_app.cpp"
    deps = [src, LIB, ROOT / "include" / "gx_graphps.hpp", ROOT / "include" / "gx.h"]
    if APP.exists() and APP.stat().st_mtime >= max(d.stat().st_mtime for d in deps):
        return APP
    cmd = ["g++", "-O2", "-std=c++17", "-I", str(ROOT / "include"), str(src), "-o", str(APP),
           "-L", str(PKG), "-lgx", "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"app build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return APP


EXAMPLE = PKG / "libgx_program_example.so"


def build_program_example() -> Path:
    """Vertex programs plugged in from outside the library
    (apps/gx_program_example.cu over include/gx_program.cuh), compiled like an
    application would compile its own: nvcc against the headers and libgx.so."""
    src = PKG / "apps" / "gx_program_example.cu"
    deps = [src, LIB, ROOT / "include" / "gx_program.cuh", ROOT / "include" / "gx.h"]
    if EXAMPLE.exists() and EXAMPLE.stat().st_mtime >= max(d.stat().st_mtime for d in deps):
        return EXAMPLE
    cmd = [NVCC] + ARCH + ["-O3", "-std=c++17", "-shared", "-Xcompiler", "-fPIC", "-I", str(ROOT / "include"),
                           str(src), "-o", str(EXAMPLE), "-L", str(PKG), "-lgx", "-Xlinker", "-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"program example build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return EXAMPLE


# Where the build looks for the reference tree (read only, to compile the
# reference's own apps as the oracle's pin); GX_REFERENCE_ROOT overrides it.
REFERENCE_MOUNT = "/root/reference"


def build_oracle() -> None:
    """Compiles the oracle's CPU restatement; and the reference's own apps
    when the reference tree is present on this machine.  Where it is not but
    the working tree carries the recipe's patched copies of the reference
    sources (oracle/_ref/, never committed), the reference's PageRank app is
    compiled from them for this host, as the CPU baseline; a host that cannot
    compile it keeps the oracle's restatement as the baseline."""
    oracle = ROOT / "oracle"
    r = subprocess.run(["make", "-s", "-C", str(oracle), "oracle"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    ref_root = os.environ.get("GX_REFERENCE_ROOT", REFERENCE_MOUNT)
    if Path(ref_root, "GraphMP", "system", "Comp.h").exists():
        r = subprocess.run(["make", "-s", "-C", str(oracle), "ref", f"REF={ref_root}"],
                           capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"reference build failed:\n{r.stdout}\n{r.stderr}")
    elif (oracle / "_ref" / "src_cached" / ".stamp").exists() and not _runs(oracle / "_ref" / "ref_pagerank_cached"):
        subprocess.run(["make", "-s", "-C", str(oracle), "ref-from-copies"], capture_output=True, text=True)


def _runs(binary: Path) -> bool:
    """The binary exists and starts on this host (it prints its usage)."""
    if not binary.exists():
        return False
    try:
        r = subprocess.run([str(binary)], capture_output=True, text=True, timeout=30)
    except OSError:
        return False
    return "usage" in r.stderr


def build(force: bool = False) -> None:
    build_lib(force)
    build_apps()
    build_program_example()
    build_oracle()


if __name__ == "__main__":
    build(force="--force" in sys.argv)
    print(LIB)
