"""Build libdlgpu.so (the C-ABI library) in-tree: drawlab_gb300/_build/.

CUDA sources are compiled by nvcc for sm_103a only; host C++ by g++ with
-ffp-contract=off (scene tables are computed with the reference's float
operations).  Translation units compile in parallel; nothing is rebuilt when
sources are unchanged.

    python -m drawlab_gb300.build [--force] [--verbose] [--checked]

--checked builds the bounds-checked variant (-DDL_CHECKS: every queue, slot,
path, node and triangle index checked before its access; a violation sets an
error bit and the call fails with a message) into _build/checked/, for tests;
DRAWLAB_GB300_LIBRARY points drawlab_gb300.api at it.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
REPO = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = BUILD / "libdlgpu.so"
CHECKED_BUILD = BUILD / "checked"
CHECKED_LIB = CHECKED_BUILD / "libdlgpu_checked.so"

CUDA_HOME = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
NVCC = str(CUDA_HOME / "bin" / "nvcc") if (CUDA_HOME / "bin" / "nvcc").exists() else "nvcc"
GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = GENCODE + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                        "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr"]
CXX = os.environ.get("CXX", "g++")
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-ffp-contract=off", "-pthread",
             "-I", str(CUDA_HOME / "include")]

CU_SOURCES = ["trace.cu", "render.cu", "noalloc.cu", "guide.cu", "query.cu"]
CPP_SOURCES = ["api.cpp", "bvh.cpp", "image.cpp", "scene.cpp", "xml.cpp"]


def _headers():
    return list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + [REPO / "include" / "drawlab.h"]


def _stale(out: Path, deps) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps if Path(d).exists())


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stdout + r.stderr


def build(force: bool = False, verbose: bool = False, checked: bool = False) -> Path:
    """Compile and link libdlgpu.so (or, checked=True, the bounds-checked
    libdlgpu_checked.so); returns its path."""
    out_dir = CHECKED_BUILD if checked else BUILD
    lib_path = CHECKED_LIB if checked else LIB
    out_dir.mkdir(parents=True, exist_ok=True)
    defs = ["-DDL_CHECKS"] if checked else []
    hdrs = _headers()
    jobs, objs = [], []
    for src in CU_SOURCES:
        s = CSRC / src
        o = out_dir / (src + ".o")
        objs.append(o)
        if force or _stale(o, [s, *hdrs]):
            extra = ["-Xptxas", "-v"] if verbose else []
            jobs.append([NVCC, *NVCC_FLAGS, *defs, *extra, "-c", str(s), "-o", str(o)])
    for src in CPP_SOURCES:
        s = CSRC / src
        o = out_dir / (src + ".o")
        objs.append(o)
        if force or _stale(o, [s, *hdrs]):
            jobs.append([CXX, *CXX_FLAGS, *defs, "-c", str(s), "-o", str(o)])
    logs = []
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            logs = list(ex.map(_run, jobs))
    if force or jobs or not lib_path.exists():
        tmp = lib_path.with_suffix(".so.tmp%d" % os.getpid())
        _run([NVCC, *GENCODE, "-shared", "-o", str(tmp), *map(str, objs), "-cudart", "shared",
              "-Xcompiler", "-pthread"])
        os.replace(tmp, lib_path)
    if verbose:
        for l in logs:
            if l.strip():
                print(l)
    return lib_path


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="--verbose" in sys.argv, checked="--checked" in sys.argv))
