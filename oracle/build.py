"""Build recipe for the oracle (test infrastructure, never shipped).

* ``build_oracle()`` compiles the CPU restatement ``oracle/oracle.cpp`` into
  ``oracle/_build/liboracle.so`` (g++, no dependencies).  It builds on any
  host, x86_64 or Arm.
* ``build_ref()`` compiles the reference's own CPU hot-path sources from where
  they lie (``$DRAWLAB_REFERENCE``, else a ``reference`` directory beside the
  repository) against the stand-in headers in ``oracle/ref_shim`` and links
  them with ``oracle/ref_driver.cpp`` and ``oracle/ref_host_setup.cpp`` into
  ``oracle/_ref/libdlref.so``.  It also compiles the reference's OptiX-only
  math (GGX material, envmap emitter, miss shader, OpenCV camera, hit data)
  as host code through ``oracle/ref_optix.cpp`` against
  ``oracle/ref_shim_optix`` into ``oracle/_ref/libdlref_optix.so``.  When the
  reference tree is absent it does nothing and returns None.

Both use ``-O3 -ffp-contract=off`` so that no fused multiply-add changes the
float results between x86 and Arm hosts.

Run as a script: ``python oracle/build.py`` builds both.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
REPO = HERE.parent
BUILD_DIR = HERE / "_build"
REF_DIR = HERE / "_ref"

# The reference's CPU hot path (relative to the reference root).
REF_SOURCES = [
    "src/core/base/common.cpp",
    "src/core/base/string.cpp",
    "src/core/bitmap/block.cpp",
    "src/core/math/math.cpp",
    "src/core/math/matrix.cpp",
    "src/core/math/wrap.cpp",
    "src/core/parser/object.cpp",
    "src/core/parser/proplist.cpp",
    "src/tracer/accel/octree.cpp",
    "src/tracer/bsdf/aniso_ggx.cpp",
    "src/tracer/bsdf/dielectric.cpp",
    "src/tracer/bsdf/diffuse.cpp",
    "src/tracer/bsdf/microfacet.cpp",
    "src/tracer/bsdf/mirror.cpp",
    "src/tracer/camera/opencv.cpp",
    "src/tracer/camera/perspective.cpp",
    "src/tracer/camera/virtual.cpp",
    "src/tracer/emitter/area.cpp",
    "src/tracer/emitter/point.cpp",
    "src/tracer/integrator/normal.cpp",
    "src/tracer/integrator/path.cpp",
    "src/tracer/mesh/mesh.cpp",
    "src/tracer/mesh/rectangle.cpp",
    "src/tracer/rfilter/rfilter.cpp",
    "src/tracer/sampler/independent.cpp",
    "src/tracer/scene/scene.cpp",
    "src/tracer/texture/texture.cpp",
]

CXX = os.environ.get("CXX", "g++")
COMMON_FLAGS = ["-std=c++17", "-O3", "-ffp-contract=off", "-fPIC", "-pthread"]


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.exists() and d.stat().st_mtime > t for d in deps)


def build_oracle(force: bool = False) -> Path:
    """Compile the CPU restatement; returns the path of liboracle.so."""
    BUILD_DIR.mkdir(exist_ok=True)
    out = BUILD_DIR / "liboracle.so"
    src = HERE / "oracle.cpp"
    deps = [src, HERE / "oracle.h", REPO / "include" / "drawlab.h"]
    if force or _stale(out, deps):
        tmp = out.with_suffix(".so.tmp%d" % os.getpid())
        _run([CXX, *COMMON_FLAGS, "-shared", "-I", str(REPO / "include"), str(src), "-o", str(tmp)])
        os.replace(tmp, out)
    return out


def reference_root() -> Path | None:
    root = Path(os.environ.get("DRAWLAB_REFERENCE", str(REPO.parent / "reference")))
    return root if (root / "src" / "tracer" / "integrator" / "path.cpp").exists() else None


def build_ref(force: bool = False) -> Path | None:
    """Compile the reference CPU path + harness; None if the reference is absent."""
    root = reference_root()
    if root is None:
        return None
    obj_dir = REF_DIR / "obj"
    obj_dir.mkdir(parents=True, exist_ok=True)
    out = REF_DIR / "libdlref.so"
    shim = HERE / "ref_shim"
    inc = ["-I", str(shim), "-I", str(root / "include"), "-I", "/usr/local/cuda/include"]
    flags = COMMON_FLAGS + ["-w"]
    shim_files = [p for p in shim.rglob("*.h")]
    jobs = []
    objs = []
    for rel in REF_SOURCES:
        src = root / rel
        obj = obj_dir / (rel.replace("/", "_") + ".o")
        objs.append(obj)
        if force or _stale(obj, [src, *shim_files]):
            jobs.append([CXX, *flags, *inc, "-c", str(src), "-o", str(obj)])
    own = [(HERE / "ref_driver.cpp", obj_dir / "ref_driver.o", []),
           (shim / "link_stubs.cpp", obj_dir / "link_stubs.o", []),
           (HERE / "ref_host_setup.cpp", obj_dir / "ref_host_setup.o", [root / "src/tracer/emitter/envmap.cpp"])]
    for src, obj, extra_deps in own:
        objs.append(obj)
        if force or _stale(obj, [src, REPO / "include" / "drawlab.h", *shim_files, *extra_deps]):
            jobs.append([CXX, *flags, *inc, "-I", str(root), "-c", str(src), "-o", str(obj)])
    # The OptiX-only code: compiled as host C++ with __CUDACC__ defined (its
    # host/device members compiled, the CUDA qualifiers ignored attributes),
    # in a library of its own so its inline helpers never meet the CPU
    # build's differently configured copies.
    optix_shim = HERE / "ref_shim_optix"
    optix_obj = obj_dir / "ref_optix.o"
    optix_out = REF_DIR / "libdlref_optix.so"
    optix_src = HERE / "ref_optix.cpp"
    optix_deps = [optix_src, *optix_shim.glob("*.h"), *(root / "src/optix/cuda").rglob("*"),
                  *(root / "include/optix").rglob("*.h")]
    optix_job = None
    if force or _stale(optix_obj, optix_deps):
        optix_job = [CXX, *flags, "-D__CUDACC__", "-I", str(optix_shim), "-I", str(root / "include"),
                     "-I", str(root / "src/optix/cuda"), "-I", "/usr/local/cuda/include",
                     "-c", str(optix_src), "-o", str(optix_obj)]
        jobs.append(optix_job)
    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        list(ex.map(_run, jobs))
    if force or jobs or not out.exists():
        tmp = out.with_suffix(".so.tmp%d" % os.getpid())
        _run([CXX, *COMMON_FLAGS, "-shared", *map(str, objs), "-o", str(tmp)])
        os.replace(tmp, out)
    if force or optix_job or not optix_out.exists():
        tmp = optix_out.with_suffix(".so.tmp%d" % os.getpid())
        _run([CXX, *COMMON_FLAGS, "-shared", str(optix_obj), "-o", str(tmp)])
        os.replace(tmp, optix_out)
    return out


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv))
