"""The C-ABI library without a GPU: it builds, loads, exports every entry
point include/drawlab.h declares, and fails cleanly where a device is needed."""
import ctypes as C
import os
import re

import pytest

from drawlab_gb300 import abi, api
from drawlab_gb300 import build as gpu_build

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    names = []
    for fn in os.listdir(os.path.join(REPO, "include")):
        if fn.endswith(".h"):
            src = open(os.path.join(REPO, "include", fn)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names += re.findall(r"^\s*(?:int|const char\*)\s+(dl_\w+)\s*\(", src, flags=re.M)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    gpu_build.build()
    return api.lib()


def test_library_exports_every_header_function(lib):
    names = header_functions()
    assert len(names) >= 19
    for n in names:
        assert hasattr(lib, n), n


def test_binding_covers_every_header_function():
    assert sorted(api.SIGNATURES) == header_functions()


def test_abi_version(lib):
    assert lib.dl_abi_version() == abi.DL_ABI_VERSION


def test_struct_sizes_match_header():
    # sizes of the descriptor structs as laid out by a C compiler (x86-64/aarch64 LP64)
    assert C.sizeof(abi.dl_mesh_desc) == 4 * 8 + 2 * 8 + 2 * 4
    assert C.sizeof(abi.dl_material_desc) == 4 * (1 + 3 + 3 + 2 + 2) + 4 + 5 * 16
    assert C.sizeof(abi.dl_render_opts) == 4 * 4 + 8 + 4 + 4 + 8
    assert C.sizeof(abi.dl_camera_desc) == 4 * (3 + 9 + 1 + 16 + 2 + 4)


STRUCTS = ["dl_mesh_desc", "dl_texture_desc", "dl_material_desc", "dl_light_desc", "dl_camera_desc", "dl_render_opts", "dl_request",
           "dl_tune_params", "dl_guide_config",
           "dl_scene_info", "dl_stats", "dl_traversal_counts"]


def test_struct_layouts_match_a_c_compiler(tmp_path):
    # every field offset and struct size of the ctypes mirrors against gcc
    # compiling the header itself
    import shutil
    import subprocess
    if shutil.which("gcc") is None:
        pytest.skip("no C compiler")
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "drawlab.h"', "int main(void) {"]
    for name in STRUCTS:
        cls = getattr(abi, name)
        lines.append('printf("%s %%zu\\n", sizeof(%s));' % (name, name))
        for f, _ in cls._fields_:
            lines.append('printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (name, f, name, f))
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", inc, str(src), "-o", str(exe)], check=True)
    out = dict(l.split() for l in subprocess.run([str(exe)], check=True, capture_output=True,
                                                 text=True).stdout.splitlines())
    for name in STRUCTS:
        cls = getattr(abi, name)
        assert int(out[name]) == C.sizeof(cls), name
        for f, _ in cls._fields_:
            assert int(out["%s.%s" % (name, f)]) == getattr(cls, f).offset, (name, f)


def test_null_handles_are_rejected(lib):
    assert lib.dl_scene_destroy(None) == abi.DL_ERR_INVALID_ARG
    assert lib.dl_context_destroy(None) == abi.DL_ERR_INVALID_ARG
    assert lib.dl_render(None, None, None) == abi.DL_ERR_INVALID_ARG
    assert lib.dl_stats_get(None, None) == abi.DL_ERR_INVALID_ARG
    h = C.c_void_p()
    assert lib.dl_context_create(0, None) == abi.DL_ERR_INVALID_ARG


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_has_gpu(), reason="a GPU is present")
def test_context_creation_fails_cleanly_without_gpu(lib):
    h = C.c_void_p()
    rc = lib.dl_context_create(0, C.byref(h))
    assert rc == abi.DL_ERR_CUDA
    assert b"CUDA" in lib.dl_last_error(None)
    assert not h.value
