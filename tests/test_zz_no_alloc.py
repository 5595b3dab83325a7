"""dl_li_static -- the entry point for callers that may not allocate device
memory while they render (an engine that owns all device memory after
start-up, a loop with a fixed memory budget).  It must give the same
per-path radiance as dl_li, call after call, although its path state lives
in a fixed array inside the library and is reused by every call, and it
must not allocate device memory.

This file sorts last so that a failure here leaves every other test run.
"""
import ctypes as C

import numpy as np
import pytest

from drawlab_gb300 import abi, api, scenes

pytestmark = pytest.mark.gpu


def _static(ctx, gs, opts, n, d_xys, d_L, d_pos):
    return ctx.lib.dl_li_static(gs.h, C.byref(opts), n, C.c_void_p(d_xys.data_ptr()),
                                C.c_void_p(d_L.data_ptr()), C.c_void_p(d_pos.data_ptr()))


def test_static_li_matches_dl_li_twice():
    torch = pytest.importorskip("torch")
    # a fresh context whose first render call is dl_li_static: none of the
    # context's own render buffers exist yet
    ctx = api.Context(0)
    sc = scenes.reference_spheres(width=48, height=32)
    gs = api.Scene.from_data(ctx, sc)
    opts = abi.make_opts(seed=21, max_depth=10, flags=abi.DL_RENDER_FIX_POINT_LIGHT)
    xys = np.array([(x, y, s) for y in range(32) for x in range(48) for s in range(12)], np.int32)
    n = xys.shape[0]                     # 18432 paths: more than the 16384-slot pool

    # the caller owns inputs and outputs (device memory it allocated itself)
    d_xys = torch.from_numpy(xys).cuda()
    d_L = torch.empty((n, 3), dtype=torch.float32, device="cuda")
    d_pos = torch.empty((n, 2), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    results = []
    free_after = []
    for call in range(2):
        d_L.fill_(float("nan"))
        d_pos.fill_(float("nan"))
        torch.cuda.synchronize()
        rc = _static(ctx, gs, opts, n, d_xys, d_L, d_pos)
        assert rc == abi.DL_OK, ctx.lib.dl_last_error(ctx.h)
        torch.cuda.synchronize()
        free_after.append(torch.cuda.mem_get_info()[0])
        results.append((d_L.cpu().numpy(), d_pos.cpu().numpy()))
    # the second call (after the first has loaded its kernels) leaves the
    # device's free memory exactly as it was
    assert free_after[1] == free_after[0], free_after

    L_ref, pos_ref = gs.li(opts, xys)
    for call, (L, pos) in enumerate(results):
        np.testing.assert_array_equal(pos, pos_ref, err_msg="call %d" % call)
        np.testing.assert_allclose(L, L_ref, rtol=1e-5, atol=1e-7, err_msg="call %d" % call)

    # a path pool larger than the fixed array is refused, with a message
    big = abi.make_opts(seed=21, max_paths_in_flight=16385)
    rc = _static(ctx, gs, big, n, d_xys, d_L, d_pos)
    assert rc == abi.DL_ERR_INVALID_ARG
    assert b"16384" in ctx.lib.dl_last_error(ctx.h)
    gs.close()
    ctx.close()
