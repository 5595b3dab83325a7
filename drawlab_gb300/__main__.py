"""Render a scene in the reference's XML format on the GPU and write the image
next to it, as the reference's renderer does (CPURenderer::renderAsync,
src/tracer/backend/cpu_renderer.cpp:129-134: `scene.xml` -> `scene.exr` and
`scene.png`).

    python -m drawlab_gb300 scene.xml [--spp N] [--seed S] [--device D]

Sample count, filter and integrator come from the file unless overridden.
"""
from __future__ import annotations

import argparse
import os
import sys
import time


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(prog="python -m drawlab_gb300", description=__doc__.split("\n\n")[0])
    ap.add_argument("scene", help="scene file in the reference's XML format")
    ap.add_argument("--spp", type=int, default=None, help="samples per pixel (default: the file's sampler)")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--device", type=int, default=0)
    args = ap.parse_args(argv)

    from . import api

    ctx = api.Context(args.device)
    scene = api.Scene.from_xml(ctx, args.scene)
    opts = scene.default_opts()
    if args.spp is not None:
        opts.spp = args.spp
    opts.seed = args.seed
    t0 = time.perf_counter()
    rgb = scene.render(opts)
    wall = time.perf_counter() - t0
    base = os.path.splitext(args.scene)[0]
    api.write_image(base + ".exr", rgb)
    api.write_image(base + ".png", rgb)
    st = ctx.stats()
    h, w = rgb.shape[:2]
    print("%dx%d, %d spp: %.1f ms on the device (%.1f ms wall) -> %s.exr, %s.png"
          % (w, h, opts.spp, st.render_ms, wall * 1e3, base, base))
    return 0


if __name__ == "__main__":
    sys.exit(main())
