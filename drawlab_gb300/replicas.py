"""Replica rendering over processes, one per GPU.

Pixel samples are independent, so the path shards without any exchange
during rendering: rank r renders its own contiguous range of samples per
pixel (dl_render_opts.spp_offset / spp) into its own film, and a single sum
of the films -- RGB and filter weight, one all-reduce -- yields the film of
the whole range.  The reference merges per-thread image blocks into one
film under a mutex (ImageBlock::put(ImageBlock&), src/core/bitmap/
block.cpp:115-129); this is the same merge, across processes.

The renderer is passed in (`render_film(opts) -> film array`), so the same
code drives Scene.render_film on GPUs (NCCL) and any film producer in
multi-process CPU tests (gloo).
"""
from __future__ import annotations

import copy

import numpy as np

from . import abi


def split_spp(spp: int, world_size: int, rank: int) -> tuple[int, int]:
    """(first sample, count) of `rank`: contiguous, balanced to within one."""
    if spp < 0 or world_size <= 0 or not 0 <= rank < world_size:
        raise ValueError("bad split arguments")
    base, extra = divmod(spp, world_size)
    count = base + (1 if rank < extra else 0)
    first = rank * base + min(rank, extra)
    return first, count


def film_shape(width: int, height: int, filter: int) -> tuple[int, int, int]:
    b = 0 if filter == abi.DL_FILTER_BOX else 2
    return height + 2 * b, width + 2 * b, 4


def resolve(film: np.ndarray, filter: int) -> np.ndarray:
    """Film (RGB + weight, with the filter border) -> normalised RGB image
    (ImageBlock::toBitmap, src/core/bitmap/block.cpp:58-66)."""
    b = 0 if filter == abi.DL_FILTER_BOX else 2
    h, w = film.shape[0] - 2 * b, film.shape[1] - 2 * b
    inner = film[b:b + h, b:b + w]
    wgt = inner[..., 3:4]
    return np.where(wgt != 0, inner[..., :3] / np.where(wgt != 0, wgt, 1), 0).astype(np.float32)


def render_replicated(render_film, opts: abi.dl_render_opts, width: int, height: int, group=None,
                      device=None) -> np.ndarray:
    """Render `opts.spp` samples per pixel split over the ranks of `group`
    and return the summed film on every rank.  `device` is where the
    all-reduce runs (a CUDA device for NCCL, None for CPU/gloo)."""
    import torch
    import torch.distributed as dist

    ws = dist.get_world_size(group)
    rank = dist.get_rank(group)
    first, count = split_spp(opts.spp, ws, rank)
    if count > 0:
        local = copy.copy(opts)
        local.spp = count
        local.spp_offset = opts.spp_offset + first
        film = np.ascontiguousarray(render_film(local), dtype=np.float32)
    else:
        film = np.zeros(film_shape(width, height, opts.filter), np.float32)
    t = torch.from_numpy(film)
    if device is not None:
        t = t.to(device)
    dist.all_reduce(t, group=group)
    return t.cpu().numpy()
