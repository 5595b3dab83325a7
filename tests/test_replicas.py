"""Replica rendering over two processes (gloo, CPU): each rank renders its own
sample range, one all-reduce sums the films, and the result equals the film
of the whole range rendered in one process.  The oracle's per-path renderer
stands in for the GPU (same per-path streams, same film)."""
import os
import socket

import numpy as np
import pytest

from drawlab_gb300 import abi, replicas, scenes


def test_split_spp_partitions_the_range():
    for spp in (0, 1, 5, 16, 17, 256):
        for ws in (1, 2, 3, 8):
            parts = [replicas.split_spp(spp, ws, r) for r in range(ws)]
            assert sum(c for _, c in parts) == spp
            nxt = 0
            for first, count in parts:
                assert first == nxt and count >= 0
                nxt += count
            assert max(c for _, c in parts) - min(c for _, c in parts) <= 1
    with pytest.raises(ValueError):
        replicas.split_spp(4, 2, 2)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, spp, out_dir):
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    repo = os.path.dirname(here)
    sys.path[:0] = [repo, os.path.join(repo, "oracle")]
    import torch.distributed as dist
    import pyoracle as po
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sc = scenes.cornell(width=24, height=20)
    orc = po.OracleScene(sc)
    opts = abi.make_opts(spp=spp, max_depth=6, seed=21)
    film = replicas.render_replicated(lambda o: orc.render_paths(o, threads=2, film=True)[1], opts, 24, 20)
    np.save(os.path.join(out_dir, "film%d.npy" % rank), film)
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("spp", [5, 1])
def test_two_replicas_sum_to_the_whole_range(tmp_path, spp):
    import torch.multiprocessing as mp
    import pyoracle as po
    port = _free_port()
    mp.start_processes(_rank_main, args=(2, port, spp, str(tmp_path)), nprocs=2, join=True,
                       start_method="spawn")
    f0, f1 = (np.load(tmp_path / ("film%d.npy" % r)) for r in range(2))
    np.testing.assert_array_equal(f0, f1)
    sc = scenes.cornell(width=24, height=20)
    whole = po.OracleScene(sc).render_paths(abi.make_opts(spp=spp, max_depth=6, seed=21), threads=2,
                                            film=True)[1]
    np.testing.assert_allclose(f0, whole, rtol=1e-5, atol=1e-6)
    rgb = replicas.resolve(f0, abi.DL_FILTER_GAUSSIAN)
    assert rgb.shape == (20, 24, 3) and np.isfinite(rgb).all()
