"""Host-side logic of bench.py that decides what the CPU baseline and the
reference arm render: the seeded block subset and the reference arm's
per-step sample size (every host core busy, K steps within minutes)."""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402


def test_block_subset_is_seeded_uniform_and_sorted():
    a = bench.cpu_block_subset(2040)
    b = bench.cpu_block_subset(2040)
    np.testing.assert_array_equal(a, b)
    assert len(a) == bench.CPU_BLOCKS == 64
    assert len(np.unique(a)) == 64 and (np.diff(a) > 0).all()
    assert a.min() >= 0 and a.max() < 2040
    # drawn over the whole frame, not the spiral's first (central) blocks
    assert a.max() > 1500 and a.min() < 500


def test_reference_step_keeps_every_core_busy():
    for cores in (1, 8, 16, 72):
        for steps in (1, 2, 5, 8, 10, 20, 100):
            k = bench.ref_blocks_per_step(cores, steps)
            assert 1 <= k <= bench.CPU_BLOCKS
            assert k >= min(cores, bench.CPU_BLOCKS)
    # 16 cores: 64 blocks per step for short runs, one block per core for long ones
    assert bench.ref_blocks_per_step(16, 1) == 64
    assert bench.ref_blocks_per_step(16, 5) == 48
    assert bench.ref_blocks_per_step(16, 20) == 16
    # about 8 s of one core per block: K steps on 16 cores stay within a few
    # minutes (48 blocks x 5 steps: about 2 minutes; 16 x 20: under 3)
    for steps in (5, 8, 10, 20):
        assert steps * bench.ref_blocks_per_step(16, steps) * 8.0 / 16 < 200
