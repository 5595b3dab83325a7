"""PCG32 known answers.  The reference draws every random number from the
wjakob/pcg32 generator of its un-vendored ext/pcg32 submodule
(src/tracer/sampler/independent.cpp:3,31-45); the oracle, the reference
build's stand-in header and the device generator restate it.  The known
answer is the published output of the PCG reference demo for
seed(initstate = 42, initseq = 54): its first six 32-bit outputs.

A small Python model of the same generator (checked against the known
answer here) predicts the device's draws, which reach the host through
dl_li's film positions: a path's first two draws are its pixel sample.
"""
import ctypes as C

import numpy as np
import pytest

import pyoracle as po
from drawlab_gb300 import abi, api, scenes

KAT_42_54 = [0xA15C02B7, 0x7B47F409, 0xBA1D3330, 0x83D2F293, 0xBFA4784B, 0xCBED606E]
M64 = (1 << 64) - 1


class Pcg32:
    """XSH-RR 64 -> 32 with the pcg32_srandom_r seeding."""

    def __init__(self, initstate, initseq):
        self.state = 0
        self.inc = ((initseq << 1) | 1) & M64
        self.u32()
        self.state = (self.state + initstate) & M64
        self.u32()

    def u32(self):
        old = self.state
        self.state = (old * 0x5851F42D4C957F2D + self.inc) & M64
        xs = (((old >> 18) ^ old) >> 27) & 0xFFFFFFFF
        rot = old >> 59
        return ((xs >> rot) | (xs << ((-rot) & 31))) & 0xFFFFFFFF

    def f32(self):
        # top 23 bits as the mantissa of a float in [1, 2), minus 1
        bits = (self.u32() >> 9) | 0x3F800000
        return np.float32(np.frombuffer(np.uint32(bits).tobytes(), np.float32)[0] - np.float32(1.0))


def splitmix64(z):
    z = (z + 0x9E3779B97F4A7C15) & M64
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M64
    return z ^ (z >> 31)


def _lib_outputs(fn, n=6):
    out = np.empty(n, np.uint32)
    fl = np.empty(n, np.float32)
    fn(C.c_uint64(42), C.c_uint64(54), n, out.ctypes.data_as(C.c_void_p), fl.ctypes.data_as(C.c_void_p))
    return out, fl


def test_python_model_known_answer():
    g = Pcg32(42, 54)
    assert [g.u32() for _ in range(6)] == KAT_42_54


def test_oracle_known_answer():
    out, fl = _lib_outputs(po.oracle_lib().orc_pcg32)
    assert out.tolist() == KAT_42_54
    want = np.array([(v >> 9) / float(1 << 23) for v in KAT_42_54], np.float32)
    np.testing.assert_array_equal(fl, want)


def test_reference_build_generator_known_answer():
    lib = po.ref_lib()
    if lib is None:
        pytest.skip("reference sources not present")
    out, _ = _lib_outputs(lib.ref_pcg32)
    assert out.tolist() == KAT_42_54


@pytest.mark.gpu
def test_device_generator_draws_the_pixel_samples():
    # per-path streams: initseq = s*W*H + y*W + x, initstate =
    # splitmix64(initseq ^ splitmix64(seed)); the pixel sample is
    # (x + second draw, y + first draw)
    sc = scenes.cornell(width=40, height=24, spp=4, max_depth=2)
    ctx = api.Context(0)
    gs = api.Scene.from_data(ctx, sc)
    seed = 1234567
    opts = abi.make_opts(seed=seed, max_depth=2)
    rng = np.random.default_rng(5)
    xys = np.stack([rng.integers(0, 40, 300), rng.integers(0, 24, 300), rng.integers(0, 64, 300)], 1)
    xys = xys.astype(np.int32)
    _, pos = gs.li(opts, xys)
    want = np.empty((len(xys), 2), np.float32)
    for i, (x, y, s) in enumerate(xys.tolist()):
        seq = s * 40 * 24 + y * 40 + x
        g = Pcg32(splitmix64(seq ^ splitmix64(seed)), seq)
        first, second = g.f32(), g.f32()
        want[i] = (np.float32(x) + second, np.float32(y) + first)
    np.testing.assert_array_equal(pos, want)
    gs.close()
    ctx.close()
