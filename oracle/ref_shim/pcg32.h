// PCG32 restated from M. E. O'Neill, "PCG: A Family of Simple Fast
// Space-Efficient Statistically Good Algorithms for Random Number Generation"
// (2014): 64-bit LCG state, XSH-RR output permutation, stream selected by the
// increment; with the interface of the wjakob/pcg32 header that the reference
// includes from its un-vendored ext/pcg32 submodule (call sites:
// src/tracer/sampler/independent.cpp:3,31-34,42,45,56): default state/stream
// constants, seed(initstate, initseq) as pcg32_srandom_r, nextUInt(), and
// nextFloat() built from the top 23 bits as a float in [1,2) minus 1.
#pragma once
#include <cstdint>
struct pcg32 {
    uint64_t state = 0x853c49e6748fea9bULL;
    uint64_t inc = 0xda3e39cb94b95bdbULL;
    pcg32() {}
    pcg32(uint64_t initstate, uint64_t initseq = 1u) { seed(initstate, initseq); }
    void seed(uint64_t initstate, uint64_t initseq = 1) {
        state = 0u;
        inc = (initseq << 1u) | 1u;
        nextUInt();
        state += initstate;
        nextUInt();
    }
    uint32_t nextUInt() {
        uint64_t old = state;
        state = old * 0x5851f42d4c957f2dULL + inc;
        uint32_t xorshifted = (uint32_t)(((old >> 18u) ^ old) >> 27u);
        uint32_t rot = (uint32_t)(old >> 59u);
        return (xorshifted >> rot) | (xorshifted << ((~rot + 1u) & 31));
    }
    float nextFloat() {
        union { uint32_t u; float f; } x;
        x.u = (nextUInt() >> 9) | 0x3f800000u;
        return x.f - 1.0f;
    }
};
