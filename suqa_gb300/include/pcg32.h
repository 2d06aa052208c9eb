// PCG32 (PCG-XSH-RR with 64-bit state, 32-bit output; M. O'Neill, "PCG: A Family
// of Simple Fast Space-Efficient Statistically Good Algorithms for Random Number
// Generation", 2014), with the seeding procedure and the [0,1) double mapping of
// the reference's vendored generator (include/pcg32.h:53-68, :121-130 there):
//   seed(s, seq): state = 0; inc = 2*seq + 1; step; state += s; step
//   next():       old = state; state = old * 6364136223846793005 + inc;
//                 x = ((old >> 18) ^ old) >> 27; rot = old >> 59; rotate-right(x, rot)
//   nextDouble(): 32 random bits placed in the top of the mantissa of a double
//                 in [1, 2), minus 1.
#pragma once
#include <cstdint>
#include <cstring>

struct pcg32 {
    uint64_t state = 0x853c49e6748fea9bULL;
    uint64_t inc = 0xda3e39cb94b95bdbULL;

    pcg32() = default;
    explicit pcg32(uint64_t initstate, uint64_t initseq = 1u) { seed(initstate, initseq); }

    void seed(uint64_t initstate, uint64_t initseq = 1) {
        state = 0U;
        inc = (initseq << 1u) | 1u;
        nextUInt();
        state += initstate;
        nextUInt();
    }

    uint32_t nextUInt() {
        const uint64_t old = state;
        state = old * 6364136223846793005ULL + inc;
        const uint32_t x = (uint32_t)(((old >> 18u) ^ old) >> 27u);
        const uint32_t rot = (uint32_t)(old >> 59u);
        return (x >> rot) | (x << ((0u - rot) & 31u));
    }

    double nextDouble() {
        const uint64_t bits = ((uint64_t)nextUInt() << 20) | 0x3ff0000000000000ULL;
        double d;
        std::memcpy(&d, &bits, sizeof d);
        return d - 1.0;
    }
};
