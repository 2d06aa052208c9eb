// Drop-in replacement of the generator part of the reference's include/Rand.hpp:
// class pcg (include/Rand.hpp:249-291 there) over PCG32.  A seed of 0 means a
// time-based seed, as in the reference.  pcg_state carries inc as well as state,
// so a restored generator continues the same stream (the reference restores
// only state and falls back to the default stream).
#pragma once
#include <chrono>
#include <cstdint>
#include "pcg32.h"

typedef unsigned long long Ullong;

struct pcg_state {
    uint64_t state;
    uint64_t inc = 3u;
};

class pcg {
    pcg32 rng;
    Ullong seed;

  public:
    pcg() : pcg(0ULL) {}

    explicit pcg(Ullong j) {
        if (j == 0) {
            const auto us = std::chrono::duration_cast<std::chrono::microseconds>(
                std::chrono::system_clock::now().time_since_epoch()).count();
            j = (Ullong)us;
        }
        seed = j;
        rng.seed(j);
    }

    explicit pcg(pcg_state st) : seed(0) {
        rng.state = st.state;
        rng.inc = st.inc;
    }

    double doub() { return rng.nextDouble(); }

    int randint(int x0, int x1) { return x0 + (int)(rng.nextUInt() % (uint32_t)(x1 - x0)); }

    pcg_state get_state() {
        pcg_state r;
        r.state = rng.state;
        r.inc = rng.inc;
        return r;
    }

    void set_seed(const Ullong& iseed) {
        seed = iseed;
        rng.seed(iseed);
    }

    inline Ullong get_seed() { return seed; }
};
