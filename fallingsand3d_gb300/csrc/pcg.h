// PCG32 (XSH-RR 64/32, O'Neill 2014) for host and device, plus the
// logarithmic-time LCG jump (Brown 1994, "Random number generation with
// arbitrary strides") so a device thread can start at any draw index.
#pragma once

#include <stdint.h>

#include "fs3d_common.h"

namespace fs3d {

constexpr uint64_t kPcgMult = 6364136223846793005ULL;

FS3D_HD uint32_t pcg_output(uint64_t old) {
    const uint32_t xs = (uint32_t)(((old >> 18) ^ old) >> 27);
    const uint32_t rot = (uint32_t)(old >> 59);
    return (xs >> rot) | (xs << ((0u - rot) & 31u));
}

// state after `delta` further steps of state' = state * kPcgMult + inc
FS3D_HD uint64_t pcg_jump(uint64_t state, uint64_t delta, uint64_t inc) {
    uint64_t acc_mult = 1u, acc_plus = 0u, cur_mult = kPcgMult, cur_plus = inc;
    while (delta > 0) {
        if (delta & 1u) {
            acc_mult *= cur_mult;
            acc_plus = acc_plus * cur_mult + cur_plus;
        }
        cur_plus = (cur_mult + 1u) * cur_plus;
        cur_mult *= cur_mult;
        delta >>= 1u;
    }
    return acc_mult * state + acc_plus;
}

struct Pcg32 {
    uint64_t state = 0, inc = 1;
    FS3D_HD Pcg32(uint64_t initstate, uint64_t initseq) {
        inc = (initseq << 1u) | 1u;
        next();
        state += initstate;
        next();
    }
    FS3D_HD uint32_t next() {
        const uint64_t old = state;
        state = old * kPcgMult + inc;
        return pcg_output(old);
    }
    FS3D_HD uint32_t bounded(uint32_t bound) {
        const uint32_t threshold = (0u - bound) % bound;
        for (;;) {
            const uint32_t v = next();
            if (v >= threshold) return v % bound;
        }
    }
};

// integer thresholds of the synthetic worlds: floor(p * 2^32)
constexpr uint32_t kP05 = 214748364u, kP10 = 429496729u, kP20 = 858993459u, kP25 = 1073741824u,
                   kP30 = 1288490188u, kP35 = 1503238553u, kP40 = 1717986918u;
constexpr uint64_t kBatchWorldStream = 0xC3Du;

// Parameters of one batch world: its fill thresholds and the generator state
// of its first cell draw (cells with y >= Y/2 draw once each, in index order).
struct BatchWorldGen {
    uint32_t sand_thr, water_thr;
    uint64_t fill_state, inc;
};

inline BatchWorldGen batch_world_gen(uint64_t world_seed) {
    Pcg32 r(world_seed, kBatchWorldStream);
    const uint32_t u1 = r.next(), u2 = r.next();
    BatchWorldGen g;
    g.sand_thr = kP05 + (uint32_t)(((uint64_t)u1 * kP35) >> 32);
    g.water_thr = g.sand_thr + (uint32_t)(((uint64_t)u2 * kP20) >> 32);
    g.fill_state = r.state;
    g.inc = r.inc;
    return g;
}

}  // namespace fs3d
