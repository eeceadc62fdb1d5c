// Device-side FS3D-rule v1: the scalar per-block rule (bytes) and the
// bit-sliced rule that runs 32 blocks per 32-bit word (bit planes).
#pragma once

#include <stdint.h>

#include "fs3d_common.h"

namespace fs3d {

__device__ __forceinline__ uint32_t draw_dev(uint32_t n, uint32_t rk, uint32_t i, uint32_t s) {
    if (n < 2u) return 0u;
    const uint32_t g = i >> 5, b = i & 31u;
    if (n == 2u) return (plane(rk, g, s, 0u) >> b) & 1u;
    uint32_t u = 0;
#pragma unroll
    for (uint32_t w = 0; w < 8u; ++w) u |= ((plane(rk, g, s, w) >> b) & 1u) << w;
    return u < 85u ? 0u : (u < 170u ? 1u : 2u);
}

__device__ __forceinline__ uint32_t has_zero_byte(uint32_t v) {
    return (v - 0x01010101u) & ~v & 0x80808080u;
}

// Can the block (top layer T, bottom layer B; byte q = column q, cells outside
// the grid hold 1) change?  Exact, by the stability property of the rule.
__device__ __forceinline__ bool block_can_move(uint32_t T, uint32_t B) {
    const uint32_t eT = has_zero_byte(T), eB = has_zero_byte(B);
    const uint32_t pT = has_zero_byte((T & 0xFEFEFEFEu) ^ 0x02020202u);
    const uint32_t wT = has_zero_byte(T ^ 0x03030303u), wB = has_zero_byte(B ^ 0x03030303u);
    return (pT && eB) || (wT && eT) || (wB && eB);
}

__device__ __forceinline__ uint32_t get_byte(uint64_t V, int s) { return (uint32_t)(V >> (8 * s)) & 0xFFu; }

// Runs the rule on one block held as 8 bytes (byte s = slot s; slots 0-3 top
// layer, 4-7 bottom layer, column q = dz*2+dx).  Returns the new bytes.
__device__ __forceinline__ uint64_t block_rule(uint64_t V, uint32_t rk, uint32_t i) {
    uint32_t moved = 0;
#pragma unroll
    for (int s = 0; s < 8; ++s) {
        const uint32_t m = get_byte(V, s);
        if ((m != 2u && m != 3u) || ((moved >> s) & 1u)) continue;
        const int q = s & 3;
        int dst = -1;
        if (s < 4) {
            if (get_byte(V, 4 + q) == 0u) {
                dst = 4 + q;
            } else {
                uint32_t cand = 0;
#pragma unroll
                for (int q2 = 0; q2 < 4; ++q2)
                    if (q2 != q && get_byte(V, 4 + q2) == 0u) cand |= 1u << (4 + q2);
                if (cand) {
                    uint32_t r = draw_dev(__popc(cand), rk, i, (uint32_t)s);
                    while (r--) cand &= cand - 1u;
                    dst = __ffs(cand) - 1;
                }
            }
        }
        if (dst < 0 && m == 3u) {
            const int base = s & 4;
            uint32_t cand = 0;
#pragma unroll
            for (int q2 = 0; q2 < 4; ++q2)
                if (q2 != q && get_byte(V, base + q2) == 0u) cand |= 1u << (base + q2);
            if (cand) {
                uint32_t r = draw_dev(__popc(cand), rk, i, (uint32_t)s);
                while (r--) cand &= cand - 1u;
                dst = __ffs(cand) - 1;
            }
        }
        if (dst >= 0) {
            V &= ~(0xFFull << (8 * s));
            V = (V & ~(0xFFull << (8 * dst))) | ((uint64_t)m << (8 * dst));
            moved |= 1u << dst;
        }
    }
    return V;
}


// ---------------------------------------------------------------------------
// Bit-sliced rule.  Each 32-bit word holds one predicate for 32 consecutive
// blocks i = 32g .. 32g+31 of a block row (bit i & 31).  Per slot s the input
// is (A, B): (0,0) empty, (0,1) solid, (1,0) sand, (1,1) water.
// ---------------------------------------------------------------------------

// bit-sliced u < c for the 8-bit numbers u whose bit w is plane p[w]
template <uint32_t C>
__device__ __forceinline__ uint32_t lt_const(const uint32_t (&p)[8]) {
    uint32_t lt = 0, eq = 0xFFFFFFFFu;
#pragma unroll
    for (int w = 7; w >= 0; --w) {
        if ((C >> w) & 1u) {
            lt |= eq & ~p[w];
            eq &= p[w];
        } else {
            eq &= ~p[w];
        }
    }
    return lt;
}

// Chooses among up to three ordered candidate masks c1..c3 for the blocks in
// `mov`; r = draw(n) with n = the number of candidates, from the slot's random
// words P_w = plane(rk, g, s, w) (draw(2) = P_0; draw(3) compares u = sum_w
// P_w << w with 85 and 170).  Outputs destination masks.
__device__ __forceinline__ void bs_select(uint32_t mov, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t rk,
                                          uint32_t g, uint32_t s, uint32_t& d1, uint32_t& d2, uint32_t& d3) {
    const uint32_t two = (c1 & c2) | (c1 & c3) | (c2 & c3);
    const uint32_t three = c1 & c2 & c3;
    uint32_t r1 = 0, r2 = 0;
    if (mov & two) {
        const uint32_t p0 = plane(rk, g, s, 0u);
        r1 = p0 & two & ~three;
        if (mov & three) {
            uint32_t p[8];
            p[0] = p0;
#pragma unroll
            for (uint32_t w = 1; w < 8u; ++w) p[w] = plane(rk, g, s, w);
            const uint32_t lt85 = lt_const<85u>(p), lt170 = lt_const<170u>(p);
            r1 |= three & ~lt85 & lt170;
            r2 = three & ~lt170;
        }
    }
    const uint32_t r0 = ~(r1 | r2);
    d1 = mov & r0 & c1;
    d2 = mov & ((r0 & ~c1 & c2) | (r1 & c1 & c2));
    d3 = mov & ((r0 & ~c1 & ~c2 & c3) | (r1 & c3 & (c1 ^ c2)) | r2);
}

// The three other columns of q, in increasing order.
__host__ __device__ constexpr int other_col(int q, int n) { return n < q ? n : n + 1; }

// The rule's activity mask of 32 blocks (W = water, E = empty per slot): the
// blocks with a particle that has an empty candidate (a top particle over an
// empty bottom cell, or water beside an empty cell of its layer).  A block
// outside the mask does not change, whatever the draws; a block in it does.
__device__ __forceinline__ uint32_t activity_mask(const uint32_t (&A)[8], const uint32_t (&W)[8],
                                                  const uint32_t (&E)[8]) {
    const uint32_t etop = E[0] | E[1] | E[2] | E[3], ebot = E[4] | E[5] | E[6] | E[7];
    return ((A[0] | A[1] | A[2] | A[3]) & ebot) | ((W[0] | W[1] | W[2] | W[3]) & etop) |
           ((W[4] | W[5] | W[6] | W[7]) & ebot);
}

// Runs one step of the rule on 32 blocks.  A[s], B[s] in/out per slot s.
// Returns the mask of blocks that changed.
__device__ __forceinline__ uint32_t bs_rule(uint32_t (&A)[8], uint32_t (&B)[8], uint32_t rk, uint32_t g) {
    // Only the empty and water planes change as slots are visited.  A slot
    // acts exactly on the particles it held at the start (A[s]): a particle
    // only ever moves into an empty cell, so a cell's own particle is still
    // there when its slot comes, and a particle that arrives is never moved
    // again.  The particle plane is rebuilt at the end from E and the solids.
    uint32_t W[8], E[8];
#pragma unroll
    for (int s = 0; s < 8; ++s) {
        W[s] = A[s] & B[s];
        E[s] = ~(A[s] | B[s]);
    }
    const uint32_t active = activity_mask(A, W, E);
    if (!active) return 0u;
#pragma unroll
    for (int s = 0; s < 8; ++s) B[s] = ~A[s] & B[s];  // from here on B holds the solids, which never change
    uint32_t changed = 0;  // a block changes iff one of its particles moves
#pragma unroll
    for (int s = 0; s < 8; ++s) {
        const int q = s & 3, base = s & 4;
        const uint32_t act = A[s] & active;
        if (!act) continue;
        const uint32_t wat = W[s];  // on the acting blocks: the slot's own water, untouched so far
        uint32_t fall = 0, dg1 = 0, dg2 = 0, dg3 = 0, side;
        if (s < 4) {
            const int b = 4 + q;
            fall = act & E[b];
            const uint32_t rest = act & ~E[b];
            const uint32_t c1 = E[4 + other_col(q, 0)], c2 = E[4 + other_col(q, 1)], c3 = E[4 + other_col(q, 2)];
            const uint32_t any = c1 | c2 | c3;
            bs_select(rest & any, c1, c2, c3, rk, g, (uint32_t)s, dg1, dg2, dg3);
            side = rest & ~any & wat;
        } else {
            side = act & wat;
        }
        const uint32_t e1 = E[base + other_col(q, 0)], e2 = E[base + other_col(q, 1)],
                       e3 = E[base + other_col(q, 2)];
        uint32_t sd1 = 0, sd2 = 0, sd3 = 0;
        const uint32_t smov = side & (e1 | e2 | e3);
        if (smov) bs_select(smov, e1, e2, e3, rk, g, (uint32_t)s, sd1, sd2, sd3);
        const uint32_t moved = fall | dg1 | dg2 | dg3 | smov;
        if (!moved) continue;
        changed |= moved;
        W[s] &= ~moved;
        E[s] |= moved;
        auto put = [&](int t, uint32_t m) {
            E[t] &= ~m;
            W[t] |= m & wat;
        };
        if (s < 4) {
            put(4 + q, fall);
            put(4 + other_col(q, 0), dg1);
            put(4 + other_col(q, 1), dg2);
            put(4 + other_col(q, 2), dg3);
        }
        put(base + other_col(q, 0), sd1);
        put(base + other_col(q, 1), sd2);
        put(base + other_col(q, 2), sd3);
    }
#pragma unroll
    for (int s = 0; s < 8; ++s) {
        const uint32_t solid = B[s];
        A[s] = ~E[s] & ~solid;
        B[s] = W[s] | solid;
    }
    return changed;
}


// The half block at the right end of an odd-phase row (x = X-1 present,
// x = X outside) has only its dx=0 column: cells r = layer*2 + dz with bit r
// of P (sand or water), W (water), E (empty).  Every candidate set has at
// most one cell there, so no random draw is ever taken.
__device__ __forceinline__ void half_block_rule(uint32_t& P, uint32_t& W, uint32_t& E) {
    uint32_t M = 0;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const uint32_t bit = 1u << r;
        if (!(P & bit) || (M & bit)) continue;
        int dst = -1;
        if (r < 2) {
            const int below = 2 + r, diag = 3 - r;  // straight down, then the other bottom cell
            if (E & (1u << below))
                dst = below;
            else if (E & (1u << diag))
                dst = diag;
        }
        if (dst < 0 && (W & bit)) {
            const int side = r ^ 1;  // the other cell of the same layer
            if (E & (1u << side)) dst = side;
        }
        if (dst >= 0) {
            const uint32_t d = 1u << dst;
            if (W & bit) W |= d;
            W &= ~bit;
            P = (P & ~bit) | d;
            E = (E | bit) & ~d;
            M |= d;
        }
    }
}

// The bit-sliced slots (A, B per slot) of the 32 blocks of a block row-pair
// that lane gl holds, in the layout rowpair_core describes.  Every lane of the
// warp calls this together (the odd phase takes a bit from the left lane).
__device__ __forceinline__ void rowpair_slots(const uint4 (&q)[4], int o, int gl, int G, uint32_t (&A)[8],
                                              uint32_t (&B)[8]) {
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        const int s0 = (a >> 1) * 4 + (a & 1) * 2;
        if (o == 0) {
            A[s0] = q[a].x;
            B[s0] = q[a].z;
            A[s0 + 1] = q[a].y;
            B[s0 + 1] = q[a].w;
        } else {
            uint32_t ua = 0u, ub = 0xFFFFFFFFu;  // x = -1 lies outside: solid
            if (G > 1) {
                const uint32_t sa = __shfl_up_sync(0xFFFFFFFFu, q[a].y, 1);
                const uint32_t sb = __shfl_up_sync(0xFFFFFFFFu, q[a].w, 1);
                if (gl > 0) {
                    ua = sa;
                    ub = sb;
                }
            }
            A[s0] = (q[a].y << 1) | (ua >> 31);
            B[s0] = (q[a].w << 1) | (ub >> 31);
            A[s0 + 1] = q[a].x;
            B[s0 + 1] = q[a].z;
        }
    }
}

// One step of one block row-pair held as plane words.  The pair's four rows
// (a = layer*2 + dz: top z0, top z1, bottom z0, bottom z1) cover x in
// [64*gl, 64*gl+64): lane gl of a group of G consecutive lanes (G a power of
// two; every lane of the warp must call this together, `has` false for lanes
// without a word).  q[a] = {A even, A odd, B even, B odd}, updated in place;
// rows outside the world are passed as solid.  In the odd phase the dx=0 word
// is the odd word shifted up one bit with bit 31 of the left lane's odd word
// carried in (x = -1 is solid), and the left lane receives its new bit 31
// back; when the row width is a multiple of 64 (`half_at_end`) the last lane
// also runs the half block at x = 64*nw - 1.
__device__ __forceinline__ void rowpair_core(uint4 (&q)[4], bool has, int o, uint32_t rk, int gl, int G, int nw,
                                             bool half_at_end) {
    uint32_t A[8], B[8];
    rowpair_slots(q, o, gl, G, A, B);
    if (has) bs_rule(A, B, rk, (uint32_t)gl);
    if (o == 0) {
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            const int s0 = (a >> 1) * 4 + (a & 1) * 2;
            q[a] = make_uint4(A[s0], A[s0 + 1], B[s0], B[s0 + 1]);
        }
        return;
    }
    // new bit 31 of this lane's odd words: from the right neighbour's dx=0
    // word, from the half block, or unchanged (padding past X)
    uint32_t ta = 0, tb = 0;
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        ta |= (q[a].y >> 31) << a;
        tb |= (q[a].w >> 31) << a;
    }
    if (has && gl == nw - 1 && half_at_end) {
        uint32_t P = ta, W = ta & tb, E = ~(ta | tb) & 0xFu;
        half_block_rule(P, W, E);
        ta = P;
        tb = (W | (~P & ~E)) & 0xFu;
    }
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        const int s0 = (a >> 1) * 4 + (a & 1) * 2;
        uint32_t na = (ta >> a) & 1u, nb = (tb >> a) & 1u;
        if (G > 1) {
            const uint32_t da = __shfl_down_sync(0xFFFFFFFFu, A[s0], 1);
            const uint32_t db = __shfl_down_sync(0xFFFFFFFFu, B[s0], 1);
            if (gl < nw - 1) {
                na = da & 1u;
                nb = db & 1u;
            }
        }
        q[a] = make_uint4(A[s0 + 1], (A[s0] >> 1) | (na << 31), B[s0 + 1], (B[s0] >> 1) | (nb << 31));
    }
}

// Whether lane gl's blocks of a block row-pair (q as for rowpair_core, only
// read) can change in phase o: the rule's activity mask, and for the half
// block at the end of an odd-phase row (`half_at_end`, last lane) a particle
// and an empty cell in it (a superset of its moves).  Every lane of the warp
// calls this together; lanes with `has` false answer false.
__device__ __forceinline__ bool rowpair_can_change(const uint4 (&q)[4], bool has, int o, int gl, int G, int nw,
                                                   bool half_at_end) {
    uint32_t A[8], B[8], W[8], E[8];
    rowpair_slots(q, o, gl, G, A, B);
#pragma unroll
    for (int s = 0; s < 8; ++s) {
        W[s] = A[s] & B[s];
        E[s] = ~(A[s] | B[s]);
    }
    bool can = has && activity_mask(A, W, E) != 0u;
    if (o == 1 && has && half_at_end && gl == nw - 1) {
        uint32_t ta = 0, tb = 0;
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            ta |= (q[a].y >> 31) << a;
            tb |= (q[a].w >> 31) << a;
        }
        if (ta != 0u && (~(ta | tb) & 0xFu) != 0u) can = true;
    }
    return can;
}

}  // namespace fs3d
