// Exact per-brick counts of non-empty cells, kept by the plane step kernels
// for a world that renders (bricks of 8x8x8 cells).
#pragma once

#include <stdint.h>

#include "planes.h"

namespace fs3d {

// Non-empty cells of each 8-cell group of a plane word, as bytes: lo byte k
// counts group 2k, hi byte k group 2k + 1 (at most 8 each).
__device__ __forceinline__ void group_counts(const uint4& q, uint32_t& lo, uint32_t& hi) {
    uint32_t e = q.x | q.z, o = q.y | q.w;  // bit m of nibble i: a non-empty cell of group i
    e = e - ((e >> 1) & 0x55555555u);
    e = (e & 0x33333333u) + ((e >> 2) & 0x33333333u);
    o = o - ((o >> 1) & 0x55555555u);
    o = (o & 0x33333333u) + ((o >> 2) & 0x33333333u);
    lo = (e & 0x0F0F0F0Fu) + (o & 0x0F0F0F0Fu);
    hi = ((e >> 4) & 0x0F0F0F0Fu) + ((o >> 4) & 0x0F0F0F0Fu);
}

// Adds one row pair's net change of non-empty cells to the per-brick counts
// (bricks of 8x8x8 cells, index bx + BX*(bz + BZ*by)).  The four rows are
// split by the brick they lie in (they share one unless the pair straddles a
// brick face in y or z); per part the group counts are summed bytewise,
// before and after, and only the groups whose sum moved reach an atomic, so
// cells moving within a brick cost none.  The counts stay exact: a brick is
// empty exactly when its count is 0.
__device__ __forceinline__ void count_bricks(int* __restrict__ counts, const PlaneWorld& w, int y0, int z0, int gl,
                                             const uint4 (&q)[4], const uint4 (&q0)[4], const bool (&in)[4]) {
    const int BX = (w.X + 7) >> 3, BZ = (w.Z + 7) >> 3;
    const bool ysplit = ((y0 + 1) & 7) == 0, zsplit = ((z0 + 1) & 7) == 0;
#pragma unroll
    for (int part = 0; part < 4; ++part) {
        if ((part & 1) && !ysplit) continue;
        if ((part & 2) && !zsplit) continue;
        uint32_t nlo = 0, nhi = 0, olo = 0, ohi = 0;
        bool any = false;
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            // rows a = 0, 1 are layer y0 + 1 (part bit 0 when the pair straddles y),
            // rows a = 1, 3 are z0 + 1 (part bit 1 when it straddles z)
            const int pa = (ysplit && a < 2 ? 1 : 0) | (zsplit && (a & 1) ? 2 : 0);
            if (pa != part || !in[a]) continue;
            uint32_t l, h;
            group_counts(q[a], l, h);
            nlo += l;
            nhi += h;
            group_counts(q0[a], l, h);
            olo += l;
            ohi += h;
            any = true;
        }
        if (!any || (nlo == olo && nhi == ohi)) continue;
        const int y = (part & 1) ? y0 + 1 : (ysplit ? y0 : y0 + 1);
        const int z = (part & 2) ? z0 + 1 : z0;
        const int64_t row = (int64_t)BX * ((z >> 3) + (int64_t)BZ * (y >> 3));
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            const uint32_t nb = (((i & 1) ? nhi : nlo) >> (8 * (i >> 1))) & 0xFFu;
            const uint32_t ob = (((i & 1) ? ohi : olo) >> (8 * (i >> 1))) & 0xFFu;
            const int bx = 8 * gl + i;
            if (nb != ob && bx < BX) atomicAdd(counts + row + bx, (int)nb - (int)ob);
        }
    }
}

}  // namespace fs3d
