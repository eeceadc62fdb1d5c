// Byte grid <-> bit-plane conversion of 64-cell chunks with byte-parallel
// (SWAR) arithmetic, shared by the byte step kernel and the conversion
// kernels.  A plane word is {A even, A odd, B even, B odd}: bit m of an even
// word is cell 2m of the chunk, of an odd word cell 2m + 1.  A value 0..3 is
// its own 2-bit code (A = bit 1, B = bit 0); any value >= 4 is static and
// solid, code (0,1).
#pragma once

#include <stdint.h>

namespace fs3d {

// bits 0, 8, 16, 24 -> bits 0..3
__device__ __forceinline__ uint32_t gather_lo4(uint32_t m) { return (m * 0x10204080u) >> 28; }
// bits 0..3 -> bit 0 of bytes 0..3
__device__ __forceinline__ uint32_t spread4(uint32_t n) { return (n * 0x00204081u) & 0x01010101u; }

// Four cells (one byte each) -> nibbles of A (sand or water) and B (water or solid).
__device__ __forceinline__ void classify4(uint32_t v, uint32_t& a4, uint32_t& b4) {
    const uint32_t big = v & 0xFCFCFCFCu;
    if (big) {
        const uint32_t nz = ((big & 0x7F7F7F7Fu) + 0x7F7F7F7Fu) | big;  // bit 7 set iff byte >= 4
        const uint32_t m = ((nz & 0x80808080u) >> 7) * 0xFFu;
        v = (v & ~m) | (0x01010101u & m);
    }
    a4 = gather_lo4((v >> 1) & 0x01010101u);
    b4 = gather_lo4(v & 0x01010101u);
}

// 64 cells (16 little-endian words, cell 4k + i in byte i of word k) -> plane word
__device__ __forceinline__ uint4 bytes_to_planes64(const uint32_t (&w)[16]) {
    uint32_t ae = 0, ao = 0, be = 0, bo = 0;
#pragma unroll
    for (int p = 0; p < 8; ++p) {
        uint32_t a, b;
        classify4(__byte_perm(w[2 * p], w[2 * p + 1], 0x6420), a, b);  // x = 8p, 8p+2, 8p+4, 8p+6
        ae |= a << (4 * p);
        be |= b << (4 * p);
        classify4(__byte_perm(w[2 * p], w[2 * p + 1], 0x7531), a, b);  // x = 8p+1, +3, +5, +7
        ao |= a << (4 * p);
        bo |= b << (4 * p);
    }
    return make_uint4(ae, ao, be, bo);
}

// plane word -> the codes of its 64 cells as 16 little-endian words
__device__ __forceinline__ void planes_to_words64(const uint4& q, uint32_t (&w)[16]) {
#pragma unroll
    for (int p = 0; p < 8; ++p) {
        const uint32_t ve = (spread4((q.x >> (4 * p)) & 0xFu) << 1) | spread4((q.z >> (4 * p)) & 0xFu);
        const uint32_t vo = (spread4((q.y >> (4 * p)) & 0xFu) << 1) | spread4((q.w >> (4 * p)) & 0xFu);
        w[2 * p] = __byte_perm(ve, vo, 0x5140);      // x = 8p, 8p+1, 8p+2, 8p+3
        w[2 * p + 1] = __byte_perm(ve, vo, 0x7362);  // x = 8p+4 .. 8p+7
    }
}

// Loads n (1..64) bytes from p into 16 words; cells past n read as solid (1).
// Sets *big when a loaded byte is a static material (>= 4).
__device__ __forceinline__ void load_chunk64(const uint8_t* p, int n, uint32_t (&w)[16], bool& big) {
    uint32_t any = 0;
    if (n == 64 && (reinterpret_cast<uintptr_t>(p) & 15u) == 0) {
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const uint4 v = reinterpret_cast<const uint4*>(p)[u];
            w[4 * u] = v.x;
            w[4 * u + 1] = v.y;
            w[4 * u + 2] = v.z;
            w[4 * u + 3] = v.w;
            any |= v.x | v.y | v.z | v.w;
        }
    } else if ((reinterpret_cast<uintptr_t>(p) & 3u) == 0) {
#pragma unroll
        for (int k = 0; k < 16; ++k) {
            uint32_t v;
            if (4 * k + 4 <= n) {
                v = reinterpret_cast<const uint32_t*>(p)[k];
            } else {
                v = 0x01010101u;
                for (int i = 0; i < 4; ++i)
                    if (4 * k + i < n) v = (v & ~(0xFFu << (8 * i))) | ((uint32_t)p[4 * k + i] << (8 * i));
            }
            w[k] = v;
            any |= v;
        }
    } else {
#pragma unroll
        for (int k = 0; k < 16; ++k) {
            uint32_t v = 0x01010101u;
            for (int i = 0; i < 4; ++i)
                if (4 * k + i < n) v = (v & ~(0xFFu << (8 * i))) | ((uint32_t)p[4 * k + i] << (8 * i));
            w[k] = v;
            any |= v;
        }
    }
    big = (any & 0xFCFCFCFCu) != 0;
}

// Stores the first n (1..64) cells of 16 words to p.
__device__ __forceinline__ void store_chunk64(uint8_t* p, int n, const uint32_t (&w)[16]) {
    if (n == 64 && (reinterpret_cast<uintptr_t>(p) & 15u) == 0) {
#pragma unroll
        for (int u = 0; u < 4; ++u)
            reinterpret_cast<uint4*>(p)[u] = make_uint4(w[4 * u], w[4 * u + 1], w[4 * u + 2], w[4 * u + 3]);
    } else if ((reinterpret_cast<uintptr_t>(p) & 3u) == 0) {
#pragma unroll
        for (int k = 0; k < 16; ++k) {
            if (4 * k + 4 <= n)
                reinterpret_cast<uint32_t*>(p)[k] = w[k];
            else
                for (int i = 0; i < 4; ++i)
                    if (4 * k + i < n) p[4 * k + i] = (uint8_t)(w[k] >> (8 * i));
        }
    } else {
        for (int x = 0; x < n; ++x) p[x] = (uint8_t)(w[x >> 2] >> (8 * (x & 3)));
    }
}

// Replaces the code of every solid cell of the chunk by its static byte
// (statics_row: the world's static bytes at the chunk's first cell).
__device__ __forceinline__ void patch_statics64(const uint4& q, const uint8_t* statics_row, int n, uint32_t (&w)[16]) {
    uint32_t se = ~q.x & q.z, so = ~q.y & q.w;  // solid cells, even and odd
    while (se) {
        const int m = __ffs(se) - 1;
        se &= se - 1;
        const int x = 2 * m;
        if (x < n) w[x >> 2] = (w[x >> 2] & ~(0xFFu << (8 * (x & 3)))) | ((uint32_t)statics_row[x] << (8 * (x & 3)));
    }
    while (so) {
        const int m = __ffs(so) - 1;
        so &= so - 1;
        const int x = 2 * m + 1;
        if (x < n) w[x >> 2] = (w[x >> 2] & ~(0xFFu << (8 * (x & 3)))) | ((uint32_t)statics_row[x] << (8 * (x & 3)));
    }
}

}  // namespace fs3d
