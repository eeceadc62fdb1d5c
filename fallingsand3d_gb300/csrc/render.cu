// Headless render kernels.  Built with --fmad=false: every float expression is
// a sequence of single IEEE operations (+ - * /, sqrtf correctly rounded), in
// the same order as the CPU restatement, so frames are reproducible bit for
// bit on the host.
//
//  * k_render_sdf: shaders/fs_raymarch.frag:10-81 as a CUDA kernel, one thread
//    per pixel: 64-step sphere tracing of a radius-0.5 sphere at the origin,
//    hit at d < 0.001, bail at t > 1000, central-difference normal (h=0.001),
//    diffuse = max(0.05, dot(n, normalize(p - light))) (the shader's vector
//    points away from the light), red surface, black miss, alpha 1.
//    Ray set-up follows fs_raymarch.vert:30-37 (origin = camPos, aspect =
//    aspect.x) and the fullscreen quad of renderer.cpp:1253-1267.
//  * k_render_dda: Amanatides & Woo (1987) traversal of the world grid with
//    the same ray generation and shading conventions; the face normal of the
//    entered voxel is shaded with the material's colour.
#include <math.h>
#include <stdint.h>

#include "fs3d_common.h"
#include "planes.h"

namespace fs3d {

struct CamDev {
    float o[3], f[3], r[3], u[3];
    float tan_half_fov, aspect;
    float light[3];
};

__device__ __forceinline__ float dot3(const float* a, const float* b) {
    return __fadd_rn(__fadd_rn(__fmul_rn(a[0], b[0]), __fmul_rn(a[1], b[1])), __fmul_rn(a[2], b[2]));
}
__device__ __forceinline__ void normalize3(float* v) {
    const float len = __fsqrt_rn(dot3(v, v));
    v[0] = __fdiv_rn(v[0], len);
    v[1] = __fdiv_rn(v[1], len);
    v[2] = __fdiv_rn(v[2], len);
}
__device__ __forceinline__ void pixel_uv2(int px, int py, int W, int H, float& ux, float& uy) {
    const float u = __fsub_rn(1.0f, __fdiv_rn(__fadd_rn((float)px, 0.5f), (float)W));
    const float v = __fdiv_rn(__fadd_rn((float)py, 0.5f), (float)H);
    ux = __fsub_rn(__fmul_rn(u, 2.0f), 1.0f);
    uy = __fsub_rn(__fmul_rn(v, 2.0f), 1.0f);
}
__device__ __forceinline__ float sdf_world(float x, float y, float z) {
    return __fsub_rn(__fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y)), __fmul_rn(z, z))), 0.5f);
}

__global__ void k_render_sdf(CamDev cam, int W, int H, float4* __restrict__ out) {
    const int px = blockIdx.x * blockDim.x + threadIdx.x;
    const int py = blockIdx.y * blockDim.y + threadIdx.y;
    if (px >= W || py >= H) return;
    float ux, uy;
    pixel_uv2(px, py, W, H, ux, uy);
    uy = __fmul_rn(uy, __fdiv_rn(1.0f, cam.aspect));
    float d[3] = {ux, uy, 1.0f};
    normalize3(d);
    float col = 0.0f, t = 0.0f;
    for (int it = 0; it < 64; ++it) {
        const float p[3] = {__fadd_rn(cam.o[0], __fmul_rn(t, d[0])), __fadd_rn(cam.o[1], __fmul_rn(t, d[1])),
                            __fadd_rn(cam.o[2], __fmul_rn(t, d[2]))};
        const float dist = sdf_world(p[0], p[1], p[2]);
        if (dist < 0.001f) {
            const float h = 0.001f;
            float n[3] = {
                __fsub_rn(sdf_world(__fadd_rn(p[0], h), p[1], p[2]), sdf_world(__fsub_rn(p[0], h), p[1], p[2])),
                __fsub_rn(sdf_world(p[0], __fadd_rn(p[1], h), p[2]), sdf_world(p[0], __fsub_rn(p[1], h), p[2])),
                __fsub_rn(sdf_world(p[0], p[1], __fadd_rn(p[2], h)), sdf_world(p[0], p[1], __fsub_rn(p[2], h)))};
            normalize3(n);
            float l[3] = {__fsub_rn(p[0], cam.light[0]), __fsub_rn(p[1], cam.light[1]), __fsub_rn(p[2], cam.light[2])};
            normalize3(l);
            col = fmaxf(0.05f, dot3(n, l));
            break;
        } else if (t > 1000.0f) {
            break;
        }
        t = __fadd_rn(t, dist);
    }
    out[(size_t)py * W + px] = make_float4(col, 0.0f, 0.0f, 1.0f);
}

__constant__ float c_palette[5][3] = {
    {0.0f, 0.0f, 0.0f}, {0.50f, 0.50f, 0.52f}, {0.86f, 0.74f, 0.46f}, {0.20f, 0.42f, 0.90f}, {0.65f, 0.35f, 0.30f}};

// material lookup: canonical bytes
struct BytesGrid {
    const uint8_t* g;
    int X, Y, Z;
    __device__ __forceinline__ uint32_t at(int x, int y, int z) const {
        return g[(int64_t)x + (int64_t)X * ((int64_t)z + (int64_t)Z * y)];
    }
};

// material lookup: bit planes (A,B) + optional static byte overlay for solids
struct PlaneGrid {
    const uint32_t* p;  // rows of nw x {A even, A odd, B even, B odd}
    const uint8_t* statics;  // nullable: every solid is stone
    int X, Y, Z, nw;
    __device__ __forceinline__ uint32_t at(int x, int y, int z) const {
        const uint32_t* row = p + (size_t)4 * nw * ((size_t)y * Z + z);
        const int word = x >> 6, bit = (x >> 1) & 31, odd = x & 1;
        const uint32_t a = (__ldg(row + 4 * word + odd) >> bit) & 1u;
        const uint32_t b = (__ldg(row + 4 * word + 2 + odd) >> bit) & 1u;
        if (a) return b ? 3u : 2u;
        if (!b) return 0u;
        return statics ? statics[(int64_t)x + (int64_t)X * ((int64_t)z + (int64_t)Z * y)] : 1u;
    }
};

// Occupancy of 8x8x8 bricks: bit b set when brick b = bx + BX*(bz + BZ*by)
// holds a non-empty cell.  Built per frame; the traversal skips the material
// loads inside empty bricks but keeps every DDA step, so the visited-cell
// sequence (and the hit) is exactly the flat traversal's.
struct BrickMap {
    const uint32_t* bits;
    int BX, BY, BZ;
    const uint32_t* sbits;  // one bit per 64^3 super-brick (8^3 bricks): set when any of its bricks is
    int SBX, SBY, SBZ;
    __device__ __forceinline__ bool occupied(int x, int y, int z) const {
        const int b = (x >> 3) + BX * ((z >> 3) + BZ * (y >> 3));
        return (__ldg(bits + (b >> 5)) >> (b & 31)) & 1u;
    }
    __device__ __forceinline__ bool super_occupied(int sb) const { return (__ldg(sbits + (sb >> 5)) >> (sb & 31)) & 1u; }
};

__device__ __forceinline__ void mark_brick(uint32_t* bits, int BX, int BZ, int bx, int by, int bz) {
    const int b = bx + BX * (bz + BZ * by);
    const uint32_t bit = 1u << (b & 31);
    if (!(bits[b >> 5] & bit)) atomicOr(bits + (b >> 5), bit);
}

// planes: a thread per 64-cell word; each 8-cell chunk with a non-empty cell marks its brick
__global__ void k_brickmap_planes(const uint4* __restrict__ rows, int X, int Y, int Z, int nw, uint32_t* bits,
                                  int BX, int BZ) {
    const int64_t n = (int64_t)Y * Z * nw;
    for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < n; u += (int64_t)gridDim.x * blockDim.x) {
        const int g = (int)(u % nw);
        const int64_t r = u / nw;
        const int y = (int)(r / Z), z = (int)(r % Z);
        const uint4 q = rows[u];
        const uint32_t nz = q.x | q.y | q.z | q.w;  // bit m: cell 64g+2m or 64g+2m+1 is not empty
        if (!nz) continue;
        // the word's 8 chunks are 8 consecutive bricks along x: one atomic per
        // 32-bit bitmap word they fall in (at most two)
        uint32_t m8 = 0;
#pragma unroll
        for (int c = 0; c < 8; ++c)
            if (((nz >> (4 * c)) & 0xFu) && 64 * g + 8 * c < X) m8 |= 1u << c;
        if (!m8) continue;
        const int b0 = 8 * g + BX * ((z >> 3) + BZ * (y >> 3));
        const int sh = b0 & 31;
        atomicOr(bits + (b0 >> 5), m8 << sh);
        if (sh > 24 && (m8 >> (32 - sh))) atomicOr(bits + (b0 >> 5) + 1, m8 >> (32 - sh));
    }
}

// Counts of non-empty cells per brick, from the planes (one thread per row word)
__global__ void k_brickcount_planes(const uint4* __restrict__ rows, int X, int Y, int Z, int nw, int* counts, int BX,
                                    int BZ) {
    const int64_t n = (int64_t)Y * Z * nw;
    for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < n; u += (int64_t)gridDim.x * blockDim.x) {
        const int g = (int)(u % nw);
        const int64_t r = u / nw;
        const int y = (int)(r / Z), z = (int)(r % Z);
        const uint4 q = rows[u];
        const uint32_t e = q.x | q.z, o = q.y | q.w;
        if (!(e | o)) continue;
        const int64_t base = (int64_t)BX * ((z >> 3) + (int64_t)BZ * (y >> 3));
#pragma unroll
        for (int c = 0; c < 8; ++c) {
            const int cnt = __popc((e >> (4 * c)) & 0xFu) + __popc((o >> (4 * c)) & 0xFu);
            if (cnt && 8 * g + c < BX) atomicAdd(counts + base + 8 * g + c, cnt);
        }
    }
}

// bit b of the brick map = (counts[b] > 0): a warp builds 32 map words,
// one ballot over 32 consecutive counts each
__global__ void k_counts_to_bits(const int* __restrict__ counts, int64_t n, uint32_t* bits) {
    const int lane = threadIdx.x & 31;
    const int64_t nwords = (n + 31) / 32;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t w = (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32; w < nwords; w += nwarps * 32) {
        uint32_t mine = 0;
        for (int k = 0; k < 32; ++k) {
            const int64_t b = (w + k) * 32 + lane;
            const uint32_t m = __ballot_sync(0xFFFFFFFFu, b < n && counts[b] > 0);
            if (lane == k) mine = m;
        }
        if (w + lane < nwords) bits[w + lane] = mine;
    }
}

// bytes: a thread per 8-cell chunk of a row
__global__ void k_brickmap_bytes(const uint8_t* __restrict__ g, int X, int Y, int Z, uint32_t* bits, int BX, int BZ) {
    const int64_t n = (int64_t)Y * Z * BX;
    for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < n; u += (int64_t)gridDim.x * blockDim.x) {
        const int c = (int)(u % BX);
        const int64_t r = u / BX;
        const int y = (int)(r / Z), z = (int)(r % Z);
        const uint8_t* row = g + r * X;
        bool any = false;
        for (int x = 8 * c; x < 8 * c + 8 && x < X; ++x) any |= row[x] != 0;
        if (any) mark_brick(bits, BX, BZ, c, y >> 3, z >> 3);
    }
}

// Crossing an empty region (an 8^3 brick or a 64^3 super-brick) at once, with
// the cell-by-cell walk's exact result.  The walk steps, at every cell, the
// axis whose next boundary key is smallest; on equal keys z goes before y
// before x.  Axis a's key after n steps is fma(n, e_a, b_a), a non-decreasing
// function of n, so the walk's steps are the merge of the three axes' key
// sequences in that order.  It leaves the region at the first of the three
// axes' leaving steps (axis a's key at step n_a + k_a - 1, k_a the cells to
// the region's face); every step that comes before it in the merge is taken
// (for each other axis a prefix of its keys, found from an estimate and
// checked key by key), and nothing in between can hit, since the region is
// empty.  The state after the crossing (cells, steps, keys, last axis, t) is
// therefore bit for bit the walk's.
__device__ __forceinline__ bool key_before(float p, int pa, float q, int pb) {
    return p < q || (p == q && pa > pb);  // axis index as the tie priority: z (2) > y (1) > x (0)
}

// cells axis a takes to leave its region of R cells (or the grid): k, and whether that leaves the grid
__device__ __forceinline__ int cells_to_leave(int v, int s, int n, int R, bool& out) {
    if (s > 0) {
        const int kb = R - (v & (R - 1)), kg = n - v;
        out = kg <= kb;
        return out ? kg : kb;
    }
    const int k = (v & (R - 1)) + 1;
    out = v - k < 0;
    return k;
}

// Takes the steps of one axis (steps n.., at most k - 1 of them: its k-th
// leaves the region) whose keys come before the leaving step's key ke of axis ax.
__device__ __forceinline__ void advance_before(int& v, int s, int& n, float b, float e, float& m, int k, int pa,
                                               float ke, int ax) {
    const int lo = n, hi = n + k - 2;  // candidate steps
    if (hi < lo) return;
    // estimate the last step before ke, then correct it key by key
    const float q = __fdiv_rn(__fsub_rn(ke, b), e);
    int j = q < (float)lo ? lo - 1 : (q > (float)hi ? hi : (int)q);
    while (j < hi && key_before(__fmaf_rn((float)(j + 1), e, b), pa, ke, ax)) ++j;
    while (j >= lo && !key_before(__fmaf_rn((float)j, e, b), pa, ke, ax)) --j;
    v += s * (j + 1 - n);
    n = j + 1;
    m = __fmaf_rn((float)n, e, b);
}

template <class G>
__global__ void __launch_bounds__(256) k_render_dda(G grid, BrickMap bm, CamDev cam, int W, int H,
                                                   float4* __restrict__ out) {
    const int px = blockIdx.x * blockDim.x + threadIdx.x;
    const int py = blockIdx.y * blockDim.y + threadIdx.y;
    if (px >= W || py >= H) return;
    const int NX = grid.X, NY = grid.Y, NZ = grid.Z;
    float ux, uy;
    pixel_uv2(px, py, W, H, ux, uy);
    const float sx = __fmul_rn(__fmul_rn(ux, cam.tan_half_fov), cam.aspect);
    const float sy = __fmul_rn(uy, cam.tan_half_fov);
    float d[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) d[a] = __fadd_rn(__fadd_rn(cam.f[a], __fmul_rn(cam.r[a], sx)), __fmul_rn(cam.u[a], sy));
    normalize3(d);
    float4 res = make_float4(0.0f, 0.0f, 0.0f, 1.0f);
    // slab entry: per axis in the same order as the CPU restatement
    float inv[3];
    float tmin = 0.0f, tmax = INFINITY;
    int entry_axis = -1;
    bool miss = false;
    const int N[3] = {NX, NY, NZ};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        if (d[a] == 0.0f) {
            inv[a] = INFINITY;
            if (cam.o[a] < 0.0f || cam.o[a] >= (float)N[a]) miss = true;
            continue;
        }
        inv[a] = __fdiv_rn(1.0f, d[a]);
        float t0 = __fmul_rn(__fsub_rn(0.0f, cam.o[a]), inv[a]);
        float t1 = __fmul_rn(__fsub_rn((float)N[a], cam.o[a]), inv[a]);
        if (t0 > t1) {
            const float tmp = t0;
            t0 = t1;
            t1 = tmp;
        }
        if (t0 > tmin) {
            tmin = t0;
            entry_axis = a;
        }
        if (t1 < tmax) tmax = t1;
    }
    if (!miss && tmin <= tmax) {
        // per-axis state as scalars (no local-memory arrays): cell v, step s, steps
        // taken n, first boundary t b, t per cell e; the next boundary key is
        // m = fma(n, e, b), one rounding, as in the CPU walk
        int v0, v1, v2, s0, s1, s2, n0 = 0, n1 = 0, n2 = 0;
        float b0, b1, b2, e0, e1, e2;
        auto setup = [&](int a, int& v, int& st, float& bt, float& td) {
            const float p = __fadd_rn(cam.o[a], __fmul_rn(d[a], tmin));
            int c = (int)floorf(p);
            c = c < 0 ? 0 : (c > N[a] - 1 ? N[a] - 1 : c);
            v = c;
            st = d[a] > 0.0f ? 1 : (d[a] < 0.0f ? -1 : 0);
            if (d[a] == 0.0f) {
                bt = INFINITY;
                td = INFINITY;
            } else {
                bt = __fmul_rn(__fsub_rn((float)(c + (st > 0 ? 1 : 0)), cam.o[a]), inv[a]);
                td = fabsf(inv[a]);
            }
        };
        setup(0, v0, s0, b0, e0);
        setup(1, v1, s1, b1, e1);
        setup(2, v2, s2, b2, e2);
        float m0 = b0, m1 = b1, m2 = b2;
        int last = entry_axis;
        float tcur = tmin;
        const int max_iter = NX + NY + NZ + 3;
        int cur_brick = -1, cur_super = -1;
        bool brick_occ = true, super_occ = true;
        for (int it = 0; it < max_iter; ++it) {
            const int sb = (v0 >> 6) + bm.SBX * ((v2 >> 6) + bm.SBZ * (v1 >> 6));
            if (sb != cur_super) {
                cur_super = sb;
                super_occ = bm.super_occupied(sb);
            }
            int R = 0;  // an empty region around the cell: a 64^3 super-brick or an 8^3 brick
            if (!super_occ) {
                R = 64;
            } else {
                const int b = (v0 >> 3) + bm.BX * ((v2 >> 3) + bm.BZ * (v1 >> 3));
                if (b != cur_brick) {
                    cur_brick = b;
                    brick_occ = bm.occupied(v0, v1, v2);
                }
                if (!brick_occ) R = 8;
            }
            if (R) {
                // cross the empty region: take every step up to and including the first
                // that leaves it, with the walk's exact keys (see key_before)
                bool out0 = false, out1 = false, out2 = false;
                const int k0 = s0 ? cells_to_leave(v0, s0, NX, R, out0) : 0;
                const int k1 = s1 ? cells_to_leave(v1, s1, NY, R, out1) : 0;
                const int k2 = s2 ? cells_to_leave(v2, s2, NZ, R, out2) : 0;
                // each axis's key at its leaving step
                const float x0 = s0 ? __fmaf_rn((float)(n0 + k0 - 1), e0, b0) : INFINITY;
                const float x1 = s1 ? __fmaf_rn((float)(n1 + k1 - 1), e1, b1) : INFINITY;
                const float x2 = s2 ? __fmaf_rn((float)(n2 + k2 - 1), e2, b2) : INFINITY;
                int ax = -1;
                float ke = INFINITY;
                if (s0) { ax = 0; ke = x0; }
                if (s1 && (ax < 0 || key_before(x1, 1, ke, ax))) { ax = 1; ke = x1; }
                if (s2 && (ax < 0 || key_before(x2, 2, ke, ax))) { ax = 2; ke = x2; }
                // the other axes take their steps that come before it (a prefix of their keys)
                if (ax != 0 && s0) advance_before(v0, s0, n0, b0, e0, m0, k0, 0, ke, ax);
                if (ax != 1 && s1) advance_before(v1, s1, n1, b1, e1, m1, k1, 1, ke, ax);
                if (ax != 2 && s2) advance_before(v2, s2, n2, b2, e2, m2, k2, 2, ke, ax);
                tcur = ke;
                last = ax;
                if (ax == 0) {
                    if (out0) break;
                    v0 += s0 * k0;
                    n0 += k0;
                    m0 = __fmaf_rn((float)n0, e0, b0);
                } else if (ax == 1) {
                    if (out1) break;
                    v1 += s1 * k1;
                    n1 += k1;
                    m1 = __fmaf_rn((float)n1, e1, b1);
                } else {
                    if (out2) break;
                    v2 += s2 * k2;
                    n2 += k2;
                    m2 = __fmaf_rn((float)n2, e2, b2);
                }
                continue;
            }
            const uint32_t m = grid.at(v0, v1, v2);
            if (m != 0u) {
                float n[3] = {0.0f, 0.0f, 0.0f};
                if (last == 0) n[0] = s0 > 0 ? -1.0f : 1.0f;
                if (last == 1) n[1] = s1 > 0 ? -1.0f : 1.0f;
                if (last == 2) n[2] = s2 > 0 ? -1.0f : 1.0f;
                float l[3];
#pragma unroll
                for (int a = 0; a < 3; ++a)
                    l[a] = __fsub_rn(__fadd_rn(cam.o[a], __fmul_rn(d[a], tcur)), cam.light[a]);
                normalize3(l);
                const float diff = fmaxf(0.05f, dot3(n, l));
                const int ci = m < 4u ? (int)m : 4;
                res = make_float4(__fmul_rn(c_palette[ci][0], diff), __fmul_rn(c_palette[ci][1], diff),
                                  __fmul_rn(c_palette[ci][2], diff), 1.0f);
                break;
            }
            // next cell: the axis whose boundary key comes first (equal keys: z, then y, then x)
            if (m0 < m1 ? m0 < m2 : false) {
                tcur = m0;
                v0 += s0;
                if (v0 < 0 || v0 >= NX) break;
                m0 = __fmaf_rn((float)++n0, e0, b0);
                last = 0;
            } else if (!(m0 < m1) && m1 < m2) {
                tcur = m1;
                v1 += s1;
                if (v1 < 0 || v1 >= NY) break;
                m1 = __fmaf_rn((float)++n1, e1, b1);
                last = 1;
            } else {
                tcur = m2;
                v2 += s2;
                if (v2 < 0 || v2 >= NZ) break;
                m2 = __fmaf_rn((float)++n2, e2, b2);
                last = 2;
            }
        }
    }
    out[(size_t)py * W + px] = res;
}

static CamDev to_dev(const fs3d_camera* c) {
    CamDev d;
    for (int a = 0; a < 3; ++a) {
        d.o[a] = c->origin[a];
        d.f[a] = c->forward[a];
        d.r[a] = c->right[a];
        d.u[a] = c->up[a];
        d.light[a] = c->light_pos[a];
    }
    d.tan_half_fov = c->tan_half_fov;
    d.aspect = c->aspect;
    return d;
}

fs3d_status launch_render_sdf(const fs3d_camera* cam, int W, int H, float* rgba_dev, cudaStream_t st) {
    const dim3 blk(16, 16), grd((W + 15) / 16, (H + 15) / 16);
    k_render_sdf<<<grd, blk, 0, st>>>(to_dev(cam), W, H, reinterpret_cast<float4*>(rgba_dev));
    FS3D_CHECK_LAUNCH("render sdf launch");
    return FS3D_OK;
}

static int map_grid(int64_t n) {
    const int64_t need = (n + 255) / 256, cap = (int64_t)sm_count_public() * 8;
    return (int)(need < 1 ? 1 : (need < cap ? need : cap));
}

// One bit per 64^3 super-brick: set when any of its (up to 8^3) bricks is.
// One warp per super-brick; each lane reads the 8-brick x runs of two of its
// 64 (y, z) brick rows (a run is 8 consecutive bits, in one or two words).
__global__ void k_superbits(const uint32_t* __restrict__ bits, int BX, int BY, int BZ, uint32_t* sbits, int SBX,
                            int SBY, int SBZ) {
    const int64_t n = (int64_t)SBX * SBY * SBZ;
    const int lane = threadIdx.x & 31;
    const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n; i += warps) {
        const int sx = (int)(i % SBX), sz = (int)((i / SBX) % SBZ), sy = (int)(i / ((int64_t)SBX * SBZ));
        const int bx0 = 8 * sx, nx = min(8, BX - bx0);
        bool any = false;
        for (int p = lane; p < 64; p += 32) {
            const int by = 8 * sy + (p >> 3), bz = 8 * sz + (p & 7);
            if (by >= BY || bz >= BZ) continue;
            const int64_t b0 = bx0 + (int64_t)BX * (bz + (int64_t)BZ * by);
            const uint64_t w = (uint64_t)__ldg(bits + (b0 >> 5)) |
                               ((b0 & 31) + nx > 32 ? (uint64_t)__ldg(bits + (b0 >> 5) + 1) << 32 : 0ull);
            any |= ((w >> (b0 & 31)) & ((1ull << nx) - 1ull)) != 0ull;
        }
        if (__any_sync(0xFFFFFFFFu, any) && lane == 0) atomicOr(sbits + (i >> 5), 1u << (i & 31));
    }
}

static int64_t brick_words(int X, int Y, int Z) {
    return (((int64_t)(X + 7) / 8) * ((Y + 7) / 8) * ((Z + 7) / 8) + 31) / 32;
}

// The brick map of a frame: the bricks' bits (filled by the caller's map
// kernel), then the super-bricks' bits after them, derived here.
static fs3d_status superbits_and_map(uint32_t* bm_bits, int X, int Y, int Z, cudaStream_t st, BrickMap* bm) {
    const int BX = (X + 7) / 8, BY = (Y + 7) / 8, BZ = (Z + 7) / 8;
    const int SBX = (X + 63) / 64, SBY = (Y + 63) / 64, SBZ = (Z + 63) / 64;
    uint32_t* sbits = bm_bits + brick_words(X, Y, Z);
    const int64_t ns = (int64_t)SBX * SBY * SBZ;
    FS3D_CUDA(cudaMemsetAsync(sbits, 0, (size_t)((ns + 31) / 32) * 4, st));
    k_superbits<<<map_grid(ns * 32), 256, 0, st>>>(bm_bits, BX, BY, BZ, sbits, SBX, SBY, SBZ);
    FS3D_CHECK_LAUNCH("super-brick map launch");
    *bm = BrickMap{bm_bits, BX, BY, BZ, sbits, SBX, SBY, SBZ};
    return FS3D_OK;
}

// bm_bits: brickmap_bytes(X, Y, Z) of device scratch the caller provides
fs3d_status launch_render_dda_bytes(const uint8_t* g, int X, int Y, int Z, uint32_t* bm_bits, const fs3d_camera* cam,
                                    int W, int H, float* rgba_dev, cudaStream_t st) {
    const int BX = (X + 7) / 8, BZ = (Z + 7) / 8;
    FS3D_CUDA(cudaMemsetAsync(bm_bits, 0, (size_t)brick_words(X, Y, Z) * 4, st));
    k_brickmap_bytes<<<map_grid((int64_t)Y * Z * BX), 256, 0, st>>>(g, X, Y, Z, bm_bits, BX, BZ);
    FS3D_CHECK_LAUNCH("brick map (bytes) launch");
    BrickMap bm;
    const fs3d_status s = superbits_and_map(bm_bits, X, Y, Z, st, &bm);
    if (s != FS3D_OK) return s;
    const dim3 blk(16, 16), grd((W + 15) / 16, (H + 15) / 16);
    k_render_dda<BytesGrid><<<grd, blk, 0, st>>>(BytesGrid{g, X, Y, Z}, bm, to_dev(cam), W, H,
                                                 reinterpret_cast<float4*>(rgba_dev));
    FS3D_CHECK_LAUNCH("render dda launch");
    return FS3D_OK;
}

fs3d_status launch_render_dda_planes(const uint4* rows, const uint8_t* statics, int X, int Y, int Z, int nw,
                                     uint32_t* bm_bits, const fs3d_camera* cam, int W, int H, float* rgba_dev,
                                     cudaStream_t st, int* brick_counts, bool recount) {
    const int BX = (X + 7) / 8, BY = (Y + 7) / 8, BZ = (Z + 7) / 8;
    const int64_t nb = (int64_t)BX * BY * BZ;
    if (brick_counts) {
        if (recount) {
            FS3D_CUDA(cudaMemsetAsync(brick_counts, 0, brick_count_bytes(X, Y, Z), st));
            k_brickcount_planes<<<map_grid((int64_t)Y * Z * nw), 256, 0, st>>>(rows, X, Y, Z, nw, brick_counts, BX, BZ);
            FS3D_CHECK_LAUNCH("brick counts (planes) launch");
        }
        k_counts_to_bits<<<map_grid((nb + 31) / 32 + 32), 256, 0, st>>>(brick_counts, nb, bm_bits);
        FS3D_CHECK_LAUNCH("brick map from counts launch");
    } else {
        FS3D_CUDA(cudaMemsetAsync(bm_bits, 0, (size_t)brick_words(X, Y, Z) * 4, st));
        k_brickmap_planes<<<map_grid((int64_t)Y * Z * nw), 256, 0, st>>>(rows, X, Y, Z, nw, bm_bits, BX, BZ);
        FS3D_CHECK_LAUNCH("brick map (planes) launch");
    }
    BrickMap bm;
    const fs3d_status s = superbits_and_map(bm_bits, X, Y, Z, st, &bm);
    if (s != FS3D_OK) return s;
    const dim3 blk(16, 16), grd((W + 15) / 16, (H + 15) / 16);
    k_render_dda<PlaneGrid><<<grd, blk, 0, st>>>(PlaneGrid{reinterpret_cast<const uint32_t*>(rows), statics, X, Y, Z, nw},
                                                 bm, to_dev(cam), W, H, reinterpret_cast<float4*>(rgba_dev));
    FS3D_CHECK_LAUNCH("render dda (planes) launch");
    return FS3D_OK;
}

size_t brick_count_bytes(int X, int Y, int Z) {
    return (size_t)((X + 7) / 8) * ((Y + 7) / 8) * ((Z + 7) / 8) * sizeof(int);
}

size_t brickmap_bytes(int X, int Y, int Z) {
    const size_t super_words = (((size_t)(X + 63) / 64) * ((Y + 63) / 64) * ((Z + 63) / 64) + 31) / 32;
    return ((size_t)brick_words(X, Y, Z) + super_words) * 4;
}

}  // namespace fs3d

extern "C" fs3d_status fs3d_render_sdf(const fs3d_camera* cam, int W, int H, float* rgba_dev, void* stream) {
    if (!cam || !rgba_dev || W <= 0 || H <= 0)
        return fs3d::set_error(FS3D_ERR_INVALID_ARG, "fs3d_render_sdf: bad args");
    return fs3d::launch_render_sdf(cam, W, H, rgba_dev, (cudaStream_t)stream);
}
