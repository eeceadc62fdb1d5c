// Drop-in step on a canonical uint8 grid in device memory (FS3D-rule v1).
//
// Two kernels, both in place (Margolus blocks of one step are disjoint):
//  * k_step_simple: one thread per 2x2x2 block, byte loads; any dims.
//  * k_step_rows16: X % 16 == 0.  A thread owns a 16-byte chunk of x in the
//    four rows (2 y x 2 z) of one block row-pair, loads them as uint4, checks
//    each block for possible motion with byte-parallel tests, runs the rule
//    only on blocks that can move and stores uint4 rows back.  In the odd
//    phase the blocks start at odd x, so one block straddles each chunk
//    boundary: the chunk on the left owns it, receives the neighbour's first
//    byte through a warp shuffle and hands the updated byte back the same way;
//    across a warp boundary the owner reads/writes that byte itself and the
//    right-hand thread stores only bytes 1..15.  Every cell is read for
//    computation and written by exactly one thread, so there is no race.
#include <stdint.h>

#include "fs3d_common.h"
#include "conv_device.cuh"
#include "rule_device.cuh"

namespace fs3d {

// ---------------------------------------------------------------------------
// simple kernel: one thread per block
// ---------------------------------------------------------------------------
__global__ void k_step_simple(uint8_t* __restrict__ grid, int X, int Y, int Z, int o, uint32_t sk) {
    const int NBX = nblocks(X, o), NBY = nblocks(Y, o), NBZ = nblocks(Z, o);
    const int64_t nb = (int64_t)NBX * NBY * NBZ;
    for (int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; b < nb;
         b += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(b % NBX);
        const int k = (int)((b / NBX) % NBZ);
        const int j = (int)(b / ((int64_t)NBX * NBZ));
        const int bx = 2 * i - o, by = 2 * j - o, bz = 2 * k - o;
        uint64_t V = 0;
        int64_t idx[8];
#pragma unroll
        for (int s = 0; s < 8; ++s) {
            const int x = bx + (s & 1), y = by + 1 - (s >> 2), z = bz + ((s >> 1) & 1);
            const bool in = x >= 0 && x < X && y >= 0 && y < Y && z >= 0 && z < Z;
            idx[s] = in ? (int64_t)x + (int64_t)X * ((int64_t)z + (int64_t)Z * y) : -1;
            V |= (uint64_t)(in ? grid[idx[s]] : (uint8_t)1) << (8 * s);
        }
        if (!block_can_move((uint32_t)V, (uint32_t)(V >> 32))) continue;
        const uint64_t N = block_rule(V, rowkey(sk, (uint32_t)j, (uint32_t)k), (uint32_t)i);
#pragma unroll
        for (int s = 0; s < 8; ++s)
            if (idx[s] >= 0 && get_byte(N, s) != get_byte(V, s)) grid[idx[s]] = (uint8_t)get_byte(N, s);
    }
}

// ---------------------------------------------------------------------------
// vectorised kernel (X % 16 == 0, grid 16-byte aligned)
// ---------------------------------------------------------------------------
struct Row16 {
    uint32_t w[4];
};

__device__ __forceinline__ Row16 load_row(const uint8_t* p) {
    const uint4 v = *reinterpret_cast<const uint4*>(p);
    return Row16{{v.x, v.y, v.z, v.w}};
}
__device__ __forceinline__ void store_row(uint8_t* p, const Row16& r) {
    *reinterpret_cast<uint4*>(p) = make_uint4(r.w[0], r.w[1], r.w[2], r.w[3]);
}
// bytes 1..15 only (byte 0 belongs to a block owned by another warp)
__device__ __forceinline__ void store_row_tail15(uint8_t* p, const Row16& r) {
    p[1] = (uint8_t)(r.w[0] >> 8);
    *reinterpret_cast<uint16_t*>(p + 2) = (uint16_t)(r.w[0] >> 16);
    *reinterpret_cast<uint32_t*>(p + 4) = r.w[1];
    *reinterpret_cast<uint2*>(p + 8) = make_uint2(r.w[2], r.w[3]);
}
__device__ __forceinline__ Row16 solid_row() { return Row16{{0x01010101u, 0x01010101u, 0x01010101u, 0x01010101u}}; }

// row' = row >> 8 bytes, with `next` as byte 15: byte p of row' is cell 16c+1+p
__device__ __forceinline__ Row16 shift_down(const Row16& r, uint32_t next) {
    Row16 o;
    o.w[0] = __funnelshift_r(r.w[0], r.w[1], 8);
    o.w[1] = __funnelshift_r(r.w[1], r.w[2], 8);
    o.w[2] = __funnelshift_r(r.w[2], r.w[3], 8);
    o.w[3] = __funnelshift_r(r.w[3], next, 8);
    return o;
}
// inverse: row = (row' << 8 bytes) | first
__device__ __forceinline__ Row16 shift_up(const Row16& r, uint32_t first) {
    Row16 o;
    o.w[0] = (r.w[0] << 8) | (first & 0xFFu);
    o.w[1] = __funnelshift_l(r.w[0], r.w[1], 8);
    o.w[2] = __funnelshift_l(r.w[1], r.w[2], 8);
    o.w[3] = __funnelshift_l(r.w[2], r.w[3], 8);
    return o;
}

// Runs the 8 blocks whose cells are bytes (2p, 2p+1) of the four rows.
// rows: [0] top z0, [1] top z1, [2] bottom z0, [3] bottom z1.
__device__ __forceinline__ void run_chunk(Row16 (&r)[4], uint32_t rk, uint32_t i0) {
#pragma unroll
    for (int p = 0; p < 8; ++p) {
        const int w = p >> 1;
        const uint32_t sel = (p & 1) ? 0x7632u : 0x5410u;
        const uint32_t T = __byte_perm(r[0].w[w], r[1].w[w], sel);
        const uint32_t B = __byte_perm(r[2].w[w], r[3].w[w], sel);
        if (!block_can_move(T, B)) continue;
        const uint64_t V = (uint64_t)T | ((uint64_t)B << 32);
        const uint64_t N = block_rule(V, rk, i0 + (uint32_t)p);
        if (N == V) continue;
        const uint32_t nT = (uint32_t)N, nB = (uint32_t)(N >> 32);
        const uint32_t s0 = (p & 1) ? 0x5410u : 0x3254u;  // layer bytes 0,1 -> row bytes
        const uint32_t s1 = (p & 1) ? 0x7610u : 0x3276u;  // layer bytes 2,3 -> row bytes
        r[0].w[w] = __byte_perm(r[0].w[w], nT, s0);
        r[1].w[w] = __byte_perm(r[1].w[w], nT, s1);
        r[2].w[w] = __byte_perm(r[2].w[w], nB, s0);
        r[3].w[w] = __byte_perm(r[3].w[w], nB, s1);
    }
}

__global__ void __launch_bounds__(256) k_step_rows16(uint8_t* __restrict__ grid, int X, int Y, int Z,
                                                    int o, uint32_t sk) {
    const int NC = X >> 4;
    const int NBY = nblocks(Y, o), NBZ = nblocks(Z, o);
    const int64_t units = (int64_t)NC * NBY * NBZ;
    const int lane = threadIdx.x & 31;
    // every lane of a warp runs the same number of iterations (shuffles)
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t u0 = (int64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31); u0 < units; u0 += stride) {
        const int64_t u = u0 + lane;
        const bool valid = u < units;
        const int c = valid ? (int)(u % NC) : 0;
        const int64_t rp = valid ? u / NC : 0;
        const int k = (int)(rp % NBZ), j = (int)(rp / NBZ);
        const int y0 = 2 * j - o, z0 = 2 * k - o;
        // rows: top z0, top z1, bottom z0, bottom z1
        const int ry[4] = {y0 + 1, y0 + 1, y0, y0};
        const int rz[4] = {z0, z0 + 1, z0, z0 + 1};
        bool rin[4];
        uint8_t* rptr[4];
        Row16 r[4];
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            rin[a] = valid && ry[a] >= 0 && ry[a] < Y && rz[a] >= 0 && rz[a] < Z;
            rptr[a] = rin[a] ? grid + ((int64_t)X * ((int64_t)rz[a] + (int64_t)Z * ry[a]) + 16 * (int64_t)c)
                             : grid;
            r[a] = rin[a] ? load_row(rptr[a]) : solid_row();
        }
        const uint32_t rk = rowkey(sk, (uint32_t)j, (uint32_t)k);
        // neighbours inside this warp hold the adjacent chunks of the same rows
        const bool left_in_warp = valid && c > 0 && lane > 0;
        const bool right_in_warp = valid && c < NC - 1 && lane < 31 && (u + 1) < units;
        if (o == 0) {
            run_chunk(r, rk, 8u * (uint32_t)c);
#pragma unroll
            for (int a = 0; a < 4; ++a)
                if (rin[a]) store_row(rptr[a], r[a]);
        } else {
            Row16 s[4];
            uint32_t half[4];
#pragma unroll
            for (int a = 0; a < 4; ++a) {
                // first byte of the chunk on the right (cell 16c+16)
                uint32_t nxt = __shfl_down_sync(0xffffffffu, r[a].w[0], 1) & 0xFFu;
                if (!right_in_warp) {
                    nxt = 1u;  // outside the grid: solid
                    if (rin[a] && c < NC - 1) nxt = rptr[a][16];
                }
                s[a] = shift_down(r[a], nxt);
                half[a] = r[a].w[0] & 0xFFu;  // cell 16c (used only when c == 0)
            }
            run_chunk(s, rk, 8u * (uint32_t)c + 1u);
            if (c == 0 && valid) {
                // half block at bx = -1: only its dx=1 cells (x = 0) exist
                const uint32_t T = 0x00010001u | (half[0] << 8) | (half[1] << 24);
                const uint32_t B = 0x00010001u | (half[2] << 8) | (half[3] << 24);
                if (block_can_move(T, B)) {
                    const uint64_t V = (uint64_t)T | ((uint64_t)B << 32);
                    const uint64_t N = block_rule(V, rk, 0u);
                    half[0] = (uint32_t)(N >> 8) & 0xFFu;
                    half[1] = (uint32_t)(N >> 24) & 0xFFu;
                    half[2] = (uint32_t)(N >> 40) & 0xFFu;
                    half[3] = (uint32_t)(N >> 56) & 0xFFu;
                }
            }
#pragma unroll
            for (int a = 0; a < 4; ++a) {
                // updated cell 16c comes from the owner on the left
                const uint32_t from_left = __shfl_up_sync(0xffffffffu, s[a].w[3] >> 24, 1);
                const Row16 out = shift_up(s[a], c == 0 ? half[a] : from_left);
                if (!rin[a]) continue;
                if (c == 0 || left_in_warp)
                    store_row(rptr[a], out);
                else
                    store_row_tail15(rptr[a], out);
                if (!right_in_warp && c < NC - 1) rptr[a][16] = (uint8_t)(s[a].w[3] >> 24);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// bit-sliced byte kernel (X % 64 == 0, X <= 2048, grid 16-byte aligned)
//
// A lane owns 64 cells of each of the four rows of a block row-pair (16 uint4
// loads), turns them into plane words in registers, runs the shared
// bit-sliced row-pair step (32 blocks per 32-bit operation) and writes back
// only the 16-byte pieces whose cells changed class.
// ---------------------------------------------------------------------------

// Merges the new class of every changed cell of one 16-byte piece u (word
// pairs 2u, 2u+1 of a 64-cell chunk) into its bytes.  Only empty, sand and
// water cells change, and their byte is their code (A << 1) | B.
__device__ __forceinline__ uint4 merge_piece(uint4 v, int u, uint32_t che, uint32_t cho, const uint4& n) {
    uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int p = 2 * u + h;
        const uint32_t ce = (che >> (4 * p)) & 0xFu, co = (cho >> (4 * p)) & 0xFu;
        const uint32_t ve = (spread4((n.x >> (4 * p)) & 0xFu) << 1) | spread4((n.z >> (4 * p)) & 0xFu);
        const uint32_t vo = (spread4((n.y >> (4 * p)) & 0xFu) << 1) | spread4((n.w >> (4 * p)) & 0xFu);
        const uint32_t me = spread4(ce) * 0xFFu, mo = spread4(co) * 0xFFu;
        const uint32_t m0 = __byte_perm(me, mo, 0x5140), m1 = __byte_perm(me, mo, 0x7362);
        w[2 * h] = (w[2 * h] & ~m0) | (__byte_perm(ve, vo, 0x5140) & m0);
        w[2 * h + 1] = (w[2 * h + 1] & ~m1) | (__byte_perm(ve, vo, 0x7362) & m1);
    }
    return make_uint4(w[0], w[1], w[2], w[3]);
}

// `rev` walks the row-pairs from the top: consecutive steps alternate, so a
// step starts on the rows the previous one touched last (still in L2).  The
// loaded bytes are not kept across the rule (that would cost 64 registers);
// the 16-byte pieces with changed cells are read again (L1) when merging.
#ifndef FS3D_ROWS64_CTAS_PER_SM
#define FS3D_ROWS64_CTAS_PER_SM 6  // register cap: 6 CTAs of 128 threads per SM (measured best)
#endif
__global__ void __launch_bounds__(128, FS3D_ROWS64_CTAS_PER_SM)
    k_step_rows64(uint8_t* __restrict__ grid, int X, int Y, int Z, int o,
                                                       uint32_t sk, int lg, int rev) {
    const int NC = X >> 6, G = 1 << lg, per = 32 >> lg;
    const int NBZ = nblocks(Z, o), NRP = nblocks(Y, o) * NBZ;
    const int lane = threadIdx.x & 31, gl = lane & (G - 1);
    const int warps = (gridDim.x * blockDim.x) >> 5;
    const int n_items = (NRP + per - 1) / per;
    for (int it0 = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; it0 < n_items; it0 += warps) {
        const int it = rev ? n_items - 1 - it0 : it0;
        const int rp = it * per + (lane >> lg);
        const bool valid = rp < NRP;  // every lane takes part in the row-pair step
        const int j = valid ? rp / NBZ : 0, k = valid ? rp - j * NBZ : 0;
        const uint32_t rk = rowkey(sk, (uint32_t)j, (uint32_t)k);
        const int y0 = 2 * j - o, z0 = 2 * k - o;
        const bool has = valid && gl < NC;
        uint4 q[4], q0[4];
        uint4* ptr[4];
        bool in[4];
        // Settled-work skip: without a sand or water cell nothing can move, and
        // a byte without bit 1 (values 0, 1, 4, 5, ...) is neither.  The test is
        // warp-uniform, so the cells a lane borrows from its neighbour for the
        // straddling blocks are covered too.  The loads hit L1 again below.
        uint32_t part = 0;
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            const int y = (a < 2) ? y0 + 1 : y0, z = z0 + (a & 1);
            in[a] = has && y >= 0 && y < Y && z >= 0 && z < Z;
            ptr[a] = reinterpret_cast<uint4*>(in[a] ? grid + ((int64_t)y * Z + z) * X + 64 * gl : grid);
            if (in[a])
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const uint4 v = ptr[a][u];
                    part |= v.x | v.y | v.z | v.w;
                }
        }
        if (__all_sync(0xFFFFFFFFu, (part & 0x02020202u) == 0u)) continue;
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            if (in[a]) {
                uint32_t w[16];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const uint4 v = ptr[a][u];
                    w[4 * u] = v.x;
                    w[4 * u + 1] = v.y;
                    w[4 * u + 2] = v.z;
                    w[4 * u + 3] = v.w;
                }
                q[a] = bytes_to_planes64(w);
            } else {
                q[a] = make_uint4(0u, 0u, 0xFFFFFFFFu, 0xFFFFFFFFu);
            }
            q0[a] = q[a];
        }
        rowpair_core(q, has, o, rk, gl, G, NC, true);
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            if (!in[a]) continue;
            const uint32_t che = (q[a].x ^ q0[a].x) | (q[a].z ^ q0[a].z);
            const uint32_t cho = (q[a].y ^ q0[a].y) | (q[a].w ^ q0[a].w);
            if (!(che | cho)) continue;
#pragma unroll
            for (int u = 0; u < 4; ++u)
                if (((che | cho) >> (8 * u)) & 0xFFu) ptr[a][u] = merge_piece(ptr[a][u], u, che, cho, q[a]);
        }
    }
}

// ---------------------------------------------------------------------------
// hash and first difference
// ---------------------------------------------------------------------------
__global__ void k_hash_bytes(const uint8_t* __restrict__ g, int64_t n, unsigned long long* out) {
    uint64_t h = 0;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t n16 = ((reinterpret_cast<uintptr_t>(g) & 15u) == 0) ? n / 16 : 0;
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n16; v += stride) {
        const uint4 q = reinterpret_cast<const uint4*>(g)[v];
        const uint32_t w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
        for (int b = 0; b < 16; ++b)
            h += fmix64((uint64_t)(16 * v + b) * 256u + ((w[b >> 2] >> (8 * (b & 3))) & 0xFFu));
    }
    for (int64_t i = 16 * n16 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        h += fmix64((uint64_t)i * 256u + g[i]);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) h += __shfl_xor_sync(0xffffffffu, h, off);
    if ((threadIdx.x & 31) == 0 && h) atomicAdd(out, (unsigned long long)h);
}

__global__ void k_first_diff(const uint8_t* __restrict__ a, const uint8_t* __restrict__ b, int64_t n,
                             unsigned long long* out) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        if (a[i] != b[i]) {
            atomicMin(out, (unsigned long long)i);
            return;
        }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
// device properties, looked up once per process (thread-safe static initialisation)
static int sm_count() {
    static const int n = [] {
        int dev = 0, v = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
        return v > 0 ? v : 148;
    }();
    return n;
}

static int grid_for(int64_t work, int threads, int per_sm) {
    const int64_t need = (work + threads - 1) / threads;
    const int64_t cap = (int64_t)sm_count() * per_sm;
    return (int)(need < cap ? (need > 0 ? need : 1) : cap);
}

bool rows16_ok(const void* grid, int X) {
    return (X % 16) == 0 && (reinterpret_cast<uintptr_t>(grid) & 15u) == 0;
}

bool rows64_ok(const void* grid, int X) {
    return (X % 64) == 0 && X <= 2048 && (reinterpret_cast<uintptr_t>(grid) & 15u) == 0;
}

static int rows64_lg(int X) {
    int lg = 0;
    while ((1 << lg) < (X >> 6)) ++lg;
    return lg;
}

static int rows64_ctas_per_sm() {
    static const int n = [] {
        int v = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, k_step_rows64, 128, 0) != cudaSuccess || v < 1) v = 1;
        return v;
    }();
    return n;
}

fs3d_status launch_step_bytes(uint8_t* grid, int X, int Y, int Z, uint64_t seed, uint64_t t0, int n_steps,
                              cudaStream_t st) {
    for (int a = 0; a < n_steps; ++a) {
        const uint64_t t = t0 + (uint64_t)a;
        const int o = (int)(t & 1u);
        const uint32_t sk = stepkey(seed, t);
        if (rows64_ok(grid, X)) {
            const int lg = rows64_lg(X);
            const int per = 32 >> lg;
            const int64_t items = ((int64_t)nblocks(Y, o) * nblocks(Z, o) + per - 1) / per;
            k_step_rows64<<<grid_for(items * 32, 128, rows64_ctas_per_sm()), 128, 0, st>>>(grid, X, Y, Z, o, sk,
                                                                                          lg, (int)(a & 1));
        } else if (rows16_ok(grid, X)) {
            const int64_t units = (int64_t)(X >> 4) * nblocks(Y, o) * nblocks(Z, o);
            k_step_rows16<<<grid_for(units, 256, 8), 256, 0, st>>>(grid, X, Y, Z, o, sk);
        } else {
            const int64_t nb = (int64_t)nblocks(X, o) * nblocks(Y, o) * nblocks(Z, o);
            k_step_simple<<<grid_for(nb, 256, 8), 256, 0, st>>>(grid, X, Y, Z, o, sk);
        }
        FS3D_CHECK_LAUNCH("step kernel launch");
    }
    return FS3D_OK;
}

// forces the one-thread-per-block kernel (used to cross-check the fast one)
fs3d_status launch_step_simple(uint8_t* grid, int X, int Y, int Z, uint64_t seed, uint64_t t0, int n_steps,
                               cudaStream_t st) {
    for (int a = 0; a < n_steps; ++a) {
        const uint64_t t = t0 + (uint64_t)a;
        const int o = (int)(t & 1u);
        const int64_t nb = (int64_t)nblocks(X, o) * nblocks(Y, o) * nblocks(Z, o);
        k_step_simple<<<grid_for(nb, 256, 8), 256, 0, st>>>(grid, X, Y, Z, o, stepkey(seed, t));
        FS3D_CHECK_LAUNCH("simple step kernel launch");
    }
    return FS3D_OK;
}

fs3d_status hash_bytes_async(const uint8_t* g, int64_t n, unsigned long long* out_dev, cudaStream_t st) {
    FS3D_CUDA(cudaMemsetAsync(out_dev, 0, sizeof(unsigned long long), st));
    k_hash_bytes<<<grid_for((n + 15) / 16, 256, 8), 256, 0, st>>>(g, n, out_dev);
    FS3D_CHECK_LAUNCH("hash kernel launch");
    return FS3D_OK;
}

int sm_count_public() { return sm_count(); }

}  // namespace fs3d

using namespace fs3d;

static bool dims_valid(int X, int Y, int Z) {
    return X > 0 && Y > 0 && Z > 0 && X <= (1 << 20) && Y <= (1 << 20) && Z <= (1 << 20);
}

extern "C" {

fs3d_status fs3d_step_device(uint8_t* grid_dev, int X, int Y, int Z, uint64_t seed, uint64_t t0, int n_steps,
                             void* stream) {
    if (!grid_dev || !dims_valid(X, Y, Z) || n_steps < 0)
        return set_error(FS3D_ERR_INVALID_ARG, "fs3d_step_device: null grid, bad dims or negative n_steps");
    return launch_step_bytes(grid_dev, X, Y, Z, seed, t0, n_steps, (cudaStream_t)stream);
}

fs3d_status fs3d_step_device_many(int n, uint8_t* const* grids_dev, const int* dims, const uint64_t* seeds,
                                  uint64_t t0, int n_steps, void* stream) {
    if (n < 0 || n_steps < 0 || (n > 0 && (!grids_dev || !dims || !seeds)))
        return set_error(FS3D_ERR_INVALID_ARG, "fs3d_step_device_many: bad args");
    for (int w = 0; w < n; ++w)
        if (!grids_dev[w] || !dims_valid(dims[3 * w], dims[3 * w + 1], dims[3 * w + 2]))
            return set_error(FS3D_ERR_INVALID_ARG, "fs3d_step_device_many: null grid or bad dims");
    // step-major, one launch per world per step: every world takes step t
    // before any takes step t + 1, as separate callers stepping their own
    // worlds would
    for (int a = 0; a < n_steps; ++a)
        for (int w = 0; w < n; ++w) {
            const fs3d_status s = launch_step_bytes(grids_dev[w], dims[3 * w], dims[3 * w + 1], dims[3 * w + 2],
                                                    seeds[w], t0 + (uint64_t)a, 1, (cudaStream_t)stream);
            if (s != FS3D_OK) return s;
        }
    return FS3D_OK;
}

fs3d_status fs3d_step_device_simple(uint8_t* grid_dev, int X, int Y, int Z, uint64_t seed, uint64_t t0,
                                    int n_steps, void* stream) {
    if (!grid_dev || !dims_valid(X, Y, Z) || n_steps < 0)
        return set_error(FS3D_ERR_INVALID_ARG, "fs3d_step_device_simple: bad args");
    return launch_step_simple(grid_dev, X, Y, Z, seed, t0, n_steps, (cudaStream_t)stream);
}

fs3d_status fs3d_hash_device(const uint8_t* grid_dev, int64_t n, void* stream, uint64_t* out) {
    if (!grid_dev || n < 0 || !out) return set_error(FS3D_ERR_INVALID_ARG, "fs3d_hash_device: bad args");
    cudaStream_t st = (cudaStream_t)stream;
    unsigned long long* d = nullptr;
    FS3D_CUDA(cudaMallocAsync((void**)&d, sizeof(*d), st));
    fs3d_status s = hash_bytes_async(grid_dev, n, d, st);
    unsigned long long h = 0;
    if (s == FS3D_OK) {
        cudaError_t e = cudaMemcpyAsync(&h, d, sizeof(h), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) s = cuda_fail(e, "fs3d_hash_device readback");
    }
    cudaFreeAsync(d, st);
    if (s == FS3D_OK) *out = (uint64_t)h;
    return s;
}

fs3d_status fs3d_first_diff_device(const uint8_t* a, const uint8_t* b, int64_t n, void* stream, int64_t* out) {
    if (!a || !b || n < 0 || !out) return set_error(FS3D_ERR_INVALID_ARG, "fs3d_first_diff_device: bad args");
    cudaStream_t st = (cudaStream_t)stream;
    unsigned long long* d = nullptr;
    FS3D_CUDA(cudaMallocAsync((void**)&d, sizeof(*d), st));
    fs3d_status s = FS3D_OK;
    cudaError_t e = cudaMemsetAsync(d, 0xFF, sizeof(*d), st);
    if (e != cudaSuccess) s = cuda_fail(e, "first_diff memset");
    if (s == FS3D_OK && n > 0) {
        k_first_diff<<<grid_for(n, 256, 8), 256, 0, st>>>(a, b, n, d);
        e = cudaGetLastError();
        if (e != cudaSuccess) s = cuda_fail(e, "first_diff launch");
        else note_launch();
    }
    unsigned long long r = ~0ull;
    if (s == FS3D_OK) {
        e = cudaMemcpyAsync(&r, d, sizeof(r), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) s = cuda_fail(e, "first_diff readback");
    }
    cudaFreeAsync(d, st);
    if (s == FS3D_OK) *out = (r == ~0ull) ? -1 : (int64_t)r;
    return s;
}

}  // extern "C"
