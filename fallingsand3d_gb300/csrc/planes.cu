// Bit-plane world format and the multi-world bit-sliced step.
//
// Format.  A world of X*Y*Z cells is stored as Y*Z rows (row r = y*Z + z) of
// nw = ceil(X/64) uint4 words; word g of a row covers x in [64g, 64g+64) and
// holds {A even, A odd, B even, B odd}: bit m of an even word is x = 64g+2m,
// of an odd word x = 64g+2m+1.  (A,B) = (0,0) empty, (0,1) solid, (1,0) sand,
// (1,1) water; cells past X are solid.  Static cells never change, so their
// byte values (stone, or any material >= 4) are taken from an optional byte
// copy of the initial grid when the world is read back.
//
// Step.  The blocks of a block row that start in word g (i = 32g .. 32g+31)
// are evaluated together: in the even phase their dx=0 / dx=1 cells are the
// even / odd words of g; in the odd phase (blocks start at odd x) the dx=0
// cells are the odd word shifted up one bit with the top bit of word g-1
// carried in, and the dx=1 cells are the even word.  A lane group of
// G = pow2ceil(nw) lanes handles one block row-pair (4 rows); lane g owns
// storage word g and the carried bit travels by warp shuffle, so each bit is
// read for computation and written by exactly one lane.  When X is a multiple
// of 64 the odd phase has one extra half block per row-pair (cells x = X-1,
// x = X outside), which the last lane runs with the scalar rule.
#include <cooperative_groups.h>
#include <stdint.h>

#include <algorithm>
#include <mutex>

#include "fs3d_common.h"
#include "pcg.h"
#include "planes.h"
#include "conv_device.cuh"
#include "rule_device.cuh"
#include "bricks_device.cuh"

namespace fs3d {

// ---------------------------------------------------------------------------
// conversions
// ---------------------------------------------------------------------------
// One (row, word) unit: the 64-cell chunk at x = 64w of row r.
__device__ __forceinline__ uint4 chunk_to_planes(const uint8_t* row, int X, int w, bool& big) {
    uint32_t v[16];
    load_chunk64(row + 64 * w, min(64, X - 64 * w), v, big);
    return bytes_to_planes64(v);
}

__device__ __forceinline__ void planes_to_chunk(const uint4& q, const uint8_t* statics_row, uint8_t* row, int X,
                                                int w) {
    uint32_t v[16];
    planes_to_words64(q, v);
    const int n = min(64, X - 64 * w);
    if (statics_row) patch_statics64(q, statics_row + 64 * w, n, v);
    store_chunk64(row + 64 * w, n, v);
}

__global__ void k_bytes_to_planes(const uint8_t* __restrict__ g, int X, int Y, int Z, int nw,
                                  uint4* __restrict__ rows) {
    const int64_t n = (int64_t)Y * Z * nw;
    for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < n; u += (int64_t)gridDim.x * blockDim.x) {
        const int w = (int)(u % nw);
        const int64_t r = u / nw;
        bool big;
        rows[u] = chunk_to_planes(g + r * X, X, w, big);
    }
}

// the byte value of one cell of a plane word (static cells from `statics`, or stone)
__device__ __forceinline__ uint32_t cell_value(const uint4& q, int m, int odd, const uint8_t* statics, int64_t idx) {
    const uint32_t a = ((odd ? q.y : q.x) >> m) & 1u, b = ((odd ? q.w : q.z) >> m) & 1u;
    if (a) return b ? 3u : 2u;
    if (!b) return 0u;
    return statics ? statics[idx] : 1u;
}

__global__ void k_planes_to_bytes(const uint4* __restrict__ rows, const uint8_t* __restrict__ statics, int X,
                                  int Y, int Z, int nw, uint8_t* __restrict__ g, const int* skip_if_set) {
    if (skip_if_set && *(volatile const int*)skip_if_set) return;
    const int64_t n = (int64_t)Y * Z * nw;
    for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < n; u += (int64_t)gridDim.x * blockDim.x) {
        const int w = (int)(u % nw);
        const int64_t r = u / nw;
        planes_to_chunk(rows[u], statics ? statics + r * X : nullptr, g + r * X, X, w);
    }
}

__global__ void k_hash_planes(const uint4* __restrict__ rows, const uint8_t* __restrict__ statics, int X, int Y,
                              int Z, int nw, unsigned long long* out) {
    const int64_t n = (int64_t)Y * Z * nw;
    uint64_t h = 0;
    for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < n; u += (int64_t)gridDim.x * blockDim.x) {
        const int w = (int)(u % nw);
        const int64_t r = u / nw;
        const uint4 q = rows[u];
        for (int x = 64 * w; x < 64 * w + 64 && x < X; ++x) {
            const int64_t idx = r * X + x;
            h += fmix64((uint64_t)idx * 256u + cell_value(q, (x >> 1) & 31, x & 1, statics, idx));
        }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) h += __shfl_xor_sync(0xffffffffu, h, off);
    if ((threadIdx.x & 31) == 0 && h) atomicAdd(out, (unsigned long long)h);
}

// Whole-grid hashes of many worlds in one launch: CTA j hashes world j
// (jobs[j]) and writes its sum to out[j].
__global__ void __launch_bounds__(256) k_hash_planes_many(const HashJob* __restrict__ jobs,
                                                         unsigned long long* __restrict__ out) {
    const HashJob jb = jobs[blockIdx.x];
    const int64_t n = (int64_t)jb.Y * jb.Z * jb.nw;
    uint64_t h = 0;
    for (int64_t u = threadIdx.x; u < n; u += blockDim.x) {
        const int w = (int)(u % jb.nw);
        const int64_t r = u / jb.nw;
        const uint4 q = jb.rows[u];
        for (int x = 64 * w; x < 64 * w + 64 && x < jb.X; ++x) {
            const int64_t idx = r * jb.X + x;
            h += fmix64((uint64_t)idx * 256u + cell_value(q, (x >> 1) & 31, x & 1, jb.statics, idx));
        }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) h += __shfl_xor_sync(0xffffffffu, h, off);
    __shared__ unsigned long long part[8];
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = h;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long t = 0;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += part[i];
        out[blockIdx.x] = t;
    }
}

// Many worlds per launch (admission and retirement of a batch): job j covers
// units [unit_off[j], unit_off[j+1]) of (row, word) pairs; its bytes sit at
// byte_off in one staging buffer.
__device__ __forceinline__ int find_job(const int64_t* __restrict__ unit_off, int njobs, int64_t u) {
    int lo = 0, hi = njobs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(unit_off + mid) <= u)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

// The job of a unit: the job of its block's first unit (block_job, from the
// host), then at most a few steps forward (a block of kConvBlock consecutive
// units spans few worlds).
__device__ __forceinline__ int unit_job(const int64_t* __restrict__ unit_off, const int* __restrict__ block_job,
                                        int njobs, int64_t u) {
    int j = __ldg(block_job + u / kConvBlock);
    while (j + 1 < njobs && __ldg(unit_off + j + 1) <= u) ++j;
    return j;
}

// Read-back: a CTA converts kConvBlock consecutive units per pass.  Their
// bytes are one contiguous span of the staging buffer (rows are back to back;
// a span may cross into the next world over at most a few padding bytes), so
// each thread writes its 64-cell chunk into shared memory and the span goes
// out in coalesced 16-byte stores (254 µs for 2048 worlds against 290 µs with
// per-thread stores of rows 16-48 bytes wide).  Rows whose width is not a
// multiple of 8 (chunks not 8-byte aligned), or spans wider than the buffer
// (many tiny worlds), take the direct per-thread path.
constexpr int kConvSpan = kConvBlock * 64 + 64;

struct UnitAt {
    int j;
    int64_t lu, r, pos;  // unit within its world, row, first byte in the staging buffer
    int w, n;            // word within the row, bytes of the chunk
};

__device__ __forceinline__ UnitAt unit_at(const ConvJob& jb, int j, int64_t lu) {
    UnitAt a;
    a.j = j;
    a.lu = lu;
    a.w = jb.nw == 1 ? 0 : (int)(lu % jb.nw);
    a.r = jb.nw == 1 ? lu : lu / jb.nw;
    a.n = min(64, jb.X - 64 * a.w);
    a.pos = jb.byte_off + a.r * jb.X + 64 * a.w;
    return a;
}

// Stores len bytes (a multiple of 8) from shared memory at sm to global g
// (8-byte aligned; sm congruent to g modulo 16) in 16-byte pieces with an
// 8-byte head and tail.
__device__ __forceinline__ void store_span(uint8_t* g, const uint8_t* sm, uint64_t len) {
    const uint64_t head = (reinterpret_cast<uintptr_t>(g) & 15u) ? 8u : 0u;
    const uint64_t body = (len - head) & ~(uint64_t)15;
    if (threadIdx.x == 0 && head) *reinterpret_cast<uint2*>(g) = *reinterpret_cast<const uint2*>(sm);
    for (uint64_t o = head + 16u * threadIdx.x; o < head + body; o += 16u * kConvBlock)
        *reinterpret_cast<uint4*>(g + o) = *reinterpret_cast<const uint4*>(sm + o);
    const uint64_t t = head + body;
    if (threadIdx.x == 0 && t < len) *reinterpret_cast<uint2*>(g + t) = *reinterpret_cast<const uint2*>(sm + t);
}

// Admission: each thread loads and converts its own chunk straight from the
// staging bytes.  (A version staging the span in shared memory, as the
// read-back does, took twice as long: a thread's chunk is X bytes apart from
// its neighbour's, so reading it from shared memory meets 4- to 16-way bank
// conflicts, and loads no longer overlap the conversion.)
__global__ void __launch_bounds__(kConvBlock) k_bytes_to_planes_multi(const ConvJob* __restrict__ jobs,
                                                                      const int64_t* __restrict__ unit_off,
                                                                      const int* __restrict__ block_job, int njobs,
                                                                      int64_t total, const uint8_t* __restrict__ staging,
                                                                      int* flags) {
    for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < total; u += (int64_t)gridDim.x * blockDim.x) {
        const int j = unit_job(unit_off, block_job, njobs, u);
        const ConvJob jb = jobs[j];
        const UnitAt at = unit_at(jb, j, u - unit_off[j]);
        uint32_t v[16];
        bool big;
        load_chunk64(staging + at.pos, at.n, v, big);
        jb.rows[at.lu] = bytes_to_planes64(v);
        if (big) atomicOr(flags + j, 1);  // holds a static material >= 4: keep its bytes
    }
}

__global__ void __launch_bounds__(kConvBlock) k_planes_to_bytes_multi(const ConvJob* __restrict__ jobs,
                                                                      const int64_t* __restrict__ unit_off,
                                                                      const int* __restrict__ block_job, int njobs,
                                                                      int64_t total, uint8_t* __restrict__ staging) {
    __shared__ __align__(16) uint8_t span[kConvSpan + 16];
    __shared__ unsigned long long s_start, s_len;
    for (int64_t base = (int64_t)blockIdx.x * kConvBlock; base < total; base += (int64_t)gridDim.x * kConvBlock) {
        const int64_t u = base + threadIdx.x;
        const bool live = u < total;
        UnitAt at{};
        int X = 0;
        uint32_t v[16];
        if (live) {
            const int j = unit_job(unit_off, block_job, njobs, u);
            const ConvJob jb = jobs[j];
            X = jb.X;
            at = unit_at(jb, j, u - unit_off[j]);
            const uint4 q = jb.rows[at.lu];
            planes_to_words64(q, v);
            const uint8_t* st = jb.statics;
            if (!st && jb.static_flag && *jb.static_flag) st = jb.static_src;
            if (st) patch_statics64(q, st + at.r * jb.X + 64 * at.w, at.n, v);
        }
        if (threadIdx.x == 0) {
            s_start = (unsigned long long)at.pos;  // unit `base` is live
            s_len = 0;
        }
        __syncthreads();
        const uint64_t start = s_start;
        bool direct = live && ((X & 7) != 0 || (uint64_t)at.pos - start + (uint64_t)at.n > (uint64_t)kConvSpan);
        if (live && !direct) atomicMax(&s_len, (unsigned long long)((uint64_t)at.pos - start + (uint64_t)at.n));
        direct = __syncthreads_or(direct) != 0;
        uint8_t* sm = span + (start & 15u);
        if (direct) {
            if (live) store_chunk64(staging + at.pos, at.n, v);
        } else {
            if (live) store_chunk64(sm + ((uint64_t)at.pos - start), at.n, v);
            __syncthreads();
            // the span's padding bytes between two worlds (if any) are written
            // too: they belong to no world
            store_span(staging + start, sm, s_len);
        }
        __syncthreads();  // the span and s_start are rewritten by the next pass
    }
}

// The mixed-size batch world generated straight into planes: stone at y < 2,
// empty below Y/2, and above it one PCG32 draw per cell in index order; each
// thread jumps its generator to the first draw of its 64-cell word.
__global__ void k_gen_batch_planes(int X, int Y, int Z, int nw, BatchWorldGen p, uint4* __restrict__ rows) {
    const int64_t n = (int64_t)Y * Z * nw;
    const int yf = Y / 2;
    for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < n; u += (int64_t)gridDim.x * blockDim.x) {
        const int w = (int)(u % nw);
        const int64_t r = u / nw;
        const int y = (int)(r / Z), z = (int)(r % Z);
        uint32_t ae = 0, ao = 0, be = 0, bo = 0;
        uint64_t st = 0;
        if (y >= yf) st = pcg_jump(p.fill_state, ((uint64_t)(y - yf) * Z + z) * X + 64u * w, p.inc);
        for (int m = 0; m < 64; ++m) {
            const int x = 64 * w + m;
            uint32_t v;
            if (x >= X || y < 2) {
                v = 1u;
            } else if (y < yf) {
                v = 0u;
            } else {
                const uint32_t d = pcg_output(st);
                st = st * kPcgMult + p.inc;
                v = d < p.sand_thr ? 2u : (d < p.water_thr ? 3u : 0u);
            }
            const uint32_t a = v >> 1, b = v & 1u;  // codes 0..3 are their own (A, B)
            if (m & 1) {
                ao |= a << (m >> 1);
                bo |= b << (m >> 1);
            } else {
                ae |= a << (m >> 1);
                be |= b << (m >> 1);
            }
        }
        rows[u] = make_uint4(ae, ao, be, bo);
    }
}

// ---------------------------------------------------------------------------
// step
// ---------------------------------------------------------------------------
// One block row-pair of one world; lane gl of a group of G lanes.  Every lane
// of the warp calls this (valid = false for groups past the last row-pair).
__device__ __forceinline__ void plane_rowpair(const PlaneWorld& w, int o, uint32_t sk, int rp, bool valid, int gl,
                                              int G, int* counts) {
    const int NBZ = nblocks(w.Z, o);
    const int j = valid ? rp / NBZ : 0, k = valid ? rp - j * NBZ : 0;
    const uint32_t rk = rowkey(sk, (uint32_t)j, (uint32_t)k);
    const int y0 = 2 * j - o, z0 = 2 * k - o;
    const bool has = valid && gl < w.nw;
    uint4 q[4], q0[4];
    uint4* ptr[4];
    bool in[4];
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        const int y = (a < 2) ? y0 + 1 : y0, z = z0 + (a & 1);
        in[a] = has && y >= 0 && y < w.Y && z >= 0 && z < w.Z;
        ptr[a] = in[a] ? w.rows + ((int64_t)y * w.Z + z) * w.nw + gl : w.rows;
        q[a] = in[a] ? *ptr[a] : make_uint4(0u, 0u, 0xFFFFFFFFu, 0xFFFFFFFFu);
        q0[a] = q[a];
    }
    rowpair_core(q, has, o, rk, gl, G, w.nw, (w.X & 63) == 0);
    bool any = false;
#pragma unroll
    for (int a = 0; a < 4; ++a)
        if (in[a] && (q[a].x != q0[a].x || q[a].y != q0[a].y || q[a].z != q0[a].z || q[a].w != q0[a].w)) {
            *ptr[a] = q[a];
            any = true;
        }
    if (counts && any) count_bricks(counts, w, y0, z0, gl, q, q0, in);
}

// One launch = one step (segment step s_seg) of every live world.  Work items
// are warp-sized: item = (world, first row-pair); a warp covers 32 >> lg
// row-pairs of that world.  Warps loop over items; the item count lives in
// device memory so a captured graph keeps working as worlds come and go.
__global__ void __launch_bounds__(256) k_plane_step(const PlaneWorld* __restrict__ worlds,
                                                   const PlaneItem* __restrict__ items,
                                                   const int* __restrict__ n_items_p, int s_seg, int* counts) {
    const int n_items = *n_items_p;
    const int lane = threadIdx.x & 31;
    const int warps = (gridDim.x * blockDim.x) >> 5;
    for (int it = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; it < n_items; it += warps) {
        const PlaneItem item = items[it];
        const PlaneWorld& w = worlds[item.world];
        if (s_seg >= w.steps) continue;
        const uint64_t t = w.t + (uint64_t)s_seg;
        const int o = (int)(t & 1u);
        const int G = 1 << w.lg;
        const int gl = lane & (G - 1);
        const int rp = item.rp0 + (lane >> w.lg);
        const int nrp = nblocks(w.Y, o) * nblocks(w.Z, o);
        plane_rowpair(w, o, stepkey(w.seed, t), rp, rp < nrp, gl, G, item.world == 0 ? counts : nullptr);
    }
}

// One step of one large world (too large for the resident kernels), skipping
// settled row-pairs exactly.  Per row (y, z) one byte holds the low 8 bits of
// the last step that changed the row.  A block row-pair of phase o at step t
// is evaluated when one of its four rows changed at step t-1 or t-2 (age
// (t - flag) & 255 of 1 or 2; an older change that aliases to those ages only
// adds work).  Otherwise its cells are those it had when last evaluated (at
// t-2, same phase), which changed nothing, and whether a block can change
// depends on its own cells alone, so it would change nothing again.  Each
// row belongs to one row-pair per step, so the row-pair reads and writes its
// rows' bytes with no other reader in the step.  A fresh world starts with
// every byte at t0 - 1 (every row changed just before).  Warps take
// (32 >> lg) row-pairs each in order; a warp whose row-pairs are all settled
// loads nothing.
__device__ __forceinline__ bool rows_changed_recently(const uint8_t* __restrict__ rf, int Y, int Z, int y0, int z0,
                                                      uint32_t tb) {
    bool d = false;
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        const int y = y0 + (a >> 1), z = z0 + (a & 1);
        if (y >= 0 && y < Y && z >= 0 && z < Z) d |= ((tb - (uint32_t)rf[(int64_t)y * Z + z]) & 0xFFu) - 1u < 2u;
    }
    return d;
}

// three CTAs per SM (80 registers, a few bytes spilled): 24 warps hide the
// rule's dependent chain better than 16 at 118 registers (1024^3 dunes:
// 118 us per step against 133 us, 123 us at four CTAs)
__global__ void __launch_bounds__(256, 3) k_plane_step_skip(const PlaneWorld w, uint8_t* __restrict__ rflags,
                                                        int* counts) {
    const uint64_t t = w.t;
    const int o = (int)(t & 1u);
    const int lane = threadIdx.x & 31;
    const int G = 1 << w.lg, per = 32 >> w.lg, gl = lane & (G - 1);
    const int NBZ = nblocks(w.Z, o), nrp = nblocks(w.Y, o) * NBZ, n_items = (nrp + per - 1) / per;
    const uint32_t sk = stepkey(w.seed, t), tb = (uint32_t)t & 0xFFu;
    const uint32_t gmask = G == 32 ? 0xFFFFFFFFu : ((1u << G) - 1u) << (lane & ~(G - 1));
    const bool half_at_end = (w.X & 63) == 0;
    const int warps = (gridDim.x * blockDim.x) >> 5;
    for (int it = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; it < n_items; it += warps) {
        const int rp = it * per + (lane >> w.lg);
        const bool valid = rp < nrp;
        const int j = valid ? rp / NBZ : 0, k = valid ? rp - j * NBZ : 0;
        const int y0 = 2 * j - o, z0 = 2 * k - o;
        bool dirty = false;
        if (valid && gl == 0) dirty = rows_changed_recently(rflags, w.Y, w.Z, y0, z0, tb);
        dirty = __shfl_sync(0xFFFFFFFFu, dirty, lane & ~(G - 1));
        if (!__any_sync(0xFFFFFFFFu, dirty)) continue;
        const bool has = dirty && gl < w.nw;
        uint4 q[4], q0[4];
        uint4* ptr[4];
        bool in[4];
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            const int y = (a < 2) ? y0 + 1 : y0, z = z0 + (a & 1);
            in[a] = has && y >= 0 && y < w.Y && z >= 0 && z < w.Z;
            ptr[a] = in[a] ? w.rows + ((int64_t)y * w.Z + z) * w.nw + gl : w.rows;
            q[a] = in[a] ? *ptr[a] : make_uint4(0u, 0u, 0xFFFFFFFFu, 0xFFFFFFFFu);
            q0[a] = q[a];
        }
        rowpair_core(q, has, o, rowkey(sk, (uint32_t)j, (uint32_t)k), gl, G, w.nw, half_at_end);
        bool any = false;
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            const bool chg =
                in[a] && (q[a].x != q0[a].x || q[a].y != q0[a].y || q[a].z != q0[a].z || q[a].w != q0[a].w);
            if (chg) {
                *ptr[a] = q[a];
                any = true;
            }
            const uint32_t bal = __ballot_sync(0xFFFFFFFFu, chg);
            if (gl == 0 && (bal & gmask)) {
                const int y = (a < 2) ? y0 + 1 : y0, z = z0 + (a & 1);
                rflags[(int64_t)y * w.Z + z] = (uint8_t)tb;
            }
        }
        if (counts && any) count_bricks(counts, w, y0, z0, gl, q, q0, in);
    }
}

// ---------------------------------------------------------------------------
// change flags of a world with no history, from its cells
// ---------------------------------------------------------------------------
// A world admitted (or loaded, or written) at step t0 has no record of its
// last changes.  Marking every layer or row changed at t0 - 1 makes its first
// two steps evaluate every row-pair.  Instead a layer or row is marked changed
// at t0 - 1 only when a block row-pair of either phase that covers it can
// change (rowpair_can_change), and at t0 - 3 (two steps before the window the
// skip reads) otherwise.  Exact: at t0 and t0 + 1 a skipped pair has no block
// that can change and no row of it changed since t0 (at t0 + 1 a change at t0
// marks it); from t0 + 2 on the skip's usual argument holds, since a pair not
// evaluated at t0 could not change then.

// the four rows of block row-pair (j, k) of phase o for lane gl, solid outside the world
__device__ __forceinline__ void load_rowpair(const uint4* __restrict__ rows, int Y, int Z, int nw, int y0, int z0,
                                             int gl, bool has, uint4 (&q)[4]) {
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        const int y = (a < 2) ? y0 + 1 : y0, z = z0 + (a & 1);
        const bool in = has && y >= 0 && y < Y && z >= 0 && z < Z;
        q[a] = in ? rows[((int64_t)y * Z + z) * nw + gl] : make_uint4(0u, 0u, 0xFFFFFFFFu, 0xFFFFFFFFu);
    }
}

__device__ __forceinline__ int lanes_lg(int nw) { return nw <= 1 ? 0 : 32 - __clz(nw - 1); }

// One warp per layer y of each job (blockIdx.x: job, blockIdx.y * 8 + warp: y).
// `one` stands for the job table when jobs is null.
__global__ void __launch_bounds__(256) k_layer_flags_from_cells(const ConvJob* __restrict__ jobs, ConvJob one) {
    const ConvJob jb = jobs ? jobs[blockIdx.x] : one;
    const int y = (int)blockIdx.y * 8 + (int)(threadIdx.x >> 5);
    if (!jb.lflags || y >= jb.Y) return;  // warp-uniform
    const int lane = threadIdx.x & 31, lg = lanes_lg(jb.nw);
    const int G = 1 << lg, per = 32 >> lg, gl = lane & (G - 1), gi = lane >> lg;
    const bool half_at_end = (jb.X & 63) == 0;
    bool any = false;
    for (int o = 0; o < 2 && !any; ++o) {
        const int y0 = 2 * ((y + o) >> 1) - o;  // the pair of phase o covering y: layers y0, y0 + 1
        const int nbz = nblocks(jb.Z, o);
        for (int k0 = 0; k0 < nbz && !any; k0 += per) {
            const int k = k0 + gi;
            const bool has = k < nbz && gl < jb.nw;
            uint4 q[4];
            load_rowpair(jb.rows, jb.Y, jb.Z, jb.nw, y0, 2 * k - o, gl, has, q);
            any = __any_sync(0xFFFFFFFFu, rowpair_can_change(q, has, o, gl, G, jb.nw, half_at_end));
        }
    }
    if (lane == 0) jb.lflags[y] = (uint8_t)(jb.t0b - (any ? 1u : 3u));
}

// Row flags, already set to t0 - 3: every block row-pair of both phases that
// can change marks its rows changed at t0 - 1 (rows shared by two such pairs
// get the same value from both).
__global__ void __launch_bounds__(256) k_row_flags_from_cells(const uint4* __restrict__ rows,
                                                              uint8_t* __restrict__ rflags, int X, int Y, int Z,
                                                              int nw, uint32_t t0b) {
    const int lane = threadIdx.x & 31, lg = lanes_lg(nw);
    const int G = 1 << lg, per = 32 >> lg, gl = lane & (G - 1), gi = lane >> lg;
    const uint32_t gmask = G == 32 ? 0xFFFFFFFFu : ((1u << G) - 1u) << (lane & ~(G - 1));
    const bool half_at_end = (X & 63) == 0;
    const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int64_t first = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    for (int o = 0; o < 2; ++o) {
        const int nbz = nblocks(Z, o), chunks = (nbz + per - 1) / per;
        const int64_t items = (int64_t)nblocks(Y, o) * chunks;
        for (int64_t it = first; it < items; it += warps) {
            const int j = (int)(it / chunks), k = (int)(it - (int64_t)j * chunks) * per + gi;
            const int y0 = 2 * j - o, z0 = 2 * k - o;
            const bool has = k < nbz && gl < nw;
            uint4 q[4];
            load_rowpair(rows, Y, Z, nw, y0, z0, gl, has, q);
            const uint32_t m = __ballot_sync(0xFFFFFFFFu, rowpair_can_change(q, has, o, gl, G, nw, half_at_end));
            if (gl == 0 && k < nbz && (m & gmask)) {
#pragma unroll
                for (int a = 0; a < 4; ++a) {
                    const int y = (a < 2) ? y0 + 1 : y0, z = z0 + (a & 1);
                    if (y >= 0 && y < Y && z >= 0 && z < Z) rflags[(int64_t)y * Z + z] = (uint8_t)(t0b - 1u);
                }
            }
        }
    }
}

// ---------------------------------------------------------------------------
// shared-memory resident segment: one CTA steps one whole world
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Waits for the mbarrier phase for at most limit_ns nanoseconds of the global
// timer (try_wait itself may suspend for a while, so the bound is on time, not
// on tries); false if it gave up.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t phase, uint64_t limit_ns) {
    const uint64_t t0 = global_ns();
    for (uint32_t it = 0;; ++it) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(smem_u32(bar)), "r"(phase)
            : "memory");
        if (done) return true;
        if (it > 64) __nanosleep(64);
        if ((it & 63u) == 63u && global_ns() - t0 > limit_ns) return false;
    }
}

// The bulk-copy wait's limit: two seconds, far beyond any copy's time (one
// slab of at most a few hundred KB); 20 ms under the copy-stall test hook, so
// a test that makes every wait run out stays short.
constexpr uint64_t kCopyWaitNs = 2000000000ull, kCopyWaitInjectedNs = 20000000ull;

// Test hook (fs3d_test_inject): extra bytes every resident kernel announces
// on its mbarrier beyond what its bulk copy delivers.  With it set, the copy
// lands in full but the barrier's phase never completes, so each wait runs to
// its iteration limit and reports a timeout; nothing else changes.  0 in
// normal operation.
static __device__ uint32_t g_inject_tx_extra;

// TMA bulk copy global -> shared, completion counted in bytes on `bar`
// (`expect` = bytes, or more under the test hook above)
__device__ __forceinline__ void bulk_load(void* smem_dst, const void* gsrc, uint32_t bytes, uint32_t expect,
                                          uint64_t* bar) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(expect)
                 : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(smem_dst)),
                 "l"(gsrc), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

// TMA bulk copy shared -> global, waited for before the buffer is reused
__device__ __forceinline__ void bulk_store_wait(void* gdst, const void* smem_src, uint32_t bytes) {
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(gdst), "r"(smem_u32(smem_src)),
                 "r"(bytes)
                 : "memory");
    asm volatile("cp.async.bulk.commit_group;" ::: "memory");
    asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
}

// The rows of one world held in shared memory by the CTAs of a cluster: CTA
// r holds rows y in [lo_r, hi_r) (lo_r even), stored as ((y - lo_r)*Z + z)*nw
// + word, followed (at the next 16-byte boundary) by four change buffers of
// one byte per layer y (buffer t & 3: 1 if step t changed a row of the
// layer) and a list of up to (hi_r - lo_r)/2 + 2 16-bit layer-pair indices.
// Step t writes buffer t & 3, reads buffers (t-1) & 3 and (t-2) & 3 and
// clears buffer (t+1) & 3, so no buffer is both read and written in a step.
// `left` is the shared memory of CTA r-1 (null for r == 0): the only layer a
// CTA touches outside its slab is y = lo_r - 1, in the odd phase.
template <bool CL>
struct SlabView {
    uint4* mine;
    uint4* left;
    uint8_t* fmine;
    uint8_t* fleft;
    int lo, hi, left_lo, Z, nw;
    __device__ __forceinline__ uint4* at(int y, int z, int g) const {
        if (!CL || y >= lo) return mine + ((y - lo) * Z + z) * nw + g;
        return left + ((y - left_lo) * Z + z) * nw + g;
    }
    __device__ __forceinline__ uint8_t* flag(int y, uint32_t b) const {
        if (!CL || y >= lo) return fmine + b * flag_stride(hi - lo) + (y - lo);
        return fleft + b * flag_stride(lo - left_lo) + (y - left_lo);
    }
    __host__ __device__ static __forceinline__ uint32_t flag_stride(int layers) { return ((uint32_t)layers + 15u) & ~15u; }
};

// shared-memory bytes after a slab's planes: change buffers and the layer list
__host__ __device__ __forceinline__ uint32_t slab_aux_bytes(uint32_t layers) {
    return 4u * ((layers + 15u) & ~15u) + ((2u * (layers / 2u + 2u) + 15u) & ~15u);
}

// index of the n-th (from 0) set bit of m; m has more than n set bits
__device__ __forceinline__ int select_bit(uint32_t m, int n) {
    int pos = 0, c = __popc(m & 0xFFFFu);
    if (n >= c) { n -= c; m >>= 16; pos += 16; }
    c = __popc(m & 0xFFu);
    if (n >= c) { n -= c; m >>= 8; pos += 8; }
    c = __popc(m & 0xFu);
    if (n >= c) { n -= c; m >>= 4; pos += 4; }
    c = __popc(m & 0x3u);
    if (n >= c) { n -= c; m >>= 2; pos += 2; }
    return pos + (n >= (int)(m & 1u) ? 1 : 0);
}

// bytes of a slab's planes, rounded up so its change buffers start 16-byte aligned
__host__ __device__ __forceinline__ uint32_t slab_flag_offset(uint32_t plane_bytes) {
    return (plane_bytes + 15u) & ~15u;
}

// Whether the block row-pairs of layer pair j (all k) must be evaluated: a
// row of layer 2j - o or 2j - o + 1 changed in one of the two previous steps.
// Otherwise every pair's cells are those of its last evaluation in the same
// phase, two steps back, which changed nothing, and whether a block can
// change depends on its cells alone (the rule's activity mask), so it would
// change nothing again.  A world without kept flags starts with every layer
// changed at steps t0 - 1 and t0 - 2.
template <bool CL>
__device__ __forceinline__ bool layer_dirty(const SlabView<CL>& v, const PlaneWorld& w, int o, uint32_t tb, int j) {
    uint32_t dirty = 0;
#pragma unroll
    for (int a = 0; a < 2; ++a) {
        const int y = 2 * j - o + a;
        if (y >= 0 && y < w.Y) dirty |= (uint32_t)*v.flag(y, (tb + 3u) & 3u) | (uint32_t)*v.flag(y, (tb + 2u) & 3u);
    }
    return dirty != 0;
}

// Evaluates block row-pair (j, k) of a world held in shared memory when `run`
// is set.  Every lane of the warp calls this together (the odd phase passes
// carry bits between lanes).  Layers with a changed row get the step's flag.
template <bool CL>
__device__ __forceinline__ void slab_rowpair(const SlabView<CL>& v, const PlaneWorld& w, int o, uint32_t sk,
                                             uint32_t tt /* step & 3 */, int j, int k, bool run, int gl,
                                             int G) {
    if (!__any_sync(0xFFFFFFFFu, run)) return;
    const int y0 = 2 * j - o, z0 = 2 * k - o;
    const uint32_t rk = rowkey(sk, (uint32_t)j, (uint32_t)k);
    const bool has = run && gl < w.nw;
    uint4 q[4], q0[4];
    uint4* ptr[4];
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        const int y = (a < 2) ? y0 + 1 : y0, z = z0 + (a & 1);
        ptr[a] = (has && y >= 0 && y < w.Y && z >= 0 && z < w.Z) ? v.at(y, z, gl) : nullptr;
        q[a] = ptr[a] ? *ptr[a] : make_uint4(0u, 0u, 0xFFFFFFFFu, 0xFFFFFFFFu);
        q0[a] = q[a];
    }
    rowpair_core(q, has, o, rk, gl, G, w.nw, (w.X & 63) == 0);
#pragma unroll
    for (int a = 0; a < 4; ++a)
        if (ptr[a] && (q[a].x != q0[a].x || q[a].y != q0[a].y || q[a].z != q0[a].z || q[a].w != q0[a].w)) {
            *ptr[a] = q[a];
            *v.flag((a < 2) ? y0 + 1 : y0, tt) = 1u;
        }
}

// first row of slab r of CS slabs (even, so even-phase row-pairs never straddle)
__device__ __forceinline__ int slab_lo(int Y, int r, int CS) { return 2 * ((r * ((Y + 1) / 2)) / CS); }

// Persistent resident segment kernel.  A group of CS CTAs (a thread-block
// cluster when CS > 1) takes worlds of its class, largest first, from
// `counter`.  Each CTA loads its slab of the world's planes into shared
// memory with one TMA bulk copy, the group runs the world's segment steps
// (one CTA / cluster barrier per step: the next phase pairs different rows;
// the one row a CTA reads from its neighbour travels through distributed
// shared memory), and each CTA writes its slab back with one TMA bulk store.
// Worlds are independent, so groups never wait on one another.
// meta: [0] per-step items, [1 + c] resident worlds of class c, [1 + kAllClasses + c] their offset in order[].
// CTAs of each single-CTA class that share an SM (the register cap that lets
// them: 24 warps of at most 80 registers per SM)
template <int NT>
constexpr int resident_ctas_per_sm() {
    return NT == 128 ? 6 : (NT == 256 ? 3 : 1);
}

// GM: the world stays in global memory (L2) and the CTA keeps only the layer
// flags and list in shared memory, so as many worlds are in flight as warps
// allow; no bulk copies.  CTAs per SM of a GM kernel: kGmThreadsPerSm threads.
#ifndef FS3D_GM_THREADS_PER_SM
#define FS3D_GM_THREADS_PER_SM 768
#endif
constexpr int kGmThreadsPerSm = FS3D_GM_THREADS_PER_SM;
template <int NT, bool CL, bool GM = false>
__global__ void __launch_bounds__(NT, CL ? 1 : (GM ? kGmThreadsPerSm / NT : resident_ctas_per_sm<NT>()))
    k_plane_segment_resident(const PlaneWorld* __restrict__ worlds,
                                                             const int* __restrict__ order,
                                                             const int* __restrict__ meta, int cls, int CS,
                                                             int* counter, int* err,
                                                             unsigned long long* processed_cells) {
    extern __shared__ __align__(128) uint4 srows[];
    __shared__ __align__(8) uint64_t bar;
    __shared__ int item;
    namespace cg = cooperative_groups;
    const int n = meta[1 + cls], off = meta[1 + kAllClasses + cls];
    if (!CL) CS = 1;
    const int r = CL ? (int)cg::this_cluster().block_rank() : 0;
    auto group_sync = [&]() {
        if (CL)
            cg::this_cluster().sync();
        else
            __syncthreads();
    };
    if (threadIdx.x == 0) mbar_init(&bar, 1);
    __syncthreads();
    const uint32_t tx_extra = g_inject_tx_extra;
    uint32_t phase = 0;
    const int lane = threadIdx.x & 31;
    uint4* left = (CL && r > 0) ? cg::this_cluster().map_shared_rank(srows, r - 1) : nullptr;
    __shared__ unsigned long long s_processed;  // cell-steps evaluated (the rest were skipped as settled)
    __shared__ int s_count[2];                   // work-list length, by step parity
    constexpr int kKeys = 32;                    // step keys computed together, one per thread
    __shared__ uint32_t s_keys[kKeys];
    // per phase o: the world's block rows along z, and the multiplier that
    // divides by it (e / n = umulhi(e, m), exact for e, n < 2^16)
    __shared__ uint32_t s_nbz[2], s_magic[2];
    if (threadIdx.x == 0) {
        s_processed = 0;
        s_count[0] = s_count[1] = 0;
    }
    for (;;) {
        // after an error every group stops taking worlds (and all of a cluster stop together)
        if (r == 0 && threadIdx.x == 0) item = *(volatile int*)err ? n : atomicAdd(counter, 1);
        group_sync();
        const int it = CL ? *cg::this_cluster().map_shared_rank(&item, 0) : item;
        group_sync();
        if (it >= n) break;
        const PlaneWorld w = worlds[order[off + it]];
        if (w.steps <= 0) continue;
        SlabView<CL> v;
        v.lo = slab_lo(w.Y, r, CS);
        v.hi = r == CS - 1 ? w.Y : slab_lo(w.Y, r + 1, CS);
        v.left_lo = r > 0 ? slab_lo(w.Y, r - 1, CS) : 0;
        const uint32_t row_bytes = (uint32_t)w.Z * (uint32_t)w.nw * 16u;
        const uint32_t bytes = GM ? 0u : (uint32_t)(v.hi - v.lo) * row_bytes;  // bulk-copied bytes
        uint4* gslab = w.rows + (int64_t)v.lo * w.Z * w.nw;
        v.mine = GM ? gslab : srows;
        v.left = left;
        v.Z = w.Z;
        v.nw = w.nw;
        v.fmine = reinterpret_cast<uint8_t*>(srows) + slab_flag_offset(bytes);
        v.fleft = left ? reinterpret_cast<uint8_t*>(left) + slab_flag_offset((uint32_t)(v.lo - v.left_lo) * row_bytes)
                       : nullptr;
        if (threadIdx.x == 0 && bytes) bulk_load(srows, gslab, bytes, bytes + tx_extra, &bar);
        if (threadIdx.x < 2) {
            s_nbz[threadIdx.x] = (uint32_t)nblocks(w.Z, (int)threadIdx.x);
            s_magic[threadIdx.x] = 0xFFFFFFFFu / (uint32_t)nblocks(w.Z, (int)threadIdx.x) + 1u;
        }
        // change buffers from the kept flags (the low 8 bits of the last step
        // that changed the layer), or every layer changed at t0 - 1 and t0 - 2
        {
            const bool kept = w.lflags != nullptr && !w.lflags_fresh;
            const uint32_t t0b = (uint32_t)w.t & 3u, fs = SlabView<CL>::flag_stride(v.hi - v.lo);
            for (int i = threadIdx.x; i < v.hi - v.lo; i += NT) {
                const uint32_t age = kept ? (((uint32_t)w.t - (uint32_t)w.lflags[v.lo + i]) & 0xFFu) : 0u;
                v.fmine[((t0b + 3u) & 3u) * fs + i] = kept ? (age == 1u) : 1u;
                v.fmine[((t0b + 2u) & 3u) * fs + i] = kept ? (age == 2u) : 1u;
                v.fmine[t0b * fs + i] = 0u;
                v.fmine[((t0b + 1u) & 3u) * fs + i] = 0u;
            }
        }
        bool ok = true;
        if (bytes) {
            ok = mbar_wait(&bar, phase, tx_extra ? kCopyWaitInjectedNs : kCopyWaitNs);
            phase ^= 1u;
        }
        // A copy that never landed poisons the world: the error record is
        // set (err[0] = 1, err[2..3] = the world's step at the start of this
        // launch, by the first group to fail), this CTA still takes part in
        // every barrier of its group but touches no memory, and the group
        // stops before its next world.
        const bool poisoned = __syncthreads_or(!ok) != 0;
        if (poisoned && threadIdx.x == 0 && atomicCAS(err, 0, 1) == 0)
            *reinterpret_cast<unsigned long long*>(err + 2) = (unsigned long long)w.t;
        group_sync();  // every slab is loaded before a neighbour reads it
        const int G = 1 << w.lg, per = NT >> w.lg;
        const int gl = lane & (G - 1);
        // layer pairs to evaluate in a step (16-bit offsets from j_lo), after the buffers
        const uint32_t fs = SlabView<CL>::flag_stride(v.hi - v.lo);
        uint16_t* jlist = reinterpret_cast<uint16_t*>(v.fmine + 4u * fs);
        for (int s = 0; s < w.steps; ++s) {
            if ((s & (kKeys - 1)) == 0) {
                // the next kKeys steps' keys, one thread each (the previous step's
                // barrier is behind every reader of the last ones)
                for (int i = threadIdx.x; i < kKeys; i += NT)
                    if (s + i < w.steps) s_keys[i] = stepkey(w.seed, w.t + (uint64_t)(s + i));
                __syncthreads();
            }
            if (poisoned) {
                group_sync();
                continue;
            }
            const uint64_t t = w.t + (uint64_t)s;
            const int o = (int)(t & 1u);
            const uint32_t sk = s_keys[s & (kKeys - 1)];
            const int NBZ = (int)s_nbz[o];
            const int j_lo = v.lo / 2, j_hi = (r == CS - 1) ? nblocks(w.Y, o) : v.hi / 2;
            const int nj = j_hi - j_lo;
            const uint32_t tb = (uint32_t)t & 3u;
            // the buffer the next step writes: read and written by no one in this step
            for (int i = threadIdx.x; i < v.hi - v.lo; i += NT) v.fmine[((tb + 1u) & 3u) * fs + i] = 0u;
            // dirty layer pairs: up to 96 as bit masks every warp computes for
            // itself (the buffers it reads are not written in this step), more
            // through the shared list
            uint32_t dm0 = 0, dm1 = 0, dm2 = 0;
            int n_layers;
            const bool masked = nj <= 96;
            if (masked) {
                dm0 = __ballot_sync(0xFFFFFFFFu, lane < nj && layer_dirty(v, w, o, tb, j_lo + lane));
                if (nj > 32) dm1 = __ballot_sync(0xFFFFFFFFu, lane + 32 < nj && layer_dirty(v, w, o, tb, j_lo + 32 + lane));
                if (nj > 64) dm2 = __ballot_sync(0xFFFFFFFFu, lane + 64 < nj && layer_dirty(v, w, o, tb, j_lo + 64 + lane));
                n_layers = __popc(dm0) + __popc(dm1) + __popc(dm2);
            } else {
                int* cnt = &s_count[s & 1];
                for (int base = 0; base < nj; base += NT) {
                    const int i = base + (int)threadIdx.x;
                    const bool add = i < nj && layer_dirty(v, w, o, tb, j_lo + i);
                    const uint32_t m = __ballot_sync(0xFFFFFFFFu, add);
                    if (m) {
                        int pos = 0;
                        if (lane == __ffs(m) - 1) pos = atomicAdd(cnt, __popc(m));
                        pos = __shfl_sync(0xFFFFFFFFu, pos, __ffs(m) - 1) + __popc(m & ((1u << lane) - 1u));
                        if (add) jlist[pos] = (uint16_t)i;
                    }
                }
                __syncthreads();
                n_layers = *cnt;
            }
            if (threadIdx.x == 0) {
                s_count[(s + 1) & 1] = 0;  // the next step's counter (read before this step)
                // cells evaluated: the rows of every dirty layer pair inside the world, X*Z cells each
                int rows = 2 * n_layers;
                if (n_layers) {
                    if (2 * j_lo - o < 0 && layer_dirty(v, w, o, tb, j_lo)) --rows;
                    if (2 * (j_hi - 1) - o + 1 >= w.Y && layer_dirty(v, w, o, tb, j_hi - 1)) --rows;
                }
                s_processed += (unsigned long long)rows * (unsigned long long)(w.X * w.Z);
            }
            const int npairs = n_layers * NBZ;
            const uint32_t nbz_magic = s_magic[o];
            for (int base = 0; base < npairs; base += per) {
                const int e = base + (int)(threadIdx.x >> w.lg);
                const bool valid = e < npairs;
                const int jd =
                    valid ? (NBZ == 1 ? e : (npairs <= 65536 ? (int)__umulhi((uint32_t)e, nbz_magic) : e / NBZ)) : 0;
                const int kk = valid ? e - jd * NBZ : 0;
                int jj = 0;
                if (valid) {
                    if (!masked)
                        jj = (int)jlist[jd];
                    else if (jd == 0 && dm0)
                        jj = __ffs(dm0) - 1;
                    else if (jd < __popc(dm0))
                        jj = select_bit(dm0, jd);
                    else if (jd < __popc(dm0) + __popc(dm1))
                        jj = 32 + select_bit(dm1, jd - __popc(dm0));
                    else
                        jj = 64 + select_bit(dm2, jd - __popc(dm0) - __popc(dm1));
                }
                slab_rowpair(v, w, o, sk, tb, j_lo + jj, kk, valid, gl, G);
            }
            group_sync();
        }
        if (w.lflags && !poisoned) {
            // kept for the next segment: the last of the final two steps that changed the layer
            const uint64_t te = w.t + (uint64_t)w.steps;
            const uint32_t b1 = (uint32_t)(te - 1u) & 3u, b2 = (uint32_t)(te - 2u) & 3u;
            for (int i = threadIdx.x; i < v.hi - v.lo; i += NT)
                w.lflags[v.lo + i] = (uint8_t)(v.fmine[b1 * fs + i] ? te - 1u : (v.fmine[b2 * fs + i] ? te - 2u : te - 3u));
        }
        // make the threads' shared-memory writes visible to the bulk copy
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (threadIdx.x == 0 && bytes && !poisoned) bulk_store_wait(gslab, srows, bytes);
        group_sync();  // the slab is free again (and no neighbour still reads it)
    }
    __syncthreads();
    if (threadIdx.x == 0 && processed_cells && s_processed) atomicAdd(processed_cells, s_processed);
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
namespace {

struct ResidentCfg {
    int threads, ctas_per_sm, cs;
    int smem;  // dynamic shared memory per CTA (bytes), 0 = class unavailable
    const void* fn;
};

// filled once per process (the first device the library is used on), from any thread
ResidentCfg g_classes[kResidentClasses];
std::once_flag g_classes_once;

template <int NT, bool CL>
const void* resident_fn() {
    return reinterpret_cast<const void*>(&k_plane_segment_resident<NT, CL>);
}

void fill_classes() {
    int dev = 0, per_sm = 0, optin = 0, reserved = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev);
    const int kStatic = 256;  // the kernel's own shared variables, rounded up
    const ResidentCfg base[kResidentClasses] = {
        {128, resident_ctas_per_sm<128>(), 1, 0, resident_fn<128, false>()},
        {256, resident_ctas_per_sm<256>(), 1, 0, resident_fn<256, false>()},
        {768, resident_ctas_per_sm<768>(), 1, 0, resident_fn<768, false>()},
        {512, 1, 2, 0, resident_fn<512, true>()},
        {512, 1, 4, 0, resident_fn<512, true>()},
        {512, 1, 8, 0, resident_fn<512, true>()}};
    for (int c = 0; c < kResidentClasses; ++c) {
        ResidentCfg k = base[c];
        int stat = kStatic;
        cudaFuncAttributes fa;
        if (cudaFuncGetAttributes(&fa, k.fn) == cudaSuccess && (int)fa.sharedSizeBytes > stat)
            stat = ((int)fa.sharedSizeBytes + 127) & ~127;
        int smem = per_sm / k.ctas_per_sm - reserved - stat;
        if (smem > optin - stat) smem = optin - stat;
        smem = smem / 16 * 16;
        if (smem <= 0 || cudaFuncSetAttribute(k.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess)
            smem = 0;
        int fit = 0;
        if (smem && (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fit, k.fn, k.threads, smem) != cudaSuccess ||
                     fit < k.ctas_per_sm))
            smem = 0;
        k.smem = smem;
        g_classes[c] = k;
    }
    cudaGetLastError();  // a refused attribute leaves the class unused, not an error
}

void init_classes() { std::call_once(g_classes_once, fill_classes); }

}  // namespace

int resident_class(int X, int Y, int Z) {
    init_classes();
    const int64_t row_bytes = (int64_t)Z * plane_nw(X) * 16;
    for (int c = 0; c < kResidentClasses; ++c) {
        const ResidentCfg& k = g_classes[c];
        if (!k.smem) continue;
        // every slab holds at most 2*ceil(NYP/CS) rows (NYP = row pairs); each
        // slab must be non-empty so the row below a slab is in its neighbour
        const int64_t nyp = (Y + 1) / 2;
        const int64_t mx = k.cs == 1 ? Y : 2 * ((nyp + k.cs - 1) / k.cs);
        // planes, then the layer flags and the layer list
        const int64_t need = ((mx * row_bytes + 15) & ~(int64_t)15) + (int64_t)slab_aux_bytes((uint32_t)mx);
        if (need <= k.smem && (k.cs == 1 || nyp >= k.cs)) return c;
    }
    return -1;
}

// ---- global-memory segment classes: one CTA per world; the planes stay in
// global memory (L2-resident for a batch of a few hundred MB) and shared
// memory holds only the change buffers and the layer list.  A step's work is
// the dirty layer pairs (a few per step: the moving surface), each of
// ceil(Z/2) block row-pairs times the lanes per pair, so the CTA is sized by
// that layer work, not by the world's volume: idle warps would wait at every
// step's barrier.  Each class caps the layers it holds flags for so that its
// CTAs per SM (24 warps in all) fit in shared memory.
namespace {
constexpr int kGmThreads[kGmClasses] = {32, 64, 128, 256, 768};
constexpr int kGmMaxY[kGmClasses] = {1024, 1024, 2048, 4096, 4096};
std::once_flag g_gm_once;
}  // namespace

int resident_class_gm(int X, int Y, int Z) {
    const int lanes = nblocks(Z, 1) << plane_lg(plane_nw(X));  // lane tasks of one layer pair
    int c = lanes <= 16 ? 0 : (lanes <= 48 ? 1 : (lanes <= 96 ? 2 : 3));
    while (c < kGmDense && Y > kGmMaxY[c]) ++c;
    return c < kGmDense ? c : -1;
}

template <int NT>
static cudaError_t launch_gm(int cls, int grid, size_t smem, cudaStream_t st, const PlaneWorld* worlds,
                             const int* order, const int* meta, int* counter, int* err,
                             unsigned long long* processed_cells, bool first) {
    cudaLaunchConfig_t lc = {};
    lc.gridDim = dim3((unsigned)grid);
    lc.blockDim = dim3((unsigned)NT);
    lc.dynamicSmemBytes = smem;
    lc.stream = st;
    cudaLaunchAttribute attr[1];
    if (first) {
        // the greatest priority: its CTAs take the SMs before the other
        // classes' grids, which are pending at the same moment in a segment graph
        static const int greatest = [] {
            int least = 0, g = 0;
            if (cudaDeviceGetStreamPriorityRange(&least, &g) != cudaSuccess) g = 0;
            return g;
        }();
        attr[0].id = cudaLaunchAttributePriority;
        attr[0].val.priority = greatest;
    }
    lc.attrs = attr;
    lc.numAttrs = first ? 1 : 0;
    return cudaLaunchKernelEx(&lc, k_plane_segment_resident<NT, false, true>, worlds, order, meta,
                              kResidentClasses + cls, 1, counter, err, processed_cells);
}

fs3d_status launch_plane_segment_gm(int cls, const PlaneWorld* worlds, const int* order, const int* meta,
                                    int* counter, int* err, cudaStream_t st, unsigned long long* processed_cells,
                                    bool first) {
    if (cls < 0 || cls >= kGmClasses) return set_error(FS3D_ERR_INVALID_ARG, "global-memory class out of range");
    std::call_once(g_gm_once, [] {
        // the planes are read through L1: leave most of the unified memory to it
        const void* fns[kGmClasses] = {reinterpret_cast<const void*>(&k_plane_segment_resident<32, false, true>),
                                       reinterpret_cast<const void*>(&k_plane_segment_resident<64, false, true>),
                                       reinterpret_cast<const void*>(&k_plane_segment_resident<128, false, true>),
                                       reinterpret_cast<const void*>(&k_plane_segment_resident<256, false, true>),
                                       reinterpret_cast<const void*>(&k_plane_segment_resident<768, false, true>)};
        for (const void* fn : fns) cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, 50);
        cudaGetLastError();
    });
    FS3D_CUDA(cudaMemsetAsync(counter, 0, sizeof(int), st));
    const int nt = kGmThreads[cls];
    const int grid = sm_count_public() * (kGmThreadsPerSm / nt);
    const size_t smem = slab_aux_bytes((uint32_t)kGmMaxY[cls]);
    cudaError_t e;
    if (nt == 32)
        e = launch_gm<32>(cls, grid, smem, st, worlds, order, meta, counter, err, processed_cells, first);
    else if (nt == 64)
        e = launch_gm<64>(cls, grid, smem, st, worlds, order, meta, counter, err, processed_cells, first);
    else if (nt == 128)
        e = launch_gm<128>(cls, grid, smem, st, worlds, order, meta, counter, err, processed_cells, first);
    else if (nt == 256)
        e = launch_gm<256>(cls, grid, smem, st, worlds, order, meta, counter, err, processed_cells, first);
    else
        e = launch_gm<768>(cls, grid, smem, st, worlds, order, meta, counter, err, processed_cells, first);
    if (e != cudaSuccess) return cuda_fail(e, "global-memory segment launch");
    note_launch();
    return FS3D_OK;
}

fs3d_status set_inject_tx_extra(uint32_t bytes) {
    FS3D_CUDA(cudaMemcpyToSymbol(g_inject_tx_extra, &bytes, sizeof(bytes)));
    return FS3D_OK;
}

int smem_world_limit() {
    init_classes();
    return g_classes[2].smem;
}

fs3d_status launch_plane_segment_resident(int cls, const PlaneWorld* worlds, const int* order, const int* meta,
                                          int* counter, int* err, cudaStream_t st,
                                          unsigned long long* processed_cells) {
    init_classes();
    const ResidentCfg& k = g_classes[cls];
    if (!k.smem) return set_error(FS3D_ERR_CUDA, "resident segment kernel unavailable for this class");
    FS3D_CUDA(cudaMemsetAsync(counter, 0, sizeof(int), st));
    const int groups = sm_count_public() * k.ctas_per_sm / k.cs;
    cudaLaunchConfig_t lc = {};
    lc.gridDim = dim3((unsigned)(groups * k.cs));
    lc.blockDim = dim3((unsigned)k.threads);
    lc.dynamicSmemBytes = (size_t)k.smem;
    lc.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)k.cs;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    lc.attrs = attr;
    lc.numAttrs = k.cs > 1 ? 1 : 0;
    const int CS = k.cs;
    cudaError_t e;
    if (k.cs > 1)
        e = cudaLaunchKernelEx(&lc, k_plane_segment_resident<512, true>, worlds, order, meta, cls, CS, counter, err,
                               processed_cells);
    else if (k.threads == 128)
        e = cudaLaunchKernelEx(&lc, k_plane_segment_resident<128, false>, worlds, order, meta, cls, CS, counter, err,
                               processed_cells);
    else if (k.threads == 256)
        e = cudaLaunchKernelEx(&lc, k_plane_segment_resident<256, false>, worlds, order, meta, cls, CS, counter, err,
                               processed_cells);
    else
        e = cudaLaunchKernelEx(&lc, k_plane_segment_resident<768, false>, worlds, order, meta, cls, CS, counter, err,
                               processed_cells);
    if (e != cudaSuccess) return cuda_fail(e, "resident segment launch");
    note_launch();
    return FS3D_OK;
}

int sm_count_public();

static int conv_grid(int64_t n) {
    const int64_t need = (n + 255) / 256, cap = (int64_t)sm_count_public() * 8;
    return (int)(need < 1 ? 1 : (need < cap ? need : cap));
}

int plane_lg(int nw) {
    int lg = 0;
    while ((1 << lg) < nw) ++lg;
    return lg;
}

int plane_items_for(int Y, int Z, int nw) {
    const int per = 32 >> plane_lg(nw);
    const int nrp = nblocks(Y, 1) * nblocks(Z, 1);
    return (nrp + per - 1) / per;
}

fs3d_status planes_from_bytes(const uint8_t* g, int X, int Y, int Z, uint4* rows, cudaStream_t st) {
    const int nw = plane_nw(X);
    k_bytes_to_planes<<<conv_grid((int64_t)Y * Z * nw), 256, 0, st>>>(g, X, Y, Z, nw, rows);
    FS3D_CHECK_LAUNCH("bytes->planes launch");
    return FS3D_OK;
}

fs3d_status planes_from_bytes_multi(const ConvJob* jobs, const int64_t* unit_off, const int* block_job, int njobs,
                                    int64_t total_units, const uint8_t* staging, int* flags, cudaStream_t st) {
    if (njobs <= 0 || total_units <= 0) return FS3D_OK;
    k_bytes_to_planes_multi<<<conv_grid(total_units), kConvBlock, 0, st>>>(jobs, unit_off, block_job, njobs,
                                                                            total_units, staging, flags);
    FS3D_CHECK_LAUNCH("bytes->planes (many worlds) launch");
    return FS3D_OK;
}

// Each warp moves 2 KB blocks: lane l takes the 16-byte chunks 32i + l of its
// block (contiguous 512 bytes per instruction), all four loads before the
// stores; one job search per block (a block spans at most a few jobs).
__global__ void k_copy_many(const CopyJob* __restrict__ jobs, const int64_t* __restrict__ chunk_off, int njobs,
                            int64_t total) {
    const int lane = threadIdx.x & 31;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t blk = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; blk * 128 < total; blk += nwarps) {
        int j = find_job(chunk_off, njobs, blk * 128);
        const uint8_t* src[4];
        uint8_t* dst[4];
        int n[4];
        uint4 v[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int64_t u = blk * 128 + 32 * i + lane;
            n[i] = 0;
            if (u >= total) continue;
            while (j + 1 < njobs && __ldg(chunk_off + j + 1) <= u) ++j;
            const CopyJob& jb = jobs[j];
            const int64_t off = (u - __ldg(chunk_off + j)) * 16;
            n[i] = (int)(jb.bytes - off < 16 ? jb.bytes - off : 16);
            src[i] = jb.src + off;
            dst[i] = jb.dst + off;
            if (n[i] == 16 && ((reinterpret_cast<uintptr_t>(src[i]) | reinterpret_cast<uintptr_t>(dst[i])) & 15u) == 0)
                v[i] = *reinterpret_cast<const uint4*>(src[i]);
        }
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            if (!n[i]) continue;
            if (n[i] == 16 && ((reinterpret_cast<uintptr_t>(src[i]) | reinterpret_cast<uintptr_t>(dst[i])) & 15u) == 0)
                *reinterpret_cast<uint4*>(dst[i]) = v[i];
            else
                for (int k = 0; k < n[i]; ++k) dst[i][k] = src[i][k];
        }
    }
}

// A small copy done by the SMs (16-byte pieces, then the last bytes one by
// one): either side may be page-locked host memory the device can address.
__global__ void k_copy_small(const uint8_t* __restrict__ src, uint8_t* __restrict__ dst, size_t bytes) {
    const size_t n16 = bytes / 16;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n16; i += (size_t)gridDim.x * blockDim.x)
        reinterpret_cast<uint4*>(dst)[i] = reinterpret_cast<const uint4*>(src)[i];
    if (blockIdx.x == 0 && threadIdx.x == 0)
        for (size_t i = n16 * 16; i < bytes; ++i) dst[i] = src[i];
}

cudaError_t copy_small_async(void* dst, const void* src, size_t bytes, cudaStream_t st) {
    if (bytes == 0) return cudaSuccess;
    if (((reinterpret_cast<uintptr_t>(dst) | reinterpret_cast<uintptr_t>(src)) & 15u) != 0)
        return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, st);
    const size_t n16 = bytes / 16;
    const int64_t need = (int64_t)((n16 + 255) / 256), cap = (int64_t)sm_count_public() * 2;
    const int grid = (int)(need < 1 ? 1 : (need < cap ? need : cap));
    k_copy_small<<<grid, 256, 0, st>>>(static_cast<const uint8_t*>(src), static_cast<uint8_t*>(dst), bytes);
    const cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) note_launch();
    return e;
}

fs3d_status copy_many(const CopyJob* jobs, const int64_t* chunk_off, int njobs, int64_t total_chunks,
                      cudaStream_t st) {
    if (njobs <= 0 || total_chunks <= 0) return FS3D_OK;
    const int64_t blocks_needed = (total_chunks + 128 * 8 - 1) / (128 * 8), cap = (int64_t)sm_count_public() * 8;
    const int grid = (int)(blocks_needed < cap ? blocks_needed : cap);
    k_copy_many<<<grid < 1 ? 1 : grid, 256, 0, st>>>(jobs, chunk_off, njobs, total_chunks);
    FS3D_CHECK_LAUNCH("many-copy launch");
    return FS3D_OK;
}

uint8_t* device_view(const void* p) {
    cudaPointerAttributes a{};
    if (!p || cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged)
        return static_cast<uint8_t*>(const_cast<void*>(p));
    if (a.type == cudaMemoryTypeHost && a.devicePointer) return static_cast<uint8_t*>(a.devicePointer);
    return nullptr;
}

bool alloc_range(const void* p, uintptr_t* start, size_t* bytes) {
    // cuPointerGetAttributes, looked up once through the runtime (no link
    // dependency on the driver library)
    using GetAttrs = int (*)(unsigned int, int*, void**, unsigned long long);
    static GetAttrs fn = [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuPointerGetAttributes", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            f = nullptr;
        cudaGetLastError();
        return reinterpret_cast<GetAttrs>(f);
    }();
    if (!fn || !p) return false;
    unsigned long long base = 0, size = 0;
    int attrs[2] = {11, 12};  // CU_POINTER_ATTRIBUTE_RANGE_START_ADDR, CU_POINTER_ATTRIBUTE_RANGE_SIZE
    void* data[2] = {&base, &size};
    if (fn(2, attrs, data, (unsigned long long)reinterpret_cast<uintptr_t>(p)) != 0 || size == 0) return false;
    if (reinterpret_cast<uintptr_t>(p) < base || reinterpret_cast<uintptr_t>(p) >= base + size) return false;
    *start = (uintptr_t)base;
    *bytes = (size_t)size;
    return true;
}

fs3d_status planes_to_bytes_multi(const ConvJob* jobs, const int64_t* unit_off, const int* block_job, int njobs,
                                  int64_t total_units, uint8_t* staging, cudaStream_t st) {
    if (njobs <= 0 || total_units <= 0) return FS3D_OK;
    k_planes_to_bytes_multi<<<conv_grid(total_units), kConvBlock, 0, st>>>(jobs, unit_off, block_job, njobs,
                                                                            total_units, staging);
    FS3D_CHECK_LAUNCH("planes->bytes (many worlds) launch");
    return FS3D_OK;
}

fs3d_status planes_generate_batch_world(uint64_t world_seed, int X, int Y, int Z, uint4* rows, cudaStream_t st) {
    const int nw = plane_nw(X);
    k_gen_batch_planes<<<conv_grid((int64_t)Y * Z * nw), 256, 0, st>>>(X, Y, Z, nw, batch_world_gen(world_seed),
                                                                       rows);
    FS3D_CHECK_LAUNCH("generate batch world launch");
    return FS3D_OK;
}

fs3d_status planes_to_bytes(const uint4* rows, const uint8_t* statics, int X, int Y, int Z, uint8_t* g,
                            cudaStream_t st, const int* skip_if_set) {
    const int nw = plane_nw(X);
    k_planes_to_bytes<<<conv_grid((int64_t)Y * Z * nw), 256, 0, st>>>(rows, statics, X, Y, Z, nw, g, skip_if_set);
    FS3D_CHECK_LAUNCH("planes->bytes launch");
    return FS3D_OK;
}

fs3d_status planes_hash_async(const uint4* rows, const uint8_t* statics, int X, int Y, int Z,
                              unsigned long long* out_dev, cudaStream_t st) {
    const int nw = plane_nw(X);
    FS3D_CUDA(cudaMemsetAsync(out_dev, 0, sizeof(unsigned long long), st));
    k_hash_planes<<<conv_grid((int64_t)Y * Z * nw), 256, 0, st>>>(rows, statics, X, Y, Z, nw, out_dev);
    FS3D_CHECK_LAUNCH("hash planes launch");
    return FS3D_OK;
}

fs3d_status planes_hash_many(const HashJob* jobs, int njobs, unsigned long long* out_dev, cudaStream_t st) {
    if (njobs <= 0) return FS3D_OK;
    k_hash_planes_many<<<njobs, 256, 0, st>>>(jobs, out_dev);
    FS3D_CHECK_LAUNCH("hash many worlds launch");
    return FS3D_OK;
}

fs3d_status launch_plane_step(const PlaneWorld* worlds, const PlaneItem* items, const int* n_items_dev,
                              int grid, int s_seg, cudaStream_t st, int* brick_counts) {
    k_plane_step<<<grid, 256, 0, st>>>(worlds, items, n_items_dev, s_seg, brick_counts);
    FS3D_CHECK_LAUNCH("plane step launch");
    return FS3D_OK;
}

__global__ void k_advance_worlds(PlaneWorld* __restrict__ worlds, const int* __restrict__ meta) {
    const int n = meta[kMetaWorlds];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        PlaneWorld& w = worlds[i];
        w.t += (uint64_t)w.steps;
        if (w.lflags) w.lflags_fresh = 0;
    }
}

fs3d_status launch_advance_worlds(PlaneWorld* worlds, const int* meta, cudaStream_t st) {
    k_advance_worlds<<<8, 256, 0, st>>>(worlds, meta);
    FS3D_CHECK_LAUNCH("advance worlds launch");
    return FS3D_OK;
}

fs3d_status init_row_flags(const uint4* rows, uint8_t* rflags, int X, int Y, int Z, uint64_t t0, cudaStream_t st) {
    FS3D_CUDA(cudaMemsetAsync(rflags, (int)((t0 - 3u) & 0xFFu), (size_t)Y * (size_t)Z, st));
    const int nw = plane_nw(X), per = 32 >> plane_lg(nw);
    const int64_t items = (int64_t)nblocks(Y, 0) * ((nblocks(Z, 0) + per - 1) / per);  // the larger phase's
    const int64_t blocks = std::min<int64_t>((items + 7) / 8, (int64_t)sm_count_public() * 8);
    k_row_flags_from_cells<<<(unsigned)std::max<int64_t>(blocks, 1), 256, 0, st>>>(rows, rflags, X, Y, Z, nw,
                                                                                   (uint32_t)t0 & 0xFFu);
    FS3D_CUDA(cudaGetLastError());
    note_launch();
    return FS3D_OK;
}

fs3d_status layer_flags_from_cells_multi(const ConvJob* jobs, int njobs, int max_Y, cudaStream_t st) {
    if (njobs <= 0 || max_Y <= 0) return FS3D_OK;
    k_layer_flags_from_cells<<<dim3((unsigned)njobs, (unsigned)((max_Y + 7) / 8)), 256, 0, st>>>(jobs, ConvJob{});
    FS3D_CUDA(cudaGetLastError());
    note_launch();
    return FS3D_OK;
}

fs3d_status layer_flags_from_cells(const uint4* rows, uint8_t* lflags, int X, int Y, int Z, uint64_t t0,
                                   cudaStream_t st) {
    ConvJob one{};
    one.rows = const_cast<uint4*>(rows);
    one.X = X;
    one.Y = Y;
    one.Z = Z;
    one.nw = plane_nw(X);
    one.lflags = lflags;
    one.t0b = (uint32_t)t0 & 0xFFu;
    k_layer_flags_from_cells<<<dim3(1u, (unsigned)((Y + 7) / 8)), 256, 0, st>>>(nullptr, one);
    FS3D_CUDA(cudaGetLastError());
    note_launch();
    return FS3D_OK;
}

fs3d_status launch_plane_step_skip(const PlaneWorld& w, uint8_t* rflags, int* counts, cudaStream_t st) {
    static const int per_sm = [] {
        int v = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, k_plane_step_skip, 256, 0) != cudaSuccess || v < 1) v = 1;
        cudaGetLastError();
        return v;
    }();
    const int per = 32 >> w.lg;
    const int64_t nrp = (int64_t)nblocks(w.Y, 1) * nblocks(w.Z, 1);
    const int64_t need = ((nrp + per - 1) / per + 7) / 8;  // eight warps per CTA
    const int64_t cap = (int64_t)sm_count_public() * per_sm;
    const int grid = (int)(need < 1 ? 1 : (need < cap ? need : cap));
    k_plane_step_skip<<<grid, 256, 0, st>>>(w, rflags, counts);
    FS3D_CHECK_LAUNCH("plane step (settled skip) launch");
    return FS3D_OK;
}

// CTAs of the step kernel that fit on one SM at once
int plane_step_ctas_per_sm() {
    static const int n = [] {
        int v = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, k_plane_step, 256, 0) != cudaSuccess || v < 1) v = 1;
        return v;
    }();
    return n;
}

// persistent grid: every CTA resident, so warps pick items without tail waves
int plane_step_grid(int64_t n_items) {
    const int64_t warps_per_cta = 8;
    const int64_t need = (n_items + warps_per_cta - 1) / warps_per_cta;
    const int64_t cap = (int64_t)sm_count_public() * plane_step_ctas_per_sm();
    return (int)(need < 1 ? 1 : (need < cap ? need : cap));
}

}  // namespace fs3d
