// Per-step kernel for one large world in the bit-plane layout (too large for
// the shared-memory resident kernels): TMA tensor tiles, a producer warp, and
// an exact skip of settled tiles.
//
// Tile.  A tile is one layer pair j (block row-pairs (j, k) of the step's
// phase o) times KT consecutive k, all words of every row: the box
// {x: all nw words, z: TZ = 2*KT rows from 2*k0 - o, y: the 2 rows from
// 2*j - o} of the planes viewed as a 3-D tensor (x in 32-bit elements, z, y).
// One cp.async.bulk.tensor load brings it into shared memory; rows outside
// the world arrive zero-filled and are treated as solid by the rule, which
// never reads them.  The x coordinate is always 0, so every load starts on a
// 16-byte boundary.
//
// Pipeline.  Each CTA holds kTiledStages tile buffers.  Its producer warp
// walks the CTA's tiles (every gridDim.x-th tile), decides for 32 tiles at a
// time which of them can change, and issues the loads of those into the ring
// (full barrier: the bytes landed; empty barrier: the kTiledWarps consumer
// warps are done with the buffer).  Consumer warps run the bit-sliced rule on
// their row-pairs of the tile straight from shared memory and store only the
// changed words to global memory.
//
// Exact skip.  Per row (y, z) and step t, one bit records whether the step
// changed the row: four rotating buffers of Y x ceil(Z/32) words; step t sets
// bits in buffer t&3, reads (t-1)&3 and (t-2)&3, and clears (t+1)&3, so no
// buffer is read and written in one step.  A block of phase o at step t whose
// cells did not change in steps t-1 and t-2 holds the cells it had when it
// was last evaluated (at t-2, same phase), which changed nothing; whether a
// block can change depends on its own cells only, so it changes nothing
// again.  A tile is evaluated when any row of its two layers in its z range
// changed in t-1 or t-2 (whole flag words: a superset, still exact).  Changed
// rows are gathered per tile in shared memory and written with one atomicOr
// per flag word.  A world without valid flags starts with every row changed
// at t0-1 and t0-2.
//
// Bounded waits.  Every mbarrier wait gives up after a time limit; the CTA
// then records the error (err[0] = 1, err[2..3] = the step) and stops.  Tiles
// already stored stay stored, so after such a failure the planes hold a
// partly stepped state; launches given a set record do nothing.
#include <cuda.h>
#include <stdint.h>
#include <string.h>

#include <mutex>

#include "fs3d_common.h"
#include "planes.h"
#include "rule_device.cuh"
#include "bricks_device.cuh"

namespace fs3d {

namespace {

constexpr int kTiledWarps = 8;                        // consumer warps per CTA
constexpr int kTiledThreads = 32 * (kTiledWarps + 1);  // + one producer warp
constexpr int kTiledStages = 3;
constexpr int kTileMaskWords = 8;  // changed-row bits per layer of a tile (TZ <= 256)
constexpr uint64_t kTileWaitNs = 2000000000ull, kTileWaitInjectedNs = 20000000ull;

struct TiledArgs {
    PlaneWorld w;      // rows, seed, t = this step, X, Y, Z, nw, lg
    uint32_t* flags;   // 4 buffers of Y * zw words
    int zw;            // flag words per row of z: ceil(Z / 32)
    int KT, TZ;        // row-pairs and z rows per tile
    int* counts;       // nullable: per-brick counts of non-empty cells
    uint32_t tx_extra; // test hook: bytes announced beyond each tile's load
};

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t now_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void bar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void bar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

// waits for the phase of parity `parity` for at most limit_ns; false if it gave up
__device__ __forceinline__ bool bar_wait(uint64_t* bar, uint32_t parity, uint64_t limit_ns) {
    const uint64_t t0 = now_ns();
    for (uint32_t it = 0;; ++it) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(smem_addr(bar)), "r"(parity)
            : "memory");
        if (done) return true;
        if (it > 16) __nanosleep(32);
        if ((it & 63u) == 63u && now_ns() - t0 > limit_ns) return false;
    }
}

// the tile at tensor coordinates (0, z, y) into shared memory, completion on `bar`
__device__ __forceinline__ void tile_load(void* dst, const CUtensorMap* tm, int z, int y, uint64_t* bar,
                                          uint32_t expect) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(expect)
                 : "memory");
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(smem_addr(dst)),
        "l"(reinterpret_cast<uint64_t>(tm)), "r"(0), "r"(z), "r"(y), "r"(smem_addr(bar))
        : "memory");
}

__device__ __forceinline__ void record_error(int* err, uint64_t t) {
    if (atomicCAS(err, 0, 1) == 0) *reinterpret_cast<unsigned long long*>(err + 2) = (unsigned long long)t;
}

// Whether tile (j, kt) may change at step t: a row of its two layers in its z
// range changed at t-1 or t-2 (flag words read whole).
__device__ __forceinline__ bool tile_dirty(const TiledArgs& p, int o, uint32_t b1, uint32_t b2, int j, int kt) {
    const int zs = 2 * kt * p.KT - o;
    const int zlo = zs < 0 ? 0 : zs, zhi = (zs + p.TZ < p.w.Z ? zs + p.TZ : p.w.Z) - 1;
    const int wlo = zlo >> 5, whi = zhi >> 5;
    const size_t fbuf = (size_t)p.w.Y * p.zw;
    for (int ly = 0; ly < 2; ++ly) {
        const int y = 2 * j - o + ly;
        if (y < 0 || y >= p.w.Y) continue;
        const uint32_t* f1 = p.flags + b1 * fbuf + (size_t)y * p.zw;
        const uint32_t* f2 = p.flags + b2 * fbuf + (size_t)y * p.zw;
        for (int wi = wlo; wi <= whi; ++wi)
            if (__ldcg(f1 + wi) | __ldcg(f2 + wi)) return true;
    }
    return false;
}

__global__ void __launch_bounds__(kTiledThreads, 2)
    k_plane_step_tiled(const __grid_constant__ CUtensorMap tmap, const TiledArgs p, int* err) {
    extern __shared__ uint8_t sraw[];
    __shared__ __align__(8) uint64_t full_bar[kTiledStages], empty_bar[kTiledStages];
    __shared__ int tile_id[kTiledStages], done_cnt[kTiledStages];
    __shared__ uint32_t masks[kTiledStages][2][kTileMaskWords];
    __shared__ int abort_flag;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const PlaneWorld& w = p.w;
    const uint32_t stage_bytes = 2u * (uint32_t)p.TZ * (uint32_t)w.nw * 16u;
    uint8_t* sbase = sraw + ((1024u - (smem_addr(sraw) & 1023u)) & 1023u);
    if (threadIdx.x == 0) {
        for (int s = 0; s < kTiledStages; ++s) {
            bar_init(&full_bar[s], 1);
            bar_init(&empty_bar[s], kTiledWarps);
            tile_id[s] = -1;
            done_cnt[s] = 0;
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        abort_flag = *(volatile int*)err;  // a failed earlier launch: step nothing
    }
    for (int i = threadIdx.x; i < kTiledStages * 2 * kTileMaskWords; i += blockDim.x) (&masks[0][0][0])[i] = 0u;
    __syncthreads();
    if (abort_flag) return;
    const uint64_t t = w.t;
    const int o = (int)(t & 1u);
    const int NBY = nblocks(w.Y, o), NBZ = nblocks(w.Z, o);
    const int ntz = (NBZ + p.KT - 1) / p.KT;  // tiles per layer pair
    const int ntiles = NBY * ntz;
    const uint32_t b_cur = (uint32_t)t & 3u, b_next = (b_cur + 1u) & 3u, b1 = (b_cur + 3u) & 3u,
                   b2 = (b_cur + 2u) & 3u;
    const size_t fbuf = (size_t)w.Y * p.zw;
    const uint64_t limit = p.tx_extra ? kTileWaitInjectedNs : kTileWaitNs;

    if (warp == kTiledWarps) {
        // ---- producer
        // the next step's flag buffer is read and written by no one in this step
        for (size_t i = (size_t)blockIdx.x * 32 + lane; i < fbuf; i += (size_t)gridDim.x * 32)
            p.flags[b_next * fbuf + i] = 0u;
        int issued = 0;
        bool stop = false;
        for (int base = blockIdx.x; base < ntiles && !stop; base += 32 * gridDim.x) {
            const int tl = base + lane * gridDim.x;
            const bool d = tl < ntiles && tile_dirty(p, o, b1, b2, tl / ntz, tl % ntz);
            uint32_t m = __ballot_sync(0xFFFFFFFFu, d);
            while (m && !stop) {
                const int b = __ffs(m) - 1;
                m &= m - 1u;
                const int tile = base + b * gridDim.x;
                const int s = issued % kTiledStages;
                int ok = 1;
                if (lane == 0) {
                    if (issued >= kTiledStages)
                        ok = bar_wait(&empty_bar[s], (uint32_t)((issued / kTiledStages) - 1) & 1u, limit);
                    if (ok) {
                        tile_id[s] = tile;
                        const int j = tile / ntz, kt = tile - j * ntz;
                        tile_load(sbase + (size_t)s * stage_bytes, &tmap, 2 * kt * p.KT - o, 2 * j - o, &full_bar[s],
                                  stage_bytes + p.tx_extra);
                    } else {
                        record_error(err, t);
                        abort_flag = 1;
                    }
                }
                stop = __shfl_sync(0xFFFFFFFFu, ok, 0) == 0;
                ++issued;
            }
        }
        if (lane == 0 && !stop) {
            // the end of the tile list: a plain arrival with tile -1 stops the consumers
            const int s = issued % kTiledStages;
            const bool ok =
                issued < kTiledStages || bar_wait(&empty_bar[s], (uint32_t)((issued / kTiledStages) - 1) & 1u, limit);
            if (ok) {
                tile_id[s] = -1;
                bar_arrive(&full_bar[s]);
            } else {
                record_error(err, t);
                abort_flag = 1;
            }
        }
        return;
    }

    // ---- consumers
    const uint32_t sk = stepkey(w.seed, t);
    const int G = 1 << w.lg, per = 32 >> w.lg;
    const int gl = lane & (G - 1);
    const uint32_t gmask = G == 32 ? 0xFFFFFFFFu : ((1u << G) - 1u) << (lane & ~(G - 1));
    const bool half_at_end = (w.X & 63) == 0;
    for (int it = 0;; ++it) {
        const int s = it % kTiledStages;
        int ok = 1;
        if (lane == 0) ok = bar_wait(&full_bar[s], (uint32_t)(it / kTiledStages) & 1u, limit);
        ok = __shfl_sync(0xFFFFFFFFu, ok, 0);
        if (!ok) {
            if (lane == 0) {
                record_error(err, t);
                abort_flag = 1;
            }
            break;
        }
        const int tile = *(volatile int*)&tile_id[s];
        if (tile < 0 || *(volatile int*)&abort_flag) break;
        const int j = tile / ntz, kt = tile - j * ntz, k0 = kt * p.KT;
        const int y0 = 2 * j - o;
        const uint4* st = reinterpret_cast<const uint4*>(sbase + (size_t)s * stage_bytes);
        for (int e0 = warp * per; e0 < p.KT; e0 += kTiledWarps * per) {
            const int e = e0 + (lane >> w.lg), k = k0 + e;
            const bool has = k < NBZ && gl < w.nw;
            const int z0 = 2 * k - o;
            uint4 q[4], q0[4];
            bool in[4];
#pragma unroll
            for (int a = 0; a < 4; ++a) {
                const int ly = a < 2 ? 1 : 0, zz = 2 * e + (a & 1);
                const int y = y0 + ly, z = z0 + (a & 1);
                in[a] = has && y >= 0 && y < w.Y && z >= 0 && z < w.Z;
                q[a] = in[a] ? st[(ly * p.TZ + zz) * w.nw + gl] : make_uint4(0u, 0u, 0xFFFFFFFFu, 0xFFFFFFFFu);
                q0[a] = q[a];
            }
            rowpair_core(q, has, o, rowkey(sk, (uint32_t)j, (uint32_t)(has ? k : 0)), gl, G, w.nw, half_at_end);
            bool any = false;
#pragma unroll
            for (int a = 0; a < 4; ++a) {
                const bool chg =
                    in[a] && (q[a].x != q0[a].x || q[a].y != q0[a].y || q[a].z != q0[a].z || q[a].w != q0[a].w);
                if (chg) {
                    const int y = y0 + (a < 2 ? 1 : 0), z = z0 + (a & 1);
                    w.rows[((int64_t)y * w.Z + z) * w.nw + gl] = q[a];
                    any = true;
                }
                const uint32_t bal = __ballot_sync(0xFFFFFFFFu, chg);
                if (gl == 0 && (bal & gmask)) {
                    const int ly = a < 2 ? 1 : 0, zz = 2 * e + (a & 1);
                    atomicOr(&masks[s][ly][zz >> 5], 1u << (zz & 31));
                }
            }
            if (p.counts && any) count_bricks(p.counts, w, y0, z0, gl, q, q0, in);
        }
        // the last consumer warp of the tile writes its changed-row bits to
        // the step's flag buffer, then every warp releases the buffer
        __syncwarp();
        __threadfence_block();
        int last = 0;
        if (lane == 0) last = atomicAdd(&done_cnt[s], 1) == kTiledWarps - 1;
        last = __shfl_sync(0xFFFFFFFFu, last, 0);
        if (last) {
            __threadfence_block();
            const int nmw = p.TZ >> 5, W = (2 * k0) >> 5;
            if (lane < 2 * nmw) {
                const int ly = lane / nmw, i = lane - ly * nmw;
                const uint32_t m = masks[s][ly][i];
                if (m) {
                    uint32_t* F = p.flags + b_cur * fbuf + (size_t)(y0 + ly) * p.zw;
                    if (o == 0) {
                        atomicOr(F + W + i, m);
                    } else {
                        // tile row zz is z = 2*k0 - 1 + zz
                        if (m >> 1) atomicOr(F + W + i, m >> 1);
                        if (m & 1u) atomicOr(F + W + i - 1, 1u << 31);
                    }
                }
                masks[s][ly][i] = 0u;
            }
            if (lane == 0) done_cnt[s] = 0;
            __syncwarp();
        }
        if (lane == 0) bar_arrive(&empty_bar[s]);
    }
}

// cuTensorMapEncodeTiled, looked up once through the runtime
using EncodeTiled = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                 const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encode_fn() {
    static EncodeTiled fn = [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            f = nullptr;
        cudaGetLastError();
        return reinterpret_cast<EncodeTiled>(f);
    }();
    return fn;
}

void tile_shape(int nw, int* KT, int* TZ) {
    const int per = 32 >> plane_lg(nw);
    *KT = kTiledWarps * per < 16 ? 16 : kTiledWarps * per;
    *TZ = 2 * *KT;
}

size_t tiled_smem(int nw) {
    int KT, TZ;
    tile_shape(nw, &KT, &TZ);
    return (size_t)kTiledStages * 2u * (size_t)TZ * (size_t)nw * 16u + 1024u;
}

std::once_flag g_tiled_once;
int g_tiled_ctas_per_sm[2] = {1, 1};  // rows of at most 16 words, rows of 17..32 words

}  // namespace

bool tiled_supported(int X, int Y, int Z) {
    const int nw = plane_nw(X);
    return nw >= 2 && nw <= 32 && Y >= 1 && Z >= 1 && encode_fn() != nullptr;
}

size_t tiled_flag_bytes(int Y, int Z) { return 4u * (size_t)Y * (size_t)((Z + 31) / 32) * sizeof(uint32_t); }

fs3d_status tiled_encode(const uint4* rows, int X, int Y, int Z, void* tmap_out) {
    EncodeTiled fn = encode_fn();
    if (!fn) return set_error(FS3D_ERR_CUDA, "cuTensorMapEncodeTiled is unavailable");
    const int nw = plane_nw(X);
    int KT, TZ;
    tile_shape(nw, &KT, &TZ);
    const cuuint64_t dims[3] = {(cuuint64_t)nw * 4u, (cuuint64_t)Z, (cuuint64_t)Y};
    const cuuint64_t strides[2] = {(cuuint64_t)nw * 16u, (cuuint64_t)Z * nw * 16u};
    const cuuint32_t box[3] = {(cuuint32_t)nw * 4u, (cuuint32_t)TZ, 2u};
    const cuuint32_t estr[3] = {1u, 1u, 1u};
    const CUresult r = fn(static_cast<CUtensorMap*>(tmap_out), CU_TENSOR_MAP_DATA_TYPE_UINT32, 3,
                          const_cast<uint4*>(rows), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                          CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_error(FS3D_ERR_CUDA, "cuTensorMapEncodeTiled failed for the world's planes");
    return FS3D_OK;
}

fs3d_status tiled_init_flags(uint32_t* flags, int Y, int Z, uint64_t t0, cudaStream_t st) {
    const size_t buf = tiled_flag_bytes(Y, Z) / 4u;
    // every row changed at t0-1 and t0-2; nothing yet in the other two buffers
    for (uint32_t b = 0; b < 4u; ++b) {
        const bool prev = b == ((uint32_t)(t0 + 3u) & 3u) || b == ((uint32_t)(t0 + 2u) & 3u);
        FS3D_CUDA(cudaMemsetAsync(reinterpret_cast<uint8_t*>(flags) + b * buf, prev ? 0xFF : 0x00, buf, st));
    }
    return FS3D_OK;
}

fs3d_status launch_plane_step_tiled(const void* tmap, const PlaneWorld& w, uint32_t* flags, int* counts, int* err,
                                    cudaStream_t st) {
    std::call_once(g_tiled_once, [] {
        // the largest tile ring (rows of 32 words) sets the attribute for every size
        const size_t mx = tiled_smem(32);
        cudaFuncSetAttribute(k_plane_step_tiled, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)mx);
        for (int c = 0; c < 2; ++c) {
            int n = 0;
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_plane_step_tiled, kTiledThreads,
                                                              tiled_smem(c ? 32 : 16)) != cudaSuccess ||
                n < 1)
                n = 1;
            g_tiled_ctas_per_sm[c] = n;
        }
        cudaGetLastError();
    });
    TiledArgs a;
    a.w = w;
    a.flags = flags;
    a.zw = (w.Z + 31) / 32;
    tile_shape(w.nw, &a.KT, &a.TZ);
    a.counts = counts;
    a.tx_extra = inject_tx_extra();
    const size_t smem = tiled_smem(w.nw);
    const int grid = sm_count_public() * g_tiled_ctas_per_sm[w.nw > 16 ? 1 : 0];
    CUtensorMap tm;
    memcpy(&tm, tmap, sizeof(tm));
    k_plane_step_tiled<<<grid, kTiledThreads, smem, st>>>(tm, a, err);
    FS3D_CHECK_LAUNCH("tiled plane step launch");
    return FS3D_OK;
}

}  // namespace fs3d
