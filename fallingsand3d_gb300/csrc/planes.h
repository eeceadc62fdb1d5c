// Bit-plane world format: device descriptors and host entry points.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "fs3d_common.h"

namespace fs3d {

// One world as the step kernel sees it (device memory, 64 bytes).
struct PlaneWorld {
    uint4* rows;      // Y*Z rows of nw uint4 words
    uint64_t seed;
    uint64_t t;       // step counter at the start of the current segment
    int32_t X, Y, Z, nw;
    int32_t steps;    // steps this world takes in the current segment
    int32_t lg;       // log2 of the lane-group size (pow2ceil(nw))
    uint8_t* lflags;       // nullable: per-layer last-changed step (low 8 bits), kept across segments
    int32_t lflags_fresh;  // 1: lflags hold nothing yet (start from "every layer changed")
    int32_t pad;
};
static_assert(sizeof(PlaneWorld) == 64, "PlaneWorld layout");

// Warp-sized work item: 32 >> lg block row-pairs of one world.
struct PlaneItem {
    int32_t world;
    int32_t rp0;
};

inline int plane_nw(int X) { return (X + 63) / 64; }
inline size_t plane_bytes(int X, int Y, int Z) { return (size_t)Y * Z * plane_nw(X) * sizeof(uint4); }
// layer flags stored after a world's planes in the same allocation
inline size_t layer_flag_bytes(int Y) { return ((size_t)Y + 15) & ~(size_t)15; }
constexpr int kPlaneMaxX = 2048;  // lane groups of at most 32 words

// Resident segment classes: worlds whose planes fit in shared memory take
// all their segment steps in one launch.  Classes 0..2 hold a world in one CTA
// of 128 / 256 / 768 threads (6 / 3 / 1 CTAs per SM); classes 3..5 split a
// world into y-slabs over a cluster of 2 / 4 / 8 CTAs of 512 threads.
constexpr int kResidentClasses = 6;
constexpr int kSingleCtaClasses = 3;  // classes 0..2 hold a world in one CTA
// Global-memory segment classes (the world stays in L2/HBM; one CTA of
// 32/64/128/256 threads per world, by the work of one layer pair; -1 if the
// world has too many layers), and kGmDense: one CTA of 768 threads per SM
// for a young (dense) world too large for one CTA's shared memory.
constexpr int kGmClasses = 5;
constexpr int kGmDense = 4;
int resident_class_gm(int X, int Y, int Z);
// Class ids of a segment's tables: shared-memory classes 0..5, then the
// global-memory classes 6..9.  meta = {per-step items, worlds per class,
// offset of each class in the order array, worlds in the table}.
constexpr int kAllClasses = kResidentClasses + kGmClasses;
constexpr int kMetaWorlds = 1 + 2 * kAllClasses;
constexpr int kMetaInts = kMetaWorlds + 1;
// smallest class that holds a world of these dims, -1 if none does
int resident_class(int X, int Y, int Z);
// Whether a call of n steps on one world of class cls takes them in one
// resident launch (one CTA or cluster: its load, store and launch paid once
// per call, then about 3-4.3 us per step up to 112^3) rather than n launches
// of the per-step kernel (each step on the whole GPU, about 6.2-7.4 us).
// Measured crossovers: 64^3 at 3-4 steps per call, 80^3 at 5, 96^3 at 7-8,
// 112^3 at 11; 128^3 (a cluster) the per-step kernel at 1 and 8 steps per
// call (7.1 against 9.8-22 us resident).
inline bool prefer_resident(int cls, int n_steps, int64_t cells) {
    return cls >= 0 && n_steps >= 4 && cells <= 1500000 && (int64_t)n_steps * 120000 >= cells;
}
// largest plane buffer (bytes) one CTA can hold; 0 if unavailable
int smem_world_limit();
constexpr int kErrInts = 4;  // size of the error record a resident launch is given
// test hook: resident kernels announce `bytes` more than each bulk copy delivers
fs3d_status set_inject_tx_extra(uint32_t bytes);
// test hook: the next n stream-ordered allocations of batch admissions fail as out of memory
void set_inject_alloc_failures(int n);
// One launch steps every world of class `cls` (order[meta[1+K+cls] ...],
// meta[1+cls] of them) through its segment steps in shared memory.  err
// points to 4 ints (8-byte aligned): a bulk copy that does not complete
// within the wait limit sets err[0] = 1 and err[2..3] = the failing world's
// step at the start of the launch (first failure only); while err[0] is set,
// launches given it step nothing.  Row
// pairs whose rows are settled are skipped; the cell-steps actually evaluated
// are added to *processed_cells when it is not null.
fs3d_status launch_plane_segment_resident(int cls, const PlaneWorld* worlds, const int* order, const int* meta,
                                          int* counter, int* err, cudaStream_t st,
                                          unsigned long long* processed_cells = nullptr);

// `first`: launched with the greatest priority, so that in a segment graph,
// where every class's grid is pending at once, its CTAs are placed first.
fs3d_status launch_plane_segment_gm(int cls, const PlaneWorld* worlds, const int* order, const int* meta,
                                    int* counter, int* err, cudaStream_t st, unsigned long long* processed_cells,
                                    bool first = false);

// One world of a many-world conversion: its planes, its static bytes
// (nullable) and the offset of its canonical bytes in a shared staging buffer.
struct ConvJob {
    uint4* rows;
    const uint8_t* statics;
    int64_t byte_off;
    int32_t X, Y, Z, nw;
    // read-back of a world whose static-material flag has not reached the
    // host yet: when *static_flag is set, its static bytes are at static_src
    const int* static_flag;
    const uint8_t* static_src;
    // admission: the world's layer flags (set from its cells by
    // layer_flags_from_cells_multi; null: none) and its first step's low 8 bits
    uint8_t* lflags = nullptr;
    uint32_t t0b = 0;
};
// bytes -> planes for njobs worlds in one launch; unit_off[j] = sum of Y*Z*nw
// over jobs before j; block_job[i] = the job of unit kConvBlock*i (from
// conv_block_jobs); flags[j] |= 1 when world j holds a material >= 4
constexpr int kConvBlock = 256;  // units per CTA pass of the conversion kernels
inline int64_t conv_blocks(int64_t total_units) { return (total_units + kConvBlock - 1) / kConvBlock; }
inline void conv_block_jobs(const int64_t* unit_off, int njobs, int64_t total_units, int* block_job) {
    int j = 0;
    for (int64_t i = 0; i < conv_blocks(total_units); ++i) {
        while (j + 1 < njobs && unit_off[j + 1] <= i * kConvBlock) ++j;
        block_job[i] = j;
    }
}
fs3d_status planes_from_bytes_multi(const ConvJob* jobs, const int64_t* unit_off, const int* block_job, int njobs,
                                    int64_t total_units, const uint8_t* staging, int* flags, cudaStream_t st);
fs3d_status planes_to_bytes_multi(const ConvJob* jobs, const int64_t* unit_off, const int* block_job, int njobs,
                                  int64_t total_units, uint8_t* staging, cudaStream_t st);

// Many byte copies in one launch (each thread moves a 16-byte chunk): used
// instead of one cudaMemcpyAsync per world when both sides are addressable
// by the device (device memory, or page-locked host memory, which the GPU
// reads and writes directly).  chunk_off[j] = sum of ceil(bytes/16) before j.
struct CopyJob {
    const uint8_t* src;
    uint8_t* dst;
    int64_t bytes;
};
fs3d_status copy_many(const CopyJob* jobs, const int64_t* chunk_off, int njobs, int64_t total_chunks, cudaStream_t st);
// A small copy (tables, flags) done by a kernel instead of a copy engine, so
// it does not queue behind large transfers on the copy engines.  Both
// pointers must be device-addressable (device memory, or the device view of
// page-locked host memory); pointers not 16-byte aligned take cudaMemcpyAsync.
cudaError_t copy_small_async(void* dst, const void* src, size_t bytes, cudaStream_t st);
// A device-addressable alias of p (itself for device or managed memory, the
// mapped address for page-locked host memory), or nullptr for pageable memory.
uint8_t* device_view(const void* p);
// The allocation that holds p (start, bytes), as the driver reports it; false
// if it cannot tell.  A copy over several grids must stay inside one.
bool alloc_range(const void* p, uintptr_t* start, size_t* bytes);

int plane_lg(int nw);
int plane_items_for(int Y, int Z, int nw);
int plane_step_grid(int64_t n_items);
int plane_step_ctas_per_sm();
fs3d_status planes_from_bytes(const uint8_t* g, int X, int Y, int Z, uint4* rows, cudaStream_t st);
// the batch world of `world_seed` written straight into planes (needs Y >= 4)
fs3d_status planes_generate_batch_world(uint64_t world_seed, int X, int Y, int Z, uint4* rows, cudaStream_t st);
// skip_if_set (nullable): the conversion writes nothing when *skip_if_set is
// non-zero (a drop-in run whose step kernel recorded a failure leaves the
// caller's grid as it was)
fs3d_status planes_to_bytes(const uint4* rows, const uint8_t* statics, int X, int Y, int Z, uint8_t* g,
                            cudaStream_t st, const int* skip_if_set = nullptr);

// ---- per-step kernel of one large world with an exact skip of settled
// row-pairs: one byte per row (y, z) holds the low 8 bits of the last step
// that changed it (Y*Z bytes).  init_row_flags: a world about to take step t0
// with no history: a row is marked changed at t0 - 1 when a block row-pair of
// either phase that covers it can change (the rule's activity mask on its
// cells), else at t0 - 3.
fs3d_status init_row_flags(const uint4* rows, uint8_t* rflags, int X, int Y, int Z, uint64_t t0, cudaStream_t st);

// Layer flags of newly admitted worlds (jobs with lflags set), the same way
// per layer: marked changed at t0 - 1 when a block row-pair of either phase
// covering the layer can change, else at t0 - 3.  max_Y: the largest Y of the jobs.
fs3d_status layer_flags_from_cells_multi(const ConvJob* jobs, int njobs, int max_Y, cudaStream_t st);
// the same for one world
fs3d_status layer_flags_from_cells(const uint4* rows, uint8_t* lflags, int X, int Y, int Z, uint64_t t0,
                                   cudaStream_t st);
// one step (w.t) of the world; counts as for launch_plane_step
fs3d_status launch_plane_step_skip(const PlaneWorld& w, uint8_t* rflags, int* counts, cudaStream_t st);
fs3d_status planes_hash_async(const uint4* rows, const uint8_t* statics, int X, int Y, int Z,
                              unsigned long long* out_dev, cudaStream_t st);
// whole-grid hashes of njobs worlds in one launch: out_dev[j] for jobs[j]
struct HashJob {
    const uint4* rows;
    const uint8_t* statics;  // nullable
    int32_t X, Y, Z, nw;
};
fs3d_status planes_hash_many(const HashJob* jobs, int njobs, unsigned long long* out_dev, cudaStream_t st);
// One step of many worlds at once (the batch's worlds too large to be
// resident).  brick_counts: nullable per-brick counts of non-empty cells of
// world 0, kept exact as it steps.
fs3d_status launch_plane_step(const PlaneWorld* worlds, const PlaneItem* items, const int* n_items_dev, int grid,
                              int s_seg, cudaStream_t st, int* brick_counts = nullptr);

// After a segment: every world of the table (meta[kMetaWorlds] of them) moves
// on by its segment steps, and its layer flags count as kept, so the next
// segment of an unchanged batch reuses the table as it stands.
fs3d_status launch_advance_worlds(PlaneWorld* worlds, const int* meta, cudaStream_t st);

// byte-grid kernels (step_bytes.cu)
bool rows16_ok(const void* grid, int X);
fs3d_status launch_step_bytes(uint8_t* grid, int X, int Y, int Z, uint64_t seed, uint64_t t0, int n_steps,
                              cudaStream_t st);
fs3d_status hash_bytes_async(const uint8_t* g, int64_t n, unsigned long long* out_dev, cudaStream_t st);
int sm_count_public();

// render (render.cu)
fs3d_status launch_render_sdf(const fs3d_camera* cam, int W, int H, float* rgba_dev, cudaStream_t st);
// the DDA kernels take a per-frame brick occupancy bitmap of brickmap_bytes() bytes
size_t brickmap_bytes(int X, int Y, int Z);
fs3d_status launch_render_dda_bytes(const uint8_t* g, int X, int Y, int Z, uint32_t* bm_bits, const fs3d_camera* cam,
                                    int W, int H, float* rgba_dev, cudaStream_t st);
// brick_counts (nullable): exact per-brick counts of non-empty cells; the
// frame then derives its brick map from them (rebuild: recount from the
// planes first) instead of a pass over the planes
fs3d_status launch_render_dda_planes(const uint4* rows, const uint8_t* statics, int X, int Y, int Z, int nw,
                                     uint32_t* bm_bits, const fs3d_camera* cam, int W, int H, float* rgba_dev,
                                     cudaStream_t st, int* brick_counts = nullptr, bool recount = true);
size_t brick_count_bytes(int X, int Y, int Z);

}  // namespace fs3d
