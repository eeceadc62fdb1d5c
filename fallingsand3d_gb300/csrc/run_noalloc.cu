// fs3d_run_device_noalloc: fs3d_run_device for callers that cannot allocate
// device memory.
//
// Some embedders of the step cannot call cudaMalloc (or any allocating
// routine) at the point where they advance the world.  Examples: an engine
// that reserves all of the GPU's memory for its own allocator at start-up, a
// frame loop on a real-time budget where an allocation may stall or
// synchronise the device, and a host that gives the library a stream but no
// allocator of its own.  This entry point runs the same bit-plane
// computation as fs3d_run_device, but its scratch (the world's planes and the
// step tables) lives in one file-scope static device array, so a call
// allocates nothing.  The caller still passes the grid, in device memory.
//
// Limits and contract:
//  * the world's planes must fit kNoAllocPlaneBytes (64 MiB: about 268 M
//    cells, e.g. 512^3), and rows wider than 2048 cells are refused; larger
//    worlds are rejected with FS3D_ERR_INVALID_ARG and a message;
//  * every GPU that loads this library holds the array (64 MiB of planes +
//    4 MiB of row flags and a few hundred bytes of tables) until the process
//    exits;
//  * the first call on a device looks up the array's device address with
//    cudaGetSymbolAddress (with that device current) and caches it for the
//    device's current context (a new context after cudaDeviceReset looks it
//    up again); make that first call before any stream capture;
//  * every call shares the array and it keeps the last call's contents; the
//    call clears what must start at zero itself.  Calls that overlap on the
//    GPU (two streams, or two host threads) race on the array: serialise them;
//  * one word of the array records a bulk copy whose bounded wait gave up
//    (the run leaves the grid as it was).  It is not cleared by the calls, so
//    later runs on the device also leave their grids unchanged until
//    fs3d_run_device_check reads and clears it.
#include <mutex>

#include "fs3d_common.h"
#include "planes.h"

namespace fs3d {
namespace {

constexpr size_t kNoAllocPlaneBytes = (size_t)64 << 20;
constexpr int kMaxDevices = 64;

// scratch layout: [planes][one-world descriptor][ints][sticky error record][row flags]
constexpr size_t kDescOff = kNoAllocPlaneBytes;
constexpr size_t kIntsOff = kDescOff + 256;
constexpr int kOrder = kMetaInts, kCounter = kOrder + 1, kInts = kCounter + 1;
constexpr size_t kErrOff = kIntsOff + 256;  // set by a timed-out copy, cleared by fs3d_run_device_check only
constexpr size_t kFlagsOff = kErrOff + 256;
// one byte per row of the per-step kernel: a world of at most 64 MiB of
// planes has at most 4 Mi rows (one 16-byte word each at the least)
constexpr size_t kNoAllocFlagBytes = kNoAllocPlaneBytes / sizeof(uint4);
constexpr size_t kScratchBytes = kFlagsOff + kNoAllocFlagBytes;
static_assert(kInts * sizeof(int) <= 256, "ints region");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// the array's device address per device, for the context it was looked up in
struct ScratchAddr {
    unsigned long long ctx = 0;  // 0: unknown, look it up again
    unsigned char* p = nullptr;
};
ScratchAddr g_scratch_addr[kMaxDevices];
std::mutex g_scratch_mu;

// Writes the one-world tables into the scratch and clears the work counter
// (the array keeps whatever the previous call left; the sticky error record
// is left alone).
__global__ void k_noalloc_tables(PlaneWorld d, int cls, unsigned char* base) {
    PlaneWorld* desc = reinterpret_cast<PlaneWorld*>(base + kDescOff);
    int* ints = reinterpret_cast<int*>(base + kIntsOff);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        *desc = d;
        for (int a = 0; a < kInts; ++a) ints[a] = 0;
        if (cls >= 0) ints[1 + cls] = 1;
    }
}

}  // namespace

// The array's device address on the current device.  Host code cannot use
// the array's name as a device address (it names a host-side stand-in), so
// the address is looked up with cudaGetSymbolAddress, with the device
// current, and kept per device for the context it belongs to.
fs3d_status noalloc_scratch_base(unsigned char** out) {
    int dev = 0;
    FS3D_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return set_error(FS3D_ERR_INVALID_ARG, "fs3d_run_device_noalloc: device index");
    unsigned long long ctx = 0;
    const bool known = current_context_id(&ctx);
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    ScratchAddr& c = g_scratch_addr[dev];
    if (!known || !c.p || !c.ctx || c.ctx != ctx) {
        void* p = nullptr;
        FS3D_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        c.p = static_cast<unsigned char*>(p);
        // the lookup made the device's context current if none was
        c.ctx = current_context_id(&ctx) ? ctx : 0;
    }
    *out = c.p;
    return FS3D_OK;
}

fs3d_status noalloc_error_word(int** out) {
    unsigned char* base = nullptr;
    const fs3d_status s = noalloc_scratch_base(&base);
    if (s == FS3D_OK) *out = reinterpret_cast<int*>(base + kErrOff);
    return s;
}

}  // namespace fs3d

using namespace fs3d;

extern "C" fs3d_status fs3d_run_device_noalloc(uint8_t* grid_dev, int X, int Y, int Z, uint64_t seed, uint64_t t0,
                                               int n_steps, void* stream) {
    if (!grid_dev || X <= 0 || Y <= 0 || Z <= 0 || n_steps < 0)
        return set_error(FS3D_ERR_INVALID_ARG, "fs3d_run_device_noalloc: null grid, bad dims or negative n_steps");
    if (X > kPlaneMaxX || Y > (1 << 20) || Z > (1 << 20) || plane_bytes(X, Y, Z) > kNoAllocPlaneBytes)
        return set_error(FS3D_ERR_INVALID_ARG,
                         "fs3d_run_device_noalloc: world too large for the static scratch (planes of at most "
                         "64 MiB, about 268 M cells, and rows of at most 2048 cells)");
    const int nw = plane_nw(X), lg = plane_lg(nw);
    // a resident launch, or the per-step kernel (prefer_resident)
    const int cls = prefer_resident(resident_class(X, Y, Z), n_steps, (int64_t)X * Y * Z) ? resident_class(X, Y, Z) : -1;
    if (n_steps == 0) return FS3D_OK;
    unsigned char* base = nullptr;
    fs3d_status s = noalloc_scratch_base(&base);
    if (s != FS3D_OK) return s;
    cudaStream_t st = (cudaStream_t)stream;
    uint4* rows = reinterpret_cast<uint4*>(base);
    PlaneWorld d{};
    d.rows = rows;
    d.seed = seed;
    d.t = t0;
    d.X = X;
    d.Y = Y;
    d.Z = Z;
    d.nw = nw;
    d.steps = n_steps;
    d.lg = lg;
    uint8_t* flags = base + kFlagsOff;  // per-row flags (per-step kernel) or per-layer flags (resident launch)
    if (cls >= 0) d.lflags = flags;     // set from the cells below: no dense first steps
    k_noalloc_tables<<<1, 32, 0, st>>>(d, cls, base);
    FS3D_CHECK_LAUNCH("noalloc tables launch");
    PlaneWorld* desc = reinterpret_cast<PlaneWorld*>(base + kDescOff);
    int* ints = reinterpret_cast<int*>(base + kIntsOff);
    int* err = reinterpret_cast<int*>(base + kErrOff);
    s = planes_from_bytes(grid_dev, X, Y, Z, rows, st);
    if (s == FS3D_OK) {
        if (cls >= 0) {
            s = layer_flags_from_cells(rows, flags, X, Y, Z, t0, st);
            if (s == FS3D_OK) s = launch_plane_segment_resident(cls, desc, ints + kOrder, ints, ints + kCounter, err, st);
        } else {
            uint8_t* rflags = flags;
            s = init_row_flags(rows, rflags, X, Y, Z, t0, st);
            for (int a = 0; a < n_steps && s == FS3D_OK; ++a) {
                d.t = t0 + (uint64_t)a;
                s = launch_plane_step_skip(d, rflags, nullptr, st);
            }
        }
    }
    // static cells never change: their values are read back from the grid
    // itself; a recorded failure leaves the grid as it was
    if (s == FS3D_OK) s = planes_to_bytes(rows, grid_dev, X, Y, Z, grid_dev, st, err);
    return s;
}
