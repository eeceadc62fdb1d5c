// fs3d_run_device: n steps of a caller-owned device byte grid through the bit
// plane kernels.  The grid is converted once into 2-bit planes (scratch), the
// steps run there (all of them in one resident launch when the world fits in
// shared memory, one per-step launch each otherwise), and the planes are
// converted back.  Static cells never change, so their byte values are read
// back from the caller's grid itself.  Rows wider than 2048 cells take the
// byte kernels instead.
//
// A resident launch whose bulk copy does not land within its bounded wait
// leaves the grid as it was and sets a sticky per-device word; while it is
// set, later runs on the device leave their grids unchanged too, and
// fs3d_run_device_check reports FS3D_ERR_TIMEOUT and clears it.
#include <chrono>
#include <mutex>
#include <thread>
#include <vector>

#include "fs3d_common.h"
#include "planes.h"

namespace fs3d {
fs3d_status noalloc_error_word(int** out);  // run_noalloc.cu
}

using namespace fs3d;

namespace {

static __device__ __align__(16) int g_run_device_err[kErrInts];  // the resident kernel's error record

constexpr int kMaxDevices = 64;
struct ErrAddr {
    unsigned long long ctx = 0;
    int* p = nullptr;
};
ErrAddr g_err_addr[kMaxDevices];
std::mutex g_err_mu;

// The sticky word's device address on the current device, looked up per
// device for the context it belongs to.
fs3d_status run_error_word(int** out) {
    int dev = 0;
    FS3D_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return set_error(FS3D_ERR_INVALID_ARG, "fs3d_run_device: device index");
    unsigned long long ctx = 0;
    const bool known = current_context_id(&ctx);
    std::lock_guard<std::mutex> lock(g_err_mu);
    ErrAddr& c = g_err_addr[dev];
    if (!known || !c.p || !c.ctx || c.ctx != ctx) {
        void* p = nullptr;
        FS3D_CUDA(cudaGetSymbolAddress(&p, g_run_device_err));
        c.p = static_cast<int*>(p);
        c.ctx = current_context_id(&ctx) ? ctx : 0;
    }
    *out = c.p;
    return FS3D_OK;
}

// device scratch of one run: the planes and the one-world step tables
struct RunScratch {
    uint4* rows = nullptr;
    PlaneWorld* desc = nullptr;
    int* ints = nullptr;  // meta (1 + 2*classes), order[0], counter
};

constexpr int kOrder = kMetaInts, kCounter = kOrder + 1, kInts = kCounter + 1;

}  // namespace

extern "C" fs3d_status fs3d_run_device(uint8_t* grid_dev, int X, int Y, int Z, uint64_t seed, uint64_t t0,
                                       int n_steps, void* stream) {
    if (!grid_dev || X <= 0 || Y <= 0 || Z <= 0 || X > (1 << 20) || Y > (1 << 20) || Z > (1 << 20) || n_steps < 0)
        return set_error(FS3D_ERR_INVALID_ARG, "fs3d_run_device: null grid, bad dims or negative n_steps");
    cudaStream_t st = (cudaStream_t)stream;
    if (n_steps == 0) return FS3D_OK;
    if (X > kPlaneMaxX) return launch_step_bytes(grid_dev, X, Y, Z, seed, t0, n_steps, st);
    const int nw = plane_nw(X), lg = plane_lg(nw);
    // a resident launch, or the per-step kernel (prefer_resident)
    const int cls = prefer_resident(resident_class(X, Y, Z), n_steps, (int64_t)X * Y * Z) ? resident_class(X, Y, Z) : -1;
    // worlds too large for shared memory, and short calls: the per-step
    // kernel that skips settled row-pairs (per-row flags in the scratch)
    int* err = nullptr;
    {
        const fs3d_status se = run_error_word(&err);
        if (se != FS3D_OK) return se;
    }
    RunScratch sc;
    uint8_t* rflags = nullptr;
    cudaError_t e = cudaMallocAsync((void**)&sc.rows, plane_bytes(X, Y, Z), st);
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&sc.desc, sizeof(PlaneWorld), st);
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&sc.ints, sizeof(int) * kInts, st);
    // per-row flags for the per-step kernel, per-layer flags for a resident launch
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&rflags, cls < 0 ? (size_t)Y * Z : layer_flag_bytes(Y), st);
    fs3d_status s = e == cudaSuccess ? FS3D_OK : cuda_fail(e, "fs3d_run_device scratch");
    PlaneWorld d{};
    d.rows = sc.rows;
    d.seed = seed;
    d.t = t0;
    d.X = X;
    d.Y = Y;
    d.Z = Z;
    d.nw = nw;
    d.steps = n_steps;
    d.lg = lg;
    if (cls >= 0) d.lflags = rflags;  // set from the cells below: no dense first steps
    int ints[kInts] = {};
    if (cls >= 0) ints[1 + cls] = 1;
    // pageable sources: staged before each call returns
    if (s == FS3D_OK) e = cudaMemcpyAsync(sc.desc, &d, sizeof(d), cudaMemcpyHostToDevice, st);
    if (s == FS3D_OK && e == cudaSuccess) e = cudaMemcpyAsync(sc.ints, ints, sizeof(ints), cudaMemcpyHostToDevice, st);
    if (s == FS3D_OK && e != cudaSuccess) s = cuda_fail(e, "fs3d_run_device tables");
    if (s == FS3D_OK) s = planes_from_bytes(grid_dev, X, Y, Z, sc.rows, st);
    if (s == FS3D_OK) {
        if (cls >= 0) {
            s = layer_flags_from_cells(sc.rows, rflags, X, Y, Z, t0, st);
            if (s == FS3D_OK)
                s = launch_plane_segment_resident(cls, sc.desc, sc.ints + kOrder, sc.ints, sc.ints + kCounter, err, st);
        } else {
            s = init_row_flags(sc.rows, rflags, X, Y, Z, t0, st);
            for (int a = 0; a < n_steps && s == FS3D_OK; ++a) {
                d.t = t0 + (uint64_t)a;
                s = launch_plane_step_skip(d, rflags, nullptr, st);
            }
        }
    }
    // a recorded failure (this run's or an earlier one's) leaves the grid as it was
    if (s == FS3D_OK) s = planes_to_bytes(sc.rows, grid_dev, X, Y, Z, grid_dev, st, err);
    // only what was allocated (the allocations stop at the first failure)
    for (void* p : {(void*)sc.rows, (void*)sc.desc, (void*)sc.ints, (void*)rflags})
        if (p) cudaFreeAsync(p, st);
    return s;
}

namespace {

fs3d_status wait_bounded(cudaStream_t st, int64_t timeout_ns) {
    if (timeout_ns < 0) {
        FS3D_CUDA(cudaStreamSynchronize(st));
        return FS3D_OK;
    }
    const auto t0 = std::chrono::steady_clock::now();
    for (;;) {
        const cudaError_t e = cudaStreamQuery(st);
        if (e == cudaSuccess) return FS3D_OK;
        if (e != cudaErrorNotReady) return cuda_fail(e, "cudaStreamQuery");
        if (std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now() - t0).count() >=
            timeout_ns)
            return set_error(FS3D_ERR_TIMEOUT, "fs3d_run_device_check: the stream did not finish within the timeout");
        std::this_thread::sleep_for(std::chrono::microseconds(20));
    }
}

// reads an error record's flag on `st` and clears the record; *was = the flag
fs3d_status take_word(int* word, cudaStream_t st, int* was) {
    FS3D_CUDA(cudaMemcpyAsync(was, word, sizeof(int), cudaMemcpyDeviceToHost, st));
    FS3D_CUDA(cudaStreamSynchronize(st));
    if (*was) {
        FS3D_CUDA(cudaMemsetAsync(word, 0, sizeof(int) * kErrInts, st));
        FS3D_CUDA(cudaStreamSynchronize(st));
    }
    return FS3D_OK;
}

}  // namespace

extern "C" fs3d_status fs3d_run_device_check(void* stream, int64_t timeout_ns) {
    cudaStream_t st = (cudaStream_t)stream;
    fs3d_status s = wait_bounded(st, timeout_ns);
    if (s != FS3D_OK) return s;
    int* a = nullptr;
    int* b = nullptr;
    s = run_error_word(&a);
    if (s == FS3D_OK) s = noalloc_error_word(&b);
    if (s != FS3D_OK) return s;
    int va = 0, vb = 0;
    s = take_word(a, st, &va);
    if (s == FS3D_OK) s = take_word(b, st, &vb);
    if (s != FS3D_OK) return s;
    if (va || vb)
        return set_error(FS3D_ERR_TIMEOUT,
                         "a bulk copy of a drop-in run did not complete in time; that run and the runs after it "
                         "left their grids unchanged");
    return FS3D_OK;
}
