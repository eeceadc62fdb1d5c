// fs3d_world: one library-owned world on the device, its stream, step,
// read-back, hash, render and checkpoint entry points.
//
// The world sits between the engine's event poll and its draw call
// (src/engine/engine.cpp:60-68 upstream): step() advances it, render()
// produces the frame from the same device-resident grid.
#include <stdio.h>
#include <string.h>
#include <time.h>

#include <chrono>
#include <thread>
#include <vector>

#include "fs3d_common.h"
#include "planes.h"

using namespace fs3d;

struct fs3d_world {
    int X = 0, Y = 0, Z = 0, layout = FS3D_LAYOUT_BYTES;
    uint64_t seed = 0, step = 0;
    cudaStream_t stream = nullptr;
    uint8_t* bytes = nullptr;    // BYTES: the state
    uint4* rows = nullptr;       // PLANES: the state
    uint8_t* statics = nullptr;  // PLANES: initial bytes when some cell holds a material >= 4
    PlaneWorld* desc = nullptr;  // PLANES: one-world descriptor of the resident kernels
    int* aux = nullptr;          // resident tables, see kAux*
    int cls = -1;        // resident class (-1: stepped by the per-step kernel)
    unsigned long long* hash_dev = nullptr;
    uint32_t* brickmap = nullptr;  // render: per-frame occupancy of 8x8x8 bricks
    int* brick_counts = nullptr;   // PLANES render: non-empty cells per brick, kept by the per-step kernel
    bool counts_valid = false;     // brick_counts match the planes
    // change flags kept from one call to the next: per row (Y*Z bytes) for the
    // per-step kernel, per layer (Y bytes, padded) for a resident launch
    uint8_t* rflags = nullptr;
    bool flags_ok = false;  // rflags describe the state at step flags_t
    uint64_t flags_t = 0;
    uint8_t* lflags = nullptr;  // resident class only
    bool lflags_ok = false;     // lflags describe the state at step lflags_t
    uint64_t lflags_t = 0;
    int64_t cells() const { return (int64_t)X * Y * Z; }
};

namespace {

// layout of fs3d_world::aux (device ints)
constexpr int kAuxMeta = 0;                              // kMetaInts ints
constexpr int kAuxOrder = kMetaInts;      // order[0] = 0
constexpr int kAuxCounter = kAuxOrder + 1;
constexpr int kAuxErr = (kAuxCounter + 2) & ~1;   // kErrInts ints, 8-byte aligned
constexpr int kAuxInts = kAuxErr + kErrInts;

bool dims_ok(int X, int Y, int Z) {
    return X > 0 && Y > 0 && Z > 0 && X <= (1 << 16) && Y <= (1 << 16) && Z <= (1 << 16);
}

fs3d_status bounded_wait(cudaStream_t st, int64_t timeout_ns) {
    if (timeout_ns < 0) {
        FS3D_CUDA(cudaStreamSynchronize(st));
        return FS3D_OK;
    }
    const auto t0 = std::chrono::steady_clock::now();
    for (;;) {
        const cudaError_t e = cudaStreamQuery(st);
        if (e == cudaSuccess) return FS3D_OK;
        if (e != cudaErrorNotReady) return cuda_fail(e, "cudaStreamQuery");
        const auto ns = std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now() - t0).count();
        if (ns >= timeout_ns) return set_error(FS3D_ERR_TIMEOUT, "stream did not finish within the timeout");
        std::this_thread::sleep_for(std::chrono::microseconds(20));
    }
}

bool any_static(const uint8_t* g, int64_t n) {
    for (int64_t i = 0; i < n; ++i)
        if (g[i] >= 4) return true;
    return false;
}

void destroy(fs3d_world* w) {
    if (!w) return;
    if (w->stream) cudaStreamSynchronize(w->stream);
    cudaFree(w->bytes);
    cudaFree(w->rows);
    cudaFree(w->statics);
    cudaFree(w->desc);
    cudaFree(w->aux);
    cudaFree(w->hash_dev);
    cudaFree(w->brickmap);
    cudaFree(w->brick_counts);
    cudaFree(w->rflags);
    cudaFree(w->lflags);
    if (w->stream) cudaStreamDestroy(w->stream);
    delete w;
}

// upload a host grid into the world's state
fs3d_status upload(fs3d_world* w, const uint8_t* g) {
    const int64_t n = w->cells();
    if (w->layout == FS3D_LAYOUT_BYTES) {
        FS3D_CUDA(cudaMemcpyAsync(w->bytes, g, (size_t)n, cudaMemcpyHostToDevice, w->stream));
        FS3D_CUDA(cudaStreamSynchronize(w->stream));
        return FS3D_OK;
    }
    const bool stat = any_static(g, n);
    if (stat && !w->statics) FS3D_CUDA(cudaMalloc((void**)&w->statics, (size_t)n));
    if (!stat && w->statics) {
        cudaFree(w->statics);
        w->statics = nullptr;
    }
    uint8_t* staging = w->statics;
    if (!staging) FS3D_CUDA(cudaMallocAsync((void**)&staging, (size_t)n, w->stream));
    FS3D_CUDA(cudaMemcpyAsync(staging, g, (size_t)n, cudaMemcpyHostToDevice, w->stream));
    fs3d_status s = planes_from_bytes(staging, w->X, w->Y, w->Z, w->rows, w->stream);
    if (staging != w->statics) cudaFreeAsync(staging, w->stream);
    if (s != FS3D_OK) return s;
    FS3D_CUDA(cudaStreamSynchronize(w->stream));
    return FS3D_OK;
}

}  // namespace

extern "C" {

fs3d_status fs3d_world_create(const uint8_t* grid_host, int X, int Y, int Z, uint64_t seed, uint64_t start_step,
                              int layout, fs3d_world** out) {
    if (!out) return set_error(FS3D_ERR_INVALID_ARG, "fs3d_world_create: out is NULL");
    *out = nullptr;
    if (!grid_host || !dims_ok(X, Y, Z))
        return set_error(FS3D_ERR_INVALID_ARG, "fs3d_world_create: NULL grid or dims outside 1..65536");
    if (layout != FS3D_LAYOUT_BYTES && layout != FS3D_LAYOUT_PLANES)
        return set_error(FS3D_ERR_INVALID_ARG, "fs3d_world_create: unknown layout");
    if (layout == FS3D_LAYOUT_PLANES && X > kPlaneMaxX)
        return set_error(FS3D_ERR_INVALID_ARG, "fs3d_world_create: PLANES layout needs X <= 2048");
    fs3d_world* w = new fs3d_world();
    w->X = X;
    w->Y = Y;
    w->Z = Z;
    w->layout = layout;
    w->seed = seed;
    w->step = start_step;
    fs3d_status s = FS3D_OK;
    auto fail = [&](cudaError_t e, const char* what) {
        s = cuda_fail(e, what);
        destroy(w);
        return s;
    };
    cudaError_t e = cudaStreamCreateWithFlags(&w->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return fail(e, "cudaStreamCreate");
    e = cudaMalloc((void**)&w->hash_dev, sizeof(unsigned long long));
    if (e != cudaSuccess) return fail(e, "cudaMalloc(hash)");
    if (layout == FS3D_LAYOUT_BYTES) {
        e = cudaMalloc((void**)&w->bytes, (size_t)w->cells());
        if (e != cudaSuccess) return fail(e, "cudaMalloc(grid)");
    } else {
        e = cudaMalloc((void**)&w->rows, plane_bytes(X, Y, Z));
        if (e != cudaSuccess) return fail(e, "cudaMalloc(planes)");
        e = cudaMalloc((void**)&w->desc, sizeof(PlaneWorld));
        // resident tables: meta (one world in its class), order {0}, work counter, error record
        int aux[kAuxInts] = {};
        w->cls = resident_class(X, Y, Z);
        if (w->cls >= 0) aux[1 + w->cls] = 1;
        if (e == cudaSuccess) e = cudaMalloc((void**)&w->aux, sizeof(aux));
        if (e == cudaSuccess) e = cudaMemcpy(w->aux, aux, sizeof(aux), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return fail(e, "cudaMalloc/copy(step tables)");
        e = cudaMalloc((void**)&w->rflags, (size_t)Y * Z);
        if (e == cudaSuccess && w->cls >= 0) e = cudaMalloc((void**)&w->lflags, layer_flag_bytes(Y));
        if (e != cudaSuccess) return fail(e, "cudaMalloc(change flags)");
    }
    s = upload(w, grid_host);
    if (s != FS3D_OK) {
        destroy(w);
        return s;
    }
    *out = w;
    return FS3D_OK;
}

fs3d_status fs3d_world_step(fs3d_world* w, int n_steps) {
    if (!w || n_steps < 0) return set_error(FS3D_ERR_INVALID_ARG, "fs3d_world_step: bad args");
    if (n_steps == 0) return FS3D_OK;
    fs3d_status s;
    if (w->layout == FS3D_LAYOUT_BYTES) {
        s = launch_step_bytes(w->bytes, w->X, w->Y, w->Z, w->seed, w->step, n_steps, w->stream);
    } else {
        const int nw = plane_nw(w->X);
        PlaneWorld d{};
        d.rows = w->rows;
        d.seed = w->seed;
        d.t = w->step;
        d.X = w->X;
        d.Y = w->Y;
        d.Z = w->Z;
        d.nw = nw;
        d.steps = n_steps;
        d.lg = plane_lg(nw);
        s = FS3D_OK;
        // one resident launch, or one per-step launch per step (prefer_resident)
        const bool resident = prefer_resident(w->cls, n_steps, w->cells());
        if (!resident) {
            // one launch per step, settled row-pairs skipped; the row flags
            // carry over from the previous call when nothing else touched the
            // world since.  Once a frame has counted the bricks, the kernel
            // keeps the counts exact, so later frames read no pass over the planes
            if (!w->flags_ok || w->flags_t != w->step) {
                s = init_row_flags(w->rows, w->rflags, w->X, w->Y, w->Z, w->step, w->stream);
                w->flags_ok = s == FS3D_OK;
            }
            int* counts = w->counts_valid ? w->brick_counts : nullptr;
            int launched = 0;
            while (s == FS3D_OK && launched < n_steps) {
                d.t = w->step + (uint64_t)launched;
                s = launch_plane_step_skip(d, w->rflags, counts, w->stream);
                if (s == FS3D_OK) ++launched;
            }
            w->step += (uint64_t)launched;  // the steps that went out before a failed launch still count
            if (s == FS3D_OK)
                w->flags_t = w->step;
            else
                w->flags_ok = false;
            return s;
        }
        // the world fits in shared memory (one CTA or a cluster): all n steps
        // in one launch, the layer flags kept from the previous call (or set
        // from the cells); the descriptor's pageable source is staged before
        // the call returns
        if (!w->lflags_ok || w->lflags_t != w->step) {
            s = layer_flags_from_cells(w->rows, w->lflags, w->X, w->Y, w->Z, w->step, w->stream);
            w->lflags_ok = s == FS3D_OK;
        }
        d.lflags = w->lflags;
        if (s == FS3D_OK) {
            const cudaError_t ce = cudaMemcpyAsync(w->desc, &d, sizeof(d), cudaMemcpyHostToDevice, w->stream);
            s = ce == cudaSuccess ? FS3D_OK : cuda_fail(ce, "fs3d_world_step descriptor");
        }
        if (s == FS3D_OK)
            s = launch_plane_segment_resident(w->cls, w->desc, w->aux + kAuxOrder, w->aux + kAuxMeta,
                                              w->aux + kAuxCounter, w->aux + kAuxErr, w->stream);
        if (s == FS3D_OK)
            w->lflags_t = w->step + (uint64_t)n_steps;
        else
            w->lflags_ok = false;
        w->counts_valid = false;  // the next frame recounts
    }
    if (s == FS3D_OK) w->step += (uint64_t)n_steps;
    return s;
}

fs3d_status fs3d_world_sync(fs3d_world* w, int64_t timeout_ns) {
    if (!w) return set_error(FS3D_ERR_INVALID_ARG, "fs3d_world_sync: NULL world");
    fs3d_status s = bounded_wait(w->stream, timeout_ns);
    if (s != FS3D_OK) return s;
    if (w->aux) {
        int err[kErrInts] = {};
        FS3D_CUDA(cudaMemcpy(err, w->aux + kAuxErr, sizeof(err), cudaMemcpyDeviceToHost));
        if (err[0]) {
            uint64_t t_fail = 0;
            memcpy(&t_fail, err + 2, sizeof(t_fail));
            FS3D_CUDA(cudaMemset(w->aux + kAuxErr, 0, sizeof(err)));
            w->counts_valid = false;
            // the failed launch and every launch after it stepped nothing: the
            // state is the one the failed launch started from
            w->step = t_fail;
            return set_error(FS3D_ERR_TIMEOUT,
                             "a shared-memory bulk copy did not complete in time; the world was set back to the "
                             "step its state holds");
        }
    }
    return FS3D_OK;
}

fs3d_status fs3d_world_read(fs3d_world* w, uint8_t* out) {
    if (!w || !out) return set_error(FS3D_ERR_INVALID_ARG, "fs3d_world_read: bad args");
    const size_t n = (size_t)w->cells();
    if (w->layout == FS3D_LAYOUT_BYTES) {
        FS3D_CUDA(cudaMemcpyAsync(out, w->bytes, n, cudaMemcpyDeviceToHost, w->stream));
        FS3D_CUDA(cudaStreamSynchronize(w->stream));
        return FS3D_OK;
    }
    uint8_t* staging = nullptr;
    FS3D_CUDA(cudaMallocAsync((void**)&staging, n, w->stream));
    fs3d_status s = planes_to_bytes(w->rows, w->statics, w->X, w->Y, w->Z, staging, w->stream);
    cudaError_t e = cudaSuccess;
    if (s == FS3D_OK) e = cudaMemcpyAsync(out, staging, n, cudaMemcpyDeviceToHost, w->stream);
    cudaFreeAsync(staging, w->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(w->stream);
    if (s == FS3D_OK && e != cudaSuccess) s = cuda_fail(e, "fs3d_world_read");
    return s;
}

fs3d_status fs3d_world_write(fs3d_world* w, const uint8_t* g) {
    if (!w || !g) return set_error(FS3D_ERR_INVALID_ARG, "fs3d_world_write: bad args");
    w->counts_valid = false;
    w->flags_ok = false;
    w->lflags_ok = false;
    return upload(w, g);
}

fs3d_status fs3d_world_hash(fs3d_world* w, uint64_t* out) {
    if (!w || !out) return set_error(FS3D_ERR_INVALID_ARG, "fs3d_world_hash: bad args");
    fs3d_status s = (w->layout == FS3D_LAYOUT_BYTES)
                        ? hash_bytes_async(w->bytes, w->cells(), w->hash_dev, w->stream)
                        : planes_hash_async(w->rows, w->statics, w->X, w->Y, w->Z, w->hash_dev, w->stream);
    if (s != FS3D_OK) return s;
    unsigned long long h = 0;
    FS3D_CUDA(cudaMemcpyAsync(&h, w->hash_dev, sizeof(h), cudaMemcpyDeviceToHost, w->stream));
    FS3D_CUDA(cudaStreamSynchronize(w->stream));
    *out = (uint64_t)h;
    return FS3D_OK;
}

fs3d_status fs3d_world_info(const fs3d_world* w, int* X, int* Y, int* Z, uint64_t* seed, uint64_t* step,
                            int* layout) {
    if (!w) return set_error(FS3D_ERR_INVALID_ARG, "fs3d_world_info: NULL world");
    if (X) *X = w->X;
    if (Y) *Y = w->Y;
    if (Z) *Z = w->Z;
    if (seed) *seed = w->seed;
    if (step) *step = w->step;
    if (layout) *layout = w->layout;
    return FS3D_OK;
}

fs3d_status fs3d_world_device_ptr(fs3d_world* w, const void** dev, int* layout) {
    if (!w || !dev) return set_error(FS3D_ERR_INVALID_ARG, "fs3d_world_device_ptr: bad args");
    *dev = w->layout == FS3D_LAYOUT_BYTES ? (const void*)w->bytes : (const void*)w->rows;
    if (layout) *layout = w->layout;
    return FS3D_OK;
}

fs3d_status fs3d_world_stream(fs3d_world* w, void** stream) {
    if (!w || !stream) return set_error(FS3D_ERR_INVALID_ARG, "fs3d_world_stream: bad args");
    *stream = (void*)w->stream;
    return FS3D_OK;
}

fs3d_status fs3d_world_destroy(fs3d_world* w) {
    if (!w) return set_error(FS3D_ERR_INVALID_ARG, "fs3d_world_destroy: NULL world");
    destroy(w);
    return FS3D_OK;
}

// ---- checkpoint ----
struct CkpHeader {
    char magic[8];
    uint32_t version, reserved;
    int32_t X, Y, Z, pad;
    uint64_t seed, step;
};

fs3d_status fs3d_world_save(fs3d_world* w, const char* path) {
    if (!w || !path) return set_error(FS3D_ERR_INVALID_ARG, "fs3d_world_save: bad args");
    std::vector<uint8_t> g((size_t)w->cells());
    fs3d_status s = fs3d_world_read(w, g.data());
    if (s != FS3D_OK) return s;
    CkpHeader h{};
    memcpy(h.magic, "FS3DCKP1", 8);
    h.version = 1;
    h.X = w->X;
    h.Y = w->Y;
    h.Z = w->Z;
    h.seed = w->seed;
    h.step = w->step;
    FILE* f = fopen(path, "wb");
    if (!f) return set_error(FS3D_ERR_IO, std::string("fs3d_world_save: cannot open ") + path);
    const bool ok = fwrite(&h, sizeof(h), 1, f) == 1 && fwrite(g.data(), 1, g.size(), f) == g.size();
    const bool closed = fclose(f) == 0;
    if (!ok || !closed) return set_error(FS3D_ERR_IO, "fs3d_world_save: short write");
    return FS3D_OK;
}

fs3d_status fs3d_world_load(const char* path, int layout, fs3d_world** out) {
    if (!path || !out) return set_error(FS3D_ERR_INVALID_ARG, "fs3d_world_load: bad args");
    *out = nullptr;
    FILE* f = fopen(path, "rb");
    if (!f) return set_error(FS3D_ERR_IO, std::string("fs3d_world_load: cannot open ") + path);
    CkpHeader h{};
    if (fread(&h, sizeof(h), 1, f) != 1 || memcmp(h.magic, "FS3DCKP1", 8) != 0 || h.version != 1 ||
        !dims_ok(h.X, h.Y, h.Z)) {
        fclose(f);
        return set_error(FS3D_ERR_IO, "fs3d_world_load: not an fs3d checkpoint");
    }
    std::vector<uint8_t> g((size_t)h.X * h.Y * h.Z);
    const bool ok = fread(g.data(), 1, g.size(), f) == g.size();
    fclose(f);
    if (!ok) return set_error(FS3D_ERR_IO, "fs3d_world_load: truncated checkpoint");
    return fs3d_world_create(g.data(), h.X, h.Y, h.Z, h.seed, h.step, layout, out);
}

// ---- render ----
fs3d_status fs3d_render(fs3d_world* w, const fs3d_camera* cam, int W, int H, int mode, float* rgba,
                        int out_on_device) {
    if (!w || !cam || !rgba || W <= 0 || H <= 0 || (mode != FS3D_RENDER_DDA && mode != FS3D_RENDER_SDF_SPHERE))
        return set_error(FS3D_ERR_INVALID_ARG, "fs3d_render: bad args");
    float* dst = rgba;
    const size_t bytes = (size_t)W * H * 4 * sizeof(float);
    if (mode == FS3D_RENDER_DDA && !w->brickmap)
        FS3D_CUDA(cudaMalloc((void**)&w->brickmap, brickmap_bytes(w->X, w->Y, w->Z)));
    // planes worlds stepped by the per-step kernel keep exact brick counts
    if (mode == FS3D_RENDER_DDA && w->layout == FS3D_LAYOUT_PLANES && w->cls < 0 && !w->brick_counts)
        FS3D_CUDA(cudaMalloc((void**)&w->brick_counts, brick_count_bytes(w->X, w->Y, w->Z)));
    if (!out_on_device) FS3D_CUDA(cudaMallocAsync((void**)&dst, bytes, w->stream));
    fs3d_status s;
    if (mode == FS3D_RENDER_SDF_SPHERE)
        s = launch_render_sdf(cam, W, H, dst, w->stream);
    else if (w->layout == FS3D_LAYOUT_BYTES)
        s = launch_render_dda_bytes(w->bytes, w->X, w->Y, w->Z, w->brickmap, cam, W, H, dst, w->stream);
    else {
        s = launch_render_dda_planes(w->rows, w->statics, w->X, w->Y, w->Z, plane_nw(w->X), w->brickmap, cam, W, H, dst,
                                     w->stream, w->brick_counts, !w->counts_valid);
        if (s == FS3D_OK && w->brick_counts) w->counts_valid = true;
    }
    if (!out_on_device) {
        cudaError_t e = cudaSuccess;
        if (s == FS3D_OK) e = cudaMemcpyAsync(rgba, dst, bytes, cudaMemcpyDeviceToHost, w->stream);
        cudaFreeAsync(dst, w->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(w->stream);
        if (s == FS3D_OK && e != cudaSuccess) s = cuda_fail(e, "fs3d_render readback");
    }
    return s;
}

}  // extern "C"
