// fs3d_run_device: n steps of a caller-owned device byte grid through the bit
// plane kernels.  The grid is converted once into 2-bit planes (scratch), the
// steps run there (all of them in one resident launch when the world fits in
// shared memory, one per-step launch each otherwise), and the planes are
// converted back.  Static cells never change, so their byte values are read
// back from the caller's grid itself.  Rows wider than 2048 cells take the
// byte kernels instead.
#include <vector>

#include "fs3d_common.h"
#include "planes.h"

using namespace fs3d;

namespace {

// device scratch of one run: the planes and the one-world step tables
struct RunScratch {
    uint4* rows = nullptr;
    PlaneWorld* desc = nullptr;
    int* ints = nullptr;  // meta (1 + 2*classes), order[0], counter, error flag
    PlaneItem* items = nullptr;
};

constexpr int kOrder = kMetaInts, kCounter = kOrder + 1, kErr = kCounter + 1, kInts = kErr + 1;

}  // namespace

extern "C" fs3d_status fs3d_run_device(uint8_t* grid_dev, int X, int Y, int Z, uint64_t seed, uint64_t t0,
                                       int n_steps, void* stream) {
    if (!grid_dev || X <= 0 || Y <= 0 || Z <= 0 || X > (1 << 20) || Y > (1 << 20) || Z > (1 << 20) || n_steps < 0)
        return set_error(FS3D_ERR_INVALID_ARG, "fs3d_run_device: null grid, bad dims or negative n_steps");
    cudaStream_t st = (cudaStream_t)stream;
    if (n_steps == 0) return FS3D_OK;
    if (X > kPlaneMaxX) return launch_step_bytes(grid_dev, X, Y, Z, seed, t0, n_steps, st);
    const int nw = plane_nw(X), lg = plane_lg(nw), cls = resident_class(X, Y, Z);
    const int n_items = cls >= 0 ? 0 : plane_items_for(Y, Z, nw);
    RunScratch sc;
    cudaError_t e = cudaMallocAsync((void**)&sc.rows, plane_bytes(X, Y, Z), st);
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&sc.desc, sizeof(PlaneWorld), st);
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&sc.ints, sizeof(int) * kInts, st);
    if (e == cudaSuccess && n_items) e = cudaMallocAsync((void**)&sc.items, sizeof(PlaneItem) * n_items, st);
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
    int ints[kInts] = {};
    ints[0] = n_items;
    if (cls >= 0) ints[1 + cls] = 1;
    std::vector<PlaneItem> items((size_t)n_items);
    for (int a = 0; a < n_items; ++a) items[(size_t)a] = PlaneItem{0, a * (32 >> lg)};
    // pageable sources: staged before each call returns
    if (s == FS3D_OK) e = cudaMemcpyAsync(sc.desc, &d, sizeof(d), cudaMemcpyHostToDevice, st);
    if (s == FS3D_OK && e == cudaSuccess) e = cudaMemcpyAsync(sc.ints, ints, sizeof(ints), cudaMemcpyHostToDevice, st);
    if (s == FS3D_OK && e == cudaSuccess && n_items)
        e = cudaMemcpyAsync(sc.items, items.data(), sizeof(PlaneItem) * n_items, cudaMemcpyHostToDevice, st);
    if (s == FS3D_OK && e != cudaSuccess) s = cuda_fail(e, "fs3d_run_device tables");
    if (s == FS3D_OK) s = planes_from_bytes(grid_dev, X, Y, Z, sc.rows, st);
    if (s == FS3D_OK) {
        if (cls >= 0) {
            s = launch_plane_segment_resident(cls, sc.desc, sc.ints + kOrder, sc.ints, sc.ints + kCounter,
                                              sc.ints + kErr, st);
        } else {
            const int grid = plane_step_grid(n_items);
            for (int a = 0; a < n_steps && s == FS3D_OK; ++a)
                s = launch_plane_step(sc.desc, sc.items, sc.ints, grid, a, st);
        }
    }
    if (s == FS3D_OK) s = planes_to_bytes(sc.rows, grid_dev, X, Y, Z, grid_dev, st);
    cudaFreeAsync(sc.rows, st);
    cudaFreeAsync(sc.desc, st);
    cudaFreeAsync(sc.ints, st);
    if (sc.items) cudaFreeAsync(sc.items, st);
    return s;
}
