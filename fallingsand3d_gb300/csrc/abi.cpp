// Library-level entry points: version, status strings, last-error message,
// launch accounting, default configuration and camera presets.
#include <math.h>
#include <string.h>

#include <atomic>
#include <string>
#include <utility>

#include "fs3d_common.h"
#include "planes.h"

namespace fs3d {

static thread_local std::string g_last_error;
static std::atomic<uint64_t> g_launches{0};

fs3d_status set_error(fs3d_status s, const std::string& msg) {
    g_last_error = msg;
    return s;
}

fs3d_status cuda_fail(cudaError_t e, const char* what) {
    g_last_error = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
    // the error is reported here: taken off the runtime's per-thread slot, so
    // that a later launch check of this thread does not report it again (an
    // error that leaves the context unusable keeps coming back regardless)
    cudaGetLastError();
    if (e == cudaErrorMemoryAllocation) return FS3D_ERR_OOM;
    return FS3D_ERR_CUDA;
}

void note_launch(uint64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

bool current_context_id(unsigned long long* id) {
    // cuCtxGetCurrent and cuCtxGetId, looked up once through the runtime (no
    // link dependency on the driver library)
    using GetCurrent = int (*)(void**);
    using GetId = int (*)(void*, unsigned long long*);
    static const std::pair<GetCurrent, GetId> fns = [] {
        void *a = nullptr, *b = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &a, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            a = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &b, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            b = nullptr;
        cudaGetLastError();
        return std::make_pair(reinterpret_cast<GetCurrent>(a), reinterpret_cast<GetId>(b));
    }();
    if (!fns.first || !fns.second) return false;
    void* ctx = nullptr;  // null: no context is current on this thread yet
    if (fns.first(&ctx) != 0 || !ctx) return false;
    return fns.second(ctx, id) == 0;
}

}  // namespace fs3d

extern "C" {

int fs3d_abi_version(void) { return FS3D_ABI_VERSION; }

const char* fs3d_status_string(fs3d_status s) {
    switch (s) {
        case FS3D_OK: return "ok";
        case FS3D_ERR_INVALID_ARG: return "invalid argument";
        case FS3D_ERR_OOM: return "out of device memory";
        case FS3D_ERR_BUDGET: return "over the memory budget";
        case FS3D_ERR_CUDA: return "CUDA error";
        case FS3D_ERR_TIMEOUT: return "timed out";
        case FS3D_ERR_MISMATCH: return "mismatch";
        case FS3D_ERR_STATE: return "invalid state";
        case FS3D_ERR_NOT_FOUND: return "not found";
        case FS3D_ERR_IO: return "i/o error";
        default: return "unknown status";
    }
}

const char* fs3d_last_error(void) { return fs3d::g_last_error.c_str(); }

uint64_t fs3d_kernel_launch_count(void) { return fs3d::g_launches.load(); }

fs3d_status fs3d_test_inject(int what, int count) {
    switch (what) {
        case FS3D_INJECT_NONE:
            fs3d::set_inject_alloc_failures(0);
            return fs3d::set_inject_tx_extra(0u);
        case FS3D_INJECT_COPY_STALL:
            return fs3d::set_inject_tx_extra(count > 0 ? 16u : 0u);
        case FS3D_INJECT_ALLOC_FAIL:
            fs3d::set_inject_alloc_failures(count);
            return FS3D_OK;
        default:
            return fs3d::set_error(FS3D_ERR_INVALID_ARG, "fs3d_test_inject: unknown injection");
    }
}

fs3d_config fs3d_default_config(void) {
    fs3d_config c;
    memset(&c, 0, sizeof(c));
    c.steps_per_segment = 64;
    c.use_graphs = 1;
    c.use_smem = 3;
    return c;
}

void fs3d_camera_fs_raymarch(fs3d_camera* cam) {
    if (!cam) return;
    memset(cam, 0, sizeof(*cam));
    cam->origin[2] = -5.0f;  // renderer.h:148 camPos {0,0,-5}
    cam->forward[2] = 1.0f;
    cam->right[0] = 1.0f;
    cam->up[1] = 1.0f;
    cam->tan_half_fov = 1.0f;
    cam->aspect = 1700.0f / 900.0f;  // materials.cpp:540
    cam->light_pos[0] = 2.0f;        // fs_raymarch.frag:51
    cam->light_pos[1] = 5.0f;
    cam->light_pos[2] = 3.0f;
}

void fs3d_camera_world_view(fs3d_camera* cam, int X, int Y, int Z, int W, int H) {
    if (!cam) return;
    memset(cam, 0, sizeof(*cam));
    const double o[3] = {-0.25 * X, 0.9 * Y, -0.25 * Z};
    const double c[3] = {0.5 * X, 0.5 * Y, 0.5 * Z};
    double f[3] = {c[0] - o[0], c[1] - o[1], c[2] - o[2]};
    double fl = sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
    for (double& v : f) v /= fl;
    // camera right = forward x world-up, camera up = right x forward
    double r[3] = {f[1] * 0.0 - f[2] * 1.0, f[2] * 0.0 - f[0] * 0.0, f[0] * 1.0 - f[1] * 0.0};
    double rl = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
    for (double& v : r) v /= rl;
    double u[3] = {r[1] * f[2] - r[2] * f[1], r[2] * f[0] - r[0] * f[2], r[0] * f[1] - r[1] * f[0]};
    for (int a = 0; a < 3; ++a) {
        cam->origin[a] = (float)o[a];
        cam->forward[a] = (float)f[a];
        // image x grows as ux falls and image y grows with uy (the fullscreen
        // quad's convention), so the basis is stored negated to keep the
        // picture upright and unmirrored
        cam->right[a] = (float)(-r[a]);
        cam->up[a] = (float)(-u[a]);
    }
    cam->tan_half_fov = (float)tan(35.0 * M_PI / 180.0);
    cam->aspect = (float)W / (float)H;
    // the fs_raymarch shading points its light vector away from the light,
    // so the light sits below the world to light the upward faces
    cam->light_pos[0] = (float)(0.3 * X);
    cam->light_pos[1] = (float)(-2.0 * Y);
    cam->light_pos[2] = (float)(0.2 * Z);
}

}  // extern "C"
