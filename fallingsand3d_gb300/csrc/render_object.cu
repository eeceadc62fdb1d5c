// The raymarch_sphere material, the one object the upstream scene draws
// (renderer.cpp:1320-1326: the cube mesh with this material, identity model).
//
// Upstream it is a Vulkan pipeline: raymarch_sphere.vert:30-45 transforms the
// cube's vertices by viewproj*model and passes two noperspective attributes,
// the camera in object space invModel*(-camPos) and the object-space vertex;
// the rasteriser covers pixels with no culling (pipelines.cpp:114) and keeps
// the nearest fragment under LESS_OR_EQUAL against depth cleared to 1
// (renderer.cpp:502-503, 1233); raymarch_sphere.frag:18-51 marches a box SDF
// of half-extent 0.5 from the object-space camera along
// normalize(localPos - origin) for at most 64 steps, colour
// (max(0.05, 1 - 0.05*steps), 0, 0) on a hit and black on a miss.
//
// Here the fixed-function part is written out: the host transforms the mesh
// (matrices of materials.cpp:531-545, column-major, sums left to right),
// orients each triangle, and marks its top-left edges; one thread per pixel
// tests the pixel centre against every triangle with edge functions,
// interpolates depth and position linearly in screen space (noperspective),
// keeps the nearest, and marches.  Built with --fmad=false and explicit
// round-to-nearest intrinsics, so the frame is bit-identical to a CPU that
// evaluates the same expressions in the same order.  Near/far clipping is not
// restated: a vertex outside the depth range is rejected.
#include <math.h>
#include <string.h>

#include "fs3d_common.h"
#include "planes.h"

namespace fs3d {

constexpr int kObjectMaxTris = 48;  // keeps the launch parameters under 4 KB

struct ObjTri {
    float sx[3], sy[3], sz[3];  // screen position (pixels, y down) and depth
    float ax[3], ay[3], az[3];  // object-space position (the noperspective attribute)
    float area;                 // twice the signed screen area after orientation (> 0), else skipped
    int tl;                     // bit k: edge opposite vertex k is a top or left edge
};

struct ObjScene {
    float o[3];      // camera in object space
    float clear[4];  // colour where no triangle covers the pixel
    int ntri;
    ObjTri t[kObjectMaxTris];
};
static_assert(sizeof(ObjScene) + 32 < 4096, "object scene must fit the launch parameters");

// ---- host: matrices and triangle set-up (same expressions as the CPU restatement)

static void mat4_mul(const float* a, const float* b, float* out) {
    float r[16];
    for (int c = 0; c < 4; ++c)
        for (int i = 0; i < 4; ++i)
            r[c * 4 + i] = a[0 * 4 + i] * b[c * 4 + 0] + a[1 * 4 + i] * b[c * 4 + 1] + a[2 * 4 + i] * b[c * 4 + 2] +
                           a[3 * 4 + i] * b[c * 4 + 3];
    memcpy(out, r, sizeof(r));
}

// Inverse from the 2x2 minors of the upper and lower row pairs (Laplace
// expansion, D. Eberly, "The Laplace Expansion Theorem", 2008).
static bool mat4_inverse(const float* m, float* out) {
    auto a = [m](int r, int c) { return m[c * 4 + r]; };
    const float s0 = a(0, 0) * a(1, 1) - a(1, 0) * a(0, 1), s1 = a(0, 0) * a(1, 2) - a(1, 0) * a(0, 2);
    const float s2 = a(0, 0) * a(1, 3) - a(1, 0) * a(0, 3), s3 = a(0, 1) * a(1, 2) - a(1, 1) * a(0, 2);
    const float s4 = a(0, 1) * a(1, 3) - a(1, 1) * a(0, 3), s5 = a(0, 2) * a(1, 3) - a(1, 2) * a(0, 3);
    const float c5 = a(2, 2) * a(3, 3) - a(3, 2) * a(2, 3), c4 = a(2, 1) * a(3, 3) - a(3, 1) * a(2, 3);
    const float c3 = a(2, 1) * a(3, 2) - a(3, 1) * a(2, 2), c2 = a(2, 0) * a(3, 3) - a(3, 0) * a(2, 3);
    const float c1 = a(2, 0) * a(3, 2) - a(3, 0) * a(2, 2), c0 = a(2, 0) * a(3, 1) - a(3, 0) * a(2, 1);
    const float det = s0 * c5 - s1 * c4 + s2 * c3 + s3 * c2 - s4 * c1 + s5 * c0;
    if (det == 0.0f || det != det) return false;
    const float k = 1.0f / det;
    float b[16];
    auto set = [&b](int r, int c, float v) { b[c * 4 + r] = v; };
    set(0, 0, (a(1, 1) * c5 - a(1, 2) * c4 + a(1, 3) * c3) * k);
    set(0, 1, (-a(0, 1) * c5 + a(0, 2) * c4 - a(0, 3) * c3) * k);
    set(0, 2, (a(3, 1) * s5 - a(3, 2) * s4 + a(3, 3) * s3) * k);
    set(0, 3, (-a(2, 1) * s5 + a(2, 2) * s4 - a(2, 3) * s3) * k);
    set(1, 0, (-a(1, 0) * c5 + a(1, 2) * c2 - a(1, 3) * c1) * k);
    set(1, 1, (a(0, 0) * c5 - a(0, 2) * c2 + a(0, 3) * c1) * k);
    set(1, 2, (-a(3, 0) * s5 + a(3, 2) * s2 - a(3, 3) * s1) * k);
    set(1, 3, (a(2, 0) * s5 - a(2, 2) * s2 + a(2, 3) * s1) * k);
    set(2, 0, (a(1, 0) * c4 - a(1, 1) * c2 + a(1, 3) * c0) * k);
    set(2, 1, (-a(0, 0) * c4 + a(0, 1) * c2 - a(0, 3) * c0) * k);
    set(2, 2, (a(3, 0) * s4 - a(3, 1) * s2 + a(3, 3) * s0) * k);
    set(2, 3, (-a(2, 0) * s4 + a(2, 1) * s2 - a(2, 3) * s0) * k);
    set(3, 0, (-a(1, 0) * c3 + a(1, 1) * c1 - a(1, 2) * c0) * k);
    set(3, 1, (a(0, 0) * c3 - a(0, 1) * c1 + a(0, 2) * c0) * k);
    set(3, 2, (-a(3, 0) * s3 + a(3, 1) * s1 - a(3, 2) * s0) * k);
    set(3, 3, (a(2, 0) * s3 - a(2, 1) * s1 + a(2, 2) * s0) * k);
    memcpy(out, b, sizeof(b));
    return true;
}

// projection (gluPerspective form, OpenGL depth range, y negated for
// Vulkan) * rotation about y by camRot.y * translation by camPos * model
static void object_mvp(const fs3d_object_view* v, float* mvp) {
    const float fovy = v->fovy_deg * 0.0174532925199432957692f;
    const float th = tanf(fovy * 0.5f);
    float P[16] = {0};
    P[0] = 1.0f / (v->aspect * th);
    P[5] = -(1.0f / th);
    P[10] = -(v->zfar + v->znear) / (v->zfar - v->znear);
    P[11] = -1.0f;
    P[14] = -(2.0f * v->zfar * v->znear) / (v->zfar - v->znear);
    const float ang = v->cam_rot_y_deg * 0.0174532925199432957692f;
    const float c = cosf(ang), s = sinf(ang);
    const float R[16] = {c, 0, -s, 0, 0, 1, 0, 0, s, 0, c, 0, 0, 0, 0, 1};
    const float T[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, v->cam_pos[0], v->cam_pos[1], v->cam_pos[2], 1};
    float V[16];
    mat4_mul(R, T, V);
    mat4_mul(P, V, mvp);
    mat4_mul(mvp, v->model, mvp);
}

static inline float edge_host(float ax, float ay, float bx, float by, float px, float py) {
    return (bx - ax) * (py - ay) - (by - ay) * (px - ax);
}
static inline int top_left_host(float ax, float ay, float bx, float by) {
    return by < ay || (by == ay && bx > ax);
}

static fs3d_status object_setup(const fs3d_object_view* v, const float* tri, int ntri, int W, int H,
                                ObjScene* sc) {
    memset(sc, 0, sizeof(*sc));
    float mvp[16], inv[16];
    object_mvp(v, mvp);
    if (!mat4_inverse(v->model, inv)) return set_error(FS3D_ERR_INVALID_ARG, "fs3d_render_object: singular model");
    const float ncp[3] = {-v->cam_pos[0], -v->cam_pos[1], -v->cam_pos[2]};
    for (int i = 0; i < 3; ++i)
        sc->o[i] = inv[0 * 4 + i] * ncp[0] + inv[1 * 4 + i] * ncp[1] + inv[2 * 4 + i] * ncp[2] + inv[3 * 4 + i];
    memcpy(sc->clear, v->clear, sizeof(sc->clear));
    sc->ntri = ntri;
    const float hw = (float)W * 0.5f, hh = (float)H * 0.5f;
    for (int t = 0; t < ntri; ++t) {
        float s[3][3], at[3][3];
        for (int k = 0; k < 3; ++k) {
            const float* p = tri + 9 * t + 3 * k;
            float cl[4];
            for (int i = 0; i < 4; ++i)
                cl[i] = mvp[0 * 4 + i] * p[0] + mvp[1 * 4 + i] * p[1] + mvp[2 * 4 + i] * p[2] + mvp[3 * 4 + i];
            if (!(cl[3] > 0.0f))
                return set_error(FS3D_ERR_INVALID_ARG, "fs3d_render_object: a vertex is behind the camera");
            const float nx = cl[0] / cl[3], ny = cl[1] / cl[3], nz = cl[2] / cl[3];
            if (!(nz >= 0.0f && nz <= 1.0f))
                return set_error(FS3D_ERR_INVALID_ARG,
                                 "fs3d_render_object: a vertex lies outside the depth range (clipping is not done)");
            s[k][0] = nx * hw + hw;
            s[k][1] = ny * hh + hh;
            s[k][2] = nz;
            memcpy(at[k], p, sizeof(at[k]));
        }
        float area = edge_host(s[0][0], s[0][1], s[1][0], s[1][1], s[2][0], s[2][1]);
        if (area < 0.0f) {  // orient counter-clockwise in y-down pixels: swap vertices 1 and 2
            for (int i = 0; i < 3; ++i) {
                float x = s[1][i];
                s[1][i] = s[2][i];
                s[2][i] = x;
                x = at[1][i];
                at[1][i] = at[2][i];
                at[2][i] = x;
            }
            area = edge_host(s[0][0], s[0][1], s[1][0], s[1][1], s[2][0], s[2][1]);
        }
        ObjTri& d = sc->t[t];
        for (int k = 0; k < 3; ++k) {
            d.sx[k] = s[k][0];
            d.sy[k] = s[k][1];
            d.sz[k] = s[k][2];
            d.ax[k] = at[k][0];
            d.ay[k] = at[k][1];
            d.az[k] = at[k][2];
        }
        d.area = area;
        d.tl = top_left_host(s[1][0], s[1][1], s[2][0], s[2][1]) | top_left_host(s[2][0], s[2][1], s[0][0], s[0][1]) << 1 |
               top_left_host(s[0][0], s[0][1], s[1][0], s[1][1]) << 2;
    }
    return FS3D_OK;
}

// ---- device

__device__ __forceinline__ float edge_dev(float ax, float ay, float bx, float by, float px, float py) {
    return __fsub_rn(__fmul_rn(__fsub_rn(bx, ax), __fsub_rn(py, ay)), __fmul_rn(__fsub_rn(by, ay), __fsub_rn(px, ax)));
}
__device__ __forceinline__ bool inside_edge(float w, int tl, int k) { return w > 0.0f || (w == 0.0f && ((tl >> k) & 1)); }
__device__ __forceinline__ float lerp3(float l0, float l1, float l2, const float* v) {
    return __fadd_rn(__fadd_rn(__fmul_rn(l0, v[0]), __fmul_rn(l1, v[1])), __fmul_rn(l2, v[2]));
}
__device__ __forceinline__ float box_sdf(float x, float y, float z) {
    const float qx = __fsub_rn(fabsf(x), 0.5f), qy = __fsub_rn(fabsf(y), 0.5f), qz = __fsub_rn(fabsf(z), 0.5f);
    const float mx = fmaxf(qx, 0.0f), my = fmaxf(qy, 0.0f), mz = fmaxf(qz, 0.0f);
    const float len = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(mx, mx), __fmul_rn(my, my)), __fmul_rn(mz, mz)));
    return __fadd_rn(len, fminf(fmaxf(qx, fmaxf(qy, qz)), 0.0f));
}

__global__ void k_render_object(const __grid_constant__ ObjScene sc, int W, int H, float4* __restrict__ out) {
    const int px = blockIdx.x * blockDim.x + threadIdx.x;
    const int py = blockIdx.y * blockDim.y + threadIdx.y;
    if (px >= W || py >= H) return;
    const float fx = __fadd_rn((float)px, 0.5f), fy = __fadd_rn((float)py, 0.5f);
    float best = 1.0f, pos[3] = {0.0f, 0.0f, 0.0f};
    bool hit = false;
    for (int t = 0; t < sc.ntri; ++t) {
        const ObjTri& T = sc.t[t];
        if (!(T.area > 0.0f)) continue;
        const float w0 = edge_dev(T.sx[1], T.sy[1], T.sx[2], T.sy[2], fx, fy);
        const float w1 = edge_dev(T.sx[2], T.sy[2], T.sx[0], T.sy[0], fx, fy);
        const float w2 = edge_dev(T.sx[0], T.sy[0], T.sx[1], T.sy[1], fx, fy);
        if (!inside_edge(w0, T.tl, 0) || !inside_edge(w1, T.tl, 1) || !inside_edge(w2, T.tl, 2)) continue;
        const float l0 = __fdiv_rn(w0, T.area), l1 = __fdiv_rn(w1, T.area), l2 = __fdiv_rn(w2, T.area);
        const float z = lerp3(l0, l1, l2, T.sz);
        if (!(z <= best)) continue;
        best = z;
        hit = true;
        pos[0] = lerp3(l0, l1, l2, T.ax);
        pos[1] = lerp3(l0, l1, l2, T.ay);
        pos[2] = lerp3(l0, l1, l2, T.az);
    }
    if (!hit) {
        out[(size_t)py * W + px] = make_float4(sc.clear[0], sc.clear[1], sc.clear[2], sc.clear[3]);
        return;
    }
    float d[3] = {__fsub_rn(pos[0], sc.o[0]), __fsub_rn(pos[1], sc.o[1]), __fsub_rn(pos[2], sc.o[2])};
    const float len = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(d[0], d[0]), __fmul_rn(d[1], d[1])), __fmul_rn(d[2], d[2])));
    d[0] = __fdiv_rn(d[0], len);
    d[1] = __fdiv_rn(d[1], len);
    d[2] = __fdiv_rn(d[2], len);
    float col = 0.0f, t = 0.0f, density = 1.0f;
    for (int it = 0; it < 64; ++it) {
        const float dist = box_sdf(__fadd_rn(sc.o[0], __fmul_rn(d[0], t)), __fadd_rn(sc.o[1], __fmul_rn(d[1], t)),
                                   __fadd_rn(sc.o[2], __fmul_rn(d[2], t)));
        if (dist < 0.001f) {
            col = fmaxf(0.05f, density);
            break;
        } else if (t > 1000.0f) {
            break;
        }
        t = __fadd_rn(t, dist);
        density = __fsub_rn(density, 0.05f);
    }
    out[(size_t)py * W + px] = make_float4(col, 0.0f, 0.0f, 1.0f);
}

}  // namespace fs3d

extern "C" {

void fs3d_object_view_scene(fs3d_object_view* v) {
    if (!v) return;
    memset(v, 0, sizeof(*v));
    v->cam_pos[2] = -5.0f;  // renderer.h:148
    v->fovy_deg = 70.0f;    // materials.cpp:533
    v->aspect = 1700.0f / 900.0f;
    v->znear = 0.01f;
    v->zfar = 200.0f;
    for (int i = 0; i < 4; ++i) v->model[i * 5] = 1.0f;
    v->clear[2] = 1.0f;  // renderer.cpp:499
    v->clear[3] = 1.0f;
}

int fs3d_mesh_cube(float* tri_xyz) {
    // assets/cube2.obj: eight corners of the +-1 cube and its twelve faces in file order
    static const float vtx[8][3] = {{1, 1, -1}, {1, -1, -1}, {1, 1, 1}, {1, -1, 1},
                                    {-1, 1, -1}, {-1, -1, -1}, {-1, 1, 1}, {-1, -1, 1}};
    static const int face[12][3] = {{5, 3, 1}, {3, 8, 4}, {7, 6, 8}, {2, 8, 6}, {1, 4, 2}, {5, 2, 6},
                                    {5, 7, 3}, {3, 7, 8}, {7, 5, 6}, {2, 4, 8}, {1, 3, 4}, {5, 1, 2}};
    if (tri_xyz)
        for (int t = 0; t < 12; ++t)
            for (int k = 0; k < 3; ++k) memcpy(tri_xyz + 9 * t + 3 * k, vtx[face[t][k] - 1], 3 * sizeof(float));
    return 12;
}

fs3d_status fs3d_render_object(const fs3d_object_view* v, const float* tri_xyz, int ntri, int W, int H,
                               float* rgba_dev, void* stream) {
    using namespace fs3d;
    if (!v || !tri_xyz || !rgba_dev || ntri < 0 || ntri > kObjectMaxTris || W <= 0 || H <= 0)
        return set_error(FS3D_ERR_INVALID_ARG, "fs3d_render_object: bad args (at most 48 triangles)");
    ObjScene sc;
    const fs3d_status s = object_setup(v, tri_xyz, ntri, W, H, &sc);
    if (s != FS3D_OK) return s;
    const dim3 blk(16, 16), grd((W + 15) / 16, (H + 15) / 16);
    k_render_object<<<grd, blk, 0, (cudaStream_t)stream>>>(sc, W, H, reinterpret_cast<float4*>(rgba_dev));
    FS3D_CHECK_LAUNCH("render object launch");
    return FS3D_OK;
}

}  // extern "C"
