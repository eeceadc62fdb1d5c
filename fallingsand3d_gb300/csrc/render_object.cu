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

#include <vector>

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

// ---- mesh materials: basic_mat / textured_mat / tri ------------------------
// Restated pipelines: basic_mat.{vert,frag} (flat colour), textured_mat (the
// colour plus the texel, alpha + 1), tri (the texel, alpha 1), with the
// fixed-function state they are drawn with (no culling, depth LESS_OR_EQUAL
// against 1, one sample per pixel, NEAREST filtering with REPEAT addressing
// of R8G8B8A8_SRGB textures).  Three passes: per primitive, transform by
// P*V*model and clip against 0 <= z <= w (Vulkan's depth range) into up to
// three screen triangles; per screen triangle, test the pixel centres of its
// box with edge functions and keep per pixel the smallest 64-bit key
// (depth bits, then the later primitive first: LESS_OR_EQUAL lets a later
// fragment at equal depth win); per pixel, shade the winner with
// perspective-correct texture coordinates.  The order in which fragments
// arrive does not matter, so the frame is deterministic and equals the CPU
// restatement bit for bit (every float operation single-rounded, in the same
// order).

struct MeshDrawDev {
    float mvp[16];
    float color[4];
    const float* verts;
    const uint8_t* tex;
    int tex_w, tex_h, material, n_tri;
    long long prim0;
};

struct ScrTri {
    float sx[3], sy[3], sz[3], iw[3], uw[3], vw[3];
    float area;
    int tl;
    int valid;
};

struct ClipVtx {
    float x, y, z, w, u, v;
};

__device__ __forceinline__ int floor_to_int_dev(float x) {
    if (x != x) return 0;
    x = floorf(x);
    if (x >= 2147483647.0f) return 2147483647;
    if (x <= -2147483648.0f) return -2147483647 - 1;
    return (int)x;
}

__device__ __forceinline__ ClipVtx clip_lerp_dev(const ClipVtx& a, const ClipVtx& b, float t) {
    ClipVtx r;
    r.x = __fadd_rn(a.x, __fmul_rn(t, __fsub_rn(b.x, a.x)));
    r.y = __fadd_rn(a.y, __fmul_rn(t, __fsub_rn(b.y, a.y)));
    r.z = __fadd_rn(a.z, __fmul_rn(t, __fsub_rn(b.z, a.z)));
    r.w = __fadd_rn(a.w, __fmul_rn(t, __fsub_rn(b.w, a.w)));
    r.u = __fadd_rn(a.u, __fmul_rn(t, __fsub_rn(b.u, a.u)));
    r.v = __fadd_rn(a.v, __fmul_rn(t, __fsub_rn(b.v, a.v)));
    return r;
}

// keeps the part with d >= 0, d = z (plane 0) or w - z (plane 1)
__device__ __forceinline__ int clip_plane_dev(const ClipVtx* in, int n, ClipVtx* out, int plane) {
    int m = 0;
    for (int i = 0; i < n; ++i) {
        const ClipVtx& a = in[i];
        const ClipVtx& b = in[(i + 1) % n];
        const float da = plane ? __fsub_rn(a.w, a.z) : a.z, db = plane ? __fsub_rn(b.w, b.z) : b.z;
        if (da >= 0.0f) out[m++] = a;
        if ((da >= 0.0f) != (db >= 0.0f)) out[m++] = clip_lerp_dev(a, b, __fdiv_rn(da, __fsub_rn(da, db)));
    }
    return m;
}

__device__ __forceinline__ float dot4_dev(float m0, float m1, float m2, float m3, const float* p) {
    return __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(m0, p[0]), __fmul_rn(m1, p[1])), __fmul_rn(m2, p[2])), m3);
}

__device__ __forceinline__ int top_left_dev(float ax, float ay, float bx, float by) {
    return by < ay || (by == ay && bx > ax);
}

// the draw holding primitive p: the last one whose first primitive is <= p
__device__ __forceinline__ int find_draw(const MeshDrawDev* __restrict__ draws, int n_draws, long long p) {
    int lo = 0, hi = n_draws - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (draws[mid].prim0 <= p)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

__global__ void k_mesh_setup(const MeshDrawDev* __restrict__ draws, int n_draws, long long n_prims, int W, int H,
                             ScrTri* __restrict__ tris) {
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n_prims) return;
    const int d = find_draw(draws, n_draws, p);
    const MeshDrawDev& dr = draws[d];
    const float* v = dr.verts + 15 * (p - dr.prim0);
    const float* m = dr.mvp;
    ClipVtx a[8], b[8];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float* q = v + 5 * k;
        a[k].x = dot4_dev(m[0], m[4], m[8], m[12], q);
        a[k].y = dot4_dev(m[1], m[5], m[9], m[13], q);
        a[k].z = dot4_dev(m[2], m[6], m[10], m[14], q);
        a[k].w = dot4_dev(m[3], m[7], m[11], m[15], q);
        a[k].u = q[3];
        a[k].v = q[4];
    }
    int n = clip_plane_dev(a, 3, b, 0);
    n = clip_plane_dev(b, n, a, 1);
    const float hw = __fmul_rn((float)W, 0.5f), hh = __fmul_rn((float)H, 0.5f);
    for (int t = 0; t < 3; ++t) {
        ScrTri s;
        s.valid = 0;
        bool ok = t + 2 < n;
        const int idx[3] = {0, t + 1, t + 2};
        for (int k = 0; k < 3 && ok; ++k) {
            const ClipVtx& c = a[idx[k]];
            if (!(c.w > 0.0f)) {
                ok = false;
                break;
            }
            s.sx[k] = __fadd_rn(__fmul_rn(__fdiv_rn(c.x, c.w), hw), hw);
            s.sy[k] = __fadd_rn(__fmul_rn(__fdiv_rn(c.y, c.w), hh), hh);
            s.sz[k] = __fdiv_rn(c.z, c.w);
            s.iw[k] = __fdiv_rn(1.0f, c.w);
            s.uw[k] = __fmul_rn(c.u, s.iw[k]);
            s.vw[k] = __fmul_rn(c.v, s.iw[k]);
        }
        if (ok) {
            s.area = edge_dev(s.sx[0], s.sy[0], s.sx[1], s.sy[1], s.sx[2], s.sy[2]);
            ok = !(s.area == 0.0f || s.area != s.area);
        }
        if (ok) {
            if (s.area < 0.0f) {
                float* f[6] = {s.sx, s.sy, s.sz, s.iw, s.uw, s.vw};
                for (int q = 0; q < 6; ++q) {
                    const float x = f[q][1];
                    f[q][1] = f[q][2];
                    f[q][2] = x;
                }
                s.area = -s.area;
            }
            s.tl = top_left_dev(s.sx[1], s.sy[1], s.sx[2], s.sy[2]) | top_left_dev(s.sx[2], s.sy[2], s.sx[0], s.sy[0]) << 1 |
                   top_left_dev(s.sx[0], s.sy[0], s.sx[1], s.sy[1]) << 2;
            s.valid = 1;
        }
        tris[3 * p + t] = s;
    }
}

__device__ __forceinline__ bool tri_cover_dev(const ScrTri& s, float fx, float fy, float (&l)[3]) {
    const float w0 = edge_dev(s.sx[1], s.sy[1], s.sx[2], s.sy[2], fx, fy);
    const float w1 = edge_dev(s.sx[2], s.sy[2], s.sx[0], s.sy[0], fx, fy);
    const float w2 = edge_dev(s.sx[0], s.sy[0], s.sx[1], s.sy[1], fx, fy);
    if (!inside_edge(w0, s.tl, 0) || !inside_edge(w1, s.tl, 1) || !inside_edge(w2, s.tl, 2)) return false;
    l[0] = __fdiv_rn(w0, s.area);
    l[1] = __fdiv_rn(w1, s.area);
    l[2] = __fdiv_rn(w2, s.area);
    return true;
}

// one warp per screen triangle: the lanes walk the pixels of its box
__global__ void k_mesh_cover(const ScrTri* __restrict__ tris, long long n_slots, int W, int H,
                             unsigned long long* __restrict__ key) {
    const int lane = threadIdx.x & 31;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long sl = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; sl < n_slots; sl += nwarps) {
        const ScrTri& s = tris[sl];
        if (!s.valid) continue;
        const float xmin = fminf(fminf(s.sx[0], s.sx[1]), s.sx[2]), xmax = fmaxf(fmaxf(s.sx[0], s.sx[1]), s.sx[2]);
        const float ymin = fminf(fminf(s.sy[0], s.sy[1]), s.sy[2]), ymax = fmaxf(fmaxf(s.sy[0], s.sy[1]), s.sy[2]);
        const int x0 = max(0, floor_to_int_dev(xmin)), x1 = min(W - 1, floor_to_int_dev(ceilf(xmax)));
        const int y0 = max(0, floor_to_int_dev(ymin)), y1 = min(H - 1, floor_to_int_dev(ceilf(ymax)));
        if (x0 > x1 || y0 > y1) continue;
        const long long bw = x1 - x0 + 1, npx = bw * (long long)(y1 - y0 + 1);
        const uint32_t code = 0xFFFFFFFFu - (uint32_t)sl / 3u * 4u - (uint32_t)(sl % 3);
        for (long long i = lane; i < npx; i += 32) {
            const int px = x0 + (int)(i % bw), py = y0 + (int)(i / bw);
            float l[3];
            if (!tri_cover_dev(s, __fadd_rn((float)px, 0.5f), __fadd_rn((float)py, 0.5f), l)) continue;
            const float z = lerp3(l[0], l[1], l[2], s.sz);
            if (!(z >= 0.0f && z <= 1.0f)) continue;
            const unsigned long long k = ((unsigned long long)__float_as_uint(z) << 32) | code;
            atomicMin(key + (size_t)py * W + px, k);
        }
    }
}

__device__ __forceinline__ float clamp01_dev(float x) { return x < 0.0f ? 0.0f : (x > 1.0f ? 1.0f : x); }

__global__ void k_mesh_resolve(const MeshDrawDev* __restrict__ draws, int n_draws, const ScrTri* __restrict__ tris,
                               const unsigned long long* __restrict__ key, const float* __restrict__ lut, int W, int H,
                               float c0, float c1, float c2, float c3, float4* __restrict__ out) {
    const int px = blockIdx.x * blockDim.x + threadIdx.x;
    const int py = blockIdx.y * blockDim.y + threadIdx.y;
    if (px >= W || py >= H) return;
    const unsigned long long k = key[(size_t)py * W + px];
    if (k == ~0ull) {
        out[(size_t)py * W + px] = make_float4(c0, c1, c2, c3);
        return;
    }
    const uint32_t code = 0xFFFFFFFFu - (uint32_t)(k & 0xFFFFFFFFull);
    const long long prim = code >> 2;
    const int q = (int)(code & 3u);
    const int d = find_draw(draws, n_draws, prim);
    const MeshDrawDev& dr = draws[d];
    const ScrTri& s = tris[3 * prim + q];
    float l[3];
    tri_cover_dev(s, __fadd_rn((float)px, 0.5f), __fadd_rn((float)py, 0.5f), l);
    float r = dr.color[0], g = dr.color[1], b = dr.color[2], a = dr.color[3];
    if (dr.material != FS3D_MAT_BASIC) {
        const float den = lerp3(l[0], l[1], l[2], s.iw);
        const float u = __fdiv_rn(lerp3(l[0], l[1], l[2], s.uw), den);
        const float v = __fdiv_rn(lerp3(l[0], l[1], l[2], s.vw), den);
        int ti = floor_to_int_dev(__fmul_rn(u, (float)dr.tex_w)) % dr.tex_w;
        int tj = floor_to_int_dev(__fmul_rn(v, (float)dr.tex_h)) % dr.tex_h;
        if (ti < 0) ti += dr.tex_w;
        if (tj < 0) tj += dr.tex_h;
        const uchar4 t = reinterpret_cast<const uchar4*>(dr.tex)[(size_t)tj * dr.tex_w + ti];
        const float tr = lut[t.x], tg = lut[t.y], tb = lut[t.z];
        if (dr.material == FS3D_MAT_TEXTURED) {
            r = __fadd_rn(r, tr);
            g = __fadd_rn(g, tg);
            b = __fadd_rn(b, tb);
            a = __fadd_rn(a, 1.0f);
        } else {
            r = tr;
            g = tg;
            b = tb;
            a = 1.0f;
        }
    }
    out[(size_t)py * W + px] = make_float4(clamp01_dev(r), clamp01_dev(g), clamp01_dev(b), clamp01_dev(a));
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

extern "C" fs3d_status fs3d_render_meshes(const fs3d_object_view* v, const fs3d_mesh_draw* draws, int n_draws, int W,
                                          int H, float* rgba_dev, void* stream) {
    using namespace fs3d;
    if (!v || (n_draws > 0 && !draws) || n_draws < 0 || n_draws > 65536 || !rgba_dev || W <= 0 || H <= 0)
        return set_error(FS3D_ERR_INVALID_ARG, "fs3d_render_meshes: bad args");
    cudaStream_t st = (cudaStream_t)stream;
    fs3d_object_view cam = *v;
    for (int i = 0; i < 16; ++i) cam.model[i] = (i % 5 == 0) ? 1.0f : 0.0f;
    float vp[16];
    object_mvp(&cam, vp);
    std::vector<MeshDrawDev> dd((size_t)(n_draws > 0 ? n_draws : 1));
    long long prims = 0;
    // draws usually share their buffers: look each distinct pointer up once
    const void* last_v = nullptr;
    const void* last_t = nullptr;
    const uint8_t* last_vdev = nullptr;
    const uint8_t* last_tdev = nullptr;
    for (int d = 0; d < n_draws; ++d) {
        const fs3d_mesh_draw& m = draws[d];
        if (m.n_vertices < 0 || m.n_vertices % 3 || (m.n_vertices && !m.vertices) || m.material < FS3D_MAT_BASIC ||
            m.material > FS3D_MAT_TEXTURE ||
            (m.material != FS3D_MAT_BASIC && (!m.texture || m.tex_width <= 0 || m.tex_height <= 0)))
            return set_error(FS3D_ERR_INVALID_ARG, "fs3d_render_meshes: bad draw");
        // the kernels read the vertices and texels: they must be device or
        // page-locked memory (used through its device alias), 4-byte aligned
        const uint8_t* vdev = nullptr;
        const uint8_t* tdev = nullptr;
        if (m.n_vertices) {
            if (m.vertices != last_v) {
                last_v = m.vertices;
                last_vdev = device_view(m.vertices);
            }
            vdev = last_vdev;
        }
        if (m.material != FS3D_MAT_BASIC) {
            if (m.texture != last_t) {
                last_t = m.texture;
                last_tdev = device_view(m.texture);
            }
            tdev = last_tdev;
        }
        if ((m.n_vertices && (!vdev || (reinterpret_cast<uintptr_t>(vdev) & 3))) ||
            (m.material != FS3D_MAT_BASIC && (!tdev || (reinterpret_cast<uintptr_t>(tdev) & 3))))
            return set_error(FS3D_ERR_INVALID_ARG,
                             "fs3d_render_meshes: vertices and textures must be 4-byte aligned device or page-locked memory");
        MeshDrawDev& x = dd[(size_t)d];
        mat4_mul(vp, m.model, x.mvp);
        memcpy(x.color, m.color, sizeof(x.color));
        x.verts = reinterpret_cast<const float*>(vdev);
        x.tex = tdev;
        x.tex_w = m.tex_width;
        x.tex_h = m.tex_height;
        x.material = m.material;
        x.n_tri = m.n_vertices / 3;
        x.prim0 = prims;
        prims += x.n_tri;
    }
    if (prims >= (1ll << 30)) return set_error(FS3D_ERR_INVALID_ARG, "fs3d_render_meshes: too many triangles");
    // sRGB texels to linear, as the sampler of an _SRGB format does (built once)
    static const std::vector<float> lut = [] {
        std::vector<float> t(256);
        for (int i = 0; i < 256; ++i) {
            const double c = i / 255.0;
            t[(size_t)i] = (float)(c <= 0.04045 ? c / 12.92 : pow((c + 0.055) / 1.055, 2.4));
        }
        return t;
    }();
    const size_t draws_b = sizeof(MeshDrawDev) * dd.size(), lut_b = sizeof(float) * 256;
    const size_t tris_b = sizeof(ScrTri) * 3 * (size_t)(prims > 0 ? prims : 1), key_b = sizeof(unsigned long long) * W * H;
    const size_t o_lut = (draws_b + 255) & ~(size_t)255, o_tris = (o_lut + lut_b + 255) & ~(size_t)255,
                 o_key = (o_tris + tris_b + 255) & ~(size_t)255;
    char* scratch = nullptr;
    FS3D_CUDA(cudaMallocAsync((void**)&scratch, o_key + key_b, st));
    MeshDrawDev* ddev = reinterpret_cast<MeshDrawDev*>(scratch);
    float* lut_dev = reinterpret_cast<float*>(scratch + o_lut);
    ScrTri* tris = reinterpret_cast<ScrTri*>(scratch + o_tris);
    unsigned long long* key = reinterpret_cast<unsigned long long*>(scratch + o_key);
    cudaError_t e = cudaMemcpyAsync(ddev, dd.data(), draws_b, cudaMemcpyHostToDevice, st);  // pageable: staged
    if (e == cudaSuccess) e = cudaMemcpyAsync(lut_dev, lut.data(), lut_b, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(key, 0xFF, key_b, st);
    fs3d_status s = e == cudaSuccess ? FS3D_OK : cuda_fail(e, "fs3d_render_meshes upload");
    if (s == FS3D_OK && prims > 0) {
        k_mesh_setup<<<(unsigned)((prims + 127) / 128), 128, 0, st>>>(ddev, n_draws, prims, W, H, tris);
        s = FS3D_OK;
        if (cudaGetLastError() != cudaSuccess) s = set_error(FS3D_ERR_CUDA, "mesh setup launch");
        if (s == FS3D_OK) {
            const long long slots = 3 * prims, warps_per_block = 8;
            long long blocks = (slots + warps_per_block - 1) / warps_per_block;
            const long long cap = (long long)sm_count_public() * 16;
            if (blocks > cap) blocks = cap;
            k_mesh_cover<<<(unsigned)blocks, 256, 0, st>>>(tris, slots, W, H, key);
            if (cudaGetLastError() != cudaSuccess) s = set_error(FS3D_ERR_CUDA, "mesh cover launch");
        }
        note_launch(2);
    }
    if (s == FS3D_OK) {
        const dim3 blk(16, 16), grd((W + 15) / 16, (H + 15) / 16);
        k_mesh_resolve<<<grd, blk, 0, st>>>(ddev, n_draws, tris, key, lut_dev, W, H, v->clear[0], v->clear[1],
                                            v->clear[2], v->clear[3], reinterpret_cast<float4*>(rgba_dev));
        if (cudaGetLastError() != cudaSuccess) s = set_error(FS3D_ERR_CUDA, "mesh resolve launch");
        note_launch(1);
    }
    cudaFreeAsync(scratch, st);
    return s;
}
