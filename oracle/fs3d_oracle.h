/*
 * fs3d oracle — CPU restatement of the falling-sand voxel step, its world
 * generators, the whole-grid hash and the two render paths.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: the parity tests,
 * the smoke check and the CPU-baseline leg of the benchmark load it.  The
 * product (libfs3d) never links, loads or calls it.
 *
 * Parity status: "parity unpinned" with respect to the upstream project.
 * The upstream FallingSand3D source tree contains no voxel update step
 * (src/engine holds only engine, window and rendering sources), so there is
 * nothing of its own to compile or compare against.  The step below follows
 * the written rule "FS3D-rule v1" (stated in full in fs3d_oracle.c and in
 * include/fs3d.h); golden hashes under tests/golden are self-recorded from
 * this oracle.  The render restatements follow the upstream shader sources:
 *   shaders/fs_raymarch.frag:10-81   (sphere tracer, shading quirks)
 *   shaders/fs_raymarch.vert:30-37   (origin = camPos, aspect = aspect.x)
 *   src/engine/rendering/renderer.cpp:1253-1267 (fullscreen quad UVs)
 *   src/engine/rendering/materials.cpp:531-545  (aspect 1700/900, camPos)
 */
#ifndef FS3D_ORACLE_H
#define FS3D_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- hashing / RNG primitives ---- */
uint32_t orc_fmix32(uint32_t h);
uint64_t orc_fmix64(uint64_t k);
uint32_t orc_stepkey(uint64_t seed, uint64_t t);
uint32_t orc_rowkey(uint32_t stepkey, uint32_t j, uint32_t k);
uint32_t orc_plane(uint32_t rowkey, uint32_t g, uint32_t s, uint32_t w);

typedef struct { uint64_t state, inc; } orc_pcg32;
void     orc_pcg32_seed(orc_pcg32* r, uint64_t initstate, uint64_t initseq);
uint32_t orc_pcg32_next(orc_pcg32* r);
uint32_t orc_pcg32_bounded(orc_pcg32* r, uint32_t bound);

/* ---- the step ---- */
void orc_step(uint8_t* grid, int X, int Y, int Z, uint64_t seed, uint64_t t);
/* same step, blocks visited in a pseudo-random order (order-independence test) */
void orc_step_shuffled(uint8_t* grid, int X, int Y, int Z, uint64_t seed, uint64_t t,
                       uint64_t order_seed);
/* same step, block rows split over nthreads OpenMP threads (nthreads<=0: all) */
void orc_step_omp(uint8_t* grid, int X, int Y, int Z, uint64_t seed, uint64_t t, int nthreads);
/* n steps from t0; if hashes != NULL, hashes[i] = hash after step t0+i */
void orc_run(uint8_t* grid, int X, int Y, int Z, uint64_t seed, uint64_t t0, int n,
             uint64_t* hashes, int nthreads);
/* 1 if the block with lattice index (i,j,k) at step t changes, else 0 */
int  orc_block_would_change(const uint8_t* grid, int X, int Y, int Z, uint64_t t,
                            int i, int j, int k);

/* ---- hash / diff ---- */
uint64_t orc_hash(const uint8_t* grid, int64_t n);
int64_t  orc_first_diff(const uint8_t* a, const uint8_t* b, int64_t n);

/* ---- generators (canonical layout idx = x + X*(z + Z*y)) ---- */
void orc_gen_c1(uint64_t seed, int X, int Y, int Z, uint8_t* grid);
void orc_gen_c2(uint64_t seed, int X, int Y, int Z, uint8_t* grid);
void orc_gen_c3_dims(uint64_t master, int count, int* dims /*3*count*/, uint64_t* seeds);
void orc_gen_c3_world(uint64_t world_seed, int X, int Y, int Z, uint8_t* grid);
void orc_gen_c5(uint64_t seed, int X, int Y, int Z, uint8_t* grid);
double orc_perlin(const uint8_t* perm512, double x, double y, double z);

/* ---- render ---- */
typedef struct {
    float origin[3];
    float forward[3];
    float right[3];
    float up[3];
    float tan_half_fov;
    float aspect;
    float light_pos[3];
    int32_t reserved;
} orc_camera;

void orc_render_sdf(const orc_camera* cam, int W, int H, float* rgba);
void orc_render_dda(const uint8_t* grid, int X, int Y, int Z, const orc_camera* cam,
                    int W, int H, float* rgba);

/* raymarch_sphere material: a triangle mesh rasterised with noperspective
 * attributes, each covered pixel marching a box SDF in object space */
#define ORC_OBJECT_MAX_TRIS 48
typedef struct {
    float cam_pos[3];     /* engine camPos; the eye sits at -cam_pos */
    float cam_rot_y_deg;  /* camRot.y */
    float fovy_deg, aspect, znear, zfar;
    float model[16];      /* column-major */
    float clear[4];
} orc_object_view;
void orc_object_mvp(const orc_object_view* v, float* mvp);
/* 0, or -1 when a vertex falls outside the depth range or the model is singular */
int orc_render_object(const orc_object_view* v, const float* tri, int ntri, int W, int H, float* rgba);
int orc_mesh_cube(float* tri /* 108 floats */);

/* mesh materials basic_mat / textured_mat / tri: triangle meshes rasterised
 * with depth test, perspective-correct texture coordinates, nearest sRGB
 * texels with repeat addressing */
#define ORC_MAT_BASIC 0
#define ORC_MAT_TEXTURED 1
#define ORC_MAT_TEXTURE 2
typedef struct {
    const float* vertices; /* n_vertices x {x, y, z, u, v}, three per triangle */
    int n_vertices;
    int material;
    float model[16];
    float color[4];
    const uint8_t* texture; /* RGBA8, row-major, sRGB */
    int tex_width, tex_height;
} orc_mesh_draw;
void orc_srgb_table(float* lut /* 256 */);
/* the camera of `view` (its model is ignored); 0, or -1 on allocation failure */
int orc_render_meshes(const orc_object_view* view, const orc_mesh_draw* draws, int n_draws, int W, int H,
                      float* rgba);

#ifdef __cplusplus
}
#endif
#endif
