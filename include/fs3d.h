/*
 * fs3d — C ABI of the GB300 falling-sand voxel engine (libfs3d.so).
 *
 * The upstream engine (FallingSand3D) exposes only C++ classes:
 *   VulkanEngine::{init,run,cleanup}           src/engine/engine.h:16-35
 *   Renderer::{init,draw,cleanup,...}          src/engine/rendering/renderer.h:81-95
 * and has no world/step interface, no plugin layer and no FFI.  Its main loop
 * (src/engine/engine.cpp:54-74) polls events and draws; a world step belongs
 * between handleEvents() and draw() (engine.cpp:60-68).  This header is the
 * boundary such a caller binds: plain pointers and sizes, status codes, no
 * exceptions, no torch or CUDA types (streams travel as void*).
 *
 * The rule is FS3D-rule v1:
 *   grid uint8, idx = x + X*(z + Z*y), gravity -y; 0 empty, 1 stone, 2 sand,
 *   3 water, >= 4 static solid; outside the grid is solid.  Step t uses
 *   Margolus 2x2x2 blocks with min corner (2i-o, 2j-o, 2k-o), o = t & 1.  In
 *   each block, slots are visited top layer first; a sand/water particle that
 *   has not moved falls straight down, else slides diagonally down into a
 *   random empty bottom cell, else (water only) moves sideways into a random
 *   empty cell of its layer.  Random choices come from a counter-based hash of
 *   (seed, t, block), so every implementation is bit-identical.
 *
 * Threading: a handle is used by one thread at a time; different handles may
 * be used concurrently.  Each world / batch owns one CUDA stream.
 */
#ifndef FS3D_H
#define FS3D_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FS3D_ABI_VERSION 1

typedef int fs3d_status;
#define FS3D_OK 0
#define FS3D_ERR_INVALID_ARG (-1)
#define FS3D_ERR_OOM (-2)
#define FS3D_ERR_BUDGET (-3)
#define FS3D_ERR_CUDA (-4)
#define FS3D_ERR_TIMEOUT (-5)
#define FS3D_ERR_MISMATCH (-6)
#define FS3D_ERR_STATE (-7)
#define FS3D_ERR_NOT_FOUND (-8)
#define FS3D_ERR_IO (-9)

/* world storage layouts */
#define FS3D_LAYOUT_BYTES 0  /* dense uint8, canonical index order            */
#define FS3D_LAYOUT_PLANES 1 /* 2 bits per cell, bit planes (see fs3d_world_device_ptr) */

/* render modes */
#define FS3D_RENDER_DDA 0        /* voxel grid traversal of the world          */
#define FS3D_RENDER_SDF_SPHERE 1 /* restatement of shaders/fs_raymarch.frag    */

typedef struct fs3d_world fs3d_world;
typedef struct fs3d_batch fs3d_batch;

/* Pinhole camera.  Ray for pixel (px,py) of a W x H image (row 0 = top):
 *   u = 1 - (px+0.5)/W, v = (py+0.5)/H, (ux,uy) = (2u-1, 2v-1)
 *   DDA: dir = normalize(forward + right*(ux*tan_half_fov*aspect) + up*(uy*tan_half_fov))
 *   SDF: dir = normalize(ux, uy*(1/aspect), 1), as fs_raymarch.frag:67-81. */
typedef struct fs3d_camera {
    float origin[3];
    float forward[3];
    float right[3];
    float up[3];
    float tan_half_fov;
    float aspect;
    float light_pos[3];
    int32_t reserved;
} fs3d_camera;

typedef struct fs3d_config {
    int steps_per_segment; /* steps per segment (graph length); default 64          */
    int ctas_per_sm;       /* persistent grid of the step kernel; 0 = all resident  */
    int use_graphs;        /* 1 (default) = run each segment as one CUDA graph       */
    int use_smem;          /* resident segments (all of a world's segment steps in
                              one launch): 1 = the planes are held in shared memory
                              (worlds that fit); 2 = the planes stay in global
                              memory (L2), one CTA per world sized by the work of
                              one layer; 3 (default) = 1 while the world's step
                              counter is below 128, then 2; 0 = the per-step
                              kernel only                                          */
    int reserved[12];
} fs3d_config;

/* ---- library ---- */
int fs3d_abi_version(void);
const char* fs3d_status_string(fs3d_status s);
/* message of the last failing call on this thread ("" if none) */
const char* fs3d_last_error(void);
/* number of this library's kernels launched so far in this process */
uint64_t fs3d_kernel_launch_count(void);
fs3d_config fs3d_default_config(void);

/* ---- drop-in step on a caller-owned device grid --------------------------
 * Replaces the CPU update of the engine loop (engine.cpp:68 hook point):
 * advances `grid_dev` (canonical layout, X*Y*Z bytes, device memory) in place
 * by n_steps steps starting at step t0.  Asynchronous on `stream` (NULL =
 * legacy default stream).  No device memory is allocated. */
fs3d_status fs3d_step_device(uint8_t* grid_dev, int X, int Y, int Z, uint64_t seed, uint64_t t0,
                             int n_steps, void* stream);
/* fs3d_step_device for n separate worlds, called from native code: for each
 * of n_steps steps, one launch of the drop-in kernel per world (worlds i with
 * dims[3i..3i+2] = X, Y, Z and seed seeds[i], all at step t0 + step).  The
 * plain per-world baseline the batched pool is measured against.  No
 * counterpart in the upstream project. */
fs3d_status fs3d_step_device_many(int n, uint8_t* const* grids_dev, const int* dims, const uint64_t* seeds,
                                  uint64_t t0, int n_steps, void* stream);
/* Same contract as fs3d_step_device, through the bit-plane kernels: the grid is
 * converted into 2-bit planes held in device scratch taken from the
 * stream-ordered pool (about X*Y*Z/4 bytes, freed on `stream` when done), the
 * n steps run there (one launch for all of them when the world fits in shared
 * memory and n repays the launch: n >= 4 and at least one step per 120 000
 * cells, up to 1.5 M cells; otherwise one launch per step over the whole GPU) and the planes are converted back.  Settled rows or
 * layers are skipped exactly, starting from flags computed from the cells.
 * Asynchronous on `stream`. */
fs3d_status fs3d_run_device(uint8_t* grid_dev, int X, int Y, int Z, uint64_t seed, uint64_t t0,
                            int n_steps, void* stream);
/* fs3d_run_device for callers that cannot allocate device memory (an engine
 * whose own allocator owns all GPU memory, a real-time frame loop that must
 * not stall on an allocation): same arguments and results, but the scratch
 * lives in one static device array (64 MiB of planes plus 4 MiB of row flags)
 * that every GPU loading this library holds until exit, so the call allocates
 * nothing.  Worlds whose planes exceed 64 MiB (about 268 M cells) or whose
 * rows exceed 2048 cells are rejected with FS3D_ERR_INVALID_ARG.  The first
 * call on a device looks the array up (cudaGetSymbolAddress) and should come
 * before any stream capture.  All calls share the array: calls that overlap
 * on the GPU race and must be serialised.  No counterpart in the upstream
 * project (it has no step). */
fs3d_status fs3d_run_device_noalloc(uint8_t* grid_dev, int X, int Y, int Z, uint64_t seed,
                                    uint64_t t0, int n_steps, void* stream);
/* Waits for `stream` (timeout_ns < 0: without limit; FS3D_ERR_TIMEOUT when
 * the limit passes first), then reports whether a drop-in run on the current
 * device (fs3d_run_device or fs3d_run_device_noalloc) met a bulk copy that
 * did not complete within its bounded wait since the last check:
 * FS3D_ERR_TIMEOUT if so, and the record is cleared.  Such a run leaves its
 * grid as it was, and so does every drop-in run on the device after it until
 * this check.  The runs are asynchronous, so this is where a caller learns of
 * it.  No counterpart in the upstream project (it has no step). */
fs3d_status fs3d_run_device_check(void* stream, int64_t timeout_ns);
/* Same contract, one thread per 2x2x2 block and byte loads: the plain
 * reference kernel the vectorised one is checked against. */
fs3d_status fs3d_step_device_simple(uint8_t* grid_dev, int X, int Y, int Z, uint64_t seed,
                                    uint64_t t0, int n_steps, void* stream);
/* Whole-grid hash H = sum_i fmix64(i*256 + v_i) mod 2^64 of a device grid;
 * synchronous (waits on `stream`). */
fs3d_status fs3d_hash_device(const uint8_t* grid_dev, int64_t n_cells, void* stream,
                             uint64_t* out);
/* Smallest index where two device grids differ, -1 if equal; synchronous. */
fs3d_status fs3d_first_diff_device(const uint8_t* a_dev, const uint8_t* b_dev, int64_t n_cells,
                                   void* stream, int64_t* out);

/* ---- world objects (library-owned device state) ---- */
fs3d_status fs3d_world_create(const uint8_t* grid_host, int X, int Y, int Z, uint64_t seed,
                              uint64_t start_step, int layout, fs3d_world** out);
/* async; a PLANES world takes the call's steps in one resident launch (a world
 * fitting shared memory, n_steps >= 4 and at least one step per 120 000 cells,
 * up to 1.5 M cells) or one launch per step over the whole GPU, and keeps its
 * change flags from call to call */
fs3d_status fs3d_world_step(fs3d_world* w, int n_steps);
/* Bounded wait (timeout_ns < 0: without limit).  FS3D_ERR_TIMEOUT also when a
 * step launch of the world met a bulk copy that did not complete within its
 * bounded wait: that launch and the ones after it stepped nothing, so the
 * world's step counter is set back to the step its state holds, and the
 * world is usable again. */
fs3d_status fs3d_world_sync(fs3d_world* w, int64_t timeout_ns);
fs3d_status fs3d_world_read(fs3d_world* w, uint8_t* grid_host_out); /* canonical layout */
fs3d_status fs3d_world_write(fs3d_world* w, const uint8_t* grid_host); /* replace contents */
fs3d_status fs3d_world_hash(fs3d_world* w, uint64_t* out);
fs3d_status fs3d_world_info(const fs3d_world* w, int* X, int* Y, int* Z, uint64_t* seed,
                            uint64_t* step, int* layout);
/* Device pointer of the current state.  BYTES: X*Y*Z canonical bytes.
 * PLANES: rows r = y*Z + z of nw = ceil(X/64) groups of four uint32 words
 * {A even, A odd, B even, B odd}; in group g, bit m of an even word is
 * x = 64g + 2m and of an odd word x = 64g + 2m + 1; (A,B) = (0,0) empty,
 * (0,1) solid, (1,0) sand, (1,1) water; cells past X are solid. */
fs3d_status fs3d_world_device_ptr(fs3d_world* w, const void** dev, int* layout);
fs3d_status fs3d_world_stream(fs3d_world* w, void** stream);
fs3d_status fs3d_world_destroy(fs3d_world* w);
/* checkpoint: header {magic "FS3DCKP1", version, X, Y, Z, seed, step} + dense grid */
fs3d_status fs3d_world_save(fs3d_world* w, const char* path);
fs3d_status fs3d_world_load(const char* path, int layout, fs3d_world** out);

/* ---- batch / serving pool ----
 * Worlds of any size share one device pool in the PLANES layout.  Each
 * admitted world has its own step counter and step budget; run_segment
 * advances every live world by min(steps_per_segment, steps left).  Worlds
 * may be admitted and retired between segments. */
fs3d_status fs3d_batch_create(size_t hbm_budget_bytes, const fs3d_config* cfg, fs3d_batch** out);
/* FS3D_ERR_BUDGET if the world does not fit in the budget right now */
fs3d_status fs3d_batch_admit(fs3d_batch* b, const uint8_t* grid_host, int X, int Y, int Z,
                             uint64_t seed, uint64_t start_step, int64_t n_steps,
                             uint64_t* ticket);
/* Admits the mixed-size synthetic world of `seed` (fs3d_gen_batch_world), generated
 * on the device straight into the pool: no host grid, no upload.  Needs Y >= 4. */
fs3d_status fs3d_batch_admit_generated(fs3d_batch* b, int X, int Y, int Z, uint64_t seed,
                                       uint64_t start_step, int64_t n_steps, uint64_t* ticket);
/* Many admissions with one host wait: admits specs[0..n) in order until one
 * does not fit (FS3D_ERR_BUDGET) or fails; *n_admitted counts the admitted. */
typedef struct fs3d_world_spec {
    const uint8_t* grid; /* host, canonical layout                               */
    int X, Y, Z;
    int pad;
    uint64_t seed, start_step;
    int64_t n_steps;
} fs3d_world_spec;
fs3d_status fs3d_batch_admit_many(fs3d_batch* b, int n, const fs3d_world_spec* specs, uint64_t* tickets,
                                  int* n_admitted);
/* The same, returning once the uploads and conversions are enqueued on the
 * admission stream (no host wait): the grids must stay unchanged until
 * fs3d_batch_wait_copies returns.  Segments wait for the conversions by
 * themselves; uploads overlap a segment already running. */
fs3d_status fs3d_batch_admit_many_async(fs3d_batch* b, int n, const fs3d_world_spec* specs, uint64_t* tickets,
                                        int* n_admitted);
fs3d_status fs3d_batch_run_segment(fs3d_batch* b); /* async on the batch stream */
/* Builds and uploads the next segment's tables now (host work and small
 * uploads on the batch stream), so the next fs3d_batch_run_segment only
 * launches it: a caller overlaps the build with a segment still running.
 * An admission or retirement in between makes the next segment build them
 * again.  No counterpart in the upstream project. */
fs3d_status fs3d_batch_prepare(fs3d_batch* b);
fs3d_status fs3d_batch_sync(fs3d_batch* b, int64_t timeout_ns);
/* done = 1 once the world has taken all its steps; hash valid when done */
fs3d_status fs3d_batch_poll(fs3d_batch* b, uint64_t ticket, int* done, uint64_t* hash);
/* fs3d_batch_poll for n worlds at once: done[i] as there; with `hashes`
 * (nullable), hashes[i] for every world that is done, those not hashed yet
 * computed together in one launch and one wait.  No counterpart in the
 * upstream project. */
fs3d_status fs3d_batch_poll_many(fs3d_batch* b, int n, const uint64_t* tickets, int* done, uint64_t* hashes);
/* frees the world's pool space; grid_out (nullable) receives the final grid */
fs3d_status fs3d_batch_retire(fs3d_batch* b, uint64_t ticket, uint8_t* grid_out);
/* retire n worlds with one host wait; grids_out (nullable) holds n host pointers (nullable each) */
fs3d_status fs3d_batch_retire_many(fs3d_batch* b, int n, const uint64_t* tickets, uint8_t* const* grids_out);
/* The same without the host wait: the read-backs run on their own stream after
 * each world's last segment (downloads overlap later segments); grids_out
 * holds the grids once fs3d_batch_wait_copies returns. */
fs3d_status fs3d_batch_retire_many_async(fs3d_batch* b, int n, const uint64_t* tickets, uint8_t* const* grids_out);
/* Reads n live worlds back without retiring them (a snapshot of their state
 * after the segments enqueued so far; the grids are in grids_out when the call
 * returns; a NULL entry skips that world).  The worlds keep running: the next
 * segment waits for the read-back.  No counterpart in the upstream project. */
fs3d_status fs3d_batch_read_many(fs3d_batch* b, int n, const uint64_t* tickets, uint8_t* const* grids_out);
/* Waits (timeout_ns < 0: without limit) until every admission and read-back
 * enqueued so far has run. */
fs3d_status fs3d_batch_wait_copies(fs3d_batch* b, int64_t timeout_ns);
/* Autotuner: times each candidate launch configuration on trial_segments real
 * segments of the live worlds (they advance as usual), keeps the fastest per
 * voxel-update and remembers it for batches of the same make-up (live worlds
 * per size class).  Knobs: resident segments in global or shared memory
 * (use_smem 2 or 1), worlds may run in the next wider CTA class (promote), and
 * the per-step kernel's CTAs per SM when some world needs that kernel. */
typedef struct fs3d_tune_report {
    int mode;               /* chosen fs3d_config.use_smem                         */
    int promote;            /* chosen class promotion (0 = smallest fitting CTA)  */
    int ctas_per_sm;        /* chosen CTAs per SM of the per-step kernel           */
    int trials;             /* configurations timed                                */
    int cached;             /* 1: taken from an earlier tuning of the same make-up */
    int segments;           /* segments run while tuning (the worlds advanced)    */
    double best_vox_per_ms; /* voxel-updates per ms of the choice                  */
    double trial_vox_per_ms[8];
} fs3d_tune_report;
fs3d_status fs3d_batch_autotune(fs3d_batch* b, int trial_segments, fs3d_tune_report* out);
/* Work counters since creation (waits for the batch stream): every cell of
 * every stepped world once per step (dense), and the cell-steps actually
 * evaluated: resident worlds skip block row-pairs whose rows did not change
 * in the two previous steps (exact: such blocks cannot change). */
fs3d_status fs3d_batch_counters(fs3d_batch* b, uint64_t* dense_cell_steps, uint64_t* processed_cell_steps);
fs3d_status fs3d_batch_stats(const fs3d_batch* b, int64_t* live_worlds, int64_t* live_cells,
                             size_t* bytes_used, size_t* bytes_budget);
fs3d_status fs3d_batch_stream(fs3d_batch* b, void** stream);
fs3d_status fs3d_batch_destroy(fs3d_batch* b);

/* ---- serving ----
 * A seeded Poisson stream of requests (dims iid from {16,24,32,48,64,96,128}^3,
 * the synthetic batch world of the request's seed, n_steps log-uniform in
 * [min_steps, max_steps]) served by one batch with continuous batching:
 * arrivals are admitted (generated on the device) while a segment runs, as
 * the memory budget allows, and join at the next segment. */
typedef struct fs3d_serve_params {
    double lambda;           /* mean arrivals per second                          */
    double duration_s;       /* arrival window                                     */
    int64_t max_requests;    /* cap on the number of requests (0 = none)           */
    uint64_t master_seed;
    size_t hbm_budget;       /* pool budget in bytes (0 = 150 GiB)                 */
    int steps_per_segment;   /* 0 = 64                                             */
    int min_steps;           /* 0 = 10                                             */
    int max_steps;           /* 0 = 1000                                           */
    int with_hash;           /* 1 = hash every finished world (request.hash)       */
    int segment_timeout_ms;  /* bound on the wait for one segment (0 = 10000); the
                                run ends with FS3D_ERR_TIMEOUT when it passes       */
    int reserved[7];
} fs3d_serve_params;

typedef struct fs3d_serve_request {
    double arrival_s, admitted_s, finished_s; /* seconds from the start of the run */
    int32_t X, Y, Z, n_steps;
    uint64_t seed, hash;
} fs3d_serve_request;

typedef struct fs3d_serve_stats {
    int64_t requests, completed, segments, peak_live_worlds;
    size_t peak_bytes;
    double wall_s, p50_ms, p99_ms, mean_ms, max_ms;
    double voxel_updates, voxel_updates_per_s, offered_voxel_updates_per_s;
    double reserved[8];
} fs3d_serve_stats;

/* The request stream of `p` (no GPU work): fills up to `capacity` requests and
 * sets *n_reqs to the stream's length. */
fs3d_status fs3d_serve_plan(const fs3d_serve_params* p, int64_t capacity, fs3d_serve_request* reqs,
                            int64_t* n_reqs);
/* Serves the n planned requests in real time; fills their admitted/finished
 * times and hashes and the summary statistics.  A request waits for memory
 * while other worlds are live; FS3D_ERR_BUDGET if one needs more than the
 * whole budget (nothing live and still no room); FS3D_ERR_TIMEOUT if a
 * segment does not end within segment_timeout_ms (default 10 s). */
fs3d_status fs3d_serve_run(const fs3d_serve_params* p, int64_t n, fs3d_serve_request* reqs,
                           fs3d_serve_stats* stats);

/* ---- render (headless) ----
 * Writes W*H RGBA float32 pixels (row 0 = top).  out_on_device = 1: `rgba`
 * is a device pointer (async on the world's stream); 0: host pointer
 * (synchronous).  SDF_SPHERE ignores the world's contents (world may be NULL
 * when out_on_device = 1 and `stream` is given via fs3d_render_sdf). */
fs3d_status fs3d_render(fs3d_world* w, const fs3d_camera* cam, int W, int H, int mode,
                        float* rgba, int out_on_device);
fs3d_status fs3d_render_sdf(const fs3d_camera* cam, int W, int H, float* rgba_dev, void* stream);
/* Camera presets: the fs_raymarch defaults (camPos (0,0,-5), aspect 1700/900,
 * light (2,5,3)) and the large-world view (origin (-X/4, 0.9Y, -Z/4) looking
 * at the centre, vertical FOV 70 degrees, aspect W/H). */
void fs3d_camera_fs_raymarch(fs3d_camera* cam);
void fs3d_camera_world_view(fs3d_camera* cam, int X, int Y, int Z, int W, int H);

/* ---- the raymarch_sphere material (the object the upstream scene draws) ----
 * Restates raymarch_sphere.vert:30-45 and .frag:18-51 with the fixed-function
 * stages between them: the mesh (object space) is transformed by
 * proj * rotY(cam_rot_y) * translate(cam_pos) * model (materials.cpp:531-536,
 * OpenGL depth range, y negated), rasterised with no culling and a top-left
 * rule at pixel centres, attributes interpolated linearly in screen space
 * (noperspective), nearest fragment kept under LESS_OR_EQUAL against depth 1;
 * each covered pixel marches a box SDF of half-extent 0.5 from the camera in
 * object space, invModel * (-cam_pos), towards the interpolated position:
 * (max(0.05, 1 - 0.05*steps), 0, 0, 1) on a hit, (0,0,0,1) on a miss; other
 * pixels get `clear`.  W*H RGBA float32 into device memory, async on `stream`.
 * A vertex behind the camera or outside the depth range (near/far clipping is
 * not done) or a singular model gives FS3D_ERR_INVALID_ARG. */
typedef struct fs3d_object_view {
    float cam_pos[3];     /* the engine's camPos (renderer.h:148); the eye sits at -cam_pos */
    float cam_rot_y_deg;  /* camRot.y in degrees (renderer.h:149)                            */
    float fovy_deg;       /* vertical field of view                                          */
    float aspect;
    float znear, zfar;
    float model[16];      /* column-major object transform                                  */
    float clear[4];       /* colour of uncovered pixels                                      */
} fs3d_object_view;
/* the upstream scene: camPos (0,0,-5), camRot 0, 70 degrees, aspect
 * 1700/900, depth 0.01..200, identity model, clear colour (0,0,1,1) */
void fs3d_object_view_scene(fs3d_object_view* v);
/* writes the scene's cube (assets/cube2.obj, +-1) as 12 triangles of 3
 * vertices x 3 floats into tri_xyz (108 floats, may be NULL); returns 12 */
int fs3d_mesh_cube(float* tri_xyz);
/* ntri <= 48 triangles of 9 floats each (host memory) */
fs3d_status fs3d_render_object(const fs3d_object_view* v, const float* tri_xyz, int ntri, int W, int H,
                               float* rgba_dev, void* stream);

/* ---- mesh materials: basic_mat, textured_mat, tri ----
 * Restates the scene's mesh pipelines (basic_mat.{vert,frag}: flat colour;
 * textured_mat: colour + texel, alpha colour.a + 1; tri: texel, alpha 1) with
 * the state they are drawn with: no culling, depth LESS_OR_EQUAL against 1
 * (later draws win ties), one sample per pixel, NEAREST filtering with REPEAT
 * addressing of sRGB texels (decoded to linear), triangles clipped against
 * the depth range 0 <= z <= w, texture coordinates interpolated
 * perspective-correctly, the result clamped to [0,1] as the attachment stores
 * it.  Camera and projection from `view` (its model is ignored; each draw has
 * its own).  W*H RGBA float32 into device memory, async on `stream`; the same
 * frame as the CPU restatement bit for bit. */
#define FS3D_MAT_BASIC 0
#define FS3D_MAT_TEXTURED 1
#define FS3D_MAT_TEXTURE 2
typedef struct fs3d_mesh_draw {
    const float* vertices;  /* n_vertices x {x, y, z, u, v} (three per triangle), device or page-locked */
    int n_vertices;         /* a multiple of 3                                           */
    int material;           /* FS3D_MAT_*                                                */
    float model[16];        /* column-major                                              */
    float color[4];         /* the material's colour (BASIC, TEXTURED)                   */
    const uint8_t* texture; /* RGBA8 texels, row-major, sRGB; device or page-locked      */
    int tex_width, tex_height;
} fs3d_mesh_draw;
/* n_draws <= 65536, fewer than 2^30 triangles in all */
fs3d_status fs3d_render_meshes(const fs3d_object_view* view, const fs3d_mesh_draw* draws, int n_draws, int W, int H,
                               float* rgba_dev, void* stream);

/* ---- test hooks (failure injection without a GPU fault) ----
 * COPY_STALL (count > 0: on, 0: off): the resident step kernels announce 16
 * bytes more on their mbarrier than each bulk copy delivers; the copy lands
 * in full, the barrier's phase never completes, and every such wait runs to
 * its iteration limit (about a second) and reports a timeout.
 * ALLOC_FAIL: the next `count` world-memory allocations of batch admissions
 * fail as out of device memory (decided on the host; nothing is launched).
 * NONE clears both.  For tests only. */
#define FS3D_INJECT_NONE 0
#define FS3D_INJECT_COPY_STALL 1
#define FS3D_INJECT_ALLOC_FAIL 2
fs3d_status fs3d_test_inject(int what, int count);

/* ---- synthetic worlds (seeded, bit-reproducible) ---- */
fs3d_status fs3d_gen_parity(uint64_t seed, int X, int Y, int Z, uint8_t* grid_host);
fs3d_status fs3d_gen_pillars(uint64_t seed, int X, int Y, int Z, uint8_t* grid_host);
fs3d_status fs3d_gen_batch_dims(uint64_t master, int count, int* dims, uint64_t* seeds);
fs3d_status fs3d_gen_batch_world(uint64_t world_seed, int X, int Y, int Z, uint8_t* grid_host);
fs3d_status fs3d_gen_dunes(uint64_t seed, int X, int Y, int Z, uint8_t* grid_host);

#ifdef __cplusplus
}
#endif
#endif /* FS3D_H */
