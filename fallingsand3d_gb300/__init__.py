"""fallingsand3d_gb300 — Python binding of libfs3d (the GB300 voxel step).

A thin ctypes layer over the C ABI in ``include/fs3d.h``; every call goes to
the CUDA library and there is no CPU fallback: importing works without a GPU
(so host-side code and tests can run), but any call that needs the device
fails loudly if the library or the GPU is missing.

Grids are numpy ``uint8`` arrays in the canonical layout
``idx = x + X*(z + Z*y)``, i.e. shape ``(Y, Z, X)``.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libfs3d.so")

LAYOUT_BYTES = 0
LAYOUT_PLANES = 1
RENDER_DDA = 0
RENDER_SDF_SPHERE = 1

OK = 0
ERR_INVALID_ARG = -1
ERR_OOM = -2
ERR_BUDGET = -3
ERR_CUDA = -4
ERR_TIMEOUT = -5
ERR_MISMATCH = -6
ERR_STATE = -7
ERR_NOT_FOUND = -8
ERR_IO = -9

# every entry point of include/fs3d.h (checked by the tests)
EXPORTS = (
    "fs3d_abi_version", "fs3d_status_string", "fs3d_last_error", "fs3d_kernel_launch_count",
    "fs3d_default_config", "fs3d_step_device", "fs3d_step_device_many", "fs3d_step_device_simple", "fs3d_run_device",
    "fs3d_run_device_noalloc", "fs3d_run_device_check", "fs3d_hash_device", "fs3d_first_diff_device",
    "fs3d_world_create", "fs3d_world_step", "fs3d_world_sync", "fs3d_world_read", "fs3d_world_write",
    "fs3d_world_hash", "fs3d_world_info", "fs3d_world_device_ptr", "fs3d_world_stream",
    "fs3d_world_destroy", "fs3d_world_save", "fs3d_world_load", "fs3d_batch_create", "fs3d_batch_admit", "fs3d_batch_admit_generated", "fs3d_batch_admit_many",
    "fs3d_batch_retire_many", "fs3d_batch_admit_many_async", "fs3d_batch_retire_many_async", "fs3d_batch_wait_copies",
    "fs3d_batch_read_many",
    "fs3d_batch_run_segment", "fs3d_batch_prepare", "fs3d_batch_sync", "fs3d_batch_poll", "fs3d_batch_poll_many", "fs3d_batch_retire",
    "fs3d_batch_stats", "fs3d_batch_counters", "fs3d_batch_autotune", "fs3d_batch_stream", "fs3d_batch_destroy", "fs3d_serve_plan", "fs3d_serve_run", "fs3d_render", "fs3d_render_sdf",
    "fs3d_camera_fs_raymarch", "fs3d_camera_world_view", "fs3d_object_view_scene", "fs3d_mesh_cube",
    "fs3d_render_object", "fs3d_render_meshes", "fs3d_gen_parity", "fs3d_gen_pillars",
    "fs3d_gen_batch_dims", "fs3d_gen_batch_world", "fs3d_gen_dunes", "fs3d_test_inject",
)


class Fs3dError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"fs3d status {status}: {msg}")
        self.status = status


class Camera(C.Structure):
    _fields_ = [("origin", C.c_float * 3), ("forward", C.c_float * 3), ("right", C.c_float * 3),
                ("up", C.c_float * 3), ("tan_half_fov", C.c_float), ("aspect", C.c_float),
                ("light_pos", C.c_float * 3), ("reserved", C.c_int32)]


class ServeParams(C.Structure):
    _fields_ = [("lambda_", C.c_double), ("duration_s", C.c_double), ("max_requests", C.c_int64),
                ("master_seed", C.c_uint64), ("hbm_budget", C.c_size_t), ("steps_per_segment", C.c_int),
                ("min_steps", C.c_int), ("max_steps", C.c_int), ("with_hash", C.c_int),
                ("segment_timeout_ms", C.c_int), ("reserved", C.c_int * 7)]


class ServeRequest(C.Structure):
    _fields_ = [("arrival_s", C.c_double), ("admitted_s", C.c_double), ("finished_s", C.c_double),
                ("X", C.c_int32), ("Y", C.c_int32), ("Z", C.c_int32), ("n_steps", C.c_int32),
                ("seed", C.c_uint64), ("hash", C.c_uint64)]


class ServeStats(C.Structure):
    _fields_ = [("requests", C.c_int64), ("completed", C.c_int64), ("segments", C.c_int64),
                ("peak_live_worlds", C.c_int64), ("peak_bytes", C.c_size_t), ("wall_s", C.c_double),
                ("p50_ms", C.c_double), ("p99_ms", C.c_double), ("mean_ms", C.c_double), ("max_ms", C.c_double),
                ("voxel_updates", C.c_double), ("voxel_updates_per_s", C.c_double),
                ("offered_voxel_updates_per_s", C.c_double), ("reserved", C.c_double * 8)]


class WorldSpec(C.Structure):
    _fields_ = [("grid", C.c_void_p), ("X", C.c_int), ("Y", C.c_int), ("Z", C.c_int), ("pad", C.c_int),
                ("seed", C.c_uint64), ("start_step", C.c_uint64), ("n_steps", C.c_int64)]


# numpy view of fs3d_world_spec (same field offsets), for building many at once
_SPEC_DTYPE = np.dtype([("grid", np.uint64), ("X", np.int32), ("Y", np.int32), ("Z", np.int32), ("pad", np.int32),
                        ("seed", np.uint64), ("start_step", np.uint64), ("n_steps", np.int64)])
assert _SPEC_DTYPE.itemsize == C.sizeof(WorldSpec)


class TuneReport(C.Structure):
    _fields_ = [("mode", C.c_int), ("promote", C.c_int), ("ctas_per_sm", C.c_int), ("trials", C.c_int), ("cached", C.c_int),
                ("segments", C.c_int), ("best_vox_per_ms", C.c_double), ("trial_vox_per_ms", C.c_double * 8)]


class ObjectView(C.Structure):
    _fields_ = [("cam_pos", C.c_float * 3), ("cam_rot_y_deg", C.c_float), ("fovy_deg", C.c_float),
                ("aspect", C.c_float), ("znear", C.c_float), ("zfar", C.c_float), ("model", C.c_float * 16),
                ("clear", C.c_float * 4)]


MAT_BASIC, MAT_TEXTURED, MAT_TEXTURE = 0, 1, 2


class MeshDraw(C.Structure):
    _fields_ = [("vertices", C.c_void_p), ("n_vertices", C.c_int), ("material", C.c_int), ("model", C.c_float * 16),
                ("color", C.c_float * 4), ("texture", C.c_void_p), ("tex_width", C.c_int), ("tex_height", C.c_int)]


class Config(C.Structure):
    _fields_ = [("steps_per_segment", C.c_int), ("ctas_per_sm", C.c_int), ("use_graphs", C.c_int),
                ("use_smem", C.c_int), ("reserved", C.c_int * 12)]


_lib: Optional[C.CDLL] = None

u8p = C.POINTER(C.c_uint8)
vp = C.c_void_p
i32, i64, u64 = C.c_int, C.c_int64, C.c_uint64


def _bind(lib: C.CDLL) -> None:
    S = C.c_int
    sig = {
        "fs3d_abi_version": (C.c_int, []),
        "fs3d_status_string": (C.c_char_p, [S]),
        "fs3d_last_error": (C.c_char_p, []),
        "fs3d_kernel_launch_count": (u64, []),
        "fs3d_default_config": (Config, []),
        "fs3d_step_device": (S, [vp, i32, i32, i32, u64, u64, i32, vp]),
        "fs3d_step_device_simple": (S, [vp, i32, i32, i32, u64, u64, i32, vp]),
        "fs3d_step_device_many": (S, [i32, C.POINTER(vp), vp, vp, u64, i32, vp]),
        "fs3d_run_device": (S, [vp, i32, i32, i32, u64, u64, i32, vp]),
        "fs3d_run_device_noalloc": (S, [vp, i32, i32, i32, u64, u64, i32, vp]),
        "fs3d_run_device_check": (S, [vp, i64]),
        "fs3d_test_inject": (S, [i32, i32]),
        "fs3d_hash_device": (S, [vp, i64, vp, C.POINTER(u64)]),
        "fs3d_first_diff_device": (S, [vp, vp, i64, vp, C.POINTER(i64)]),
        "fs3d_world_create": (S, [vp, i32, i32, i32, u64, u64, i32, C.POINTER(vp)]),
        "fs3d_world_step": (S, [vp, i32]),
        "fs3d_world_sync": (S, [vp, i64]),
        "fs3d_world_read": (S, [vp, vp]),
        "fs3d_world_write": (S, [vp, vp]),
        "fs3d_world_hash": (S, [vp, C.POINTER(u64)]),
        "fs3d_world_info": (S, [vp, C.POINTER(i32), C.POINTER(i32), C.POINTER(i32), C.POINTER(u64),
                                C.POINTER(u64), C.POINTER(i32)]),
        "fs3d_world_device_ptr": (S, [vp, C.POINTER(vp), C.POINTER(i32)]),
        "fs3d_world_stream": (S, [vp, C.POINTER(vp)]),
        "fs3d_world_destroy": (S, [vp]),
        "fs3d_world_save": (S, [vp, C.c_char_p]),
        "fs3d_world_load": (S, [C.c_char_p, i32, C.POINTER(vp)]),
        "fs3d_batch_create": (S, [C.c_size_t, C.POINTER(Config), C.POINTER(vp)]),
        "fs3d_batch_admit": (S, [vp, vp, i32, i32, i32, u64, u64, i64, C.POINTER(u64)]),
        "fs3d_batch_admit_generated": (S, [vp, i32, i32, i32, u64, u64, i64, C.POINTER(u64)]),
        "fs3d_batch_admit_many": (S, [vp, i32, C.POINTER(WorldSpec), C.POINTER(u64), C.POINTER(i32)]),
        "fs3d_batch_retire_many": (S, [vp, i32, C.POINTER(u64), C.POINTER(vp)]),
        "fs3d_batch_admit_many_async": (S, [vp, i32, C.POINTER(WorldSpec), C.POINTER(u64), C.POINTER(i32)]),
        "fs3d_batch_retire_many_async": (S, [vp, i32, C.POINTER(u64), C.POINTER(vp)]),
        "fs3d_batch_wait_copies": (S, [vp, i64]),
        "fs3d_batch_read_many": (S, [vp, i32, C.POINTER(u64), C.POINTER(vp)]),
        "fs3d_batch_run_segment": (S, [vp]),
        "fs3d_batch_prepare": (S, [vp]),
        "fs3d_batch_sync": (S, [vp, i64]),
        "fs3d_batch_poll": (S, [vp, u64, C.POINTER(i32), C.POINTER(u64)]),
        "fs3d_batch_poll_many": (S, [vp, i32, C.POINTER(u64), C.POINTER(i32), C.POINTER(u64)]),
        "fs3d_batch_retire": (S, [vp, u64, vp]),
        "fs3d_batch_autotune": (S, [vp, i32, C.POINTER(TuneReport)]),
        "fs3d_batch_counters": (S, [vp, C.POINTER(u64), C.POINTER(u64)]),
        "fs3d_batch_stats": (S, [vp, C.POINTER(i64), C.POINTER(i64), C.POINTER(C.c_size_t),
                                 C.POINTER(C.c_size_t)]),
        "fs3d_batch_stream": (S, [vp, C.POINTER(vp)]),
        "fs3d_batch_destroy": (S, [vp]),
        "fs3d_serve_plan": (S, [C.POINTER(ServeParams), i64, C.POINTER(ServeRequest), C.POINTER(i64)]),
        "fs3d_serve_run": (S, [C.POINTER(ServeParams), i64, C.POINTER(ServeRequest), C.POINTER(ServeStats)]),
        "fs3d_render": (S, [vp, C.POINTER(Camera), i32, i32, i32, vp, i32]),
        "fs3d_render_sdf": (S, [C.POINTER(Camera), i32, i32, vp, vp]),
        "fs3d_camera_fs_raymarch": (None, [C.POINTER(Camera)]),
        "fs3d_camera_world_view": (None, [C.POINTER(Camera), i32, i32, i32, i32, i32]),
        "fs3d_object_view_scene": (None, [C.POINTER(ObjectView)]),
        "fs3d_mesh_cube": (C.c_int, [vp]),
        "fs3d_render_object": (S, [C.POINTER(ObjectView), vp, i32, i32, i32, vp, vp]),
        "fs3d_render_meshes": (S, [C.POINTER(ObjectView), C.POINTER(MeshDraw), i32, i32, i32, vp, vp]),
        "fs3d_gen_parity": (S, [u64, i32, i32, i32, vp]),
        "fs3d_gen_pillars": (S, [u64, i32, i32, i32, vp]),
        "fs3d_gen_batch_dims": (S, [u64, i32, vp, vp]),
        "fs3d_gen_batch_world": (S, [u64, i32, i32, i32, vp]),
        "fs3d_gen_dunes": (S, [u64, i32, i32, i32, vp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args


def lib() -> C.CDLL:
    """The loaded libfs3d; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: run `python -m fallingsand3d_gb300.build` first")
        lib_ = C.CDLL(LIB_PATH)
        _bind(lib_)
        _lib = lib_
    return _lib


def check(status: int) -> None:
    if status != OK:
        L = lib()
        raise Fs3dError(status, f"{L.fs3d_status_string(status).decode()}: {L.fs3d_last_error().decode()}")


def _ptr(a: np.ndarray) -> int:
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data


def kernel_launches() -> int:
    return int(lib().fs3d_kernel_launch_count())


# ---------------------------------------------------------------- generators
def _gen(fn: str, seed: int, X: int, Y: int, Z: int) -> np.ndarray:
    g = np.empty((Y, Z, X), np.uint8)
    check(getattr(lib(), fn)(seed, X, Y, Z, _ptr(g)))
    return g


def gen_parity(seed: int, X: int = 64, Y: int = 64, Z: int = 64) -> np.ndarray:
    """Stone floor, upper half iid sand 0.25 / water 0.15."""
    return _gen("fs3d_gen_parity", seed, X, Y, Z)


def gen_pillars(seed: int, X: int = 512, Y: int = 512, Z: int = 512) -> np.ndarray:
    """Stone floor + 256 stone pillars, upper 60% iid sand 0.30 / water 0.10."""
    return _gen("fs3d_gen_pillars", seed, X, Y, Z)


def gen_batch_world(seed: int, X: int, Y: int, Z: int) -> np.ndarray:
    return _gen("fs3d_gen_batch_world", seed, X, Y, Z)


def gen_dunes(seed: int, X: int = 1024, Y: int = 1024, Z: int = 1024) -> np.ndarray:
    return _gen("fs3d_gen_dunes", seed, X, Y, Z)


def gen_batch_dims(master: int, count: int):
    dims = np.empty((count, 3), np.int32)
    seeds = np.empty(count, np.uint64)
    check(lib().fs3d_gen_batch_dims(master, count, _ptr(dims), _ptr(seeds)))
    return dims, seeds


# ---------------------------------------------------------------- cameras
def camera_fs_raymarch() -> Camera:
    c = Camera()
    lib().fs3d_camera_fs_raymarch(C.byref(c))
    return c


def camera_world_view(X: int, Y: int, Z: int, W: int, H: int) -> Camera:
    c = Camera()
    lib().fs3d_camera_world_view(C.byref(c), X, Y, Z, W, H)
    return c


def object_view_scene(cam_pos=None, rot_y: Optional[float] = None, model=None) -> ObjectView:
    """The upstream scene's view of its one object, optionally moved: camPos,
    camRot.y in degrees, a 4x4 model matrix (row-major numpy, stored
    column-major)."""
    v = ObjectView()
    lib().fs3d_object_view_scene(C.byref(v))
    if cam_pos is not None:
        v.cam_pos[:] = [float(x) for x in cam_pos]
    if rot_y is not None:
        v.cam_rot_y_deg = float(rot_y)
    if model is not None:
        v.model[:] = [float(x) for x in np.asarray(model, np.float32).T.reshape(-1)]
    return v


def mesh_cube() -> np.ndarray:
    """The scene's +-1 cube as (12, 3, 3) float32 triangles."""
    tri = np.empty((12, 3, 3), np.float32)
    lib().fs3d_mesh_cube(_ptr(tri))
    return tri


def render_object_device(view: ObjectView, tri: np.ndarray, W: int, H: int, rgba_ptr: int, stream: int = 0) -> None:
    """The raymarch_sphere material over a triangle mesh into W*H RGBA float32 at rgba_ptr."""
    tri = np.ascontiguousarray(tri, np.float32).reshape(-1, 9)
    check(lib().fs3d_render_object(C.byref(view), _ptr(tri), tri.shape[0], W, H, rgba_ptr, stream))


def mesh_draw(vertices_ptr: int, n_vertices: int, material: int = MAT_BASIC, model=None, color=(1.0, 1.0, 1.0, 1.0),
              texture_ptr: int = 0, tex_width: int = 0, tex_height: int = 0) -> MeshDraw:
    """One draw of fs3d_render_meshes: vertices as {x,y,z,u,v} float32 (device or
    page-locked), model a row-major 4x4 (stored column-major), RGBA8 sRGB texture."""
    d = MeshDraw()
    d.vertices, d.n_vertices, d.material = vertices_ptr, n_vertices, material
    d.model[:] = [float(x) for x in np.asarray(model if model is not None else np.eye(4), np.float32).T.reshape(-1)]
    d.color[:] = [float(c) for c in color]
    d.texture, d.tex_width, d.tex_height = texture_ptr, tex_width, tex_height
    return d


def mesh_draws(draws) -> C.Array:
    """A ctypes array of MeshDraw, to pass to render_meshes_device frame after frame."""
    return (MeshDraw * max(len(draws), 1))(*draws)


def render_meshes_device(view: ObjectView, draws, W: int, H: int, rgba_ptr: int, stream: int = 0) -> None:
    """The basic_mat / textured_mat / tri materials over the given draws (a list of
    MeshDraw, or the array mesh_draws built) into W*H RGBA float32."""
    arr = draws if isinstance(draws, C.Array) else mesh_draws(draws)
    check(lib().fs3d_render_meshes(C.byref(view), arr, len(draws), W, H, rgba_ptr, stream))


# ---------------------------------------------------------------- device entry points
def step_device(grid_ptr: int, X: int, Y: int, Z: int, seed: int, t0: int, n_steps: int, stream: int = 0) -> None:
    """Drop-in step of a device grid (pointer) in place; async on `stream`."""
    check(lib().fs3d_step_device(grid_ptr, X, Y, Z, seed, t0, n_steps, stream))


def step_device_many(grid_ptrs, dims, seeds, t0: int, n_steps: int, stream: int = 0) -> None:
    """The drop-in kernel launched once per world per step from native code
    (device grids at grid_ptrs, dims an n x 3 array of X, Y, Z)."""
    n = len(grid_ptrs)
    ptrs = np.asarray(grid_ptrs if n else [0], dtype=np.uint64)
    d = np.ascontiguousarray(np.asarray(dims if n else [[1, 1, 1]], dtype=np.int32).reshape(-1, 3))
    sd = np.asarray(seeds if n else [0], dtype=np.uint64)
    check(lib().fs3d_step_device_many(n, ptrs.ctypes.data_as(C.POINTER(vp)), _ptr(d), _ptr(sd), t0, n_steps, stream))


def run_device(grid_ptr: int, X: int, Y: int, Z: int, seed: int, t0: int, n_steps: int, stream: int = 0) -> None:
    """n steps of a device grid through the bit-plane kernels (device scratch)."""
    check(lib().fs3d_run_device(grid_ptr, X, Y, Z, seed, t0, n_steps, stream))


def run_device_check(stream: int = 0, timeout_ns: int = -1) -> None:
    """Waits for `stream`, then raises Fs3dError(ERR_TIMEOUT) if a drop-in run on
    this device gave up a bounded copy wait since the last check (and clears it)."""
    check(lib().fs3d_run_device_check(stream, timeout_ns))


INJECT_NONE, INJECT_COPY_STALL, INJECT_ALLOC_FAIL = 0, 1, 2


def inject(what: int, count: int = 1) -> None:
    """Failure injection for tests (fs3d_test_inject); INJECT_NONE clears it."""
    check(lib().fs3d_test_inject(what, count))


def step_device_simple(grid_ptr: int, X: int, Y: int, Z: int, seed: int, t0: int, n_steps: int,
                       stream: int = 0) -> None:
    """One-thread-per-block reference kernel (same contract as step_device)."""
    check(lib().fs3d_step_device_simple(grid_ptr, X, Y, Z, seed, t0, n_steps, stream))


def hash_device(grid_ptr: int, n_cells: int, stream: int = 0) -> int:
    out = u64(0)
    check(lib().fs3d_hash_device(grid_ptr, n_cells, stream, C.byref(out)))
    return int(out.value)


def first_diff_device(a_ptr: int, b_ptr: int, n_cells: int, stream: int = 0) -> int:
    out = i64(0)
    check(lib().fs3d_first_diff_device(a_ptr, b_ptr, n_cells, stream, C.byref(out)))
    return int(out.value)


def render_sdf_device(cam: Camera, W: int, H: int, rgba_ptr: int, stream: int = 0) -> None:
    check(lib().fs3d_render_sdf(C.byref(cam), W, H, rgba_ptr, stream))


# ---------------------------------------------------------------- world
class World:
    """One device-resident world (library-owned memory and stream)."""

    def __init__(self, grid: np.ndarray, seed: int, start_step: int = 0, layout: int = LAYOUT_PLANES):
        g = np.ascontiguousarray(grid, dtype=np.uint8)
        if g.ndim != 3:
            raise ValueError("grid must have shape (Y, Z, X)")
        Y, Z, X = g.shape
        h = vp()
        check(lib().fs3d_world_create(_ptr(g), X, Y, Z, seed, start_step, layout, C.byref(h)))
        self._h = h
        self.X, self.Y, self.Z, self.seed, self.layout = X, Y, Z, seed, layout

    @classmethod
    def load(cls, path: str, layout: int = LAYOUT_PLANES) -> "World":
        self = cls.__new__(cls)
        h = vp()
        check(lib().fs3d_world_load(path.encode(), layout, C.byref(h)))
        self._h = h
        X, Y, Z, L = i32(), i32(), i32(), i32()
        seed, step = u64(), u64()
        check(lib().fs3d_world_info(h, C.byref(X), C.byref(Y), C.byref(Z), C.byref(seed), C.byref(step),
                                    C.byref(L)))
        self.X, self.Y, self.Z, self.seed, self.layout = X.value, Y.value, Z.value, seed.value, L.value
        return self

    @property
    def handle(self):
        if self._h is None:
            raise Fs3dError(ERR_STATE, "world destroyed")
        return self._h

    @property
    def step_counter(self) -> int:
        s = u64()
        check(lib().fs3d_world_info(self.handle, None, None, None, None, C.byref(s), None))
        return int(s.value)

    def step(self, n: int = 1) -> None:
        check(lib().fs3d_world_step(self.handle, n))

    def sync(self, timeout_ns: int = -1) -> None:
        check(lib().fs3d_world_sync(self.handle, timeout_ns))

    def read(self, out: Optional[np.ndarray] = None) -> np.ndarray:
        g = out if out is not None else np.empty((self.Y, self.Z, self.X), np.uint8)
        check(lib().fs3d_world_read(self.handle, _ptr(g)))
        return g

    def write(self, grid: np.ndarray) -> None:
        g = np.ascontiguousarray(grid, dtype=np.uint8)
        if g.shape != (self.Y, self.Z, self.X):
            raise ValueError("shape mismatch")
        check(lib().fs3d_world_write(self.handle, _ptr(g)))

    def hash(self) -> int:
        out = u64()
        check(lib().fs3d_world_hash(self.handle, C.byref(out)))
        return int(out.value)

    def device_ptr(self) -> int:
        p, L = vp(), i32()
        check(lib().fs3d_world_device_ptr(self.handle, C.byref(p), C.byref(L)))
        return int(p.value or 0)

    def stream(self) -> int:
        p = vp()
        check(lib().fs3d_world_stream(self.handle, C.byref(p)))
        return int(p.value or 0)

    def save(self, path: str) -> None:
        check(lib().fs3d_world_save(self.handle, path.encode()))

    def render(self, cam: Camera, W: int, H: int, mode: int = RENDER_DDA, out_ptr: Optional[int] = None):
        if out_ptr is not None:
            check(lib().fs3d_render(self.handle, C.byref(cam), W, H, mode, out_ptr, 1))
            return None
        img = np.empty((H, W, 4), np.float32)
        check(lib().fs3d_render(self.handle, C.byref(cam), W, H, mode, _ptr(img), 0))
        return img

    def close(self) -> None:
        if self._h is not None:
            check(lib().fs3d_world_destroy(self._h))
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------- batch
class Batch:
    """Pool of many worlds stepped together in graph-captured segments."""

    def __init__(self, budget_bytes: int, steps_per_segment: int = 64, use_graphs: bool = True,
                 ctas_per_sm: int = 0, use_smem=None):
        """use_smem: None = the library default; False/0 = per-step kernel only;
        True/1 = shared-memory resident segments; 2 = global-memory segments;
        3 = shared memory while a world's step counter is below 128, then
        global memory."""
        cfg = lib().fs3d_default_config()
        cfg.steps_per_segment = steps_per_segment
        cfg.use_graphs = 1 if use_graphs else 0
        if use_smem is not None:
            cfg.use_smem = int(use_smem)
        cfg.ctas_per_sm = ctas_per_sm
        h = vp()
        check(lib().fs3d_batch_create(budget_bytes, C.byref(cfg), C.byref(h)))
        self._h = h

    @property
    def handle(self):
        if self._h is None:
            raise Fs3dError(ERR_STATE, "batch destroyed")
        return self._h

    def admit(self, grid: np.ndarray, seed: int, n_steps: int, start_step: int = 0) -> int:
        g = np.ascontiguousarray(grid, dtype=np.uint8)
        Y, Z, X = g.shape
        t = u64()
        check(lib().fs3d_batch_admit(self.handle, _ptr(g), X, Y, Z, seed, start_step, n_steps, C.byref(t)))
        return int(t.value)

    def admit_generated(self, X: int, Y: int, Z: int, seed: int, n_steps: int, start_step: int = 0) -> int:
        """Admits the synthetic batch world of `seed`, generated on the device."""
        t = u64()
        check(lib().fs3d_batch_admit_generated(self.handle, X, Y, Z, seed, start_step, n_steps, C.byref(t)))
        return int(t.value)

    def admit_many(self, grids, seeds, n_steps, start_steps=None, ptrs=None, dims=None, wait=True):
        """Admits many grids with one host wait.  `ptrs` may give raw pointers
        (page-locked host or device buffers are gathered on the device in one
        pass) instead of the numpy arrays'; with `ptrs`, `dims` (an n x 3 array
        of X, Y, Z) may replace `grids`.  Returns the tickets of the admitted
        worlds (in order).  wait=False (with `ptrs`) returns once the uploads
        are enqueued: the buffers must stay unchanged until wait_copies()."""
        if not wait and ptrs is None:
            raise ValueError("admit_many(wait=False) needs ptrs to buffers the caller keeps alive")
        n = len(ptrs) if grids is None else len(grids)
        spec = np.zeros(max(n, 1), dtype=_SPEC_DTYPE)
        keep = None
        if n:
            if dims is not None:
                xyz = np.asarray(dims, dtype=np.int64).reshape(n, 3)
            else:
                shp = np.array([tuple(g.shape) for g in grids], dtype=np.int64).reshape(n, 3)  # (Y, Z, X)
                xyz = shp[:, [2, 0, 1]]
            if ptrs is None:
                keep = [np.ascontiguousarray(g, dtype=np.uint8) for g in grids]
                ptrs = [k.ctypes.data for k in keep]
            spec["grid"][:n] = np.asarray(ptrs, dtype=np.uint64)
            spec["X"][:n], spec["Y"][:n], spec["Z"][:n] = xyz[:, 0], xyz[:, 1], xyz[:, 2]
            spec["seed"][:n] = np.asarray(seeds, dtype=np.uint64)
            spec["start_step"][:n] = np.asarray(start_steps if start_steps is not None else 0, dtype=np.uint64)
            spec["n_steps"][:n] = np.asarray(n_steps, dtype=np.int64)
        tickets = np.zeros(max(n, 1), dtype=np.uint64)
        done = i32()
        fn = lib().fs3d_batch_admit_many if wait else lib().fs3d_batch_admit_many_async
        st = fn(self.handle, n, spec.ctypes.data_as(C.POINTER(WorldSpec)), tickets.ctypes.data_as(C.POINTER(u64)),
                C.byref(done))
        if st not in (OK, ERR_BUDGET):
            check(st)
        del keep
        return tickets[:done.value].tolist()

    def retire_many(self, tickets, out_ptrs=None, wait=True) -> None:
        """Retires worlds with one host wait; out_ptrs: host (or device) buffers, or None.
        wait=False returns once the read-backs are enqueued: the outputs hold
        the grids after wait_copies()."""
        n = len(tickets)
        ts = np.asarray(tickets if n else [0], dtype=np.uint64)
        outs = None
        if out_ptrs is not None:
            try:
                outs_arr = np.asarray(out_ptrs if n else [0], dtype=np.uint64)
            except TypeError:  # None entries: those worlds are not read back
                outs_arr = np.asarray([p or 0 for p in out_ptrs], dtype=np.uint64)
            outs = outs_arr.ctypes.data_as(C.POINTER(vp))
        fn = lib().fs3d_batch_retire_many if wait else lib().fs3d_batch_retire_many_async
        check(fn(self.handle, n, ts.ctypes.data_as(C.POINTER(u64)), outs))

    def read_many(self, tickets, out_ptrs) -> None:
        """Reads live worlds back into out_ptrs (host or device buffers) without
        retiring them; returns once the grids are there."""
        n = len(tickets)
        ts = np.asarray(tickets if n else [0], dtype=np.uint64)
        outs = np.asarray([p or 0 for p in out_ptrs] if n else [0], dtype=np.uint64)
        check(lib().fs3d_batch_read_many(self.handle, n, ts.ctypes.data_as(C.POINTER(u64)),
                                         outs.ctypes.data_as(C.POINTER(vp))))

    def wait_copies(self, timeout_ns: int = -1) -> None:
        """Waits for every admission upload and read-back enqueued so far."""
        check(lib().fs3d_batch_wait_copies(self.handle, timeout_ns))

    def try_admit(self, grid: np.ndarray, seed: int, n_steps: int, start_step: int = 0) -> Optional[int]:
        try:
            return self.admit(grid, seed, n_steps, start_step)
        except Fs3dError as e:
            if e.status == ERR_BUDGET:
                return None
            raise

    def run_segment(self) -> None:
        check(lib().fs3d_batch_run_segment(self.handle))

    def prepare(self) -> None:
        """Builds the next segment's tables now (fs3d_batch_prepare)."""
        check(lib().fs3d_batch_prepare(self.handle))

    def sync(self, timeout_ns: int = -1) -> None:
        check(lib().fs3d_batch_sync(self.handle, timeout_ns))

    def poll(self, ticket: int, with_hash: bool = True):
        done, h = i32(), u64()
        check(lib().fs3d_batch_poll(self.handle, ticket, C.byref(done), C.byref(h) if with_hash else None))
        return bool(done.value), (int(h.value) if done.value and with_hash else None)

    def poll_many(self, tickets, with_hash: bool = True):
        """(done, hashes) arrays for many worlds; hashes of the finished ones
        computed together."""
        n = len(tickets)
        ts = np.asarray(tickets if n else [0], dtype=np.uint64)
        done = np.zeros(max(n, 1), dtype=np.int32)
        hs = np.zeros(max(n, 1), dtype=np.uint64)
        check(lib().fs3d_batch_poll_many(self.handle, n, ts.ctypes.data_as(C.POINTER(u64)),
                                         done.ctypes.data_as(C.POINTER(i32)),
                                         hs.ctypes.data_as(C.POINTER(u64)) if with_hash else None))
        return done[:n].astype(bool), hs[:n]

    def retire(self, ticket: int, shape=None) -> Optional[np.ndarray]:
        if shape is None:
            check(lib().fs3d_batch_retire(self.handle, ticket, None))
            return None
        g = np.empty(shape, np.uint8)
        check(lib().fs3d_batch_retire(self.handle, ticket, _ptr(g)))
        return g

    def counters(self) -> dict:
        """Cell-steps since creation: all of them (dense) and those evaluated."""
        d, p = u64(0), u64(0)
        check(lib().fs3d_batch_counters(self.handle, C.byref(d), C.byref(p)))
        return {"dense_cell_steps": int(d.value), "processed_cell_steps": int(p.value)}

    def autotune(self, trial_segments: int = 2) -> dict:
        """Times the launch configurations on real segments and keeps the best."""
        r = TuneReport()
        check(lib().fs3d_batch_autotune(self.handle, trial_segments, C.byref(r)))
        return {"mode": r.mode, "promote": r.promote, "ctas_per_sm": r.ctas_per_sm, "trials": r.trials, "cached": bool(r.cached),
                "segments": r.segments, "best_vox_per_ms": r.best_vox_per_ms, "trial_vox_per_ms": list(r.trial_vox_per_ms)[:r.trials]}

    def stats(self):
        w, c = i64(), i64()
        u, b = C.c_size_t(), C.c_size_t()
        check(lib().fs3d_batch_stats(self.handle, C.byref(w), C.byref(c), C.byref(u), C.byref(b)))
        return {"live_worlds": w.value, "live_cells": c.value, "bytes_used": u.value, "bytes_budget": b.value}

    def stream(self) -> int:
        p = vp()
        check(lib().fs3d_batch_stream(self.handle, C.byref(p)))
        return int(p.value or 0)

    def close(self) -> None:
        if self._h is not None:
            check(lib().fs3d_batch_destroy(self._h))
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------- serving
def serve_params(lam: float, duration_s: float, master_seed: int = 1, max_requests: int = 0,
                 hbm_budget: int = 0, steps_per_segment: int = 64, min_steps: int = 10, max_steps: int = 1000,
                 with_hash: bool = True, segment_timeout_ms: int = 0) -> ServeParams:
    p = ServeParams()
    p.segment_timeout_ms = segment_timeout_ms
    p.lambda_, p.duration_s, p.max_requests, p.master_seed = lam, duration_s, max_requests, master_seed
    p.hbm_budget, p.steps_per_segment, p.min_steps, p.max_steps = hbm_budget, steps_per_segment, min_steps, max_steps
    p.with_hash = 1 if with_hash else 0
    return p


def serve_plan(p: ServeParams):
    n = i64()
    check(lib().fs3d_serve_plan(C.byref(p), 0, None, C.byref(n)))
    reqs = (ServeRequest * max(n.value, 1))()
    check(lib().fs3d_serve_plan(C.byref(p), n.value, reqs, C.byref(n)))
    return reqs, n.value


def serve(p: ServeParams):
    """Plans and serves the request stream; returns (stats dict, requests)."""
    reqs, n = serve_plan(p)
    st = ServeStats()
    check(lib().fs3d_serve_run(C.byref(p), n, reqs, C.byref(st)))
    stats = {f: getattr(st, f) for f, _ in ServeStats._fields_ if f != "reserved"}
    return stats, [reqs[i] for i in range(n)]
