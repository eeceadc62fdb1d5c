"""ctypes binding of the CPU oracle (oracle/liboracle.so) for the tests.

The oracle is the checker: tests, the smoke check and the CPU-baseline leg of
the benchmark load it; the product never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_SO = os.path.join(ORACLE_DIR, "build", "liboracle.so")


class ObjectView(C.Structure):
    _fields_ = [("cam_pos", C.c_float * 3), ("cam_rot_y_deg", C.c_float), ("fovy_deg", C.c_float),
                ("aspect", C.c_float), ("znear", C.c_float), ("zfar", C.c_float), ("model", C.c_float * 16),
                ("clear", C.c_float * 4)]


def scene_view(**kw) -> ObjectView:
    """The upstream scene: camPos (0,0,-5), camRot 0, 70 degrees, aspect
    1700/900, depth 0.01..200, identity model, blue clear colour."""
    v = ObjectView()
    v.cam_pos[:] = kw.get("cam_pos", (0.0, 0.0, -5.0))
    v.cam_rot_y_deg = kw.get("rot_y", 0.0)
    v.fovy_deg, v.aspect, v.znear, v.zfar = 70.0, 1700.0 / 900.0, 0.01, 200.0
    v.model[:] = [float(x) for x in np.asarray(kw.get("model", np.eye(4)), np.float32).T.reshape(-1)]
    v.clear[:] = (0.0, 0.0, 1.0, 1.0)
    return v


class MeshDraw(C.Structure):
    _fields_ = [("vertices", C.c_void_p), ("n_vertices", C.c_int), ("material", C.c_int), ("model", C.c_float * 16),
                ("color", C.c_float * 4), ("texture", C.c_void_p), ("tex_width", C.c_int), ("tex_height", C.c_int)]


class Camera(C.Structure):
    _fields_ = [("origin", C.c_float * 3), ("forward", C.c_float * 3), ("right", C.c_float * 3),
                ("up", C.c_float * 3), ("tan_half_fov", C.c_float), ("aspect", C.c_float),
                ("light_pos", C.c_float * 3), ("reserved", C.c_int32)]


def build() -> str:
    src = os.path.join(ORACLE_DIR, "fs3d_oracle.c")
    if not os.path.exists(ORACLE_SO) or os.path.getmtime(ORACLE_SO) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", ORACLE_DIR], check=True)
    return ORACLE_SO


class Oracle:
    def __init__(self, path: str):
        L = C.CDLL(path)
        vp, i32, i64, u32, u64 = C.c_void_p, C.c_int, C.c_int64, C.c_uint32, C.c_uint64
        sig = {
            "orc_fmix32": (u32, [u32]), "orc_fmix64": (u64, [u64]),
            "orc_stepkey": (u32, [u64, u64]), "orc_rowkey": (u32, [u32, u32, u32]),
            "orc_plane": (u32, [u32, u32, u32, u32]),
            "orc_step": (None, [vp, i32, i32, i32, u64, u64]),
            "orc_step_shuffled": (None, [vp, i32, i32, i32, u64, u64, u64]),
            "orc_step_omp": (None, [vp, i32, i32, i32, u64, u64, i32]),
            "orc_run": (None, [vp, i32, i32, i32, u64, u64, i32, vp, i32]),
            "orc_block_would_change": (i32, [vp, i32, i32, i32, u64, i32, i32, i32]),
            "orc_hash": (u64, [vp, i64]), "orc_first_diff": (i64, [vp, vp, i64]),
            "orc_gen_c1": (None, [u64, i32, i32, i32, vp]), "orc_gen_c2": (None, [u64, i32, i32, i32, vp]),
            "orc_gen_c3_dims": (None, [u64, i32, vp, vp]), "orc_gen_c3_world": (None, [u64, i32, i32, i32, vp]),
            "orc_gen_c5": (None, [u64, i32, i32, i32, vp]),
            "orc_render_sdf": (None, [C.POINTER(Camera), i32, i32, vp]),
            "orc_render_dda": (None, [vp, i32, i32, i32, C.POINTER(Camera), i32, i32, vp]),
            "orc_render_object": (i32, [C.POINTER(ObjectView), vp, i32, i32, i32, vp]),
            "orc_object_mvp": (None, [C.POINTER(ObjectView), vp]),
            "orc_mesh_cube": (i32, [vp]),
            "orc_render_meshes": (i32, [C.POINTER(ObjectView), C.POINTER(MeshDraw), i32, i32, i32, vp]),
            "orc_srgb_table": (None, [vp]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        self.L = L

    # -- rule
    def step(self, g: np.ndarray, seed: int, t: int) -> None:
        Y, Z, X = g.shape
        self.L.orc_step(g.ctypes.data, X, Y, Z, seed, t)

    def step_shuffled(self, g, seed, t, order_seed) -> None:
        Y, Z, X = g.shape
        self.L.orc_step_shuffled(g.ctypes.data, X, Y, Z, seed, t, order_seed)

    def step_omp(self, g, seed, t, nthreads=0) -> None:
        Y, Z, X = g.shape
        self.L.orc_step_omp(g.ctypes.data, X, Y, Z, seed, t, nthreads)

    def run(self, g: np.ndarray, seed: int, t0: int, n: int, nthreads: int = 1, hashes: bool = False):
        Y, Z, X = g.shape
        h = np.zeros(max(n, 1), np.uint64)
        self.L.orc_run(g.ctypes.data, X, Y, Z, seed, t0, n, h.ctypes.data if hashes else None, nthreads)
        return h[:n] if hashes else None

    def hash(self, g: np.ndarray) -> int:
        return int(self.L.orc_hash(g.ctypes.data, g.size))

    def first_diff(self, a: np.ndarray, b: np.ndarray) -> int:
        return int(self.L.orc_first_diff(a.ctypes.data, b.ctypes.data, a.size))

    def would_change(self, g, t, i, j, k) -> bool:
        Y, Z, X = g.shape
        return bool(self.L.orc_block_would_change(g.ctypes.data, X, Y, Z, t, i, j, k))

    # -- generators
    def _gen(self, fn, seed, X, Y, Z):
        g = np.empty((Y, Z, X), np.uint8)
        getattr(self.L, fn)(seed, X, Y, Z, g.ctypes.data)
        return g

    def gen_c1(self, seed, X=64, Y=64, Z=64):
        return self._gen("orc_gen_c1", seed, X, Y, Z)

    def gen_c2(self, seed, X=512, Y=512, Z=512):
        return self._gen("orc_gen_c2", seed, X, Y, Z)

    def gen_c3_world(self, seed, X, Y, Z):
        return self._gen("orc_gen_c3_world", seed, X, Y, Z)

    def gen_c5(self, seed, X=1024, Y=1024, Z=1024):
        return self._gen("orc_gen_c5", seed, X, Y, Z)

    def gen_c3_dims(self, master, count):
        dims = np.empty((count, 3), np.int32)
        seeds = np.empty(count, np.uint64)
        self.L.orc_gen_c3_dims(master, count, dims.ctypes.data, seeds.ctypes.data)
        return dims, seeds

    # -- render
    def render_sdf(self, cam: Camera, W: int, H: int) -> np.ndarray:
        img = np.empty((H, W, 4), np.float32)
        self.L.orc_render_sdf(C.byref(cam), W, H, img.ctypes.data)
        return img

    def mesh_cube(self) -> np.ndarray:
        tri = np.empty((12, 3, 3), np.float32)
        self.L.orc_mesh_cube(tri.ctypes.data)
        return tri

    def object_mvp(self, view: ObjectView) -> np.ndarray:
        m = np.empty(16, np.float32)
        self.L.orc_object_mvp(C.byref(view), m.ctypes.data)
        return m.reshape(4, 4).T  # row-major view of the column-major matrix

    def render_object(self, view: ObjectView, tri: np.ndarray, W: int, H: int):
        """RGBA image, or None when the oracle rejects the view."""
        tri = np.ascontiguousarray(tri, np.float32)
        img = np.empty((H, W, 4), np.float32)
        rc = self.L.orc_render_object(C.byref(view), tri.ctypes.data, tri.shape[0], W, H, img.ctypes.data)
        return img if rc == 0 else None

    def render_meshes(self, view: ObjectView, draws, W: int, H: int) -> np.ndarray:
        """draws: dicts with vertices (n x 5 float32), material, model (4x4 row-major), color, texture
        (h x w x 4 uint8)."""
        keep, arr = [], (MeshDraw * max(len(draws), 1))()
        for i, d in enumerate(draws):
            v = np.ascontiguousarray(d["vertices"], np.float32)
            keep.append(v)
            m = arr[i]
            m.vertices, m.n_vertices, m.material = v.ctypes.data, v.shape[0], d.get("material", 0)
            m.model[:] = [float(x) for x in np.asarray(d.get("model", np.eye(4)), np.float32).T.reshape(-1)]
            m.color[:] = [float(c) for c in d.get("color", (1, 1, 1, 1))]
            tex = d.get("texture")
            if tex is not None:
                tex = np.ascontiguousarray(tex, np.uint8)
                keep.append(tex)
                m.texture, m.tex_width, m.tex_height = tex.ctypes.data, tex.shape[1], tex.shape[0]
        img = np.empty((H, W, 4), np.float32)
        assert self.L.orc_render_meshes(C.byref(view), arr, len(draws), W, H, img.ctypes.data) == 0
        return img

    def srgb_table(self) -> np.ndarray:
        t = np.empty(256, np.float32)
        self.L.orc_srgb_table(t.ctypes.data)
        return t

    def render_dda(self, g: np.ndarray, cam: Camera, W: int, H: int) -> np.ndarray:
        Y, Z, X = g.shape
        img = np.empty((H, W, 4), np.float32)
        self.L.orc_render_dda(g.ctypes.data, X, Y, Z, C.byref(cam), W, H, img.ctypes.data)
        return img


_oracle = None


def load() -> Oracle:
    """The oracle; FS3D_ORACLE_SO names another build of the same source (the
    tests run it once more built at -O0 with the undefined-behaviour checks)."""
    global _oracle
    if _oracle is None:
        _oracle = Oracle(os.environ.get("FS3D_ORACLE_SO") or build())
    return _oracle


def camera_from(fs3d_cam) -> Camera:
    """Copies a product camera struct into the oracle's (same layout)."""
    c = Camera()
    C.memmove(C.byref(c), C.byref(fs3d_cam), C.sizeof(Camera))
    return c
