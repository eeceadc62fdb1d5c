"""GPU render parity: the CUDA restatement of fs_raymarch.frag and the voxel
DDA against the CPU restatements.  Tolerance |d| <= 1e-5 per channel per pixel
(both sides use single IEEE operations in the same order, so the expected
difference is zero)."""
import numpy as np
import pytest

from gpu_util import to_device
import oracle_lib

pytestmark = pytest.mark.gpu
TOL = 1e-5


def check_img(got, exp):
    d = np.abs(got - exp)
    if d.max() > TOL:
        y, x, c = np.unravel_index(int(np.argmax(d)), d.shape)
        pytest.fail(f"pixel (x={x}, y={y}) channel {c}: got {got[y, x, c]} expected {exp[y, x, c]}")


@pytest.mark.parametrize("wh", [(850, 450), (320, 180), (64, 48)])
def test_sdf_sphere_matches_cpu(fs3d, orc, cuda, wh):
    W, H = wh
    cam = fs3d.camera_fs_raymarch()
    out = cuda.empty((H, W, 4), dtype=cuda.float32, device="cuda")
    fs3d.render_sdf_device(cam, W, H, out.data_ptr(), cuda.cuda.current_stream().cuda_stream)
    got = out.cpu().numpy()
    exp = orc.render_sdf(oracle_lib.camera_from(cam), W, H)
    check_img(got, exp)
    assert (got[..., 0] > 0.04).sum() > 0.01 * W * H  # the sphere is in view


@pytest.mark.parametrize("layout", [0, 1])
def test_dda_matches_cpu(fs3d, orc, layout):
    g = orc.gen_c1(9)
    orc.run(g, 9, 0, 30, nthreads=0)
    W, H = 160, 90
    cam = fs3d.camera_world_view(64, 64, 64, W, H)
    with fs3d.World(g, 9, 30, layout) as w:
        got = w.render(cam, W, H, fs3d.RENDER_DDA)
    exp = orc.render_dda(g, oracle_lib.camera_from(cam), W, H)
    check_img(got, exp)
    assert (exp[..., :3].sum(-1) > 0).mean() > 0.2


def test_dda_dunes_and_inside_camera(fs3d, orc):
    X, Y, Z = 96, 80, 112
    g = orc.gen_c5(3, X, Y, Z)
    W, H = 192, 108
    cams = [fs3d.camera_world_view(X, Y, Z, W, H)]
    inside = fs3d.camera_world_view(X, Y, Z, W, H)
    inside.origin[0], inside.origin[1], inside.origin[2] = 40.5, 70.25, 30.0
    cams.append(inside)
    with fs3d.World(g, 3, 0, fs3d.LAYOUT_PLANES) as w:
        for cam in cams:
            check_img(w.render(cam, W, H), orc.render_dda(g, oracle_lib.camera_from(cam), W, H))


def axis_camera(fs3d, origin, forward, right, up, W, H):
    c = fs3d.camera_world_view(8, 8, 8, W, H)
    for a in range(3):
        c.origin[a], c.forward[a], c.right[a], c.up[a] = origin[a], forward[a], right[a], up[a]
    return c


@pytest.mark.parametrize("layout", [0, 1])
def test_dda_empty_brick_crossings(fs3d, orc, layout):
    """Rays cross empty 8^3 bricks in one go on the GPU and cell by cell on the
    CPU: a sparse world whose sides are not multiples of 8, seen from outside
    and from inside, along the axes (rays with zero direction components, and
    the ties between axes that a ray at 45 degrees meets), and obliquely."""
    X, Y, Z = 37, 29, 45
    rng = np.random.default_rng(5)
    g = np.where(rng.random((Y, Z, X)) < 0.004, rng.integers(1, 4, (Y, Z, X)), 0).astype(np.uint8)
    g[0, : Z // 2] = 1
    g[Y - 1, Z - 3:, X - 5:] = 3
    W, H = 96, 64
    cams = [fs3d.camera_world_view(X, Y, Z, W, H),
            axis_camera(fs3d, (18.5, 14.5, -20.0), (0, 0, 1), (1, 0, 0), (0, 1, 0), W, H),
            axis_camera(fs3d, (18.0, 14.0, 22.0), (0, 0, 1), (1, 0, 0), (0, 1, 0), W, H),
            axis_camera(fs3d, (-10.0, 20.0, -10.0), (0.70710677, 0, 0.70710677), (0.70710677, 0, -0.70710677),
                        (0, 1, 0), W, H),
            axis_camera(fs3d, (36.5, 28.5, 44.5), (-0.57735026, -0.57735026, -0.57735026),
                        (0.70710677, -0.70710677, 0), (-0.40824830, -0.40824830, 0.81649661), W, H),
            axis_camera(fs3d, (4.0, 40.0, 4.0), (0, -1, 0), (1, 0, 0), (0, 0, 1), W, H)]
    with fs3d.World(g, 1, 0, layout) as w:
        for cam in cams:
            exp = orc.render_dda(g, oracle_lib.camera_from(cam), W, H)
            check_img(w.render(cam, W, H), exp)


def test_world_render_to_device(fs3d, orc, cuda):
    g = orc.gen_c1(2)
    W, H = 128, 72
    cam = fs3d.camera_world_view(64, 64, 64, W, H)
    with fs3d.World(g, 2, 0, fs3d.LAYOUT_BYTES) as w:
        out = cuda.zeros((H, W, 4), dtype=cuda.float32, device="cuda")
        w.render(cam, W, H, fs3d.RENDER_DDA, out_ptr=out.data_ptr())
        w.sync()
        check_img(out.cpu().numpy(), orc.render_dda(g, oracle_lib.camera_from(cam), W, H))


def _object_cases():
    rx = np.eye(4)
    c, s = np.cos(np.radians(30)), np.sin(np.radians(30))
    rx[1:3, 1:3] = [[c, -s], [s, c]]
    ry = np.eye(4)
    c, s = np.cos(np.radians(40)), np.sin(np.radians(40))
    ry[0, 0], ry[0, 2], ry[2, 0], ry[2, 2] = c, s, -s, c
    model = rx @ ry @ np.diag([1.2, 0.8, 1.0, 1.0])
    model[:3, 3] = (0.3, -0.2, 0.5)
    return [("scene", {}, (850, 450)), ("scene", {}, (1920, 1080)), ("scene", {}, (333, 217)),
            ("rot_y", {"rot_y": 25.0}, (850, 450)), ("model", {"model": model}, (640, 360)),
            ("moved", {"cam_pos": (1.5, -1.0, -3.0), "rot_y": -20.0}, (850, 450))]


@pytest.mark.parametrize("case", _object_cases(), ids=lambda c: f"{c[0]}-{c[2][0]}x{c[2][1]}")
def test_object_material_matches_cpu_bit_exact(fs3d, orc, cuda, case):
    _, kw, (W, H) = case
    tri = fs3d.mesh_cube()
    view = fs3d.object_view_scene(**kw)
    out = cuda.full((H, W, 4), -1.0, dtype=cuda.float32, device="cuda")
    fs3d.render_object_device(view, tri, W, H, out.data_ptr(), cuda.cuda.current_stream().cuda_stream)
    got = out.cpu().numpy()
    exp = orc.render_object(oracle_lib.scene_view(**kw), tri, W, H)
    assert exp is not None
    if not np.array_equal(got, exp):
        d = np.argwhere((got != exp).any(-1))
        y, x = d[0]
        pytest.fail(f"{len(d)} pixels differ; first (x={x}, y={y}): got {got[y, x]} expected {exp[y, x]}")
    assert (got[..., 0] > 0).sum() > 0.005 * W * H


def test_object_material_custom_mesh(fs3d, orc, cuda):
    """Two cubes (the second shifted and shrunk) and a ragged triangle count."""
    a = fs3d.mesh_cube()
    b = a * 0.4 + np.array([1.3, 0.2, -0.5], np.float32)
    tri = np.concatenate([a, b, a[:5] * 0.7])
    W, H = 512, 288
    view = fs3d.object_view_scene(rot_y=10.0)
    out = cuda.empty((H, W, 4), dtype=cuda.float32, device="cuda")
    fs3d.render_object_device(view, tri, W, H, out.data_ptr(), cuda.cuda.current_stream().cuda_stream)
    exp = orc.render_object(oracle_lib.scene_view(rot_y=10.0), tri, W, H)
    assert np.array_equal(out.cpu().numpy(), exp)


def test_dda_after_steps_of_a_large_world(fs3d, orc):
    """A plane world too large for the resident kernels (per-step kernel),
    rendered between runs of steps that rain water into empty bricks: every
    frame (brick map rebuilt from the current planes) equals the CPU DDA of
    the read-back grid exactly, from outside and from inside the world."""
    X, Y, Z = 256, 160, 192
    g = orc.gen_c5(11, X, Y, Z)
    W, H = 192, 108
    cam = fs3d.camera_world_view(X, Y, Z, W, H)
    low = fs3d.camera_world_view(X, Y, Z, W, H)
    low.origin[0], low.origin[1], low.origin[2] = 20.5, 30.25, 10.0
    with fs3d.World(g, 11, 0, fs3d.LAYOUT_PLANES) as w:
        check_img(w.render(cam, W, H), orc.render_dda(g, oracle_lib.camera_from(cam), W, H))
        for n in (40, 1, 75):
            w.step(n)
            cur = w.read()
            for c in (cam, low):
                check_img(w.render(c, W, H), orc.render_dda(cur, oracle_lib.camera_from(c), W, H))


def _mesh_scene(fs3d, orc, cuda, n_cubes=10, seed=3):
    """A few cubes with every material, as (gpu draws, oracle draws, tensors to keep)."""
    rng = np.random.default_rng(seed)
    v = orc.mesh_cube().reshape(-1, 3)
    cube = np.c_[v, (v[:, :2] + 1) * rng.uniform(0.5, 3.0)].astype(np.float32)
    tex = rng.integers(0, 256, (32, 24, 4), dtype=np.uint8)
    dv, dt = cuda.from_numpy(cube).cuda(), cuda.from_numpy(tex).cuda()
    gpu, cpu = [], []
    for i in range(n_cubes):
        m = np.eye(4)
        a = rng.uniform(0, 2 * np.pi)
        m[:3, :3] = [[np.cos(a), 0, np.sin(a)], [0, 1, 0], [-np.sin(a), 0, np.cos(a)]]
        m[:3, :3] *= rng.uniform(0.2, 0.7)
        m[:3, 3] = rng.uniform(-2.5, 2.5, 3)
        mat = i % 3
        col = tuple(rng.uniform(0, 1, 4))
        gpu.append(fs3d.mesh_draw(dv.data_ptr(), cube.shape[0], mat, m, col,
                                  dt.data_ptr() if mat else 0, tex.shape[1], tex.shape[0]))
        cpu.append(dict(vertices=cube, material=mat, model=m, color=col, texture=tex if mat else None))
    return gpu, cpu, (dv, dt)


@pytest.mark.parametrize("case", [("scene", {}, (850, 450)), ("turned", {"rot_y": 35.0}, (1920, 1080)),
                                  ("odd", {"cam_pos": (0.3, -0.2, -3.0)}, (333, 217)),
                                  ("inside", {"cam_pos": (0.0, 0.0, 0.0), "rot_y": 20.0}, (320, 180))],
                         ids=lambda c: c[0])
def test_mesh_materials_match_cpu_bit_exact(fs3d, orc, cuda, case):
    _, kw, (W, H) = case
    gpu, cpu, keep = _mesh_scene(fs3d, orc, cuda)
    if case[0] == "inside":  # one big cube around the camera, textured, plus the small ones
        big = np.eye(4) * 3.0
        big[3, 3] = 1.0
        gpu.append(fs3d.mesh_draw(gpu[1].vertices, 36, fs3d.MAT_TEXTURE, big, (1, 1, 1, 1), gpu[1].texture,
                                  gpu[1].tex_width, gpu[1].tex_height))
        cpu.append(dict(cpu[1], model=big, material=2))
    out = cuda.full((H, W, 4), -1.0, dtype=cuda.float32, device="cuda")
    fs3d.render_meshes_device(fs3d.object_view_scene(**kw), gpu, W, H, out.data_ptr(),
                              cuda.cuda.current_stream().cuda_stream)
    got = out.cpu().numpy()
    exp = orc.render_meshes(oracle_lib.scene_view(**kw), cpu, W, H)
    if not np.array_equal(got, exp):
        d = np.argwhere((got != exp).any(-1))
        y, x = d[0]
        pytest.fail(f"{len(d)} pixels differ; first (x={x}, y={y}): got {got[y, x]} expected {exp[y, x]}")
    assert ((got != [0, 0, 1, 1]).any(-1)).mean() > 0.01
    del keep


def test_mesh_pinned_vertices_and_pageable_rejected(fs3d, orc, cuda):
    v = orc.mesh_cube().reshape(-1, 3)
    cube = np.c_[v, np.zeros((36, 2))].astype(np.float32)
    pinned = cuda.from_numpy(cube).pin_memory()
    W, H = 128, 72
    out = cuda.empty((H, W, 4), dtype=cuda.float32, device="cuda")
    view = fs3d.object_view_scene(rot_y=10.0)
    fs3d.render_meshes_device(view, [fs3d.mesh_draw(pinned.data_ptr(), 36, fs3d.MAT_BASIC, None, (0, 1, 0, 1))],
                              W, H, out.data_ptr(), cuda.cuda.current_stream().cuda_stream)
    exp = orc.render_meshes(oracle_lib.scene_view(rot_y=10.0), [dict(vertices=cube, color=(0, 1, 0, 1))], W, H)
    assert np.array_equal(out.cpu().numpy(), exp)
    with pytest.raises(fs3d.Fs3dError) as e:
        fs3d.render_meshes_device(view, [fs3d.mesh_draw(cube.ctypes.data, 36)], W, H, out.data_ptr())
    assert e.value.status == fs3d.ERR_INVALID_ARG
