"""CPU checks of the oracle: known-answer blocks for every rule clause, an
independent Python statement of the rule, invariants, order independence and
the self-recorded golden vectors (parity with the upstream project is
unpinned: it contains no step to compare against)."""
import json
import os

import numpy as np
import pytest

import oracle_lib
import rule_py

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "golden.json")
EMPTY, STONE, SAND, WATER = 0, 1, 2, 3


def cube(fill=EMPTY, X=2, Y=2, Z=2):
    return np.full((Y, Z, X), fill, np.uint8)


def test_hash_primitives_match_python(orc):
    for v in [0, 1, 0xDEADBEEF, 0xFFFFFFFF, 12345]:
        assert orc.L.orc_fmix32(v) == rule_py.fmix32(v)
    for v in [0, 1, 2**63 + 5, 0xFFFFFFFFFFFFFFFF]:
        assert orc.L.orc_fmix64(v) == rule_py.fmix64(v)
    for seed, t in [(0, 0), (1, 7), (2**40 + 3, 2**33 + 1)]:
        sk = orc.L.orc_stepkey(seed, t)
        assert sk == rule_py.stepkey(seed, t)
        assert orc.L.orc_rowkey(sk, 3, 5) == rule_py.rowkey(sk, 3, 5)
        assert orc.L.orc_plane(sk, 2, 7, 4) == rule_py.plane(sk, 2, 7, 4)


def test_kat_fall_straight_down(orc):
    for m in (SAND, WATER):
        g = cube()
        g[1, 0, 0] = m  # (y=1, z=0, x=0): top layer, column 0
        orc.step(g, 1, 0)
        exp = cube()
        exp[0, 0, 0] = m
        assert (g == exp).all()


def test_kat_stone_and_static_materials_hold(orc):
    g = cube()
    g[1, 0, 0] = STONE
    g[1, 1, 1] = 9
    g0 = g.copy()
    orc.step(g, 1, 0)
    assert (g == g0).all()


@pytest.mark.parametrize("seed", range(6))
def test_kat_diagonal_slide_uses_draw(orc, seed):
    g = cube()
    g[1, 0, 0] = SAND
    g[0, 0, 0] = STONE  # straight below is blocked; 3 empty bottom candidates
    orc.step(g, seed, 0)
    rk = rule_py.rowkey(rule_py.stepkey(seed, 0), 0, 0)
    r = rule_py.draw(3, rk, 0, 0)
    q = [1, 2, 3][r]  # candidates in column order
    exp = cube()
    exp[0, 0, 0] = STONE
    exp[0, q >> 1, q & 1] = SAND
    assert (g == exp).all()


@pytest.mark.parametrize("seed", range(6))
def test_kat_water_sideways_bottom(orc, seed):
    g = cube()
    g[0, 1, 1] = WATER  # bottom layer, column 3
    g[0, 0, 0] = STONE  # candidates: columns 1, 2
    orc.step(g, seed, 0)
    rk = rule_py.rowkey(rule_py.stepkey(seed, 0), 0, 0)
    q = [1, 2][rule_py.draw(2, rk, 0, 7)]
    exp = cube()
    exp[0, 0, 0] = STONE
    exp[0, q >> 1, q & 1] = WATER
    assert (g == exp).all()


def test_kat_sand_never_moves_sideways(orc):
    g = cube()
    g[0, 0, 0] = SAND
    g0 = g.copy()
    orc.step(g, 3, 0)
    assert (g == g0).all()


def test_kat_sand_does_not_displace_water(orc):
    g = cube(fill=STONE)
    g[1, 0, 0] = SAND
    g[0, 0, 0] = WATER
    g0 = g.copy()
    orc.step(g, 3, 0)
    assert (g == g0).all()


def test_kat_outside_cells_are_solid(orc):
    # X = 1: every block is missing its dx=1 column
    g = np.zeros((2, 2, 1), np.uint8)
    g[1, 0, 0] = SAND
    g[0, 0, 0] = STONE
    orc.step(g, 5, 0)  # only diagonal candidate is (y=0, z=1)
    assert g[0, 1, 0] == SAND and g[1, 0, 0] == EMPTY
    # one layer, two cells along z: in the even phase both cells share a block
    # (the layer is its bottom, y = 1 lies outside) and the water spreads to
    # z = 1; in the odd phase z = 0 and z = 1 sit in different blocks
    g = np.zeros((1, 2, 1), np.uint8)
    g[0, 0, 0] = WATER
    orc.step(g, 5, 1)
    assert g[0, 0, 0] == WATER and g[0, 1, 0] == EMPTY
    orc.step(g, 5, 0)
    assert g[0, 1, 0] == WATER and g[0, 0, 0] == EMPTY


@pytest.mark.parametrize("seed", range(8))
def test_kat_moved_particle_moves_once(orc, seed):
    g = cube()
    g[0] = STONE
    g[1, 0, 0] = WATER  # slides to a random top column, then stays there
    orc.step(g, seed, 0)
    assert (g[0] == STONE).all()
    assert (g[1] == WATER).sum() == 1 and g[1, 0, 0] == EMPTY
    rk = rule_py.rowkey(rule_py.stepkey(seed, 0), 0, 0)
    q = [1, 2, 3][rule_py.draw(3, rk, 0, 0)]
    assert g[1, q >> 1, q & 1] == WATER


@pytest.mark.parametrize("dims", [(5, 4, 3), (7, 6, 9), (8, 8, 8), (1, 6, 5), (13, 3, 2)])
def test_oracle_matches_python_statement(orc, dims):
    X, Y, Z = dims
    rng = np.random.default_rng(X * 100 + Y * 10 + Z)
    g = rng.choice(np.array([0, 0, 0, 1, 2, 3, 5], np.uint8), size=(Y, Z, X))
    p = g.copy()
    for t in range(6):
        orc.step(g, 99, t)
        rule_py.step(p, 99, t)
        assert (g == p).all(), f"step {t}: first diff {orc.first_diff(g, p)}"
    assert orc.hash(g) == rule_py.grid_hash(g)


def test_invariants_and_order_independence(orc):
    g = orc.gen_c1(7, 48, 40, 36)
    st = g == STONE
    counts = np.bincount(g.reshape(-1), minlength=4)
    a, b, c = g.copy(), g.copy(), g.copy()
    for t in range(40):
        orc.step(a, 7, t)
        orc.step_shuffled(b, 7, t, 1000 + t)
        orc.step_omp(c, 7, t, 4)
        assert (a == b).all() and (a == c).all(), t
    assert (np.bincount(a.reshape(-1), minlength=4) == counts).all()
    assert ((a == STONE) == st).all()


def test_stability_does_not_depend_on_draws(orc):
    rng = np.random.default_rng(3)
    for _ in range(300):
        g = rng.choice(np.array([0, 1, 2, 3], np.uint8), size=(2, 2, 2), p=[0.4, 0.2, 0.2, 0.2])
        changed = []
        for seed in range(4):
            h = g.copy()
            orc.step(h, seed, 0)
            changed.append(not (h == g).all())
        assert len(set(changed)) == 1
        assert orc.would_change(g, 0, 0, 0, 0) == changed[0]


def test_generators_are_stable(orc):
    a = orc.gen_c1(11)
    b = orc.gen_c1(11)
    assert (a == b).all() and not (a == orc.gen_c1(12)).all()
    counts = np.bincount(a.reshape(-1), minlength=4)
    upper = 64 * 64 * 32
    assert abs(counts[SAND] / upper - 0.25) < 0.01 and abs(counts[WATER] / upper - 0.15) < 0.01
    dims, seeds = orc.gen_c3_dims(1, 2048)
    assert set(np.unique(dims)) <= {16, 24, 32, 48, 64, 96, 128}


def test_golden_vectors(orc):
    with open(GOLDEN) as f:
        gold = json.load(f)
    for key, exp in gold["parity_runs"].items():
        seed = int(key)
        g = orc.gen_c1(seed)
        hs = orc.run(g, seed, 0, len(exp), nthreads=0, hashes=True)
        assert [int(h) for h in hs] == [int(h) for h in exp], seed
    gen = gold["generators"]
    assert orc.hash(orc.gen_c1(1)) == int(gen["parity_s1_64"])
    assert orc.hash(orc.gen_c2(1, 128, 160, 96)) == int(gen["pillars_s1_128x160x96"])
    assert orc.hash(orc.gen_c5(1, 128, 128, 128)) == int(gen["dunes_s1_128"])
    dims, seeds = orc.gen_c3_dims(1, 2048)
    assert rule_py.fmix64(int(np.bitwise_xor.reduce(seeds))) == int(gen["batch_seeds_m1_2048"])
    assert int(dims.sum()) == int(gen["batch_dims_sum_m1_2048"])
    for w in range(4):
        X, Y, Z = (int(v) for v in dims[w])
        assert orc.hash(orc.gen_c3_world(int(seeds[w]), X, Y, Z)) == int(gen["batch_world_%d" % w])
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(os.path.dirname(GOLDEN), "make_golden.py"))
    make_golden = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(make_golden)
    assert make_golden.dda_digest(orc) == gold["renders"]["dda_dunes64_s1_t30_64x48"]


# ---- raymarch_sphere material (rasterised mesh + box SDF march)

def _rot(axis, deg):
    c, s = np.cos(np.radians(deg)), np.sin(np.radians(deg))
    m = np.eye(4)
    i, j = [(1, 2), (2, 0), (0, 1)][axis]
    m[i, i] = m[j, j] = c
    m[i, j], m[j, i] = -s, s
    return m


def _object_views():
    model = _rot(0, 30) @ _rot(1, 40)
    model[:3, 3] = (0.3, -0.2, 0.5)
    return {"scene": {}, "rot_y": {"rot_y": 25.0}, "model": {"model": model},
            "moved": {"cam_pos": (1.5, -1.0, -3.0), "rot_y": -20.0}}


def _ray_box(o, d, h):
    with np.errstate(divide="ignore", invalid="ignore"):
        t0, t1 = (-h - o) / d, (h - o) / d
    tmin = np.nanmax(np.minimum(t0, t1), -1)
    tmax = np.nanmin(np.maximum(t0, t1), -1)
    return tmax >= np.maximum(tmin, 0)


def _numpy_statement(orc, view, tri, W, H):
    """Independent float64 statement: rasterise with screen-space (noperspective)
    barycentrics and nearest depth, then intersect the ray from the object-space
    camera through the interpolated position with the half-extent-0.5 box
    analytically.  Returns (covered, box hit)."""
    mvp = orc.object_mvp(view).astype(np.float64)
    model = np.array(view.model, np.float64).reshape(4, 4).T
    o = (np.linalg.inv(model) @ np.r_[-np.array(view.cam_pos, np.float64), 1.0])[:3]
    px, py = np.meshgrid(np.arange(W) + 0.5, np.arange(H) + 0.5)
    best = np.full((H, W), np.inf)
    pos = np.zeros((H, W, 3))
    for t in tri.astype(np.float64):
        c = np.c_[t, np.ones(3)] @ mvp.T
        s = c[:, :3] / c[:, 3:]
        sx, sy, sz = (s[:, 0] + 1) * W / 2, (s[:, 1] + 1) * H / 2, s[:, 2]
        area = (sx[1] - sx[0]) * (sy[2] - sy[0]) - (sy[1] - sy[0]) * (sx[2] - sx[0])
        if area == 0:
            continue
        lam = []
        for a, b in ((1, 2), (2, 0), (0, 1)):
            lam.append(((sx[b] - sx[a]) * (py - sy[a]) - (sy[b] - sy[a]) * (px - sx[a])) / area)
        inside = (lam[0] >= 0) & (lam[1] >= 0) & (lam[2] >= 0)
        z = lam[0] * sz[0] + lam[1] * sz[1] + lam[2] * sz[2]
        take = inside & (z <= best)
        best[take] = z[take]
        p = lam[0][..., None] * t[0] + lam[1][..., None] * t[1] + lam[2][..., None] * t[2]
        pos[take] = p[take]
    covered = np.isfinite(best)
    hit = _ray_box(np.broadcast_to(o, pos.shape), pos - o, 0.5) & covered
    return covered, hit


@pytest.mark.parametrize("name", list(_object_views()))
def test_object_render_matches_independent_statement(orc, name):
    tri = orc.mesh_cube()
    view = oracle_lib.scene_view(**_object_views()[name])
    W, H = 425, 225
    img = orc.render_object(view, tri, W, H)
    assert img is not None
    covered, hit = _numpy_statement(orc, view, tri, W, H)
    got_cov = ~((img[..., 0] == 0) & (img[..., 1] == 0) & (img[..., 2] == 1))
    got_hit = img[..., 0] > 0
    # pixel centres on a triangle edge or grazing the box may fall either way
    assert (got_cov != covered).sum() <= 2e-3 * covered.sum() + 2, name
    assert (got_hit != hit).sum() <= 1e-2 * hit.sum() + 4, name
    assert covered.sum() > 0 and hit.sum() > 0
    # shading: 1 - 0.05 per march step, at least 0.05; alpha 1 wherever covered
    vals = np.unique(img[..., 0][got_hit])
    assert ((vals >= 0.05) & (vals <= 1.0)).all()
    assert (img[..., 3] == 1).all()


def test_object_render_scene_is_axis_aligned_exact(orc):
    """The scene's default view looks straight at the cube's front face, where
    screen-space interpolation is exact: cube and box coverage equal a
    true-perspective ray-vs-box test pixel for pixel."""
    tri = orc.mesh_cube()
    view = oracle_lib.scene_view()
    W, H = 850, 450
    img = orc.render_object(view, tri, W, H)
    inv = np.linalg.inv(orc.object_mvp(view).astype(np.float64))
    px, py = np.meshgrid(np.arange(W) + 0.5, np.arange(H) + 0.5)

    def unproject(z):
        p = np.stack([px / (W / 2) - 1, py / (H / 2) - 1, np.full_like(px, z), np.ones_like(px)], -1) @ inv.T
        return p[..., :3] / p[..., 3:]

    a, b = unproject(0.3), unproject(0.9)
    assert ((img[..., 2] != 1) == _ray_box(a, b - a, 1.0)).all()
    assert ((img[..., 0] > 0) == _ray_box(a, b - a, 0.5)).all()


def test_object_render_noperspective_bends_oblique_rays(orc):
    """The material's noperspective attributes bend the rays of faces seen at
    an angle: with the camera turned 25 degrees a large share of the box's
    pixels differ from a true-perspective ray test (the upstream image does
    this too), while the cube's silhouette stays exact."""
    tri = orc.mesh_cube()
    view = oracle_lib.scene_view(rot_y=25.0)
    W, H = 425, 225
    img = orc.render_object(view, tri, W, H)
    inv = np.linalg.inv(orc.object_mvp(view).astype(np.float64))
    px, py = np.meshgrid(np.arange(W) + 0.5, np.arange(H) + 0.5)
    p = [np.stack([px / (W / 2) - 1, py / (H / 2) - 1, np.full_like(px, z), np.ones_like(px)], -1) @ inv.T
         for z in (0.3, 0.9)]
    a, b = (q[..., :3] / q[..., 3:] for q in p)
    true_box = _ray_box(a, b - a, 0.5)
    assert ((img[..., 2] != 1) == _ray_box(a, b - a, 1.0)).all()
    assert ((img[..., 0] > 0) != true_box).sum() > 0.1 * true_box.sum()


def test_object_render_translation_equivalence_and_rejections(orc):
    tri = orc.mesh_cube()
    T = np.eye(4)
    T[:3, 3] = (0.4, -0.3, 0.2)
    a = orc.render_object(oracle_lib.scene_view(model=T), tri, 320, 180)
    b = orc.render_object(oracle_lib.scene_view(cam_pos=(0.4, -0.3, -4.8)), tri, 320, 180)
    assert np.array_equal(a, b)
    assert orc.render_object(oracle_lib.scene_view(cam_pos=(0.0, 0.0, -1.0)), tri, 64, 32) is None  # eye in the cube
    assert orc.render_object(oracle_lib.scene_view(model=np.zeros((4, 4))), tri, 64, 32) is None


# ---- mesh materials (rasterised triangles, depth test, textures)

def _cube_uv(orc):
    v = orc.mesh_cube().reshape(-1, 3)
    return np.c_[v, (v[:, :2] + 1) * 0.5].astype(np.float32)


def _rays(orc, view, W, H):
    inv = np.linalg.inv(orc.object_mvp(view).astype(np.float64))
    px, py = np.meshgrid(np.arange(W) + 0.5, np.arange(H) + 0.5)
    p = [np.stack([px / (W / 2) - 1, py / (H / 2) - 1, np.full_like(px, z), np.ones_like(px)], -1) @ inv.T
         for z in (0.3, 0.9)]
    a, b = (q[..., :3] / q[..., 3:] for q in p)
    return a, b - a


@pytest.mark.parametrize("rot", [0.0, 25.0, -60.0])
def test_mesh_basic_coverage_matches_analytic(orc, rot):
    view = oracle_lib.scene_view(rot_y=rot)
    W, H = 320, 180
    img = orc.render_meshes(view, [dict(vertices=_cube_uv(orc), material=0, color=(1, 0, 0, 1))], W, H)
    o, d = _rays(orc, view, W, H)
    cov = _ray_box(o, d, 1.0)
    got = img[..., 2] != 1
    assert (got != cov).sum() <= 2e-3 * cov.sum() + 2
    assert (img[got][:, 0] == 1).all() and (img[~got] == [0, 0, 1, 1]).all()


def test_mesh_camera_inside_cube_is_clipped(orc):
    """Triangles crossing the near plane are clipped, not dropped: from the
    cube's centre every pixel sees a face."""
    img = orc.render_meshes(oracle_lib.scene_view(cam_pos=(0.0, 0.0, 0.0), rot_y=33.0),
                            [dict(vertices=_cube_uv(orc), material=0, color=(0, 1, 0, 1))], 160, 90)
    assert (img[..., 1] == 1).all()


@pytest.mark.parametrize("rot", [0.0, 40.0])
def test_mesh_texture_perspective_correct(orc, rot):
    """A textured quad, head-on and turned: the texel of each pixel equals the
    one a float64 ray-plane intersection gives (nearest, repeat), except for
    pixels within 1e-3 texel of a texel boundary."""
    rng = np.random.default_rng(5)
    tex = rng.integers(0, 256, (16, 16, 4), dtype=np.uint8)
    quad = np.array([[-1, -1, 0, 0, 0], [1, -1, 0, 2, 0], [1, 1, 0, 2, 2],
                     [-1, -1, 0, 0, 0], [1, 1, 0, 2, 2], [-1, 1, 0, 0, 2]], np.float32)  # uv 0..2: repeats
    c, s = np.cos(np.radians(rot)), np.sin(np.radians(rot))
    model = np.array([[c, 0, s, 0], [0, 1, 0, 0], [-s, 0, c, 0], [0, 0, 0, 1]], np.float64)
    view = oracle_lib.scene_view(cam_pos=(0.0, 0.0, -2.5))
    W, H = 256, 144
    img = orc.render_meshes(view, [dict(vertices=quad, material=2, texture=tex, model=model)], W, H)
    o, d = _rays(orc, view, W, H)
    n = model[:3, :3] @ [0, 0, 1.0]
    t = -(o @ n) / (d @ n)
    hit = o + t[..., None] * d
    local = hit @ model[:3, :3]  # back to object space (orthonormal)
    inside = (np.abs(local[..., 0]) <= 1) & (np.abs(local[..., 1]) <= 1) & (t > 0)
    u, v = (local[..., 0] + 1), (local[..., 1] + 1)  # 0..2
    fu, fv = u * 16, v * 16
    sure = inside & (np.abs(fu - np.round(fu)) > 1e-3) & (np.abs(fv - np.round(fv)) > 1e-3)
    sure &= (np.abs(local[..., 0]) < 0.999) & (np.abs(local[..., 1]) < 0.999)
    ti, tj = np.floor(fu).astype(int) % 16, np.floor(fv).astype(int) % 16
    lut = orc.srgb_table()
    exp = lut[tex[tj, ti, 0]]
    assert sure.sum() > 1000
    assert (img[..., 0][sure] == exp[sure]).mean() > 0.995
    assert (img[..., 3][inside] == 1).all()


def test_mesh_depth_ties_and_materials(orc):
    """Coplanar quads: the later draw wins (LESS_OR_EQUAL); a farther one is
    hidden; textured_mat adds the colour to the texel and 1 to alpha (the
    attachment clamps to [0,1])."""
    quad = np.array([[-1, -1, 0, 0, 0], [1, -1, 0, 1, 0], [1, 1, 0, 1, 1],
                     [-1, -1, 0, 0, 0], [1, 1, 0, 1, 1], [-1, 1, 0, 0, 1]], np.float32)
    back = quad.copy()
    back[:, 2] = -0.5
    tex = np.full((2, 2, 4), 128, np.uint8)
    view = oracle_lib.scene_view()
    W, H = 160, 90
    img = orc.render_meshes(view, [dict(vertices=quad, material=0, color=(1, 0, 0, 1)),
                                   dict(vertices=quad, material=1, color=(0.1, 0.2, 0.3, 0.5), texture=tex),
                                   dict(vertices=back, material=0, color=(0, 0, 0, 1))], W, H)
    cov = img[..., 2] != 1
    cov &= ~((img[..., 0] == 0) & (img[..., 1] == 0) & (img[..., 2] == 1))
    lut = orc.srgb_table()
    exp = np.float32([0.1, 0.2, 0.3]) + lut[128]
    assert cov.sum() > 500
    assert np.allclose(img[cov][:, :3], exp, atol=0) and (img[cov][:, 3] == 1).all()


def _camera(origin, forward, right, up, W, H):
    c = oracle_lib.Camera()
    for a in range(3):
        c.origin[a], c.forward[a], c.right[a], c.up[a] = origin[a], forward[a], right[a], up[a]
    c.tan_half_fov, c.aspect = 0.6, W / H
    c.light_pos[0], c.light_pos[1], c.light_pos[2] = 20.0, 30.0, 10.0
    return c


def test_dda_oracle_matches_python_walk(orc):
    """The oracle's voxel DDA against an independent Python statement of the
    same walk (float32 operations, boundary keys fma(n, e, b) rounded once):
    equal image for image, from outside the grid and from inside it along an
    axis (direction components of zero)."""
    import dda_py
    rng = np.random.default_rng(17)
    g = np.where(rng.random((10, 14, 12)) < 0.08, rng.choice(np.array([1, 2, 3, 7], np.uint8), (10, 14, 12)), 0)
    g = g.astype(np.uint8)
    W, H = 20, 12
    s = np.float32(np.sqrt(0.5))
    cams = [_camera((-6.3, 14.2, -8.1), (0.6, -0.48, 0.64), (0.7271, 0.0, -0.6865), (0.3295, 0.8776, 0.349), W, H),
            _camera((5.5, 4.25, 1.0), (0.0, 0.0, 1.0), (1.0, 0.0, 0.0), (0.0, 1.0, 0.0), W, H),
            _camera((-3.0, 12.0, -3.0), (s, 0.0, s), (s, 0.0, -s), (0.0, 1.0, 0.0), W, H)]
    for cam in cams:
        got = orc.render_dda(g, cam, W, H)
        exp = dda_py.render(g, cam, W, H)
        assert np.array_equal(got, exp), np.argwhere(np.any(got != exp, axis=-1))[:5]
        assert (exp[..., :3].sum(-1) > 0).any()
