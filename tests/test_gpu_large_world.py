"""GPU parity of the per-step kernel of one large world (exact skip of settled
row-pairs by per-row change bytes) against the CPU oracle, whole-grid hash
after every step, first differing voxel on failure.  The worlds are too large
for the shared-memory resident kernels, so the world object steps them with
the per-step kernel; rows of 1 to 32 plane words, odd sizes in y and z,
static materials.  Integer work: bit-exact."""
import numpy as np
import oracle_lib
import pytest

from gpu_util import describe_diff, stream_ptr, to_device

pytestmark = pytest.mark.gpu


def mixed_grid(X, Y, Z, seed):
    rng = np.random.default_rng(seed)
    g = rng.choice(np.array([0, 0, 0, 0, 1, 2, 2, 3, 3, 7], np.uint8), size=(Y, Z, X))
    g[Y // 3:2 * Y // 3] = np.where(g[Y // 3:2 * Y // 3] == 1, 0, g[Y // 3:2 * Y // 3])
    g[: Y // 4] = np.where(g[: Y // 4] == 0, 2, g[: Y // 4])  # a settled bottom region (no empty cells)
    return g


# (X, Y, Z): plane words per row 16, 17 (groups of 32 lanes), 3, 2, 8, 16 (partial last word), 32, 1
DIMS = [(1024, 64, 256), (1088, 63, 200), (130, 300, 260), (100, 600, 333), (512, 257, 97), (1000, 33, 300),
        (2048, 64, 96), (64, 700, 700)]


def check_every_step(fs3d, orc, g, seed, t0, n, layout=1):
    Y, Z, X = g.shape
    exp = orc.run(g.copy(), seed, t0, n, nthreads=0, hashes=True)
    with fs3d.World(g, seed, t0, layout) as w:
        for t in range(n):
            w.step(1)
            if w.hash() != int(exp[t]):
                ref = g.copy()
                orc.run(ref, seed, t0, t + 1, nthreads=0)
                pytest.fail(describe_diff(w.read(), ref, t0 + t))
        w.sync()
        return w.read()


@pytest.mark.parametrize("dims", DIMS)
def test_large_world_every_step(fs3d, orc, dims):
    X, Y, Z = dims
    seed = X * 131 + Y * 7 + Z
    g = mixed_grid(X, Y, Z, seed)
    check_every_step(fs3d, orc, g, seed, 3, 40)


def test_settled_dunes_every_step(fs3d, orc):
    """256^3 dunes (rows of 4 words): the sand settles and the rain lands, so
    ever more row-pairs are skipped; every step still equals the oracle."""
    g = orc.gen_c5(4, 256, 256, 256)
    assert (g == fs3d.gen_dunes(4, 256, 256, 256)).all()
    check_every_step(fs3d, orc, g, 4, 0, 300)


def test_steps_in_several_calls_and_after_write(fs3d, orc):
    """The row change flags carry over between step calls (the same results as
    one call), and a rewrite of the world's contents starts them afresh."""
    X, Y, Z = 512, 200, 160
    g = mixed_grid(X, Y, Z, 5)
    ref = g.copy()
    orc.run(ref, 5, 0, 37, nthreads=0)
    with fs3d.World(g, 5, 0, fs3d.LAYOUT_PLANES) as w:
        for n in (1, 2, 13, 21):
            w.step(n)
        got = w.read()
        assert (got == ref).all(), describe_diff(got, ref, 36)
        g2 = mixed_grid(X, Y, Z, 6)
        w.write(g2)
        w.step(9)
        ref2 = g2.copy()
        orc.run(ref2, 5, 37, 9, nthreads=0)
        got = w.read()
        assert (got == ref2).all(), describe_diff(got, ref2, 45)


@pytest.mark.parametrize("entry", ["fs3d_run_device", "fs3d_run_device_noalloc"])
def test_drop_in_runs_of_large_worlds(fs3d, orc, cuda, entry):
    """The drop-in runs take the per-step kernel for worlds too large for
    shared memory: two runs in a row equal the oracle."""
    X, Y, Z = 1024, 96, 200
    seed = 77
    g = mixed_grid(X, Y, Z, seed)
    d = to_device(cuda, g)
    st = stream_ptr(cuda)
    fn = getattr(fs3d.lib(), entry)
    assert fn(d.data_ptr(), X, Y, Z, seed, 11, 17, st) == 0
    assert fn(d.data_ptr(), X, Y, Z, seed, 28, 6, st) == 0
    fs3d.run_device_check(st)
    ref = g.copy()
    orc.run(ref, seed, 11, 23, nthreads=0)
    got = d.cpu().numpy()
    assert (got == ref).all(), describe_diff(got, ref, 33)


def test_render_counts_stay_exact(fs3d, orc):
    """A rendered world keeps its per-brick counts through the per-step kernel:
    frames after stepping equal the CPU DDA of the oracle's grid."""
    X, Y, Z = 512, 160, 192
    g = mixed_grid(X, Y, Z, 9)
    cam = fs3d.camera_world_view(X, Y, Z, 160, 90)
    ref = g.copy()
    with fs3d.World(g, 9, 0, fs3d.LAYOUT_PLANES) as w:
        for s in range(12):
            w.step(1)
            orc.step(ref, 9, s)
            img = w.render(cam, 160, 90)
        exp = orc.render_dda(ref, oracle_lib.camera_from(cam), 160, 90)
        assert float(np.abs(img - exp).max()) <= 1e-5
