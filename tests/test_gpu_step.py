"""GPU parity of the single-world paths against the CPU oracle: the drop-in
byte kernels (vectorised and one-thread-per-block) and the world object in
both layouts, compared by whole-grid hash after every step, with the first
differing voxel reported on failure.  Integer work: bit-exact."""
import numpy as np
import pytest

from gpu_util import describe_diff, stream_ptr, to_device

pytestmark = pytest.mark.gpu

SEEDS = list(range(1, 33))


@pytest.mark.parametrize("seed", SEEDS)
def test_parity_64_drop_in_every_step(fs3d, orc, cuda, seed):
    g = orc.gen_c1(seed)
    exp_hashes = orc.run(g.copy(), seed, 0, 200, nthreads=0, hashes=True)
    d = to_device(cuda, g)
    st = stream_ptr(cuda)
    for t in range(200):
        fs3d.step_device(d.data_ptr(), 64, 64, 64, seed, t, 1, st)
        h = fs3d.hash_device(d.data_ptr(), d.numel(), st)
        if h != int(exp_hashes[t]):
            ref = g.copy()
            orc.run(ref, seed, 0, t + 1, nthreads=0)
            pytest.fail(describe_diff(d.cpu().numpy(), ref, t))


@pytest.mark.parametrize("layout", [0, 1])
@pytest.mark.parametrize("seed", SEEDS[:8])
def test_parity_64_world_every_step(fs3d, orc, seed, layout):
    g = orc.gen_c1(seed)
    exp_hashes = orc.run(g.copy(), seed, 0, 200, nthreads=0, hashes=True)
    with fs3d.World(g, seed, 0, layout) as w:
        for t in range(200):
            w.step(1)
            if w.hash() != int(exp_hashes[t]):
                ref = g.copy()
                orc.run(ref, seed, 0, t + 1, nthreads=0)
                pytest.fail(describe_diff(w.read(), ref, t))
        assert w.step_counter == 200


DIMS = [(24, 40, 33), (96, 20, 70), (128, 30, 17), (1, 5, 7), (17, 9, 64), (130, 12, 10), (192, 8, 8),
        (64, 3, 2), (2, 64, 3), (48, 1, 48), (1024, 6, 6), (2048, 4, 3), (16, 128, 16), (80, 33, 7)]


def mixed_grid(X, Y, Z, seed):
    rng = np.random.default_rng(seed)
    g = rng.choice(np.array([0, 0, 0, 0, 1, 2, 2, 3, 3, 7], np.uint8), size=(Y, Z, X))
    g[Y // 3:2 * Y // 3] = np.where(g[Y // 3:2 * Y // 3] == 1, 0, g[Y // 3:2 * Y // 3])
    return g


@pytest.mark.parametrize("dims", DIMS)
def test_parity_odd_dims_all_paths(fs3d, orc, cuda, dims):
    X, Y, Z = dims
    seed = X * 7919 + Y * 31 + Z
    g = mixed_grid(X, Y, Z, seed)
    n = 24
    ref = g.copy()
    exp = orc.run(ref, seed, 5, n, nthreads=0, hashes=True)
    st = stream_ptr(cuda)
    fast, simple = to_device(cuda, g), to_device(cuda, g)
    worlds = [fs3d.World(g, seed, 5, layout) for layout in ((0, 1) if X <= 2048 else (0,))]
    for t in range(n):
        fs3d.step_device(fast.data_ptr(), X, Y, Z, seed, 5 + t, 1, st)
        fs3d.step_device_simple(simple.data_ptr(), X, Y, Z, seed, 5 + t, 1, st)
        for w in worlds:
            w.step(1)
        got = {"fast": fs3d.hash_device(fast.data_ptr(), fast.numel(), st),
               "simple": fs3d.hash_device(simple.data_ptr(), simple.numel(), st)}
        for w in worlds:
            got["world%d" % w.layout] = w.hash()
        bad = {k: v for k, v in got.items() if v != int(exp[t])}
        if bad:
            r = g.copy()
            orc.run(r, seed, 5, t + 1, nthreads=0)
            name = sorted(bad)[0]
            arr = (fast.cpu().numpy() if name == "fast" else simple.cpu().numpy() if name == "simple"
                   else worlds[int(name[-1])].read())
            pytest.fail(f"{sorted(bad)} differ; {name}: " + describe_diff(arr, r, t))
    assert (fast.cpu().numpy() == ref).all()
    for w in worlds:
        assert (w.read() == ref).all()
        w.close()


def test_hash_and_first_diff_device(fs3d, orc, cuda):
    rng = np.random.default_rng(5)
    for n in (1, 15, 16, 17, 1000, 4097, 1 << 20):
        a = rng.integers(0, 256, n, dtype=np.uint8)
        da = to_device(cuda, a)
        assert fs3d.hash_device(da.data_ptr(), n) == orc.hash(a)
        b = a.copy()
        assert fs3d.first_diff_device(da.data_ptr(), to_device(cuda, b).data_ptr(), n) == -1
        k = n // 2
        b[k] ^= 1
        b[-1] ^= 2
        assert fs3d.first_diff_device(da.data_ptr(), to_device(cuda, b).data_ptr(), n) == k
    # unaligned base pointer
    big = to_device(cuda, rng.integers(0, 4, 4099, dtype=np.uint8))
    assert fs3d.hash_device(big.data_ptr() + 3, 4096) == orc.hash(big.cpu().numpy()[3:4099])


def test_checkpoint_resume_is_exact(fs3d, orc, tmp_path):
    g = orc.gen_c1(21)
    path = str(tmp_path / "w.fs3d")
    with fs3d.World(g, 21, 0, fs3d.LAYOUT_PLANES) as a:
        a.step(50)
        a.save(path)
        a.step(70)
        ha = a.hash()
    with fs3d.World.load(path, fs3d.LAYOUT_BYTES) as b:
        assert b.step_counter == 50 and b.seed == 21
        b.step(70)
        assert b.hash() == ha
    ref = g.copy()
    orc.run(ref, 21, 0, 120, nthreads=0)
    assert orc.hash(ref) == ha


def test_bounded_sync_and_launch_count(fs3d, orc):
    g = orc.gen_c1(3)
    with fs3d.World(g, 3, 0, fs3d.LAYOUT_BYTES) as w:
        before = fs3d.kernel_launches()
        w.step(300)
        try:
            w.sync(0)  # may still be running: a timeout is a clean status, not a hang
        except fs3d.Fs3dError as e:
            assert e.status == fs3d.ERR_TIMEOUT
        w.sync(-1)
        w.sync(0)
        assert fs3d.kernel_launches() - before == 300


@pytest.mark.parametrize("dims", [(64, 64, 64), (24, 40, 33), (128, 256, 128), (512, 64, 96), (3000, 5, 4)])
def test_run_device_matches_oracle(fs3d, orc, cuda, dims):
    X, Y, Z = dims
    seed = X + Y + Z
    g = mixed_grid(X, Y, Z, seed)
    ref = g.copy()
    orc.run(ref, seed, 9, 33, nthreads=0)
    d = to_device(cuda, g)
    st = stream_ptr(cuda)
    fs3d.run_device(d.data_ptr(), X, Y, Z, seed, 9, 20, st)
    fs3d.run_device(d.data_ptr(), X, Y, Z, seed, 29, 13, st)
    cuda.cuda.synchronize()
    out = d.cpu().numpy()
    assert (out == ref).all(), describe_diff(out, ref, 32)


def test_step_device_many_native_launch_loop(fs3d, orc, cuda):
    """One launch per world per step from native code: each world equals the
    oracle."""
    dims = [(24, 40, 33), (64, 64, 64), (128, 30, 17), (48, 16, 96)]
    grids = [mixed_grid(X, Y, Z, 100 + i) for i, (X, Y, Z) in enumerate(dims)]
    devs = [to_device(cuda, g) for g in grids]
    seeds = [7 + i for i in range(len(dims))]
    fs3d.step_device_many([d.data_ptr() for d in devs], dims, seeds, 4, 15, stream_ptr(cuda))
    cuda.cuda.synchronize()
    for g, d, s in zip(grids, devs, seeds):
        ref = g.copy()
        orc.run(ref, s, 4, 15, nthreads=0)
        got = d.cpu().numpy()
        assert (got == ref).all(), describe_diff(got, ref, 18)
