"""Worlds that arrive with no change history (admitted, created, written or
run at some step t0) get their change flags from their cells: a layer (batch)
or row (per-step kernel) is marked changed at t0 - 1 only when a block
row-pair of either phase that covers it can change, so the first two steps
evaluate only those row-pairs instead of every one.  Exactness is checked
against the CPU oracle on mostly settled worlds, at even and odd start steps
and at start steps whose low 8 bits wrap (t0 - 3 mod 256); the batch also
shows that the first segment evaluates fewer cell-steps than two dense steps.
Integer work: bit-exact."""
import numpy as np
import pytest

from gpu_util import describe_diff, stream_ptr, to_device

pytestmark = pytest.mark.gpu

GiB = 1 << 30
STARTS = [130, 255, 256, 257, 1025]


def settled(orc, X, Y, Z, seed, steps=150):
    """Random sand, water, solids and statics, fallen for `steps` steps on the
    CPU: the bottom is packed and only the surface still moves."""
    rng = np.random.default_rng(seed)
    g = rng.choice(np.array([0, 0, 0, 1, 2, 2, 3, 3, 7], np.uint8), size=(Y, Z, X))
    g[: Y // 3] = np.where(g[: Y // 3] == 0, 2, g[: Y // 3])
    orc.run(g, seed, 0, steps, nthreads=0)
    return g


@pytest.mark.parametrize("use_smem", [1, 2, 3])
def test_batch_admission_flags_exact_and_sparse(fs3d, orc, use_smem):
    dims, seeds = fs3d.gen_batch_dims(23, 10)
    dims = [(int(X), int(Y), int(Z)) for X, Y, Z in dims]
    dims[0] = (128, 40, 24)  # rows of two full words: the odd phase's half block at the row end
    dims[1] = (64, 33, 31)
    grids = [settled(orc, X, Y, Z, int(s)) for (X, Y, Z), s in zip(dims, seeds)]
    starts = [STARTS[i % len(STARTS)] for i in range(len(dims))]
    S, n = 2, 12
    cells = sum(X * Y * Z for X, Y, Z in dims)
    with fs3d.Batch(GiB, steps_per_segment=S, use_smem=use_smem) as b:
        ts = b.admit_many(grids, [int(s) for s in seeds], n, start_steps=starts)
        b.run_segment()
        b.sync()
        first = b.counters()["processed_cell_steps"]
        # without flags from the cells these first two steps evaluate every cell twice
        assert first < 2 * cells, (first, cells)
        for _ in range(n // S - 1):
            b.run_segment()
        b.sync()
        for t, (X, Y, Z), s, t0, g in zip(ts, dims, seeds, starts, grids):
            ref = g.copy()
            orc.run(ref, int(s), t0, n, nthreads=0)
            got = b.retire(t, (Y, Z, X))
            assert (got == ref).all(), ((X, Y, Z), t0, describe_diff(got, ref, t0 + n - 1))


def test_batch_single_admissions(fs3d, orc):
    dims = [(96, 48, 40), (130, 37, 20), (64, 64, 64)]
    with fs3d.Batch(GiB, steps_per_segment=8) as b:
        items = []
        for i, (X, Y, Z) in enumerate(dims):
            seed, t0 = 300 + i, STARTS[i + 1]
            g = settled(orc, X, Y, Z, seed)
            items.append((b.admit(g, seed, 24, start_step=t0), g, (X, Y, Z), seed, t0))
        for _ in range(3):
            b.run_segment()
        b.sync()
        for t, g, (X, Y, Z), seed, t0 in items:
            ref = g.copy()
            orc.run(ref, seed, t0, 24, nthreads=0)
            got = b.retire(t, (Y, Z, X))
            assert (got == ref).all(), describe_diff(got, ref, t0 + 23)


@pytest.mark.parametrize("t0", [256, 257])
def test_world_created_settled_every_step(fs3d, orc, t0):
    """The per-step kernel of a large world (rows of 8 words): created from a
    settled grid at t0, every step's hash equals the oracle's."""
    X, Y, Z = 512, 72, 300
    g = settled(orc, X, Y, Z, 31, steps=120)
    n = 12
    exp = orc.run(g.copy(), 31, t0, n, nthreads=0, hashes=True)
    with fs3d.World(g, 31, t0, fs3d.LAYOUT_PLANES) as w:
        for s in range(n):
            w.step(1)
            if w.hash() != int(exp[s]):
                ref = g.copy()
                orc.run(ref, 31, t0, s + 1, nthreads=0)
                pytest.fail(describe_diff(w.read(), ref, t0 + s))
        # a rewrite starts the flags afresh from the new cells
        g2 = settled(orc, X, Y, Z, 32, steps=90)
        w.write(g2)
        w.step(5)
        ref2 = g2.copy()
        orc.run(ref2, 31, t0 + n, 5, nthreads=0)
        got = w.read()
        assert (got == ref2).all(), describe_diff(got, ref2, t0 + n + 4)


@pytest.mark.parametrize("dims", [(1024, 48, 160), (64, 48, 40), (96, 40, 64)])
@pytest.mark.parametrize("entry", ["fs3d_run_device", "fs3d_run_device_noalloc"])
def test_drop_in_run_of_settled_world(fs3d, orc, cuda, entry, dims):
    """Settled worlds through both drop-in entries at start steps across the
    8-bit wrap: the per-step kernel (1024 x 48 x 160, too large for shared
    memory, and every call of fewer than four steps: row flags) and the
    resident launch (the smaller worlds' longer calls: layer flags)."""
    X, Y, Z = dims
    seed = 57
    g = settled(orc, X, Y, Z, seed, steps=100)
    d = to_device(cuda, g)
    st = stream_ptr(cuda)
    fn = getattr(fs3d.lib(), entry)
    t = 255
    for n in (9, 4, 2, 1):
        assert fn(d.data_ptr(), X, Y, Z, seed, t, n, st) == 0
        t += n
    fs3d.run_device_check(st)
    ref = g.copy()
    orc.run(ref, seed, 255, t - 255, nthreads=0)
    got = d.cpu().numpy()
    assert (got == ref).all(), describe_diff(got, ref, t - 1)


@pytest.mark.parametrize("dims", [(2048, 1, 700), (2048, 700, 1), (1000, 3, 333), (1, 900, 900), (4, 2, 4)])
def test_thin_and_tiny_worlds(fs3d, orc, dims):
    """Single-layer, single-row and one-cell-wide worlds: the pairs at the
    world's edges (a layer or row of the pair outside it) are handled as solid
    by the flags from the cells too.  Created at an odd step, stepped once per
    call, every hash against the oracle."""
    X, Y, Z = dims
    seed = X + 3 * Y + 7 * Z
    rng = np.random.default_rng(seed)
    g = rng.choice(np.array([0, 0, 1, 2, 2, 3, 3, 7], np.uint8), size=(Y, Z, X))
    orc.run(g, seed, 0, 6, nthreads=0)
    t0, n = 513, 8
    exp = orc.run(g.copy(), seed, t0, n, nthreads=0, hashes=True)
    with fs3d.World(g, seed, t0, fs3d.LAYOUT_PLANES) as w:
        for s in range(n):
            w.step(1)
            if w.hash() != int(exp[s]):
                ref = g.copy()
                orc.run(ref, seed, t0, s + 1, nthreads=0)
                pytest.fail(describe_diff(w.read(), ref, t0 + s))
    with fs3d.Batch(GiB, steps_per_segment=3, use_smem=3) as b:
        t = b.admit(g, seed, n, start_step=t0)
        for _ in range(3):
            b.run_segment()
        b.sync()
        ref = g.copy()
        orc.run(ref, seed, t0, n, nthreads=0)
        got = b.retire(t, (Y, Z, X))
        assert (got == ref).all(), describe_diff(got, ref, t0 + n - 1)


@pytest.mark.parametrize("dims", [(64, 48, 40), (96, 96, 96), (130, 70, 90)])
def test_world_calls_of_few_and_many_steps(fs3d, orc, dims):
    """A world that fits the resident kernels, stepped in calls of one to
    eight steps, as an engine's frame loop would: short calls take the
    per-step kernel (row flags), longer ones a resident launch (layer flags)
    when the world is small; each kind of flags carries from call to call or
    is set again from the cells, and every call's hash equals the oracle's,
    across the 8-bit wrap of the flags."""
    X, Y, Z = dims
    seed = 900 + X
    g = settled(orc, X, Y, Z, seed, steps=80)
    t0 = 250
    calls = [1, 1, 5, 1, 8, 2, 4, 1, 1, 6, 3, 4]
    n = sum(calls)
    exp = orc.run(g.copy(), seed, t0, n, nthreads=0, hashes=True)
    with fs3d.World(g, seed, t0, fs3d.LAYOUT_PLANES) as w:
        done = 0
        for c in calls:
            w.step(c)
            done += c
            if w.hash() != int(exp[done - 1]):
                ref = g.copy()
                orc.run(ref, seed, t0, done, nthreads=0)
                pytest.fail(describe_diff(w.read(), ref, t0 + done - 1))
        g2 = settled(orc, X, Y, Z, seed + 1, steps=60)
        w.write(g2)
        for _ in range(5):
            w.step(1)
        w.step(3)
        ref2 = g2.copy()
        orc.run(ref2, seed, t0 + n, 8, nthreads=0)
        got = w.read()
        assert (got == ref2).all(), describe_diff(got, ref2, t0 + n + 7)
        w.step(16)  # a resident launch (small worlds) after the rewrite's per-step calls
        orc.run(ref2, seed, t0 + n + 8, 16, nthreads=0)
        got = w.read()
        assert (got == ref2).all(), describe_diff(got, ref2, t0 + n + 23)
