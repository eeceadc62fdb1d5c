"""Parity at the workloads' full sizes against the CPU oracle (slow: the
oracle runs the same steps on the host cores).

* 512^3 pillars, 1000 steps: the drop-in byte kernel's whole-grid hash every
  10 steps and the final grid; the same world in the plane layout (per-step
  kernel with the exact skip of settled row-pairs) by hash after the 1000 steps.
* 1024^3 dunes, 500 steps: the plane-layout world (the same kernel) by hash
  after every one of the first 50 steps, and the whole final grid after step 500.

On a mismatch the first differing voxel is reported.  Integer work: bit-exact."""
import numpy as np
import pytest

from gpu_util import describe_diff, stream_ptr, to_device

pytestmark = [pytest.mark.gpu, pytest.mark.slow]


def test_pillars_512_1000_steps(fs3d, orc, cuda):
    X = Y = Z = 512
    seed, every, n = 1, 10, 1000
    g = fs3d.gen_pillars(seed, X, Y, Z)
    assert (g == orc.gen_c2(seed, X, Y, Z)).all()
    st = stream_ptr(cuda)
    d = to_device(cuda, g)
    got = []
    for c in range(n // every):
        fs3d.step_device(d.data_ptr(), X, Y, Z, seed, every * c, every, st)
        got.append(fs3d.hash_device(d.data_ptr(), d.numel(), st))
    final = d.cpu().numpy()
    del d
    with fs3d.World(g, seed, 0, fs3d.LAYOUT_PLANES) as w:
        w.step(n)
        planes_hash = w.hash()
    ref = g.copy()
    for c in range(n // every):
        orc.run(ref, seed, every * c, every, nthreads=0)
        if orc.hash(ref) != got[c]:
            again = to_device(cuda, g)
            fs3d.step_device(again.data_ptr(), X, Y, Z, seed, 0, every * (c + 1), st)
            pytest.fail("byte kernel: " + describe_diff(again.cpu().numpy(), ref, every * (c + 1) - 1))
    assert (final == ref).all(), describe_diff(final, ref, n - 1)
    assert planes_hash == orc.hash(ref), "plane layout (per-step kernel) differs after 1000 steps"


def test_dunes_1024_500_steps(fs3d, orc):
    N = 1024
    seed, first, n = 1, 50, 500
    g = fs3d.gen_dunes(seed, N, N, N)
    assert (g == orc.gen_c5(seed, N, N, N)).all()
    got = []
    with fs3d.World(g, seed, 0, fs3d.LAYOUT_PLANES) as w:
        for _ in range(first):
            w.step(1)
            got.append(w.hash())
        w.step(n - first)
        final = w.read()
    ref = g  # the world holds its own copy
    exp = orc.run(ref, seed, 0, first, nthreads=0, hashes=True)
    bad = [t for t in range(first) if int(exp[t]) != got[t]]
    if bad:
        t = bad[0]
        again = orc.gen_c5(seed, N, N, N)
        with fs3d.World(again, seed, 0, fs3d.LAYOUT_PLANES) as w:
            w.step(t + 1)
            mine = w.read()
        orc.run(again, seed, 0, t + 1, nthreads=0)
        pytest.fail(describe_diff(mine, again, t))
    orc.run(ref, seed, first, n - first, nthreads=0)
    assert (final == ref).all(), describe_diff(final, ref, n - 1)
