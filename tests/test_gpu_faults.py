"""Failure detection without a GPU fault.

Device side: the resident step kernels wait for their bulk copies with an
iteration limit.  The test hook makes every such wait run out in a form that
cannot fault: the kernel announces 16 bytes more on its mbarrier than the
copy delivers, so the copy lands in full and only the barrier's phase never
completes.  The kernel then records the failure, steps nothing, and the host
reports FS3D_ERR_TIMEOUT; the next normal call is bit-exact.

Host side: an admission whose device allocation is refused returns
FS3D_ERR_OOM, admits nothing and leaves the batch usable."""
import numpy as np
import pytest

from gpu_util import describe_diff, stream_ptr, to_device

pytestmark = pytest.mark.gpu

GiB = 1 << 30


@pytest.fixture
def stall(fs3d):
    """The copy-stall injection, switched off again whatever the test does."""
    fs3d.inject(fs3d.INJECT_COPY_STALL, 1)
    try:
        yield
    finally:
        fs3d.inject(fs3d.INJECT_NONE, 0)


def test_world_resident_copy_timeout_rewinds_and_recovers(fs3d, orc):
    seed = 41
    g = orc.gen_c1(seed)  # 64^3: one CTA holds it in shared memory (bulk copies)
    with fs3d.World(g, seed, 0, fs3d.LAYOUT_PLANES) as w:
        w.step(10)
        w.sync()
        h10 = w.hash()
        fs3d.inject(fs3d.INJECT_COPY_STALL, 1)
        try:
            w.step(5)  # its copy never completes: records the failure, steps nothing
            w.step(7)  # launched after the failure: steps nothing either
            with pytest.raises(fs3d.Fs3dError) as e:
                w.sync()
            assert e.value.status == fs3d.ERR_TIMEOUT
        finally:
            fs3d.inject(fs3d.INJECT_NONE, 0)
        # set back to the step its state holds, state unchanged
        assert w.step_counter == 10
        assert w.hash() == h10
        w.sync()  # the record was cleared
        w.step(20)
        w.sync()
        ref = g.copy()
        orc.run(ref, seed, 0, 30, nthreads=0)
        got = w.read()
        assert (got == ref).all(), describe_diff(got, ref, 29)


@pytest.mark.parametrize("entry", ["fs3d_run_device", "fs3d_run_device_noalloc"])
def test_drop_in_run_copy_timeout_reported_by_check(fs3d, orc, cuda, entry):
    X = Y = Z = 64
    seed = 43
    g = orc.gen_c1(seed)
    d = to_device(cuda, g)
    st = stream_ptr(cuda)
    fn = getattr(fs3d.lib(), entry)
    fs3d.run_device_check(st)  # nothing recorded before
    fs3d.inject(fs3d.INJECT_COPY_STALL, 1)
    try:
        assert fn(d.data_ptr(), X, Y, Z, seed, 0, 12, st) == 0
        with pytest.raises(fs3d.Fs3dError) as e:
            fs3d.run_device_check(st)
        assert e.value.status == fs3d.ERR_TIMEOUT
    finally:
        fs3d.inject(fs3d.INJECT_NONE, 0)
    cuda.cuda.synchronize()
    assert (d.cpu().numpy() == g).all()  # the run left the grid as it was
    fs3d.run_device_check(st)  # cleared
    assert fn(d.data_ptr(), X, Y, Z, seed, 0, 12, st) == 0
    fs3d.run_device_check(st)
    ref = g.copy()
    orc.run(ref, seed, 0, 12, nthreads=0)
    got = d.cpu().numpy()
    assert (got == ref).all(), describe_diff(got, ref, 11)


def test_batch_resident_copy_timeout_is_reported(fs3d, orc, stall):
    dims, seeds = fs3d.gen_batch_dims(9, 4)
    with fs3d.Batch(GiB, steps_per_segment=16, use_smem=1) as b:
        for (X, Y, Z), s in zip(dims, seeds):
            b.admit(fs3d.gen_batch_world(int(s), int(X), int(Y), int(Z)), int(s), 16)
        b.run_segment()
        with pytest.raises(fs3d.Fs3dError) as e:
            b.sync()
        assert e.value.status == fs3d.ERR_TIMEOUT


def test_admission_allocation_refused_is_oom_and_batch_stays_usable(fs3d, orc):
    dims, seeds = fs3d.gen_batch_dims(17, 6)
    worlds = [((int(X), int(Y), int(Z)), int(s)) for (X, Y, Z), s in zip(np.minimum(dims, 64), seeds)]
    grids = [fs3d.gen_batch_world(s, *d) for d, s in worlds]
    n = 40
    with fs3d.Batch(GiB, steps_per_segment=32) as b:
        t0 = b.admit(grids[0], worlds[0][1], n)
        before = b.stats()
        fs3d.inject(fs3d.INJECT_ALLOC_FAIL, 1)
        try:
            with pytest.raises(fs3d.Fs3dError) as e:
                b.admit(grids[1], worlds[1][1], n)
            assert e.value.status == fs3d.ERR_OOM
            assert b.stats() == before
            fs3d.inject(fs3d.INJECT_ALLOC_FAIL, 1)
            with pytest.raises(fs3d.Fs3dError) as e:
                b.admit_many(grids[1:], [s for _, s in worlds[1:]], n)
            assert e.value.status == fs3d.ERR_OOM
            assert b.stats() == before
        finally:
            fs3d.inject(fs3d.INJECT_NONE, 0)
        ts = [t0] + b.admit_many(grids[1:], [s for _, s in worlds[1:]], n)
        for _ in range(2):
            b.run_segment()
        b.sync()
        for t, (d, s), g in zip(ts, worlds, grids):
            X, Y, Z = d
            ref = g.copy()
            orc.run(ref, s, 0, n, nthreads=0)
            assert (b.retire(t, (Y, Z, X)) == ref).all(), d
