"""GPU checks of the serving loop: continuous batching keeps every result
identical to the world run alone and to the oracle (every served request is
checked), also when the memory budget forces arrivals to wait."""
import concurrent.futures as cf
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def oracle_hashes(orc, reqs):
    """The oracle's final hash of every request, worlds run in parallel on the
    host cores (one thread each)."""
    def one(r):
        g = orc.gen_c3_world(r.seed, r.X, r.Y, r.Z)
        orc.L.orc_run(g.ctypes.data, r.X, r.Y, r.Z, r.seed, 0, r.n_steps, None, 1)
        return orc.hash(g)
    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        return list(ex.map(one, reqs))


def alone_hash(fs3d, r):
    with fs3d.Batch(1 << 30, steps_per_segment=64) as b:
        t = b.admit_generated(r.X, r.Y, r.Z, r.seed, r.n_steps)
        for _ in range((r.n_steps + 63) // 64):
            b.run_segment()
        b.sync()
        return b.poll(t)[1]


def test_served_results_equal_alone_and_oracle(fs3d, orc):
    p = fs3d.serve_params(2000.0, 0.5, master_seed=3, min_steps=10, max_steps=150)
    stats, reqs = fs3d.serve(p)
    assert stats["completed"] == stats["requests"] == len(reqs) > 500
    assert stats["p50_ms"] <= stats["p99_ms"] <= stats["max_ms"]
    assert stats["peak_live_worlds"] > 1  # work overlapped on the device
    for r in reqs:
        assert r.arrival_s <= r.admitted_s <= r.finished_s
    exp = oracle_hashes(orc, reqs)
    bad = [i for i, (r, h) in enumerate(zip(reqs, exp)) if r.hash != h]
    assert not bad, f"{len(bad)} of {len(reqs)} served requests differ from the oracle, first {bad[0]}"
    rng = np.random.default_rng(0)
    for i in rng.choice(len(reqs), 6, replace=False):
        assert reqs[int(i)].hash == alone_hash(fs3d, reqs[int(i)])


def test_tight_budget_defers_but_stays_exact(fs3d, orc):
    budget = 600 << 10  # room for one of the largest worlds (512 KiB of planes) at a time
    p = fs3d.serve_params(4000.0, 0.1, master_seed=5, min_steps=50, max_steps=300, hbm_budget=budget)
    stats, reqs = fs3d.serve(p)
    assert stats["completed"] == len(reqs)
    assert stats["peak_bytes"] <= budget
    waited = [r for r in reqs if r.admitted_s - r.arrival_s > 2e-3]
    assert waited, "the budget should have made some arrivals wait"
    assert [r.hash for r in reqs] == oracle_hashes(orc, reqs)
    for r in waited[:4]:
        assert r.hash == alone_hash(fs3d, r)


def test_request_larger_than_the_whole_budget_is_an_error(fs3d):
    """A request that cannot fit even with nothing else live ends the run with
    FS3D_ERR_BUDGET instead of waiting for memory that never frees."""
    budget = 48 << 10  # a 16^3 or 48^3 world fits, a 64 x 64 cross-section does not
    p = fs3d.serve_params(2000.0, 0.05, master_seed=6, min_steps=10, max_steps=40, hbm_budget=budget)
    reqs, n = fs3d.serve_plan(p)
    planes = [r.Y * r.Z * ((r.X + 63) // 64) * 16 for r in reqs[:n]]
    assert max(planes) > budget and min(planes) < budget
    with pytest.raises(fs3d.Fs3dError) as e:
        fs3d.serve(p)
    assert e.value.status == fs3d.ERR_BUDGET
    stats, done = fs3d.serve(fs3d.serve_params(2000.0, 0.05, master_seed=6, min_steps=10, max_steps=40))
    assert stats["completed"] == len(done) == n


def test_serving_reports_a_device_wait_that_gave_up(fs3d):
    """Young requests run in the shared-memory step kernels; with every bulk
    copy wait made to run out (test hook), the first segment's wait reports
    FS3D_ERR_TIMEOUT and the run ends with it instead of serving wrong results."""
    p = fs3d.serve_params(2000.0, 0.05, master_seed=8, min_steps=10, max_steps=40, segment_timeout_ms=5000)
    fs3d.inject(fs3d.INJECT_COPY_STALL, 1)
    try:
        with pytest.raises(fs3d.Fs3dError) as e:
            fs3d.serve(p)
        assert e.value.status == fs3d.ERR_TIMEOUT
    finally:
        fs3d.inject(fs3d.INJECT_NONE, 0)
    stats, reqs = fs3d.serve(p)  # and serving works again
    assert stats["completed"] == len(reqs) > 0
