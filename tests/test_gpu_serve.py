"""GPU checks of the serving loop: continuous batching keeps every result
identical to the world run alone (and to the oracle), also when the memory
budget forces arrivals to wait."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


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
    rng = np.random.default_rng(0)
    for i in rng.choice(len(reqs), 6, replace=False):
        r = reqs[int(i)]
        assert r.arrival_s <= r.admitted_s <= r.finished_s
        assert r.hash == alone_hash(fs3d, r)
        g = orc.gen_c3_world(r.seed, r.X, r.Y, r.Z)
        orc.run(g, r.seed, 0, r.n_steps, nthreads=0)
        assert r.hash == orc.hash(g)


def test_tight_budget_defers_but_stays_exact(fs3d):
    budget = 600 << 10  # room for one of the largest worlds (512 KiB of planes) at a time
    p = fs3d.serve_params(4000.0, 0.1, master_seed=5, min_steps=50, max_steps=300, hbm_budget=budget)
    stats, reqs = fs3d.serve(p)
    assert stats["completed"] == len(reqs)
    assert stats["peak_bytes"] <= budget
    waited = [r for r in reqs if r.admitted_s - r.arrival_s > 2e-3]
    assert waited, "the budget should have made some arrivals wait"
    for r in waited[:4]:
        assert r.hash == alone_hash(fs3d, r)
