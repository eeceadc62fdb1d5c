"""CPU checks of the serving request stream (no GPU work)."""
import numpy as np


def test_plan_is_seeded_poisson(fs3d):
    p = fs3d.serve_params(2000.0, 2.0, master_seed=7)
    reqs, n = fs3d.serve_plan(p)
    reqs2, n2 = fs3d.serve_plan(p)
    assert n == n2 and all(a.seed == b.seed and a.arrival_s == b.arrival_s for a, b in zip(reqs, reqs2))
    arr = np.array([r.arrival_s for r in reqs[:n]])
    assert (np.diff(arr) > 0).all() and arr[-1] <= 2.0
    assert abs(n / 2.0 - 2000) < 5 * np.sqrt(2000 * 2.0) / 2.0
    steps = np.array([r.n_steps for r in reqs[:n]])
    assert steps.min() >= 10 and steps.max() <= 1000
    # log-uniform: the median of exp(U[ln 10, ln 1000]) is 100
    assert 80 < np.median(steps) < 125
    dims = {r.X for r in reqs[:n]} | {r.Y for r in reqs[:n]} | {r.Z for r in reqs[:n]}
    assert dims == {16, 24, 32, 48, 64, 96, 128}
    assert len({r.seed for r in reqs[:n]}) == n


def test_plan_caps(fs3d):
    p = fs3d.serve_params(8000.0, 10.0, master_seed=1, max_requests=123, min_steps=5, max_steps=7)
    reqs, n = fs3d.serve_plan(p)
    assert n == 123 and {r.n_steps for r in reqs[:n]} <= {5, 6, 7}
