"""CPU checks of the oracle: known-answer blocks for every rule clause, an
independent Python statement of the rule, invariants, order independence and
the self-recorded golden vectors (parity with the upstream project is
unpinned: it contains no step to compare against)."""
import json
import os

import numpy as np
import pytest

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
