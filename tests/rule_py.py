"""Pure-Python statement of FS3D-rule v1, written from the rule text (not from
the C oracle), used to cross-check the oracle on small grids."""
from __future__ import annotations

import numpy as np

M32 = 0xFFFFFFFF
M64 = 0xFFFFFFFFFFFFFFFF


def fmix32(h: int) -> int:
    h &= M32
    h ^= h >> 16
    h = (h * 0x85EBCA6B) & M32
    h ^= h >> 13
    h = (h * 0xC2B2AE35) & M32
    h ^= h >> 16
    return h


def fmix64(k: int) -> int:
    k &= M64
    k ^= k >> 33
    k = (k * 0xFF51AFD7ED558CCD) & M64
    k ^= k >> 33
    k = (k * 0xC4CEB9FE1A85EC53) & M64
    k ^= k >> 33
    return k


def stepkey(seed: int, t: int) -> int:
    h = fmix32(0x243F6A88 ^ (seed & M32))
    h = fmix32(h ^ ((seed >> 32) & M32))
    h = fmix32(h ^ (t & M32))
    return fmix32(h ^ ((t >> 32) & M32))


def rowkey(sk: int, j: int, k: int) -> int:
    h = fmix32(sk ^ ((0x85EBCA77 * (j + 1)) & M32))
    return fmix32(h ^ ((0xC2B2AE3D * (k + 1)) & M32))


def plane(rk: int, g: int, s: int, w: int) -> int:
    return fmix32((rk + 0x9E3779B9 * (1 + w + 8 * s + 64 * g)) & M32)


def draw(n: int, rk: int, i: int, s: int) -> int:
    if n <= 1:
        return 0
    g, b = i >> 5, i & 31
    if n == 2:
        return (plane(rk, g, s, 0) >> b) & 1
    u = sum(((plane(rk, g, s, w) >> b) & 1) << w for w in range(8))
    return 0 if u < 85 else (1 if u < 170 else 2)


def block(val, rk: int, i: int) -> list:
    """The rule on block i of its row-pair (row key rk): val[s] are the eight
    slot values (slots 0-3 the top layer, 4-7 the bottom one, column q = s & 3;
    a cell outside the grid holds 1).  Returns the new values."""
    val = [int(v) for v in val]
    empty = lambda s: val[s] == 0  # noqa: E731
    moved = set()
    for s in range(8):
        m = val[s]
        if m not in (2, 3) or s in moved:
            continue
        q = s & 3
        dst = None
        if s < 4:
            if empty(4 + q):
                dst = 4 + q
            else:
                cand = [4 + q2 for q2 in range(4) if q2 != q and empty(4 + q2)]
                if cand:
                    dst = cand[draw(len(cand), rk, i, s)]
        if dst is None and m == 3:
            base = s & 4
            cand = [base + q2 for q2 in range(4) if q2 != q and empty(base + q2)]
            if cand:
                dst = cand[draw(len(cand), rk, i, s)]
        if dst is not None:
            val[dst], val[s] = m, 0
            moved.add(dst)
    return val


def step(grid: np.ndarray, seed: int, t: int) -> None:
    """One step in place; grid shape (Y, Z, X)."""
    Y, Z, X = grid.shape
    o = t & 1
    sk = stepkey(seed, t)
    nb = lambda n: (n + o + 1) // 2  # noqa: E731
    for j in range(nb(Y)):
        for k in range(nb(Z)):
            rk = rowkey(sk, j, k)
            for i in range(nb(X)):
                cells = []
                for s in range(8):
                    layer, q = s >> 2, s & 3
                    x, y, z = 2 * i - o + (q & 1), 2 * j - o + (1 - layer), 2 * k - o + (q >> 1)
                    inside = 0 <= x < X and 0 <= y < Y and 0 <= z < Z
                    cells.append((y, z, x) if inside else None)
                val = block([int(grid[c]) if c else 1 for c in cells], rk, i)
                for s in range(8):
                    if cells[s]:
                        grid[cells[s]] = val[s]


def grid_hash(grid: np.ndarray) -> int:
    flat = grid.reshape(-1)
    return sum(fmix64(i * 256 + int(v)) for i, v in enumerate(flat)) & M64
