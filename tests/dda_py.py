"""An independent statement of the voxel DDA walk in Python, every float32
operation rounded as in the C oracle (numpy float32 scalars; the fused
multiply-add computed exactly and rounded once to nearest, ties to even).
Slow: for small images only.  Test infrastructure."""
from fractions import Fraction

import numpy as np

F = np.float32
PALETTE = [(0.0, 0.0, 0.0), (0.50, 0.50, 0.52), (0.86, 0.74, 0.46), (0.20, 0.42, 0.90), (0.65, 0.35, 0.30)]


def fma32(a, b, c) -> np.float32:
    """fmaf(a, b, c): the exact a*b + c rounded once to float32 (nearest, ties to even)."""
    exact = Fraction(float(a)) * Fraction(float(b)) + Fraction(float(c))
    f = F(float(exact))  # within one ulp of the answer (double rounding)
    best = None
    for cand in (np.nextafter(f, F(-np.inf)), f, np.nextafter(f, F(np.inf))):
        key = (abs(Fraction(float(cand)) - exact), int(np.array(cand, F).view(np.uint32)) & 1)
        if best is None or key < best[0]:
            best = (key, cand)
    return F(best[1])


def normalize3(v):
    ln = np.sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2])
    return [v[0] / ln, v[1] / ln, v[2] / ln]


def render(g: np.ndarray, cam, W: int, H: int) -> np.ndarray:
    """g[y, z, x] uint8; cam with origin, forward, right, up, tan_half_fov, aspect, light_pos."""
    Y, Z, X = g.shape
    N = [X, Y, Z]
    o = [F(cam.origin[a]) for a in range(3)]
    fw = [F(cam.forward[a]) for a in range(3)]
    rt = [F(cam.right[a]) for a in range(3)]
    up = [F(cam.up[a]) for a in range(3)]
    lp = [F(cam.light_pos[a]) for a in range(3)]
    th, asp = F(cam.tan_half_fov), F(cam.aspect)
    img = np.zeros((H, W, 4), F)
    img[..., 3] = 1
    for py in range(H):
        for px in range(W):
            u = F(1) - (F(px) + F(0.5)) / F(W)
            v = (F(py) + F(0.5)) / F(H)
            ux, uy = u * F(2) - F(1), v * F(2) - F(1)
            sx, sy = ux * th * asp, uy * th
            d = normalize3([fw[a] + rt[a] * sx + up[a] * sy for a in range(3)])
            inv = [F(np.inf)] * 3
            tmin, tmax, entry, miss = F(0), F(np.inf), -1, False
            for a in range(3):
                if d[a] == 0:
                    if o[a] < 0 or o[a] >= F(N[a]):
                        miss = True
                    continue
                inv[a] = F(1) / d[a]
                t0 = (F(0) - o[a]) * inv[a]
                t1 = (F(N[a]) - o[a]) * inv[a]
                if t0 > t1:
                    t0, t1 = t1, t0
                if t0 > tmin:
                    tmin, entry = t0, a
                if t1 < tmax:
                    tmax = t1
            if miss or not tmin <= tmax:
                continue
            cell, step, base, per, nst = [0] * 3, [0] * 3, [F(np.inf)] * 3, [F(np.inf)] * 3, [0] * 3
            for a in range(3):
                c = int(np.floor(o[a] + d[a] * tmin))
                cell[a] = min(max(c, 0), N[a] - 1)
                step[a] = 1 if d[a] > 0 else (-1 if d[a] < 0 else 0)
                if d[a] != 0:
                    base[a] = (F(cell[a] + (1 if step[a] > 0 else 0)) - o[a]) * inv[a]
                    per[a] = F(abs(inv[a]))
            key = list(base)
            last, tcur = entry, tmin
            for _ in range(X + Y + Z + 3):
                m = int(g[cell[1], cell[2], cell[0]])
                if m:
                    n = [F(0)] * 3
                    if last >= 0:
                        n[last] = F(-1) if step[last] > 0 else F(1)
                    lv = normalize3([o[a] + d[a] * tcur - lp[a] for a in range(3)])
                    diff = max(F(0.05), n[0] * lv[0] + n[1] * lv[1] + n[2] * lv[2])
                    col = PALETTE[m if m < 4 else 4]
                    img[py, px, :3] = [F(col[k]) * diff for k in range(3)]
                    break
                if key[0] < key[1]:
                    a = 0 if key[0] < key[2] else 2
                else:
                    a = 1 if key[1] < key[2] else 2
                tcur = key[a]
                cell[a] += step[a]
                if cell[a] < 0 or cell[a] >= N[a]:
                    break
                nst[a] += 1
                key[a] = fma32(F(nst[a]), per[a], base[a])
                last = a
    return img
