"""Writes tests/golden/golden.json from the CPU oracle.

These vectors are self-recorded (the upstream project has no step, tests or
fixtures to take them from); they pin the oracle, the generators and the rule
against silent change and across hosts (x86_64 here, aarch64 on the GPU host).
Run from the repository root: python tests/golden/make_golden.py
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
import oracle_lib  # noqa: E402
import rule_py  # noqa: E402


def dda_camera():
    """A fixed camera looking into a 64^3 world from outside (oracle_lib.Camera)."""
    c = oracle_lib.Camera()
    vals = {"origin": (-20.5, 70.25, -30.0), "forward": (0.48, -0.6, 0.64), "right": (0.8, 0.0, -0.6),
            "up": (0.36, 0.8, 0.48)}
    for k, v in vals.items():
        for a in range(3):
            getattr(c, k)[a] = v[a]
    c.tan_half_fov, c.aspect = 0.7, 64 / 48
    c.light_pos[0], c.light_pos[1], c.light_pos[2] = 30.0, 90.0, 20.0
    return c


def dda_digest(orc) -> str:
    """SHA-256 of the float32 RGBA image of the voxel DDA on the 64^3 dunes
    world after 30 oracle steps."""
    g = orc.gen_c5(1, 64, 64, 64)
    orc.run(g, 1, 0, 30, nthreads=0)
    img = orc.render_dda(g, dda_camera(), 64, 48)
    return hashlib.sha256(np.ascontiguousarray(img, dtype=np.float32).tobytes()).hexdigest()


def main():
    orc = oracle_lib.load()
    out = {"rule": "FS3D-rule v1", "parity_runs": {}, "generators": {}}
    for seed in (1, 2, 3, 4):
        g = orc.gen_c1(seed)
        out["parity_runs"][str(seed)] = [str(int(h)) for h in orc.run(g, seed, 0, 200, nthreads=0, hashes=True)]
    gen = out["generators"]
    gen["parity_s1_64"] = str(orc.hash(orc.gen_c1(1)))
    gen["pillars_s1_128x160x96"] = str(orc.hash(orc.gen_c2(1, 128, 160, 96)))
    gen["dunes_s1_128"] = str(orc.hash(orc.gen_c5(1, 128, 128, 128)))
    dims, seeds = orc.gen_c3_dims(1, 2048)
    gen["batch_seeds_m1_2048"] = str(rule_py.fmix64(int(np.bitwise_xor.reduce(seeds))))
    gen["batch_dims_sum_m1_2048"] = str(int(dims.sum()))
    for w in range(4):
        X, Y, Z = (int(v) for v in dims[w])
        gen["batch_world_%d" % w] = str(orc.hash(orc.gen_c3_world(int(seeds[w]), X, Y, Z)))
    out["renders"] = {"dda_dunes64_s1_t30_64x48": dda_digest(orc)}
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(out, f, indent=1)
        f.write("\n")


if __name__ == "__main__":
    main()
