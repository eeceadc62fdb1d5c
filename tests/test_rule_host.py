"""The device rule code itself, compiled for the host (g++ over
fallingsand3d_gb300/csrc/rule_device.cuh, the few CUDA intrinsics it uses
given host definitions), checked block by block against the independent
Python statement of the rule on random blocks of every density: the
bit-sliced rule (32 blocks per word), the scalar block rule, the activity
mask (exactly the blocks that change) and the scalar can-move predicate.
No GPU: this checks the rule's logic; the GPU tests check the kernels."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

import rule_py

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "fallingsand3d_gb300", "csrc")

HARNESS = r"""
#include <stdint.h>
#include <stdlib.h>
static inline int __popc(uint32_t v) { return __builtin_popcount(v); }
static inline int __ffs(uint32_t v) { return __builtin_ffs((int)v); }
// warp shuffles appear in the row-pair helpers, which this harness never calls
static inline uint32_t __shfl_up_sync(unsigned, uint32_t v, int) { abort(); return v; }
static inline uint32_t __shfl_down_sync(unsigned, uint32_t v, int) { abort(); return v; }
#include "rule_device.cuh"
extern "C" uint32_t h_bs_rule(uint32_t* A, uint32_t* B, uint32_t rk, uint32_t g, uint32_t* active) {
    uint32_t a[8], b[8], W[8], E[8];
    for (int s = 0; s < 8; ++s) {
        a[s] = A[s];
        b[s] = B[s];
        W[s] = a[s] & b[s];
        E[s] = ~(a[s] | b[s]);
    }
    *active = fs3d::activity_mask(a, W, E);
    const uint32_t c = fs3d::bs_rule(a, b, rk, g);
    for (int s = 0; s < 8; ++s) {
        A[s] = a[s];
        B[s] = b[s];
    }
    return c;
}
extern "C" uint64_t h_block_rule(uint64_t V, uint32_t rk, uint32_t i) { return fs3d::block_rule(V, rk, i); }
extern "C" int h_block_can_move(uint32_t T, uint32_t B) { return fs3d::block_can_move(T, B) ? 1 : 0; }
"""


@pytest.fixture(scope="module")
def host_rule(tmp_path_factory):
    cuda_inc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
    if not shutil.which("g++") or not os.path.exists(os.path.join(cuda_inc, "cuda_runtime.h")):
        pytest.skip("g++ or the CUDA headers not found")
    d = tmp_path_factory.mktemp("host_rule")
    src, so = d / "harness.cpp", d / "libhostrule.so"
    src.write_text(HARNESS)
    subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-w", "-I", cuda_inc, "-I", CSRC,
                    "-o", str(so), str(src)], check=True)
    L = C.CDLL(str(so))
    u32p = C.POINTER(C.c_uint32)
    L.h_bs_rule.restype = C.c_uint32
    L.h_bs_rule.argtypes = [u32p, u32p, C.c_uint32, C.c_uint32, u32p]
    L.h_block_rule.restype = C.c_uint64
    L.h_block_rule.argtypes = [C.c_uint64, C.c_uint32, C.c_uint32]
    L.h_block_can_move.restype = C.c_int
    L.h_block_can_move.argtypes = [C.c_uint32, C.c_uint32]
    return L


def planes_of(vals):
    """(A, B) per slot for 32 blocks: empty (0,0), solid (0,1), sand (1,0), water (1,1)."""
    bits = 1 << np.arange(32, dtype=np.uint64)
    A = [int(((vals[:, s] >= 2) * bits).sum()) for s in range(8)]
    B = [int((((vals[:, s] == 1) | (vals[:, s] == 3)) * bits).sum()) for s in range(8)]
    return A, B


def values_of(A, B):
    out = np.zeros((32, 8), np.int64)
    for s in range(8):
        for b in range(32):
            a, bb = (A[s] >> b) & 1, (B[s] >> b) & 1
            out[b, s] = 2 + bb if a else bb
    return out


def test_device_rule_equals_python_statement(host_rule):
    L = host_rule
    rng = np.random.default_rng(20241204)
    trials = 0
    for density in (0.1, 0.35, 0.6, 0.9):  # share of non-empty cells
        for _ in range(150):
            p_empty = 1.0 - density
            w = rng.dirichlet([1.0, 1.0, 1.0]) * density  # solid, sand, water
            vals = rng.choice(4, size=(32, 8), p=[p_empty, *w])
            rk, g = int(rng.integers(0, 1 << 32)), int(rng.integers(0, 4))
            exp = np.array([rule_py.block(vals[b], rk, 32 * g + b) for b in range(32)])
            A, B = planes_of(vals)
            a = (C.c_uint32 * 8)(*A)
            bb = (C.c_uint32 * 8)(*B)
            active = C.c_uint32()
            changed = L.h_bs_rule(a, bb, rk, g, C.byref(active))
            got = values_of(list(a), list(bb))
            assert np.array_equal(got, exp), (density, rk, g)
            moved = sum(1 << b for b in range(32) if not np.array_equal(exp[b], vals[b]))
            assert changed == moved and active.value == moved, (density, rk, g)
            for b in range(32):
                V = sum(int(vals[b, s]) << (8 * s) for s in range(8))
                out = L.h_block_rule(V, rk, 32 * g + b)
                assert [(out >> (8 * s)) & 0xFF for s in range(8)] == list(exp[b]), (rk, g, b)
                T = sum(int(vals[b, q]) << (8 * q) for q in range(4))
                Bo = sum(int(vals[b, 4 + q]) << (8 * q) for q in range(4))
                assert L.h_block_can_move(T, Bo) == int((moved >> b) & 1), (rk, g, b)
            trials += 1
    assert trials == 600
