"""The library's host-only code (the seeded generators, the request planner,
the status and error plumbing) built once more at -O0 with gcc's
undefined-behaviour checks and, where its runtime is installed, its address
checks (every report aborts), and run on odd and full sizes: its outputs must
equal the shipped library's byte for byte.  The batch
entry points the server calls are stubbed (the planner never reaches them);
nothing here touches a GPU."""
import ctypes as C
import os
import shutil
import subprocess
import sys

import numpy as np
import pytest

from sanitize_util import report_found, sanitize_flags

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "fallingsand3d_gb300", "csrc")

STUBS = r"""
#include "fs3d_common.h"
#include "planes.h"
namespace fs3d {
fs3d_status set_inject_tx_extra(uint32_t) { return FS3D_OK; }
void set_inject_alloc_failures(int) {}
}
extern "C" {
#define STUB(name, ...) fs3d_status name(__VA_ARGS__) { return FS3D_ERR_STATE; }
STUB(fs3d_batch_create, size_t, const fs3d_config*, fs3d_batch**)
STUB(fs3d_batch_destroy, fs3d_batch*)
STUB(fs3d_batch_stream, fs3d_batch*, void**)
STUB(fs3d_batch_admit_generated, fs3d_batch*, int, int, int, uint64_t, uint64_t, int64_t, uint64_t*)
STUB(fs3d_batch_run_segment, fs3d_batch*)
STUB(fs3d_batch_sync, fs3d_batch*, int64_t)
STUB(fs3d_batch_poll, fs3d_batch*, uint64_t, int*, uint64_t*)
STUB(fs3d_batch_poll_many, fs3d_batch*, int, const uint64_t*, int*, uint64_t*)
STUB(fs3d_batch_retire, fs3d_batch*, uint64_t, uint8_t*)
STUB(fs3d_batch_retire_many, fs3d_batch*, int, const uint64_t*, uint8_t* const*)
STUB(fs3d_batch_stats, const fs3d_batch*, int64_t*, int64_t*, size_t*, size_t*)
}
"""

# (generator, seed, X, Y, Z): default sizes and odd ones
GRIDS = [("fs3d_gen_parity", 1, 64, 64, 64), ("fs3d_gen_parity", 7, 37, 29, 41),
         ("fs3d_gen_pillars", 1, 128, 160, 96), ("fs3d_gen_pillars", 3, 33, 17, 65),
         ("fs3d_gen_dunes", 1, 128, 128, 128), ("fs3d_gen_dunes", 5, 45, 70, 23),
         ("fs3d_gen_batch_world", 11, 48, 96, 16), ("fs3d_gen_batch_world", 12, 17, 5, 130)]
PLANS = [(2000.0, 0.5, 3, 10, 150), (8000.0, 1.0, 9, 1, 1000), (50.0, 2.0, 1, 500, 500)]

CHILD = r"""
import ctypes as C, sys
import numpy as np
d = np.load(sys.argv[2], allow_pickle=True)
L = C.CDLL(sys.argv[1])
L.fs3d_gen_batch_dims.argtypes = [C.c_uint64, C.c_int, C.c_void_p, C.c_void_p]
for i, (name, seed, X, Y, Z) in enumerate(d["grids"]):
    fn = getattr(L, str(name))
    fn.argtypes = [C.c_uint64, C.c_int, C.c_int, C.c_int, C.c_void_p]
    g = np.empty((int(Y), int(Z), int(X)), np.uint8)
    assert fn(int(seed), int(X), int(Y), int(Z), g.ctypes.data) == 0
    assert np.array_equal(g, d["grid%d" % i]), name
dims = np.empty((2048, 3), np.int32); seeds = np.empty(2048, np.uint64)
assert L.fs3d_gen_batch_dims(1, 2048, dims.ctypes.data, seeds.ctypes.data) == 0
assert np.array_equal(dims, d["dims"]) and np.array_equal(seeds, d["seeds"])
for i, blob in enumerate(d["plans"]):
    p = (C.c_char * len(d["params%d" % i].tobytes())).from_buffer_copy(d["params%d" % i].tobytes())
    n = C.c_int64()
    assert L.fs3d_serve_plan(p, C.c_int64(0), None, C.byref(n)) == 0
    buf = (C.c_char * (len(blob.tobytes()) or 1))()
    assert L.fs3d_serve_plan(p, n, buf, C.byref(n)) == 0
    assert bytes(buf)[:len(blob.tobytes())] == blob.tobytes(), i
print("ok")
"""


def test_host_code_under_sanitizers_at_O0(fs3d, tmp_path):
    cuda_inc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
    cuda_lib = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "lib64")
    if not shutil.which("g++") or not os.path.exists(os.path.join(cuda_inc, "cuda_runtime.h")):
        pytest.skip("g++ or the CUDA headers not found")
    stub = tmp_path / "stubs.cpp"
    stub.write_text(STUBS)
    flags, env_add, _ = sanitize_flags()
    so = tmp_path / "libhost_checked.so"
    r = subprocess.run(["g++", "-O0", "-std=c++17", "-fPIC", *flags, "-I", cuda_inc, "-I", CSRC, "-shared", "-o", str(so),
                        *(os.path.join(CSRC, f) for f in ("gen.cpp", "abi.cpp", "serve.cpp")), str(stub),
                        "-L", cuda_lib, "-lcudart"], capture_output=True, text=True)
    if r.returncode != 0 and "san" in r.stderr:
        pytest.skip("gcc's sanitizer runtime is not installed")
    assert r.returncode == 0, r.stderr
    # the shipped library's outputs
    L = fs3d.lib()
    data = {"grids": np.array(GRIDS, dtype=object)}
    for i, (name, seed, X, Y, Z) in enumerate(GRIDS):
        g = np.empty((Y, Z, X), np.uint8)
        assert getattr(L, name)(seed, X, Y, Z, g.ctypes.data) == 0
        data["grid%d" % i] = g
    data["dims"], data["seeds"] = fs3d.gen_batch_dims(1, 2048)
    plans = []
    for i, (lam, dur, seed, lo, hi) in enumerate(PLANS):
        p = fs3d.serve_params(lam, dur, master_seed=seed, min_steps=lo, max_steps=hi)
        reqs, n = fs3d.serve_plan(p)
        plans.append(np.frombuffer(C.string_at(C.addressof(reqs), C.sizeof(fs3d.ServeRequest) * n), np.uint8))
        data["params%d" % i] = np.frombuffer(C.string_at(C.addressof(p), C.sizeof(p)), np.uint8)
    data["plans"] = np.array(plans + [None], dtype=object)[:-1]
    npz = tmp_path / "expected.npz"
    np.savez(npz, **data)
    t = subprocess.run([sys.executable, "-c", CHILD, str(so), str(npz)], capture_output=True, text=True,
                       env=dict(os.environ, **env_add), timeout=600)
    out = t.stdout + t.stderr
    assert t.returncode == 0 and not report_found(out) and "ok" in t.stdout, out[-3000:]
