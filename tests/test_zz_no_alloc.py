"""GPU check of fs3d_run_device_noalloc, the entry point for callers that
cannot allocate device memory (an engine whose own allocator owns the GPU's
memory, or a real-time frame loop that must not stall on an allocation).

Called through the C ABI, it must give exactly what fs3d_run_device gives
(integer work: bit-exact), on two calls in a row, since every call shares the
same static scratch array and inherits the previous call's contents; it must
equal the CPU oracle; and it must allocate nothing.  The file is named so
pytest collects it last."""
import ctypes as C
import os

import numpy as np
import pytest

from gpu_util import describe_diff, stream_ptr, to_device

pytestmark = pytest.mark.gpu

# cudaMemPoolAttr values (driver_types.h)
_USED_MEM_CURRENT, _USED_MEM_HIGH = 0x7, 0x8


def _grid(X, Y, Z, seed):
    rng = np.random.default_rng(seed)
    return rng.choice(np.array([0, 0, 0, 0, 1, 2, 2, 3, 3, 6], np.uint8), size=(Y, Z, X))


# a world one CTA holds in shared memory, one stepped by the per-step kernel
# (too large for shared memory), and a small odd-sized one
CASES = [((64, 64, 64), 11, 3, 40), ((512, 128, 512), 12, 0, 9), ((24, 40, 33), 13, 7, 21)]


def test_noalloc_matches_allocating_entry_point(fs3d, cuda):
    L = fs3d.lib()
    st = stream_ptr(cuda)
    for (X, Y, Z), seed, t0, n in CASES + CASES[:1]:  # the first case twice: reuse after other worlds
        g = _grid(X, Y, Z, seed)
        a, b = to_device(cuda, g), to_device(cuda, g)
        assert L.fs3d_run_device(C.c_void_p(a.data_ptr()), X, Y, Z, seed, t0, n, C.c_void_p(st)) == 0
        # two calls in a row on the no-allocation entry point, continuing the same world
        half = n // 2
        assert L.fs3d_run_device_noalloc(C.c_void_p(b.data_ptr()), X, Y, Z, seed, t0, half, C.c_void_p(st)) == 0
        assert L.fs3d_run_device_noalloc(C.c_void_p(b.data_ptr()), X, Y, Z, seed, t0 + half, n - half,
                                         C.c_void_p(st)) == 0
        cuda.cuda.synchronize()
        want, got = a.cpu().numpy(), b.cpu().numpy()
        assert (got == want).all(), describe_diff(got, want, n - 1)
        assert not (got == g).all()


def test_noalloc_rejects_worlds_beyond_its_scratch(fs3d, cuda):
    L = fs3d.lib()
    d = cuda.zeros(16, dtype=cuda.uint8, device="cuda")
    # 2048 x 256 x 2048 cells: 256 MiB of planes, four times the static scratch
    assert L.fs3d_run_device_noalloc(C.c_void_p(d.data_ptr()), 2048, 256, 2048, 1, 0, 1, None) == fs3d.ERR_INVALID_ARG
    assert b"64 MiB" in L.fs3d_last_error()
    # rows wider than 2048 cells
    assert L.fs3d_run_device_noalloc(C.c_void_p(d.data_ptr()), 4096, 2, 2, 1, 0, 1, None) == fs3d.ERR_INVALID_ARG


@pytest.mark.parametrize("dims", [(64, 64, 64), (512, 128, 512), (24, 40, 33), (130, 30, 70)])
def test_noalloc_matches_oracle(fs3d, orc, cuda, dims):
    X, Y, Z = dims
    seed = X * 31 + Y * 7 + Z
    g = _grid(X, Y, Z, seed)
    d = to_device(cuda, g)
    L = fs3d.lib()
    st = stream_ptr(cuda)
    # two calls in a row continue one world: the second inherits the scratch the first left
    assert L.fs3d_run_device_noalloc(C.c_void_p(d.data_ptr()), X, Y, Z, seed, 5, 11, C.c_void_p(st)) == 0
    assert L.fs3d_run_device_noalloc(C.c_void_p(d.data_ptr()), X, Y, Z, seed, 16, 9, C.c_void_p(st)) == 0
    fs3d.run_device_check(st)
    ref = g.copy()
    orc.run(ref, seed, 5, 20, nthreads=0)
    got = d.cpu().numpy()
    assert (got == ref).all(), describe_diff(got, ref, 24)


def _cudart():
    for name in ("/usr/local/cuda/lib64/libcudart.so.13", "libcudart.so.13", "libcudart.so"):
        try:
            return C.CDLL(name)
        except OSError:
            continue
    return None


def test_noalloc_allocates_nothing(fs3d, cuda):
    """Neither the stream-ordered pool nor plain device memory grows while the
    calls run: the pool's high-water mark stays at its level before them, and
    the device's free memory is unchanged after them."""
    rt = _cudart()
    if rt is None:
        pytest.skip("the CUDA runtime library is not loadable here")
    X, Y, Z = 128, 96, 80
    g = _grid(X, Y, Z, 3)
    d = to_device(cuda, g)
    L = fs3d.lib()
    st = stream_ptr(cuda)
    # a first call (the array's address is looked up once per device) and a warm torch
    assert L.fs3d_run_device_noalloc(C.c_void_p(d.data_ptr()), X, Y, Z, 3, 0, 4, C.c_void_p(st)) == 0
    cuda.cuda.synchronize()
    pool = C.c_void_p()
    assert rt.cudaDeviceGetDefaultMemPool(C.byref(pool), cuda.cuda.current_device()) == 0
    used, high, zero = C.c_uint64(), C.c_uint64(), C.c_uint64(0)
    assert rt.cudaMemPoolSetAttribute(pool, _USED_MEM_HIGH, C.byref(zero)) == 0  # high mark := current
    assert rt.cudaMemPoolGetAttribute(pool, _USED_MEM_CURRENT, C.byref(used)) == 0
    free0 = cuda.cuda.mem_get_info()[0]
    for t0 in (4, 10):
        assert L.fs3d_run_device_noalloc(C.c_void_p(d.data_ptr()), X, Y, Z, 3, t0, 6, C.c_void_p(st)) == 0
    cuda.cuda.synchronize()
    assert rt.cudaMemPoolGetAttribute(pool, _USED_MEM_HIGH, C.byref(high)) == 0
    assert high.value == used.value, (high.value, used.value)
    assert cuda.cuda.mem_get_info()[0] == free0
