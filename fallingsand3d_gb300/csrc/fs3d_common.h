// Shared helpers of libfs3d: the counter-based hash of FS3D-rule v1, status
// plumbing and launch accounting.  Host and device see the same definitions.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <string>

#include "../../include/fs3d.h"

#define FS3D_HD __host__ __device__ __forceinline__

namespace fs3d {

// MurmurHash3 finalizers (Appleby, public domain).
FS3D_HD uint32_t fmix32(uint32_t h) {
    h ^= h >> 16;
    h *= 0x85ebca6bu;
    h ^= h >> 13;
    h *= 0xc2b2ae35u;
    h ^= h >> 16;
    return h;
}

FS3D_HD uint64_t fmix64(uint64_t k) {
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdULL;
    k ^= k >> 33;
    k *= 0xc4ceb9fe1a85ec53ULL;
    k ^= k >> 33;
    return k;
}

// Per (world seed, step) key; computed once per step on the host.
FS3D_HD uint32_t stepkey(uint64_t seed, uint64_t t) {
    uint32_t h = fmix32(0x243F6A88u ^ (uint32_t)seed);
    h = fmix32(h ^ (uint32_t)(seed >> 32));
    h = fmix32(h ^ (uint32_t)t);
    h = fmix32(h ^ (uint32_t)(t >> 32));
    return h;
}

// Per block row (j along y, k along z).
FS3D_HD uint32_t rowkey(uint32_t sk, uint32_t j, uint32_t k) {
    uint32_t h = fmix32(sk ^ (0x85EBCA77u * (j + 1u)));
    return fmix32(h ^ (0xC2B2AE3Du * (k + 1u)));
}

// Random word w of slot s for the 32 blocks i in [32g, 32g+32) of a block
// row: bit (i & 31) belongs to block i.
FS3D_HD uint32_t plane(uint32_t rk, uint32_t g, uint32_t s, uint32_t w) {
    return fmix32(rk + 0x9E3779B9u * (1u + w + 8u * s + 64u * g));
}

FS3D_HD int nblocks(int n, int o) { return (n + o + 1) >> 1; }

// ---- status plumbing ----
fs3d_status set_error(fs3d_status s, const std::string& msg);
fs3d_status cuda_fail(cudaError_t e, const char* what);
void note_launch(uint64_t n = 1);
// Unique id of the calling thread's current CUDA context; false if no context
// is current yet (the runtime makes one current on its first device call) or
// the driver cannot tell.  A device address cached for one context is stale
// in another (after cudaDeviceReset, for example).
bool current_context_id(unsigned long long* id);

}  // namespace fs3d

#define FS3D_CUDA(call)                                              \
    do {                                                             \
        cudaError_t e_ = (call);                                     \
        if (e_ != cudaSuccess) return ::fs3d::cuda_fail(e_, #call);  \
    } while (0)

#define FS3D_CHECK_LAUNCH(what)                                      \
    do {                                                             \
        cudaError_t e_ = cudaGetLastError();                         \
        if (e_ != cudaSuccess) return ::fs3d::cuda_fail(e_, what);   \
        ::fs3d::note_launch();                                       \
    } while (0)
