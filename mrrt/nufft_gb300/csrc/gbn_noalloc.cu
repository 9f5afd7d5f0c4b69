// Fixed scratch array for gbn_interp_adjoint_noalloc.
//
// The adjoint spread splits a crowded tile over several CTAs; each writes its
// partial sums to scratch memory and reduce_kernel adds them up in part order.
// gbn_interp_adjoint keeps that scratch in a per-plan buffer that it grows
// with cudaMalloc.  Callers that cannot allocate during a call (a fixed
// device-memory budget, or no room for the device-wide synchronisation a
// cudaMalloc / cudaFree may cause) use this array instead: it is part of the
// module image, so the CUDA driver reserves it when the module loads and no
// allocator is ever called for it.
//
// The array lives in its own translation unit so that the module holding it
// (and its 64 MiB) is only loaded by processes that use the no-alloc entry
// point.
#include <cuda_runtime.h>

#include <mutex>

#include "../../../include/gbnufft.h"
#include "gbn_internal.h"

// Nothing in it has to start at zero: every part of a split tile writes all
// cells that reduce_kernel later reads, before it reads them.
static __device__ __align__(256) unsigned char g_noalloc_scratch[GBN_NOALLOC_SCRATCH_BYTES];

namespace gbn {

namespace {
constexpr int NOALLOC_MAX_DEVICES = 64;
std::mutex g_noalloc_mu;
void* g_noalloc_addr[NOALLOC_MAX_DEVICES] = {};
}  // namespace

// Device address of the array on the current device.  The first request on
// a device looks it up (with that device current) and caches it; later
// requests only read the cache.
cudaError_t noalloc_scratch(void** ptr, size_t* bytes) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        if (!p) return cudaErrorInvalidSymbol;
        g_noalloc_addr[dev] = p;
    }
    *ptr = g_noalloc_addr[dev];
    *bytes = sizeof(g_noalloc_scratch);
    return cudaSuccess;
}

}  // namespace gbn
