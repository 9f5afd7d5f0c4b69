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
// The array lives in its own translation unit.  Under lazy module loading
// (CUDA_MODULE_LOADING=LAZY, the default since CUDA 12.2) the module holding
// it, and its 64 MiB, is loaded on a device only when a process first uses
// the no-alloc entry point there.  With CUDA_MODULE_LOADING=EAGER every
// process that loads libgbnufft reserves the 64 MiB on each device it
// initialises.
#include <cuda_runtime.h>

#include "../../../include/gbnufft.h"
#include "gbn_internal.h"

// Nothing in it has to start at zero: every part of a split tile writes all
// cells that reduce_kernel later reads, before it reads them.
static __device__ __align__(256) unsigned char g_noalloc_scratch[GBN_NOALLOC_SCRATCH_BYTES];

namespace gbn {

// Device address of the array on the current device, looked up on every
// call.  The lookup allocates nothing once the module is loaded, and a
// fresh lookup stays right after cudaDeviceReset or a re-created primary
// context, which may load the module (and the array) at another address.
cudaError_t noalloc_scratch(void** ptr, size_t* bytes) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    if (!p) return cudaErrorInvalidSymbol;
    *ptr = p;
    *bytes = sizeof(g_noalloc_scratch);
    return cudaSuccess;
}

}  // namespace gbn
