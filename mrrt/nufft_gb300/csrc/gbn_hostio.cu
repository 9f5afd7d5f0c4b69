// Host-to-device copy done by a kernel that reads pageable host memory in
// place.  On a system whose GPU shares the host's page tables (the device
// attribute cudaDevAttrPageableMemoryAccess is 1, e.g. Grace over
// NVLink-C2C) this moves a caller's ordinary (unpinned) array at the link's
// rate without the CUDA driver's staging through pinned bounce buffers, and,
// unlike a copy from pageable memory, it does not hold the calling thread
// while the data move.  The host-buffer transforms use it for inputs that
// are not pinned; pinned inputs and every output go through the copy engines.
#include <cuda_runtime.h>

#include <cstdint>

#include "gbn_internal.h"

namespace gbn {

// 16-byte words, grid-stride; four independent loads in flight per thread
// keep enough requests outstanding to cover the link's latency.
__global__ void __launch_bounds__(256) host_read_kernel(const int4* __restrict__ src, int4* __restrict__ dst,
                                                        int64_t n) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (; i + 3 * stride < n; i += 4 * stride) {
        const int4 a = src[i], b = src[i + stride], c = src[i + 2 * stride], d = src[i + 3 * stride];
        dst[i] = a;
        dst[i + stride] = b;
        dst[i + 2 * stride] = c;
        dst[i + 3 * stride] = d;
    }
    for (; i < n; i += stride) dst[i] = src[i];
}

cudaError_t launch_host_read(void* dst, const void* src, size_t bytes, int sms, cudaStream_t s) {
    if (bytes == 0) return cudaSuccess;
    if ((reinterpret_cast<uintptr_t>(dst) | reinterpret_cast<uintptr_t>(src) | bytes) & 15)
        return cudaErrorInvalidValue;
    const int64_t n = (int64_t)(bytes / 16);
    // two CTAs per SM saturate the host link; more only add contention with
    // the transform kernels running beside the copy
    int64_t blocks = (n + 255) / 256;
    if (blocks > 2 * (int64_t)sms) blocks = 2 * (int64_t)sms;
    host_read_kernel<<<(unsigned)blocks, 256, 0, s>>>(reinterpret_cast<const int4*>(src), reinterpret_cast<int4*>(dst),
                                                      n);
    return cudaGetLastError();
}

}  // namespace gbn
