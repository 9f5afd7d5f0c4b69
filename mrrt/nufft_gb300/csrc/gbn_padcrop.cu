// Deapodisation + zero-pad (forward) and crop + deapodisation (adjoint).
//
// Forward (mrrt/nufft/_nufft.py:1325-1331): xk = x * sn, zero-padded to Kd.
// The padded buffer is persistent and its padding stays zero, so only the
// Nd-sized corner is written per call.
// Adjoint (mrrt/nufft/_nufft.py:1561-1572): x = grid[:N] * scale * conj(sn),
// where the grid holds the unnormalised inverse FFT and scale folds the
// reference's prod(Kd) * adjoint_scalefactor with ifftn's 1/prod(Kd)
// (or the orthonormal factors).
//
// One warp per image row (memory axis 0); rows are enumerated over
// (plane, axis 1, axis 2).
#include <cuda_runtime.h>

#include "gbn_device.cuh"
#include "gbn_internal.h"

namespace gbn {

template <typename R>
__global__ void __launch_bounds__(256) pad_kernel(const PadParams<R> p) {
    typedef typename Cx<R>::T C;
    const int lane = threadIdx.x & 31;
    const int64_t rows_per_plane = (int64_t)p.N[1] * p.N[2];
    const int64_t nrows = rows_per_plane * p.planes;
    const int64_t wid = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t row = wid; row < nrows; row += nw) {
        const int64_t pl = row / rows_per_plane;
        const int64_t rr = row - pl * rows_per_plane;
        const int n1 = (int)(rr % p.N[1]);
        const int n2 = (int)(rr / p.N[1]);
        const C* src = p.x + pl * p.Nprod + rr * p.N[0];
        const R* s = p.sn + rr * p.N[0];
        C* dst = p.out + pl * p.Kprod + ((int64_t)n2 * p.K[1] + n1) * p.K[0];
        for (int n0 = lane; n0 < p.N[0]; n0 += 32) {
            C v = src[n0];
            const R w = s[n0];
            v.x *= w;
            v.y *= w;
            dst[n0] = v;
        }
    }
}

template <typename R>
__global__ void __launch_bounds__(256) crop_kernel(const CropParams<R> p) {
    typedef typename Cx<R>::T C;
    const int lane = threadIdx.x & 31;
    const int64_t rows_per_plane = (int64_t)p.N[1] * p.N[2];
    const int64_t nrows = rows_per_plane * p.planes;
    const int64_t wid = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t row = wid; row < nrows; row += nw) {
        const int64_t pl = row / rows_per_plane;
        const int64_t rr = row - pl * rows_per_plane;
        const int n1 = (int)(rr % p.N[1]);
        const int n2 = (int)(rr / p.N[1]);
        const C* src = p.grid + pl * p.Kprod + ((int64_t)n2 * p.K[1] + n1) * p.K[0];
        const R* s = p.sn + rr * p.N[0];
        C* dst = p.x + pl * p.Nprod + rr * p.N[0];
        for (int n0 = lane; n0 < p.N[0]; n0 += 32) {
            C v = src[n0];
            v.x *= p.scale;
            v.y *= p.scale;
            const R w = s[n0];
            v.x *= w;
            v.y *= w;
            dst[n0] = v;
        }
    }
}

static int row_grid(int64_t nrows) {
    int64_t warps = nrows;
    int64_t blocks = (warps + 7) / 8;
    if (blocks > 152 * 32) blocks = 152 * 32;
    if (blocks < 1) blocks = 1;
    return (int)blocks;
}

template <typename R>
cudaError_t launch_pad(const PadParams<R>& p, cudaStream_t s) {
    if (p.planes == 0 || p.Nprod == 0) return cudaSuccess;
    const int64_t nrows = (int64_t)p.N[1] * p.N[2] * p.planes;
    pad_kernel<R><<<row_grid(nrows), 256, 0, s>>>(p);
    return cudaGetLastError();
}

template <typename R>
cudaError_t launch_crop(const CropParams<R>& p, cudaStream_t s) {
    if (p.planes == 0 || p.Nprod == 0) return cudaSuccess;
    const int64_t nrows = (int64_t)p.N[1] * p.N[2] * p.planes;
    crop_kernel<R><<<row_grid(nrows), 256, 0, s>>>(p);
    return cudaGetLastError();
}

template cudaError_t launch_pad<float>(const PadParams<float>&, cudaStream_t);
template cudaError_t launch_pad<double>(const PadParams<double>&, cudaStream_t);
template cudaError_t launch_crop<float>(const CropParams<float>&, cudaStream_t);
template cudaError_t launch_crop<double>(const CropParams<double>&, cudaStream_t);

}  // namespace gbn
