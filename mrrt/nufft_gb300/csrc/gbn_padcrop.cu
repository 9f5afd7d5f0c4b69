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
// (plane, axis 1, axis 2).  The coil-sensitivity variants fuse the MRI
// system operator's coil-map multiply (forward) and conjugate-map coil sum
// (adjoint) into these passes.
#include <cuda_runtime.h>

#include <cstdint>

#include "gbn_device.cuh"
#include "gbn_internal.h"

namespace gbn {

// PAIRS: single precision with even rows and 16-byte aligned rows on both
// sides; a lane then moves two adjacent complex values per access (16-byte
// loads and stores, 8-byte loads of sn), four accesses in flight.
template <typename R, bool PAIRS>
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
        const int64_t xo = pl * p.Nprod + rr * p.N[0];
        const int64_t oo = pl * p.gsp + (int64_t)n1 * p.gs1 + (int64_t)n2 * p.gs2;
        if (!GBN_INB(p.check, xo + p.N[0] <= p.x_elems, CHK_IMAGE) ||
            !GBN_INB(p.check, oo + p.N[0] <= p.out_elems, CHK_GRID_WRITE))
            continue;
        const C* src = p.x + xo;
        const R* s = p.sn + rr * p.N[0];
        C* dst = p.out + oo;
        if constexpr (PAIRS) {
            const float4* s4 = reinterpret_cast<const float4*>(src);
            const float2* w2 = reinterpret_cast<const float2*>(s);
            float4* d4 = reinterpret_cast<float4*>(dst);
            const int np = p.N[0] >> 1;
#pragma unroll 4
            for (int q = lane; q < np; q += 32) {
                float4 v = s4[q];
                const float2 w = w2[q];
                v.x *= w.x;
                v.y *= w.x;
                v.z *= w.y;
                v.w *= w.y;
                d4[q] = v;
            }
        } else {
            for (int n0 = lane; n0 < p.N[0]; n0 += 32) {
                C v = src[n0];
                const R w = s[n0];
                v.x *= w;
                v.y *= w;
                dst[n0] = v;
            }
        }
    }
}

template <typename R, bool PAIRS>
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
        const int64_t go = pl * p.gsp + (int64_t)n1 * p.gs1 + (int64_t)n2 * p.gs2;
        const int64_t xo = pl * p.Nprod + rr * p.N[0];
        if (!GBN_INB(p.check, go + p.N[0] <= p.grid_elems, CHK_GRID_READ) ||
            !GBN_INB(p.check, xo + p.N[0] <= p.x_elems, CHK_IMAGE))
            continue;
        const C* src = p.grid + go;
        const R* s = p.sn + rr * p.N[0];
        C* dst = p.x + xo;
        if constexpr (PAIRS) {
            const float4* s4 = reinterpret_cast<const float4*>(src);
            const float2* w2 = reinterpret_cast<const float2*>(s);
            float4* d4 = reinterpret_cast<float4*>(dst);
            const int np = p.N[0] >> 1;
            const float sc = (float)p.scale;
#pragma unroll 4
            for (int q = lane; q < np; q += 32) {
                float4 v = s4[q];
                const float2 w = w2[q];
                v.x *= sc;
                v.y *= sc;
                v.z *= sc;
                v.w *= sc;
                v.x *= w.x;
                v.y *= w.x;
                v.z *= w.y;
                v.w *= w.y;
                d4[q] = v;
            }
        } else {
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
}

// Rows of both buffers start on 16-byte boundaries and hold whole pairs.
template <typename R>
static bool pairs_ok(int N0, int64_t Nprod, int64_t gsp, int64_t gs1, int64_t gs2, const void* a, const void* b) {
    return sizeof(R) == 4 && (N0 % 2) == 0 && (Nprod % 2) == 0 && (gsp % 2) == 0 && (gs1 % 2) == 0 &&
           (gs2 % 2) == 0 && (reinterpret_cast<uintptr_t>(a) & 15) == 0 && (reinterpret_cast<uintptr_t>(b) & 15) == 0;
}

// Coil-sensitivity pad: plane f * coils + c gets sn * maps[c] * x[f] (the
// multiply an MRI system operator applies before the NUFFT, here fused into
// the deapodisation pass so the coil images are never materialised).
template <typename R>
__global__ void __launch_bounds__(256) pad_sense_kernel(const PadParams<R> p) {
    typedef typename Cx<R>::T C;
    const int lane = threadIdx.x & 31;
    const int64_t rows_per_plane = (int64_t)p.N[1] * p.N[2];
    const int64_t nrows = rows_per_plane * p.planes;
    const int64_t wid = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t row = wid; row < nrows; row += nw) {
        const int64_t pl = row / rows_per_plane;
        const int64_t rr = row - pl * rows_per_plane;
        const int64_t f = pl / p.coils, c = pl - f * p.coils;
        const int n1 = (int)(rr % p.N[1]);
        const int n2 = (int)(rr / p.N[1]);
        const int64_t oo = pl * p.gsp + (int64_t)n1 * p.gs1 + (int64_t)n2 * p.gs2;
        if (!GBN_INB(p.check, (f * p.Nprod + rr * p.N[0]) + p.N[0] <= p.x_elems, CHK_IMAGE) ||
            !GBN_INB(p.check, oo + p.N[0] <= p.out_elems, CHK_GRID_WRITE))
            continue;
        const C* src = p.x + f * p.Nprod + rr * p.N[0];
        const C* mp = p.maps + c * p.Nprod + rr * p.N[0];
        const R* s = p.sn + rr * p.N[0];
        C* dst = p.out + oo;
        for (int n0 = lane; n0 < p.N[0]; n0 += 32) {
            C v = cmul(src[n0], mp[n0]);
            const R w = s[n0];
            v.x *= w;
            v.y *= w;
            dst[n0] = v;
        }
    }
}

// Coil-combining crop: x[f] = sum over c (in coil order) of conj(maps[c]) *
// (scale * sn * cropped plane f * coils + c), one image per frame.
template <typename R>
__global__ void __launch_bounds__(256) crop_sense_kernel(const CropParams<R> p) {
    typedef typename Cx<R>::T C;
    const int lane = threadIdx.x & 31;
    const int64_t rows_per_plane = (int64_t)p.N[1] * p.N[2];
    const int64_t frames = p.planes / p.coils;
    const int64_t nrows = rows_per_plane * frames;
    const int64_t wid = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t row = wid; row < nrows; row += nw) {
        const int64_t f = row / rows_per_plane;
        const int64_t rr = row - f * rows_per_plane;
        const int n1 = (int)(rr % p.N[1]);
        const int n2 = (int)(rr / p.N[1]);
        const int64_t goff = (int64_t)n1 * p.gs1 + (int64_t)n2 * p.gs2;
        if (!GBN_INB(p.check, ((f + 1) * p.coils - 1) * p.gsp + goff + p.N[0] <= p.grid_elems, CHK_GRID_READ) ||
            !GBN_INB(p.check, f * p.Nprod + rr * p.N[0] + p.N[0] <= p.x_elems, CHK_IMAGE))
            continue;
        const R* s = p.sn + rr * p.N[0];
        C* dst = p.x + f * p.Nprod + rr * p.N[0];
        for (int n0 = lane; n0 < p.N[0]; n0 += 32) {
            const R w = s[n0];
            C acc = cmake<R>((R)0, (R)0);
            for (int c = 0; c < p.coils; ++c) {
                C v = p.grid[(f * p.coils + c) * p.gsp + goff + n0];
                v.x *= p.scale;
                v.y *= p.scale;
                v.x *= w;
                v.y *= w;
                const C t = cmulc(v, p.maps[(int64_t)c * p.Nprod + rr * p.N[0] + n0]);
                acc.x += t.x;
                acc.y += t.y;
            }
            dst[n0] = acc;
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
    if (p.maps) {
        if (p.coils < 1) return cudaErrorInvalidValue;
        pad_sense_kernel<R><<<row_grid(nrows), 256, 0, s>>>(p);
    } else if (pairs_ok<R>(p.N[0], p.Nprod, p.gsp, p.gs1, p.gs2, p.x, p.out)) {
        pad_kernel<R, true><<<row_grid(nrows), 256, 0, s>>>(p);
    } else {
        pad_kernel<R, false><<<row_grid(nrows), 256, 0, s>>>(p);
    }
    return cudaGetLastError();
}

template <typename R>
cudaError_t launch_crop(const CropParams<R>& p, cudaStream_t s) {
    if (p.planes == 0 || p.Nprod == 0) return cudaSuccess;
    if (p.maps) {
        if (p.coils < 1 || p.planes % p.coils) return cudaErrorInvalidValue;
        const int64_t nrows = (int64_t)p.N[1] * p.N[2] * (p.planes / p.coils);
        crop_sense_kernel<R><<<row_grid(nrows), 256, 0, s>>>(p);
    } else {
        const int64_t nrows = (int64_t)p.N[1] * p.N[2] * p.planes;
        if (pairs_ok<R>(p.N[0], p.Nprod, p.gsp, p.gs1, p.gs2, p.grid, p.x))
            crop_kernel<R, true><<<row_grid(nrows), 256, 0, s>>>(p);
        else
            crop_kernel<R, false><<<row_grid(nrows), 256, 0, s>>>(p);
    }
    return cudaGetLastError();
}

template cudaError_t launch_pad<float>(const PadParams<float>&, cudaStream_t);
template cudaError_t launch_pad<double>(const PadParams<double>&, cudaStream_t);
template cudaError_t launch_crop<float>(const CropParams<float>&, cudaStream_t);
template cudaError_t launch_crop<double>(const CropParams<double>&, cudaStream_t);

}  // namespace gbn
