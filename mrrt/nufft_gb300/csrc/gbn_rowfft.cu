// Row passes of the 2-D and 3-D oversampled FFTs with the deapodisation,
// zero-pad and crop folded in.
//
// Forward (mrrt/nufft/_nufft.py:1325-1331, then the first axis of fftn): each
// image row x[plane][n2][n1][:N0] is multiplied by sn[n2][n1][:N0], taken as
// the first N0 of K0 values (the rest zero, never stored or read) and
// transformed along memory axis 0 into its grid row (offset plane * gsp +
// n2 * gs2 + n1 * gs1: the row-interleaved 2-D grid or the plane-major 3-D
// grid).  This replaces the pad kernel's write of the zero-padded planes and
// the row FFT's read of them.
// Inverse (the first axis of ifftn, then :1561-1572): each grid row the crop
// keeps (n1 < N1, n2 < N2) is transformed back and only its first N0 outputs
// are formed into the image, scaled by scale * sn: the row FFT's write and
// the crop's read of the transformed rows are gone.
//
// Same four-step split as the last-axis pass (gbn_colfft.cu), with a CTA
// owning TR whole rows: step A thread (row, n1) loads elements n1 + L1 n2 of
// its row (consecutive threads on consecutive elements), step B thread
// (row, k2) writes elements k2 + L2 k1.  The shared rows of the exchange are
// padded to L1 + 1 so that step B's reads across k2 hit distinct banks.
// Plain transforms only: the coil-map (SENSE) variants keep the pad / crop
// kernels around the cuFFT row pass.
#include <cuda_runtime.h>

#include <cstdint>

#include "gbn_device.cuh"
#include "gbn_fft.cuh"
#include "gbn_internal.h"

namespace gbn {

namespace {

// D3: rows of a 3-D image (N2 > 1; a separate instantiation keeps the 2-D
// kernel's row arithmetic to one division).
template <int L1, int L2, int TR, int SIGN, bool D3>
__global__ void __launch_bounds__(TR * L1) rowfft_kernel(const RowFftParams p) {
    constexpr int LP = L1 + 1;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2* sm = reinterpret_cast<float2*>(smem_raw);
    const int64_t rpp = D3 ? (int64_t)p.N1 * p.N2 : p.N1;   // rows per plane
    const int64_t rows = (int64_t)p.planes * rpp;
    const int64_t r0 = (int64_t)blockIdx.x * TR;
    const int64_t Nprod = rpp * p.N0;

    // step A: (row, n1), L2-point transforms of elements n1 + L1 n2
    {
        const int n1 = threadIdx.x % L1, rl = threadIdx.x / L1;
        const int64_t r = r0 + rl;
        float2 v[L2];
#pragma unroll
        for (int n2 = 0; n2 < L2; ++n2) v[n2] = make_float2(0.f, 0.f);
        if (r < rows) {
            const int64_t pl = r / rpp;
            const int rr = (int)(r - pl * rpp);   // image row within the plane
            if (SIGN < 0) {
                // image row times sn, zero past N0
                const int64_t xo = pl * Nprod + (int64_t)rr * p.N0;
                const float* s = p.sn + (int64_t)rr * p.N0;
#pragma unroll
                for (int n2 = 0; n2 < L2; ++n2) {
                    const int n = n1 + L1 * n2;
                    if (n < p.N0 && GBN_INB(p.check, xo + n < p.in_elems, CHK_IMAGE)) {
                        const float2 x = p.in[xo + n];
                        const float w = s[n];
                        v[n2] = make_float2(x.x * w, x.y * w);
                    }
                }
            } else {
                const int n2r = D3 ? rr / p.N1 : 0;
                const int64_t go = pl * p.gsp + (int64_t)n2r * p.gs2 + (int64_t)(rr - n2r * p.N1) * p.gs1;
#pragma unroll
                for (int n2 = 0; n2 < L2; ++n2) {
                    const int n = n1 + L1 * n2;
                    if (GBN_INB(p.check, go + n >= 0 && go + n < p.in_elems, CHK_GRID_READ)) v[n2] = p.in[go + n];
                }
            }
        }
        stockham<L2, 1, SIGN>(v);
#pragma unroll
        for (int k2 = 1; k2 < L2; ++k2) {
            float2 w = __ldg(p.tw + n1 * k2);   // n1 k2 < L
            if (SIGN > 0) w.y = -w.y;
            v[k2] = cmul(v[k2], w);
        }
#pragma unroll
        for (int k2 = 0; k2 < L2; ++k2) sm[(rl * L2 + k2) * LP + n1] = v[k2];
    }
    __syncthreads();
    // step B: (row, k2), L1-point transforms, elements k2 + L2 k1 out
    for (int q = threadIdx.x; q < TR * L2; q += TR * L1) {
        const int k2 = q % L2, rl = q / L2;
        const int64_t r = r0 + rl;
        float2 u[L1];
#pragma unroll
        for (int n1 = 0; n1 < L1; ++n1) u[n1] = sm[(rl * L2 + k2) * LP + n1];
        stockham<L1, 1, SIGN>(u);
        if (r >= rows) continue;
        const int64_t pl = r / rpp;
        const int rr = (int)(r - pl * rpp);
        if (SIGN < 0) {
            const int n2r = D3 ? rr / p.N1 : 0;
            const int64_t go = pl * p.gsp + (int64_t)n2r * p.gs2 + (int64_t)(rr - n2r * p.N1) * p.gs1;
#pragma unroll
            for (int k1 = 0; k1 < L1; ++k1) {
                const int k = k2 + L2 * k1;
                if (GBN_INB(p.check, go + k >= 0 && go + k < p.out_elems, CHK_GRID_WRITE)) p.out[go + k] = u[k1];
            }
        } else {
            // the crop: first N0 outputs, times scale, times sn
            const int64_t xo = pl * Nprod + (int64_t)rr * p.N0;
            const float* s = p.sn + (int64_t)rr * p.N0;
#pragma unroll
            for (int k1 = 0; k1 < L1; ++k1) {
                const int k = k2 + L2 * k1;
                if (k < p.N0 && GBN_INB(p.check, xo + k < p.out_elems, CHK_IMAGE)) {
                    float2 t = make_float2(u[k1].x * p.scale, u[k1].y * p.scale);
                    const float w = s[k];
                    t.x *= w;
                    t.y *= w;
                    p.out[xo + k] = t;
                }
            }
        }
    }
}

template <int L1, int L2, int TR>
cudaError_t rowfft_launch(const RowFftParams& p, int sign, cudaStream_t s) {
    const size_t smem = (size_t)TR * L2 * (L1 + 1) * sizeof(float2);
    const bool d3 = p.N2 > 1;
    const void* k = sign < 0 ? (d3 ? reinterpret_cast<const void*>(rowfft_kernel<L1, L2, TR, -1, true>)
                                   : reinterpret_cast<const void*>(rowfft_kernel<L1, L2, TR, -1, false>))
                             : (d3 ? reinterpret_cast<const void*>(rowfft_kernel<L1, L2, TR, 1, true>)
                                   : reinterpret_cast<const void*>(rowfft_kernel<L1, L2, TR, 1, false>));
    cudaError_t e = ensure_dynamic_smem(k, smem);
    if (e != cudaSuccess) return e;
    const int64_t ctas = ((int64_t)p.planes * p.N1 * p.N2 + TR - 1) / TR;
    if (ctas > INT32_MAX) return cudaErrorInvalidValue;
    if (sign < 0 && d3)
        rowfft_kernel<L1, L2, TR, -1, true><<<(unsigned)ctas, TR * L1, smem, s>>>(p);
    else if (sign < 0)
        rowfft_kernel<L1, L2, TR, -1, false><<<(unsigned)ctas, TR * L1, smem, s>>>(p);
    else if (d3)
        rowfft_kernel<L1, L2, TR, 1, true><<<(unsigned)ctas, TR * L1, smem, s>>>(p);
    else
        rowfft_kernel<L1, L2, TR, 1, false><<<(unsigned)ctas, TR * L1, smem, s>>>(p);
    return cudaGetLastError();
}

}  // namespace

bool rowfft_supported(int L) { return colfft_supported(L); }

// Rows per CTA and splits measured on a GB300 (pad + forward, inverse + crop):
//   512, 32 planes x 256 rows: 16 x 32 with 8 rows 16.3 + 18.0 us, 16 rows
//     18.2 + 20.7 us (cuFFT's row pass alone 13.3 us each way, plus the pad
//     or crop kernel);
//   384, 512 planes x 192 rows: 16 x 24 with 8 rows 99.7 + 110.1 us, 16 rows
//     100.2 + 117.5 us (cuFFT's row pass alone 161.5 us).
cudaError_t launch_rowfft(const RowFftParams& p, int sign, cudaStream_t s) {
    if (p.planes <= 0 || p.N1 <= 0 || p.N2 <= 0 || p.N0 <= 0 || p.N0 > p.L) return cudaErrorInvalidValue;
    switch (p.L) {
        case 64: return rowfft_launch<8, 8, 16>(p, sign, s);
        case 96: return rowfft_launch<8, 12, 16>(p, sign, s);
        case 128: return rowfft_launch<8, 16, 16>(p, sign, s);
        case 192: return rowfft_launch<16, 12, 16>(p, sign, s);
        case 256: return rowfft_launch<8, 32, 16>(p, sign, s);
        case 384: return rowfft_launch<16, 24, 8>(p, sign, s);
        case 512: return rowfft_launch<16, 32, 8>(p, sign, s);
        case 768: return rowfft_launch<32, 24, 8>(p, sign, s);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace gbn
