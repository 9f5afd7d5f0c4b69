// Pruned FFT pass along a strided axis of the oversampled grid.
//
// The oversampled FFT (mrrt/nufft/_nufft.py:1330-1350 forward fftn of the
// zero-padded image, :1561-1572 adjoint ifftn before the crop) is done in
// passes.  Every pass but the first runs along a strided memory axis (axis 1
// in 2-D; axes 1 and 2 in 3-D): an [L][S] array -- S columns, row stride S
// -- transformed along L for every column, for a set of such arrays at two
// strides (planes; z-slabs within a plane).  Half of that axis is zero
// padding:
//   * forward, only the first nin = N_last rows hold data; rows past nin are
//     zero and are not read;
//   * inverse, only the first nout = N_last rows are used afterwards (the
//     crop reads them); the others are not written.
// cuFFT reads and writes all L rows; this pass moves 3/4 of that traffic.
//
// Algorithm: the four-step split L = L1 L2 of the Cooley-Tukey FFT,
//   X[k2 + L2 k1] = sum_n1 W_L1^(n1 k1) W_L^(n1 k2) sum_n2 x[n1 + L1 n2] W_L2^(n2 k2),
// with W_M = exp(-2 pi i / M) forward and its conjugate inverse.
//   step A: a thread per (column, n1) loads the L2 rows n1 + L1 n2 of its
//     column (16 or 8 adjacent columns per CTA: 128- or 64-byte row segments), transforms
//     them in registers, multiplies by W_L^(n1 k2) and stores to shared memory;
//   step B: a thread per (column, k2) reads its L1 values back, transforms
//     them in registers and stores rows k2 + L2 k1.
// The register transforms are Stockham autosort FFTs (Govindaraju et al.,
// "High performance discrete Fourier transforms on graphics processors",
// SC 2008), radix 4, 2 and 3 stages fully unrolled; their roots are compile-
// time constants in constant memory, the W_L^(n1 k2) twiddles a per-plan
// table computed on the host in double precision.  Single precision only;
// other lengths and double precision run the pass through cuFFT.
#include <cuda_runtime.h>

#include <cstdint>

#include "gbn_device.cuh"
#include "gbn_fft.cuh"
#include "gbn_internal.h"

namespace gbn {

namespace {

// Z: the arrays have a second stride (blockIdx.z; the 3-D axis-1 pass).  A
// separate instantiation: with the second term in every kernel the 2-D
// 512-point pass compiled to 86 instead of 80 registers, two 256-thread CTAs
// per SM instead of three, and ran 40% slower.
template <int L1, int L2, int CF_TC, int SIGN, bool Z>
__global__ void __launch_bounds__(CF_TC * L1) colfft_kernel(const ColFftParams p) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2* sm = reinterpret_cast<float2*>(smem_raw);
    const int64_t c0 = (int64_t)blockIdx.x * CF_TC;
    const int64_t pb = (int64_t)blockIdx.y * p.ps + (Z ? (int64_t)blockIdx.z * p.ps2 : 0);

    // step A: (column, n1), L2-point transforms of rows n1 + L1 n2
    {
        const int col = threadIdx.x % CF_TC, n1 = threadIdx.x / CF_TC;
        const int64_t c = c0 + col;
        float2 v[L2];
#pragma unroll
        for (int n2 = 0; n2 < L2; ++n2) {
            const int n = n1 + L1 * n2;
            const int64_t i = pb + (int64_t)n * p.S + c;
            v[n2] = make_float2(0.f, 0.f);
            if (n < p.nin && c < p.S && GBN_INB(p.check, i >= 0 && i < p.in_elems, CHK_GRID_READ)) v[n2] = p.in[i];
        }
        stockham<L2, 1, SIGN>(v);
#pragma unroll
        for (int k2 = 1; k2 < L2; ++k2) {
            float2 w = __ldg(p.tw + n1 * k2);   // n1 k2 < L
            if (SIGN > 0) w.y = -w.y;
            v[k2] = cmul(v[k2], w);
        }
#pragma unroll
        for (int k2 = 0; k2 < L2; ++k2) sm[(k2 * L1 + n1) * CF_TC + col] = v[k2];
    }
    __syncthreads();
    // step B: (column, k2), L1-point transforms, rows k2 + L2 k1 out
    for (int q = threadIdx.x; q < CF_TC * L2; q += CF_TC * L1) {
        const int col = q % CF_TC, k2 = q / CF_TC;
        const int64_t c = c0 + col;
        float2 u[L1];
#pragma unroll
        for (int n1 = 0; n1 < L1; ++n1) u[n1] = sm[(k2 * L1 + n1) * CF_TC + col];
        stockham<L1, 1, SIGN>(u);
#pragma unroll
        for (int k1 = 0; k1 < L1; ++k1) {
            const int k = k2 + L2 * k1;
            const int64_t i = pb + (int64_t)k * p.S + c;
            if (k < p.nout && c < p.S && GBN_INB(p.check, i >= 0 && i < p.out_elems, CHK_GRID_WRITE)) p.out[i] = u[k1];
        }
    }
}

// CF_TC columns per CTA: 16 (128-byte row segments), 8 for 32-point second
// stages (a 256-thread CTA, so that the 32-point transforms need no spills).
template <int L1, int L2, int CF_TC>
cudaError_t colfft_launch(const ColFftParams& p, int sign, cudaStream_t s) {
    constexpr int L = L1 * L2;
    const size_t smem = (size_t)CF_TC * L * sizeof(float2);
    const bool z = p.planes2 > 1;
    const void* k = sign < 0 ? (z ? reinterpret_cast<const void*>(colfft_kernel<L1, L2, CF_TC, -1, true>)
                                  : reinterpret_cast<const void*>(colfft_kernel<L1, L2, CF_TC, -1, false>))
                             : (z ? reinterpret_cast<const void*>(colfft_kernel<L1, L2, CF_TC, 1, true>)
                                  : reinterpret_cast<const void*>(colfft_kernel<L1, L2, CF_TC, 1, false>));
    cudaError_t e = ensure_dynamic_smem(k, smem);
    if (e != cudaSuccess) return e;
    const int64_t ctas = (p.S + CF_TC - 1) / CF_TC;
    if (ctas > INT32_MAX || p.planes > 65535 || p.planes2 > 65535) return cudaErrorInvalidValue;
    const dim3 grid((unsigned)ctas, (unsigned)p.planes, (unsigned)p.planes2);
    if (sign < 0 && z)
        colfft_kernel<L1, L2, CF_TC, -1, true><<<grid, CF_TC * L1, smem, s>>>(p);
    else if (sign < 0)
        colfft_kernel<L1, L2, CF_TC, -1, false><<<grid, CF_TC * L1, smem, s>>>(p);
    else if (z)
        colfft_kernel<L1, L2, CF_TC, 1, true><<<grid, CF_TC * L1, smem, s>>>(p);
    else
        colfft_kernel<L1, L2, CF_TC, 1, false><<<grid, CF_TC * L1, smem, s>>>(p);
    return cudaGetLastError();
}

}  // namespace

// Lengths with a compile-time split L1 x L2 (both dividing 96, at most 32)
// that measured faster than cuFFT.
bool colfft_supported(int L) {
    switch (L) {
        case 64: case 96: case 128: case 192: case 256: case 384: case 512: case 768:
            return true;
        default:
            return false;
    }
}

cudaError_t launch_colfft(const ColFftParams& p, int sign, cudaStream_t s) {
    if (p.S <= 0 || p.planes <= 0 || p.planes2 <= 0 || p.nin < 0 || p.nin > p.L || p.nout < 0 || p.nout > p.L)
        return cudaErrorInvalidValue;
    // Splits measured on a GB300 (forward + inverse, packed butterflies):
    //   512, 16384 columns: 16 x 32 with 16 columns per CTA 57 us, 32 x 16
    //     with 8 columns 58 us, cuFFT 62 us;
    //   384, 196608 columns: 16 x 24 321 us, 24 x 16 337 us, cuFFT 694 us;
    //   256, 8 planes of 65536 columns: 8 x 32 554 us, 16 x 16 662 us,
    //     cuFFT 808 us;
    //   128, 4 planes of 32768 columns: 8 x 16 73 us, 16 x 8 81 us, cuFFT 134 us;
    //   192: 16 x 12 116 us, 8 x 24 120 us, cuFFT 214 us; 768: 32 x 24 109 us,
    //     24 x 32 128 us, cuFFT 255 us.
    // 1024 (32 x 32, one CTA per SM at 242 registers) ran slower than cuFFT
    // (152 against about 139 us at 16384 columns) and is left to cuFFT.
    switch (p.L) {
        case 64: return colfft_launch<8, 8, 16>(p, sign, s);
        case 96: return colfft_launch<8, 12, 16>(p, sign, s);
        case 128: return colfft_launch<8, 16, 16>(p, sign, s);
        case 192: return colfft_launch<16, 12, 16>(p, sign, s);
        case 256: return colfft_launch<8, 32, 16>(p, sign, s);
        case 384: return colfft_launch<16, 24, 16>(p, sign, s);
        case 512: return colfft_launch<16, 32, 16>(p, sign, s);
        case 768: return colfft_launch<32, 24, 8>(p, sign, s);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace gbn
