// In-register FFTs shared by the FFT pass kernels (gbn_colfft.cu,
// gbn_rowfft.cu): Stockham autosort transforms (Govindaraju et al., "High
// performance discrete Fourier transforms on graphics processors", SC 2008)
// of length N dividing 96, radix 4, 2 and 3 stages fully unrolled, and the
// four-step twiddle multiply.  Included by one translation unit each (the
// constant table is per unit).
#pragma once

#include <cuda_runtime.h>

#include "gbn_device.cuh"

namespace gbn {
namespace {

// exp(-2 pi i m / 96), m < 96: the roots of every register transform (its
// length divides 96).  cos and sin by their Taylor series on [-pi, pi]
// (30 terms, error far below float rounding), evaluated by the compiler.
constexpr double kPi = 3.14159265358979323846;
constexpr double reduce_angle(int m) { return 2 * kPi * m / 96 > kPi ? 2 * kPi * m / 96 - 2 * kPi : 2 * kPi * m / 96; }
constexpr double series_cos(double x) {
    double t = 1, s = 1;
    for (int k = 1; k < 30; ++k) {
        t *= -x * x / ((2.0 * k - 1) * (2.0 * k));
        s += t;
    }
    return s;
}
constexpr double series_sin(double x) {
    double t = x, s = x;
    for (int k = 1; k < 30; ++k) {
        t *= -x * x / ((2.0 * k) * (2.0 * k + 1));
        s += t;
    }
    return s;
}
#define GBN_ROOT(m) {(float)series_cos(reduce_angle(m)), (float)-series_sin(reduce_angle(m))}
#define GBN_ROOT4(m) GBN_ROOT(m), GBN_ROOT(m + 1), GBN_ROOT(m + 2), GBN_ROOT(m + 3)
#define GBN_ROOT16(m) GBN_ROOT4(m), GBN_ROOT4(m + 4), GBN_ROOT4(m + 8), GBN_ROOT4(m + 12)
__constant__ float2 c_root96[96] = {GBN_ROOT16(0), GBN_ROOT16(16), GBN_ROOT16(32),
                                    GBN_ROOT16(48), GBN_ROOT16(64), GBN_ROOT16(80)};
#undef GBN_ROOT16
#undef GBN_ROOT4
#undef GBN_ROOT

// Complex add and subtract as one packed f32x2 instruction each (the
// butterflies' adds are most of their work: 2-D 512-point pass 61 -> 57 us,
// 3-D 256-point 661 -> 554 us with the split below).
__device__ __forceinline__ unsigned long long pack2(float2 a) {
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a.x), "f"(a.y));
    return r;
}
__device__ __forceinline__ float2 unpack2(unsigned long long r) {
    float2 d;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(d.x), "=f"(d.y) : "l"(r));
    return d;
}
__device__ __forceinline__ float2 padd(float2 a, float2 b) {
    unsigned long long r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(pack2(a)), "l"(pack2(b)));
    return unpack2(r);
}
__device__ __forceinline__ float2 psub(float2 a, float2 b) {
    unsigned long long r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(pack2(a)), "l"(pack2(b)));
    return unpack2(r);
}
// multiply by i^(SIGN), i.e. -i forward, +i inverse
template <int SIGN>
__device__ __forceinline__ float2 mul_si(float2 a) { return SIGN < 0 ? make_float2(a.y, -a.x) : make_float2(-a.y, a.x); }

// v * (root m of 96, conjugated for the inverse); m is a compile-time value
// once the loops are unrolled, so the quarter turns cost no multiply.
template <int SIGN>
__device__ __forceinline__ float2 root_mul(float2 v, int m) {
    if (m == 0) return v;
    if (m == 48) return make_float2(-v.x, -v.y);
    if (m == 24) return mul_si<SIGN>(v);
    if (m == 72) return mul_si<-SIGN>(v);
    float2 w = c_root96[m];
    if (SIGN > 0) w.y = -w.y;
    return cmul(v, w);
}

template <int R, int SIGN>
__device__ __forceinline__ void butterfly(float2 (&v)[R]) {
    if constexpr (R == 2) {
        const float2 a = v[0];
        v[0] = padd(a, v[1]);
        v[1] = psub(a, v[1]);
    } else if constexpr (R == 4) {
        const float2 t0 = padd(v[0], v[2]), t1 = psub(v[0], v[2]);
        const float2 t2 = padd(v[1], v[3]), t3 = mul_si<SIGN>(psub(v[1], v[3]));
        v[0] = padd(t0, t2);
        v[2] = psub(t0, t2);
        v[1] = padd(t1, t3);
        v[3] = psub(t1, t3);
    } else {
        static_assert(R == 3, "radix 2, 3 or 4");
        // w = exp(SIGN 2 pi i / 3) = -1/2 + SIGN i sqrt(3)/2
        constexpr float h = 0.866025403784438646763723f;   // sqrt(3) / 2
        const float2 t = padd(v[1], v[2]);
        const float2 d = psub(v[1], v[2]);
        const float2 u = SIGN < 0 ? make_float2(h * d.y, -h * d.x) : make_float2(-h * d.y, h * d.x);
        const float2 m = make_float2(v[0].x - 0.5f * t.x, v[0].y - 0.5f * t.y);
        v[0] = padd(v[0], t);
        v[1] = padd(m, u);
        v[2] = psub(m, u);
    }
}

constexpr int stage_radix(int n) { return n % 4 == 0 ? 4 : (n % 2 == 0 ? 2 : 3); }

// In-register Stockham FFT of length N (N divides 96), stages of NS -> NS R.
template <int N, int NS, int SIGN>
__device__ __forceinline__ void stockham(float2 (&x)[N]) {
    if constexpr (NS < N) {
        constexpr int R = stage_radix(N / NS);
        constexpr int Q = N / R;
        static_assert(96 % (NS * R) == 0, "register transform lengths divide 96");
        float2 y[N];
#pragma unroll
        for (int j = 0; j < Q; ++j) {
            const int jm = j % NS;
            float2 v[R];
#pragma unroll
            for (int r = 0; r < R; ++r) v[r] = x[j + r * Q];
#pragma unroll
            for (int r = 1; r < R; ++r) v[r] = root_mul<SIGN>(v[r], jm * r * (96 / (NS * R)));
            butterfly<R, SIGN>(v);
            const int base = (j / NS) * NS * R + jm;
#pragma unroll
            for (int r = 0; r < R; ++r) y[base + r * NS] = v[r];
        }
#pragma unroll
        for (int i = 0; i < N; ++i) x[i] = y[i];
        stockham<N, NS * R, SIGN>(x);
    }
}

}  // namespace
}  // namespace gbn
