// Device helpers shared by the NUFFT kernels.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

#include "gbn_internal.h"

// Checked builds (compiled with GBN_CHECKED, libgbnufft_checked.so): every
// global index the kernels form from plan data is tested against the extent
// of its buffer before the access.  A failed test sets a bit in the plan's
// status word (gbn_debug_check_status) and the access is skipped: nothing
// traps or faults.  In the normal build the test is the constant true.
#ifdef GBN_CHECKED
#define GBN_INB(word, cond, bit) ((cond) ? true : (atomicOr((word), (bit)), false))
#else
#define GBN_INB(word, cond, bit) true
#endif

namespace gbn {

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
// a * conj(b)
__device__ __forceinline__ float2 cmulc(float2 a, float2 b) {
    return make_float2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
__device__ __forceinline__ double2 cmulc(double2 a, double2 b) {
    return make_double2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}

template <typename R> __device__ __forceinline__ typename Cx<R>::T cmake(R re, R im);
template <> __device__ __forceinline__ float2 cmake<float>(float re, float im) {
    return make_float2(re, im);
}
template <> __device__ __forceinline__ double2 cmake<double>(double re, double im) {
    return make_double2(re, im);
}

__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ void sincos_r(float x, float* s, float* c) { sincosf(x, s, c); }
__device__ __forceinline__ void sincos_r(double x, double* s, double* c) { sincos(x, s, c); }

// k mod K for k in a few periods around [0, K).
__device__ __forceinline__ int wrapk(int k, int K) {
    int r = k % K;
    return r < 0 ? r + K : r;
}

// First tap of the window: 1 + floor(t - J/2), evaluated in double exactly as
// the reference C does (nufft_table.template.c:577-578).
template <typename R>
__device__ __forceinline__ int first_tap(R t, int J) {
    return 1 + (int)floor((double)t - 0.5 * (double)J);
}

// phase_before(k) = exp(i * sum_d c_d k_d) with every product and partial sum
// rounded in the working precision, summed in the reference's axis order
// (mrrt/nufft/_nufft.py:703-715).
template <typename R>
__device__ __forceinline__ typename Cx<R>::T phase_before(const Geom<R>& g, const int* k) {
    R ph[3];
#pragma unroll
    for (int d = 0; d < 3; ++d)
        ph[d] = d < g.ndim ? mul_rn(g.pbc[d], (R)k[d]) : (R)0;
    R s = ph[g.pbo[0]];
    for (int i = 1; i < g.ndim; ++i) s = add_rn(s, ph[g.pbo[i]]);
    R sn, cs;
    sincos_r(s, &sn, &cs);
    return cmake<R>(cs, sn);
}

// (1 - alf) h0 + alf h1 with both products and the sum rounded separately
// (no contraction into a fused multiply-add), as the reference's C
// evaluates it: the same bits wherever the compiler inlines it.
template <typename R>
__device__ __forceinline__ R lerp_rn(R alf, R h0, R h1) {
    return add_rn(mul_rn((R)1 - alf, h0), mul_rn(alf, h1));
}

// Linearly interpolated table coefficient for tap k of coordinate t
// (nufft_table.template.c:581-585):  p = (t - k) L, n = floor(p),
// coef = (1 - alf) h[n] + alf h[n + 1].  Tables are zero-padded by two
// entries on each side on the device, so the one-past-the-end read that
// occurs when t - J/2 is an integer stays in bounds.
template <typename R, bool CX>
__device__ __forceinline__ void table_coef(const Geom<R>& g, int d, R t, int k, R& cr, R& ci) {
    const R pp = (t - (R)k) * (R)g.L;
    const R nf = floor(pp);
    // the host bounds |t| so this index lies in [-1, J*L+1]; the clamp keeps
    // every read inside the zero-padded table regardless
    const int n = min(max((int)nf + g.ncenter[d], -2), g.J[d] * g.L + 1);
    const R alf = pp - nf;
    const R* h = g.hr[d];
    cr = lerp_rn(alf, __ldg(h + n), __ldg(h + n + 1));
    if (CX) {
        const R* hi = g.hi[d];
        ci = lerp_rn(alf, __ldg(hi + n), __ldg(hi + n + 1));
    } else {
        ci = (R)0;
    }
}

// Tile coordinates of a linear tile index (axis 0 fastest).
template <int NDIM>
__device__ __forceinline__ void tile_origin(int tile, const int* nt, const int* T, int* org) {
    int rem = tile;
#pragma unroll
    for (int d = 0; d < NDIM; ++d) {
        const int tc = rem % nt[d];
        rem /= nt[d];
        org[d] = tc * T[d];
    }
}

template <typename R>
__device__ __forceinline__ int region_dims(const Geom<R>& g, int ndim, int* Rd) {
    int tot = 1;
    for (int d = 0; d < 3; ++d) {
        Rd[d] = d < ndim ? g.T[d] + g.J[d] - 1 : 1;
        tot *= Rd[d];
    }
    return tot;
}

// Packed single-precision pairs (Blackwell f32x2 pipe): one instruction for
// two IEEE round-to-nearest operations, bitwise identical to two scalar
// fmaf / multiplications.
__device__ __forceinline__ float2 ffma2(float2 a, float2 b, float2 c) {
    unsigned long long ra, rb, rc, rd;
    asm("mov.b64 %0, {%1, %2};" : "=l"(ra) : "f"(a.x), "f"(a.y));
    asm("mov.b64 %0, {%1, %2};" : "=l"(rb) : "f"(b.x), "f"(b.y));
    asm("mov.b64 %0, {%1, %2};" : "=l"(rc) : "f"(c.x), "f"(c.y));
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(rd) : "l"(ra), "l"(rb), "l"(rc));
    float2 d;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(d.x), "=f"(d.y) : "l"(rd));
    return d;
}
__device__ __forceinline__ float2 fmul2(float2 a, float2 b) {
    unsigned long long ra, rb, rd;
    asm("mov.b64 %0, {%1, %2};" : "=l"(ra) : "f"(a.x), "f"(a.y));
    asm("mov.b64 %0, {%1, %2};" : "=l"(rb) : "f"(b.x), "f"(b.y));
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(rd) : "l"(ra), "l"(rb));
    float2 d;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(d.x), "=f"(d.y) : "l"(rd));
    return d;
}
// Asynchronous global -> shared copies (cp.async, cached in L1 and L2).
// BYTES is 4, 8 or 16; both addresses must be aligned to BYTES.
template <int BYTES>
__device__ __forceinline__ void cp_async(void* smem, const void* gmem) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2;" ::"r"(s), "l"(gmem), "n"(BYTES) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
// Wait until every copy this thread issued has landed (bounded by memory
// latency; no polling in this code).
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }


// Element-wise pair operations: a * b and a * b + c on (re, im) pairs.
__device__ __forceinline__ float2 pmul(float2 a, float2 b) { return fmul2(a, b); }
__device__ __forceinline__ double2 pmul(double2 a, double2 b) { return make_double2(a.x * b.x, a.y * b.y); }
__device__ __forceinline__ float2 pfma(float2 a, float2 b, float2 c) { return ffma2(a, b, c); }
__device__ __forceinline__ double2 pfma(double2 a, double2 b, double2 c) {
    return make_double2(fma(a.x, b.x, c.x), fma(a.y, b.y, c.y));
}


// acc += c * v with c given as a pair: (c, c) for a real kernel, the complex
// coefficient (Re c, Im c) otherwise.
template <bool CX, typename C>
__device__ __forceinline__ void qfma(C& acc, C c, C v) {
    if (CX) {
        acc.x += c.x * v.x;
        acc.y += c.x * v.y;
        acc.x -= c.y * v.y;
        acc.y += c.y * v.x;
    } else {
        acc = pfma(c, v, acc);
    }
}


// Work distribution of the persistent interpolation kernels.  tickets[0]
// hands out (work item, coil chunk) pairs in item order (items are sorted
// heaviest first); tickets[1] counts the CTAs that found no more work, and
// the last of them resets both to zero for the next launch (stream-ordered,
// so graph replays work too).  Nothing waits on another CTA.
__device__ __forceinline__ int next_ticket(int* tickets, int* slot) {
    if (threadIdx.x == 0) *slot = atomicAdd(&tickets[0], 1);
    __syncthreads();
    const int t = *slot;
    __syncthreads();   // every thread has its ticket before thread 0 takes the next
    return t;
}
__device__ __forceinline__ void retire_ctas(int* tickets) {
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(&tickets[1], 1) == (int)gridDim.x - 1) {
            tickets[0] = 0;
            tickets[1] = 0;
        }
    }
}

// Two adjacent complex values in one 16-byte store (single precision; the
// address must be 16-byte aligned).  Double precision stores them singly.
__device__ __forceinline__ void store_pair(float2* dst, float2 a, float2 b) {
    *reinterpret_cast<float4*>(dst) = make_float4(a.x, a.y, b.x, b.y);
}
__device__ __forceinline__ void store_pair(double2* dst, double2 a, double2 b) {
    dst[0] = a;
    dst[1] = b;
}

}  // namespace gbn
