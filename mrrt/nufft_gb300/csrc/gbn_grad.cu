// Gradient of a real loss L with respect to the sample coordinates tm.
//
// The forward output is y[m,c] = ph[m] * G[m,c] with
//   G[m,c] = sum_k w(t_m - k) g_c[k],  w(u) = prod_d h_d(u_d)
// where g_c is the oversampled grid after phase_before (and the orthonormal
// scale) and ph[m] = exp(i omega_m . s), s = n_shift - n_mid (real phasing,
// mrrt/nufft/_nufft.py:717-724).  With t_d = omega_d / gamma_d,
//   dy/dt_d = ph * sum_k h_d'(..) prod_{e != d} h_e(..) g_c[k]
//           + i s_d gamma_d y .
// h_d' is a table of the analytic derivative of the Kaiser-Bessel kernel on
// the same sample points as h_d, linearly interpolated the same way.  With
// torch's convention for the incoming gradient gy = dL/dRe(y) + i dL/dIm(y),
//   dL/dt_d = sum_c Re(conj(gy[m,c]) dy[m,c]/dt_d).
// One thread per sample (samples in gather-list order, so neighbouring
// threads read neighbouring grid taps); coils are summed inside the thread.
// phase_before is separable, so it is folded into the per-axis coefficients
// (J sincos per axis per sample instead of one per tap per coil).  The
// kernel has no counterpart in the reference, which has no autograd.
#include <cuda_runtime.h>

#include "gbn_device.cuh"
#include "gbn_internal.h"

namespace gbn {

template <typename R, int NDIM>
__global__ void __launch_bounds__(128) grad_kernel(const GradParams<R> p) {
    typedef typename Cx<R>::T C;
    const Geom<R>& g = p.g;
    const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= p.M) return;
    // Per axis and tap: the table coefficient and its derivative, each
    // times that axis's factor of phase_before.  phase_before(k) =
    // exp(i sum_d c_d k_d) is a product over axes, so the phases cost
    // J sincos per axis per sample instead of one per tap per coil.
    C cc[NDIM][JMAX], dd[NDIM][JMAX];
    int kf[3] = {0, 0, 0};
#pragma unroll
    for (int d = 0; d < NDIM; ++d) {
        const R t = p.t[d][m];
        kf[d] = first_tap(t, g.J[d]);
#pragma unroll
        for (int j = 0; j < JMAX; ++j) {
            cc[d][j] = cmake<R>((R)0, (R)0);
            dd[d][j] = cmake<R>((R)0, (R)0);
            if (j < g.J[d]) {
                R c, ci;
                table_coef<R, false>(g, d, t, kf[d] + j, c, ci);
                const R pp = (t - (R)(kf[d] + j)) * (R)g.L;
                const R nf = floor(pp);
                const int n = min(max((int)nf + g.ncenter[d], -2), g.J[d] * g.L + 1);
                const R dc = lerp_rn(pp - nf, __ldg(p.dh[d] + n), __ldg(p.dh[d] + n + 1));
                R sn = (R)0, cs = (R)1;
                if (p.apply_pb) sincos_r(mul_rn(g.pbc[d], (R)wrapk(kf[d] + j, g.K[d])), &sn, &cs);
                cc[d][j] = cmake<R>(c * cs, c * sn);
                dd[d][j] = cmake<R>(dc * cs, dc * sn);
            }
        }
    }
    const C ph = p.ph ? p.ph[m] : cmake<R>((R)1, (R)0);
    const R inv_scale = (R)1 / p.grid_scale;
    R out[3] = {0, 0, 0};
    constexpr int D1 = NDIM > 1 ? 1 : 0, D2 = NDIM > 2 ? 2 : 0;
    for (int co = 0; co < p.coils; ++co) {
        const C* gb = p.grid + (int64_t)co * g.gsp;
        C G = cmake<R>(0, 0), D[3] = {cmake<R>(0, 0), cmake<R>(0, 0), cmake<R>(0, 0)};
#pragma unroll 1
        for (int j2 = 0; j2 < (NDIM > 2 ? g.J[D2] : 1); ++j2) {
            C G1 = cmake<R>(0, 0), D10 = cmake<R>(0, 0), D11 = cmake<R>(0, 0);
            const int64_t o2 = NDIM > 2 ? (int64_t)wrapk(kf[D2] + j2, g.K[D2]) * g.gs2 : 0;
#pragma unroll 1
            for (int j1 = 0; j1 < (NDIM > 1 ? g.J[D1] : 1); ++j1) {
                const int64_t o1 = NDIM > 1 ? (int64_t)wrapk(kf[D1] + j1, g.K[D1]) * g.gs1 : 0;
                C r = cmake<R>(0, 0), rd = cmake<R>(0, 0);
#pragma unroll
                for (int j0 = 0; j0 < JMAX; ++j0) {
                    if (j0 >= g.J[0]) continue;
                    const C v = gb[wrapk(kf[0] + j0, g.K[0]) + o1 + o2];
                    r = cadd(r, cmul(cc[0][j0], v));
                    rd = cadd(rd, cmul(dd[0][j0], v));
                }
                if (NDIM > 1) {
                    const C w1 = cc[D1][j1], dw1 = dd[D1][j1];
                    G1 = cadd(G1, cmul(w1, r));
                    D10 = cadd(D10, cmul(w1, rd));
                    D11 = cadd(D11, cmul(dw1, r));
                } else {
                    G1 = r;
                    D10 = rd;
                }
            }
            if (NDIM > 2) {
                const C w2 = cc[D2][j2], dw2 = dd[D2][j2];
                G = cadd(G, cmul(w2, G1));
                D[0] = cadd(D[0], cmul(w2, D10));
                D[1] = cadd(D[1], cmul(w2, D11));
                D[2] = cadd(D[2], cmul(dw2, G1));
            } else {
                G = G1;
                D[0] = D10;
                D[1] = D11;
            }
        }
        const C gy = p.gy[(int64_t)co * p.M + p.idx[m]];
        const C y = cmul(ph, G);
        // Re(conj(gy) * i * y) = Re(gy) * (-Im y) + Im(gy) * Re(y)
        const R ry = (-gy.x * y.y + gy.y * y.x) * inv_scale;
#pragma unroll
        for (int d = 0; d < NDIM; ++d) {
            const C dv = cmul(ph, D[d]);
            out[d] += (gy.x * dv.x + gy.y * dv.y) * inv_scale + p.phase_shift[d] * ry;
        }
    }
#pragma unroll
    for (int d = 0; d < NDIM; ++d) p.gtm[(int64_t)p.idx[m] * NDIM + d] = out[d];
}

// 2-D: a group of 8 lanes per sample, lane j holding window row j (and the
// coefficients of tap j of both axes); the rows' partial sums are combined
// by three butterfly shuffles.  One thread per sample left most of the GPU
// idle on a 65,536-sample trajectory (19% of warp slots, long-scoreboard
// bound); the group gives 8 times the threads and a sixth of the serial taps.
template <typename R>
__global__ void __launch_bounds__(256) grad2d_group_kernel(const GradParams<R> p) {
    typedef typename Cx<R>::T C;
    const Geom<R>& g = p.g;
    const int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t m = gid >> 3;
    const int lane = threadIdx.x & 31;
    const int j = lane & 7;
    const int base = lane & ~7;
    const bool ok = m < p.M;
    const int64_t mm = ok ? m : 0;
    // tap j of each axis: coefficient and derivative times the axis's phase_before factor
    C cc[2], dd[2];
    int kf[2];
#pragma unroll
    for (int d = 0; d < 2; ++d) {
        const R t = p.t[d][mm];
        kf[d] = first_tap(t, g.J[d]);
        cc[d] = cmake<R>((R)0, (R)0);
        dd[d] = cmake<R>((R)0, (R)0);
        if (ok && j < g.J[d]) {
            R c, ci;
            table_coef<R, false>(g, d, t, kf[d] + j, c, ci);
            const R pp = (t - (R)(kf[d] + j)) * (R)g.L;
            const R nf = floor(pp);
            const int n = min(max((int)nf + g.ncenter[d], -2), g.J[d] * g.L + 1);
            const R dc = lerp_rn(pp - nf, __ldg(p.dh[d] + n), __ldg(p.dh[d] + n + 1));
            R sn = (R)0, cs = (R)1;
            if (p.apply_pb) sincos_r(mul_rn(g.pbc[d], (R)wrapk(kf[d] + j, g.K[d])), &sn, &cs);
            cc[d] = cmake<R>(c * cs, c * sn);
            dd[d] = cmake<R>(dc * cs, dc * sn);
        }
    }
    const bool row = ok && j < g.J[1];
    const int64_t o1 = (int64_t)wrapk(kf[1] + j, g.K[1]) * g.gs1;
    const C ph = (ok && p.ph) ? p.ph[mm] : cmake<R>((R)1, (R)0);
    const R inv_scale = (R)1 / p.grid_scale;
    R out[2] = {0, 0};
    for (int co = 0; co < p.coils; ++co) {
        const C* gb = p.grid + (int64_t)co * g.gsp;
        C r = cmake<R>(0, 0), rd = cmake<R>(0, 0);
        for (int j0 = 0; j0 < g.J[0]; ++j0) {
            C c0, d0;
            c0.x = __shfl_sync(0xffffffffu, cc[0].x, base + j0);
            c0.y = __shfl_sync(0xffffffffu, cc[0].y, base + j0);
            d0.x = __shfl_sync(0xffffffffu, dd[0].x, base + j0);
            d0.y = __shfl_sync(0xffffffffu, dd[0].y, base + j0);
            if (row) {
                const C v = gb[wrapk(kf[0] + j0, g.K[0]) + o1];
                r = cadd(r, cmul(c0, v));
                rd = cadd(rd, cmul(d0, v));
            }
        }
        // this row's contributions; rows j >= J1 contribute zero
        C G = cmul(cc[1], r), D0 = cmul(cc[1], rd), D1 = cmul(dd[1], r);
#pragma unroll
        for (int off = 1; off < 8; off <<= 1) {
            G.x += __shfl_xor_sync(0xffffffffu, G.x, off);
            G.y += __shfl_xor_sync(0xffffffffu, G.y, off);
            D0.x += __shfl_xor_sync(0xffffffffu, D0.x, off);
            D0.y += __shfl_xor_sync(0xffffffffu, D0.y, off);
            D1.x += __shfl_xor_sync(0xffffffffu, D1.x, off);
            D1.y += __shfl_xor_sync(0xffffffffu, D1.y, off);
        }
        if (ok && j == 0) {
            const C gy = p.gy[(int64_t)co * p.M + p.idx[mm]];
            const C y = cmul(ph, G);
            const R ry = (-gy.x * y.y + gy.y * y.x) * inv_scale;
            const C dv0 = cmul(ph, D0), dv1 = cmul(ph, D1);
            out[0] += (gy.x * dv0.x + gy.y * dv0.y) * inv_scale + p.phase_shift[0] * ry;
            out[1] += (gy.x * dv1.x + gy.y * dv1.y) * inv_scale + p.phase_shift[1] * ry;
        }
    }
    if (ok && j == 0) {
        p.gtm[(int64_t)p.idx[mm] * 2 + 0] = out[0];
        p.gtm[(int64_t)p.idx[mm] * 2 + 1] = out[1];
    }
}

template <typename R>
cudaError_t launch_grad(const GradParams<R>& p, cudaStream_t s) {
    if (p.M == 0) return cudaSuccess;
    const unsigned blocks = (unsigned)((p.M + 127) / 128);
    switch (p.g.ndim) {
        case 1: grad_kernel<R, 1><<<blocks, 128, 0, s>>>(p); break;
        case 2:
            grad2d_group_kernel<R><<<(unsigned)((p.M * 8 + 255) / 256), 256, 0, s>>>(p);
            break;
        case 3: grad_kernel<R, 3><<<blocks, 128, 0, s>>>(p); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

template cudaError_t launch_grad<float>(const GradParams<float>&, cudaStream_t);
template cudaError_t launch_grad<double>(const GradParams<double>&, cudaStream_t);

}  // namespace gbn
