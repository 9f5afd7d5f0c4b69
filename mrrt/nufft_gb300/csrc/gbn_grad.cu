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
// One thread per sample; coils are summed inside the thread.  The kernel has
// no counterpart in the reference, which has no autograd.
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
    R t[3];
    int kf[3];
#pragma unroll
    for (int d = 0; d < NDIM; ++d) {
        t[d] = p.t[d][m];
        kf[d] = first_tap(t[d], g.J[d]);
    }
    R c[NDIM][JMAX], dc[NDIM][JMAX];
#pragma unroll
    for (int d = 0; d < NDIM; ++d) {
#pragma unroll
        for (int j = 0; j < JMAX; ++j) {
            c[d][j] = (R)0;
            dc[d][j] = (R)0;
            if (j < g.J[d]) {
                R ci;
                table_coef<R, false>(g, d, t[d], kf[d] + j, c[d][j], ci);
                const R pp = (t[d] - (R)(kf[d] + j)) * (R)g.L;
                const R nf = floor(pp);
                const int n = min(max((int)nf + g.ncenter[d], -2), g.J[d] * g.L + 1);
                const R alf = pp - nf;
                dc[d][j] = lerp_rn(alf, __ldg(p.dh[d] + n), __ldg(p.dh[d] + n + 1));
            }
        }
    }
    const C ph = p.ph ? p.ph[m] : cmake<R>((R)1, (R)0);
    R out[3] = {0, 0, 0};
    for (int cc = 0; cc < p.coils; ++cc) {
        const C* gb = p.grid + (int64_t)cc * g.gsp;
        C G = cmake<R>(0, 0), D[3] = {cmake<R>(0, 0), cmake<R>(0, 0), cmake<R>(0, 0)};
#pragma unroll 1
        for (int j2 = 0; j2 < (NDIM > 2 ? JMAX : 1); ++j2) {
            if (NDIM > 2 && j2 >= g.J[2]) continue;
#pragma unroll 1
            for (int j1 = 0; j1 < (NDIM > 1 ? JMAX : 1); ++j1) {
                if (NDIM > 1 && j1 >= g.J[1]) continue;
                C rc = cmake<R>(0, 0), rd = cmake<R>(0, 0);
#pragma unroll
                for (int j0 = 0; j0 < JMAX; ++j0) {
                    if (j0 >= g.J[0]) continue;
                    int k[3] = {0, 0, 0};
                    k[0] = wrapk(kf[0] + j0, g.K[0]);
                    if (NDIM > 1) k[1] = wrapk(kf[NDIM > 1 ? 1 : 0] + j1, g.K[1]);
                    if (NDIM > 2) k[2] = wrapk(kf[NDIM > 2 ? 2 : 0] + j2, g.K[2]);
                    const int64_t off = k[0] + (int64_t)k[1] * g.gs1 + (int64_t)k[2] * g.gs2;
                    C v = gb[off];
                    if (p.apply_pb) v = cmul(v, phase_before(g, k));
                    v.x /= p.grid_scale;
                    v.y /= p.grid_scale;
                    rc.x += c[0][j0] * v.x;
                    rc.y += c[0][j0] * v.y;
                    rd.x += dc[0][j0] * v.x;
                    rd.y += dc[0][j0] * v.y;
                }
                R w1 = (R)1, dw1 = (R)0;
                if (NDIM > 1) {
                    w1 = c[NDIM > 1 ? 1 : 0][j1];
                    dw1 = dc[NDIM > 1 ? 1 : 0][j1];
                }
                R w2 = (R)1, dw2 = (R)0;
                if (NDIM > 2) {
                    w2 = c[NDIM > 2 ? 2 : 0][j2];
                    dw2 = dc[NDIM > 2 ? 2 : 0][j2];
                }
                const R a = w1 * w2;
                G.x += a * rc.x;
                G.y += a * rc.y;
                D[0].x += a * rd.x;
                D[0].y += a * rd.y;
                if (NDIM > 1) {
                    D[1].x += dw1 * w2 * rc.x;
                    D[1].y += dw1 * w2 * rc.y;
                }
                if (NDIM > 2) {
                    D[2].x += w1 * dw2 * rc.x;
                    D[2].y += w1 * dw2 * rc.y;
                }
            }
        }
        const C gy = p.gy[(int64_t)cc * p.M + p.idx[m]];
        const C y = cmul(ph, G);
        // Re(conj(gy) * i * y) = Re(gy) * (-Im y) + Im(gy) * Re(y)
        const R ry = -gy.x * y.y + gy.y * y.x;
#pragma unroll
        for (int d = 0; d < NDIM; ++d) {
            const C dd = cmul(ph, D[d]);
            out[d] += gy.x * dd.x + gy.y * dd.y + p.phase_shift[d] * ry;
        }
    }
#pragma unroll
    for (int d = 0; d < NDIM; ++d) p.gtm[(int64_t)p.idx[m] * NDIM + d] = out[d];
}

template <typename R>
cudaError_t launch_grad(const GradParams<R>& p, cudaStream_t s) {
    if (p.M == 0) return cudaSuccess;
    const unsigned blocks = (unsigned)((p.M + 127) / 128);
    switch (p.g.ndim) {
        case 1: grad_kernel<R, 1><<<blocks, 128, 0, s>>>(p); break;
        case 2: grad_kernel<R, 2><<<blocks, 128, 0, s>>>(p); break;
        case 3: grad_kernel<R, 3><<<blocks, 128, 0, s>>>(p); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

template cudaError_t launch_grad<float>(const GradParams<float>&, cudaStream_t);
template cudaError_t launch_grad<double>(const GradParams<double>&, cudaStream_t);

}  // namespace gbn
