// Exact direct NUDFT in double precision (the reference's dtft / dtft_adj,
// mrrt/nufft/_dtft.py:16-216), used to state the error of the fast
// transform and exported as the package's dtft / dtft_adj.
//
//   forward: y[r][m] = sum_n x[r][n] exp(-i sum_d omega[m][d] (n_d - s_d))
//   adjoint: x[r][n] = sum_m y[r][m] exp(+i sum_d omega[m][d] (n_d - s_d))
//
// Forward: one thread per sample; along memory axis 0 the phase factor is
// advanced by complex rotation and re-seeded with sincos at every row start,
// which keeps the error at the 1e-14 level for rows of a few hundred pixels.
// Adjoint: one thread per pixel, samples staged through shared memory,
// one sincos per (pixel, sample).
#include <cuda_runtime.h>

#include "gbn_internal.h"

namespace gbn {

constexpr int DTFT_REPS = 4;

__global__ void __launch_bounds__(128)
dtft_fwd_kernel(int ndim, int N0, int N1, int N2, double s0, double s1, double s2,
                const double* __restrict__ omega, int64_t M, const double2* __restrict__ x,
                double2* __restrict__ y, int reps, int r0) {
    const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= M) return;
    const double w0 = omega[m * ndim + 0];
    const double w1 = ndim > 1 ? omega[m * ndim + 1] : 0.0;
    const double w2 = ndim > 2 ? omega[m * ndim + 2] : 0.0;
    const int nr = min(DTFT_REPS, reps - r0);
    const int64_t Nprod = (int64_t)N0 * N1 * N2;
    double ar[DTFT_REPS], ai[DTFT_REPS];
#pragma unroll
    for (int r = 0; r < DTFT_REPS; ++r) ar[r] = ai[r] = 0.0;
    double rs, rc;
    sincos(-w0, &rs, &rc);
    for (int n2 = 0; n2 < N2; ++n2) {
        for (int n1 = 0; n1 < N1; ++n1) {
            double ps, pc;
            sincos(-(w0 * (0.0 - s0) + w1 * (n1 - s1) + w2 * (n2 - s2)), &ps, &pc);
            const int64_t rowoff = ((int64_t)n2 * N1 + n1) * N0;
            for (int n0 = 0; n0 < N0; ++n0) {
#pragma unroll
                for (int r = 0; r < DTFT_REPS; ++r) {
                    if (r < nr) {
                        const double2 v = x[(int64_t)(r0 + r) * Nprod + rowoff + n0];
                        ar[r] += v.x * pc - v.y * ps;
                        ai[r] += v.x * ps + v.y * pc;
                    }
                }
                const double npc = pc * rc - ps * rs;
                ps = ps * rc + pc * rs;
                pc = npc;
            }
        }
    }
    for (int r = 0; r < nr; ++r) y[(int64_t)(r0 + r) * M + m] = make_double2(ar[r], ai[r]);
}

__global__ void __launch_bounds__(128)
dtft_adj_kernel(int ndim, int N0, int N1, int N2, double s0, double s1, double s2,
                const double* __restrict__ omega, int64_t M, const double2* __restrict__ y,
                double2* __restrict__ x, int reps, int r0) {
    __shared__ double so[128 * 3];
    __shared__ double2 sy[128 * DTFT_REPS];
    const int64_t Nprod = (int64_t)N0 * N1 * N2;
    const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int n0 = 0, n1 = 0, n2 = 0;
    if (n < Nprod) {
        n0 = (int)(n % N0);
        n1 = (int)((n / N0) % N1);
        n2 = (int)(n / ((int64_t)N0 * N1));
    }
    const double d0 = n0 - s0, d1 = n1 - s1, d2 = n2 - s2;
    const int nr = min(DTFT_REPS, reps - r0);
    double ar[DTFT_REPS], ai[DTFT_REPS];
#pragma unroll
    for (int r = 0; r < DTFT_REPS; ++r) ar[r] = ai[r] = 0.0;
    for (int64_t base = 0; base < M; base += 128) {
        const int cnt = (int)min((int64_t)128, M - base);
        __syncthreads();
        if (threadIdx.x < cnt) {
            for (int d = 0; d < ndim; ++d) so[threadIdx.x * 3 + d] = omega[(base + threadIdx.x) * ndim + d];
            for (int r = 0; r < nr; ++r)
                sy[threadIdx.x * DTFT_REPS + r] = y[(int64_t)(r0 + r) * M + base + threadIdx.x];
        }
        __syncthreads();
        for (int j = 0; j < cnt; ++j) {
            double ph = so[j * 3] * d0;
            if (ndim > 1) ph += so[j * 3 + 1] * d1;
            if (ndim > 2) ph += so[j * 3 + 2] * d2;
            double s, c;
            sincos(ph, &s, &c);
#pragma unroll
            for (int r = 0; r < DTFT_REPS; ++r) {
                if (r < nr) {
                    const double2 v = sy[j * DTFT_REPS + r];
                    ar[r] += v.x * c - v.y * s;
                    ai[r] += v.x * s + v.y * c;
                }
            }
        }
    }
    if (n < Nprod)
        for (int r = 0; r < nr; ++r) x[(int64_t)(r0 + r) * Nprod + n] = make_double2(ar[r], ai[r]);
}

cudaError_t launch_dtft(bool adjoint, int ndim, const int* Nd, const double* n_shift,
                        const double* omega, int64_t M, const double2* in, double2* out,
                        int reps, cudaStream_t st) {
    const int N0 = Nd[0], N1 = ndim > 1 ? Nd[1] : 1, N2 = ndim > 2 ? Nd[2] : 1;
    const double s0 = n_shift[0], s1 = ndim > 1 ? n_shift[1] : 0.0, s2 = ndim > 2 ? n_shift[2] : 0.0;
    const int64_t Nprod = (int64_t)N0 * N1 * N2;
    for (int r0 = 0; r0 < reps; r0 += DTFT_REPS) {
        if (!adjoint) {
            if (M == 0) break;
            const int64_t blocks = (M + 127) / 128;
            dtft_fwd_kernel<<<(unsigned)blocks, 128, 0, st>>>(ndim, N0, N1, N2, s0, s1, s2, omega, M,
                                                              in, out, reps, r0);
        } else {
            const int64_t blocks = (Nprod + 127) / 128;
            dtft_adj_kernel<<<(unsigned)blocks, 128, 0, st>>>(ndim, N0, N1, N2, s0, s1, s2, omega, M,
                                                              in, out, reps, r0);
        }
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

}  // namespace gbn
