// Plan-time interpolation coefficients in list order.
//
// The coefficients of a sample depend only on its coordinates, which are
// fixed per plan, so the gather and spread kernels can read them instead of
// interpolating the lookup tables for every call: one coalesced read of
// jsum values per entry replaces 2 * jsum scattered table reads (the main
// L1 traffic of both kernels besides the staged grid values).  Table mode
// fills them with table_coef, the same device function the kernels use, so
// results are bitwise those of the table path.  Sparse-matrix mode fills
// them from the per-sample weights of the reference's precomputed
// interpolation matrix (mrrt/nufft/_nufft.py:750-877).
#include <cuda_runtime.h>

#include "gbn_device.cuh"
#include "gbn_internal.h"

namespace gbn {

template <typename R, bool CX>
__global__ void __launch_bounds__(256) coef_kernel(const CoefParams<R> p) {
    const int4 it = p.items[blockIdx.x];
    const int f = it.x, start = it.z, count = it.w;
    const Geom<R>& g = p.g;
    const int jsum = p.jsum;
    const int64_t fo = p.foff[f];
    for (int q = threadIdx.x; q < count * jsum; q += blockDim.x) {
        const int el = q / jsum;
        int j = q - el * jsum;
        int d = 0;
        while (d + 1 < g.ndim && j >= g.J[d]) {
            j -= g.J[d];
            ++d;
        }
        const int64_t e = start + el;
        R cr, ci = (R)0;
        if (p.wr[0]) {
            const int64_t w = (fo + p.s.idx[e]) * g.J[d] + j;
            cr = p.wr[d][w];
            if (CX) ci = p.wi[d][w];
        } else {
            const R t = p.s.t[d][e];
            table_coef<R, CX>(g, d, t, first_tap(t, g.J[d]) + j, cr, ci);
        }
        p.out_r[e * jsum + (q - el * jsum)] = cr;
        if (CX) p.out_i[e * jsum + (q - el * jsum)] = ci;
    }
}

template <typename R>
cudaError_t launch_coef(const CoefParams<R>& p, cudaStream_t s) {
    if (p.nitems == 0) return cudaSuccess;
    if (p.cx)
        coef_kernel<R, true><<<p.nitems, 256, 0, s>>>(p);
    else
        coef_kernel<R, false><<<p.nitems, 256, 0, s>>>(p);
    return cudaGetLastError();
}

template cudaError_t launch_coef<float>(const CoefParams<float>&, cudaStream_t);
template cudaError_t launch_coef<double>(const CoefParams<double>&, cudaStream_t);

}  // namespace gbn
