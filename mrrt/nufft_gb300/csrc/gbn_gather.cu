// Forward table interpolation (grid -> samples), tiled over the oversampled
// grid.  Replaces the reference's one-thread-per-sample gathers
// (mrrt/nufft/_extensions/c/nufft_table.template.c:43-141, 538-921 on the
// CPU; mrrt/nufft/cuda/jinja/table_{1,2,3}d_forward.jinja on the GPU) with
// the same per-tap arithmetic and a different work decomposition:
//
// * samples are pre-sorted by grid tile (host planner, gbn_plan.cu);
// * a CTA owns one work item (frame, tile, sample range) and one chunk of
//   LS coils; the lanes of a warp are (sample slot, coil), so a sample's
//   J^d coefficients are computed once and applied to LS coils;
// * the tile plus its (J-1)-cell halo is staged once in shared memory for
//   all LS coils, with phase_before and the orthonormal scale applied while
//   staging; every sample of the tile then reads its window from shared
//   memory.
#include <cuda_runtime.h>

#include "gbn_device.cuh"
#include "gbn_internal.h"

namespace gbn {

constexpr int GATHER_THREADS = 256;

// ---------------------------------------------------------------------------
// forward gather
// ---------------------------------------------------------------------------
template <typename R, int NDIM, bool CX>
__global__ void __launch_bounds__(GATHER_THREADS)
gather_kernel(const GatherParams<R> p) {
    typedef typename Cx<R>::T C;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C* S = reinterpret_cast<C*>(smem_raw);
    const Geom<R>& g = p.g;

    const int4 it = p.items[blockIdx.x];
    const int f = it.x, tile = it.y, start = it.z, count = it.w;
    const int LS = p.ln.LS, lsh = p.ln.lsh, LSP = p.ln.LSP, swz = p.ln.swz;
    const int c0 = blockIdx.y << lsh;
    const int nc = min(LS, p.coils - c0);

    int org[3] = {0, 0, 0};
    tile_origin<NDIM>(tile, g.nt, g.T, org);
    int Rd[3];
    const int Rtot = region_dims(g, NDIM, Rd);

    // ---- stage tile + halo for nc coils -----------------------------------
    const C* gb = p.grid + ((int64_t)f * p.coils + c0) * g.Kprod;
    for (int cell = threadIdx.x; cell < Rtot; cell += blockDim.x) {
        int r[3];
        int rem = cell;
        r[0] = rem % Rd[0];
        rem /= Rd[0];
        r[1] = rem % Rd[1];
        r[2] = rem / Rd[1];
        int k[3] = {0, 0, 0};
        int64_t off = 0, stride = 1;
#pragma unroll
        for (int d = 0; d < NDIM; ++d) {
            k[d] = wrapk(org[d] + r[d], g.K[d]);
            off += (int64_t)k[d] * stride;
            stride *= g.K[d];
        }
        C ph = cmake<R>((R)1, (R)0);
        if (p.apply_pb) ph = phase_before(g, k);
        C* dst = S + (int64_t)cell * LSP;
        const int sw = cell & swz;
        for (int c = 0; c < nc; ++c) {
            C v = gb[(int64_t)c * g.Kprod + off];
            if (p.apply_pb) v = cmul(v, ph);
            if (p.grid_scale != (R)1) {
                v.x = v.x / p.grid_scale;
                v.y = v.y / p.grid_scale;
            }
            dst[c ^ sw] = v;
        }
    }
    __syncthreads();

    // ---- per-sample gather from shared memory -----------------------------
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nwarps = blockDim.x >> 5;
    const int SW = 32 >> lsh;
    const int slot = lane >> lsh, coil = lane & (LS - 1);
    const int64_t fo = p.foff[f];
    const int Mf = (int)(p.foff[f + 1] - fo);
    C* yb = p.y + fo * p.coils + (int64_t)(c0 + coil) * Mf;

    for (int i0 = warp * SW; i0 < count; i0 += nwarps * SW) {
        const int i = i0 + slot;
        if (i >= count) continue;
        const int e = start + i;
        R t[3];
        int kf[3], loc[3];
#pragma unroll
        for (int d = 0; d < NDIM; ++d) {
            t[d] = p.s.t[d][e];
            kf[d] = first_tap(t[d], g.J[d]);
            loc[d] = wrapk(kf[d], g.K[d]) - org[d];
        }
        R cr[NDIM][JMAX], ci[NDIM][JMAX];
#pragma unroll
        for (int d = 0; d < NDIM; ++d) {
#pragma unroll
            for (int j = 0; j < JMAX; ++j) {
                if (j < g.J[d]) {
                    table_coef<R, CX>(g, d, t[d], kf[d] + j, cr[d][j], ci[d][j]);
                } else {
                    cr[d][j] = (R)0;
                    ci[d][j] = (R)0;
                }
            }
        }
        C acc = cmake<R>((R)0, (R)0);
        if (NDIM == 1) {
#pragma unroll
            for (int j0 = 0; j0 < JMAX; ++j0) {
                if (j0 < g.J[0]) {
                    const int cell = loc[0] + j0;
                    cfma<CX>(acc, cr[0][j0], ci[0][j0], S[(int64_t)cell * LSP + (coil ^ (cell & swz))]);
                }
            }
        } else if (NDIM == 2) {
#pragma unroll
            for (int j1 = 0; j1 < JMAX; ++j1) {
                if (j1 < g.J[1]) {
                    const int base = (loc[1] + j1) * Rd[0] + loc[0];
                    C row = cmake<R>((R)0, (R)0);
#pragma unroll
                    for (int j0 = 0; j0 < JMAX; ++j0) {
                        if (j0 < g.J[0]) {
                            const int cell = base + j0;
                            cfma<CX>(row, cr[0][j0], ci[0][j0],
                                     S[(int64_t)cell * LSP + (coil ^ (cell & swz))]);
                        }
                    }
                    cfma<CX>(acc, cr[NDIM > 1 ? 1 : 0][j1], ci[NDIM > 1 ? 1 : 0][j1], row);
                }
            }
        } else {
#pragma unroll 1
            for (int j2 = 0; j2 < JMAX; ++j2) {
                if (j2 < g.J[2]) {
                    C plane = cmake<R>((R)0, (R)0);
#pragma unroll
                    for (int j1 = 0; j1 < JMAX; ++j1) {
                        if (j1 < g.J[1]) {
                            const int base = ((loc[2] + j2) * Rd[1] + loc[1] + j1) * Rd[0] + loc[0];
                            C row = cmake<R>((R)0, (R)0);
#pragma unroll
                            for (int j0 = 0; j0 < JMAX; ++j0) {
                                if (j0 < g.J[0]) {
                                    const int cell = base + j0;
                                    cfma<CX>(row, cr[0][j0], ci[0][j0],
                                             S[(int64_t)cell * LSP + (coil ^ (cell & swz))]);
                                }
                            }
                            cfma<CX>(plane, cr[NDIM > 1 ? 1 : 0][j1], ci[NDIM > 1 ? 1 : 0][j1], row);
                        }
                    }
                    cfma<CX>(acc, cr[NDIM > 2 ? 2 : 0][j2], ci[NDIM > 2 ? 2 : 0][j2], plane);
                }
            }
        }
        if (coil < nc) {
            if (p.apply_ph) acc = cmul(acc, p.s.ph[e]);
            yb[p.s.idx[e]] = acc;
        }
    }
}

template <typename R>
size_t gather_smem(const Geom<R>& g, const Lanes& ln) {
    size_t cells = 1;
    for (int d = 0; d < g.ndim; ++d) cells *= (size_t)(g.T[d] + g.J[d] - 1);
    return cells * (size_t)ln.LSP * sizeof(typename Cx<R>::T);
}

template <typename K>
static cudaError_t ensure_smem(K kernel, size_t bytes) {
    if (bytes <= 48 * 1024) return cudaSuccess;
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

template <typename R, int NDIM, bool CX>
static cudaError_t gather_dispatch(const GatherParams<R>& p, cudaStream_t s) {
    const size_t smem = gather_smem(p.g, p.ln);
    cudaError_t e = ensure_smem(gather_kernel<R, NDIM, CX>, smem);
    if (e != cudaSuccess) return e;
    dim3 grid(p.nitems, (p.coils + p.ln.LS - 1) / p.ln.LS);
    gather_kernel<R, NDIM, CX><<<grid, GATHER_THREADS, smem, s>>>(p);
    return cudaGetLastError();
}

template <typename R>
cudaError_t launch_gather(const GatherParams<R>& p, cudaStream_t s) {
    if (p.nitems == 0 || p.coils == 0) return cudaSuccess;
    const bool cx = p.g.hi[0] != nullptr;
    switch (p.g.ndim * 2 + (cx ? 1 : 0)) {
        case 2: return gather_dispatch<R, 1, false>(p, s);
        case 3: return gather_dispatch<R, 1, true>(p, s);
        case 4: return gather_dispatch<R, 2, false>(p, s);
        case 5: return gather_dispatch<R, 2, true>(p, s);
        case 6: return gather_dispatch<R, 3, false>(p, s);
        case 7: return gather_dispatch<R, 3, true>(p, s);
    }
    return cudaErrorInvalidValue;
}

template size_t gather_smem<float>(const Geom<float>&, const Lanes&);
template size_t gather_smem<double>(const Geom<double>&, const Lanes&);
template cudaError_t launch_gather<float>(const GatherParams<float>&, cudaStream_t);
template cudaError_t launch_gather<double>(const GatherParams<double>&, cudaStream_t);

}  // namespace gbn
