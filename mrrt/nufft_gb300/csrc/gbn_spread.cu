// Adjoint table interpolation (samples -> grid), tiled over the oversampled
// grid.  Replaces the reference's scatters (serial per coil on the CPU,
// mrrt/nufft/_extensions/c/nufft_table.template.c:144-531, 924-1206; global
// atomicAdd per tap on the GPU, mrrt/nufft/cuda/jinja/table_*_adjoint.jinja)
// with an "owner computes" decomposition:
//
// * a CTA owns one grid tile and one chunk of LS coils; it accumulates, in
//   shared memory, the contributions that land in ITS tile from every sample
//   whose window touches the tile (the planner lists halo samples in each
//   tile they reach);
// * each grid cell is then written exactly once, with conj(phase_before)
//   applied -- no global atomics and no zero-fill of the grid;
// * tiles too heavy for one CTA are split into parts whose partial tiles go
//   to a scratch buffer and are summed in a fixed order by reduce_kernel.
#include <cuda_runtime.h>

#include "gbn_device.cuh"
#include "gbn_internal.h"

namespace gbn {

constexpr int SPREAD_THREADS = 256;

// ---------------------------------------------------------------------------
// adjoint spread (owner computes)
// ---------------------------------------------------------------------------
template <typename R, int NDIM, bool CX>
__global__ void __launch_bounds__(SPREAD_THREADS)
spread_kernel(const SpreadParams<R> p) {
    typedef typename Cx<R>::T C;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    R* A = reinterpret_cast<R*>(smem_raw);
    const Geom<R>& g = p.g;

    const int4 it = p.items[blockIdx.x];
    const int2 part = p.parts[blockIdx.x];
    const int f = it.x, tile = it.y, start = it.z, count = it.w;
    const int LS = p.ln.LS, lsh = p.ln.lsh;
    const int CS = 2 * LS + 1;  // floats per cell: re[LS], im[LS], pad
    const int c0 = blockIdx.y << lsh;
    const int nc = min(LS, p.coils - c0);

    int org[3] = {0, 0, 0}, ext[3] = {1, 1, 1}, Td[3] = {1, 1, 1};
    tile_origin<NDIM>(tile, g.nt, g.T, org);
#pragma unroll
    for (int d = 0; d < NDIM; ++d) {
        Td[d] = g.T[d];
        ext[d] = min(g.T[d], g.K[d] - org[d]);
    }
    const int TT = Td[0] * Td[1] * Td[2];

    for (int q = threadIdx.x; q < TT * CS; q += blockDim.x) A[q] = (R)0;
    __syncthreads();

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nwarps = blockDim.x >> 5;
    const int SW = 32 >> lsh;
    const int slot = lane >> lsh, coil = lane & (LS - 1);
    const int64_t fo = p.foff[f];
    const int Mf = (int)(p.foff[f + 1] - fo);
    const C* yb = p.y + fo * p.coils + (int64_t)(c0 + min(coil, nc - 1)) * Mf;

    for (int i0 = warp * SW; i0 < count; i0 += nwarps * SW) {
        const int i = i0 + slot;
        if (i >= count || coil >= nc) continue;
        const int e = start + i;
        C v = yb[p.s.idx[e]];
        if (p.apply_ph) v = cmulc(v, p.s.ph[e]);
        R t[3];
        int kf[3];
#pragma unroll
        for (int d = 0; d < NDIM; ++d) {
            t[d] = p.s.t[d][e];
            kf[d] = first_tap(t[d], g.J[d]);
        }
        R cr[NDIM][JMAX], ci[NDIM][JMAX];
        int lr[NDIM][JMAX];
#pragma unroll
        for (int d = 0; d < NDIM; ++d) {
#pragma unroll
            for (int j = 0; j < JMAX; ++j) {
                lr[d][j] = -1;
                cr[d][j] = (R)0;
                ci[d][j] = (R)0;
                if (j < g.J[d]) {
                    const int l = wrapk(kf[d] + j, g.K[d]) - org[d];
                    if (l >= 0 && l < ext[d]) {
                        lr[d][j] = l;
                        table_coef<R, CX>(g, d, t[d], kf[d] + j, cr[d][j], ci[d][j]);
                    }
                }
            }
        }
        if (NDIM == 1) {
#pragma unroll
            for (int j0 = 0; j0 < JMAX; ++j0) {
                if (lr[0][j0] >= 0) {
                    const C w = cscale_conj<CX>(cr[0][j0], ci[0][j0], v);
                    R* a = A + lr[0][j0] * CS + coil;
                    atomicAdd(a, w.x);
                    atomicAdd(a + LS, w.y);
                }
            }
        } else if (NDIM == 2) {
#pragma unroll
            for (int j1 = 0; j1 < JMAX; ++j1) {
                if (lr[NDIM > 1 ? 1 : 0][j1] >= 0) {
                    const C v1 = cscale_conj<CX>(cr[NDIM > 1 ? 1 : 0][j1], ci[NDIM > 1 ? 1 : 0][j1], v);
                    const int rowc = lr[NDIM > 1 ? 1 : 0][j1] * Td[0];
#pragma unroll
                    for (int j0 = 0; j0 < JMAX; ++j0) {
                        if (lr[0][j0] >= 0) {
                            const C w = cscale_conj<CX>(cr[0][j0], ci[0][j0], v1);
                            R* a = A + (rowc + lr[0][j0]) * CS + coil;
                            atomicAdd(a, w.x);
                            atomicAdd(a + LS, w.y);
                        }
                    }
                }
            }
        } else {
#pragma unroll 1
            for (int j2 = 0; j2 < JMAX; ++j2) {
                if (lr[NDIM > 2 ? 2 : 0][j2] >= 0) {
                    const C v2 = cscale_conj<CX>(cr[NDIM > 2 ? 2 : 0][j2], ci[NDIM > 2 ? 2 : 0][j2], v);
                    const int pc = lr[NDIM > 2 ? 2 : 0][j2] * Td[1];
#pragma unroll
                    for (int j1 = 0; j1 < JMAX; ++j1) {
                        if (lr[NDIM > 1 ? 1 : 0][j1] >= 0) {
                            const C v1 = cscale_conj<CX>(cr[NDIM > 1 ? 1 : 0][j1], ci[NDIM > 1 ? 1 : 0][j1], v2);
                            const int rowc = (pc + lr[NDIM > 1 ? 1 : 0][j1]) * Td[0];
#pragma unroll
                            for (int j0 = 0; j0 < JMAX; ++j0) {
                                if (lr[0][j0] >= 0) {
                                    const C w = cscale_conj<CX>(cr[0][j0], ci[0][j0], v1);
                                    R* a = A + (rowc + lr[0][j0]) * CS + coil;
                                    atomicAdd(a, w.x);
                                    atomicAdd(a + LS, w.y);
                                }
                            }
                        }
                    }
                }
            }
        }
    }
    __syncthreads();

    // ---- flush: each owned cell written once ------------------------------
    const int slot_id = part.x;
    for (int q = threadIdx.x; q < TT * nc; q += blockDim.x) {
        const int c = q / TT;
        const int cell = q - c * TT;
        int r[3];
        r[0] = cell % Td[0];
        r[1] = (cell / Td[0]) % Td[1];
        r[2] = cell / (Td[0] * Td[1]);
        bool inside = true;
#pragma unroll
        for (int d = 0; d < NDIM; ++d) inside = inside && (r[d] < ext[d]);
        if (!inside) continue;
        C val = cmake<R>(A[cell * CS + c], A[cell * CS + LS + c]);
        if (slot_id < 0) {
            int k[3] = {0, 0, 0};
            int64_t off = 0, stride = 1;
#pragma unroll
            for (int d = 0; d < NDIM; ++d) {
                k[d] = org[d] + r[d];
                off += (int64_t)k[d] * stride;
                stride *= g.K[d];
            }
            if (p.apply_pb) val = cmulc(val, phase_before(g, k));
            p.grid[((int64_t)f * p.coils + c0 + c) * g.Kprod + off] = val;
        } else {
            p.scratch[(((int64_t)slot_id * gridDim.y + blockIdx.y) * LS + c) * p.tile_cells + cell] = val;
        }
    }
}

// Sum the parts of split tiles in part order and write the grid.
template <typename R, int NDIM>
__global__ void __launch_bounds__(256) reduce_kernel(const ReduceParams<R> p) {
    typedef typename Cx<R>::T C;
    const Geom<R>& g = p.g;
    const int4 tl = p.tiles[blockIdx.x];
    const int f = tl.x, tile = tl.y, slot0 = tl.z, nparts = tl.w;
    const int LS = p.ln.LS, lsh = p.ln.lsh;
    const int c0 = blockIdx.y << lsh;
    const int nc = min(LS, p.coils - c0);
    int org[3] = {0, 0, 0}, ext[3] = {1, 1, 1}, Td[3] = {1, 1, 1};
    tile_origin<NDIM>(tile, g.nt, g.T, org);
#pragma unroll
    for (int d = 0; d < NDIM; ++d) {
        Td[d] = g.T[d];
        ext[d] = min(g.T[d], g.K[d] - org[d]);
    }
    const int TT = Td[0] * Td[1] * Td[2];
    for (int q = threadIdx.x; q < TT * nc; q += blockDim.x) {
        const int c = q / TT;
        const int cell = q - c * TT;
        int r[3];
        r[0] = cell % Td[0];
        r[1] = (cell / Td[0]) % Td[1];
        r[2] = cell / (Td[0] * Td[1]);
        bool inside = true;
#pragma unroll
        for (int d = 0; d < NDIM; ++d) inside = inside && (r[d] < ext[d]);
        if (!inside) continue;
        C acc = cmake<R>((R)0, (R)0);
        for (int s = 0; s < nparts; ++s) {
            const C v = p.scratch[(((int64_t)(slot0 + s) * gridDim.y + blockIdx.y) * LS + c) * p.tile_cells + cell];
            acc.x += v.x;
            acc.y += v.y;
        }
        int k[3] = {0, 0, 0};
        int64_t off = 0, stride = 1;
#pragma unroll
        for (int d = 0; d < NDIM; ++d) {
            k[d] = org[d] + r[d];
            off += (int64_t)k[d] * stride;
            stride *= g.K[d];
        }
        if (p.apply_pb) acc = cmulc(acc, phase_before(g, k));
        p.grid[((int64_t)f * p.coils + c0 + c) * g.Kprod + off] = acc;
    }
}

template <typename R>
size_t spread_smem(const Geom<R>& g, const Lanes& ln) {
    size_t cells = 1;
    for (int d = 0; d < g.ndim; ++d) cells *= (size_t)g.T[d];
    return cells * (size_t)(2 * ln.LS + 1) * sizeof(R);
}

template <typename K>
static cudaError_t ensure_smem(K kernel, size_t bytes) {
    if (bytes <= 48 * 1024) return cudaSuccess;
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

template <typename R, int NDIM, bool CX>
static cudaError_t spread_dispatch(const SpreadParams<R>& p, cudaStream_t s) {
    const size_t smem = spread_smem(p.g, p.ln);
    cudaError_t e = ensure_smem(spread_kernel<R, NDIM, CX>, smem);
    if (e != cudaSuccess) return e;
    dim3 grid(p.nitems, (p.coils + p.ln.LS - 1) / p.ln.LS);
    spread_kernel<R, NDIM, CX><<<grid, SPREAD_THREADS, smem, s>>>(p);
    return cudaGetLastError();
}

template <typename R>
cudaError_t launch_spread(const SpreadParams<R>& p, cudaStream_t s) {
    if (p.nitems == 0 || p.coils == 0) return cudaSuccess;
    const bool cx = p.g.hi[0] != nullptr;
    switch (p.g.ndim * 2 + (cx ? 1 : 0)) {
        case 2: return spread_dispatch<R, 1, false>(p, s);
        case 3: return spread_dispatch<R, 1, true>(p, s);
        case 4: return spread_dispatch<R, 2, false>(p, s);
        case 5: return spread_dispatch<R, 2, true>(p, s);
        case 6: return spread_dispatch<R, 3, false>(p, s);
        case 7: return spread_dispatch<R, 3, true>(p, s);
    }
    return cudaErrorInvalidValue;
}

template <typename R>
cudaError_t launch_reduce(const ReduceParams<R>& p, cudaStream_t s) {
    if (p.ntiles == 0 || p.coils == 0) return cudaSuccess;
    dim3 grid(p.ntiles, (p.coils + p.ln.LS - 1) / p.ln.LS);
    switch (p.g.ndim) {
        case 1: reduce_kernel<R, 1><<<grid, 256, 0, s>>>(p); break;
        case 2: reduce_kernel<R, 2><<<grid, 256, 0, s>>>(p); break;
        case 3: reduce_kernel<R, 3><<<grid, 256, 0, s>>>(p); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

template size_t spread_smem<float>(const Geom<float>&, const Lanes&);
template size_t spread_smem<double>(const Geom<double>&, const Lanes&);
template cudaError_t launch_spread<float>(const SpreadParams<float>&, cudaStream_t);
template cudaError_t launch_spread<double>(const SpreadParams<double>&, cudaStream_t);
template cudaError_t launch_reduce<float>(const ReduceParams<float>&, cudaStream_t);
template cudaError_t launch_reduce<double>(const ReduceParams<double>&, cudaStream_t);

}  // namespace gbn
