// Sample binning on the device (the planner's sort of samples by tile,
// without a trip through host memory).
//
// The host planner (gbn_plan.cu, build_lists) and these kernels build the
// same lists from the same coordinates:
//   * gather list: one entry per sample, sorted (stably) by the gather tile
//     of its first tap, chunks of at most GATHER_CHUNK samples per work item;
//   * spread list: one entry per (spread tile, periodic image of the window)
//     the sample's window touches, carrying the window start in tile
//     coordinates, sorted stably by tile; a tile's entries are one work item,
//     or several parts whose partial tiles are reduced in part order.
// Work items are ordered heaviest first.  The sorts are stable radix sorts
// keyed by (frame, tile), so entries of a tile are in sample order and the
// spread's summation order, hence its result, is the same in every run.
// (The host planner additionally reorders the entries of heavy 3-D tiles by
// a hash of the sample index for balance; the device lists keep sample
// order, which gives the same result up to float rounding.)
//
// The reference has no such step: its CPU kernels loop over samples and its
// CuPy kernels scatter with global atomics
// (mrrt/nufft/cuda/jinja/table_2d_adjoint.jinja); the coordinates it bins
// are tm = omega / gamma (mrrt/nufft/_nufft.py:338-342).
#include <cuda_runtime.h>

#include "gbn_device.cuh"
#include "gbn_internal.h"

namespace gbn {

namespace {

__device__ __forceinline__ int frame_of(const int64_t* foff, int F, int64_t m) {
    int lo = 0, hi = F;   // foff[lo] <= m < foff[hi]
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (foff[mid] <= m) lo = mid;
        else hi = mid;
    }
    return lo;
}

struct AxisHits {
    int n;
    int tile[JMAX];
    int ls[JMAX];
};

// distinct (tile, window start in tile coordinates) pairs of one axis, in
// tap order (as the host planner's axis_hits)
__device__ __forceinline__ void axis_hits(int kf, int J, int K, int T, AxisHits& h) {
    h.n = 0;
    for (int j = 0; j < J; ++j) {
        const int c = wrapk(kf + j, K);
        const int tl = c / T;
        const int ls = c - tl * T - j;
        bool seen = false;
        for (int q = 0; q < h.n; ++q) seen = seen || (h.tile[q] == tl && h.ls[q] == ls);
        if (!seen) {
            h.tile[h.n] = tl;
            h.ls[h.n] = ls;
            ++h.n;
        }
    }
}

// first taps of sample m; false (and taps of t = 0) for an invalid coordinate
template <typename R>
__device__ __forceinline__ bool sample_taps(const BinParams<R>& p, int64_t m, int* kf) {
    bool ok = true;
    for (int d = 0; d < p.ndim; ++d) {
        R t = p.tm[m * p.ndim + d];
        if (!(fabs((double)t) <= p.tm_limit)) {   // false for NaN as well
            ok = false;
            t = (R)0;
        }
        kf[d] = first_tap(t, p.J[d]);
    }
    return ok;
}

template <typename R>
__global__ void __launch_bounds__(256) bin_count_kernel(const BinParams<R> p) {
    const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= p.M) return;
    int kf[3] = {0, 0, 0};
    if (!sample_taps(p, m, kf)) atomicOr(p.err, 1);
    const int f = frame_of(p.foff, p.F, m);
    int lin = 0, mul = 1;
    int n = 1;
    for (int d = 0; d < p.ndim; ++d) {
        lin += (wrapk(kf[d], p.K[d]) / p.Tg[d]) * mul;
        mul *= p.ntg[d];
        AxisHits h;
        axis_hits(kf[d], p.J[d], p.K[d], p.Ts[d], h);
        n *= h.n;
    }
    p.gkey[m] = (unsigned)(f * p.ntiles_g + lin);
    p.gval[m] = (unsigned)m;
    p.ecount[m] = n;
}

template <typename R>
__global__ void __launch_bounds__(256) bin_emit_kernel(const BinParams<R> p) {
    const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= p.M) return;
    int kf[3] = {0, 0, 0};
    sample_taps(p, m, kf);
    const int f = frame_of(p.foff, p.F, m);
    AxisHits h[3];
    for (int d = 0; d < 3; ++d) {
        h[d].n = 1;
        h[d].tile[0] = 0;
        h[d].ls[0] = 0;
    }
    for (int d = 0; d < p.ndim; ++d) axis_hits(kf[d], p.J[d], p.K[d], p.Ts[d], h[d]);
    int e = p.eoff[m];
    for (int a2 = 0; a2 < h[2].n; ++a2)
        for (int a1 = 0; a1 < h[1].n; ++a1)
            for (int a0 = 0; a0 < h[0].n; ++a0) {
                const int lin = h[0].tile[a0] + p.nts[0] * (h[1].tile[a1] + p.nts[1] * h[2].tile[a2]);
                p.skey[e] = (unsigned)(f * p.ntiles_s + lin);
                p.sval[e] = (unsigned)e;
                p.em[e] = (int)m;
                p.els[e] = make_short4((short)h[0].ls[a0], (short)h[1].ls[a1], (short)h[2].ls[a2], 0);
                ++e;
            }
}

// Counts per bin of sorted keys: lanes holding the same key (a run of the
// sort) add once, through their lowest lane.
__global__ void __launch_bounds__(256) bin_hist_kernel(const unsigned* keys, int64_t n, int* counts) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned lane = threadIdx.x & 31;
    const bool ok = i < n;
    const unsigned k = ok ? keys[i] : 0xffffffffu;
    const unsigned peers = __match_any_sync(0xffffffffu, k);
    if (ok && (peers & ((1u << lane) - 1u)) == 0) atomicAdd(&counts[k], __popc(peers));
}

// parts per bin: gather chunks (none for an empty tile), spread parts (at
// least one: an empty tile still writes its zeros), split-tile slots
__global__ void __launch_bounds__(256) bin_parts_kernel(const ItemParams p) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b < p.nbins_g) p.gparts[b] = (p.gcnt[b] + p.gchunk - 1) / p.gchunk;
    if (b < p.nbins_s) {
        const int c = p.scnt[b];
        const int parts = max(1, (c + p.schunk - 1) / p.schunk);
        p.sparts[b] = parts;
        p.rslots[b] = parts > 1 ? parts : 0;
        p.rflag[b] = parts > 1 ? 1 : 0;
    }
}

__global__ void __launch_bounds__(256) bin_items_kernel(const ItemParams p) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b < p.nbins_g) {
        const int f = b / p.ntiles_g, tile = b - f * p.ntiles_g;
        const int g0 = p.gstart[b], gn = p.gcnt[b];
        int it = p.goff[b];
        for (int q = 0; q < gn; q += p.gchunk) {
            p.gitems[it] = make_int4(f, tile, g0 + q, min(p.gchunk, gn - q));
            p.gsize[it] = (unsigned)(p.gchunk - min(p.gchunk, gn - q));
            p.gorder[it] = (unsigned)it;
            ++it;
        }
    }
    if (b < p.nbins_s) {
        const int f = b / p.ntiles_s, tile = b - f * p.ntiles_s;
        const int s0 = p.sstart[b], sn = p.scnt[b];
        const int parts = p.sparts[b];
        const int it0 = p.soff[b];
        if (parts == 1) {
            p.sitems[it0] = make_int4(f, tile, s0, sn);
            p.sslot[it0] = make_int2(-1, 1);
            p.ssize[it0] = (unsigned)(p.schunk - sn);
            p.sorder[it0] = (unsigned)it0;
        } else {
            const int per = (sn + parts - 1) / parts;
            const int slot0 = p.slotoff[b];
            for (int q = 0; q < parts; ++q) {
                const int a = s0 + q * per;
                const int n = min(per, s0 + sn - a);
                p.sitems[it0 + q] = make_int4(f, tile, a, n);
                p.sslot[it0 + q] = make_int2(slot0 + q, parts);
                p.ssize[it0 + q] = (unsigned)(p.schunk - n);
                p.sorder[it0 + q] = (unsigned)(it0 + q);
            }
            p.rtiles[p.roff[b]] = make_int4(f, tile, slot0, parts);
        }
    }
}

template <typename T>
__global__ void __launch_bounds__(256) permute_kernel(const T* in, const unsigned* order, int64_t n, T* out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = in[order[i]];
}

template <typename R>
__global__ void __launch_bounds__(256) bin_pack_kernel(const PackParams<R> p) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.len) return;
    const unsigned e = p.order[i];
    const int64_t m = p.em ? (int64_t)p.em[e] : (int64_t)e;
    if (p.ls_out) p.ls_out[i] = p.els[e];
    if (p.ph_out) p.ph_out[i] = p.ph[m];
    for (int d = 0; d < p.ndim; ++d) p.t_out[d][i] = p.tm[m * p.ndim + d];
    const int f = frame_of(p.foff, p.F, m);
    p.idx_out[i] = (int)(m - p.foff[f]);
}

inline unsigned grid_for(int64_t n, int threads) { return (unsigned)((n + threads - 1) / threads); }

}  // namespace

template <typename R>
cudaError_t launch_bin_count(const BinParams<R>& p, cudaStream_t s) {
    if (p.M == 0) return cudaSuccess;
    bin_count_kernel<R><<<grid_for(p.M, 256), 256, 0, s>>>(p);
    return cudaGetLastError();
}

template <typename R>
cudaError_t launch_bin_emit(const BinParams<R>& p, cudaStream_t s) {
    if (p.M == 0) return cudaSuccess;
    bin_emit_kernel<R><<<grid_for(p.M, 256), 256, 0, s>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_bin_hist(const unsigned* keys, int64_t n, int* counts, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    bin_hist_kernel<<<grid_for(n, 256), 256, 0, s>>>(keys, n, counts);
    return cudaGetLastError();
}

cudaError_t launch_bin_parts(const ItemParams& p, cudaStream_t s) {
    const int nb = max(p.nbins_g, p.nbins_s);
    if (nb == 0) return cudaSuccess;
    bin_parts_kernel<<<grid_for(nb, 256), 256, 0, s>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_bin_items(const ItemParams& p, cudaStream_t s) {
    const int nb = max(p.nbins_g, p.nbins_s);
    if (nb == 0) return cudaSuccess;
    bin_items_kernel<<<grid_for(nb, 256), 256, 0, s>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_permute_int4(const int4* in, const unsigned* order, int64_t n, int4* out, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    permute_kernel<int4><<<grid_for(n, 256), 256, 0, s>>>(in, order, n, out);
    return cudaGetLastError();
}

cudaError_t launch_permute_int2(const int2* in, const unsigned* order, int64_t n, int2* out, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    permute_kernel<int2><<<grid_for(n, 256), 256, 0, s>>>(in, order, n, out);
    return cudaGetLastError();
}

template <typename R>
cudaError_t launch_bin_pack(const PackParams<R>& p, cudaStream_t s) {
    if (p.len == 0) return cudaSuccess;
    bin_pack_kernel<R><<<grid_for(p.len, 256), 256, 0, s>>>(p);
    return cudaGetLastError();
}

template cudaError_t launch_bin_count<float>(const BinParams<float>&, cudaStream_t);
template cudaError_t launch_bin_count<double>(const BinParams<double>&, cudaStream_t);
template cudaError_t launch_bin_emit<float>(const BinParams<float>&, cudaStream_t);
template cudaError_t launch_bin_emit<double>(const BinParams<double>&, cudaStream_t);
template cudaError_t launch_bin_pack<float>(const PackParams<float>&, cudaStream_t);
template cudaError_t launch_bin_pack<double>(const PackParams<double>&, cudaStream_t);

}  // namespace gbn
