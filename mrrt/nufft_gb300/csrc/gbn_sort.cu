// Device-side scan and stable radix sort used by the sample binning
// (gbn_bin.cu).  Written for this project (no CUB): a three-kernel
// exclusive scan and an LSD radix sort with 8-bit digits whose scatter ranks
// equal keys in input order, so the sort is stable and its output is the
// same in every run.
#include <cuda_runtime.h>

#include "gbn_sort.cuh"

namespace gbn {

namespace {

constexpr int SCAN_THREADS = 512;
constexpr int SCAN_PER_THREAD = 4;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_PER_THREAD;   // 2048 elements per CTA

constexpr int RADIX_THREADS = 256;
constexpr int RADIX_WARPS = RADIX_THREADS / 32;
constexpr int RADIX_BUCKETS = 256;
// Items per lane: 16 (4096 items per CTA) for large sorts; 2 (512 per CTA)
// below RADIX_SMALL items, where 4096-item tiles would leave most SMs idle.
constexpr int RADIX_ROUNDS_LARGE = 16, RADIX_ROUNDS_SMALL = 2;
constexpr int64_t RADIX_SMALL = 1 << 20;
inline int radix_rounds(int64_t n) { return n < RADIX_SMALL ? RADIX_ROUNDS_SMALL : RADIX_ROUNDS_LARGE; }

inline size_t round256(size_t v) { return (v + 255) & ~(size_t)255; }

// Exclusive scan of a CTA's values held one per thread; *out_total gets the
// CTA total.
__device__ __forceinline__ int block_exclusive_scan(int v, int* warp_sums, int* out_total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        const int nw = blockDim.x >> 5;
        int w = lane < nw ? warp_sums[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < nw) warp_sums[lane] = w;   // inclusive
    }
    __syncthreads();
    const int before = warp > 0 ? warp_sums[warp - 1] : 0;
    *out_total = warp_sums[(blockDim.x >> 5) - 1];
    return before + x - v;
}

__global__ void __launch_bounds__(SCAN_THREADS) scan_tile_kernel(const int* in, int* out, int64_t n, int* bsum) {
    __shared__ int ws[32];
    const int64_t base = (int64_t)blockIdx.x * SCAN_TILE + (int64_t)threadIdx.x * SCAN_PER_THREAD;
    int v[SCAN_PER_THREAD];
    int s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_PER_THREAD; ++k) {
        v[k] = base + k < n ? in[base + k] : 0;
        s += v[k];
    }
    int total;
    int run = block_exclusive_scan(s, ws, &total);
#pragma unroll
    for (int k = 0; k < SCAN_PER_THREAD; ++k) {
        if (base + k < n) out[base + k] = run;
        run += v[k];
    }
    if (threadIdx.x == 0 && bsum) bsum[blockIdx.x] = total;
}

__global__ void __launch_bounds__(SCAN_THREADS) scan_add_kernel(int* out, int64_t n, const int* boff) {
    const int64_t base = (int64_t)blockIdx.x * SCAN_TILE + (int64_t)threadIdx.x * SCAN_PER_THREAD;
    const int add = boff[blockIdx.x];
#pragma unroll
    for (int k = 0; k < SCAN_PER_THREAD; ++k)
        if (base + k < n) out[base + k] += add;
}

__global__ void scan_total_kernel(const int* in, const int* out, int64_t n, int* total) {
    *total = n > 0 ? out[n - 1] + in[n - 1] : 0;
}

__device__ __forceinline__ int digit_of(unsigned key, int shift) { return (int)((key >> shift) & 0xffu); }

template <int RADIX_ROUNDS>
__global__ void __launch_bounds__(RADIX_THREADS) radix_hist_kernel(const unsigned* keys, int64_t n, int shift,
                                                                   int nblk, int* hist) {
    constexpr int RADIX_TILE = RADIX_THREADS * RADIX_ROUNDS;
    __shared__ int h[RADIX_BUCKETS];
    for (int q = threadIdx.x; q < RADIX_BUCKETS; q += blockDim.x) h[q] = 0;
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t base = (int64_t)blockIdx.x * RADIX_TILE + (int64_t)warp * (32 * RADIX_ROUNDS) + lane;
#pragma unroll 4
    for (int r = 0; r < RADIX_ROUNDS; ++r) {
        const int64_t i = base + r * 32;
        if (i < n) atomicAdd(&h[digit_of(keys[i], shift)], 1);
    }
    __syncthreads();
    // digit-major: the scan of hist gives, for digit d and CTA b, the output
    // position of the CTA's first item with digit d
    for (int q = threadIdx.x; q < RADIX_BUCKETS; q += blockDim.x) hist[(int64_t)q * nblk + blockIdx.x] = h[q];
}

// Items of a CTA in index order are (warp, round, lane); each lands after
// every earlier item with the same digit, so the pass is stable.
template <int RADIX_ROUNDS>
__global__ void __launch_bounds__(RADIX_THREADS) radix_scatter_kernel(const unsigned* keys, const unsigned* vals,
                                                                      int64_t n, int shift, int nblk,
                                                                      const int* offs, unsigned* keys_out,
                                                                      unsigned* vals_out) {
    constexpr int RADIX_TILE = RADIX_THREADS * RADIX_ROUNDS;
    __shared__ int wh[RADIX_WARPS][RADIX_BUCKETS];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int q = lane; q < RADIX_BUCKETS; q += 32) wh[warp][q] = 0;
    __syncwarp();
    const int64_t base = (int64_t)blockIdx.x * RADIX_TILE + (int64_t)warp * (32 * RADIX_ROUNDS) + lane;
    const unsigned lt = (1u << lane) - 1u;
    unsigned k[RADIX_ROUNDS], v[RADIX_ROUNDS];
    // sweep 1: digit counts of this warp's items
#pragma unroll
    for (int r = 0; r < RADIX_ROUNDS; ++r) {
        const int64_t i = base + r * 32;
        const bool ok = i < n;
        k[r] = ok ? keys[i] : 0u;
        v[r] = ok ? vals[i] : 0u;
        const int d = ok ? digit_of(k[r], shift) : RADIX_BUCKETS + lane;   // out of range: matches no one
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        if (ok && (peers & lt) == 0) wh[warp][d] += __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    // warp offsets within the CTA, per digit, in warp order
    for (int d = threadIdx.x; d < RADIX_BUCKETS; d += blockDim.x) {
        int acc = offs[(int64_t)d * nblk + blockIdx.x];
        for (int w = 0; w < RADIX_WARPS; ++w) {
            const int c = wh[w][d];
            wh[w][d] = acc;
            acc += c;
        }
    }
    __syncthreads();
    // sweep 2: scatter
#pragma unroll
    for (int r = 0; r < RADIX_ROUNDS; ++r) {
        const int64_t i = base + r * 32;
        const bool ok = i < n;
        const int d = ok ? digit_of(k[r], shift) : RADIX_BUCKETS + lane;
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        if (ok) {
            const int pos = wh[warp][d] + __popc(peers & lt);
            keys_out[pos] = k[r];
            vals_out[pos] = v[r];
        }
        __syncwarp();
        if (ok && (peers & lt) == 0) wh[warp][d] += __popc(peers);
        __syncwarp();
    }
}

}  // namespace

size_t scan_temp_bytes(int64_t n) {
    size_t bytes = 0;
    while (n > SCAN_TILE) {
        const int64_t nb = (n + SCAN_TILE - 1) / SCAN_TILE;
        bytes += 2 * round256((size_t)nb * sizeof(int));
        n = nb;
    }
    return bytes + 256;
}

cudaError_t exclusive_scan(const int* in, int* out, int64_t n, int* total, void* temp, cudaStream_t s) {
    if (n <= 0) {
        if (total) return cudaMemsetAsync(total, 0, sizeof(int), s);
        return cudaSuccess;
    }
    const int64_t nb = (n + SCAN_TILE - 1) / SCAN_TILE;
    if (nb == 1) {
        scan_tile_kernel<<<1, SCAN_THREADS, 0, s>>>(in, out, n, nullptr);
    } else {
        char* t = reinterpret_cast<char*>(temp);
        int* bsum = reinterpret_cast<int*>(t);
        int* boff = reinterpret_cast<int*>(t + round256((size_t)nb * sizeof(int)));
        void* rest = t + 2 * round256((size_t)nb * sizeof(int));
        scan_tile_kernel<<<(unsigned)nb, SCAN_THREADS, 0, s>>>(in, out, n, bsum);
        cudaError_t e = exclusive_scan(bsum, boff, nb, nullptr, rest, s);
        if (e != cudaSuccess) return e;
        scan_add_kernel<<<(unsigned)nb, SCAN_THREADS, 0, s>>>(out, n, boff);
    }
    if (total) scan_total_kernel<<<1, 1, 0, s>>>(in, out, n, total);
    return cudaGetLastError();
}

// temp layout: keys and values of the other ping-pong side, the digit
// histogram, its scan, the scan's own temporaries (each 256-byte aligned)
size_t radix_temp_bytes(int64_t n) {
    // the larger of the two tilings' histograms (either may run for a
    // smaller sort sharing this workspace)
    const int64_t nblk = (n + RADIX_THREADS * RADIX_ROUNDS_SMALL - 1) / (RADIX_THREADS * RADIX_ROUNDS_SMALL);
    const int64_t nh = nblk * RADIX_BUCKETS;
    return 2 * round256((size_t)n * sizeof(unsigned)) + 2 * round256((size_t)nh * sizeof(int)) +
           scan_temp_bytes(nh);
}

cudaError_t radix_sort_pairs(unsigned* keys, unsigned* vals, int64_t n, int bits, void* temp, cudaStream_t s) {
    if (n <= 1 || bits <= 0) return cudaSuccess;
    const int rounds = radix_rounds(n);
    const int tile = RADIX_THREADS * rounds;
    const int nblk = (int)((n + tile - 1) / tile);
    const int64_t nh = (int64_t)nblk * RADIX_BUCKETS;
    char* t = reinterpret_cast<char*>(temp);
    unsigned* k2 = reinterpret_cast<unsigned*>(t);
    t += round256((size_t)n * sizeof(unsigned));
    unsigned* v2 = reinterpret_cast<unsigned*>(t);
    t += round256((size_t)n * sizeof(unsigned));
    int* hist = reinterpret_cast<int*>(t);
    t += round256((size_t)nh * sizeof(int));
    int* offs = reinterpret_cast<int*>(t);
    t += round256((size_t)nh * sizeof(int));
    void* stmp = t;
    unsigned *ka = keys, *va = vals, *kb = k2, *vb = v2;
    int passes = 0;
    for (int shift = 0; shift < bits; shift += 8, ++passes) {
        if (rounds == RADIX_ROUNDS_SMALL)
            radix_hist_kernel<RADIX_ROUNDS_SMALL><<<nblk, RADIX_THREADS, 0, s>>>(ka, n, shift, nblk, hist);
        else
            radix_hist_kernel<RADIX_ROUNDS_LARGE><<<nblk, RADIX_THREADS, 0, s>>>(ka, n, shift, nblk, hist);
        cudaError_t e = exclusive_scan(hist, offs, nh, nullptr, stmp, s);
        if (e != cudaSuccess) return e;
        if (rounds == RADIX_ROUNDS_SMALL)
            radix_scatter_kernel<RADIX_ROUNDS_SMALL><<<nblk, RADIX_THREADS, 0, s>>>(ka, va, n, shift, nblk, offs, kb, vb);
        else
            radix_scatter_kernel<RADIX_ROUNDS_LARGE><<<nblk, RADIX_THREADS, 0, s>>>(ka, va, n, shift, nblk, offs, kb, vb);
        unsigned* tk = ka; ka = kb; kb = tk;
        unsigned* tv = va; va = vb; vb = tv;
    }
    if (passes & 1) {
        cudaError_t e = cudaMemcpyAsync(keys, ka, (size_t)n * sizeof(unsigned), cudaMemcpyDeviceToDevice, s);
        if (e != cudaSuccess) return e;
        e = cudaMemcpyAsync(vals, va, (size_t)n * sizeof(unsigned), cudaMemcpyDeviceToDevice, s);
        if (e != cudaSuccess) return e;
    }
    return cudaGetLastError();
}

}  // namespace gbn
