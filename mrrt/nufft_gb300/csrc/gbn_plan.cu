// Host side of libgbnufft: plan construction (tile planner), cuFFT plans,
// device buffers and the C ABI declared in include/gbnufft.h.
//
// The plan corresponds to the reference's operator set-up in table mode
// (mrrt/nufft/_nufft.py:216-390): tables, deapodisation and sample
// coordinates are uploaded once; in addition the planner sorts samples by
// grid tile (the reference's GPU path has no such step -- it scatters with
// global atomics, mrrt/nufft/cuda/jinja/table_2d_adjoint.jinja).
#include <cuda_runtime.h>
#include <cufft.h>
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <atomic>
#include <mutex>
#include <string>
#include <vector>

#include "../../../include/gbnufft.h"
#include "gbn_internal.h"
#include "gbn_sort.cuh"

using namespace gbn;

namespace gbn {

cudaError_t ensure_dynamic_smem(const void* kernel, size_t bytes) {
    // without the attribute a launch may use 48 KB of shared memory, static
    // and dynamic together
    if (bytes <= 40 * 1024) return cudaSuccess;
    struct Entry { const void* k; int dev; size_t bytes; };
    static std::mutex mu;
    static std::vector<Entry> done;
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lk(mu);
    for (auto& x : done)
        if (x.k == kernel && x.dev == dev && x.bytes >= bytes) return cudaSuccess;
    cudaFuncAttributes fa;
    e = cudaFuncGetAttributes(&fa, kernel);
    if (e != cudaSuccess) return e;
    if (bytes + fa.sharedSizeBytes > 48 * 1024) {
        e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
        if (e != cudaSuccess) return e;
    }
    for (auto& x : done)
        if (x.k == kernel && x.dev == dev) {
            x.bytes = bytes;
            return cudaSuccess;
        }
    done.push_back({kernel, dev, bytes});
    return cudaSuccess;
}

int resident_ctas(const void* kernel, int threads, size_t smem) {
    struct Entry { const void* k; int dev, threads; size_t smem; int ctas; };
    static std::mutex mu;
    static std::vector<Entry> done;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    std::lock_guard<std::mutex> lk(mu);
    for (auto& x : done)
        if (x.k == kernel && x.dev == dev && x.threads == threads && x.smem == smem) return x.ctas;
    int per_sm = 0, sms = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    const int ctas = std::max(1, per_sm) * std::max(1, sms);
    done.push_back({kernel, dev, threads, smem, ctas});
    return ctas;
}

}  // namespace gbn

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
    g_last_error = msg;
    return code;
}

int cuda_fail(cudaError_t e, const char* where) {
    // an allocation that failed is reported as such, whatever the call site
    const int code = e == cudaErrorMemoryAllocation ? GBN_ERR_NOMEM : GBN_ERR_CUDA;
    return fail(code, std::string(where) + ": " + cudaGetErrorString(e));
}

int cufft_fail(cufftResult r, const char* where) {
    return fail(GBN_ERR_CUFFT, std::string(where) + ": cuFFT error " + std::to_string((int)r));
}

#define GBN_CUDA(call, where)                          \
    do {                                               \
        cudaError_t e__ = (call);                      \
        if (e__ != cudaSuccess) return cuda_fail(e__, where); \
    } while (0)

int next_pow2(int v) {
    int p = 1;
    while (p < v) p <<= 1;
    return p;
}

int ilog2(int v) {
    int l = 0;
    while ((1 << l) < v) ++l;
    return l;
}

// Largest number of coil lanes per sample for a given dimensionality.
int lane_cap(int ndim) { return ndim >= 3 ? 8 : 32; }

Lanes make_lanes(int ndim, int coils) {
    Lanes ln;
    ln.LS = std::min(lane_cap(ndim), next_pow2(std::max(coils, 1)));
    ln.lsh = ilog2(ln.LS);
    ln.LSP = ln.LS == 1 ? 1 : ln.LS + 1;
    return ln;
}

// Host-side fault injection for tests (gbn_debug_fail_alloc): the number of
// further device allocations that succeed before one fails, or -1 (off).
std::atomic<long long> g_fail_alloc_after{-1};

// True when the injection says this allocation is the one that fails.
bool injected_alloc_failure() {
    long long n = g_fail_alloc_after.load();
    while (n >= 0) {
        if (g_fail_alloc_after.compare_exchange_weak(n, n - 1)) return n == 0;
    }
    return false;
}

struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    ~DevBuf() {
        if (p) cudaFree(p);
    }
    cudaError_t alloc(size_t b) {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
        if (b == 0) return cudaSuccess;
        if (injected_alloc_failure()) return cudaErrorMemoryAllocation;
        cudaError_t e = cudaMalloc(&p, b);
        if (e == cudaSuccess) bytes = b;
        return e;
    }
};

struct FftEntry {
    int planes;
    cufftHandle h;        // full transform (1-D, 3-D)
    cufftHandle hx, hy;   // pruned passes: slabs holding data, then the last axis (hy
                          // only when the plan's own last-axis pass cannot run)
};

// State of the host-buffer transforms: two copy streams, events, device
// staging for one call's input and output.
struct HostIo {
    cudaStream_t h2d = nullptr, d2h = nullptr;
    std::vector<cudaEvent_t> ev;
    DevBuf in, out;
    ~HostIo() {
        for (cudaEvent_t e : ev) cudaEventDestroy(e);
        if (h2d) cudaStreamDestroy(h2d);
        if (d2h) cudaStreamDestroy(d2h);
    }
};

constexpr int GATHER_CHUNK = 512;   // samples per gather work item
constexpr int SPREAD_CHUNK = 512;   // list entries per spread work item (1-D)
// Entries per spread work item: tiles with more are split into parts whose
// partial sums are reduced.  2-D: 768 (the 32-coil radial workload's spread
// + reduce measured 0.160 / 0.152 / 0.179 ms at 512 / 768 / 1024).  3-D: a
// sample enters about 8 spread tiles, so the tiles are lighter and the
// per-item overhead weighs more: 1024 (measured).
int spread_part_entries(int ndim) { return ndim == 3 ? 2 * SPREAD_CHUNK : ndim == 2 ? 768 : SPREAD_CHUNK; }
constexpr size_t SMEM_BUDGET = 112 * 1024;   // tile choice: two CTAs per SM
constexpr size_t SMEM_LIMIT = 227 * 1024;    // per-CTA hardware limit
// |tm| bound: keeps t - k exact in float32 (both below 2^24) so table indices
// stay inside the table.
constexpr double TM_LIMIT = 4194304.0;

}  // namespace

struct gbn_plan {
    int device = 0;
    gbn_geometry geom;
    bool dbl = false;
    bool cx = false;
    int F = 1;
    int64_t M_total = 0;
    std::vector<int64_t> foff;
    int Tg[3] = {1, 1, 1}, ntg[3] = {1, 1, 1};   // gather tiling
    int Ts[3] = {1, 1, 1}, nts[3] = {1, 1, 1};   // spread tiling
    int ntiles_g = 1, ntiles_s = 1;               // per frame
    int64_t Kprod = 1, Nprod = 1;
    int rsize = 4;        // sizeof(R)
    bool has_phase = false;

    DevBuf tables, dtables, sn, dfoff;
    DevBuf check;         // status word of the checked build's bounds tests
    DevBuf tickets;       // work counters of the persistent gather launch
    DevBuf weights;       // sparse-matrix mode: per-axis [M_total][J] weights (re, then im)
    DevBuf gcoef, scoef;  // precomputed coefficients in gather / spread list order
    bool coefs = false;   // gcoef / scoef hold the current lists' coefficients
    DevBuf glist, gitems;
    DevBuf bin_ws, bin_ws2;   // device binning workspaces (grown on demand)
    DevBuf slist, sitems, sparts, rtiles;
    int n_gitems = 0, n_sitems = 0, n_rtiles = 0, n_slots = 0;
    int64_t glen = 0, slen = 0;
    DevBuf pad, grid, scratch;
    DevBuf mid;           // output of the forward's slab pass (2-D rows, 3-D z-planes); the
                          // slabs >= N_last the last-axis pass reads stay zero
    int64_t mid_clean = 0;     // 2-D: slabs from which mid is known to be zero
    bool colfft = false;       // last-axis pass by gbn_colfft.cu (else cuFFT)
    bool rowfft = false;       // every pass on the plan's kernels, the row passes with the pad
                               // and crop folded in (gbn_rowfft.cu, gbn_colfft.cu)
    DevBuf fft_tw[3];          // per axis d: exp(-2 pi i m / K_d), m < K_d (axes those use)
    int mid_planes = 0;        // planes the mid buffer holds
    int cap_planes = 0;        // planes the pad/grid buffers hold
    int64_t scratch_cap = 0;   // complex elements
    std::vector<FftEntry> ffts;
    HostIo hio;
    std::mutex mu;

    ~gbn_plan() {
        for (auto& f : ffts) {
            if (f.h) cufftDestroy(f.h);
            if (f.hx) cufftDestroy(f.hx);
            if (f.hy) cufftDestroy(f.hy);
        }
    }
};

namespace {

// NVTX range over a host scope: the stages of a transform appear by name
// (and nest) in a profiler's timeline.  Header-only NVTX v3: without a tool
// attached a push/pop is a branch on a null function pointer.
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev) {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DeviceGuard() {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

template <typename R>
Geom<R> make_geom(const gbn_plan* P, bool spread) {
    Geom<R> g;
    std::memset(&g, 0, sizeof(g));
    const gbn_geometry& G = P->geom;
    g.ndim = G.ndim;
    const R* base = reinterpret_cast<const R*>(P->tables.p);
    size_t off = 0;
    for (int d = 0; d < 3; ++d) {
        const bool on = d < G.ndim;
        g.N[d] = on ? G.Nd[d] : 1;
        g.K[d] = on ? G.Kd[d] : 1;
        g.J[d] = on ? G.Jd[d] : 1;
        g.T[d] = spread ? P->Ts[d] : P->Tg[d];
        g.nt[d] = spread ? P->nts[d] : P->ntg[d];
        g.ncenter[d] = on ? (int)std::floor((double)G.Jd[d] * (double)G.L / 2.0) : 0;
        g.pbc[d] = on ? (R)G.pb_coef[d] : (R)0;
        g.pbo[d] = on ? G.pb_order[d] : d;
        if (on) {
            const size_t len = (size_t)G.Jd[d] * G.L + 1 + 4;
            g.hr[d] = base + off + 2;
            off += len;
        }
    }
    for (int d = 0; d < G.ndim && P->cx; ++d) {
        const size_t len = (size_t)G.Jd[d] * G.L + 1 + 4;
        g.hi[d] = base + off + 2;
        off += len;
    }
    g.L = G.L;
    g.Kprod = P->Kprod;
    g.Nprod = P->Nprod;
    // plane-major layout (the C ABI's grids); transform-internal grids of
    // 2-D and 3-D plans are re-strided by internal_layout
    g.gsp = P->Kprod;
    g.gs1 = g.K[0];
    g.gs2 = (int64_t)g.K[0] * g.K[1];
    g.check = reinterpret_cast<unsigned*>(P->check.p);
    return g;
}

// The 2-D transform keeps its grids row-interleaved, [K1][planes][K0]: row
// r of every plane is one contiguous block, so the row FFT pass runs over the
// first N1 * planes rows only (the others hold zero padding on the way in and
// are cropped away on the way out) and the column pass is one strided batch.
// The 3-D transform keeps the plane-major layout and prunes plane by plane
// (up to PRUNE3_MAX_PLANES planes): a batched 2-D FFT of the first N2
// z-planes, then the z-pass at the plane's own stride.  Interleaving z-planes
// too would stretch the z-pass's stride to planes x K1 x K0, which measured
// slower than the pruning saves.
constexpr int PRUNE3_MAX_PLANES = 16;
bool pruned_3d(const gbn_plan* P, int planes) { return P->geom.ndim == 3 && planes <= PRUNE3_MAX_PLANES; }

// cells of one slab (a row in 2-D, a z-plane in 3-D), and the image extent
// along the last axis
int64_t slab_cells(const gbn_plan* P) {
    return P->geom.ndim == 2 ? P->geom.Kd[0] : (int64_t)P->geom.Kd[0] * P->geom.Kd[1];
}
int last_n(const gbn_plan* P) { return P->geom.Nd[P->geom.ndim - 1]; }

template <typename T>
void internal_layout(const gbn_plan* P, int planes, T& g) {
    if (P->geom.ndim == 2) {
        g.gsp = P->geom.Kd[0];
        g.gs1 = (int64_t)planes * P->geom.Kd[0];
        g.gs2 = 0;
    } else {
        g.gsp = P->Kprod;
        g.gs1 = P->geom.Kd[0];
        g.gs2 = P->geom.ndim > 2 ? slab_cells(P) : 0;
    }
}

// Sample-list buffer layout: window starts (spread list only), sample
// phase (if any), one coordinate array per axis, sample index.  Every
// section starts on a 16-byte boundary (double2 phases need it).
inline size_t align16(size_t v) { return (v + 15) & ~(size_t)15; }

template <typename R>
struct ListLayout {
    size_t ls = 0, ph = 0, t[3] = {0, 0, 0}, idx = 0, bytes = 0;
    ListLayout(const gbn_plan* P, int64_t len, bool with_ls) {
        size_t off = 0;
        if (with_ls) {
            ls = off;
            off = align16(off + sizeof(short4) * (size_t)len);
        }
        if (P->has_phase) {
            ph = off;
            off = align16(off + sizeof(typename Cx<R>::T) * (size_t)len);
        }
        for (int d = 0; d < P->geom.ndim; ++d) {
            t[d] = off;
            off = align16(off + sizeof(R) * (size_t)len);
        }
        idx = off;
        bytes = align16(off + sizeof(int) * (size_t)len) + 16;
    }
};

template <typename R>
SampleList<R> make_list(const gbn_plan* P, const DevBuf& buf, int64_t len, bool with_ls) {
    typedef typename Cx<R>::T C;
    SampleList<R> s;
    std::memset(&s, 0, sizeof(s));
    const char* b = reinterpret_cast<const char*>(buf.p);
    const ListLayout<R> L(P, len, with_ls);
    if (with_ls) s.ls = reinterpret_cast<const short4*>(b + L.ls);
    if (P->has_phase) s.ph = reinterpret_cast<const C*>(b + L.ph);
    for (int d = 0; d < P->geom.ndim; ++d) s.t[d] = reinterpret_cast<const R*>(b + L.t[d]);
    s.idx = reinterpret_cast<const int*>(b + L.idx);
    s.len = len;
    if (P->coefs) {
        const DevBuf& cb = with_ls ? P->scoef : P->gcoef;
        int jsum = 0;
        for (int d = 0; d < P->geom.ndim; ++d) jsum += P->geom.Jd[d];
        s.jsum = jsum;
        s.cr = reinterpret_cast<const R*>(cb.p);
        if (P->cx) s.ci = s.cr + (size_t)len * jsum;
    }
    return s;
}

template <typename R>
size_t list_bytes(const gbn_plan* P, int64_t len, bool with_ls) {
    return ListLayout<R>(P, len, with_ls).bytes;
}

// Gather tiling: start from a per-dimension default and halve the largest
// edge until the staged tile + halo fits the shared-memory budget.
// Spread tiling: up to 8 register blocks per CTA, one warp each; edges are
// multiples of the block edges and may exceed Kd (the cells past Kd are
// never written).
void choose_tiles(gbn_plan* P) {
    const gbn_geometry& G = P->geom;
    const int ndim = G.ndim;
    const Lanes ln = make_lanes(ndim, G.max_coils);
    int T[3] = {1, 1, 1};
    if (ndim == 1) {
        T[0] = 256;
    } else if (ndim == 2) {
        if (ln.LS >= 16) { T[0] = 16; T[1] = 8; }
        else if (ln.LS >= 4) { T[0] = 32; T[1] = 16; }
        else { T[0] = 32; T[1] = 32; }
    } else {
        if (ln.LS >= 4) { T[0] = 8; T[1] = 8; T[2] = 4; }
        else { T[0] = 8; T[1] = 8; T[2] = 8; }
    }
    for (int d = 0; d < ndim; ++d)
        if (G.tile[d] > 0) T[d] = G.tile[d];
    const size_t csz = (size_t)2 * P->rsize;
    for (int it = 0; it < 32; ++it) {
        size_t cells = 1;
        for (int d = 0; d < ndim; ++d) cells *= (size_t)(std::min(T[d], G.Kd[d]) + G.Jd[d] - 1);
        if (cells * ln.LSP * csz <= SMEM_BUDGET) break;
        int dm = 0;
        for (int d = 1; d < ndim; ++d)
            if (T[d] > T[dm]) dm = d;
        if (T[dm] <= 1) break;
        T[dm] /= 2;
    }
    for (int d = 0; d < 3; ++d) {
        P->Tg[d] = d < ndim ? std::max(1, std::min(T[d], G.Kd[d])) : 1;
        P->ntg[d] = d < ndim ? (G.Kd[d] + P->Tg[d] - 1) / P->Tg[d] : 1;
    }
    P->ntiles_g = P->ntg[0] * P->ntg[1] * P->ntg[2];
    // spread: 8 register blocks (warps) per tile by default
    int B[3] = {1, 1, 1}, S[3] = {1, 1, 1};
    if (ndim == 1) { B[0] = SpreadBlock<1>::B0; S[0] = 8 * B[0]; }
    else if (ndim == 2) { B[0] = SpreadBlock<2>::B0; B[1] = SpreadBlock<2>::B1; S[0] = 4 * B[0]; S[1] = 2 * B[1]; }
    else {
        B[0] = SpreadBlock<3>::B0; B[1] = SpreadBlock<3>::B1; B[2] = SpreadBlock<3>::B2;
        // 8 x 4 x 4: measured best of the 8-block shapes on a 3-D kooshball
        S[0] = 2 * B[0]; S[1] = B[1]; S[2] = 4 * B[2];
    }
    for (int d = 0; d < ndim; ++d) {
        if (G.stile[d] > 0) S[d] = std::max(B[d], (G.stile[d] / B[d]) * B[d]);
        // no wider than the grid rounded up to whole blocks
        const int kmax = ((G.Kd[d] + B[d] - 1) / B[d]) * B[d];
        S[d] = std::min(S[d], kmax);
    }
    // at most 8 warps per CTA
    for (int it = 0; it < 32; ++it) {
        int w = 1;
        for (int d = 0; d < ndim; ++d) w *= S[d] / B[d];
        if (w <= 8) break;
        int dm = 0;
        for (int d = 1; d < ndim; ++d)
            if (S[d] / B[d] > S[dm] / B[dm]) dm = d;
        S[dm] = std::max(B[dm], ((S[dm] / 2) / B[dm]) * B[dm]);
    }
    for (int d = 0; d < 3; ++d) {
        P->Ts[d] = d < ndim ? S[d] : 1;
        P->nts[d] = d < ndim ? (G.Kd[d] + P->Ts[d] - 1) / P->Ts[d] : 1;
    }
    P->ntiles_s = P->nts[0] * P->nts[1] * P->nts[2];
}

template <typename R>
int build_lists(gbn_plan* P, const R* tm, const R* phase) {
    typedef typename Cx<R>::T C;
    const gbn_geometry& G = P->geom;
    const int ndim = G.ndim;
    const int64_t Mt = P->M_total;
    const int ntg = P->ntiles_g, nts = P->ntiles_s;
    const int64_t nbins_g = (int64_t)P->F * ntg, nbins_s = (int64_t)P->F * nts;

    // first tap of every sample, per axis (validated)
    std::vector<int> kf((size_t)Mt * ndim);
    for (int64_t m = 0; m < Mt; ++m) {
        for (int d = 0; d < ndim; ++d) {
            const R t = tm[m * ndim + d];
            if (!std::isfinite((double)t) || std::fabs((double)t) > TM_LIMIT)
                return fail(GBN_ERR_INVALID, "sample coordinate is not finite or |tm| > 2^22");
            kf[(size_t)m * ndim + d] = 1 + (int)std::floor((double)t - 0.5 * (double)G.Jd[d]);
        }
    }
    auto wrap = [](int k, int K) {
        int r = k % K;
        return r < 0 ? r + K : r;
    };
    // ---- gather list: stable counting sort by the tile of the first tap ----
    std::vector<int64_t> gbin((size_t)Mt);
    for (int f = 0; f < P->F; ++f) {
        for (int64_t m = P->foff[f]; m < P->foff[f + 1]; ++m) {
            int lin = 0, mul = 1;
            for (int d = 0; d < ndim; ++d) {
                lin += (wrap(kf[(size_t)m * ndim + d], G.Kd[d]) / P->Tg[d]) * mul;
                mul *= P->ntg[d];
            }
            gbin[(size_t)m] = (int64_t)f * ntg + lin;
        }
    }
    std::vector<int64_t> gcount((size_t)nbins_g + 1, 0);
    for (int64_t m = 0; m < Mt; ++m) gcount[(size_t)gbin[m] + 1]++;
    for (int64_t b = 0; b < nbins_g; ++b) gcount[b + 1] += gcount[b];
    std::vector<int64_t> gorder((size_t)Mt);
    {
        std::vector<int64_t> cur(gcount.begin(), gcount.end() - 1);
        for (int64_t m = 0; m < Mt; ++m) gorder[(size_t)cur[gbin[m]]++] = m;
    }
    // ---- spread list: one entry per (tile, periodic image of the window)
    // that touches the tile; the entry carries the window start in tile
    // coordinates, so the kernel never wraps.
    struct AxisHit { int tile; int ls; };
    auto axis_hits = [&](int64_t m, int d, AxisHit* out) {
        int n = 0;
        for (int j = 0; j < G.Jd[d]; ++j) {
            const int c = wrap(kf[(size_t)m * ndim + d] + j, G.Kd[d]);
            const int tl = c / P->Ts[d];
            const int ls = c - tl * P->Ts[d] - j;
            bool seen = false;
            for (int q = 0; q < n; ++q) seen = seen || (out[q].tile == tl && out[q].ls == ls);
            if (!seen) out[n++] = AxisHit{tl, ls};
        }
        return n;
    };
    auto for_each_entry = [&](int64_t m, int f, auto&& fn) {
        AxisHit h[3][JMAX];
        int nh[3] = {1, 1, 1};
        for (int d = 0; d < 3; ++d) h[d][0] = AxisHit{0, 0};
        for (int d = 0; d < ndim; ++d) nh[d] = axis_hits(m, d, h[d]);
        for (int a2 = 0; a2 < nh[2]; ++a2)
            for (int a1 = 0; a1 < nh[1]; ++a1)
                for (int a0 = 0; a0 < nh[0]; ++a0) {
                    const int lin = h[0][a0].tile + P->nts[0] * (h[1][a1].tile + P->nts[1] * h[2][a2].tile);
                    short4 ls;
                    ls.x = (short)h[0][a0].ls;
                    ls.y = (short)h[1][a1].ls;
                    ls.z = (short)h[2][a2].ls;
                    ls.w = 0;
                    fn((int64_t)f * nts + lin, ls);
                }
    };
    std::vector<int64_t> scount((size_t)nbins_s + 1, 0);
    for (int f = 0; f < P->F; ++f)
        for (int64_t m = P->foff[f]; m < P->foff[f + 1]; ++m)
            for_each_entry(m, f, [&](int64_t b, short4) { scount[(size_t)b + 1]++; });
    for (int64_t b = 0; b < nbins_s; ++b) scount[b + 1] += scount[b];
    const int64_t slen = scount[(size_t)nbins_s];
    if (Mt > INT32_MAX || slen > INT32_MAX)
        return fail(GBN_ERR_TOOLARGE, "more than 2^31 list entries");
    std::vector<int64_t> sorder((size_t)slen);
    std::vector<short4> sls((size_t)slen);
    {
        std::vector<int64_t> cur(scount.begin(), scount.end() - 1);
        for (int f = 0; f < P->F; ++f)
            for (int64_t m = P->foff[f]; m < P->foff[f + 1]; ++m)
                for_each_entry(m, f, [&](int64_t b, short4 ls) {
                    const int64_t at = cur[b]++;
                    sorder[(size_t)at] = m;
                    sls[(size_t)at] = ls;
                });
    }
    // 3-D: within a tile, entries in sample order come in a few trajectory
    // segments at a time, so a staged chunk loads some warps' register
    // blocks much more than others, and every warp waits for the busiest one
    // at the chunk's barrier.  Runs of four consecutive samples (one 32-byte
    // sector of each coil's values) are put in a fixed pseudo-random order
    // instead, so every chunk spreads over the whole tile (kooshball spread
    // 6.08 -> 5.73 ms).  2-D keeps sample order: with 32 coils a chunk's
    // values are 16 KB, and scattering their reads cost more than the
    // balance gained (0.159 -> 0.180 ms).
    if (ndim == 3) {
        std::vector<std::pair<uint32_t, int64_t>> key;
        std::vector<int64_t> o2;
        std::vector<short4> l2;
        for (int64_t b = 0; b < nbins_s; ++b) {
            const int64_t lo = scount[(size_t)b], hi = scount[(size_t)b + 1];
            if (hi - lo <= SPREAD_CHUNK_ENTRIES) continue;   // one chunk: order irrelevant
            key.resize((size_t)(hi - lo));
            for (int64_t i = lo; i < hi; ++i) {
                const uint32_t run = (uint32_t)(sorder[(size_t)i] >> 2);
                key[(size_t)(i - lo)] = {run * 2654435761u, i};
            }
            std::sort(key.begin(), key.end());
            o2.resize(key.size());
            l2.resize(key.size());
            for (size_t q = 0; q < key.size(); ++q) {
                o2[q] = sorder[(size_t)key[q].second];
                l2[q] = sls[(size_t)key[q].second];
            }
            std::copy(o2.begin(), o2.end(), sorder.begin() + lo);
            std::copy(l2.begin(), l2.end(), sls.begin() + lo);
        }
    }
    // ---- pack lists (SoA) -------------------------------------------------
    auto pack = [&](const std::vector<int64_t>& order, const short4* ls, DevBuf& dst, int64_t len) -> int {
        const ListLayout<R> L(P, len, ls != nullptr);
        const size_t bytes = L.bytes;
        std::vector<char> host(bytes, 0);
        if (ls) std::memcpy(host.data() + L.ls, ls, sizeof(short4) * (size_t)len);
        if (P->has_phase) {
            C* ph = reinterpret_cast<C*>(host.data() + L.ph);
            for (int64_t i = 0; i < len; ++i) {
                ph[i].x = phase[2 * order[i]];
                ph[i].y = phase[2 * order[i] + 1];
            }
        }
        for (int d = 0; d < ndim; ++d) {
            R* t = reinterpret_cast<R*>(host.data() + L.t[d]);
            for (int64_t i = 0; i < len; ++i) t[i] = tm[order[i] * ndim + d];
        }
        int* idx = reinterpret_cast<int*>(host.data() + L.idx);
        for (int64_t i = 0; i < len; ++i) {
            const int64_t m = order[i];
            const int f = (int)(std::upper_bound(P->foff.begin(), P->foff.end(), m) - P->foff.begin()) - 1;
            idx[i] = (int)(m - P->foff[f]);
        }
        cudaError_t e = dst.alloc(bytes);
        if (e != cudaSuccess) return cuda_fail(e, "list allocation");
        e = cudaMemcpy(dst.p, host.data(), bytes, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return cuda_fail(e, "list upload");
        return GBN_OK;
    };
    int rc = pack(gorder, nullptr, P->glist, Mt);
    if (rc) return rc;
    rc = pack(sorder, sls.data(), P->slist, slen);
    if (rc) return rc;
    P->glen = Mt;
    P->slen = slen;

    // ---- work items ---------------------------------------------------------
    struct Item { int4 a; int2 b; };
    std::vector<Item> gi, si;
    std::vector<int4> rt;
    int slots = 0;
    for (int64_t b = 0; b < nbins_g; ++b) {
        const int f = (int)(b / ntg), tile = (int)(b % ntg);
        const int64_t g0 = gcount[b], gn = gcount[b + 1] - g0;
        for (int64_t q = 0; q < gn; q += GATHER_CHUNK)
            gi.push_back({make_int4(f, tile, (int)(g0 + q), (int)std::min<int64_t>(GATHER_CHUNK, gn - q)),
                          make_int2(-1, 1)});
    }
    for (int64_t b = 0; b < nbins_s; ++b) {
        const int f = (int)(b / nts), tile = (int)(b % nts);
        const int64_t s0 = scount[b], sn = scount[b + 1] - s0;
        const int SCH = spread_part_entries(G.ndim);
        const int parts = (int)std::max<int64_t>(1, (sn + SCH - 1) / SCH);
        if (parts == 1) {
            si.push_back({make_int4(f, tile, (int)s0, (int)sn), make_int2(-1, 1)});
        } else {
            const int64_t per = (sn + parts - 1) / parts;
            for (int q = 0; q < parts; ++q) {
                const int64_t a = s0 + q * per;
                const int64_t n = std::min<int64_t>(per, s0 + sn - a);
                si.push_back({make_int4(f, tile, (int)a, (int)n), make_int2(slots + q, parts)});
            }
            rt.push_back(make_int4(f, tile, slots, parts));
            slots += parts;
        }
    }
    auto heavy_first = [](const Item& x, const Item& y) { return x.a.w > y.a.w; };
    std::stable_sort(gi.begin(), gi.end(), heavy_first);
    std::stable_sort(si.begin(), si.end(), heavy_first);
    std::vector<int4> ga(gi.size()), sa(si.size());
    std::vector<int2> sb(si.size());
    for (size_t i = 0; i < gi.size(); ++i) ga[i] = gi[i].a;
    for (size_t i = 0; i < si.size(); ++i) {
        sa[i] = si[i].a;
        sb[i] = si[i].b;
    }
    auto upload = [&](DevBuf& dst, const void* src, size_t bytes) -> int {
        cudaError_t e = dst.alloc(std::max<size_t>(bytes, 16));
        if (e != cudaSuccess) return cuda_fail(e, "item allocation");
        if (bytes) {
            e = cudaMemcpy(dst.p, src, bytes, cudaMemcpyHostToDevice);
            if (e != cudaSuccess) return cuda_fail(e, "item upload");
        }
        return GBN_OK;
    };
    if ((rc = upload(P->gitems, ga.data(), ga.size() * sizeof(int4)))) return rc;
    if ((rc = upload(P->sitems, sa.data(), sa.size() * sizeof(int4)))) return rc;
    if ((rc = upload(P->sparts, sb.data(), sb.size() * sizeof(int2)))) return rc;
    if ((rc = upload(P->rtiles, rt.data(), rt.size() * sizeof(int4)))) return rc;
    P->n_gitems = (int)ga.size();
    P->n_sitems = (int)sa.size();
    P->n_rtiles = (int)rt.size();
    P->n_slots = slots;
    return GBN_OK;
}

// Scratch for the partial tiles of split spread work items.
int ensure_scratch(gbn_plan* P, int coils) {
    const size_t csz = (size_t)2 * P->rsize;
    const Lanes ln = make_lanes(P->geom.ndim, coils);
    const int64_t tile_cells = (int64_t)P->Ts[0] * P->Ts[1] * P->Ts[2];
    const int64_t chunks = (coils + ln.LS - 1) / ln.LS;
    // an upper bound for any lane count call_lanes may pick (halving LS
    // never increases chunks * LS)
    const int64_t need = (int64_t)P->n_slots * chunks * ln.LS * tile_cells;
    if (need > P->scratch_cap) {
        cudaError_t e = P->scratch.alloc((size_t)need * csz);
        if (e != cudaSuccess) return fail(GBN_ERR_NOMEM, "scratch allocation failed");
        P->scratch_cap = need;
    }
    return GBN_OK;
}

// Zero-padded FFT input, FFT output grid and scratch for F * coils planes.
// `fused`: the call runs the 3-D transform on the plan's own passes (in
// place on the grid), which need no slab-pass buffer.
int ensure_buffers(gbn_plan* P, int coils, bool fused = false) {
    const int planes = P->F * coils;
    const size_t csz = (size_t)2 * P->rsize;
    if (planes > P->cap_planes) {
        const size_t bytes = (size_t)planes * P->Kprod * csz;
        cudaError_t e = P->pad.alloc(bytes);
        if (e != cudaSuccess) return fail(GBN_ERR_NOMEM, "pad buffer allocation failed");
        e = cudaMemset(P->pad.p, 0, bytes);
        if (e != cudaSuccess) return cuda_fail(e, "pad buffer clear");
        e = P->grid.alloc(bytes);
        if (e != cudaSuccess) return fail(GBN_ERR_NOMEM, "grid buffer allocation failed");
        P->cap_planes = planes;
    }
    // the pruned FFT's intermediate buffer: every plane in 2-D, the planes of
    // a pruned call in 3-D (none beyond PRUNE3_MAX_PLANES)
    const int mid_need = P->geom.ndim == 2 || (pruned_3d(P, planes) && !fused) ? planes : 0;
    if (mid_need > P->mid_planes) {
        const size_t bytes = (size_t)mid_need * P->Kprod * csz;
        cudaError_t e = P->mid.alloc(bytes);
        if (e != cudaSuccess) return fail(GBN_ERR_NOMEM, "slab-pass buffer allocation failed");
        e = cudaMemset(P->mid.p, 0, bytes);
        if (e != cudaSuccess) return cuda_fail(e, "slab-pass buffer clear");
        P->mid_planes = mid_need;
        P->mid_clean = 0;
    }
    return ensure_scratch(P, coils);
}

// The last-axis pass runs on the plan's own pruned kernel (gbn_colfft.cu) in
// single precision, 2-D and 3-D, for the lengths it implements, unless the
// geometry asks for cuFFT throughout.  Its twiddles are computed here in
// double precision and rounded once.
int upload_twiddles(DevBuf& dst, int L) {
    std::vector<float> tw(2 * (size_t)L);
    for (int m = 0; m < L; ++m) {
        const double a = 6.283185307179586476925286766559 * (double)m / (double)L;   // 2 pi m / L
        tw[2 * m] = (float)std::cos(a);
        tw[2 * m + 1] = (float)-std::sin(a);
    }
    cudaError_t e = dst.alloc(tw.size() * sizeof(float));
    if (e == cudaSuccess) e = cudaMemcpy(dst.p, tw.data(), tw.size() * sizeof(float), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(e, "FFT twiddle table");
    return GBN_OK;
}

// When every axis has a supported length, the whole transform runs on the
// plan's kernels, the row passes with the pad and the crop folded in
// (gbn_rowfft.cu).
int setup_colfft(gbn_plan* P) {
    const gbn_geometry& G = P->geom;
    const int L = G.Kd[G.ndim - 1];
    P->colfft = !P->dbl && G.ndim >= 2 && !(G.flags & GBN_FLAG_CUFFT_ONLY) && colfft_supported(L);
    if (!P->colfft) return GBN_OK;
    P->rowfft = rowfft_supported(G.Kd[0]) && (G.ndim == 2 || colfft_supported(G.Kd[1]));
    for (int d = 0; d < G.ndim; ++d) {
        if (d < G.ndim - 1 && !P->rowfft) continue;
        int rc = upload_twiddles(P->fft_tw[d], G.Kd[d]);
        if (rc) return rc;
    }
    return GBN_OK;
}

// Row pass with the pad (sign -1: image -> grid rows) or the crop (sign +1:
// grid rows -> image) folded in; 2-D: image rows to the row-interleaved
// layout (into mid), 3-D: to the plane-major layout (the grid in place).
int run_rowfft(gbn_plan* P, const void* in, int64_t in_elems, void* out, int64_t out_elems, int planes, int sign,
               cudaStream_t s) {
    const gbn_geometry& G = P->geom;
    RowFftParams p;
    std::memset(&p, 0, sizeof(p));
    p.in = static_cast<const float2*>(in);
    p.out = static_cast<float2*>(out);
    p.sn = static_cast<const float*>(P->sn.p);
    p.scale = G.ortho ? (float)(G.adjoint_scale / std::sqrt((double)P->Kprod)) : (float)G.adjoint_scale;
    p.planes = planes;
    p.N0 = G.Nd[0];
    p.N1 = G.Nd[1];
    p.N2 = G.ndim > 2 ? G.Nd[2] : 1;
    p.L = G.Kd[0];
    internal_layout(P, planes, p);
    p.tw = static_cast<const float2*>(P->fft_tw[0].p);
    p.check = static_cast<unsigned*>(P->check.p);
    p.in_elems = in_elems;
    p.out_elems = out_elems;
    GBN_CUDA(launch_rowfft(p, sign, s), sign < 0 ? "pad + row FFT pass" : "row FFT pass + crop");
    return GBN_OK;
}

// Pass along memory axis `axis` (1 or 2) over planes x planes2 arrays of
// [K_axis][S] at strides ps, ps2: rows >= nin read as zero, rows >= nout not
// written.
struct AxisPass {
    const void* in;
    int64_t in_elems;
    void* out;
    int64_t out_elems;
    int axis;
    int64_t S, ps, ps2;
    int planes, planes2;
    int nin, nout;
};
int run_colfft(gbn_plan* P, const AxisPass& a, int sign, cudaStream_t s) {
    ColFftParams p;
    std::memset(&p, 0, sizeof(p));
    p.in = static_cast<const float2*>(a.in);
    p.out = static_cast<float2*>(a.out);
    p.S = a.S;
    p.ps = a.ps;
    p.ps2 = a.ps2;
    p.planes = a.planes;
    p.planes2 = a.planes2;
    p.L = P->geom.Kd[a.axis];
    p.nin = a.nin;
    p.nout = a.nout;
    p.tw = static_cast<const float2*>(P->fft_tw[a.axis].p);
    p.check = static_cast<unsigned*>(P->check.p);
    p.in_elems = a.in_elems;
    p.out_elems = a.out_elems;
    GBN_CUDA(launch_colfft(p, sign, s), "strided-axis FFT pass");
    return GBN_OK;
}

int get_fft(gbn_plan* P, int planes, FftEntry** out) {
    for (auto& f : P->ffts)
        if (f.planes == planes) {
            *out = &f;
            return GBN_OK;
        }
    const gbn_geometry& G = P->geom;
    const cufftType type = P->dbl ? CUFFT_Z2Z : CUFFT_C2C;
    FftEntry f{planes, 0, 0, 0};
    cufftResult r;
    if (G.ndim == 2 || pruned_3d(P, planes)) {
        // 2-D: all planes' rows at once (interleaved layout); 3-D: one plane
        // at a time (its z-planes are contiguous, plane-major layout)
        const int slab = (int)slab_cells(P), Kl = G.Kd[G.ndim - 1], Nl = last_n(P);
        const int batch_planes = G.ndim == 2 ? planes : 1;
        // slabs k < N_last: transformed as rows (2-D) or as K1 x K0 planes (3-D)
        int nx[2] = {G.ndim == 2 ? G.Kd[0] : G.Kd[1], G.Kd[0]};
        r = cufftPlanMany(&f.hx, G.ndim - 1, nx, nullptr, 1, slab, nullptr, 1, slab, type, Nl * batch_planes);
        if (r != CUFFT_SUCCESS) return cufft_fail(r, "cufftPlanMany (slabs)");
        // every column along the last axis: stride batch_planes * slab, adjacent columns
        const int zs = batch_planes * slab;
        int ny[1] = {Kl}, emb[1] = {Kl};
        if (!P->colfft) r = cufftPlanMany(&f.hy, 1, ny, emb, zs, 1, emb, zs, 1, type, zs);
        if (r != CUFFT_SUCCESS) {
            cufftDestroy(f.hx);
            return cufft_fail(r, "cufftPlanMany (last axis)");
        }
    } else {
        int n[3];
        for (int d = 0; d < G.ndim; ++d) n[d] = G.Kd[G.ndim - 1 - d];
        r = cufftPlanMany(&f.h, G.ndim, n, nullptr, 1, (int)P->Kprod, nullptr, 1, (int)P->Kprod, type, planes);
        if (r != CUFFT_SUCCESS) return cufft_fail(r, "cufftPlanMany");
    }
    P->ffts.push_back(f);
    *out = &P->ffts.back();
    return GBN_OK;
}

int exec_fft(gbn_plan* P, cufftHandle h, void* in, void* out, int dir, cudaStream_t s) {
    cufftResult r = cufftSetStream(h, s);
    if (r != CUFFT_SUCCESS) return cufft_fail(r, "cufftSetStream");
    if (P->dbl)
        r = cufftExecZ2Z(h, (cufftDoubleComplex*)in, (cufftDoubleComplex*)out, dir);
    else
        r = cufftExecC2C(h, (cufftComplex*)in, (cufftComplex*)out, dir);
    if (r != CUFFT_SUCCESS) return cufft_fail(r, "cufftExec");
    return GBN_OK;
}

// 2-D last-axis pass: forward mid -> grid (the N_1 slabs with data read),
// inverse grid -> grid in place (the N_1 slabs the crop reads written).
int colfft_2d(gbn_plan* P, int planes, int sign, cudaStream_t s) {
    const int64_t ge = (int64_t)P->cap_planes * P->Kprod;
    AxisPass a{P->grid.p, ge, P->grid.p, ge, 1, (int64_t)planes * P->geom.Kd[0], 0, 0, 1, 1,
               P->geom.Kd[1], last_n(P)};
    if (sign < 0) {
        a.in = P->mid.p;
        a.in_elems = (int64_t)P->mid_planes * P->Kprod;
        a.nin = last_n(P);
        a.nout = P->geom.Kd[1];
    }
    return run_colfft(P, a, sign, s);
}

// 3-D passes along axes 1 and 2 of the grid, in place: forward axis 1 over
// the N_2 z-slabs with data (N_1 rows read), then axis 2 (N_2 z-slabs read);
// inverse axis 2 (N_2 z-slabs written), then axis 1 over those slabs (N_1
// rows written).
int colfft_3d(gbn_plan* P, int planes, int sign, cudaStream_t s) {
    const gbn_geometry& G = P->geom;
    const int64_t ge = (int64_t)P->cap_planes * P->Kprod;
    const int64_t slab = (int64_t)G.Kd[0] * G.Kd[1];
    AxisPass a1{P->grid.p, ge, P->grid.p, ge, 1, G.Kd[0], slab, P->Kprod, G.Nd[2], planes, 0, 0};
    AxisPass a2{P->grid.p, ge, P->grid.p, ge, 2, slab, P->Kprod, 0, planes, 1, 0, 0};
    int rc;
    if (sign < 0) {
        a1.nin = G.Nd[1];
        a1.nout = G.Kd[1];
        a2.nin = G.Nd[2];
        a2.nout = G.Kd[2];
        if ((rc = run_colfft(P, a1, -1, s))) return rc;
        return run_colfft(P, a2, -1, s);
    }
    a2.nin = G.Kd[2];
    a2.nout = G.Nd[2];
    a1.nin = G.Kd[1];
    a1.nout = G.Nd[1];
    if ((rc = run_colfft(P, a2, 1, s))) return rc;
    return run_colfft(P, a1, 1, s);
}

// Forward Kd-point FFT of the padded planes into the grid.  2-D and 3-D:
// the slab pass only over the N_last slabs that hold data (pad -> mid), then
// the last-axis pass over every column (mid -> grid).
int fft_forward(gbn_plan* P, int planes, cudaStream_t s) {
    FftEntry* f = nullptr;
    int rc = get_fft(P, planes, &f);
    if (rc) return rc;
    if (pruned_3d(P, planes)) {
        // the first N2 z-planes of each plane into mid, whose other z-planes
        // are never written and stay zero; then each plane's z-pass
        const size_t pb = (size_t)P->Kprod * 2 * P->rsize;
        char* pad = static_cast<char*>(P->pad.p);
        char* mid = static_cast<char*>(P->mid.p);
        char* grid = static_cast<char*>(P->grid.p);
        for (int pl = 0; pl < planes; ++pl)
            if ((rc = exec_fft(P, f->hx, pad + pl * pb, mid + pl * pb, CUFFT_FORWARD, s))) return rc;
        if (P->colfft)
            return run_colfft(P,
                              AxisPass{mid, (int64_t)P->mid_planes * P->Kprod, grid,
                                       (int64_t)P->cap_planes * P->Kprod, 2, slab_cells(P), P->Kprod, 0, planes,
                                       1, last_n(P), P->geom.Kd[2]},
                              -1, s);
        for (int pl = 0; pl < planes; ++pl)
            if ((rc = exec_fft(P, f->hy, mid + pl * pb, grid + pl * pb, CUFFT_FORWARD, s))) return rc;
        return GBN_OK;
    }
    if (P->geom.ndim == 2 && P->colfft) {
        // the last-axis pass reads only the N_last * planes slabs the row
        // pass writes
        if ((rc = exec_fft(P, f->hx, P->pad.p, P->mid.p, CUFFT_FORWARD, s))) return rc;
        return colfft_2d(P, planes, -1, s);
    }
    if (P->geom.ndim == 2) {
        // The last-axis pass reads slabs [N_last * planes, K_last * planes)
        // of mid as zero.  A call with more planes wrote slabs below
        // N_last * cap_planes, so slabs in [N_last * planes, mid_clean) are
        // cleared first.  A stream being captured into a graph clears up to
        // N_last * cap_planes on every replay, since eager calls between
        // replays may write there.
        const int64_t row = slab_cells(P) * 2 * P->rsize;
        const int64_t lo = (int64_t)last_n(P) * planes;
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        GBN_CUDA(cudaStreamIsCapturing(s, &cs), "capture status");
        const bool capturing = cs != cudaStreamCaptureStatusNone;
        const int64_t hi = capturing ? (int64_t)last_n(P) * P->mid_planes : P->mid_clean;
        if (hi > lo)
            GBN_CUDA(cudaMemsetAsync(static_cast<char*>(P->mid.p) + lo * row, 0, (size_t)((hi - lo) * row), s),
                     "row-pass buffer clear");
        P->mid_clean = capturing ? std::max(P->mid_clean, lo) : lo;
        if ((rc = exec_fft(P, f->hx, P->pad.p, P->mid.p, CUFFT_FORWARD, s))) return rc;
        return exec_fft(P, f->hy, P->mid.p, P->grid.p, CUFFT_FORWARD, s);
    }
    return exec_fft(P, f->h, P->pad.p, P->grid.p, CUFFT_FORWARD, s);
}

// Inverse FFT of the grid in place.  2-D and 3-D: every column along the
// last axis, then only the N_last slabs the crop reads.
int fft_inverse(gbn_plan* P, int planes, cudaStream_t s) {
    FftEntry* f = nullptr;
    int rc = get_fft(P, planes, &f);
    if (rc) return rc;
    if (pruned_3d(P, planes)) {
        const size_t pb = (size_t)P->Kprod * 2 * P->rsize;
        char* grid = static_cast<char*>(P->grid.p);
        if (P->colfft) {
            const int64_t ge = (int64_t)P->cap_planes * P->Kprod;
            if ((rc = run_colfft(P, AxisPass{grid, ge, grid, ge, 2, slab_cells(P), P->Kprod, 0, planes, 1,
                                             P->geom.Kd[2], last_n(P)},
                                 1, s)))
                return rc;
        } else {
            for (int pl = 0; pl < planes; ++pl)
                if ((rc = exec_fft(P, f->hy, grid + pl * pb, grid + pl * pb, CUFFT_INVERSE, s))) return rc;
        }
        for (int pl = 0; pl < planes; ++pl)
            if ((rc = exec_fft(P, f->hx, grid + pl * pb, grid + pl * pb, CUFFT_INVERSE, s))) return rc;
        return GBN_OK;
    }
    if (P->geom.ndim == 2) {
        if (P->colfft) {
            if ((rc = colfft_2d(P, planes, 1, s))) return rc;
        } else if ((rc = exec_fft(P, f->hy, P->grid.p, P->grid.p, CUFFT_INVERSE, s))) {
            return rc;
        }
        return exec_fft(P, f->hx, P->grid.p, P->grid.p, CUFFT_INVERSE, s);
    }
    return exec_fft(P, f->h, P->grid.p, P->grid.p, CUFFT_INVERSE, s);
}

// Coil lanes for a call: as many as the coil count asks for, halved until
// the gather and spread shared memory fit the per-CTA limit with the plan's
// tiles (a plan tiled for few coils still runs wide batches, in more chunks).
// Both directions use the same lane count so the scratch bound holds.
template <typename R>
Lanes call_lanes(const gbn_plan* P, int coils) {
    const Geom<R> gg = make_geom<R>(P, false), gs = make_geom<R>(P, true);
    Lanes ln = make_lanes(P->geom.ndim, coils);
    while (ln.LS > 1 && (gather_smem<R>(gg, ln) > SMEM_LIMIT || spread_smem<R>(gs, ln) > SMEM_LIMIT))
        ln = make_lanes(P->geom.ndim, ln.LS / 2);
    return ln;
}

template <typename R>
int run_gather(gbn_plan* P, const void* grid, void* y, int coils, bool phases, cudaStream_t s) {
    typedef typename Cx<R>::T C;
    GatherParams<R> p;
    std::memset(&p, 0, sizeof(p));
    p.g = make_geom<R>(P, false);
    p.ln = call_lanes<R>(P, coils);
    p.s = make_list<R>(P, P->glist, P->glen, false);
    p.items = reinterpret_cast<const int4*>(P->gitems.p);
    p.nitems = P->n_gitems;
    p.coils = coils;
    p.foff = reinterpret_cast<const int64_t*>(P->dfoff.p);
    if (phases) internal_layout(P, P->F * coils, p.g);   // the transform's own grid
    p.grid = reinterpret_cast<const C*>(grid);
    p.y = reinterpret_cast<C*>(y);
    p.apply_pb = phases && P->geom.phasing == GBN_PHASING_REAL;
    p.grid_scale = (phases && P->geom.ortho) ? (R)std::sqrt((double)P->Kprod) : (R)1;
    p.apply_ph = phases && P->has_phase;
    p.g.grid_elems = (int64_t)P->F * coils * P->Kprod;
    p.g.sample_elems = (int64_t)coils * P->M_total;
    // work counters of the persistent (3-D) gather launch; unused in 1-D, 2-D
    p.tickets = reinterpret_cast<int*>(P->tickets.p);
    p.chunks = (coils + p.ln.LS - 1) / p.ln.LS;
    GBN_CUDA(launch_gather<R>(p, s), "gather launch");
    return GBN_OK;
}

template <typename R>
int run_spread(gbn_plan* P, const void* y, void* grid, int coils, bool phases, cudaStream_t s) {
    typedef typename Cx<R>::T C;
    int rc = ensure_scratch(P, coils);
    if (rc) return rc;
    SpreadParams<R> p;
    std::memset(&p, 0, sizeof(p));
    p.g = make_geom<R>(P, true);
    p.ln = call_lanes<R>(P, coils);
    p.s = make_list<R>(P, P->slist, P->slen, true);
    p.items = reinterpret_cast<const int4*>(P->sitems.p);
    p.parts = reinterpret_cast<const int2*>(P->sparts.p);
    p.nitems = P->n_sitems;
    p.coils = coils;
    p.foff = reinterpret_cast<const int64_t*>(P->dfoff.p);
    if (phases) internal_layout(P, P->F * coils, p.g);   // the transform's own grid
    p.y = reinterpret_cast<const C*>(y);
    p.grid = reinterpret_cast<C*>(grid);
    p.scratch = reinterpret_cast<C*>(P->scratch.p);
    p.tile_cells = (int64_t)P->Ts[0] * P->Ts[1] * P->Ts[2];
    p.scratch_elems = P->scratch_cap;
    p.chunks = (coils + p.ln.LS - 1) / p.ln.LS;
    p.g.grid_elems = (int64_t)P->F * coils * P->Kprod;
    p.g.sample_elems = (int64_t)coils * P->M_total;
    p.apply_pb = phases && P->geom.phasing == GBN_PHASING_REAL;
    p.apply_ph = phases && P->has_phase;
    GBN_CUDA(launch_spread<R>(p, s), "spread launch");
    if (P->n_rtiles) {
        ReduceParams<R> q;
        std::memset(&q, 0, sizeof(q));
        q.g = p.g;
        q.ln = p.ln;
        q.tiles = reinterpret_cast<const int4*>(P->rtiles.p);
        q.ntiles = P->n_rtiles;
        q.coils = coils;
        q.scratch = p.scratch;
        q.grid = p.grid;
        q.tile_cells = p.tile_cells;
        q.scratch_elems = p.scratch_elems;
        q.apply_pb = p.apply_pb;
        GBN_CUDA(launch_reduce<R>(q, s), "reduce launch");
    }
    return GBN_OK;
}

// The spread of run_spread with the split-tile partial sums kept in the
// fixed no-alloc array instead of the plan's scratch buffer.  Nothing here
// allocates: the size check happens before any launch, and the array's
// address comes from a lookup on the current device at every call.
template <typename R>
int run_spread_noalloc(gbn_plan* P, const void* y, void* grid, int coils, cudaStream_t s) {
    typedef typename Cx<R>::T C;
    void* scratch = nullptr;
    size_t cap = 0;
    cudaError_t e = noalloc_scratch(&scratch, &cap);
    if (e != cudaSuccess) return cuda_fail(e, "no-alloc scratch address lookup");
    const Lanes ln = call_lanes<R>(P, coils);
    const int64_t tile_cells = (int64_t)P->Ts[0] * P->Ts[1] * P->Ts[2];
    const int64_t chunks = (coils + ln.LS - 1) / ln.LS;
    const int64_t need = (int64_t)P->n_slots * chunks * ln.LS * tile_cells * 2 * (int64_t)P->rsize;
    if (need > (int64_t)cap) {
        char msg[256];
        std::snprintf(msg, sizeof(msg),
                      "no-alloc adjoint needs %lld bytes of scratch for %d coils but its fixed array "
                      "holds %zu; call with fewer coils or use gbn_interp_adjoint",
                      (long long)need, coils, cap);
        return fail(GBN_ERR_TOOLARGE, msg);
    }
    SpreadParams<R> p;
    std::memset(&p, 0, sizeof(p));
    p.g = make_geom<R>(P, true);
    p.ln = ln;
    p.s = make_list<R>(P, P->slist, P->slen, true);
    p.items = reinterpret_cast<const int4*>(P->sitems.p);
    p.parts = reinterpret_cast<const int2*>(P->sparts.p);
    p.nitems = P->n_sitems;
    p.coils = coils;
    p.foff = reinterpret_cast<const int64_t*>(P->dfoff.p);
    p.y = reinterpret_cast<const C*>(y);
    p.grid = reinterpret_cast<C*>(grid);
    p.scratch = reinterpret_cast<C*>(scratch);
    p.tile_cells = tile_cells;
    p.scratch_elems = (int64_t)(cap / sizeof(C));
    p.chunks = (coils + ln.LS - 1) / ln.LS;
    p.g.grid_elems = (int64_t)P->F * coils * P->Kprod;
    p.g.sample_elems = (int64_t)coils * P->M_total;
    p.apply_pb = 0;
    p.apply_ph = 0;
    GBN_CUDA(launch_spread<R>(p, s), "no-alloc spread launch");
    if (P->n_rtiles) {
        ReduceParams<R> q;
        std::memset(&q, 0, sizeof(q));
        q.g = p.g;
        q.ln = p.ln;
        q.tiles = reinterpret_cast<const int4*>(P->rtiles.p);
        q.ntiles = P->n_rtiles;
        q.coils = coils;
        q.scratch = p.scratch;
        q.grid = p.grid;
        q.tile_cells = p.tile_cells;
        q.scratch_elems = p.scratch_elems;
        q.apply_pb = 0;
        GBN_CUDA(launch_reduce<R>(q, s), "no-alloc reduce launch");
    }
    return GBN_OK;
}

template <typename R>
int run_forward(gbn_plan* P, const void* x, void* y, int coils, cudaStream_t s, const void* maps = nullptr) {
    int rc = ensure_buffers(P, coils, P->rowfft && !maps);
    if (rc) return rc;
    if (!P->pad.p || !P->grid.p) return fail(GBN_ERR_NOMEM, "transform buffers missing");
    const gbn_geometry& G = P->geom;
    PadParams<R> pp;
    std::memset(&pp, 0, sizeof(pp));
    pp.ndim = G.ndim;
    for (int d = 0; d < 3; ++d) {
        pp.N[d] = d < G.ndim ? G.Nd[d] : 1;
        pp.K[d] = d < G.ndim ? G.Kd[d] : 1;
    }
    pp.Nprod = P->Nprod;
    pp.Kprod = P->Kprod;
    pp.planes = P->F * coils;
    pp.x = reinterpret_cast<const typename Cx<R>::T*>(x);
    pp.sn = reinterpret_cast<const R*>(P->sn.p);
    pp.out = reinterpret_cast<typename Cx<R>::T*>(P->pad.p);
    pp.maps = reinterpret_cast<const typename Cx<R>::T*>(maps);
    pp.coils = coils;
    pp.check = reinterpret_cast<unsigned*>(P->check.p);
    pp.x_elems = (int64_t)(maps ? P->F : P->F * coils) * P->Nprod;
    pp.out_elems = (int64_t)P->cap_planes * P->Kprod;
    internal_layout(P, P->F * coils, pp);
    if (P->rowfft && !maps) {
        // single precision only (rowfft is off for double plans); 2-D rows
        // into mid, 3-D rows into the grid, whose passes run in place
        {
            NvtxRange r("gbn forward: pad + fft");
            const int planes = P->F * coils;
            const bool d2 = G.ndim == 2;
            if ((rc = run_rowfft(P, x, pp.x_elems, d2 ? P->mid.p : P->grid.p,
                                 (int64_t)(d2 ? P->mid_planes : P->cap_planes) * P->Kprod, planes, -1, s)))
                return rc;
            if ((rc = d2 ? colfft_2d(P, planes, -1, s) : colfft_3d(P, planes, -1, s))) return rc;
        }
        NvtxRange r("gbn forward: gather");
        return run_gather<R>(P, P->grid.p, y, coils, true, s);
    }
    {
        NvtxRange r("gbn forward: pad");
        GBN_CUDA(launch_pad<R>(pp, s), "pad launch");
    }
    {
        NvtxRange r("gbn forward: fft");
        if ((rc = fft_forward(P, P->F * coils, s))) return rc;
    }
    NvtxRange r("gbn forward: gather");
    return run_gather<R>(P, P->grid.p, y, coils, true, s);
}

template <typename R>
int run_adjoint(gbn_plan* P, const void* y, void* x, int coils, cudaStream_t s, const void* maps = nullptr) {
    // allocate first: the grid pointer handed to the spread must be the
    // buffer this call will use (it is null before the first call)
    int rc = ensure_buffers(P, coils, P->rowfft && !maps);
    if (rc) return rc;
    if (!P->grid.p) return fail(GBN_ERR_NOMEM, "grid buffer missing");
    {
        NvtxRange r("gbn adjoint: spread");
        rc = run_spread<R>(P, y, P->grid.p, coils, true, s);
        if (rc) return rc;
    }
    if (P->rowfft && !maps) {
        NvtxRange r("gbn adjoint: fft + crop");
        if ((rc = P->geom.ndim == 2 ? colfft_2d(P, P->F * coils, 1, s) : colfft_3d(P, P->F * coils, 1, s)))
            return rc;
        return run_rowfft(P, P->grid.p, (int64_t)P->cap_planes * P->Kprod, x, (int64_t)P->F * coils * P->Nprod,
                          P->F * coils, 1, s);
    }
    {
        NvtxRange r("gbn adjoint: fft");
        if ((rc = fft_inverse(P, P->F * coils, s))) return rc;
    }
    const gbn_geometry& G = P->geom;
    CropParams<R> cp;
    std::memset(&cp, 0, sizeof(cp));
    cp.ndim = G.ndim;
    for (int d = 0; d < 3; ++d) {
        cp.N[d] = d < G.ndim ? G.Nd[d] : 1;
        cp.K[d] = d < G.ndim ? G.Kd[d] : 1;
    }
    cp.Nprod = P->Nprod;
    cp.Kprod = P->Kprod;
    cp.planes = P->F * coils;
    cp.grid = reinterpret_cast<const typename Cx<R>::T*>(P->grid.p);
    cp.sn = reinterpret_cast<const R*>(P->sn.p);
    cp.scale = G.ortho ? (R)(G.adjoint_scale / std::sqrt((double)P->Kprod)) : (R)G.adjoint_scale;
    cp.x = reinterpret_cast<typename Cx<R>::T*>(x);
    cp.maps = reinterpret_cast<const typename Cx<R>::T*>(maps);
    cp.coils = coils;
    cp.check = reinterpret_cast<unsigned*>(P->check.p);
    cp.x_elems = (int64_t)(maps ? P->F : P->F * coils) * P->Nprod;
    cp.grid_elems = (int64_t)P->cap_planes * P->Kprod;
    internal_layout(P, P->F * coils, cp);
    NvtxRange r("gbn adjoint: crop");
    GBN_CUDA(launch_crop<R>(cp, s), "crop launch");
    return GBN_OK;
}

// ---------------------------------------------------------------------------
// Host-buffer transforms.  One call copies the input to the device,
// transforms it and copies the result back, returning once the result is in
// host memory.  A single-frame batch of 2 * HOST_CHUNK coils or more runs as
// a pipeline of HOST_CHUNK-coil chunks: all chunks' input copies are queued
// on one copy stream and their transforms on the caller's stream (chunk k
// waits for its own copy only), then the output copies on a second copy
// stream, each waiting for its chunk's transform.  So chunk k is transformed
// while chunk k + 1 is copied in and chunk k - 1 copied out.  16 coils keep
// the batched kernels efficient (half the batch costs 0.6-0.7 of the full
// one) while halving the exposed copy at each end; the forward starts with
// two 8-coil chunks, since its output (the samples, 3x the image at the 2-D
// workload) is the longer copy and starts sooner (forward 0.477 -> 0.459 ms
// at 32 coils).  Every copy runs on the copy engines, pageable memory too:
// reading pageable input with SM loads (the device can, over NVLink-C2C) ran
// at the same 203 GB/s but took SMs from the transforms (0.491 against
// 0.477 ms).
constexpr int HOST_CHUNK = 16;

int host_io_init(gbn_plan* P, int nev) {
    HostIo& h = P->hio;
    if (!h.h2d) GBN_CUDA(cudaStreamCreateWithFlags(&h.h2d, cudaStreamNonBlocking), "copy stream");
    if (!h.d2h) GBN_CUDA(cudaStreamCreateWithFlags(&h.d2h, cudaStreamNonBlocking), "copy stream");
    while ((int)h.ev.size() < nev) {
        cudaEvent_t e;
        GBN_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "copy event");
        h.ev.push_back(e);
    }
    return GBN_OK;
}

// cudaMemoryTypeUnregistered for pageable host memory, cudaMemoryTypeHost for
// pinned or registered memory.
int host_kind(const void* p, cudaMemoryType* kind) {
    cudaPointerAttributes a;
    GBN_CUDA(cudaPointerGetAttributes(&a, p), "pointer attributes");
    if (a.type == cudaMemoryTypeDevice) return fail(GBN_ERR_INVALID, "host-buffer transforms take host memory");
    *kind = a.type;
    return GBN_OK;
}

int grow(DevBuf& b, size_t bytes, const char* what) {
    bytes = std::max<size_t>(bytes, 256);
    if (b.bytes >= bytes) return GBN_OK;
    if (b.alloc(bytes) != cudaSuccess) return fail(GBN_ERR_NOMEM, what);
    return GBN_OK;
}

template <typename R>
int run_host(gbn_plan* P, bool forward, const void* in, void* out, int coils, cudaStream_t s) {
    const size_t csz = (size_t)2 * P->rsize;
    const size_t img = (size_t)P->F * P->Nprod * csz, smp = (size_t)P->M_total * csz;   // per coil
    const size_t in_per = forward ? img : smp, out_per = forward ? smp : img;
    // chunk k covers coils [cstart[k], cstart[k + 1])
    std::vector<int> cstart{0};
    if (P->F == 1 && coils >= 2 * HOST_CHUNK) {
        // the forward's first two chunks are half size: its output (the
        // samples) starts copying out sooner
        while (cstart.back() < coils) {
            const int k = (int)cstart.size() - 1;
            const int want = (forward && k < 2) ? HOST_CHUNK / 2 : HOST_CHUNK;
            cstart.push_back(std::min(coils, cstart.back() + want));
        }
    } else {
        cstart.push_back(coils);
    }
    const int nchunks = (int)cstart.size() - 1;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    GBN_CUDA(cudaStreamIsCapturing(s, &cs), "capture status");
    if (cs != cudaStreamCaptureStatusNone)
        return fail(GBN_ERR_UNSUPPORTED, "host-buffer transforms cannot be captured into a graph");
    cudaMemoryType kin = cudaMemoryTypeHost, kout = cudaMemoryTypeHost;
    int rc;
    if (in_per && (rc = host_kind(in, &kin))) return rc;
    if (out_per && (rc = host_kind(out, &kout))) return rc;
    if ((rc = host_io_init(P, 2 * nchunks + 2))) return rc;
    HostIo& h = P->hio;
    // staging is idle here: every host-buffer call waits for its copies
    if ((rc = grow(h.in, in_per * coils, "host input staging allocation failed"))) return rc;
    if ((rc = grow(h.out, out_per * coils, "host output staging allocation failed"))) return rc;
    char* din = static_cast<char*>(h.in.p);
    char* dout = static_cast<char*>(h.out.p);
    cudaEvent_t* ev = h.ev.data();
    // the copies follow work already queued on the caller's stream
    GBN_CUDA(cudaEventRecord(ev[0], s), "event record");
    GBN_CUDA(cudaStreamWaitEvent(h.h2d, ev[0], 0), "stream wait");
    GBN_CUDA(cudaStreamWaitEvent(h.d2h, ev[0], 0), "stream wait");
    int issued = 0;
    for (int k = 0; k < nchunks && rc == GBN_OK; ++k) {
        const int c0 = cstart[k], n = cstart[k + 1] - c0;
        const size_t off = (size_t)c0 * in_per, bytes = (size_t)n * in_per;
        cudaError_t e = cudaSuccess;
        if (bytes)
            e = cudaMemcpyAsync(din + off, static_cast<const char*>(in) + off, bytes, cudaMemcpyHostToDevice, h.h2d);
        if (e == cudaSuccess) e = cudaEventRecord(ev[1 + 2 * k], h.h2d);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(s, ev[1 + 2 * k], 0);
        if (e != cudaSuccess) {
            rc = cuda_fail(e, "host-to-device copy");
            break;
        }
        char* xin = din + off;
        char* xout = dout + (size_t)c0 * out_per;
        rc = forward ? run_forward<R>(P, xin, xout, n, s) : run_adjoint<R>(P, xin, xout, n, s);
        if (rc) break;
        e = cudaEventRecord(ev[2 + 2 * k], s);
        if (e != cudaSuccess) rc = cuda_fail(e, "event record");
        issued = k + 1;
    }
    for (int k = 0; k < issued && rc == GBN_OK; ++k) {
        const int c0 = cstart[k], n = cstart[k + 1] - c0;
        const size_t off = (size_t)c0 * out_per, bytes = (size_t)n * out_per;
        cudaError_t e = cudaStreamWaitEvent(h.d2h, ev[2 + 2 * k], 0);
        if (e == cudaSuccess && bytes)
            e = cudaMemcpyAsync(static_cast<char*>(out) + off, dout + off, bytes, cudaMemcpyDeviceToHost, h.d2h);
        if (e != cudaSuccess) rc = cuda_fail(e, "device-to-host copy");
    }
    cudaEvent_t done = ev[2 * nchunks + 1];
    if (rc == GBN_OK) {
        cudaError_t e = cudaEventRecord(done, h.d2h);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(s, done, 0);   // the caller's stream sees the result
        if (e == cudaSuccess) e = cudaEventSynchronize(done);
        if (e != cudaSuccess) rc = cuda_fail(e, "host-buffer transform");
    }
    if (rc != GBN_OK) {
        // leave no copy in flight on the caller's memory
        cudaStreamSynchronize(h.h2d);
        cudaStreamSynchronize(s);
        cudaStreamSynchronize(h.d2h);
    }
    return rc;
}


template <typename R>
int upload_static(gbn_plan* P, const void* const* h_re, const void* const* h_im, const void* sn) {
    const gbn_geometry& G = P->geom;
    size_t total = 0;
    for (int d = 0; d < G.ndim; ++d) total += (size_t)G.Jd[d] * G.L + 1 + 4;
    const size_t n_tab = P->cx ? 2 * total : total;
    std::vector<R> host(n_tab, (R)0);
    size_t off = 0;
    for (int part = 0; part < (P->cx ? 2 : 1); ++part) {
        for (int d = 0; d < G.ndim; ++d) {
            const size_t len = (size_t)G.Jd[d] * G.L + 1;
            const R* src = reinterpret_cast<const R*>(part == 0 ? h_re[d] : h_im[d]);
            if (!src) return fail(GBN_ERR_INVALID, "missing lookup table");
            std::memcpy(host.data() + off + 2, src, len * sizeof(R));
            off += len + 4;
        }
    }
    cudaError_t e = P->tables.alloc(n_tab * sizeof(R));
    if (e != cudaSuccess) return cuda_fail(e, "table allocation");
    GBN_CUDA(cudaMemcpy(P->tables.p, host.data(), n_tab * sizeof(R), cudaMemcpyHostToDevice), "table upload");
    e = P->sn.alloc((size_t)P->Nprod * sizeof(R));
    if (e != cudaSuccess) return cuda_fail(e, "sn allocation");
    if (!sn) return fail(GBN_ERR_INVALID, "missing deapodisation array");
    GBN_CUDA(cudaMemcpy(P->sn.p, sn, (size_t)P->Nprod * sizeof(R), cudaMemcpyHostToDevice), "sn upload");
    e = P->dfoff.alloc(P->foff.size() * sizeof(int64_t));
    if (e != cudaSuccess) return cuda_fail(e, "offset allocation");
    GBN_CUDA(cudaMemcpy(P->dfoff.p, P->foff.data(), P->foff.size() * sizeof(int64_t), cudaMemcpyHostToDevice),
             "offset upload");
    return GBN_OK;
}

int validate(const gbn_geometry* g) {
    if (!g) return fail(GBN_ERR_INVALID, "null geometry");
    if (g->ndim < 1 || g->ndim > 3) return fail(GBN_ERR_UNSUPPORTED, "ndim must be 1, 2 or 3");
    if (g->precision != GBN_PRECISION_SINGLE && g->precision != GBN_PRECISION_DOUBLE)
        return fail(GBN_ERR_INVALID, "precision must be single or double");
    if (g->phasing != GBN_PHASING_REAL && g->phasing != GBN_PHASING_COMPLEX)
        return fail(GBN_ERR_INVALID, "phasing must be real or complex");
    if (g->L < 1) return fail(GBN_ERR_INVALID, "table oversampling L must be >= 1");
    if (g->n_frames < 1) return fail(GBN_ERR_INVALID, "n_frames must be >= 1");
    if (g->max_coils < 1) return fail(GBN_ERR_INVALID, "max_coils must be >= 1");
    int64_t K = 1;
    for (int d = 0; d < g->ndim; ++d) {
        if (g->Nd[d] < 1 || g->Kd[d] < 1) return fail(GBN_ERR_INVALID, "sizes must be positive");
        if (g->Kd[d] < g->Nd[d]) return fail(GBN_ERR_INVALID, "Kd must be >= Nd on every axis");
        if (g->Jd[d] < 1) return fail(GBN_ERR_INVALID, "kernel width J must be >= 1");
        if (g->Jd[d] > JMAX) return fail(GBN_ERR_UNSUPPORTED, "kernel width J > 8 is not built");
        if (g->Jd[d] > g->Kd[d]) return fail(GBN_ERR_INVALID, "kernel width J exceeds Kd");
        if (g->tile[d] < 0) return fail(GBN_ERR_INVALID, "tile edges must be >= 0");
        K *= g->Kd[d];
        if (g->pb_order[d] < 0 || g->pb_order[d] >= g->ndim)
            return fail(GBN_ERR_INVALID, "pb_order entries must name axes");
    }
    if (K > INT32_MAX) return fail(GBN_ERR_TOOLARGE, "prod(Kd) must be < 2^31");
    if ((int64_t)g->L * JMAX > (1 << 28)) return fail(GBN_ERR_TOOLARGE, "table too long");
    return GBN_OK;
}

// Precompute both lists' interpolation coefficients (list order): from the
// sparse-mode weights when set, else from the tables unless the geometry
// asks for table interpolation inside the kernels (GBN_FLAG_TABLE_ONLY).
template <typename R>
int fill_coefs(gbn_plan* P, cudaStream_t stream = 0, bool sync = true) {
    P->coefs = false;
    const gbn_geometry& G = P->geom;
    if (!P->weights.p && (G.flags & GBN_FLAG_TABLE_ONLY)) {
        GBN_CUDA(P->gcoef.alloc(0), "coefficient release");
        GBN_CUDA(P->scoef.alloc(0), "coefficient release");
        return GBN_OK;
    }
    int jsum = 0;
    for (int d = 0; d < G.ndim; ++d) jsum += G.Jd[d];
    const size_t parts = P->cx ? 2 : 1;
    const size_t gb = (size_t)P->glen * jsum * parts * sizeof(R);
    const size_t sb = (size_t)P->slen * jsum * parts * sizeof(R);
    GBN_CUDA(P->gcoef.alloc(std::max<size_t>(gb, 16)), "gather coefficient allocation");
    GBN_CUDA(P->scoef.alloc(std::max<size_t>(sb, 16)), "spread coefficient allocation");
    for (int which = 0; which < 2; ++which) {
        const bool spread = which == 1;
        CoefParams<R> c;
        std::memset(&c, 0, sizeof(c));
        c.g = make_geom<R>(P, spread);
        c.s = make_list<R>(P, spread ? P->slist : P->glist, spread ? P->slen : P->glen, spread);
        c.items = reinterpret_cast<const int4*>(spread ? P->sitems.p : P->gitems.p);
        c.nitems = spread ? P->n_sitems : P->n_gitems;
        c.foff = reinterpret_cast<const int64_t*>(P->dfoff.p);
        if (P->weights.p) {
            const R* w = reinterpret_cast<const R*>(P->weights.p);
            size_t woff = 0;
            for (int d = 0; d < G.ndim; ++d) {
                c.wr[d] = w + woff;
                woff += (size_t)P->M_total * G.Jd[d];
            }
            for (int d = 0; d < G.ndim && P->cx; ++d) {
                c.wi[d] = w + woff;
                woff += (size_t)P->M_total * G.Jd[d];
            }
        }
        const int64_t len = spread ? P->slen : P->glen;
        c.out_r = reinterpret_cast<R*>(spread ? P->scoef.p : P->gcoef.p);
        c.out_i = P->cx ? c.out_r + (size_t)len * jsum : nullptr;
        c.jsum = jsum;
        c.cx = P->cx ? 1 : 0;
        GBN_CUDA(launch_coef<R>(c, stream), "coefficient launch");
    }
    if (sync) GBN_CUDA(cudaDeviceSynchronize(), "coefficient precompute");
    P->coefs = true;
    return GBN_OK;
}

template <typename R>
int plan_points(gbn_plan* P, const void* tm, const void* phase) {
    if (!tm && P->M_total > 0) return fail(GBN_ERR_INVALID, "null coordinate array");
    P->has_phase = phase != nullptr;
    int rc = build_lists<R>(P, reinterpret_cast<const R*>(tm), reinterpret_cast<const R*>(phase));
    if (rc) return rc;
    return fill_coefs<R>(P);
}

}  // namespace

// ---------------------------------------------------------------------------
// Device binning: the lists of build_lists built by kernels (gbn_bin.cu,
// gbn_sort.cu) from device coordinates.  Two small reads come back to the
// host (the entry count, to size the spread list, and the item counts, to
// size the launches); the coordinates and lists stay on the device.
namespace {

// Bump allocation of 256-byte aligned pieces of a workspace; with a null
// base it only sums the sizes (sizing pass).
struct Bump {
    char* base;
    size_t off = 0;
    explicit Bump(void* b) : base(reinterpret_cast<char*>(b)) {}
    template <typename T>
    T* take(int64_t n) {
        T* p = base ? reinterpret_cast<T*>(base + off) : nullptr;
        off += ((size_t)std::max<int64_t>(n, 1) * sizeof(T) + 255) & ~(size_t)255;
        return p;
    }
};

int bits_for(int64_t n) {
    int b = 0;
    while ((int64_t(1) << b) < n) ++b;
    return std::max(b, 1);
}

template <typename R>
int device_build_lists(gbn_plan* P, const R* tm, const typename Cx<R>::T* ph, cudaStream_t s) {
    typedef typename Cx<R>::T C;
    const gbn_geometry& G = P->geom;
    const int ndim = G.ndim;
    const int64_t M = P->M_total;
    const int ntg = P->ntiles_g, nts = P->ntiles_s;
    const int64_t nbg = (int64_t)P->F * ntg, nbs = (int64_t)P->F * nts;
    int64_t bound = M;
    for (int d = 0; d < ndim; ++d) bound *= G.Jd[d];
    if (bound > INT32_MAX || nbg > INT32_MAX / 2 || nbs > INT32_MAX / 2)
        return fail(GBN_ERR_TOOLARGE, "device binning: more than 2^31 possible list entries");
    const int SCH = spread_part_entries(ndim);

    // ---- phase A: per-sample tiles and entry counts ----------------------
    const int64_t nmax = std::max<int64_t>(std::max<int64_t>(M, nbg), nbs);
    int *err, *tot, *ecount, *eoff;
    unsigned *gkey, *gval;
    void* scan_tmp;
    auto layout_a = [&](Bump& b) {
        err = b.take<int>(16);
        tot = b.take<int>(16);
        gkey = b.take<unsigned>(M);
        gval = b.take<unsigned>(M);
        ecount = b.take<int>(M);
        eoff = b.take<int>(M);
        scan_tmp = b.take<char>((int64_t)scan_temp_bytes(nmax));
    };
    {
        Bump sz(nullptr);
        layout_a(sz);
        if (sz.off > P->bin_ws.bytes) {
            cudaError_t e = P->bin_ws.alloc(sz.off);
            if (e != cudaSuccess) return cuda_fail(e, "binning workspace");
        }
        Bump b(P->bin_ws.p);
        layout_a(b);
    }
    BinParams<R> bp;
    std::memset(&bp, 0, sizeof(bp));
    bp.ndim = ndim;
    bp.F = P->F;
    for (int d = 0; d < 3; ++d) {
        bp.K[d] = d < ndim ? G.Kd[d] : 1;
        bp.J[d] = d < ndim ? G.Jd[d] : 1;
        bp.Tg[d] = P->Tg[d];
        bp.ntg[d] = P->ntg[d];
        bp.Ts[d] = P->Ts[d];
        bp.nts[d] = P->nts[d];
    }
    bp.ntiles_g = ntg;
    bp.ntiles_s = nts;
    bp.tm_limit = TM_LIMIT;
    bp.M = M;
    bp.tm = tm;
    bp.foff = reinterpret_cast<const int64_t*>(P->dfoff.p);
    bp.err = err;
    bp.gkey = gkey;
    bp.gval = gval;
    bp.ecount = ecount;
    bp.eoff = eoff;
    GBN_CUDA(cudaMemsetAsync(err, 0, 32 * sizeof(int), s), "binning reset");
    GBN_CUDA(launch_bin_count<R>(bp, s), "bin count launch");
    GBN_CUDA(exclusive_scan(ecount, eoff, M, tot, scan_tmp, s), "entry scan");
    int hA[2] = {0, 0};
    GBN_CUDA(cudaMemcpyAsync(&hA[0], err, sizeof(int), cudaMemcpyDeviceToHost, s), "binning readback");
    GBN_CUDA(cudaMemcpyAsync(&hA[1], tot, sizeof(int), cudaMemcpyDeviceToHost, s), "binning readback");
    GBN_CUDA(cudaStreamSynchronize(s), "binning readback");
    if (hA[0]) return fail(GBN_ERR_INVALID, "sample coordinate is not finite or |tm| > 2^22");
    const int64_t slen = hA[1];

    // ---- phase B: spread entries, sorts, bins, items ---------------------
    const int64_t nsort = std::max<int64_t>(std::max<int64_t>(M, slen), nbs);
    const int64_t nitem_max = nbg + M / GATHER_CHUNK + 1 + nbs + slen / SCH + 1;
    unsigned *skey, *sval, *gsize, *gorder, *ssize, *sorder;
    int *em, *cg, *cs, *sg, *ss, *gp, *sp, *rs, *rf, *go, *so, *slo, *ro;
    short4* els;
    int4 *gi_tmp, *si_tmp;
    int2* sl_tmp;
    void* rtmp;
    auto layout_b = [&](Bump& b) {
        skey = b.take<unsigned>(slen);
        sval = b.take<unsigned>(slen);
        em = b.take<int>(slen);
        els = b.take<short4>(slen);
        cg = b.take<int>(nbg);
        cs = b.take<int>(nbs);
        sg = b.take<int>(nbg);
        ss = b.take<int>(nbs);
        gp = b.take<int>(nbg);
        sp = b.take<int>(nbs);
        rs = b.take<int>(nbs);
        rf = b.take<int>(nbs);
        go = b.take<int>(nbg);
        so = b.take<int>(nbs);
        slo = b.take<int>(nbs);
        ro = b.take<int>(nbs);
        gi_tmp = b.take<int4>(nitem_max);
        si_tmp = b.take<int4>(nitem_max);
        sl_tmp = b.take<int2>(nitem_max);
        gsize = b.take<unsigned>(nitem_max);
        gorder = b.take<unsigned>(nitem_max);
        ssize = b.take<unsigned>(nitem_max);
        sorder = b.take<unsigned>(nitem_max);
        rtmp = b.take<char>((int64_t)radix_temp_bytes(nsort));
    };
    {
        Bump sz(nullptr);
        layout_b(sz);
        if (sz.off > P->bin_ws2.bytes) {
            cudaError_t e = P->bin_ws2.alloc(sz.off);
            if (e != cudaSuccess) return cuda_fail(e, "binning workspace");
        }
        Bump b(P->bin_ws2.p);
        layout_b(b);
    }
    bp.skey = skey;
    bp.sval = sval;
    bp.em = em;
    bp.els = els;
    GBN_CUDA(launch_bin_emit<R>(bp, s), "bin emit launch");
    GBN_CUDA(radix_sort_pairs(gkey, gval, M, bits_for(nbg), rtmp, s), "gather sort");
    GBN_CUDA(radix_sort_pairs(skey, sval, slen, bits_for(nbs), rtmp, s), "spread sort");
    GBN_CUDA(cudaMemsetAsync(cg, 0, sizeof(int) * nbg, s), "bin count reset");
    GBN_CUDA(cudaMemsetAsync(cs, 0, sizeof(int) * nbs, s), "bin count reset");
    GBN_CUDA(launch_bin_hist(gkey, M, cg, s), "gather bin counts");
    GBN_CUDA(launch_bin_hist(skey, slen, cs, s), "spread bin counts");
    GBN_CUDA(exclusive_scan(cg, sg, nbg, nullptr, scan_tmp, s), "gather bin scan");
    GBN_CUDA(exclusive_scan(cs, ss, nbs, nullptr, scan_tmp, s), "spread bin scan");
    ItemParams ip;
    std::memset(&ip, 0, sizeof(ip));
    ip.nbins_g = (int)nbg;
    ip.nbins_s = (int)nbs;
    ip.ntiles_g = ntg;
    ip.ntiles_s = nts;
    ip.gchunk = GATHER_CHUNK;
    ip.schunk = SCH;
    ip.gcnt = cg;
    ip.gstart = sg;
    ip.scnt = cs;
    ip.sstart = ss;
    ip.gparts = gp;
    ip.sparts = sp;
    ip.rslots = rs;
    ip.rflag = rf;
    GBN_CUDA(launch_bin_parts(ip, s), "bin parts launch");
    GBN_CUDA(exclusive_scan(gp, go, nbg, tot + 1, scan_tmp, s), "gather item scan");
    GBN_CUDA(exclusive_scan(sp, so, nbs, tot + 2, scan_tmp, s), "spread item scan");
    GBN_CUDA(exclusive_scan(rs, slo, nbs, tot + 3, scan_tmp, s), "slot scan");
    GBN_CUDA(exclusive_scan(rf, ro, nbs, tot + 4, scan_tmp, s), "split tile scan");
    int hB[4] = {0, 0, 0, 0};
    GBN_CUDA(cudaMemcpyAsync(hB, tot + 1, 4 * sizeof(int), cudaMemcpyDeviceToHost, s), "binning readback");
    GBN_CUDA(cudaStreamSynchronize(s), "binning readback");
    const int n_gi = hB[0], n_si = hB[1], n_slots = hB[2], n_rt = hB[3];
    auto ensure = [&](DevBuf& b, size_t bytes, const char* what) -> int {
        bytes = std::max<size_t>(bytes, 16);
        if (b.bytes < bytes) {
            cudaError_t e = b.alloc(bytes);
            if (e != cudaSuccess) return cuda_fail(e, what);
        }
        return GBN_OK;
    };
    int rc;
    if ((rc = ensure(P->gitems, (size_t)n_gi * sizeof(int4), "item allocation"))) return rc;
    if ((rc = ensure(P->sitems, (size_t)n_si * sizeof(int4), "item allocation"))) return rc;
    if ((rc = ensure(P->sparts, (size_t)n_si * sizeof(int2), "item allocation"))) return rc;
    if ((rc = ensure(P->rtiles, (size_t)n_rt * sizeof(int4), "item allocation"))) return rc;
    ip.goff = go;
    ip.soff = so;
    ip.slotoff = slo;
    ip.roff = ro;
    ip.gitems = gi_tmp;
    ip.gsize = gsize;
    ip.gorder = gorder;
    ip.sitems = si_tmp;
    ip.sslot = sl_tmp;
    ip.ssize = ssize;
    ip.sorder = sorder;
    ip.rtiles = reinterpret_cast<int4*>(P->rtiles.p);
    GBN_CUDA(launch_bin_items(ip, s), "bin items launch");
    // heaviest first, ties in bin order (a stable sort by chunk - count), as
    // the host planner's stable_sort
    GBN_CUDA(radix_sort_pairs(gsize, gorder, n_gi, bits_for(GATHER_CHUNK + 1), rtmp, s), "gather item sort");
    GBN_CUDA(radix_sort_pairs(ssize, sorder, n_si, bits_for(SCH + 1), rtmp, s), "spread item sort");
    GBN_CUDA(launch_permute_int4(gi_tmp, gorder, n_gi, reinterpret_cast<int4*>(P->gitems.p), s), "item order");
    GBN_CUDA(launch_permute_int4(si_tmp, sorder, n_si, reinterpret_cast<int4*>(P->sitems.p), s), "item order");
    GBN_CUDA(launch_permute_int2(sl_tmp, sorder, n_si, reinterpret_cast<int2*>(P->sparts.p), s), "item order");

    // ---- lists (SoA, the layout of build_lists) --------------------------
    P->has_phase = ph != nullptr;
    if ((rc = ensure(P->glist, list_bytes<R>(P, M, false), "list allocation"))) return rc;
    if ((rc = ensure(P->slist, list_bytes<R>(P, slen, true), "list allocation"))) return rc;
    for (int which = 0; which < 2; ++which) {
        const bool spread = which == 1;
        const int64_t len = spread ? slen : M;
        const ListLayout<R> L(P, len, spread);
        char* base = reinterpret_cast<char*>(spread ? P->slist.p : P->glist.p);
        PackParams<R> pk;
        std::memset(&pk, 0, sizeof(pk));
        pk.ndim = ndim;
        pk.F = P->F;
        pk.len = len;
        pk.order = spread ? sval : gval;
        pk.em = spread ? em : nullptr;
        pk.els = spread ? els : nullptr;
        pk.tm = tm;
        pk.ph = ph;
        pk.foff = reinterpret_cast<const int64_t*>(P->dfoff.p);
        pk.ls_out = spread ? reinterpret_cast<short4*>(base + L.ls) : nullptr;
        pk.ph_out = ph ? reinterpret_cast<C*>(base + L.ph) : nullptr;
        for (int d = 0; d < ndim; ++d) pk.t_out[d] = reinterpret_cast<R*>(base + L.t[d]);
        pk.idx_out = reinterpret_cast<int*>(base + L.idx);
        GBN_CUDA(launch_bin_pack<R>(pk, s), "list pack launch");
    }
    P->glen = M;
    P->slen = slen;
    P->n_gitems = n_gi;
    P->n_sitems = n_si;
    P->n_rtiles = n_rt;
    P->n_slots = n_slots;
    return fill_coefs<R>(P, s, false);
}

}  // namespace

namespace {
template <typename R>
int run_grad(gbn_plan* P, const void* grid, const void* gy, const double* shift, void* gtm, int coils,
             cudaStream_t s) {
    typedef typename Cx<R>::T C;
    GradParams<R> p;
    std::memset(&p, 0, sizeof(p));
    p.g = make_geom<R>(P, false);
    internal_layout(P, P->F * coils, p.g);   // the grid a forward call with these coils left
    const SampleList<R> L = make_list<R>(P, P->glist, P->glen, false);
    const R* db = reinterpret_cast<const R*>(P->dtables.p);
    size_t off = 0;
    for (int d = 0; d < P->geom.ndim; ++d) {
        p.t[d] = L.t[d];
        p.dh[d] = db + off + 2;
        off += (size_t)P->geom.Jd[d] * P->geom.L + 1 + 4;
        p.phase_shift[d] = shift ? (R)shift[d] : (R)0;
    }
    p.idx = L.idx;
    p.ph = L.ph;
    p.M = P->glen;
    p.coils = coils;
    p.apply_pb = P->geom.phasing == GBN_PHASING_REAL;
    p.grid_scale = P->geom.ortho ? (R)std::sqrt((double)P->Kprod) : (R)1;
    p.grid = reinterpret_cast<const C*>(grid);
    p.gy = reinterpret_cast<const C*>(gy);
    p.gtm = reinterpret_cast<R*>(gtm);
    GBN_CUDA(launch_grad<R>(p, s), "gradient launch");
    return GBN_OK;
}
}  // namespace

extern "C" {

int gbn_plan_create(gbn_plan** out, const gbn_geometry* geom, const void* const* h_re,
                    const void* const* h_im, const void* sn, const int64_t* frame_offsets,
                    const void* tm, const void* sample_phase, int device) {
    if (!out) return fail(GBN_ERR_INVALID, "null plan pointer");
    *out = nullptr;
    int rc = validate(geom);
    if (rc) return rc;
    if (!h_re || !frame_offsets) return fail(GBN_ERR_INVALID, "null table or offset array");
    DeviceGuard guard(device);
    gbn_plan* P = new (std::nothrow) gbn_plan();
    if (!P) return fail(GBN_ERR_NOMEM, "host allocation failed");
    P->device = device;
    P->geom = *geom;
    P->dbl = geom->precision == GBN_PRECISION_DOUBLE;
    P->rsize = P->dbl ? 8 : 4;
    P->cx = geom->phasing == GBN_PHASING_COMPLEX;
    if (P->cx && (!h_im || !h_im[0])) {
        delete P;
        return fail(GBN_ERR_INVALID, "complex phasing needs imaginary tables");
    }
    P->F = geom->n_frames;
    P->foff.assign(frame_offsets, frame_offsets + P->F + 1);
    if (P->foff[0] != 0) {
        delete P;
        return fail(GBN_ERR_INVALID, "frame_offsets[0] must be 0");
    }
    for (int f = 0; f < P->F; ++f)
        if (P->foff[f + 1] < P->foff[f]) {
            delete P;
            return fail(GBN_ERR_INVALID, "frame offsets must be non-decreasing");
        }
    P->M_total = P->foff[P->F];
    for (int d = 0; d < geom->ndim; ++d) {
        P->Kprod *= geom->Kd[d];
        P->Nprod *= geom->Nd[d];
    }
    choose_tiles(P);
    if ((rc = setup_colfft(P))) {
        delete P;
        return rc;
    }
    {
        cudaError_t e = P->check.alloc(16);
        if (e == cudaSuccess) e = cudaMemset(P->check.p, 0, 16);
        if (e == cudaSuccess) e = P->tickets.alloc(16);
        if (e == cudaSuccess) e = cudaMemset(P->tickets.p, 0, 16);
        if (e != cudaSuccess) {
            delete P;
            return cuda_fail(e, "status word");
        }
    }
    rc = P->dbl ? upload_static<double>(P, h_re, h_im, sn) : upload_static<float>(P, h_re, h_im, sn);
    if (!rc) rc = P->dbl ? plan_points<double>(P, tm, sample_phase) : plan_points<float>(P, tm, sample_phase);
    if (rc) {
        delete P;
        return rc;
    }
    *out = P;
    return GBN_OK;
}

int gbn_plan_set_points(gbn_plan* P, const void* tm, const void* sample_phase) {
    if (!P) return fail(GBN_ERR_INVALID, "null plan");
    std::lock_guard<std::mutex> lk(P->mu);
    DeviceGuard guard(P->device);
    GBN_CUDA(cudaDeviceSynchronize(), "synchronise before replanning");
    // weights belong to the old coordinates
    GBN_CUDA(P->weights.alloc(0), "weight release");
    return P->dbl ? plan_points<double>(P, tm, sample_phase) : plan_points<float>(P, tm, sample_phase);
}

int gbn_plan_set_points_device(gbn_plan* P, const void* tm, const void* sample_phase, void* stream) {
    if (!P) return fail(GBN_ERR_INVALID, "null plan");
    if (!tm && P->M_total > 0) return fail(GBN_ERR_INVALID, "null coordinate array");
    std::lock_guard<std::mutex> lk(P->mu);
    DeviceGuard guard(P->device);
    for (const void* q : {tm, sample_phase}) {
        if (!q) continue;
        cudaPointerAttributes a;
        if (cudaPointerGetAttributes(&a, q) != cudaSuccess || a.type != cudaMemoryTypeDevice) {
            cudaGetLastError();
            return fail(GBN_ERR_INVALID, "gbn_plan_set_points_device takes device pointers");
        }
    }
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    // calls queued before on other streams may still read the lists
    GBN_CUDA(cudaDeviceSynchronize(), "synchronise before replanning");
    GBN_CUDA(P->weights.alloc(0), "weight release");
    return P->dbl ? device_build_lists<double>(P, reinterpret_cast<const double*>(tm),
                                               reinterpret_cast<const double2*>(sample_phase), s)
                  : device_build_lists<float>(P, reinterpret_cast<const float*>(tm),
                                              reinterpret_cast<const float2*>(sample_phase), s);
}

int gbn_plan_destroy(gbn_plan* P) {
    if (!P) return GBN_OK;
    DeviceGuard guard(P->device);
    cudaDeviceSynchronize();
    delete P;
    return GBN_OK;
}

static int check_call(gbn_plan* P, const void* a, const void* b, int coils) {
    if (!P) return fail(GBN_ERR_INVALID, "null plan");
    if (coils < 1) return fail(GBN_ERR_INVALID, "coils must be >= 1");
    if ((!a || !b) && P->M_total > 0) return fail(GBN_ERR_INVALID, "null data pointer");
    if ((int64_t)coils * P->F * P->Kprod > ((int64_t)1 << 40))
        return fail(GBN_ERR_TOOLARGE, "batch too large");
    return GBN_OK;
}

int gbn_forward(gbn_plan* P, const void* x, void* y, int coils, void* stream) {
    int rc = check_call(P, x, y, coils);
    if (rc) return rc;
    if (!x) return fail(GBN_ERR_INVALID, "null image");   // read even without samples
    std::lock_guard<std::mutex> lk(P->mu);
    DeviceGuard guard(P->device);
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    return P->dbl ? run_forward<double>(P, x, y, coils, s) : run_forward<float>(P, x, y, coils, s);
}

int gbn_adjoint(gbn_plan* P, const void* y, void* x, int coils, void* stream) {
    int rc = check_call(P, y, x, coils);
    if (rc) return rc;
    if (!x) return fail(GBN_ERR_INVALID, "null image");   // written even without samples
    std::lock_guard<std::mutex> lk(P->mu);
    DeviceGuard guard(P->device);
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    return P->dbl ? run_adjoint<double>(P, y, x, coils, s) : run_adjoint<float>(P, y, x, coils, s);
}

int gbn_forward_host(gbn_plan* P, const void* x, void* y, int coils, void* stream) {
    int rc = check_call(P, x, y, coils);
    if (rc) return rc;
    if (!x) return fail(GBN_ERR_INVALID, "null image");
    std::lock_guard<std::mutex> lk(P->mu);
    DeviceGuard guard(P->device);
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    return P->dbl ? run_host<double>(P, true, x, y, coils, s) : run_host<float>(P, true, x, y, coils, s);
}

int gbn_adjoint_host(gbn_plan* P, const void* y, void* x, int coils, void* stream) {
    int rc = check_call(P, y, x, coils);
    if (rc) return rc;
    if (!x) return fail(GBN_ERR_INVALID, "null image");
    std::lock_guard<std::mutex> lk(P->mu);
    DeviceGuard guard(P->device);
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    return P->dbl ? run_host<double>(P, false, y, x, coils, s) : run_host<float>(P, false, y, x, coils, s);
}

int gbn_forward_sense(gbn_plan* P, const void* image, const void* maps, void* y, int coils, void* stream) {
    int rc = check_call(P, image, y, coils);
    if (rc) return rc;
    if (!maps || !image) return fail(GBN_ERR_INVALID, "null image or coil maps");
    std::lock_guard<std::mutex> lk(P->mu);
    DeviceGuard guard(P->device);
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    return P->dbl ? run_forward<double>(P, image, y, coils, s, maps) : run_forward<float>(P, image, y, coils, s, maps);
}

int gbn_adjoint_sense(gbn_plan* P, const void* y, const void* maps, void* image, int coils, void* stream) {
    int rc = check_call(P, y, image, coils);
    if (rc) return rc;
    if (!maps || !image) return fail(GBN_ERR_INVALID, "null image or coil maps");
    std::lock_guard<std::mutex> lk(P->mu);
    DeviceGuard guard(P->device);
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    return P->dbl ? run_adjoint<double>(P, y, image, coils, s, maps) : run_adjoint<float>(P, y, image, coils, s, maps);
}

int gbn_interp_forward(gbn_plan* P, const void* grid, void* y, int coils, void* stream) {
    int rc = check_call(P, grid, y, coils);
    if (rc) return rc;
    std::lock_guard<std::mutex> lk(P->mu);
    DeviceGuard guard(P->device);
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    return P->dbl ? run_gather<double>(P, grid, y, coils, false, s)
                  : run_gather<float>(P, grid, y, coils, false, s);
}

int gbn_interp_adjoint(gbn_plan* P, const void* y, void* grid, int coils, void* stream) {
    int rc = check_call(P, y, grid, coils);
    if (rc) return rc;
    if (!grid) return fail(GBN_ERR_INVALID, "null grid");   // written even without samples
    std::lock_guard<std::mutex> lk(P->mu);
    DeviceGuard guard(P->device);
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    return P->dbl ? run_spread<double>(P, y, grid, coils, false, s)
                  : run_spread<float>(P, y, grid, coils, false, s);
}

int gbn_interp_adjoint_noalloc(gbn_plan* P, const void* y, void* grid, int coils, void* stream) {
    int rc = check_call(P, y, grid, coils);
    if (rc) return rc;
    if (!grid) return fail(GBN_ERR_INVALID, "null grid");
    std::lock_guard<std::mutex> lk(P->mu);
    DeviceGuard guard(P->device);
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    return P->dbl ? run_spread_noalloc<double>(P, y, grid, coils, s)
                  : run_spread_noalloc<float>(P, y, grid, coils, s);
}

int gbn_forward_grid(gbn_plan* P, void** grid) {
    if (!P || !grid) return fail(GBN_ERR_INVALID, "null argument");
    *grid = P->grid.p;
    return GBN_OK;
}

int gbn_plan_set_dtables(gbn_plan* P, const void* const* dtab) {
    if (!P || !dtab) return fail(GBN_ERR_INVALID, "null argument");
    std::lock_guard<std::mutex> lk(P->mu);
    DeviceGuard guard(P->device);
    const gbn_geometry& G = P->geom;
    size_t total = 0;
    for (int d = 0; d < G.ndim; ++d) total += (size_t)G.Jd[d] * G.L + 1 + 4;
    std::vector<char> host(total * P->rsize, 0);
    size_t off = 0;
    for (int d = 0; d < G.ndim; ++d) {
        const size_t len = (size_t)G.Jd[d] * G.L + 1;
        if (!dtab[d]) return fail(GBN_ERR_INVALID, "missing derivative table");
        std::memcpy(host.data() + (off + 2) * P->rsize, dtab[d], len * P->rsize);
        off += len + 4;
    }
    cudaError_t e = P->dtables.alloc(host.size());
    if (e != cudaSuccess) return cuda_fail(e, "derivative table allocation");
    GBN_CUDA(cudaMemcpy(P->dtables.p, host.data(), host.size(), cudaMemcpyHostToDevice),
             "derivative table upload");
    return GBN_OK;
}

int gbn_plan_set_weights(gbn_plan* P, const void* const* w_re, const void* const* w_im) {
    if (!P) return fail(GBN_ERR_INVALID, "null plan");
    std::lock_guard<std::mutex> lk(P->mu);
    DeviceGuard guard(P->device);
    GBN_CUDA(cudaDeviceSynchronize(), "synchronise before replacing weights");
    if (!w_re) {
        GBN_CUDA(P->weights.alloc(0), "weight release");
        return P->dbl ? fill_coefs<double>(P) : fill_coefs<float>(P);
    }
    const gbn_geometry& G = P->geom;
    if (P->cx && !w_im) return fail(GBN_ERR_INVALID, "complex phasing needs imaginary weights");
    size_t per = 0;
    for (int d = 0; d < G.ndim; ++d) {
        if (!w_re[d] || (P->cx && !w_im[d])) return fail(GBN_ERR_INVALID, "missing weight array");
        per += (size_t)P->M_total * G.Jd[d];
    }
    const size_t bytes = per * (P->cx ? 2 : 1) * P->rsize;
    if (bytes == 0) return GBN_OK;
    GBN_CUDA(P->weights.alloc(bytes), "weight allocation");
    size_t off = 0;
    for (int part = 0; part < (P->cx ? 2 : 1); ++part)
        for (int d = 0; d < G.ndim; ++d) {
            const size_t n = (size_t)P->M_total * G.Jd[d] * P->rsize;
            const void* src = part == 0 ? w_re[d] : w_im[d];
            GBN_CUDA(cudaMemcpy(static_cast<char*>(P->weights.p) + off, src, n, cudaMemcpyHostToDevice),
                     "weight upload");
            off += n;
        }
    return P->dbl ? fill_coefs<double>(P) : fill_coefs<float>(P);
}

int gbn_grad_tm(gbn_plan* P, const void* grid, const void* gy, const double* phase_shift, void* gtm,
                int coils, void* stream) {
    int rc = check_call(P, grid, gy, coils);
    if (rc) return rc;
    if (!gtm && P->M_total > 0) return fail(GBN_ERR_INVALID, "null gradient output");
    if (P->F != 1) return fail(GBN_ERR_UNSUPPORTED, "coordinate gradient needs a single-frame plan");
    if (P->cx) return fail(GBN_ERR_UNSUPPORTED, "coordinate gradient needs phasing real");
    if (!P->dtables.p) return fail(GBN_ERR_INVALID, "derivative tables not set (gbn_plan_set_dtables)");
    if (P->weights.p) return fail(GBN_ERR_UNSUPPORTED, "coordinate gradient needs table interpolation");
    std::lock_guard<std::mutex> lk(P->mu);
    DeviceGuard guard(P->device);
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    return P->dbl ? run_grad<double>(P, grid, gy, phase_shift, gtm, coils, s)
                  : run_grad<float>(P, grid, gy, phase_shift, gtm, coils, s);
}

int gbn_dtft_forward(int ndim, const int* Nd, const double* n_shift, const void* omega, int64_t M,
                     const void* x, void* y, int reps, void* stream) {
    if (ndim < 1 || ndim > 3 || !Nd || !n_shift || M < 0 || reps < 1)
        return fail(GBN_ERR_INVALID, "bad dtft arguments");
    if (M > 0 && (!omega || !x || !y)) return fail(GBN_ERR_INVALID, "null dtft pointer");
    GBN_CUDA(launch_dtft(false, ndim, Nd, n_shift, (const double*)omega, M, (const double2*)x, (double2*)y, reps,
                         reinterpret_cast<cudaStream_t>(stream)),
             "dtft forward");
    return GBN_OK;
}

int gbn_dtft_adjoint(int ndim, const int* Nd, const double* n_shift, const void* omega, int64_t M,
                     const void* y, void* x, int reps, void* stream) {
    if (ndim < 1 || ndim > 3 || !Nd || !n_shift || M < 0 || reps < 1)
        return fail(GBN_ERR_INVALID, "bad dtft arguments");
    if (!x || (M > 0 && (!omega || !y))) return fail(GBN_ERR_INVALID, "null dtft pointer");
    GBN_CUDA(launch_dtft(true, ndim, Nd, n_shift, (const double*)omega, M, (const double2*)y, (double2*)x, reps,
                         reinterpret_cast<cudaStream_t>(stream)),
             "dtft adjoint");
    return GBN_OK;
}

int gbn_plan_stats(const gbn_plan* P, int64_t* o) {
    if (!P || !o) return fail(GBN_ERR_INVALID, "null argument");
    o[0] = P->n_gitems;
    o[1] = P->n_sitems;
    o[2] = P->n_rtiles;
    o[3] = P->glen;
    o[4] = P->slen;
    o[5] = (int64_t)P->ntiles_s * P->F;
    o[6] = (int64_t)(P->tables.bytes + P->weights.bytes + P->gcoef.bytes + P->scoef.bytes + P->mid.bytes + P->sn.bytes + P->glist.bytes + P->slist.bytes + P->pad.bytes +
                     P->grid.bytes + P->scratch.bytes);
    o[7] = P->M_total;
    return GBN_OK;
}

int gbn_debug_check_status(gbn_plan* P, unsigned* out) {
    if (!P || !out) return fail(GBN_ERR_INVALID, "null argument");
    *out = 0;
#ifdef GBN_CHECKED
    std::lock_guard<std::mutex> lk(P->mu);
    DeviceGuard guard(P->device);
    GBN_CUDA(cudaDeviceSynchronize(), "status read");
    GBN_CUDA(cudaMemcpy(out, P->check.p, sizeof(unsigned), cudaMemcpyDeviceToHost), "status read");
    GBN_CUDA(cudaMemset(P->check.p, 0, sizeof(unsigned)), "status reset");
    return GBN_OK;
#else
    return fail(GBN_ERR_UNSUPPORTED, "bounds checks are compiled only into libgbnufft_checked.so");
#endif
}

const char* gbn_last_error(void) { return g_last_error.c_str(); }

int gbn_debug_fail_alloc(long long after) {
    g_fail_alloc_after.store(after < 0 ? -1 : after);
    return GBN_OK;
}

const char* gbn_version(void) { return "gbnufft 0.1.0 (sm_103a)"; }

}  // extern "C"
