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
//   all LS coils ([cell][coil], padded row), with phase_before and the
//   orthonormal scale applied while staging;
// * a warp prepares 32 samples at a time, one per lane (coefficients,
//   window position, output index, phase), then gathers them SW at a time
//   from shared memory, reading the prepared values by shuffle.
//
// The kernel is compiled generically (run-time kernel width J <= 8 and lane
// count) and, for the common single-precision real-kernel cases, with J and
// the lane count fixed at compile time (no predication, constant strides).
#include <cuda_runtime.h>

#include <algorithm>

#include "gbn_device.cuh"
#include "gbn_internal.h"

namespace gbn {

constexpr int GATHER_THREADS = 256;

// Read one entry's precomputed coefficients (jsum values: the taps of axis
// 0, then axis 1, ...) into per-axis register arrays; 16-byte loads when the
// width is fixed and the entry size is a multiple of 16 bytes.
template <typename R, int NDIM, int JJ, int JL>
__device__ __forceinline__ void load_coefs(const R* src, const Geom<R>& g, R (&c)[NDIM][JL]) {
    if (JJ > 0 && sizeof(R) == 4 && (NDIM * JJ) % 4 == 0) {
        constexpr int NV = (JJ > 0 ? NDIM * JJ : 4) / 4;
        float4 v[NV];
#pragma unroll
        for (int i = 0; i < NV; ++i) v[i] = __ldg(reinterpret_cast<const float4*>(src) + i);
        const float* f = reinterpret_cast<const float*>(v);
#pragma unroll
        for (int d = 0; d < NDIM; ++d)
#pragma unroll
            for (int j = 0; j < JL; ++j) c[d][j] = (R)f[d * JJ + j];
    } else {
        int off = 0;
#pragma unroll
        for (int d = 0; d < NDIM; ++d) {
#pragma unroll
            for (int j = 0; j < JL; ++j)
                if (JJ > 0 || j < g.J[d]) c[d][j] = __ldg(src + off + j);
            off += JJ > 0 ? JJ : g.J[d];
        }
    }
}

// Element-wise staging (per-cell offsets and phases in shared memory, then
// one thread per staged value): the 2-D kernels with 16 or 32 coil lanes
// (2-D workload gather 0.134 -> 0.128 ms).  With 8 lanes the extra shared
// memory cost more than the balanced loads gained (series gather 0.413 ->
// 0.448 ms), and in 3-D it would leave one CTA per SM.
__host__ __device__ constexpr bool gather_elem_staging(int ndim, int lsc) { return ndim == 2 && lsc >= 16; }

// The 3-D kernels run persistent: as many CTAs as are resident at once,
// each taking (work item, coil chunk) tickets in item order, heaviest items
// first, so that the long tail of light items fills the SMs the heavy ones
// leave (3-D kooshball gather 3.88 -> 3.39 ms).  In 2-D one CTA per (item,
// chunk) is as fast or faster: the items are evenly sized there.
// (Written as one loop around the whole body: with the body in a separate
// inlined function the 3-D persistent kernel compiled to 102 instead of 126
// registers and ran at 4.04 ms.)
__host__ __device__ constexpr bool gather_persistent(int ndim) { return ndim == 3; }

template <typename R, int NDIM, bool CX, int JJ, int LSC>
__global__ void __launch_bounds__(GATHER_THREADS)
gather_kernel(const GatherParams<R> p) {
    typedef typename Cx<R>::T C;
    constexpr int JL = JJ > 0 ? JJ : JMAX;    // loop bound of the tap loops
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C* S = reinterpret_cast<C*>(smem_raw);
    const Geom<R>& g = p.g;

    // One (work item, coil chunk) per round: a ticket when persistent, else
    // the CTA's own (blockIdx.x, blockIdx.y) and a single round.
    __shared__ int ticket_slot;
    const int total = p.nitems * p.chunks;
    for (int round = 0;; ++round) {
    int ticket;
    if constexpr (gather_persistent(NDIM)) {
        ticket = next_ticket(p.tickets, &ticket_slot);
    } else {
        if (round > 0) break;
        ticket = blockIdx.x * p.chunks + blockIdx.y;
    }
    if (ticket >= total) break;
    const int item = ticket / p.chunks, chunk = ticket - item * p.chunks;
    const int4 it = p.items[item];
    const int f = it.x, tile = it.y, start = it.z, count = it.w;
    if (!GBN_INB(g.check, start >= 0 && count >= 0 && start + (int64_t)count <= p.s.len, CHK_LIST)) continue;
    const int LS = LSC > 0 ? LSC : p.ln.LS;
    const int lsh = LSC > 0 ? (LSC == 32 ? 5 : LSC == 16 ? 4 : LSC == 8 ? 3 : LSC == 4 ? 2 : LSC == 2 ? 1 : 0)
                            : p.ln.lsh;
    // Tap split (3-D, 8 coil lanes, even width, single precision): a
    // half-warp serves one sample, its two 8-lane halves taking the even and
    // odd taps along axis 0.  Cell rows are 8 coils wide, coil c of a cell at region
    // x-position x stored at slot c ^ (x & 7): the two cells a half-warp
    // reads (x and x + 1) then fill complementary halves of the 16 bank pairs,
    // where two independent samples' padded rows would mostly collide.  In
    // 2-D (36 taps per sample) the extra per-sample shuffles cost more than
    // the conflicts, so 2-D keeps four samples per warp.
    constexpr bool TS = LSC == 8 && NDIM == 3 && JJ > 0 && (JJ % 2) == 0 && sizeof(R) == 4;
    constexpr bool ES = gather_elem_staging(NDIM, LSC);
    const int LSP = TS ? 8 : (LSC > 0 ? (LSC == 1 ? 1 : LSC + 1) : p.ln.LSP);
    const int c0 = chunk << lsh;
    const int nc = min(LS, p.coils - c0);

    int org[3] = {0, 0, 0};
    tile_origin<NDIM>(tile, g.nt, g.T, org);
    int Rd[3];
    const int Rtot = region_dims(g, NDIM, Rd);

    // ---- stage tile + halo for nc coils --------------------------------------
    const C* gb = p.grid + ((int64_t)f * p.coils + c0) * g.gsp;
    if constexpr (ES) {
        // (1) thread per cell: grid offset and phase_before into shared
        // memory; (2) thread per (coil, cell), consecutive threads on
        // consecutive cells, eight independent loads in flight.  Every
        // thread gets the same share of loads, where a thread per cell
        // serialises all the coils of its cells.
        int64_t* soff = reinterpret_cast<int64_t*>(S + (size_t)Rtot * LSP);
        C* sph = reinterpret_cast<C*>(soff + Rtot);
        for (int cell = threadIdx.x; cell < Rtot; cell += blockDim.x) {
            int r[3];
            int rem = cell;
            r[0] = rem % Rd[0];
            rem /= Rd[0];
            r[1] = rem % Rd[1];
            r[2] = rem / Rd[1];
            int k[3] = {0, 0, 0};
#pragma unroll
            for (int d = 0; d < NDIM; ++d) k[d] = wrapk(org[d] + r[d], g.K[d]);
            soff[cell] = k[0] + (int64_t)k[1] * g.gs1 + (int64_t)k[2] * g.gs2;
            if (p.apply_pb) sph[cell] = phase_before(g, k);
        }
        __syncthreads();
        const int E = Rtot * nc;
        const int step = blockDim.x;
        int cell = threadIdx.x, c = 0;
        while (cell >= Rtot && c < nc) cell -= Rtot, ++c;
        for (int e = threadIdx.x; e < E; e += 8 * step) {
            C v[8];
            int cc[8], cl[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                cc[u] = c;
                cl[u] = cell;
                if (e + u * step < E) {
                    const int64_t gi = ((int64_t)f * p.coils + c0 + c) * g.gsp + soff[cell];
                    if (GBN_INB(g.check, gi >= 0 && gi < g.grid_elems, CHK_GRID_READ))
                        v[u] = gb[(int64_t)c * g.gsp + soff[cell]];
                }
                cell += step;
                while (cell >= Rtot) cell -= Rtot, ++c;
            }
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                if (e + u * step < E) {
                    C w = v[u];
                    if (p.apply_pb) w = cmul(w, sph[cl[u]]);
                    if (p.grid_scale != (R)1) {
                        w.x = w.x / p.grid_scale;
                        w.y = w.y / p.grid_scale;
                    }
                    S[cl[u] * LSP + cc[u]] = w;
                }
            }
        }
    } else {
    // thread per cell, coils in batches of four independent loads
    for (int cell = threadIdx.x; cell < Rtot; cell += blockDim.x) {
        int r[3];
        int rem = cell;
        r[0] = rem % Rd[0];
        rem /= Rd[0];
        r[1] = rem % Rd[1];
        r[2] = rem / Rd[1];
        int k[3] = {0, 0, 0};
#pragma unroll
        for (int d = 0; d < NDIM; ++d) k[d] = wrapk(org[d] + r[d], g.K[d]);
        const int64_t off = k[0] + (int64_t)k[1] * g.gs1 + (int64_t)k[2] * g.gs2;
        C ph = cmake<R>((R)1, (R)0);
        if (p.apply_pb) ph = phase_before(g, k);
        const int dst = cell * LSP;
        const C* src = gb + off;
        for (int c = 0; c < nc; c += 4) {
            C v[4];
#pragma unroll
            for (int u = 0; u < 4; ++u)
                if (c + u < nc) {
                    const int64_t gi = ((int64_t)f * p.coils + c0 + c + u) * g.gsp + off;
                    if (GBN_INB(g.check, gi >= 0 && gi < g.grid_elems, CHK_GRID_READ))
                        v[u] = src[(int64_t)(c + u) * g.gsp];
                }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                if (c + u < nc) {
                    C w = v[u];
                    if (p.apply_pb) w = cmul(w, ph);
                    if (p.grid_scale != (R)1) {
                        w.x = w.x / p.grid_scale;
                        w.y = w.y / p.grid_scale;
                    }
                    S[dst + (TS ? ((c + u) ^ (r[0] & 7)) : c + u)] = w;
                }
            }
        }
    }
    }
    __syncthreads();

    // ---- per-sample gather from shared memory -------------------------------
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nwarps = blockDim.x >> 5;
    const int SW = TS ? 2 : 32 >> lsh;
    const int slot = TS ? lane >> 4 : lane >> lsh, coil = lane & (LS - 1);
    const int th = TS ? (lane >> 3) & 1 : 0;   // tap half (tap split)
    const int64_t fo = p.foff[f];
    const int Mf = (int)(p.foff[f + 1] - fo);
    if (!GBN_INB(g.check, (fo + Mf) * p.coils <= g.sample_elems, CHK_SAMPLE_WRITE)) {
        __syncthreads();
        continue;
    }
    C* yb = p.y + fo * p.coils + (int64_t)(c0 + coil) * Mf;
    const int J0 = JJ > 0 ? JJ : g.J[0];
    const int J1 = JJ > 0 ? JJ : g.J[NDIM > 1 ? 1 : 0];
    const int J2 = JJ > 0 ? JJ : g.J[NDIM > 2 ? 2 : 0];
    const int rowstride = Rd[0] * LSP;
    const int planestride = Rd[0] * Rd[1] * LSP;
    int pidx = -1;                          // held output, waiting for its pair
    C pacc = cmake<R>((R)0, (R)0);

    for (int base = warp * 32; base < count; base += nwarps * 32) {
        const int nb = min(32, count - base);
        R mcr[NDIM][JL], mci[NDIM][JL];
        int mbase = 0;  // shared-memory index of the window's first cell
        int mx0 = 0;    // region x-position of the window's first cell
        int midx = 0;
        C mph = cmake<R>((R)1, (R)0);
#pragma unroll
        for (int d = 0; d < NDIM; ++d)
#pragma unroll
            for (int j = 0; j < JL; ++j) mcr[d][j] = mci[d][j] = (R)0;
        if (lane < nb) {
            const int e = start + base + lane;
            midx = p.s.idx[e];
            int loc[3] = {0, 0, 0};
            R tt[3];
            int kf[3];
#pragma unroll
            for (int d = 0; d < NDIM; ++d) {
                tt[d] = p.s.t[d][e];
                kf[d] = first_tap(tt[d], g.J[d]);
                loc[d] = wrapk(kf[d], g.K[d]) - org[d];
            }
            if (p.s.cr) {
                // precomputed coefficients: jsum contiguous values per entry
                load_coefs<R, NDIM, JJ, JL>(p.s.cr + (int64_t)e * p.s.jsum, g, mcr);
                if (CX) load_coefs<R, NDIM, JJ, JL>(p.s.ci + (int64_t)e * p.s.jsum, g, mci);
            } else {
#pragma unroll
                for (int d = 0; d < NDIM; ++d)
#pragma unroll
                    for (int j = 0; j < JL; ++j)
                        if (JJ > 0 || j < g.J[d]) table_coef<R, CX>(g, d, tt[d], kf[d] + j, mcr[d][j], mci[d][j]);
            }
            mbase = ((loc[2] * Rd[1] + loc[1]) * Rd[0] + loc[0]) * LSP;
            mx0 = loc[0];
            if (p.apply_ph) mph = p.s.ph[e];
        }
        for (int s0 = 0; s0 < nb; s0 += SW) {
            const int src = s0 + slot;
            R cr[NDIM][JL], ci[NDIM][JL];
#pragma unroll
            for (int d = 0; d < NDIM; ++d) {
#pragma unroll
                for (int j = 0; j < JL; ++j) {
                    cr[d][j] = (R)0;
                    ci[d][j] = (R)0;
                    if (JJ > 0 || j < g.J[d]) {
                        cr[d][j] = __shfl_sync(0xffffffffu, mcr[d][j], src);
                        if (CX) ci[d][j] = __shfl_sync(0xffffffffu, mci[d][j], src);
                    }
                }
            }
            // coefficient pairs, built once per sample: (c, c) for a real kernel
            // (packed multiply-add on re and im), (Re c, Im c) for a complex one
            C q[NDIM][JL];
#pragma unroll
            for (int d = 0; d < NDIM; ++d)
#pragma unroll
                for (int j = 0; j < JL; ++j) q[d][j] = CX ? cmake<R>(cr[d][j], ci[d][j]) : cmake<R>(cr[d][j], cr[d][j]);
            const int sbase = __shfl_sync(0xffffffffu, mbase, src) + (TS ? 0 : coil);
            const int x0 = TS ? __shfl_sync(0xffffffffu, mx0, src) : 0;
            const int idx = __shfl_sync(0xffffffffu, midx, src);
            C ph;
            ph.x = __shfl_sync(0xffffffffu, mph.x, src);
            ph.y = __shfl_sync(0xffffffffu, mph.y, src);

            C acc = cmake<R>((R)0, (R)0);
            if constexpr (TS) {
                // lanes past the last sample run on zero coefficients (their
                // window is cell 0) so that the whole warp reaches the shuffle
                constexpr int JH = (JJ > 0 ? JJ : 2) / 2;
                int off[JH];
                C qh[JH];
#pragma unroll
                for (int jj = 0; jj < JH; ++jj) {
                    const int j0 = 2 * jj + th;
                    off[jj] = j0 * 8 + (coil ^ ((x0 + j0) & 7));
                    qh[jj] = th ? q[0][2 * jj + 1] : q[0][2 * jj];
                }
#pragma unroll
                for (int j2 = 0; j2 < (NDIM > 2 ? JL : 1); ++j2) {
                    C plane = cmake<R>((R)0, (R)0);
#pragma unroll
                    for (int j1 = 0; j1 < JL; ++j1) {
                        const int rb = sbase + j2 * planestride + j1 * rowstride;
                        C row = cmake<R>((R)0, (R)0);
#pragma unroll
                        for (int jj = 0; jj < JH; ++jj) qfma<CX>(row, qh[jj], S[rb + off[jj]]);
                        qfma<CX>(plane, q[NDIM > 1 ? 1 : 0][j1], row);
                    }
                    if (NDIM > 2)
                        qfma<CX>(acc, q[NDIM > 2 ? 2 : 0][j2], plane);
                    else
                        acc = plane;
                }
                acc.x += __shfl_xor_sync(0xffffffffu, acc.x, 8);
                acc.y += __shfl_xor_sync(0xffffffffu, acc.y, 8);
                if (src >= nb || th) continue;
            } else {
            if (src >= nb) continue;
            if (NDIM == 1) {
#pragma unroll
                for (int j0 = 0; j0 < JL; ++j0)
                    if (JJ > 0 || j0 < J0) qfma<CX>(acc, q[0][j0], S[sbase + j0 * LSP]);
            } else if (NDIM == 2) {
#pragma unroll
                for (int j1 = 0; j1 < JL; ++j1) {
                    if (JJ > 0 || j1 < J1) {
                        const int rb = sbase + j1 * rowstride;
                        C row = cmake<R>((R)0, (R)0);
#pragma unroll
                        for (int j0 = 0; j0 < JL; ++j0)
                            if (JJ > 0 || j0 < J0) qfma<CX>(row, q[0][j0], S[rb + j0 * LSP]);
                        qfma<CX>(acc, q[NDIM > 1 ? 1 : 0][j1], row);
                    }
                }
            } else {
#pragma unroll
                for (int j2 = 0; j2 < JL; ++j2) {
                    if (JJ > 0 || j2 < J2) {
                        C plane = cmake<R>((R)0, (R)0);
#pragma unroll
                        for (int j1 = 0; j1 < JL; ++j1) {
                            if (JJ > 0 || j1 < J1) {
                                const int rb = sbase + j2 * planestride + j1 * rowstride;
                                C row = cmake<R>((R)0, (R)0);
#pragma unroll
                                for (int j0 = 0; j0 < JL; ++j0)
                                    if (JJ > 0 || j0 < J0) qfma<CX>(row, q[0][j0], S[rb + j0 * LSP]);
                                qfma<CX>(plane, q[NDIM > 1 ? 1 : 0][j1], row);
                            }
                        }
                        qfma<CX>(acc, q[NDIM > 2 ? 2 : 0][j2], plane);
                    }
                }
            }
            }
            if (coil < nc) {
                if (p.apply_ph) acc = cmul(acc, ph);
                if (sizeof(R) == 4 && (LSC == 32 || (LSC > 0 && NDIM == 3))) {
                    // samples idx, idx + 1 (idx even) in consecutive list
                    // entries leave as one 16-byte store: half the store
                    // sectors along a trajectory's runs of consecutive samples
                    // (enabled where measured faster: 32 lanes, and 3-D)
                    if (pidx >= 0 && idx == pidx + 1 &&
                        (reinterpret_cast<uintptr_t>(yb + pidx) & 15) == 0) {
                        if (GBN_INB(g.check, idx < Mf, CHK_SAMPLE_WRITE)) store_pair(yb + pidx, pacc, acc);
                        pidx = -1;
                    } else {
                        if (pidx >= 0) yb[pidx] = pacc;
                        pidx = -1;
                        if ((idx & 1) == 0 && GBN_INB(g.check, idx >= 0 && idx < Mf, CHK_SAMPLE_WRITE)) {
                            pidx = idx;
                            pacc = acc;
                        } else if (GBN_INB(g.check, idx >= 0 && idx < Mf, CHK_SAMPLE_WRITE)) {
                            yb[idx] = acc;
                        }
                    }
                } else if (GBN_INB(g.check, idx >= 0 && idx < Mf, CHK_SAMPLE_WRITE)) {
                    yb[idx] = acc;
                }
            }
        }
    }
    if (pidx >= 0 && coil < nc) yb[pidx] = pacc;
    if constexpr (gather_persistent(NDIM)) __syncthreads();   // the next item restages the tile
    }
    if constexpr (gather_persistent(NDIM)) retire_ctas(p.tickets);
}

template <typename R>
size_t gather_smem(const Geom<R>& g, const Lanes& ln) {
    size_t cells = 1;
    for (int d = 0; d < g.ndim; ++d) cells *= (size_t)(g.T[d] + g.J[d] - 1);
    return cells * (size_t)ln.LSP * sizeof(typename Cx<R>::T);
}

// Shared memory of one launch: the tap-split kernels keep unpadded 8-coil rows.
template <typename R, int NDIM, int JJ, int LSC>
static size_t gather_smem_of(const Geom<R>& g, const Lanes& ln) {
    constexpr bool TS = LSC == 8 && NDIM == 3 && JJ > 0 && (JJ % 2) == 0 && sizeof(R) == 4;
    size_t cells = 1;
    for (int d = 0; d < g.ndim; ++d) cells *= (size_t)(g.T[d] + g.J[d] - 1);
    if (TS) return cells * 8 * sizeof(typename Cx<R>::T);
    if (gather_elem_staging(NDIM, LSC))   // + per-cell grid offset and phase
        return gather_smem(g, ln) + cells * sizeof(int64_t) + cells * sizeof(typename Cx<R>::T);
    return gather_smem(g, ln);
}

template <typename K>
static cudaError_t ensure_smem(K kernel, size_t bytes) {
    return ensure_dynamic_smem(reinterpret_cast<const void*>(kernel), bytes);
}

template <typename R, int NDIM, bool CX, int JJ, int LSC>
static cudaError_t gather_launch(const GatherParams<R>& p, cudaStream_t s) {
    const size_t smem = gather_smem_of<R, NDIM, JJ, LSC>(p.g, p.ln);
    cudaError_t e = ensure_smem(gather_kernel<R, NDIM, CX, JJ, LSC>, smem);
    if (e != cudaSuccess) return e;
    const int64_t total = (int64_t)p.nitems * p.chunks;
    if (p.chunks != (p.coils + p.ln.LS - 1) / p.ln.LS || total > INT32_MAX) return cudaErrorInvalidValue;
    if constexpr (gather_persistent(NDIM)) {
        if (!p.tickets) return cudaErrorInvalidValue;
        const int ctas = resident_ctas(reinterpret_cast<const void*>(gather_kernel<R, NDIM, CX, JJ, LSC>),
                                       GATHER_THREADS, smem);
        const int grid = (int)std::min<int64_t>(total, ctas > 0 ? ctas : total);
        gather_kernel<R, NDIM, CX, JJ, LSC><<<grid, GATHER_THREADS, smem, s>>>(p);
    } else {
        gather_kernel<R, NDIM, CX, JJ, LSC><<<dim3(p.nitems, p.chunks), GATHER_THREADS, smem, s>>>(p);
    }
    return cudaGetLastError();
}

// Kernel width shared by every axis, or 0.
template <typename R>
static int uniform_j(const Geom<R>& g) {
    for (int d = 1; d < g.ndim; ++d)
        if (g.J[d] != g.J[0]) return 0;
    return g.J[0];
}

template <int NDIM>
static cudaError_t gather_specialised(const GatherParams<float>& p, cudaStream_t s, bool* done) {
    *done = true;
    const int J = uniform_j(p.g);
    const int LS = p.ln.LS;
#define GBN_G(JV, LV) \
    if (J == JV && LS == LV) return gather_launch<float, NDIM, false, JV, LV>(p, s);
    GBN_G(6, 32) GBN_G(6, 16) GBN_G(6, 8) GBN_G(6, 1) GBN_G(4, 32) GBN_G(4, 16) GBN_G(4, 8) GBN_G(4, 1)
#undef GBN_G
    *done = false;
    return cudaSuccess;
}

template <typename R>
static cudaError_t launch_generic(const GatherParams<R>& p, cudaStream_t s) {
    const bool cx = p.g.hi[0] != nullptr;
    switch (p.g.ndim * 2 + (cx ? 1 : 0)) {
        case 2: return gather_launch<R, 1, false, 0, 0>(p, s);
        case 3: return gather_launch<R, 1, true, 0, 0>(p, s);
        case 4: return gather_launch<R, 2, false, 0, 0>(p, s);
        case 5: return gather_launch<R, 2, true, 0, 0>(p, s);
        case 6: return gather_launch<R, 3, false, 0, 0>(p, s);
        case 7: return gather_launch<R, 3, true, 0, 0>(p, s);
    }
    return cudaErrorInvalidValue;
}

static cudaError_t gather_any(const GatherParams<float>& p, cudaStream_t s) {
    const bool cx = p.g.hi[0] != nullptr;
    if (!cx && (p.g.ndim == 2 || p.g.ndim == 3)) {
        bool done = false;
        cudaError_t e = p.g.ndim == 2 ? gather_specialised<2>(p, s, &done) : gather_specialised<3>(p, s, &done);
        if (done) return e;
    }
    return launch_generic<float>(p, s);
}

static cudaError_t gather_any(const GatherParams<double>& p, cudaStream_t s) {
    return launch_generic<double>(p, s);
}

template <typename R>
cudaError_t launch_gather(const GatherParams<R>& p, cudaStream_t s) {
    if (p.nitems == 0 || p.coils == 0) return cudaSuccess;
    return gather_any(p, s);
}

template cudaError_t launch_gather<float>(const GatherParams<float>&, cudaStream_t);
template cudaError_t launch_gather<double>(const GatherParams<double>&, cudaStream_t);
template size_t gather_smem<float>(const Geom<float>&, const Lanes&);
template size_t gather_smem<double>(const Geom<double>&, const Lanes&);

}  // namespace gbn
