// Adjoint table interpolation (samples -> grid), tiled over the oversampled
// grid.  Replaces the reference's scatters (serial per coil on the CPU,
// mrrt/nufft/_extensions/c/nufft_table.template.c:144-531, 924-1206; global
// atomicAdd per tap on the GPU, mrrt/nufft/cuda/jinja/table_*_adjoint.jinja)
// with an "owner computes" decomposition and register accumulation:
//
// * a CTA owns one grid tile and one chunk of LS coils; each of its warps
//   owns a register block of SB0 x SB1 x SB2 = 16 (8 in 1-D) cells of the
//   tile, held as accumulators in every lane (lane = (sample slot, coil));
// * the planner lists every sample whose window touches the tile, with the
//   window start in tile coordinates (one entry per periodic image that
//   touches it, so the kernel never wraps);
// * entries are staged by chunk in shared memory: zero-padded per-axis
//   coefficient rows and the sample values for the LS coils;
// * each warp ballots which staged entries touch its block and accumulates
//   them in entry order: no atomics, no write conflicts, a fixed summation
//   order (bitwise repeatable);
// * sample slots of a warp are combined with warp shuffles and every grid
//   cell is written exactly once, with conj(phase_before) applied.  Tiles
//   too heavy for one CTA are split into parts whose partial tiles go to a
//   scratch buffer and are summed in part order by reduce_kernel.
#include <cuda_runtime.h>

#include "gbn_device.cuh"
#include "gbn_internal.h"

namespace gbn {

__host__ __device__ constexpr int cpad_len(int B) { return ((2 * (B - 1) + JMAX + 3) / 4) * 4; }

// Shared memory per CTA up to which the coefficient prefetch is used: four
// CTAs of it fit an SM's 228 KB.
constexpr size_t SPREAD_CPF_SMEM = 56 * 1024;

template <int NDIM>
struct SpreadLayout {
    static constexpr int B0 = SpreadBlock<NDIM>::B0, B1 = SpreadBlock<NDIM>::B1, B2 = SpreadBlock<NDIM>::B2;
    static constexpr int NB = B0 * B1 * B2;
    static constexpr int P0 = cpad_len(B0), P1 = cpad_len(B1), P2 = cpad_len(B2);
    static constexpr int PSUM = P0 + (NDIM > 1 ? P1 : 0) + (NDIM > 2 ? P2 : 0);
    // row stride of the staged coefficient rows: odd, so the thread-per-entry
    // staging stores fall in different banks
    static constexpr int PSTR = PSUM + 1;
};

// One staged entry's contribution to a warp's register block: its value
// for this lane's coil and the block's slice of its coefficient rows
// (loaded), then B0 x B1 x B2 multiply-adds (accumulate).
template <typename R, int NDIM, bool CX, typename SL, bool ROWSKIP = false>
struct EntryOps {
    typedef typename Cx<R>::T C;
    static constexpr int B0 = SL::B0, B1 = SL::B1, B2 = SL::B2;
    C v;
    C a0[B0], a1[B1], a2[B2];

    __device__ __forceinline__ void load(const C* cp, const C* vb, const short4* sls, int el, int VS, int coil,
                                         int bo0, int bo1, int bo2) {
        const short4 s = sls[el];
        v = vb[el * VS + coil];
        const C* row = cp + el * SL::PSTR;
        const int i0 = bo0 - s.x + (B0 - 1);
#pragma unroll
        for (int k = 0; k < B0; ++k) a0[k] = row[i0 + k];
        if (NDIM > 1) {
            const int i1 = SL::P0 + bo1 - s.y + (B1 - 1);
#pragma unroll
            for (int k = 0; k < B1; ++k) a1[k] = row[i1 + k];
        } else {
            a1[0] = CX ? cmake<R>((R)1, (R)0) : cmake<R>((R)1, (R)1);   // neutral factor
        }
        if (NDIM > 2) {
            const int i2 = SL::P0 + SL::P1 + bo2 - s.z + (B2 - 1);
#pragma unroll
            for (int k = 0; k < B2; ++k) a2[k] = row[i2 + k];
        } else {
            a2[0] = CX ? cmake<R>((R)1, (R)0) : cmake<R>((R)1, (R)1);
        }
    }

    // ROWSKIP: window start along axis 1 relative to the block, and the
    // kernel width; rows of the block the window misses are skipped
    int ry = 0, Jy = 0;
    template <int NB>
    __device__ __forceinline__ void accumulate(C (&acc)[NB]) const {
#pragma unroll
        for (int k2 = 0; k2 < B2; ++k2) {
#pragma unroll
            for (int k1 = 0; k1 < B1; ++k1) {
                if (ROWSKIP && (unsigned)(k1 - ry) >= (unsigned)Jy) continue;
                C tv;
                if (CX) {
                    // conj(c2 c1) v, the pairs already hold conj
                    const C w = cmul(a1[k1], a2[k2]);
                    tv = cmul(w, v);
                } else {
                    // pairs (c, c): w12 = c1 c2 on both halves, tv = w12 v
                    const C w12 = NDIM > 2 ? pmul(a1[k1], a2[k2]) : a1[k1];
                    tv = pmul(w12, v);
                }
#pragma unroll
                for (int k0 = 0; k0 < B0; ++k0) {
                    const int q = (k2 * B1 + k1) * B0 + k0;
                    if (CX) {
                        const C w0 = cmul(a0[k0], tv);
                        acc[q].x += w0.x;
                        acc[q].y += w0.y;
                    } else {
                        acc[q] = pfma(a0[k0], tv, acc[q]);
                    }
                }
            }
        }
    }
};

int spread_threads(int ndim, const int* T) {
    int b[3];
    if (ndim == 1) { b[0] = SpreadBlock<1>::B0; b[1] = b[2] = 1; }
    else if (ndim == 2) { b[0] = SpreadBlock<2>::B0; b[1] = SpreadBlock<2>::B1; b[2] = 1; }
    else { b[0] = SpreadBlock<3>::B0; b[1] = SpreadBlock<3>::B1; b[2] = SpreadBlock<3>::B2; }
    int warps = 1;
    for (int d = 0; d < ndim; ++d) warps *= T[d] / b[d];
    return 32 * warps;
}

template <typename R, int NDIM, bool CX, int JJ, int LSC, bool ROWSKIP = false>
__global__ void __launch_bounds__(256, 4)
spread_kernel(const SpreadParams<R> p) {
    typedef typename Cx<R>::T C;
    typedef SpreadLayout<NDIM> SL;
    constexpr int B0 = SL::B0, B1 = SL::B1, B2 = SL::B2, NB = SL::NB;
    constexpr int CH = SPREAD_CHUNK_ENTRIES;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const Geom<R>& g = p.g;

    const int LS = LSC > 0 ? LSC : p.ln.LS;
    const int lsh = LSC > 0 ? (LSC == 32 ? 5 : LSC == 16 ? 4 : LSC == 8 ? 3 : LSC == 4 ? 2 : LSC == 2 ? 1 : 0)
                            : p.ln.lsh;
    const int Jx = JJ > 0 ? JJ : g.J[0];
    const int Jy = JJ > 0 ? JJ : g.J[NDIM > 1 ? 1 : 0];
    const int Jz = JJ > 0 ? JJ : g.J[NDIM > 2 ? 2 : 0];
    const int VS = LS + 1;
    // shared layout (two buffers for the copied-in chunk data, one for the
    // coefficient rows computed from it):
    //   vbuf[2][CH][VS]   sample values of the LS coils
    //   cp[CH][PSTR]      coefficient pairs: (c, c) for a real kernel (a packed
    //                     multiply applies c to re and im at once),
    //                     (Re c, -Im c) = conj(c) for a complex kernel
    //   tb[2][NDIM][CH]   coordinates, lsb[2][CH] window starts
    //   craw[CX ? 2 : 1][CH * jsum]  (cpf) the next chunk's precomputed
    //                     coefficients as stored, copied in beside its values
    C* vbuf = reinterpret_cast<C*>(smem_raw);
    C* cp = vbuf + 2 * CH * VS;
    short4* lsb = reinterpret_cast<short4*>(cp + CH * SL::PSTR);
    R* tb = reinterpret_cast<R*>(lsb + 2 * CH);
    R* craw = tb + 2 * NDIM * CH;

    // One CTA per (work item, coil chunk).  (A persistent launch, resident
    // CTAs taking work tickets as the 3-D gather does, measured slower here:
    // 0.191 against 0.151 ms at the 2-D 32-coil workload, 5.78 against
    // 5.71 ms at the 3-D kooshball.)
    __shared__ unsigned char hitpos[8][32];   // per warp: positions of the current group's hits
    const int item = blockIdx.x, chunk = blockIdx.y;
    const int4 it = p.items[item];
    const int2 part = p.parts[item];
    const int f = it.x, tile = it.y, start = it.z, count = it.w;
    if (!GBN_INB(g.check, start >= 0 && count >= 0 && start + (int64_t)count <= p.s.len, CHK_LIST)) return;
    const int c0 = chunk << lsh;
    const int nc = min(LS, p.coils - c0);

    int org[3] = {0, 0, 0}, ext[3] = {1, 1, 1}, Td[3] = {1, 1, 1};
    tile_origin<NDIM>(tile, g.nt, g.T, org);
#pragma unroll
    for (int d = 0; d < NDIM; ++d) {
        Td[d] = g.T[d];
        ext[d] = min(g.T[d], g.K[d] - org[d]);
    }

    const int tid = threadIdx.x;
    const int warp = tid >> 5, lane = tid & 31;
    const int SW = 32 >> lsh;
    const int slot = lane >> lsh, coil = lane & (LS - 1);
    // this warp's register block
    const int nb0 = Td[0] / B0, nb1 = NDIM > 1 ? Td[1] / B1 : 1;
    const int bo0 = (warp % nb0) * B0;
    const int bo1 = NDIM > 1 ? ((warp / nb0) % nb1) * B1 : 0;
    const int bo2 = NDIM > 2 ? (warp / (nb0 * nb1)) * B2 : 0;

    C acc[NB];
#pragma unroll
    for (int q = 0; q < NB; ++q) acc[q] = cmake<R>((R)0, (R)0);

    const int64_t fo = p.foff[f];
    const int Mf = (int)(p.foff[f + 1] - fo);
    if (!GBN_INB(g.check, (fo + Mf) * p.coils <= g.sample_elems, CHK_SAMPLE_READ)) return;
    const C* yb = p.y + fo * p.coils + (int64_t)c0 * Mf;

    // zero padding of the coefficient rows: written once, the J coefficient
    // slots of each row are overwritten per chunk.  Only the rows of entries
    // the item has are ever read (a tile of 25 entries zeroes 25 rows, not
    // 64); an empty tile -- no entry touches it -- needs none: it only writes
    // zeros
    for (int q = tid; q < min(count, CH) * SL::PSTR; q += blockDim.x) cp[q] = cmake<R>((R)0, (R)0);
    const int Jsum = Jx + (NDIM > 1 ? Jy : 0) + (NDIM > 2 ? Jz : 0);

    // Copy-in assignment: each thread owns up to two entries of a chunk and
    // the coils cg, cg + ng, ... of them.
    const int nthr = blockDim.x;
    const int ng = nthr >= CH ? nthr / CH : 1;
    const int cg = nthr >= CH ? tid / CH : 0;
    const int EPT = nthr >= CH ? 1 : CH / nthr;    // 1 or 2 (CTAs have >= 32 threads)
    const int elo = nthr >= CH ? tid % CH : tid;
    const int nchunks = (count + CH - 1) / CH;

    // index and phase of this thread's entries, one chunk ahead of the copies
    int nidx[2] = {0, 0};
    C nph[2] = {cmake<R>((R)1, (R)0), cmake<R>((R)1, (R)0)};
    C cph[2] = {cmake<R>((R)1, (R)0), cmake<R>((R)1, (R)0)};
    auto load_meta = [&](int chunk) {
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            const int el = elo + u * nthr;
            const int n = min(CH, count - chunk * CH);
            if (u < EPT && chunk < nchunks && el < n) {
                const int e = start + chunk * CH + el;
                nidx[u] = p.s.idx[e];
                if (p.apply_ph) nph[u] = p.s.ph[e];
            }
        }
    };
    // issue the asynchronous copies of chunk `chunk` into buffer `b`
    auto issue = [&](int chunk, int b) {
        const int n = min(CH, count - chunk * CH);
        const int e0 = start + chunk * CH;
        C* vb = vbuf + b * CH * VS;
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            const int el = elo + u * nthr;
            if (u < EPT && el < n && GBN_INB(g.check, nidx[u] >= 0 && nidx[u] < Mf, CHK_SAMPLE_READ)) {
                const C* src = yb + nidx[u];
                for (int c = cg; c < nc; c += ng) cp_async<sizeof(C)>(vb + el * VS + c, src + (int64_t)c * Mf);
            }
        }
        for (int q = tid; q < n; q += nthr) {
            cp_async<sizeof(short4)>(lsb + b * CH + q, p.s.ls + e0 + q);
            if (!p.s.cr) {
#pragma unroll
                for (int d = 0; d < NDIM; ++d)
                    cp_async<sizeof(R)>(tb + (b * NDIM + d) * CH + q, p.s.t[d] + e0 + q);
            }
        }
    };
    // (cpf) the chunk's coefficients, contiguous in list order, into the one
    // raw buffer: issued once the previous chunk's rows are built
    auto issue_coefs = [&](int chunk) {
        if (!p.cpf) return;
        const int n = min(CH, count - chunk * CH);
        const int64_t e0 = (int64_t)start + chunk * CH;
        const int nq = n * p.s.jsum;
        for (int q = tid; q < nq; q += nthr) {
            cp_async<sizeof(R)>(craw + q, p.s.cr + e0 * p.s.jsum + q);
            if (CX) cp_async<sizeof(R)>(craw + CH * p.s.jsum + q, p.s.ci + e0 * p.s.jsum + q);
        }
    };

    if (nchunks > 0) {
        load_meta(0);
        issue(0, 0);
        issue_coefs(0);
        cp_async_commit();
#pragma unroll
        for (int u = 0; u < 2; ++u) cph[u] = nph[u];
        load_meta(1);
    }

    for (int k = 0; k < nchunks; ++k) {
        const int b = k & 1;
        const int n = min(CH, count - k * CH);
        const C* vb = vbuf + b * CH * VS;
        const short4* sls = lsb + b * CH;
        // ---- chunk k has landed: apply conj(sample phase) to own values ------
        cp_async_wait_all();
        if (p.apply_ph) {
            C* vw = vbuf + b * CH * VS;
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                const int el = elo + u * nthr;
                if (u < EPT && el < n)
                    for (int c = cg; c < nc; c += ng) vw[el * VS + c] = cmulc(vw[el * VS + c], cph[u]);
            }
        }
        __syncthreads();
        // ---- coefficient rows of chunk k (the J taps of each axis) -------------
        for (int q = tid; q < n * Jsum; q += nthr) {
            const int el = q / Jsum;
            int j = q - el * Jsum;
            int d = 0, slot0 = B0 - 1, Jd = Jx;
            if (NDIM > 1 && j >= Jx) {
                j -= Jx;
                d = 1;
                slot0 = SL::P0 + B1 - 1;
                Jd = Jy;
                if (NDIM > 2 && j >= Jy) {
                    j -= Jy;
                    d = 2;
                    slot0 = SL::P0 + SL::P1 + B2 - 1;
                    Jd = Jz;
                }
            }
            R cr, ci = (R)0;
            if (p.cpf) {
                cr = craw[q];
                if (CX) ci = craw[CH * Jsum + q];
            } else if (p.s.cr) {
                const int64_t ce = (int64_t)(start + k * CH + el) * Jsum + (q - el * Jsum);
                cr = p.s.cr[ce];
                if (CX) ci = p.s.ci[ce];
            } else {
                const R t = tb[(b * NDIM + d) * CH + el];
                table_coef<R, CX>(g, d, t, first_tap(t, Jd) + j, cr, ci);
            }
            cp[el * SL::PSTR + slot0 + j] = CX ? cmake<R>(cr, -ci) : cmake<R>(cr, cr);
        }
        // ---- copy-in of chunk k+1 overlaps with the accumulation of chunk k ----
        if (k + 1 < nchunks) {
            issue(k + 1, b ^ 1);
#pragma unroll
            for (int u = 0; u < 2; ++u) cph[u] = nph[u];
            load_meta(k + 2);
        }
        __syncthreads();
        // every row of chunk k is built: the raw buffer takes chunk k+1's
        if (k + 1 < nchunks) issue_coefs(k + 1);
        cp_async_commit();
        // ---- accumulate: each warp takes the entries touching its block --------
        for (int gb = 0; gb < n; gb += 32) {
            const int l = gb + lane;
            bool hit = false;
            if (l < n) {
                const short4 s = sls[l];
                hit = s.x < bo0 + B0 && s.x + Jx > bo0;
                if (NDIM > 1) hit = hit && s.y < bo1 + B1 && s.y + Jy > bo1;
                if (NDIM > 2) hit = hit && s.z < bo2 + B2 && s.z + Jz > bo2;
            }
            unsigned mask = __ballot_sync(0xffffffffu, hit);
            if (SW > 1) {
                // several samples per warp: the hits' positions are compacted
                // into this warp's list, and slot k takes hits k, k + SW,
                // k + 2 SW, ... in entry order (the order, hence the sums, of
                // a serial pick)
                if (hit) hitpos[warp][__popc(mask & ((1u << lane) - 1u))] = (unsigned char)lane;
                __syncwarp();
                const int nh = __popc(mask);
                for (int r = slot; r < nh; r += SW) {
                    const int pos = hitpos[warp][r];
                    if (coil < nc) {
                        EntryOps<R, NDIM, CX, SL, ROWSKIP> A;
                        A.load(cp, vb, sls, gb + pos, VS, coil, bo0, bo1, bo2);
                        if (ROWSKIP) {
                            A.ry = sls[gb + pos].y - bo1;
                            A.Jy = Jy;
                        }
                        A.accumulate(acc);
                    }
                }
                __syncwarp();   // the list is rewritten for the next group
                continue;
            }
            while (mask) {
                const int pos = __ffs(mask) - 1;
                mask &= mask - 1;
                if (coil < nc) {
                    EntryOps<R, NDIM, CX, SL, ROWSKIP> A;
                    A.load(cp, vb, sls, gb + pos, VS, coil, bo0, bo1, bo2);
                    if (ROWSKIP) {
                        A.ry = sls[gb + pos].y - bo1;
                        A.Jy = Jy;
                    }
                    A.accumulate(acc);
                }
            }
        }
    }

    // ---- combine the sample slots of the warp ------------------------------
    for (int off = LS; off < 32; off <<= 1) {
#pragma unroll
        for (int q = 0; q < NB; ++q) {
            acc[q].x += __shfl_xor_sync(0xffffffffu, acc[q].x, off);
            acc[q].y += __shfl_xor_sync(0xffffffffu, acc[q].y, off);
        }
    }

    // ---- flush: each owned cell written once -------------------------------
    // phase_before of the block's cells: lane q computes cell q (q < NB), the
    // others read it by shuffle
    C myph = cmake<R>((R)1, (R)0);
    const int slot_id = part.x;
    const bool direct = slot_id < 0;
    // zeros need no phase: an empty tile skips the per-cell sincos
    if (direct && p.apply_pb && lane < NB && count > 0) {
        const int k0 = lane % B0, k1 = (lane / B0) % B1, k2 = lane / (B0 * B1);
        int k[3] = {org[0] + bo0 + k0, org[1] + bo1 + k1, org[2] + bo2 + k2};
        bool in = bo0 + k0 < ext[0];
        if (NDIM > 1) in = in && bo1 + k1 < ext[1];
        if (NDIM > 2) in = in && bo2 + k2 < ext[2];
        if (in) myph = phase_before(g, k);
    }
    // cells are written in adjacent pairs: one 16-byte store when both are
    // inside the grid and the address is aligned (single precision, even K0)
    const bool vec_ok = sizeof(R) == 4 && (g.K[0] % 2) == 0 && (g.gsp % 2) == 0 && (g.gs1 % 2) == 0 &&
                        (g.gs2 % 2) == 0;
#pragma unroll
    for (int q = 0; q < NB; q += 2) {
        const int k0 = q % B0, k1 = (q / B0) % B1, k2 = q / (B0 * B1);
        C ph0 = cmake<R>((R)1, (R)0), ph1 = cmake<R>((R)1, (R)0);
        if (direct && p.apply_pb && count > 0) {
            ph0.x = __shfl_sync(0xffffffffu, myph.x, q);
            ph0.y = __shfl_sync(0xffffffffu, myph.y, q);
            ph1.x = __shfl_sync(0xffffffffu, myph.x, q + 1);
            ph1.y = __shfl_sync(0xffffffffu, myph.y, q + 1);
        }
        const int l0 = bo0 + k0, l1 = bo1 + k1, l2 = bo2 + k2;
        bool row_in = true;
        if (NDIM > 1) row_in = row_in && l1 < ext[1];
        if (NDIM > 2) row_in = row_in && l2 < ext[2];
        const bool in0 = row_in && l0 < ext[0], in1 = row_in && l0 + 1 < ext[0];
        if (slot != 0 || coil >= nc) continue;
        C v0 = acc[q], v1 = acc[q + 1];
        if (direct) {
            if (p.apply_pb && count > 0) {
                v0 = cmulc(v0, ph0);
                v1 = cmulc(v1, ph1);
            }
            const int64_t off = (int64_t)(org[0] + l0) + (int64_t)(org[1] + l1) * g.gs1 +
                                (int64_t)(org[2] + l2) * g.gs2;
            // the cells this lane writes: gi (if in0) and gi + 1 (if in1)
            const int64_t gi = ((int64_t)f * p.coils + c0 + coil) * g.gsp + off;
            if ((in0 || in1) &&
                !GBN_INB(g.check, gi + (in0 ? 0 : 1) >= 0 && gi + (in1 ? 1 : 0) < g.grid_elems, CHK_GRID_WRITE))
                continue;
            C* dst = p.grid + ((int64_t)f * p.coils + c0 + coil) * g.gsp + off;
            if (in0 && in1 && vec_ok) {
                store_pair(dst, v0, v1);
            } else {
                if (in0) dst[0] = v0;
                if (in1) dst[1] = v1;
            }
        } else {
            const int cell = l0 + Td[0] * (l1 + Td[1] * l2);
            const int64_t si = (((int64_t)slot_id * p.chunks + chunk) * LS + coil) * p.tile_cells + cell;
            if ((in0 || in1) &&
                !GBN_INB(g.check, si + (in0 ? 0 : 1) >= 0 && si + (in1 ? 1 : 0) < p.scratch_elems, CHK_SCRATCH))
                continue;
            C* dst = p.scratch + si;
            if (in0) dst[0] = v0;
            if (in1) dst[1] = v1;
        }
    }
}

// Sum the parts of split tiles in part order and write the grid.  One
// thread per (coil, cell) of a tile; a tile's TT x LS elements are spread
// over `nsub` CTAs (blockIdx.x = tile * nsub + sub) so that the many small
// partial-sum reads are in flight at once.  The parts are loaded four at a
// time and added in part order, so the result is the same in every run.
template <typename R, int NDIM>
__global__ void __launch_bounds__(256) reduce_kernel(const ReduceParams<R> p, const int nsub) {
    typedef typename Cx<R>::T C;
    const Geom<R>& g = p.g;
    const int ti = blockIdx.x / nsub;
    const int sub = blockIdx.x - ti * nsub;
    const int4 tl = p.tiles[ti];
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
    const int q = sub * blockDim.x + threadIdx.x;
    if (q >= TT * nc) return;
    const int c = q / TT;
    const int cell = q - c * TT;
    int r[3];
    r[0] = cell % Td[0];
    r[1] = (cell / Td[0]) % Td[1];
    r[2] = cell / (Td[0] * Td[1]);
    bool inside = true;
#pragma unroll
    for (int d = 0; d < NDIM; ++d) inside = inside && (r[d] < ext[d]);
    if (!inside) return;
    const int64_t pstride = (int64_t)gridDim.y * LS * p.tile_cells;
    const int64_t s0 = (((int64_t)slot0 * gridDim.y + blockIdx.y) * LS + c) * p.tile_cells + cell;
    if (!GBN_INB(g.check, slot0 >= 0 && nparts >= 1 && s0 + (int64_t)(nparts - 1) * pstride < p.scratch_elems,
                 CHK_SCRATCH))
        return;
    const C* src = p.scratch + s0;
    C acc = cmake<R>((R)0, (R)0);
    int s = 0;
    for (; s + 4 <= nparts; s += 4) {
        const C v0 = src[(int64_t)s * pstride];
        const C v1 = src[(int64_t)(s + 1) * pstride];
        const C v2 = src[(int64_t)(s + 2) * pstride];
        const C v3 = src[(int64_t)(s + 3) * pstride];
        acc.x += v0.x; acc.y += v0.y;
        acc.x += v1.x; acc.y += v1.y;
        acc.x += v2.x; acc.y += v2.y;
        acc.x += v3.x; acc.y += v3.y;
    }
    for (; s < nparts; ++s) {
        const C v = src[(int64_t)s * pstride];
        acc.x += v.x;
        acc.y += v.y;
    }
    int k[3] = {0, 0, 0};
#pragma unroll
    for (int d = 0; d < NDIM; ++d) k[d] = org[d] + r[d];
    const int64_t off = k[0] + (int64_t)k[1] * g.gs1 + (int64_t)k[2] * g.gs2;
    if (p.apply_pb) acc = cmulc(acc, phase_before(g, k));
    const int64_t gi = ((int64_t)f * p.coils + c0 + c) * g.gsp + off;
    if (GBN_INB(g.check, gi >= 0 && gi < g.grid_elems, CHK_GRID_WRITE)) p.grid[gi] = acc;
}

template <typename R>
size_t spread_smem(const Geom<R>& g, const Lanes& ln) {
    int pstr = 0;
    if (g.ndim == 1) pstr = SpreadLayout<1>::PSTR;
    else if (g.ndim == 2) pstr = SpreadLayout<2>::PSTR;
    else pstr = SpreadLayout<3>::PSTR;
    const size_t CH = SPREAD_CHUNK_ENTRIES;
    const size_t csz = sizeof(typename Cx<R>::T);
    return 2 * CH * (size_t)(ln.LS + 1) * csz + CH * (size_t)pstr * csz + 2 * CH * sizeof(short4) +
           2 * (size_t)g.ndim * CH * sizeof(R);
}

template <typename K>
static cudaError_t ensure_smem(K kernel, size_t bytes) {
    return ensure_dynamic_smem(reinterpret_cast<const void*>(kernel), bytes);
}

template <typename R, int NDIM, bool CX, int JJ, int LSC, bool ROWSKIP = false>
static cudaError_t spread_launch(const SpreadParams<R>& p0, cudaStream_t s) {
    // Precomputed coefficients are copied into shared memory a chunk ahead
    // (cp.async, with the values) when the extra buffer still leaves four
    // CTAs per SM; otherwise the row staging reads them from global memory
    // between the chunk's barriers.
    SpreadParams<R> p = p0;
    const size_t base = spread_smem(p.g, p.ln);
    const size_t raw = p.s.cr ? (size_t)(CX ? 2 : 1) * SPREAD_CHUNK_ENTRIES * p.s.jsum * sizeof(R) : 0;
    p.cpf = p.s.cr && base + raw <= SPREAD_CPF_SMEM;
    const size_t smem = base + (p.cpf ? raw : 0);
    cudaError_t e = ensure_smem(spread_kernel<R, NDIM, CX, JJ, LSC, ROWSKIP>, smem);
    if (e != cudaSuccess) return e;
    const int threads = spread_threads(NDIM, p.g.T);
    if (threads < 32 || threads > 256) return cudaErrorInvalidConfiguration;
    if (p.chunks != (p.coils + p.ln.LS - 1) / p.ln.LS) return cudaErrorInvalidValue;
    spread_kernel<R, NDIM, CX, JJ, LSC, ROWSKIP><<<dim3(p.nitems, p.chunks), threads, smem, s>>>(p);
    return cudaGetLastError();
}

template <typename R>
static cudaError_t spread_generic(const SpreadParams<R>& p, cudaStream_t s) {
    const bool cx = p.g.hi[0] != nullptr;
    switch (p.g.ndim * 2 + (cx ? 1 : 0)) {
        case 2: return spread_launch<R, 1, false, 0, 0>(p, s);
        case 3: return spread_launch<R, 1, true, 0, 0>(p, s);
        case 4: return spread_launch<R, 2, false, 0, 0>(p, s);
        case 5: return spread_launch<R, 2, true, 0, 0>(p, s);
        case 6: return spread_launch<R, 3, false, 0, 0>(p, s);
        case 7: return spread_launch<R, 3, true, 0, 0>(p, s);
    }
    return cudaErrorInvalidValue;
}

template <int NDIM>
static cudaError_t spread_specialised(const SpreadParams<float>& p, cudaStream_t s, bool* done) {
    *done = true;
    int J = p.g.J[0];
    for (int d = 1; d < p.g.ndim; ++d)
        if (p.g.J[d] != J) J = 0;
    const int LS = p.ln.LS;
    // J 6, 32 coil lanes: skip the rows of a 4 x 4 block the window misses
    // (measured at the 2-D 32-coil workload: 0.152 against 0.154 ms)
    if (NDIM == 2 && J == 6 && LS == 32) return spread_launch<float, NDIM, false, 6, 32, true>(p, s);
#define GBN_S(JV, LV) \
    if (J == JV && LS == LV) return spread_launch<float, NDIM, false, JV, LV>(p, s);
    GBN_S(6, 32) GBN_S(6, 16) GBN_S(6, 8) GBN_S(6, 1) GBN_S(4, 32) GBN_S(4, 16) GBN_S(4, 8) GBN_S(4, 1)
#undef GBN_S
    *done = false;
    return cudaSuccess;
}

static cudaError_t spread_any(const SpreadParams<float>& p, cudaStream_t s) {
    const bool cx = p.g.hi[0] != nullptr;
    if (!cx && (p.g.ndim == 2 || p.g.ndim == 3)) {
        bool done = false;
        cudaError_t e = p.g.ndim == 2 ? spread_specialised<2>(p, s, &done) : spread_specialised<3>(p, s, &done);
        if (done) return e;
    }
    return spread_generic<float>(p, s);
}

static cudaError_t spread_any(const SpreadParams<double>& p, cudaStream_t s) {
    return spread_generic<double>(p, s);
}

template <typename R>
cudaError_t launch_spread(const SpreadParams<R>& p, cudaStream_t s) {
    if (p.nitems == 0 || p.coils == 0) return cudaSuccess;
    return spread_any(p, s);
}

template <typename R>
cudaError_t launch_reduce(const ReduceParams<R>& p, cudaStream_t s) {
    if (p.ntiles == 0 || p.coils == 0) return cudaSuccess;
    const int64_t tt = (int64_t)p.g.T[0] * (p.g.ndim > 1 ? p.g.T[1] : 1) * (p.g.ndim > 2 ? p.g.T[2] : 1);
    const int nsub = (int)((tt * p.ln.LS + 255) / 256);
    dim3 grid((unsigned)((int64_t)p.ntiles * nsub), (p.coils + p.ln.LS - 1) / p.ln.LS);
    switch (p.g.ndim) {
        case 1: reduce_kernel<R, 1><<<grid, 256, 0, s>>>(p, nsub); break;
        case 2: reduce_kernel<R, 2><<<grid, 256, 0, s>>>(p, nsub); break;
        case 3: reduce_kernel<R, 3><<<grid, 256, 0, s>>>(p, nsub); break;
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
