// Internal declarations shared by the host planner (gbn_plan.cu) and the
// device kernels (gbn_gather.cu, gbn_spread.cu, gbn_padcrop.cu, gbn_grad.cu,
// gbn_colfft.cu, ...).
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

namespace gbn {

// Kernel width limit of the register-resident coefficient arrays.
constexpr int JMAX = 8;

// Spread register blocks: each warp of a spread CTA (at most 8 warps) owns
// SB0 x SB1 x SB2 cells of its tile (16 accumulators per lane).
template <int NDIM> struct SpreadBlock;
template <> struct SpreadBlock<1> { static constexpr int B0 = 16, B1 = 1, B2 = 1; };
template <> struct SpreadBlock<2> { static constexpr int B0 = 4, B1 = 4, B2 = 1; };
template <> struct SpreadBlock<3> { static constexpr int B0 = 4, B1 = 4, B2 = 1; };
// Entries staged per spread chunk (two chunks in flight: one accumulated
// while the next is copied in).
constexpr int SPREAD_CHUNK_ENTRIES = 64;

template <typename R> struct Cx;
template <> struct Cx<float> { typedef float2 T; };
template <> struct Cx<double> { typedef double2 T; };

// Geometry in memory-axis order (axis 0 fastest) with the tiling of the
// list being processed.
template <typename R>
struct Geom {
    int ndim;
    int N[3], K[3], J[3], T[3], nt[3];
    int L;
    int ncenter[3];          // floor(J*L/2): table index of t = 0
    const R* hr[3];          // device tables (shifted past their zero padding)
    const R* hi[3];          // imaginary tables, nullptr for a real kernel
    int64_t Kprod, Nprod;
    // Grid layout: cell (k0, k1, k2) of plane pl (= frame * coils + coil) at
    // pl * gsp + k0 + k1 * gs1 + k2 * gs2.  Plane-major ([planes][K...]:
    // gsp = Kprod, gs1 = K0, gs2 = K0 K1) or, for the 2-D transform's own
    // grid, row-interleaved ([K1][planes][K0]: gsp = K0, gs1 = planes K0),
    // the layout its pruned FFT passes need.
    int64_t gsp, gs1, gs2;
    R pbc[3];                // phase_before coefficient per memory axis
    int pbo[3];              // summation order of the per-axis phases
    // Checked builds (GBN_CHECKED): the plan's status word and the extents
    // (complex elements) of the grid and sample buffers of the call
    unsigned* check;
    int64_t grid_elems, sample_elems;
};

// Status bits of a checked build: which kind of index failed its bound.
constexpr unsigned CHK_GRID_READ = 1u, CHK_GRID_WRITE = 2u, CHK_SAMPLE_READ = 4u, CHK_SAMPLE_WRITE = 8u,
                   CHK_SCRATCH = 16u, CHK_LIST = 32u, CHK_IMAGE = 64u;

// Coil-lane layout of a CTA: LS lanes per sample (power of two <= 32),
// SW = 32 / LS samples per warp.  Staged grid values for one cell occupy
// LSP complex slots (LS + 1 for LS > 1: conflict-free transposed staging).
struct Lanes {
    int LS, lsh, LSP;
};

// Sorted sample list (one per direction).
template <typename R>
struct SampleList {
    const R* t[3];                  // coordinate per memory axis, list order
    const int* idx;                 // sample index within its frame
    const typename Cx<R>::T* ph;    // per-sample phase (list order) or nullptr
    const short4* ls;               // spread list: window start in tile coordinates
    // Interpolation coefficients precomputed in list order, or nullptr (the
    // kernels then interpolate the tables): entry e holds jsum values, the
    // J_0 taps of axis 0, then the J_1 taps of axis 1, ...; ci the imaginary
    // parts for a complex kernel.
    const R* cr;
    const R* ci;
    int jsum;
    int64_t len;                    // entries in the list
};

// Fill a list's precomputed coefficients, for every entry of every work
// item: from the tables (bitwise the values the kernels would interpolate)
// or, in sparse-matrix mode, from per-sample weights wr[d] / wi[d]
// ([M_total][J_d], sample order = frame offset + index).
template <typename R>
struct CoefParams {
    Geom<R> g;
    SampleList<R> s;
    const int4* items;              // {frame, tile, start, count}
    int nitems;
    const int64_t* foff;
    const R* wr[3];
    const R* wi[3];
    R* out_r;
    R* out_i;
    int jsum;
    int cx;
};

template <typename R>
struct GatherParams {
    Geom<R> g;
    Lanes ln;
    SampleList<R> s;
    const int4* items;              // {frame, tile, start, count}
    int nitems;
    int coils;
    const int64_t* foff;            // device frame offsets [F+1]
    const typename Cx<R>::T* grid;  // [F][coils][Kprod]
    typename Cx<R>::T* y;           // samples
    int apply_pb;                   // multiply staged cells by phase_before
    R grid_scale;                   // divide staged cells by this (ortho)
    int apply_ph;                   // multiply outputs by the sample phase
    int* tickets;                   // work counter pair of the persistent (3-D) launch, zero
                                    // between launches; the 1-D and 2-D kernels ignore it
    int chunks;                     // coil chunks of LS lanes
};

template <typename R>
struct SpreadParams {
    Geom<R> g;
    Lanes ln;
    SampleList<R> s;
    const int4* items;              // {frame, tile, start, count}
    const int2* parts;              // {scratch slot or -1, nparts}
    int nitems;
    int coils;
    const int64_t* foff;
    const typename Cx<R>::T* y;
    typename Cx<R>::T* grid;
    typename Cx<R>::T* scratch;     // [slot][chunk][LS][tile cells] partial sums
    int64_t tile_cells;             // T0*T1*T2
    int64_t scratch_elems;          // scratch extent (complex elements)
    int apply_pb;
    int apply_ph;
    int chunks;                     // coil chunks of LS lanes (gridDim.y)
    int cpf;                        // set by the launcher: precomputed coefficients prefetched
                                    // into shared memory a chunk ahead
};

template <typename R>
struct ReduceParams {
    Geom<R> g;
    Lanes ln;
    const int4* tiles;              // {frame, tile, first slot, nparts}
    int ntiles;
    int coils;
    const typename Cx<R>::T* scratch;
    typename Cx<R>::T* grid;
    int64_t tile_cells;
    int64_t scratch_elems;
    int apply_pb;
};

template <typename R>
struct PadParams {
    int ndim;
    int N[3], K[3];
    int64_t Nprod, Kprod;
    int64_t gsp, gs1, gs2;          // layout of the padded grid (see Geom)
    int planes;
    const typename Cx<R>::T* x;
    const R* sn;
    typename Cx<R>::T* out;
    // coil-sensitivity fusion: x is one image per frame [F][N] and plane
    // f * coils + c receives sn * maps[c] * x[f]; nullptr for the plain pad
    const typename Cx<R>::T* maps;
    int coils;
    unsigned* check;                // checked builds: status word
    int64_t x_elems, out_elems;     // extents of x and out
};

template <typename R>
struct CropParams {
    int ndim;
    int N[3], K[3];
    int64_t Nprod, Kprod;
    int64_t gsp, gs1, gs2;          // layout of the grid read (see Geom)
    int planes;
    const typename Cx<R>::T* grid;
    const R* sn;
    R scale;
    typename Cx<R>::T* x;
    // coil combination: x[f] = sum_c conj(maps[c]) * (cropped plane f * coils
    // + c), one image per frame; nullptr for the plain crop
    const typename Cx<R>::T* maps;
    int coils;
    unsigned* check;                // checked builds: status word
    int64_t grid_elems, x_elems;    // extents of grid and x
};

template <typename R>
struct GradParams {
    Geom<R> g;
    const R* t[3];                  // coordinates, gather-list order
    const int* idx;                 // sample index of each list entry
    const R* dh[3];                 // derivative tables (shifted like hr)
    const typename Cx<R>::T* ph;    // sample phase, list order, or nullptr
    R phase_shift[3];               // s_d * gamma_d: d(phase)/d(tm_d) / i
    int64_t M;                      // list length (single frame)
    int coils;
    int apply_pb;
    R grid_scale;
    const typename Cx<R>::T* grid;  // [coils][Kprod], before phase_before
    const typename Cx<R>::T* gy;    // [coils][M] incoming gradient
    R* gtm;                         // [M][ndim] out
};

// Device binning (gbn_bin.cu): per-sample pass over coordinates tm
// ([M][ndim], plan precision, device) for the plan's tilings.
template <typename R>
struct BinParams {
    int ndim, F;
    int K[3], J[3], Tg[3], ntg[3], Ts[3], nts[3];
    int ntiles_g, ntiles_s;        // per frame
    double tm_limit;               // |tm| bound (larger or non-finite: err)
    int64_t M;
    const R* tm;
    const int64_t* foff;           // device frame offsets [F+1]
    int* err;                      // set to 1 on an invalid coordinate
    unsigned* gkey;                // [M] gather bin (frame * ntiles_g + tile)
    unsigned* gval;                // [M] sample index (sort payload)
    int* ecount;                   // [M] spread entries of each sample
    const int* eoff;               // [M] exclusive scan of ecount (emit pass)
    unsigned* skey;                // [entries] spread bin
    unsigned* sval;                // [entries] entry index (sort payload)
    int* em;                       // [entries] sample index
    short4* els;                   // [entries] window start in tile coordinates
};

// Work items from per-bin counts (starts = exclusive scans of the counts).
struct ItemParams {
    int nbins_g, nbins_s, ntiles_g, ntiles_s;
    int gchunk, schunk;
    const int* gcnt;
    const int* gstart;
    const int* scnt;
    const int* sstart;
    int* gparts;                   // parts pass: gather items per bin
    int* sparts;                   //   spread items per bin
    int* rslots;                   //   scratch slots per bin (parts of split tiles)
    int* rflag;                    //   1 for a split tile
    const int* goff;               // items pass: scans of the above
    const int* soff;
    const int* slotoff;
    const int* roff;
    int4* gitems;
    unsigned* gsize;               // sort key: chunk - count (heaviest first)
    unsigned* gorder;
    int4* sitems;
    int2* sslot;
    unsigned* ssize;
    unsigned* sorder;
    int4* rtiles;
};

// List packing: position i of a sorted list takes sample em[order[i]] (or
// order[i] itself when em is null, the gather list).
template <typename R>
struct PackParams {
    int ndim, F;
    int64_t len;
    const unsigned* order;
    const int* em;
    const short4* els;
    const R* tm;
    const typename Cx<R>::T* ph;
    const int64_t* foff;
    short4* ls_out;
    typename Cx<R>::T* ph_out;
    R* t_out[3];
    int* idx_out;
};

template <typename R> cudaError_t launch_bin_count(const BinParams<R>& p, cudaStream_t s);
template <typename R> cudaError_t launch_bin_emit(const BinParams<R>& p, cudaStream_t s);
cudaError_t launch_bin_hist(const unsigned* keys, int64_t n, int* counts, cudaStream_t s);
cudaError_t launch_bin_parts(const ItemParams& p, cudaStream_t s);
cudaError_t launch_bin_items(const ItemParams& p, cudaStream_t s);
cudaError_t launch_permute_int4(const int4* in, const unsigned* order, int64_t n, int4* out, cudaStream_t s);
cudaError_t launch_permute_int2(const int2* in, const unsigned* order, int64_t n, int2* out, cudaStream_t s);
template <typename R> cudaError_t launch_bin_pack(const PackParams<R>& p, cudaStream_t s);

// Pruned FFT pass along a strided axis (gbn_colfft.cu): planes x planes2
// arrays at offsets y * ps + z * ps2, each [L][S] (S columns, row stride S);
// rows >= nin are read as zero, rows >= nout are not written.  in == out is
// allowed.
struct ColFftParams {
    const float2* in;
    float2* out;
    int64_t S;                      // columns per array, and the row stride (elements)
    int64_t ps, ps2;                // array strides (elements)
    int planes, planes2;
    int L, nin, nout;
    const float2* tw;               // exp(-2 pi i m / L), m < L
    unsigned* check;                // checked builds: status word and extents
    int64_t in_elems, out_elems;
};
bool colfft_supported(int L);
// sign -1: forward (exp(-2 pi i nk / L)), +1: inverse (unnormalised)
cudaError_t launch_colfft(const ColFftParams& p, int sign, cudaStream_t s);

// Row passes of the 2-D and 3-D transforms with pad / crop folded in
// (gbn_rowfft.cu).  Rows r < planes * N2 * N1 (N2 = 1 in 2-D): plane
// r / (N1 N2), image row (n2, n1) of [planes][N2][N1][N0] and grid row at
// plane * gsp + n2 * gs2 + n1 * gs1 (L = K0 values).  sign -1: sn * image ->
// forward FFT -> grid row; +1: grid row -> inverse FFT -> first N0 values *
// scale * sn -> image.
struct RowFftParams {
    const float2* in;               // forward: image; inverse: grid
    float2* out;                    // forward: grid; inverse: image
    const float* sn;                // [N2][N1][N0]
    float scale;                    // inverse only
    int planes, N0, N1, N2, L;
    int64_t gsp, gs1, gs2;
    const float2* tw;               // exp(-2 pi i m / L), m < L
    unsigned* check;                // checked builds: status word and extents
    int64_t in_elems, out_elems;
};
bool rowfft_supported(int L);
cudaError_t launch_rowfft(const RowFftParams& p, int sign, cudaStream_t s);

template <typename R> cudaError_t launch_gather(const GatherParams<R>& p, cudaStream_t s);
template <typename R> cudaError_t launch_spread(const SpreadParams<R>& p, cudaStream_t s);
template <typename R> cudaError_t launch_reduce(const ReduceParams<R>& p, cudaStream_t s);
template <typename R> cudaError_t launch_pad(const PadParams<R>& p, cudaStream_t s);
template <typename R> cudaError_t launch_crop(const CropParams<R>& p, cudaStream_t s);
template <typename R> cudaError_t launch_grad(const GradParams<R>& p, cudaStream_t s);
template <typename R> cudaError_t launch_coef(const CoefParams<R>& p, cudaStream_t s);

// Shared-memory bytes needed by the gather / spread kernels for a lane layout.
template <typename R> size_t gather_smem(const Geom<R>& g, const Lanes& ln);
template <typename R> size_t spread_smem(const Geom<R>& g, const Lanes& ln);
// Threads of a spread CTA for a tiling (one warp per register block).
int spread_threads(int ndim, const int* T);

// Raise a kernel's dynamic shared-memory limit to at least `bytes` on the
// current device.  The attribute is set once per (kernel, device) and size
// (later launches needing no more skip the call), so launches recorded in a
// CUDA graph after a warm-up call make no attribute call.
cudaError_t ensure_dynamic_smem(const void* kernel, size_t bytes);

// CTAs of `kernel` (with this block size and dynamic shared memory) that fit
// on the current device at once: the grid of a persistent launch.  Cached
// per (kernel, device, threads, smem); 0 if the query fails.
int resident_ctas(const void* kernel, int threads, size_t smem);

// Address and size of the fixed no-alloc scratch array on the current device
// (gbn_noalloc.cu); looked up on every request.
cudaError_t noalloc_scratch(void** ptr, size_t* bytes);

cudaError_t launch_dtft(bool adjoint, int ndim, const int* Nd, const double* n_shift,
                        const double* omega, int64_t M, const double2* in, double2* out,
                        int reps, cudaStream_t s);

}  // namespace gbn
