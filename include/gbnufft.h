/* gbnufft.h -- C ABI of the GB300 table-mode NUFFT (libgbnufft.so).
 *
 * Plain C types only: host pointers, device pointers (void*), sizes, a CUDA
 * stream passed as void* (0 = legacy default stream).  Every entry point
 * returns a status code (GBN_OK on success); gbn_last_error() describes the
 * most recent failure on the calling thread.  No entry point aborts.
 *
 * A plan owns device working storage (the oversampled grid, the partial sums
 * of split tiles, the work counters of the 3-D interpolation launch): the
 * calls on one plan must not overlap in time.  Issue them on one stream, or
 * synchronise between streams; separate plans may run concurrently.
 *
 * Axis convention.  The plan is described in MEMORY-AXIS order: axis 0 is
 * the fastest-varying index of the image and of the oversampled grid.  A
 * Fortran-ordered numpy image of shape Nd (the reference's layout,
 * mrrt/nufft/_nufft.py:1306) maps omega column d to memory axis d; a
 * C-ordered [batch, N0, N1] tensor maps omega column d to memory axis
 * ndim-1-d.  The Python layer performs that mapping.
 *
 * Data layouts (complex values are interleaved re/im, complex64 for single
 * precision, complex128 for double):
 *   image   x : [frames][coils][N_{ndim-1}]...[N_0]
 *   grid      : [frames][coils][K_{ndim-1}]...[K_0]
 *   samples y : frame f occupies [coils][M_f] starting at
 *               coils * frame_offsets[f]
 *   tm        : host, [M_total][ndim] with column d = coordinate on memory
 *               axis d, in units of oversampled-grid cells (omega / (2 pi / K)),
 *               the reference's tm (mrrt/nufft/_nufft.py:338-342).
 */
#ifndef GBNUFFT_H
#define GBNUFFT_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GBN_OK 0
#define GBN_ERR_INVALID 1     /* bad argument (shape, size, pointer, flag)   */
#define GBN_ERR_CUDA 2        /* CUDA runtime error                           */
#define GBN_ERR_CUFFT 3       /* cuFFT error                                  */
#define GBN_ERR_NOMEM 4       /* device or host allocation failed             */
#define GBN_ERR_UNSUPPORTED 5 /* valid request outside what is implemented    */
#define GBN_ERR_TOOLARGE 6    /* request exceeds a fixed capacity             */

#define GBN_PRECISION_SINGLE 0
#define GBN_PRECISION_DOUBLE 1
#define GBN_PHASING_REAL 0
#define GBN_PHASING_COMPLEX 1

/* Geometry flags.  By default a plan precomputes every sample's table
 * coefficients once (list order, jsum = sum(Jd) values per sample and per
 * spread-list entry) and the kernels read them; TABLE_ONLY keeps no such
 * buffers and interpolates the tables inside the kernels instead (same
 * results bit for bit, less device memory).                               */
#define GBN_FLAG_TABLE_ONLY 1
/* By default the single-precision 2-D and 3-D plans run the FFT's pass
 * along the slowest axis on the library's own pruned kernel when that
 * axis's length is 64, 96, 128, 192, 256, 384, 512 or 768 (it reads
 * only the rows that hold data and writes only the rows the crop reads);
 * CUFFT_ONLY runs every pass through cuFFT instead.                         */
#define GBN_FLAG_CUFFT_ONLY 2

/* Geometry of one operator (or of a series of frames sharing it). */
typedef struct gbn_geometry {
    int ndim;              /* 1, 2 or 3                                       */
    int Nd[3];             /* image size per memory axis                      */
    int Kd[3];             /* oversampled grid size per memory axis           */
    int Jd[3];             /* kernel width per memory axis (1..8)             */
    int L;                 /* table samples per grid unit                     */
    int precision;         /* GBN_PRECISION_*                                 */
    int phasing;           /* GBN_PHASING_*                                   */
    int ortho;             /* 1: orthonormal FFT scaling                      */
    double adjoint_scale;  /* adjoint_scalefactor                             */
    /* real phasing: phase_before(k) = exp(i * sum_d c_d k_d), the per-axis
     * coefficient c_d = 2 pi n_mid_d / K_d; the partial sums are rounded in
     * the working precision in the order given by pb_order (reference axis
     * order, mrrt/nufft/_nufft.py:703-715).                                  */
    double pb_coef[3];
    int pb_order[3];
    int n_frames;          /* number of sample sets (1 for a plain operator) */
    int tile[3];           /* gather tile edge per memory axis, 0 = default   */
    int stile[3];          /* spread tile edge per memory axis, 0 = default   */
    int max_coils;         /* largest coil count a call will use              */
    int flags;             /* GBN_FLAG_* bits, 0 by default                   */
} gbn_geometry;

typedef struct gbn_plan gbn_plan;

/* Create a plan.  Replaces the reference's per-operator set-up
 * (NufftBase.__init__ table branch, mrrt/nufft/_nufft.py:216-390).
 *   h_re[d], h_im[d] : host lookup tables of length Jd[d]*L+1 for memory axis d
 *                      (h_im NULL or all-NULL for phasing real).
 *   sn               : host deapodisation [N_{ndim-1}]...[N_0] (real).
 *   frame_offsets    : host [n_frames+1] sample offsets (frame_offsets[0] = 0).
 *   tm               : host [M_total][ndim] coordinates (see header note).
 *   sample_phase     : host [M_total] complex, applied after interpolation and
 *                      conjugated before spreading (phase_after for real
 *                      phasing, phase_shift for complex phasing); may be NULL.
 * Table, tm and phase arrays are in the plan precision (float or double).    */
int gbn_plan_create(gbn_plan** plan, const gbn_geometry* geom,
                    const void* const* h_re, const void* const* h_im,
                    const void* sn, const int64_t* frame_offsets,
                    const void* tm, const void* sample_phase, int device);

/* Replace the sample coordinates (and sample phase) of an existing plan with
 * the same frame offsets; rebuilds the tile lists.                          */
int gbn_plan_set_points(gbn_plan* plan, const void* tm,
                        const void* sample_phase);

/* gbn_plan_set_points with DEVICE arrays: tm [M_total][ndim] and
 * sample_phase [M_total] (or NULL) in device memory, plan precision.  The
 * tile lists are built on the device by a sort of the samples (stable, so
 * the spread's summation order, hence its result, is the same in every
 * run); the coordinates never pass through host memory.  The call waits
 * for work already queued on the device, and for two 4-to-16-byte counts it
 * reads back on `stream` (to size the lists and launches), then returns with
 * the rest queued on `stream`.  Invalid coordinates (non-finite, |tm| >
 * 2^22) return GBN_ERR_INVALID and keep the previous lists.  Replaces the
 * host-side tm = omega / gamma recomputation of the reference
 * (mrrt/nufft/_nufft.py:338-342) when a trajectory is optimised on the GPU. */
int gbn_plan_set_points_device(gbn_plan* plan, const void* tm,
                               const void* sample_phase, void* stream);

int gbn_plan_destroy(gbn_plan* plan);

/* Forward NUFFT, image -> samples, `coils` coils per frame.
 * Replaces nufft_forward (mrrt/nufft/_nufft.py:1275-1397) in table mode:
 * deapodise + zero-pad, Kd-point FFT, phase_before, table interpolation
 * (interp{1,2,3}_table, mrrt/nufft/_interp_table.py:26-159, C kernels
 * {float,double}_interp{1,2,3}_table1_{real,complex}_forward,
 * mrrt/nufft/_extensions/c/nufft_table.template.h:98-342), sample phase.   */
int gbn_forward(gbn_plan* plan, const void* x, void* y, int coils,
                void* stream);

/* Adjoint NUFFT, samples -> image.  Replaces nufft_adj
 * (mrrt/nufft/_nufft.py:1459-1578) in table mode, including the adjoint
 * spread interp{1,2,3}_table_adj (C kernels *_adj in the same header).     */
int gbn_adjoint(gbn_plan* plan, const void* y, void* x, int coils,
                void* stream);

/* The same transforms on HOST buffers, as the reference's NufftBase.fft /
 * NufftBase.adj take and return host arrays (mrrt/nufft/_nufft.py:425-452
 * and 454-481).  x and y are host pointers in the layouts above (pageable
 * or pinned); the call copies the input in, transforms on `stream` and
 * returns once the result is in host memory.  Single-frame batches of 32
 * coils or more run as a copy / transform pipeline of 16-coil chunks (the
 * forward starts with two 8-coil chunks) on two copy streams the plan owns;
 * every copy, pageable or pinned, runs on the copy engines.  Pinned outputs
 * let the copies run at the link's full rate.  Device pointers and calls
 * during graph capture are rejected.                                        */
int gbn_forward_host(gbn_plan* plan, const void* x_host, void* y_host,
                     int coils, void* stream);
int gbn_adjoint_host(gbn_plan* plan, const void* y_host, void* x_host,
                     int coils, void* stream);

/* Coil-sensitivity (SENSE) forward: y = NUFFT(maps[c] * image[f]) for every
 * frame f and coil c, the coil-map multiply fused into the deapodisation
 * pass (the coil images are never stored).  The MRI system operator of
 * mrrt.operators, built on the reference's NUFFT, applies maps before
 * nufft_forward (mrrt/nufft/_nufft.py:3-5 names it); this fuses that step.
 *   image : [frames][N...]   one image per frame
 *   maps  : [coils][N...]    coil sensitivities, shared by all frames
 *   y     : as for gbn_forward.                                             */
int gbn_forward_sense(gbn_plan* plan, const void* image, const void* maps,
                      void* y, int coils, void* stream);

/* Coil-combining adjoint: image[f] = sum_c conj(maps[c]) * adjoint_c, the
 * sum (in coil order) fused into the crop pass.                             */
int gbn_adjoint_sense(gbn_plan* plan, const void* y, const void* maps,
                      void* image, int coils, void* stream);

/* Table interpolation alone: oversampled grid -> samples, no phases, no FFT.
 * Replaces interp{1,2,3}_table (mrrt/nufft/_interp_table.py:26-159).        */
int gbn_interp_forward(gbn_plan* plan, const void* grid, void* y, int coils,
                       void* stream);

/* Adjoint table interpolation alone: samples -> oversampled grid.  Replaces
 * interp{1,2,3}_table_adj (mrrt/nufft/_interp_table.py:46-191).            */
int gbn_interp_adjoint(gbn_plan* plan, const void* y, void* grid, int coils,
                       void* stream);

/* Capacity of the fixed scratch array behind gbn_interp_adjoint_noalloc.
 * Under lazy module loading (CUDA_MODULE_LOADING=LAZY, the CUDA default) the
 * array is reserved on a device only once a process first calls the no-alloc
 * entry point there; with CUDA_MODULE_LOADING=EAGER every process that loads
 * libgbnufft reserves it on each device it initialises.                     */
#define GBN_NOALLOC_SCRATCH_BYTES (64u * 1024u * 1024u)

/* Same result as gbn_interp_adjoint, for callers that must not allocate
 * device memory during a call: a process whose device memory is committed
 * up front to a fixed budget, or a pipeline that cannot let a cudaMalloc or
 * cudaFree (which may synchronise the whole device) happen between its
 * launches.  gbn_interp_adjoint grows a per-plan buffer for the partial sums
 * of tiles split across CTAs; this variant keeps them in one statically
 * sized array per device instead and never calls an allocator.
 * No counterpart in the reference.
 *   - Limit: the partial sums of one call must fit GBN_NOALLOC_SCRATCH_BYTES
 *     (64 MiB); a larger request returns GBN_ERR_TOOLARGE before anything
 *     is launched.  Fewer coils per call, or gbn_interp_adjoint, fit it.
 *   - Every call looks up the array's address on the current device (no
 *     allocation; it stays right after a device reset).  The first call on
 *     a device can also load the module holding the array: make that first
 *     call before any stream capture.
 *   - Every plan on a device shares the one array: calls whose kernels can
 *     overlap in time (unordered streams, or several host threads) race on
 *     it and corrupt each other's results.  Order them on one stream or
 *     synchronise between them.                                            */
int gbn_interp_adjoint_noalloc(gbn_plan* plan, const void* y, void* grid,
                               int coils, void* stream);

/* Sparse-matrix mode: interpolate with precomputed weights instead of the
 * tables.  w_re[d] (and w_im[d] for phasing complex) are host arrays
 * [M_total][Jd[d]] in the plan precision: the coefficient of tap j of
 * sample m on memory axis d, the tap cells being first_tap + j as in table
 * mode.  The interpolation matrix is their per-sample outer product, as in
 * the reference's sparse operator (_init_sparsemat,
 * mrrt/nufft/_nufft.py:750-877, applied as p * xk / p.H * xk at
 * _nufft.py:1384 and 1505).  w_re NULL returns to table mode;
 * gbn_plan_set_points drops the weights.                                     */
int gbn_plan_set_weights(gbn_plan* plan, const void* const* w_re,
                         const void* const* w_im);

/* Upload derivative tables dh/dt (host, length Jd[d]*L+1 per memory axis, plan
 * precision) used by gbn_grad_tm.  No counterpart in the reference.          */
int gbn_plan_set_dtables(gbn_plan* plan, const void* const* dtab);

/* Gradient of a real loss with respect to the sample coordinates tm
 * (single-frame plans, real phasing).
 *   grid : the forward's oversampled grid before phase_before, i.e. the FFT
 *          output a gbn_forward call with the same coil count leaves in the
 *          buffer that gbn_forward_grid returns (callers copy it if they need
 *          it later), in that buffer's layout.
 *   gy   : [coils][M] dL/dy in torch's convention (dL/dRe + i dL/dIm).
 *   phase_shift : host [ndim], d(sample phase)/d(tm_d) divided by i, i.e.
 *          (n_shift_d - n_mid_d) * 2 pi / Kd[d] for phase_after.
 *   gtm  : out, [M][ndim] dL/dtm (plan precision), summed over coils.
 * No counterpart in the reference (it has no autograd).                     */
int gbn_grad_tm(gbn_plan* plan, const void* grid, const void* gy,
                const double* phase_shift, void* gtm, int coils, void* stream);

/* Device pointer of the plan's forward grid buffer (valid until the next
 * call on the plan).  Its layout is the transform's own: [K1][coils][K0] for
 * 2-D plans (row k1 of every coil plane together, so the FFT's row pass skips
 * the zero-padded rows), [coils][K...] for 1-D and 3-D plans.  The
 * interpolation-only entry points keep the [planes][K...] layout.           */
int gbn_forward_grid(gbn_plan* plan, void** grid);

/* Exact direct NUDFT in double precision on the GPU (the reference's
 * dtft / dtft_adj, mrrt/nufft/_dtft.py:16-216).
 *   omega : device [M][ndim] (double), column d pairs with memory axis d.
 *   x     : device [reps][N_{ndim-1}]...[N_0] complex128.
 *   y     : device [reps][M] complex128.                                     */
int gbn_dtft_forward(int ndim, const int* Nd, const double* n_shift,
                     const void* omega, int64_t M, const void* x, void* y,
                     int reps, void* stream);
int gbn_dtft_adjoint(int ndim, const int* Nd, const double* n_shift,
                     const void* omega, int64_t M, const void* y, void* x,
                     int reps, void* stream);

/* Plan statistics: 8 int64 values (gather items, spread items, split tiles,
 * gather list length, spread list length, tiles, device bytes held, M_total). */
int gbn_plan_stats(const gbn_plan* plan, int64_t* out8);

/* Message of the last failure on the calling thread ("" if none). */
const char* gbn_last_error(void);

/* Library version string. */
const char* gbn_version(void);

/* Testing hook, no counterpart in the reference: the bounds-check status of
 * a plan in the checked build (libgbnufft_checked.so, compiled with
 * GBN_CHECKED).  That build tests every global index its kernels form from
 * plan data against the extent of the buffer it addresses, skips an access
 * that fails, and records the failure as a bit in *out: 1 grid read, 2 grid
 * write, 4 sample read, 8 sample write, 16 split-tile scratch, 32 list
 * range, 64 image.  The call waits for the device, returns the bits
 * recorded since the last call and clears them.  In the normal build it
 * returns GBN_ERR_UNSUPPORTED with *out = 0.                               */
int gbn_debug_check_status(gbn_plan* plan, unsigned* out);

/* Testing hook, no counterpart in the reference: host-side fault injection
 * for the allocation-failure paths.  After this call, `after` more device
 * allocations made by the library succeed and the next one fails as if
 * cudaMalloc had reported cudaErrorMemoryAllocation (nothing is requested
 * from the device for it); the call that needed it returns GBN_ERR_NOMEM.
 * A negative value turns the injection off.  Process-wide.                 */
int gbn_debug_fail_alloc(long long after);

#ifdef __cplusplus
}
#endif

#endif /* GBNUFFT_H */
