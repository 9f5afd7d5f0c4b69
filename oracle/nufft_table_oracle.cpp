// Oracle (test infrastructure only): a CPU restatement of the reference's
// table-mode interpolation, used to check the CUDA path and as the timed
// CPU baseline ("port").  It is never linked into the product library.
//
// Algorithm followed (reference file:line):
//   forward 1-D  mrrt/nufft/_extensions/c/nufft_table.template.c:43-141
//   adjoint 1-D  nufft_table.template.c:144-305
//   adjoint 2-D  nufft_table.template.c:308-531
//   forward 2-D  nufft_table.template.c:538-707
//   forward 3-D  nufft_table.template.c:710-921
//   adjoint 3-D  nufft_table.template.c:924-1206
//
// Per tap the reference computes, in the working precision T:
//   koff = 1 + floor(t - J/2)           (double)
//   p    = (t - k) * L                  (T)
//   n    = floor(p), alf = p - n        (T)
//   coef = (1 - alf) h[n] + alf h[n+1]  (table centred at floor(J L / 2))
//   kmod = k mod K                      (periodic wrap, k may be negative)
// The forward is a separable gather (axis 0 innermost); the adjoint is the
// matching scatter with conj(coef).  Parallelisation mirrors the reference:
// OpenMP over samples for the forward, over repetitions (coils) for the
// adjoint, so one coil's adjoint is single-threaded as it is there.
//
// Arrays follow the reference's Fortran layout: tm is [M, ndim] (column d
// at tm + d*M), the grid is [K1, K2, K3, N] with axis 0 fastest, samples are
// [M, N].  Real and imaginary parts are separate planes, as in the Cython
// wrapper (mrrt/nufft/_extensions/_nufft_table.pyx:215-441).
#include <cmath>
#include <cstring>
#include <cstdint>

namespace {

template <typename T>
struct Axis {
    const T* hr;   // real table, already shifted to its centre
    const T* hi;   // imaginary table (nullptr for a real kernel)
    int J, K, L;
};

template <typename T>
inline Axis<T> make_axis(const T* hr, const T* hi, int J, int K, int L) {
    const int ncenter = (int)std::floor((double)J * (double)L / 2.0);
    Axis<T> a;
    a.hr = hr + ncenter;
    a.hi = hi ? hi + ncenter : nullptr;
    a.J = J; a.K = K; a.L = L;
    return a;
}

inline int wrap(int k, int K) {
    int r = k % K;
    return r < 0 ? r + K : r;
}

// Coefficient of tap k for coordinate t (complex in general).
template <typename T, bool CX>
inline void tap(const Axis<T>& a, T t, int k, T* cr, T* ci) {
    const T p = (t - (T)k) * (T)a.L;
    const int n = (int)std::floor(p);
    const T alf = p - (T)n;
    *cr = ((T)1 - alf) * a.hr[n] + alf * a.hr[n + 1];
    if (CX) *ci = ((T)1 - alf) * a.hi[n] + alf * a.hi[n + 1];
    else *ci = (T)0;
}

template <typename T>
inline int first_tap(T t, int J) {
    return 1 + (int)std::floor((double)t - (double)J / 2.0);
}

// ---- forward (gather) -----------------------------------------------------

template <typename T, bool CX>
void fwd_1d(const Axis<T>& a0, const T* tm, int64_t M,
            const T* ckr, const T* cki, T* fr, T* fi) {
#pragma omp parallel for schedule(static)
    for (int64_t m = 0; m < M; ++m) {
        const T t0 = tm[m];
        int k = first_tap(t0, a0.J);
        T sr = 0, si = 0;
        for (int j = 0; j < a0.J; ++j, ++k) {
            T cr, ci;
            tap<T, CX>(a0, t0, k, &cr, &ci);
            const int q = wrap(k, a0.K);
            if (CX) {
                sr += cr * ckr[q] - ci * cki[q];
                si += cr * cki[q] + ci * ckr[q];
            } else {
                sr += cr * ckr[q];
                si += cr * cki[q];
            }
        }
        fr[m] = sr;
        fi[m] = si;
    }
}

template <typename T, bool CX>
void fwd_2d(const Axis<T>& a0, const Axis<T>& a1, const T* tm, int64_t M,
            const T* ckr, const T* cki, T* fr, T* fi) {
#pragma omp parallel for schedule(dynamic, 1000)
    for (int64_t m = 0; m < M; ++m) {
        const T t0 = tm[m];
        const T t1 = tm[M + m];
        const int k0s = first_tap(t0, a0.J);
        int k1 = first_tap(t1, a1.J);
        T s2r = 0, s2i = 0;
        for (int j1 = 0; j1 < a1.J; ++j1, ++k1) {
            T c1r, c1i;
            tap<T, CX>(a1, t1, k1, &c1r, &c1i);
            const int64_t row = (int64_t)wrap(k1, a1.K) * a0.K;
            T s1r = 0, s1i = 0;
            int k0 = k0s;
            for (int j0 = 0; j0 < a0.J; ++j0, ++k0) {
                T c0r, c0i;
                tap<T, CX>(a0, t0, k0, &c0r, &c0i);
                const int64_t q = row + wrap(k0, a0.K);
                s1r += c0r * ckr[q] - c0i * cki[q];
                s1i += c0r * cki[q] + c0i * ckr[q];
            }
            s2r += c1r * s1r - c1i * s1i;
            s2i += c1r * s1i + c1i * s1r;
        }
        fr[m] = s2r;
        fi[m] = s2i;
    }
}

template <typename T, bool CX>
void fwd_3d(const Axis<T>& a0, const Axis<T>& a1, const Axis<T>& a2,
            const T* tm, int64_t M, const T* ckr, const T* cki, T* fr, T* fi) {
#pragma omp parallel for schedule(dynamic, 1000)
    for (int64_t m = 0; m < M; ++m) {
        const T t0 = tm[m], t1 = tm[M + m], t2 = tm[2 * M + m];
        const int k0s = first_tap(t0, a0.J);
        const int k1s = first_tap(t1, a1.J);
        int k2 = first_tap(t2, a2.J);
        T s3r = 0, s3i = 0;
        for (int j2 = 0; j2 < a2.J; ++j2, ++k2) {
            T c2r, c2i;
            tap<T, CX>(a2, t2, k2, &c2r, &c2i);
            const int k2m = wrap(k2, a2.K);
            T s2r = 0, s2i = 0;
            int k1 = k1s;
            for (int j1 = 0; j1 < a1.J; ++j1, ++k1) {
                T c1r, c1i;
                tap<T, CX>(a1, t1, k1, &c1r, &c1i);
                const int64_t row =
                    ((int64_t)k2m * a1.K + wrap(k1, a1.K)) * a0.K;
                T s1r = 0, s1i = 0;
                int k0 = k0s;
                for (int j0 = 0; j0 < a0.J; ++j0, ++k0) {
                    T c0r, c0i;
                    tap<T, CX>(a0, t0, k0, &c0r, &c0i);
                    const int64_t q = row + wrap(k0, a0.K);
                    s1r += c0r * ckr[q] - c0i * cki[q];
                    s1i += c0r * cki[q] + c0i * ckr[q];
                }
                s2r += c1r * s1r - c1i * s1i;
                s2i += c1r * s1i + c1i * s1r;
            }
            s3r += c2r * s2r - c2i * s2i;
            s3i += c2r * s2i + c2i * s2r;
        }
        fr[m] = s3r;
        fi[m] = s3i;
    }
}

// ---- adjoint (scatter), one repetition; the caller loops over coils ----

template <typename T, bool CX>
void adj_1d(const Axis<T>& a0, const T* tm, int64_t M,
            const T* fr, const T* fi, T* ckr, T* cki) {
    for (int64_t m = 0; m < M; ++m) {
        const T t0 = tm[m];
        const T vr = fr[m], vi = fi[m];
        int k = first_tap(t0, a0.J);
        for (int j = 0; j < a0.J; ++j, ++k) {
            T cr, ci;
            tap<T, CX>(a0, t0, k, &cr, &ci);
            const int q = wrap(k, a0.K);
            ckr[q] += cr * vr + ci * vi;
            cki[q] += cr * vi - ci * vr;
        }
    }
}

template <typename T, bool CX>
void adj_2d(const Axis<T>& a0, const Axis<T>& a1, const T* tm, int64_t M,
            const T* fr, const T* fi, T* ckr, T* cki) {
    for (int64_t m = 0; m < M; ++m) {
        const T t0 = tm[m], t1 = tm[M + m];
        const T vr = fr[m], vi = fi[m];
        const int k0s = first_tap(t0, a0.J);
        int k1 = first_tap(t1, a1.J);
        for (int j1 = 0; j1 < a1.J; ++j1, ++k1) {
            T c1r, c1i;
            tap<T, CX>(a1, t1, k1, &c1r, &c1i);
            const int64_t row = (int64_t)wrap(k1, a1.K) * a0.K;
            const T v1r = c1r * vr + c1i * vi;
            const T v1i = c1r * vi - c1i * vr;
            int k0 = k0s;
            for (int j0 = 0; j0 < a0.J; ++j0, ++k0) {
                T c0r, c0i;
                tap<T, CX>(a0, t0, k0, &c0r, &c0i);
                const int64_t q = row + wrap(k0, a0.K);
                ckr[q] += c0r * v1r + c0i * v1i;
                cki[q] += c0r * v1i - c0i * v1r;
            }
        }
    }
}

template <typename T, bool CX>
void adj_3d(const Axis<T>& a0, const Axis<T>& a1, const Axis<T>& a2,
            const T* tm, int64_t M, const T* fr, const T* fi,
            T* ckr, T* cki) {
    for (int64_t m = 0; m < M; ++m) {
        const T t0 = tm[m], t1 = tm[M + m], t2 = tm[2 * M + m];
        const T vr = fr[m], vi = fi[m];
        const int k0s = first_tap(t0, a0.J);
        const int k1s = first_tap(t1, a1.J);
        int k2 = first_tap(t2, a2.J);
        for (int j2 = 0; j2 < a2.J; ++j2, ++k2) {
            T c2r, c2i;
            tap<T, CX>(a2, t2, k2, &c2r, &c2i);
            const int k2m = wrap(k2, a2.K);
            const T v2r = c2r * vr + c2i * vi;
            const T v2i = c2r * vi - c2i * vr;
            int k1 = k1s;
            for (int j1 = 0; j1 < a1.J; ++j1, ++k1) {
                T c1r, c1i;
                tap<T, CX>(a1, t1, k1, &c1r, &c1i);
                const int64_t row =
                    ((int64_t)k2m * a1.K + wrap(k1, a1.K)) * a0.K;
                const T v1r = c1r * v2r + c1i * v2i;
                const T v1i = c1r * v2i - c1i * v2r;
                int k0 = k0s;
                for (int j0 = 0; j0 < a0.J; ++j0, ++k0) {
                    T c0r, c0i;
                    tap<T, CX>(a0, t0, k0, &c0r, &c0i);
                    const int64_t q = row + wrap(k0, a0.K);
                    ckr[q] += c0r * v1r + c0i * v1i;
                    cki[q] += c0r * v1i - c0i * v1r;
                }
            }
        }
    }
}

template <typename T>
int interp_forward(int ndim, const int* K, const int* J, int L,
                   const T* const* hr, const T* const* hi, const T* tm,
                   int64_t M, const T* ckr, const T* cki, int N,
                   T* fr, T* fi) {
    if (ndim < 1 || ndim > 3 || M < 0 || N < 0 || L < 1) return -1;
    Axis<T> ax[3];
    int64_t Kprod = 1;
    bool cx = hi != nullptr;
    for (int d = 0; d < ndim; ++d) {
        if (J[d] < 1 || K[d] < J[d]) return -1;
        ax[d] = make_axis<T>(hr[d], hi ? hi[d] : nullptr, J[d], K[d], L);
        Kprod *= K[d];
        if (!ax[d].hi) cx = false;
    }
    for (int n = 0; n < N; ++n) {
        const T* gr = ckr + (int64_t)n * Kprod;
        const T* gi = cki + (int64_t)n * Kprod;
        T* yr = fr + (int64_t)n * M;
        T* yi = fi + (int64_t)n * M;
        if (cx) {
            if (ndim == 1) fwd_1d<T, true>(ax[0], tm, M, gr, gi, yr, yi);
            else if (ndim == 2)
                fwd_2d<T, true>(ax[0], ax[1], tm, M, gr, gi, yr, yi);
            else fwd_3d<T, true>(ax[0], ax[1], ax[2], tm, M, gr, gi, yr, yi);
        } else {
            if (ndim == 1) fwd_1d<T, false>(ax[0], tm, M, gr, gi, yr, yi);
            else if (ndim == 2)
                fwd_2d<T, false>(ax[0], ax[1], tm, M, gr, gi, yr, yi);
            else fwd_3d<T, false>(ax[0], ax[1], ax[2], tm, M, gr, gi, yr, yi);
        }
    }
    return 0;
}

template <typename T>
int interp_adjoint(int ndim, const int* K, const int* J, int L,
                   const T* const* hr, const T* const* hi, const T* tm,
                   int64_t M, const T* fr, const T* fi, int N,
                   T* ckr, T* cki) {
    if (ndim < 1 || ndim > 3 || M < 0 || N < 0 || L < 1) return -1;
    Axis<T> ax[3];
    int64_t Kprod = 1;
    bool cx = hi != nullptr;
    for (int d = 0; d < ndim; ++d) {
        if (J[d] < 1 || K[d] < J[d]) return -1;
        ax[d] = make_axis<T>(hr[d], hi ? hi[d] : nullptr, J[d], K[d], L);
        Kprod *= K[d];
        if (!ax[d].hi) cx = false;
    }
#pragma omp parallel for schedule(static)
    for (int n = 0; n < N; ++n) {
        T* gr = ckr + (int64_t)n * Kprod;
        T* gi = cki + (int64_t)n * Kprod;
        std::memset(gr, 0, sizeof(T) * (size_t)Kprod);
        std::memset(gi, 0, sizeof(T) * (size_t)Kprod);
        const T* yr = fr + (int64_t)n * M;
        const T* yi = fi + (int64_t)n * M;
        if (cx) {
            if (ndim == 1) adj_1d<T, true>(ax[0], tm, M, yr, yi, gr, gi);
            else if (ndim == 2)
                adj_2d<T, true>(ax[0], ax[1], tm, M, yr, yi, gr, gi);
            else adj_3d<T, true>(ax[0], ax[1], ax[2], tm, M, yr, yi, gr, gi);
        } else {
            if (ndim == 1) adj_1d<T, false>(ax[0], tm, M, yr, yi, gr, gi);
            else if (ndim == 2)
                adj_2d<T, false>(ax[0], ax[1], tm, M, yr, yi, gr, gi);
            else adj_3d<T, false>(ax[0], ax[1], ax[2], tm, M, yr, yi, gr, gi);
        }
    }
    return 0;
}

}  // namespace

extern "C" {

// hi == nullptr (or all entries null) selects the real-kernel variant.
int oracle_interp_forward_f32(int ndim, const int* K, const int* J, int L,
                              const float* const* hr, const float* const* hi,
                              const float* tm, int64_t M, const float* ckr,
                              const float* cki, int N, float* fr, float* fi) {
    return interp_forward<float>(ndim, K, J, L, hr, hi, tm, M, ckr, cki, N,
                                 fr, fi);
}

int oracle_interp_forward_f64(int ndim, const int* K, const int* J, int L,
                              const double* const* hr,
                              const double* const* hi, const double* tm,
                              int64_t M, const double* ckr, const double* cki,
                              int N, double* fr, double* fi) {
    return interp_forward<double>(ndim, K, J, L, hr, hi, tm, M, ckr, cki, N,
                                  fr, fi);
}

int oracle_interp_adjoint_f32(int ndim, const int* K, const int* J, int L,
                              const float* const* hr, const float* const* hi,
                              const float* tm, int64_t M, const float* fr,
                              const float* fi, int N, float* ckr,
                              float* cki) {
    return interp_adjoint<float>(ndim, K, J, L, hr, hi, tm, M, fr, fi, N,
                                 ckr, cki);
}

int oracle_interp_adjoint_f64(int ndim, const int* K, const int* J, int L,
                              const double* const* hr,
                              const double* const* hi, const double* tm,
                              int64_t M, const double* fr, const double* fi,
                              int N, double* ckr, double* cki) {
    return interp_adjoint<double>(ndim, K, J, L, hr, hi, tm, M, fr, fi, N,
                                  ckr, cki);
}

}  // extern "C"
