/*
 * Oracle library (TEST INFRASTRUCTURE ONLY): a CPU restatement of the
 * reference's tiled singular-value path, evelyne-ringoot/Avocado-sandwich
 * my_CU_svdval (CUDAbasedSVD/SVD_GPU.jl:257-283) on the KernelAbstractions
 * building blocks (the .jl files of KAbasedSVD/src).  It is the parity reference for the CUDA
 * library and the timed CPU baseline; the product never links or calls it.
 *
 * Stage 3 of the reference is LAPACK bdsdc('U','N') (KAbasedSVD/src/
 * bulgechasing.jl:50-53; OpenBLAS_jll 0.3.27 LAPACK, not vendored in the
 * reference).  The oracle restates the same quantity -- the singular values of
 * the upper bidiagonal -- with Kahan's bisection on the Golub-Kahan tridiagonal
 * (the published method of LAPACK dstebz), in double; the tests pin it against
 * LAPACK gesdd on the dense bidiagonal.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define OT float
#define OT_SUFFIX _s
#include "oracle_impl.h"
#undef OT
#undef OT_SUFFIX

#define OT double
#define OT_SUFFIX _d
#include "oracle_impl.h"
#undef OT
#undef OT_SUFFIX

int oracle_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void oracle_set_threads(int nthreads) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
}

/* Number of eigenvalues of the Golub-Kahan tridiagonal TGK(d, e) (zero
 * diagonal, off-diagonal d0, e0, d1, e1, ..., d_{n-1}) that are < x, via the
 * LDL^T pivot recurrence with the dstebz pivot guard. */
static int64_t tgk_count(const double *d, const double *e, int64_t n, double x, double pivmin) {
    int64_t cnt = 0;
    double q = -x;
    if (fabs(q) < pivmin) q = -pivmin;
    if (q < 0) ++cnt;
    for (int64_t i = 0; i < 2 * n - 1; ++i) {
        double off = (i & 1) ? e[i >> 1] : d[i >> 1];
        q = -x - off * off / q;
        if (fabs(q) < pivmin) q = -pivmin;
        if (q < 0) ++cnt;
    }
    return cnt;
}

/* Singular values of the upper bidiagonal (d[0..n-1], e[0..n-2]) in
 * descending order, each bisected to an absolute width of rel_tol * bound. */
void oracle_bidiag_svals(const double *d, const double *e, int64_t n, double *sigma, double rel_tol) {
    double bound = 0, maxsq = 0;
    for (int64_t i = 0; i < n; ++i) {
        double r = fabs(d[i]) + (i > 0 ? fabs(e[i - 1]) : 0.0) + (i + 1 < n ? fabs(e[i]) : 0.0);
        if (r > bound) bound = r;
        if (d[i] * d[i] > maxsq) maxsq = d[i] * d[i];
        if (i + 1 < n && e[i] * e[i] > maxsq) maxsq = e[i] * e[i];
    }
    double pivmin = 2.2250738585072014e-308 * (maxsq > 1 ? maxsq : 1);
    if (bound == 0) {
        for (int64_t k = 0; k < n; ++k) sigma[k] = 0;
        return;
    }
    double tol = rel_tol * bound;
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t k = 0; k < n; ++k) {
        /* k-th largest singular value = the (n + (n-1-k))-th smallest TGK eigenvalue
         * (0-based), i.e. the smallest x with count(x) > 2n-1-k. */
        int64_t target = 2 * n - 1 - k;
        double lo = 0, hi = bound * (1 + 1e-15) + pivmin;
        for (int it = 0; it < 200 && hi - lo > tol; ++it) {
            double mid = 0.5 * (lo + hi);
            if (tgk_count(d, e, n, mid, pivmin) > target)
                hi = mid;
            else
                lo = mid;
        }
        sigma[k] = 0.5 * (lo + hi);
    }
}

/* Extract diag / superdiag of a column-major n x n matrix. */
#define EXTRACT_BIDIAG(OTT)                                                              \
    for (int64_t i = 0; i < n; ++i) d[i] = (double)((const OTT *)a)[i + i * lda];         \
    for (int64_t i = 0; i + 1 < n; ++i) e[i] = (double)((const OTT *)a)[i + (i + 1) * lda];

void oracle_extract_bidiag_s(const float *a, int64_t n, int64_t lda, double *d, double *e) { EXTRACT_BIDIAG(float) }
void oracle_extract_bidiag_d(const double *a, int64_t n, int64_t lda, double *d, double *e) { EXTRACT_BIDIAG(double) }

/*
 * The whole reference path on the CPU: copy (SVD_GPU.jl:259), GE2BND
 * (Blockbidiag!), band -> bidiagonal (bidiagonalize), bidiagonal singular
 * values.  a is not modified.  Returns 0, or -1 when the arguments are outside
 * the reference's contract (SVD_GPU.jl:261-262: power-of-two tile >= 16
 * dividing n).
 */
#define SVDVALS_BODY(OTT, SUF)                                                          \
    if (b < 16 || (b & (b - 1)) != 0 || n <= 0 || n % b != 0) return -1;                  \
    OTT *w = (OTT *)malloc(sizeof(OTT) * (size_t)n * (size_t)n);                         \
    if (!w) return -2;                                                                   \
    for (int64_t j = 0; j < n; ++j) memcpy(w + j * n, a + j * lda, sizeof(OTT) * (size_t)n); \
    oracle_blockbidiag##SUF(w, n, n, b);                                                 \
    oracle_bidiagonalize##SUF(w, n, n, b);                                               \
    double *d = (double *)malloc(sizeof(double) * (size_t)n);                            \
    double *e = (double *)malloc(sizeof(double) * (size_t)(n > 1 ? n - 1 : 1));          \
    oracle_extract_bidiag##SUF(w, n, n, d, e);                                           \
    oracle_bidiag_svals(d, e, n, sigma, rel_tol);                                        \
    free(d);                                                                             \
    free(e);                                                                             \
    free(w);                                                                             \
    return 0;

int oracle_svdvals_s(const float *a, int64_t n, int64_t lda, int b, double *sigma, double rel_tol) {
    SVDVALS_BODY(float, _s)
}
int oracle_svdvals_d(const double *a, int64_t n, int64_t lda, int b, double *sigma, double rel_tol) {
    SVDVALS_BODY(double, _d)
}
