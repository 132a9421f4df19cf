/*
 * avs.h -- C ABI of the GB300-native tiled SVD (singular values only).
 *
 * Drop-in for the tiled-matrix singular-value entry point of
 * evelyne-ringoot/Avocado-sandwich:
 *
 *     my_CU_svdval(A::Matrix{Float32}, block_size)    CUDAbasedSVD/SVD_GPU.jl:257-270
 *     my_CU_svdval(A::CuMatrix{Float32}, block_size)  CUDAbasedSVD/SVD_GPU.jl:272-283
 *
 * and for the KernelAbstractions building blocks behind it
 * (TiledMatrix -> Blockbidiag! -> bidiagonalize -> diag_lapack,
 *  KAbasedSVD/src/TiledMatrix.jl:41, tiledalgos.jl:17, bulgechasing.jl:33,50).
 *
 * Every function is plain C: pointers, sizes and status codes.  Matrices are
 * column-major (Julia's layout) with a leading dimension.  "Host" entry points
 * take host pointers and do the host<->device copies themselves (the
 * Matrix{Float32} method); "_dev" entry points take device pointers that the
 * caller owns (the CuMatrix{Float32} method).  The input matrix of the SVD
 * entry points is never modified (the reference copies it first,
 * SVD_GPU.jl:259,273); the building blocks and the out-of-core calls work in
 * place, as their reference counterparts do.  Singular
 * values are returned in descending order, like LAPACK bdsdc.
 *
 * Status codes: 0 success; -i the i-th argument is invalid (LAPACK info
 * style); AVS_ERR_NOT_IMPLEMENTED for the reference's "Not implemented" cases
 * (non-square, tile not a power of two, tile < 16, tile not dividing n); > 0
 * runtime errors.  A Julia binding turns AVS_ERR_NOT_IMPLEMENTED into
 * error("Not implemented").
 *
 * Threading: a handle owns one CUDA stream, a second (highest-priority)
 * stream on which stage 1 of the tensor-core modes runs its next panel ahead
 * (joined back before the call returns; ordered after the caller's stream by
 * events, so capture and stream semantics are the caller's), and a grow-only
 * device workspace; calls on one handle are serialised by the caller (one
 * handle per host thread).  Entry points block until their results are ready.
 */
#ifndef AVS_H
#define AVS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define AVS_VERSION_MAJOR 0
#define AVS_VERSION_MINOR 2

/* ---- status codes -------------------------------------------------------- */
#define AVS_SUCCESS 0
#define AVS_ERR_NOT_IMPLEMENTED (-100) /* SVD_GPU.jl:261-262 / 275-276 */
#define AVS_ERR_CUDA 1                 /* a CUDA runtime call failed */
#define AVS_ERR_OOM 2                  /* device memory exhausted */
#define AVS_ERR_TIMEOUT 3              /* a bounded device-side wait gave up */
#define AVS_ERR_NONFINITE 4            /* NaN/Inf met in the factorisation */
#define AVS_ERR_NO_DEVICE 5            /* no usable CUDA device */
#define AVS_ERR_UNSUPPORTED 6          /* valid request the library does not support */
#define AVS_ERR_INTERNAL 7
#define AVS_ERR_TOO_LARGE 8            /* n above the static scratch of avs_bidiag_svals_noalloc */

/* ---- precision modes of the trailing WY updates (stage 1) ---------------- */
/* Householder generation/scaling, bulge chase and bisection run in FP64 (plain
 * mode) or double-float (FP32-class modes, see the flags below) scalars; these
 * modes select the storage type of the tiles and the arithmetic of the
 * compact-WY trailing updates. */
#define AVS_PREC_DEFAULT 0 /* FP64 for the _d entry points, FP32 for _s */
#define AVS_PREC_FP64 1    /* plain path: FP64 tiles, FP64 updates */
#define AVS_PREC_FP32 2    /* FP32 tiles, FP32 SIMT updates */
#define AVS_PREC_TF32 3    /* FP32 tiles, TF32 tensor-core updates, FP32 accumulate */
#define AVS_PREC_TF32X3 4  /* FP32 tiles, split TF32 (3 products) tensor-core updates */
#define AVS_PREC_BF16 5    /* FP32 tiles, BF16 tensor-core updates, FP32 accumulate */
#define AVS_PREC_BF16X3 6  /* FP32 tiles, split BF16 (3 products) tensor-core updates */
#define AVS_PREC_FP64X2 7  /* FP64 tiles and panels; the full compact-WY trailing updates of tiles >= 128
                              in double-float (two-term split FP32 products) on the FP32 pipe, stages 2
                              and 3 in double-float: FP64-level accuracy (1e-12) at the FP32 pipe's rate */

/* ---- avs_opts.flags ---------------------------------------------------------
 * Stages 2 and 3 (bulge chase, bisection) run in FP64 for AVS_PREC_FP64 and in
 * double-float arithmetic (pairs of FP32, ~44-48 significant bits; GB300 issues
 * FP64 at 1/64 of the FP32 rate) for the FP32-class modes.  These flags
 * override that choice. */
#define AVS_FLAG_FP64_STAGES 1
#define AVS_FLAG_DF64_STAGES 2
/* Stage 2 is hierarchical by default in the FP32-class modes, as the
 * reference's bidiag! (BRD/src/bulgechasing2.jl:22-45) and the halving of
 * bidiagonalize (KAbasedSVD/src/bulgechasing.jl:33-42): a blocked band
 * reduction (T rows per sweep, compact-WY applies, FP32 arithmetic) takes the
 * band of width tile (64, 128 or 256) to width 16, then the element chase
 * (double-float) takes it to the bidiagonal.  With FP64 stages the element
 * chase runs from the band of width tile (the FP64 block stage is slower on
 * GB300's FP64 pipe) unless AVS_FLAG_HIER_CHASE asks for the hierarchy (FP64
 * block stage).  Batched groups make the same choices as single calls. */
#define AVS_FLAG_ONE_STAGE_CHASE 4 /* element chase straight from the band of width tile */
#define AVS_FLAG_BAND32 8          /* intermediate band of width 32 instead of 16 */
#define AVS_FLAG_HIER_CHASE 32     /* hierarchical stage 2 with FP64 stages too */
/* The element chase of the narrow band runs G sweeps per CTA inside a
 * shared-memory window by default; this flag runs it with one thread-block
 * cluster per sweep on the band in global memory instead. */
#define AVS_FLAG_CLUSTER_CHASE 16

typedef struct avs_handle avs_handle;

typedef struct avs_opts {
    int32_t precision;      /* AVS_PREC_* (0 = default for the entry point's type) */
    int32_t flags;          /* AVS_FLAG_* (0 = defaults) */
    double bisect_rel_tol;  /* bisection width relative to ||B|| (0 = 2 * DBL_EPSILON in FP64,
                               4e-14 in double-float on FP64 tiles, 1e-10 in double-float
                               for the FP32-class modes) */
    void *stream;           /* cudaStream_t for the _dev entry points (NULL = handle stream) */
} avs_opts;

typedef struct avs_report {
    double t_total_ms;   /* device time of the whole call (events on the call's stream) */
    double t_stage1_ms;  /* GE2BND: tile QR/LQ band reduction */
    double t_stage2_ms;  /* band -> bidiagonal bulge chase (incl. band extraction) */
    double t_stage3_ms;  /* bidiagonal singular values (bisection) */
    double t_h2d_ms;     /* host entry points: input copy */
    double t_d2h_ms;     /* host entry points: output copy */
    int64_t kernel_launches;
    int64_t workspace_bytes;
    int32_t precision;   /* precision mode that ran */
    int32_t status;
    double t_update_ms;  /* tensor-core modes: the trailing updates inside stage 1 (copies of Y,
                            the two tcgen05 GEMMs and the chain), summed over the half-steps */
    double t_band_ms;    /* hierarchical stage 2: the blocked band reduction (band extraction
                            included); the element chase is t_stage2_ms - t_band_ms */
} avs_report;

/* ---- handle ---------------------------------------------------------------- */
/* Replaces the implicit CUDA.jl context/stream of the reference. */
int avs_create(avs_handle **h, int device);
int avs_destroy(avs_handle *h);
/* Pre-grow the workspace for (n, tile, precision) so that later calls allocate nothing. */
int avs_reserve(avs_handle *h, int64_t n, int32_t tile, int32_t precision);
/* Message of a status code; for AVS_ERR_CUDA it names the last CUDA runtime error the calling
 * thread met inside the library. */
const char *avs_strerror(int status);
int avs_version(void);

/* ---- entry point: my_CU_svdval ------------------------------------------------
 * m x n column-major A (ld lda >= m), tile = block_size; sigma receives n
 * values in descending order.  m != n, tile not a power of two, tile < 16 or
 * n % tile != 0 return AVS_ERR_NOT_IMPLEMENTED (SVD_GPU.jl:261-262).
 * opts and report may be NULL. */
/* Host matrices: my_CU_svdval(::Matrix{Float32}, b), SVD_GPU.jl:257-270. */
int avs_svdvals_s(avs_handle *h, int64_t m, int64_t n, int64_t lda, int32_t tile, const float *A, float *sigma,
                  const avs_opts *opts, avs_report *report);
/* Float64 host matrices (the reference has no Float64 method; same contract). */
int avs_svdvals_d(avs_handle *h, int64_t m, int64_t n, int64_t lda, int32_t tile, const double *A, double *sigma,
                  const avs_opts *opts, avs_report *report);
/* Device matrices: my_CU_svdval(::CuMatrix{Float32}, b), SVD_GPU.jl:272-283. */
int avs_svdvals_dev_s(avs_handle *h, int64_t m, int64_t n, int64_t lda, int32_t tile, const float *dA,
                      float *dsigma, const avs_opts *opts, avs_report *report);
int avs_svdvals_dev_d(avs_handle *h, int64_t m, int64_t n, int64_t lda, int32_t tile, const double *dA,
                      double *dsigma, const avs_opts *opts, avs_report *report);

/* ---- building blocks (device pointers) ----------------------------------------
 * Blockbidiag! (KAbasedSVD/src/tiledalgos.jl:17-34) on a TiledMatrix
 * (TiledMatrix.jl:41-67) in place: on return dA holds the upper band
 * 0 <= j - i <= tile.  Entries outside the band hold Householder vectors
 * (the reference zeroes them with triu!/tril!/.= 0, tiledalgos.jl:40,46,52,58);
 * avs_extract_band_* reads only the band. */
int avs_blockbidiag_dev_s(avs_handle *h, int64_t n, int64_t lda, int32_t tile, float *dA, const avs_opts *opts,
                          avs_report *report);
int avs_blockbidiag_dev_d(avs_handle *h, int64_t n, int64_t lda, int32_t tile, double *dA, const avs_opts *opts,
                          avs_report *report);
/* Blockbidiag! with its reflectors kept: the band reduction above, plus the tau
 * of every Householder reflector, so that Q and P of A = Q B P^T can be rebuilt
 * from the vectors left in dA (the orthogonality / backward-error check of the
 * band reduction).  The reference keeps tau in the TiledMatrix's nt x nt Tau
 * grid (KAbasedSVD/src/TiledMatrix.jl:53-58; slots Tau[k,k] and Tau[row,k] of
 * the QR half-step, Tau[k,k] and Tau[col,k] of the LQ half-step,
 * TiledMatrix.jl:92-113), where the LQ half-step overwrites the QR one; here
 * both are kept.  nt = n / tile; each array holds nt * nt * tile elements and
 * may be NULL:
 *   dtau_q[(k*nt + r)*tile + l]  QR half-step k, tile row r >= k, reflector l:
 *       r == k: GEQRT of tile (k,k), v = unit lower column l of tile (k,k);
 *       r >  k: TSQRT of [R_kk; A_rk], v = e_l on top, column l of tile (r,k) below;
 *   dtau_p[(k*nt + c)*tile + l]  LQ half-step k, tile column c >= k+1, reflector l
 *       (right reflectors, stored as rows): c == k+1: GELQT of tile (k,k+1), v =
 *       unit upper row l of that tile; c > k+1: TSLQT, v = e_l on the left
 *       (tile column k+1), row l of tile (k,c) on the right.
 * opts->precision selects the update arithmetic of the _s form (FP32 SIMT or a
 * tensor-core mode), as for avs_svdvals; the tiles keep the input's type. */
int avs_blockbidiag_tau_dev_s(avs_handle *h, int64_t n, int64_t lda, int32_t tile, float *dA, float *dtau_q,
                              float *dtau_p, const avs_opts *opts, avs_report *report);
int avs_blockbidiag_tau_dev_d(avs_handle *h, int64_t n, int64_t lda, int32_t tile, double *dA, double *dtau_q,
                              double *dtau_p, const avs_opts *opts, avs_report *report);
/* tiled_QR! (KAbasedSVD/src/tiledalgos.jl:6-15) on a TiledMatrix in place: the QR
 * half-steps of Blockbidiag! alone (GEQRT of the diagonal tile, TSQRT down the
 * panel, compact-WY updates of the trailing tiles).  On return R is in the upper
 * triangle, the Householder vectors below it (unit lower V in the diagonal
 * tiles, V in the tiles below, as the reference leaves them).  dtau (may be
 * NULL; nt * nt * tile elements, nt = n / tile) receives the tau of panel k,
 * tile row r >= k, reflector l at dtau[(k * nt + r) * tile + l].  opts->precision
 * selects the update arithmetic as for avs_svdvals (FP32: SIMT or tensor cores). */
int avs_geqrf_dev_s(avs_handle *h, int64_t n, int64_t lda, int32_t tile, float *dA, float *dtau,
                    const avs_opts *opts, avs_report *report);
int avs_geqrf_dev_d(avs_handle *h, int64_t n, int64_t lda, int32_t tile, double *dA, double *dtau,
                    const avs_opts *opts, avs_report *report);

/* ---- out of core (host matrices larger than the device budget) -----------------
 * OOC_Bidiag! / OOC_SVD! / OOC_QR! (KAbasedSVD/src/tiledalgos.jl:232-260) over a
 * LargeTiledMatrix (TiledMatrix.jl:121-186): A stays in host memory
 * (column-major, lda) and is overwritten in place, as in the reference.  Each
 * half-step streams the tile rows (QR) or tile columns (LQ) of its trailing
 * block through the device in slabs sized by device_bytes (0 = 90% of the
 * free device memory), the top tile carried from slab to slab; once the
 * trailing block fits, it is finished in device memory (the reference's
 * kswitch tail).  The band and the Householder vectors come out bit for bit
 * as those of avs_blockbidiag_dev / avs_geqrf_dev in the input's type (the
 * same kernels in the same order; FP32 or FP64, other precision modes return
 * AVS_ERR_UNSUPPORTED).  A is pinned with
 * cudaHostRegister for the call when possible.  avs_svdvals_ooc_* then copies
 * the band to the device and returns sigma (descending) in host memory, where
 * the reference's OOC_SVD! returns the bidiagonal (tiledalgos.jl:256-259).
 * tau of the QR form: host, nt * nt * tile elements, layout of avs_geqrf_dev
 * (may be NULL).  device_bytes below what one slab needs returns AVS_ERR_OOM. */
int avs_blockbidiag_ooc_s(avs_handle *h, int64_t n, int64_t lda, int32_t tile, float *A, int64_t device_bytes,
                          avs_report *report);
int avs_blockbidiag_ooc_d(avs_handle *h, int64_t n, int64_t lda, int32_t tile, double *A, int64_t device_bytes,
                          avs_report *report);
int avs_svdvals_ooc_s(avs_handle *h, int64_t n, int64_t lda, int32_t tile, float *A, float *sigma,
                      int64_t device_bytes, const avs_opts *opts, avs_report *report);
int avs_svdvals_ooc_d(avs_handle *h, int64_t n, int64_t lda, int32_t tile, double *A, double *sigma,
                      int64_t device_bytes, const avs_opts *opts, avs_report *report);
int avs_geqrf_ooc_s(avs_handle *h, int64_t n, int64_t lda, int32_t tile, float *A, float *tau, int64_t device_bytes,
                    avs_report *report);
/* The slab plan of the calls above (host only, no device needed): for order n,
 * tile, element size (4 or 8) and device_bytes > 0, *slab = tile rows per slab
 * (0: device_bytes too small), *bytes = device bytes the call holds,
 * *incore_from = the step k from which the trailing block is finished in
 * device memory in the band form (nt: never).  Pointers may be NULL. */
int avs_ooc_plan(int64_t n, int32_t tile, int32_t elem_bytes, int64_t device_bytes, int32_t *slab, int64_t *bytes,
                 int32_t *incore_from);
int avs_geqrf_ooc_d(avs_handle *h, int64_t n, int64_t lda, int32_t tile, double *A, double *tau,
                    int64_t device_bytes, avs_report *report);
/* Copy the upper band 0 <= j - i <= bw of a dense n x n matrix into a dense
 * FP64 n x n matrix with zeros elsewhere (the reference's banded array). */
int avs_extract_band_dev_s(avs_handle *h, int64_t n, int64_t lda, int32_t bw, const float *dA, double *dB,
                           int64_t ldb);
int avs_extract_band_dev_d(avs_handle *h, int64_t n, int64_t lda, int32_t bw, const double *dA, double *dB,
                           int64_t ldb);
/* bidiagonalize(A, bw) (KAbasedSVD/src/bulgechasing.jl:33-42): upper band of
 * width bw in a dense FP64 n x n matrix -> diagonal d (n) and superdiagonal e
 * (n-1) of an upper bidiagonal with the same singular values (FP64 bulge chase). */
int avs_band_to_bidiag_dev(avs_handle *h, int64_t n, int32_t bw, const double *dB, int64_t ldb, double *dd,
                           double *de, avs_report *report);
/* One stage of the hierarchical band reduction: bidiag! with factor bw / tbw
 * (BRD/src/bulgechasing2.jl:22-45; LQ_QMUL / QR_QMUL, :4-20).  The upper band
 * 0 <= j - i <= bw of the dense n x n matrix dB (leading dimension ldb;
 * entries outside it are ignored) is reduced to an upper band of width tbw
 * with the same singular values; dB receives every entry of the working band
 * storage (rows j-2bw+1 .. j+bw-1 of column j; zero outside width tbw on
 * return) and zeros elsewhere.  (bw, tbw) in {(256, 32), (256, 16), (128, 32),
 * (128, 16), (64, 16)}, other pairs AVS_ERR_UNSUPPORTED.  _s: FP32 arithmetic,
 * _d: FP64. */
int avs_band_reduce_dev_s(avs_handle *h, int64_t n, int32_t bw, int32_t tbw, float *dB, int64_t ldb,
                          avs_report *report);
int avs_band_reduce_dev_d(avs_handle *h, int64_t n, int32_t bw, int32_t tbw, double *dB, int64_t ldb,
                          avs_report *report);

/* diag_lapack / LAPACK.bdsdc!('U','N',d,e) (bulgechasing.jl:50-53): singular
 * values of the upper bidiagonal, descending, by FP64 bisection on the
 * Golub-Kahan tridiagonal.  rel_tol as avs_opts.bisect_rel_tol. */
int avs_bidiag_svals_dev(avs_handle *h, int64_t n, const double *dd, const double *de, double *dsigma,
                         double rel_tol, avs_report *report);

/* Allocation-free variant of avs_bidiag_svals_dev.  No counterpart in the
 * reference.  For callers that cannot call cudaMalloc when they need the
 * values -- a host whose device memory belongs to its own pool allocator
 * (Julia's CUDA.jl, PyTorch's caching allocator), or a latency-critical loop
 * that must not pay cudaMalloc's implicit synchronisation.  Needs no handle;
 * runs on the current device and on `stream` (a cudaStream_t, NULL = legacy
 * default stream), and synchronises that stream before it returns, so the
 * values are in dsigma on return.  Its scratch is a static device array in the
 * library (~512 KiB per GPU, held until exit), so n <= 65536; larger n returns
 * AVS_ERR_TOO_LARGE.  The first call on a device looks the array's address up.
 * Because every call synchronises its stream, no call can be recorded by a
 * stream capture (CUDA graph).  Calls share the array: calls that overlap on
 * the GPU race on it. */
int avs_bidiag_svals_noalloc(int64_t n, const double *dd, const double *de, double *dsigma, double rel_tol,
                             void *stream);

/* Batched singular values of `count` independent square FP32 matrices of mixed
 * orders, all on the device (the many-small-matrices workload of RMT/rmt.jl:9-36,
 * which calls LAPACK once per matrix).  Matrix i is n[i] x n[i], column-major
 * with leading dimension lda[i], at dA[i]; its n[i] values go to dsigma[i]
 * (descending, FP32).  tile[i] = 0 (or tile == NULL) lets the autotuner choose
 * the tile for that order; otherwise the same "Not implemented" rules as
 * avs_svdvals_dev_s apply per matrix.  Matrices of equal (n, tile) run as one
 * group: stage-1 launches cover the whole group, one cluster chase kernel runs
 * all the group's sweeps, one bisection kernel all its values.  Each group's
 * launch sequence is captured once in a CUDA graph (kept per (n, tile, group
 * size) on the handle) and replayed.  Results of a matrix do not depend on the
 * other matrices of the call.  Precision: FP32 tiles with double-float stages
 * 2 and 3 (the `precision` field of opts is ignored; bisect_rel_tol is used;
 * the Float64 form below takes AVS_PREC_FP64X2).
 * The pointer arrays are host arrays.  The work runs on the handle's stream,
 * after the work queued so far on opts->stream (when given); the call blocks
 * until all values are written.  report->t_total_ms covers all groups. */
int avs_svdvals_batched_dev_s(avs_handle *h, int32_t count, const int64_t *n, const int64_t *lda,
                              const int32_t *tile, const float *const *dA, float *const *dsigma,
                              const avs_opts *opts, avs_report *report);
/* The same batched pipeline stopped after the bulge chase: the bidiagonal B of
 * each matrix (A = U B V^T, V e1 = e1), d (n values) and e (n values, the last
 * one 0) to the caller's FP64 device vectors dd[i], de[i].  B is unique up to
 * the signs of its entries, so |d| and |e| equal those of LAPACK gebrd on the
 * same matrix to the FP32 rounding of the band reduction: the quantity the
 * random-matrix sampling client reads (RMT/rmt.jl:24-31, d of gebrd!). */
int avs_bidiag_batched_dev_s(avs_handle *h, int32_t count, const int64_t *n, const int64_t *lda,
                             const int32_t *tile, const float *const *dA, double *const *dd, double *const *de,
                             const avs_opts *opts, avs_report *report);
/* The same two batched calls for Float64 matrices, FP64 throughout (tiles,
 * updates, bulge chase, bisection; the random-matrix client of RMT/rmt.jl runs
 * gebrd! in Float64, rmt.jl:23,28).  Each matrix's values are bit-identical to
 * those of avs_svdvals_dev_d / the FP64 pipeline on the same matrix.
 * opts->precision == AVS_PREC_FP64X2 runs the groups' trailing updates, bulge
 * chase and bisection in double-float, as avs_svdvals_dev_d does in that mode
 * (values then equal its values bit for bit; AVS_FLAG_FP64_STAGES keeps FP64
 * stages 2-3). */
int avs_svdvals_batched_dev_d(avs_handle *h, int32_t count, const int64_t *n, const int64_t *lda,
                              const int32_t *tile, const double *const *dA, double *const *dsigma,
                              const avs_opts *opts, avs_report *report);
int avs_bidiag_batched_dev_d(avs_handle *h, int32_t count, const int64_t *n, const int64_t *lda,
                             const int32_t *tile, const double *const *dA, double *const *dd, double *const *de,
                             const avs_opts *opts, avs_report *report);

/* Autotuner of the batched path: times tiles 32, 64 and 128 (those that divide
 * n with at least two tiles) on `sample` seeded random matrices of order n,
 * stores the fastest on the handle (used for tile 0 in the batched call) and
 * returns it in *best (may be NULL).  sample <= 0 means 16. */
int avs_autotune_tile(avs_handle *h, int64_t n, int32_t sample, int32_t *best);

/* Failure-path check: a kernel waits, with a short bound (about 0.3 s), on a
 * flag that nothing sets -- the bounded wait that every cross-CTA dependency
 * of the library uses.  Returns AVS_ERR_TIMEOUT, and the handle and the CUDA
 * context stay usable. */
int avs_selftest_timeout(avs_handle *h);

/* Diagnostics (no counterpart in the reference): the architecture of the
 * device code the runtime loaded from this library on `device`
 * (cudaFuncAttributes binaryVersion, 103 for sm_103a, and ptxVersion). */
int avs_kernel_arch(int device, int32_t *binary_version, int32_t *ptx_version);
/* Diagnostics (no counterpart in the reference): the compute roof of the bulge
 * chase on `device` -- flops per second of its inner arithmetic (compensated
 * dot products and reflector updates, 4 flops per element step) in
 * double-float (fp64 == 0), FP64 (fp64 == 1) or FP32 (fp64 == 2: the
 * arithmetic of the blocked band reduction), from registers on every SM.  The call
 * allocates and frees a small output buffer and synchronises the device. */
int avs_measure_chase_rate(int device, int32_t fp64, double *flops_per_s);

/* Release the handle's cached device workspace, pinned tables and captured
 * graphs (the handle stays usable; the next call allocates again). */
int avs_trim(avs_handle *h);
/* Device bytes the handle currently holds: the workspace of the single-matrix
 * entry points and that of the batched entry point (either pointer may be NULL). */
int avs_workspace_bytes(avs_handle *h, int64_t *single_bytes, int64_t *batched_bytes);
/* Device workspace one call needs: count == 0 -> one avs_svdvals_{s,d} call of
 * order n with this tile and precision; count >= 1 -> one batched group of
 * `count` matrices of order n (FP64 group for AVS_PREC_FP64, FP32 otherwise;
 * the caller's inputs and outputs not included). */
int avs_estimate_bytes(int64_t n, int32_t tile, int32_t precision, int32_t count, int64_t *bytes);

/* ---- serving loop ---------------------------------------------------------------
 * An SVD request server with continuous batching (no counterpart in the
 * reference, whose entry point is one blocking call).  Requests (host matrices,
 * FP32 or FP64, any supported order) are queued by avs_serve_submit and run by
 * `workers` execution slots, each with its own handle and CUDA stream, so the
 * work of several requests overlaps on the GPU.  A free slot takes the oldest
 * queued request and every other queued request of the same order and type
 * (up to max_batch) into one batched call (avs_svdvals_batched_dev_s / _d);
 * avs_serve_plan says which precision mode and tile a request gets and
 * whether it is batched.  Admission is by device
 * memory: a slot starts a group only while the bytes held by all slots stay
 * within hbm_budget_bytes; otherwise it shrinks the group, releases its own
 * cached workspace, or waits until others finish.  Each result equals the
 * result of the same request served alone (the batched kernels are
 * batch-invariant).  Latency = completion - submission (host steady clock). */
typedef struct avs_server avs_server;

#define AVS_DTYPE_F32 0
#define AVS_DTYPE_F64 1

typedef struct avs_serve_config {
    int32_t device;
    int32_t workers;          /* execution slots (0 = 4) */
    int32_t max_batch;        /* requests per batched group (0 = 512) */
    int32_t autotune;         /* 1 = autotune FP32 tiles per order, 0 = fixed rule */
    int64_t hbm_budget_bytes; /* 0 = 80% of the device memory free at creation */
} avs_serve_config;

typedef struct avs_serve_stats {
    int64_t submitted, completed, failed, queued, batches;
    double p50_ms, p99_ms, mean_ms, max_ms; /* latency of completed requests */
    double throughput_rps;                  /* completed / (last completion - first submission) */
    double mean_batch;                      /* requests per group */
    int64_t peak_bytes;                     /* peak device bytes held by the slots */
    int64_t budget_bytes;
} avs_serve_stats;

int avs_serve_create(avs_server **srv, const avs_serve_config *cfg);
/* How the server runs a request of order n and type dtype (host only, no
 * device needed): *tile_out (tile 0 = the server's rule), *precision (an
 * AVS_PREC_* mode: FP32 SIMT updates for FP32 requests below order 2048,
 * split-BF16 tensor-core updates above, AVS_PREC_FP64X2 for FP64 requests) and
 * *batched (1: requests of the same order and type share batched calls; 0: the
 * request runs alone).  A served result equals the single-matrix entry point's
 * with this tile and precision, bit for bit.  Pointers may be NULL. */
int avs_serve_plan(int64_t n, int32_t dtype, int32_t tile, int32_t *tile_out, int32_t *precision, int32_t *batched);
/* Queue one request: n x n column-major A (ld lda) of type dtype in host memory,
 * n values to sigma (same type).  Both buffers must stay valid until the request
 * completes.  tile = 0 picks the tile.  Returns its id in *id. */
int avs_serve_submit(avs_server *srv, int64_t n, int64_t lda, int32_t dtype, int32_t tile, const void *A, void *sigma,
                     int64_t *id);
/* Block until request id completes; its status and latency (ms) are returned.
 * timeout_ms < 0 waits forever; a timeout returns AVS_ERR_TIMEOUT. */
int avs_serve_wait(avs_server *srv, int64_t id, double timeout_ms, int32_t *status, double *latency_ms);
int avs_serve_stats_get(avs_server *srv, avs_serve_stats *out);
/* Drain the queue, stop the slots and free everything. */
int avs_serve_destroy(avs_server *srv);

/* Tile kernels, one tile (b x b, column-major, ld b), device pointers.
 * QR_unsafe_kernel! (QRkernels.jl:3-66): R above, unit-lower V below, tau[0..b-2]. */
int avs_geqrt_tile_dev_s(avs_handle *h, int32_t b, float *dA, float *dtau);
int avs_geqrt_tile_dev_d(avs_handle *h, int32_t b, double *dA, double *dtau);
/* QR_unsafe_kernel2! (QRkernels.jl:71-129): R (upper triangle of dR) and the
 * full bottom tile dB, which receives V; tau[0..b-1]. */
int avs_tsqrt_tile_dev_s(avs_handle *h, int32_t b, float *dR, float *dB, float *dtau);
int avs_tsqrt_tile_dev_d(avs_handle *h, int32_t b, double *dR, double *dB, double *dtau);

#ifdef __cplusplus
}
#endif
#endif /* AVS_H */
