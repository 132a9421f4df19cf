// Stage 3: singular values of an upper bidiagonal B (d, e) by per-value FP64
// bisection on the Golub-Kahan tridiagonal TGK(B) (zero diagonal,
// off-diagonal d0, e0, d1, e1, ..., d_{n-1}; eigenvalues +-sigma_i).
//
// Replaces LAPACK.bdsdc!('U','N', d, e) (KAbasedSVD/src/bulgechasing.jl:50-53,
// CUDAbasedSVD/SVD_GPU.jl:267,281), which the reference runs on the CPU.
// Method: Sturm counts from the LDL^T pivots of TGK - x I with the pivot guard
// of LAPACK dstebz (Kahan's bisection); one thread per singular value, every
// loop bounded.  Output is descending, like bdsdc.
#include <algorithm>
#include <cfloat>
#include <cmath>

#include "avs_common.cuh"
#include "df64.cuh"

namespace avs {
namespace {

// scratch[0] = Gershgorin bound of TGK, scratch[1] = pivmin (one block).
__device__ void tgk_bound_body(const double *d, const double *e, int64_t n, double *scratch) {
    __shared__ double sb[32], sm[32];
    double bound = 0.0, maxsq = 0.0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
        const double di = fabs(d[i]);
        const double el = i > 0 ? fabs(e[i - 1]) : 0.0;
        const double er = i + 1 < n ? fabs(e[i]) : 0.0;
        bound = fmax(bound, di + el + er);
        maxsq = fmax(maxsq, fmax(di * di, er * er));
    }
    for (int o = 16; o > 0; o >>= 1) {
        bound = fmax(bound, __shfl_xor_sync(0xffffffffu, bound, o));
        maxsq = fmax(maxsq, __shfl_xor_sync(0xffffffffu, maxsq, o));
    }
    if ((threadIdx.x & 31) == 0) {
        sb[threadIdx.x >> 5] = bound;
        sm[threadIdx.x >> 5] = maxsq;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double b2 = 0.0, m2 = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
            b2 = fmax(b2, sb[w]);
            m2 = fmax(m2, sm[w]);
        }
        scratch[0] = b2;
        scratch[1] = DBL_MIN * fmax(m2, 1.0);
    }
}

__global__ void tgk_bound_kernel(const double *d, const double *e, int64_t n, double *scratch) {
    tgk_bound_body(d, e, n, scratch);
}

// Pivot recurrence q_i = -x - a_i / q_{i-1} (a_i = squared off-diagonal of
// TGK), counting negative pivots.  The division is replaced by a reciprocal:
// a single-precision estimate (hardware rcp) refined by one Newton-Raphson
// step r' = r (2 - q r), which leaves a relative error near 2^-46; pivots
// outside the single-precision range fall back to an FP64 division.  The
// count is then exact for off-diagonals perturbed by ~1e-14 relatively.
__device__ __forceinline__ double recip_nr(double q) {
    const double aq = fabs(q);
    if (aq > 1e-36 && aq < 1e36) {
        const double r = (double)__frcp_rn((float)q);
        const double e = fma(-q, r, 1.0);
        return fma(r, e, r);
    }
    return 1.0 / q;
}

__device__ __forceinline__ int tgk_count(const double *__restrict__ d, const double *__restrict__ e, int64_t n,
                                         double x, double pivmin) {
    int cnt = 0;
    double q = -x;
    if (fabs(q) < pivmin) q = -pivmin;
    cnt += (q < 0.0);
    for (int64_t i = 0; i < n; ++i) {
        const double di = __ldg(d + i);
        q = fma(-(di * di), recip_nr(q), -x);
        if (fabs(q) < pivmin) q = -pivmin;
        cnt += (q < 0.0);
        if (i + 1 < n) {
            const double ei = __ldg(e + i);
            q = fma(-(ei * ei), recip_nr(q), -x);
            if (fabs(q) < pivmin) q = -pivmin;
            cnt += (q < 0.0);
        }
    }
    return cnt;
}

// The same count in FP32 (used only to narrow the bracket; every bracket it
// produces is re-checked with FP64 counts before it is trusted).
__device__ __forceinline__ int tgk_count_f32(const double *__restrict__ d, const double *__restrict__ e, int64_t n,
                                             float x, float pivmin) {
    int cnt = 0;
    float q = -x;
    if (fabsf(q) < pivmin) q = -pivmin;
    cnt += (q < 0.0f);
    for (int64_t i = 0; i < n; ++i) {
        const float di = (float)__ldg(d + i);
        q = -x - __fdividef(di * di, q);
        if (fabsf(q) < pivmin || !isfinite(q)) q = -pivmin;
        cnt += (q < 0.0f);
        if (i + 1 < n) {
            const float ei = (float)__ldg(e + i);
            q = -x - __fdividef(ei * ei, q);
            if (fabsf(q) < pivmin || !isfinite(q)) q = -pivmin;
            cnt += (q < 0.0f);
        }
    }
    return cnt;
}

// The k-th largest singular value of the upper bidiagonal (d, e) of order n,
// from the bound and pivot guard in scratch[0..1].
__device__ double bisect_value(const double *d, const double *e, int64_t n, int64_t k, double rel_tol,
                               const double *scratch) {
    const double bound = scratch[0];
    const double pivmin = scratch[1];
    if (bound == 0.0) return 0.0;
    const double tol = rel_tol * bound;
    const int64_t target = 2 * n - 1 - k;  // TGK index (ascending) of the k-th largest sigma
    double lo = 0.0, hi = bound * (1.0 + 4.0 * DBL_EPSILON) + pivmin;
    // phase 1: FP32 counts shrink the bracket to ~2^-18 of its width
    if (bound < 1e30 && bound > 1e-30) {
        float flo = 0.0f, fhi = (float)hi;
        const float fpiv = fmaxf((float)pivmin, 1e-37f);
        for (int it = 0; it < 18; ++it) {
            const float mid = 0.5f * (flo + fhi);
            if (mid <= flo || mid >= fhi) break;
            if (tgk_count_f32(d, e, n, mid, fpiv) > target)
                fhi = mid;
            else
                flo = mid;
        }
        // widen by a few FP32 ulps of the bracket and verify it in FP64
        const double w = fmax((double)(fhi - flo), 1e-7 * bound);
        const double tlo = fmax(0.0, (double)flo - w), thi = fmin(hi, (double)fhi + w);
        if (tgk_count(d, e, n, tlo, pivmin) <= target) lo = tlo;
        if (tgk_count(d, e, n, thi, pivmin) > target) hi = thi;
    }
    // phase 2: FP64 bisection to the requested width
    for (int it = 0; it < 128 && hi - lo > tol; ++it) {
        const double mid = 0.5 * (lo + hi);
        if (mid <= lo || mid >= hi) break;
        if (tgk_count(d, e, n, mid, pivmin) > target)
            hi = mid;
        else
            lo = mid;
    }
    return 0.5 * (lo + hi);
}

__global__ void bisect_kernel(const double *d, const double *e, int64_t n, double rel_tol, const double *scratch,
                              double *sigma) {
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= n) return;
    sigma[k] = bisect_value(d, e, n, k, rel_tol, scratch);
}

// ---- double-float bisection (the pipeline's stage 3 for FP32-class modes) ----
// B is scaled by 1/bound so every quantity stays inside FP32's exponent range;
// the squared TGK off-diagonals a_i = (off_i / bound)^2 are formed once in FP64
// and stored as df64 pairs.  A count costs ~60 FP32 instructions per pivot
// instead of an FP64 division; relative errors of ~1e-14 per pivot keep the
// count exact for a matrix within ~1e-14 of TGK(B) (the backward-stability
// argument of the FP64 recurrence).
__global__ void tgk_prep_df_kernel(const double *d, const double *e, int64_t n, const double *scratch, float2 *a) {
    const double inv = scratch[0] > 0.0 ? 1.0 / scratch[0] : 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < 2 * n - 1;
         i += (int64_t)gridDim.x * blockDim.x) {
        const double off = ((i & 1) ? e[i >> 1] : d[i >> 1]) * inv;
        const double sq = off * off;
        const float h = (float)sq;
        a[i] = make_float2(h, (float)(sq - (double)h));
    }
}

// 1 / q in double-float: hardware reciprocal estimate of q.hi (relative error
// ~2^-23) refined by one Newton-Raphson step r' = r + r (1 - q r) in df64.
__device__ __forceinline__ df64 df_rcp_fast(df64 q) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(q.hi));
    const df64 e = df_sub(df64{1.0f, 0.0f}, df_mul_f(q, r));
    return df_add(df64{r, 0.0f}, df_mul_f(e, r));
}

// Sturm counts of TGK at K shifts at once (one pass over a, K independent
// recurrences interleaved for instruction-level parallelism).
template <int K>
__device__ __forceinline__ void tgk_count_df_k(const float2 *__restrict__ a, int64_t m, const df64 (&x)[K],
                                               float pivmin, int (&cnt)[K]) {
    df64 nx[K], q[K];
#pragma unroll
    for (int j = 0; j < K; ++j) {
        nx[j] = df_neg(x[j]);
        q[j] = nx[j];
        if (fabsf(q[j].hi) < pivmin) q[j] = df64{-pivmin, 0.0f};
        cnt[j] = df_lt0(q[j]);
    }
    for (int64_t i = 0; i < m; ++i) {
        const float2 ai = __ldg(a + i);
        const df64 av{ai.x, ai.y};
#pragma unroll
        for (int j = 0; j < K; ++j) {
            q[j] = df_sub(nx[j], df_mul(av, df_rcp_fast(q[j])));
            if (fabsf(q[j].hi) < pivmin) q[j] = df64{-pivmin, 0.0f};
            cnt[j] += df_lt0(q[j]);
        }
    }
}

template <int K>
__device__ __forceinline__ void tgk_count_f_k(const float2 *__restrict__ a, int64_t m, const float (&x)[K],
                                              float pivmin, int (&cnt)[K]) {
    float q[K];
#pragma unroll
    for (int j = 0; j < K; ++j) {
        q[j] = -x[j];
        if (fabsf(q[j]) < pivmin) q[j] = -pivmin;
        cnt[j] = (q[j] < 0.0f);
    }
    for (int64_t i = 0; i < m; ++i) {
        const float ai = __ldg(a + i).x;
#pragma unroll
        for (int j = 0; j < K; ++j) {
            q[j] = -x[j] - __fdividef(ai, q[j]);
            if (fabsf(q[j]) < pivmin || !isfinite(q[j])) q[j] = -pivmin;
            cnt[j] += (q[j] < 0.0f);
        }
    }
}

// k-th largest singular value of the scaled problem (a = squared scaled
// off-diagonals, bound = the scale), returned unscaled.  Multisection by a
// group of G consecutive lanes: each lane counts at K = 3 shifts (one pass
// over a, three interleaved recurrences), so a pass splits the bracket into
// G*K + 1 parts; the group agrees on the first shift whose count exceeds the
// target with G-lane shuffles.  FP32 passes first (to ~1e-6 of the scale),
// then a double-float verified bracket and double-float passes to rel_tol.
template <int G>
__device__ double bisect_df_grp(const float2 *a, int64_t n, int64_t k, double rel_tol, double bound, int gl,
                                unsigned gmask) {
    if (bound == 0.0) return 0.0;
    constexpr int K = 3, NSH = G * K, NI = NSH + 1;
    const int64_t m = 2 * n - 1;
    const float pivmin = 1e-36f;
    const int64_t target = 2 * n - 1 - k;
    auto group_first = [&](const int (&c)[K]) {
        int first = NSH;
#pragma unroll
        for (int j = K - 1; j >= 0; --j)
            if (c[j] > target) first = gl * K + j;
#pragma unroll
        for (int o = G / 2; o >= 1; o >>= 1) first = min(first, __shfl_xor_sync(gmask, first, o));
        return first;
    };
    // FP32 phase on the scaled problem (all values in [0, 1]); count(x) > target <=> x > sigma_k
    float flo = 0.0f, fhi = 1.0f + 1e-6f;
    for (int it = 0; it < 24 && fhi - flo > 1e-6f; ++it) {
        const float w = (fhi - flo) * (1.0f / NI);
        if (!(flo + w > flo) || !(fhi - w < fhi)) break;
        float x[K];
#pragma unroll
        for (int j = 0; j < K; ++j) x[j] = flo + w * (float)(gl * K + j + 1);
        int c[K];
        tgk_count_f_k<K>(a, m, x, pivmin, c);
        const int first = group_first(c);
        const float nlo = flo + w * (float)first;
        const float nhi = first == NSH ? fhi : flo + w * (float)(first + 1);
        flo = nlo;
        fhi = nhi;
    }
    // verified bracket in double-float
    df64 lo = df64{0.0f, 0.0f}, hi = df64{1.0f + 1e-6f, 0.0f};
    {
        const float w = fmaxf(fhi - flo, 4e-7f);
        df64 t[2] = {df64{fmaxf(0.0f, flo - w), 0.0f}, df64{fminf(1.0f + 1e-6f, fhi + w), 0.0f}};
        int c[2];
        tgk_count_df_k<2>(a, m, t, pivmin, c);
        if (c[0] <= target) lo = t[0];
        if (c[1] > target) hi = t[1];
    }
    const float tol = (float)fmax(rel_tol, 1e-15);
    for (int it = 0; it < 60; ++it) {
        const df64 width = df_sub(hi, lo);
        if (width.hi <= tol) break;
        const df64 q = df64{width.hi * (1.0f / NI), width.lo * (1.0f / NI)};
        df64 x[K];
#pragma unroll
        for (int j = 0; j < K; ++j) x[j] = df_add(lo, df_mul_f(q, (float)(gl * K + j + 1)));
        int c[K];
        tgk_count_df_k<K>(a, m, x, pivmin, c);
        const int first = group_first(c);
        const df64 nlo = first == 0 ? lo : df_add(lo, df_mul_f(q, (float)first));
        const df64 nhi = first == NSH ? hi : df_add(lo, df_mul_f(q, (float)(first + 1)));
        lo = nlo;
        hi = nhi;
    }
    const df64 c = df_add(lo, hi);
    return bound * 0.5 * df_to_double(c);
}

// Lanes per value, a function of the order alone: the single-matrix and the
// batched calls of one order run the same multisection, so a matrix's values
// are identical alone and in a batch (the final bracket depends on G).  A group
// of G lanes does more counts per value (about 1.3, 2.3 and 3.2 times those of
// one lane for G = 2, 4, 8) in fewer dependent passes; G = 2 measured fastest
// at n = 16384 on GB300 (121 ms with G = 1, 98 ms with G = 2, 146 ms with
// G = 4) and keeps the batched workloads, where values are plentiful, close
// to the one-lane work.
inline int bisect_group(int64_t n) { return n >= 65536 ? 1 : 2; }

template <int G>
__global__ void bisect_df_kernel(const float2 *a, int64_t n, double rel_tol, const double *scratch, double *sigma) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t k = t / G;
    const int gl = (int)(t % G);
    if (k >= n) return;  // whole groups: G divides the block size
    const unsigned gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << ((threadIdx.x & 31) & ~(G - 1)));
    const double v = bisect_df_grp<G>(a, n, k, rel_tol, scratch[0], gl, gmask);
    if (gl == 0) sigma[k] = v;
}

template <typename T>
__global__ void cast_kernel(const double *src, T *dst, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        dst[i] = (T)src[i];
}

template <typename TI, typename TO>
__global__ void copy2d_kernel(const TI *src, int64_t lds, TO *dst, int64_t ldd, int64_t rows, int64_t cols) {
    for (int64_t c = blockIdx.y; c < cols; c += gridDim.y)
        for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < rows; r += (int64_t)gridDim.x * blockDim.x)
            dst[r + c * ldd] = (TO)src[r + c * lds];
}

// Threads per CTA: small enough that the values spread over every SM.
inline int bisect_threads(int64_t n) {
    int t = 128;
    while (t > 32 && (n + t - 1) / t < 2 * 152) t >>= 1;
    return t;
}

}  // namespace

int stage3_bisect(const double *dd, const double *de, int64_t n, double rel_tol, double *dsigma, double *dscratch,
                  cudaStream_t s, int64_t *launches) {
    if (n <= 0) return AVS_SUCCESS;
    if (!(rel_tol > 0.0)) rel_tol = 2.0 * DBL_EPSILON;
    tgk_bound_kernel<<<1, 1024, 0, s>>>(dd, de, n, dscratch);
    AVS_CUDA_TRY(cudaGetLastError());
    const int threads = bisect_threads(n);
    bisect_kernel<<<(unsigned)((n + threads - 1) / threads), threads, 0, s>>>(dd, de, n, rel_tol, dscratch, dsigma);
    AVS_CUDA_TRY(cudaGetLastError());
    if (launches) *launches += 2;
    return AVS_SUCCESS;
}

// ---------------------------------------------------------------------------
// Allocation-free variant of the bisection (avs_bidiag_svals_noalloc).
//
// Some callers cannot call cudaMalloc at the moment they need singular values:
// a host that has handed all device memory to its own pool allocator (Julia's
// CUDA.jl, PyTorch's caching allocator) and forbids allocations behind the
// pool's back, or a latency-critical loop that must not pay cudaMalloc's
// implicit device synchronisation.  For them the scratch of the bisection --
// the Gershgorin bound and pivot guard of TGK(B), and a zero-padded copy of the
// superdiagonal -- lives in the file-scope device array below instead of a
// workspace.  Every GPU that loads the library holds it (about 512 KiB) until
// the process exits.  Every call shares it and it keeps the last call's
// contents; calls that overlap on the GPU race on it.
constexpr int64_t kNoAllocMaxN = 65536;
constexpr int64_t kNoAllocHead = 8;  // [0] bound, [1] pivmin, rest unused
static __device__ __align__(256) double g_noalloc_scratch[kNoAllocHead + kNoAllocMaxN + 1];

}  // namespace avs

#include <mutex>

namespace avs {
namespace {
constexpr int kMaxDevices = 64;
double *g_noalloc_ptr[kMaxDevices] = {};
std::mutex g_noalloc_mu;
}  // namespace

// Device address of the static scratch for the current device.  Host code may
// not use g_noalloc_scratch as a device pointer (it names a host-side shadow),
// so the address is looked up once per device with that device current.
static int noalloc_scratch(double **out) {
    int dev = 0;
    AVS_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return AVS_ERR_UNSUPPORTED;
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void *p = nullptr;
        AVS_CUDA_TRY(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        g_noalloc_ptr[dev] = static_cast<double *>(p);
    }
    *out = g_noalloc_ptr[dev];
    return AVS_SUCCESS;
}

int bidiag_svals_noalloc(int64_t n, const double *dd, const double *de, double *dsigma, double rel_tol,
                         cudaStream_t s) {
    if (n < 0) return -1;
    if (n > kNoAllocMaxN) return AVS_ERR_TOO_LARGE;
    if (n > 0 && !dd) return -2;
    if (n > 1 && !de) return -3;
    if (n > 0 && !dsigma) return -4;
    if (n == 0) return AVS_SUCCESS;
    double *scr = nullptr;
    int rc = noalloc_scratch(&scr);
    if (rc != AVS_SUCCESS) return rc;
    double *te = scr + kNoAllocHead;
    // the previous call's contents are still there: rewrite the whole padded copy
    if (n > 1) AVS_CUDA_TRY(cudaMemcpyAsync(te, de, sizeof(double) * (size_t)(n - 1), cudaMemcpyDeviceToDevice, s));
    AVS_CUDA_TRY(cudaMemsetAsync(te + (n - 1), 0, sizeof(double) * 2, s));
    if (!(rel_tol > 0.0)) rel_tol = 2.0 * DBL_EPSILON;
    tgk_bound_kernel<<<1, 1024, 0, s>>>(dd, te, n, scr);
    AVS_CUDA_TRY(cudaGetLastError());
    const int threads = bisect_threads(n);
    bisect_kernel<<<(unsigned)((n + threads - 1) / threads), threads, 0, s>>>(dd, te, n, rel_tol, scr, dsigma);
    AVS_CUDA_TRY(cudaGetLastError());
    AVS_CUDA_TRY(cudaStreamSynchronize(s));
    return AVS_SUCCESS;
}

int stage3_bisect_df(const double *dd, const double *de, int64_t n, double rel_tol, double *dsigma, double *dscratch,
                     float2 *dpairs, cudaStream_t s, int64_t *launches) {
    if (n <= 0) return AVS_SUCCESS;
    if (!(rel_tol > 0.0)) rel_tol = 1e-14;
    tgk_bound_kernel<<<1, 1024, 0, s>>>(dd, de, n, dscratch);
    AVS_CUDA_TRY(cudaGetLastError());
    const int pb = (int)std::min<int64_t>((2 * n + 255) / 256, 1024);
    tgk_prep_df_kernel<<<pb, 256, 0, s>>>(dd, de, n, dscratch, dpairs);
    AVS_CUDA_TRY(cudaGetLastError());
    const int G = bisect_group(n);
    const int64_t nt = n * G;
    const unsigned blocks = (unsigned)((nt + 127) / 128);
    if (G == 1)
        bisect_df_kernel<1><<<blocks, 128, 0, s>>>(dpairs, n, rel_tol, dscratch, dsigma);
    else if (G == 2)
        bisect_df_kernel<2><<<blocks, 128, 0, s>>>(dpairs, n, rel_tol, dscratch, dsigma);
    else if (G == 4)
        bisect_df_kernel<4><<<blocks, 128, 0, s>>>(dpairs, n, rel_tol, dscratch, dsigma);
    else
        bisect_df_kernel<8><<<blocks, 128, 0, s>>>(dpairs, n, rel_tol, dscratch, dsigma);
    AVS_CUDA_TRY(cudaGetLastError());
    if (launches) *launches += 3;
    return AVS_SUCCESS;
}

template <typename T>
int cast_from_double(const double *src, T *dst, int64_t n, cudaStream_t s) {
    const int nb = (int)std::min<int64_t>((n + 255) / 256, 1024);
    cast_kernel<T><<<nb > 0 ? nb : 1, 256, 0, s>>>(src, dst, n);
    AVS_CUDA_TRY(cudaGetLastError());
    return AVS_SUCCESS;
}
template int cast_from_double<float>(const double *, float *, int64_t, cudaStream_t);
template int cast_from_double<double>(const double *, double *, int64_t, cudaStream_t);

template <typename TI, typename TO>
int copy_convert_2d(const TI *src, int64_t lds, TO *dst, int64_t ldd, int64_t rows, int64_t cols, cudaStream_t s) {
    dim3 grid((unsigned)std::min<int64_t>((rows + 255) / 256, 64), (unsigned)std::min<int64_t>(cols, 65535));
    copy2d_kernel<TI, TO><<<grid, 256, 0, s>>>(src, lds, dst, ldd, rows, cols);
    AVS_CUDA_TRY(cudaGetLastError());
    return AVS_SUCCESS;
}
template int copy_convert_2d<float, float>(const float *, int64_t, float *, int64_t, int64_t, int64_t, cudaStream_t);
template int copy_convert_2d<double, double>(const double *, int64_t, double *, int64_t, int64_t, int64_t,
                                             cudaStream_t);
template int copy_convert_2d<float, double>(const float *, int64_t, double *, int64_t, int64_t, int64_t,
                                            cudaStream_t);
template int copy_convert_2d<double, float>(const double *, int64_t, float *, int64_t, int64_t, int64_t,
                                            cudaStream_t);

// ---------------------------------------------------------------------------
// Batched double-float bisection: `batch` bidiagonals of order n stacked at
// stride n (d, e), singular values to dsigma (stride n).
namespace {
__global__ void tgk_bound_batched(const double *d, const double *e, int64_t n, double *scratch) {
    const int64_t zb = blockIdx.x;
    tgk_bound_body(d + zb * n, e + zb * n, n, scratch + zb * 4);
}
__global__ void tgk_prep_df_batched(const double *d, const double *e, int64_t n, int batch, const double *scratch,
                                    float2 *a) {
    const int64_t m = 2 * n - 1;
    const int64_t total = m * (int64_t)batch;
    for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < total; g += (int64_t)gridDim.x * blockDim.x) {
        const int64_t zb = g / m, i = g % m;
        const double bnd = scratch[zb * 4];
        const double inv = bnd > 0.0 ? 1.0 / bnd : 0.0;
        const double off = ((i & 1) ? e[zb * n + (i >> 1)] : d[zb * n + (i >> 1)]) * inv;
        const double sq = off * off;
        const float h = (float)sq;
        a[zb * (2 * n) + i] = make_float2(h, (float)(sq - (double)h));
    }
}
template <int G>
__global__ void bisect_df_batched(const float2 *a, int64_t n, int batch, double rel_tol, const double *scratch,
                                  double *sigma) {
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t g = t / G;
    const int gl = (int)(t % G);
    if (g >= n * (int64_t)batch) return;
    const int64_t zb = g / n, k = g % n;
    const unsigned gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << ((threadIdx.x & 31) & ~(G - 1)));
    const double v = bisect_df_grp<G>(a + zb * (2 * n), n, k, rel_tol, scratch[zb * 4], gl, gmask);
    if (gl == 0) sigma[g] = v;
}
}  // namespace

// Batched FP64 bisection: the single-matrix kernel's per-value code, one
// thread per value of every matrix (values identical to stage3_bisect's).
namespace {
__global__ void bisect_batched(const double *d, const double *e, int64_t n, int batch, double rel_tol,
                               const double *scratch, double *sigma) {
    const int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (g >= n * (int64_t)batch) return;
    const int64_t zb = g / n, k = g % n;
    sigma[g] = bisect_value(d + zb * n, e + zb * n, n, k, rel_tol, scratch + zb * 4);
}
}  // namespace

int stage3_bisect_batched(const double *dd, const double *de, int64_t n, int batch, double rel_tol, double *dsigma,
                          double *dscratch, cudaStream_t s, int64_t *launches) {
    if (n <= 0 || batch <= 0) return AVS_SUCCESS;
    if (!(rel_tol > 0.0)) rel_tol = 2.0 * DBL_EPSILON;
    tgk_bound_batched<<<batch, 256, 0, s>>>(dd, de, n, dscratch);
    AVS_CUDA_TRY(cudaGetLastError());
    const int64_t nv = n * (int64_t)batch;
    const int threads = bisect_threads(nv);
    bisect_batched<<<(unsigned)((nv + threads - 1) / threads), threads, 0, s>>>(dd, de, n, batch, rel_tol, dscratch,
                                                                               dsigma);
    AVS_CUDA_TRY(cudaGetLastError());
    if (launches) *launches += 2;
    return AVS_SUCCESS;
}

int stage3_bisect_df_batched(const double *dd, const double *de, int64_t n, int batch, double rel_tol,
                             double *dsigma, double *dscratch, float2 *dpairs, cudaStream_t s, int64_t *launches) {
    if (n <= 0 || batch <= 0) return AVS_SUCCESS;
    if (!(rel_tol > 0.0)) rel_tol = 4e-14;
    tgk_bound_batched<<<batch, 256, 0, s>>>(dd, de, n, dscratch);
    AVS_CUDA_TRY(cudaGetLastError());
    const int64_t total = (2 * n - 1) * (int64_t)batch;
    tgk_prep_df_batched<<<(unsigned)std::min<int64_t>((total + 255) / 256, 8192), 256, 0, s>>>(dd, de, n, batch,
                                                                                              dscratch, dpairs);
    AVS_CUDA_TRY(cudaGetLastError());
    const int64_t nv = n * (int64_t)batch;
    const int G = bisect_group(n);
    const unsigned blocks = (unsigned)((nv * G + 127) / 128);
    if (G == 1)
        bisect_df_batched<1><<<blocks, 128, 0, s>>>(dpairs, n, batch, rel_tol, dscratch, dsigma);
    else if (G == 2)
        bisect_df_batched<2><<<blocks, 128, 0, s>>>(dpairs, n, batch, rel_tol, dscratch, dsigma);
    else if (G == 4)
        bisect_df_batched<4><<<blocks, 128, 0, s>>>(dpairs, n, batch, rel_tol, dscratch, dsigma);
    else
        bisect_df_batched<8><<<blocks, 128, 0, s>>>(dpairs, n, batch, rel_tol, dscratch, dsigma);
    AVS_CUDA_TRY(cudaGetLastError());
    if (launches) *launches += 3;
    return AVS_SUCCESS;
}

}  // namespace avs
