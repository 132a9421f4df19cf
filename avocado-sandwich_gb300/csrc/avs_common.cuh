// Internal helpers shared by the stage kernels and the C ABI.
#pragma once

#include <cuda_runtime.h>
#include <atomic>
#include <stdint.h>

#include "avs.h"

namespace avs {

// Error flag values written by kernels into the workspace's status word.
enum DeviceError : int {
    kDevOk = 0,
    kDevTimeout = 1,   // a bounded spin on a progress flag ran out
    kDevNonfinite = 2, // NaN/Inf met while generating a reflector
    kDevInternal = 3,  // a kernel found its own bookkeeping inconsistent
};

// Bounds of any dependency wait: at most kSpinLimit polls (an acquire load and
// a 32 ns sleep each, about 1 us with the load's latency) and at most
// kWaitNs of %globaltimer, whichever comes first -- far beyond any legitimate
// wait, short enough that a lost dependency returns AVS_ERR_TIMEOUT instead of
// hanging the GPU.
constexpr long long kSpinLimit = 1ll << 27;
constexpr long long kWaitNs = 4000000000ll;  // 4 s

// Column-major view of a matrix, optionally transposed: element (i, j) of the
// view is a[i + j*lda] (LAYOUT 0) or a[j + i*lda] (LAYOUT 1).  The LQ half of
// each GE2BND step is the QR half on the transposed view, as the reference
// does with adjoint views (KAbasedSVD/src/TiledMatrix.jl:85-88).
template <typename T, int LAYOUT>
struct View {
    T *a;
    int64_t lda;
    __device__ __forceinline__ T &operator()(int64_t i, int64_t j) const {
        return LAYOUT == 0 ? a[i + j * lda] : a[j + i * lda];
    }
};

// Acquire-load of a progress counter written by another CTA.
__device__ __forceinline__ int ld_acquire(const int *p) {
    int v;
    asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Release-store of a progress counter (after the CTA's writes are complete).
__device__ __forceinline__ void st_release(int *p, int v) {
    asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Bounded wait until *flag >= target.  Called by one thread; returns false on
// timeout (after recording kDevTimeout in *err) or when another CTA already
// failed.  Never spins forever: at most kSpinLimit polls and limit_ns of
// %globaltimer.
__device__ __forceinline__ bool wait_geq_n(const int *flag, int target, int *err, long long limit_ns) {
    if (ld_acquire(flag) >= target) return true;
    const unsigned long long t0 = global_ns();
    for (long long it = 0;; ++it) {
        if (ld_acquire(flag) >= target) return true;
        if ((it & 15) == 15) {  // another CTA's failure, the bounds: every 16 polls
            if (ld_acquire(err) != kDevOk) return false;
            if (it > kSpinLimit || (long long)(global_ns() - t0) > limit_ns) {
                atomicCAS(err, kDevOk, kDevTimeout);
                return false;
            }
        }
        __nanosleep(32);
    }
}
__device__ __forceinline__ bool wait_geq(const int *flag, int target, int *err) {
    return wait_geq_n(flag, target, err, kWaitNs);
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

}  // namespace avs

#define AVS_CUDA_TRY(expr)                                   \
    do {                                                     \
        cudaError_t _e = (expr);                             \
        if (_e != cudaSuccess) {                             \
            avs::set_last_cuda_error(_e);                    \
            return (_e == cudaErrorMemoryAllocation) ? AVS_ERR_OOM : AVS_ERR_CUDA; \
        }                                                    \
    } while (0)

namespace avs {
void set_last_cuda_error(cudaError_t e);

// Host-side launchers (defined in the stage .cu files).
struct Stage1Work {
    void *tau;        // [nt][b] of T
    void *tblk;       // [nt][b/ib][ib*ib] of T
    int *flags;       // ticket (1) + two progress counters per tile (2 nt), reset per launch
    int *err;         // device status word (shared with other stages)
    void *tfull;      // [nt][b*b] of T: full compact-WY factors (tiles 128, 256)
    void *tc_ws = nullptr;  // tensor-core update buffers (stage1_tc_bytes), FP32 tiles
    int tc_split = 0;       // operand format of the tensor-core update (tc::Fmt); 0: SIMT update
    int df_update = 0;      // FP64 tiles: full-T trailing updates in double-float on the FP32 pipe
    // optional timing of the tensor-core updates: event pairs (start, end) per
    // half-step, at most ev_cap pairs; *ev_used counts the pairs recorded
    cudaEvent_t *ev_pairs = nullptr;
    int ev_cap = 0;
    int *ev_used = nullptr;
    // optional (one matrix): the tau of every half-step, copied out after its
    // panel -- QR half-step k, tile row r >= k at tau_q_out[(k * nt + r) * b + l];
    // LQ half-step k, tile column c >= k + 1 at tau_p_out[(k * nt + c) * b + l]
    void *tau_q_out = nullptr, *tau_p_out = nullptr;
    // batched mode: `batch` matrices at dA + z*sA, each with its own tau / T
    // blocks / full T / flag block at the given strides (elements, ints)
    int batch = 1;
    int64_t sA = 0, sTau = 0, sTblk = 0, sTfull = 0, sFlags = 0;
    // optional (tensor-core path): a second stream (high priority) and three
    // events on which the next half-step's panel and T build run while the
    // current trailing update finishes (lookahead); without them everything
    // runs on the caller's stream in the same order
    cudaStream_t aux = nullptr;
    cudaEvent_t la_fork = nullptr, la_panel = nullptr, la_tb = nullptr;
    // the panel may start beside the chain, waiting for its tiles, only when
    // the call holds a reservation of its panel CTAs (the waiting panels of
    // all running calls together stay within half of the SMs)
    bool la_ready = false;
};
template <typename T>
int stage1_tbuild(const T *dA, int64_t lda, int b, int layout, int pr, int pc, int P, const Stage1Work &w,
                  cudaStream_t s);

// Tensor-core update buffers (carved from Stage1Work::tc_ws).
struct TcBufs {
    float *xt;        // n x n: the transposed working matrix
    void *ph, *pl;    // n x n operand planes of the trailing block
    void *ych, *ycl;  // [nt][b][b] Y^T planes (GEMM 1)
    void *yrh, *yrl;  // [nt][b][b] Y planes (GEMM 2)
    float *S;         // [nt][n][b] S_p = Y_p^T A_p
    void *wh, *wl;    // [nt][n][b] W_p planes
    void *th, *tl;    // [nt][b][b] T_p planes
    int *ready;       // [nt + 1] per-tile counters of finished chain strips
    size_t bytes;
};
TcBufs stage1_tc_carve(void *ws, int64_t n, int b, int fmt);
size_t stage1_tc_bytes(int64_t n, int b, int fmt);
int stage1_tc_planes(const float *x, int64_t n, int fmt, const TcBufs &tb, cudaStream_t s);
int stage1_tc_planes_block(const float *x, int64_t n, int64_t r0, int64_t j0, int fmt, const TcBufs &tb,
                           cudaStream_t s);
int stage1_tc_transpose(const float *src, float *dst, int64_t n, int64_t i0, int64_t j0, int fmt, const TcBufs &tb,
                        cudaStream_t s);
// transpose of the box rows [i0, i0 + ni) x columns [j0, j0 + nj) of src
// (ld n) into dst, with dst's operand planes (multiples of 32)
int stage1_tc_transpose_box(const float *src, float *dst, int64_t n, int64_t i0, int64_t ni, int64_t j0, int64_t nj,
                            int fmt, const TcBufs &tb, cudaStream_t s);
enum TcParts : int { kTcS = 1, kTcChain = 2, kTcUpdate = 4, kTcPlanes = 8, kTcAll = 15 };
// columns of the chain's strips: the chain signals a tile of the top row
// (ready[tile] += 1 per strip, b / kChainStrip strips per tile) once the
// strip's final values are in memory
constexpr int kChainStrip = 32;
int stage1_tc_update(float *x, int64_t n, int b, int pr, int pc, int P, const Stage1Work &w, const TcBufs &tb,
                     cudaStream_t s, int64_t *launches, int parts = kTcAll, float *xt_out = nullptr,
                     int *ready = nullptr);
int stage1_chain_tplanes(const float *tfull, int b, int P, int fmt, void *t_hi, void *t_lo, cudaStream_t s);
int stage1_chain_tc2(float *x, int64_t n, int b, int pr, int pc, int P, void *t_hi, void *t_lo, const void *y_hi,
                     const void *y_lo, const float *S, int64_t ntr, void *w_hi, void *w_lo, int fmt, int *err,
                     cudaStream_t s, float *xt_out = nullptr, int *ready = nullptr);

template <typename T>
int stage1_update_full(T *dA, int64_t lda, int64_t n, int b, int layout, int pr, int pc, int P, const Stage1Work &w,
                       cudaStream_t s, int first_role = 0);

template <typename T>
int stage1_ge2bnd(T *dA, int64_t n, int64_t lda, int b, const Stage1Work &w, cudaStream_t s, int64_t *launches);
template <typename T>
int stage1_panel(T *dA, int64_t lda, int b, int layout, int pr, int pc, int P, int first_role, const Stage1Work &w,
                 cudaStream_t s);
template <typename T>
int stage1_update(T *dA, int64_t lda, int64_t ncols, int b, int layout, int pr, int pc, int P, int first_role,
                  const Stage1Work &w, cudaStream_t s);

// Out-of-core GE2BND / tiled QR on a host matrix (column-major, lda), through
// device memory dws of ws_bytes (ooc_plan gives the slab size and the bytes).
struct OocPlan {
    int slab;            // tile rows (columns) per slab below the top tile
    size_t bytes;        // device bytes the driver uses
    size_t slab_bytes;   // one slab buffer
};
OocPlan ooc_plan(int64_t n, int b, size_t elem, size_t budget);
struct OocStats {
    double h2d_bytes = 0, d2h_bytes = 0;
    int64_t launches = 0, slabs = 0;
    int64_t incore_from = -1;  // step at which the trailing block went in core (-1: never)
};
template <typename T>
int ooc_ge2bnd(T *A, int64_t n, int64_t lda, int b, bool qr_only, T *tau_host, const OocPlan &plan, void *dws,
               int *err, cudaStream_t s, OocStats *st);
template <typename T>
int stage1_geqrf(T *dA, int64_t n, int64_t lda, int b, const Stage1Work &w, T *dtau, cudaStream_t s,
                 int64_t *launches);

template <typename T>
int stage1_geqrt_tile(T *dA, int b, T *dtau, const Stage1Work &w, cudaStream_t s);
template <typename T>
int stage1_tsqrt_pair(T *dRB, int b, T *dtau, const Stage1Work &w, cudaStream_t s);

template <typename T>
int extract_band_compact(const T *dA, int64_t n, int64_t lda, int bw, double *dAB, int64_t ldab, cudaStream_t s);
template <typename T>
int extract_band_dense(const T *dA, int64_t n, int64_t lda, int bw, double *dB, int64_t ldb, cudaStream_t s);
int dense_band_to_compact(const double *dB, int64_t n, int64_t ldb, int bw, double *dAB, int64_t ldab,
                          cudaStream_t s);

struct Stage2Work {
    int *flags;  // ticket (1) + done (n) ; reset per launch
    int *err;
};
// window: bands 8/16/32 by the shared-memory window kernel (ldab == 3 bw)
int stage2_chase(double *dAB, int64_t n, int bw, int64_t ldab, double *dd, double *de, const Stage2Work &w,
                 cudaStream_t s, int num_sms, int64_t *launches, bool window = false);
int stage2_rate(int fp64, int num_sms, double *flops_per_s);

template <typename T>
int stage2_chase_df(const T *dW, int64_t n, int64_t ldw, int bw, float2 *dAB, int64_t ldab, double *dd, double *de,
                    const Stage2Work &w, cudaStream_t s, int num_sms, int64_t *launches, bool window = false);
// Batched stage 2 (stage2_chase.cu): tbw > 0 runs the blocked band reduction
// to width tbw first (dAB then holds the FP32 / FP64 band, 3 bw x n per
// matrix; dAB2 the narrow band, 3 tbw x n per matrix); window: the element
// chase in the shared-memory window where the band width allows it.
int stage2_chase_df_batched(const float *dW, int64_t n, int bw, int batch, float2 *dAB, int64_t ldab, double *dd,
                            double *de, const Stage2Work &w, cudaStream_t s, int num_sms, int64_t *launches, int tbw,
                            bool window, float2 *dAB2);
// FP64 tiles, double-float chase (the batched groups of AVS_PREC_FP64X2)
int stage2_chase_df_batched(const double *dW, int64_t n, int bw, int batch, float2 *dAB, int64_t ldab, double *dd,
                            double *de, const Stage2Work &w, cudaStream_t s, int num_sms, int64_t *launches,
                            bool window);
// Blocked band reduction bw -> tbw (stage2_band.cu), on a compact band with
// 16-byte aligned column segments: A(r, c) at dAB[(r - c + band_ku(bw)) + c *
// ldab], ldab = band_ldab(bw) (rows c-2bw .. c+bw of column c; a segment that
// starts at a row divisible by 4 starts on 16 bytes).
__host__ __device__ constexpr int band_ku(int bw) { return 2 * bw; }
__host__ __device__ constexpr int64_t band_ldab(int bw) { return 3 * (int64_t)bw + 1; }
// elements from one matrix's compact band to the next in a batch (a multiple
// of 4, so every matrix's segments stay on 16 bytes)
__host__ __device__ constexpr int64_t band_stride(int bw, int64_t n) { return (band_ldab(bw) * n + 3) / 4 * 4; }
template <typename R>
int band_stage(R *dAB, int64_t n, int bw, int tbw, int64_t ldab, const Stage2Work &w, cudaStream_t s, int num_sms,
               int batch, int64_t sAB, int64_t sDone);
bool band_stage_supported(int bw, int tbw);
template <typename TI, typename R>
int dense_to_band(const TI *dA, int64_t n, int64_t lda, int64_t sA, int bw, R *dAB, int64_t ldab, int64_t sAB,
                  int batch, cudaStream_t s);
template <typename R, typename St>
int band_to_band(const R *dAB1, int64_t n, int bw1, int64_t ldab1, int64_t sAB1, int bw2, St *dAB2, int64_t ldab2,
                 int64_t sAB2, int batch, cudaStream_t s);
template <typename R>
int band_to_dense(const R *dAB, int64_t n, int bw, int64_t ldab, R *dA, int64_t lda, cudaStream_t s);
// Hierarchical stage 2 (stage2_chase.cu): the band of width bw of dW
// (W[r + c*ldw]) -> width tbw by the blocked band reduction, then the element
// chase tbw -> 1; d and e out.  _df: FP32 band reduction, double-float chase;
// _fp64: FP64 throughout.  dAB1 holds 3 bw x n elements, dAB2 3 tbw x n.
// window: the narrow band's element chase by the windowed multi-sweep kernel
// (stage2_window.cu) instead of the cluster kernel.
// after_band (optional): recorded on s between the band reduction and the chase.
int stage2_chase_hier_df(const float *dW, int64_t n, int64_t ldw, int bw, int tbw, float *dAB1, float2 *dAB2,
                         double *dd, double *de, const Stage2Work &w, cudaStream_t s, int num_sms, int64_t *launches,
                         bool window, cudaEvent_t after_band = nullptr);
int stage2_chase_hier_fp64(const double *dW, int64_t n, int64_t ldw, int bw, int tbw, double *dAB1, double *dAB2,
                           double *dd, double *de, const Stage2Work &w, cudaStream_t s, int num_sms,
                           int64_t *launches, bool window, cudaEvent_t after_band = nullptr);
// Element chase of a narrow band (width 8, 16 or 32; compact storage, ldab =
// 3 bw) with G sweeps per CTA in a shared-memory window (stage2_window.cu).
bool chase_window_supported(int bw);
// batch matrices at stride sAB elements; w.flags: 1 + batch (n + 1) ints.
int stage2_chase_window_df(float2 *dAB, int64_t n, int bw, const Stage2Work &w, cudaStream_t s, int num_sms,
                           int batch = 1, int64_t sAB = 0);
int stage2_chase_window_fp64(double *dAB, int64_t n, int bw, const Stage2Work &w, cudaStream_t s, int num_sms,
                             int batch = 1, int64_t sAB = 0);
int stage3_bisect_df_batched(const double *dd, const double *de, int64_t n, int batch, double rel_tol,
                             double *dsigma, double *dscratch, float2 *dpairs, cudaStream_t s, int64_t *launches);
int stage2_chase_fp64_batched(const double *dW, int64_t n, int bw, int batch, double *dAB, int64_t ldab, double *dd,
                              double *de, const Stage2Work &w, cudaStream_t s, int num_sms, int64_t *launches,
                              int tbw, bool window, double *dAB2);
int stage3_bisect_batched(const double *dd, const double *de, int64_t n, int batch, double rel_tol, double *dsigma,
                          double *dscratch, cudaStream_t s, int64_t *launches);
int bidiag_svals_noalloc(int64_t n, const double *dd, const double *de, double *dsigma, double rel_tol,
                         cudaStream_t s);
int stage3_bisect_df(const double *dd, const double *de, int64_t n, double rel_tol, double *dsigma, double *dscratch,
                     float2 *dpairs, cudaStream_t s, int64_t *launches);
int stage3_bisect(const double *dd, const double *de, int64_t n, double rel_tol, double *dsigma, double *dscratch,
                  cudaStream_t s, int64_t *launches);

template <typename T>
int cast_from_double(const double *src, T *dst, int64_t n, cudaStream_t s);
template <typename TI, typename TO>
int copy_convert_2d(const TI *src, int64_t lds, TO *dst, int64_t ldd, int64_t rows, int64_t cols, cudaStream_t s);

}  // namespace avs
