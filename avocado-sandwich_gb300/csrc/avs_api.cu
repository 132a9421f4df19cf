// C ABI of the GB300 tiled SVD: handle, workspace, argument checks and the
// three-stage pipeline behind my_CU_svdval (CUDAbasedSVD/SVD_GPU.jl:257-283).
#include <algorithm>
#include <atomic>
#include <cfloat>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <new>
#include <tuple>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "avs_common.cuh"
#include "tc_gemm.cuh"

namespace avs {
static thread_local cudaError_t g_last_cuda = cudaSuccess;
void set_last_cuda_error(cudaError_t e) { g_last_cuda = e; }
}  // namespace avs

using namespace avs;

struct avs_handle {
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t aux = nullptr;  // stage 1's lookahead stream (panels and T builds)
    cudaEvent_t la_ev[3] = {};   // its hand-off events
    void *ws = nullptr;
    size_t ws_bytes = 0;
    cudaEvent_t ev[7] = {};  // 6: after the blocked band reduction of stage 2
    int *h_err = nullptr;  // pinned status word
    // batched path: its own grow-only workspace, pinned pointer tables,
    // captured graphs per group shape, autotuned tiles per order n
    void *bws = nullptr;
    size_t bws_bytes = 0;
    void *pinned = nullptr;
    size_t pinned_bytes = 0;
    std::vector<cudaEvent_t> upd_ev;  // event pairs timing the tensor-core updates
    struct Graph {
        cudaGraphExec_t exec = nullptr;
        int64_t kernels = 0;
        cudaEvent_t ev[4] = {};  // recorded inside the graph: start, after stage 1, 2, 3
    };
    std::map<std::tuple<int64_t, int, int, int>, Graph> graphs;  // (n, tile, count, output form)
    void drop_graphs() {
        for (auto &kv : graphs) {
            cudaGraphExecDestroy(kv.second.exec);
            for (cudaEvent_t e : kv.second.ev)
                if (e) cudaEventDestroy(e);
        }
        graphs.clear();
    }
    std::map<int64_t, int> tuned;
};

namespace {

constexpr int kMaxTile = 256;
constexpr int kMaxNarrowBand = 32;  // widest intermediate band of the hierarchical chase

inline size_t align_up(size_t x) { return (x + 255) & ~size_t(255); }

inline bool is_pow2(int64_t x) { return x > 0 && (x & (x - 1)) == 0; }

// Workspace carve-up for one call.
struct Layout {
    size_t off_w, off_stage, off_tau, off_tblk, off_flags1, off_flags2, off_err, off_ab, off_ab2, off_d, off_e,
        off_sig, off_scr, off_out, off_tfull, off_pairs, off_tc, total;
    int64_t ldab;
};

Layout make_layout(int64_t n, int b, size_t elem, size_t stage_elem, int tc_fmt = 0) {
    Layout L{};
    const int64_t nt = n / b;
    size_t o = 0;
    L.off_err = o;
    o = align_up(o + 64);
    L.off_w = o;
    o = align_up(o + elem * (size_t)n * (size_t)n);
    L.off_stage = o;
    o = align_up(o + stage_elem * (size_t)n * (size_t)n);
    L.off_tau = o;
    o = align_up(o + elem * (size_t)(nt + 1) * (size_t)b);
    L.off_tblk = o;
    o = align_up(o + elem * (size_t)(nt + 1) * (size_t)(b / 16) * 256);
    L.off_tfull = o;
    o = align_up(o + (b >= 128 ? elem * (size_t)(nt + 1) * (size_t)b * (size_t)b : 0));
    L.off_flags1 = o;
    o = align_up(o + sizeof(int) * (size_t)(2 * nt + 4));
    L.off_flags2 = o;
    o = align_up(o + sizeof(int) * (size_t)(n + 4));
    L.ldab = 3 * (int64_t)b;
    L.off_ab = o;
    // the one-stage chase's band (3b x n) or the block stage's (band_ldab(b) x n)
    o = align_up(o + sizeof(double) * (size_t)band_stride(b, n));
    L.off_ab2 = o;  // the narrow band of the hierarchical chase (width <= kMaxNarrowBand)
    o = align_up(o + sizeof(double) * (size_t)(3 * kMaxNarrowBand) * (size_t)n);
    L.off_d = o;
    o = align_up(o + sizeof(double) * (size_t)n);
    L.off_e = o;
    o = align_up(o + sizeof(double) * (size_t)(n + 1));
    L.off_sig = o;
    o = align_up(o + sizeof(double) * (size_t)n);
    L.off_scr = o;
    o = align_up(o + sizeof(double) * 8);
    L.off_out = o;
    o = align_up(o + sizeof(double) * (size_t)n);
    L.off_pairs = o;
    o = align_up(o + sizeof(float2) * (size_t)(2 * n + 1));
    L.off_tc = o;
    o = align_up(o + (tc_fmt ? stage1_tc_bytes(n, b, tc_fmt) : 0));
    L.total = o;
    return L;
}

int ensure_ws(avs_handle *h, size_t bytes) {
    if (h->ws_bytes >= bytes) return AVS_SUCCESS;
    if (h->ws) {
        cudaStreamSynchronize(h->stream);
        cudaFree(h->ws);
        h->ws = nullptr;
        h->ws_bytes = 0;
    }
    cudaError_t e = cudaMalloc(&h->ws, bytes);
    if (e != cudaSuccess) {
        set_last_cuda_error(e);
        cudaGetLastError();
        return AVS_ERR_OOM;
    }
    h->ws_bytes = bytes;
    return AVS_SUCCESS;
}

inline char *ws_at(avs_handle *h, size_t off) { return reinterpret_cast<char *>(h->ws) + off; }

int resolve_precision(int32_t requested, bool input_double) {
    if (requested == AVS_PREC_DEFAULT) return input_double ? AVS_PREC_FP64 : AVS_PREC_FP32;
    return requested;
}

// Storage element size of the stage-1 tiles for a precision mode (0 = mode not provided).
size_t storage_elem(int prec) {
    switch (prec) {
        case AVS_PREC_FP64:
        case AVS_PREC_FP64X2: return 8;
        case AVS_PREC_FP32:
        case AVS_PREC_TF32:
        case AVS_PREC_TF32X3:
        case AVS_PREC_BF16:
        case AVS_PREC_BF16X3: return 4;
        default: return 0;
    }
}

// Operand format of the tensor-core trailing update for a precision mode
// (tc::Fmt: 1 TF32, 3 split TF32, 4 BF16, 5 split BF16); 0 = SIMT update.
// Tiles below 128 keep the 16-block SIMT update (their updates are small).
int tc_split_of(int prec, int tile) {
    if (tile < 128) return 0;
    switch (prec) {
        case AVS_PREC_TF32: return tc::kTF32;
        case AVS_PREC_TF32X3: return tc::kTF32X3;
        case AVS_PREC_BF16: return tc::kBF16;
        case AVS_PREC_BF16X3: return tc::kBF16X3;
        default: return 0;
    }
}

// Arithmetic of stages 2 and 3: FP64 for the plain FP64 path (or on request),
// double-float (two FP32, ~44-48 bits) for the FP32-class modes.
bool fp64_stages(int prec, const avs_opts *opts) {
    if (opts && (opts->flags & AVS_FLAG_FP64_STAGES)) return true;
    if (opts && (opts->flags & AVS_FLAG_DF64_STAGES)) return false;
    return prec == AVS_PREC_FP64;
}

// FP64 tiles with the full-T trailing updates in double-float (AVS_PREC_FP64X2).
inline bool df_update_of(int prec) { return prec == AVS_PREC_FP64X2; }

inline int flags_of(const avs_opts *opts) { return opts ? opts->flags : 0; }

// Stage 2 of a single call: the band of width b goes to width
// narrow_band_of(b, flags, fp64) by the blocked band reduction, then to the
// bidiagonal by the element chase (0: the element chase from width b).  FP64
// stages keep the one-stage chase unless asked (the FP64 block stage runs on
// the FP64 pipe, 1/64 of the FP32 rate: slower than the one-stage FP64 chase,
// measured 537 vs 315 ms at n = 8192, tile 128).
int narrow_band_of(int b, int flags, bool fp64) {
    if (flags & AVS_FLAG_ONE_STAGE_CHASE) return 0;
    if (fp64 && !(flags & AVS_FLAG_HIER_CHASE)) return 0;
    const int t = (flags & AVS_FLAG_BAND32) ? 32 : 16;
    return band_stage_supported(b, t) ? t : 0;
}

// Bisection width relative to ||B||: 2 eps in FP64; 4e-14 in double-float
// when the tiles are FP64 (FP64X2: FP64-level results); 1e-10 in double-float
// for the FP32-class modes, whose values carry the ~1e-7..1e-5 error of their
// FP32 stage 1: the bracket is then 1000x below FP32's unit roundoff and the
// multisection stops four passes earlier.
double bisect_tol(bool f64, bool fp32_tiles, const avs_opts *opts) {
    if (opts && opts->bisect_rel_tol > 0) return opts->bisect_rel_tol;
    return f64 ? 2.0 * DBL_EPSILON : (fp32_tiles ? 1e-10 : 4e-14);
}

int check_common(avs_handle *h, int64_t m, int64_t n, int64_t lda, int32_t tile, const void *A, const void *sigma) {
    if (!h) return -1;
    if (m < 0) return -2;
    if (n < 0) return -3;
    if (lda < (m > 1 ? m : 1)) return -4;
    if (m != n) return AVS_ERR_NOT_IMPLEMENTED;
    if (!is_pow2(tile) || tile < 16 || (n > 0 && n % tile != 0)) return AVS_ERR_NOT_IMPLEMENTED;
    if (tile > kMaxTile) return AVS_ERR_UNSUPPORTED;
    if (n > 0 && !A) return -6;
    if (n > 0 && !sigma) return -7;
    return AVS_SUCCESS;
}

int finish_status(avs_handle *h, cudaStream_t s) {
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        set_last_cuda_error(e);
        return AVS_ERR_CUDA;
    }
    int dev_err = *h->h_err;
    if (dev_err == kDevTimeout) return AVS_ERR_TIMEOUT;
    if (dev_err == kDevNonfinite) return AVS_ERR_NONFINITE;
    if (dev_err != kDevOk) return AVS_ERR_INTERNAL;
    return AVS_SUCCESS;
}

// NVTX range around the host side of a stage (the launches it enqueues), for
// profilers' timelines.
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};

float ev_ms(cudaEvent_t a, cudaEvent_t b) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, a, b) != cudaSuccess) {
        cudaGetLastError();
        return 0.f;
    }
    return ms;
}

// Stages 2 and 3 from the band of W (entries W[r + c*ldw], 0 <= c - r <= b):
// bulge chase, bisection, sigma_out (type TO, device).  Records ev[2] between
// the stages and ev[3] at the end; the status word is the layout's.
template <typename S, typename TO>
int run_stages23(avs_handle *h, const Layout &L, int64_t n, int b, const S *W, int64_t ldw, TO *sigma_out,
                 double rel_tol, bool fp64_stages, cudaStream_t s, int64_t *launches, int flags,
                 bool *band_ran = nullptr) {
    int rc;
    int *err = reinterpret_cast<int *>(ws_at(h, L.off_err));
    double *AB = reinterpret_cast<double *>(ws_at(h, L.off_ab));
    double *dd = reinterpret_cast<double *>(ws_at(h, L.off_d));
    double *de = reinterpret_cast<double *>(ws_at(h, L.off_e));
    Stage2Work w2;
    w2.flags = reinterpret_cast<int *>(ws_at(h, L.off_flags2));
    w2.err = err;
    const int tbw = narrow_band_of(b, flags, fp64_stages);
    if (tbw > 0 && sizeof(S) == 8 && fp64_stages) {
        if ((rc = stage2_chase_hier_fp64(reinterpret_cast<const double *>(W), n, ldw, b, tbw, AB,
                                         reinterpret_cast<double *>(ws_at(h, L.off_ab2)), dd, de, w2, s, h->num_sms,
                                         launches, !(flags & AVS_FLAG_CLUSTER_CHASE), h->ev[6])) != AVS_SUCCESS)
            return rc;
        if (band_ran) *band_ran = true;
    } else if (tbw > 0 && sizeof(S) == 4 && !fp64_stages) {
        // the FP32 band of width b in the first half of AB (3b x n floats)
        if ((rc = stage2_chase_hier_df(reinterpret_cast<const float *>(W), n, ldw, b, tbw,
                                       reinterpret_cast<float *>(AB), reinterpret_cast<float2 *>(ws_at(h, L.off_ab2)),
                                       dd, de, w2, s, h->num_sms, launches, !(flags & AVS_FLAG_CLUSTER_CHASE),
                                       h->ev[6])) != AVS_SUCCESS)
            return rc;
        if (band_ran) *band_ran = true;
    } else if (fp64_stages) {
        if ((rc = extract_band_compact<S>(W, n, ldw, b, AB, L.ldab, s)) != AVS_SUCCESS) return rc;
        ++*launches;
        if ((rc = stage2_chase(AB, n, b, L.ldab, dd, de, w2, s, h->num_sms, launches,
                               !(flags & AVS_FLAG_CLUSTER_CHASE))) != AVS_SUCCESS)
            return rc;
    } else {
        // the FP64 band buffer holds the float2 band (same size)
        if ((rc = stage2_chase_df<S>(W, n, ldw, b, reinterpret_cast<float2 *>(AB), L.ldab, dd, de, w2, s,
                                     h->num_sms, launches, !(flags & AVS_FLAG_CLUSTER_CHASE))) != AVS_SUCCESS)
            return rc;
    }
    AVS_CUDA_TRY(cudaEventRecord(h->ev[2], s));
    double *sig = reinterpret_cast<double *>(ws_at(h, L.off_sig));
    if (fp64_stages)
        rc = stage3_bisect(dd, de, n, rel_tol, sig, reinterpret_cast<double *>(ws_at(h, L.off_scr)), s, launches);
    else
        rc = stage3_bisect_df(dd, de, n, rel_tol, sig, reinterpret_cast<double *>(ws_at(h, L.off_scr)),
                              reinterpret_cast<float2 *>(ws_at(h, L.off_pairs)), s, launches);
    if (rc != AVS_SUCCESS) return rc;
    if ((rc = cast_from_double<TO>(sig, sigma_out, n, s)) != AVS_SUCCESS) return rc;
    ++*launches;
    AVS_CUDA_TRY(cudaEventRecord(h->ev[3], s));
    return AVS_SUCCESS;
}

// Panel CTAs that calls of the process may keep waiting on the GPU for their
// tiles beside their chains.  A call reserves its largest panel (nt - 1 CTAs)
// for its whole duration, and only if all reservations together stay within
// half of the SMs: the chains of all running calls then always have the other
// half (waiting panels hold their SMs; every other kernel finishes by itself).
// Held until the call's stream is synchronised.
std::atomic<int> g_lookahead_ctas{0};
struct LookaheadSlot {
    int held = 0;
    LookaheadSlot(int want, int limit) {
        if (want <= 0) return;
        int cur = g_lookahead_ctas.load();
        while (cur + want <= limit) {
            if (g_lookahead_ctas.compare_exchange_weak(cur, cur + want)) {
                held = want;
                break;
            }
        }
    }
    ~LookaheadSlot() {
        if (held) g_lookahead_ctas.fetch_sub(held);
    }
    LookaheadSlot(const LookaheadSlot &) = delete;
    LookaheadSlot &operator=(const LookaheadSlot &) = delete;
};

// The pipeline on device data.  S = tile storage type.  src holds the input
// (type TI, leading dimension lds) on the device; sigma_out (type TO) on the device.
template <typename S, typename TI, typename TO>
int run_pipeline(avs_handle *h, const Layout &L, int64_t n, int b, const TI *src, int64_t lds, TO *sigma_out,
                 double rel_tol, bool fp64_stages, int tc_split, cudaStream_t s, avs_report *rep,
                 bool df_update = false, int chase_flags = 0) {
    int rc;
    int64_t launches = 0;
    S *W = reinterpret_cast<S *>(ws_at(h, L.off_w));
    int *err = reinterpret_cast<int *>(ws_at(h, L.off_err));
    AVS_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int), s));
    AVS_CUDA_TRY(cudaEventRecord(h->ev[0], s));
    if ((rc = copy_convert_2d<TI, S>(src, lds, W, n, n, n, s)) != AVS_SUCCESS) return rc;
    ++launches;
    Stage1Work w1;
    w1.tau = ws_at(h, L.off_tau);
    w1.tblk = ws_at(h, L.off_tblk);
    w1.flags = reinterpret_cast<int *>(ws_at(h, L.off_flags1));
    w1.err = err;
    w1.tfull = ws_at(h, L.off_tfull);
    w1.tc_split = tc_split;
    w1.tc_ws = tc_split ? ws_at(h, L.off_tc) : nullptr;
    w1.df_update = df_update ? 1 : 0;
    w1.aux = h->aux;
    w1.la_fork = h->la_ev[0];
    w1.la_panel = h->la_ev[1];
    w1.la_tb = h->la_ev[2];
    const LookaheadSlot slot(tc_split ? (int)(n / b) - 1 : 0, h->num_sms / 2);
    w1.la_ready = slot.held > 0;
    int upd_used = 0;
    if (tc_split && rep) {
        const int pairs = (int)(8 * (n / b));  // four parts per half-step
        while ((int)h->upd_ev.size() < 2 * pairs) {
            cudaEvent_t e;
            AVS_CUDA_TRY(cudaEventCreate(&e));
            h->upd_ev.push_back(e);
        }
        w1.ev_pairs = h->upd_ev.data();
        w1.ev_cap = pairs;
        w1.ev_used = &upd_used;
    }
    {
        NvtxRange r("avs stage 1: GE2BND");
        if ((rc = stage1_ge2bnd<S>(W, n, n, b, w1, s, &launches)) != AVS_SUCCESS) return rc;
    }
    AVS_CUDA_TRY(cudaEventRecord(h->ev[1], s));
    bool band_ran = false;
    {
        NvtxRange r("avs stages 2-3: chase, bisection");
        if ((rc = run_stages23<S, TO>(h, L, n, b, W, n, sigma_out, rel_tol, fp64_stages, s, &launches,
                                      chase_flags, &band_ran)) !=
            AVS_SUCCESS)
            return rc;
    }
    AVS_CUDA_TRY(cudaMemcpyAsync(h->h_err, err, sizeof(int), cudaMemcpyDeviceToHost, s));
    rc = finish_status(h, s);
    if (rep) {
        rep->t_stage1_ms = ev_ms(h->ev[0], h->ev[1]);
        rep->t_stage2_ms = ev_ms(h->ev[1], h->ev[2]);
        rep->t_stage3_ms = ev_ms(h->ev[2], h->ev[3]);
        rep->t_total_ms = ev_ms(h->ev[0], h->ev[3]);
        rep->t_update_ms = 0.0;
        rep->t_band_ms = band_ran ? ev_ms(h->ev[1], h->ev[6]) : 0.0;
        for (int q = 0; q < upd_used; ++q) rep->t_update_ms += ev_ms(h->upd_ev[2 * q], h->upd_ev[2 * q + 1]);
        rep->kernel_launches = launches;
        rep->workspace_bytes = (int64_t)h->ws_bytes;
        rep->status = rc;
    }
    return rc;
}

template <typename TI, typename TO>
int svdvals_dev(avs_handle *h, int64_t m, int64_t n, int64_t lda, int32_t tile, const TI *dA, TO *dsigma,
                const avs_opts *opts, avs_report *rep) {
    int rc = check_common(h, m, n, lda, tile, dA, dsigma);
    if (rep) {
        std::memset(rep, 0, sizeof(*rep));
        rep->status = rc;
    }
    if (rc != AVS_SUCCESS || n == 0) return rc;
    const int prec = resolve_precision(opts ? opts->precision : 0, sizeof(TI) == 8);
    const size_t elem = storage_elem(prec);
    if (elem == 0) return AVS_ERR_UNSUPPORTED;
    if (rep) rep->precision = prec;
    cudaStream_t s = (opts && opts->stream) ? reinterpret_cast<cudaStream_t>(opts->stream) : h->stream;
    AVS_CUDA_TRY(cudaSetDevice(h->device));
    const int split = tc_split_of(prec, tile);
    if (split < 0) return AVS_ERR_UNSUPPORTED;
    const Layout L = make_layout(n, tile, elem, 0, split);
    if ((rc = ensure_ws(h, L.total)) != AVS_SUCCESS) return rc;
    const bool f64 = fp64_stages(prec, opts);
    const double tol = bisect_tol(f64, elem == 4, opts);
    if (elem == 8)
        return run_pipeline<double, TI, TO>(h, L, n, tile, dA, lda, dsigma, tol, f64, 0, s, rep, df_update_of(prec),
                                            flags_of(opts));
    return run_pipeline<float, TI, TO>(h, L, n, tile, dA, lda, dsigma, tol, f64, split, s, rep, false,
                                       flags_of(opts));
}

// Page-locks a caller's host range for the duration of a call (large ranges
// only): the copy from page-locked memory is one DMA at the link's rate, where a
// pageable copy goes through the driver's staging buffers.  A range that
// cannot be registered (already page-locked, or refused) is copied as it is.
// The stream is drained before the range is released.
struct HostPin {
    void *p = nullptr;
    cudaStream_t s = nullptr;
    HostPin(const void *ptr, size_t bytes, cudaStream_t stream) : s(stream) {
        if (bytes < (size_t(32) << 20)) return;
        void *q = const_cast<void *>(ptr);
        if (cudaHostRegister(q, bytes, cudaHostRegisterDefault) == cudaSuccess ||
            (cudaGetLastError(), cudaHostRegister(q, bytes, cudaHostRegisterReadOnly) == cudaSuccess))
            p = q;
        else
            cudaGetLastError();
    }
    ~HostPin() {
        if (!p) return;
        cudaStreamSynchronize(s);
        cudaHostUnregister(p);
    }
};

template <typename T>
int svdvals_host(avs_handle *h, int64_t m, int64_t n, int64_t lda, int32_t tile, const T *A, T *sigma,
                 const avs_opts *opts, avs_report *rep) {
    int rc = check_common(h, m, n, lda, tile, A, sigma);
    if (rep) {
        std::memset(rep, 0, sizeof(*rep));
        rep->status = rc;
    }
    if (rc != AVS_SUCCESS || n == 0) return rc;
    const int prec = resolve_precision(opts ? opts->precision : 0, sizeof(T) == 8);
    const size_t elem = storage_elem(prec);
    if (elem == 0) return AVS_ERR_UNSUPPORTED;
    AVS_CUDA_TRY(cudaSetDevice(h->device));
    const int split = tc_split_of(prec, tile);
    if (split < 0) return AVS_ERR_UNSUPPORTED;
    const Layout L = make_layout(n, tile, elem, sizeof(T), split);
    if ((rc = ensure_ws(h, L.total)) != AVS_SUCCESS) return rc;
    cudaStream_t s = h->stream;
    T *stage = reinterpret_cast<T *>(ws_at(h, L.off_stage));
    const HostPin pin(A, sizeof(T) * ((size_t)lda * (size_t)(n - 1) + (size_t)n), s);
    AVS_CUDA_TRY(cudaEventRecord(h->ev[4], s));
    AVS_CUDA_TRY(cudaMemcpy2DAsync(stage, sizeof(T) * (size_t)n, A, sizeof(T) * (size_t)lda, sizeof(T) * (size_t)n,
                                   (size_t)n, cudaMemcpyHostToDevice, s));
    avs_report r2{};
    const bool f64 = fp64_stages(prec, opts);
    const double tol = bisect_tol(f64, elem == 4, opts);
    T *dout = reinterpret_cast<T *>(ws_at(h, L.off_out));
    if (elem == 8)
        rc = run_pipeline<double, T, T>(h, L, n, tile, stage, n, dout, tol, f64, 0, s, &r2, df_update_of(prec),
                                        flags_of(opts));
    else
        rc = run_pipeline<float, T, T>(h, L, n, tile, stage, n, dout, tol, f64, split, s, &r2, false,
                                       flags_of(opts));
    if (rc == AVS_SUCCESS) {
        AVS_CUDA_TRY(cudaMemcpyAsync(sigma, dout, sizeof(T) * (size_t)n, cudaMemcpyDeviceToHost, s));
        AVS_CUDA_TRY(cudaEventRecord(h->ev[5], s));
        AVS_CUDA_TRY(cudaStreamSynchronize(s));
    }
    if (rep) {
        *rep = r2;
        rep->precision = prec;
        if (rc == AVS_SUCCESS) {
            rep->t_h2d_ms = ev_ms(h->ev[4], h->ev[0]);
            rep->t_d2h_ms = ev_ms(h->ev[3], h->ev[5]);
            rep->t_total_ms = ev_ms(h->ev[4], h->ev[5]);
        }
        rep->status = rc;
    }
    return rc;
}

}  // namespace

extern "C" {

int avs_version(void) { return AVS_VERSION_MAJOR * 100 + AVS_VERSION_MINOR; }

const char *avs_strerror(int status) {
    switch (status) {
        case AVS_SUCCESS: return "success";
        case AVS_ERR_NOT_IMPLEMENTED: return "Not implemented";
        case AVS_ERR_CUDA: {  // names the last CUDA error this thread met in the library
            static thread_local char msg[192];
            std::snprintf(msg, sizeof msg, "CUDA runtime error (%s)", cudaGetErrorString(g_last_cuda));
            return msg;
        }
        case AVS_ERR_OOM: return "out of device memory";
        case AVS_ERR_TIMEOUT: return "a bounded device-side wait timed out";
        case AVS_ERR_NONFINITE: return "non-finite value met in the factorisation";
        case AVS_ERR_NO_DEVICE: return "no usable CUDA device";
        case AVS_ERR_UNSUPPORTED: return "valid request not supported by the library";
        case AVS_ERR_INTERNAL: return "internal error";
        case AVS_ERR_TOO_LARGE: return "size exceeds the static scratch of the allocation-free entry point";
        default: return status < 0 ? "invalid argument" : "unknown error";
    }
}

int avs_create(avs_handle **out, int device) {
    if (!out) return -1;
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count <= 0) {
        cudaGetLastError();
        return AVS_ERR_NO_DEVICE;
    }
    if (device < 0 || device >= count) return -2;
    avs_handle *h = new (std::nothrow) avs_handle();
    if (!h) return AVS_ERR_INTERNAL;
    h->device = device;
    AVS_CUDA_TRY(cudaSetDevice(device));
    AVS_CUDA_TRY(cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, device));
    AVS_CUDA_TRY(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
    {
        // the lookahead stream at the highest priority: the panels are a latency-bound chain on
        // few SMs, and the block scheduler then places them ahead of the update's tiles
        int least = 0, greatest = 0;
        AVS_CUDA_TRY(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        AVS_CUDA_TRY(cudaStreamCreateWithPriority(&h->aux, cudaStreamNonBlocking, greatest));
    }
    for (auto &e : h->ev) AVS_CUDA_TRY(cudaEventCreate(&e));
    for (auto &e : h->la_ev) AVS_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    AVS_CUDA_TRY(cudaMallocHost(&h->h_err, sizeof(int)));
    *h->h_err = 0;
    *out = h;
    return AVS_SUCCESS;
}

int avs_destroy(avs_handle *h) {
    if (!h) return AVS_SUCCESS;
    cudaSetDevice(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    if (h->ws) cudaFree(h->ws);
    for (auto &e : h->ev)
        if (e) cudaEventDestroy(e);
    if (h->h_err) cudaFreeHost(h->h_err);
    h->drop_graphs();
    if (h->bws) cudaFree(h->bws);
    if (h->pinned) cudaFreeHost(h->pinned);
    for (cudaEvent_t e : h->upd_ev) cudaEventDestroy(e);
    for (cudaEvent_t e : h->la_ev)
        if (e) cudaEventDestroy(e);
    if (h->aux) {
        cudaStreamSynchronize(h->aux);
        cudaStreamDestroy(h->aux);
    }
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return AVS_SUCCESS;
}

int avs_reserve(avs_handle *h, int64_t n, int32_t tile, int32_t precision) {
    if (!h) return -1;
    if (n < 0) return -2;
    if (!is_pow2(tile) || tile < 16 || (n > 0 && n % tile != 0)) return AVS_ERR_NOT_IMPLEMENTED;
    if (tile > kMaxTile) return AVS_ERR_UNSUPPORTED;
    const int prec = resolve_precision(precision, true);
    const size_t elem = storage_elem(prec);
    if (elem == 0) return AVS_ERR_UNSUPPORTED;
    AVS_CUDA_TRY(cudaSetDevice(h->device));
    return ensure_ws(h, make_layout(n, tile, elem, 8, tc_split_of(prec, tile)).total);
}

int avs_svdvals_s(avs_handle *h, int64_t m, int64_t n, int64_t lda, int32_t tile, const float *A, float *sigma,
                  const avs_opts *opts, avs_report *report) {
    return svdvals_host<float>(h, m, n, lda, tile, A, sigma, opts, report);
}
int avs_svdvals_d(avs_handle *h, int64_t m, int64_t n, int64_t lda, int32_t tile, const double *A, double *sigma,
                  const avs_opts *opts, avs_report *report) {
    return svdvals_host<double>(h, m, n, lda, tile, A, sigma, opts, report);
}
int avs_svdvals_dev_s(avs_handle *h, int64_t m, int64_t n, int64_t lda, int32_t tile, const float *dA,
                      float *dsigma, const avs_opts *opts, avs_report *report) {
    return svdvals_dev<float, float>(h, m, n, lda, tile, dA, dsigma, opts, report);
}
int avs_svdvals_dev_d(avs_handle *h, int64_t m, int64_t n, int64_t lda, int32_t tile, const double *dA,
                      double *dsigma, const avs_opts *opts, avs_report *report) {
    return svdvals_dev<double, double>(h, m, n, lda, tile, dA, dsigma, opts, report);
}

}  // extern "C"

namespace {
// Blockbidiag! in place.  with_prec: opts->precision selects the update
// arithmetic of FP32 tiles (tensor-core modes included), as in avs_svdvals;
// otherwise the input type's SIMT update runs.  dtq / dtp (may be NULL)
// receive the tau of the QR / LQ half-steps.
template <typename T>
int blockbidiag_dev(avs_handle *h, int64_t n, int64_t lda, int32_t tile, T *dA, const avs_opts *opts,
                    avs_report *rep, T *dtq = nullptr, T *dtp = nullptr, bool with_prec = false) {
    int rc = check_common(h, n, n, lda, tile, dA, dA);
    if (rep) {
        std::memset(rep, 0, sizeof(*rep));
        rep->status = rc;
    }
    if (rc != AVS_SUCCESS || n == 0) return rc;
    int prec = sizeof(T) == 8 ? AVS_PREC_FP64 : AVS_PREC_FP32;
    if (with_prec) {
        prec = resolve_precision(opts ? opts->precision : 0, sizeof(T) == 8);
        if (storage_elem(prec) != sizeof(T)) return AVS_ERR_UNSUPPORTED;  // tiles are the input type
    }
    AVS_CUDA_TRY(cudaSetDevice(h->device));
    const int split = sizeof(T) == 4 ? tc_split_of(prec, tile) : 0;
    const Layout L = make_layout(n, tile, sizeof(T), 0, split);
    if ((rc = ensure_ws(h, L.total)) != AVS_SUCCESS) return rc;
    cudaStream_t s = (opts && opts->stream) ? reinterpret_cast<cudaStream_t>(opts->stream) : h->stream;
    int *err = reinterpret_cast<int *>(ws_at(h, L.off_err));
    AVS_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int), s));
    Stage1Work w1;
    w1.tau = ws_at(h, L.off_tau);
    w1.tblk = ws_at(h, L.off_tblk);
    w1.flags = reinterpret_cast<int *>(ws_at(h, L.off_flags1));
    w1.err = err;
    w1.tfull = ws_at(h, L.off_tfull);
    w1.tc_split = split;
    w1.tc_ws = split ? ws_at(h, L.off_tc) : nullptr;
    w1.tau_q_out = dtq;
    w1.tau_p_out = dtp;
    w1.df_update = (sizeof(T) == 8 && df_update_of(prec)) ? 1 : 0;
    int64_t launches = 0;
    AVS_CUDA_TRY(cudaEventRecord(h->ev[0], s));
    // the stage-1 kernels move 16-byte vectors: a matrix that is not 16-byte
    // aligned (pointer or leading dimension) runs on an aligned copy
    const bool aligned = (reinterpret_cast<uintptr_t>(dA) % 16 == 0) && ((size_t)lda * sizeof(T)) % 16 == 0;
    if (aligned) {
        if ((rc = stage1_ge2bnd<T>(dA, n, lda, tile, w1, s, &launches)) != AVS_SUCCESS) return rc;
    } else {
        T *W = reinterpret_cast<T *>(ws_at(h, L.off_w));
        AVS_CUDA_TRY(cudaMemcpy2DAsync(W, sizeof(T) * n, dA, sizeof(T) * lda, sizeof(T) * n, n,
                                       cudaMemcpyDeviceToDevice, s));
        if ((rc = stage1_ge2bnd<T>(W, n, n, tile, w1, s, &launches)) != AVS_SUCCESS) return rc;
        AVS_CUDA_TRY(cudaMemcpy2DAsync(dA, sizeof(T) * lda, W, sizeof(T) * n, sizeof(T) * n, n,
                                       cudaMemcpyDeviceToDevice, s));
    }
    AVS_CUDA_TRY(cudaEventRecord(h->ev[1], s));
    AVS_CUDA_TRY(cudaMemcpyAsync(h->h_err, err, sizeof(int), cudaMemcpyDeviceToHost, s));
    rc = finish_status(h, s);
    if (rep) {
        rep->t_stage1_ms = rep->t_total_ms = ev_ms(h->ev[0], h->ev[1]);
        rep->kernel_launches = launches;
        rep->precision = prec;
        rep->status = rc;
    }
    return rc;
}

// tiled_QR! (KAbasedSVD/src/tiledalgos.jl:6-15) in place on a device matrix.
template <typename T>
int geqrf_dev(avs_handle *h, int64_t n, int64_t lda, int32_t tile, T *dA, T *dtau, const avs_opts *opts,
              avs_report *rep) {
    int rc = check_common(h, n, n, lda, tile, dA, dA);
    if (rep) {
        std::memset(rep, 0, sizeof(*rep));
        rep->status = rc;
    }
    if (rc != AVS_SUCCESS || n == 0) return rc;
    const int prec = resolve_precision(opts ? opts->precision : 0, sizeof(T) == 8);
    if (storage_elem(prec) != sizeof(T)) return AVS_ERR_UNSUPPORTED;  // tiles are the input type
    AVS_CUDA_TRY(cudaSetDevice(h->device));
    const int split = sizeof(T) == 4 ? tc_split_of(prec, tile) : 0;
    const Layout L = make_layout(n, tile, sizeof(T), 0, split);
    if ((rc = ensure_ws(h, L.total)) != AVS_SUCCESS) return rc;
    cudaStream_t s = (opts && opts->stream) ? reinterpret_cast<cudaStream_t>(opts->stream) : h->stream;
    int *err = reinterpret_cast<int *>(ws_at(h, L.off_err));
    AVS_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int), s));
    Stage1Work w1;
    w1.tau = ws_at(h, L.off_tau);
    w1.tblk = ws_at(h, L.off_tblk);
    w1.flags = reinterpret_cast<int *>(ws_at(h, L.off_flags1));
    w1.err = err;
    w1.tfull = ws_at(h, L.off_tfull);
    w1.tc_split = split;
    w1.tc_ws = split ? ws_at(h, L.off_tc) : nullptr;
    int64_t launches = 0;
    AVS_CUDA_TRY(cudaEventRecord(h->ev[0], s));
    const bool aligned = (reinterpret_cast<uintptr_t>(dA) % 16 == 0) && lda == n;
    if (aligned) {
        if ((rc = stage1_geqrf<T>(dA, n, n, tile, w1, dtau, s, &launches)) != AVS_SUCCESS) return rc;
    } else {  // the kernels want a 16-byte aligned matrix with ld n: run on a copy
        T *W = reinterpret_cast<T *>(ws_at(h, L.off_w));
        AVS_CUDA_TRY(cudaMemcpy2DAsync(W, sizeof(T) * n, dA, sizeof(T) * lda, sizeof(T) * n, n,
                                       cudaMemcpyDeviceToDevice, s));
        if ((rc = stage1_geqrf<T>(W, n, n, tile, w1, dtau, s, &launches)) != AVS_SUCCESS) return rc;
        AVS_CUDA_TRY(cudaMemcpy2DAsync(dA, sizeof(T) * lda, W, sizeof(T) * n, sizeof(T) * n, n,
                                       cudaMemcpyDeviceToDevice, s));
    }
    AVS_CUDA_TRY(cudaEventRecord(h->ev[1], s));
    AVS_CUDA_TRY(cudaMemcpyAsync(h->h_err, err, sizeof(int), cudaMemcpyDeviceToHost, s));
    rc = finish_status(h, s);
    if (rep) {
        rep->t_stage1_ms = rep->t_total_ms = ev_ms(h->ev[0], h->ev[1]);
        rep->kernel_launches = launches;
        rep->precision = prec;
        rep->status = rc;
    }
    return rc;
}

template <typename T>
int extract_band_dev(avs_handle *h, int64_t n, int64_t lda, int32_t bw, const T *dA, double *dB, int64_t ldb) {
    if (!h) return -1;
    if (n < 0) return -2;
    if (lda < (n > 1 ? n : 1)) return -3;
    if (bw < 0) return -4;
    if (n > 0 && !dA) return -5;
    if (n > 0 && !dB) return -6;
    if (ldb < (n > 1 ? n : 1)) return -7;
    if (n == 0) return AVS_SUCCESS;
    AVS_CUDA_TRY(cudaSetDevice(h->device));
    int rc = extract_band_dense<T>(dA, n, lda, bw, dB, ldb, h->stream);
    if (rc != AVS_SUCCESS) return rc;
    AVS_CUDA_TRY(cudaStreamSynchronize(h->stream));
    return AVS_SUCCESS;
}

template <typename T>
int tile_kernel(avs_handle *h, int32_t b, T *dA, T *dB, T *dtau, bool ts) {
    if (!h) return -1;
    if (!is_pow2(b) || b < 16) return AVS_ERR_NOT_IMPLEMENTED;
    if (b > kMaxTile) return AVS_ERR_UNSUPPORTED;
    if (!dA) return -3;
    if (ts && !dB) return -4;
    if (!dtau) return ts ? -5 : -4;
    AVS_CUDA_TRY(cudaSetDevice(h->device));
    const Layout L = make_layout(2 * b, b, sizeof(T), 0);
    int rc = ensure_ws(h, L.total);
    if (rc != AVS_SUCCESS) return rc;
    cudaStream_t s = h->stream;
    int *err = reinterpret_cast<int *>(ws_at(h, L.off_err));
    AVS_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int), s));
    Stage1Work w1;
    w1.tau = ws_at(h, L.off_tau);
    w1.tblk = ws_at(h, L.off_tblk);
    w1.flags = reinterpret_cast<int *>(ws_at(h, L.off_flags1));
    w1.err = err;
    w1.tfull = ws_at(h, L.off_tfull);
    if (!ts) {
        if (reinterpret_cast<uintptr_t>(dA) % 16 == 0) {
            rc = stage1_geqrt_tile<T>(dA, b, dtau, w1, s);
        } else {  // 16-byte vectors in the kernel: run on an aligned copy
            T *cp = reinterpret_cast<T *>(ws_at(h, L.off_w));
            AVS_CUDA_TRY(cudaMemcpyAsync(cp, dA, sizeof(T) * (size_t)b * b, cudaMemcpyDeviceToDevice, s));
            rc = stage1_geqrt_tile<T>(cp, b, dtau, w1, s);
            if (rc == AVS_SUCCESS)
                AVS_CUDA_TRY(cudaMemcpyAsync(dA, cp, sizeof(T) * (size_t)b * b, cudaMemcpyDeviceToDevice, s));
        }
    } else {
        T *pair = reinterpret_cast<T *>(ws_at(h, L.off_w));  // 2b x b, ld 2b
        AVS_CUDA_TRY(cudaMemcpy2DAsync(pair, sizeof(T) * 2 * b, dA, sizeof(T) * b, sizeof(T) * b, b,
                                       cudaMemcpyDeviceToDevice, s));
        AVS_CUDA_TRY(cudaMemcpy2DAsync(pair + b, sizeof(T) * 2 * b, dB, sizeof(T) * b, sizeof(T) * b, b,
                                       cudaMemcpyDeviceToDevice, s));
        rc = stage1_tsqrt_pair<T>(pair, b, dtau, w1, s);
        if (rc == AVS_SUCCESS) {
            AVS_CUDA_TRY(cudaMemcpy2DAsync(dA, sizeof(T) * b, pair, sizeof(T) * 2 * b, sizeof(T) * b, b,
                                           cudaMemcpyDeviceToDevice, s));
            AVS_CUDA_TRY(cudaMemcpy2DAsync(dB, sizeof(T) * b, pair + b, sizeof(T) * 2 * b, sizeof(T) * b, b,
                                           cudaMemcpyDeviceToDevice, s));
        }
    }
    if (rc != AVS_SUCCESS) return rc;
    AVS_CUDA_TRY(cudaMemcpyAsync(h->h_err, err, sizeof(int), cudaMemcpyDeviceToHost, s));
    return finish_status(h, s);
}

// Out-of-core entry points (OOC_Bidiag! / OOC_SVD! / OOC_QR!, tiledalgos.jl:232-260).
enum OocMode { kOocBand = 0, kOocSvd = 1, kOocQr = 2 };

// Upper band (0 <= c - r <= b) of the host matrix A into band storage on the
// device: element (r, c) at band[b + r + c*b], i.e. the band of the matrix
// (band + b) with leading dimension b.  Columns c >= b are one strided copy.
template <typename T>
int band_to_device(const T *A, int64_t n, int64_t lda, int b, T *band, cudaStream_t s) {
    for (int64_t c = 0; c < std::min<int64_t>(b, n); ++c)
        AVS_CUDA_TRY(cudaMemcpyAsync(band + b + c * b, A + c * lda, sizeof(T) * (size_t)(c + 1),
                                     cudaMemcpyHostToDevice, s));
    if (n > b)
        AVS_CUDA_TRY(cudaMemcpy2DAsync(band + (int64_t)b * (b + 1), sizeof(T) * (size_t)(b + 1), A + (int64_t)b * lda,
                                       sizeof(T) * (size_t)(lda + 1), sizeof(T) * (size_t)(b + 1), (size_t)(n - b),
                                       cudaMemcpyHostToDevice, s));
    return AVS_SUCCESS;
}

template <typename T>
int ooc_call(avs_handle *h, int64_t n, int64_t lda, int32_t tile, T *A, T *sigma, T *tau, int mode,
             int64_t device_bytes, const avs_opts *opts, avs_report *rep) {
    int rc = check_common(h, n, n, lda, tile, A, mode == kOocSvd ? static_cast<const void *>(sigma) : A);
    if (rep) {
        std::memset(rep, 0, sizeof(*rep));
        rep->status = rc;
    }
    if (rc != AVS_SUCCESS || n == 0) return rc;
    if (device_bytes < 0) return -8;
    const int prec = resolve_precision(opts ? opts->precision : 0, sizeof(T) == 8);
    // the slabs run the SIMT 16-reflector-block update in the input's type
    if (prec != (sizeof(T) == 8 ? AVS_PREC_FP64 : AVS_PREC_FP32)) return AVS_ERR_UNSUPPORTED;
    AVS_CUDA_TRY(cudaSetDevice(h->device));
    size_t budget = (size_t)device_bytes;
    if (budget == 0) {
        size_t fr = 0, tot = 0;
        AVS_CUDA_TRY(cudaMemGetInfo(&fr, &tot));
        budget = fr / 10 * 9 + h->ws_bytes;
    }
    if (budget <= 256) return AVS_ERR_OOM;
    const OocPlan plan = ooc_plan(n, tile, sizeof(T), budget - 256);
    if (plan.slab < 1) return AVS_ERR_OOM;
    const Layout L = make_layout(n, tile, 0, 0, 0);  // stages 2-3 only (no n x n buffers)
    const size_t band_off = L.total;
    const size_t need23 = mode == kOocSvd ? band_off + align_up(sizeof(T) * (size_t)n * (tile + 1)) : 0;
    if ((rc = ensure_ws(h, std::max(256 + plan.bytes, need23))) != AVS_SUCCESS) return rc;
    cudaStream_t s = h->stream;
    // pin the caller's matrix for the duration of the call (pageable copies
    // still work when it cannot be registered)
    const size_t a_bytes = sizeof(T) * ((size_t)lda * (size_t)(n - 1) + (size_t)n);
    bool registered = cudaHostRegister(A, a_bytes, cudaHostRegisterDefault) == cudaSuccess;
    if (!registered) cudaGetLastError();
    int *err = reinterpret_cast<int *>(ws_at(h, L.off_err));  // offset 0, outside the slab region
    OocStats st;
    int64_t launches = 0;
    rc = AVS_SUCCESS;
    auto step = [&]() -> int {
        AVS_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int), s));
        AVS_CUDA_TRY(cudaEventRecord(h->ev[0], s));
        NvtxRange range("avs out-of-core stage 1");
        int r = ooc_ge2bnd<T>(A, n, lda, tile, mode == kOocQr, mode == kOocQr ? tau : nullptr, plan, ws_at(h, 256),
                              err, s, &st);
        if (r != AVS_SUCCESS) return r;
        AVS_CUDA_TRY(cudaEventRecord(h->ev[1], s));
        if (mode == kOocSvd) {
            T *band = reinterpret_cast<T *>(ws_at(h, band_off));
            if ((r = band_to_device<T>(A, n, lda, tile, band, s)) != AVS_SUCCESS) return r;
            const bool f64 = fp64_stages(prec, opts);
            T *dout = reinterpret_cast<T *>(ws_at(h, L.off_out));
            const double tol = bisect_tol(f64, sizeof(T) == 4, opts);
            if ((r = run_stages23<T, T>(h, L, n, tile, band + tile, tile, dout, tol, f64, s, &launches,
                                        opts ? opts->flags : 0)) != AVS_SUCCESS)
                return r;
            AVS_CUDA_TRY(cudaMemcpyAsync(sigma, dout, sizeof(T) * (size_t)n, cudaMemcpyDeviceToHost, s));
        } else {
            AVS_CUDA_TRY(cudaEventRecord(h->ev[2], s));
            AVS_CUDA_TRY(cudaEventRecord(h->ev[3], s));
        }
        AVS_CUDA_TRY(cudaMemcpyAsync(h->h_err, err, sizeof(int), cudaMemcpyDeviceToHost, s));
        return finish_status(h, s);
    };
    rc = step();
    if (rc != AVS_SUCCESS) cudaStreamSynchronize(s);  // no copy into A may be left in flight
    if (registered) cudaHostUnregister(A);
    if (rep) {
        if (rc == AVS_SUCCESS) {
            rep->t_stage1_ms = ev_ms(h->ev[0], h->ev[1]);
            rep->t_stage2_ms = ev_ms(h->ev[1], h->ev[2]);
            rep->t_stage3_ms = ev_ms(h->ev[2], h->ev[3]);
            rep->t_total_ms = ev_ms(h->ev[0], h->ev[3]);
        }
        rep->kernel_launches = launches + st.launches;
        rep->workspace_bytes = (int64_t)h->ws_bytes;
        rep->precision = prec;
        rep->status = rc;
    }
    return rc;
}
}  // namespace

template <typename R>
int band_reduce_dev(avs_handle *h, int64_t n, int32_t bw, int32_t tbw, R *dB, int64_t ldb, avs_report *rep) {
    if (!h) return -1;
    if (n < 0) return -2;
    if (bw < 1) return -3;
    if (tbw < 1 || tbw >= bw) return -4;
    if (n > 0 && !dB) return -5;
    if (ldb < (n > 1 ? n : 1)) return -6;
    if (rep) std::memset(rep, 0, sizeof(*rep));
    if (!band_stage_supported(bw, tbw)) return AVS_ERR_UNSUPPORTED;
    if (n == 0) return AVS_SUCCESS;
    AVS_CUDA_TRY(cudaSetDevice(h->device));
    const Layout L = make_layout(n, 1, 8, 0);
    const int64_t ldab = band_ldab(bw);
    const size_t ab_off = align_up(L.total);
    const size_t fl_off = align_up(ab_off + sizeof(R) * (size_t)band_stride(bw, n));
    int rc = ensure_ws(h, align_up(fl_off + sizeof(int) * (size_t)(n + 4)));
    if (rc != AVS_SUCCESS) return rc;
    cudaStream_t s = h->stream;
    int *err = reinterpret_cast<int *>(ws_at(h, L.off_err));
    AVS_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int), s));
    R *AB = reinterpret_cast<R *>(ws_at(h, ab_off));
    AVS_CUDA_TRY(cudaEventRecord(h->ev[0], s));
    if ((rc = dense_to_band<R, R>(dB, n, ldb, 0, bw, AB, ldab, 0, 1, s)) != AVS_SUCCESS) return rc;
    Stage2Work w2;
    w2.flags = reinterpret_cast<int *>(ws_at(h, fl_off));
    w2.err = err;
    if ((rc = band_stage<R>(AB, n, bw, tbw, ldab, w2, s, h->num_sms, 1, 0, 0)) != AVS_SUCCESS) return rc;
    AVS_CUDA_TRY(cudaEventRecord(h->ev[1], s));
    if ((rc = band_to_dense<R>(AB, n, bw, ldab, dB, ldb, s)) != AVS_SUCCESS) return rc;
    AVS_CUDA_TRY(cudaMemcpyAsync(h->h_err, err, sizeof(int), cudaMemcpyDeviceToHost, s));
    rc = finish_status(h, s);
    if (rep) {
        rep->t_stage2_ms = rep->t_total_ms = ev_ms(h->ev[0], h->ev[1]);
        rep->kernel_launches = 3;
        rep->status = rc;
    }
    return rc;
}

extern "C" {

int avs_ooc_plan(int64_t n, int32_t tile, int32_t elem_bytes, int64_t device_bytes, int32_t *slab, int64_t *bytes,
                 int32_t *incore_from) {
    if (n < 0) return -1;
    if (!is_pow2(tile) || tile < 16 || (n > 0 && n % tile != 0)) return AVS_ERR_NOT_IMPLEMENTED;
    if (tile > kMaxTile) return AVS_ERR_UNSUPPORTED;
    if (elem_bytes != 4 && elem_bytes != 8) return -3;
    if (device_bytes <= 0) return -4;
    const OocPlan p = device_bytes > 256 ? ooc_plan(n, tile, (size_t)elem_bytes, (size_t)device_bytes - 256)
                                         : OocPlan{};
    const int64_t nt = n / tile;
    int64_t from = nt;
    for (int64_t k = 0; p.slab > 0 && k < nt; ++k) {
        const int64_t m = n - k * tile;
        if ((size_t)elem_bytes * (size_t)m * (size_t)m <= 2 * p.slab_bytes) {
            from = k;
            break;
        }
    }
    if (slab) *slab = p.slab;
    if (bytes) *bytes = p.slab > 0 ? (int64_t)(p.bytes + 256) : 0;
    if (incore_from) *incore_from = (int32_t)from;
    return AVS_SUCCESS;
}

int avs_blockbidiag_ooc_s(avs_handle *h, int64_t n, int64_t lda, int32_t tile, float *A, int64_t device_bytes,
                          avs_report *report) {
    return ooc_call<float>(h, n, lda, tile, A, nullptr, nullptr, kOocBand, device_bytes, nullptr, report);
}
int avs_blockbidiag_ooc_d(avs_handle *h, int64_t n, int64_t lda, int32_t tile, double *A, int64_t device_bytes,
                          avs_report *report) {
    return ooc_call<double>(h, n, lda, tile, A, nullptr, nullptr, kOocBand, device_bytes, nullptr, report);
}
int avs_svdvals_ooc_s(avs_handle *h, int64_t n, int64_t lda, int32_t tile, float *A, float *sigma,
                      int64_t device_bytes, const avs_opts *opts, avs_report *report) {
    return ooc_call<float>(h, n, lda, tile, A, sigma, nullptr, kOocSvd, device_bytes, opts, report);
}
int avs_svdvals_ooc_d(avs_handle *h, int64_t n, int64_t lda, int32_t tile, double *A, double *sigma,
                      int64_t device_bytes, const avs_opts *opts, avs_report *report) {
    return ooc_call<double>(h, n, lda, tile, A, sigma, nullptr, kOocSvd, device_bytes, opts, report);
}
int avs_geqrf_ooc_s(avs_handle *h, int64_t n, int64_t lda, int32_t tile, float *A, float *tau, int64_t device_bytes,
                    avs_report *report) {
    return ooc_call<float>(h, n, lda, tile, A, nullptr, tau, kOocQr, device_bytes, nullptr, report);
}
int avs_geqrf_ooc_d(avs_handle *h, int64_t n, int64_t lda, int32_t tile, double *A, double *tau,
                    int64_t device_bytes, avs_report *report) {
    return ooc_call<double>(h, n, lda, tile, A, nullptr, tau, kOocQr, device_bytes, nullptr, report);
}

int avs_blockbidiag_dev_s(avs_handle *h, int64_t n, int64_t lda, int32_t tile, float *dA, const avs_opts *opts,
                          avs_report *report) {
    return blockbidiag_dev<float>(h, n, lda, tile, dA, opts, report);
}
int avs_blockbidiag_dev_d(avs_handle *h, int64_t n, int64_t lda, int32_t tile, double *dA, const avs_opts *opts,
                          avs_report *report) {
    return blockbidiag_dev<double>(h, n, lda, tile, dA, opts, report);
}

int avs_blockbidiag_tau_dev_s(avs_handle *h, int64_t n, int64_t lda, int32_t tile, float *dA, float *dtau_q,
                              float *dtau_p, const avs_opts *opts, avs_report *report) {
    return blockbidiag_dev<float>(h, n, lda, tile, dA, opts, report, dtau_q, dtau_p, true);
}
int avs_blockbidiag_tau_dev_d(avs_handle *h, int64_t n, int64_t lda, int32_t tile, double *dA, double *dtau_q,
                              double *dtau_p, const avs_opts *opts, avs_report *report) {
    return blockbidiag_dev<double>(h, n, lda, tile, dA, opts, report, dtau_q, dtau_p, true);
}
int avs_geqrf_dev_s(avs_handle *h, int64_t n, int64_t lda, int32_t tile, float *dA, float *dtau,
                    const avs_opts *opts, avs_report *report) {
    return geqrf_dev<float>(h, n, lda, tile, dA, dtau, opts, report);
}
int avs_geqrf_dev_d(avs_handle *h, int64_t n, int64_t lda, int32_t tile, double *dA, double *dtau,
                    const avs_opts *opts, avs_report *report) {
    return geqrf_dev<double>(h, n, lda, tile, dA, dtau, opts, report);
}
int avs_extract_band_dev_s(avs_handle *h, int64_t n, int64_t lda, int32_t bw, const float *dA, double *dB,
                           int64_t ldb) {
    return extract_band_dev<float>(h, n, lda, bw, dA, dB, ldb);
}
int avs_extract_band_dev_d(avs_handle *h, int64_t n, int64_t lda, int32_t bw, const double *dA, double *dB,
                           int64_t ldb) {
    return extract_band_dev<double>(h, n, lda, bw, dA, dB, ldb);
}

int avs_band_to_bidiag_dev(avs_handle *h, int64_t n, int32_t bw, const double *dB, int64_t ldb, double *dd,
                           double *de, avs_report *rep) {
    if (!h) return -1;
    if (n < 0) return -2;
    if (bw < 1) return -3;
    if (n > 0 && !dB) return -4;
    if (ldb < (n > 1 ? n : 1)) return -5;
    if (n > 0 && !dd) return -6;
    if (n > 1 && !de) return -7;
    if (rep) std::memset(rep, 0, sizeof(*rep));
    if (n == 0) return AVS_SUCCESS;
    AVS_CUDA_TRY(cudaSetDevice(h->device));
    const Layout L = make_layout(n, 1, 8, 0);
    const int64_t ldab = 3 * (int64_t)bw;
    // compact band + flags after the standard layout
    const size_t ab_off = align_up(L.total);
    const size_t fl_off = align_up(ab_off + sizeof(double) * (size_t)ldab * (size_t)n);
    const size_t d_off = align_up(fl_off + sizeof(int) * (size_t)(n + 4));
    const size_t e_off = align_up(d_off + sizeof(double) * (size_t)n);
    int rc = ensure_ws(h, align_up(e_off + sizeof(double) * (size_t)(n + 1)));
    if (rc != AVS_SUCCESS) return rc;
    cudaStream_t s = h->stream;
    int *err = reinterpret_cast<int *>(ws_at(h, L.off_err));
    AVS_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int), s));
    double *AB = reinterpret_cast<double *>(ws_at(h, ab_off));
    double *td = reinterpret_cast<double *>(ws_at(h, d_off));
    double *te = reinterpret_cast<double *>(ws_at(h, e_off));
    AVS_CUDA_TRY(cudaEventRecord(h->ev[0], s));
    if ((rc = dense_band_to_compact(dB, n, ldb, bw, AB, ldab, s)) != AVS_SUCCESS) return rc;
    Stage2Work w2;
    w2.flags = reinterpret_cast<int *>(ws_at(h, fl_off));
    w2.err = err;
    int64_t launches = 1;
    if ((rc = stage2_chase(AB, n, bw, ldab, td, te, w2, s, h->num_sms, &launches)) != AVS_SUCCESS) return rc;
    AVS_CUDA_TRY(cudaEventRecord(h->ev[1], s));
    AVS_CUDA_TRY(cudaMemcpyAsync(dd, td, sizeof(double) * (size_t)n, cudaMemcpyDeviceToDevice, s));
    if (n > 1)
        AVS_CUDA_TRY(cudaMemcpyAsync(de, te, sizeof(double) * (size_t)(n - 1), cudaMemcpyDeviceToDevice, s));
    AVS_CUDA_TRY(cudaMemcpyAsync(h->h_err, err, sizeof(int), cudaMemcpyDeviceToHost, s));
    rc = finish_status(h, s);
    if (rep) {
        rep->t_stage2_ms = rep->t_total_ms = ev_ms(h->ev[0], h->ev[1]);
        rep->kernel_launches = launches;
        rep->status = rc;
    }
    return rc;
}

int avs_band_reduce_dev_s(avs_handle *h, int64_t n, int32_t bw, int32_t tbw, float *dB, int64_t ldb,
                          avs_report *rep) {
    return band_reduce_dev<float>(h, n, bw, tbw, dB, ldb, rep);
}
int avs_band_reduce_dev_d(avs_handle *h, int64_t n, int32_t bw, int32_t tbw, double *dB, int64_t ldb,
                          avs_report *rep) {
    return band_reduce_dev<double>(h, n, bw, tbw, dB, ldb, rep);
}

int avs_bidiag_svals_dev(avs_handle *h, int64_t n, const double *dd, const double *de, double *dsigma,
                         double rel_tol, avs_report *rep) {
    if (!h) return -1;
    if (n < 0) return -2;
    if (n > 0 && !dd) return -3;
    if (n > 1 && !de) return -4;
    if (n > 0 && !dsigma) return -5;
    if (rep) std::memset(rep, 0, sizeof(*rep));
    if (n == 0) return AVS_SUCCESS;
    AVS_CUDA_TRY(cudaSetDevice(h->device));
    const Layout L = make_layout(n, 1, 8, 0);
    const size_t e_off = align_up(L.total);
    int rc = ensure_ws(h, align_up(e_off + sizeof(double) * (size_t)(n + 1)));
    if (rc != AVS_SUCCESS) return rc;
    cudaStream_t s = h->stream;
    // e may have n-1 entries; pad a private copy to n.
    double *te = reinterpret_cast<double *>(ws_at(h, e_off));
    AVS_CUDA_TRY(cudaMemsetAsync(te, 0, sizeof(double) * (size_t)(n + 1), s));
    if (n > 1) AVS_CUDA_TRY(cudaMemcpyAsync(te, de, sizeof(double) * (size_t)(n - 1), cudaMemcpyDeviceToDevice, s));
    int64_t launches = 0;
    AVS_CUDA_TRY(cudaEventRecord(h->ev[0], s));
    rc = stage3_bisect(dd, te, n, rel_tol, dsigma, reinterpret_cast<double *>(ws_at(h, L.off_scr)), s, &launches);
    if (rc != AVS_SUCCESS) return rc;
    AVS_CUDA_TRY(cudaEventRecord(h->ev[1], s));
    AVS_CUDA_TRY(cudaStreamSynchronize(s));
    if (rep) {
        rep->t_stage3_ms = rep->t_total_ms = ev_ms(h->ev[0], h->ev[1]);
        rep->kernel_launches = launches;
    }
    return AVS_SUCCESS;
}

int avs_bidiag_svals_noalloc(int64_t n, const double *dd, const double *de, double *dsigma, double rel_tol,
                             void *stream) {
    return bidiag_svals_noalloc(n, dd, de, dsigma, rel_tol, reinterpret_cast<cudaStream_t>(stream));
}

int avs_geqrt_tile_dev_s(avs_handle *h, int32_t b, float *dA, float *dtau) {
    return tile_kernel<float>(h, b, dA, nullptr, dtau, false);
}
int avs_geqrt_tile_dev_d(avs_handle *h, int32_t b, double *dA, double *dtau) {
    return tile_kernel<double>(h, b, dA, nullptr, dtau, false);
}
int avs_tsqrt_tile_dev_s(avs_handle *h, int32_t b, float *dR, float *dB, float *dtau) {
    return tile_kernel<float>(h, b, dR, dB, dtau, true);
}
int avs_tsqrt_tile_dev_d(avs_handle *h, int32_t b, double *dR, double *dB, double *dtau) {
    return tile_kernel<double>(h, b, dR, dB, dtau, true);
}

}  // extern "C"

// ===========================================================================
// Batched singular values (many independent matrices of mixed orders).
namespace {

struct BatchLayout {
    size_t err, W, tau, tblk, tfull, f1, ab, ab2, f2, d, e, sig, scr, pairs, ptrs, total;
};

// elem: bytes of the tile type (4: FP32 tiles and double-float stages 2-3;
// 8: FP64 throughout).  The band takes 8 bytes per entry either way.
BatchLayout batch_layout(int64_t n, int b, int cnt, size_t elem = 4) {
    BatchLayout L{};
    const int64_t nt = n / b;
    size_t o = 0;
    auto take = [&](size_t bytes) {
        const size_t at = o;
        o = align_up(o + bytes);
        return at;
    };
    L.err = take(64);
    L.W = take(elem * (size_t)cnt * n * n);
    L.tau = take(elem * (size_t)cnt * (nt + 1) * b);
    L.tblk = take(elem * (size_t)cnt * (nt + 1) * (b / 16) * 256);
    L.tfull = take(b >= 128 ? elem * (size_t)cnt * (nt + 1) * b * b : 0);
    L.f1 = take(sizeof(int) * (size_t)cnt * (2 * nt + 4));
    L.ab = take(sizeof(double) * (size_t)cnt * (size_t)band_stride(b, n));
    L.ab2 = take(sizeof(double) * (size_t)cnt * 3 * kMaxNarrowBand * n);  // narrow band of the hierarchical chase
    L.f2 = take(sizeof(int) * ((size_t)cnt * (n + 1) + 4));
    L.d = take(sizeof(double) * (size_t)cnt * n);
    L.e = take(sizeof(double) * (size_t)cnt * n);
    L.sig = take(sizeof(double) * (size_t)cnt * n);
    L.scr = take(sizeof(double) * (size_t)cnt * 4);
    L.pairs = take(sizeof(float2) * (size_t)cnt * 2 * n);
    L.ptrs = take(sizeof(void *) * 4 * (size_t)cnt + 64);
    L.total = o + 256;
    return L;
}

template <typename T>
__global__ void gather_kernel(const T *const *src, const int64_t *lds, T *dst, int64_t n) {
    const int64_t zb = blockIdx.y;
    const T *a = src[zb];
    const int64_t ld = lds[zb];
    T *w = dst + zb * n * n;
    for (int64_t c = blockIdx.x; c < n; c += gridDim.x)
        for (int64_t r = threadIdx.x; r < n; r += blockDim.x) w[r + c * n] = a[r + c * ld];
}

__global__ void scatter_de_kernel(const double *d, const double *e, double *const *dst_d, double *const *dst_e,
                                  int64_t n, int cnt) {
    const int64_t total = n * (int64_t)cnt;
    for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < total; g += (int64_t)gridDim.x * blockDim.x) {
        dst_d[g / n][g % n] = d[g];
        dst_e[g / n][g % n] = (g % n) + 1 < n ? e[g] : 0.0;
    }
}

template <typename T>
__global__ void scatter_kernel(const double *sig, T *const *dst, int64_t n, int cnt) {
    const int64_t total = n * (int64_t)cnt;
    for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < total; g += (int64_t)gridDim.x * blockDim.x)
        dst[g / n][g % n] = (T)sig[g];
}

int ensure_bws(avs_handle *h, size_t bytes) {
    if (h->bws_bytes >= bytes) return AVS_SUCCESS;
    cudaStreamSynchronize(h->stream);
    h->drop_graphs();  // graphs hold pointers into the old workspace
    if (h->bws) cudaFree(h->bws);
    h->bws = nullptr;
    h->bws_bytes = 0;
    cudaError_t e = cudaMalloc(&h->bws, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return AVS_ERR_OOM;
    }
    h->bws_bytes = bytes;
    return AVS_SUCCESS;
}

int ensure_pinned(avs_handle *h, size_t bytes) {
    if (h->pinned_bytes >= bytes) return AVS_SUCCESS;
    cudaStreamSynchronize(h->stream);
    if (h->pinned) cudaFreeHost(h->pinned);
    h->pinned = nullptr;
    h->pinned_bytes = 0;
    AVS_CUDA_TRY(cudaMallocHost(&h->pinned, bytes));
    h->pinned_bytes = bytes;
    return AVS_SUCCESS;
}

// The launches of one group (gather .. scatter), captured once per shape.
// T = float: FP32 tiles, double-float stages 2-3.  T = double: FP64 tiles;
// stages 2-3 in FP64 (f64_stages) or in double-float (AVS_PREC_FP64X2, as its
// single call).
template <typename T>
int group_launches(avs_handle *h, const BatchLayout &L, int64_t n, int b, int cnt, double tol, cudaStream_t s,
                   const cudaEvent_t *ev, int64_t *launches, bool bidiag, bool df_update, bool f64_stages,
                   int flags) {
    char *base = reinterpret_cast<char *>(h->bws);
    T *W = reinterpret_cast<T *>(base + L.W);
    const T *const *src = reinterpret_cast<const T *const *>(base + L.ptrs);
    T *const *dst = reinterpret_cast<T *const *>(base + L.ptrs + sizeof(void *) * cnt);
    const int64_t *lds = reinterpret_cast<const int64_t *>(base + L.ptrs + 2 * sizeof(void *) * cnt);
    double *const *dst_e = reinterpret_cast<double *const *>(base + L.ptrs + 3 * sizeof(void *) * cnt);
    int *err = reinterpret_cast<int *>(base + L.err);
    const int64_t nt = n / b;
    AVS_CUDA_TRY(cudaEventRecordWithFlags(ev[0], s, cudaEventRecordExternal));
    AVS_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int), s));
    gather_kernel<T><<<dim3((unsigned)std::min<int64_t>(n, 1024), (unsigned)cnt), 256, 0, s>>>(src, lds, W, n);
    AVS_CUDA_TRY(cudaGetLastError());
    Stage1Work w1;
    w1.tau = base + L.tau;
    w1.tblk = base + L.tblk;
    w1.tfull = b >= 128 ? base + L.tfull : nullptr;
    w1.flags = reinterpret_cast<int *>(base + L.f1);
    w1.err = err;
    w1.batch = cnt;
    w1.sA = n * n;
    w1.sTau = (nt + 1) * b;
    w1.sTblk = (nt + 1) * (b / 16) * 256;
    w1.sTfull = (nt + 1) * (int64_t)b * b;
    w1.sFlags = 2 * nt + 4;
    w1.df_update = (sizeof(T) == 8 && df_update) ? 1 : 0;
    int rc = stage1_ge2bnd<T>(W, n, n, b, w1, s, launches);
    if (rc != AVS_SUCCESS) return rc;
    AVS_CUDA_TRY(cudaEventRecordWithFlags(ev[1], s, cudaEventRecordExternal));
    Stage2Work w2;
    w2.flags = reinterpret_cast<int *>(base + L.f2);
    w2.err = err;
    double *dd = reinterpret_cast<double *>(base + L.d);
    double *de = reinterpret_cast<double *>(base + L.e);
    // stage 2 as a single call of the same mode runs it (run_stages23)
    const int tbw = narrow_band_of(b, flags, sizeof(T) == 8 && f64_stages);
    const bool window = !(flags & AVS_FLAG_CLUSTER_CHASE);
    if constexpr (sizeof(T) == 8) {
        if (f64_stages)
            rc = stage2_chase_fp64_batched(W, n, b, cnt, reinterpret_cast<double *>(base + L.ab), 3 * (int64_t)b, dd,
                                           de, w2, s, h->num_sms, launches, tbw, window,
                                           reinterpret_cast<double *>(base + L.ab2));
        else
            rc = stage2_chase_df_batched(W, n, b, cnt, reinterpret_cast<float2 *>(base + L.ab), 3 * (int64_t)b, dd,
                                         de, w2, s, h->num_sms, launches, window);
    } else {
        rc = stage2_chase_df_batched(W, n, b, cnt, reinterpret_cast<float2 *>(base + L.ab), 3 * (int64_t)b, dd, de,
                                     w2, s, h->num_sms, launches, tbw, window, reinterpret_cast<float2 *>(base + L.ab2));
    }
    if (rc != AVS_SUCCESS) return rc;
    AVS_CUDA_TRY(cudaEventRecordWithFlags(ev[2], s, cudaEventRecordExternal));
    if (bidiag) {  // the bidiagonal itself: d and e of each matrix to the caller's vectors
        scatter_de_kernel<<<(unsigned)std::min<int64_t>((n * cnt + 255) / 256, 8192), 256, 0, s>>>(
            dd, de, reinterpret_cast<double *const *>(dst), dst_e, n, cnt);
        AVS_CUDA_TRY(cudaGetLastError());
        AVS_CUDA_TRY(cudaEventRecordWithFlags(ev[3], s, cudaEventRecordExternal));
        if (launches) *launches += 2;
        return AVS_SUCCESS;
    }
    double *sig = reinterpret_cast<double *>(base + L.sig);
    if (sizeof(T) == 8 && f64_stages)
        rc = stage3_bisect_batched(dd, de, n, cnt, tol, sig, reinterpret_cast<double *>(base + L.scr), s, launches);
    else
        rc = stage3_bisect_df_batched(dd, de, n, cnt, tol, sig, reinterpret_cast<double *>(base + L.scr),
                                      reinterpret_cast<float2 *>(base + L.pairs), s, launches);
    if (rc != AVS_SUCCESS) return rc;
    scatter_kernel<T><<<(unsigned)std::min<int64_t>((n * cnt + 255) / 256, 8192), 256, 0, s>>>(sig, dst, n, cnt);
    AVS_CUDA_TRY(cudaGetLastError());
    AVS_CUDA_TRY(cudaEventRecordWithFlags(ev[3], s, cudaEventRecordExternal));
    if (launches) *launches += 2;
    return AVS_SUCCESS;
}

// Seeded N(0,1)-like fill for the autotuner's sample matrices (sum of four
// uniforms from a 32-bit integer hash; the distribution only needs to be generic).
__global__ void fill_sample_kernel(float *a, int64_t count, uint32_t seed) {
    for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < count; g += (int64_t)gridDim.x * blockDim.x) {
        float acc = 0.f;
        for (uint32_t k = 0; k < 4; ++k) {
            uint32_t x = (uint32_t)g * 4u + k + seed * 0x9E3779B9u;
            x ^= x >> 16;
            x *= 0x7feb352dU;
            x ^= x >> 15;
            x *= 0x846ca68bU;
            x ^= x >> 16;
            acc += (float)(x >> 8) * (1.0f / 16777216.0f);
        }
        a[g] = (acc - 2.0f) * 1.7320508f;
    }
}

bool valid_tile(int64_t n, int t) { return is_pow2(t) && t >= 16 && t <= kMaxTile && n % t == 0 && t <= n; }

}  // namespace

// Batched calls: out1 = sigma (type T) or d (FP64), out2 = e (FP64, bidiagonal form only).
template <typename T>
static int batched_call(avs_handle *h, int32_t count, const int64_t *n, const int64_t *lda, const int32_t *tile,
                        const T *const *dA, void *const *out1, void *const *out2, bool bidiag,
                        const avs_opts *opts, avs_report *rep) {
    void *const *dsigma = out1;
    if (rep) std::memset(rep, 0, sizeof(*rep));
    if (!h) return -1;
    if (count < 0) return -2;
    if (count == 0) return AVS_SUCCESS;
    if (!n) return -3;
    if (!lda) return -4;
    if (!dA) return -6;
    if (!dsigma) return -7;
    if (bidiag && !out2) return -8;
    std::vector<int> tiles(count);
    for (int i = 0; i < count; ++i) {
        if (n[i] < 0) return -3;
        if (lda[i] < (n[i] > 1 ? n[i] : 1)) return -4;
        const int t = tile ? tile[i] : 0;
        if (t != 0 && !valid_tile(n[i], t)) return (t > kMaxTile && is_pow2(t)) ? AVS_ERR_UNSUPPORTED
                                                                                : AVS_ERR_NOT_IMPLEMENTED;
        if (n[i] > 0 && (!dA[i] || !dsigma[i])) return dA[i] ? -7 : -6;
        if (bidiag && n[i] > 0 && !out2[i]) return -8;
        tiles[i] = t;
    }
    AVS_CUDA_TRY(cudaSetDevice(h->device));
    // tiles left to the autotuner
    for (int i = 0; i < count; ++i) {
        if (tiles[i] != 0 || n[i] == 0) continue;
        auto it = h->tuned.find(n[i]);
        if (it == h->tuned.end()) {
            int rc = avs_autotune_tile(h, n[i], 16, nullptr);
            if (rc != AVS_SUCCESS) return rc;
            it = h->tuned.find(n[i]);
        }
        tiles[i] = it->second;
    }
    // groups of equal (n, tile)
    std::map<std::pair<int64_t, int>, std::vector<int>> groups;
    for (int i = 0; i < count; ++i)
        if (n[i] > 0) groups[{n[i], tiles[i]}].push_back(i);
    size_t need = 0;
    size_t pin_need = sizeof(int) * 16 * (groups.size() + 1);
    for (auto &g : groups) {
        need = std::max(need, batch_layout(g.first.first, g.first.second, (int)g.second.size(), sizeof(T)).total);
        pin_need += sizeof(void *) * 4 * g.second.size();
    }
    int rc;
    if ((rc = ensure_bws(h, need)) != AVS_SUCCESS) return rc;
    if ((rc = ensure_pinned(h, pin_need)) != AVS_SUCCESS) return rc;
    if (h->graphs.size() > 256) h->drop_graphs();  // bound the cache of group shapes
    cudaStream_t s = h->stream;  // graphs are captured and replayed on the handle's stream
    if (opts && opts->stream) {  // order after the caller's work on its stream
        AVS_CUDA_TRY(cudaEventRecord(h->ev[4], reinterpret_cast<cudaStream_t>(opts->stream)));
        AVS_CUDA_TRY(cudaStreamWaitEvent(s, h->ev[4], 0));
    }
    // FP64 groups: AVS_PREC_FP64X2 takes the double-float trailing updates and
    // double-float stages 2-3 (FP64 stages on AVS_FLAG_FP64_STAGES), as its single call
    const bool dfu = sizeof(T) == 8 && opts && df_update_of(opts->precision);
    const bool f64s = sizeof(T) == 8 && (!dfu || (opts->flags & AVS_FLAG_FP64_STAGES));
    const double tol = bisect_tol(f64s, sizeof(T) == 4, opts);
    // pinned layout: one status word per group (16 ints apart), then the pointer tables
    int *h_status = reinterpret_cast<int *>(h->pinned);
    void **tab = reinterpret_cast<void **>(h_status + 16 * (groups.size() + 1));
    AVS_CUDA_TRY(cudaEventRecord(h->ev[0], s));
    int64_t launches = 0;
    size_t gi = 0;
    std::vector<const avs_handle::Graph *> ran;
    for (auto &g : groups) {
        const int64_t gn = g.first.first;
        const int gb = g.first.second;
        const int cnt = (int)g.second.size();
        const BatchLayout L = batch_layout(gn, gb, cnt, sizeof(T));
        NvtxRange range("avs batched group");
        // pointer tables: sources, destinations, leading dimensions
        for (int q = 0; q < cnt; ++q) {
            tab[q] = const_cast<T *>(dA[g.second[q]]);
            tab[cnt + q] = dsigma[g.second[q]];
            tab[3 * cnt + q] = bidiag ? out2[g.second[q]] : nullptr;
            reinterpret_cast<int64_t *>(tab + 2 * cnt)[q] = lda[g.second[q]];
        }
        AVS_CUDA_TRY(cudaMemcpyAsync(reinterpret_cast<char *>(h->bws) + L.ptrs, tab, sizeof(void *) * 4 * cnt,
                                     cudaMemcpyHostToDevice, s));
        const int cflags = flags_of(opts) & (AVS_FLAG_ONE_STAGE_CHASE | AVS_FLAG_BAND32 | AVS_FLAG_CLUSTER_CHASE |
                                             AVS_FLAG_HIER_CHASE);
        const auto key = std::make_tuple(gn, gb, cnt,
                                         (bidiag ? 1 : 0) + (sizeof(T) == 8 ? 2 : 0) + (dfu ? 4 : 0) + (f64s ? 8 : 0) +
                                             (cflags << 4));
        auto it = h->graphs.find(key);
        if (it == h->graphs.end()) {
            avs_handle::Graph gr;
            for (cudaEvent_t &e : gr.ev) AVS_CUDA_TRY(cudaEventCreate(&e));
            cudaGraph_t graph;
            AVS_CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
            rc = group_launches<T>(h, L, gn, gb, cnt, tol, s, gr.ev, &gr.kernels, bidiag, dfu, f64s, cflags);
            cudaError_t ce = cudaStreamEndCapture(s, &graph);
            if (rc == AVS_SUCCESS && ce == cudaSuccess) {
                ce = cudaGraphInstantiate(&gr.exec, graph, 0);
                cudaGraphDestroy(graph);
            }
            if (rc != AVS_SUCCESS || ce != cudaSuccess) {
                for (cudaEvent_t e : gr.ev) cudaEventDestroy(e);
                if (rc != AVS_SUCCESS) return rc;
                AVS_CUDA_TRY(ce);
            }
            it = h->graphs.emplace(key, gr).first;
        }
        AVS_CUDA_TRY(cudaGraphLaunch(it->second.exec, s));
        launches += it->second.kernels;
        ran.push_back(&it->second);
        AVS_CUDA_TRY(cudaMemcpyAsync(h_status + 16 * gi, reinterpret_cast<char *>(h->bws) + L.err, sizeof(int),
                                     cudaMemcpyDeviceToHost, s));
        tab += 4 * cnt;
        ++gi;
    }
    AVS_CUDA_TRY(cudaEventRecord(h->ev[1], s));
    {
        cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            set_last_cuda_error(e);
            return AVS_ERR_CUDA;
        }
    }
    rc = AVS_SUCCESS;
    for (size_t q = 0; q < gi && rc == AVS_SUCCESS; ++q) {
        const int dev_err = h_status[16 * q];
        if (dev_err == kDevTimeout) rc = AVS_ERR_TIMEOUT;
        else if (dev_err == kDevNonfinite) rc = AVS_ERR_NONFINITE;
        else if (dev_err != kDevOk) rc = AVS_ERR_INTERNAL;
    }
    if (rep) {
        rep->t_total_ms = ev_ms(h->ev[0], h->ev[1]);
        for (const avs_handle::Graph *g : ran) {
            rep->t_stage1_ms += ev_ms(g->ev[0], g->ev[1]);
            rep->t_stage2_ms += ev_ms(g->ev[1], g->ev[2]);
            rep->t_stage3_ms += ev_ms(g->ev[2], g->ev[3]);
        }
        rep->kernel_launches = launches;
        rep->workspace_bytes = (int64_t)h->bws_bytes;
        rep->precision = sizeof(T) == 8 ? (dfu ? AVS_PREC_FP64X2 : AVS_PREC_FP64) : AVS_PREC_FP32;
        rep->status = rc;
    }
    return rc;
}

extern "C" int avs_svdvals_batched_dev_s(avs_handle *h, int32_t count, const int64_t *n, const int64_t *lda,
                                         const int32_t *tile, const float *const *dA, float *const *dsigma,
                                         const avs_opts *opts, avs_report *rep) {
    return batched_call(h, count, n, lda, tile, dA, reinterpret_cast<void *const *>(dsigma), nullptr, false, opts,
                        rep);
}

extern "C" int avs_bidiag_batched_dev_s(avs_handle *h, int32_t count, const int64_t *n, const int64_t *lda,
                                        const int32_t *tile, const float *const *dA, double *const *dd,
                                        double *const *de, const avs_opts *opts, avs_report *rep) {
    return batched_call(h, count, n, lda, tile, dA, reinterpret_cast<void *const *>(dd),
                        reinterpret_cast<void *const *>(de), true, opts, rep);
}

extern "C" int avs_svdvals_batched_dev_d(avs_handle *h, int32_t count, const int64_t *n, const int64_t *lda,
                                         const int32_t *tile, const double *const *dA, double *const *dsigma,
                                         const avs_opts *opts, avs_report *rep) {
    return batched_call(h, count, n, lda, tile, dA, reinterpret_cast<void *const *>(dsigma), nullptr, false, opts,
                        rep);
}

extern "C" int avs_bidiag_batched_dev_d(avs_handle *h, int32_t count, const int64_t *n, const int64_t *lda,
                                        const int32_t *tile, const double *const *dA, double *const *dd,
                                        double *const *de, const avs_opts *opts, avs_report *rep) {
    return batched_call(h, count, n, lda, tile, dA, reinterpret_cast<void *const *>(dd),
                        reinterpret_cast<void *const *>(de), true, opts, rep);
}

// Autotuner: time each valid tile in {32, 64, 128} on `sample` seeded random
// matrices of order n through the batched path; keep the fastest.
extern "C" int avs_autotune_tile(avs_handle *h, int64_t n, int32_t sample, int32_t *best) {
    if (!h) return -1;
    if (n <= 0) return -2;
    if (sample <= 0) sample = 16;
    const int cands[3] = {32, 64, 128};
    std::vector<int> valid;
    for (int t : cands)
        if (valid_tile(n, t) && n / t >= 2) valid.push_back(t);
    if (valid.empty())
        for (int t : {16, 32, 64, 128, 256})
            if (valid_tile(n, t)) { valid.push_back(t); break; }
    if (valid.empty()) return AVS_ERR_NOT_IMPLEMENTED;
    AVS_CUDA_TRY(cudaSetDevice(h->device));
    float *A = nullptr, *S = nullptr;
    AVS_CUDA_TRY(cudaMalloc(&A, sizeof(float) * (size_t)sample * n * n));
    if (cudaMalloc(&S, sizeof(float) * (size_t)sample * n) != cudaSuccess) {
        cudaFree(A);
        return AVS_ERR_OOM;
    }
    fill_sample_kernel<<<1024, 256, 0, h->stream>>>(A, (int64_t)sample * n * n, 7u);
    std::vector<const float *> pa(sample);
    std::vector<float *> ps(sample);
    std::vector<int64_t> nn(sample, n), ll(sample, n);
    for (int i = 0; i < sample; ++i) {
        pa[i] = A + (size_t)i * n * n;
        ps[i] = S + (size_t)i * n;
    }
    int bt = valid[0];
    float bestms = 1e30f;
    int rc = AVS_SUCCESS;
    for (int t : valid) {
        std::vector<int32_t> tt(sample, t);
        avs_report r;
        for (int rep = 0; rep < 2 && rc == AVS_SUCCESS; ++rep)  // first call captures the graph
            rc = avs_svdvals_batched_dev_s(h, sample, nn.data(), ll.data(), tt.data(), pa.data(), ps.data(), nullptr,
                                           &r);
        if (rc != AVS_SUCCESS) break;
        if (r.t_total_ms < bestms) {
            bestms = (float)r.t_total_ms;
            bt = t;
        }
    }
    cudaFree(A);
    cudaFree(S);
    if (rc != AVS_SUCCESS) return rc;
    h->tuned[n] = bt;
    if (best) *best = bt;
    return AVS_SUCCESS;
}

// ===========================================================================
// Failure path check: one thread waits, with a short bound, on a flag that
// nothing sets -- the wait every cross-CTA dependency of the library uses.
namespace {
__global__ void timeout_probe_kernel(const int *flag, int *err, long long limit) {
    if (threadIdx.x == 0 && blockIdx.x == 0) wait_geq_n(flag, 1, err, limit);
}
}  // namespace

extern "C" int avs_selftest_timeout(avs_handle *h) {
    if (!h) return -1;
    AVS_CUDA_TRY(cudaSetDevice(h->device));
    int rc = ensure_ws(h, 256);
    if (rc != AVS_SUCCESS) return rc;
    cudaStream_t s = h->stream;
    int *err = reinterpret_cast<int *>(h->ws);
    int *flag = err + 16;
    AVS_CUDA_TRY(cudaMemsetAsync(h->ws, 0, 256, s));
    timeout_probe_kernel<<<1, 32, 0, s>>>(flag, err, 100000000ll);  // 100 ms
    AVS_CUDA_TRY(cudaGetLastError());
    AVS_CUDA_TRY(cudaMemcpyAsync(h->h_err, err, sizeof(int), cudaMemcpyDeviceToHost, s));
    return finish_status(h, s);
}

// Architecture the library's kernels were built for, read back from the loaded
// image by the runtime (binaryVersion 103 = sm_103).
extern "C" int avs_kernel_arch(int device, int32_t *binary_version, int32_t *ptx_version) {
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count <= 0) {
        cudaGetLastError();
        return AVS_ERR_NO_DEVICE;
    }
    if (device < 0 || device >= count) return -1;
    AVS_CUDA_TRY(cudaSetDevice(device));
    cudaFuncAttributes fa{};
    AVS_CUDA_TRY(cudaFuncGetAttributes(&fa, timeout_probe_kernel));
    if (binary_version) *binary_version = fa.binaryVersion;
    if (ptx_version) *ptx_version = fa.ptxVersion;
    return AVS_SUCCESS;
}

// Compute roof of the bulge chase on `device`: flops/s of its inner arithmetic
// (double-float, or FP64 with fp64 != 0) with every SM busy and no memory traffic.
extern "C" int avs_measure_chase_rate(int device, int32_t fp64, double *flops_per_s) {
    if (!flops_per_s) return -3;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count <= 0) {
        cudaGetLastError();
        return AVS_ERR_NO_DEVICE;
    }
    if (device < 0 || device >= count) return -1;
    AVS_CUDA_TRY(cudaSetDevice(device));
    int sms = 0;
    AVS_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    return stage2_rate(fp64, sms, flops_per_s);
}

// ===========================================================================
// Memory accounting helpers (used by admission control of the serving loop).
extern "C" int avs_trim(avs_handle *h) {
    if (!h) return -1;
    AVS_CUDA_TRY(cudaSetDevice(h->device));
    AVS_CUDA_TRY(cudaStreamSynchronize(h->stream));
    h->drop_graphs();
    if (h->ws) cudaFree(h->ws);
    if (h->bws) cudaFree(h->bws);
    if (h->pinned) cudaFreeHost(h->pinned);
    h->ws = h->bws = h->pinned = nullptr;
    h->ws_bytes = h->bws_bytes = h->pinned_bytes = 0;
    return AVS_SUCCESS;
}

extern "C" int avs_workspace_bytes(avs_handle *h, int64_t *single_bytes, int64_t *batched_bytes) {
    if (!h) return -1;
    if (single_bytes) *single_bytes = (int64_t)h->ws_bytes;
    if (batched_bytes) *batched_bytes = (int64_t)h->bws_bytes;
    return AVS_SUCCESS;
}

extern "C" int avs_estimate_bytes(int64_t n, int32_t tile, int32_t precision, int32_t count, int64_t *bytes) {
    if (n < 0) return -1;
    if (!is_pow2(tile) || tile < 16 || (n > 0 && n % tile != 0) || tile > n) return AVS_ERR_NOT_IMPLEMENTED;
    if (tile > kMaxTile) return AVS_ERR_UNSUPPORTED;
    if (count < 0) return -4;
    if (!bytes) return -5;
    if (count >= 1) {  // batched group: FP64 tiles for AVS_PREC_FP64, FP32 otherwise
        *bytes = (int64_t)batch_layout(n, tile, count, precision == AVS_PREC_FP64 ? 8 : 4).total;
        return AVS_SUCCESS;
    }
    const int prec = resolve_precision(precision, true);
    const size_t elem = storage_elem(prec);
    if (elem == 0) return AVS_ERR_UNSUPPORTED;
    *bytes = (int64_t)make_layout(n, tile, elem, elem, tc_split_of(prec, tile)).total;
    return AVS_SUCCESS;
}
