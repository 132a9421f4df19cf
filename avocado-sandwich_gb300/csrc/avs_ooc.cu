// Out-of-core GE2BND and tiled QR: the matrix stays in host memory and passes
// through the GPU in slabs.  This is the GB300 form of the reference's
// OOC_alg! / OOC_Bidiag! / OOC_QR! (KAbasedSVD/src/tiledalgos.jl:232-251) over
// LargeTiledMatrix (TiledMatrix.jl:121-186), which streams one tile row at a
// time through three device tile-row buffers and finishes the last kswitch
// tiles in device memory.
//
// A QR half-step k touches tile rows k..nt-1 of columns kb..n-1.  The top tile
// row k stays on the device for the whole half-step; the tile rows below it
// come in slabs of `slab` tile rows.  Each slab buffer holds [top row; slab
// rows] as one column-major matrix, so the in-core panel kernel (GEQRT on the
// first slab, TSQRT roles 1..slab after it) and the in-core trailing update
// (full-T for tiles >= 128, 16-reflector blocks below) run on it unchanged; the
// top row is carried to the next slab buffer by a device copy.  The flat-tree
// order of the TSQRTs and the update kernels are the in-core ones, so the
// result is the in-core SIMT result bit for bit.  An LQ half-step is the same
// on tile columns (the kernels' transposed view of the buffer).  Once the
// trailing block fits in the slab memory it is copied in, finished by the
// in-core driver and copied back.
#include <algorithm>
#include <utility>

#include "avs_common.cuh"

namespace avs {
namespace {

inline size_t al256(size_t x) { return (x + 255) & ~size_t(255); }

struct OocBufs {
    void *tau, *tblk, *tfull;
    int *flags;
    char *X[2];      // slab buffers
    char *region;    // both slab buffers as one region (the in-core tail)
    size_t region_bytes;
};

OocBufs carve(void *ws, int64_t n, int b, size_t elem, int slab) {
    const int64_t nt = n / b;
    OocBufs o{};
    char *p = static_cast<char *>(ws);
    size_t off = 0;
    o.tau = p + off;
    off = al256(off + elem * (size_t)(nt + 1) * b);
    o.tblk = p + off;
    off = al256(off + elem * (size_t)(nt + 1) * (b / 16) * 256);
    o.tfull = b >= 128 ? p + off : nullptr;
    off = al256(off + (b >= 128 ? elem * (size_t)(nt + 1) * b * b : 0));
    o.flags = reinterpret_cast<int *>(p + off);
    off = al256(off + sizeof(int) * (size_t)(2 * nt + 4));
    const size_t sb = al256(elem * (size_t)(1 + slab) * b * n);
    o.region = p + off;
    o.X[0] = p + off;
    o.X[1] = p + off + sb;
    o.region_bytes = 2 * sb;
    return o;
}

size_t fixed_bytes(int64_t n, int b, size_t elem) {
    const int64_t nt = n / b;
    return al256(elem * (size_t)(nt + 1) * b) + al256(elem * (size_t)(nt + 1) * (b / 16) * 256) +
           al256(b >= 128 ? elem * (size_t)(nt + 1) * b * b : 0) + al256(sizeof(int) * (size_t)(2 * nt + 4)) + 256;
}

// cudaMemcpy2DAsync of `height` runs of `width` elements
template <typename T>
int copy2d(T *dst, int64_t dld, const T *src, int64_t sld, int64_t width, int64_t height, cudaMemcpyKind kind,
           cudaStream_t s, double *bytes) {
    if (width <= 0 || height <= 0) return AVS_SUCCESS;
    AVS_CUDA_TRY(cudaMemcpy2DAsync(dst, sizeof(T) * (size_t)dld, src, sizeof(T) * (size_t)sld,
                                   sizeof(T) * (size_t)width, (size_t)height, kind, s));
    if (bytes) *bytes += (double)sizeof(T) * (double)width * (double)height;
    return AVS_SUCCESS;
}

// One half-step through slab buffers.  layout 0 (QR, tile rows of the block
// rows r0.., columns c0..n-1) or 1 (LQ, tile columns of the block columns c0..,
// rows r0..n-1).  `tiles` tiles in the panel; the top tile is tile 0.  tau of
// role p goes to tau_host + p*b (QR only).
template <typename T>
int half_step(T *A, int64_t n, int64_t lda, int b, int layout, int64_t r0, int64_t c0, int tiles, int slab,
              const OocBufs &ob, const Stage1Work &w, T *tau_host, cudaStream_t s, OocStats *st) {
    // the block: QR: rows r0 + [0, tiles*b), columns c0..n-1 (m columns);
    //            LQ: columns c0 + [0, tiles*b), rows r0..n-1 (m rows)
    const int64_t m = layout == 0 ? n - c0 : n - r0;
    const int64_t ld = layout == 0 ? (int64_t)(1 + slab) * b : m;
    T *X[2] = {reinterpret_cast<T *>(ob.X[0]), reinterpret_cast<T *>(ob.X[1])};
    double *up = st ? &st->h2d_bytes : nullptr;
    double *down = st ? &st->d2h_bytes : nullptr;
    // host address of tile t of the panel (row offset q within it) and the
    // buffer address of buffer tile u
    auto host_at = [&](int t) -> T * {
        return layout == 0 ? A + (r0 + (int64_t)t * b) + c0 * lda : A + r0 + (c0 + (int64_t)t * b) * lda;
    };
    auto buf_at = [&](T *x, int u) -> T * { return layout == 0 ? x + (int64_t)u * b : x + (int64_t)u * b * ld; };
    // tiles [u0, u0 + cnt) of buffer x  <->  panel tiles [t0, t0 + cnt)
    auto move = [&](T *x, int u0, int t0, int cnt, bool in) -> int {
        const int64_t rows = (int64_t)cnt * b;
        if (layout == 0) {
            return in ? copy2d<T>(buf_at(x, u0), ld, host_at(t0), lda, rows, m, cudaMemcpyHostToDevice, s, up)
                      : copy2d<T>(host_at(t0), lda, buf_at(x, u0), ld, rows, m, cudaMemcpyDeviceToHost, s, down);
        }
        return in ? copy2d<T>(buf_at(x, u0), ld, host_at(t0), lda, m, rows, cudaMemcpyHostToDevice, s, up)
                  : copy2d<T>(host_at(t0), lda, buf_at(x, u0), ld, m, rows, cudaMemcpyDeviceToHost, s, down);
    };
    int rc;
    int cur = 0, done = 0;  // tiles below the top already through
    int first = std::min(slab, tiles - 1);
    if ((rc = move(X[0], 0, 0, 1 + first, true)) != AVS_SUCCESS) return rc;
    for (bool lead = true;; lead = false) {
        const int cnt = lead ? first : std::min(slab, tiles - 1 - done);
        const int P = 1 + cnt;
        const int fr = lead ? 0 : 1;
        if ((rc = stage1_panel<T>(X[cur], ld, b, layout, 0, 0, P, fr, w, s)) != AVS_SUCCESS) return rc;
        if ((rc = stage1_update<T>(X[cur], ld, m, b, layout, 0, 0, P, fr, w, s)) != AVS_SUCCESS) return rc;
        if (st) st->launches += 2, ++st->slabs;
        if (tau_host)
            AVS_CUDA_TRY(cudaMemcpyAsync(tau_host + (size_t)(lead ? 0 : 1 + done) * b,
                                         static_cast<T *>(w.tau) + (size_t)fr * b, sizeof(T) * (size_t)(P - fr) * b,
                                         cudaMemcpyDeviceToHost, s));
        // the slab's own tiles go home; the top tile moves on
        if ((rc = move(X[cur], 1, 1 + done, cnt, false)) != AVS_SUCCESS) return rc;
        done += cnt;
        if (done >= tiles - 1) break;
        const int nx = 1 - cur;
        if (layout == 0) rc = copy2d<T>(X[nx], ld, X[cur], ld, b, m, cudaMemcpyDeviceToDevice, s, nullptr);
        else rc = copy2d<T>(X[nx], ld, X[cur], ld, m, b, cudaMemcpyDeviceToDevice, s, nullptr);
        if (rc != AVS_SUCCESS) return rc;
        if ((rc = move(X[nx], 1, 1 + done, std::min(slab, tiles - 1 - done), true)) != AVS_SUCCESS) return rc;
        cur = nx;
    }
    return move(X[cur], 0, 0, 1, false);
}

}  // namespace

OocPlan ooc_plan(int64_t n, int b, size_t elem, size_t budget) {
    OocPlan p{};
    const int64_t nt = n / b;
    const size_t fixed = fixed_bytes(n, b, elem);
    const size_t per_tile = 2 * elem * (size_t)b * (size_t)n;  // one tile row in each slab buffer
    if (budget <= fixed + 2 * per_tile) return p;             // not even a top tile and one slab tile
    int64_t slab = (int64_t)((budget - fixed) / per_tile) - 1;
    slab = std::max<int64_t>(1, std::min<int64_t>(slab, std::max<int64_t>(1, nt - 1)));
    p.slab = (int)slab;
    p.slab_bytes = al256(elem * (size_t)(1 + slab) * b * n);
    p.bytes = fixed + 2 * p.slab_bytes;
    return p;
}

template <typename T>
int ooc_ge2bnd(T *A, int64_t n, int64_t lda, int b, bool qr_only, T *tau_host, const OocPlan &plan, void *dws,
               int *err, cudaStream_t s, OocStats *st) {
    if (plan.slab < 1) return AVS_ERR_OOM;
    const int nt = (int)(n / b);
    const OocBufs ob = carve(dws, n, b, sizeof(T), plan.slab);
    Stage1Work w;
    w.tau = ob.tau;
    w.tblk = ob.tblk;
    w.flags = ob.flags;
    w.err = err;
    w.tfull = ob.tfull;  // full-T updates for tiles >= 128, as in core
    int rc;
    for (int k = 0; k < nt; ++k) {
        const int64_t kb = (int64_t)k * b, m = n - kb;
        const int ntt = nt - k;
        // the trailing block (and, for QR, its tau) fits: finish it in core
        const size_t need = sizeof(T) * ((size_t)m * m + (qr_only && tau_host ? (size_t)ntt * ntt * b : 0));
        if (need <= ob.region_bytes) {
            T *X = reinterpret_cast<T *>(ob.region);
            T *dtau = reinterpret_cast<T *>(ob.region) + (size_t)m * m;
            if ((rc = copy2d<T>(X, m, A + kb + kb * lda, lda, m, m, cudaMemcpyHostToDevice, s,
                                st ? &st->h2d_bytes : nullptr)) != AVS_SUCCESS)
                return rc;
            int64_t launches = 0;
            if (qr_only) rc = stage1_geqrf<T>(X, m, m, b, w, tau_host ? dtau : nullptr, s, &launches);
            else rc = stage1_ge2bnd<T>(X, m, m, b, w, s, &launches);
            if (rc != AVS_SUCCESS) return rc;
            if (qr_only && tau_host) {
                for (int q = 0; q < ntt; ++q)  // tail panel q -> panel k + q, tile rows k + q..
                    AVS_CUDA_TRY(cudaMemcpyAsync(tau_host + ((size_t)(k + q) * nt + k + q) * b,
                                                 dtau + ((size_t)q * ntt + q) * b, sizeof(T) * (size_t)(ntt - q) * b,
                                                 cudaMemcpyDeviceToHost, s));
            }
            if ((rc = copy2d<T>(A + kb + kb * lda, lda, X, m, m, m, cudaMemcpyDeviceToHost, s,
                                st ? &st->d2h_bytes : nullptr)) != AVS_SUCCESS)
                return rc;
            if (st) {
                st->launches += launches;
                st->incore_from = k;
            }
            return AVS_SUCCESS;
        }
        // QR half-step k: tile rows k..nt-1 of tile column k
        if ((rc = half_step<T>(A, n, lda, b, 0, kb, kb, ntt, plan.slab, ob, w,
                               tau_host ? tau_host + ((size_t)k * nt + k) * b : nullptr, s, st)) != AVS_SUCCESS)
            return rc;
        if (qr_only || k == nt - 1) continue;
        // LQ half-step k: tile columns k+1..nt-1 of tile row k
        if ((rc = half_step<T>(A, n, lda, b, 1, kb, kb + b, ntt - 1, plan.slab, ob, w, nullptr, s, st)) !=
            AVS_SUCCESS)
            return rc;
    }
    return AVS_SUCCESS;
}

template int ooc_ge2bnd<float>(float *, int64_t, int64_t, int, bool, float *, const OocPlan &, void *, int *,
                               cudaStream_t, OocStats *);
template int ooc_ge2bnd<double>(double *, int64_t, int64_t, int, bool, double *, const OocPlan &, void *, int *,
                                cudaStream_t, OocStats *);

}  // namespace avs
