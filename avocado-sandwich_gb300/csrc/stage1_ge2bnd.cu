// Stage 1: tile QR/LQ block-bidiagonalisation (GE2BND), FP64 and FP32 tiles.
//
// Reference: Blockbidiag! (KAbasedSVD/src/tiledalgos.jl:17-59) on the tile
// views of KAbasedSVD/src/TiledMatrix.jl:77-113, with the GEQRT / TSQRT tile
// kernels of KAbasedSVD/src/QRkernels.jl:3-129 and the reflector applies of
// QRkernels.jl:131-197.
//
// Each GE2BND step k is two half-steps, both written as "QR of a column panel
// plus left-apply to the trailing columns" on a view of the matrix:
//   QR half: view = A,   top tile row pr = k,   panel column tile pc = k
//   LQ half: view = A^T, top tile row pr = k+1, panel column tile pc = k
// (the reference runs the LQ half as QR kernels on adjoint views,
//  TiledMatrix.jl:85-88, 98-102).
//
// Panel kernel.  Role 0 runs GEQRT on the top tile; role p >= 1 runs TSQRT on
// [R; tile p], exactly the flat tree of the reference.  Reflectors of
// different roles that touch different rows commute, so role p may process
// its column block cb as soon as role p-1 has finished block cb: the roles form
// a systolic pipeline over the row tiles whose critical path is
// (#tiles + b/16) block steps instead of #tiles * b reflector steps.  Within a
// block the 16 reflectors are generated one column at a time, their
// compact-WY factor T (16 x 16) is formed, and the block is applied to the rest
// of the tile with it.  A role hands block cb on in two parts: the 16 x 16
// diagonal block of the top rows right after its reflectors (all the next
// role's reflectors read), and the trailing top rows after its apply (which the
// next role reads only in its own apply), so the step between roles is one
// reflector loop.  Roles are handed out by an atomic ticket in launch order,
// so a role only ever waits on a role already running: no co-residency
// assumption, and every wait is bounded.  The panel computes in its tile type,
// except with the double-float trailing updates of FP64 tiles (AVS_PREC_FP64X2),
// where it computes in double-float too (FP64 storage).  In the lookahead of the
// tensor-core path (stage1_ge2bnd_tc) a role may also wait for its own tile,
// which the previous update's chain finishes on the other stream.
//
// Trailing update kernel.  One CTA owns a column strip of the trailing matrix,
// keeps the strip of the top tile row in shared memory, and applies the GEQRT
// blocks and then, row tile by row tile, the TSQRT blocks (compact WY per 16
// reflectors) -- the serial order of the reference's Qtapply1_par! /
// Qtapply2_par! (TiledMatrix.jl:107-113) per column, all columns in parallel.
//
// Householder vectors stay where the reference leaves them before it zeroes
// them (tiledalgos.jl:40,46,52,58); later stages read only the band, so the
// zeroing launches are not needed.
#include <algorithm>
#include <cmath>
#include <cstdio>

#include <type_traits>

#include "avs_common.cuh"
#include "df64.cuh"

namespace avs {
namespace {

constexpr int kIB = 16;    // reflectors per compact-WY block
constexpr int kNT = 256;   // threads per CTA (16 columns x 16 row groups)

struct PanelArgs {
    void *a;
    int64_t lda;
    int b;
    int pr, pc;      // top tile row, panel tile column (view coordinates)
    int P;           // number of roles (tiles in the panel)
    int first_role;  // 0, or 1 for a lone TSQRT
    void *tau;       // [P][b]
    void *tblk;      // [P][b/kIB][kIB*kIB]
    int *ticket;
    int *progress;   // [2P]: diagonal block handed on, trailing top rows handed on
    int *err;
    const int *ready;  // optional: role p's tile is final once ready[p] >= ready_need
    int ready_need;
    int64_t sA, sTau, sTblk, sFlags;  // per-matrix strides (blockIdx.y = matrix)
};

struct UpdateArgs {
    void *a;
    int64_t lda;
    int64_t n;
    int b;
    int pr, pc, P;
    int first_role;  // 1: the top tile's own (GEQRT) blocks were applied earlier
    int width;       // strip width
    const void *tblk;
    int64_t sA, sTblk;  // per-matrix strides (blockIdx.y = matrix)
};

__host__ __device__ inline int ldpad(int b) { return b + 1; }

// ---------------------------------------------------------------------------
// Reflector scalars.  The reference's expressions (QRkernels.jl:27-31) in
// closed form: n1 = ||x||, nu = alpha + sign(alpha) n1,
// tau = 2 nu^2 / (s + nu^2) = |nu| / n1, tau / nu = sign(nu) / n1,
// tau / nu^2 = 1 / (n1 |nu|), new diagonal beta = -sign(alpha) n1; evaluated in
// FP64 for FP64 tiles and in double-float for FP32 tiles (GB300 issues FP64 at
// 1/64 of the FP32 rate).

// Reflector scalars from s = sum of squares of the sub-column (as a pair) and
// alpha.  Writes nu, tau, tau/nu, tau/nu^2, 1/nu, beta (the new diagonal).
struct PScalars {
    double nu, tau, tc, f, inv, beta;
};

__device__ __forceinline__ PScalars pscal_double(double s, double alpha) {
    PScalars r;
    const double n1 = sqrt(s + alpha * alpha);
    const double sg = alpha < 0.0 ? -1.0 : 1.0;
    r.nu = alpha + sg * n1;
    if (r.nu == 0.0) {
        r.tau = r.tc = r.f = r.inv = 0.0;
        r.beta = alpha;
        return r;
    }
    const double rn1 = 1.0 / n1;
    const double anu = fabs(r.nu);
    r.tau = anu * rn1;
    r.tc = (r.nu < 0.0 ? -rn1 : rn1);
    r.inv = 1.0 / r.nu;
    r.f = rn1 * fabs(r.inv);
    r.beta = -sg * n1;
    return r;
}

// FP32 tiles: the same closed forms in double-float, rounded to FP32 at the
// end -- no FP64 instruction (GB300 runs those at 1/64 of the FP32 rate).
struct PScalarsF {
    float nu, tau, tc, f, inv, beta;
};

__device__ __forceinline__ PScalarsF pscal_float(df64 s, float alpha) {
    PScalarsF r;
    const df64 x = df_add(s, two_prod(alpha, alpha));  // n1^2
    if (x.hi <= 0.0f) {  // zero column: identity reflector
        r.nu = r.tau = r.tc = r.f = r.inv = 0.0f;
        r.beta = alpha;
        return r;
    }
    // 1/n1: hardware rsqrt estimate, one Newton step in double-float:
    // y' = y + y (1 - x y^2) / 2
    const float y0 = rsqrtf(x.hi);
    const df64 e = df_sub(df64{1.0f, 0.0f}, df_mul(x, two_prod(y0, y0)));
    const df64 rn1 = df_add(df64{y0, 0.0f}, df_mul_f(e, 0.5f * y0));
    const df64 n1 = df_mul(x, rn1);
    const bool neg = alpha < 0.0f;
    const df64 a = df64{alpha, 0.0f};
    const df64 nu = neg ? df_sub(a, n1) : df_add(a, n1);  // |nu| = |alpha| + n1 > 0
    // 1/nu: hardware reciprocal estimate, one Newton step: z' = z + z (1 - nu z)
    const float z0 = __fdividef(1.0f, nu.hi);
    const df64 ez = df_sub(df64{1.0f, 0.0f}, df_mul_f(nu, z0));
    const df64 inv = df_add(df64{z0, 0.0f}, df_mul_f(ez, z0));
    const df64 anu = neg ? df_neg(nu) : nu;
    const df64 ainv = neg ? df_neg(inv) : inv;
    const df64 tau = df_mul(anu, rn1);
    const df64 f = df_mul(rn1, ainv);
    r.nu = nu.hi + nu.lo;
    r.tau = tau.hi + tau.lo;
    r.tc = neg ? -(rn1.hi + rn1.lo) : (rn1.hi + rn1.lo);
    r.inv = inv.hi + inv.lo;
    r.f = f.hi + f.lo;
    r.beta = neg ? (n1.hi + n1.lo) : -(n1.hi + n1.lo);
    return r;
}

template <typename T>
struct PScal;
template <>
struct PScal<double> {
    using Acc = double;
    static __device__ __forceinline__ Acc zero() { return 0.0; }
    static __device__ __forceinline__ Acc sq(double x, Acc a) { return fma(x, x, a); }
    static __device__ __forceinline__ Acc shfl_add(Acc a, int o) { return a + __shfl_xor_sync(0xffffffffu, a, o); }
    static __device__ __forceinline__ Acc shfl_add_local(Acc a, Acc b) { return a + b; }
    static __device__ __forceinline__ void compute(Acc s, double alpha, double *out) {
        const PScalars r = pscal_double(s, alpha);
        out[0] = r.nu; out[1] = r.tc; out[2] = r.f; out[3] = r.inv; out[4] = r.beta; out[5] = r.tau;
    }
};
template <>
struct PScal<float> {
    using Acc = df64;
    static __device__ __forceinline__ Acc zero() { return df64{0.0f, 0.0f}; }
    static __device__ __forceinline__ Acc sq(float x, Acc a) { return df_add(a, two_prod(x, x)); }
    static __device__ __forceinline__ Acc shfl_add(Acc a, int o) {
        return df_add(a, df64{__shfl_xor_sync(0xffffffffu, a.hi, o), __shfl_xor_sync(0xffffffffu, a.lo, o)});
    }
    static __device__ __forceinline__ Acc shfl_add_local(Acc a, Acc b) { return df_add(a, b); }
    static __device__ __forceinline__ void compute(Acc s, float alpha, float *out) {
        const PScalarsF r = pscal_float(s, alpha);
        out[0] = r.nu; out[1] = r.tc; out[2] = r.f; out[3] = r.inv; out[4] = r.beta; out[5] = r.tau;
    }
};

// FP64 tiles in double-float arithmetic (AVS_PREC_FP64X2): the same closed
// forms with alpha and the results as double-float values.
struct PScalarsD {
    df64 nu, tau, tc, f, inv, beta;
};

__device__ __forceinline__ PScalarsD pscal_df(df64 s, df64 alpha) {
    PScalarsD r;
    const df64 x = df_add(s, df_mul(alpha, alpha));  // n1^2
    const df64 z{0.0f, 0.0f};
    if (x.hi <= 0.0f) {  // zero column: identity reflector
        r.nu = r.tau = r.tc = r.f = r.inv = z;
        r.beta = alpha;
        return r;
    }
    // 1/n1 and 1/nu: FP32 estimates refined by one Newton step in double-float
    const float y0 = rsqrtf(x.hi);
    const df64 e = df_sub(df64{1.0f, 0.0f}, df_mul(x, two_prod(y0, y0)));
    const df64 rn1 = df_add(df64{y0, 0.0f}, df_mul_f(e, 0.5f * y0));
    const df64 n1 = df_mul(x, rn1);
    const bool neg = df_lt0(alpha);
    const df64 nu = neg ? df_sub(alpha, n1) : df_add(alpha, n1);  // |nu| = |alpha| + n1 > 0
    const df64 inv = df_rcp(nu);
    const df64 anu = neg ? df_neg(nu) : nu;
    const df64 ainv = neg ? df_neg(inv) : inv;
    r.nu = nu;
    r.tau = df_mul(anu, rn1);
    r.tc = neg ? df_neg(rn1) : rn1;
    r.inv = inv;
    r.f = df_mul(rn1, ainv);
    r.beta = neg ? n1 : df_neg(n1);
    return r;
}

template <>
struct PScal<dfx> {
    using Acc = df64;
    static __device__ __forceinline__ Acc zero() { return df64{0.0f, 0.0f}; }
    static __device__ __forceinline__ Acc sq(dfx x, Acc a) { return df_add(a, df_mul(x.v, x.v)); }
    static __device__ __forceinline__ Acc shfl_add(Acc a, int o) {
        return df_add(a, df64{__shfl_xor_sync(0xffffffffu, a.hi, o), __shfl_xor_sync(0xffffffffu, a.lo, o)});
    }
    static __device__ __forceinline__ Acc shfl_add_local(Acc a, Acc b) { return df_add(a, b); }
    static __device__ __forceinline__ void compute(Acc s, dfx alpha, dfx *out) {
        const PScalarsD r = pscal_df(s, alpha.v);
        out[0] = dfx(r.nu); out[1] = dfx(r.tc); out[2] = dfx(r.f); out[3] = dfx(r.inv); out[4] = dfx(r.beta);
        out[5] = dfx(r.tau);
    }
};

// Warp shuffles and finiteness of the panel's compute types.
__device__ __forceinline__ float vshfl_xor(float v, int o) { return __shfl_xor_sync(0xffffffffu, v, o); }
__device__ __forceinline__ double vshfl_xor(double v, int o) { return __shfl_xor_sync(0xffffffffu, v, o); }
__device__ __forceinline__ dfx vshfl_xor(dfx v, int o) {
    return dfx(df64{__shfl_xor_sync(0xffffffffu, v.v.hi, o), __shfl_xor_sync(0xffffffffu, v.v.lo, o)});
}
__device__ __forceinline__ float vshfl(float v, int src) { return __shfl_sync(0xffffffffu, v, src); }
__device__ __forceinline__ double vshfl(double v, int src) { return __shfl_sync(0xffffffffu, v, src); }
__device__ __forceinline__ dfx vshfl(dfx v, int src) {
    return dfx(df64{__shfl_sync(0xffffffffu, v.v.hi, src), __shfl_sync(0xffffffffu, v.v.lo, src)});
}
__device__ __forceinline__ bool vfinite(float v) { return isfinite(v); }
__device__ __forceinline__ bool vfinite(double v) { return isfinite(v); }
__device__ __forceinline__ bool vfinite(dfx v) { return isfinite(v.v.hi) && isfinite(v.v.lo); }

// ---------------------------------------------------------------------------
// Panel kernel (roles, schedule and outputs as described at the top):
//   * every thread owns one row of the 16-column slice (b <= 256 rows, 256
//     threads); the 16 dot products of a reflector step are reduced with a
//     warp reduce-scatter (16 shuffles) and one double-buffered shared-memory
//     pass across warps: one barrier per reflector;
//   * the masked reflector block Y is written once per block (row-major, so the
//     apply reads a row of it as 16 consecutive values);
//   * the apply to the rest of the tile is Z = Y^T C (thread j owns column j; C
//     streams through shared memory in row chunks, cp.async ring issued at the
//     start of the block), W = T^T Z (+ top rows), C -= Y W (threads own rows,
//     W broadcast from shared memory).

template <typename T>
__device__ __forceinline__ void ld4(const T *p, T (&v)[4]) {
    if (sizeof(T) == 4) {
        const float4 x = __ldcg(reinterpret_cast<const float4 *>(p));
        v[0] = x.x; v[1] = x.y; v[2] = x.z; v[3] = x.w;
    } else {
        const double2 x = __ldcg(reinterpret_cast<const double2 *>(p));
        const double2 y = __ldcg(reinterpret_cast<const double2 *>(p) + 1);
        v[0] = x.x; v[1] = x.y; v[2] = y.x; v[3] = y.y;
    }
}

// Rows of the trailing tile staged per chunk in the apply's first product
// (two chunks in flight), and the padded leading dimension of a chunk.
template <typename T>
__host__ __device__ constexpr int chunk_rows() { return sizeof(T) == 8 ? 16 : 32; }
template <typename T, int LAYOUT>
__host__ __device__ inline int chunk_ld(int b) { return LAYOUT == 0 ? chunk_rows<T>() + 4 : b + 4; }
// chunks in flight: the first ones are issued when a block starts, so their
// loads overlap the block's reflectors
template <typename T>
__host__ __device__ constexpr int chunk_bufs() { return sizeof(T) == 8 ? 2 : 4; }
template <typename T>
__host__ __device__ inline size_t chunk_elems(int b) {
    // the larger of the two layouts: [b][CR + 4] or [CR][b + 4]
    const size_t a0 = (size_t)b * (chunk_rows<T>() + 4), a1 = (size_t)chunk_rows<T>() * (b + 4);
    return a0 > a1 ? a0 : a1;
}

template <typename T>
size_t panel3_smem_bytes(int b) {
    return sizeof(T) * (32 /* tau, scalars */ + (size_t)ldpad(b) * kIB /* X */ + (size_t)b * kIB /* Yr */ +
                        (size_t)kIB * b /* Rt */ + (size_t)kIB * b /* Ws */ + 2 * kIB * kIB /* Tm, G */ +
                        16 * kIB /* part */ + 8 + 2 * kIB /* spart, dsum, rvs */ + 4 /* align */ +
                        chunk_bufs<T>() * chunk_elems<T>(b) /* C chunks */) +
           sizeof(double) * 16;
}

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((uint32_t)__cvta_generic_to_shared(smem)),
                 "l"(gmem)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

template <typename T, int LAYOUT, typename CT = T>
__global__ void __launch_bounds__(kNT) panel3_kernel(PanelArgs args) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int b = args.b;
    const int nb = b / kIB;
    const int ldx = ldpad(b);
    using Acc = typename PScal<CT>::Acc;
    Acc *spart = reinterpret_cast<Acc *>(smem_raw);         // 8 warps
    CT *stau = reinterpret_cast<CT *>(smem_raw + sizeof(double) * 16);
    CT *scal = stau + kIB;                                   // 16
    CT *X = scal + 16;                                       // ldx * kIB (column-major)
    CT *Yr = X + (size_t)ldx * kIB;                          // b * kIB (row-major: Yr[t*16 + l])
    CT *Rt = Yr + (size_t)b * kIB;                           // kIB * b, Rt[l + j*kIB]
    CT *Ws = Rt + (size_t)kIB * b;                           // kIB * b, Ws[l + j*kIB]
    CT *Tm = Ws + (size_t)kIB * b;                           // kIB * kIB, Tm[l + i*kIB]
    CT *G = Tm + kIB * kIB;                                  // kIB * kIB
    CT *part = G + kIB * kIB;                                // 2 x 8 * kIB (double-buffered)
    CT *dsum = part + 16 * kIB;                              // end of the small arrays
    // C chunks (16-byte aligned): LAYOUT 0 [column][row], LAYOUT 1 [row][column]
    T *cbuf0 = reinterpret_cast<T *>((reinterpret_cast<uintptr_t>(dsum + 2 * kIB + 8) + 15) & ~(uintptr_t)15);

    __shared__ int s_role, s_ok;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int64_t zb = blockIdx.y;
    int *ticket = args.ticket + zb * args.sFlags;
    int *progress = args.progress + zb * args.sFlags;
    if (tid == 0) s_role = atomicAdd(ticket, 1) + args.first_role;
    __syncthreads();
    const int p = s_role;
    if (p >= args.P) return;

    View<T, LAYOUT> V{reinterpret_cast<T *>(args.a) + zb * args.sA, args.lda};
    const int64_t row0 = (int64_t)(args.pr + p) * b;
    const int64_t top0 = (int64_t)args.pr * b;
    const int64_t col0 = (int64_t)args.pc * b;
    const bool geqrt = (p == 0);
    T *tau_out = reinterpret_cast<T *>(args.tau) + zb * args.sTau + (size_t)p * b;
    T *tblk_out = reinterpret_cast<T *>(args.tblk) + zb * args.sTblk + (size_t)p * nb * kIB * kIB;
    const int t = tid;  // my row (b <= 256)

    if (args.ready) {  // the tile is still being written by the previous update's chain
        if (tid == 0) s_ok = wait_geq(args.ready + p, args.ready_need, args.err);
        __syncthreads();
        if (!s_ok) return;
    }
    int *full = progress + args.P;  // per role: block cb's trailing top rows are final
    for (int cb = 0; cb < nb; ++cb) {
        const int c0 = cb * kIB;
        // ---- the role's own tile (no other role writes it): the block's 16
        // columns and the first chunks of its trailing columns load while the
        // role waits for the previous one
        for (int idx = tid; idx < b * kIB; idx += kNT) {
            int tt, l;
            if (LAYOUT == 0) { tt = idx % b; l = idx / b; } else { l = idx % kIB; tt = idx / kIB; }
            X[tt + l * ldx] = CT(__ldcg(&V(row0 + tt, col0 + c0 + l)));
        }
        const int jbase = c0 + kIB;
        const int nrest = b - jbase;
        const int tstart = geqrt ? c0 : 0;  // rows above c0 have Y = 0 for GEQRT
        constexpr int CR = chunk_rows<T>();
        constexpr int NBUF = chunk_bufs<T>();
        const int cld = chunk_ld<T, LAYOUT>(b);
        const int nch = nrest > 0 ? (b - tstart + CR - 1) / CR : 0;
        auto issue = [&](int ch) {  // one cp.async group per chunk (empty past the last)
            if (ch < nch) {
                constexpr int VEC = 16 / (int)sizeof(T);  // elements per 16-byte copy
                T *buf = cbuf0 + (size_t)(ch % NBUF) * chunk_elems<T>(b);
                const int t0 = tstart + ch * CR;
                const int rows = min(CR, b - t0);
                if (LAYOUT == 0) {  // column j: rows t0.. contiguous
                    const int per = rows / VEC;
                    for (int idx = tid; idx < nrest * per; idx += kNT) {
                        const int j = idx / per, r = (idx % per) * VEC;
                        cp_async16(buf + j * cld + r, &V(row0 + t0 + r, col0 + jbase + j));
                    }
                } else {  // row t: columns contiguous
                    const int per = nrest / VEC;
                    for (int idx = tid; idx < rows * per; idx += kNT) {
                        const int r = idx / per, j = (idx % per) * VEC;
                        cp_async16(buf + r * cld + j, &V(row0 + t0 + r, col0 + jbase + j));
                    }
                }
            }
            cp_async_commit();
        };
        if (nrest > 0) {
#pragma unroll
            for (int q = 0; q < NBUF; ++q) issue(q);
        }
        // ---- the diagonal 16 x 16 block of the top rows, once the previous
        // role's reflectors of this block are in it (TSQRT)
        if (tid == 0) {
            bool ok = true;
            if (p > args.first_role) ok = wait_geq(progress + p - 1, cb + 1, args.err);
            s_ok = ok;
        }
        __syncthreads();
        if (!s_ok) {
            cp_async_wait<0>();
            return;
        }
        if (!geqrt) {
            for (int idx = tid; idx < kIB * kIB; idx += kNT) {
                int l, j;
                if (LAYOUT == 0) { l = idx % kIB; j = idx / kIB; } else { j = idx % kIB; l = idx / kIB; }
                Rt[l + (c0 + j) * kIB] = CT(__ldcg(&V(top0 + c0 + l, col0 + c0 + j)));
            }
        }
        __syncthreads();

        // ---- the 16 reflectors of the block, one per step, all threads.  One
        // barrier per reflector: the warp partial sums are double-buffered, and
        // every warp forms the (identical) scalars and column sums itself.
        // Every warp reads the pivot row (alpha and the row the reflector
        // updates) after the step's barrier, so warp 0 keeps the updated pivot
        // row in registers and stores it after the next barrier: no later step
        // reads that row before the Gram matrix below.
        CT *pend_at = nullptr;
        CT pend_v = CT(0);
        for (int i = 0; i < kIB; ++i) {
            const int c = c0 + i;
            const int pb = i & 1;
            if (geqrt && c == b - 1) {
                if (tid == 0) stau[i] = CT(0);
                continue;
            }
            const bool live = (t < b) && (geqrt ? (t > c) : true);
            const CT x = live ? X[t + i * ldx] : CT(0);
            CT pv[kIB];
#pragma unroll
            for (int jj = 0; jj < kIB; ++jj) pv[jj] = (live && jj > i) ? x * X[t + jj * ldx] : CT(0);
            Acc sq = PScal<CT>::zero();
            if (live) sq = PScal<CT>::sq(x, sq);
            // warp reduce-scatter of pv[0..15]: lane L ends with the warp sum of pv[L & 15]
#pragma unroll
            for (int h = 8; h >= 1; h >>= 1) {
                const bool upper = (lane & h) != 0;
#pragma unroll
                for (int q = 0; q < h; ++q) {
                    const CT send = upper ? pv[q] : pv[q + h];
                    const CT keep = upper ? pv[q + h] : pv[q];
                    pv[q] = keep + vshfl_xor(send, h);
                }
            }
            pv[0] += vshfl_xor(pv[0], 16);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) sq = PScal<CT>::shfl_add(sq, o);
            if (lane < kIB) part[pb * 8 * kIB + wid * kIB + lane] = pv[0];  // lane L holds index L & 15
            if (lane == 0) spart[pb * 8 + wid] = sq;
            __syncthreads();
            if (pend_at) {  // the previous step's pivot row, read by every warp before this barrier
                *pend_at = pend_v;
                pend_at = nullptr;
            }
            const CT alpha = geqrt ? X[c + i * ldx] : Rt[i + c * kIB];
            CT out[6];
            if constexpr (!std::is_same<CT, double>::value) {
                // FP32 tiles: every lane forms the (double-float) scalars -- no
                // divergence, and the loads below overlap them.  The 8 warp
                // partials are summed by a 3-level shuffle tree; df_add is
                // commutative, so every lane of every warp gets the same sum.
                Acc s_all = spart[pb * 8 + (lane & 7)];
                s_all = PScal<CT>::shfl_add(s_all, 1);
                s_all = PScal<CT>::shfl_add(s_all, 2);
                s_all = PScal<CT>::shfl_add(s_all, 4);
                PScal<CT>::compute(s_all, alpha, out);
                if (!vfinite(out[5]) || !vfinite(out[0])) {
                    if (tid == 0) atomicCAS(args.err, kDevOk, kDevNonfinite);
                    out[5] = out[1] = out[2] = out[3] = CT(0);
                    out[4] = alpha;
                }
            } else {
                // FP64 tiles: lane 0 of each warp forms the scalars (FP64 is
                // costly on every lane), the warp reads them with shuffles
                if (lane == 0) {
                    Acc s_all = PScal<CT>::zero();
#pragma unroll
                    for (int w = 0; w < kNT / 32; ++w) s_all = PScal<CT>::shfl_add_local(s_all, spart[pb * 8 + w]);
                    PScal<CT>::compute(s_all, alpha, out);
                    if (!vfinite(out[5]) || !vfinite(out[0])) {
                        if (tid == 0) atomicCAS(args.err, kDevOk, kDevNonfinite);
                        out[5] = out[1] = out[2] = out[3] = CT(0);
                        out[4] = alpha;
                    }
                }
#pragma unroll
                for (int q = 0; q < 6; ++q) out[q] = vshfl(out[q], 0);
            }
            // column sums of the 16 dot products: lane L sums column L & 15
            CT dmine = CT(0);
#pragma unroll
            for (int w = 0; w < kNT / 32; ++w) dmine += part[pb * 8 * kIB + w * kIB + (lane & 15)];
            CT rvr[kIB];
#pragma unroll
            for (int jj = 0; jj < kIB; ++jj) rvr[jj] = geqrt ? X[c + jj * ldx] : Rt[i + (c0 + jj) * kIB];
            const CT tv = out[5];
            if (tid == 0) stau[i] = tv;
            if (tv == CT(0)) {
                if (live) X[t + i * ldx] = CT(0);
                continue;  // the next step reads only own rows until its barrier
            }
            const CT nu = out[0], tc = out[1], f = out[2], inv = out[3];
            CT dsv[kIB];
#pragma unroll
            for (int jj = 0; jj < kIB; ++jj) dsv[jj] = vshfl(dmine, jj);
            if (live) {
#pragma unroll
                for (int jj = 0; jj < kIB; ++jj)
                    if (jj > i) X[t + jj * ldx] -= x * (f * (nu * rvr[jj] + dsv[jj]));
                X[t + i * ldx] = x * inv;
            }
            if (tid < kIB && tid >= i) {
                pend_v = (tid == i) ? out[4] : rvr[tid] - tc * (nu * rvr[tid] + dmine);
                pend_at = geqrt ? &X[c + tid * ldx] : &Rt[i + (c0 + tid) * kIB];
            }
        }
        __syncthreads();
        if (pend_at) *pend_at = pend_v;
        __syncthreads();
        // the diagonal block of the top rows is final for this role: back to
        // global memory and handed on -- a TSQRT role's successor needs only
        // this block for its own reflectors
        if (!geqrt) {
            for (int idx = tid; idx < kIB * kIB; idx += kNT) {
                int l, jx;
                if (LAYOUT == 0) { l = idx % kIB; jx = idx / kIB; } else { jx = idx % kIB; l = idx / kIB; }
                V(top0 + c0 + l, col0 + c0 + jx) = (T)Rt[l + (c0 + jx) * kIB];
            }
            __syncthreads();
            if (tid == 0) {
                __threadfence();
                st_release(progress + p, cb + 1);
            }
        }

        // ---- Gram matrix of the block's reflectors, CT (warp 0), masked Y
        {
            const int pi = tid >> 1, h = tid & 1;
            int l = -1, i = 0;
            if (pi < kIB * (kIB - 1) / 2) {
                int acc = 0;
                for (int ii = 1; ii < kIB; ++ii) {
                    if (pi < acc + ii) { i = ii; l = pi - acc; break; }
                    acc += ii;
                }
            }
            CT pt = CT(0);
            if (l >= 0) {
                const int half = (b + 1) / 2;
                const int tlo = h * half, thi = min(b, tlo + half);
                for (int tt = tlo; tt < thi; ++tt)
                    if (geqrt ? (tt > c0 + i) : true) pt += X[tt + l * ldx] * X[tt + i * ldx];
            }
            pt += vshfl_xor(pt, 1);
            if (l >= 0 && h == 0) G[l + i * kIB] = pt + (geqrt ? X[c0 + i + l * ldx] : CT(0));
        }
        if (tid < kIB * kIB) Tm[tid] = CT(0);
        for (int idx = tid; idx < b * kIB; idx += kNT) {
            const int tt = idx / kIB, l = idx % kIB;
            CT y = X[tt + l * ldx];
            if (geqrt) y = (tt == c0 + l) ? CT(1) : (tt > c0 + l ? y : CT(0));
            Yr[tt * kIB + l] = y;
        }
        __syncthreads();
        if (wid == 0) {
            if (lane < kIB) Tm[lane + lane * kIB] = stau[lane];
            __syncwarp();
            for (int i = 1; i < kIB; ++i) {
                if (lane < i) {
                    CT acc = CT(0);
                    for (int m = lane; m < i; ++m) acc += Tm[lane + m * kIB] * G[m + i * kIB];
                    Tm[lane + i * kIB] = -stau[i] * acc;
                }
                __syncwarp();
            }
        }
        for (int idx = tid; idx < b * kIB; idx += kNT) {
            int tt, l;
            if (LAYOUT == 0) { tt = idx % b; l = idx / b; } else { l = idx % kIB; tt = idx / kIB; }
            if (!geqrt || tt >= c0) V(row0 + tt, col0 + c0 + l) = (T)X[tt + l * ldx];
        }
        if (tid < kIB) tau_out[c0 + tid] = (T)stau[tid];
        __syncthreads();
        if (geqrt && tid == 0) {  // the block's rows of the top tile are written back above
            __threadfence();
            st_release(progress, cb + 1);
        }
        if (tid < kIB * kIB) tblk_out[(size_t)cb * kIB * kIB + tid] = (T)Tm[tid];

        // ---- apply to the rest of the tile
        if (nrest > 0) {
            // (a) Z = Y^CT C: the rows tstart..b-1 of C stream through shared
            // memory in chunks of CR rows (cp.async ring of NBUF chunks, issued
            // since the block started); thread j owns column j and all 16
            // reflectors (Y rows broadcast).
            {
                CT z[kIB];
#pragma unroll
                for (int l = 0; l < kIB; ++l) z[l] = CT(0);
                for (int ch = 0; ch < nch; ++ch) {
                    cp_async_wait<NBUF - 1>();
                    __syncthreads();
                    const T *buf = cbuf0 + (size_t)(ch % NBUF) * chunk_elems<T>(b);
                    const int t0 = tstart + ch * CR;
                    const int rows = min(CR, b - t0);
                    const int j = tid;
                    if (j < nrest) {
                        for (int r = 0; r < rows; ++r) {
                            const CT cv = CT(LAYOUT == 0 ? buf[j * cld + r] : buf[r * cld + j]);
                            const CT *yrow = Yr + (t0 + r) * kIB;
#pragma unroll
                            for (int l = 0; l < kIB; ++l) z[l] += yrow[l] * cv;
                        }
                    }
                    __syncthreads();
                    issue(ch + NBUF);
                }
                cp_async_wait<0>();
                if (tid < nrest) {
#pragma unroll
                    for (int l = 0; l < kIB; ++l) Ws[l + tid * kIB] = z[l];
                }
            }
            __syncthreads();
            // the trailing top rows, once the previous role's (b) is in them
            if (!geqrt) {
                if (tid == 0) s_ok = (p > args.first_role) ? wait_geq(full + p - 1, cb + 1, args.err) : true;
                __syncthreads();
                if (!s_ok) return;
                for (int idx = tid; idx < kIB * nrest; idx += kNT) {
                    int l, j;
                    if (LAYOUT == 0) { l = idx % kIB; j = idx / kIB; } else { j = idx % nrest; l = idx / nrest; }
                    Rt[l + (jbase + j) * kIB] = CT(__ldcg(&V(top0 + c0 + l, col0 + jbase + j)));
                }
                __syncthreads();
            }
            // (b) W = CT^CT (Z + top rows); top rows -= W
            for (int jr = tid; jr < nrest; jr += kNT) {
                CT zc[kIB];
#pragma unroll
                for (int l = 0; l < kIB; ++l) {
                    zc[l] = Ws[l + jr * kIB];
                    if (!geqrt) zc[l] += Rt[l + (jbase + jr) * kIB];
                }
#pragma unroll
                for (int l = 0; l < kIB; ++l) {
                    CT acc = CT(0);
#pragma unroll
                    for (int m = 0; m <= l; ++m) acc += Tm[m + l * kIB] * zc[m];
                    Ws[l + jr * kIB] = acc;
                    if (!geqrt) Rt[l + (jbase + jr) * kIB] -= acc;
                }
            }
            __syncthreads();
            // The trailing top rows are final for this block: a TSQRT role
            // hands them to the next role now, before updating its own tile (c).
            if (!geqrt) {
                for (int idx = tid; idx < kIB * nrest; idx += kNT) {
                    int l, jx;
                    if (LAYOUT == 0) { l = idx % kIB; jx = idx / kIB; } else { jx = idx % nrest; l = idx / nrest; }
                    V(top0 + c0 + l, col0 + jbase + jx) = (T)Rt[l + (jbase + jx) * kIB];
                }
                __syncthreads();
                if (tid == 0) {
                    __threadfence();
                    st_release(full + p, cb + 1);
                }
            }
            // (c) C -= Y W: thread owns row t; 16 columns per group, the next
            // group's loads issued before the current group's arithmetic
            if (t >= tstart && t < b) {
                CT yv[kIB];
#pragma unroll
                for (int l = 0; l < kIB; ++l) yv[l] = Yr[t * kIB + l];
                CT cur[16], nxt[16];
                auto load16 = [&](int jr, CT (&v)[16]) {
                    if (LAYOUT == 0) {
#pragma unroll
                        for (int q = 0; q < 16; ++q) v[q] = CT(__ldcg(&V(row0 + t, col0 + jbase + jr + q)));
                    } else {
#pragma unroll
                        for (int q4 = 0; q4 < 4; ++q4) {
                            T w4[4];
                            ld4(&V(row0 + t, col0 + jbase + jr + 4 * q4), w4);
#pragma unroll
                            for (int q = 0; q < 4; ++q) v[4 * q4 + q] = CT(w4[q]);
                        }
                    }
                };
                load16(0, cur);
                for (int jr = 0; jr < nrest; jr += 16) {
                    if (jr + 16 < nrest) load16(jr + 16, nxt);
#pragma unroll
                    for (int q = 0; q < 16; ++q) {
                        CT s2 = CT(0);
#pragma unroll
                        for (int l = 0; l < kIB; ++l) s2 += yv[l] * Ws[l + (jr + q) * kIB];
                        cur[q] -= s2;
                    }
                    if (LAYOUT == 0) {
#pragma unroll
                        for (int q = 0; q < 16; ++q) V(row0 + t, col0 + jbase + jr + q) = (T)cur[q];
                    } else {
#pragma unroll
                        for (int q = 0; q < 16; ++q) V(row0 + t, col0 + jbase + jr + q) = (T)cur[q];
                    }
#pragma unroll
                    for (int q = 0; q < 16; ++q) cur[q] = nxt[q];
                }
            }
        } else if (!geqrt) {
            // no columns right of the block (the diagonal block went back above)
            if (tid == 0) st_release(full + p, cb + 1);
        }
        __syncthreads();
        if (geqrt && tid == 0) {
            __threadfence();
            st_release(full, cb + 1);
        }
    }
}

template <typename T>
size_t update_smem_bytes(int b, int width) {
    return sizeof(T) * ((size_t)2 * ldpad(b) * width + (size_t)ldpad(b) * kIB + 2 * (size_t)kIB * width +
                        (size_t)kIB * kIB);
}

template <typename T, int LAYOUT>
__global__ void __launch_bounds__(kNT) update_kernel(UpdateArgs args) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int b = args.b;
    const int nb = b / kIB;
    const int ld = ldpad(b);
    const int W = args.width;
    T *Top = reinterpret_cast<T *>(smem_raw);  // ld * W
    T *Ap = Top + (size_t)ld * W;              // ld * W
    T *Vs = Ap + (size_t)ld * W;               // ld * kIB
    T *Zs = Vs + (size_t)ld * kIB;             // kIB * W
    T *Ws = Zs + (size_t)kIB * W;              // kIB * W
    T *Tm = Ws + (size_t)kIB * W;              // kIB * kIB

    const int tid = threadIdx.x;
    const int64_t j0 = (int64_t)(args.pc + 1) * b + (int64_t)blockIdx.x * W;
    const int wc = (int)min((int64_t)W, args.n - j0);
    if (wc <= 0) return;
    const int64_t zb = blockIdx.y;
    View<T, LAYOUT> V{reinterpret_cast<T *>(args.a) + zb * args.sA, args.lda};
    const int64_t top0 = (int64_t)args.pr * b;
    const int64_t col0 = (int64_t)args.pc * b;
    const T *tblk = reinterpret_cast<const T *>(args.tblk) + zb * args.sTblk;

    auto load_strip = [&](T *S, int64_t r0) {
        for (int idx = tid; idx < b * wc; idx += kNT) {
            int t, c;
            if (LAYOUT == 0) { t = idx % b; c = idx / b; } else { c = idx % wc; t = idx / wc; }
            S[t + c * ld] = V(r0 + t, j0 + c);
        }
    };
    auto store_strip = [&](const T *S, int64_t r0) {
        for (int idx = tid; idx < b * wc; idx += kNT) {
            int t, c;
            if (LAYOUT == 0) { t = idx % b; c = idx / b; } else { c = idx % wc; t = idx / wc; }
            V(r0 + t, j0 + c) = S[t + c * ld];
        }
    };

    load_strip(Top, top0);
    for (int p = args.first_role; p < args.P; ++p) {
        const bool geqrt = (p == 0);
        const int64_t r0 = (int64_t)(args.pr + p) * b;
        T *Tp = geqrt ? Top : Ap;
        if (!geqrt) load_strip(Ap, r0);
        for (int cb = 0; cb < nb; ++cb) {
            const int c0 = cb * kIB;
            for (int idx = tid; idx < b * kIB; idx += kNT) {
                int t, l;
                if (LAYOUT == 0) { t = idx % b; l = idx / b; } else { l = idx % kIB; t = idx / kIB; }
                Vs[t + l * ld] = V(r0 + t, col0 + c0 + l);
            }
            if (tid < kIB * kIB) Tm[tid] = tblk[((size_t)p * nb + cb) * kIB * kIB + tid];
            __syncthreads();
            // Z = Y^T Tp (+ top rows for TSQRT blocks)
            for (int o = tid; o < kIB * wc; o += kNT) {
                const int l = o % kIB, c = o / kIB;
                T z;
                if (geqrt) {
                    const int ts = c0 + l;
                    z = Tp[ts + c * ld];
                    for (int t = ts + 1; t < b; ++t) z += Vs[t + l * ld] * Tp[t + c * ld];
                } else {
                    z = Top[c0 + l + c * ld];
                    for (int t = 0; t < b; ++t) z += Vs[t + l * ld] * Tp[t + c * ld];
                }
                Zs[l + c * kIB] = z;
            }
            __syncthreads();
            // W = T^T Z
            for (int o = tid; o < kIB * wc; o += kNT) {
                const int l = o % kIB, c = o / kIB;
                T w = T(0);
                for (int m = 0; m <= l; ++m) w += Tm[m + l * kIB] * Zs[m + c * kIB];
                Ws[l + c * kIB] = w;
            }
            __syncthreads();
            // Tp -= Y W ; top rows -= W (TSQRT)
            for (int idx = tid; idx < b * wc; idx += kNT) {
                const int t = idx % b, c = idx / b;
                if (geqrt) {
                    if (t >= c0) {
                        const int lmax = min(kIB - 1, t - c0);
                        T acc = T(0);
                        for (int l = 0; l <= lmax; ++l) {
                            const T y = (t == c0 + l) ? T(1) : Vs[t + l * ld];
                            acc += y * Ws[l + c * kIB];
                        }
                        Tp[t + c * ld] -= acc;
                    }
                } else {
                    T acc = T(0);
#pragma unroll
                    for (int l = 0; l < kIB; ++l) acc += Vs[t + l * ld] * Ws[l + c * kIB];
                    Tp[t + c * ld] -= acc;
                }
            }
            if (!geqrt) {
                for (int o = tid; o < kIB * wc; o += kNT) {
                    const int l = o % kIB, c = o / kIB;
                    Top[c0 + l + c * ld] -= Ws[l + c * kIB];
                }
            }
            __syncthreads();
        }
        if (!geqrt) store_strip(Ap, r0);
        __syncthreads();
    }
    store_strip(Top, top0);
}

// FP64 tiles with the double-float trailing updates (AVS_PREC_FP64X2) run
// the panel in double-float arithmetic too (CT = dfx: FP64 storage, each value
// converted on load and rounded back on store); GB300 issues FP64 at 1/64 of
// the FP32 rate and the panel's reflectors and applies are FP64-issue-bound.
template <typename T, int LAYOUT>
int launch_panel(T *dA, int64_t lda, int b, int pr, int pc, int P, int first_role, const Stage1Work &w,
                 cudaStream_t s, const int *ready = nullptr) {
    static std::atomic<bool> attr_set{false};
    const size_t smem = panel3_smem_bytes<T>(b);
    const bool dfp = sizeof(T) == 8 && w.df_update;
    if (!attr_set) {
        AVS_CUDA_TRY(cudaFuncSetAttribute(panel3_kernel<T, LAYOUT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)panel3_smem_bytes<T>(256)));
        if constexpr (sizeof(T) == 8)
            AVS_CUDA_TRY(cudaFuncSetAttribute(panel3_kernel<T, LAYOUT, dfx>,
                                              cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)panel3_smem_bytes<T>(256)));
        attr_set = true;
    }
    const int batch = w.batch > 0 ? w.batch : 1;
    AVS_CUDA_TRY(cudaMemsetAsync(w.flags, 0, sizeof(int) * (size_t)(batch > 1 ? w.sFlags * batch : 2 * P + 1), s));
    PanelArgs a;
    a.a = dA;
    a.lda = lda;
    a.b = b;
    a.pr = pr;
    a.pc = pc;
    a.P = P;
    a.first_role = first_role;
    a.tau = w.tau;
    a.tblk = w.tblk;
    a.ticket = w.flags;
    a.progress = w.flags + 1;
    a.err = w.err;
    a.sA = w.sA;
    a.sTau = w.sTau;
    a.sTblk = w.sTblk;
    a.sFlags = w.sFlags;
    a.ready = ready;
    a.ready_need = b / kChainStrip;
    if constexpr (sizeof(T) == 8) {
        if (dfp) {
            panel3_kernel<T, LAYOUT, dfx><<<dim3(P - first_role, batch), kNT, smem, s>>>(a);
            AVS_CUDA_TRY(cudaGetLastError());
            return AVS_SUCCESS;
        }
    }
    panel3_kernel<T, LAYOUT><<<dim3(P - first_role, batch), kNT, smem, s>>>(a);
    AVS_CUDA_TRY(cudaGetLastError());
    return AVS_SUCCESS;
}

template <typename T, int LAYOUT>
int launch_update(T *dA, int64_t lda, int64_t n, int b, int pr, int pc, int P, const Stage1Work &w,
                  cudaStream_t s, int first_role = 0) {
    const int width = sizeof(T) == 8 ? 32 : 64;
    static std::atomic<bool> attr_set{false};
    if (!attr_set) {
        AVS_CUDA_TRY(cudaFuncSetAttribute(update_kernel<T, LAYOUT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)update_smem_bytes<T>(256, width)));
        attr_set = true;
    }
    const int64_t ncols = n - (int64_t)(pc + 1) * b;
    if (ncols <= 0) return AVS_SUCCESS;
    UpdateArgs a;
    a.a = dA;
    a.lda = lda;
    a.n = n;
    a.b = b;
    a.pr = pr;
    a.pc = pc;
    a.P = P;
    a.first_role = first_role;
    a.width = width;
    a.tblk = w.tblk;
    a.sA = w.sA;
    a.sTblk = w.sTblk;
    const unsigned grid = (unsigned)((ncols + width - 1) / width);
    update_kernel<T, LAYOUT><<<dim3(grid, w.batch > 0 ? w.batch : 1), kNT, update_smem_bytes<T>(b, width), s>>>(a);
    AVS_CUDA_TRY(cudaGetLastError());
    return AVS_SUCCESS;
}

// The tau of the panel just launched (roles 0..P-1 of half-step k, tile index
// first + p) to the caller's array, when it asked for them.
template <typename T>
int copy_tau_out(void *out, const Stage1Work &w, int nt, int k, int first, int P, int b, cudaStream_t s) {
    if (!out) return AVS_SUCCESS;
    AVS_CUDA_TRY(cudaMemcpyAsync(reinterpret_cast<T *>(out) + ((size_t)k * nt + first) * b, w.tau,
                                 sizeof(T) * (size_t)P * b, cudaMemcpyDeviceToDevice, s));
    return AVS_SUCCESS;
}

}  // namespace

// Tensor-core trailing update (the parts of stage1_tc_update in `parts`) of
// one half-step, bracketed by a pair of the caller's events when it asked for
// timing.
int timed_update(float *X, int64_t n, int b, int pr, int pc, int P, const Stage1Work &w, const TcBufs &tb,
                 cudaStream_t s, int64_t *launches, int parts = kTcAll, float *xt_out = nullptr,
                 int *ready = nullptr) {
    const bool timed = w.ev_pairs && w.ev_used && *w.ev_used < w.ev_cap;
    if (timed) AVS_CUDA_TRY(cudaEventRecord(w.ev_pairs[2 * *w.ev_used], s));
    const int rc = stage1_tc_update(X, n, b, pr, pc, P, w, tb, s, launches, parts, xt_out, ready);
    if (rc != AVS_SUCCESS) return rc;
    if (timed) {
        AVS_CUDA_TRY(cudaEventRecord(w.ev_pairs[2 * *w.ev_used + 1], s));
        ++*w.ev_used;
    }
    return AVS_SUCCESS;
}

// GE2BND with tensor-core trailing updates (FP32 tiles, b = 128 or 256, one
// matrix, lda = n): QR half-steps on X, LQ half-steps as QR half-steps on the
// transposed trailing block in XT.
//
// Lookahead: the next half-step's panel works on the top tile row that the
// chain of the current update computes (the chain writes it into the other
// buffer as well, transposed, and counts finished strips per tile), so the
// panel runs on the aux stream (high priority) beside the chain, each role
// waiting for its own tile, and beside the rest of the update (A_p -= Y_p W_p
// and the transpose of the rows below) on the caller's stream; its T build
// follows on aux.  The Y copies and S_p = Y_p^T A_p need the panel only and
// run beside the T build; the chain waits for both.  Every kernel touches the
// same data in the same order as without the overlap:
//   QR half-step k: the chain writes X row tile k (columns >= k+1) and its
//     transpose, XT column tile k = the LQ panel, which overlaps the rest of
//     the update of X rows >= k+1 and the transpose X -> XT of rows and
//     columns >= k+1.
//   LQ half-step k: the chain writes XT row tile k+1 and its transpose, X
//     column tile k+1 (rows >= k+1) = the next QR panel, which overlaps the
//     update of XT rows >= k+2 and the transposes back (XT rows >= k+2, and
//     the one tile XT(k+1, k) -> X(k, k+1)).
int stage1_ge2bnd_tc(float *X, int64_t n, int b, const Stage1Work &w, cudaStream_t s, int64_t *launches) {
    const int nt = (int)(n / b);
    const int fmt = w.tc_split;
    const TcBufs tb = stage1_tc_carve(w.tc_ws, n, b, fmt);
    float *XT = tb.xt;
    const bool la = w.aux && w.la_fork && w.la_panel && w.la_tb;
    cudaStream_t a = la ? w.aux : s;
    int rc, dev = 0, sms = 0;
    AVS_CUDA_TRY(cudaGetDevice(&dev));
    AVS_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    if ((rc = stage1_tc_planes(X, n, fmt, tb, s)) != AVS_SUCCESS) return rc;
    // panel + tau copy + T build of one half-step on the aux stream, after the
    // caller's stream has reached this point (or the point where it recorded
    // la_fork: forked = true); hand-offs back after the panel and after the T
    // build
    auto panel_tb = [&](float *M, int pr, int pc, int P, void *tau_out, int k, int first, const int *ready,
                        bool forked = false) -> int {
        int r;
        if (la) {
            if (!forked) AVS_CUDA_TRY(cudaEventRecord(w.la_fork, s));
            AVS_CUDA_TRY(cudaStreamWaitEvent(a, w.la_fork, 0));
        }
        if ((r = launch_panel<float, 0>(M, n, b, pr, pc, P, 0, w, a, ready)) != AVS_SUCCESS) return r;
        if ((r = copy_tau_out<float>(tau_out, w, nt, k, first, P, b, a)) != AVS_SUCCESS) return r;
        if (la) AVS_CUDA_TRY(cudaEventRecord(w.la_panel, a));
        if ((int64_t)(pc + 1) * b < n && (r = stage1_tbuild<float>(M, n, b, 0, pr, pc, P, w, a)) != AVS_SUCCESS)
            return r;
        if (la) AVS_CUDA_TRY(cudaEventRecord(w.la_tb, a));
        if (launches) *launches += 2;
        return AVS_SUCCESS;
    };
    // one half-step's update on the caller's stream, with the next panel
    // (on M2, panel tile (pr2, pc2), P2 tiles) started beside its chain
    auto half_step = [&](float *M, int pr, int pc, int P, float *M2, int pr2, int pc2, int P2, void *tau_out,
                         int k2, int first2) -> int {
        int r;
        if (la) AVS_CUDA_TRY(cudaStreamWaitEvent(s, w.la_panel, 0));
        if ((r = timed_update(M, n, b, pr, pc, P, w, tb, s, launches, kTcS)) != AVS_SUCCESS) return r;
        if (la) AVS_CUDA_TRY(cudaStreamWaitEvent(s, w.la_tb, 0));
        // The panel starts beside the chain (its roles wait for their tiles)
        // only while its P2 CTAs, on at most P2 SMs, leave at least half of the
        // SMs to the chain and the call holds its reservation (w.la_ready: the
        // waiting panels of all running calls within half of the SMs);
        // otherwise after it.  The chain is launched first:
        // where the two streams share a hardware queue the panel then simply
        // runs after it, so the panel's waits never hold the chain back.
        int *ready = (la && w.la_ready && 2 * P2 <= sms) ? tb.ready : nullptr;
        if ((r = timed_update(M, n, b, pr, pc, P, w, tb, s, launches, kTcPlanes, nullptr, ready)) != AVS_SUCCESS)
            return r;
        if (ready) AVS_CUDA_TRY(cudaEventRecord(w.la_fork, s));
        if ((r = timed_update(M, n, b, pr, pc, P, w, tb, s, launches, kTcChain, M2, ready)) != AVS_SUCCESS) return r;
        if ((r = panel_tb(M2, pr2, pc2, P2, tau_out, k2, first2, ready, ready != nullptr)) != AVS_SUCCESS) return r;
        return timed_update(M, n, b, pr, pc, P, w, tb, s, launches, kTcUpdate);
    };
    auto finish = [&](int r) -> int {  // the aux stream joins the caller's before any return
        if (la) {
            cudaEventRecord(w.la_fork, a);
            cudaStreamWaitEvent(s, w.la_fork, 0);
        }
        return r;
    };
    if ((rc = panel_tb(X, 0, 0, nt, w.tau_q_out, 0, 0, nullptr)) != AVS_SUCCESS) return finish(rc);
    for (int k = 0; k + 1 < nt; ++k) {
        const int64_t k1b = (int64_t)(k + 1) * b, k2b = (int64_t)(k + 2) * b;
        const int P = nt - k, PL = nt - k - 1;
        // QR half-step k (its panel and T build done or in flight on aux), the LQ panel beside it
        if ((rc = half_step(X, k, k, P, XT, k + 1, k, PL, w.tau_p_out, k, k + 1)) != AVS_SUCCESS) return finish(rc);
        // X rows, columns >= k+1 -> XT
        if ((rc = stage1_tc_transpose_box(X, XT, n, k1b, n - k1b, k1b, n - k1b, fmt, tb, s)) != AVS_SUCCESS)
            return finish(rc);
        // LQ half-step k, the next QR panel beside it
        if ((rc = half_step(XT, k + 1, k, PL, X, k + 1, k + 1, P - 1, w.tau_q_out, k + 1, k + 1)) != AVS_SUCCESS)
            return finish(rc);
        // and back: XT rows >= k+2 (all columns >= k) -> X, and the LQ panel's top tile
        if ((rc = stage1_tc_transpose_box(XT, X, n, k2b, n - k2b, (int64_t)k * b, n - (int64_t)k * b, fmt, tb, s)) !=
            AVS_SUCCESS)
            return finish(rc);
        if ((rc = stage1_tc_transpose_box(XT, X, n, k1b, b, (int64_t)k * b, b, fmt, tb, s)) != AVS_SUCCESS)
            return finish(rc);
        if (launches) *launches += 3;
    }
    // the last QR panel (one tile, no trailing columns) ran on aux
    return finish(AVS_SUCCESS);
}

template <typename T>
int stage1_ge2bnd(T *dA, int64_t n, int64_t lda, int b, const Stage1Work &w, cudaStream_t s, int64_t *launches) {
    const int nt = (int)(n / b);
    int rc;
    if constexpr (sizeof(T) == 4) {
        if (w.tc_split && w.tc_ws && b >= 128 && lda == n && (w.batch <= 1))
            return stage1_ge2bnd_tc(reinterpret_cast<float *>(dA), n, b, w, s, launches);
    }
    for (int k = 0; k < nt; ++k) {
        // QR half-step: GEQRT(k,k) + TSQRT(row,k), Q^T applied to the row panels.
        const int P = nt - k;
        if ((rc = launch_panel<T, 0>(dA, lda, b, k, k, P, 0, w, s)) != AVS_SUCCESS) return rc;
        if ((rc = copy_tau_out<T>(w.tau_q_out, w, nt, k, k, P, b, s)) != AVS_SUCCESS) return rc;
        if (b >= 128 && w.tfull)
            rc = stage1_update_full<T>(dA, lda, n, b, 0, k, k, P, w, s);
        else
            rc = launch_update<T, 0>(dA, lda, n, b, k, k, P, w, s);
        if (rc != AVS_SUCCESS) return rc;
        if (launches) *launches += (k + 1 < nt) ? ((b >= 128 && w.tfull) ? 3 : 2) : 1;
        if (k == nt - 1) break;
        // LQ half-step: the same on the transposed view, top tile (k, k+1).
        const int PL = nt - k - 1;
        if ((rc = launch_panel<T, 1>(dA, lda, b, k + 1, k, PL, 0, w, s)) != AVS_SUCCESS) return rc;
        if ((rc = copy_tau_out<T>(w.tau_p_out, w, nt, k, k + 1, PL, b, s)) != AVS_SUCCESS) return rc;
        if (b >= 128 && w.tfull)
            rc = stage1_update_full<T>(dA, lda, n, b, 1, k + 1, k, PL, w, s);
        else
            rc = launch_update<T, 1>(dA, lda, n, b, k + 1, k, PL, w, s);
        if (rc != AVS_SUCCESS) return rc;
        if (launches) *launches += (b >= 128 && w.tfull) ? 3 : 2;
    }
    return AVS_SUCCESS;
}

// Tiled QR (tiled_QR!, KAbasedSVD/src/tiledalgos.jl:6-15): the QR half-steps
// of GE2BND alone.  On return R is in the upper triangle and the reflectors
// below it (unit lower V in the diagonal tiles, full V in the tiles below);
// dtau (optional) receives the tau of panel k, tile row r, reflector l at
// dtau[(k * nt + r) * b + l] (rows r >= k).
template <typename T>
int stage1_geqrf(T *dA, int64_t n, int64_t lda, int b, const Stage1Work &w, T *dtau, cudaStream_t s,
                 int64_t *launches) {
    const int nt = (int)(n / b);
    int rc;
    const bool tc = sizeof(T) == 4 && w.tc_split && w.tc_ws && b >= 128 && lda == n && w.batch <= 1;
    TcBufs tb{};
    if (tc) tb = stage1_tc_carve(w.tc_ws, n, b, w.tc_split);
    for (int k = 0; k < nt; ++k) {
        const int P = nt - k;
        if ((rc = launch_panel<T, 0>(dA, lda, b, k, k, P, 0, w, s)) != AVS_SUCCESS) return rc;
        if (launches) ++*launches;
        if (dtau)
            AVS_CUDA_TRY(cudaMemcpyAsync(dtau + ((size_t)k * nt + k) * b, w.tau, sizeof(T) * (size_t)P * b,
                                         cudaMemcpyDeviceToDevice, s));
        if (k == nt - 1) break;
        if constexpr (sizeof(T) == 4) {
            if (tc) {
                // operand planes of the trailing block as the update reads it now
                const int64_t r0 = (int64_t)k * b, j0 = (int64_t)(k + 1) * b;
                if ((rc = stage1_tc_planes_block(reinterpret_cast<float *>(dA), n, r0, j0, w.tc_split, tb, s)) !=
                    AVS_SUCCESS)
                    return rc;
                if ((rc = stage1_tbuild<float>(reinterpret_cast<float *>(dA), n, b, 0, k, k, P, w, s)) != AVS_SUCCESS)
                    return rc;
                if ((rc = timed_update(reinterpret_cast<float *>(dA), n, b, k, k, P, w, tb, s, launches)) !=
                    AVS_SUCCESS)
                    return rc;
                if (launches) *launches += 2;
                continue;
            }
        }
        if (b >= 128 && w.tfull)
            rc = stage1_update_full<T>(dA, lda, n, b, 0, k, k, P, w, s);
        else
            rc = launch_update<T, 0>(dA, lda, n, b, k, k, P, w, s);
        if (rc != AVS_SUCCESS) return rc;
        if (launches) *launches += (b >= 128 && w.tfull) ? 2 : 1;
    }
    return AVS_SUCCESS;
}

template <typename T>
int stage1_geqrt_tile(T *dA, int b, T *dtau, const Stage1Work &w, cudaStream_t s) {
    int rc = launch_panel<T, 0>(dA, b, b, 0, 0, 1, 0, w, s);
    if (rc != AVS_SUCCESS) return rc;
    AVS_CUDA_TRY(cudaMemcpyAsync(dtau, w.tau, sizeof(T) * (size_t)(b - 1), cudaMemcpyDeviceToDevice, s));
    return AVS_SUCCESS;
}

// dRB: contiguous 2b x b buffer [R; B] (ld 2b); role 1 of a two-tile panel.
template <typename T>
int stage1_tsqrt_pair(T *dRB, int b, T *dtau, const Stage1Work &w, cudaStream_t s) {
    int rc = launch_panel<T, 0>(dRB, 2 * b, b, 0, 0, 2, 1, w, s);
    if (rc != AVS_SUCCESS) return rc;
    AVS_CUDA_TRY(cudaMemcpyAsync(dtau, reinterpret_cast<T *>(w.tau) + b, sizeof(T) * (size_t)b,
                                 cudaMemcpyDeviceToDevice, s));
    return AVS_SUCCESS;
}

// One panel (P tiles down tile column pc from tile row pr, roles first_role..P-1)
// and its trailing update over the columns right of the panel up to ncols, on
// the view `layout` (0: columns, 1: transposed) of dA: the full-T update for
// tiles >= 128 when w.tfull is given (as in stage1_ge2bnd), else the
// 16-reflector-block one.  The building blocks of the out-of-core driver,
// which runs a half-step as a sequence of such slabs with the top tile row
// carried from slab to slab.
template <typename T>
int stage1_panel(T *dA, int64_t lda, int b, int layout, int pr, int pc, int P, int first_role, const Stage1Work &w,
                 cudaStream_t s) {
    return layout == 0 ? launch_panel<T, 0>(dA, lda, b, pr, pc, P, first_role, w, s)
                       : launch_panel<T, 1>(dA, lda, b, pr, pc, P, first_role, w, s);
}
template <typename T>
int stage1_update(T *dA, int64_t lda, int64_t ncols, int b, int layout, int pr, int pc, int P, int first_role,
                  const Stage1Work &w, cudaStream_t s) {
    if (b >= 128 && w.tfull) return stage1_update_full<T>(dA, lda, ncols, b, layout, pr, pc, P, w, s, first_role);
    return layout == 0 ? launch_update<T, 0>(dA, lda, ncols, b, pr, pc, P, w, s, first_role)
                       : launch_update<T, 1>(dA, lda, ncols, b, pr, pc, P, w, s, first_role);
}
template int stage1_panel<float>(float *, int64_t, int, int, int, int, int, int, const Stage1Work &, cudaStream_t);
template int stage1_panel<double>(double *, int64_t, int, int, int, int, int, int, const Stage1Work &, cudaStream_t);
template int stage1_update<float>(float *, int64_t, int64_t, int, int, int, int, int, int, const Stage1Work &,
                                  cudaStream_t);
template int stage1_update<double>(double *, int64_t, int64_t, int, int, int, int, int, int, const Stage1Work &,
                                   cudaStream_t);

template int stage1_ge2bnd<float>(float *, int64_t, int64_t, int, const Stage1Work &, cudaStream_t, int64_t *);
template int stage1_ge2bnd<double>(double *, int64_t, int64_t, int, const Stage1Work &, cudaStream_t, int64_t *);
template int stage1_geqrt_tile<float>(float *, int, float *, const Stage1Work &, cudaStream_t);
template int stage1_geqrf<float>(float *, int64_t, int64_t, int, const Stage1Work &, float *, cudaStream_t,
                                 int64_t *);
template int stage1_geqrf<double>(double *, int64_t, int64_t, int, const Stage1Work &, double *, cudaStream_t,
                                  int64_t *);
template int stage1_geqrt_tile<double>(double *, int, double *, const Stage1Work &, cudaStream_t);
template int stage1_tsqrt_pair<float>(float *, int, float *, const Stage1Work &, cudaStream_t);
template int stage1_tsqrt_pair<double>(double *, int, double *, const Stage1Work &, cudaStream_t);

}  // namespace avs
