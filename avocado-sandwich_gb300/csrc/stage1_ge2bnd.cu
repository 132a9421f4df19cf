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
// block the 16 reflectors are generated one column at a time with the
// reference's nu/tau formulas (scalars in FP64), their compact-WY factor T
// (16 x 16) is formed, and the block is applied to the rest of the tile with
// it.  Roles are handed out by an atomic ticket in launch order, so a role only
// ever waits on a role already running: no co-residency assumption, and every
// wait is bounded.
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

#include "avs_common.cuh"
#include "df64.cuh"

namespace avs {
namespace {

constexpr int kIB = 16;    // reflectors per compact-WY block
constexpr int kNT = 256;   // threads per CTA (16 columns x 16 row groups)
constexpr int kCW = 32;    // column chunk of the in-panel apply

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
    int *progress;   // [P]
    int *err;
};

struct UpdateArgs {
    void *a;
    int64_t lda;
    int64_t n;
    int b;
    int pr, pc, P;
    int width;  // strip width
    const void *tblk;
};

__host__ __device__ inline int ldpad(int b) { return b + 1; }

template <typename T>
size_t panel_smem_bytes(int b) {
    size_t doubles = 2 * kIB + kIB * kIB + 8;                    // dsum, tau, G, scalars
    size_t ts = (size_t)ldpad(b) * kIB        /* X  */
                + (size_t)kIB * b             /* Rt */
                + (size_t)ldpad(b) * kCW      /* C  */
                + 2 * (size_t)kIB * kCW       /* Z, W */
                + (size_t)kIB * kIB;          /* Tm */
    return doubles * sizeof(double) + ts * sizeof(T);
}

template <typename T, int LAYOUT>
__global__ void __launch_bounds__(kNT) panel_kernel(PanelArgs args) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int b = args.b;
    const int nb = b / kIB;
    const int ldx = ldpad(b);
    double *dsum = reinterpret_cast<double *>(smem_raw);  // kIB
    double *stau = dsum + kIB;                             // kIB
    double *G = stau + kIB;                                // kIB*kIB, G[l + i*kIB]
    double *scal = G + kIB * kIB;                          // 8
    T *X = reinterpret_cast<T *>(scal + 8);                // ldx * kIB
    T *Rt = X + (size_t)ldx * kIB;                         // kIB * b, Rt[l + j*kIB]
    T *C = Rt + (size_t)kIB * b;                           // ldx * kCW
    T *Zs = C + (size_t)ldx * kCW;                         // kIB * kCW
    T *Ws = Zs + kIB * kCW;                                // kIB * kCW
    T *Tm = Ws + kIB * kCW;                                // kIB * kIB, Tm[l + i*kIB]

    __shared__ int s_role, s_ok;
    const int tid = threadIdx.x;
    const int jj = tid >> 4;  // column within the block
    const int g = tid & 15;   // row group
    if (tid == 0) s_role = atomicAdd(args.ticket, 1) + args.first_role;
    __syncthreads();
    const int p = s_role;
    if (p >= args.P) return;

    View<T, LAYOUT> V{reinterpret_cast<T *>(args.a), args.lda};
    const int64_t row0 = (int64_t)(args.pr + p) * b;  // my tile (view rows)
    const int64_t top0 = (int64_t)args.pr * b;        // top tile (view rows)
    const int64_t col0 = (int64_t)args.pc * b;        // panel (view cols)
    const bool geqrt = (p == 0);
    T *tau_out = reinterpret_cast<T *>(args.tau) + (size_t)p * b;
    T *tblk_out = reinterpret_cast<T *>(args.tblk) + (size_t)p * nb * kIB * kIB;
    const int rows_per_g = b / 16;

    for (int cb = 0; cb < nb; ++cb) {
        const int c0 = cb * kIB;
        // ---- wait for the previous role to release block cb of the top rows
        if (tid == 0) {
            bool ok = true;
            if (p > args.first_role) ok = wait_geq(args.progress + p - 1, cb + 1, args.err);
            s_ok = ok;
        }
        __syncthreads();
        if (!s_ok) return;

        // ---- load my 16-column slice (and, for TSQRT, the top rows c0..c0+15)
        for (int idx = tid; idx < b * kIB; idx += kNT) {
            int t, l;
            if (LAYOUT == 0) { t = idx % b; l = idx / b; } else { l = idx % kIB; t = idx / kIB; }
            X[t + l * ldx] = __ldcg(&V(row0 + t, col0 + c0 + l));
        }
        if (!geqrt) {
            const int ncols = b - c0;
            for (int idx = tid; idx < kIB * ncols; idx += kNT) {
                int l, j;
                if (LAYOUT == 0) { l = idx % kIB; j = idx / kIB; } else { j = idx % ncols; l = idx / ncols; }
                Rt[l + (c0 + j) * kIB] = __ldcg(&V(top0 + c0 + l, col0 + c0 + j));
            }
        }
        __syncthreads();

        // ---- 16 reflectors, one column at a time (QRkernels.jl:17-58 / 87-120)
        for (int i = 0; i < kIB; ++i) {
            const int c = c0 + i;  // column (and, for GEQRT, pivot row) in the tile
            if (geqrt && c == b - 1) {  // the reference loops iter = 1:N-1 for GEQRT
                if (tid == 0) { stau[i] = 0.0; }
                __syncthreads();
                continue;
            }
            T xr[16];
            double acc = 0.0;
            T accT = T(0);
            T rv = T(0);
            if (jj >= i) rv = geqrt ? X[c + jj * ldx] : Rt[i + (c0 + jj) * kIB];
#pragma unroll
            for (int m = 0; m < 16; ++m) {
                xr[m] = T(0);
                if (m < rows_per_g) {
                    const int t = g + 16 * m;
                    const bool live = geqrt ? (t > c) : true;
                    xr[m] = live ? X[t + i * ldx] : T(0);
                    if (jj >= i) {
                        if (jj == i) acc += (double)xr[m] * (double)xr[m];
                        else accT += xr[m] * X[t + jj * ldx];
                    }
                }
            }
#pragma unroll
            for (int o = 8; o > 0; o >>= 1) {
                accT += __shfl_xor_sync(0xffffffffu, accT, o);
                acc += __shfl_xor_sync(0xffffffffu, acc, o);
            }
            if (g == 0 && jj >= i) dsum[jj] = (jj == i) ? acc : (double)accT;
            __syncthreads();
            if (tid == 0) {
                const double s = dsum[i];
                const double alpha = geqrt ? (double)X[c + i * ldx] : (double)Rt[i + c * kIB];
                const double n1 = sqrt(s + alpha * alpha);
                const double nu = alpha + (alpha < 0.0 ? -n1 : n1);
                double tv = 0.0;
                if (nu != 0.0) {
                    const double n2 = sqrt(s + nu * nu);
                    const double q = nu / n2;
                    tv = 2.0 * (q * q);
                }
                if (!isfinite(tv) || !isfinite(nu)) { atomicCAS(args.err, kDevOk, kDevNonfinite); tv = 0.0; }
                scal[0] = nu;
                scal[1] = (tv != 0.0) ? 1.0 / nu : 0.0;         // scaling of V
                scal[2] = (tv != 0.0) ? (tv / nu) / nu : 0.0;   // taucorr / nu
                stau[i] = tv;
            }
            __syncthreads();
            const double nu = scal[0];
            const double tv = stau[i];
            const T inv_nu = (T)scal[1];
            const T f_upd = (T)scal[2];
            if (tv == 0.0) {
                // identity reflector: zero column (or the GEQRT tail) -> V column = 0
                if (jj == i) {
                    for (int m = 0; m < rows_per_g; ++m) {
                        const int t = g + 16 * m;
                        if (geqrt ? (t > c) : true) X[t + i * ldx] = T(0);
                    }
                }
                __syncthreads();
                continue;
            }
            const double tc = tv / nu;  // taucorr
            if (jj >= i) {
                const double w = nu * (double)rv + dsum[jj];
                const T wT = (T)w;
                const T fw = f_upd * wT;  // (x_t / nu) * (tau / nu) * w_j = x_t * fw
#pragma unroll
                for (int m = 0; m < 16; ++m) {
                    if (m >= rows_per_g) break;
                    const int t = g + 16 * m;
                    if (geqrt) {
                        if (t > c) {
                            if (jj > i) X[t + jj * ldx] -= xr[m] * fw;
                            else X[t + i * ldx] = xr[m] * inv_nu;
                        } else if (t == c) {
                            X[c + jj * ldx] = (T)((double)rv - tc * w);
                        }
                    } else {
                        if (jj > i) X[t + jj * ldx] -= xr[m] * fw;
                        else X[t + i * ldx] = xr[m] * inv_nu;
                    }
                }
                if (!geqrt && g == 0) Rt[i + (c0 + jj) * kIB] = (T)((double)rv - tc * w);
            }
            __syncthreads();
        }

        // ---- compact-WY factor of the block: G = Y^T Y (strict upper), T recurrence
        {
            const int i = jj;
            for (int l = 0; l < kIB; ++l) {
                double part = 0.0;
                if (l < i) {
                    T pt = T(0);
                    for (int m = 0; m < rows_per_g; ++m) {
                        const int t = g + 16 * m;
                        if (geqrt ? (t > c0 + i) : true) pt += X[t + l * ldx] * X[t + i * ldx];
                    }
                    part = (double)pt;
                }
#pragma unroll
                for (int o = 8; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
                if (g == 0) {
                    if (l < i && geqrt) part += (double)X[c0 + i + l * ldx];  // unit entry of y_i
                    G[l + i * kIB] = (l < i) ? part : 0.0;
                }
            }
        }
        if (tid < kIB * kIB) Tm[tid] = T(0);
        __syncthreads();
        if (tid < kIB) Tm[tid + tid * kIB] = (T)stau[tid];
        __syncthreads();
        for (int i = 1; i < kIB; ++i) {
            if (tid < i) {
                double sacc = 0.0;
                for (int m = tid; m < i; ++m) sacc += (double)Tm[tid + m * kIB] * G[m + i * kIB];
                Tm[tid + i * kIB] = (T)(-stau[i] * sacc);
            }
            __syncthreads();
        }

        // ---- write V (and the block's R rows), tau, T.  GEQRT writes only rows
        // >= c0: rows above are top rows that the next role may be updating.
        for (int idx = tid; idx < b * kIB; idx += kNT) {
            int t, l;
            if (LAYOUT == 0) { t = idx % b; l = idx / b; } else { l = idx % kIB; t = idx / kIB; }
            if (!geqrt || t >= c0) V(row0 + t, col0 + c0 + l) = X[t + l * ldx];
        }
        if (tid < kIB) tau_out[c0 + tid] = (T)stau[tid];
        if (tid < kIB * kIB) tblk_out[(size_t)cb * kIB * kIB + tid] = Tm[tid];

        // ---- apply the block to the rest of the tile (and the top rows), chunked
        for (int j = c0 + kIB; j < b; j += kCW) {
            const int cw = min(kCW, b - j);
            for (int idx = tid; idx < b * cw; idx += kNT) {
                int t, cc;
                if (LAYOUT == 0) { t = idx % b; cc = idx / b; } else { cc = idx % cw; t = idx / cw; }
                C[t + cc * ldx] = __ldcg(&V(row0 + t, col0 + j + cc));
            }
            __syncthreads();
            for (int o = tid; o < kIB * cw; o += kNT) {
                const int l = o % kIB, cc = o / kIB;
                T z = geqrt ? T(0) : Rt[l + (j + cc) * kIB];
                const int tstart = geqrt ? (c0 + l) : 0;
                if (geqrt) z += C[tstart + cc * ldx];  // unit diagonal of Y
                for (int t = geqrt ? tstart + 1 : 0; t < b; ++t) z += X[t + l * ldx] * C[t + cc * ldx];
                Zs[l + cc * kIB] = z;
            }
            __syncthreads();
            for (int o = tid; o < kIB * cw; o += kNT) {
                const int l = o % kIB, cc = o / kIB;
                T w = T(0);
                for (int m = 0; m <= l; ++m) w += Tm[m + l * kIB] * Zs[m + cc * kIB];
                Ws[l + cc * kIB] = w;
                if (!geqrt) Rt[l + (j + cc) * kIB] -= w;
            }
            __syncthreads();
            for (int idx = tid; idx < b * cw; idx += kNT) {
                const int t = idx % b, cc = idx / b;
                T acc2 = T(0);
                if (geqrt) {
                    if (t >= c0) {
                        const int lmax = min(kIB - 1, t - c0);
                        for (int l = 0; l <= lmax; ++l) {
                            const T y = (t == c0 + l) ? T(1) : X[t + l * ldx];
                            acc2 += y * Ws[l + cc * kIB];
                        }
                        C[t + cc * ldx] -= acc2;
                    }
                } else {
#pragma unroll
                    for (int l = 0; l < kIB; ++l) acc2 += X[t + l * ldx] * Ws[l + cc * kIB];
                    C[t + cc * ldx] -= acc2;
                }
            }
            __syncthreads();
            for (int idx = tid; idx < b * cw; idx += kNT) {
                int t, cc;
                if (LAYOUT == 0) { t = idx % b; cc = idx / b; } else { cc = idx % cw; t = idx / cw; }
                if (!geqrt || t >= c0) V(row0 + t, col0 + j + cc) = C[t + cc * ldx];
            }
            __syncthreads();
        }
        if (!geqrt) {
            const int ncols = b - c0;
            for (int idx = tid; idx < kIB * ncols; idx += kNT) {
                int l, jx;
                if (LAYOUT == 0) { l = idx % kIB; jx = idx / kIB; } else { jx = idx % ncols; l = idx / ncols; }
                V(top0 + c0 + l, col0 + c0 + jx) = Rt[l + (c0 + jx) * kIB];
            }
        }
        __syncthreads();
        if (tid == 0) {
            __threadfence();
            st_release(args.progress + p, cb + 1);
        }
    }
}

// ---------------------------------------------------------------------------
// Panel kernel, warp-synchronous reflector generation.
//
// Same roles, systolic schedule, outputs (V in place, tau, 16 x 16 T blocks)
// and arithmetic as panel_kernel, restructured for latency: warp 0 generates
// the 16 reflectors of a block with warp-level synchronisation only; the
// reflector scalars use the closed forms of the reference's expressions
// (n1 = ||x||, nu = alpha + sign(alpha) n1, tau = 2 nu^2 / (s + nu^2) = |nu| / n1,
// tau / nu = sign(nu) / n1, tau / nu^2 = 1 / (n1 |nu|)) evaluated in FP64 for
// FP64 tiles and in double-float for FP32 tiles (GB300 issues FP64 at 1/64 of
// the FP32 rate); the block's Gram matrix uses the whole CTA; the apply to the
// rest of the tile runs four threads per column with the column in registers.

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
    const df64 a = df64{alpha, 0.0f};
    const df64 n1 = df_sqrt(df_add(s, two_prod(alpha, alpha)));
    const bool neg = alpha < 0.0f;
    const df64 nu = neg ? df_sub(a, n1) : df_add(a, n1);
    r.nu = nu.hi + nu.lo;
    if (nu.hi == 0.0f) {
        r.tau = r.tc = r.f = r.inv = 0.0f;
        r.beta = alpha;
        return r;
    }
    const df64 rn1 = df_rcp(n1);
    const df64 anu = nu.hi < 0.0f ? df_neg(nu) : nu;
    const df64 inv = df_rcp(nu);
    const df64 tau = df_mul(anu, rn1);
    const df64 f = df_mul(rn1, inv.hi < 0.0f ? df_neg(inv) : inv);
    r.tau = tau.hi + tau.lo;
    r.tc = nu.hi < 0.0f ? -(rn1.hi + rn1.lo) : (rn1.hi + rn1.lo);
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
    static __device__ __forceinline__ void compute(Acc s, float alpha, float *out) {
        const PScalarsF r = pscal_float(s, alpha);
        out[0] = r.nu; out[1] = r.tc; out[2] = r.f; out[3] = r.inv; out[4] = r.beta; out[5] = r.tau;
    }
};

__device__ __forceinline__ PScalars pscal_df(df64 s, float alpha) {
    PScalars r;
    const df64 a = df64{alpha, 0.0f};
    const df64 n1 = df_sqrt(df_add(s, two_prod(alpha, alpha)));
    const bool neg = alpha < 0.0f;
    const df64 nu = neg ? df_sub(a, n1) : df_add(a, n1);
    r.nu = df_to_double(nu);
    if (nu.hi == 0.0f) {
        r.tau = r.tc = r.f = r.inv = 0.0;
        r.beta = alpha;
        return r;
    }
    const df64 rn1 = df_rcp(n1);
    const df64 anu = nu.hi < 0.0f ? df_neg(nu) : nu;
    const df64 inv = df_rcp(nu);
    r.tau = df_to_double(df_mul(anu, rn1));
    r.tc = df_to_double(nu.hi < 0.0f ? df_neg(rn1) : rn1);
    r.inv = df_to_double(inv);
    r.f = df_to_double(df_mul(rn1, inv.hi < 0.0f ? df_neg(inv) : inv));
    r.beta = df_to_double(neg ? n1 : df_neg(n1));
    return r;
}

template <typename T>
size_t panel2_smem_bytes(int b) {
    return sizeof(T) * 32 /* tau, scalars */ +
           sizeof(T) * ((size_t)ldpad(b) * kIB /* X */ + (size_t)kIB * b /* Rt */ + 2 * kIB * kIB /* Tm, G */ +
                        (size_t)kIB * 33 /* red */ + 2 * kIB /* dsum, wbuf */);
}

template <typename T, int LAYOUT>
__global__ void __launch_bounds__(kNT) panel2_kernel(PanelArgs args) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int b = args.b;
    const int nb = b / kIB;
    const int ldx = ldpad(b);
    T *stau = reinterpret_cast<T *>(smem_raw);             // kIB
    T *scal = stau + kIB;                                  // 16
    T *X = scal + 16;                                      // ldx * kIB
    T *Rt = X + (size_t)ldx * kIB;                         // kIB * b, Rt[l + j*kIB]
    T *Tm = Rt + (size_t)kIB * b;                          // kIB * kIB, Tm[l + i*kIB]
    T *G = Tm + kIB * kIB;                                 // kIB * kIB, G[l + i*kIB]
    T *red = G + kIB * kIB;                                // kIB * 33
    T *dsum = red + kIB * 33;                              // kIB
    T *wbuf = dsum + kIB;                                  // kIB

    __shared__ int s_role, s_ok;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    if (tid == 0) s_role = atomicAdd(args.ticket, 1) + args.first_role;
    __syncthreads();
    const int p = s_role;
    if (p >= args.P) return;

    View<T, LAYOUT> V{reinterpret_cast<T *>(args.a), args.lda};
    const int64_t row0 = (int64_t)(args.pr + p) * b;
    const int64_t top0 = (int64_t)args.pr * b;
    const int64_t col0 = (int64_t)args.pc * b;
    const bool geqrt = (p == 0);
    T *tau_out = reinterpret_cast<T *>(args.tau) + (size_t)p * b;
    T *tblk_out = reinterpret_cast<T *>(args.tblk) + (size_t)p * nb * kIB * kIB;
    const int R = (b + 31) / 32;  // rows per lane in the reflector loop
    const int RQ = b / 4;         // rows per thread in the apply

    for (int cb = 0; cb < nb; ++cb) {
        const int c0 = cb * kIB;
        if (tid == 0) {
            bool ok = true;
            if (p > args.first_role) ok = wait_geq(args.progress + p - 1, cb + 1, args.err);
            s_ok = ok;
        }
        __syncthreads();
        if (!s_ok) return;
        for (int idx = tid; idx < b * kIB; idx += kNT) {
            int t, l;
            if (LAYOUT == 0) { t = idx % b; l = idx / b; } else { l = idx % kIB; t = idx / kIB; }
            X[t + l * ldx] = __ldcg(&V(row0 + t, col0 + c0 + l));
        }
        if (!geqrt) {
            const int ncols = b - c0;
            for (int idx = tid; idx < kIB * ncols; idx += kNT) {
                int l, j;
                if (LAYOUT == 0) { l = idx % kIB; j = idx / kIB; } else { j = idx % ncols; l = idx / ncols; }
                Rt[l + (c0 + j) * kIB] = __ldcg(&V(top0 + c0 + l, col0 + c0 + j));
            }
        }
        __syncthreads();

        // ---- warp 0: the 16 reflectors of the block
        if (wid == 0) {
            for (int i = 0; i < kIB; ++i) {
                const int c = c0 + i;
                if (geqrt && c == b - 1) {  // the reference's GEQRT loops iter = 1:N-1
                    if (lane == 0) stau[i] = T(0);
                    __syncwarp();
                    continue;
                }
                T xr[8];
                T dp[kIB];
#pragma unroll
                for (int jj = 0; jj < kIB; ++jj) dp[jj] = T(0);
                typename PScal<T>::Acc sq = PScal<T>::zero();
#pragma unroll
                for (int r = 0; r < 8; ++r) {
                    xr[r] = T(0);
                    if (r < R) {
                        const int t = lane + 32 * r;
                        const bool live = (t < b) && (geqrt ? (t > c) : true);
                        if (live) {
                            const T x = X[t + i * ldx];
                            xr[r] = x;
                            sq = PScal<T>::sq(x, sq);
#pragma unroll
                            for (int jj = 0; jj < kIB; ++jj)
                                if (jj > i) dp[jj] += x * X[t + jj * ldx];
                        }
                    }
                }
#pragma unroll
                for (int jj = 0; jj < kIB; ++jj) red[jj * 33 + lane] = dp[jj];
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) sq = PScal<T>::shfl_add(sq, o);
                __syncwarp();
                if (lane < kIB && lane > i) {
                    T acc = T(0);
#pragma unroll 8
                    for (int q = 0; q < 32; ++q) acc += red[lane * 33 + q];
                    dsum[lane] = acc;
                }
                if (lane == 0) {
                    const T alpha = geqrt ? X[c + i * ldx] : Rt[i + c * kIB];
                    T out[6];
                    PScal<T>::compute(sq, alpha, out);
                    if (!isfinite(out[5]) || !isfinite(out[0])) {
                        atomicCAS(args.err, kDevOk, kDevNonfinite);
                        out[5] = out[1] = out[2] = out[3] = T(0);
                        out[4] = alpha;
                    }
                    stau[i] = out[5];
                    scal[0] = out[0];
                    scal[1] = out[1];
                    scal[2] = out[2];
                    scal[3] = out[3];
                    scal[4] = out[4];
                }
                __syncwarp();
                if (stau[i] == T(0)) {
#pragma unroll
                    for (int r = 0; r < 8; ++r) {
                        const int t = lane + 32 * r;
                        if (r < R && t < b && (geqrt ? (t > c) : true)) X[t + i * ldx] = T(0);
                    }
                    __syncwarp();
                    continue;
                }
                const T nu = scal[0], tc = scal[1], f = scal[2], inv = scal[3];
                if (lane < kIB && lane > i) {
                    const T rv = geqrt ? X[c + lane * ldx] : Rt[i + (c0 + lane) * kIB];
                    const T w = nu * rv + dsum[lane];
                    wbuf[lane] = w;
                    if (geqrt) X[c + lane * ldx] = rv - tc * w;
                    else Rt[i + (c0 + lane) * kIB] = rv - tc * w;
                }
                if (lane == 0) {
                    if (geqrt) X[c + i * ldx] = scal[4];
                    else Rt[i + c * kIB] = scal[4];
                }
                __syncwarp();
#pragma unroll
                for (int r = 0; r < 8; ++r) {
                    const int t = lane + 32 * r;
                    if (r < R && t < b && (geqrt ? (t > c) : true)) {
                        const T x = xr[r];
#pragma unroll
                        for (int jj = 0; jj < kIB; ++jj)
                            if (jj > i) X[t + jj * ldx] -= x * (f * wbuf[jj]);
                        X[t + i * ldx] = x * inv;
                    }
                }
                __syncwarp();
            }
        }
        __syncthreads();

        // ---- Gram matrix of the block's reflectors (whole CTA), then T (warp 0)
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
            T part = T(0);
            if (l >= 0) {
                const int half = (b + 1) / 2;
                const int tlo = h * half, thi = min(b, tlo + half);
                for (int t = tlo; t < thi; ++t)
                    if (geqrt ? (t > c0 + i) : true) part += X[t + l * ldx] * X[t + i * ldx];
            }
            part += __shfl_xor_sync(0xffffffffu, part, 1);
            if (l >= 0 && h == 0) G[l + i * kIB] = part + (geqrt ? X[c0 + i + l * ldx] : T(0));
        }
        if (tid < kIB * kIB) Tm[tid] = T(0);
        __syncthreads();
        if (wid == 0) {
            if (lane < kIB) Tm[lane + lane * kIB] = stau[lane];
            __syncwarp();
            for (int i = 1; i < kIB; ++i) {
                if (lane < i) {
                    T acc = T(0);
                    for (int m = lane; m < i; ++m) acc += Tm[lane + m * kIB] * G[m + i * kIB];
                    Tm[lane + i * kIB] = -stau[i] * acc;
                }
                __syncwarp();
            }
        }
        __syncthreads();

        // ---- write V, tau, T
        for (int idx = tid; idx < b * kIB; idx += kNT) {
            int t, l;
            if (LAYOUT == 0) { t = idx % b; l = idx / b; } else { l = idx % kIB; t = idx / kIB; }
            if (!geqrt || t >= c0) V(row0 + t, col0 + c0 + l) = X[t + l * ldx];
        }
        if (tid < kIB) tau_out[c0 + tid] = stau[tid];
        if (tid < kIB * kIB) tblk_out[(size_t)cb * kIB * kIB + tid] = Tm[tid];

        // ---- apply the block to the rest of the tile: 4 threads per column
        const int nrest = b - c0 - kIB;
        const int quad = tid >> 2, qq = tid & 3;
        for (int base = 0; base < nrest; base += kNT / 4) {
            const int jrel = base + quad;
            const bool cv = jrel < nrest;
            const int j = c0 + kIB + (cv ? jrel : 0);
            T cr[64];
            T z[kIB];
#pragma unroll
            for (int l = 0; l < kIB; ++l) z[l] = T(0);
#pragma unroll
            for (int r = 0; r < 64; ++r) {
                cr[r] = T(0);
                if (r < RQ) {
                    const int t = qq * RQ + r;
                    if (cv && (!geqrt || t >= c0)) {
                        const T cval = __ldcg(&V(row0 + t, col0 + j));
                        cr[r] = cval;
#pragma unroll
                        for (int l = 0; l < kIB; ++l) {
                            T y;
                            if (geqrt) y = (t == c0 + l) ? T(1) : (t > c0 + l ? X[t + l * ldx] : T(0));
                            else y = X[t + l * ldx];
                            z[l] += y * cval;
                        }
                    }
                }
            }
#pragma unroll
            for (int l = 0; l < kIB; ++l) {
                z[l] += __shfl_xor_sync(0xffffffffu, z[l], 1);
                z[l] += __shfl_xor_sync(0xffffffffu, z[l], 2);
                if (!geqrt && cv) z[l] += Rt[l + j * kIB];
            }
            T w[kIB];
#pragma unroll
            for (int l = 0; l < kIB; ++l) {
                T acc = T(0);
#pragma unroll
                for (int m = 0; m <= l; ++m) acc += Tm[m + l * kIB] * z[m];
                w[l] = acc;
            }
            if (!geqrt && cv) {
#pragma unroll
                for (int l = 0; l < kIB; ++l)
                    if ((l >> 2) == qq) Rt[l + j * kIB] -= w[l];
            }
#pragma unroll
            for (int r = 0; r < 64; ++r) {
                if (r < RQ) {
                    const int t = qq * RQ + r;
                    if (cv && (!geqrt || t >= c0)) {
                        T acc = cr[r];
#pragma unroll
                        for (int l = 0; l < kIB; ++l) {
                            T y;
                            if (geqrt) y = (t == c0 + l) ? T(1) : (t > c0 + l ? X[t + l * ldx] : T(0));
                            else y = X[t + l * ldx];
                            acc -= y * w[l];
                        }
                        V(row0 + t, col0 + j) = acc;
                    }
                }
            }
        }
        __syncthreads();
        if (!geqrt) {
            const int ncols = b - c0;
            for (int idx = tid; idx < kIB * ncols; idx += kNT) {
                int l, jx;
                if (LAYOUT == 0) { l = idx % kIB; jx = idx / kIB; } else { jx = idx % ncols; l = idx / ncols; }
                V(top0 + c0 + l, col0 + c0 + jx) = Rt[l + (c0 + jx) * kIB];
            }
        }
        __syncthreads();
        if (tid == 0) {
            __threadfence();
            st_release(args.progress + p, cb + 1);
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
    View<T, LAYOUT> V{reinterpret_cast<T *>(args.a), args.lda};
    const int64_t top0 = (int64_t)args.pr * b;
    const int64_t col0 = (int64_t)args.pc * b;
    const T *tblk = reinterpret_cast<const T *>(args.tblk);

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
    for (int p = 0; p < args.P; ++p) {
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

template <typename T, int LAYOUT>
int launch_panel(T *dA, int64_t lda, int b, int pr, int pc, int P, int first_role, const Stage1Work &w,
                 cudaStream_t s) {
    static bool attr_set = false;
    const size_t smem = panel2_smem_bytes<T>(b);
    if (!attr_set) {
        AVS_CUDA_TRY(cudaFuncSetAttribute(panel2_kernel<T, LAYOUT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)panel2_smem_bytes<T>(256)));
        attr_set = true;
    }
    AVS_CUDA_TRY(cudaMemsetAsync(w.flags, 0, sizeof(int) * (size_t)(P + 1), s));
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
    panel2_kernel<T, LAYOUT><<<P - first_role, kNT, smem, s>>>(a);
    AVS_CUDA_TRY(cudaGetLastError());
    return AVS_SUCCESS;
}

template <typename T, int LAYOUT>
int launch_update(T *dA, int64_t lda, int64_t n, int b, int pr, int pc, int P, const Stage1Work &w,
                  cudaStream_t s) {
    const int width = sizeof(T) == 8 ? 32 : 64;
    static bool attr_set = false;
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
    a.width = width;
    a.tblk = w.tblk;
    const unsigned grid = (unsigned)((ncols + width - 1) / width);
    update_kernel<T, LAYOUT><<<grid, kNT, update_smem_bytes<T>(b, width), s>>>(a);
    AVS_CUDA_TRY(cudaGetLastError());
    return AVS_SUCCESS;
}

// Tensor-core trailing update: T build (shared with the SIMT path) + the
// tcgen05 GEMM sequence.
template <typename T>
int update_tc_half(T *dA, int64_t lda, int64_t n, int b, int layout, int pr, int pc, int P, const Stage1Work &w,
                   cudaStream_t s) {
    if constexpr (sizeof(T) != 4) {
        return AVS_ERR_INTERNAL;
    } else {
        int rc = stage1_tbuild<T>(dA, lda, b, layout, pr, pc, P, w.tblk, w.tfull, s);
        if (rc != AVS_SUCCESS) return rc;
        return stage1_update_tc(reinterpret_cast<float *>(dA), lda, n, b, layout, pr, pc, P,
                                reinterpret_cast<const float *>(w.tfull), w.tc_S, w.tc_W, w.tc_split, w.err, s);
    }
}

}  // namespace

template <typename T>
int stage1_ge2bnd(T *dA, int64_t n, int64_t lda, int b, const Stage1Work &w, cudaStream_t s, int64_t *launches) {
    const int nt = (int)(n / b);
    int rc;
    for (int k = 0; k < nt; ++k) {
        // QR half-step: GEQRT(k,k) + TSQRT(row,k), Q^T applied to the row panels.
        const int P = nt - k;
        if ((rc = launch_panel<T, 0>(dA, lda, b, k, k, P, 0, w, s)) != AVS_SUCCESS) return rc;
        if (b >= 128 && w.tfull && w.tc_split && sizeof(T) == 4)
            rc = update_tc_half<T>(dA, lda, n, b, 0, k, k, P, w, s);
        else if (b >= 128 && w.tfull)
            rc = stage1_update_full<T>(dA, lda, n, b, 0, k, k, P, w.tblk, w.tfull, s);
        else
            rc = launch_update<T, 0>(dA, lda, n, b, k, k, P, w, s);
        if (rc != AVS_SUCCESS) return rc;
        if (launches) *launches += (k + 1 < nt) ? ((b >= 128 && w.tfull) ? 3 : 2) : 1;
        if (k == nt - 1) break;
        // LQ half-step: the same on the transposed view, top tile (k, k+1).
        const int PL = nt - k - 1;
        if ((rc = launch_panel<T, 1>(dA, lda, b, k + 1, k, PL, 0, w, s)) != AVS_SUCCESS) return rc;
        if (b >= 128 && w.tfull && w.tc_split && sizeof(T) == 4)
            rc = update_tc_half<T>(dA, lda, n, b, 1, k + 1, k, PL, w, s);
        else if (b >= 128 && w.tfull)
            rc = stage1_update_full<T>(dA, lda, n, b, 1, k + 1, k, PL, w.tblk, w.tfull, s);
        else
            rc = launch_update<T, 1>(dA, lda, n, b, k + 1, k, PL, w, s);
        if (rc != AVS_SUCCESS) return rc;
        if (launches) *launches += (b >= 128 && w.tfull) ? 3 : 2;
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

template int stage1_ge2bnd<float>(float *, int64_t, int64_t, int, const Stage1Work &, cudaStream_t, int64_t *);
template int stage1_ge2bnd<double>(double *, int64_t, int64_t, int, const Stage1Work &, cudaStream_t, int64_t *);
template int stage1_geqrt_tile<float>(float *, int, float *, const Stage1Work &, cudaStream_t);
template int stage1_geqrt_tile<double>(double *, int, double *, const Stage1Work &, cudaStream_t);
template int stage1_tsqrt_pair<float>(float *, int, float *, const Stage1Work &, cudaStream_t);
template int stage1_tsqrt_pair<double>(double *, int, double *, const Stage1Work &, cudaStream_t);

}  // namespace avs
