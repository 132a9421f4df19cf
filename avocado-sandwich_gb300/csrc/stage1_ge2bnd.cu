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
    const size_t smem = panel_smem_bytes<T>(b);
    if (!attr_set) {
        AVS_CUDA_TRY(cudaFuncSetAttribute(panel_kernel<T, LAYOUT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)panel_smem_bytes<T>(256)));
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
    panel_kernel<T, LAYOUT><<<P - first_role, kNT, smem, s>>>(a);
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

}  // namespace

template <typename T>
int stage1_ge2bnd(T *dA, int64_t n, int64_t lda, int b, const Stage1Work &w, cudaStream_t s, int64_t *launches) {
    const int nt = (int)(n / b);
    int rc;
    for (int k = 0; k < nt; ++k) {
        // QR half-step: GEQRT(k,k) + TSQRT(row,k), Q^T applied to the row panels.
        const int P = nt - k;
        if ((rc = launch_panel<T, 0>(dA, lda, b, k, k, P, 0, w, s)) != AVS_SUCCESS) return rc;
        if (b >= 128 && w.tfull)
            rc = stage1_update_full<T>(dA, lda, n, b, 0, k, k, P, w.tblk, w.tfull, s);
        else
            rc = launch_update<T, 0>(dA, lda, n, b, k, k, P, w, s);
        if (rc != AVS_SUCCESS) return rc;
        if (launches) *launches += (k + 1 < nt) ? ((b >= 128 && w.tfull) ? 3 : 2) : 1;
        if (k == nt - 1) break;
        // LQ half-step: the same on the transposed view, top tile (k, k+1).
        const int PL = nt - k - 1;
        if ((rc = launch_panel<T, 1>(dA, lda, b, k + 1, k, PL, 0, w, s)) != AVS_SUCCESS) return rc;
        if (b >= 128 && w.tfull)
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
