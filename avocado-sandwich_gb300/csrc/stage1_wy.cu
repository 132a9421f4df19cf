// Stage 1, trailing update with the full compact-WY factor of each tile
// (tiles of 128 and 256).
//
// The reflectors a panel role generated for its tile (GEQRT: b - 1 of them,
// TSQRT: b) are applied to the trailing columns as one block reflector
// Q_p = I - Y_p T_p Y_p^T, in the reference's order (GEQRT first, then the
// TSQRT tiles top to bottom, TiledMatrix.jl:107-113 / QRkernels.jl:131-197):
//
//   GEQRT tile:  Z = Y0^T Top,          W = T0^T Z,  Top -= Y0 W
//   TSQRT tile:  Z = Top + V_p^T A_p,   W = T_p^T Z, Top -= W, A_p -= V_p W
//
// tbuild_kernel forms T_p (b x b, upper triangular) from the 16 x 16 diagonal
// blocks the panel kernel produced and the Gram matrix G = Y_p^T Y_p:
// T[0:c0, J] = -T[0:c0, 0:c0] G[0:c0, J] T_JJ for the column blocks J (FP64
// tiles; in double-float with the double-float updates); tbuild_f32_kernel
// forms the same T for FP32 tiles with T's upper block triangle in shared
// memory.
//
// update_full_kernel: one CTA per column strip keeps the strip of the top tile
// row in shared memory for the whole half-step; each of the three products is
// a register-blocked GEMM (8 rows x CB columns per thread, K = b streamed
// through shared memory in chunks that the next chunk's loads overlap).  FP64
// tiles use 16-column strips when 32-column strips would leave SMs idle; in
// double-float the products accumulate with the compensated dot product.
#include <algorithm>
#include <type_traits>

#include "avs_common.cuh"
#include "df64.cuh"

namespace avs {
namespace {

constexpr int kWIB = 16;     // diagonal block size of T (the panel's compact-WY blocks)
constexpr int kWNT = 256;    // threads per CTA

template <typename T>
struct WCfg {
    static constexpr int W = sizeof(T) == 8 ? 32 : 64;   // strip width
    static constexpr int KC = sizeof(T) == 8 ? 8 : 16;   // K chunk
};

struct TBuildArgs {
    const void *a;
    int64_t lda;
    int b;
    int pr, pc, P;
    const void *tblk;  // [P][b/16][256]
    void *tfull;       // [P][b*b], T(l, i) at l + i*b
    int64_t sA, sTblk, sTfull;  // per-matrix strides (blockIdx.y = matrix)
    int first_role;    // tiles first_role..P-1 (1: the top tile's T was built earlier)
};

// ---------------------------------------------------------------------------
// T build.  One CTA per tile.
template <typename T, int LAYOUT, typename CT = T>
__global__ void __launch_bounds__(kWNT) tbuild_kernel(TBuildArgs args) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int b = args.b;
    const int nb = b / kWIB;
    const int p = blockIdx.x + args.first_role;
    const int64_t zb = blockIdx.y;
    const bool geqrt = (p == 0);
    const int tid = threadIdx.x;
    View<const T, LAYOUT> V{reinterpret_cast<const T *>(args.a) + zb * args.sA, args.lda};
    const int64_t row0 = (int64_t)(args.pr + p) * b;
    const int64_t col0 = (int64_t)args.pc * b;
    T *Tf = reinterpret_cast<T *>(args.tfull) + zb * args.sTfull + (size_t)p * b * b;
    const T *tb = reinterpret_cast<const T *>(args.tblk) + zb * args.sTblk + (size_t)p * nb * kWIB * kWIB;

    // ---- 1. G(l, i) = y_l^CT y_i for l < i in different 16-blocks, into Tf
    constexpr int KC = 32;
    CT *chunk = reinterpret_cast<CT *>(smem_raw);  // KC x (b + 1)
    const int ldc = b + 1;
    // 4 x 4 micro-blocks (lb, ib) of G with block16(lb*4) < block16(ib*4)
    const int nmb = b / 4;
    int total = 0;
    for (int ib = 0; ib < nmb; ++ib) total += (ib * 4 / kWIB) * (kWIB / 4);
    for (int base = 0; base < total; base += kWNT) {
        // locate this thread's micro-block (lb, ib)
        int my = base + tid, lb = -1, ibk = -1;
        if (my < total) {
            int acc = 0;
            for (int ib = 0; ib < nmb; ++ib) {
                const int cnt = (ib * 4 / kWIB) * (kWIB / 4);
                if (my < acc + cnt) { ibk = ib; lb = my - acc; break; }
                acc += cnt;
            }
        }
        CT g[4][4];
#pragma unroll
        for (int x = 0; x < 4; ++x)
#pragma unroll
            for (int y = 0; y < 4; ++y) g[x][y] = CT(0);
        for (int k0 = 0; k0 < b; k0 += KC) {
            __syncthreads();
            for (int idx = tid; idx < KC * b; idx += kWNT) {
                int k, m;
                if (LAYOUT == 0) { k = idx % KC; m = idx / KC; } else { m = idx % b; k = idx / b; }
                const int t = k0 + k;
                CT v = CT(V(row0 + t, col0 + m));
                if (geqrt) v = (t == m) ? CT(1) : (t > m ? v : CT(0));
                chunk[k * ldc + m] = v;
            }
            __syncthreads();
            if (lb >= 0) {
                for (int k = 0; k < KC; ++k) {
                    CT a[4], c[4];
#pragma unroll
                    for (int x = 0; x < 4; ++x) a[x] = chunk[k * ldc + lb * 4 + x];
#pragma unroll
                    for (int y = 0; y < 4; ++y) c[y] = chunk[k * ldc + ibk * 4 + y];
#pragma unroll
                    for (int x = 0; x < 4; ++x)
#pragma unroll
                        for (int y = 0; y < 4; ++y) g[x][y] += a[x] * c[y];
                }
            }
        }
        if (lb >= 0) {
#pragma unroll
            for (int x = 0; x < 4; ++x)
#pragma unroll
                for (int y = 0; y < 4; ++y) Tf[(lb * 4 + x) + (size_t)(ibk * 4 + y) * b] = (T)g[x][y];
        }
    }
    __syncthreads();
    // ---- 2. diagonal blocks and zeros below them; first column block
    for (int idx = tid; idx < b * b; idx += kWNT) {
        const int l = idx % b, i = idx / b;
        const int bl = l / kWIB, bi = i / kWIB;
        if (bl == bi) Tf[l + (size_t)i * b] = tb[(size_t)bi * kWIB * kWIB + (l % kWIB) + (i % kWIB) * kWIB];
        else if (bl > bi) Tf[l + (size_t)i * b] = T(0);
    }
    __syncthreads();
    // ---- 3. column blocks J = 1..nb-1: CT[0:c0, J] = -CT[0:c0,0:c0] G[0:c0, J] T_JJ.
    // G's block (in Tf's column block J) and T_JJ are staged in shared memory;
    // thread r owns row r: 16 accumulators over m (CT upper triangular, zeros
    // below the diagonal), one coalesced load of CT(r, m) per m, then the 16 x 16
    // product with T_JJ in registers.
    CT *Gs = chunk;              // c0 x kWIB, Gs[m * kWIB + q]
    CT *TJ = Gs + b * kWIB;      // kWIB x kWIB, TJ[qq + q * kWIB]
    for (int J = 1; J < nb; ++J) {
        const int c0 = J * kWIB;
        for (int idx = tid; idx < c0 * kWIB; idx += kWNT) {
            const int m = idx % c0, q = idx / c0;
            Gs[m * kWIB + q] = CT(Tf[m + (size_t)(c0 + q) * b]);
        }
        for (int idx = tid; idx < kWIB * kWIB; idx += kWNT) TJ[idx] = CT(tb[(size_t)J * kWIB * kWIB + idx]);
        __syncthreads();
        const int r = tid;
        if (r < c0) {
            CT acc[kWIB];
#pragma unroll
            for (int q = 0; q < kWIB; ++q) acc[q] = CT(0);
#pragma unroll 8
            for (int m = 0; m < c0; ++m) {
                const CT t = CT(Tf[r + (size_t)m * b]);
#pragma unroll
                for (int q = 0; q < kWIB; ++q) acc[q] += t * Gs[m * kWIB + q];
            }
#pragma unroll
            for (int q = 0; q < kWIB; ++q) {
                CT v = CT(0);
#pragma unroll
                for (int qq = 0; qq < kWIB; ++qq) v += acc[qq] * TJ[qq + q * kWIB];
                Tf[r + (size_t)(c0 + q) * b] = (T)(-v);
            }
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// T build in shared memory (FP32 tiles).  One CTA per tile, the same T as
// tbuild_kernel with T's upper block triangle held in shared memory, packed by
// 16-column blocks (column block J: rows 0 .. 16(J+1), column-major, at
// offset 256 J (J+1) / 2):
//   1. the Gram blocks G_IJ = Y_I^T Y_J (I < J) in two passes over the tile's
//      rows (8 x 8 output tiles per thread, rows of Y staged 32 at a time with
//      the next chunk's loads in flight during the current chunk's products),
//      written straight into their places in the packed T;
//   2. the diagonal blocks T_JJ from the panel;
//   3. column blocks J = 1.. in order: H = G[0:c0, J] T_JJ, then
//      T[0:c0, J] = -T[0:c0, 0:c0] H, one thread per row, every operand in
//      shared memory (the recurrence is latency-bound when it reads T back
//      from global memory);
//   4. T to tfull (zeros below the diagonal blocks), coalesced.
constexpr int kTbKC = 32;  // rows of Y per staged chunk

__host__ __device__ constexpr int tb_off(int J) { return 256 * J * (J + 1) / 2; }
inline size_t tbuild_f32_smem(int b) {
    const int nb = b / kWIB;
    return sizeof(float) * ((size_t)tb_off(nb) + (size_t)kTbKC * (b + 4));
}

template <int LAYOUT>
__global__ void __launch_bounds__(kWNT) tbuild_f32_kernel(TBuildArgs args) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int b = args.b;
    const int nb = b / kWIB;
    const int p = blockIdx.x + args.first_role;
    const int64_t zb = blockIdx.y;
    const bool geqrt = (p == 0);
    const int tid = threadIdx.x;
    View<const float, LAYOUT> V{reinterpret_cast<const float *>(args.a) + zb * args.sA, args.lda};
    const int64_t row0 = (int64_t)(args.pr + p) * b;
    const int64_t col0 = (int64_t)args.pc * b;
    float *Tf = reinterpret_cast<float *>(args.tfull) + zb * args.sTfull + (size_t)p * b * b;
    const float *tb = reinterpret_cast<const float *>(args.tblk) + zb * args.sTblk + (size_t)p * nb * kWIB * kWIB;
    float *Tp = reinterpret_cast<float *>(smem_raw);  // packed upper block triangle
    float *ch = Tp + tb_off(nb);                        // [kTbKC][b + 4] rows of Y, then H
    const int ldc = b + 4;
    auto tp = [&](int r, int i) -> float & {  // T(r, i), r < 16 (i / 16 + 1)
        const int J = i / kWIB;
        return Tp[tb_off(J) + (i % kWIB) * (kWIB * (J + 1)) + r];
    };

    // ---- 1. Gram blocks
    const int ntiles = 2 * nb * (nb - 1);  // 8 x 8 tiles: 4 per block pair
    const int per = kTbKC * b / kWNT;      // staged values per thread and chunk
    for (int base = 0; base < ntiles; base += kWNT) {
        const int u = base + tid;
        int l0 = -1, i0 = -1;
        if (u < ntiles) {
            const int pair = u >> 2;
            int J = 1;
            while (J * (J + 1) / 2 <= pair) ++J;
            const int I = pair - J * (J - 1) / 2;
            l0 = I * kWIB + 8 * ((u >> 1) & 1);
            i0 = J * kWIB + 8 * (u & 1);
        }
        float g[8][8];
#pragma unroll
        for (int x = 0; x < 8; ++x)
#pragma unroll
            for (int y = 0; y < 8; ++y) g[x][y] = 0.0f;
        // staged value e of this thread: (k, m) = (k_0 + e dk, m_0 + e dm), one
        // pointer stepped by a fixed stride (coalesced along the tile's storage)
        const int k_0 = (LAYOUT == 0) ? tid % kTbKC : tid / b;
        const int m_0 = (LAYOUT == 0) ? tid / kTbKC : tid % b;
        const int dk = (LAYOUT == 0) ? 0 : kWNT / b;
        const int dm = (LAYOUT == 0) ? kWNT / kTbKC : 0;
        const int64_t dp = (LAYOUT == 0) ? (int64_t)dm * args.lda : (int64_t)dk * args.lda;
        float nx[32];
        auto fetch = [&](int k0) {
            const float *ptr = &V(row0 + k0 + k_0, col0 + m_0);
#pragma unroll
            for (int e = 0; e < 32; ++e) {
                if (e < per) {
                    float v = __ldcg(ptr + e * dp);
                    if (geqrt) {
                        const int t = k0 + k_0 + e * dk, m = m_0 + e * dm;
                        v = (t == m) ? 1.0f : (t > m ? v : 0.0f);
                    }
                    nx[e] = v;
                }
            }
        };
        fetch(0);
        for (int k0 = 0; k0 < b; k0 += kTbKC) {
            __syncthreads();  // the previous chunk's products are done
#pragma unroll
            for (int e = 0; e < 32; ++e)
                if (e < per) ch[(k_0 + e * dk) * ldc + m_0 + e * dm] = nx[e];
            __syncthreads();
            if (k0 + kTbKC < b) fetch(k0 + kTbKC);
            if (l0 >= 0) {
#pragma unroll 4
                for (int k = 0; k < kTbKC; ++k) {
                    const float4 a0 = *reinterpret_cast<const float4 *>(ch + k * ldc + l0);
                    const float4 a1 = *reinterpret_cast<const float4 *>(ch + k * ldc + l0 + 4);
                    const float4 c0 = *reinterpret_cast<const float4 *>(ch + k * ldc + i0);
                    const float4 c1 = *reinterpret_cast<const float4 *>(ch + k * ldc + i0 + 4);
                    const float a[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
                    const float c[8] = {c0.x, c0.y, c0.z, c0.w, c1.x, c1.y, c1.z, c1.w};
#pragma unroll
                    for (int x = 0; x < 8; ++x)
#pragma unroll
                        for (int y = 0; y < 8; ++y) g[x][y] = fmaf(a[x], c[y], g[x][y]);
                }
            }
        }
        if (l0 >= 0) {
#pragma unroll
            for (int y = 0; y < 8; ++y)
#pragma unroll
                for (int x = 0; x < 8; ++x) tp(l0 + x, i0 + y) = g[x][y];
        }
    }
    // ---- 2. diagonal blocks
    for (int idx = tid; idx < nb * kWIB * kWIB; idx += kWNT) {
        const int J = idx / (kWIB * kWIB), e = idx % (kWIB * kWIB), r = e % kWIB, q = e / kWIB;
        tp(J * kWIB + r, J * kWIB + q) = tb[idx];
    }
    __syncthreads();
    // ---- 3. column blocks
    float *H = ch;  // [c0][16]
    for (int J = 1; J < nb; ++J) {
        const int c0 = J * kWIB;
        const int r = tid;
        if (r < c0) {  // H[r] = G[r, J] T_JJ (T_JJ upper triangular)
            float gq[kWIB], h[kWIB];
#pragma unroll
            for (int q = 0; q < kWIB; ++q) gq[q] = tp(r, c0 + q);
#pragma unroll
            for (int q = 0; q < kWIB; ++q) {
                float v = 0.0f;
#pragma unroll
                for (int qq = 0; qq <= q; ++qq) v = fmaf(gq[qq], tp(c0 + qq, c0 + q), v);
                h[q] = v;
            }
#pragma unroll
            for (int q = 0; q < kWIB; q += 4)
                *reinterpret_cast<float4 *>(H + r * kWIB + q) = make_float4(h[q], h[q + 1], h[q + 2], h[q + 3]);
        }
        __syncthreads();
        if (r < c0) {  // T[r, J] = -sum_{m >= block start of r} T(r, m) H[m]
            float acc[kWIB];
#pragma unroll
            for (int q = 0; q < kWIB; ++q) acc[q] = 0.0f;
            for (int m = (r / kWIB) * kWIB; m < c0; ++m) {
                const float t = tp(r, m);
                const float4 *hm = reinterpret_cast<const float4 *>(H + m * kWIB);
#pragma unroll
                for (int q4 = 0; q4 < kWIB / 4; ++q4) {
                    const float4 hv = hm[q4];
                    acc[4 * q4] = fmaf(t, hv.x, acc[4 * q4]);
                    acc[4 * q4 + 1] = fmaf(t, hv.y, acc[4 * q4 + 1]);
                    acc[4 * q4 + 2] = fmaf(t, hv.z, acc[4 * q4 + 2]);
                    acc[4 * q4 + 3] = fmaf(t, hv.w, acc[4 * q4 + 3]);
                }
            }
#pragma unroll
            for (int q = 0; q < kWIB; ++q) tp(r, c0 + q) = -acc[q];
        }
        __syncthreads();
    }
    // ---- 4. out, zeros below the diagonal blocks
    for (int idx = tid; idx < b * b; idx += kWNT) {
        const int l = idx % b, i = idx / b;
        Tf[l + (size_t)i * b] = (l < kWIB * (i / kWIB + 1)) ? tp(l, i) : 0.0f;
    }
}

// ---------------------------------------------------------------------------
// Trailing update with full T.
struct UpdFullArgs {
    void *a;
    int64_t lda;
    int64_t n;
    int b;
    int pr, pc, P;
    const void *tfull;
    int64_t sA, sTfull;  // per-matrix strides (blockIdx.y = matrix)
    int first_role;      // 1: the top tile's own reflectors were applied earlier
};

// A-operand sources for the three products.
enum ASrc { kVrows = 0, kTrows = 1, kVcols = 2 };

template <typename T, int B, int WW = WCfg<T>::W>
struct UCfg {
    static constexpr int W = WW;
    static constexpr int KC = WCfg<T>::KC;
    static constexpr int MB = 8;                  // rows per thread
    static constexpr int TM = B / MB;             // threads along rows
    static constexpr int TC = kWNT / TM;          // threads along columns
    static constexpr int CB = W / TC;             // columns per thread
    static constexpr int LDB = B + 4;             // leading dimension of strip buffers (rows)
    static constexpr int LDC = B + 4;             // leading dimension of A chunks (m)
    static constexpr int PER = KC * B / kWNT;     // chunk elements per thread
    static_assert(CB >= 1 && PER >= 1, "update configuration");
};

// T: element type in memory; CT: compute type (T itself, or dfx for FP64 data
// updated in double-float arithmetic).
template <typename T, int LAYOUT, int B, int WW = WCfg<T>::W, typename CT = T>
struct UpdCtx {
    using C = UCfg<T, B, WW>;
    View<T, LAYOUT> V;
    const T *Tf;      // T of the current tile, ld B
    int64_t row0, col0;
    bool geqrt;
    // element (k, m) of the A operand for source s (chunk-relative k0 added by caller)
    __device__ __forceinline__ CT a_elem(int s, int k, int m) const {
        if (s == kVrows) {  // V(k, m): Z = V^T ...
            if (geqrt && k <= m) return (k == m) ? CT(1) : CT(0);
            return CT(V(row0 + k, col0 + m));
        } else if (s == kTrows) {  // T(k, m)
            return CT(Tf[k + (size_t)m * B]);
        } else {  // V(m, k): ... -= V W
            if (geqrt && m <= k) return (m == k) ? CT(1) : CT(0);
            return CT(V(row0 + m, col0 + k));
        }
    }
    // chunk element index -> (k, m), coalesced for the source
    __device__ __forceinline__ void map(int s, int idx, int &k, int &m) const {
        const bool kfast = (s == kTrows) || (s == kVrows && LAYOUT == 0) || (s == kVcols && LAYOUT == 1);
        if (kfast) { k = idx % C::KC; m = idx / C::KC; } else { m = idx % B; k = idx / B; }
    }
};

// acc (+|-)= A(k, m)^T-view ... : acc[i][j] += sign * sum_k A(k, m0+i) * Bop(k, c0+j)
template <typename T, int LAYOUT, int B, int WW = WCfg<T>::W, typename CT = T>
__device__ __forceinline__ void gemm(const UpdCtx<T, LAYOUT, B, WW, CT> &ctx, int src,
                                     CT (&acc)[8][UCfg<T, B, WW>::CB], const CT *Bop, CT *chunk0, CT *chunk1,
                                     bool neg) {
    using C = UCfg<T, B, WW>;
    const int tid = threadIdx.x;
    const int m0 = tid % C::TM;  // rows m0 + TM*i: consecutive lanes, consecutive rows
    const int c0 = (tid / C::TM) * C::CB;
    CT pre[C::PER];
    // prologue: chunk 0 into registers
#pragma unroll
    for (int e = 0; e < C::PER; ++e) {
        int k, m;
        ctx.map(src, tid + e * kWNT, k, m);
        pre[e] = ctx.a_elem(src, k, m);
    }
    CT *bufs[2] = {chunk0, chunk1};
    const int nchunk = B / C::KC;
    for (int ch = 0; ch < nchunk; ++ch) {
        CT *cur = bufs[ch & 1];
#pragma unroll
        for (int e = 0; e < C::PER; ++e) {
            int k, m;
            ctx.map(src, tid + e * kWNT, k, m);
            cur[k * C::LDC + m] = pre[e];
        }
        __syncthreads();
        if (ch + 1 < nchunk) {
            const int k0n = (ch + 1) * C::KC;
#pragma unroll
            for (int e = 0; e < C::PER; ++e) {
                int k, m;
                ctx.map(src, tid + e * kWNT, k, m);
                pre[e] = ctx.a_elem(src, k0n + k, m);
            }
        }
        const int k0 = ch * C::KC;
        if constexpr (std::is_same<CT, dfx>::value) {
            // double-float: compensated accumulation (Dot2, Ogita-Rump-Oishi) on
            // the pairs (s, c) = (acc.hi, acc.lo): the product's error terms and
            // the sum's rounding error go to c, renormalised once per call below
#pragma unroll 4
            for (int k = 0; k < C::KC; ++k) {
                CT av[8], bv[C::CB];
#pragma unroll
                for (int i = 0; i < 8; ++i) av[i] = cur[k * C::LDC + m0 + C::TM * i];
#pragma unroll
                for (int j = 0; j < C::CB; ++j) {
                    bv[j] = Bop[(k0 + k) + (c0 + j) * C::LDB];
                    if (neg) bv[j] = -bv[j];
                }
#pragma unroll
                for (int i = 0; i < 8; ++i)
#pragma unroll
                    for (int j = 0; j < C::CB; ++j) {
                        const df64 x = av[i].v, y = bv[j].v;
                        const float pr = __fmul_rn(x.hi, y.hi);
                        float ep = __fmaf_rn(x.hi, y.hi, -pr);
                        ep = __fmaf_rn(x.hi, y.lo, ep);
                        ep = __fmaf_rn(x.lo, y.hi, ep);
                        df64 &a = acc[i][j].v;
                        const float t = __fadd_rn(a.hi, pr);
                        const float z = __fsub_rn(t, a.hi);
                        const float es = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(t, z)), __fsub_rn(pr, z));
                        a.hi = t;
                        a.lo = __fadd_rn(a.lo, __fadd_rn(es, ep));
                    }
            }
            continue;
        }
#pragma unroll 4
        for (int k = 0; k < C::KC; ++k) {
            CT av[8], bv[C::CB];
#pragma unroll
            for (int i = 0; i < 8; ++i) av[i] = cur[k * C::LDC + m0 + C::TM * i];
#pragma unroll
            for (int j = 0; j < C::CB; ++j) bv[j] = Bop[(k0 + k) + (c0 + j) * C::LDB];
            if (neg) {
#pragma unroll
                for (int i = 0; i < 8; ++i)
#pragma unroll
                    for (int j = 0; j < C::CB; ++j) acc[i][j] -= av[i] * bv[j];
            } else {
#pragma unroll
                for (int i = 0; i < 8; ++i)
#pragma unroll
                    for (int j = 0; j < C::CB; ++j) acc[i][j] += av[i] * bv[j];
            }
        }
    }
    if constexpr (std::is_same<CT, dfx>::value) {
#pragma unroll
        for (int i = 0; i < 8; ++i)
#pragma unroll
            for (int j = 0; j < C::CB; ++j) acc[i][j].v = two_sum(acc[i][j].v.hi, acc[i][j].v.lo);
    }
    __syncthreads();
}

template <typename T, int LAYOUT, int B, typename CT = T, int WW = WCfg<T>::W>
__global__ void __launch_bounds__(kWNT) update_full_kernel(UpdFullArgs args) {
    using C = UCfg<T, B, WW>;
    static_assert(sizeof(CT) == sizeof(T), "compute type of the element's size");
    extern __shared__ __align__(16) unsigned char smem_raw[];
    CT *Top = reinterpret_cast<CT *>(smem_raw);    // LDB x W, column-major
    CT *Buf = Top + (size_t)C::LDB * C::W;         // LDB x W
    CT *ch0 = Buf + (size_t)C::LDB * C::W;         // KC x LDC
    CT *ch1 = ch0 + (size_t)C::KC * C::LDC;
    const int tid = threadIdx.x;
    const int64_t j0 = (int64_t)(args.pc + 1) * B + (int64_t)blockIdx.x * C::W;
    const int wc = (int)min((int64_t)C::W, args.n - j0);
    if (wc <= 0) return;
    const int64_t zb = blockIdx.y;
    View<T, LAYOUT> V{reinterpret_cast<T *>(args.a) + zb * args.sA, args.lda};
    const int64_t top0 = (int64_t)args.pr * B;
    const int m0 = tid % C::TM;
    const int c0 = (tid / C::TM) * C::CB;

    auto load_strip = [&](CT *S, int64_t r0) {
        for (int idx = tid; idx < B * C::W; idx += kWNT) {
            int t, c;
            if (LAYOUT == 0) { t = idx % B; c = idx / B; } else { c = idx % C::W; t = idx / C::W; }
            S[t + c * C::LDB] = (c < wc) ? CT(V(r0 + t, j0 + c)) : CT(0);
        }
    };
    auto store_strip = [&](const CT *S, int64_t r0) {
        for (int idx = tid; idx < B * C::W; idx += kWNT) {
            int t, c;
            if (LAYOUT == 0) { t = idx % B; c = idx / B; } else { c = idx % C::W; t = idx / C::W; }
            if (c < wc) V(r0 + t, j0 + c) = (T)S[t + c * C::LDB];
        }
    };
    auto get_blk = [&](const CT *S, CT (&r)[8][C::CB]) {
#pragma unroll
        for (int i = 0; i < 8; ++i)
#pragma unroll
            for (int j = 0; j < C::CB; ++j) r[i][j] = S[(m0 + C::TM * i) + (c0 + j) * C::LDB];
    };
    auto put_blk = [&](CT *S, const CT (&r)[8][C::CB]) {
#pragma unroll
        for (int i = 0; i < 8; ++i)
#pragma unroll
            for (int j = 0; j < C::CB; ++j) S[(m0 + C::TM * i) + (c0 + j) * C::LDB] = r[i][j];
    };
    auto zero = [&](CT (&r)[8][C::CB]) {
#pragma unroll
        for (int i = 0; i < 8; ++i)
#pragma unroll
            for (int j = 0; j < C::CB; ++j) r[i][j] = CT(0);
    };

    load_strip(Top, top0);
    __syncthreads();
    CT acc[8][C::CB];
    CT apr[8][C::CB];
    for (int p = args.first_role; p < args.P; ++p) {
        UpdCtx<T, LAYOUT, B, WW, CT> ctx;
        ctx.V = V;
        ctx.Tf = reinterpret_cast<const T *>(args.tfull) + zb * args.sTfull + (size_t)p * B * B;
        ctx.row0 = (int64_t)(args.pr + p) * B;
        ctx.col0 = (int64_t)args.pc * B;
        ctx.geqrt = (p == 0);
        if (p == 0) {
            zero(acc);
            gemm(ctx, kVrows, acc, Top, ch0, ch1, false);   // Z = Y0^T Top
            put_blk(Buf, acc);
            __syncthreads();
            zero(acc);
            gemm(ctx, kTrows, acc, Buf, ch0, ch1, false);   // W = T0^T Z
            put_blk(Buf, acc);
            __syncthreads();
            get_blk(Top, acc);
            gemm(ctx, kVcols, acc, Buf, ch0, ch1, true);    // Top -= Y0 W
            put_blk(Top, acc);
            __syncthreads();
        } else {
            load_strip(Buf, ctx.row0);
            __syncthreads();
            get_blk(Top, acc);
            gemm(ctx, kVrows, acc, Buf, ch0, ch1, false);   // Z = Top + V^T A_p
            get_blk(Buf, apr);
            __syncthreads();
            put_blk(Buf, acc);
            __syncthreads();
            zero(acc);
            gemm(ctx, kTrows, acc, Buf, ch0, ch1, false);   // W = T^T Z
            {
                CT tp[8][C::CB];
                get_blk(Top, tp);
#pragma unroll
                for (int i = 0; i < 8; ++i)
#pragma unroll
                    for (int j = 0; j < C::CB; ++j) tp[i][j] -= acc[i][j];
                put_blk(Top, tp);                                             // Top -= W
            }
            put_blk(Buf, acc);
            __syncthreads();
            gemm(ctx, kVcols, apr, Buf, ch0, ch1, true);    // A_p -= V W
            put_blk(Buf, apr);
            __syncthreads();
            store_strip(Buf, ctx.row0);
            __syncthreads();
        }
    }
    store_strip(Top, top0);
}

template <typename T, int B, int WW = WCfg<T>::W>
size_t upd_full_smem() {
    using C = UCfg<T, B, WW>;
    return sizeof(T) * (2 * (size_t)C::LDB * C::W + 2 * (size_t)C::KC * C::LDC);
}

template <typename T, int LAYOUT, int B, typename CT = T, int WW = WCfg<T>::W>
int launch_upd_full(T *dA, int64_t lda, int64_t n, int pr, int pc, int P, const Stage1Work &w, cudaStream_t s,
                    int first_role) {
    using C = UCfg<T, B, WW>;
    static std::atomic<bool> attr{false};
    const size_t smem = upd_full_smem<T, B, WW>();
    if (!attr) {
        AVS_CUDA_TRY(cudaFuncSetAttribute(update_full_kernel<T, LAYOUT, B, CT, WW>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        attr = true;
    }
    const int64_t ncols = n - (int64_t)(pc + 1) * B;
    if (ncols <= 0) return AVS_SUCCESS;
    UpdFullArgs a{dA, lda, n, B, pr, pc, P, w.tfull, w.sA, w.sTfull, first_role};
    const unsigned gx = (unsigned)((ncols + C::W - 1) / C::W);
    update_full_kernel<T, LAYOUT, B, CT, WW><<<dim3(gx, w.batch > 0 ? w.batch : 1), kWNT, smem, s>>>(a);
    AVS_CUDA_TRY(cudaGetLastError());
    return AVS_SUCCESS;
}

// FP64 tiles: the update in FP64, or in double-float when the work asks for it.
// FP64 tiles: 32-column strips, or 16 when the 32-column strips (times the
// batch) would not give every SM two CTAs -- a strip runs its P tiles in
// sequence, so the strips are the launch's only parallelism.  A column's values
// do not depend on the strip width (columns are independent, the sums run in
// the same order), so single and batched calls agree bit for bit.
template <typename T, int LAYOUT, int B>
int launch_upd_full_any(T *dA, int64_t lda, int64_t n, int pr, int pc, int P, const Stage1Work &w, cudaStream_t s,
                        int first_role) {
    if constexpr (sizeof(T) == 8) {
        static int sms = 0;
        if (sms == 0) {
            int dev = 0;
            AVS_CUDA_TRY(cudaGetDevice(&dev));
            AVS_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        }
        const int64_t ncols = n - (int64_t)(pc + 1) * B;
        const bool narrow = ((ncols + 31) / 32) * (int64_t)(w.batch > 0 ? w.batch : 1) < 2 * (int64_t)sms;
        if (w.df_update)
            return narrow ? launch_upd_full<T, LAYOUT, B, dfx, 16>(dA, lda, n, pr, pc, P, w, s, first_role)
                          : launch_upd_full<T, LAYOUT, B, dfx>(dA, lda, n, pr, pc, P, w, s, first_role);
        return narrow ? launch_upd_full<T, LAYOUT, B, T, 16>(dA, lda, n, pr, pc, P, w, s, first_role)
                      : launch_upd_full<T, LAYOUT, B>(dA, lda, n, pr, pc, P, w, s, first_role);
    }
    return launch_upd_full<T, LAYOUT, B>(dA, lda, n, pr, pc, P, w, s, first_role);
}

template <typename T, int LAYOUT>
int launch_tbuild(const T *dA, int64_t lda, int b, int pr, int pc, int P, const Stage1Work &w, cudaStream_t s,
                  int first_role = 0) {
    if constexpr (sizeof(T) == 4) {
        static std::atomic<bool> attr32{false};
        if (!attr32) {
            AVS_CUDA_TRY(cudaFuncSetAttribute(tbuild_f32_kernel<LAYOUT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)tbuild_f32_smem(256)));
            attr32 = true;
        }
        TBuildArgs a{dA, lda, b, pr, pc, P, w.tblk, w.tfull, w.sA, w.sTblk, w.sTfull, first_role};
        tbuild_f32_kernel<LAYOUT><<<dim3(P - first_role, w.batch > 0 ? w.batch : 1), kWNT, tbuild_f32_smem(b), s>>>(a);
        AVS_CUDA_TRY(cudaGetLastError());
        return AVS_SUCCESS;
    }
    static std::atomic<bool> attr{false};
    const size_t smem = sizeof(T) * (size_t)32 * (256 + 1) > sizeof(T) * (size_t)256 * 256 / 16
                            ? sizeof(T) * (size_t)32 * (256 + 1)
                            : sizeof(T) * (size_t)256 * 16;
    if (!attr) {
        AVS_CUDA_TRY(
            cudaFuncSetAttribute(tbuild_kernel<T, LAYOUT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        if constexpr (sizeof(T) == 8)
            AVS_CUDA_TRY(cudaFuncSetAttribute(tbuild_kernel<T, LAYOUT, dfx>,
                                              cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        attr = true;
    }
    TBuildArgs a{dA, lda, b, pr, pc, P, w.tblk, w.tfull, w.sA, w.sTblk, w.sTfull, first_role};
    if constexpr (sizeof(T) == 8) {
        // FP64 tiles with the double-float updates: the T build in double-float
        // too (FP64 storage; GB300 issues FP64 at 1/64 of the FP32 rate)
        if (w.df_update) {
            tbuild_kernel<T, LAYOUT, dfx><<<dim3(P - first_role, w.batch > 0 ? w.batch : 1), kWNT, smem, s>>>(a);
            AVS_CUDA_TRY(cudaGetLastError());
            return AVS_SUCCESS;
        }
    }
    tbuild_kernel<T, LAYOUT><<<dim3(P - first_role, w.batch > 0 ? w.batch : 1), kWNT, smem, s>>>(a);
    AVS_CUDA_TRY(cudaGetLastError());
    return AVS_SUCCESS;
}

}  // namespace

// T build alone (for the tensor-core update path).
template <typename T>
int stage1_tbuild(const T *dA, int64_t lda, int b, int layout, int pr, int pc, int P, const Stage1Work &w,
                  cudaStream_t s) {
    return layout == 0 ? launch_tbuild<T, 0>(dA, lda, b, pr, pc, P, w, s)
                       : launch_tbuild<T, 1>(dA, lda, b, pr, pc, P, w, s);
}
template int stage1_tbuild<float>(const float *, int64_t, int, int, int, int, int, const Stage1Work &, cudaStream_t);
template int stage1_tbuild<double>(const double *, int64_t, int, int, int, int, int, const Stage1Work &,
                                   cudaStream_t);

// Full-T trailing update of one half-step (tiles 128 and 256), tiles
// first_role..P-1 of the panel.
template <typename T>
int stage1_update_full(T *dA, int64_t lda, int64_t n, int b, int layout, int pr, int pc, int P, const Stage1Work &w,
                       cudaStream_t s, int first_role) {
    int rc;
    if (layout == 0) {
        if ((rc = launch_tbuild<T, 0>(dA, lda, b, pr, pc, P, w, s, first_role)) != AVS_SUCCESS) return rc;
        return b == 256 ? launch_upd_full_any<T, 0, 256>(dA, lda, n, pr, pc, P, w, s, first_role)
                        : launch_upd_full_any<T, 0, 128>(dA, lda, n, pr, pc, P, w, s, first_role);
    }
    if ((rc = launch_tbuild<T, 1>(dA, lda, b, pr, pc, P, w, s, first_role)) != AVS_SUCCESS) return rc;
    return b == 256 ? launch_upd_full_any<T, 1, 256>(dA, lda, n, pr, pc, P, w, s, first_role)
                    : launch_upd_full_any<T, 1, 128>(dA, lda, n, pr, pc, P, w, s, first_role);
}

template int stage1_update_full<float>(float *, int64_t, int64_t, int, int, int, int, int, const Stage1Work &,
                                       cudaStream_t, int);

template int stage1_update_full<double>(double *, int64_t, int64_t, int, int, int, int, int, const Stage1Work &,
                                        cudaStream_t, int);

}  // namespace avs
