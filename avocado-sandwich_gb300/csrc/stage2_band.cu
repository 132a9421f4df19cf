// Stage 2a: blocked band reduction, upper band of width B -> upper band of
// width T (T < B, T | B), the first stage of the hierarchical bulge chase.
//
// Reference: one stage of bidiag! (BRD/src/bulgechasing2.jl:22-45) with
// factor B / T, i.e. cbw = B, tbw = ts = T: a sweep reduces T rows at once;
// its first op is LQ_QMUL on those rows, then QR_QMUL / LQ_QMUL pairs chase
// the bulge down the band (bulgechasing2.jl:4-20).  The reference also uses
// the halving form of this step in bidiagonalize (KAbasedSVD/src/
// bulgechasing.jl:33-42).
//
// Sweep s (rows p = sT .. p+T-1), step m, with c0 = p + T + mB:
//   R op (LQ_QMUL): the T pivot rows [rho, rho+T) (rho = p for m = 0, else
//     c0 - B) over the columns [c0, c0+B) are factored X = L Q (T
//     Householder reflectors from the right); the rows below, [rho+T, c0+B),
//     are multiplied by Q^T = I - V T V^T; X becomes [L 0].
//   L op (QR_QMUL): the rows [c0, c0+B) over the T pivot columns [c0, c0+T)
//     are factored QR (T reflectors from the left); the columns to their
//     right, [c0+T, c0+2B), are multiplied by Q^T = I - V T^T V^T.
// Every index range is clipped to n.  With T = 1 this is the element chase
// of stage2_chase.cu.  Op k of sweep s touches nothing that ops >= k+4 of
// sweep s-1 touch (the same lag as the element chase: R op m of sweep s
// overlaps sweep s-1's ops up to L op m+1 in a T x T corner, L op m up to R
// op m+2), so sweep s runs op k once sweep s-1 has finished k+4 ops, and the
// result is bit-identical to running the sweeps one after another.
//
// One thread-block cluster of C CTAs owns a sweep.  Every CTA loads the
// panel and factors it itself (same data, same code: the same bits), builds
// the compact-WY factor T (LAPACK xLARFT, forward, columnwise), then applies
// the block reflector to its share of the rows (R op) or columns (L op) as
// two small GEMMs on the FP32 (or FP64) pipe, operands in shared memory.
// The band is in compact storage A(r, c) at AB[(r - c + 2B) + c * ldab],
// ldab = 3B + 1 (band_ku / band_ldab): rows c-2B .. c+B of column c (band,
// upper bulge up to 2B-1, lower bulge up to B-1), laid out so that every
// column segment an op moves starts on 16 bytes: staging and write-back move
// 16-byte vectors.
//
// Arithmetic: the element type R throughout (FP32 for the FP32-class modes,
// FP64 for the FP64 path), reflector scalars included.
#include <cooperative_groups.h>

#include <algorithm>
#include <type_traits>

#include "avs_common.cuh"

namespace cg = cooperative_groups;

namespace avs {
namespace {

template <int B, int T, int C>
struct BandCfg {
    static constexpr int NT = 256;                // threads per CTA
    static constexpr int NW = NT / 32;            // warps
    static constexpr int MR = 2 * B - T;          // rows (R op) / columns (L op) of the apply, at most
    static constexpr int PER = (MR + C - 1) / C;  // per CTA
    static constexpr int RQ = 4096 / B;           // granule that makes every micro-tile split exact
    static constexpr int RPC = (PER + RQ - 1) / RQ * RQ;  // rows (R op) / columns (L op) per CTA
    static constexpr int LDP = B + 4;             // panel: column stride (QR form, B rows)
    static constexpr int LDA_R = RPC + 4;         // R op staging: column stride (RPC rows)
    static constexpr int LDA_L = B + 4;           // L op staging: column stride (B rows)
    static constexpr int ASZ = (B * LDA_R > RPC * LDA_L) ? B * LDA_R : RPC * LDA_L;
    static constexpr int LDW = RPC + 4;           // W / Y buffer: [k][r or cc]
    // GEMM 1 / Y: 4 rows (R op) or 4 columns (L op) x KPT reflectors per thread
    static constexpr int NG4 = RPC / 4;
    static constexpr int NKG = NT / NG4;
    static constexpr int KPT = (T >= NKG) ? T / NKG : 1;
    // GEMM 2, R op: 4 rows x CPT2R columns per thread
    static constexpr int NCG_R = NT / NG4;
    static constexpr int CPT2R = B / NCG_R;
    // GEMM 2, L op: 4 rows x CPT2L columns per thread
    static constexpr int NIG = B / 4;
    static constexpr int NCG_L = NT / NIG;
    static constexpr int CPT2L = RPC / NCG_L;
    static_assert(B % 32 == 0 && T <= 32 && T < B && B % T == 0, "band stage shape");
    static_assert(NT % NG4 == 0 && (T >= NKG ? T % NKG == 0 : true), "GEMM 1 split");
    static_assert(CPT2R % 4 == 0 && CPT2R * NCG_R == B, "R op GEMM 2 split");
    static_assert(NT % NIG == 0 && CPT2L % 4 == 0 && CPT2L * NCG_L == RPC, "L op GEMM 2 split");
    template <typename R>
    static constexpr size_t smem_bytes() {
        return sizeof(R) * ((size_t)T * LDP + ASZ + (size_t)T * LDW + (size_t)T * (T + 1) * 2 + T);
    }
};

template <typename R>
struct Vec4;
template <>
struct Vec4<float> {
    static __device__ __forceinline__ void ld(const float *p, float (&o)[4]) {
        const float4 v = *reinterpret_cast<const float4 *>(p);
        o[0] = v.x;
        o[1] = v.y;
        o[2] = v.z;
        o[3] = v.w;
    }
};
template <>
struct Vec4<double> {
    static __device__ __forceinline__ void ld(const double *p, double (&o)[4]) {
        const double2 a = *reinterpret_cast<const double2 *>(p);
        const double2 b = *reinterpret_cast<const double2 *>(p + 2);
        o[0] = a.x;
        o[1] = a.y;
        o[2] = b.x;
        o[3] = b.y;
    }
};

// 16-byte vectors of the element type: 4 floats or 2 doubles.
template <typename R>
struct Vec16;
template <>
struct Vec16<float> {
    static constexpr int N = 4;
    static __device__ __forceinline__ void ld(const float *p, float (&o)[4]) {
        const float4 v = __ldcg(reinterpret_cast<const float4 *>(p));
        o[0] = v.x;
        o[1] = v.y;
        o[2] = v.z;
        o[3] = v.w;
    }
    static __device__ __forceinline__ void st(float *p, const float (&v)[4]) {
        *reinterpret_cast<float4 *>(p) = make_float4(v[0], v[1], v[2], v[3]);
    }
};
template <>
struct Vec16<double> {
    static constexpr int N = 2;
    static __device__ __forceinline__ void ld(const double *p, double (&o)[2]) {
        const double2 v = __ldcg(reinterpret_cast<const double2 *>(p));
        o[0] = v.x;
        o[1] = v.y;
    }
    static __device__ __forceinline__ void st(double *p, const double (&v)[2]) {
        *reinterpret_cast<double2 *>(p) = make_double2(v[0], v[1]);
    }
};

// Staging copy global (L2) -> shared of NV 16-byte vectors spread over NT
// threads: vector idx = tid + u * NT comes from src(idx) (nullptr: zeros) and
// goes to dst(idx, v).  The loads of a batch of 8 are all in flight before the
// first store, so a thread waits for about one L2 latency per batch instead of
// one per vector.
template <typename R, int NT, int NV, typename Src, typename Dst>
__device__ __forceinline__ void stage_in_vec(int tid, Src src, Dst dst) {
    constexpr int N = Vec16<R>::N;
    constexpr int PER = (NV + NT - 1) / NT;
    constexpr int BATCH = PER < 8 ? PER : 8;
#pragma unroll
    for (int u0 = 0; u0 < PER; u0 += BATCH) {
        R v[BATCH][N];
#pragma unroll
        for (int u = 0; u < BATCH; ++u) {
            const int idx = tid + (u0 + u) * NT;
            const R *p = (u0 + u < PER && idx < NV) ? src(idx) : nullptr;
            if (p) {
                Vec16<R>::ld(p, v[u]);
            } else {
#pragma unroll
                for (int e = 0; e < N; ++e) v[u][e] = R(0);
            }
        }
#pragma unroll
        for (int u = 0; u < BATCH; ++u) {
            const int idx = tid + (u0 + u) * NT;
            if (u0 + u < PER && idx < NV) dst(idx, v[u]);
        }
    }
}

__device__ __forceinline__ void cl_arrive() { asm volatile("barrier.cluster.arrive.aligned;" ::: "memory"); }
__device__ __forceinline__ void cl_wait() { asm volatile("barrier.cluster.wait.aligned;" ::: "memory"); }

// Scalars of the LAPACK-convention reflector of x = (alpha, x2) with s =
// ||x2||^2 > 0: beta = -sign(alpha) ||x||, tau = (beta - alpha) / beta =
// 1 + |alpha| / ||x||, scal = 1 / (alpha - beta).  FP32: the norm from the
// hardware reciprocal square root with one Newton step (about 0.5 ulp), the
// reciprocals correctly rounded -- a short dependent chain on the panel's
// critical path; FP64: divisions and sqrt.
__device__ __forceinline__ void reflector_scalars(float alpha, float s, float &tau, float &beta, float &scal) {
    const float a2s = fmaf(alpha, alpha, s);
    const float r = rsqrtf(a2s);
    float nrm = a2s * r;
    nrm = fmaf(0.5f * r, fmaf(-nrm, nrm, a2s), nrm);
    beta = alpha >= 0.0f ? -nrm : nrm;
    scal = __frcp_rn(alpha - beta);
    tau = fmaf(fabsf(alpha), __frcp_rn(nrm), 1.0f);
}
__device__ __forceinline__ void reflector_scalars(double alpha, double s, double &tau, double &beta, double &scal) {
    const double nrm = sqrt(fma(alpha, alpha, s));
    beta = alpha >= 0.0 ? -nrm : nrm;
    tau = (beta - alpha) / beta;
    scal = 1.0 / (alpha - beta);
}

// Householder QR of the panel P (B rows x T columns, column k at P + k*LDP,
// zero rows below the valid part), LAPACK convention per column: beta =
// -sign(alpha) ||x||, v = x / (alpha - beta) below the diagonal, v_k = 1,
// tau = (beta - alpha) / beta; tau = 0 when the part below the diagonal is
// zero.  On return P holds R on and above the diagonal and V below it;
// s_tau the taus; gram[j * (T+1) + k] = v_j^T v_k for j < k.  Warp w owns
// columns w, w + NW, ...; lane l rows l, l + 32, ...; one barrier per
// reflector.
template <typename R, int B, int T, int NW>
__device__ __forceinline__ void panel_qr(R *P, R *s_tau, R *gram) {
    constexpr int LDP = B + 4;
    constexpr int CPW = (T + NW - 1) / NW;
    constexpr int RPL = B / 32;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    R x[CPW][RPL];
#pragma unroll
    for (int jj = 0; jj < CPW; ++jj) {
        const int j = w + NW * jj;
#pragma unroll
        for (int u = 0; u < RPL; ++u) x[jj][u] = (j < T) ? P[j * LDP + lane + 32 * u] : R(0);
    }
#pragma unroll
    for (int k = 0; k < T; ++k) {
        const int ow = k % NW, jk = k / NW;
        if (w == ow) {
            R s = R(0);
#pragma unroll
            for (int u = 0; u < RPL; ++u) {
                const int i = lane + 32 * u;
                if (i > k) s = fma(x[jk][u], x[jk][u], s);
            }
            s = warp_sum(s);
            const R alpha = __shfl_sync(0xffffffffu, x[jk][k / 32], k % 32);
            R tau = R(0), beta = alpha, scal = R(0);
            if (s > R(0)) reflector_scalars(alpha, s, tau, beta, scal);
#pragma unroll
            for (int u = 0; u < RPL; ++u) {
                const int i = lane + 32 * u;
                if (i > k) x[jk][u] *= scal;
                else if (i == k) x[jk][u] = beta;
                P[k * LDP + i] = x[jk][u];
            }
            if (lane == 0) s_tau[k] = tau;
        }
        __syncthreads();
        const R tau = s_tau[k];
        R v[RPL];
#pragma unroll
        for (int u = 0; u < RPL; ++u) {
            const int i = lane + 32 * u;
            v[u] = (i > k) ? P[k * LDP + i] : (i == k ? R(1) : R(0));
        }
        // columns right of k get H_k (column k+1's slot first: the critical path);
        // columns left of k give the Gram entries v_j^T v_k
#pragma unroll
        for (int jj0 = 0; jj0 < CPW; ++jj0) {
            const int jj = (jj0 + ((k + 1) / NW)) % CPW;
            const int j = w + NW * jj;
            if (j < T && j != k) {
                R d = R(0);
#pragma unroll
                for (int u = 0; u < RPL; ++u) d = fma(v[u], x[jj][u], d);
                d = warp_sum(d);
                if (j > k) {
                    const R t = d * tau;
#pragma unroll
                    for (int u = 0; u < RPL; ++u) x[jj][u] = fma(-t, v[u], x[jj][u]);
                } else if (lane == 0) {
                    gram[j * (T + 1) + k] = d;  // x holds v_j below its diagonal
                }
            }
        }
    }
}

// Compact-WY factor of the panel's reflectors (LAPACK xLARFT, forward,
// columnwise): Tm[i*(T+1)+k], upper triangular, T[k][k] = tau_k, T[0:k, k] =
// -tau_k T[0:k, 0:k] (V^T v_k)[0:k].  Warp 0, lane i builds row i.
template <typename R, int T>
__device__ __forceinline__ void build_t(const R *s_tau, const R *gram, R *Tm) {
    const int i = threadIdx.x;
    if (i >= 32) return;
    R row[T];
#pragma unroll
    for (int k = 0; k < T; ++k) {
        const R tk = s_tau[k];
        R acc = R(0);
#pragma unroll
        for (int l = 0; l < k; ++l)
            if (l >= i) acc = fma(row[l], gram[l * (T + 1) + k], acc);
        row[k] = (i < k) ? -tk * acc : (i == k ? tk : R(0));
    }
    if (i < T) {
#pragma unroll
        for (int k = 0; k < T; ++k) Tm[i * (T + 1) + k] = row[k];
    }
}

template <int B, int T, typename R, int C>
__global__ void __launch_bounds__(256, sizeof(R) == 4 ? 2 : 1) band_stage_kernel(R *ab_base, int64_t n, int64_t ldab, int *ticket,
                                                          int *done_base, int *err, int batch, int64_t sAB,
                                                          int64_t sDone) {
    using Cfg = BandCfg<B, T, C>;
    constexpr int NT = Cfg::NT, NW = Cfg::NW, LDP = Cfg::LDP, RPC = Cfg::RPC, LDW = Cfg::LDW;
    constexpr int ku = band_ku(B);
    extern __shared__ __align__(16) unsigned char smem_raw[];
    R *P = reinterpret_cast<R *>(smem_raw);  // [T][LDP] panel (QR form), then V
    R *As = P + T * LDP;                      // apply staging
    R *Wy = As + Cfg::ASZ;                    // [T][LDW]: W / Z, then Y
    R *Tm = Wy + T * LDW;                     // [T][T+1]
    R *gram = Tm + T * (T + 1);               // [T][T+1]
    R *s_tau = gram + T * (T + 1);            // [T]
    __shared__ int s_j;
    cg::cluster_group cluster = cg::this_cluster();
    const int q = (int)cluster.block_rank();
    const int tid = threadIdx.x;

    const int64_t nsw = (n - 2 - T >= 0) ? (n - 2 - T) / T + 1 : 0;
    for (;;) {
        if (q == 0 && tid == 0) s_j = atomicAdd(ticket, 1);
        cluster.sync();
        const int64_t tk = *cluster.map_shared_rank(&s_j, 0);
        cluster.sync();
        const int64_t sw = tk / batch, zb = tk % batch;  // sweep-major over the batch
        if (sw >= nsw) return;
        R *ab = ab_base + zb * sAB;
        int *done = done_base + zb * sDone;
        auto at = [&](int64_t r, int64_t c) -> R * { return ab + (ku + r - c) + c * ldab; };
        const int64_t p = sw * T;
        const int nsteps = (int)((n - 2 - p - T) / B) + 1;
        const int ops_prev = (sw > 0) ? 2 * ((int)((n - 2 - p) / B) + 1) : 0;
        for (int op = 0; op < 2 * nsteps; ++op) {
            const int m = op >> 1;
            const bool rop = (op & 1) == 0;
            const int64_t c0 = p + T + (int64_t)m * B;
            // A wait that runs out records kDevTimeout; the cluster still runs its
            // barriers to the end (later waits return at once), so no CTA is left
            // at a cluster barrier.
            if (tid == 0 && sw > 0) wait_geq(done + sw - 1, min(op + 4, ops_prev), err);
            __syncthreads();
            const int L = (int)(n - c0 < B ? n - c0 : (int64_t)B);  // R op: columns; L op: rows
            if (rop) {
                const int64_t rho = (m == 0) ? p : c0 - B;
                const int64_t r_lo = rho + T + (int64_t)q * RPC;
                const int64_t r_hi = (c0 + B < n) ? c0 + B : n;
                constexpr int VN = Vec16<R>::N;
                // panel (QR form): P[k][c'] = A(rho + k, c0 + c'); column c' of the
                // pivot rows is T / VN vectors
                stage_in_vec<R, NT, T / VN * B>(
                    tid,
                    [&](int idx) -> const R * {
                        const int cc = idx / (T / VN), pt = idx % (T / VN);
                        return (cc < L) ? at(rho + pt * VN, c0 + cc) : nullptr;
                    },
                    [&](int idx, const R(&v)[VN]) {
                        const int cc = idx / (T / VN), pt = idx % (T / VN);
#pragma unroll
                        for (int e = 0; e < VN; ++e) P[(pt * VN + e) * LDP + cc] = v[e];
                    });
                // this CTA's rows of the apply, column-major [c][r] (a vector that
                // starts below r_hi ends below c0 + B, inside the column's segment;
                // its rows at or past r_hi are zeroed)
                stage_in_vec<R, NT, RPC / VN * B>(
                    tid,
                    [&](int idx) -> const R * {
                        const int cc = idx / (RPC / VN), pt = idx % (RPC / VN);
                        return (cc < L && r_lo + pt * VN < r_hi) ? at(r_lo + pt * VN, c0 + cc) : nullptr;
                    },
                    [&](int idx, R(&v)[VN]) {
                        const int pt = idx % (RPC / VN);
#pragma unroll
                        for (int e = 1; e < VN; ++e)
                            if (r_lo + pt * VN + e >= r_hi) v[e] = R(0);
                        Vec16<R>::st(As + (idx / (RPC / VN)) * Cfg::LDA_R + pt * VN, v);
                    });
                __syncthreads();
                cl_arrive();  // done reading the pivot rows
                panel_qr<R, B, T, NW>(P, s_tau, gram);
                __syncthreads();
                build_t<R, T>(s_tau, gram, Tm);
                cl_wait();  // every CTA has read the pivot rows: CTA 0 stores L and zeros
                if (q == 0) {
                    for (int idx = tid; idx < T * L; idx += NT) {
                        const int k = idx % T, j = idx / T;
                        *at(rho + k, c0 + j) = (j <= k) ? P[k * LDP + j] : R(0);
                    }
                }
                __syncthreads();
                for (int idx = tid; idx < T * T; idx += NT) {  // explicit V: unit diagonal, zeros above
                    const int k = idx / T, i = idx % T;
                    if (i <= k) P[k * LDP + i] = (i == k) ? R(1) : R(0);
                }
                __syncthreads();
                // W = A V: thread = 4 rows x KPT reflectors
                {
                    constexpr int KPT = Cfg::KPT;
                    const int g = tid % Cfg::NG4, kg = tid / Cfg::NG4;
                    const int k0 = kg * KPT;
                    if (k0 < T) {
                        R acc[KPT][4];
#pragma unroll
                        for (int a = 0; a < KPT; ++a)
#pragma unroll
                            for (int b2 = 0; b2 < 4; ++b2) acc[a][b2] = R(0);
#pragma unroll 2
                        for (int c = 0; c < B; c += 4) {
                            R a4[4][4], v4[KPT][4];
#pragma unroll
                            for (int cc = 0; cc < 4; ++cc) Vec4<R>::ld(As + (c + cc) * Cfg::LDA_R + 4 * g, a4[cc]);
#pragma unroll
                            for (int kk = 0; kk < KPT; ++kk) Vec4<R>::ld(P + (k0 + kk) * LDP + c, v4[kk]);
#pragma unroll
                            for (int kk = 0; kk < KPT; ++kk)
#pragma unroll
                                for (int cc = 0; cc < 4; ++cc)
#pragma unroll
                                    for (int rr = 0; rr < 4; ++rr)
                                        acc[kk][rr] = fma(a4[cc][rr], v4[kk][cc], acc[kk][rr]);
                        }
#pragma unroll
                        for (int kk = 0; kk < KPT; ++kk)
#pragma unroll
                            for (int rr = 0; rr < 4; ++rr) Wy[(k0 + kk) * LDW + 4 * g + rr] = acc[kk][rr];
                    }
                }
                __syncthreads();
                // Y = W T (all reads before the barrier, then in place)
                {
                    constexpr int KPT = Cfg::KPT;
                    const int g = tid % Cfg::NG4, kg = tid / Cfg::NG4;
                    const int k0 = kg * KPT;
                    R y[KPT][4];
                    if (k0 < T) {
#pragma unroll
                        for (int kk = 0; kk < KPT; ++kk) {
                            const int k = k0 + kk;
#pragma unroll
                            for (int rr = 0; rr < 4; ++rr) y[kk][rr] = R(0);
                            for (int l = 0; l <= k; ++l) {
                                const R t = Tm[l * (T + 1) + k];
#pragma unroll
                                for (int rr = 0; rr < 4; ++rr) y[kk][rr] = fma(Wy[l * LDW + 4 * g + rr], t, y[kk][rr]);
                            }
                        }
                    }
                    __syncthreads();
                    if (k0 < T) {
#pragma unroll
                        for (int kk = 0; kk < KPT; ++kk)
#pragma unroll
                            for (int rr = 0; rr < 4; ++rr) Wy[(k0 + kk) * LDW + 4 * g + rr] = y[kk][rr];
                    }
                }
                __syncthreads();
                // A -= Y V^T: thread = 4 rows x CPT2R columns; straight to global
                {
                    constexpr int CPT = Cfg::CPT2R;
                    const int g = tid % Cfg::NG4, cgp = tid / Cfg::NG4;
                    const int cb = cgp * CPT;
                    R acc[4][CPT];
#pragma unroll
                    for (int cc = 0; cc < CPT; ++cc)
#pragma unroll
                        for (int rr = 0; rr < 4; ++rr) acc[rr][cc] = As[(cb + cc) * Cfg::LDA_R + 4 * g + rr];
                    for (int k = 0; k < T; ++k) {
                        R y4[4];
                        Vec4<R>::ld(Wy + k * LDW + 4 * g, y4);
#pragma unroll
                        for (int c4 = 0; c4 < CPT; c4 += 4) {
                            R v4[4];
                            Vec4<R>::ld(P + k * LDP + cb + c4, v4);
#pragma unroll
                            for (int cc = 0; cc < 4; ++cc)
#pragma unroll
                                for (int rr = 0; rr < 4; ++rr)
                                    acc[rr][c4 + cc] = fma(-y4[rr], v4[cc], acc[rr][c4 + cc]);
                        }
                    }
                    constexpr int VN = Vec16<R>::N;
#pragma unroll
                    for (int cc = 0; cc < CPT; ++cc) {
                        const int c = cb + cc;
                        if (c < L) {
#pragma unroll
                            for (int r0 = 0; r0 < 4; r0 += VN) {
                                const int64_t r = r_lo + 4 * g + r0;
                                if (r + VN <= r_hi) {
                                    R v[VN];
#pragma unroll
                                    for (int e = 0; e < VN; ++e) v[e] = acc[r0 + e][cc];
                                    Vec16<R>::st(at(r, c0 + c), v);
                                } else {
#pragma unroll
                                    for (int e = 0; e < VN; ++e)
                                        if (r + e < r_hi) *at(r + e, c0 + c) = acc[r0 + e][cc];
                                }
                            }
                        }
                    }
                }
            } else {
                const int Tc = (int)(n - c0 < T ? n - c0 : (int64_t)T);  // pivot columns
                const int64_t cc_lo = c0 + T + (int64_t)q * RPC;
                const int64_t c_hi = (c0 + 2 * B < n) ? c0 + 2 * B : n;
                constexpr int VN = Vec16<R>::N;
                // panel: P[k][i] = A(c0 + i, c0 + k); a vector that starts below L
                // stays inside the column's segment, its rows at or past L are zeroed
                stage_in_vec<R, NT, B / VN * T>(
                    tid,
                    [&](int idx) -> const R * {
                        const int k = idx / (B / VN), pt = idx % (B / VN);
                        return (pt * VN < L && k < Tc) ? at(c0 + pt * VN, c0 + k) : nullptr;
                    },
                    [&](int idx, R(&v)[VN]) {
                        const int pt = idx % (B / VN);
#pragma unroll
                        for (int e = 1; e < VN; ++e)
                            if (pt * VN + e >= L) v[e] = R(0);
                        Vec16<R>::st(P + (idx / (B / VN)) * LDP + pt * VN, v);
                    });
                // this CTA's columns of the apply, column-major [cc][i]
                stage_in_vec<R, NT, B / VN * RPC>(
                    tid,
                    [&](int idx) -> const R * {
                        const int cc = idx / (B / VN), pt = idx % (B / VN);
                        return (pt * VN < L && cc_lo + cc < c_hi) ? at(c0 + pt * VN, cc_lo + cc) : nullptr;
                    },
                    [&](int idx, R(&v)[VN]) {
                        const int pt = idx % (B / VN);
#pragma unroll
                        for (int e = 1; e < VN; ++e)
                            if (pt * VN + e >= L) v[e] = R(0);
                        Vec16<R>::st(As + (idx / (B / VN)) * Cfg::LDA_L + pt * VN, v);
                    });
                __syncthreads();
                cl_arrive();  // done reading the pivot columns
                panel_qr<R, B, T, NW>(P, s_tau, gram);
                __syncthreads();
                build_t<R, T>(s_tau, gram, Tm);
                cl_wait();  // CTA 0 stores R and zeros
                if (q == 0) {
                    for (int idx = tid; idx < Tc * L; idx += NT) {
                        const int i = idx % L, k = idx / L;
                        *at(c0 + i, c0 + k) = (i <= k) ? P[k * LDP + i] : R(0);
                    }
                }
                __syncthreads();
                for (int idx = tid; idx < T * T; idx += NT) {
                    const int k = idx / T, i = idx % T;
                    if (i <= k) P[k * LDP + i] = (i == k) ? R(1) : R(0);
                }
                __syncthreads();
                // Z = V^T A: thread = 4 columns (g + cc NG4: lanes one column apart, so
                // their column reads spread over the banks) x KPT reflectors
                {
                    constexpr int KPT = Cfg::KPT;
                    const int g = tid % Cfg::NG4, kg = tid / Cfg::NG4;
                    const int k0 = kg * KPT;
                    if (k0 < T) {
                        R acc[KPT][4];
#pragma unroll
                        for (int a = 0; a < KPT; ++a)
#pragma unroll
                            for (int b2 = 0; b2 < 4; ++b2) acc[a][b2] = R(0);
#pragma unroll 2
                        for (int i = 0; i < B; i += 4) {
                            R a4[4][4], v4[KPT][4];
#pragma unroll
                            for (int cc = 0; cc < 4; ++cc)
                                Vec4<R>::ld(As + (g + cc * Cfg::NG4) * Cfg::LDA_L + i, a4[cc]);
#pragma unroll
                            for (int kk = 0; kk < KPT; ++kk) Vec4<R>::ld(P + (k0 + kk) * LDP + i, v4[kk]);
#pragma unroll
                            for (int kk = 0; kk < KPT; ++kk)
#pragma unroll
                                for (int cc = 0; cc < 4; ++cc)
#pragma unroll
                                    for (int ii = 0; ii < 4; ++ii)
                                        acc[kk][cc] = fma(v4[kk][ii], a4[cc][ii], acc[kk][cc]);
                        }
#pragma unroll
                        for (int kk = 0; kk < KPT; ++kk)
#pragma unroll
                            for (int cc = 0; cc < 4; ++cc) Wy[(k0 + kk) * LDW + g + cc * Cfg::NG4] = acc[kk][cc];
                    }
                }
                __syncthreads();
                // Y = T^T Z
                {
                    constexpr int KPT = Cfg::KPT;
                    const int g = tid % Cfg::NG4, kg = tid / Cfg::NG4;
                    const int k0 = kg * KPT;
                    R y[KPT][4];
                    if (k0 < T) {
#pragma unroll
                        for (int kk = 0; kk < KPT; ++kk) {
                            const int k = k0 + kk;
#pragma unroll
                            for (int cc = 0; cc < 4; ++cc) y[kk][cc] = R(0);
                            for (int l = 0; l <= k; ++l) {
                                const R t = Tm[l * (T + 1) + k];
#pragma unroll
                                for (int cc = 0; cc < 4; ++cc)
                                    y[kk][cc] = fma(t, Wy[l * LDW + g + cc * Cfg::NG4], y[kk][cc]);
                            }
                        }
                    }
                    __syncthreads();
                    if (k0 < T) {
#pragma unroll
                        for (int kk = 0; kk < KPT; ++kk)
#pragma unroll
                            for (int cc = 0; cc < 4; ++cc) Wy[(k0 + kk) * LDW + g + cc * Cfg::NG4] = y[kk][cc];
                    }
                }
                __syncthreads();
                // A -= V Y: thread = 4 rows x CPT2L columns; straight to global
                {
                    constexpr int CPT = Cfg::CPT2L;
                    const int ig = tid % Cfg::NIG, cgp = tid / Cfg::NIG;
                    const int cb = cgp * CPT;
                    R acc[4][CPT];
#pragma unroll
                    for (int cc = 0; cc < CPT; ++cc)
#pragma unroll
                        for (int ii = 0; ii < 4; ++ii) acc[ii][cc] = As[(cb + cc) * Cfg::LDA_L + 4 * ig + ii];
                    for (int k = 0; k < T; ++k) {
                        R v4[4];
                        Vec4<R>::ld(P + k * LDP + 4 * ig, v4);
#pragma unroll
                        for (int c4 = 0; c4 < CPT; c4 += 4) {
                            R y4[4];
                            Vec4<R>::ld(Wy + k * LDW + cb + c4, y4);
#pragma unroll
                            for (int cc = 0; cc < 4; ++cc)
#pragma unroll
                                for (int ii = 0; ii < 4; ++ii)
                                    acc[ii][c4 + cc] = fma(-v4[ii], y4[cc], acc[ii][c4 + cc]);
                        }
                    }
                    constexpr int VN = Vec16<R>::N;
#pragma unroll
                    for (int cc = 0; cc < CPT; ++cc) {
                        const int64_t c = cc_lo + cb + cc;
                        if (c < c_hi) {
#pragma unroll
                            for (int i0 = 0; i0 < 4; i0 += VN) {
                                const int i = 4 * ig + i0;
                                if (i + VN <= L) {
                                    R v[VN];
#pragma unroll
                                    for (int e = 0; e < VN; ++e) v[e] = acc[i0 + e][cc];
                                    Vec16<R>::st(at(c0 + i, c), v);
                                } else {
#pragma unroll
                                    for (int e = 0; e < VN; ++e)
                                        if (i + e < L) *at(c0 + i + e, c) = acc[i0 + e][cc];
                                }
                            }
                        }
                    }
                }
            }
            // the op's stores, made visible at GPU scope by one fence per CTA (after
            // the CTA barrier), then the cluster barrier, then the release
            __syncthreads();
            if (tid == 0) __threadfence();
            cluster.sync();
            if (q == 0 && tid == 0) st_release(done + sw, op + 1);
        }
    }
}

template <int B, int T, typename R, int C>
int launch_band_stage(R *dAB, int64_t n, int64_t ldab, const Stage2Work &w, cudaStream_t s, int num_sms, int batch,
                      int64_t sAB, int64_t sDone) {
    using Cfg = BandCfg<B, T, C>;
    const size_t smem = Cfg::template smem_bytes<R>();
    auto kern = band_stage_kernel<B, T, R, C>;
    AVS_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    if (C > 8) AVS_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = C;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.blockDim = dim3(Cfg::NT);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cfg.gridDim = dim3(C * 64);
    int max_clusters = 0;
    if (cudaOccupancyMaxActiveClusters(&max_clusters, kern, &cfg) != cudaSuccess || max_clusters <= 0) {
        cudaGetLastError();
        max_clusters = std::max(1, num_sms / C);
    }
    const int64_t nsw = (n - 2 - T >= 0) ? (n - 2 - T) / T + 1 : 0;
    if (nsw == 0) return AVS_SUCCESS;
    // sweeps in flight: a sweep's 2 n / B ops over a lag of 4 ops
    const int64_t want = std::max<int64_t>(1, ((n / B) / 2 + 2) * (int64_t)batch);
    const int64_t clusters = std::min<int64_t>(std::min<int64_t>(want, max_clusters), nsw * (int64_t)batch);
    cfg.gridDim = dim3((unsigned)(clusters * C));
    AVS_CUDA_TRY(cudaLaunchKernelEx(&cfg, kern, dAB, n, ldab, w.flags, w.flags + 1, w.err, batch, sAB, sDone));
    return AVS_SUCCESS;
}

// dense (leading dimension lda, matrix stride sA) -> compact band of width
// bw (ku = band_ku(bw)), zeros outside 0 <= c - r <= bw
template <typename TI, typename R>
__global__ void dense_to_band_kernel(const TI *a, int64_t n, int64_t lda, int64_t sA, int bw, R *ab, int64_t ldab,
                                     int64_t sAB) {
    const int64_t c = blockIdx.x;
    const int64_t zb = blockIdx.y;
    const int ku = band_ku(bw);
    const TI *az = a + zb * sA;
    R *abz = ab + zb * sAB + c * ldab;
    for (int i = threadIdx.x; i < ldab; i += blockDim.x) {
        const int64_t r = c - ku + i;
        abz[i] = (r >= 0 && r <= c && c - r <= bw) ? (R)az[r + c * lda] : R(0);
    }
}

// compact band (width bw1 storage) holding a band of width bw2 -> compact
// band of width bw2 (ku2 = 2 bw2 - 1) of storage type St (float2: double-float
// pairs; double)
template <typename R, typename St>
__global__ void band_to_band_kernel(const R *ab1, int64_t n, int bw1, int64_t ldab1, int64_t sAB1, int bw2, St *ab2,
                                    int64_t ldab2, int64_t sAB2) {
    const int64_t c = blockIdx.x;
    const int64_t zb = blockIdx.y;
    const int ku1 = band_ku(bw1), ku2 = 2 * bw2 - 1;
    const R *src = ab1 + zb * sAB1;
    St *dst = ab2 + zb * sAB2 + c * ldab2;
    for (int i = threadIdx.x; i < ldab2; i += blockDim.x) {
        const int64_t r = c - ku2 + i;
        const bool in = (r >= 0 && r <= c && c - r <= bw2);
        const R v = in ? src[(ku1 + r - c) + c * ldab1] : R(0);
        if constexpr (std::is_same<St, float2>::value) {
            const float h = (float)v;
            dst[i] = make_float2(h, (float)((double)v - (double)h));
        } else {
            dst[i] = (St)v;
        }
    }
}

// compact band (width bw storage) -> dense column-major n x n: every entry the
// compact storage holds (rows c-2bw .. c+bw of column c), zeros elsewhere
template <typename R>
__global__ void band_to_dense_kernel(const R *ab, int64_t n, int bw, int64_t ldab, R *a, int64_t lda) {
    const int64_t c = blockIdx.x;
    const int ku = band_ku(bw);
    for (int64_t r = threadIdx.x; r < n; r += blockDim.x) {
        const int64_t i = ku + r - c;
        a[r + c * lda] = (i >= 0 && i < ldab) ? ab[i + c * ldab] : R(0);
    }
}

// CTAs per cluster: the apply's 2B - T rows (columns) split C ways; FP64
// operands at band 256 take 16 CTAs (a non-portable cluster size) so that a
// CTA's staging fits in shared memory.
template <int B, typename R>
constexpr int band_cluster() {
    return B == 256 ? (sizeof(R) == 8 ? 16 : 8) : (B == 128 ? 8 : 2);
}

}  // namespace

template <typename R>
int band_stage(R *dAB, int64_t n, int bw, int tbw, int64_t ldab, const Stage2Work &w, cudaStream_t s, int num_sms,
               int batch, int64_t sAB, int64_t sDone) {
    if (n < 3) return AVS_SUCCESS;
    if (ldab != band_ldab(bw)) return AVS_ERR_INTERNAL;
    AVS_CUDA_TRY(cudaMemsetAsync(w.flags, 0, sizeof(int) * (size_t)((n + 1) * (int64_t)batch + 1), s));
#define AVS_BAND_CASE(BB, TT)                                                                                   \
    if (bw == BB && tbw == TT)                                                                                  \
        return launch_band_stage<BB, TT, R, band_cluster<BB, R>()>(dAB, n, ldab, w, s, num_sms, batch, sAB, sDone);
    AVS_BAND_CASE(256, 32)
    AVS_BAND_CASE(256, 16)
    AVS_BAND_CASE(128, 32)
    AVS_BAND_CASE(128, 16)
    AVS_BAND_CASE(64, 16)
#undef AVS_BAND_CASE
    return AVS_ERR_UNSUPPORTED;
}
template int band_stage<float>(float *, int64_t, int, int, int64_t, const Stage2Work &, cudaStream_t, int, int,
                               int64_t, int64_t);
template int band_stage<double>(double *, int64_t, int, int, int64_t, const Stage2Work &, cudaStream_t, int, int,
                                int64_t, int64_t);

bool band_stage_supported(int bw, int tbw) {
    return ((bw == 256 || bw == 128) && (tbw == 32 || tbw == 16)) || (bw == 64 && tbw == 16);
}

template <typename TI, typename R>
int dense_to_band(const TI *dA, int64_t n, int64_t lda, int64_t sA, int bw, R *dAB, int64_t ldab, int64_t sAB,
                  int batch, cudaStream_t s) {
    if (n <= 0) return AVS_SUCCESS;
    dense_to_band_kernel<TI, R><<<dim3((unsigned)n, (unsigned)batch), 128, 0, s>>>(dA, n, lda, sA, bw, dAB, ldab, sAB);
    AVS_CUDA_TRY(cudaGetLastError());
    return AVS_SUCCESS;
}
template int dense_to_band<float, float>(const float *, int64_t, int64_t, int64_t, int, float *, int64_t, int64_t,
                                         int, cudaStream_t);
template int dense_to_band<double, double>(const double *, int64_t, int64_t, int64_t, int, double *, int64_t,
                                           int64_t, int, cudaStream_t);

template <typename R, typename St>
int band_to_band(const R *dAB1, int64_t n, int bw1, int64_t ldab1, int64_t sAB1, int bw2, St *dAB2, int64_t ldab2,
                 int64_t sAB2, int batch, cudaStream_t s) {
    if (n <= 0) return AVS_SUCCESS;
    band_to_band_kernel<R, St><<<dim3((unsigned)n, (unsigned)batch), 128, 0, s>>>(dAB1, n, bw1, ldab1, sAB1, bw2,
                                                                                 dAB2, ldab2, sAB2);
    AVS_CUDA_TRY(cudaGetLastError());
    return AVS_SUCCESS;
}
template int band_to_band<float, float2>(const float *, int64_t, int, int64_t, int64_t, int, float2 *, int64_t,
                                         int64_t, int, cudaStream_t);
template int band_to_band<double, double>(const double *, int64_t, int, int64_t, int64_t, int, double *, int64_t,
                                          int64_t, int, cudaStream_t);

template <typename R>
int band_to_dense(const R *dAB, int64_t n, int bw, int64_t ldab, R *dA, int64_t lda, cudaStream_t s) {
    if (n <= 0) return AVS_SUCCESS;
    band_to_dense_kernel<R><<<(unsigned)n, 256, 0, s>>>(dAB, n, bw, ldab, dA, lda);
    AVS_CUDA_TRY(cudaGetLastError());
    return AVS_SUCCESS;
}
template int band_to_dense<float>(const float *, int64_t, int, int64_t, float *, int64_t, cudaStream_t);
template int band_to_dense<double>(const double *, int64_t, int, int64_t, double *, int64_t, cudaStream_t);

}  // namespace avs
