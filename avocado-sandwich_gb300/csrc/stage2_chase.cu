// Stage 2: upper band (width bw) -> upper bidiagonal by Householder bulge
// chasing, FP64, on the GPU.
//
// Reference: bidiagonalize / block_bidiagonalize! (KAbasedSVD/src/
// bulgechasing.jl:1-42), which the reference runs on the CPU with LAPACK on
// views of the dense n x n array.  Here the band lives in a compact FP64 band
// array with room for the bulges, and the chase is one persistent kernel.
//
// Sweep j (j = 0 .. n-2) makes row j bidiagonal.  Its step m works on the
// pivot (rho, c0) -- (j, j+1) for m = 0, then (c0_prev, c0_prev + bw):
//   R op: a right reflector of length <= bw annihilates A[rho, c0+1 .. c0+bw-1];
//         it is applied to rows rho .. c0+bw-1;
//   L op: a left reflector annihilates A[c0+1 .. c0+bw-1, c0]; it is applied to
//         columns c0 .. c0+2bw-1.
// Only the first row/column of each bulge is annihilated; what remains of a
// bulge lies where the next sweep's reflectors annihilate it.  Step m of sweep
// j touches nothing that steps >= m+3 of sweep j-1 touch, so sweep j may run
// step m once sweep j-1 has finished step m+2: the sweeps form a wavefront,
// each CTA owning one sweep at a time (sweeps handed out by an atomic ticket in
// order, so a sweep waits only on sweeps already running; every wait bounded).
// The result is bit-identical to running the sweeps one after another.
//
// For the tile sizes of the pipeline (bw = 16 .. 256) each sweep is owned by a
// thread-block cluster of C CTAs (8 for bw >= 128): every CTA forms the
// reflector itself from the pivot row/column, then applies it to its share of
// the rows (R op) or columns (L op), holding its values in registers; a
// cluster barrier separates the ops.  Dependencies are tracked per op: the
// counter of sweep j counts finished ops (R, L, R, L, ...), and op k of sweep
// j waits until sweep j-1 has finished op k+3 -- the tightest lag for which
// the wavefront stays bit-identical to the sequential order.  Along the
// critical path a sweep therefore costs 4 ops instead of 6.
//
// Band storage: A(r, c) at AB[(r - c + 2bw - 1) + c * ldab], ldab >= 3bw - 1,
// which holds 0 <= c - r <= 2bw - 1 (band + upper bulge) and
// 0 <= r - c <= bw - 1 (lower bulge).
#include <cooperative_groups.h>

#include <algorithm>
#include <type_traits>
#include <cmath>

#include "avs_common.cuh"
#include "chase_ar.cuh"
#include "df64.cuh"

namespace cg = cooperative_groups;

namespace avs {
namespace {

constexpr int kChaseThreads = 256;

struct Band {
    double *ab;
    int64_t ldab;
    int ku;  // 2bw - 1
    __device__ __forceinline__ double *at(int64_t r, int64_t c) const { return ab + (ku + r - c) + c * ldab; }
};

__device__ __forceinline__ double block_sum(double v, double *red) {
    v = warp_sum(v);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) red[wid] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x < 32) {
        s = (threadIdx.x < (blockDim.x >> 5)) ? red[threadIdx.x] : 0.0;
        s = warp_sum(s);
        if (threadIdx.x == 0) red[0] = s;
    }
    __syncthreads();
    return red[0];
}

// Householder reflector of x (length L, x[0] = alpha) in shared memory, LAPACK
// convention: beta = -sign(alpha) ||x||, v[0] = 1, v = x / (alpha - beta),
// tau = (beta - alpha) / beta; tau = 0 when x[1..] == 0.  Overwrites x with v.
__device__ void make_reflector(double *x, int L, double *red, double *out_tau, double *out_beta) {
    double part = 0.0;
    for (int i = 1 + threadIdx.x; i < L; i += blockDim.x) part += x[i] * x[i];
    const double s = block_sum(part, red);
    const double alpha = x[0];
    double tau = 0.0, beta = alpha, scal = 0.0;
    if (s > 0.0) {
        const double nrm = sqrt(alpha * alpha + s);
        beta = alpha >= 0.0 ? -nrm : nrm;
        tau = (beta - alpha) / beta;
        scal = 1.0 / (alpha - beta);
    }
    __syncthreads();
    for (int i = 1 + threadIdx.x; i < L; i += blockDim.x) x[i] *= scal;
    if (threadIdx.x == 0) x[0] = 1.0;
    __syncthreads();
    *out_tau = tau;
    *out_beta = beta;
}

__global__ void __launch_bounds__(kChaseThreads) chase_kernel(double *ab, int64_t n, int bw, int64_t ldab,
                                                              int *ticket, int *done, int *err) {
    extern __shared__ double sv[];  // bw doubles: the current reflector
    __shared__ double red[32];
    __shared__ int s_j, s_ok;
    Band A{ab, ldab, 2 * bw - 1};
    const int tid = threadIdx.x;
    const int lane = tid & 31, wid = tid >> 5, nwarps = blockDim.x >> 5;

    for (;;) {
        if (tid == 0) s_j = atomicAdd(ticket, 1);
        __syncthreads();
        const int64_t j = s_j;
        if (j >= n - 1) return;
        const int nsteps = (int)((n - j - 2) / bw) + 1;
        const int nsteps_prev = (j > 0) ? (int)((n - j - 1) / bw) + 1 : 0;
        int64_t rho = j, c0 = j + 1;
        for (int m = 0; m < nsteps; ++m) {
            if (tid == 0) {
                bool ok = true;
                if (j > 0) ok = wait_geq(done + j - 1, min(m + 3, nsteps_prev), err);
                s_ok = ok;
            }
            __syncthreads();
            if (!s_ok) return;
            const int64_t c1 = min(c0 + bw - 1, n - 1);
            const int L = (int)(c1 - c0 + 1);
            if (L >= 2) {
                // ---- R op: row rho, columns c0..c1
                for (int i = tid; i < L; i += blockDim.x) sv[i] = __ldcg(A.at(rho, c0 + i));
                __syncthreads();
                double tau, beta;
                make_reflector(sv, L, red, &tau, &beta);
                if (tau != 0.0) {
                    for (int64_t r = rho + 1 + tid; r <= c1; r += blockDim.x) {
                        double w = 0.0;
                        for (int i = 0; i < L; ++i) w += __ldcg(A.at(r, c0 + i)) * sv[i];
                        w *= tau;
                        for (int i = 0; i < L; ++i) *A.at(r, c0 + i) -= w * sv[i];
                    }
                }
                if (tid == 0) *A.at(rho, c0) = beta;
                for (int i = 1 + tid; i < L; i += blockDim.x) *A.at(rho, c0 + i) = 0.0;
                __syncthreads();
                // ---- L op: column c0, rows c0..c1, applied to columns c0..c0+2bw-1
                for (int i = tid; i < L; i += blockDim.x) sv[i] = __ldcg(A.at(c0 + i, c0));
                __syncthreads();
                make_reflector(sv, L, red, &tau, &beta);
                if (tau != 0.0) {
                    const int64_t cend = min(c0 + 2 * (int64_t)bw - 1, n - 1);
                    for (int64_t c = c0 + 1 + wid; c <= cend; c += nwarps) {
                        double w = 0.0;
                        for (int i = lane; i < L; i += 32) w += sv[i] * __ldcg(A.at(c0 + i, c));
                        w = warp_sum(w) * tau;
                        for (int i = lane; i < L; i += 32) *A.at(c0 + i, c) -= w * sv[i];
                    }
                }
                if (tid == 0) *A.at(c0, c0) = beta;
                for (int i = 1 + tid; i < L; i += blockDim.x) *A.at(c0 + i, c0) = 0.0;
            }
            __syncthreads();
            if (tid == 0) {
                __threadfence();
                st_release(done + j, m + 1);
            }
            rho = c0;
            c0 += bw;
        }
    }
}

template <int BW, int CC = (BW >= 128 ? 8 : (BW == 64 ? 4 : (BW == 32 ? 2 : 1))), int NTT = 512>
struct ChaseCfg {
    static constexpr int C = CC;  // CTAs per cluster (one sweep per cluster)
    // One matrix: 512 threads per CTA -- an op's latency (the sweep wavefront's
    // step) falls with the threads that share it (128-thread CTAs, several per
    // SM, were slower at every band width).  A batch of small bands is
    // throughput-bound instead: smaller CTAs, several sweeps per SM.
    static constexpr int NT = NTT;
    static constexpr int MINB = 512 / NTT;  // same registers per SM as one 512-thread CTA
    static constexpr int RPC = 2 * BW / C;          // R op: rows per CTA (64 or 32)
    static constexpr int G = NT / RPC;              // R op: column groups
    static constexpr int CPG = BW / G;              // R op: columns per group
    static constexpr int CPC = 2 * BW / C;          // L op: columns per CTA
    static constexpr int CPW = CPC / (NT / 32);     // L op: columns per warp
    static constexpr int RPL = BW >= 32 ? BW / 32 : 1;  // L op: rows per lane
    // R op dot products: every row's sum runs over NCH fixed chunks of W0
    // columns, each chunk accumulated in the same order and the chunks added
    // in index order, whatever C and NT are -- so every configuration of a
    // band width gives the same bits (a matrix's values do not depend on the
    // batch it runs in).
    static constexpr int NCH = 16;
    static constexpr int W0 = BW / NCH;
    static constexpr int CPT = CPG / W0;  // chunks per thread
    static_assert(CPG >= 1 && CPW >= 1, "chase configuration");
    static_assert(W0 >= 1 && CPG % W0 == 0 && G * CPT == NCH, "chase chunking");
};


template <typename S>
struct BandT {
    using Ar = ChaseAr<S>;
    typename Ar::St *ab;
    int64_t ldab;
    int ku;  // 2bw - 1
    __device__ __forceinline__ typename Ar::St *at(int64_t r, int64_t c) const { return ab + (ku + r - c) + c * ldab; }
};

// Split cluster barrier: every thread of every CTA arrives (release: its
// earlier reads and writes are ordered before) and later waits (acquire).
// Between the two a CTA keeps working; a thread waits before it arrives again.
__device__ __forceinline__ void cluster_arrive() { asm volatile("barrier.cluster.arrive.aligned;" ::: "memory"); }
__device__ __forceinline__ void cluster_wait() { asm volatile("barrier.cluster.wait.aligned;" ::: "memory"); }

template <typename S>
__device__ __forceinline__ typename ChaseAr<S>::V warp_sum_s(typename ChaseAr<S>::V v) {
    using Ar = ChaseAr<S>;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = Ar::add(v, Ar::shfl_xor(v, o));
    return v;
}

// Reflector of x[0..L) read straight from the band by one warp (lane l holds
// x[l + 32 t]): LAPACK convention, beta = -sign(alpha) ||x||, v = x / (alpha -
// beta), v0 = 1, tau = (beta - alpha) / beta; tau = 0 when x[1..] == 0.  Every
// lane forms the scalars (no broadcast); v goes to sv, tau and beta to
// s_tau / s_beta.  Every CTA of the cluster computes the same reflector from
// the same data.  row: x[i] = A(fixed, start + i); else x[i] = A(start + i, fixed).
template <typename S, int BW>
__device__ __forceinline__ void warp_reflector(const BandT<S> &A, bool row, int64_t fixed, int64_t start, int L,
                                               typename ChaseAr<S>::V *sv, typename ChaseAr<S>::V *s_tau,
                                               typename ChaseAr<S>::V *s_beta) {
    using Ar = ChaseAr<S>;
    using V = typename Ar::V;
    constexpr int PER = (BW + 31) / 32;
    const int lane = threadIdx.x & 31;
    V x[PER];
#pragma unroll
    for (int t = 0; t < PER; ++t) {  // all loads in flight before the first use
        const int i = lane + 32 * t;
        x[t] = Ar::zero();
        if (i < L) x[t] = Ar::ld(row ? A.at(fixed, start + i) : A.at(start + i, fixed));
    }
    typename Ar::Acc acc = Ar::acc_zero();
#pragma unroll
    for (int t = 0; t < PER; ++t) {
        const int i = lane + 32 * t;
        if (i >= 1 && i < L) Ar::acc_add(acc, x[t], x[t]);
    }
    const V s = warp_sum_s<S>(Ar::acc_value(acc));
    const V alpha = Ar::shfl(x[0], 0);
    V tau = Ar::zero(), beta = alpha, scal = Ar::zero();
    if (Ar::gt0(s)) {
        const V nrm = Ar::sqrt(Ar::fma(alpha, alpha, s));
        beta = Ar::ge0(alpha) ? Ar::neg(nrm) : nrm;
        tau = Ar::mul(Ar::sub(beta, alpha), Ar::rcp(beta));
        scal = Ar::rcp(Ar::sub(alpha, beta));
    }
#pragma unroll
    for (int t = 0; t < PER; ++t) {
        const int i = lane + 32 * t;
        if (i < L) sv[i] = (i == 0) ? Ar::one() : Ar::mul(x[t], scal);
    }
    if (lane == 0) {
        *s_tau = tau;
        *s_beta = beta;
    }
}

template <int BW, typename S, int CC, int NTT = 512>
__global__ void __launch_bounds__(ChaseCfg<BW, CC, NTT>::NT, ChaseCfg<BW, CC, NTT>::MINB) chase_cluster_kernel(typename ChaseAr<S>::St *ab_base, int64_t n, int64_t ldab,
                                                            int *ticket, int *done_base, int *err, int batch,
                                                            int64_t sAB, int64_t sDone) {
    using Cfg = ChaseCfg<BW, CC, NTT>;
    using Ar = ChaseAr<S>;
    using V = typename Ar::V;
    cg::cluster_group cluster = cg::this_cluster();
    const int q = (int)cluster.block_rank();
    __shared__ V sv[BW];
    __shared__ V part[Cfg::NCH][Cfg::RPC];
    __shared__ V wrow[Cfg::RPC];
    __shared__ V s_tau, s_beta;
    __shared__ int s_j;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;

    for (;;) {
        if (q == 0 && tid == 0) s_j = atomicAdd(ticket, 1);
        cluster.sync();
        const int64_t tk = *cluster.map_shared_rank(&s_j, 0);
        cluster.sync();
        // tickets are sweep-major over the batch: every matrix advances its own wavefront
        const int64_t j = tk / batch, zb = tk % batch;
        if (j >= n - 1) return;
        BandT<S> A{ab_base + zb * sAB, ldab, 2 * BW - 1};
        int *done = done_base + zb * sDone;
        const int nsteps = (int)((n - j - 2) / BW) + 1;
        const int ops_prev = (j > 0) ? 2 * ((int)((n - j - 1) / BW) + 1) : 0;
        int64_t rho = j, c0 = j + 1;
        for (int m = 0; m < nsteps; ++m) {
            const int64_t c1 = min(c0 + BW - 1, n - 1);
            const int L = (int)(c1 - c0 + 1);
            // ================= R op (op 2m) =================
            // The reflector's input (row rho, columns c0..c1) is final once this
            // sweep's previous op and op 2m of sweep j-1 are done -- already
            // waited for when m >= 1 -- so it is formed before the wait for the
            // block (op 2m+3 of sweep j-1); for m == 0 the wait comes first.
            if (m == 0) {
                if (tid == 0 && j > 0) wait_geq(done + j - 1, min(4, ops_prev), err);
                __syncthreads();
            }
            if (L >= 2) {
                if (wid == 0) warp_reflector<S, BW>(A, true, rho, c0, L, sv, &s_tau, &s_beta);
                __syncthreads();
                cluster_arrive();  // this CTA is done reading row rho
            }
            if (m > 0) {
                if (tid == 0 && j > 0) wait_geq(done + j - 1, min(2 * m + 4, ops_prev), err);
                __syncthreads();
            }
            if (L >= 2) {
                const V tau = s_tau;
                if (!Ar::iszero(tau)) {
                    const int rr = tid % Cfg::RPC, g = tid / Cfg::RPC;
                    const int64_t r = rho + 1 + (int64_t)q * Cfg::RPC + rr;
                    const bool rv = (r <= c1);
                    V vals[Cfg::CPG];
#pragma unroll
                    for (int k = 0; k < Cfg::CPG; ++k) {
                        const int ci = g * Cfg::CPG + k;
                        vals[k] = (rv && ci < L) ? Ar::ld(A.at(r, c0 + ci)) : Ar::zero();
                    }
#pragma unroll
                    for (int cc = 0; cc < Cfg::CPT; ++cc) {
                        typename Ar::Acc a0 = Ar::acc_zero(), a1 = Ar::acc_zero();
#pragma unroll
                        for (int kk = 0; kk < Cfg::W0; ++kk) {
                            const int k = cc * Cfg::W0 + kk;
                            const int ci = g * Cfg::CPG + k;
                            if (ci < L) Ar::acc_add((kk & 1) ? a1 : a0, vals[k], sv[ci]);
                        }
                        part[g * Cfg::CPT + cc][rr] = Ar::add(Ar::acc_value(a0), Ar::acc_value(a1));
                    }
                    __syncthreads();
                    if (g == 0) {
                        V w = Ar::zero();
#pragma unroll
                        for (int c = 0; c < Cfg::NCH; ++c) w = Ar::add(w, part[c][rr]);
                        wrow[rr] = Ar::mul(w, tau);
                    }
                    __syncthreads();
                    const V w = wrow[rr];
                    if (rv) {
#pragma unroll
                        for (int k = 0; k < Cfg::CPG; ++k) {
                            const int ci = g * Cfg::CPG + k;
                            if (ci < L) Ar::st(A.at(r, c0 + ci), Ar::sub(vals[k], Ar::mul(w, sv[ci])));
                        }
                    }
                }
                // Every CTA has read row rho (it arrived after its reflector);
                // only then does CTA 0 overwrite it with beta and zeros.
                cluster_wait();
                if (q == 0) {
                    if (tid == 0) Ar::st(A.at(rho, c0), s_beta);
                    for (int i = 1 + tid; i < L; i += blockDim.x) Ar::st(A.at(rho, c0 + i), Ar::zero());
                }
            }
            __threadfence();
            cluster.sync();
            if (q == 0 && tid == 0) st_release(done + j, 2 * m + 1);
            // ================= L op (op 2m+1) =================
            // Column c0 (rows c0..c1) is final after this sweep's R op and op
            // 2m+1 of sweep j-1 (covered by the R op's wait): reflector first.
            if (L >= 2) {
                if (wid == 0) warp_reflector<S, BW>(A, false, c0, c0, L, sv, &s_tau, &s_beta);
                __syncthreads();
                cluster_arrive();  // this CTA is done reading column c0
            }
            if (tid == 0 && j > 0) wait_geq(done + j - 1, min(2 * m + 5, ops_prev), err);
            __syncthreads();
            if (L >= 2) {
                const V tau = s_tau;
                if (!Ar::iszero(tau)) {
                    const int64_t cend = min(c0 + 2 * (int64_t)BW - 1, n - 1);
                    const int64_t cbase = c0 + 1 + (int64_t)q * Cfg::CPC + (int64_t)wid * Cfg::CPW;
                    V vals[Cfg::CPW][Cfg::RPL];
#pragma unroll
                    for (int k = 0; k < Cfg::CPW; ++k) {
                        const int64_t c = cbase + k;
#pragma unroll
                        for (int t = 0; t < Cfg::RPL; ++t) {
                            const int ri = lane + 32 * t;
                            vals[k][t] = (c <= cend && ri < L) ? Ar::ld(A.at(c0 + ri, c)) : Ar::zero();
                        }
                    }
#pragma unroll
                    for (int k = 0; k < Cfg::CPW; ++k) {
                        const int64_t c = cbase + k;
                        typename Ar::Acc acc = Ar::acc_zero();
#pragma unroll
                        for (int t = 0; t < Cfg::RPL; ++t) {
                            const int ri = lane + 32 * t;
                            if (ri < L) Ar::acc_add(acc, sv[ri], vals[k][t]);
                        }
                        const V w = Ar::mul(warp_sum_s<S>(Ar::acc_value(acc)), tau);
                        if (c <= cend) {
#pragma unroll
                            for (int t = 0; t < Cfg::RPL; ++t) {
                                const int ri = lane + 32 * t;
                                if (ri < L) Ar::st(A.at(c0 + ri, c), Ar::sub(vals[k][t], Ar::mul(w, sv[ri])));
                            }
                        }
                    }
                }
                cluster_wait();  // as in the R op: column c0 is overwritten after every CTA has read it
                if (q == 0) {
                    if (tid == 0) Ar::st(A.at(c0, c0), s_beta);
                    for (int i = 1 + tid; i < L; i += blockDim.x) Ar::st(A.at(c0 + i, c0), Ar::zero());
                }
            }
            __threadfence();
            cluster.sync();
            if (q == 0 && tid == 0) st_release(done + j, 2 * m + 2);
            rho = c0;
            c0 += BW;
        }
    }
}

template <int BW, typename S, int CC = ChaseCfg<BW>::C, int NTT = 512>
int launch_chase_cluster(typename ChaseAr<S>::St *dAB, int64_t n, int64_t ldab, const Stage2Work &w, cudaStream_t s,
                         int num_sms, int batch = 1, int64_t sAB = 0, int64_t sDone = 0) {
    using Cfg = ChaseCfg<BW, CC, NTT>;
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = Cfg::C;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.blockDim = dim3(Cfg::NT);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int max_clusters = 0;
    cfg.gridDim = dim3(Cfg::C * 64);
    if (cudaOccupancyMaxActiveClusters(&max_clusters, chase_cluster_kernel<BW, S, CC, NTT>, &cfg) != cudaSuccess ||
        max_clusters <= 0) {
        cudaGetLastError();
        max_clusters = std::max(1, num_sms / Cfg::C);
    }
    // Sweeps in flight are bounded by the wavefront: about (n / bw) / 2 per matrix.
    const int64_t want = std::max<int64_t>(1, ((n / BW) / 2 + 2) * (int64_t)batch);
    const int64_t clusters = std::min<int64_t>(std::min<int64_t>(want, max_clusters), (n - 1) * (int64_t)batch);
    cfg.gridDim = dim3((unsigned)(clusters * Cfg::C));
    AVS_CUDA_TRY(cudaLaunchKernelEx(&cfg, chase_cluster_kernel<BW, S, CC, NTT>, dAB, n, ldab, w.flags, w.flags + 1, w.err,
                                    batch, sAB, sDone));
    return AVS_SUCCESS;
}

template <typename S>
int launch_chase_any(typename ChaseAr<S>::St *dAB, int64_t n, int bw, int64_t ldab, const Stage2Work &w,
                     cudaStream_t s, int num_sms) {
    switch (bw) {
        case 16: return launch_chase_cluster<16, S>(dAB, n, ldab, w, s, num_sms);
        case 32: return launch_chase_cluster<32, S>(dAB, n, ldab, w, s, num_sms);
        case 64: return launch_chase_cluster<64, S>(dAB, n, ldab, w, s, num_sms);
        case 128: return launch_chase_cluster<128, S>(dAB, n, ldab, w, s, num_sms);
        case 256: return launch_chase_cluster<256, S>(dAB, n, ldab, w, s, num_sms);
        default: return AVS_ERR_UNSUPPORTED;
    }
}

// float2 band (double-float) <-> extraction
template <typename T>
__global__ void extract_band_df_kernel(const T *a, int64_t n, int64_t lda, int bw, float2 *ab, int64_t ldab) {
    const int64_t c = blockIdx.x;
    const int ku = 2 * bw - 1;
    for (int i = threadIdx.x; i <= bw; i += blockDim.x) {
        const int64_t r = c - bw + i;
        if (r >= 0) {
            if (sizeof(T) == 4) {
                ab[(ku + r - c) + c * ldab] = make_float2((float)a[r + c * lda], 0.0f);  // exact
            } else {
                const double v = (double)a[r + c * lda];
                const float h = (float)v;
                ab[(ku + r - c) + c * ldab] = make_float2(h, (float)(v - (double)h));
            }
        }
    }
}

__global__ void bidiag_out_df_kernel(const float2 *ab, int64_t n, int bw, int64_t ldab, double *d, double *e) {
    const int ku = 2 * bw - 1;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float2 x = ab[ku + i * ldab];
        d[i] = (double)x.x + (double)x.y;
        if (i + 1 < n) {
            const float2 y = ab[(ku - 1) + (i + 1) * ldab];
            e[i] = (double)y.x + (double)y.y;
        }
    }
}

template <typename T>
__global__ void extract_band_compact_kernel(const T *a, int64_t n, int64_t lda, int bw, double *ab, int64_t ldab) {
    const int64_t c = blockIdx.x;
    const int ku = 2 * bw - 1;
    for (int i = threadIdx.x; i <= bw; i += blockDim.x) {
        const int64_t r = c - bw + i;
        if (r >= 0) ab[(ku + r - c) + c * ldab] = (double)a[r + c * lda];
    }
}

template <typename T>
__global__ void extract_band_dense_kernel(const T *a, int64_t n, int64_t lda, int bw, double *bm, int64_t ldb) {
    const int64_t c = blockIdx.x;
    for (int64_t r = threadIdx.x; r < n; r += blockDim.x) {
        const int64_t d = c - r;
        bm[r + c * ldb] = (d >= 0 && d <= bw) ? (double)a[r + c * lda] : 0.0;
    }
}

__global__ void dense_to_compact_kernel(const double *bm, int64_t n, int64_t ldb, int bw, double *ab, int64_t ldab) {
    const int64_t c = blockIdx.x;
    const int ku = 2 * bw - 1;
    for (int i = threadIdx.x; i <= bw; i += blockDim.x) {
        const int64_t r = c - bw + i;
        if (r >= 0) ab[(ku + r - c) + c * ldab] = bm[r + c * ldb];
    }
}

__global__ void bidiag_out_kernel(const double *ab, int64_t n, int bw, int64_t ldab, double *d, double *e) {
    const int ku = 2 * bw - 1;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        d[i] = ab[ku + i * ldab];
        if (i + 1 < n) e[i] = ab[(ku - 1) + (i + 1) * ldab];
    }
}

// Compute roof of the chase: its inner arithmetic -- a compensated dot product
// over 16 register values, the scaled reflector update of each value -- with
// no memory traffic, on every SM.  One element step is 4 flops (multiply-add of
// the dot, multiply-subtract of the update), the accounting of the chase's flop
// count.
template <typename S>
__global__ void __launch_bounds__(512) chase_rate_kernel(typename ChaseAr<S>::St *out, int iters) {
    using Ar = ChaseAr<S>;
    using V = typename Ar::V;
    constexpr int K = 16;
    V vals[K], sv[K];
    const float seed = 1.0f + 1e-3f * (float)(threadIdx.x & 63);
#pragma unroll
    for (int k = 0; k < K; ++k) {
        vals[k] = Ar::v_from_double(seed + 0.01 * k);
        sv[k] = Ar::v_from_double(0.5 / (k + 1));
    }
    const V tau = Ar::v_from_double(1e-3);
    for (int it = 0; it < iters; ++it) {
        typename Ar::Acc a0 = Ar::acc_zero(), a1 = Ar::acc_zero();
#pragma unroll
        for (int k = 0; k < K; ++k) Ar::acc_add((k & 1) ? a1 : a0, vals[k], sv[k]);
        const V w = Ar::mul(Ar::add(Ar::acc_value(a0), Ar::acc_value(a1)), tau);
#pragma unroll
        for (int k = 0; k < K; ++k) vals[k] = Ar::sub(vals[k], Ar::mul(w, sv[k]));
    }
    V acc = Ar::zero();
#pragma unroll
    for (int k = 0; k < K; ++k) acc = Ar::add(acc, vals[k]);
    Ar::st(out + blockIdx.x * (int64_t)blockDim.x + threadIdx.x, acc);
}

// The same element steps in plain FP32 (the arithmetic of the blocked band
// reduction's applies in the FP32-class modes).
__global__ void __launch_bounds__(512) fp32_rate_kernel(float *out, int iters) {
    constexpr int K = 16;
    float vals[K], sv[K];
    const float seed = 1.0f + 1e-3f * (float)(threadIdx.x & 63);
#pragma unroll
    for (int k = 0; k < K; ++k) {
        vals[k] = seed + 0.01f * k;
        sv[k] = 0.5f / (k + 1);
    }
    for (int it = 0; it < iters; ++it) {
        float a0 = 0.f, a1 = 0.f;
#pragma unroll
        for (int k = 0; k < K; k += 2) {
            a0 = fmaf(vals[k], sv[k], a0);
            a1 = fmaf(vals[k + 1], sv[k + 1], a1);
        }
        const float w = (a0 + a1) * 1e-3f;
#pragma unroll
        for (int k = 0; k < K; ++k) vals[k] = fmaf(-w, sv[k], vals[k]);
    }
    float acc = 0.f;
#pragma unroll
    for (int k = 0; k < K; ++k) acc += vals[k];
    out[blockIdx.x * (int64_t)blockDim.x + threadIdx.x] = acc;
}

}  // namespace

// Measured rate (flops/s, 4 per element step) of the chase arithmetic in
// double-float (mode 0), FP64 (1) or FP32 (2), all SMs busy, timed with events;
// the output buffer is allocated and freed here.
int stage2_rate(int fp64, int num_sms, double *flops_per_s) {
    const int threads = 512, blocks = num_sms * 4;
    const int iters = fp64 == 1 ? 256 : (fp64 == 2 ? 32768 : 8192);
    void *out = nullptr;
    AVS_CUDA_TRY(cudaMalloc(&out, sizeof(double) * (size_t)blocks * threads));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    for (int rep = 0; rep < 4; ++rep) {  // first launch warms up
        cudaEventRecord(e0);
        if (fp64 == 1)
            chase_rate_kernel<double><<<blocks, threads>>>(reinterpret_cast<double *>(out), iters);
        else if (fp64 == 2)
            fp32_rate_kernel<<<blocks, threads>>>(reinterpret_cast<float *>(out), iters);
        else
            chase_rate_kernel<df64><<<blocks, threads>>>(reinterpret_cast<float2 *>(out), iters);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms < best) best = ms;
    }
    const cudaError_t err = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (err != cudaSuccess) {
        set_last_cuda_error(err);
        return AVS_ERR_CUDA;
    }
    *flops_per_s = 4.0 * 16.0 * (double)iters * blocks * threads / (best * 1e-3);
    return AVS_SUCCESS;
}

template <typename T>
int extract_band_compact(const T *dA, int64_t n, int64_t lda, int bw, double *dAB, int64_t ldab, cudaStream_t s) {
    AVS_CUDA_TRY(cudaMemsetAsync(dAB, 0, sizeof(double) * (size_t)ldab * (size_t)n, s));
    extract_band_compact_kernel<T><<<(unsigned)n, 128, 0, s>>>(dA, n, lda, bw, dAB, ldab);
    AVS_CUDA_TRY(cudaGetLastError());
    return AVS_SUCCESS;
}
template int extract_band_compact<float>(const float *, int64_t, int64_t, int, double *, int64_t, cudaStream_t);
template int extract_band_compact<double>(const double *, int64_t, int64_t, int, double *, int64_t, cudaStream_t);

template <typename T>
int extract_band_dense(const T *dA, int64_t n, int64_t lda, int bw, double *dB, int64_t ldb, cudaStream_t s) {
    extract_band_dense_kernel<T><<<(unsigned)n, 256, 0, s>>>(dA, n, lda, bw, dB, ldb);
    AVS_CUDA_TRY(cudaGetLastError());
    return AVS_SUCCESS;
}
template int extract_band_dense<float>(const float *, int64_t, int64_t, int, double *, int64_t, cudaStream_t);
template int extract_band_dense<double>(const double *, int64_t, int64_t, int, double *, int64_t, cudaStream_t);

int dense_band_to_compact(const double *dB, int64_t n, int64_t ldb, int bw, double *dAB, int64_t ldab,
                          cudaStream_t s) {
    AVS_CUDA_TRY(cudaMemsetAsync(dAB, 0, sizeof(double) * (size_t)ldab * (size_t)n, s));
    dense_to_compact_kernel<<<(unsigned)n, 128, 0, s>>>(dB, n, ldb, bw, dAB, ldab);
    AVS_CUDA_TRY(cudaGetLastError());
    return AVS_SUCCESS;
}

int stage2_chase(double *dAB, int64_t n, int bw, int64_t ldab, double *dd, double *de, const Stage2Work &w,
                 cudaStream_t s, int num_sms, int64_t *launches, bool window) {
    if (window && chase_window_supported(bw) && ldab == 3 * (int64_t)bw) {
        const int rc = stage2_chase_window_fp64(dAB, n, bw, w, s, num_sms);
        if (rc != AVS_SUCCESS) return rc;
        if (launches) *launches += 1;
    } else if (n >= 2 && bw >= 2) {
        AVS_CUDA_TRY(cudaMemsetAsync(w.flags, 0, sizeof(int) * (size_t)(n + 1), s));
        int rc = launch_chase_any<double>(dAB, n, bw, ldab, w, s, num_sms);
        if (rc == AVS_ERR_UNSUPPORTED) {
            // any other band width: one CTA per sweep, step-level lag 3
            const int64_t sweeps = n - 1;
            const int64_t want = std::max<int64_t>(1, (n / bw) / 3 + 4);
            const int grid = (int)std::min<int64_t>(std::min<int64_t>(sweeps, want), (int64_t)num_sms * 2);
            chase_kernel<<<grid, kChaseThreads, sizeof(double) * (size_t)bw, s>>>(dAB, n, bw, ldab, w.flags,
                                                                                   w.flags + 1, w.err);
            AVS_CUDA_TRY(cudaGetLastError());
            rc = AVS_SUCCESS;
        }
        if (rc != AVS_SUCCESS) return rc;
        if (launches) *launches += 1;
    }
    const int nb = (int)std::min<int64_t>((n + 255) / 256, 4096);
    bidiag_out_kernel<<<nb > 0 ? nb : 1, 256, 0, s>>>(dAB, n, bw, ldab, dd, de);
    AVS_CUDA_TRY(cudaGetLastError());
    if (launches) *launches += 1;
    return AVS_SUCCESS;
}

// Double-float chase for the pipeline's FP32-class modes (tiles 16..256).
template <typename T>
int stage2_chase_df(const T *dW, int64_t n, int64_t ldw, int bw, float2 *dAB, int64_t ldab, double *dd, double *de,
                    const Stage2Work &w, cudaStream_t s, int num_sms, int64_t *launches, bool window) {
    AVS_CUDA_TRY(cudaMemsetAsync(dAB, 0, sizeof(float2) * (size_t)ldab * (size_t)n, s));
    extract_band_df_kernel<T><<<(unsigned)n, 128, 0, s>>>(dW, n, ldw, bw, dAB, ldab);
    AVS_CUDA_TRY(cudaGetLastError());
    if (window && chase_window_supported(bw) && ldab == 3 * (int64_t)bw) {
        const int rc = stage2_chase_window_df(dAB, n, bw, w, s, num_sms);
        if (rc != AVS_SUCCESS) return rc;
    } else if (n >= 2) {
        AVS_CUDA_TRY(cudaMemsetAsync(w.flags, 0, sizeof(int) * (size_t)(n + 1), s));
        const int rc = launch_chase_any<df64>(dAB, n, bw, ldab, w, s, num_sms);
        if (rc != AVS_SUCCESS) return rc;
    }
    const int nb = (int)std::min<int64_t>((n + 255) / 256, 4096);
    bidiag_out_df_kernel<<<nb > 0 ? nb : 1, 256, 0, s>>>(dAB, n, bw, ldab, dd, de);
    AVS_CUDA_TRY(cudaGetLastError());
    if (launches) *launches += 3;
    return AVS_SUCCESS;
}
template int stage2_chase_df<float>(const float *, int64_t, int64_t, int, float2 *, int64_t, double *, double *,
                                    const Stage2Work &, cudaStream_t, int, int64_t *, bool);
template int stage2_chase_df<double>(const double *, int64_t, int64_t, int, float2 *, int64_t, double *, double *,
                                     const Stage2Work &, cudaStream_t, int, int64_t *, bool);

// Hierarchical stage 2: the blocked band reduction bw -> tbw (stage2_band.cu;
// the reference's bidiag! stage, BRD/src/bulgechasing2.jl:22-45), then the
// element chase tbw -> 1 above.
int stage2_chase_hier_df(const float *dW, int64_t n, int64_t ldw, int bw, int tbw, float *dAB1, float2 *dAB2,
                         double *dd, double *de, const Stage2Work &w, cudaStream_t s, int num_sms, int64_t *launches,
                         bool window, cudaEvent_t after_band) {
    const int64_t ldab1 = band_ldab(bw), ldab2 = 3 * (int64_t)tbw;
    int rc;
    if ((rc = dense_to_band<float, float>(dW, n, ldw, 0, bw, dAB1, ldab1, 0, 1, s)) != AVS_SUCCESS) return rc;
    if ((rc = band_stage<float>(dAB1, n, bw, tbw, ldab1, w, s, num_sms, 1, 0, 0)) != AVS_SUCCESS) return rc;
    if (after_band) AVS_CUDA_TRY(cudaEventRecord(after_band, s));
    if ((rc = band_to_band<float, float2>(dAB1, n, bw, ldab1, 0, tbw, dAB2, ldab2, 0, 1, s)) != AVS_SUCCESS)
        return rc;
    if (window && chase_window_supported(tbw)) {
        if ((rc = stage2_chase_window_df(dAB2, n, tbw, w, s, num_sms)) != AVS_SUCCESS) return rc;
    } else if (n >= 2) {
        AVS_CUDA_TRY(cudaMemsetAsync(w.flags, 0, sizeof(int) * (size_t)(n + 1), s));
        if ((rc = launch_chase_any<df64>(dAB2, n, tbw, ldab2, w, s, num_sms)) != AVS_SUCCESS) return rc;
    }
    const int nb = (int)std::min<int64_t>((n + 255) / 256, 4096);
    bidiag_out_df_kernel<<<nb > 0 ? nb : 1, 256, 0, s>>>(dAB2, n, tbw, ldab2, dd, de);
    AVS_CUDA_TRY(cudaGetLastError());
    if (launches) *launches += 5;
    return AVS_SUCCESS;
}

int stage2_chase_hier_fp64(const double *dW, int64_t n, int64_t ldw, int bw, int tbw, double *dAB1, double *dAB2,
                           double *dd, double *de, const Stage2Work &w, cudaStream_t s, int num_sms,
                           int64_t *launches, bool window, cudaEvent_t after_band) {
    const int64_t ldab1 = band_ldab(bw), ldab2 = 3 * (int64_t)tbw;
    int rc;
    if ((rc = dense_to_band<double, double>(dW, n, ldw, 0, bw, dAB1, ldab1, 0, 1, s)) != AVS_SUCCESS) return rc;
    if ((rc = band_stage<double>(dAB1, n, bw, tbw, ldab1, w, s, num_sms, 1, 0, 0)) != AVS_SUCCESS) return rc;
    if (after_band) AVS_CUDA_TRY(cudaEventRecord(after_band, s));
    if ((rc = band_to_band<double, double>(dAB1, n, bw, ldab1, 0, tbw, dAB2, ldab2, 0, 1, s)) != AVS_SUCCESS)
        return rc;
    if (window && chase_window_supported(tbw)) {
        if ((rc = stage2_chase_window_fp64(dAB2, n, tbw, w, s, num_sms)) != AVS_SUCCESS) return rc;
    } else if (n >= 2) {
        AVS_CUDA_TRY(cudaMemsetAsync(w.flags, 0, sizeof(int) * (size_t)(n + 1), s));
        if ((rc = launch_chase_any<double>(dAB2, n, tbw, ldab2, w, s, num_sms)) != AVS_SUCCESS) return rc;
    }
    const int nb = (int)std::min<int64_t>((n + 255) / 256, 4096);
    bidiag_out_kernel<<<nb > 0 ? nb : 1, 256, 0, s>>>(dAB2, n, tbw, ldab2, dd, de);
    AVS_CUDA_TRY(cudaGetLastError());
    if (launches) *launches += 5;
    return AVS_SUCCESS;
}

// ---------------------------------------------------------------------------
// Batched chase: `batch` matrices of the same order n and band width bw,
// stacked at stride n*n (tiles) / ldab*n (band) / n+1 (flags) / n (d, e).
// S = df64 (FP32 tiles, the FP32-class modes) or double (FP64 tiles).
namespace {
template <typename T, typename S>
__global__ void extract_band_batched(const T *a, int64_t n, int bw, typename ChaseAr<S>::St *ab, int64_t ldab) {
    const int64_t c = blockIdx.x, zb = blockIdx.y;
    const int ku = 2 * bw - 1;
    const T *az = a + zb * n * n;
    typename ChaseAr<S>::St *abz = ab + zb * ldab * n;
    for (int i = threadIdx.x; i <= bw; i += blockDim.x) {
        const int64_t r = c - bw + i;
        if (r >= 0) {
            if constexpr (sizeof(typename ChaseAr<S>::St) == sizeof(float2) && sizeof(T) == 4 &&
                          !std::is_same<S, double>::value)
                abz[(ku + r - c) + c * ldab] = make_float2((float)az[r + c * n], 0.0f);  // exact
            else
                abz[(ku + r - c) + c * ldab] = ChaseAr<S>::from_double((double)az[r + c * n]);
        }
    }
}
template <typename S>
__global__ void bidiag_out_batched(const typename ChaseAr<S>::St *ab, int64_t n, int bw, int64_t ldab, double *d,
                                   double *e, int batch, int64_t sAB) {
    const int ku = 2 * bw - 1;
    const int64_t total = n * (int64_t)batch;
    for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < total; g += (int64_t)gridDim.x * blockDim.x) {
        const int64_t zb = g / n, i = g % n;
        const typename ChaseAr<S>::St *abz = ab + zb * sAB;
        d[zb * n + i] = st_to_double(abz[ku + i * ldab]);
        e[zb * n + i] = (i + 1 < n) ? st_to_double(abz[(ku - 1) + (i + 1) * ldab]) : 0.0;
    }
}
}  // namespace

// Batched stage 2, the same choices as a single call's run_stages23 (so a
// matrix's values do not depend on its batch): tbw > 0: the blocked band
// reduction bw -> tbw (arithmetic T, band dAB as T elements, band_stride(bw,
// n) per matrix), then the element chase of the narrow band (dAB2, 3 tbw x n per
// matrix); tbw == 0: the element chase from width bw.  window: the element
// chase in the shared-memory window (bands 8/16/32) instead of clusters.
template <typename T, typename S>
int stage2_chase_batched(const T *dW, int64_t n, int bw, int batch, typename ChaseAr<S>::St *dAB, int64_t ldab,
                         double *dd, double *de, const Stage2Work &w, cudaStream_t s, int num_sms,
                         int64_t *launches, int tbw, bool window, typename ChaseAr<S>::St *dAB2) {
    using St = typename ChaseAr<S>::St;
    if (tbw > 0) {
        T *ab1 = reinterpret_cast<T *>(dAB);
        const int64_t ldab1 = band_ldab(bw), sAB1 = band_stride(bw, n), ldab2 = 3 * (int64_t)tbw, sAB2 = ldab2 * n;
        int rc;
        if ((rc = dense_to_band<T, T>(dW, n, n, n * n, bw, ab1, ldab1, sAB1, batch, s)) != AVS_SUCCESS) return rc;
        if ((rc = band_stage<T>(ab1, n, bw, tbw, ldab1, w, s, num_sms, batch, sAB1, n + 1)) != AVS_SUCCESS)
            return rc;
        if ((rc = band_to_band<T, St>(ab1, n, bw, ldab1, sAB1, tbw, dAB2, ldab2, sAB2, batch, s)) != AVS_SUCCESS)
            return rc;
        if (window && chase_window_supported(tbw)) {
            rc = std::is_same<S, df64>::value
                     ? stage2_chase_window_df(reinterpret_cast<float2 *>(dAB2), n, tbw, w, s, num_sms, batch, sAB2)
                     : stage2_chase_window_fp64(reinterpret_cast<double *>(dAB2), n, tbw, w, s, num_sms, batch,
                                                sAB2);
        } else {
            AVS_CUDA_TRY(cudaMemsetAsync(w.flags, 0, sizeof(int) * (size_t)((n + 1) * (int64_t)batch + 1), s));
            rc = tbw == 16 ? launch_chase_cluster<16, S, 1>(dAB2, n, ldab2, w, s, num_sms, batch, sAB2, n + 1)
                           : launch_chase_cluster<32, S, 2>(dAB2, n, ldab2, w, s, num_sms, batch, sAB2, n + 1);
        }
        if (rc != AVS_SUCCESS) return rc;
        const int nb = (int)std::min<int64_t>((n * batch + 255) / 256, 8192);
        bidiag_out_batched<S><<<nb > 0 ? nb : 1, 256, 0, s>>>(dAB2, n, tbw, ldab2, dd, de, batch, sAB2);
        AVS_CUDA_TRY(cudaGetLastError());
        if (launches) *launches += 5;
        return AVS_SUCCESS;
    }
    AVS_CUDA_TRY(cudaMemsetAsync(dAB, 0, sizeof(St) * (size_t)ldab * (size_t)n * batch, s));
    extract_band_batched<T, S><<<dim3((unsigned)n, (unsigned)batch), 128, 0, s>>>(dW, n, bw, dAB, ldab);
    AVS_CUDA_TRY(cudaGetLastError());
    if (window && chase_window_supported(bw) && ldab == 3 * (int64_t)bw) {
        const int rc = std::is_same<S, df64>::value
                           ? stage2_chase_window_df(reinterpret_cast<float2 *>(dAB), n, bw, w, s, num_sms, batch,
                                                    ldab * n)
                           : stage2_chase_window_fp64(reinterpret_cast<double *>(dAB), n, bw, w, s, num_sms, batch,
                                                      ldab * n);
        if (rc != AVS_SUCCESS) return rc;
    } else if (n >= 2) {
        AVS_CUDA_TRY(cudaMemsetAsync(w.flags, 0, sizeof(int) * (size_t)((n + 1) * (int64_t)batch + 1), s));
        int rc;
        // small bands: few, small CTAs per sweep (the batch supplies the
        // parallelism).  Measured on the 4096-matrix workload (orders 64..1024;
        // the matrices each band divides), stage 2, CTAs per cluster x threads:
        // band 32: 1 x 128 499 ms, 2 x 64 503, 2 x 128 554, 2 x 256 588,
        // 2 x 512 979, 1 x 512 1035; band 64: 2 x 128 670, 1 x 256 687,
        // 1 x 512 876, 2/4 x 512 1251/1223; band 128: 2 x 512 1278, 4 x 256
        // 1281, 4/8 x 512 1879/3289.
        // The small CTAs pay only while the batch keeps every SM busy with
        // several sweeps (a sweep has about (n / bw) / 2 siblings in flight);
        // a short batch is latency-bound and keeps 512-thread CTAs.  Every
        // configuration of a band width computes the same bits (fixed
        // reduction order), so a matrix's values do not depend on its batch.
        // A batch whose sweeps in flight fit twice in the GPU with the single
        // call's clusters (C = 8 at bands >= 128, 4 at 64, 2 at 32) is
        // latency-bound and takes them: e.g. one n = 8192 matrix at band 128.
        const int64_t inflight = (int64_t)batch * std::max<int64_t>(1, (n / bw) / 2);
        const bool wide = inflight >= 4 * (int64_t)num_sms;
        const int cdef = bw >= 128 ? 8 : (bw == 64 ? 4 : (bw == 32 ? 2 : 1));
        const bool narrow = inflight <= 2 * (int64_t)(num_sms / cdef);
        const int64_t sAB = ldab * n, sF = n + 1;
        switch (bw) {
            case 16: rc = launch_chase_cluster<16, S, 1>(dAB, n, ldab, w, s, num_sms, batch, sAB, sF); break;
            case 32:
                rc = wide     ? launch_chase_cluster<32, S, 1, 128>(dAB, n, ldab, w, s, num_sms, batch, sAB, sF)
                               : launch_chase_cluster<32, S, 2>(dAB, n, ldab, w, s, num_sms, batch, sAB, sF);
                break;
            case 64:
                rc = wide     ? launch_chase_cluster<64, S, 2, 128>(dAB, n, ldab, w, s, num_sms, batch, sAB, sF)
                     : narrow ? launch_chase_cluster<64, S, 4>(dAB, n, ldab, w, s, num_sms, batch, sAB, sF)
                              : launch_chase_cluster<64, S, 1>(dAB, n, ldab, w, s, num_sms, batch, sAB, sF);
                break;
            case 128:
                rc = narrow ? launch_chase_cluster<128, S, 8>(dAB, n, ldab, w, s, num_sms, batch, sAB, sF)
                            : launch_chase_cluster<128, S, 2>(dAB, n, ldab, w, s, num_sms, batch, sAB, sF);
                break;
            case 256: rc = launch_chase_cluster<256, S, 8>(dAB, n, ldab, w, s, num_sms, batch, sAB, sF); break;
            default: rc = AVS_ERR_UNSUPPORTED;
        }
        if (rc != AVS_SUCCESS) return rc;
    }
    const int nb = (int)std::min<int64_t>((n * batch + 255) / 256, 8192);
    bidiag_out_batched<S><<<nb > 0 ? nb : 1, 256, 0, s>>>(dAB, n, bw, ldab, dd, de, batch, ldab * n);
    AVS_CUDA_TRY(cudaGetLastError());
    if (launches) *launches += 3;
    return AVS_SUCCESS;
}

int stage2_chase_df_batched(const float *dW, int64_t n, int bw, int batch, float2 *dAB, int64_t ldab, double *dd,
                            double *de, const Stage2Work &w, cudaStream_t s, int num_sms, int64_t *launches, int tbw,
                            bool window, float2 *dAB2) {
    return stage2_chase_batched<float, df64>(dW, n, bw, batch, dAB, ldab, dd, de, w, s, num_sms, launches, tbw,
                                             window, dAB2);
}

int stage2_chase_df_batched(const double *dW, int64_t n, int bw, int batch, float2 *dAB, int64_t ldab, double *dd,
                            double *de, const Stage2Work &w, cudaStream_t s, int num_sms, int64_t *launches,
                            bool window) {
    return stage2_chase_batched<double, df64>(dW, n, bw, batch, dAB, ldab, dd, de, w, s, num_sms, launches, 0, window,
                                              nullptr);
}

int stage2_chase_fp64_batched(const double *dW, int64_t n, int bw, int batch, double *dAB, int64_t ldab, double *dd,
                              double *de, const Stage2Work &w, cudaStream_t s, int num_sms, int64_t *launches,
                              int tbw, bool window, double *dAB2) {
    return stage2_chase_batched<double, double>(dW, n, bw, batch, dAB, ldab, dd, de, w, s, num_sms, launches, tbw,
                                                window, dAB2);
}

}  // namespace avs
