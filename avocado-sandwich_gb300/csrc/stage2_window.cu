// Stage 2b: element bulge chase of a narrow band (width BW = 8, 16, 32) ->
// upper bidiagonal, with G consecutive sweeps per CTA in a shared-memory
// window.
//
// The ops are those of the element chase in stage2_chase.cu (the reference's
// bidiagonalize / block_bidiagonalize! with target width 1, KAbasedSVD/src/
// bulgechasing.jl:18-40): sweep j, step m, pivot column c0 = j + 1 + m BW,
// c1 = min(c0 + BW - 1, n - 1):
//   R op: a right reflector from row rho (= j for m = 0, c0 - BW after)
//     over columns c0..c1, applied to rows rho+1..c1;
//   L op: a left reflector from column c0 over rows c0..c1, applied to
//     columns c0+1..min(c0 + 2BW - 1, n - 1).
// Op k of sweep j touches nothing that ops >= k+4 of sweep j-1 touch.
//
// Layout of the work.  A CTA owns the sweeps j0 .. j0+G-1 (groups handed out
// in order by a ticket); compute warp i runs sweep j0+i, op t - 4i at tick t,
// so the G sweeps advance in lockstep with the minimal lag, and all their
// data stays in a window of W columns of the band in shared memory (column c
// in slot c mod W).  A producer warp moves the band between the window and
// global memory: before tick t it has loaded (cp.async, 16-byte chunks, L2
// only) every column the tick touches, and it prefetches the columns of tick
// t+3; after tick t it marks as retired the columns that no sweep of the
// group touches again (those left of the trailing sweep's next pivot).  A
// publisher warp writes retired columns back and publishes the boundary in
// retired[g] (fence, release), off the ticks' critical path.  The next
// group's producer loads a column only once retired[g] has passed it, so it
// sees every update of this group, and this group never touches a column
// again once it is retired: the result is the sequential chase's, bit for
// bit, whatever the timing.  Compute warps touch only shared memory;
// named barriers hand each tick between the producer and the compute warps.
// Every wait on another CTA is bounded (kDevTimeout).
//
// Band storage in global memory: the element chase's compact form, A(r, c) at
// AB[(r - c + 2BW - 1) + c * ldab], ldab = 3 BW.
#include <algorithm>

#include "avs_common.cuh"
#include "chase_ar.cuh"

namespace avs {
namespace {

template <int BW, int G>
struct WinCfg {
    static constexpr int KU = 2 * BW - 1;
    static constexpr int LDAB = 3 * BW;         // storage rows per column (global)
    static constexpr int LDW = 3 * BW + 2;      // window column stride (16-byte multiple; odd stride - 1)
    static constexpr int W = 2 * G * BW + 2 * BW;  // window columns (span of a group's ops + prefetch)
    static constexpr int NC = 32 * G;           // compute threads: one warp per sweep
    static constexpr int D = 4;                 // ticks of the mbarrier ring (producer lookahead)
    static constexpr int NT = NC + 64;          // + the producer and the publisher warps
    static constexpr int CHUNKS = LDAB * 8 / 16;  // 16-byte chunks per column
    static_assert(BW % 2 == 0 && BW <= 32, "window chase band");
    static constexpr size_t smem_bytes() { return 8 * ((size_t)W * LDW + (size_t)G * 32); }
};

__device__ __forceinline__ unsigned smem_addr(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void cp_async16(void *dst, const void *src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait_group() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }
__device__ __forceinline__ void bar_sync(int id, int cnt) { asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(cnt) : "memory"); }
__device__ __forceinline__ void bar_arrive(int id, int cnt) {
    asm volatile("bar.arrive %0, %1;" ::"r"(id), "r"(cnt) : "memory");
}

// mbarriers of the tick ring: the producer's copies arrive on them
// (cp.async.mbarrier.arrive.noinc: when all of the lane's earlier copies have
// landed), the compute warps wait on the phase of their tick
__device__ __forceinline__ void mbar_init(unsigned long long *m, unsigned cnt) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(m)), "r"(cnt) : "memory");
}
__device__ __forceinline__ void mbar_inval(unsigned long long *m) {
    asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_addr(m)) : "memory");
}
__device__ __forceinline__ void cp_async_mbar_arrive(unsigned long long *m) {
    asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" ::"r"(smem_addr(m)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long *m, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(m)), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ int ld_volatile_shared(const int *p) { return *(const volatile int *)p; }
__device__ __forceinline__ void st_volatile_shared(int *p, int v) { *(volatile int *)p = v; }
__device__ __forceinline__ int ld_relaxed(const int *p) {
    int v;
    asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Bounded waits on a shared-memory counter written by another warp of the CTA
// (kWaitNs of %globaltimer, kSpinLimit polls); on timeout kDevTimeout.
__device__ __forceinline__ bool wait_shared_geq(const int *p, int target, int *err) {
    const unsigned long long t0 = global_ns();
    for (long long it = 0; ld_volatile_shared(p) < target; ++it) {
        if (it > kSpinLimit || ((it & 255) == 255 && (long long)(global_ns() - t0) > kWaitNs)) {
            atomicCAS(err, kDevOk, kDevTimeout);
            return false;
        }
        __nanosleep(32);
    }
    return true;
}
// Bounded wait for a phase of an mbarrier (kWaitNs, kSpinLimit polls); on
// timeout kDevTimeout and false.
__device__ __forceinline__ bool mbar_wait(unsigned long long *m, unsigned parity, int *err) {
    const unsigned long long t0 = global_ns();
    for (long long it = 0; !mbar_try_wait(m, parity); ++it) {
        if (it > kSpinLimit || ((it & 63) == 63 && (long long)(global_ns() - t0) > kWaitNs)) {
            atomicCAS(err, kDevOk, kDevTimeout);
            return false;
        }
    }
    return true;
}
// returns the counter once it exceeds v (or v after a timeout)
__device__ __forceinline__ int wait_shared_gt(const int *p, int v, int *err) {
    const unsigned long long t0 = global_ns();
    for (long long it = 0;; ++it) {
        const int x = ld_volatile_shared(p);
        if (x > v) return x;
        if (it > kSpinLimit || ((it & 255) == 255 && (long long)(global_ns() - t0) > kWaitNs)) {
            atomicCAS(err, kDevOk, kDevTimeout);
            return v;
        }
        __nanosleep(32);
    }
}

template <typename S>
__device__ __forceinline__ typename ChaseAr<S>::V wsum(typename ChaseAr<S>::V v) {
    using Ar = ChaseAr<S>;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = Ar::add(v, Ar::shfl_xor(v, o));
    return v;
}

// Per-sweep op geometry.
struct WOp {
    int c0, c1, hi;  // pivot column, last column of the reflector, last column touched
};
template <int BW>
__device__ __forceinline__ int wops(int64_t n, int j) { return 2 * ((int)((n - j - 2) / BW) + 1); }
template <int BW>
__device__ __forceinline__ WOp wop(int64_t n, int j, int k) {
    WOp o;
    o.c0 = j + 1 + (k >> 1) * BW;
    const int last = (int)(n - 1);
    o.c1 = min(o.c0 + BW - 1, last);
    o.hi = min(o.c0 + ((k & 1) ? 2 * BW - 1 : BW - 1), last);
    return o;
}

template <int BW, typename S, int G>
__global__ void __launch_bounds__(WinCfg<BW, G>::NT, 1)
    chase_win_kernel(typename ChaseAr<S>::St *ab_base, int64_t n, int batch, int64_t sAB, int *ticket,
                     int *retired_base, int64_t sRet, int *err) {
    using Cfg = WinCfg<BW, G>;
    using Ar = ChaseAr<S>;
    using V = typename Ar::V;
    using St = typename Ar::St;
    static_assert(sizeof(St) == 8 && sizeof(V) == 8, "8-byte band elements");
    constexpr int KU = Cfg::KU, LDW = Cfg::LDW, W = Cfg::W, NC = Cfg::NC, NT = Cfg::NT, LDAB = Cfg::LDAB;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    St *win = reinterpret_cast<St *>(smem_raw);  // [W][LDW]
    V *vbuf = reinterpret_cast<V *>(win + (size_t)W * LDW);  // [G][32]: each compute warp's reflector
    __shared__ int s_g;
    __shared__ int s_tick, s_wb;  // ticks the compute warps have finished; columns below s_wb written back
    __shared__ __align__(8) unsigned long long s_full[Cfg::D];  // tick t's columns are in: phase t / D of [t % D]
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    if (tid == 0)
        for (int d = 0; d < Cfg::D; ++d) mbar_init(&s_full[d], 32);
    const int nsweeps = (int)(n - 1);
    const int ngroups = (nsweeps + G - 1) / G;
    auto A = [&](int r, int c) -> St * { return win + (size_t)(c % W) * LDW + (r - c + KU); };

    for (;;) {
        if (tid == 0) s_g = atomicAdd(ticket, 1);
        __syncthreads();
        const int tk = s_g;
        __syncthreads();
        // tickets are group-major over the batch: every matrix advances its own wavefront
        const int g = tk / batch, zb = tk % batch;
        if (g >= ngroups) return;
        St *ab = ab_base + (size_t)zb * sAB;
        int *retired = retired_base + (size_t)zb * sRet;
        const int j0 = g * G;
        if (tid == 0) {
            s_tick = 0;
            s_wb = j0 + 1;
        }
        __syncthreads();
        const int gs = min(G, nsweeps - j0);
        int nticks = 0;
        for (int i = 0; i < gs; ++i) nticks = max(nticks, 4 * i + wops<BW>(n, j0 + i));
        // columns [lo, .. ) not yet retired; the tick's highest column + 1
        auto tick_need = [&](int t) -> int {
            int need = 0;
            for (int i = 0; i < gs; ++i) {
                const int k = t - 4 * i;
                if (k >= 0 && k < wops<BW>(n, j0 + i)) need = max(need, wop<BW>(n, j0 + i, k).hi + 1);
            }
            return need;
        };
        // after tick t: the lowest column any op of a later tick touches (n: none)
        auto retire_after = [&](int t) -> int {
            int lo = (int)n;
            for (int i = 0; i < gs; ++i) {
                const int k = t + 1 - 4 * i;
                if (k < wops<BW>(n, j0 + i)) lo = min(lo, wop<BW>(n, j0 + i, max(k, 0)).c0);
            }
            return lo;
        };

        if (wid == G) {
            // ---------------- producer warp: global -> window ----------------
            // Each tick's copies arrive on the tick's mbarrier as they land; the
            // producer runs up to D - 1 ticks ahead of the compute warps (the
            // mbarrier ring) and never sits between two ticks.
            int issued = j0 + 1;               // columns below are requested (cp.async)
            int rp = (g == 0) ? (int)n : 0;    // retired[g-1] as last observed
            int rp_next = rp;                  // lane 0: a relaxed read in flight, used next tick
            // copies of the columns [from, to) into their slots (one column per step, lanes over chunks)
            auto copy_in = [&](int from, int to) {
                int sl = from % W;
                for (int c = from; c < to; ++c) {
                    for (int h = lane; h < Cfg::CHUNKS; h += 32)
                        cp_async16(win + (size_t)sl * LDW + 2 * h, ab + (size_t)c * LDAB + 2 * h);
                    if (++sl == W) sl = 0;
                }
            };
            for (int t = 0; t < nticks; ++t) {
                const int need = tick_need(t);
                if (t >= Cfg::D) {  // the ring slot of tick t is free once the compute warps are past tick t - D
                    if (lane == 0) wait_shared_geq(&s_tick, t - Cfg::D + 1, err);
                    __syncwarp();
                }
                if (issued < need) {
                    // not prefetched (the previous group was behind): load now
                    if (rp < need) {
                        if (lane == 0) wait_geq(retired + g - 1, need, err);
                        __syncwarp();
                        rp = max(need, __shfl_sync(0xffffffffu, lane == 0 ? ld_acquire(retired + g - 1) : 0, 0));
                    }
                    if (need > ld_volatile_shared(&s_wb) + W) {  // free slots (bounded wait on the publisher)
                        if (lane == 0) wait_shared_geq(&s_wb, need - W, err);
                        __syncwarp();
                    }
                    copy_in(issued, need);
                    issued = need;
                }
                cp_async_mbar_arrive(&s_full[t % Cfg::D]);  // tick t: when this lane's copies so far have landed
                // lane 0's read of the previous group's boundary, issued last tick.  The
                // copies of the columns it releases are issued only once the value has
                // arrived (their range depends on it) and read L2, where the previous
                // group's writes were made visible before its release.
                rp = max(rp, __shfl_sync(0xffffffffu, rp_next, 0));
                if (g > 0 && rp < (int)n && lane == 0) rp_next = ld_relaxed(retired + g - 1);
                // prefetch the columns of the next three ticks that the previous group
                // has retired and whose slots are free
                const int tgt = min(min(tick_need(t + 3), rp), min(ld_volatile_shared(&s_wb) + W, (int)n));
                if (tgt > issued) {
                    copy_in(issued, tgt);
                    issued = tgt;
                }
            }
            cp_wait_all();
        } else if (wid == G + 1) {
            // ---------------- publisher warp: window -> global, retired[g] ----------------
            // Follows the compute warps' progress: after tick t-1 the columns left
            // of retire_after(t-1) are final for this group; they are written back
            // and the boundary is released for the next group.
            int wb = j0 + 1, seen = 0;
            for (;;) {
                int tk = seen;
                if (lane == 0) tk = wait_shared_gt(&s_tick, seen, err);
                tk = __shfl_sync(0xffffffffu, tk, 0);
                if (tk <= seen) break;  // only after a timeout (recorded)
                seen = tk;
                const int r = (tk >= nticks) ? (int)n : retire_after(tk - 1);
                if (r > wb) {
                    __threadfence_block();
                    int sl = wb % W;
                    for (int c = wb; c < r; ++c) {
                        for (int h = lane; h < Cfg::CHUNKS; h += 32) {
                            const uint4 v = *reinterpret_cast<const uint4 *>(win + (size_t)sl * LDW + 2 * h);
                            *reinterpret_cast<uint4 *>(ab + (size_t)c * LDAB + 2 * h) = v;
                        }
                        if (++sl == W) sl = 0;
                    }
                    __syncwarp();
                    wb = r;
                    if (lane == 0) {
                        st_volatile_shared(&s_wb, wb);  // the slots may be refilled
                        __threadfence();
                        st_release(retired + g, wb);
                    }
                }
                if (tk >= nticks) break;
            }
        } else {
            // ---------------- compute warps: warp i runs sweep j0 + i ----------------
            // (one warp per sweep: measured faster than two warps sharing a sweep's
            // reflector and halving its apply, 239 vs 300 ms at n = 16384)
            const int sw = wid;
            const int j = j0 + sw;
            const int ops = (sw < gs) ? wops<BW>(n, j) : 0;
            V *sv = vbuf + wid * 32;
            for (int t = 0; t < nticks; ++t) {
                bar_sync(1, Cfg::NC);  // every compute warp is done with tick t-1
                if (wid == 0 && lane == 0) {
                    __threadfence_block();
                    st_volatile_shared(&s_tick, t);  // ticks < t are done (publisher, producer)
                }
                mbar_wait(&s_full[t % Cfg::D], (unsigned)(t / Cfg::D) & 1u, err);  // tick t's columns are in
                const int k = t - 4 * sw;
                if (k >= 0 && k < ops) {
                    const WOp o = wop<BW>(n, j, k);
                    const int L = o.c1 - o.c0 + 1;
                    if (L >= 2) {
                        const bool rop = (k & 1) == 0;
                        const int rho = rop ? ((k == 0) ? j : o.c0 - BW) : o.c0;
                        // reflector input: row rho (R op) or column c0 (L op), columns/rows c0..c1
                        V x = Ar::zero();
                        if (lane < L) x = Ar::lds(rop ? A(rho, o.c0 + lane) : A(o.c0 + lane, o.c0));
                        typename Ar::Acc acc = Ar::acc_zero();
                        if (lane >= 1 && lane < L) Ar::acc_add(acc, x, x);
                        const V s = wsum<S>(Ar::acc_value(acc));
                        const V alpha = Ar::shfl(x, 0);
                        V tau = Ar::zero(), beta = alpha, scal = Ar::zero();
                        if (Ar::gt0(s)) {
                            const V nrm = Ar::sqrt(Ar::fma(alpha, alpha, s));
                            beta = Ar::ge0(alpha) ? Ar::neg(nrm) : nrm;
                            tau = Ar::mul(Ar::sub(beta, alpha), Ar::rcp(beta));
                            scal = Ar::rcp(Ar::sub(alpha, beta));
                        }
                        if (lane < L) sv[lane] = (lane == 0) ? Ar::one() : Ar::mul(x, scal);
                        __syncwarp();
                        if (!Ar::iszero(tau)) {
                            // column c0 + i sits in slot s0 + i (wrapping at W): one modulo per op
                            const int s0 = o.c0 % W;
                            if (rop) {
                                // lane = row r: A(r, c0 + i) at slot(c0 + i) * LDW + (r - c0 - i + KU);
                                // from column to column the address moves by LDW - 1 (- W LDW at the wrap)
                                for (int r = rho + 1 + lane; r <= o.c1; r += 32) {
                                    St *p0 = win + (size_t)s0 * LDW + (r - o.c0 + KU);
                                    V xv[BW];
                                    typename Ar::Acc a = Ar::acc_zero();
                                    {
                                        St *p = p0;
#pragma unroll
                                        for (int i = 0; i < BW; ++i) {
                                            if (i < L) {
                                                xv[i] = Ar::lds(p);
                                                Ar::acc_add(a, xv[i], sv[i]);
                                            }
                                            p += LDW - 1;
                                            if (s0 + i + 1 == W) p -= (size_t)W * LDW;
                                        }
                                    }
                                    const V w = Ar::mul(Ar::acc_value(a), tau);
                                    St *p = p0;
#pragma unroll
                                    for (int i = 0; i < BW; ++i) {
                                        if (i < L) Ar::st(p, Ar::sub(xv[i], Ar::mul(w, sv[i])));
                                        p += LDW - 1;
                                        if (s0 + i + 1 == W) p -= (size_t)W * LDW;
                                    }
                                }
                            } else {
                                // lane = column c: rows c0 .. c0+L-1 contiguous from A(c0, c)
                                for (int c = o.c0 + 1 + lane; c <= o.hi; c += 32) {
                                    int sl = s0 + (c - o.c0);
                                    sl -= (sl >= W) ? W : 0;
                                    St *p = win + (size_t)sl * LDW + (o.c0 - c + KU);
                                    V xv[BW];
                                    typename Ar::Acc a = Ar::acc_zero();
#pragma unroll
                                    for (int i = 0; i < BW; ++i) {
                                        if (i < L) {
                                            xv[i] = Ar::lds(p + i);
                                            Ar::acc_add(a, sv[i], xv[i]);
                                        }
                                    }
                                    const V w = Ar::mul(Ar::acc_value(a), tau);
#pragma unroll
                                    for (int i = 0; i < BW; ++i)
                                        if (i < L) Ar::st(p + i, Ar::sub(xv[i], Ar::mul(w, sv[i])));
                                }
                            }
                        }
                        // the pivot row / column: beta and zeros (every lane has read it:
                        // the norm's shuffles came after the reads)
                        if (lane < L) {
                            St *p = rop ? A(rho, o.c0 + lane) : A(o.c0 + lane, o.c0);
                            Ar::st(p, lane == 0 ? beta : Ar::zero());
                        }
                    }
                }
                __syncwarp();
            }
            bar_sync(1, Cfg::NC);
            if (wid == 0 && lane == 0) {
                __threadfence_block();
                st_volatile_shared(&s_tick, nticks);  // all ticks done
            }
        }
        __syncthreads();
        if (tid == 0) {  // fresh phases for the next group
            for (int d = 0; d < Cfg::D; ++d) {
                mbar_inval(&s_full[d]);
                mbar_init(&s_full[d], 32);
            }
        }
    }
}

template <int BW, typename S, int G>
int launch_win(typename ChaseAr<S>::St *dAB, int64_t n, const Stage2Work &w, cudaStream_t s, int num_sms, int batch,
               int64_t sAB) {
    using Cfg = WinCfg<BW, G>;
    const size_t smem = Cfg::smem_bytes();
    auto kern = chase_win_kernel<BW, S, G>;
    AVS_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, Cfg::NT, smem) != cudaSuccess || per_sm < 1) {
        cudaGetLastError();
        per_sm = 1;
    }
    const int64_t ngroups = ((n - 1) + G - 1) / G;
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(ngroups * batch, (int64_t)num_sms * per_sm));
    kern<<<grid, Cfg::NT, smem, s>>>(dAB, n, batch, sAB, w.flags, w.flags + 1, n + 1, w.err);
    AVS_CUDA_TRY(cudaGetLastError());
    return AVS_SUCCESS;
}

}  // namespace

bool chase_window_supported(int bw) { return bw == 8 || bw == 16 || bw == 32; }

// The band (width bw, compact storage with ldab = 3 bw) -> bidiagonal, in
// place.  w.flags: n + 2 ints (zeroed here).
template <typename S>
static int chase_window(typename ChaseAr<S>::St *dAB, int64_t n, int bw, const Stage2Work &w, cudaStream_t s,
                        int num_sms, int batch, int64_t sAB) {
    if (n < 2 || batch < 1) return AVS_SUCCESS;
    if (n > ((int64_t)1 << 30) || (int64_t)batch * n > ((int64_t)1 << 31) - 64) return AVS_ERR_UNSUPPORTED;
    AVS_CUDA_TRY(cudaMemsetAsync(w.flags, 0, sizeof(int) * (size_t)((n + 1) * (int64_t)batch + 1), s));
    switch (bw) {
        case 8: return launch_win<8, S, 8>(dAB, n, w, s, num_sms, batch, sAB);
        // band 16: 8 sweeps per CTA for one matrix (n = 16384: 322 ms of stage 2 against 334 with 4); 4 for
        // batches, whose matrices give the launch enough groups (512 matrices of order 256: 31.8 against
        // 35.8 ms); the values do not depend on it
        case 16: return batch > 1 ? launch_win<16, S, 4>(dAB, n, w, s, num_sms, batch, sAB)
                                  : launch_win<16, S, 8>(dAB, n, w, s, num_sms, batch, sAB);
        case 32: return launch_win<32, S, 3>(dAB, n, w, s, num_sms, batch, sAB);
        default: return AVS_ERR_UNSUPPORTED;
    }
}
int stage2_chase_window_df(float2 *dAB, int64_t n, int bw, const Stage2Work &w, cudaStream_t s, int num_sms,
                           int batch, int64_t sAB) {
    return chase_window<df64>(dAB, n, bw, w, s, num_sms, batch, sAB);
}
int stage2_chase_window_fp64(double *dAB, int64_t n, int bw, const Stage2Work &w, cudaStream_t s, int num_sms,
                             int batch, int64_t sAB) {
    return chase_window<double>(dAB, n, bw, w, s, num_sms, batch, sAB);
}

}  // namespace avs
