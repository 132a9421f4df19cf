// Chain of the tensor-core trailing update on tcgen05.
//
// For one column strip of the top tile row (NS = 32 columns) the chain runs
// the tiles of the panel in order (TiledMatrix.jl:107-113 / QRkernels.jl:165-197
// order: GEQRT tile first, then the TSQRT tiles top to bottom):
//
//   p = 0 (GEQRT):  W = T0^T S_0,           Top -= Y0 W
//   p >= 1 (TSQRT): W = T_p^T (Top + S_p),  Top -= W,  W_p = W (operand planes)
//
// where S_p = Y_p^T A_p came from the batched tensor-core GEMM.  Each product
// is one tcgen05 MMA sequence: the b x b factor (T_p^T, or Y0) is the A
// operand, loaded by TMA from its K-major operand planes through a two-stage
// ring; the strip operand (Top + S_p, or W0) is the B operand, written into
// shared memory by the CTA's threads in the canonical 128-byte-swizzled
// K-major layout; the accumulator (b rows x 32 columns, two 128-lane halves
// for b = 256) lives in tensor memory.  Both factors are triangular (T_p^T
// and Y0 lower triangular in (row, k)), so the K blocks right of the first
// half's diagonal block are skipped.  Top stays in shared memory (FP32) for
// the whole chain; at the end it goes to the matrix and, transposed, to the
// other buffer (the next half-step's panel column), and each strip raises its
// tile's counter so that panel can start on the tiles already finished.
#include <cuda_bf16.h>

#include "avs_common.cuh"
#include "tc_gemm.cuh"

namespace avs {
namespace {

constexpr int NS = kChainStrip;  // strip columns

struct ChainTcArgs {
    float *x;
    int64_t n;
    int pr, pc, P;
    const float *S;  // [P][ntr][b]
    int64_t ntr;
    void *w_hi, *w_lo;  // [P][ntr][b] operand planes of W_p
    int fmt;
    int *err;
    float *xt;  // optional: the final top strip transposed, xt[(j0 + c) + (top0 + l) * n]
    int *ready; // optional: ready[strip / (B / NS)] += 1 once the strip's values are in memory
};

template <int B, bool SPLIT, bool BF16>
struct CCfg {
    // threads: one warp per TMEM lane quadrant (b = 128: two CTAs fit an SM),
    // or two (b = 256: one CTA per SM, so eight warps hide the epilogue's latency)
    static constexpr int CNT = B == 256 ? 256 : 128;
    static constexpr int EB = BF16 ? 2 : 4;
    static constexpr int BK = 128 / EB;           // K elements per 128-byte block
    static constexpr int NKB = B / BK;            // K blocks
    static constexpr int HALVES = B / 128;        // 128-row halves of the factor
    static constexpr int PL = SPLIT ? 2 : 1;      // operand planes
    static constexpr int ZT = NS * 128;           // bytes of one B tile (32 rows x 128 B)
    static constexpr int ZPLANE = NKB * ZT;       // bytes of one B plane
    static constexpr int AT = 128 * 128;          // bytes of one A tile (128 rows x 128 B)
    static constexpr int ASTAGE = HALVES * PL * AT;
    static constexpr int TS = B + 1;              // top strip: column stride (padded for the transposed read)
    static constexpr int TOP = TS * NS * 4;       // FP32 top strip
    static constexpr int SMEM = 1024 + PL * ZPLANE + 2 * ASTAGE + TOP;
    static constexpr int TCOLS = HALVES * NS;     // TMEM columns of the accumulator
    static constexpr int TALLOC = TCOLS < 32 ? 32 : TCOLS;
};

template <int B, bool SPLIT, bool BF16>
__global__ void __launch_bounds__(CCfg<B, SPLIT, BF16>::CNT, 1)
    chain_tc_kernel(const __grid_constant__ CUtensorMap tT_hi, const __grid_constant__ CUtensorMap tT_lo,
                    const __grid_constant__ CUtensorMap tY_hi, const __grid_constant__ CUtensorMap tY_lo,
                    ChainTcArgs args) {
    using C = CCfg<B, SPLIT, BF16>;
    using namespace tc;
    constexpr int CNT = C::CNT;
    extern __shared__ uint8_t smem_dyn[];
    __shared__ uint64_t full[2], empty[2], done;
    __shared__ uint32_t tmem_base;
    __shared__ int s_fail;
    uint8_t *base = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_dyn) + 1023) & ~(uintptr_t)1023);
    uint8_t *zbuf = base;                               // B operand planes
    uint8_t *abuf = zbuf + C::PL * C::ZPLANE;           // A ring: [stage][half][plane]
    float *top = reinterpret_cast<float *>(abuf + 2 * C::ASTAGE);  // [c][l], column stride TS
    const int tid = threadIdx.x, wid = tid >> 5, lane = tid & 31;
    const int64_t js = (int64_t)blockIdx.x * NS;
    const int64_t j0 = (int64_t)(args.pc + 1) * B + js;
    const int64_t top0 = (int64_t)args.pr * B;
    const int64_t n = args.n;

    if (tid == 0) {
        for (int s = 0; s < 2; ++s) {
            mbar_init(smem_u32(&full[s]), 1);
            mbar_init(smem_u32(&empty[s]), 1);
        }
        mbar_init(smem_u32(&done), 1);
        s_fail = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (wid == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                     "r"(C::TALLOC));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    // strip elements owned by this thread in the element-wise passes:
    // element i is (c, l) = ((tid + CNT i) / B, (tid + CNT i) % B)
    constexpr int E = B * NS / CNT;
    {
        float v[E];
#pragma unroll
        for (int i = 0; i < E; ++i) {
            const int idx = tid + CNT * i, c = idx / B, l = idx % B;
            v[i] = args.x[(top0 + l) + (j0 + c) * n];
        }
#pragma unroll
        for (int i = 0; i < E; ++i) {
            const int idx = tid + CNT * i;
            top[(idx / B) * C::TS + idx % B] = v[i];
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_base;
    const uint32_t id = idesc(128, NS, BF16);
    int gblk = 0;      // K blocks issued through the ring so far
    int dphase = 0;    // completed products (parity of `done`)
    bool ok = true;

    auto a_tile = [&](int s, int h, int pl) -> uint32_t {
        return smem_u32(abuf) + (uint32_t)(s * C::ASTAGE + (h * C::PL + pl) * C::AT);
    };
    auto z_tile = [&](int pl, int kb) -> uint32_t { return smem_u32(zbuf) + (uint32_t)(pl * C::ZPLANE + kb * C::ZT); };
    // halves of the factor that are nonzero in K block kb (lower triangular)
    auto halves_in = [&](int kb) { return (kb * C::BK < 128) ? 0 : 1; };  // first half used

    // One product: accumulator = factor rows [a_row0, a_row0 + B) (A) x strip operand (B).
    auto product = [&](const CUtensorMap *ah, const CUtensorMap *al, int a_row0) {
        if (tid == 0) {
            for (int kb = 0; kb < C::NKB; ++kb) {
                const int g = gblk + kb, s = g & 1;
                if (g >= 2 && !mbar_wait(smem_u32(&empty[s]), (uint32_t)(((g >> 1) - 1) & 1), args.err)) {
                    s_fail = 1;
                    break;
                }
                const int h0 = halves_in(kb);
                const uint32_t fb = smem_u32(&full[s]);
                mbar_expect_tx(fb, (uint32_t)((C::HALVES - h0) * C::PL * C::AT));
                for (int h = h0; h < C::HALVES; ++h) {
                    tma_load_2d(a_tile(s, h, 0), ah, kb * C::BK, a_row0 + h * 128, fb);
                    if (SPLIT) tma_load_2d(a_tile(s, h, 1), al, kb * C::BK, a_row0 + h * 128, fb);
                }
            }
        } else if (tid == 32) {
            for (int kb = 0; kb < C::NKB; ++kb) {
                const int g = gblk + kb, s = g & 1;
                if (!mbar_wait(smem_u32(&full[s]), (uint32_t)((g >> 1) & 1), args.err)) {
                    s_fail = 1;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                for (int h = halves_in(kb); h < C::HALVES; ++h) {
                    const uint32_t d = tmem + (uint32_t)(h * NS);
#pragma unroll
                    for (int ks = 0; ks < 4; ++ks) {
                        const uint32_t ko = ks * 32;
                        const uint64_t da = desc_sw128(a_tile(s, h, 0) + ko), db = desc_sw128(z_tile(0, kb) + ko);
                        const uint32_t acc = (kb > 0 || ks > 0) ? 1u : 0u;
                        if (SPLIT) {
                            mma<BF16>(d, desc_sw128(a_tile(s, h, 1) + ko), db, id, acc);
                            mma<BF16>(d, da, desc_sw128(z_tile(1, kb) + ko), id, 1u);
                            mma<BF16>(d, da, db, id, 1u);
                        } else {
                            mma<BF16>(d, da, db, id, acc);
                        }
                    }
                }
                mma_commit(smem_u32(&empty[s]));
            }
            mma_commit(smem_u32(&done));
        }
        gblk += C::NKB;
        __syncwarp();
        ok = mbar_wait(smem_u32(&done), (uint32_t)(dphase & 1), args.err) && ok;
        ++dphase;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        ok = ok && !*(volatile int *)&s_fail;
    };
    // strip operand element (row c, k) into the B planes
    auto put_z = [&](int c, int k, float z) {
        const int kb = k / C::BK, kk = k % C::BK;
        if constexpr (BF16) {
            const __nv_bfloat16 h = __float2bfloat16_rn(z);
            *reinterpret_cast<__nv_bfloat16 *>(zbuf + kb * C::ZT + swz2(c, kk)) = h;
            if (SPLIT)
                *reinterpret_cast<__nv_bfloat16 *>(zbuf + C::ZPLANE + kb * C::ZT + swz2(c, kk)) =
                    __float2bfloat16_rn(z - __bfloat162float(h));
        } else {
            const uint32_t h = rna_tf32(z);
            *reinterpret_cast<uint32_t *>(zbuf + kb * C::ZT + swz4(c, kk)) = h;
            if (SPLIT)
                *reinterpret_cast<uint32_t *>(zbuf + C::ZPLANE + kb * C::ZT + swz4(c, kk)) =
                    rna_tf32(z - __uint_as_float(h));
        }
    };
    // The accumulator part this thread reads back: warp w reads TMEM lanes
    // 32 (w % 4) ..; the two warps of a lane quadrant take the two 128-row
    // halves (b = 256) or the two 16-column halves of the strip (b = 128).
    // Row my_l, columns my_c0 .. my_c0 + EC - 1.
    constexpr int GRP = CNT / 128;
    constexpr bool BY_HALF = C::HALVES >= GRP;
    constexpr int EC = BY_HALF ? NS : NS / GRP;
    const int quad = wid & 3, grp = wid >> 2;
    const int my_h = BY_HALF ? grp : 0;
    const int my_c0 = BY_HALF ? 0 : grp * EC;
    const int my_l = my_h * 128 + 32 * quad + lane;
    auto read_acc = [&](float (&v)[EC]) {
        const uint32_t ta = tmem + ((uint32_t)(32 * quad) << 16) + (uint32_t)(my_h * NS + my_c0);
#pragma unroll
        for (int c16 = 0; c16 < EC; c16 += 16) {
            float a[16];
            tmem_ld16(ta + c16, a);
#pragma unroll
            for (int q = 0; q < 16; ++q) v[c16 + q] = a[q];
        }
    };

    // S_p strip values of this thread, loaded one tile ahead (in flight
    // during the previous tile's products)
    float sv[E];
    auto load_s = [&](int p) {
        const float *Sp = args.S + ((size_t)p * args.ntr + js) * B;
#pragma unroll
        for (int i = 0; i < E; ++i) sv[i] = Sp[tid + CNT * i];  // Sp[c * B + l]
    };
    load_s(0);
    for (int p = 0; p < args.P; ++p) {
#pragma unroll
        for (int i = 0; i < E; ++i) {
            const int idx = tid + CNT * i, c = idx / B, l = idx % B;
            put_z(c, l, p > 0 ? sv[i] + top[c * C::TS + l] : sv[i]);
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (p + 1 < args.P) load_s(p + 1);
        product(&tT_hi, &tT_lo, p * B);  // W = T_p^T Z
        if (p == 0) {
            // W0 becomes the strip operand of Top -= Y0 W0
            {
                float v[EC];
                read_acc(v);
#pragma unroll
                for (int c = 0; c < EC; ++c) put_z(my_c0 + c, my_l, v[c]);
            }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncthreads();
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            product(&tY_hi, &tY_lo, 0);  // Y0 W0
            {
                float v[EC];
                read_acc(v);
#pragma unroll
                for (int c = 0; c < EC; ++c) top[(my_c0 + c) * C::TS + my_l] -= v[c];
            }
        } else {
            float v[EC];
            read_acc(v);
#pragma unroll
            for (int c = 0; c < EC; ++c) {
                top[(my_c0 + c) * C::TS + my_l] -= v[c];
                if (ok)
                    tc::put_operand(args.fmt, args.w_hi, args.w_lo, ((int64_t)p * args.ntr + js + my_c0 + c) * B + my_l,
                                    v[c]);
            }
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    }
    if (ok) {
#pragma unroll
        for (int i = 0; i < E; ++i) {
            const int idx = tid + CNT * i, c = idx / B, l = idx % B;
            args.x[(top0 + l) + (j0 + c) * n] = top[c * C::TS + l];
        }
        if (args.xt) {  // a warp writes 32 consecutive columns of one row: 128 bytes
#pragma unroll
            for (int i = 0; i < E; ++i) {
                const int idx = tid + CNT * i, c = idx % NS, l = idx / NS;
                args.xt[(j0 + c) + (top0 + l) * n] = top[c * C::TS + l];
            }
        }
        if (args.ready) __threadfence();  // this thread's values, before the strip is released
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    // release the strip to the panel that waits for its tile
    if (args.ready && tid == 0 && ok) {
        __threadfence();
        atomicAdd(args.ready + blockIdx.x / (B / NS), 1);
    }
    if (wid == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(C::TALLOC));
}

__global__ void tplanes_kernel(const float *t, int64_t count, int fmt, void *hi, void *lo) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x)
        tc::put_operand(fmt, hi, lo, i, t[i]);
}

template <int B, bool SPLIT, bool BF16>
int launch_chain_tc(const ChainTcArgs &a, const CUtensorMap (&m)[4], cudaStream_t s) {
    using C = CCfg<B, SPLIT, BF16>;
    static_assert(C::SMEM <= 232448, "chain shared memory");
    static std::atomic<bool> attr{false};
    if (!attr) {
        AVS_CUDA_TRY(cudaFuncSetAttribute(chain_tc_kernel<B, SPLIT, BF16>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM));
        attr = true;
    }
    chain_tc_kernel<B, SPLIT, BF16><<<(unsigned)(a.ntr / NS), C::CNT, C::SMEM, s>>>(m[0], m[1], m[2], m[3], a);
    AVS_CUDA_TRY(cudaGetLastError());
    return AVS_SUCCESS;
}

}  // namespace

// Operand planes of the T factors of one half-step (tfull: [P][b*b] FP32, T(l,
// l') at l + l'*b) into t_hi/t_lo.
int stage1_chain_tplanes(const float *tfull, int b, int P, int fmt, void *t_hi, void *t_lo, cudaStream_t s) {
    tplanes_kernel<<<512, 256, 0, s>>>(tfull, (int64_t)P * b * b, fmt, t_hi, t_lo);
    AVS_CUDA_TRY(cudaGetLastError());
    return AVS_SUCCESS;
}

// Chain of one half-step on the tensor cores.  t_hi/t_lo: the T factors'
// operand planes (stage1_chain_tplanes); yrow: the Y planes [P][t][l] (tile 0 =
// the masked GEQRT Y0).
int stage1_chain_tc2(float *x, int64_t n, int b, int pr, int pc, int P, void *t_hi, void *t_lo, const void *y_hi,
                     const void *y_lo, const float *S, int64_t ntr, void *w_hi, void *w_lo, int fmt, int *err,
                     cudaStream_t s, float *xt_out, int *ready) {
    if (ntr <= 0) return AVS_SUCCESS;
    if (ntr % NS) return AVS_ERR_INTERNAL;
    const bool bf = tc::fmt_bf16(fmt), split = tc::fmt_split(fmt);
    CUtensorMap m[4];
    const void *planes[4] = {t_hi, split ? t_lo : t_hi, y_hi, split ? y_lo : y_hi};
    for (int i = 0; i < 4; ++i) {
        tc::Operand op{const_cast<void *>(planes[i]), nullptr, b, (int64_t)P * b, b};
        if (!tc::make_tmap(&m[i], op, op.hi, 128, bf)) return AVS_ERR_INTERNAL;
    }
    ChainTcArgs a{x, n, pr, pc, P, S, ntr, w_hi, w_lo, fmt, err, xt_out, ready};
    if (b == 256) {
        if (fmt == tc::kTF32) return launch_chain_tc<256, false, false>(a, m, s);
        if (fmt == tc::kTF32X3) return launch_chain_tc<256, true, false>(a, m, s);
        if (fmt == tc::kBF16) return launch_chain_tc<256, false, true>(a, m, s);
        if (fmt == tc::kBF16X3) return launch_chain_tc<256, true, true>(a, m, s);
    } else if (b == 128) {
        if (fmt == tc::kTF32) return launch_chain_tc<128, false, false>(a, m, s);
        if (fmt == tc::kTF32X3) return launch_chain_tc<128, true, false>(a, m, s);
        if (fmt == tc::kBF16) return launch_chain_tc<128, false, true>(a, m, s);
        if (fmt == tc::kBF16X3) return launch_chain_tc<128, true, true>(a, m, s);
    }
    return AVS_ERR_UNSUPPORTED;
}

}  // namespace avs
