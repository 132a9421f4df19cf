// tcgen05 GEMM for the tensor-core trailing updates (TF32 and split TF32).
//
// D[M x N] = A[M x K] * B[K x N] for a batch of problems, FP32 in global
// memory, TF32 tensor-core products accumulated in FP32 in tensor memory.
// One CTA (4 warps) computes a 128 x 128 tile of D:
//   * all threads stream A and B in 32-wide K blocks from global memory
//     (either major order), round each value to TF32 (and, for the split
//     mode, also the TF32 residual x - hi), and store them into shared memory
//     in the canonical K-major 128-byte-swizzled layout (8-row atoms of
//     1024 B; the 16-byte chunk c of row r sits at chunk c ^ (r & 7));
//   * one thread issues tcgen05.mma (kind::tf32, M = 128, N = 128, K = 8) on
//     shared-memory descriptors -- per K step hi*hi, or hi*hi + hi*lo + lo*hi
//     for the split mode (FP32-class products) -- and commits them to an
//     mbarrier that frees the shared-memory stage (two stages, so the loads of
//     block k+1 overlap the products of block k);
//   * the epilogue reads the accumulator with tcgen05.ld (warp w owns TMEM
//     lanes 32w..32w+31, i.e. rows of D) and applies one of the fused updates
//     the compact-WY trailing update needs.
// Every wait is bounded; a timeout sets the device status word.
#include <cuda_runtime.h>

#include "avs_common.cuh"

namespace avs {
namespace tc {

constexpr int BM = 128, BN = 128, BK = 32;
constexpr int NT = 128;
constexpr int STAGES = 2;
constexpr int TILE_BYTES = BM * BK * 4;  // 16 KB: 128 rows x 128 B
constexpr int TMEM_COLS = 256;           // accumulator uses BN = 128 of them
constexpr int SMEM_PAD = 32 * 1024;      // slack after the last stage

enum Epi : int {
    kStore = 0,     // C = D
    kSub = 1,       // C -= D
    kTopUpdate = 2  // C -= D (C is the top rows), W = D, Z += C_new (if Z)
};
enum AMask : int { kNoMask = 0, kUnitLowerT = 1, kUnitLower = 2 };

struct GemmArgs {
    const float *A;
    int64_t lda, strideA;
    int a_kmajor, a_mask;
    const float *B;
    int64_t ldb, strideB;
    int b_kmajor;
    float *C;
    int64_t ldc, strideC;
    int c_colmajor;
    float *W;
    int64_t ldw, strideW;
    float *Z;
    int64_t ldz;
    int M, N, K;
    int epi, split;
    int *err;
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ uint32_t to_tf32(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return r;
}

// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row atoms
// 1024 B apart (SBO), leading offset unused for this layout (1), version 1.
__device__ __forceinline__ uint64_t desc_sw128(uint32_t addr) {
    uint64_t d = 0;
    d |= (uint64_t)((addr >> 4) & 0x3FFFu);
    d |= (uint64_t)1u << 16;
    d |= (uint64_t)(1024u >> 4) << 32;
    d |= (uint64_t)1u << 46;
    d |= (uint64_t)2u << 61;
    return d;
}

// Instruction descriptor, kind::tf32: D FP32, A/B TF32, both K-major, M x N.
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N) {
    return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n"
        :
        : "r"(d_tmem), "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void mma_commit(uint32_t mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
                 : "memory");
}

__device__ __forceinline__ void mbar_init(uint32_t mbar, int count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar), "r"(count) : "memory");
}

// Bounded wait for the completion of phase `parity` of an mbarrier.
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity, int *err) {
    for (long long it = 0; it < kSpinLimit; ++it) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.b32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(mbar), "r"(parity)
            : "memory");
        if (done) return true;
        if ((it & 1023) == 1023 && ld_acquire(err) != kDevOk) return false;
    }
    atomicCAS(err, kDevOk, kDevTimeout);
    return false;
}

__device__ __forceinline__ uint32_t swz(int r, int k) {
    return (uint32_t)((r >> 3) * 1024 + (r & 7) * 128 + ((((k >> 2) ^ (r & 7)) << 4) | ((k & 3) << 2)));
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// Store one value of a tile: (r, k) of the tile, split into hi (and lo).
__device__ __forceinline__ void put(uint8_t *hi, uint8_t *lo, int r, int k, float x, bool split) {
    const uint32_t off = swz(r, k);
    const uint32_t h = to_tf32(x);
    *reinterpret_cast<uint32_t *>(hi + off) = h;
    if (split) *reinterpret_cast<uint32_t *>(lo + off) = to_tf32(x - __uint_as_float(h));
}

__device__ __forceinline__ void put4(uint8_t *hi, uint8_t *lo, int r, int k, float4 x, bool split) {
    const uint32_t off = swz(r, k);  // k % 4 == 0: one 16-byte chunk
    uint4 h = make_uint4(to_tf32(x.x), to_tf32(x.y), to_tf32(x.z), to_tf32(x.w));
    *reinterpret_cast<uint4 *>(hi + off) = h;
    if (split) {
        uint4 l = make_uint4(to_tf32(x.x - __uint_as_float(h.x)), to_tf32(x.y - __uint_as_float(h.y)),
                             to_tf32(x.z - __uint_as_float(h.z)), to_tf32(x.w - __uint_as_float(h.w)));
        *reinterpret_cast<uint4 *>(lo + off) = l;
    }
}

__device__ __forceinline__ float amask(int mask, int64_t m, int64_t k, float v) {
    if (mask == kUnitLowerT) return (k == m) ? 1.0f : (k > m ? v : 0.0f);
    if (mask == kUnitLower) return (m == k) ? 1.0f : (m > k ? v : 0.0f);
    return v;
}

// Load the 128 x 32 block (rows r0.., k0..) of an operand into (hi, lo).
// kmajor: element (row, k) at p[k + row * ld]; else at p[row + k * ld].
__device__ __forceinline__ void load_tile(const float *p, int64_t ld, int kmajor, int mask, int64_t r0, int64_t k0,
                                          uint8_t *hi, uint8_t *lo, bool split) {
    const int tid = threadIdx.x;
    if (kmajor) {
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            const int idx = tid + NT * i;
            const int r = idx >> 3, c4 = idx & 7;
            float4 v = __ldg(reinterpret_cast<const float4 *>(p + (k0 + 4 * c4) + (r0 + r) * ld));
            if (mask) {
                v.x = amask(mask, r0 + r, k0 + 4 * c4 + 0, v.x);
                v.y = amask(mask, r0 + r, k0 + 4 * c4 + 1, v.y);
                v.z = amask(mask, r0 + r, k0 + 4 * c4 + 2, v.z);
                v.w = amask(mask, r0 + r, k0 + 4 * c4 + 3, v.w);
            }
            put4(hi, lo, r, 4 * c4, v, split);
        }
    } else {
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            const int idx = tid + NT * i;
            const int kk = idx >> 5, m4 = idx & 31;
            const float4 v = __ldg(reinterpret_cast<const float4 *>(p + (r0 + 4 * m4) + (k0 + kk) * ld));
            const float e[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
            for (int q = 0; q < 4; ++q)
                put(hi, lo, 4 * m4 + q, kk, mask ? amask(mask, r0 + 4 * m4 + q, k0 + kk, e[q]) : e[q], split);
        }
    }
}

__global__ void __launch_bounds__(NT) tc_gemm_kernel(GemmArgs g) {
    extern __shared__ uint8_t smem_dyn[];
    __shared__ uint64_t mbar[STAGES];
    __shared__ uint32_t tmem_base;
    const bool split = g.split == 3;
    // 1024-byte aligned tiles: per stage A_hi, B_hi (, A_lo, B_lo)
    uint8_t *base = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_dyn) + 1023) & ~(uintptr_t)1023);
    const int per_stage = (split ? 4 : 2) * TILE_BYTES;
    const int tid = threadIdx.x, wid = tid >> 5, lane = tid & 31;
    const int64_t z = blockIdx.z;
    const int64_t m0 = (int64_t)blockIdx.y * BM, n0 = (int64_t)blockIdx.x * BN;
    const float *A = g.A + z * g.strideA;
    const float *B = g.B + z * g.strideB;

    if (tid == 0) {
        for (int s = 0; s < STAGES; ++s) mbar_init(smem_u32(&mbar[s]), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (wid == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                     "r"(TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_base;
    const uint32_t idesc = idesc_tf32(BM, BN);
    const int nkb = g.K / BK;
    bool ok = true;

    for (int kb = 0; kb < nkb; ++kb) {
        const int s = kb % STAGES;
        uint8_t *st = base + s * per_stage;
        uint8_t *a_hi = st, *b_hi = st + TILE_BYTES;
        uint8_t *a_lo = st + 2 * TILE_BYTES, *b_lo = st + 3 * TILE_BYTES;
        if (kb >= STAGES) ok = mbar_wait(smem_u32(&mbar[s]), (uint32_t)((kb / STAGES - 1) & 1), g.err) && ok;
        load_tile(A, g.lda, g.a_kmajor, g.a_mask, m0, (int64_t)kb * BK, a_hi, a_lo, split);
        load_tile(B, g.ldb, g.b_kmajor, kNoMask, n0, (int64_t)kb * BK, b_hi, b_lo, split);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
            for (int ks = 0; ks < BK / 8; ++ks) {
                const uint32_t koff = ks * 32;  // 8 TF32 values = 32 bytes along K
                const uint64_t ah = desc_sw128(smem_u32(a_hi) + koff), bh = desc_sw128(smem_u32(b_hi) + koff);
                mma_tf32(tmem, ah, bh, idesc, (kb > 0 || ks > 0) ? 1u : 0u);
                if (split) {
                    const uint64_t al = desc_sw128(smem_u32(a_lo) + koff), bl = desc_sw128(smem_u32(b_lo) + koff);
                    mma_tf32(tmem, ah, bl, idesc, 1u);
                    mma_tf32(tmem, al, bh, idesc, 1u);
                }
            }
            mma_commit(smem_u32(&mbar[s]));
        }
        __syncthreads();
    }
    {
        const int s = (nkb - 1) % STAGES;
        ok = mbar_wait(smem_u32(&mbar[s]), (uint32_t)(((nkb - 1) / STAGES) & 1), g.err) && ok;
    }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");

    // ---- epilogue: warp w owns rows m0 + 32w + lane
    const int64_t m = m0 + 32 * wid + lane;
    float *C = g.C + z * g.strideC;
    for (int c16 = 0; c16 < BN / 16; ++c16) {
        float v[16];
        tmem_ld16(tmem + ((uint32_t)(32 * wid) << 16) + (uint32_t)(c16 * 16), v);
        if (!ok) continue;
#pragma unroll
        for (int q = 0; q < 16; ++q) {
            const int64_t nn = n0 + c16 * 16 + q;
            float *cp = g.c_colmajor ? (C + m + nn * g.ldc) : (C + nn + m * g.ldc);
            if (g.epi == kStore) {
                *cp = v[q];
            } else if (g.epi == kSub) {
                *cp = *cp - v[q];
            } else {
                const float cn = *cp - v[q];
                *cp = cn;
                if (g.W) g.W[z * g.strideW + m + nn * g.ldw] = v[q];
                if (g.Z) g.Z[m + nn * g.ldz] += cn;
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (wid == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS));
}

}  // namespace tc

int tc_gemm(const tc::GemmArgs &a, int batch, cudaStream_t s) {
    if (a.M % tc::BM || a.N % tc::BN || a.K % tc::BK || batch <= 0) return AVS_ERR_INTERNAL;
    const int smem = (a.split == 3 ? 4 : 2) * tc::TILE_BYTES * tc::STAGES + 1024 + tc::SMEM_PAD;
    static std::atomic<bool> attr{false};
    if (!attr) {
        AVS_CUDA_TRY(cudaFuncSetAttribute(tc::tc_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          4 * tc::TILE_BYTES * tc::STAGES + 1024 + tc::SMEM_PAD));
        attr = true;
    }
    dim3 grid((unsigned)(a.N / tc::BN), (unsigned)(a.M / tc::BM), (unsigned)batch);
    tc::tc_gemm_kernel<<<grid, tc::NT, smem, s>>>(a);
    AVS_CUDA_TRY(cudaGetLastError());
    return AVS_SUCCESS;
}

// ---------------------------------------------------------------------------
// Trailing update of one half-step on the tensor cores (FP32 tiles, tile 128
// or 256).  View element (i, j) is a[i + j*lda] (layout 0) or a[j + i*lda]
// (layout 1); the panel occupies view rows pr*b.., columns pc*b..pc*b+b-1; the
// trailing columns start at j0 = (pc+1)*b.  T_p comes from tbuild (tfull,
// column-major b x b per tile); S and Wb hold P slots of b x N (ld b).
int stage1_update_tc(float *a, int64_t lda, int64_t n, int b, int layout, int pr, int pc, int P, const float *tfull,
                     float *S, float *Wb, int split, int *err, cudaStream_t s) {
    const int64_t j0 = (int64_t)(pc + 1) * b;
    const int64_t N = n - j0;
    if (N <= 0) return AVS_SUCCESS;
    const int64_t top0 = (int64_t)pr * b, col0 = (int64_t)pc * b;
    auto vptr = [&](int64_t i, int64_t j) { return layout == 0 ? a + i + j * lda : a + j + i * lda; };
    const int64_t tile_step = layout == 0 ? (int64_t)b : (int64_t)b * lda;  // view row tile -> next
    const int64_t slot = (int64_t)b * N;
    int rc;
    tc::GemmArgs g;
    auto base = [&]() {
        tc::GemmArgs x = {};
        x.M = b; x.N = (int)N; x.K = b; x.split = split; x.err = err;
        return x;
    };
    // Y^T operand (m = l, k = t) of the tile whose view rows start at r0
    auto set_yt = [&](tc::GemmArgs &x, int64_t r0) {
        x.A = vptr(r0, col0); x.lda = lda; x.a_kmajor = layout == 0 ? 1 : 0;
    };
    // Y operand (m = t, k = l)
    auto set_y = [&](tc::GemmArgs &x, int64_t r0) {
        x.A = vptr(r0, col0); x.lda = lda; x.a_kmajor = layout == 0 ? 0 : 1;
    };
    // view rows r0.., trailing columns as B (k = t, n = c) or as C (m = t, n = c)
    auto set_b_rows = [&](tc::GemmArgs &x, int64_t r0) {
        x.B = vptr(r0, j0); x.ldb = lda; x.b_kmajor = layout == 0 ? 1 : 0;
    };
    auto set_c_rows = [&](tc::GemmArgs &x, int64_t r0) {
        x.C = vptr(r0, j0); x.ldc = lda; x.c_colmajor = layout == 0 ? 1 : 0;
    };
    // 1. S_p = Y_p^T A_p for p = 1..P-1 (independent of one another)
    if (P > 1) {
        g = base();
        set_yt(g, top0 + b); g.strideA = tile_step;
        set_b_rows(g, top0 + b); g.strideB = tile_step;
        g.C = S + slot; g.ldc = b; g.strideC = slot; g.c_colmajor = 1;
        g.epi = tc::kStore;
        if ((rc = tc_gemm(g, P - 1, s)) != AVS_SUCCESS) return rc;
    }
    // 2. S_0 = Y0^T Top (unit lower Y0 from the GEQRT tile)
    g = base();
    set_yt(g, top0); g.a_mask = tc::kUnitLowerT;
    set_b_rows(g, top0);
    g.C = S; g.ldc = b; g.c_colmajor = 1; g.epi = tc::kStore;
    if ((rc = tc_gemm(g, 1, s)) != AVS_SUCCESS) return rc;
    // 3. W_0 = T_0^T S_0
    g = base();
    g.A = tfull; g.lda = b; g.a_kmajor = 1;
    g.B = S; g.ldb = b; g.b_kmajor = 1;
    g.C = Wb; g.ldc = b; g.c_colmajor = 1; g.epi = tc::kStore;
    if ((rc = tc_gemm(g, 1, s)) != AVS_SUCCESS) return rc;
    // 4. Top -= Y0 W_0, and Z_1 = Top + S_1
    g = base();
    set_y(g, top0); g.a_mask = tc::kUnitLower;
    g.B = Wb; g.ldb = b; g.b_kmajor = 1;
    set_c_rows(g, top0);
    g.epi = tc::kTopUpdate; g.W = nullptr;
    g.Z = P > 1 ? S + slot : nullptr; g.ldz = b;
    if ((rc = tc_gemm(g, 1, s)) != AVS_SUCCESS) return rc;
    // 5. for each TSQRT tile in order: W_p = T_p^T Z_p, Top -= W_p, Z_{p+1} = Top + S_{p+1}
    for (int p = 1; p < P; ++p) {
        g = base();
        g.A = tfull + (size_t)p * b * b; g.lda = b; g.a_kmajor = 1;
        g.B = S + p * slot; g.ldb = b; g.b_kmajor = 1;
        set_c_rows(g, top0);
        g.epi = tc::kTopUpdate;
        g.W = Wb + p * slot; g.ldw = b;
        g.Z = (p + 1 < P) ? S + (p + 1) * slot : nullptr; g.ldz = b;
        if ((rc = tc_gemm(g, 1, s)) != AVS_SUCCESS) return rc;
    }
    // 6. A_p -= Y_p W_p for p = 1..P-1
    if (P > 1) {
        g = base();
        set_y(g, top0 + b); g.strideA = tile_step;
        g.B = Wb + slot; g.ldb = b; g.b_kmajor = 1; g.strideB = slot;
        set_c_rows(g, top0 + b); g.strideC = tile_step;
        g.epi = tc::kSub;
        if ((rc = tc_gemm(g, P - 1, s)) != AVS_SUCCESS) return rc;
    }
    return AVS_SUCCESS;
}

// ---------------------------------------------------------------------------
// Self-test of the tensor-core GEMM against an FP64 SIMT product on the same
// device data (used by the GPU tests; allocates its own buffers).
namespace {
__global__ void fill_kernel(float *p, int64_t n, uint32_t seed) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        uint32_t h = (uint32_t)i * 2654435761u ^ seed;
        h ^= h >> 13;
        h *= 0x5bd1e995u;
        h ^= h >> 15;
        p[i] = ((float)(h & 0xFFFFFF) / 16777216.0f) * 2.0f - 1.0f;
    }
}
__global__ void ref_kernel(const float *A, int64_t lda, int akm, const float *B, int64_t ldb, int bkm, double *D,
                           int M, int N, int K) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x, n = blockIdx.y;
    if (m >= M) return;
    double acc = 0.0;
    for (int k = 0; k < K; ++k) {
        const double a = akm ? A[k + (int64_t)m * lda] : A[m + (int64_t)k * lda];
        const double b = bkm ? B[k + (int64_t)n * ldb] : B[n + (int64_t)k * ldb];
        acc += a * b;
    }
    D[m + (int64_t)n * M] = acc;
}
__global__ void cmp_kernel(const float *C, const double *D, int64_t n, float *out) {
    float mx = 0.f, ref = 0.f;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
        mx = fmaxf(mx, (float)fabs((double)C[i] - D[i]));
        ref = fmaxf(ref, (float)fabs(D[i]));
    }
    for (int o = 16; o > 0; o >>= 1) {
        mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        ref = fmaxf(ref, __shfl_xor_sync(0xffffffffu, ref, o));
    }
    __shared__ float sm[32], sr[32];
    if ((threadIdx.x & 31) == 0) { sm[threadIdx.x >> 5] = mx; sr[threadIdx.x >> 5] = ref; }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) { mx = fmaxf(mx, sm[w]); ref = fmaxf(ref, sr[w]); }
        out[0] = mx / fmaxf(ref, 1e-30f);
    }
}
}  // namespace

}  // namespace avs

extern "C" int avsx_tc_gemm_selftest(int M, int N, int K, int a_kmajor, int b_kmajor, int split, float *relerr) {
    using namespace avs;
    float *A = nullptr, *B = nullptr, *C = nullptr, *out = nullptr;
    double *D = nullptr;
    int *err = nullptr;
    int rc = AVS_SUCCESS;
    const int64_t lda = a_kmajor ? K : M, ldb = b_kmajor ? K : N;
    if (cudaMalloc(&A, sizeof(float) * (size_t)M * K) != cudaSuccess ||
        cudaMalloc(&B, sizeof(float) * (size_t)K * N) != cudaSuccess ||
        cudaMalloc(&C, sizeof(float) * (size_t)M * N) != cudaSuccess ||
        cudaMalloc(&D, sizeof(double) * (size_t)M * N) != cudaSuccess || cudaMalloc(&out, sizeof(float)) != cudaSuccess ||
        cudaMalloc(&err, sizeof(int)) != cudaSuccess) {
        rc = AVS_ERR_OOM;
    } else {
        cudaMemset(err, 0, sizeof(int));
        fill_kernel<<<256, 256>>>(A, (int64_t)M * K, 17u);
        fill_kernel<<<256, 256>>>(B, (int64_t)K * N, 91u);
        ref_kernel<<<dim3((M + 127) / 128, N), 128>>>(A, lda, a_kmajor, B, ldb, b_kmajor, D, M, N, K);
        tc::GemmArgs g = {};
        g.A = A; g.lda = lda; g.a_kmajor = a_kmajor; g.a_mask = tc::kNoMask;
        g.B = B; g.ldb = ldb; g.b_kmajor = b_kmajor;
        g.C = C; g.ldc = M; g.c_colmajor = 1;
        g.M = M; g.N = N; g.K = K; g.epi = tc::kStore; g.split = split; g.err = err;
        rc = tc_gemm(g, 1, 0);
        if (rc == AVS_SUCCESS) {
            cmp_kernel<<<1, 1024>>>(C, D, (int64_t)M * N, out);
            int herr = 0;
            if (cudaMemcpy(relerr, out, sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess ||
                cudaMemcpy(&herr, err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
                rc = AVS_ERR_CUDA;
            else if (herr == kDevTimeout)
                rc = AVS_ERR_TIMEOUT;
        }
    }
    cudaFree(A); cudaFree(B); cudaFree(C); cudaFree(D); cudaFree(out); cudaFree(err);
    return rc;
}
