// tcgen05 GEMM for the tensor-core trailing updates (TF32, split TF32, BF16,
// split BF16), fed by TMA.
//
// D[M x N] = A[M x K] * B[K x N] for a batch of problems p, FP32 accumulation
// in tensor memory.  Both operands are K-major in global memory (row m of A /
// row n of B holds K contiguous values) in one of four operand formats:
//   kTF32    fp32 planes holding rna_tf32(x) (1 product);
//   kTF32X3  two fp32 planes hi = rna_tf32(x), lo = rna_tf32(x - hi): the
//            products lo*hi + hi*lo + hi*hi give FP32-class accuracy;
//   kBF16    one bf16 plane (1 product);
//   kBF16X3  two bf16 planes hi = bf16(x), lo = bf16(x - hi) (3 products).
// The planes are produced by the kernels that write the operands (panel
// copies, transposes, the chain kernel), so the GEMM itself only moves bytes.
//
// One CTA (4 warps) computes a 128 x BN tile of D:
//   * warp 0, lane 0 issues cp.async.bulk.tensor loads of the K blocks (128
//     bytes of K per row, 128-byte swizzle -- the canonical K-major layout of
//     the tcgen05 shared-memory descriptors) into a ring of stages, each stage
//     completing on its "full" mbarrier by transaction count;
//   * warp 1, lane 0 issues tcgen05.mma (M = 128, N = BN, K = 8 for TF32 or
//     16 for BF16 per instruction) and commits each stage to its "empty"
//     mbarrier, which hands the stage back to the loader;
//   * after the last commit all four warps read the accumulator with
//     tcgen05.ld (warp w owns TMEM lanes 32w..32w+31 = rows of D) and either
//     store D or subtract it from the output (the trailing-matrix update).
// Every wait is bounded in time; a timeout sets the device status word and
// the CTA skips its stores.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <mutex>

#include "avs_common.cuh"
#include "tc_gemm.cuh"

namespace avs {
namespace tc {

namespace {

constexpr int BM = 128;
constexpr int NT = 128;
constexpr int kSmemStages = 200 * 1024;  // bytes of the stage ring

template <int BN, bool SPLIT, bool BF16>
struct KCfg {
    static constexpr int PLANES = SPLIT ? 2 : 1;
    static constexpr int A_BYTES = BM * 128;  // 128 rows x 128 B of K
    static constexpr int B_BYTES = BN * 128;
    static constexpr int STAGE = (A_BYTES + B_BYTES) * PLANES;
    static constexpr int STAGES = kSmemStages / STAGE > 6 ? 6 : kSmemStages / STAGE;
    static constexpr int SMEM = STAGE * STAGES + 1024;
    static constexpr int KSTEPS = 4;           // MMAs per 128-byte K block (32 B of K each)
    static constexpr int BK = BF16 ? 64 : 32;  // K elements per block
    static_assert(STAGES >= 2, "stage ring");
};

template <int BN, bool SPLIT, bool BF16>
__global__ void __launch_bounds__(NT, 1)
    gemm_kernel(const __grid_constant__ CUtensorMap ta_hi, const __grid_constant__ CUtensorMap ta_lo,
                const __grid_constant__ CUtensorMap tb_hi, const __grid_constant__ CUtensorMap tb_lo, GemmDesc g) {
    using C = KCfg<BN, SPLIT, BF16>;
    extern __shared__ uint8_t smem_dyn[];
    __shared__ uint64_t full[C::STAGES], empty[C::STAGES], done;
    __shared__ uint32_t tmem_base;
    __shared__ int s_fail;
    uint8_t *base = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_dyn) + 1023) & ~(uintptr_t)1023);
    const int tid = threadIdx.x, wid = tid >> 5, lane = tid & 31;
    const int p = (int)blockIdx.z + g.p0;
    const int m0 = (int)blockIdx.y * BM, n0 = (int)blockIdx.x * BN;

    if (tid == 0) {
        for (int s = 0; s < C::STAGES; ++s) {
            mbar_init(smem_u32(&full[s]), 1);
            mbar_init(smem_u32(&empty[s]), 1);
        }
        mbar_init(smem_u32(&done), 1);
        s_fail = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&ta_hi)) : "memory");
        asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tb_hi)) : "memory");
    }
    if (wid == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                     "r"(BN));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_base;
    // stage s: A hi | B hi | A lo | B lo
    auto stage_ptr = [&](int s, int which) -> uint32_t {
        const uint32_t st = smem_u32(base) + (uint32_t)(s * C::STAGE);
        switch (which) {
            case 0: return st;
            case 1: return st + C::A_BYTES;
            case 2: return st + C::A_BYTES + C::B_BYTES;
            default: return st + 2 * C::A_BYTES + C::B_BYTES;
        }
    };

    if (wid == 0 && lane == 0) {
        // ---- loader
        for (int kb = 0; kb < g.nkb; ++kb) {
            const int s = kb % C::STAGES;
            if (kb >= C::STAGES && !mbar_wait(smem_u32(&empty[s]), (uint32_t)((kb / C::STAGES - 1) & 1), g.err)) {
                s_fail = 1;
                break;
            }
            const uint32_t fb = smem_u32(&full[s]);
            mbar_expect_tx(fb, (uint32_t)C::STAGE);
            const int ax = kb * C::BK, ay = g.a_y0 + p * g.a_yp + m0;
            const int bx = g.b_x0 + p * g.b_xp + kb * C::BK, by = g.b_y0 + p * g.b_yp + n0;
            tma_load_2d(stage_ptr(s, 0), &ta_hi, ax, ay, fb);
            tma_load_2d(stage_ptr(s, 1), &tb_hi, bx, by, fb);
            if constexpr (SPLIT) {
                tma_load_2d(stage_ptr(s, 2), &ta_lo, ax, ay, fb);
                tma_load_2d(stage_ptr(s, 3), &tb_lo, bx, by, fb);
            }
        }
    } else if (wid == 1 && lane == 0) {
        // ---- MMA issue
        const uint32_t id = idesc(BM, BN, BF16);
        for (int kb = 0; kb < g.nkb; ++kb) {
            const int s = kb % C::STAGES;
            if (!mbar_wait(smem_u32(&full[s]), (uint32_t)((kb / C::STAGES) & 1), g.err)) {
                s_fail = 1;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t ah = stage_ptr(s, 0), bh = stage_ptr(s, 1);
#pragma unroll
            for (int ks = 0; ks < C::KSTEPS; ++ks) {
                const uint32_t ko = ks * 32;
                const uint64_t da = desc_sw128(ah + ko), db = desc_sw128(bh + ko);
                if constexpr (SPLIT) {
                    const uint32_t al = stage_ptr(s, 2), bl = stage_ptr(s, 3);
                    mma<BF16>(tmem, desc_sw128(al + ko), db, id, (kb > 0 || ks > 0) ? 1u : 0u);
                    mma<BF16>(tmem, da, desc_sw128(bl + ko), id, 1u);
                    mma<BF16>(tmem, da, db, id, 1u);
                } else {
                    mma<BF16>(tmem, da, db, id, (kb > 0 || ks > 0) ? 1u : 0u);
                }
            }
            mma_commit(smem_u32(&empty[s]));
        }
        mma_commit(smem_u32(&done));
    }
    __syncwarp();
    const bool ok = mbar_wait(smem_u32(&done), 0u, g.err) && !*(volatile int *)&s_fail;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");

    // ---- epilogue: warp w owns rows m0 + 32w + lane
    const int64_t row = g.o_row0 + (int64_t)p * g.o_rowp + m0 + 32 * wid + lane;
    const int64_t col0 = g.o_col0 + (int64_t)p * g.o_colp + n0;
    for (int c16 = 0; c16 < BN / 16; ++c16) {
        float v[16];
        tmem_ld16(tmem + ((uint32_t)(32 * wid) << 16) + (uint32_t)(c16 * 16), v);
        if (!ok) continue;
        float *o = g.out + row + (col0 + c16 * 16) * g.ld_out;
        if (g.epi == kEpiStore) {
#pragma unroll
            for (int q = 0; q < 16; ++q) o[q * g.ld_out] = v[q];
        } else {
            float cur[16];
#pragma unroll
            for (int q = 0; q < 16; ++q) cur[q] = o[q * g.ld_out];
#pragma unroll
            for (int q = 0; q < 16; ++q) o[q * g.ld_out] = cur[q] - v[q];
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (wid == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(BN));
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// dependency on libcuda).
using EncodeFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                              const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                              CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeFn encode_fn() {
    static EncodeFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeFn>(p);
        else
            cudaGetLastError();
    });
    return fn;
}

template <int BN, bool SPLIT, bool BF16>
int launch(const Operand &A, const Operand &B, const GemmDesc &g, int mtiles, int ntiles, int batch, cudaStream_t s) {
    using C = KCfg<BN, SPLIT, BF16>;
    static std::atomic<bool> attr{false};
    if (!attr) {
        AVS_CUDA_TRY(cudaFuncSetAttribute(gemm_kernel<BN, SPLIT, BF16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          C::SMEM));
        attr = true;
    }
    if (!encode_fn()) return AVS_ERR_UNSUPPORTED;
    CUtensorMap m[4];
    if (!make_tmap(&m[0], A, A.hi, BM, BF16) || !make_tmap(&m[1], A, A.lo, BM, BF16) ||
        !make_tmap(&m[2], B, B.hi, BN, BF16) || !make_tmap(&m[3], B, B.lo, BN, BF16))
        return AVS_ERR_INTERNAL;
    gemm_kernel<BN, SPLIT, BF16><<<dim3((unsigned)ntiles, (unsigned)mtiles, (unsigned)batch), NT, C::SMEM, s>>>(
        m[0], m[1], m[2], m[3], g);
    AVS_CUDA_TRY(cudaGetLastError());
    return AVS_SUCCESS;
}

}  // namespace

// 2-D tensor map of a K-major operand plane: box of 128 bytes of K x box_rows
// rows, 128-byte swizzle.  A null plane (unused lo) maps the hi plane.
bool make_tmap(CUtensorMap *map, const Operand &op, const void *ptr, int box_rows, bool bf16) {
    EncodeFn enc = encode_fn();
    if (!enc) return false;
    if (!ptr) ptr = op.hi;
    const int esz = bf16 ? 2 : 4;
    const cuuint64_t dims[2] = {(cuuint64_t)op.k_extent, (cuuint64_t)op.rows};
    const cuuint64_t strides[1] = {(cuuint64_t)op.ld * esz};
    const cuuint32_t box[2] = {(cuuint32_t)(128 / esz), (cuuint32_t)box_rows};
    const cuuint32_t es[2] = {1, 1};
    return enc(map, bf16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2,
               const_cast<void *>(ptr), dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
               CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

int gemm(int fmt, const Operand &A, const Operand &B, const GemmDesc &g, int M, int N, int batch, cudaStream_t s) {
    if (M % BM || batch <= 0 || N % 128) return AVS_ERR_INTERNAL;
    const bool wide = (N % 256 == 0);
    switch (fmt) {
        case kTF32:
            return wide ? launch<256, false, false>(A, B, g, M / BM, N / 256, batch, s)
                        : launch<128, false, false>(A, B, g, M / BM, N / 128, batch, s);
        case kTF32X3: return launch<128, true, false>(A, B, g, M / BM, N / 128, batch, s);
        case kBF16:
            return wide ? launch<256, false, true>(A, B, g, M / BM, N / 256, batch, s)
                        : launch<128, false, true>(A, B, g, M / BM, N / 128, batch, s);
        case kBF16X3: return launch<128, true, true>(A, B, g, M / BM, N / 128, batch, s);
        default: return AVS_ERR_UNSUPPORTED;
    }
}

}  // namespace tc

// ---------------------------------------------------------------------------
// Self-test of the tensor-core GEMM against an FP64 product of the same data
// (used by the GPU tests; allocates its own buffers).  A is M x K, B is N x K
// (both K-major), C = A B^T is stored column-major (ld M).
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
__global__ void planes_kernel(const float *x, int64_t n, int fmt, void *hi, void *lo) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        tc::put_operand(fmt, hi, lo, i, x[i]);
}
__global__ void ref_kernel(const float *A, const float *B, double *D, int M, int N, int K) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x, n = blockIdx.y;
    if (m >= M) return;
    double acc = 0.0;
    for (int k = 0; k < K; ++k) acc += (double)A[k + (int64_t)m * K] * (double)B[k + (int64_t)n * K];
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

extern "C" int avsx_tc_gemm_selftest(int M, int N, int K, int fmt, float *relerr) {
    using namespace avs;
    if (M <= 0 || N <= 0 || K <= 0 || M % 128 || N % 128 || K % 64) return AVS_ERR_INTERNAL;
    if (fmt != tc::kTF32 && fmt != tc::kTF32X3 && fmt != tc::kBF16 && fmt != tc::kBF16X3) return AVS_ERR_UNSUPPORTED;
    float *A = nullptr, *B = nullptr, *C = nullptr, *out = nullptr;
    void *ah = nullptr, *al = nullptr, *bh = nullptr, *bl = nullptr;
    double *D = nullptr;
    int *err = nullptr;
    int rc = AVS_SUCCESS;
    const size_t esz = (fmt == tc::kBF16 || fmt == tc::kBF16X3) ? 2 : 4;
    if (cudaMalloc(&A, sizeof(float) * (size_t)M * K) != cudaSuccess ||
        cudaMalloc(&B, sizeof(float) * (size_t)K * N) != cudaSuccess ||
        cudaMalloc(&C, sizeof(float) * (size_t)M * N) != cudaSuccess ||
        cudaMalloc(&D, sizeof(double) * (size_t)M * N) != cudaSuccess || cudaMalloc(&out, sizeof(float)) != cudaSuccess ||
        cudaMalloc(&err, sizeof(int)) != cudaSuccess || cudaMalloc(&ah, esz * (size_t)M * K) != cudaSuccess ||
        cudaMalloc(&al, esz * (size_t)M * K) != cudaSuccess || cudaMalloc(&bh, esz * (size_t)N * K) != cudaSuccess ||
        cudaMalloc(&bl, esz * (size_t)N * K) != cudaSuccess) {
        cudaGetLastError();
        rc = AVS_ERR_OOM;
    } else {
        cudaMemset(err, 0, sizeof(int));
        fill_kernel<<<256, 256>>>(A, (int64_t)M * K, 17u);
        fill_kernel<<<256, 256>>>(B, (int64_t)K * N, 91u);
        planes_kernel<<<256, 256>>>(A, (int64_t)M * K, fmt, ah, al);
        planes_kernel<<<256, 256>>>(B, (int64_t)N * K, fmt, bh, bl);
        ref_kernel<<<dim3((M + 127) / 128, N), 128>>>(A, B, D, M, N, K);
        tc::Operand oa{ah, al, (int64_t)K, (int64_t)M, (int64_t)K};
        tc::Operand ob{bh, bl, (int64_t)K, (int64_t)N, (int64_t)K};
        tc::GemmDesc g = {};
        g.nkb = (int)((size_t)K * esz / 128);
        g.epi = tc::kEpiStore;
        g.out = C;
        g.ld_out = M;
        g.err = err;
        rc = tc::gemm(fmt, oa, ob, g, M, N, 1, 0);
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
    cudaFree(ah); cudaFree(al); cudaFree(bh); cudaFree(bl);
    return rc;
}
