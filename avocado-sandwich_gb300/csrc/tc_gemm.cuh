// Interface of the tcgen05 GEMM (tc_gemm.cu) and the operand formats shared
// with the kernels that produce its operands.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace avs {
namespace tc {

// Operand formats (values of Stage1Work::tc_split).
enum Fmt : int { kNone = 0, kTF32 = 1, kTF32X3 = 3, kBF16 = 4, kBF16X3 = 5 };

__host__ __device__ constexpr bool fmt_bf16(int fmt) { return fmt == kBF16 || fmt == kBF16X3; }
__host__ __device__ constexpr bool fmt_split(int fmt) { return fmt == kTF32X3 || fmt == kBF16X3; }
__host__ __device__ constexpr int fmt_bytes(int fmt) { return fmt_bf16(fmt) ? 2 : 4; }

// A K-major operand: `rows` rows of `k_extent` elements, row stride `ld`
// elements, in one plane (hi) or two (hi, lo).
struct Operand {
    void *hi;
    void *lo;
    int64_t ld;
    int64_t rows;
    int64_t k_extent;
};

enum Epi : int { kEpiStore = 0, kEpiSub = 1 };

// Problem p = blockIdx.z + p0.  A tile rows: y = a_y0 + p*a_yp + m0, K blocks
// at x = kb*BK.  B tile rows: y = b_y0 + p*b_yp + n0, K at x = b_x0 + p*b_xp +
// kb*BK.  Output element (m, c) at out[(o_row0 + p*o_rowp + m) +
// (o_col0 + p*o_colp + c) * ld_out]; kEpiStore writes D, kEpiSub subtracts it.
struct GemmDesc {
    int p0;
    int a_y0, a_yp;
    int b_x0, b_xp, b_y0, b_yp;
    int nkb;
    int epi;
    float *out;
    int64_t ld_out;
    int64_t o_row0, o_rowp, o_col0, o_colp;
    int *err;
};

// D = A B^T for `batch` problems: M rows of A (multiple of 128), N rows of B
// (multiple of 128).
int gemm(int fmt, const Operand &A, const Operand &B, const GemmDesc &g, int M, int N, int batch, cudaStream_t s);

}  // namespace tc
}  // namespace avs

struct CUtensorMap_st;
namespace avs {
namespace tc {
// Tensor map (TMA descriptor) of a K-major operand plane: boxes of 128 bytes of
// K x box_rows rows, 128-byte swizzle; ptr == nullptr maps op.hi.
bool make_tmap(CUtensorMap_st *map, const Operand &op, const void *ptr, int box_rows, bool bf16);

// Store x into operand plane(s) at element i in format fmt.
__device__ __forceinline__ uint32_t rna_tf32(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return r;
}

__device__ __forceinline__ void put_operand(int fmt, void *hi, void *lo, int64_t i, float x) {
    if (fmt == kTF32) {
        static_cast<uint32_t *>(hi)[i] = rna_tf32(x);  // rounded, not the tensor core's truncation
    } else if (fmt == kTF32X3) {
        const uint32_t h = rna_tf32(x);
        static_cast<uint32_t *>(hi)[i] = h;
        static_cast<uint32_t *>(lo)[i] = rna_tf32(x - __uint_as_float(h));
    } else {
        const __nv_bfloat16 h = __float2bfloat16_rn(x);
        static_cast<__nv_bfloat16 *>(hi)[i] = h;
        if (fmt == kBF16X3) static_cast<__nv_bfloat16 *>(lo)[i] = __float2bfloat16_rn(x - __bfloat162float(h));
    }
}

}  // namespace tc
}  // namespace avs

// ---------------------------------------------------------------------------
// tcgen05 / TMA / mbarrier building blocks shared by the tensor-core kernels.
#include <cuda.h>

#include "avs_common.cuh"

namespace avs {
namespace tc {

constexpr long long kWaitNs = 2000000000ll;  // bound of every mbarrier wait: 2 s

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ unsigned long long gtimer() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row atoms
// 1024 B apart (stride byte offset), leading byte offset unused for this
// layout (1), descriptor version 1 (bits 46-47), swizzle mode 2 (bits 61-63).
__device__ __forceinline__ uint64_t desc_sw128(uint32_t addr) {
    uint64_t d = 0;
    d |= (uint64_t)((addr >> 4) & 0x3FFFu);
    d |= (uint64_t)1u << 16;
    d |= (uint64_t)(1024u >> 4) << 32;
    d |= (uint64_t)1u << 46;
    d |= (uint64_t)2u << 61;
    return d;
}

// Instruction descriptors: D FP32 (bits 4-5 = 1), A/B format (bits 7-9,
// 10-12: TF32 = 2 for kind::tf32, BF16 = 1 for kind::f16), both operands
// K-major, N >> 3 at bit 17, M >> 4 at bit 24.
__host__ __device__ constexpr uint32_t idesc(int M, int N, bool bf16) {
    return (1u << 4) | ((bf16 ? 1u : 2u) << 7) | ((bf16 ? 1u : 2u) << 10) | ((uint32_t)(N >> 3) << 17) |
           ((uint32_t)(M >> 4) << 24);
}

template <bool BF16>
__device__ __forceinline__ void mma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t id, uint32_t acc) {
    if constexpr (BF16) {
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "setp.ne.b32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n"
            :
            : "r"(d_tmem), "l"(a), "l"(b), "r"(id), "r"(acc));
    } else {
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "setp.ne.b32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n"
            :
            : "r"(d_tmem), "l"(a), "l"(b), "r"(id), "r"(acc));
    }
}

__device__ __forceinline__ void mma_commit(uint32_t mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
                 : "memory");
}

__device__ __forceinline__ void mbar_init(uint32_t mbar, int count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t mbar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(bytes) : "memory");
}

// Bounded wait for the completion of phase `parity` of an mbarrier (2 s).
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity, int *err) {
    const unsigned long long t0 = gtimer();
    for (long long it = 0;; ++it) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.b32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(mbar), "r"(parity)
            : "memory");
        if (done) return true;
        if ((it & 255) == 255) {
            if (ld_acquire(err) != kDevOk) return false;
            if ((long long)(gtimer() - t0) > kWaitNs) {
                atomicCAS(err, kDevOk, kDevTimeout);
                return false;
            }
        }
    }
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, int x, int y, uint32_t mbar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
        "[%4];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(mbar)
        : "memory");
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


// Byte offset of element (row r, k) in a K-major 128-byte-swizzled tile of
// 4-byte elements (K block of 32): 8-row atoms of 1024 B, the 16-byte chunk c
// of row r stored at chunk c ^ (r & 7).
__device__ __forceinline__ uint32_t swz4(int r, int k) {
    return (uint32_t)((r >> 3) * 1024 + (r & 7) * 128 + ((((k >> 2) ^ (r & 7)) << 4) | ((k & 3) << 2)));
}
// The same for 2-byte elements (K block of 64).
__device__ __forceinline__ uint32_t swz2(int r, int k) {
    return (uint32_t)((r >> 3) * 1024 + (r & 7) * 128 + ((((k >> 3) ^ (r & 7)) << 4) | ((k & 7) << 1)));
}

}  // namespace tc
}  // namespace avs
