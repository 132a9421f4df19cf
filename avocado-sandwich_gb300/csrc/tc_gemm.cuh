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
