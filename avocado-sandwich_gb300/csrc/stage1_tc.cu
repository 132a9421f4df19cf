// Stage 1 with tensor-core trailing updates (FP32 tiles, tiles 128 and 256).
//
// Every half-step runs as a QR half-step on a column-major matrix: the LQ
// half-step k (row panel k, LQ of tiles (k, k+1..), TiledMatrix.jl:98-113) is
// the QR half-step of the transposed matrix, so the trailing block is
// transposed into a second buffer before it and back after it.  Then both
// products of the trailing update read the large operand along contiguous
// memory (K-major), which is what the TMA-fed tcgen05 GEMM wants:
//
//   S_p  = Y_p^T A_p          p = 0..P-1   (tensor cores, one batched launch)
//   W_p  = T_p^T (Top + S_p), Top -= ...   (chain kernel, SIMT, sequential in p)
//   A_p -= Y_p W_p            p = 1..P-1   (tensor cores, one batched launch)
//
// Operand planes (rounded TF32, TF32 hi/lo, BF16, BF16 hi/lo) of the trailing
// block come out of the transposes; those of Y out of a copy kernel; those of
// W out of the chain.
#include <algorithm>

#include "avs_common.cuh"
#include "tc_gemm.cuh"

namespace avs {
namespace {

inline size_t al256(size_t x) { return (x + 255) & ~size_t(255); }

// Y copies: ycol [p][l][t] (t fastest) and yrow [p][t][l] (l fastest) of the
// panel tiles X(r0 + p*b + t, c0 + l); tile 0 (GEQRT) keeps its unit lower
// triangle only.
__global__ void ycopy_kernel(const float *X, int64_t ldx, int64_t r0, int64_t c0, int b, int fmt, void *ych,
                             void *ycl, void *yrh, void *yrl) {
    __shared__ float tile[32][33];
    const int p = blockIdx.z;
    const int t0 = blockIdx.x * 32, l0 = blockIdx.y * 32;
    const int tx = threadIdx.x, ty = threadIdx.y;
    for (int k = ty; k < 32; k += 8) {
        const int t = t0 + tx, l = l0 + k;
        float v = X[(r0 + (int64_t)p * b + t) + (c0 + l) * ldx];
        if (p == 0) v = (t == l) ? 1.0f : (t > l ? v : 0.0f);
        tc::put_operand(fmt, ych, ycl, ((int64_t)p * b + l) * b + t, v);
        tile[k][tx] = v;
    }
    __syncthreads();
    for (int k = ty; k < 32; k += 8) {
        const int t = t0 + k, l = l0 + tx;
        tc::put_operand(fmt, yrh, yrl, ((int64_t)p * b + t) * b + l, tile[tx][k]);
    }
}

// dst[j + i*ld] = src[i + j*ld] for i in [i0, n), j in [j0, n); the operand
// planes of dst (same indexing) are written too when fmt needs them.
__global__ void transpose_kernel(const float *src, float *dst, int64_t ld, int64_t i0, int64_t j0, int fmt,
                                 void *ph, void *pl) {
    __shared__ float tile[32][33];
    const int64_t ib = i0 + (int64_t)blockIdx.x * 32, jb = j0 + (int64_t)blockIdx.y * 32;
    const int tx = threadIdx.x, ty = threadIdx.y;
    for (int k = ty; k < 32; k += 8) tile[k][tx] = src[(ib + tx) + (jb + k) * ld];
    __syncthreads();
    for (int k = ty; k < 32; k += 8) {
        const float v = tile[tx][k];
        const int64_t o = (jb + tx) + (ib + k) * ld;
        dst[o] = v;
        if (ph) tc::put_operand(fmt, ph, pl, o, v);
    }
}

__global__ void planes_kernel(const float *x, int64_t count, int fmt, void *ph, void *pl) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x)
        tc::put_operand(fmt, ph, pl, i, x[i]);
}

// planes of the block rows r0.., columns j0.. of x (same indexing)
__global__ void planes_block_kernel(const float *x, int64_t n, int64_t r0, int64_t j0, int fmt, void *ph, void *pl) {
    const int64_t rows = n - r0;
    for (int64_t c = j0 + blockIdx.y; c < n; c += gridDim.y)
        for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < rows; r += (int64_t)gridDim.x * blockDim.x)
            tc::put_operand(fmt, ph, pl, (r0 + r) + c * n, x[(r0 + r) + c * n]);
}

}  // namespace

int stage1_tc_planes_block(const float *x, int64_t n, int64_t r0, int64_t j0, int fmt, const TcBufs &tb,
                           cudaStream_t s) {
    if (r0 >= n || j0 >= n) return AVS_SUCCESS;
    const unsigned gy = (unsigned)std::min<int64_t>(n - j0, 4096);
    planes_block_kernel<<<dim3((unsigned)std::min<int64_t>((n - r0 + 255) / 256, 64), gy), 256, 0, s>>>(
        x, n, r0, j0, fmt, tb.ph, tb.pl);
    AVS_CUDA_TRY(cudaGetLastError());
    return AVS_SUCCESS;
}

TcBufs stage1_tc_carve(void *ws, int64_t n, int b, int fmt) {
    TcBufs t{};
    char *p = static_cast<char *>(ws);
    const int64_t nt = n / b;
    const size_t e = (size_t)tc::fmt_bytes(fmt);
    const bool two = tc::fmt_split(fmt);
    size_t o = 0;
    auto take = [&](size_t bytes) -> void * {
        if (bytes == 0) return nullptr;
        void *q = p ? p + o : nullptr;
        o = al256(o + bytes);
        return q;
    };
    t.xt = static_cast<float *>(take(sizeof(float) * (size_t)n * n));
    t.ph = take(e * (size_t)n * n);
    t.pl = take(two ? e * (size_t)n * n : 0);
    t.ych = take(e * (size_t)nt * b * b);
    t.ycl = take(two ? e * (size_t)nt * b * b : 0);
    t.yrh = take(e * (size_t)nt * b * b);
    t.yrl = take(two ? e * (size_t)nt * b * b : 0);
    t.S = static_cast<float *>(take(sizeof(float) * (size_t)nt * b * n));
    t.wh = take(e * (size_t)nt * b * n);
    t.wl = take(two ? e * (size_t)nt * b * n : 0);
    t.th = take(e * (size_t)nt * b * b);
    t.tl = take(two ? e * (size_t)nt * b * b : 0);
    t.ready = static_cast<int *>(take(sizeof(int) * (size_t)(nt + 1)));
    t.bytes = o;
    return t;
}

size_t stage1_tc_bytes(int64_t n, int b, int fmt) { return stage1_tc_carve(nullptr, n, b, fmt).bytes; }

int stage1_tc_planes(const float *x, int64_t n, int fmt, const TcBufs &tb, cudaStream_t s) {
    planes_kernel<<<1024, 256, 0, s>>>(x, n * n, fmt, tb.ph, tb.pl);
    AVS_CUDA_TRY(cudaGetLastError());
    return AVS_SUCCESS;
}

int stage1_tc_transpose(const float *src, float *dst, int64_t n, int64_t i0, int64_t j0, int fmt, const TcBufs &tb,
                        cudaStream_t s) {
    if (i0 >= n || j0 >= n) return AVS_SUCCESS;
    const dim3 grid((unsigned)((n - i0) / 32), (unsigned)((n - j0) / 32));
    transpose_kernel<<<grid, dim3(32, 8), 0, s>>>(src, dst, n, i0, j0, fmt, tb.ph, tb.pl);
    AVS_CUDA_TRY(cudaGetLastError());
    return AVS_SUCCESS;
}

int stage1_tc_transpose_box(const float *src, float *dst, int64_t n, int64_t i0, int64_t ni, int64_t j0, int64_t nj,
                            int fmt, const TcBufs &tb, cudaStream_t s) {
    if (ni <= 0 || nj <= 0) return AVS_SUCCESS;
    if (ni % 32 || nj % 32 || i0 + ni > n || j0 + nj > n) return AVS_ERR_INTERNAL;
    transpose_kernel<<<dim3((unsigned)(ni / 32), (unsigned)(nj / 32)), dim3(32, 8), 0, s>>>(src, dst, n, i0, j0, fmt,
                                                                                          tb.ph, tb.pl);
    AVS_CUDA_TRY(cudaGetLastError());
    return AVS_SUCCESS;
}

// Trailing update of the QR half-step with panel (pr, pc) and P tiles on the
// column-major n x n matrix x (ld n), after the panel and the T build.  parts
// selects the steps (a caller that overlaps other work with the update runs
// them separately): kTcS = Y copies and S_p = Y_p^T A_p (needs the panel
// only), kTcPlanes = the T factors' operand planes (needs the T build; zeroes
// the ready counters when given), kTcChain = the chain (writes the top tile
// row, and its transpose into xt_out when given, counting finished strips per
// tile in ready), kTcUpdate = A_p -= Y_p W_p.
int stage1_tc_update(float *x, int64_t n, int b, int pr, int pc, int P, const Stage1Work &w, const TcBufs &tb,
                     cudaStream_t s, int64_t *launches, int parts, float *xt_out, int *ready) {
    const int fmt = w.tc_split;
    const int64_t r0 = (int64_t)pr * b, c0 = (int64_t)pc * b, j0 = (int64_t)(pc + 1) * b;
    const int64_t ntr = n - j0;
    if (ntr <= 0) return AVS_SUCCESS;
    int rc;
    const int nkb = b * tc::fmt_bytes(fmt) / 128;
    if (parts & kTcS) {
        ycopy_kernel<<<dim3(b / 32, b / 32, P), dim3(32, 8), 0, s>>>(x, n, r0, c0, b, fmt, tb.ych, tb.ycl, tb.yrh,
                                                                    tb.yrl);
        AVS_CUDA_TRY(cudaGetLastError());
        // S_p = Y_p^T A_p, p = 0..P-1 (A_0 = the top tile row)
        {
            tc::Operand A{tb.ych, tb.ycl, b, (int64_t)P * b, b};
            tc::Operand B{tb.ph, tb.pl, n, n, n};
            tc::GemmDesc g{};
            g.p0 = 0;
            g.a_y0 = 0;
            g.a_yp = b;
            g.b_x0 = (int)r0;
            g.b_xp = b;
            g.b_y0 = (int)j0;
            g.b_yp = 0;
            g.nkb = nkb;
            g.epi = tc::kEpiStore;
            g.out = tb.S;
            g.ld_out = b;
            g.o_row0 = 0;
            g.o_rowp = 0;
            g.o_col0 = 0;
            g.o_colp = ntr;
            g.err = w.err;
            if ((rc = tc::gemm(fmt, A, B, g, b, (int)ntr, P, s)) != AVS_SUCCESS) return rc;
        }
        if (launches) *launches += 2;
    }
    if (parts & kTcPlanes) {
        if (ready) AVS_CUDA_TRY(cudaMemsetAsync(ready, 0, sizeof(int) * (size_t)(n / b + 1), s));
        if ((rc = stage1_chain_tplanes(static_cast<const float *>(w.tfull), b, P, fmt, tb.th, tb.tl, s)) !=
            AVS_SUCCESS)
            return rc;
        if (launches) *launches += 1;
    }
    // chain along the tiles (top tile row, W_p)
    if (parts & kTcChain) {
        if ((rc = stage1_chain_tc2(x, n, b, pr, pc, P, tb.th, tb.tl, tb.yrh, tb.yrl, tb.S, ntr, tb.wh, tb.wl, fmt,
                                   w.err, s, xt_out, ready)) != AVS_SUCCESS)
            return rc;
        if (launches) *launches += 1;
    }
    // A_p -= Y_p W_p, p = 1..P-1
    if ((parts & kTcUpdate) && P > 1) {
        tc::Operand A{tb.yrh, tb.yrl, b, (int64_t)P * b, b};
        tc::Operand B{tb.wh, tb.wl, b, (int64_t)P * ntr, b};
        tc::GemmDesc g{};
        g.p0 = 1;
        g.a_y0 = 0;
        g.a_yp = b;
        g.b_x0 = 0;
        g.b_xp = 0;
        g.b_y0 = 0;
        g.b_yp = (int)ntr;
        g.nkb = nkb;
        g.epi = tc::kEpiSub;
        g.out = x;
        g.ld_out = n;
        g.o_row0 = r0;
        g.o_rowp = b;
        g.o_col0 = j0;
        g.o_colp = 0;
        g.err = w.err;
        if ((rc = tc::gemm(fmt, A, B, g, b, (int)ntr, P - 1, s)) != AVS_SUCCESS) return rc;
        if (launches) *launches += 1;
    }
    return AVS_SUCCESS;
}

}  // namespace avs
