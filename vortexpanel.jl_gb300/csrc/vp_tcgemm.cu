// FP32-class GEMM on the fifth-generation tensor cores for the trailing updates of the mixed-precision bordered LU
// (the reference factors with LAPACK's dgetrf, src/assembly/solve.jl:54,84): C -= A B with A (m x k), B (k x n) and C
// FP32, column-major.
//
// Each FP32 operand is split into three bf16 pieces, x = x1 + x2 + x3, each piece the bf16 rounding of what the
// previous ones leave (3 x 8 significant bits cover FP32's 24). The six products whose orders reach FP32's precision,
// A1B1 + A1B2 + A2B1 + A1B3 + A2B2 + A3B1, are accumulated in FP32 in tensor memory (the dropped A2B3, A3B2, A3B3 lie
// below 2^-24 |A||B|), so the factors keep FP32 accuracy and the FP64 refinement converges as with FP32 factors. A1B1
// and the five smaller products go to two accumulators, added in the epilogue, so that the small terms are not
// rounded against the large sum at every step.
//
// Layout: a split kernel writes the pieces K-major (A3[p][row][k], B3[p][col][k], bf16, k padded to 64, rows to
// 128). One CTA per 128 x 128 tile of C, 128 threads:
//   - thread 0 stages 64-wide k-slices of the six operand tiles with TMA (cp.async.bulk.tensor, 128-byte swizzle, this
//     GPU's own memory, no multicast) into two shared-memory stages of 96 KB, paced by mbarriers;
//   - thread 32 issues tcgen05.mma (kind::f16, bf16 operands, M 128, N 128, K 16) into two 128-column FP32
//     accumulators in TMEM, 24 per k-slice, and frees each stage with tcgen05.commit;
//   - the four warps read the accumulators back with tcgen05.ld (warp w holds rows 32w..32w+31) and subtract their
//     sum from C (coalesced along C's columns).
// Every mbarrier wait has an iteration limit: a wait that gives up sets the error word, the CTA skips the rest of its
// work and still frees its TMEM; the host reports VP_ERR_TIMEOUT.
#include <cuda.h>
#include <cuda_bf16.h>

#include <cstdint>
#include <cstdlib>

#include "vp_internal.h"

namespace {

constexpr int TC_BM = 128, TC_BN = 128, TC_BK = 64;
constexpr int TC_PIECES = 3, TC_STAGES = 2, TC_THREADS = 128;
constexpr int TC_TILE_BYTES = TC_BM * TC_BK * 2;                       // 16 KB: one 128 x 64 bf16 tile
constexpr int TC_STAGE_BYTES = 2 * TC_PIECES * TC_TILE_BYTES;          // 96 KB: three A and three B tiles
constexpr int TC_SMEM = TC_STAGES * TC_STAGE_BYTES + 1024;             // + alignment to 1024 bytes
constexpr int TC_TMEM_COLS = 256;  // two FP32 accumulators of 128 lanes x 128 columns: A1B1, and the five small products
constexpr long long TC_WAIT_LIMIT = 1LL << 22;                         // iterations of a bounded mbarrier wait

// the six products (A piece, B piece) of the three-piece split that reach FP32's precision
__constant__ int c_prod_a[6] = {0, 0, 1, 0, 1, 2};
__constant__ int c_prod_b[6] = {0, 1, 0, 2, 1, 0};

__device__ __forceinline__ void split3(float x, __nv_bfloat16& a, __nv_bfloat16& b, __nv_bfloat16& c) {
    a = __float2bfloat16_rn(x);
    const float r1 = x - __bfloat162float(a);  // exact: a is x rounded to 8 significant bits
    b = __float2bfloat16_rn(r1);
    const float r2 = r1 - __bfloat162float(b);
    c = __float2bfloat16_rn(r2);
}

// A (m x k, column-major, lda) -> three K-major pieces dst[p][row][kk] (rows_pad x k_pad each), through a 32 x 32
// shared-memory transpose so that both the reads (along rows) and the writes (along k) are coalesced; zero padding
__global__ void split_a_kernel(int m, int k, const float* __restrict__ A, int lda, int rows_pad, int k_pad,
                               __nv_bfloat16* __restrict__ dst) {
    __shared__ float t[32][33];
    const int r0 = blockIdx.x * 32, c0 = blockIdx.y * 32;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8
    for (int yy = ty; yy < 32; yy += 8) {
        const int r = r0 + tx, c = c0 + yy;
        t[yy][tx] = (r < m && c < k) ? A[size_t(c) * lda + r] : 0.f;
    }
    __syncthreads();
    const size_t plane = size_t(rows_pad) * k_pad;
    for (int yy = ty; yy < 32; yy += 8) {
        const int r = r0 + yy, c = c0 + tx;
        __nv_bfloat16 a, b, cc;
        split3(t[tx][yy], a, b, cc);
        const size_t o = size_t(r) * k_pad + c;
        dst[o] = a;
        dst[plane + o] = b;
        dst[2 * plane + o] = cc;
    }
}

// B (k x n, column-major, ldb: k contiguous) -> three K-major pieces dst[p][col][kk] (cols_pad x k_pad each)
__global__ void split_b_kernel(int k, int n, const float* __restrict__ B, int ldb, int cols_pad, int k_pad,
                               __nv_bfloat16* __restrict__ dst) {
    const size_t plane = size_t(cols_pad) * k_pad;
    const size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= plane) return;
    const int j = int(i / k_pad), kk = int(i % k_pad);
    const float x = (j < n && kk < k) ? B[size_t(j) * ldb + kk] : 0.f;
    __nv_bfloat16 a, b, c;
    split3(x, a, b, c);
    dst[i] = a;
    dst[plane + i] = b;
    dst[2 * plane + i] = c;
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return uint32_t(__cvta_generic_to_shared(p)); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

// wait for the phase of the given parity to complete, at most TC_WAIT_LIMIT tries; false (and the error word set)
// when it gives up
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, int* err) {
    for (long long i = 0; i < TC_WAIT_LIMIT; ++i) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
        if (done) return true;
    }
    atomicExch(err, 1);
    return false;
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
        ::"r"(dst), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
        : "memory");
}

// shared-memory matrix descriptor of a K-major bf16 tile in the 128-byte swizzled layout TMA writes: rows of 128 bytes,
// 8-row groups 1024 bytes apart (stride byte offset), descriptor version 1, swizzle mode 128B
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
    uint64_t d = 0;
    d |= uint64_t((addr & 0x3FFFF) >> 4);
    d |= uint64_t(16 >> 4) << 16;    // leading byte offset (not used by the swizzled K-major layout)
    d |= uint64_t(1024 >> 4) << 32;  // stride byte offset
    d |= uint64_t(1) << 46;          // version
    d |= uint64_t(2) << 61;          // 128-byte swizzle
    return d;
}

// instruction descriptor of tcgen05.mma kind::f16: FP32 accumulator, bf16 A and B, both K-major, N = 128, M = 128
constexpr uint32_t TC_IDESC = (1u << 4) | (1u << 7) | (1u << 10) | (uint32_t(TC_BN >> 3) << 17) | (uint32_t(TC_BM >> 4) << 24);

__device__ __forceinline__ void mma_bf16(uint32_t tmem, uint64_t ad, uint64_t bd, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
        ::"r"(tmem), "l"(ad), "l"(bd), "r"(TC_IDESC), "r"(acc)
        : "memory");
}

// 32 consecutive FP32 columns of this warp's 32 TMEM lanes (one row per thread)
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t* v) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
        "%14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]),
          "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]), "=r"(v[16]),
          "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]),
          "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
        : "r"(taddr)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

__global__ void __launch_bounds__(TC_THREADS, 1)
    tc_gemm_kernel(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB, int m, int n,
                   int ktiles, int m_pad, int n_pad, float* __restrict__ C, int ldc, int* err) {
    extern __shared__ uint8_t smem_raw[];
    __shared__ __align__(8) uint64_t full_bar[TC_STAGES], empty_bar[TC_STAGES], done_bar;
    __shared__ uint32_t tmem_holder;
    __shared__ int s_fail;
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = blockIdx.x * TC_BM, n0 = blockIdx.y * TC_BN;
    const uint32_t sbase = smem_u32(smem);
    auto tileA = [&](int s, int p) { return sbase + uint32_t(s * TC_STAGE_BYTES + p * TC_TILE_BYTES); };
    auto tileB = [&](int s, int p) { return sbase + uint32_t(s * TC_STAGE_BYTES + (TC_PIECES + p) * TC_TILE_BYTES); };
    if (threadIdx.x == 0) {
        for (int s = 0; s < TC_STAGES; ++s) {
            mbar_init(smem_u32(&full_bar[s]), 1);
            mbar_init(smem_u32(&empty_bar[s]), 1);
        }
        mbar_init(smem_u32(&done_bar), 1);
        s_fail = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_holder)),
                     "r"(TC_TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_holder;

    if (threadIdx.x == 0) {  // TMA producer
        for (int kt = 0; kt < ktiles; ++kt) {
            const int s = kt % TC_STAGES;
            if (kt >= TC_STAGES && !mbar_wait(smem_u32(&empty_bar[s]), uint32_t((kt / TC_STAGES - 1) & 1), err)) {
                s_fail = 1;
                break;
            }
            const uint32_t fb = smem_u32(&full_bar[s]);
            mbar_expect_tx(fb, TC_STAGE_BYTES);
            for (int p = 0; p < TC_PIECES; ++p) {
                tma_load_2d(tileA(s, p), &mapA, kt * TC_BK, p * m_pad + m0, fb);
                tma_load_2d(tileB(s, p), &mapB, kt * TC_BK, p * n_pad + n0, fb);
            }
        }
    } else if (threadIdx.x == 32) {  // MMA issuer
        int issued_hi = 0, issued_lo = 0;
        for (int kt = 0; kt < ktiles; ++kt) {
            const int s = kt % TC_STAGES;
            if (!mbar_wait(smem_u32(&full_bar[s]), uint32_t((kt / TC_STAGES) & 1), err)) {
                s_fail = 1;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            for (int kk = 0; kk < TC_BK / 16; ++kk)
                for (int q = 0; q < 6; ++q) {
                    const uint64_t ad = smem_desc(tileA(s, c_prod_a[q]) + uint32_t(kk * 32));
                    const uint64_t bd = smem_desc(tileB(s, c_prod_b[q]) + uint32_t(kk * 32));
                    if (q == 0)
                        mma_bf16(tmem, ad, bd, issued_hi++ > 0 ? 1u : 0u);
                    else
                        mma_bf16(tmem + uint32_t(TC_BN), ad, bd, issued_lo++ > 0 ? 1u : 0u);
                }
            mma_commit(smem_u32(&empty_bar[s]));
        }
        mma_commit(smem_u32(&done_bar));  // arrives when every MMA issued above has completed
    }
    __syncwarp();
    // epilogue: the accumulator back from TMEM, C -= D
    const bool done = mbar_wait(smem_u32(&done_bar), 0u, err);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    __syncthreads();
    if (done && !s_fail) {
        const int row = m0 + warp * 32 + lane;
        for (int c0 = 0; c0 < TC_BN; c0 += 32) {
            uint32_t v[32], u[32];
            const uint32_t taddr = tmem + (uint32_t(warp * 32) << 16) + uint32_t(c0);
            tmem_ld32(taddr, v);
            tmem_ld32(taddr + uint32_t(TC_BN), u);
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            if (row < m)
#pragma unroll
                for (int j = 0; j < 32; ++j) {
                    const int col = n0 + c0 + j;
                    if (col < n) C[size_t(col) * ldc + row] -= __uint_as_float(v[j]) + __uint_as_float(u[j]);
                }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_TMEM_COLS) : "memory");
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
    static EncodeTiledFn fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
    }
    return fn;
}

// the tensor map of three stacked K-major pieces (3 rows_pad rows of k_pad bf16), box 64 x 128, 128-byte swizzle
bool make_map(CUtensorMap* map, void* base, int rows_pad, int k_pad) {
    EncodeTiledFn fn = encode_fn();
    if (!fn) return false;
    const cuuint64_t gdim[2] = {cuuint64_t(k_pad), cuuint64_t(TC_PIECES) * cuuint64_t(rows_pad)};
    const cuuint64_t gstride[1] = {cuuint64_t(k_pad) * 2};
    const cuuint32_t box[2] = {TC_BK, TC_BM};
    const cuuint32_t estride[2] = {1, 1};
    return fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, base, gdim, gstride, box, estride, CU_TENSOR_MAP_INTERLEAVE_NONE,
              CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) ==
           CUDA_SUCCESS;
}

}  // namespace

bool vp_tc_gemm_enabled() {
    const char* e = std::getenv("VP_LU_TENSOR_CORES");
    return !(e && e[0] == '0');
}

bool vp_tc_gemm_fits(int m, int n, int k) { return m >= TC_BM && n >= TC_BN && k >= TC_BK; }

void vp_tc_work_free(TcWork* w) {
    if (w->pieces) cudaFree(w->pieces);
    if (w->err) cudaFree(w->err);
    *w = TcWork();
}

int vp_tc_gemm_sub(vp_ctx* ctx, int m, int n, int k, const float* A, int lda, const float* B, int ldb, float* C,
                   int ldc) {
    if (m <= 0 || n <= 0 || k <= 0) return VP_OK;
    TcWork* w = &ctx->tc;
    const int m_pad = (m + TC_BM - 1) / TC_BM * TC_BM, n_pad = (n + TC_BN - 1) / TC_BN * TC_BN;
    const int k_pad = (k + TC_BK - 1) / TC_BK * TC_BK;
    const size_t na = size_t(TC_PIECES) * m_pad * k_pad, nb = size_t(TC_PIECES) * n_pad * k_pad;
    if (na + nb > w->cap) {
        vp_tc_work_free(w);
        int r;
        __nv_bfloat16* pieces = nullptr;
        if ((r = vp_alloc(ctx, &pieces, na + nb)) || (r = vp_alloc(ctx, &w->err, 1))) return r;
        w->pieces = pieces;
        w->cap = na + nb;
        VP_CUDA(ctx, cudaMemsetAsync(w->err, 0, sizeof(int), ctx->stream));
    }
    if (!w->attr_set) {
        VP_CUDA(ctx, cudaFuncSetAttribute(tc_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM));
        w->attr_set = true;
    }
    __nv_bfloat16* a3 = static_cast<__nv_bfloat16*>(w->pieces);
    __nv_bfloat16* b3 = a3 + na;
    split_a_kernel<<<dim3(m_pad / 32, k_pad / 32), 256, 0, ctx->stream>>>(m, k, A, lda, m_pad, k_pad, a3);
    split_b_kernel<<<int((size_t(n_pad) * k_pad + 255) / 256), 256, 0, ctx->stream>>>(k, n, B, ldb, n_pad, k_pad, b3);
    CUtensorMap ma, mb;
    if (!make_map(&ma, a3, m_pad, k_pad) || !make_map(&mb, b3, n_pad, k_pad))
        return vp_fail(ctx, VP_ERR_CUDA, "cuTensorMapEncodeTiled failed");
    tc_gemm_kernel<<<dim3(m_pad / TC_BM, n_pad / TC_BN), TC_THREADS, TC_SMEM, ctx->stream>>>(
        ma, mb, m, n, k_pad / TC_BK, m_pad, n_pad, C, ldc, w->err);
    ctx->launches += 3;
    VP_CUDA(ctx, cudaGetLastError());
    return VP_OK;
}

int vp_tc_gemm_check(vp_ctx* ctx) {
    TcWork* w = &ctx->tc;
    if (!w->err) return VP_OK;
    int e = 0;
    VP_CUDA(ctx, vp_d2h(ctx, &e, w->err, sizeof(int)));
    VP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (e) {
        cudaMemsetAsync(w->err, 0, sizeof(int), ctx->stream);
        return vp_fail(ctx, VP_ERR_TIMEOUT, "tensor-core GEMM: a bounded wait gave up");
    }
    return VP_OK;
}

extern "C" int vp_gemm_sub_f32(vp_ctx* ctx, int m, int n, int k, const float* A, int lda, const float* B, int ldb,
                               float* C, int ldc) {
    if (!ctx || m <= 0 || n <= 0 || k <= 0 || !A || !B || !C || lda < m || ldb < k || ldc < m)
        return vp_fail(ctx, VP_ERR_ARG, "bad argument");
    DeviceGuard dg;
    if (dg.set(ctx->device) != cudaSuccess) return vp_fail(ctx, VP_ERR_CUDA, "cudaSetDevice");
    float *dA, *dB, *dC;
    int r;
    if ((r = vp_upload(ctx, &dA, A, size_t(lda) * k))) return r;
    if ((r = vp_upload(ctx, &dB, B, size_t(ldb) * n))) {
        cudaFree(dA);
        return r;
    }
    if ((r = vp_upload(ctx, &dC, C, size_t(ldc) * n))) {
        cudaFree(dA);
        cudaFree(dB);
        return r;
    }
    r = vp_tc_gemm_sub(ctx, m, n, k, dA, lda, dB, ldb, dC, ldc);
    if (!r) r = vp_tc_gemm_check(ctx);
    if (!r) {
        cudaError_t e = vp_d2h(ctx, C, dC, sizeof(float) * size_t(ldc) * n);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) r = vp_fail(ctx, VP_ERR_CUDA, std::string("vp_gemm_sub_f32: ") + cudaGetErrorString(e));
    }
    cudaFree(dA);
    cudaFree(dB);
    cudaFree(dC);
    return r;
}
