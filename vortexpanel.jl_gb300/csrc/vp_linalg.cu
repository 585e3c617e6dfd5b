// Bordered dense solve on the GPU: factorize_galerkin / solve_galerkin of src/assembly/solve.jl:15-115 over the
// Galerkin reduction C' A [C; W] of src/dofmap/system.jl:141-165.
//
//  - reduction + border: one kernel gathers M = C' A Cf (A row-major FP64, C and Cf sparse) into a column-major FP64
//    matrix through a shared-memory transpose, then the border rows/columns (scaled to the mean |diagonal|) are set;
//  - LU with partial pivoting (the reference calls LAPACK dgetrf): recursive (left half, swap, TRSM, GEMM, right
//    half). Its leaf panels (m x 16 columns) are factored by one thread-block cluster of 8 CTAs that holds the panel
//    in distributed shared memory: per column, every CTA finds its pivot candidate, one cluster barrier, every CTA
//    reads the 8 candidates and the pivot row through DSMEM, swaps and updates its rows. TRSM is cuBLAS; the
//    trailing-update GEMM is cuBLAS DGEMM for VP_FP64 and, for VP_MIXED, the tensor-core GEMM of vp_tcgemm.cu
//    (three-piece bf16 split, six tcgen05 products accumulated in FP32 in TMEM) for updates of at least one
//    128 x 128 x 64 tile, cuBLAS SGEMM for the smaller ones;
//  - VP_MIXED keeps the FP64 bordered matrix and refines every solve with FP64 residuals (iterative refinement) to
//    FP64 accuracy;
//  - the 1-norm condition estimate of dgecon (Hager/Higham, as LAPACK dlacn2) from solves with M and M'.
#include <cooperative_groups.h>

#include <algorithm>
#include <climits>
#include <cmath>

#include "vp_internal.h"

namespace cg = cooperative_groups;

namespace {

constexpr int LU_CL = 8;       // CTAs per cluster of the leaf kernel
constexpr int LU_THREADS = 512;

// M(q, q') = sum_{i in C[:,q]} C[i,q] sum_{j in Cf[:,q']} A[i, j] Cf[j,q'], written column-major (ld n)
__global__ void reduce_kernel(int nq, int n, const double* __restrict__ A, long long lda, const int* __restrict__ ctp,
                              const int* __restrict__ cti, const double* __restrict__ ctv,
                              const int* __restrict__ cfp, const int* __restrict__ cfi,
                              const double* __restrict__ cfv, double* __restrict__ M) {
    __shared__ double tile[32][33];
    const int q0 = blockIdx.y * 32, p0 = blockIdx.x * 32;  // q rows of M, p columns of M
    const int tx = threadIdx.x, ty = threadIdx.y;          // 32 x 8
    for (int yy = ty; yy < 32; yy += 8) {
        int q = q0 + yy, p = p0 + tx;
        double acc = 0;
        if (q < nq && p < nq) {
            for (int u = ctp[q]; u < ctp[q + 1]; ++u) {
                const double* Ar = A + size_t(cti[u]) * size_t(lda);
                double part = 0;
                for (int v = cfp[p]; v < cfp[p + 1]; ++v) part += Ar[cfi[v]] * cfv[v];
                acc += ctv[u] * part;
            }
        }
        tile[yy][tx] = acc;
    }
    __syncthreads();
    for (int yy = ty; yy < 32; yy += 8) {
        int p = p0 + yy, q = q0 + tx;
        if (q < nq && p < nq) M[size_t(p) * n + q] = tile[tx][yy];
    }
}

__global__ void border_kernel(int nq, int n, int nb, const double* __restrict__ ecol, const double* __restrict__ crow,
                              double* __restrict__ M) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int k = 0; k < nb; ++k) {
        // column nq+k: se_k e_k on the unknowns, 0 on the border rows; row nq+k: scaled c_k, 0 in the corner
        M[size_t(nq + k) * n + i] = i < nq ? ecol[size_t(k) * nq + i] : 0.0;
        if (i < nq) M[size_t(i) * n + nq + k] = crow[size_t(k) * nq + i];
    }
}

template <class T>
__global__ void col_abs_sum_kernel(int n, const T* __restrict__ M, double* __restrict__ out) {
    __shared__ double red[256];
    int c = blockIdx.x;
    double s = 0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) s += fabs(double(M[size_t(c) * n + i]));
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[c] = red[0];
}

// LU leaf: rows [c0, c0 + m) x columns [c0, c0 + w) (w <= W) of the column-major matrix (ld lda), partial pivoting.
// Rows are split over the 8 CTAs of the cluster (R rows each) and held in shared memory for the whole panel.
template <class T, int W>
__global__ void __cluster_dims__(LU_CL, 1, 1) __launch_bounds__(LU_THREADS)
    lu_leaf_kernel(T* __restrict__ A, long long lda, int c0, int m, int w, int R, int* __restrict__ ipiv,
                   int* __restrict__ info) {
    cg::cluster_group cl = cg::this_cluster();
    const int rank = (int)cl.block_rank();
    extern __shared__ __align__(16) unsigned char smraw[];
    T* pan = reinterpret_cast<T*>(smraw);  // R x W, row-major
    __shared__ T s_cval[2];
    __shared__ int s_cidx[2];
    __shared__ T s_crow[2][W];
    __shared__ T s_rowj[2][W];
    __shared__ T s_piv[W];
    __shared__ T red_v[LU_THREADS / 32];
    __shared__ int red_i[LU_THREADS / 32];
    __shared__ int s_p;
    __shared__ T s_gbest;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int row0 = rank * R;
    const int nloc = max(0, min(R, m - row0));
    for (int k = 0; k < W; ++k)
        for (int li = tid; li < nloc; li += LU_THREADS)
            pan[li * W + k] = k < w ? A[size_t(c0 + k) * size_t(lda) + size_t(c0 + row0 + li)] : T(0);
    __syncthreads();
    for (int j = 0; j < w; ++j) {
        const int buf = j & 1;
        // 1. this CTA's candidate: the largest |a(i, j)| over its rows i >= j (smallest index on ties)
        T best = T(-1);
        int bi = INT_MAX;
        for (int li = tid; li < nloc; li += LU_THREADS) {
            int i = row0 + li;
            if (i >= j) {
                T v = fabs(pan[li * W + j]);
                if (v > best || (v == best && i < bi)) {
                    best = v;
                    bi = i;
                }
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            T ov = __shfl_xor_sync(0xffffffffu, best, o);
            int oi = __shfl_xor_sync(0xffffffffu, bi, o);
            if (ov > best || (ov == best && oi < bi)) {
                best = ov;
                bi = oi;
            }
        }
        if (lane == 0) {
            red_v[wid] = best;
            red_i[wid] = bi;
        }
        __syncthreads();
        if (tid == 0) {
            for (int w = 1; w < LU_THREADS / 32; ++w)
                if (red_v[w] > best || (red_v[w] == best && red_i[w] < bi)) {
                    best = red_v[w];
                    bi = red_i[w];
                }
            s_cval[buf] = best;
            s_cidx[buf] = bi;
            if (bi != INT_MAX)
                for (int k = 0; k < W; ++k) s_crow[buf][k] = pan[(bi - row0) * W + k];
            if (j >= row0 && j < row0 + nloc)
                for (int k = 0; k < W; ++k) s_rowj[buf][k] = pan[(j - row0) * W + k];
        }
        __syncthreads();
        cl.sync();
        // 2. the pivot over the cluster, its row, and the old row j
        if (tid == 0) {
            T gb = T(-1);
            int gi = INT_MAX;
            for (int r = 0; r < LU_CL; ++r) {
                T v = *cl.map_shared_rank(&s_cval[buf], r);
                int ix = *cl.map_shared_rank(&s_cidx[buf], r);
                if (ix != INT_MAX && (v > gb || (v == gb && ix < gi))) {
                    gb = v;
                    gi = ix;
                }
            }
            s_p = gi;
            s_gbest = gb;
        }
        __syncthreads();
        const int p = s_p;
        const bool zero = !(s_gbest > T(0)) || p == INT_MAX;
        if (zero) {
            if (rank == 0 && tid == 0) {
                if (*info == 0) *info = c0 + j + 1;
                ipiv[c0 + j] = c0 + j;
            }
        } else {
            const int cp = p / R, cj = j / R;
            if (tid < W) {
                T pv = *cl.map_shared_rank(&s_crow[buf][tid], cp);
                T rj = *cl.map_shared_rank(&s_rowj[buf][tid], cj);
                s_piv[tid] = pv;
                if (rank == cj) pan[(j - row0) * W + tid] = pv;
                if (rank == cp && p != j) pan[(p - row0) * W + tid] = rj;
            }
            if (rank == 0 && tid == 0) ipiv[c0 + j] = c0 + p;
            __syncthreads();
            // 3. eliminate below the pivot
            const T pj = s_piv[j];
            for (int li = tid; li < nloc; li += LU_THREADS) {
                int i = row0 + li;
                if (i > j) {
                    T l = pan[li * W + j] / pj;
                    pan[li * W + j] = l;
#pragma unroll
                    for (int k = 0; k < W; ++k)
                        if (k > j) pan[li * W + k] -= l * s_piv[k];
                }
            }
        }
        __syncthreads();
    }
    for (int k = 0; k < w; ++k)
        for (int li = tid; li < nloc; li += LU_THREADS)
            A[size_t(c0 + k) * size_t(lda) + size_t(c0 + row0 + li)] = pan[li * W + k];
    cl.sync();  // no CTA leaves while another may still read its shared memory
}

// apply the row swaps ipiv[j0..j1) (in order) to the columns [cs, ce)
template <class T>
__global__ void laswp_kernel(T* __restrict__ A, long long lda, int cs, int ce, int j0, int j1, const int* __restrict__ ipiv) {
    int c = cs + blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ce) return;
    T* col = A + size_t(c) * size_t(lda);
    for (int j = j0; j < j1; ++j) {
        int p = ipiv[j];
        if (p != j) {
            T t = col[j];
            col[j] = col[p];
            col[p] = t;
        }
    }
}

// x(i, k) = b(perm[i], k) (forward) or x(perm[i], k) = b(i, k) (inverse); column-major n x nrhs
template <class T>
__global__ void permute_kernel(int n, int nrhs, const int* __restrict__ perm, int inverse, const T* __restrict__ b,
                               T* __restrict__ x) {
    size_t idx = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    if (idx >= size_t(n) * nrhs) return;
    int i = int(idx % n), k = int(idx / n);
    if (inverse)
        x[size_t(k) * n + perm[i]] = b[idx];
    else
        x[idx] = b[size_t(k) * n + perm[i]];
}

// rhs = [C' b; 0] for nrhs columns (b: nslot x nrhs column-major)
__global__ void ctb_kernel(int nq, int n, int nslot, int nrhs, const int* __restrict__ ctp, const int* __restrict__ cti,
                           const double* __restrict__ ctv, const double* __restrict__ b, double* __restrict__ rhs) {
    size_t idx = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    if (idx >= size_t(n) * nrhs) return;
    int q = int(idx % n), k = int(idx / n);
    double s = 0;
    if (q < nq)
        for (int u = ctp[q]; u < ctp[q + 1]; ++u) s += ctv[u] * b[size_t(k) * nslot + cti[u]];
    rhs[idx] = s;
}

template <class A_, class B_>
__global__ void convert_kernel(size_t n, const A_* __restrict__ a, B_* __restrict__ b) {
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x)
        b[i] = B_(a[i]);
}

__global__ void axpy_f2d_kernel(size_t n, const float* __restrict__ d, double* __restrict__ x) {
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x)
        x[i] += double(d[i]);
}

// ------------------------------------------------------------------------------------------------------------------
// host drivers

template <class T>
int gemm_sub(vp_ctx* ctx, int m, int n, int k, const T* A, int lda, const T* B, int ldb, T* C, int ldc);
template <>
int gemm_sub<double>(vp_ctx* ctx, int m, int n, int k, const double* A, int lda, const double* B, int ldb, double* C,
                     int ldc) {
    const double one = 1.0, mone = -1.0;
    VP_BLAS(ctx, cublasDgemm(ctx->blas, CUBLAS_OP_N, CUBLAS_OP_N, m, n, k, &mone, A, lda, B, ldb, &one, C, ldc));
    return VP_OK;
}
template <>
int gemm_sub<float>(vp_ctx* ctx, int m, int n, int k, const float* A, int lda, const float* B, int ldb, float* C,
                    int ldc) {
    // the trailing updates large enough for a 128 x 128 tile run on the tensor cores (three-piece bf16 split, FP32
    // accumulation in TMEM: FP32-class products); the small ones on cuBLAS
    if (vp_tc_gemm_enabled() && vp_tc_gemm_fits(m, n, k)) return vp_tc_gemm_sub(ctx, m, n, k, A, lda, B, ldb, C, ldc);
    const float one = 1.0f, mone = -1.0f;
    VP_BLAS(ctx, cublasSgemm(ctx->blas, CUBLAS_OP_N, CUBLAS_OP_N, m, n, k, &mone, A, lda, B, ldb, &one, C, ldc));
    return VP_OK;
}

template <class T>
int trsm(vp_ctx* ctx, cublasFillMode_t uplo, cublasOperation_t op, cublasDiagType_t diag, int m, int n, const T* A,
         int lda, T* B, int ldb);
template <>
int trsm<double>(vp_ctx* ctx, cublasFillMode_t uplo, cublasOperation_t op, cublasDiagType_t diag, int m, int n,
                 const double* A, int lda, double* B, int ldb) {
    const double one = 1.0;
    VP_BLAS(ctx, cublasDtrsm(ctx->blas, CUBLAS_SIDE_LEFT, uplo, op, diag, m, n, &one, A, lda, B, ldb));
    return VP_OK;
}
template <>
int trsm<float>(vp_ctx* ctx, cublasFillMode_t uplo, cublasOperation_t op, cublasDiagType_t diag, int m, int n,
                const float* A, int lda, float* B, int ldb) {
    const float one = 1.0f;
    VP_BLAS(ctx, cublasStrsm(ctx->blas, CUBLAS_SIDE_LEFT, uplo, op, diag, m, n, &one, A, lda, B, ldb));
    return VP_OK;
}

template <class T>
int leaf_width(int m) {
    // the widest leaf whose panel fits the cluster's shared memory (200 KB per CTA)
    int R = (m + LU_CL - 1) / LU_CL;
    for (int w : {16, 8, 4})
        if (size_t(R) * w * sizeof(T) <= 200 * 1024) return w;
    return 0;
}

template <class T, int W>
int launch_leaf(vp_ctx* ctx, T* A, int lda, int c0, int m, int w, int* ipiv, int* info) {
    if (w < 1 || w > W || w > m) return vp_fail(ctx, VP_ERR_ARG, "LU leaf width out of range");
    int R = (m + LU_CL - 1) / LU_CL;
    size_t smem = size_t(R) * W * sizeof(T);
    if (smem > 227 * 1024) return vp_fail(ctx, VP_ERR_ARG, "LU leaf panel does not fit shared memory");
    VP_CUDA(ctx, cudaFuncSetAttribute(lu_leaf_kernel<T, W>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    lu_leaf_kernel<T, W><<<LU_CL, LU_THREADS, smem, ctx->stream>>>(A, lda, c0, m, w, R, ipiv, info);
    ctx->launches++;
    VP_CUDA(ctx, cudaGetLastError());
    return VP_OK;
}

// factor a leaf of w columns with the smallest kernel instance that holds it
template <class T>
int leaf(vp_ctx* ctx, T* A, int lda, int c0, int w, int m, int* ipiv, int* info) {
    if (w > 8) return launch_leaf<T, 16>(ctx, A, lda, c0, m, w, ipiv, info);
    if (w > 4) return launch_leaf<T, 8>(ctx, A, lda, c0, m, w, ipiv, info);
    if (w > 2) return launch_leaf<T, 4>(ctx, A, lda, c0, m, w, ipiv, info);
    if (w > 1) return launch_leaf<T, 2>(ctx, A, lda, c0, m, w, ipiv, info);
    return launch_leaf<T, 1>(ctx, A, lda, c0, m, w, ipiv, info);
}

__global__ void iota_kernel(int n, int* __restrict__ a) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] = i;
}

template <class T>
int laswp(vp_ctx* ctx, T* A, int lda, int cs, int ce, int j0, int j1, const int* ipiv) {
    if (ce <= cs || j1 <= j0) return VP_OK;
    int nc = ce - cs;
    laswp_kernel<T><<<(nc + 127) / 128, 128, 0, ctx->stream>>>(A, lda, cs, ce, j0, j1, ipiv);
    ctx->launches++;
    VP_CUDA(ctx, cudaGetLastError());
    return VP_OK;
}

// recursive LU of the columns [c0, c0 + w) (rows c0..n-1)
template <class T>
int rgetrf(vp_ctx* ctx, T* A, int n, int c0, int w, int lw, int* ipiv, int* info) {
    int r;
    if (w <= lw) return leaf<T>(ctx, A, n, c0, w, n - c0, ipiv, info);
    int w1 = ((w / 2 + lw - 1) / lw) * lw;
    if (w1 >= w) w1 = w - lw;
    int w2 = w - w1;
    if ((r = rgetrf<T>(ctx, A, n, c0, w1, lw, ipiv, info))) return r;
    if ((r = laswp<T>(ctx, A, n, c0 + w1, c0 + w, c0, c0 + w1, ipiv))) return r;
    if ((r = trsm<T>(ctx, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_N, CUBLAS_DIAG_UNIT, w1, w2, A + size_t(c0) * n + c0, n,
                     A + size_t(c0 + w1) * n + c0, n)))
        return r;
    if (n - c0 - w1 > 0 &&
        (r = gemm_sub<T>(ctx, n - c0 - w1, w2, w1, A + size_t(c0) * n + (c0 + w1), n, A + size_t(c0 + w1) * n + c0, n,
                         A + size_t(c0 + w1) * n + (c0 + w1), n)))
        return r;
    if ((r = rgetrf<T>(ctx, A, n, c0 + w1, w2, lw, ipiv, info))) return r;
    return laswp<T>(ctx, A, n, c0, c0 + w1, c0 + w1, c0 + w, ipiv);
}

// solve with the factors: op = N: M x = b; op = T: M' x = b (b, x: n x nrhs column-major, device; may alias)
template <class T>
int lu_solve(vp_ctx* ctx, const vp_factor* F, const T* LU, const int* d_perm, int nrhs, T* b, T* work, bool trans) {
    int n = F->n, r;
    size_t tot = size_t(n) * nrhs;
    int nb = int((tot + 255) / 256);
    if (!trans) {
        permute_kernel<T><<<nb, 256, 0, ctx->stream>>>(n, nrhs, d_perm, 0, b, work);
        ctx->launches++;
        if ((r = trsm<T>(ctx, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_N, CUBLAS_DIAG_UNIT, n, nrhs, LU, n, work, n))) return r;
        if ((r = trsm<T>(ctx, CUBLAS_FILL_MODE_UPPER, CUBLAS_OP_N, CUBLAS_DIAG_NON_UNIT, n, nrhs, LU, n, work, n))) return r;
        VP_CUDA(ctx, cudaMemcpyAsync(b, work, sizeof(T) * tot, cudaMemcpyDeviceToDevice, ctx->stream));
    } else {
        if ((r = trsm<T>(ctx, CUBLAS_FILL_MODE_UPPER, CUBLAS_OP_T, CUBLAS_DIAG_NON_UNIT, n, nrhs, LU, n, b, n))) return r;
        if ((r = trsm<T>(ctx, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_T, CUBLAS_DIAG_UNIT, n, nrhs, LU, n, b, n))) return r;
        permute_kernel<T><<<nb, 256, 0, ctx->stream>>>(n, nrhs, d_perm, 1, b, work);
        ctx->launches++;
        VP_CUDA(ctx, cudaMemcpyAsync(b, work, sizeof(T) * tot, cudaMemcpyDeviceToDevice, ctx->stream));
    }
    VP_CUDA(ctx, cudaGetLastError());
    return VP_OK;
}

}  // namespace

int vp_lu_factor(vp_ctx* ctx, int precision, int n, double* M64, vp_factor* F) {
    int r;
    int* d_info;
    if ((r = vp_alloc(ctx, &d_info, 1))) return r;
    VP_CUDA(ctx, cudaMemsetAsync(d_info, 0, sizeof(int), ctx->stream));
    if ((r = vp_alloc(ctx, &F->ipiv, size_t(n)))) return r;
    iota_kernel<<<(n + 255) / 256, 256, 0, ctx->stream>>>(n, F->ipiv);  // every swap index valid from the start
    ctx->launches++;
    if (precision == VP_FP64) {
        if ((r = vp_alloc(ctx, &F->LU64, size_t(n) * n))) return r;
        VP_CUDA(ctx, cudaMemcpyAsync(F->LU64, M64, sizeof(double) * size_t(n) * n, cudaMemcpyDeviceToDevice, ctx->stream));
        int lw = leaf_width<double>(n);
        if (!lw) return vp_fail(ctx, VP_ERR_ARG, "matrix too large for the LU panel");
        r = rgetrf<double>(ctx, F->LU64, n, 0, n, lw, F->ipiv, d_info);
    } else {
        if ((r = vp_alloc(ctx, &F->LU32, size_t(n) * n))) return r;
        convert_kernel<double, float><<<4 * ctx->nsm, 256, 0, ctx->stream>>>(size_t(n) * n, M64, F->LU32);
        ctx->launches++;
        int lw = leaf_width<float>(n);
        if (!lw) return vp_fail(ctx, VP_ERR_ARG, "matrix too large for the LU panel");
        r = rgetrf<float>(ctx, F->LU32, n, 0, n, lw, F->ipiv, d_info);
        if (!r) r = vp_tc_gemm_check(ctx);
    }
    if (r) {
        cudaFree(d_info);
        return r;
    }
    int info = 0;
    F->h_ipiv.resize(n);
    VP_CUDA(ctx, vp_d2h(ctx, &info, d_info, sizeof(int)));
    VP_CUDA(ctx, vp_d2h(ctx, F->h_ipiv.data(), F->ipiv, sizeof(int) * n));
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    cudaFree(d_info);
    if (e != cudaSuccess) return vp_fail(ctx, VP_ERR_CUDA, std::string("LU: ") + cudaGetErrorString(e));
    if (info > 0) return vp_fail(ctx, VP_ERR_SINGULAR, "zero pivot in column " + std::to_string(info));
    return VP_OK;
}

// ------------------------------------------------------------------------------------------------------------------

static int solve_core(vp_ctx* ctx, const vp_factor* F, int nrhs, double* x, bool trans, int* iters,
                      SolveWork* ws = nullptr);

extern "C" int vp_factorize(vp_ctx* ctx, const vp_system* sys, int precision, int nq, const int* C_rowptr,
                            const int* C_col, const double* C_val, int nwake, const int* W_rowptr, const int* W_col,
                            const double* W_val, int nbody, const int* q_body, const double* slot_area,
                            const int* slot_body, vp_factor** out, double* cond) {
    if (!ctx || !sys || !C_rowptr || !C_col || !C_val || !out || !q_body || !slot_area || !slot_body)
        return vp_fail(ctx, VP_ERR_ARG, "null argument");
    *out = nullptr;
    if (cudaSetDevice(ctx->device) != cudaSuccess) return vp_fail(ctx, VP_ERR_CUDA, "cudaSetDevice");
    if (precision != VP_FP64 && precision != VP_MIXED) return vp_fail(ctx, VP_ERR_ARG, "unknown precision");
    const int nslot = sys->nslot;
    if (nwake != sys->nwnode)
        return vp_fail(ctx, VP_ERR_ARG, "A is " + std::to_string(nslot) + "x" + std::to_string(sys->ncols) +
                                            ", expected " + std::to_string(nslot) + "x" + std::to_string(nslot + nwake));
    if (nq <= 0 || nbody < 0) return vp_fail(ctx, VP_ERR_ARG, "nq must be positive");
    // C' and Cf' = [C; W]' as CSR over the unknowns
    std::vector<std::vector<std::pair<int, double>>> ct(nq), cft(nq);
    for (int i = 0; i < nslot; ++i)
        for (int u = C_rowptr[i]; u < C_rowptr[i + 1]; ++u) {
            int q = C_col[u];
            if (q < 0 || q >= nq) return vp_fail(ctx, VP_ERR_ARG, "C column out of range");
            ct[q].push_back({i, C_val[u]});
            cft[q].push_back({i, C_val[u]});
        }
    for (int i = 0; i < nwake; ++i)
        for (int u = W_rowptr[i]; u < W_rowptr[i + 1]; ++u) {
            int q = W_col[u];
            if (q < 0 || q >= nq) return vp_fail(ctx, VP_ERR_ARG, "W column out of range");
            cft[q].push_back({nslot + i, W_val[u]});
        }
    auto csr = [](const std::vector<std::vector<std::pair<int, double>>>& rows, std::vector<int>& p, std::vector<int>& c,
                  std::vector<double>& v) {
        p.assign(1, 0);
        for (auto& r : rows) {
            for (auto& e : r) {
                c.push_back(e.first);
                v.push_back(e.second);
            }
            p.push_back((int)c.size());
        }
        if (c.empty()) {
            c.push_back(0);
            v.push_back(0);
        }
    };
    std::vector<int> ctp, cti, cfp, cfi;
    std::vector<double> ctv, cfv;
    csr(ct, ctp, cti, ctv);
    csr(cft, cfp, cfi, cfv);
    const int nb = nbody;
    const int n = nq + nb;
    vp_factor* F = new vp_factor();
    F->n = n;
    F->nq = nq;
    F->nb = nb;
    F->nslot = nslot;
    F->ncols = sys->ncols;
    F->precision = precision;
    int r;
    auto fail = [&](int code) {
        vp_factor_free(F);
        return code;
    };
    int *d_cfp, *d_cfi;
    double* d_cfv;
    if ((r = vp_upload(ctx, &F->Ct_ptr, ctp.data(), ctp.size())) || (r = vp_upload(ctx, &F->Ct_col, cti.data(), cti.size())) ||
        (r = vp_upload(ctx, &F->Ct_val, ctv.data(), ctv.size())))
        return fail(r);
    if ((r = vp_upload(ctx, &d_cfp, cfp.data(), cfp.size()))) return fail(r);
    if ((r = vp_upload(ctx, &d_cfi, cfi.data(), cfi.size()))) { cudaFree(d_cfp); return fail(r); }
    if ((r = vp_upload(ctx, &d_cfv, cfv.data(), cfv.size()))) { cudaFree(d_cfp); cudaFree(d_cfi); return fail(r); }
    if ((r = vp_alloc(ctx, &F->M, size_t(n) * n))) { cudaFree(d_cfp); cudaFree(d_cfi); cudaFree(d_cfv); return fail(r); }
    vp_phase_begin(ctx, PH_REDUCE);
    VP_CUDA(ctx, cudaMemsetAsync(F->M, 0, sizeof(double) * size_t(n) * n, ctx->stream));
    dim3 grid((nq + 31) / 32, (nq + 31) / 32), block(32, 8);
    reduce_kernel<<<grid, block, 0, ctx->stream>>>(nq, n, sys->A, sys->ncols, F->Ct_ptr, F->Ct_col, F->Ct_val, d_cfp,
                                                   d_cfi, d_cfv, F->M);
    ctx->launches++;
    VP_CUDA(ctx, cudaGetLastError());
    // border (bordered_matrix, solve.jl:23-38): scale = mean |diag|, e_k and c_k scaled to 2-norm = scale
    std::vector<double> diag(nq);
    vp_phase_end(ctx);
    VP_CUDA(ctx, cudaMemcpy2DAsync(diag.data(), sizeof(double), F->M, sizeof(double) * (size_t(n) + 1), sizeof(double), nq,
                                   cudaMemcpyDeviceToHost, ctx->stream));
    VP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    cudaFree(d_cfp);
    cudaFree(d_cfi);
    cudaFree(d_cfv);
    double scale = 0;
    for (double d : diag) scale += std::fabs(d);
    scale /= nq;
    F->h_se.assign(nb, 0.0);
    if (nb > 0) {
        std::vector<double> ecol(size_t(nb) * nq, 0.0), crow(size_t(nb) * nq, 0.0);
        for (int k = 0; k < nb; ++k) {
            double ne = 0, nc = 0;
            std::vector<double> c(nq, 0.0);
            for (int q = 0; q < nq; ++q) {
                if (q_body[q] == k + 1) ne += 1;
                for (auto& e : ct[q])
                    if (slot_body[e.first] == k + 1) c[q] += e.second * slot_area[e.first];
            }
            for (int q = 0; q < nq; ++q) nc += c[q] * c[q];
            ne = std::sqrt(ne);
            nc = std::sqrt(nc);
            if (!(ne > 0) || !(nc > 0)) return fail(vp_fail(ctx, VP_ERR_ARG, "a body has no unknowns"));
            F->h_se[k] = scale / ne;
            for (int q = 0; q < nq; ++q) {
                ecol[size_t(k) * nq + q] = q_body[q] == k + 1 ? F->h_se[k] : 0.0;
                crow[size_t(k) * nq + q] = c[q] * (scale / nc);
            }
        }
        double *d_e, *d_c;
        if ((r = vp_upload(ctx, &d_e, ecol.data(), ecol.size()))) return fail(r);
        if ((r = vp_upload(ctx, &d_c, crow.data(), crow.size()))) { cudaFree(d_e); return fail(r); }
        border_kernel<<<(n + 255) / 256, 256, 0, ctx->stream>>>(nq, n, nb, d_e, d_c, F->M);
        ctx->launches++;
        VP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        cudaFree(d_e);
        cudaFree(d_c);
    }
    // norms of M (1-norm for the condition estimate, inf-norm for the refinement test)
    {
        double* d_cs;
        if ((r = vp_alloc(ctx, &d_cs, size_t(n)))) return fail(r);
        col_abs_sum_kernel<double><<<n, 256, 0, ctx->stream>>>(n, F->M, d_cs);
        ctx->launches++;
        std::vector<double> cs(n);
        VP_CUDA(ctx, vp_d2h(ctx, cs.data(), d_cs, sizeof(double) * n));
        VP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        cudaFree(d_cs);
        F->norm1 = *std::max_element(cs.begin(), cs.end());
    }
    vp_phase_begin(ctx, PH_LU);
    r = vp_lu_factor(ctx, precision, n, F->M, F);
    vp_phase_end(ctx);
    if (r) return fail(r);
    // permutation from the sequential swaps
    std::vector<int> perm(n);
    for (int i = 0; i < n; ++i) perm[i] = i;
    for (int j = 0; j < n; ++j) std::swap(perm[j], perm[F->h_ipiv[j]]);
    if ((r = vp_upload(ctx, &F->perm, perm.data(), perm.size()))) return fail(r);
    if (!F->h_se.empty() && (r = vp_upload(ctx, &F->se, F->h_se.data(), F->h_se.size()))) return fail(r);
    // 1-norm condition estimate (LAPACK dgecon / dlacn2: Hager's method with Higham's refinements)
    {
        vp_phase_begin(ctx, PH_COND);
        std::vector<double> hx(n), hy(n);
        double *dx;
        if ((r = vp_alloc(ctx, &dx, size_t(n)))) return fail(r);
        auto solve1 = [&](bool trans) -> int {
            VP_CUDA(ctx, vp_h2d(ctx, dx, hx.data(), sizeof(double) * n));
            int rr = solve_core(ctx, F, 1, dx, trans, nullptr);
            if (rr) return rr;
            VP_CUDA(ctx, vp_d2h(ctx, hy.data(), dx, sizeof(double) * n));
            VP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
            return VP_OK;
        };
        auto sgn = [](double v) { return v >= 0 ? 1.0 : -1.0; };
        for (int i = 0; i < n; ++i) hx[i] = 1.0 / n;
        if ((r = solve1(false))) { cudaFree(dx); return fail(r); }
        double est = 0;
        for (double v : hy) est += std::fabs(v);
        std::vector<double> xi(n);
        for (int i = 0; i < n; ++i) xi[i] = sgn(hy[i]);
        hx = xi;
        if ((r = solve1(true))) { cudaFree(dx); return fail(r); }
        int jmax = 0;
        for (int i = 1; i < n; ++i)
            if (std::fabs(hy[i]) > std::fabs(hy[jmax])) jmax = i;
        for (int iter = 2; iter <= 5; ++iter) {
            std::fill(hx.begin(), hx.end(), 0.0);
            hx[jmax] = 1.0;
            if ((r = solve1(false))) { cudaFree(dx); return fail(r); }
            double old = est;
            est = 0;
            for (double v : hy) est += std::fabs(v);
            bool same = true;
            for (int i = 0; i < n && same; ++i) same = sgn(hy[i]) == xi[i];
            if (same || est <= old) break;
            for (int i = 0; i < n; ++i) xi[i] = sgn(hy[i]);
            hx = xi;
            if ((r = solve1(true))) { cudaFree(dx); return fail(r); }
            int jlast = jmax;
            jmax = 0;
            for (int i = 1; i < n; ++i)
                if (std::fabs(hy[i]) > std::fabs(hy[jmax])) jmax = i;
            if (std::fabs(hy[jlast]) == std::fabs(hy[jmax])) break;
        }
        double altsgn = 1;
        for (int i = 0; i < n; ++i) {
            hx[i] = altsgn * (1.0 + double(i) / std::max(n - 1, 1));
            altsgn = -altsgn;
        }
        if ((r = solve1(false))) { cudaFree(dx); return fail(r); }
        double temp = 0;
        for (double v : hy) temp += std::fabs(v);
        temp = 2 * temp / (3.0 * n);
        if (temp > est) est = temp;
        cudaFree(dx);
        vp_phase_end(ctx);
        F->cond = est * F->norm1;
    }
    if (cond) *cond = F->cond;
    *out = F;
    return VP_OK;
}

int vp_solve_work_alloc(vp_ctx* ctx, const vp_factor* F, SolveWork* w) {
    const size_t n = size_t(F->n);
    int r;
    w->n = F->n;
    if ((r = vp_alloc(ctx, &w->work64, n)) || (r = vp_alloc(ctx, &w->rhs, n)) || (r = vp_alloc(ctx, &w->res, n)) ||
        (r = vp_alloc(ctx, &w->f, n)) || (r = vp_alloc(ctx, &w->fw, n))) {
        vp_solve_work_free(w);
        return r;
    }
    return VP_OK;
}

void vp_solve_work_free(SolveWork* w) {
    cudaFree(w->work64);
    cudaFree(w->rhs);
    cudaFree(w->res);
    cudaFree(w->f);
    cudaFree(w->fw);
    *w = SolveWork();
}

// solve in place (x holds the right hand side on entry); VP_MIXED refines with FP64 residuals of M. With ws (one
// right hand side) its buffers are used and nothing is allocated.
static int solve_core(vp_ctx* ctx, const vp_factor* F, int nrhs, double* x, bool trans, int* iters, SolveWork* ws) {
    const int n = F->n;
    const int* d_perm = F->perm;
    const double norm1 = F->norm1;
    const size_t tot = size_t(n) * nrhs;
    int r;
    if (ws && (nrhs != 1 || ws->n != n)) return vp_fail(ctx, VP_ERR_ARG, "solve workspace does not fit");
    if (F->precision == VP_FP64) {
        double* work;
        if (ws) {
            work = ws->work64;
        } else if ((r = vp_alloc(ctx, &work, tot))) {
            return r;
        }
        r = lu_solve<double>(ctx, F, F->LU64, d_perm, nrhs, x, work, trans);
        if (!ws) cudaFree(work);
        if (iters) *iters = 1;
        return r;
    }
    // mixed: x0 = LU32^-1 rhs; r = rhs - M x; x += LU32^-1 r until the residual is at FP64 rounding level
    double *rhs, *res;
    float *f, *fw;
    if (ws) {
        rhs = ws->rhs;
        res = ws->res;
        f = ws->f;
        fw = ws->fw;
    } else {
        if ((r = vp_alloc(ctx, &rhs, tot))) return r;
        if ((r = vp_alloc(ctx, &res, tot))) { cudaFree(rhs); return r; }
        if ((r = vp_alloc(ctx, &f, tot))) { cudaFree(rhs); cudaFree(res); return r; }
        if ((r = vp_alloc(ctx, &fw, tot))) { cudaFree(rhs); cudaFree(res); cudaFree(f); return r; }
    }
    auto cleanup = [&]() {
        if (ws) return;
        cudaFree(rhs);
        cudaFree(res);
        cudaFree(f);
        cudaFree(fw);
    };
    VP_CUDA(ctx, cudaMemcpyAsync(rhs, x, sizeof(double) * tot, cudaMemcpyDeviceToDevice, ctx->stream));
    int g = std::min<int>(4 * ctx->nsm, int((tot + 255) / 256));
    convert_kernel<double, float><<<g, 256, 0, ctx->stream>>>(tot, rhs, f);
    ctx->launches++;
    if ((r = lu_solve<float>(ctx, F, F->LU32, d_perm, nrhs, f, fw, trans))) { cleanup(); return r; }
    convert_kernel<float, double><<<g, 256, 0, ctx->stream>>>(tot, f, x);
    ctx->launches++;
    const double one = 1.0, mone = -1.0;
    const cublasOperation_t op = trans ? CUBLAS_OP_T : CUBLAS_OP_N;
    std::vector<double> rn(nrhs), xn(nrhs);
    int it = 0;
    bool conv = false;
    double prev = INFINITY;
    for (it = 1; it <= 30; ++it) {
        VP_CUDA(ctx, cudaMemcpyAsync(res, rhs, sizeof(double) * tot, cudaMemcpyDeviceToDevice, ctx->stream));
        // a matrix-vector product per column: M is read once per column at the HBM rate (a GEMM with a few columns
        // takes a tile shape that reads it far slower)
        for (int k = 0; k < nrhs; ++k)
            VP_BLAS(ctx, cublasDgemv(ctx->blas, op, n, n, &mone, F->M, n, x + size_t(k) * n, 1, &one,
                                     res + size_t(k) * n, 1));
        // convergence: every column's residual at FP64 rounding of |M| |x|
        bool ok = true;
        double worst = 0;
        for (int k = 0; k < nrhs; ++k) {
            int ir, ix;
            cublasSetPointerMode(ctx->blas, CUBLAS_POINTER_MODE_HOST);
            VP_BLAS(ctx, cublasIdamax(ctx->blas, n, res + size_t(k) * n, 1, &ir));
            VP_BLAS(ctx, cublasIdamax(ctx->blas, n, x + size_t(k) * n, 1, &ix));
            double a, bx;
            VP_CUDA(ctx, vp_d2h(ctx, &a, res + size_t(k) * n + (ir - 1), sizeof(double)));
            VP_CUDA(ctx, vp_d2h(ctx, &bx, x + size_t(k) * n + (ix - 1), sizeof(double)));
            VP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
            double ratio = std::fabs(a) / (norm1 * std::fabs(bx) + 1e-300);
            worst = std::max(worst, ratio);
            if (ratio > 4 * std::sqrt(double(n)) * 1.1102230246251565e-16) ok = false;
        }
        if (ok) {
            conv = true;
            break;
        }
        if (it > 3 && worst > 0.5 * prev) break;  // stagnation
        prev = worst;
        convert_kernel<double, float><<<g, 256, 0, ctx->stream>>>(tot, res, f);
        ctx->launches++;
        if ((r = lu_solve<float>(ctx, F, F->LU32, d_perm, nrhs, f, fw, trans))) { cleanup(); return r; }
        axpy_f2d_kernel<<<g, 256, 0, ctx->stream>>>(tot, f, x);
        ctx->launches++;
    }
    cleanup();
    if (iters) *iters = it;
    if (!conv) {
        // stagnated at a level the FP32 factors cannot improve: accept when already tiny, else report
        return vp_fail(ctx, VP_ERR_NOCONV, "iterative refinement did not converge");
    }
    return VP_OK;
}

int vp_solve_dev(vp_ctx* ctx, const vp_factor* F, const double* d_b, double* d_x, SolveWork* w) {
    const int n = F->n;
    ctb_kernel<<<(n + 255) / 256, 256, 0, ctx->stream>>>(F->nq, n, F->nslot, 1, F->Ct_ptr, F->Ct_col, F->Ct_val, d_b, d_x);
    ctx->launches++;
    VP_CUDA(ctx, cudaGetLastError());
    return solve_core(ctx, F, 1, d_x, false, nullptr, w);
}

extern "C" int vp_solve(vp_ctx* ctx, const vp_factor* F, int nrhs, const double* b, double* q, double* lambda) {
    if (!ctx || !F || !b || !q || nrhs <= 0) return vp_fail(ctx, VP_ERR_ARG, "null argument");
    const int n = F->n, nq = F->nq, nb = F->nb, nslot = F->nslot;
    const size_t tot = size_t(n) * nrhs;
    int r;
    double *db, *x;
    if ((r = vp_alloc(ctx, &db, size_t(nslot) * nrhs))) return r;
    if ((r = vp_alloc(ctx, &x, tot))) { cudaFree(db); return r; }
    VP_CUDA(ctx, vp_h2d(ctx, db, b, sizeof(double) * size_t(nslot) * nrhs));
    ctb_kernel<<<int((tot + 255) / 256), 256, 0, ctx->stream>>>(nq, n, nslot, nrhs, F->Ct_ptr, F->Ct_col, F->Ct_val, db, x);
    ctx->launches++;
    vp_phase_begin(ctx, PH_SOLVE);
    r = solve_core(ctx, F, nrhs, x, false, nullptr);
    vp_phase_end(ctx);
    if (!r) {
        std::vector<double> hx(tot);
        vp_d2h(ctx, hx.data(), x, sizeof(double) * tot);
        cudaError_t e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) r = vp_fail(ctx, VP_ERR_CUDA, cudaGetErrorString(e));
        for (int k = 0; k < nrhs && !r; ++k) {
            for (int i = 0; i < nq; ++i) q[size_t(k) * nq + i] = hx[size_t(k) * n + i];
            if (lambda)
                for (int i = 0; i < nb; ++i) lambda[size_t(k) * nb + i] = F->h_se[i] * hx[size_t(k) * n + nq + i];
        }
    }
    cudaFree(db);
    cudaFree(x);
    return r;
}

// the adjoint's transposed solve: M' [xi; eta] = [g; 0]
extern "C" int vp_solve_transposed(vp_ctx* ctx, const vp_factor* F, int nrhs, const double* g, double* xi) {
    if (!ctx || !F || !g || !xi || nrhs <= 0) return vp_fail(ctx, VP_ERR_ARG, "null argument");
    if (cudaSetDevice(ctx->device) != cudaSuccess) return vp_fail(ctx, VP_ERR_CUDA, "cudaSetDevice");
    const int n = F->n, nq = F->nq;
    const size_t tot = size_t(n) * nrhs;
    std::vector<double> hx(tot, 0.0);
    for (int k = 0; k < nrhs; ++k)
        for (int i = 0; i < nq; ++i) hx[size_t(k) * n + i] = g[size_t(k) * nq + i];
    double* x;
    int r;
    if ((r = vp_upload(ctx, &x, hx.data(), tot))) return r;
    vp_phase_begin(ctx, PH_ADJ_SOLVE);
    r = solve_core(ctx, F, nrhs, x, true, nullptr);
    vp_phase_end(ctx);
    if (!r) {
        cudaError_t e = vp_d2h(ctx, hx.data(), x, sizeof(double) * tot);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) r = vp_fail(ctx, VP_ERR_CUDA, cudaGetErrorString(e));
        for (int k = 0; k < nrhs && !r; ++k)
            for (int i = 0; i < nq; ++i) xi[size_t(k) * nq + i] = hx[size_t(k) * n + i];
    }
    cudaFree(x);
    return r;
}

extern "C" int vp_solve_system(vp_ctx* ctx, const vp_factor* F, const vp_system* sys, double* q, double* lambda,
                               double* residual) {
    if (!ctx || !F || !sys) return vp_fail(ctx, VP_ERR_ARG, "null argument");
    if (sys->nslot != F->nslot) return vp_fail(ctx, VP_ERR_ARG, "system and factorization do not match");
    const int n = F->n, nq = F->nq, nb = F->nb;
    int r;
    double *x, *rhs;
    if ((r = vp_alloc(ctx, &x, size_t(n)))) return r;
    if ((r = vp_alloc(ctx, &rhs, size_t(n)))) { cudaFree(x); return r; }
    ctb_kernel<<<(n + 255) / 256, 256, 0, ctx->stream>>>(nq, n, F->nslot, 1, F->Ct_ptr, F->Ct_col, F->Ct_val, sys->b, x);
    ctx->launches++;
    VP_CUDA(ctx, cudaMemcpyAsync(rhs, x, sizeof(double) * n, cudaMemcpyDeviceToDevice, ctx->stream));
    vp_phase_begin(ctx, PH_SOLVE);
    r = solve_core(ctx, F, 1, x, false, nullptr);
    vp_phase_end(ctx);
    if (!r) {
        std::vector<double> hx(n);
        vp_d2h(ctx, hx.data(), x, sizeof(double) * n);
        if (residual) {
            double nr = 0, nrhs = 0;
            cublasDnrm2(ctx->blas, n, rhs, 1, &nrhs);
            const double one = 1.0, mone = -1.0;
            cublasDgemv(ctx->blas, CUBLAS_OP_N, n, n, &mone, F->M, n, x, 1, &one, rhs, 1);
            cublasDnrm2(ctx->blas, n, rhs, 1, &nr);
            *residual = nrhs > 0 ? nr / nrhs : nr;
        }
        cudaError_t e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) r = vp_fail(ctx, VP_ERR_CUDA, cudaGetErrorString(e));
        if (q)
            for (int i = 0; i < nq; ++i) q[i] = hx[i];
        if (lambda)
            for (int i = 0; i < nb; ++i) lambda[i] = F->h_se[i] * hx[nq + i];
    }
    cudaFree(x);
    cudaFree(rhs);
    return r;
}

extern "C" int vp_factor_info(const vp_factor* F, int* n, double* cond) {
    if (!F) return VP_ERR_ARG;
    if (n) *n = F->n;
    if (cond) *cond = F->cond;
    return VP_OK;
}

extern "C" void vp_factor_free(vp_factor* F) {
    if (!F) return;
    cudaFree(F->perm);
    cudaFree(F->M);
    cudaFree(F->LU64);
    cudaFree(F->LU32);
    cudaFree(F->ipiv);
    cudaFree(F->se);
    cudaFree(F->Ct_ptr);
    cudaFree(F->Ct_col);
    cudaFree(F->Ct_val);
    delete F;
}
