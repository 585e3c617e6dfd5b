// Internal types of libvortexpanel_gpu: the context, the resident system and factorization, error handling.
#pragma once
#include <cublas_v2.h>
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/vortexpanel_gpu.h"

// phases timed with CUDA events on the context's stream (vp_phase_times)
enum {
    PH_SETUP = 0,   // element data and tile uploads
    PH_CLASSIFY,    // non-far source lists
    PH_FAR,         // far tier tile kernel
    PH_NEAR,        // near, touching and contact tiers
    PH_REDUCE,      // C' A [C; W] and the border
    PH_LU,          // LU factorization
    PH_COND,        // condition estimate
    PH_SOLVE,       // triangular solves and refinement
    PH_ADJOINT,     // adjoint: element data, classification and the node derivatives (finish)
    PH_ADJ_FAR,     // adjoint far tier
    PH_ADJ_NEAR,    // adjoint non-far pairs, filaments, freestream
    PH_ADJ_SOLVE,   // transposed solve
    PH_WAKE,        // free wake: blob sums, body velocity, explicit right hand side of particles
    PH_NEAR_PAIRS,  // near_kernel_pairs alone (the touching and contact pairs of the assembly)
    PH_ADJ_PAIRS,   // adj_pairs_kernel alone (the touching and contact pairs of the adjoint)
    PH_WAKE_RHS,    // free wake simulation: the explicit right hand side kernels
    PH_WAKE_VEL,    // free wake simulation: the body and blob velocities at the wake points
    PH_COUNT
};

// buffers of the tensor-core GEMM of the LU's trailing updates (vp_tcgemm.cu): the bf16 pieces of its operands,
// grown to the largest update seen, and its error word
struct TcWork {
    void* pieces = nullptr;  // bf16 elements
    size_t cap = 0;          // elements
    int* err = nullptr;
    bool attr_set = false;
};

struct vp_ctx {
    int device = 0;
    int nsm = 0;
    cudaStream_t stream = nullptr;
    cublasHandle_t blas = nullptr;
    std::string err;
    int* d_flag = nullptr;  // device error word of bounded waits and checks
    // instrumentation: per-phase device time (ms, cumulative) and launches of this library's kernels
    double phase_ms[PH_COUNT] = {};
    long long launches = 0;
    long long h2d_bytes = 0, d2h_bytes = 0;  // host<->device copies made by the library
    std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> pending;
    TcWork tc;
    // test triangles per far-tier tile, per precision (vp_precision): set by vp_set_far_tile (the autotuner's choice)
    int far_tile[2] = {4, 8};
};

// record the start/end of a phase on the context's stream; vp_phase_flush() accumulates the elapsed times
int vp_phase_begin(vp_ctx* ctx, int ph);
int vp_phase_end(vp_ctx* ctx);
void vp_phase_flush(vp_ctx* ctx);

// Element data of one triangle in FP64 (the FlatTriangle / SourceTriangle fields the kernels read).
struct TriGeo {
    double x[9];    // corners
    double n[3];    // unit normal
    double c[3];    // centroid
    double area, diam, reach;
    double gam[9];  // vortex sheet of a unit nodal value at each corner, gamma_b = -e_b / 2A
    double nu[9];   // in-plane outward unit normals of the edges (edge a from corner a to a+1)
    double len[3];  // edge lengths
    double sigma;   // source strength (0 for wake sheets)
    int node[3];    // corner nodes (for shared-corner tests)
    int slot[3];    // corner slots (body) or wake-node columns
};

struct vp_system {
    int nslot = 0, ncols = 0, nwnode = 0;
    double* A = nullptr;  // nslot x ncols, row-major
    double* b = nullptr;  // nslot
};

struct vp_factor {
    int n = 0, nq = 0, nb = 0, nslot = 0, ncols = 0, precision = 0;
    double cond = 0;
    double* M = nullptr;     // bordered matrix, FP64, column-major n x n (kept for FP64 residuals)
    double* LU64 = nullptr;  // FP64 factors (column-major n x n) for VP_FP64
    float* LU32 = nullptr;   // FP32 factors (column-major n x n) for VP_MIXED
    int* ipiv = nullptr;     // device pivots (row swapped with at each step), n
    std::vector<int> h_ipiv;
    int* perm = nullptr;     // device permutation: row of M in position i of the factors
    double norm1 = 0;        // 1-norm of M
    double* se = nullptr;    // border column scales (device, nb)
    std::vector<double> h_se;
    // C' as CSR over unknowns (nq x nslot) for the right hand side, on the device
    int *Ct_ptr = nullptr, *Ct_col = nullptr;
    double* Ct_val = nullptr;
};

int vp_fail(vp_ctx* ctx, int code, const std::string& msg);

// Makes a context's device current for the length of a call and gives the caller's current device back on return.
struct DeviceGuard {
    int prev = -1;
    cudaError_t set(int device) {
        cudaError_t e = cudaGetDevice(&prev);
        if (e != cudaSuccess) {
            prev = -1;
            return e;
        }
        return prev == device ? cudaSuccess : cudaSetDevice(device);
    }
    ~DeviceGuard() {
        int cur = -1;
        if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
    }
};

#define VP_CUDA(ctx, call)                                                                            \
    do {                                                                                              \
        cudaError_t e_ = (call);                                                                      \
        if (e_ != cudaSuccess)                                                                        \
            return vp_fail((ctx), VP_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));   \
    } while (0)

#define VP_BLAS(ctx, call)                                                                            \
    do {                                                                                              \
        cublasStatus_t s_ = (call);                                                                   \
        if (s_ != CUBLAS_STATUS_SUCCESS)                                                              \
            return vp_fail((ctx), VP_ERR_CUDA, std::string(#call) + ": cublas status " + std::to_string(int(s_))); \
    } while (0)

template <class T>
int vp_alloc(vp_ctx* ctx, T** p, size_t n) {
    *p = nullptr;
    if (n == 0) n = 1;
    cudaError_t e = cudaMalloc((void**)p, n * sizeof(T));
    if (e != cudaSuccess) {
        *p = nullptr;
        return vp_fail(ctx, VP_ERR_NOMEM, std::string("cudaMalloc of ") + std::to_string(n * sizeof(T)) + " bytes: " +
                                              cudaGetErrorString(e));
    }
    return VP_OK;
}

template <class T>
int vp_upload(vp_ctx* ctx, T** p, const T* h, size_t n) {
    int r = vp_alloc(ctx, p, n);
    if (r) return r;
    if (n) VP_CUDA(ctx, cudaMemcpyAsync(*p, h, n * sizeof(T), cudaMemcpyHostToDevice, ctx->stream));
    ctx->h2d_bytes += (long long)(n * sizeof(T));
    return VP_OK;
}

// counted copies between host and device on the context's stream
inline cudaError_t vp_h2d(vp_ctx* ctx, void* d, const void* h, size_t bytes) {
    ctx->h2d_bytes += (long long)bytes;
    return cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, ctx->stream);
}
inline cudaError_t vp_d2h(vp_ctx* ctx, void* h, const void* d, size_t bytes) {
    ctx->d2h_bytes += (long long)bytes;
    return cudaMemcpyAsync(h, d, bytes, cudaMemcpyDeviceToHost, ctx->stream);
}

// linear algebra (vp_linalg.cu)
int vp_lu_factor(vp_ctx* ctx, int precision, int n, double* M64, vp_factor* F);

// Device buffers of one right hand side's solve, allocated once by a caller that solves repeatedly (the free wake's
// steps): vp_solve_work_alloc sizes them for the factorization, vp_solve_work_free releases them.
struct SolveWork {
    int n = 0;
    double *work64 = nullptr, *rhs = nullptr, *res = nullptr;
    float *f = nullptr, *fw = nullptr;
};
int vp_solve_work_alloc(vp_ctx* ctx, const vp_factor* F, SolveWork* w);
void vp_solve_work_free(SolveWork* w);
// solve_galerkin(F, b) for one right hand side on the device, with no allocation: b (nslot, device) -> x (n, device:
// q, then the border unknowns); lambda_k = se_k x[nq + k]. Stream-ordered on the context's stream; the mixed path's
// refinement reads its residual norms back to the host.
int vp_solve_dev(vp_ctx* ctx, const vp_factor* F, const double* d_b, double* d_x, SolveWork* w);

// the tensor-core GEMM (vp_tcgemm.cu): C -= A B, FP32 column-major, as three-piece bf16 splits with six tcgen05
// products accumulated in FP32 in TMEM; stream-ordered, errors of its bounded waits read by vp_tc_gemm_check
bool vp_tc_gemm_enabled();
bool vp_tc_gemm_fits(int m, int n, int k);
int vp_tc_gemm_sub(vp_ctx* ctx, int m, int n, int k, const float* A, int lda, const float* B, int ldb, float* C,
                   int ldc);
int vp_tc_gemm_check(vp_ctx* ctx);
void vp_tc_work_free(TcWork* w);

// post-processing (vp_post.cu): u, cp and the summed force and moment of the gradient route on device data, launched
// without a synchronisation; d_part: 6 doubles per 256 triangles, d_out6: F then M
int vp_post_surface_launch(vp_ctx* ctx, int ntri, const double* d_corners, const int* d_slot, const double* d_mu,
                           const double* d_dmudt, const double* vinf, const double* origin, double* d_u, double* d_cp,
                           double* d_part, double* d_out6);
