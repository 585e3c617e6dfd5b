// C-ABI entry points of libvortexpanel_gpu: contexts, errors, system handles (include/vortexpanel_gpu.h).
#include <cstring>

#include "vp_internal.h"

int vp_assemble_impl(vp_ctx* ctx, const vp_assembly_options* o, int nnode, const double* x, int ntri, const int* tris,
                     const int* corner_slot, int nslot, int ntouch, const int* touch_pairs, const double* sigma,
                     const double* vinf, int nwnode, const double* wx, int nwtri, const int* wtris, int nfil,
                     const int* fil, vp_system** out, vp_assembly_stats* stats, int body_sources);
int vp_assemble_batch_impl(vp_ctx* ctx, const vp_assembly_options* o, int nsys, const vp_assembly_input* in,
                           vp_system** out, vp_assembly_stats* stats);
int vp_adjoint_impl(vp_ctx* ctx, const vp_assembly_options* o, int nnode, const double* x, int ntri, const int* tris,
                    const int* corner_slot, int nslot, int ntouch, const int* touch_pairs, const double* sigma,
                    const double* vinf, int nwnode, const double* wx, int nwtri, const int* wtris, int nfil,
                    const int* fil, int nadj, const double* nu, const double* mu, const double* dvinf,
                    double* grad_x, double* grad_wx, double* dalpha, vp_assembly_stats* stats);

int vp_fail(vp_ctx* ctx, int code, const std::string& msg) {
    if (ctx) ctx->err = msg;
    return code;
}

int vp_phase_begin(vp_ctx* ctx, int ph) {
    cudaEvent_t a, b;
    if (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess)
        return vp_fail(ctx, VP_ERR_CUDA, "cudaEventCreate");
    cudaEventRecord(a, ctx->stream);
    ctx->pending.push_back({ph, {a, b}});
    return VP_OK;
}

int vp_phase_end(vp_ctx* ctx) {
    if (ctx->pending.empty()) return VP_OK;
    cudaEventRecord(ctx->pending.back().second.second, ctx->stream);
    return VP_OK;
}

void vp_phase_flush(vp_ctx* ctx) {
    for (auto& p : ctx->pending) {
        float ms = 0;
        if (cudaEventSynchronize(p.second.second) == cudaSuccess &&
            cudaEventElapsedTime(&ms, p.second.first, p.second.second) == cudaSuccess)
            ctx->phase_ms[p.first] += ms;
        cudaEventDestroy(p.second.first);
        cudaEventDestroy(p.second.second);
    }
    ctx->pending.clear();
}

extern "C" {

void vp_default_options(vp_assembly_options* o) {
    if (!o) return;
    o->test = 0;
    o->far_ratio = 3.0;
    o->far_points = 3;
    o->near_points = 7;
    o->near_ratio = 1.5;
    o->near_depth = 3;
    o->touch_levels = 6;
    o->touch_ratio = 0.15;
    o->touch_order = 3;
    o->corner_angle = 75.0;
    o->contact_rel = 0.1;
    o->kernel_far = 10.0;
    o->precision = VP_FP64;
}

int vp_ctx_create(int device, vp_ctx** out) {
    if (!out) return VP_ERR_ARG;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return VP_ERR_CUDA;
    if (device < 0 || device >= ndev) return VP_ERR_ARG;
    vp_ctx* c = new vp_ctx();
    c->device = device;
    if (cudaSetDevice(device) != cudaSuccess) {
        delete c;
        return VP_ERR_CUDA;
    }
    cudaDeviceGetAttribute(&c->nsm, cudaDevAttrMultiProcessorCount, device);
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete c;
        return VP_ERR_CUDA;
    }
    if (cublasCreate(&c->blas) != CUBLAS_STATUS_SUCCESS) {
        cudaStreamDestroy(c->stream);
        delete c;
        return VP_ERR_CUDA;
    }
    cublasSetStream(c->blas, c->stream);
    cublasSetMathMode(c->blas, CUBLAS_PEDANTIC_MATH);
    if (cudaMalloc(&c->d_flag, 64 * sizeof(int)) != cudaSuccess) {
        cublasDestroy(c->blas);
        cudaStreamDestroy(c->stream);
        delete c;
        return VP_ERR_NOMEM;
    }
    cudaMemset(c->d_flag, 0, 64 * sizeof(int));
    *out = c;
    return VP_OK;
}

void vp_ctx_destroy(vp_ctx* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    vp_phase_flush(ctx);
    if (ctx->d_flag) cudaFree(ctx->d_flag);
    vp_tc_work_free(&ctx->tc);
    if (ctx->blas) cublasDestroy(ctx->blas);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

const char* vp_last_error(const vp_ctx* ctx) { return ctx ? ctx->err.c_str() : "no context"; }

int vp_phase_times(vp_ctx* ctx, double* ms, int n, long long* launches, int reset) {
    if (!ctx) return VP_ERR_ARG;
    vp_phase_flush(ctx);
    for (int k = 0; k < n && k < PH_COUNT; ++k)
        if (ms) ms[k] = ctx->phase_ms[k];
    if (launches) *launches = ctx->launches;
    if (reset) {
        for (double& v : ctx->phase_ms) v = 0;
        ctx->launches = 0;
    }
    return VP_OK;
}

int vp_transfer_bytes(vp_ctx* ctx, long long* h2d, long long* d2h, int reset) {
    if (!ctx) return VP_ERR_ARG;
    if (h2d) *h2d = ctx->h2d_bytes;
    if (d2h) *d2h = ctx->d2h_bytes;
    if (reset) ctx->h2d_bytes = ctx->d2h_bytes = 0;
    return VP_OK;
}

int vp_assemble(vp_ctx* ctx, const vp_assembly_options* opts, int nnode, const double* x, int ntri, const int* tris,
                const int* corner_slot, int nslot, int ntouch, const int* touch_pairs, const double* sigma,
                const double* vinf, int nwnode, const double* wx, int nwtri, const int* wtris, int nfil,
                const int* fil, vp_system** out, vp_assembly_stats* stats) {
    if (!ctx) return VP_ERR_ARG;
    if (cudaSetDevice(ctx->device) != cudaSuccess) return vp_fail(ctx, VP_ERR_CUDA, "cudaSetDevice");
    return vp_assemble_impl(ctx, opts, nnode, x, ntri, tris, corner_slot, nslot, ntouch, touch_pairs, sigma, vinf,
                            nwnode, wx, nwtri, wtris, nfil, fil, out, stats, 1);
}

int vp_set_far_tile(vp_ctx* ctx, int precision, int tile) {
    if (!ctx) return VP_ERR_ARG;
    if (precision != VP_FP64 && precision != VP_MIXED) return vp_fail(ctx, VP_ERR_ARG, "unknown precision");
    const bool ok = precision == VP_MIXED ? (tile == 2 || tile == 4 || tile == 8) : (tile == 1 || tile == 2 || tile == 4);
    if (!ok)
        return vp_fail(ctx, VP_ERR_ARG, "far tile: 1, 2 or 4 test triangles in FP64, 2, 4 or 8 in mixed precision");
    ctx->far_tile[precision] = tile;
    return VP_OK;
}

int vp_get_far_tile(const vp_ctx* ctx, int precision) {
    if (!ctx || (precision != VP_FP64 && precision != VP_MIXED)) return 0;
    return ctx->far_tile[precision];
}

int vp_assemble_batch(vp_ctx* ctx, const vp_assembly_options* opts, int nsys, const vp_assembly_input* in,
                      vp_system** out, vp_assembly_stats* stats) {
    if (!ctx) return VP_ERR_ARG;
    if (cudaSetDevice(ctx->device) != cudaSuccess) return vp_fail(ctx, VP_ERR_CUDA, "cudaSetDevice");
    return vp_assemble_batch_impl(ctx, opts, nsys, in, out, stats);
}

int vp_adjoint(vp_ctx* ctx, const vp_assembly_options* opts, int nnode, const double* x, int ntri, const int* tris,
               const int* corner_slot, int nslot, int ntouch, const int* touch_pairs, const double* sigma,
               const double* vinf, int nwnode, const double* wx, int nwtri, const int* wtris, int nfil, const int* fil,
               int nadj, const double* nu, const double* mu, const double* dvinf, double* grad_x, double* grad_wx,
               double* dalpha, vp_assembly_stats* stats) {
    if (!ctx) return VP_ERR_ARG;
    if (cudaSetDevice(ctx->device) != cudaSuccess) return vp_fail(ctx, VP_ERR_CUDA, "cudaSetDevice");
    return vp_adjoint_impl(ctx, opts, nnode, x, ntri, tris, corner_slot, nslot, ntouch, touch_pairs, sigma, vinf,
                           nwnode, wx, nwtri, wtris, nfil, fil, nadj, nu, mu, dvinf, grad_x, grad_wx, dalpha, stats);
}

int vp_system_shape(const vp_system* sys, int* nrows, int* ncols) {
    if (!sys) return VP_ERR_ARG;
    if (nrows) *nrows = sys->nslot;
    if (ncols) *ncols = sys->ncols;
    return VP_OK;
}

int vp_system_download(vp_ctx* ctx, const vp_system* sys, double* A, double* b) {
    if (!ctx || !sys) return vp_fail(ctx, VP_ERR_ARG, "null argument");
    if (A)
        VP_CUDA(ctx, vp_d2h(ctx, A, sys->A, sizeof(double) * size_t(sys->nslot) * sys->ncols));
    if (b) VP_CUDA(ctx, vp_d2h(ctx, b, sys->b, sizeof(double) * sys->nslot));
    VP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return VP_OK;
}

int vp_system_download_rows(vp_ctx* ctx, const vp_system* sys, int r0, int r1, double* A, double* b) {
    if (!ctx || !sys) return vp_fail(ctx, VP_ERR_ARG, "null argument");
    if (r0 < 0 || r1 > sys->nslot || r0 > r1) return vp_fail(ctx, VP_ERR_ARG, "rows out of range");
    if (r0 == r1) return VP_OK;
    if (A)
        VP_CUDA(ctx, vp_d2h(ctx, A, sys->A + size_t(r0) * sys->ncols, sizeof(double) * size_t(r1 - r0) * sys->ncols));
    if (b) VP_CUDA(ctx, vp_d2h(ctx, b, sys->b + r0, sizeof(double) * (r1 - r0)));
    VP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return VP_OK;
}

void vp_system_free(vp_system* sys) {
    if (!sys) return;
    if (sys->A) cudaFree(sys->A);
    if (sys->b) cudaFree(sys->b);
    delete sys;
}

}  // extern "C"
