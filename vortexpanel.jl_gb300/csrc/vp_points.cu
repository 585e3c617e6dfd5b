// Point evaluation of the device kernels (diagnostics and tests): the source-triangle velocity, its reverse-mode
// derivatives with the shape chain rule, and the filament's, one thread per point.
#include "vp_adjoint_common.cuh"
#include "vp_internal.h"

#include <cuda.h>

#include <mutex>

namespace {

template <class T>
__device__ SrcKern<T> kern_of(const double* t, double* c_out) {
    double c[3] = {(t[0] + t[3] + t[6]) / 3, (t[1] + t[4] + t[7]) / 3, (t[2] + t[5] + t[8]) / 3};
    v3<double> v0 = mk3(t[0], t[1], t[2]), v1 = mk3(t[3], t[4], t[5]), v2 = mk3(t[6], t[7], t[8]);
    v3<double> nA = cross(v1 - v0, v2 - v0);
    double A2 = vnorm(nA);
    v3<double> n = nA / A2;
    v3<double> V[3] = {v0, v1, v2};
    SrcKern<T> S;
    double diam = 0;
    for (int e = 0; e < 3; ++e) {
        v3<double> ed = V[(e + 1) % 3] - V[e];
        double len = vnorm(ed);
        v3<double> nu = cross(ed, n) / len;
        S.nu[e] = mk3(T(nu.x), T(nu.y), T(nu.z));
        S.len[e] = T(len);
        diam = fmax(diam, len);
        S.d[e] = mk3(T(V[e].x - c[0]), T(V[e].y - c[1]), T(V[e].z - c[2]));
    }
    S.n = mk3(T(n.x), T(n.y), T(n.z));
    S.area = T(A2 / 2);
    S.diam = T(diam);
    for (int k = 0; k < 3; ++k) c_out[k] = c[k];
    return S;
}

template <class T>
__global__ void points_kernel(int mode, int n, const double* __restrict__ tri, const double* __restrict__ x,
                              const double* __restrict__ m, int side, double kfar, double* __restrict__ out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double* t = tri + 9 * i;
    const double* p = x + 3 * i;
    if (mode == 2) {  // filament a = t[0:3], b = t[3:6], ca = t[6], cb = t[7], n = m
        v3<T> ra = mk3(T(p[0] - t[0]), T(p[1] - t[1]), T(p[2] - t[2]));
        v3<T> rb = mk3(T(p[0] - t[3]), T(p[1] - t[4]), T(p[2] - t[5]));
        v3<T> nn = mk3(T(m[3 * i]), T(m[3 * i + 1]), T(m[3 * i + 2]));
        v3<T> ga, gb;
        T s = seg_vjp(ra, rb, nn, T(t[6]), T(t[7]), ga, gb);
        double* o = out + 10 * i;
        o[0] = double(s);
        v3<T> gx = ga + gb;
        o[1] = gx.x; o[2] = gx.y; o[3] = gx.z;
        o[4] = -ga.x; o[5] = -ga.y; o[6] = -ga.z;
        o[7] = -gb.x; o[8] = -gb.y; o[9] = -gb.z;
        return;
    }
    double c[3];
    SrcKern<T> S = kern_of<T>(t, c);
    v3<T> r = mk3(T(p[0] - c[0]), T(p[1] - c[1]), T(p[2] - c[2]));
    v3<T> r0 = mk3(T(p[0] - t[0]), T(p[1] - t[1]), T(p[2] - t[2]));
    v3<T> r1 = mk3(T(p[0] - t[3]), T(p[1] - t[4]), T(p[2] - t[5]));
    v3<T> r2 = mk3(T(p[0] - t[6]), T(p[1] - t[7]), T(p[2] - t[8]));
    T fd = T(kfar) * S.diam;
    bool far = dot(r, r) > fd * fd;
    if (mode == 0) {
        v3<T> w = far ? sv_far(S, r) : sv_exact3(S, r0, r1, r2, r, side, T(1e-12));
        out[3 * i] = w.x;
        out[3 * i + 1] = w.y;
        out[3 * i + 2] = w.z;
        return;
    }
    v3<T> mm = mk3(T(m[3 * i]), T(m[3 * i + 1]), T(m[3 * i + 2]));
    AdjSums<T> acc;
    adj_zero(acc);
    if (far)
        adj_point_far(acc, S, T(1), T(1), T(0), T(0), r, mm);
    else
        adj_point_exact(acc, S, T(1), T(1), T(0), T(0), r0, r1, r2, r, mm, side, T(1e-12));
    AdjSums<double> a;
    a.Q = mk3(double(acc.Q.x), double(acc.Q.y), double(acc.Q.z));
    a.Grf = mk3(double(acc.Grf.x), double(acc.Grf.y), double(acc.Grf.z));
    for (int k = 0; k < 3; ++k) {
        a.Xg[k] = mk3(double(acc.Xg[k].x), double(acc.Xg[k].y), double(acc.Xg[k].z));
        a.Gr[k] = mk3(double(acc.Gr[k].x), double(acc.Gr[k].y), double(acc.Gr[k].z));
        a.Gd[k] = mk3(double(acc.Gd[k].x), double(acc.Gd[k].y), double(acc.Gd[k].z));
        a.L[k] = acc.L[k];
        a.N[k] = acc.N[k];
    }
    a.O = acc.O;
    a.A = acc.A;
    double* o = out + 13 * i;
    v3<double> md = mk3(m[3 * i], m[3 * i + 1], m[3 * i + 2]);
    o[0] = dot(a.Q, md);
    o[1] = a.Xg[0].x; o[2] = a.Xg[0].y; o[3] = a.Xg[0].z;
    double gS[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    adj_source_shape(t, a, md, gS);
    for (int k = 0; k < 9; ++k) o[4 + k] = gS[k];
}

}  // namespace

extern "C" int vp_eval_points(vp_ctx* ctx, int mode, int precision, int n, const double* tri, const double* x,
                              const double* m, int side, double kernel_far, double* out) {
    if (!ctx || !tri || !x || !out || n <= 0 || mode < 0 || mode > 2) return vp_fail(ctx, VP_ERR_ARG, "bad argument");
    if (mode > 0 && !m) return vp_fail(ctx, VP_ERR_ARG, "m is needed");
    if (precision != VP_FP64 && precision != VP_MIXED) return vp_fail(ctx, VP_ERR_ARG, "precision must be VP_FP64 or VP_MIXED");
    DeviceGuard dg;
    if (dg.set(ctx->device) != cudaSuccess) return vp_fail(ctx, VP_ERR_CUDA, "cudaSetDevice");
    const int nout = mode == 0 ? 3 : (mode == 1 ? 13 : 10);
    double *dt, *dx, *dm = nullptr, *dout;
    int r;
    if ((r = vp_upload(ctx, &dt, tri, size_t(9) * n))) return r;
    if ((r = vp_upload(ctx, &dx, x, size_t(3) * n))) { cudaFree(dt); return r; }
    if (m && (r = vp_upload(ctx, &dm, m, size_t(3) * n))) { cudaFree(dt); cudaFree(dx); return r; }
    if ((r = vp_alloc(ctx, &dout, size_t(nout) * n))) { cudaFree(dt); cudaFree(dx); cudaFree(dm); return r; }
    if (precision == VP_FP64)
        points_kernel<double><<<(n + 127) / 128, 128, 0, ctx->stream>>>(mode, n, dt, dx, dm, side, kernel_far, dout);
    else
        points_kernel<float><<<(n + 127) / 128, 128, 0, ctx->stream>>>(mode, n, dt, dx, dm, side, kernel_far, dout);
    ctx->launches++;
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = vp_d2h(ctx, out, dout, sizeof(double) * nout * n);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    cudaFree(dt);
    cudaFree(dx);
    cudaFree(dm);
    cudaFree(dout);
    if (e != cudaSuccess) return vp_fail(ctx, VP_ERR_CUDA, std::string("vp_eval_points: ") + cudaGetErrorString(e));
    return VP_OK;
}

// ---------------------------------------------------------------------------------------------------------------------
// vp_eval_points_static: the same evaluation as vp_eval_points with no device allocation, for callers that cannot
// allocate while they run (a host whose device memory sits in its own pool, a loop that cannot afford the device
// synchronisation of cudaMalloc/cudaFree). Inputs and outputs are staged through one file-scope device array sized
// for VP_STATIC_POINTS_MAX points. Its address is looked up with cudaGetSymbolAddress on the first call for each device
// (with that device current), so that first call has to be made before any stream capture on the device; the address
// is kept with the id of the CUDA context it was looked up in and looked up again when the device's current context
// changes (after a cudaDeviceReset, say), because the array then lives at a new address. Calls that overlap in time on
// one device (from two streams or two host threads) share the array and race: the caller serialises them. No part of
// the array has to start at zero: points_kernel writes every output slot of the n points it is given, and the inputs
// are copied in before the launch. The caller's current device is restored on return.
namespace {

constexpr size_t kStaticTri = size_t(9) * VP_STATIC_POINTS_MAX;   // triangle (or filament) rows
constexpr size_t kStaticVec = size_t(3) * VP_STATIC_POINTS_MAX;   // x and m
constexpr size_t kStaticOut = size_t(13) * VP_STATIC_POINTS_MAX;  // widest output (mode 1)
// offsets in doubles; each block starts on a 256-byte boundary (VP_STATIC_POINTS_MAX is a multiple of 32)
constexpr size_t kOffX = kStaticTri, kOffM = kOffX + kStaticVec, kOffOut = kOffM + kStaticVec;
constexpr size_t kStaticDoubles = kOffOut + kStaticOut;
static_assert(VP_STATIC_POINTS_MAX % 32 == 0, "blocks must stay 256-byte aligned");

static __device__ __align__(256) double g_points_scratch[kStaticDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
double* g_scratch_addr[kMaxDevices] = {};
unsigned long long g_scratch_ctx_id[kMaxDevices] = {};

// the unique id of the calling thread's current CUDA context (cuCtxGetId, reached through the runtime's driver entry
// points so that the library needs no link to libcuda); 0 when it cannot be had
unsigned long long current_context_id() {
    typedef CUresult (*GetCurrent)(CUcontext*);
    typedef CUresult (*GetId)(CUcontext, unsigned long long*);
    static GetCurrent get_current = nullptr;
    static GetId get_id = nullptr;
    static bool resolved = false;
    if (!resolved) {  // called under g_scratch_mu
        cudaDriverEntryPointQueryResult q1, q2;
        void *a = nullptr, *b = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &a, 12000, cudaEnableDefault, &q1) == cudaSuccess &&
            q1 == cudaDriverEntryPointSuccess &&
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &b, 12000, cudaEnableDefault, &q2) == cudaSuccess &&
            q2 == cudaDriverEntryPointSuccess) {
            get_current = reinterpret_cast<GetCurrent>(a);
            get_id = reinterpret_cast<GetId>(b);
        }
        resolved = true;
    }
    CUcontext c = nullptr;
    unsigned long long id = 0;
    if (!get_current || !get_id || get_current(&c) != CUDA_SUCCESS || !c || get_id(c, &id) != CUDA_SUCCESS) return 0;
    return id;
}

}  // namespace

extern "C" int vp_eval_points_static(vp_ctx* ctx, int mode, int precision, int n, const double* tri, const double* x,
                                     const double* m, int side, double kernel_far, double* out) {
    if (!ctx || !tri || !x || !out || n <= 0 || mode < 0 || mode > 2) return vp_fail(ctx, VP_ERR_ARG, "bad argument");
    if (mode > 0 && !m) return vp_fail(ctx, VP_ERR_ARG, "m is needed");
    if (precision != VP_FP64 && precision != VP_MIXED) return vp_fail(ctx, VP_ERR_ARG, "precision must be VP_FP64 or VP_MIXED");
    if (n > VP_STATIC_POINTS_MAX)
        return vp_fail(ctx, VP_ERR_ARG, "vp_eval_points_static: n = " + std::to_string(n) + " is above " +
                                            std::to_string(VP_STATIC_POINTS_MAX));
    if (ctx->device < 0 || ctx->device >= kMaxDevices) return vp_fail(ctx, VP_ERR_ARG, "device index");
    DeviceGuard dg;
    if (dg.set(ctx->device) != cudaSuccess) return vp_fail(ctx, VP_ERR_CUDA, "cudaSetDevice");
    double* base;
    {
        std::lock_guard<std::mutex> lk(g_scratch_mu);
        const unsigned long long id = current_context_id();
        if (!g_scratch_addr[ctx->device] || id == 0 || id != g_scratch_ctx_id[ctx->device]) {
            void* p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_points_scratch);
            if (e != cudaSuccess)
                return vp_fail(ctx, VP_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
            g_scratch_addr[ctx->device] = static_cast<double*>(p);
            g_scratch_ctx_id[ctx->device] = id;
        }
        base = g_scratch_addr[ctx->device];
    }
    const int nout = mode == 0 ? 3 : (mode == 1 ? 13 : 10);
    double *dt = base, *dx = base + kOffX, *dm = m ? base + kOffM : nullptr, *dout = base + kOffOut;
    cudaError_t e = vp_h2d(ctx, dt, tri, sizeof(double) * 9 * size_t(n));
    if (e == cudaSuccess) e = vp_h2d(ctx, dx, x, sizeof(double) * 3 * size_t(n));
    if (e == cudaSuccess && m) e = vp_h2d(ctx, dm, m, sizeof(double) * 3 * size_t(n));
    if (e == cudaSuccess) {
        if (precision == VP_FP64)
            points_kernel<double><<<(n + 127) / 128, 128, 0, ctx->stream>>>(mode, n, dt, dx, dm, side, kernel_far, dout);
        else
            points_kernel<float><<<(n + 127) / 128, 128, 0, ctx->stream>>>(mode, n, dt, dx, dm, side, kernel_far, dout);
        ctx->launches++;
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = vp_d2h(ctx, out, dout, sizeof(double) * nout * size_t(n));
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess)
        return vp_fail(ctx, VP_ERR_CUDA, std::string("vp_eval_points_static: ") + cudaGetErrorString(e));
    return VP_OK;
}
