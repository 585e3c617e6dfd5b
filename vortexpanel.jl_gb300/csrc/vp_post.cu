// The reductions that follow a solve, on the GPU in FP64, each summed in a fixed order (bit-reproducible):
//   vp_consistency    <- Assembly.consistency(dm, A, b; W)                   src/assembly/solve.jl:111-115
//                        row and column sums of A [C; W] against its infinity norm, and the sum of b;
//   vp_surface_loads  <- Post.gradient_velocity, pressure_coefficient        src/post/Post.jl:72-84
//                        and Forces.pressure_force                           src/post/forces.jl:11-20
//                        u = V - (V.n)n + grad mu per triangle, Cp (with the element mean of dmu/dt when given), and the
//                        force and moment -sum Cp A n, sum (c - o) x (-Cp A n);
//   vp_wake_loads     <- Forces.kutta_joukowski_force, trefftz_drag         src/post/forces.jl:34-39,53-81
//                        (2/|V|^2) V x sum (mu_a + mu_b)/2 (x_b - x_a) along the trailing edge lines, and the induced
//                        drag of the strips' midpoint normalwash in the Trefftz plane.
// A is read once per pass (HBM-bound); the loads are O(n) (surface) and O(nte^2) (Trefftz).
#include <cmath>
#include <string>
#include <vector>

#include "vp_internal.h"

namespace {

constexpr int RB = 256;  // threads of the reduction blocks

// sum of v over the block in a fixed order (warp trees, then the warps' sums by warp 0); every thread gets it
__device__ double block_sum(double v, double* sh) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    if (lane == 0) sh[w] = v;
    __syncthreads();
    if (w == 0) {
        v = lane < int(blockDim.x >> 5) ? sh[lane] : 0.0;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) sh[32] = v;
    }
    __syncthreads();
    return sh[32];
}

__device__ double block_max(double v, double* sh) {
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    if (lane == 0) sh[w] = v;
    __syncthreads();
    if (w == 0) {
        v = lane < int(blockDim.x >> 5) ? sh[lane] : 0.0;
        for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
        if (lane == 0) sh[32] = v;
    }
    __syncthreads();
    return sh[32];
}

// ---- consistency ----------------------------------------------------------------------------------------------------

// one block per row i of A: (A Cf)_iq = sum over the column list of q of A[i, k] Cf[k, q]; the row's sum and |.|-sum
__global__ void __launch_bounds__(RB) cons_rows_kernel(const double* __restrict__ A, long long lda, int nq,
                                                       const int* __restrict__ cp, const int* __restrict__ ci,
                                                       const double* __restrict__ cv, double* __restrict__ rowsum,
                                                       double* __restrict__ rowabs) {
    __shared__ double sh[33];
    const double* Ai = A + size_t(blockIdx.x) * lda;
    double s = 0.0, a = 0.0;
    for (int q = threadIdx.x; q < nq; q += RB) {
        double v = 0.0;
        for (int p = cp[q]; p < cp[q + 1]; ++p) v += Ai[ci[p]] * cv[p];
        s += v;
        a += fabs(v);
    }
    s = block_sum(s, sh);
    a = block_sum(a, sh);
    if (threadIdx.x == 0) {
        rowsum[blockIdx.x] = s;
        rowabs[blockIdx.x] = a;
    }
}

// partial column sums of A over row chunks: part[chunk][j] (coalesced along the row)
__global__ void __launch_bounds__(RB) cons_colpart_kernel(const double* __restrict__ A, long long lda, int nrow,
                                                          int ncol, int rows_per_chunk, double* __restrict__ part) {
    const int j = blockIdx.x * RB + threadIdx.x;
    if (j >= ncol) return;
    const int r0 = blockIdx.y * rows_per_chunk, r1 = min(nrow, r0 + rows_per_chunk);
    double s = 0.0;
    for (int i = r0; i < r1; ++i) s += A[size_t(i) * lda + j];
    part[size_t(blockIdx.y) * ncol + j] = s;
}

// the column sums of A (the chunks in order), then of A Cf: colsum_q = sum_k s_k Cf[k, q]
__global__ void __launch_bounds__(RB) cons_cols_kernel(const double* __restrict__ part, int nchunk, int ncol,
                                                       double* __restrict__ s) {
    const int j = blockIdx.x * RB + threadIdx.x;
    if (j >= ncol) return;
    double v = 0.0;
    for (int c = 0; c < nchunk; ++c) v += part[size_t(c) * ncol + j];
    s[j] = v;
}

// out: max |row sum|, max row |.|-sum, max |column sum| of A Cf, sum b, sum |b|
__global__ void __launch_bounds__(1024) cons_final_kernel(int nrow, const double* __restrict__ rowsum,
                                                          const double* __restrict__ rowabs, int nq,
                                                          const int* __restrict__ cp, const int* __restrict__ ci,
                                                          const double* __restrict__ cv, const double* __restrict__ s,
                                                          const double* __restrict__ b, double* __restrict__ out) {
    __shared__ double sh[33];
    double mr = 0.0, ma = 0.0, mc = 0.0, sb = 0.0, ab = 0.0;
    for (int i = threadIdx.x; i < nrow; i += blockDim.x) {
        mr = fmax(mr, fabs(rowsum[i]));
        ma = fmax(ma, rowabs[i]);
        sb += b[i];
        ab += fabs(b[i]);
    }
    for (int q = threadIdx.x; q < nq; q += blockDim.x) {
        double v = 0.0;
        for (int p = cp[q]; p < cp[q + 1]; ++p) v += s[ci[p]] * cv[p];
        mc = fmax(mc, fabs(v));
    }
    mr = block_max(mr, sh);
    ma = block_max(ma, sh);
    mc = block_max(mc, sh);
    sb = block_sum(sb, sh);
    ab = block_sum(ab, sh);
    if (threadIdx.x == 0) {
        out[0] = mr;
        out[1] = ma;
        out[2] = mc;
        out[3] = sb;
        out[4] = ab;
    }
}

// ---- surface loads --------------------------------------------------------------------------------------------------

struct SurfArgs {
    int ntri;
    const double* corners;   // ntri x 9
    const int* slot;         // ntri x 3
    const double* mu;        // nslot, or null when cp_in is given
    const double* dmudt;     // nslot or null
    const double* cp_in;     // ntri or null: the pressure coefficient is given
    double V[3], o[3], V2;
    double* u_out;           // ntri x 3 or null
    double* cp_out;          // ntri or null
    double* part;            // gridDim.x x 6: the blocks' sums of F and M
};

// one thread per triangle; F and M summed per block in a fixed order
__global__ void __launch_bounds__(RB) surface_kernel(SurfArgs a) {
    __shared__ double sh[33];
    const int t = blockIdx.x * RB + threadIdx.x;
    double f[6] = {0, 0, 0, 0, 0, 0};
    if (t < a.ntri) {
        const double* c = a.corners + 9 * size_t(t);
        const double e1[3] = {c[3] - c[0], c[4] - c[1], c[5] - c[2]}, e2[3] = {c[6] - c[0], c[7] - c[1], c[8] - c[2]};
        const double nA[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
        const double A2 = sqrt(nA[0] * nA[0] + nA[1] * nA[1] + nA[2] * nA[2]);
        const double n[3] = {nA[0] / A2, nA[1] / A2, nA[2] / A2};
        double cp;
        if (a.cp_in) {
            cp = a.cp_in[t];
        } else {
            // grad mu = sum_k mu_k n x e_k / (2A), e_k the edge opposite corner k (e_0 = c - b, e_1 = a - c, e_2 = b - a)
            const int* sl = a.slot + 3 * size_t(t);
            const double m0 = a.mu[sl[0]], m1 = a.mu[sl[1]], m2 = a.mu[sl[2]];
            double G[3];
            for (int z = 0; z < 3; ++z)
                G[z] = (m0 * (c[6 + z] - c[3 + z]) + m1 * (c[z] - c[6 + z]) + m2 * (c[3 + z] - c[z])) / A2;
            const double g[3] = {n[1] * G[2] - n[2] * G[1], n[2] * G[0] - n[0] * G[2], n[0] * G[1] - n[1] * G[0]};
            const double Vn = a.V[0] * n[0] + a.V[1] * n[1] + a.V[2] * n[2];
            double u[3], uu = 0.0;
            for (int z = 0; z < 3; ++z) {
                u[z] = a.V[z] - Vn * n[z] + g[z];
                uu += u[z] * u[z];
            }
            double s = uu;
            if (a.dmudt) s += 2.0 * ((a.dmudt[sl[0]] + a.dmudt[sl[1]] + a.dmudt[sl[2]]) / 3.0);
            cp = 1.0 - s / a.V2;
            if (a.u_out)
                for (int z = 0; z < 3; ++z) a.u_out[3 * size_t(t) + z] = u[z];
            if (a.cp_out) a.cp_out[t] = cp;
        }
        const double w = -cp * (A2 / 2);
        const double fv[3] = {w * n[0], w * n[1], w * n[2]};
        const double r[3] = {(c[0] + c[3] + c[6]) / 3 - a.o[0], (c[1] + c[4] + c[7]) / 3 - a.o[1],
                             (c[2] + c[5] + c[8]) / 3 - a.o[2]};
        f[0] = fv[0];
        f[1] = fv[1];
        f[2] = fv[2];
        f[3] = r[1] * fv[2] - r[2] * fv[1];
        f[4] = r[2] * fv[0] - r[0] * fv[2];
        f[5] = r[0] * fv[1] - r[1] * fv[0];
    }
    for (int k = 0; k < 6; ++k) {
        const double v = block_sum(f[k], sh);
        if (threadIdx.x == 0) a.part[6 * size_t(blockIdx.x) + k] = v;
    }
}

// the blocks' partial sums in block order
__global__ void __launch_bounds__(32) sum_parts_kernel(int nblock, int width, const double* __restrict__ part,
                                                       double* __restrict__ out) {
    const int k = threadIdx.x;
    if (k >= width) return;
    double v = 0.0;
    for (int i = 0; i < nblock; ++i) v += part[size_t(i) * width + k];
    out[k] = v;
}

// ---- wake loads -----------------------------------------------------------------------------------------------------

struct WakeArgs {
    int nseg, nvort;
    const double* x;       // nte x 3
    const double* mu;      // nte
    const int* seg;        // nseg x 2 (a, b)
    const int* vort;       // nvort x 3 (node, before segment or -1, after segment or -1)
    double V[3], d[3];
    double* part;          // nseg: each strip's drag term; then [nseg .. nseg + 3): the circulation vector G
};

__device__ __forceinline__ void proj(const double* x, const double* d, double* p) {
    const double s = x[0] * d[0] + x[1] * d[1] + x[2] * d[2];
    p[0] = x[0] - s * d[0];
    p[1] = x[1] - s * d[1];
    p[2] = x[2] - s * d[2];
}

// one block per strip k: its normalwash at the middle from every trailing vortex (threads over vortices), then
// Gamma_k (n.v) l. Block nseg sums the Kutta-Joukowski circulation vector in segment order.
__global__ void __launch_bounds__(RB) trefftz_kernel(WakeArgs a) {
    __shared__ double sh[33];
    const int k = blockIdx.x;
    if (k == a.nseg) {
        if (threadIdx.x == 0) {
            double G[3] = {0, 0, 0};
            for (int s = 0; s < a.nseg; ++s) {
                const int ia = a.seg[2 * s], ib = a.seg[2 * s + 1];
                const double g = (a.mu[ia] + a.mu[ib]) / 2;
                for (int z = 0; z < 3; ++z) G[z] += g * (a.x[3 * ib + z] - a.x[3 * ia + z]);
            }
            for (int z = 0; z < 3; ++z) a.part[a.nseg + z] = G[z];
        }
        return;
    }
    const int ia = a.seg[2 * k], ib = a.seg[2 * k + 1];
    double pa[3], pb[3];
    proj(a.x + 3 * ia, a.d, pa);
    proj(a.x + 3 * ib, a.d, pb);
    const double c[3] = {(pa[0] + pb[0]) / 2, (pa[1] + pb[1]) / 2, (pa[2] + pb[2]) / 2};
    const double e[3] = {pb[0] - pa[0], pb[1] - pa[1], pb[2] - pa[2]};
    const double l = sqrt(e[0] * e[0] + e[1] * e[1] + e[2] * e[2]);
    const double t[3] = {e[0] / l, e[1] / l, e[2] / l};
    const double n[3] = {a.d[1] * t[2] - a.d[2] * t[1], a.d[2] * t[0] - a.d[0] * t[2], a.d[0] * t[1] - a.d[1] * t[0]};
    double v[3] = {0, 0, 0};
    const double i4pi = 1.0 / (4.0 * M_PI);
    for (int p = threadIdx.x; p < a.nvort; p += RB) {
        const int node = a.vort[3 * p], sb = a.vort[3 * p + 1], sa = a.vort[3 * p + 2];
        const double Gb = sb >= 0 ? (a.mu[a.seg[2 * sb]] + a.mu[a.seg[2 * sb + 1]]) / 2 : 0.0;
        const double Ga = sa >= 0 ? (a.mu[a.seg[2 * sa]] + a.mu[a.seg[2 * sa + 1]]) / 2 : 0.0;
        double pp[3];
        proj(a.x + 3 * node, a.d, pp);
        const double r[3] = {c[0] - pp[0], c[1] - pp[1], c[2] - pp[2]};
        const double r2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
        const double s = (Ga - Gb) * i4pi / r2;
        v[0] += s * (a.d[1] * r[2] - a.d[2] * r[1]);
        v[1] += s * (a.d[2] * r[0] - a.d[0] * r[2]);
        v[2] += s * (a.d[0] * r[1] - a.d[1] * r[0]);
    }
    const double vn = block_sum(n[0] * v[0] + n[1] * v[1] + n[2] * v[2], sh);
    if (threadIdx.x == 0) a.part[k] = (a.mu[ia] + a.mu[ib]) / 2 * vn * l;
}

// device buffers freed on scope exit
struct Bufs {
    std::vector<void*> p;
    ~Bufs() {
        for (void* q : p) cudaFree(q);
    }
    template <class T>
    int alloc(vp_ctx* ctx, T** d, size_t n) {
        int r = vp_alloc(ctx, d, n);
        if (!r) p.push_back((void*)*d);
        return r;
    }
    template <class T>
    int up(vp_ctx* ctx, T** d, const T* h, size_t n) {
        int r = vp_upload(ctx, d, h, n);
        if (!r) p.push_back((void*)*d);
        return r;
    }
};

// CSR of Cf' (nq rows over the ncols = nslot + nwake columns of A) from C (nslot x nq) and W (nwake x nq)
void transpose_cf(int nslot, int nq, const int* Cp, const int* Ci, const double* Cv, int nwake, const int* Wp,
                  const int* Wi, const double* Wv, std::vector<int>& tp, std::vector<int>& ti, std::vector<double>& tv) {
    tp.assign(nq + 1, 0);
    for (int k = 0; k < nslot; ++k)
        for (int p = Cp[k]; p < Cp[k + 1]; ++p) tp[Ci[p] + 1]++;
    for (int k = 0; k < nwake; ++k)
        for (int p = Wp[k]; p < Wp[k + 1]; ++p) tp[Wi[p] + 1]++;
    for (int q = 0; q < nq; ++q) tp[q + 1] += tp[q];
    ti.assign(std::max(tp[nq], 1), 0);
    tv.assign(std::max(tp[nq], 1), 0.0);
    std::vector<int> fill(tp.begin(), tp.end() - 1);
    for (int k = 0; k < nslot; ++k)
        for (int p = Cp[k]; p < Cp[k + 1]; ++p) {
            ti[fill[Ci[p]]] = k;
            tv[fill[Ci[p]]++] = Cv[p];
        }
    for (int k = 0; k < nwake; ++k)
        for (int p = Wp[k]; p < Wp[k + 1]; ++p) {
            ti[fill[Wi[p]]] = nslot + k;
            tv[fill[Wi[p]]++] = Wv[p];
        }
}

bool csr_ok(int nrow, int ncol, const int* p, const int* i) {
    if (!p || p[0] != 0) return false;
    for (int r = 0; r < nrow; ++r)
        if (p[r + 1] < p[r]) return false;
    for (int k = 0; k < p[nrow]; ++k)
        if (!i || i[k] < 0 || i[k] >= ncol) return false;
    return true;
}

}  // namespace

extern "C" int vp_consistency(vp_ctx* ctx, const vp_system* sys, int nq, const int* C_rowptr, const int* C_col,
                              const double* C_val, int nwake, const int* W_rowptr, const int* W_col,
                              const double* W_val, double* out) {
    if (!ctx || !sys || !out || nq <= 0 || nwake < 0 || !C_val) return vp_fail(ctx, VP_ERR_ARG, "bad argument");
    if (sys->ncols != sys->nslot + nwake)
        return vp_fail(ctx, VP_ERR_ARG, "A has " + std::to_string(sys->ncols) + " columns, expected nslot + nwake = " +
                                            std::to_string(sys->nslot + nwake));
    if (!csr_ok(sys->nslot, nq, C_rowptr, C_col) || (nwake > 0 && (!csr_ok(nwake, nq, W_rowptr, W_col) || !W_val)))
        return vp_fail(ctx, VP_ERR_ARG, "C or W is not a valid CSR matrix over nq columns");
    DeviceGuard dg;
    if (dg.set(ctx->device) != cudaSuccess) return vp_fail(ctx, VP_ERR_CUDA, "cudaSetDevice");
    std::vector<int> tp, ti;
    std::vector<double> tv;
    transpose_cf(sys->nslot, nq, C_rowptr, C_col, C_val, nwake, W_rowptr, W_col, W_val, tp, ti, tv);
    const int nrow = sys->nslot, ncol = sys->ncols;
    const int nchunk = std::min(64, std::max(1, nrow / 64)), rpc = (nrow + nchunk - 1) / nchunk;
    Bufs B;
    int *dp, *di;
    double *dv, *rs, *ra, *part, *s, *dout;
    int r;
    if ((r = B.up(ctx, &dp, tp.data(), tp.size())) || (r = B.up(ctx, &di, ti.data(), ti.size())) ||
        (r = B.up(ctx, &dv, tv.data(), tv.size())) || (r = B.alloc(ctx, &rs, size_t(nrow))) ||
        (r = B.alloc(ctx, &ra, size_t(nrow))) || (r = B.alloc(ctx, &part, size_t(nchunk) * ncol)) ||
        (r = B.alloc(ctx, &s, size_t(ncol))) || (r = B.alloc(ctx, &dout, 5)))
        return r;
    cons_rows_kernel<<<nrow, RB, 0, ctx->stream>>>(sys->A, sys->ncols, nq, dp, di, dv, rs, ra);
    cons_colpart_kernel<<<dim3((ncol + RB - 1) / RB, nchunk), RB, 0, ctx->stream>>>(sys->A, sys->ncols, nrow, ncol, rpc,
                                                                                    part);
    cons_cols_kernel<<<(ncol + RB - 1) / RB, RB, 0, ctx->stream>>>(part, nchunk, ncol, s);
    cons_final_kernel<<<1, 1024, 0, ctx->stream>>>(nrow, rs, ra, nq, dp, di, dv, s, sys->b, dout);
    ctx->launches += 4;
    VP_CUDA(ctx, cudaGetLastError());
    double h[5];
    VP_CUDA(ctx, vp_d2h(ctx, h, dout, sizeof(h)));
    VP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    out[0] = h[1] > 0 ? h[0] / h[1] : 0.0;
    out[1] = h[1] > 0 ? h[2] / h[1] : 0.0;
    out[2] = h[4] > 0 ? fabs(h[3]) / h[4] : 0.0;
    return VP_OK;
}

// the gradient route's surface kernel and the ordered sum of its blocks on device data, launched on the context's
// stream without a synchronisation (the free wake's loads); d_part holds 6 doubles per block of 256 triangles
int vp_post_surface_launch(vp_ctx* ctx, int ntri, const double* d_corners, const int* d_slot, const double* d_mu,
                           const double* d_dmudt, const double* vinf, const double* origin, double* d_u, double* d_cp,
                           double* d_part, double* d_out6) {
    const int nb = std::max(1, (ntri + RB - 1) / RB);
    SurfArgs a{};
    a.ntri = ntri;
    a.corners = d_corners;
    a.slot = d_slot;
    a.mu = d_mu;
    a.dmudt = d_dmudt;
    a.cp_in = nullptr;
    for (int z = 0; z < 3; ++z) {
        a.V[z] = vinf[z];
        a.o[z] = origin ? origin[z] : 0.0;
    }
    a.V2 = a.V[0] * a.V[0] + a.V[1] * a.V[1] + a.V[2] * a.V[2];
    a.u_out = d_u;
    a.cp_out = d_cp;
    a.part = d_part;
    surface_kernel<<<nb, RB, 0, ctx->stream>>>(a);
    sum_parts_kernel<<<1, 32, 0, ctx->stream>>>(nb, 6, d_part, d_out6);
    ctx->launches += 2;
    VP_CUDA(ctx, cudaGetLastError());
    return VP_OK;
}

static int surface_common(vp_ctx* ctx, int ntri, const double* corners, const int* corner_slot, int nslot,
                          const double* mu, const double* dmudt, const double* cp_in, const double* vinf,
                          const double* origin, double* u, double* cp, double* F, double* M) {
    DeviceGuard dg;
    if (dg.set(ctx->device) != cudaSuccess) return vp_fail(ctx, VP_ERR_CUDA, "cudaSetDevice");
    const int nb = std::max(1, (ntri + RB - 1) / RB);
    Bufs B;
    double *dc, *dmu = nullptr, *ddm = nullptr, *dcp_in = nullptr, *du = nullptr, *dcp = nullptr, *part, *dout;
    int* dsl = nullptr;
    int r;
    if ((r = B.up(ctx, &dc, corners, 9 * size_t(ntri)))) return r;
    if (cp_in) {
        if ((r = B.up(ctx, &dcp_in, cp_in, size_t(ntri)))) return r;
    } else {
        if ((r = B.up(ctx, &dsl, corner_slot, 3 * size_t(ntri))) || (r = B.up(ctx, &dmu, mu, size_t(nslot)))) return r;
        if (dmudt && (r = B.up(ctx, &ddm, dmudt, size_t(nslot)))) return r;
        if (u && (r = B.alloc(ctx, &du, 3 * size_t(ntri)))) return r;
        if (cp && (r = B.alloc(ctx, &dcp, size_t(ntri)))) return r;
    }
    if ((r = B.alloc(ctx, &part, 6 * size_t(nb))) || (r = B.alloc(ctx, &dout, 6))) return r;
    SurfArgs a{};
    a.ntri = ntri;
    a.corners = dc;
    a.slot = dsl;
    a.mu = dmu;
    a.dmudt = ddm;
    a.cp_in = dcp_in;
    for (int z = 0; z < 3; ++z) {
        a.V[z] = vinf ? vinf[z] : 0.0;
        a.o[z] = origin ? origin[z] : 0.0;
    }
    a.V2 = a.V[0] * a.V[0] + a.V[1] * a.V[1] + a.V[2] * a.V[2];
    a.u_out = du;
    a.cp_out = dcp;
    a.part = part;
    surface_kernel<<<nb, RB, 0, ctx->stream>>>(a);
    sum_parts_kernel<<<1, 32, 0, ctx->stream>>>(nb, 6, part, dout);
    ctx->launches += 2;
    VP_CUDA(ctx, cudaGetLastError());
    double h[6];
    VP_CUDA(ctx, vp_d2h(ctx, h, dout, sizeof(h)));
    if (du) VP_CUDA(ctx, vp_d2h(ctx, u, du, sizeof(double) * 3 * ntri));
    if (dcp) VP_CUDA(ctx, vp_d2h(ctx, cp, dcp, sizeof(double) * ntri));
    VP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    for (int z = 0; z < 3; ++z) {
        if (F) F[z] = h[z];
        if (M) M[z] = h[3 + z];
    }
    return VP_OK;
}

extern "C" int vp_surface_loads(vp_ctx* ctx, int ntri, const double* corners, const int* corner_slot, int nslot,
                                const double* mu, const double* dmudt, const double* vinf, const double* origin,
                                double* u, double* cp, double* F, double* M) {
    if (!ctx || ntri <= 0 || nslot <= 0 || !corners || !corner_slot || !mu || !vinf)
        return vp_fail(ctx, VP_ERR_ARG, "bad argument");
    for (size_t k = 0; k < 3 * size_t(ntri); ++k)
        if (corner_slot[k] < 0 || corner_slot[k] >= nslot) return vp_fail(ctx, VP_ERR_ARG, "corner slot out of range");
    if (!(vinf[0] * vinf[0] + vinf[1] * vinf[1] + vinf[2] * vinf[2] > 0))
        return vp_fail(ctx, VP_ERR_ARG, "V∞ must not be zero");
    for (int t = 0; t < ntri; ++t) {
        const double* c = corners + 9 * size_t(t);
        const double e1[3] = {c[3] - c[0], c[4] - c[1], c[5] - c[2]}, e2[3] = {c[6] - c[0], c[7] - c[1], c[8] - c[2]};
        const double n2 = std::pow(e1[1] * e2[2] - e1[2] * e2[1], 2) + std::pow(e1[2] * e2[0] - e1[0] * e2[2], 2) +
                          std::pow(e1[0] * e2[1] - e1[1] * e2[0], 2);
        if (!(n2 > 0)) return vp_fail(ctx, VP_ERR_DEGENERATE, "degenerate triangle " + std::to_string(t));
    }
    return surface_common(ctx, ntri, corners, corner_slot, nslot, mu, dmudt, nullptr, vinf, origin, u, cp, F, M);
}

extern "C" int vp_pressure_force(vp_ctx* ctx, int ntri, const double* corners, const double* cp, const double* origin,
                                 double* F, double* M) {
    if (!ctx || ntri <= 0 || !corners || !cp) return vp_fail(ctx, VP_ERR_ARG, "bad argument");
    return surface_common(ctx, ntri, corners, nullptr, 0, nullptr, nullptr, cp, nullptr, origin, nullptr, nullptr, F, M);
}

extern "C" int vp_wake_loads(vp_ctx* ctx, int nte, const double* te_x, int nline, const int* line_ptr,
                             const int* line_nodes, const int* line_closed, const double* mu_w, const double* vinf,
                             double* F_kj, double* D_trefftz) {
    if (!ctx || nte < 0 || nline < 0 || !vinf || (nte > 0 && (!te_x || !mu_w)) ||
        (nline > 0 && (!line_ptr || !line_nodes || !line_closed)))
        return vp_fail(ctx, VP_ERR_ARG, "bad argument");
    const double V2 = vinf[0] * vinf[0] + vinf[1] * vinf[1] + vinf[2] * vinf[2];
    if (!(V2 > 0)) return vp_fail(ctx, VP_ERR_ARG, "V∞ must not be zero");
    if (nline > 0 && line_ptr[0] != 0) return vp_fail(ctx, VP_ERR_ARG, "line_ptr[0] must be 0");
    // segments (a, b) along every line and the trailing vortex at every line point with its neighbouring segments
    std::vector<int> seg, vort;
    for (int L = 0; L < nline; ++L) {
        const int p0 = line_ptr[L], m = line_ptr[L + 1] - p0;
        if (m < 0) return vp_fail(ctx, VP_ERR_ARG, "line_ptr must not decrease");
        for (int i = 0; i < m; ++i)
            if (line_nodes[p0 + i] < 0 || line_nodes[p0 + i] >= nte)
                return vp_fail(ctx, VP_ERR_ARG, "trailing edge node out of range");
        const bool closed = line_closed[L] != 0;
        const int nseg = closed ? m : m - 1;
        const int s0 = int(seg.size() / 2);
        for (int i = 0; i < nseg; ++i) {
            seg.push_back(line_nodes[p0 + i]);
            seg.push_back(line_nodes[p0 + (i + 1) % m]);
        }
        for (int i = 0; i < m; ++i) {
            vort.push_back(line_nodes[p0 + i]);
            vort.push_back(i > 0 ? s0 + i - 1 : (closed && nseg > 0 ? s0 + nseg - 1 : -1));
            vort.push_back(i < nseg ? s0 + i : -1);
        }
    }
    const int nseg = int(seg.size() / 2), nvort = int(vort.size() / 3);
    if (nseg == 0) {
        for (int z = 0; z < 3; ++z)
            if (F_kj) F_kj[z] = 0.0;
        if (D_trefftz) *D_trefftz = 0.0;
        return VP_OK;
    }
    DeviceGuard dg;
    if (dg.set(ctx->device) != cudaSuccess) return vp_fail(ctx, VP_ERR_CUDA, "cudaSetDevice");
    Bufs B;
    double *dx, *dmu, *part, *dout;
    int *dseg, *dvort;
    int r;
    if ((r = B.up(ctx, &dx, te_x, 3 * size_t(nte))) || (r = B.up(ctx, &dmu, mu_w, size_t(nte))) ||
        (r = B.up(ctx, &dseg, seg.data(), seg.size())) || (r = B.up(ctx, &dvort, vort.data(), vort.size())) ||
        (r = B.alloc(ctx, &part, size_t(nseg) + 3)) || (r = B.alloc(ctx, &dout, 1)))
        return r;
    WakeArgs a{};
    a.nseg = nseg;
    a.nvort = nvort;
    a.x = dx;
    a.mu = dmu;
    a.seg = dseg;
    a.vort = dvort;
    const double vn = std::sqrt(V2);
    for (int z = 0; z < 3; ++z) {
        a.V[z] = vinf[z];
        a.d[z] = vinf[z] / vn;
    }
    a.part = part;
    trefftz_kernel<<<nseg + 1, RB, 0, ctx->stream>>>(a);
    sum_parts_kernel<<<1, 32, 0, ctx->stream>>>(nseg, 1, part, dout);
    ctx->launches += 2;
    VP_CUDA(ctx, cudaGetLastError());
    double D, G[3];
    VP_CUDA(ctx, vp_d2h(ctx, &D, dout, sizeof(double)));
    VP_CUDA(ctx, vp_d2h(ctx, G, part + nseg, sizeof(G)));
    VP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    const double k = 2.0 / V2;
    if (F_kj) {
        F_kj[0] = k * (vinf[1] * G[2] - vinf[2] * G[1]);
        F_kj[1] = k * (vinf[2] * G[0] - vinf[0] * G[2]);
        F_kj[2] = k * (vinf[0] * G[1] - vinf[1] * G[0]);
    }
    if (D_trefftz) *D_trefftz = k * D;
    return VP_OK;
}
