// The free wake's device work (src/freewake/step.jl, src/assembly/explicit.jl, src/post/Post.jl:92-112):
//   - blob velocities: the direct Rosenhead-Moore sum of every blob at every wake point (blob_velocities,
//     step.jl:176-187), a tiled N-body kernel: one thread per point, the blobs staged through shared memory in tiles;
//   - body velocity: sigma_s w_s + gamma_s x w_s of every body triangle at every wake point (body_velocity), one
//     thread per point over shared-memory tiles of triangles, the exact kernel within kernel_far diameters and the
//     multipole beyond;
//   - explicit right hand side (explicit_rhs, explicit.jl:31-85): the wake's known sheets and filaments through the
//     assembly's own tiers (their columns assembled with the body as test triangles only, times their doublets), and
//     the particles with the far rule or, closer than far_ratio, the near rule.
#include "vp_pairs.cuh"
#include "vp_wake_kernels.cuh"

int vp_assemble_impl(vp_ctx* ctx, const vp_assembly_options* o, int nnode, const double* x, int ntri, const int* tris,
                     const int* corner_slot, int nslot, int ntouch, const int* touch_pairs, const double* sigma,
                     const double* vinf, int nwnode, const double* wx, int nwtri, const int* wtris, int nfil,
                     const int* fil, vp_system** out, vp_assembly_stats* stats, int body_sources);

namespace {

// the particles' part of explicit_rhs: one warp per test triangle, the lanes over the particles (particle_rows). Each
// triangle writes its three rows; a slot's rows (from several test triangles) are summed afterwards in triangle order.
struct BlobRhsArgs {
    const TriGeo* tri;
    int ntri, nblob;
    const double* blobs;  // x (3), alpha (3), delta
    ParticleRule pr;
    double* trow;         // ntri x 3
};

template <class T>
__global__ void __launch_bounds__(128) blob_rhs_kernel(BlobRhsArgs a) {
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (w >= a.ntri) return;
    const TriGeo& Tr = a.tri[w];
    double rows[3] = {0, 0, 0};
    for (int k = lane; k < a.nblob; k += 32) particle_rows<T>(a.pr, Tr, a.blobs + 7 * size_t(k), rows);
    for (int k = 0; k < 3; ++k) {
        const double v = warp_sum(rows[k]);
        if (lane == k) a.trow[3 * size_t(w) + k] = v;
    }
}

int points_grid(int n) { return (n + NB_THREADS - 1) / NB_THREADS; }

}  // namespace

extern "C" int vp_blob_velocities(vp_ctx* ctx, int precision, int nblob, const double* blobs, int npts, const double* X,
                                  double* U) {
    if (!ctx || npts < 0 || nblob < 0 || (npts > 0 && (!X || !U)) || (nblob > 0 && !blobs))
        return vp_fail(ctx, VP_ERR_ARG, "bad argument");
    if (npts == 0) return VP_OK;
    if (cudaSetDevice(ctx->device) != cudaSuccess) return vp_fail(ctx, VP_ERR_CUDA, "cudaSetDevice");
    if (nblob == 0) {
        for (size_t k = 0; k < 3 * size_t(npts); ++k) U[k] = 0.0;
        return VP_OK;
    }
    DevList dl;
    double *db, *dx, *du;
    int r;
    std::vector<double> hb(blobs, blobs + 7 * size_t(nblob));
    std::vector<double> hx(X, X + 3 * size_t(npts));
    if ((r = dl.up(ctx, &db, hb)) || (r = dl.up(ctx, &dx, hx)) || (r = dl.alloc(ctx, &du, 3 * size_t(npts)))) return r;
    vp_phase_begin(ctx, PH_WAKE);
    if (precision == VP_FP64)
        blob_kernel<double><<<points_grid(npts), NB_THREADS, 0, ctx->stream>>>(nblob, db, npts, dx, du);
    else
        blob_kernel<float><<<(npts + NB_THREADS * NB_PTS - 1) / (NB_THREADS * NB_PTS), NB_THREADS, 0, ctx->stream>>>(
            nblob, db, npts, dx, du);
    vp_phase_end(ctx);
    ctx->launches++;
    VP_CUDA(ctx, cudaGetLastError());
    VP_CUDA(ctx, vp_d2h(ctx, U, du, sizeof(double) * 3 * npts));
    VP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return VP_OK;
}

extern "C" int vp_body_velocity(vp_ctx* ctx, int precision, int ntri, const double* corners, const double* sigma,
                                const double* gamma, double kernel_far, int npts, const double* X, double* U) {
    if (!ctx || ntri < 0 || npts < 0 || (ntri > 0 && (!corners || !sigma || !gamma)) || (npts > 0 && (!X || !U)) ||
        !(kernel_far > 0))
        return vp_fail(ctx, VP_ERR_ARG, "bad argument");
    if (npts == 0) return VP_OK;
    if (cudaSetDevice(ctx->device) != cudaSuccess) return vp_fail(ctx, VP_ERR_CUDA, "cudaSetDevice");
    std::vector<BodySrc> hs(std::max(ntri, 1));
    for (int t = 0; t < ntri; ++t) {
        TriGeo g;
        const double* c = corners + 9 * size_t(t);
        if (!make_tri(c, c + 3, c + 6, g)) return vp_fail(ctx, VP_ERR_DEGENERATE, "degenerate triangle " + std::to_string(t));
        BodySrc& s = hs[t];
        for (int k = 0; k < 3; ++k) {
            s.c[k] = g.c[k];
            s.len[k] = g.len[k];
            s.n[k] = g.n[k];
            s.gam[k] = gamma[3 * size_t(t) + k];
        }
        for (int k = 0; k < 9; ++k) {
            s.d[k] = g.x[k] - g.c[k % 3];
            s.nu[k] = g.nu[k];
        }
        s.area = g.area;
        s.diam = g.diam;
        s.sigma = sigma[t];
    }
    DevList dl;
    BodySrc* ds;
    double *dx, *du;
    int r;
    std::vector<double> hx(X, X + 3 * size_t(npts));
    if ((r = dl.up(ctx, &ds, hs)) || (r = dl.up(ctx, &dx, hx)) || (r = dl.alloc(ctx, &du, 3 * size_t(npts)))) return r;
    vp_phase_begin(ctx, PH_WAKE);
    if (precision == VP_FP64)
        body_kernel<double><<<points_grid(npts), NB_THREADS, 0, ctx->stream>>>(ntri, ds, kernel_far, npts, dx, du);
    else
        body_kernel<float><<<points_grid(npts), NB_THREADS, 0, ctx->stream>>>(ntri, ds, kernel_far, npts, dx, du);
    vp_phase_end(ctx);
    ctx->launches++;
    VP_CUDA(ctx, cudaGetLastError());
    VP_CUDA(ctx, vp_d2h(ctx, U, du, sizeof(double) * 3 * npts));
    VP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return VP_OK;
}

extern "C" int vp_explicit_rhs(vp_ctx* ctx, const vp_assembly_options* o, int nnode, const double* x, int ntri,
                               const int* tris, const int* corner_slot, int nslot, int nsheet, const double* sheet_x,
                               const double* sheet_mu, int nseg, const double* seg_x, const double* seg_gamma,
                               int nblob, const double* blobs, double* rhs) {
    if (!ctx || !o || !x || !tris || !corner_slot || !rhs || nsheet < 0 || nseg < 0 || nblob < 0 ||
        (nsheet > 0 && (!sheet_x || !sheet_mu)) || (nseg > 0 && (!seg_x || !seg_gamma)) || (nblob > 0 && !blobs) ||
        ntri < 0 || nnode < 0 || nslot < 0)
        return vp_fail(ctx, VP_ERR_ARG, "bad argument");
    for (size_t k = 0; k < 3 * size_t(ntri); ++k) {
        if (tris[k] < 0 || tris[k] >= nnode) return vp_fail(ctx, VP_ERR_ARG, "triangle node out of range");
        if (corner_slot[k] < 0 || corner_slot[k] >= nslot) return vp_fail(ctx, VP_ERR_ARG, "corner slot out of range");
    }
    if (cudaSetDevice(ctx->device) != cudaSuccess) return vp_fail(ctx, VP_ERR_CUDA, "cudaSetDevice");
    int r;
    DevList dl;
    double* d_rhs;
    if ((r = dl.alloc(ctx, &d_rhs, size_t(nslot)))) return r;
    VP_CUDA(ctx, cudaMemsetAsync(d_rhs, 0, sizeof(double) * nslot, ctx->stream));
    // sheets and filaments: their own nodes (unshared), their columns assembled with the body's test triangles
    const int nw = 3 * nsheet + 2 * nseg;
    if (nw > 0) {
        std::vector<double> wx(3 * size_t(nw)), mu(nw);
        std::vector<int> wt(3 * size_t(std::max(nsheet, 1)), 0), fl(2 * size_t(std::max(nseg, 1)), 0);
        for (int s = 0; s < nsheet; ++s)
            for (int k = 0; k < 3; ++k) {
                for (int z = 0; z < 3; ++z) wx[3 * (3 * size_t(s) + k) + z] = sheet_x[9 * size_t(s) + 3 * k + z];
                mu[3 * s + k] = sheet_mu[3 * size_t(s) + k];
                wt[3 * size_t(s) + k] = 3 * s + k;
            }
        for (int f = 0; f < nseg; ++f)
            for (int k = 0; k < 2; ++k) {
                const int node = 3 * nsheet + 2 * f + k;
                for (int z = 0; z < 3; ++z) wx[3 * size_t(node) + z] = seg_x[6 * size_t(f) + 3 * k + z];
                mu[node] = seg_gamma[2 * size_t(f) + k];
                fl[2 * size_t(f) + k] = node;
            }
        std::vector<double> sig(ntri, 0.0);
        const double vzero[3] = {0, 0, 0};
        vp_system* sys = nullptr;
        r = vp_assemble_impl(ctx, o, nnode, x, ntri, tris, corner_slot, nslot, 0, nullptr, sig.data(), vzero, nw,
                             wx.data(), nsheet, wt.data(), nseg, fl.data(), &sys, nullptr, 0);
        if (r) return r;
        double* d_mu;
        if ((r = dl.up(ctx, &d_mu, mu))) {
            vp_system_free(sys);
            return r;
        }
        const double mone = -1.0, zero = 0.0;
        // A is row-major nslot x (nslot + nw): its wake block, read column-major, is nw x nslot with leading dim ncols
        cublasStatus_t bs = cublasDgemv(ctx->blas, CUBLAS_OP_T, nw, nslot, &mone, sys->A + nslot, sys->ncols, d_mu, 1,
                                        &zero, d_rhs, 1);
        cudaError_t e = cudaStreamSynchronize(ctx->stream);
        vp_system_free(sys);
        if (bs != CUBLAS_STATUS_SUCCESS) return vp_fail(ctx, VP_ERR_CUDA, "cublasDgemv");
        if (e != cudaSuccess) return vp_fail(ctx, VP_ERR_CUDA, std::string("explicit_rhs: ") + cudaGetErrorString(e));
    }
    // particles
    if (nblob > 0) {
        std::vector<TriGeo> tg(ntri);
        for (int t = 0; t < ntri; ++t) {
            if (!make_tri(x + 3 * tris[3 * t], x + 3 * tris[3 * t + 1], x + 3 * tris[3 * t + 2], tg[t]))
                return vp_fail(ctx, VP_ERR_DEGENERATE, "degenerate triangle " + std::to_string(t));
            for (int k = 0; k < 3; ++k) {
                tg[t].node[k] = tris[3 * t + k];
                tg[t].slot[k] = corner_slot[3 * t + k];
            }
        }
        std::vector<RulePt> rfar = triangle_rule(o->far_points), rnear = triangle_rule(o->near_points);
        std::vector<double> hb(blobs, blobs + 7 * size_t(nblob));
        TriGeo* d_tg;
        RulePt *d_rf, *d_rn;
        double *d_b, *d_trow;
        if ((r = dl.up(ctx, &d_tg, tg)) || (r = dl.up(ctx, &d_rf, rfar)) || (r = dl.up(ctx, &d_rn, rnear)) ||
            (r = dl.up(ctx, &d_b, hb)) || (r = dl.alloc(ctx, &d_trow, 3 * size_t(ntri))))
            return r;
        BlobRhsArgs a{};
        a.tri = d_tg;
        a.ntri = ntri;
        a.nblob = nblob;
        a.blobs = d_b;
        a.pr.rfar = d_rf;
        a.pr.nfar = (int)rfar.size();
        a.pr.rnear = d_rn;
        a.pr.nnear = (int)rnear.size();
        a.pr.test_mode = o->test;
        a.pr.near_depth = o->near_depth;
        a.pr.far_ratio = o->far_ratio;
        a.pr.near_ratio = o->near_ratio;
        a.trow = d_trow;
        const int nb = (ntri * 32 + 127) / 128;
        if (o->precision == VP_FP64)
            blob_rhs_kernel<double><<<nb, 128, 0, ctx->stream>>>(a);
        else
            blob_rhs_kernel<float><<<nb, 128, 0, ctx->stream>>>(a);
        ctx->launches++;
        VP_CUDA(ctx, cudaGetLastError());
        std::vector<double> trow(3 * size_t(ntri));
        VP_CUDA(ctx, vp_d2h(ctx, trow.data(), d_trow, sizeof(double) * 3 * ntri));
        VP_CUDA(ctx, vp_d2h(ctx, rhs, d_rhs, sizeof(double) * nslot));
        VP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        for (int t = 0; t < ntri; ++t)
            for (int k = 0; k < 3; ++k) rhs[corner_slot[3 * t + k]] += trow[3 * size_t(t) + k];
        return VP_OK;
    }
    VP_CUDA(ctx, vp_d2h(ctx, rhs, d_rhs, sizeof(double) * nslot));
    VP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return VP_OK;
}
