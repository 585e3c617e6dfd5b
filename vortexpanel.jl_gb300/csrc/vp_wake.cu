// The free wake as a device-resident simulation: FreeWakeSim's step!/run! (src/freewake/step.jl:113-216) over the
// state of src/freewake/state.jl, with every array on the GPU at a fixed capacity and no allocation inside a step.
//
// State (allocated once; the particle arrays grow only when a step would overflow them):
//   - node rows in a ring of keep_rows + 2 rows, newest first: positions (nte x 3) and the doublets each row was shed
//     with (nte), and mu_line, the upstream doublets of the last converted row (FreeWakeState, state.jl:132-147);
//   - particles (x, alpha, delta) with their merge tag and group, and per strip the merge batch's rows, length and
//     width;
//   - the body's element data, the factored bordered matrix of the body with its trailing edge panel and its b0.
// One step, in the reference's order (step.jl:113-146), all on the context's stream:
//   1. vortex_elements (state.jl:241-253): the free rows' sheets (two per strip and panel row), the rows' tip sides,
//      the interface filament along R0 and the far end filament, with their blobs (free_wake_blobs, state.jl:275-295);
//   2. explicit_rhs (src/assembly/explicit.jl:31-85): one warp per body triangle over the sheets (the assembly's
//      wake_pair_rule tiers: far points by lanes, contact and near pieces by the warp), the filaments (segment_rule:
//      far, vertex or near) and the particles (far rule or near quadtree); the rows are summed per slot in a fixed
//      order, then the bordered solve with the factors (no allocation) gives q, mu = C q and mu_w = K q;
//   3. the loads (step_loads, step.jl:149-163): the gradient route's Cp with the backward difference of mu, the
//      pressure force and moment, Kutta-Joukowski, and the total vorticity and impulse of every element's blobs;
//   4. the velocities at the free nodes and particles: V + the body's exact kernels + every wake element as blobs
//      (wake_velocities, step.jl:166-173), and forward Euler;
//   5. a new R0 on the trailing edge panel's downstream edge, conversion of the oldest row into particles with the
//      merge bookkeeping (convert_oldest!, merge_strip!, state.jl:300-373) and deletion beyond the limit
//      (delete_far!, step.jl:190-195), by single-block kernels that keep the particle count on the device.
// The step's record (a few doubles and mu_w) is the only copy to the host.
#include <cmath>
#include <limits>

#include "vp_pairs.cuh"
#include "vp_wake_kernels.cuh"

namespace {

constexpr int RHS_WARPS = 4;    // warps (test triangles) per block of the right hand side kernel
constexpr int BK_THREADS = 1024;  // the single-block bookkeeping kernels
constexpr int ELEM_THREADS = 128;

struct CoreDev {  // CoreRule (state.jl:64-92): 0 auto, 1 scaled, 2 fixed
    int mode;
    double overlap, factor, floor, value;
};

__device__ __forceinline__ double core_tri(const CoreDev& c, v3<double> p, v3<double> q, v3<double> r) {
    if (c.mode == 2) return c.value;
    if (c.mode == 0) return c.overlap * fmax(fmax(vnorm(q - p), vnorm(r - q)), vnorm(p - r)) / 2;
    return fmax(c.factor * sqrt(vnorm(cross(q - p, r - p))), c.floor);
}

__device__ __forceinline__ double core_seg(const CoreDev& c, v3<double> a, v3<double> b) {
    if (c.mode == 2) return c.value;
    if (c.mode == 0) return c.overlap * vnorm(b - a) / 2;
    return fmax(c.factor * vnorm(b - a) / 2, c.floor);
}

__device__ __forceinline__ void put_blob(double* o, v3<double> x, v3<double> al, double d) {
    o[0] = x.x;
    o[1] = x.y;
    o[2] = x.z;
    o[3] = al.x;
    o[4] = al.y;
    o[5] = al.z;
    o[6] = d;
}

// the particle of a sheet triangle (p, q, r) with corner doublets m: its centroid, gamma A = sum over the edges of
// (mu_a + mu_b)/2 (x_b - x_a) (sheet_vorticity, state.jl:272), and the triangle's core
__device__ __forceinline__ void sheet_blob(const CoreDev& c, v3<double> p, v3<double> q, v3<double> r, double m0,
                                           double m1, double m2, double* o) {
    v3<double> al = ((m0 + m1) * (q - p) + (m1 + m2) * (r - q) + (m2 + m0) * (p - r)) / 2.0;
    put_blob(o, (p + q + r) / 3.0, al, core_tri(c, p, q, r));
}

// the two blobs of a filament a -> b with end circulations ga, gb at its 2-point Gauss positions (blob.jl:31-38)
__device__ __forceinline__ void segment_blob_pair(const CoreDev& c, v3<double> a, v3<double> b, double ga, double gb,
                                                  double* o) {
    const double s = 1.0 / (2.0 * sqrt(3.0));
    const double d = core_seg(c, a, b);
    const double xi[2] = {0.5 - s, 0.5 + s};
    for (int h = 0; h < 2; ++h) {
        v3<double> al = (((1 - xi[h]) * ga + xi[h] * gb) / 2) * (b - a);
        put_blob(o + 7 * h, a + xi[h] * (b - a), al, d);
    }
}

// element data of a sheet triangle on the device, as make_tri builds it on the host (flat_triangle.jl:12-31); the
// node fields mark it as a wake triangle (no shared nodes with the body). Returns false for a zero area.
__device__ bool dev_make_tri(v3<double> a, v3<double> b, v3<double> c, TriGeo& g) {
    v3<double> nA = cross(b - a, c - a);
    double A2 = sqrt(dot(nA, nA));
    const v3<double> v[3] = {a, b, c};
    for (int k = 0; k < 3; ++k) {
        g.x[3 * k] = v[k].x;
        g.x[3 * k + 1] = v[k].y;
        g.x[3 * k + 2] = v[k].z;
        g.node[k] = -1;
        g.slot[k] = 0;
    }
    if (!(A2 > 0)) return false;
    v3<double> n = nA / A2;
    g.n[0] = n.x;
    g.n[1] = n.y;
    g.n[2] = n.z;
    v3<double> cc = (a + b + c) / 3.0;
    g.c[0] = cc.x;
    g.c[1] = cc.y;
    g.c[2] = cc.z;
    g.area = A2 / 2;
    v3<double> e[3];
    for (int q = 0; q < 3; ++q) {
        e[q] = v[(q + 1) % 3] - v[q];
        g.len[q] = sqrt(dot(e[q], e[q]));
        v3<double> nu = cross(e[q], n) / g.len[q];
        g.nu[3 * q] = nu.x;
        g.nu[3 * q + 1] = nu.y;
        g.nu[3 * q + 2] = nu.z;
    }
    g.diam = fmax(g.len[0], fmax(g.len[1], g.len[2]));
    const int opp[3] = {1, 2, 0};
    for (int bb = 0; bb < 3; ++bb) {
        g.gam[3 * bb] = -e[opp[bb]].x / A2;
        g.gam[3 * bb + 1] = -e[opp[bb]].y / A2;
        g.gam[3 * bb + 2] = -e[opp[bb]].z / A2;
    }
    double rch = 0;
    for (int q = 0; q < 3; ++q) rch = fmax(rch, vnorm(v[q] - cc));
    g.reach = rch;
    g.sigma = 0;
    return true;
}

// ---- 1. the free wake's vortex elements and their blobs -------------------------------------------------------------

struct ElemArgs {
    int nr, head, R, nte;
    const double* rx;   // R x nte x 3 (ring rows)
    const double* rmu;  // R x nte
    const double* mul;  // nte (mu_line)
    int nstrip, nfirst, nlast;
    const int* strips;  // nstrip x 2
    const int* first;
    const int* last;
    CoreDev core;
    int nsh, nsg;       // sheets 2 nstrip (nr - 1); segments (nfirst + nlast)(nr - 1) + 2 nstrip (nr >= 1)
    TriGeo* sheet;      // nsh
    double* sheet_G;    // nsh x 3: the sheet's vortex strength sum_b mu_b gamma_b
    int* sheet_ok;      // nsh: nondegenerate (in the right hand side)
    double* seg;        // nsg x 8: a (3), b (3), ga, gb
    double* blobs;      // the sheets' blobs (nsh), then the segments' (2 nsg)
};

__device__ __forceinline__ v3<double> row_x(const ElemArgs& a, int i, int k) {
    const double* p = a.rx + (size_t((a.head + i) % a.R) * a.nte + k) * 3;
    return mk3(p[0], p[1], p[2]);
}
__device__ __forceinline__ double row_mu(const ElemArgs& a, int i, int k) {
    return a.rmu[size_t((a.head + i) % a.R) * a.nte + k];
}

__global__ void __launch_bounds__(ELEM_THREADS) elements_kernel(ElemArgs a) {
    const int e = blockIdx.x * ELEM_THREADS + threadIdx.x;
    if (e < a.nsh) {
        // panel row i between node rows i and i + 1 (panel_row!, state.jl:203-218): two sheets per strip (A, B)
        const int i = e / (2 * a.nstrip), j = e % (2 * a.nstrip), s = j >> 1, h = j & 1;
        const int A = a.strips[2 * s], B = a.strips[2 * s + 1];
        v3<double> p, q, r;
        double m0, m1, m2;
        if (h == 0) {
            p = row_x(a, i, A), q = row_x(a, i + 1, A), r = row_x(a, i, B);
            m0 = row_mu(a, i, A), m1 = row_mu(a, i + 1, A), m2 = row_mu(a, i, B);
        } else {
            p = row_x(a, i + 1, A), q = row_x(a, i + 1, B), r = row_x(a, i, B);
            m0 = row_mu(a, i + 1, A), m1 = row_mu(a, i + 1, B), m2 = row_mu(a, i, B);
        }
        // nondegenerate (state.jl:155): |(q - p) x (r - p)| > 1e-12 max of the squared edges
        const double big = fmax(fmax(dot(q - p, q - p), dot(r - p, r - p)), dot(r - q, r - q));
        TriGeo& g = a.sheet[e];
        const bool ok = vnorm(cross(q - p, r - p)) > 1e-12 * big && dev_make_tri(p, q, r, g);
        a.sheet_ok[e] = ok ? 1 : 0;
        double G[3] = {0, 0, 0};
        if (ok)
            for (int z = 0; z < 3; ++z) G[z] = m0 * g.gam[z] + m1 * g.gam[3 + z] + m2 * g.gam[6 + z];
        for (int z = 0; z < 3; ++z) a.sheet_G[3 * size_t(e) + z] = G[z];
        sheet_blob(a.core, p, q, r, m0, m1, m2, a.blobs + 7 * size_t(e));
        return;
    }
    const int f = e - a.nsh;
    if (f >= a.nsg) return;
    const int ntip = a.nfirst + a.nlast, ntips = ntip * (a.nr - 1);
    v3<double> x0, x1;
    double g0, g1;
    if (f < ntips) {  // tip sides of panel row i: first nodes upstream (x1 -> x0), last nodes downstream (x0 -> x1)
        const int i = f / ntip, k = f % ntip;
        if (k < a.nfirst) {
            const int nd = a.first[k];
            x0 = row_x(a, i + 1, nd), x1 = row_x(a, i, nd), g0 = row_mu(a, i + 1, nd), g1 = row_mu(a, i, nd);
        } else {
            const int nd = a.last[k - a.nfirst];
            x0 = row_x(a, i, nd), x1 = row_x(a, i + 1, nd), g0 = row_mu(a, i, nd), g1 = row_mu(a, i + 1, nd);
        }
    } else if (f < ntips + a.nstrip) {  // the interface filament along R0, A -> B, strength mu(R0)
        const int s = f - ntips, A = a.strips[2 * s], B = a.strips[2 * s + 1];
        x0 = row_x(a, 0, A), x1 = row_x(a, 0, B), g0 = row_mu(a, 0, A), g1 = row_mu(a, 0, B);
    } else {  // the far end filament along the oldest row, B -> A, strength mu - mu_line (far_end!, state.jl:221-230)
        const int s = f - ntips - a.nstrip, A = a.strips[2 * s], B = a.strips[2 * s + 1], o = a.nr - 1;
        x0 = row_x(a, o, B), x1 = row_x(a, o, A), g0 = row_mu(a, o, B) - a.mul[B], g1 = row_mu(a, o, A) - a.mul[A];
    }
    double* sg = a.seg + 8 * size_t(f);
    sg[0] = x0.x, sg[1] = x0.y, sg[2] = x0.z, sg[3] = x1.x, sg[4] = x1.y, sg[5] = x1.z, sg[6] = g0, sg[7] = g1;
    segment_blob_pair(a.core, x0, x1, g0, g1, a.blobs + 7 * (size_t(a.nsh) + 2 * size_t(f)));
}

// the trailing edge panel's elements with the doublets mu_w of its trailing edge nodes, as blobs
// (vortex_elements(w::RigidWake, mu_w), state.jl:256-265, and free_wake_blobs)
struct TeBlobArgs {
    int npt, npf;
    const double* x;   // panel nodes
    const int* te;     // panel node -> trailing edge node
    const int* tris;   // npt x 3
    const int* fil;    // npf x 2
    const double* muw; // nte
    CoreDev core;
    double* blobs;     // npt + 2 npf
};

__global__ void te_blobs_kernel(TeBlobArgs a) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e < a.npt) {
        const int* t = a.tris + 3 * e;
        v3<double> p = ld3(a.x + 3 * t[0]), q = ld3(a.x + 3 * t[1]), r = ld3(a.x + 3 * t[2]);
        sheet_blob(a.core, p, q, r, a.muw[a.te[t[0]]], a.muw[a.te[t[1]]], a.muw[a.te[t[2]]], a.blobs + 7 * size_t(e));
    } else if (e < a.npt + a.npf) {
        const int f = e - a.npt, ia = a.fil[2 * f], ib = a.fil[2 * f + 1];
        segment_blob_pair(a.core, ld3(a.x + 3 * ia), ld3(a.x + 3 * ib), a.muw[a.te[ia]], a.muw[a.te[ib]],
                          a.blobs + 7 * (size_t(a.npt) + 2 * size_t(f)));
    }
}

// ---- 2. the explicit right hand side ------------------------------------------------------------------------------

struct RhsArgs {
    NearArgs na;        // the body (tri), the sheets (wtri), the rules and options
    const double* sheet_G;
    const int* sheet_ok;
    int nsh, nsg, npart;
    const double* seg;   // nsg x 8
    const double* part;  // npart x 7
    ParticleRule pr;
    double* trow;        // ntri x 3: the rows of every test triangle
};

// the source velocity w of sheet S at the point x: the multipole beyond kernel_far diameters, else the exact kernel;
// FP32 under the guard in mixed precision, FP64 where the guard refuses (source_velocity, source_triangle.jl:134-138)
template <class T>
__device__ v3<double> sheet_w(const TriGeo& S, v3<double> x, double kfar) {
    const v3<double> r64 = x - ld3(S.c);
    const double fd = kfar * S.diam;
    if (sizeof(T) == 4) {
        SrcKern<float> K;
        for (int k = 0; k < 3; ++k) {
            K.d[k] = mk3(float(S.x[3 * k] - S.c[0]), float(S.x[3 * k + 1] - S.c[1]), float(S.x[3 * k + 2] - S.c[2]));
            K.nu[k] = mk3(float(S.nu[3 * k]), float(S.nu[3 * k + 1]), float(S.nu[3 * k + 2]));
            K.len[k] = float(S.len[k]);
        }
        K.n = mk3(float(S.n[0]), float(S.n[1]), float(S.n[2]));
        K.area = float(S.area);
        K.diam = float(S.diam);
        const v3<float> r = mk3(float(r64.x), float(r64.y), float(r64.z));
        v3<float> w;
        bool done = true;
        if (dot(r64, r64) > fd * fd) {
            w = sv_far(K, r);
        } else {
            const Fp32Guard g{PAIR_GUARD};
            done = sv_exact3_guarded(K, r - K.d[0], r - K.d[1], r - K.d[2], 0, g, w);
        }
        if (done) return mk3(double(w.x), double(w.y), double(w.z));
    }
    SrcKern<double> K;
    for (int k = 0; k < 3; ++k) {
        K.d[k] = mk3(S.x[3 * k] - S.c[0], S.x[3 * k + 1] - S.c[1], S.x[3 * k + 2] - S.c[2]);
        K.nu[k] = ld3(S.nu + 3 * k);
        K.len[k] = S.len[k];
    }
    K.n = ld3(S.n);
    K.area = S.area;
    K.diam = S.diam;
    if (dot(r64, r64) > fd * fd) return sv_far(K, r64);
    return sv_exact3(K, r64 - K.d[0], r64 - K.d[1], r64 - K.d[2], r64, 0, 1e-12);
}

// one warp per body test triangle: rows_a = -sum over the sheets of the pair block times their doublets, - the
// filaments' end parts times their circulations, - the particles' normal velocity, each against psi_a
template <class T>
__global__ void __launch_bounds__(32 * RHS_WARPS) wake_rhs_kernel(RhsArgs ra) {
    __shared__ WarpSh shm[RHS_WARPS];
    const NearArgs& a = ra.na;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int t = blockIdx.x * RHS_WARPS + w;
    if (t >= a.ntri) return;
    const TriGeo& Tr = a.tri[t];
    const v3<double> nT = ld3(Tr.n);
    PairCtx pc;
    pc.a = &a;
    pc.T = &Tr;
    pc.sh = &shm[w];
    pc.lane = lane;
    pc.nleaf = 0;
    pc.nq64 = 0;
    double rows[3] = {0, 0, 0};
    const RulePt* RF = a.rule[R_FAR];
    const int nfar = a.nrule[R_FAR];
    // sheets (wake_pair_rule, assemble.jl:288-293): a far one by its lane, the others by the warp
    for (int s0 = 0; s0 < ra.nsh; s0 += 32) {
        const int s = s0 + lane;
        bool nonfar = false;
        if (s < ra.nsh && ra.sheet_ok[s]) {
            const TriGeo& S = a.wtri[s];
            const double dc = vnorm(ld3(S.c) - ld3(Tr.c));
            if (dc > a.far_ratio * fmax(Tr.diam, S.diam)) {
                const v3<double> G = ld3(ra.sheet_G + 3 * size_t(s));
                for (int q = 0; q < nfar; ++q) {
                    const RulePt m = RF[q];
                    const v3<double> wv = sheet_w<T>(S, tpoint(Tr, &m.l0), a.kernel_far);
                    const double c = (m.w * Tr.area) * dot(cross(wv, nT), G);
                    const v3<double> psi = test_weights(a.test_mode, m.l0, m.l1, m.l2);
                    rows[0] -= c * psi.x;
                    rows[1] -= c * psi.y;
                    rows[2] -= c * psi.z;
                }
            } else {
                nonfar = true;
            }
        }
        unsigned msk = __ballot_sync(0xffffffffu, nonfar);
        while (msk) {
            const int q = __ffs(msk) - 1;
            msk &= msk - 1;
            const int sq = s0 + q;
            FwdAcc acc = {};
            pc.kind = 0;
            pc.npts = 0;
            pc.n64 = 0;
            tri_pair(pc, acc, t, sq, true);
            fold32(acc);
            const v3<double> G = ld3(ra.sheet_G + 3 * size_t(sq));
            for (int k = 0; k < 3; ++k) {
                const v3<double> P = mk3(warp_sum(acc.P[k].x), warp_sum(acc.P[k].y), warp_sum(acc.P[k].z));
                if (lane == 0) rows[k] -= dot(cross(P, nT), G);
            }
            __syncwarp();
        }
    }
    // filaments (segment_rule, assemble.jl:299-306; segment_block, :312-321): far by the lane, vertex or near by the warp
    const double corners[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    for (int f0 = 0; f0 < ra.nsg; f0 += 32) {
        const int f = f0 + lane;
        bool nonfar = false;
        if (f < ra.nsg) {
            const double* sg = ra.seg + 8 * size_t(f);
            const v3<double> fa = ld3(sg), fb = ld3(sg + 3);
            if (vnorm((fa + fb) / 2.0 - ld3(Tr.c)) > a.far_ratio * fmax(Tr.diam, vnorm(fb - fa))) {
                for (int q = 0; q < nfar; ++q) {
                    const RulePt m = RF[q];
                    const v3<double> x = tpoint(Tr, &m.l0);
                    v3<double> va, vb;
                    segment_velocity(x - fa, x - fb, va, vb);
                    const double c = (m.w * Tr.area) * (dot(va, nT) * sg[6] + dot(vb, nT) * sg[7]);
                    const v3<double> psi = test_weights(a.test_mode, m.l0, m.l1, m.l2);
                    rows[0] -= c * psi.x;
                    rows[1] -= c * psi.y;
                    rows[2] -= c * psi.z;
                }
            } else {
                nonfar = true;
            }
        }
        unsigned msk = __ballot_sync(0xffffffffu, nonfar);
        while (msk) {
            const int q = __ffs(msk) - 1;
            msk &= msk - 1;
            const double* sg = ra.seg + 8 * size_t(f0 + q);
            const v3<double> fa = ld3(sg), fb = ld3(sg + 3);
            if (lane == 0)
                for (int k = 0; k < 3; ++k) {
                    pc.sh->E[9 * k + 0] = Tr.x[3 * k + 0] - fa.x;
                    pc.sh->E[9 * k + 1] = Tr.x[3 * k + 1] - fa.y;
                    pc.sh->E[9 * k + 2] = Tr.x[3 * k + 2] - fa.z;
                    pc.sh->E[9 * k + 3] = Tr.x[3 * k + 0] - fb.x;
                    pc.sh->E[9 * k + 4] = Tr.x[3 * k + 1] - fb.y;
                    pc.sh->E[9 * k + 5] = Tr.x[3 * k + 2] - fb.z;
                }
            __syncwarp();
            FwdAcc acc = {};
            pc.kind = 1;
            pc.npts = 0;
            pc.n64 = 0;
            pc.side = 0;
            pc.fp32 = 0;
            int kv = -1;
            for (int k = 0; k < 3 && kv < 0; ++k)
                if (fmin(vnorm(ld3(Tr.x + 3 * k) - fa), vnorm(ld3(Tr.x + 3 * k) - fb)) <= 1e-12 * Tr.diam) kv = k;
            if (kv >= 0) {
                vertex_rule(pc, acc, kv);
            } else {
                SrcRef src{1, nullptr, fa, fb};
                near_pieces(pc, acc, src, corners, 1.0, a.near_depth);
                flush_leaves(pc, acc);
            }
            for (int k = 0; k < 3; ++k) {
                const double ca = warp_sum(acc.ca[k]), cb = warp_sum(acc.cb[k]);
                if (lane == 0) rows[k] -= ca * sg[6] + cb * sg[7];
            }
            __syncwarp();
        }
    }
    // particles (explicit.jl:63-76)
    for (int k = lane; k < ra.npart; k += 32) particle_rows<T>(ra.pr, Tr, ra.part + 7 * size_t(k), rows);
    for (int k = 0; k < 3; ++k) {
        const double v = warp_sum(rows[k]);
        if (lane == 0) ra.trow[3 * size_t(t) + k] = v;
    }
}

// rhs_s = b0_s + the rows of the slot's corners in a fixed order (the slot's list of triangle corners)
__global__ void slot_gather_kernel(int nslot, const int* __restrict__ ptr, const int* __restrict__ ent,
                                   const double* __restrict__ trow, const double* __restrict__ b0,
                                   double* __restrict__ rhs) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nslot) return;
    double v = 0.0;
    for (int p = ptr[s]; p < ptr[s + 1]; ++p) v += trow[ent[p]];
    rhs[s] = b0[s] + v;
}

// y = M x for a CSR matrix (the DOF map's C and K)
__global__ void csr_mv_kernel(int nrow, const int* __restrict__ p, const int* __restrict__ c,
                              const double* __restrict__ v, const double* __restrict__ x, double* __restrict__ y) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nrow) return;
    double s = 0.0;
    for (int k = p[i]; k < p[i + 1]; ++k) s += v[k] * x[c[k]];
    y[i] = s;
}

// ---- the mixed path's FP32 kernels of the particles' right hand side and of the body velocity ----------------------
// Both are N-body sums in FP32 with FP64 accumulation across tiles. Offsets are formed from hi/lo FP32 splits of the
// FP64 positions ((x_hi - y_hi) + (x_lo - y_lo): the first difference is exact where it matters), so they keep FP64
// accuracy near the wing. A 2-D grid spreads the targets over blocks and the sources over chunks; each chunk's
// partial sums go to their own slot and are added in chunk order (no atomics, bit-reproducible). The rare pairs that
// need the reference's near rule or FP64 (a particle within far_ratio of a test triangle, a point where the FP32 exact
// kernel cancels, a distance within rounding of a switch) take the FP64 path of the same pair.

constexpr int NB_CHUNK = 1024;  // sources per chunk of the 2-D N-body grids
constexpr int NB_TPB = 128;     // targets per block

__device__ __forceinline__ void split_hi_lo(double x, float& hi, float& lo) {
    hi = float(x);
    lo = float(x - double(hi));
}

// per particle: (x_hi, delta^2), (x_lo, delta), alpha / 4 pi
__global__ void particle_prep_kernel(int n, const double* __restrict__ part, float4* __restrict__ ph,
                                     float4* __restrict__ pl, float4* __restrict__ pa) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double* p = part + 7 * size_t(i);
    float h[3], l[3];
    for (int z = 0; z < 3; ++z) split_hi_lo(p[z], h[z], l[z]);
    const float i4pi = 1.f / (4.f * vp_pi<float>());
    ph[i] = make_float4(h[0], h[1], h[2], float(p[6] * p[6]));
    pl[i] = make_float4(l[0], l[1], l[2], float(p[6]));
    pa[i] = make_float4(float(p[3]) * i4pi, float(p[4]) * i4pi, float(p[5]) * i4pi, 0.f);
}

struct PRhsArgs {
    int ntri, npart, nchunk;
    const TriGeo* tri;
    const double* part;  // npart x 7 (the FP64 path of near and ambiguous pairs)
    const float4* ph;
    const float4* pl;
    const float4* pa;
    ParticleRule pr;
    double* out;         // nchunk x ntri x 3
};

// one thread per body test triangle (its far-rule points), the block's chunk of particles through shared memory:
// -int psi_a n.u dA of every particle of the chunk (explicit.jl:63-76)
__global__ void __launch_bounds__(NB_TPB) particle_rhs_kernel(PRhsArgs a) {
    __shared__ float4 sh[NB_TPB], sl[NB_TPB], sa[NB_TPB];
    const int t = blockIdx.x * NB_TPB + threadIdx.x;
    const bool valid = t < a.ntri;
    const TriGeo& Tr = a.tri[valid ? t : 0];
    const int nf = a.pr.nfar;
    float qh[NQMAX][3], ql[NQMAX][3];
    double U[NQMAX][3];
    float ch[3], cl[3];
    for (int z = 0; z < 3; ++z) split_hi_lo(Tr.c[z], ch[z], cl[z]);
#pragma unroll
    for (int q = 0; q < NQMAX; ++q) {
        const RulePt m = a.pr.rfar[q < nf ? q : 0];
        const v3<double> x = tpoint(Tr, &m.l0);
        split_hi_lo(x.x, qh[q][0], ql[q][0]);
        split_hi_lo(x.y, qh[q][1], ql[q][1]);
        split_hi_lo(x.z, qh[q][2], ql[q][2]);
        U[q][0] = U[q][1] = U[q][2] = 0.0;
    }
    const float diam = float(Tr.diam), fr = float(a.pr.far_ratio);
    double rows[3] = {0, 0, 0};
    const int j0 = blockIdx.y * NB_CHUNK, j1 = min(a.npart, j0 + NB_CHUNK);
    for (int b0 = j0; b0 < j1; b0 += NB_TPB) {
        const int nb = min(NB_TPB, j1 - b0);
        __syncthreads();
        if (threadIdx.x < nb) {
            sh[threadIdx.x] = a.ph[b0 + threadIdx.x];
            sl[threadIdx.x] = a.pl[b0 + threadIdx.x];
            sa[threadIdx.x] = a.pa[b0 + threadIdx.x];
        }
        __syncthreads();
        if (!valid) continue;
        float u[NQMAX][3];
#pragma unroll
        for (int q = 0; q < NQMAX; ++q) u[q][0] = u[q][1] = u[q][2] = 0.f;
        for (int k = 0; k < nb; ++k) {
            const float4 h = sh[k], l = sl[k], al = sa[k];
            const float dx = (ch[0] - h.x) + (cl[0] - l.x), dy = (ch[1] - h.y) + (cl[1] - l.y),
                        dz = (ch[2] - h.z) + (cl[2] - l.z);
            const float d2 = dx * dx + dy * dy + dz * dz;
            const float thr = fr * fmaxf(diam, l.w);
            if (d2 > thr * thr * 1.00001f) {  // far, beyond rounding: the far rule's points in FP32
#pragma unroll
                for (int q = 0; q < NQMAX; ++q) {
                    if (q >= nf) break;
                    const float rx = (qh[q][0] - h.x) + (ql[q][0] - l.x), ry = (qh[q][1] - h.y) + (ql[q][1] - l.y),
                                rz = (qh[q][2] - h.z) + (ql[q][2] - l.z);
                    const float r2 = fmaf(rx, rx, fmaf(ry, ry, fmaf(rz, rz, h.w)));
                    const float inv = rsqrtf(r2);
                    const float sc = inv * inv * inv;
                    u[q][0] = fmaf(sc, al.y * rz - al.z * ry, u[q][0]);
                    u[q][1] = fmaf(sc, al.z * rx - al.x * rz, u[q][1]);
                    u[q][2] = fmaf(sc, al.x * ry - al.y * rx, u[q][2]);
                }
            } else {  // near, or within rounding of the switch: the reference's decision and rule in FP64
                particle_rows<float>(a.pr, Tr, a.part + 7 * size_t(b0 + k), rows);
            }
        }
#pragma unroll
        for (int q = 0; q < NQMAX; ++q)
            for (int z = 0; z < 3; ++z) U[q][z] += double(u[q][z]);
    }
    if (!valid) return;
#pragma unroll
    for (int q = 0; q < NQMAX; ++q) {
        if (q >= nf) break;
        const RulePt m = a.pr.rfar[q];
        const double un = (m.w * Tr.area) * (U[q][0] * Tr.n[0] + U[q][1] * Tr.n[1] + U[q][2] * Tr.n[2]);
        const v3<double> psi = test_weights(a.pr.test_mode, m.l0, m.l1, m.l2);
        rows[0] -= un * psi.x;
        rows[1] -= un * psi.y;
        rows[2] -= un * psi.z;
    }
    double* o = a.out + (size_t(blockIdx.y) * a.ntri + t) * 3;
    o[0] = rows[0];
    o[1] = rows[1];
    o[2] = rows[2];
}

// out[i] += the chunks' partial sums of element i, in chunk order
__global__ void add_chunks_kernel(int n, int nchunk, const double* __restrict__ part, double* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double v = out[i];
    for (int c = 0; c < nchunk; ++c) v += part[size_t(c) * n + i];
    out[i] = v;
}

// body triangles as FP32 sources: centroid hi (3) and lo (3), corner offsets (9), edge normals (9), edge lengths (3),
// normal (3), area, diameter, sigma, gamma (3): 37 floats
constexpr int BS32 = 37;

__global__ void body_src32_kernel(int ntri, const BodySrc* __restrict__ bs, float* __restrict__ out) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntri) return;
    const BodySrc& b = bs[t];
    float* o = out + size_t(t) * BS32;
    for (int z = 0; z < 3; ++z) split_hi_lo(b.c[z], o[z], o[3 + z]);
    for (int k = 0; k < 9; ++k) {
        o[6 + k] = float(b.d[k]);
        o[15 + k] = float(b.nu[k]);
    }
    for (int k = 0; k < 3; ++k) {
        o[24 + k] = float(b.len[k]);
        o[27 + k] = float(b.n[k]);
        o[33 + k] = float(b.gam[k]);
    }
    o[30] = float(b.area);
    o[31] = float(b.diam);
    o[32] = float(b.sigma);
}

struct BVelArgs {
    int ntri, npts, nchunk;
    const float* src32;    // ntri x BS32
    const BodySrc* src64;  // the FP64 sources (guarded points, ambiguous far tests)
    const double* X;       // npts x 3
    double kernel_far;
    double* out;           // nchunk x npts x 3
};

constexpr int BV_TILE = 64;

// one thread per point, the block's chunk of body triangles through shared memory: sigma_s w_s + gamma_s x w_s
// (body_velocity, Post.jl:92-112): the multipole beyond kernel_far diameters, the exact kernel in FP32 under the
// guard within, FP64 where the guard refuses or the far switch is within rounding
__global__ void __launch_bounds__(NB_TPB) body_vel_kernel(BVelArgs a) {
    __shared__ float ss[BV_TILE * BS32];
    const int i = blockIdx.x * NB_TPB + threadIdx.x;
    const bool valid = i < a.npts;
    const v3<double> x = valid ? ld3(a.X + 3 * size_t(i)) : mk3(0.0, 0.0, 0.0);
    float xh[3], xl[3];
    split_hi_lo(x.x, xh[0], xl[0]);
    split_hi_lo(x.y, xh[1], xl[1]);
    split_hi_lo(x.z, xh[2], xl[2]);
    const float kf = float(a.kernel_far);
    const Fp32Guard g{PAIR_GUARD};
    v3<double> acc = mk3(0.0, 0.0, 0.0);
    const int s0 = blockIdx.y * NB_CHUNK, s1 = min(a.ntri, s0 + NB_CHUNK);
    for (int t0 = s0; t0 < s1; t0 += BV_TILE) {
        const int nt = min(BV_TILE, s1 - t0);
        __syncthreads();
        for (int k = threadIdx.x; k < nt * BS32; k += NB_TPB) ss[k] = a.src32[size_t(t0) * BS32 + k];
        __syncthreads();
        if (!valid) continue;
        v3<float> part = mk3(0.f, 0.f, 0.f);
        for (int k = 0; k < nt; ++k) {
            const float* o = ss + k * BS32;
            const v3<float> r = mk3((xh[0] - o[0]) + (xl[0] - o[3]), (xh[1] - o[1]) + (xl[1] - o[4]),
                                    (xh[2] - o[2]) + (xl[2] - o[5]));
            SrcKern<float> K;
            for (int e = 0; e < 3; ++e) {
                K.d[e] = mk3(o[6 + 3 * e], o[7 + 3 * e], o[8 + 3 * e]);
                K.nu[e] = mk3(o[15 + 3 * e], o[16 + 3 * e], o[17 + 3 * e]);
                K.len[e] = o[24 + e];
            }
            K.n = mk3(o[27], o[28], o[29]);
            K.area = o[30];
            K.diam = o[31];
            const float fd = kf * K.diam;
            const float r2 = dot(r, r);
            v3<float> w;
            bool ok = true;
            if (r2 > fd * fd * 1.00001f) {
                w = sv_far(K, r);
            } else if (r2 < fd * fd * 0.99999f) {
                ok = sv_exact3_guarded(K, r - K.d[0], r - K.d[1], r - K.d[2], 0, g, w);
            } else {
                ok = false;
            }
            if (ok) {
                const v3<float> gm = mk3(o[33], o[34], o[35]);
                part += o[32] * w + cross(gm, w);
            } else {  // FP64: the reference's far switch and kernel for this pair
                const BodySrc& b = a.src64[t0 + k];
                SrcKern<double> K64 = kern_from<double>(b);
                const v3<double> w64 = sv_rel(K64, x - mk3(b.c[0], b.c[1], b.c[2]), 0, a.kernel_far, 1e-12);
                acc += b.sigma * w64 + cross(mk3(b.gam[0], b.gam[1], b.gam[2]), w64);
            }
        }
        acc += mk3(double(part.x), double(part.y), double(part.z));
    }
    if (!valid) return;
    double* out = a.out + (size_t(blockIdx.y) * a.npts + i) * 3;
    out[0] = acc.x;
    out[1] = acc.y;
    out[2] = acc.z;
}

// ---- 3. the loads --------------------------------------------------------------------------------------------------

// dmu/dt by backward difference (zero on the first step), the sheets gamma of the body triangles from mu
// (sheet_strengths, Post.jl:19-23) into the body-velocity sources
__global__ void body_state_kernel(int ntri, int nslot, const TriGeo* __restrict__ tg, const double* __restrict__ mu,
                                  const double* __restrict__ mu_prev, double inv_dt, int first, double* __restrict__ dmu,
                                  BodySrc* __restrict__ bs) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nslot) dmu[i] = first ? 0.0 : (mu[i] - mu_prev[i]) * inv_dt;
    if (i < ntri) {
        const TriGeo& g = tg[i];
        const double m0 = mu[g.slot[0]], m1 = mu[g.slot[1]], m2 = mu[g.slot[2]];
        for (int z = 0; z < 3; ++z) bs[i].gam[z] = m0 * g.gam[z] + m1 * g.gam[3 + z] + m2 * g.gam[6 + z];
    }
}

// sum of v over the block in a fixed order; every thread gets it
__device__ double bsum(double v, double* sh) {
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

__device__ double bmax(double v, double* sh) {
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

// the total vorticity Omega = sum alpha and impulse I = 1/2 sum x x alpha (vorticity_moments, state.jl:381-385) of
// the body's sheets as blobs (centroid, gamma A) and of the blob list, per block; then in block order
__global__ void __launch_bounds__(256) moments_kernel(int ntri, const TriGeo* __restrict__ tg,
                                                      const BodySrc* __restrict__ bs, int nblob,
                                                      const double* __restrict__ blobs, double* __restrict__ part) {
    __shared__ double sh[33];
    const int i = blockIdx.x * 256 + threadIdx.x;
    v3<double> x = mk3(0.0, 0.0, 0.0), al = mk3(0.0, 0.0, 0.0);
    if (i < ntri) {
        x = ld3(tg[i].c);
        al = tg[i].area * mk3(bs[i].gam[0], bs[i].gam[1], bs[i].gam[2]);
    } else if (i < ntri + nblob) {
        const double* b = blobs + 7 * size_t(i - ntri);
        x = ld3(b);
        al = ld3(b + 3);
    }
    const v3<double> I = cross(x, al) / 2.0;
    const double v[6] = {al.x, al.y, al.z, I.x, I.y, I.z};
    for (int k = 0; k < 6; ++k) {
        const double s = bsum(v[k], sh);
        if (threadIdx.x == 0) part[6 * size_t(blockIdx.x) + k] = s;
    }
}

// out[0..6): the moments' blocks summed in order; out[6..9): the Kutta-Joukowski circulation vector
// G = sum over the trailing edge segments of (mu_a + mu_b)/2 (x_b - x_a) (kutta_joukowski_force, forces.jl:34-39)
__global__ void finish_loads_kernel(int nblock, const double* __restrict__ part, int nseg, const int* __restrict__ seg,
                                    const double* __restrict__ tex, const double* __restrict__ muw,
                                    double* __restrict__ out) {
    const int k = threadIdx.x;
    if (k < 6) {
        double v = 0.0;
        for (int b = 0; b < nblock; ++b) v += part[6 * size_t(b) + k];
        out[k] = v;
    } else if (k < 9) {
        const int z = k - 6;
        double v = 0.0;
        for (int s = 0; s < nseg; ++s) {
            const int ia = seg[2 * s], ib = seg[2 * s + 1];
            v += (muw[ia] + muw[ib]) / 2 * (tex[3 * ib + z] - tex[3 * ia + z]);
        }
        out[k] = v;
    }
}

// ---- 4. velocities and forward Euler ------------------------------------------------------------------------------

struct PointArgs {
    int nr, head, R, nte, npart;
    double* rx;    // ring rows
    double* part;  // particles
    double* X;     // nr nte + npart points
};

// the free nodes (rows newest first) and the particles as one list of points
__global__ void gather_points_kernel(PointArgs a) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int nn = a.nr * a.nte;
    if (k < nn) {
        const int i = k / a.nte, j = k % a.nte;
        const double* p = a.rx + (size_t((a.head + i) % a.R) * a.nte + j) * 3;
        for (int z = 0; z < 3; ++z) a.X[3 * size_t(k) + z] = p[z];
    } else if (k < nn + a.npart) {
        const double* p = a.part + 7 * size_t(k - nn);
        for (int z = 0; z < 3; ++z) a.X[3 * size_t(k) + z] = p[z];
    }
}

// U = V + body + blobs (or V alone for a prescribed wake); x += dt U on the rows and particles; the blocks' max |U|
__global__ void __launch_bounds__(256) advect_kernel(PointArgs a, double vx, double vy, double vz, int freestream,
                                                     double dt, const double* __restrict__ ub,
                                                     const double* __restrict__ uw, double* __restrict__ umax_part) {
    __shared__ double sh[33];
    const int k = blockIdx.x * 256 + threadIdx.x;
    const int nn = a.nr * a.nte;
    double um = 0.0;
    if (k < nn + a.npart) {
        double U[3] = {vx, vy, vz};
        if (!freestream)
            for (int z = 0; z < 3; ++z) U[z] += ub[3 * size_t(k) + z] + uw[3 * size_t(k) + z];
        double* p = k < nn ? a.rx + (size_t((a.head + k / a.nte) % a.R) * a.nte + k % a.nte) * 3
                           : a.part + 7 * size_t(k - nn);
        for (int z = 0; z < 3; ++z) p[z] += dt * U[z];
        um = sqrt(U[0] * U[0] + U[1] * U[1] + U[2] * U[2]);
    }
    um = bmax(um, sh);
    if (threadIdx.x == 0) umax_part[blockIdx.x] = um;
}

__global__ void max_parts_kernel(int n, const double* __restrict__ part, double* __restrict__ out) {
    if (threadIdx.x != 0) return;
    double m = 0.0;
    for (int i = 0; i < n; ++i) m = fmax(m, part[i]);
    *out = m;
}

// a new R0: the trailing edge panel's downstream edge, shed with this step's mu_w
__global__ void shed_kernel(int nte, int row, const double* __restrict__ edge, const double* __restrict__ muw,
                            double* __restrict__ rx, double* __restrict__ rmu) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nte) return;
    for (int z = 0; z < 3; ++z) rx[(size_t(row) * nte + k) * 3 + z] = edge[3 * k + z];
    rmu[size_t(row) * nte + k] = muw[k];
}

// ---- 5. conversion, merging and deletion (single block; the particle count stays on the device) -----------------

struct BookArgs {
    int nte, R, up, down;   // ring rows of the converted panel row's upstream and downstream node rows
    double* rx;
    double* rmu;
    double* mul;
    int nstrip, nfirst, nlast;
    const int* strips;
    const int* first;
    const int* last;
    const int* merge;       // per strip, or null
    CoreDev core;
    int cap;
    int* np;                // particle count (device)
    double* part;
    int* tag;
    signed char* group;
    int* brows;
    double* blen;
    double* bwid;
    int* err;               // set to 1 when the particles would exceed the capacity
    double delete_limit, d[3];
};

// stable in-place removal of the particles for which drop() holds (keep_particles!, state.jl:150-155); returns the
// new count (every thread)
template <class Drop>
__device__ int compact(const BookArgs& a, int n, Drop drop) {
    __shared__ int s_scan[BK_THREADS];
    __shared__ int s_base;
    if (threadIdx.x == 0) s_base = 0;
    __syncthreads();
    for (int c0 = 0; c0 < n; c0 += BK_THREADS) {
        const int i = c0 + threadIdx.x;
        const bool keep = i < n && !drop(i);
        double pv[7];
        int tg = 0;
        signed char gr = 0;
        if (keep) {
            for (int z = 0; z < 7; ++z) pv[z] = a.part[7 * size_t(i) + z];
            tg = a.tag[i];
            gr = a.group[i];
        }
        s_scan[threadIdx.x] = keep ? 1 : 0;
        __syncthreads();
        for (int o = 1; o < BK_THREADS; o <<= 1) {  // inclusive scan (Hillis-Steele)
            const int v = threadIdx.x >= o ? s_scan[threadIdx.x - o] : 0;
            __syncthreads();
            s_scan[threadIdx.x] += v;
            __syncthreads();
        }
        const int pos = s_base + s_scan[threadIdx.x] - 1;
        if (keep) {
            for (int z = 0; z < 7; ++z) a.part[7 * size_t(pos) + z] = pv[z];
            a.tag[pos] = tg;
            a.group[pos] = gr;
        }
        __syncthreads();
        if (threadIdx.x == BK_THREADS - 1) s_base += s_scan[BK_THREADS - 1];
        __syncthreads();
    }
    const int r = s_base;
    __syncthreads();
    return r;
}

// merge_strip! (state.jl:352-373): strip s's batch into one particle per side of the merged quad's diagonal, the sum
// of the strengths at their strength-weighted centre, with the core of the merged quad
__device__ void merge_strip(const BookArgs& a, int s) {
    __shared__ double sh[33];
    const int n = *a.np;
    double acc[2][11];  // per group: alpha (3), sum w, sum w x (3), sum x (3), count
    for (int g = 0; g < 2; ++g)
        for (int z = 0; z < 11; ++z) acc[g][z] = 0.0;
    for (int i = threadIdx.x; i < n; i += BK_THREADS) {
        if (a.tag[i] != s + 1) continue;
        const int g = a.group[i] == 1 ? 0 : 1;
        const double* p = a.part + 7 * size_t(i);
        const double w = sqrt(p[3] * p[3] + p[4] * p[4] + p[5] * p[5]);
        for (int z = 0; z < 3; ++z) {
            acc[g][z] += p[3 + z];
            acc[g][4 + z] += w * p[z];
            acc[g][7 + z] += p[z];
        }
        acc[g][3] += w;
        acc[g][10] += 1.0;
    }
    for (int g = 0; g < 2; ++g)
        for (int z = 0; z < 11; ++z) acc[g][z] = bsum(acc[g][z], sh);
    const double W = a.bwid[s], L = a.blen[s];
    const v3<double> o = mk3(0.0, 0.0, 0.0);
    const double delta = core_tri(a.core, o, mk3(W, 0.0, 0.0), mk3(W, L, 0.0));
    int m = compact(a, n, [&](int i) { return a.tag[i] == s + 1; });
    if (threadIdx.x == 0) {
        for (int g = 0; g < 2; ++g) {
            if (acc[g][10] == 0.0) continue;
            v3<double> x = acc[g][3] > 0 ? mk3(acc[g][4], acc[g][5], acc[g][6]) / acc[g][3]
                                         : mk3(acc[g][7], acc[g][8], acc[g][9]) / acc[g][10];
            put_blob(a.part + 7 * size_t(m), x, mk3(acc[g][0], acc[g][1], acc[g][2]), delta);
            a.tag[m] = 0;
            a.group[m] = 0;
            ++m;
        }
        *a.np = m;
        a.brows[s] = 0;
        a.blen[s] = 0.0;
    }
    __syncthreads();
}

// convert_oldest! (state.jl:300-343): the oldest panel row (node rows up and down) into particles; the caller drops
// the downstream node row afterwards
__global__ void __launch_bounds__(BK_THREADS) convert_kernel(BookArgs a) {
    __shared__ int s_scan[BK_THREADS];
    __shared__ int s_nfar;
    __shared__ int s_np0;
    if (threadIdx.x == 0) {
        s_nfar = 0;
        s_np0 = *a.np;
    }
    __syncthreads();
    const int np0 = s_np0;
    auto X = [&](int row, int k) {
        const double* p = a.rx + (size_t(row) * a.nte + k) * 3;
        return mk3(p[0], p[1], p[2]);
    };
    auto M = [&](int row, int k) { return a.rmu[size_t(row) * a.nte + k]; };
    // the far end's filaments with a strength (mu - mu_line nonzero at either end), counted
    for (int c0 = 0; c0 < a.nstrip; c0 += BK_THREADS) {
        const int s = c0 + threadIdx.x;
        int f = 0;
        if (s < a.nstrip) {
            const int A = a.strips[2 * s], B = a.strips[2 * s + 1];
            f = (M(a.down, A) - a.mul[A] != 0.0 || M(a.down, B) - a.mul[B] != 0.0) ? 1 : 0;
        }
        const int v = __syncthreads_count(f);
        if (threadIdx.x == 0) s_nfar += v;
        __syncthreads();
    }
    const int ntip = a.nfirst + a.nlast;
    const int total = 2 * a.nstrip + 2 * ntip + 2 * s_nfar;
    if (np0 + total > a.cap) {
        if (threadIdx.x == 0) *a.err = 1;
        return;
    }
    // sheet particles, two per strip in strip order, with the merge tags
    for (int s = threadIdx.x; s < a.nstrip; s += BK_THREADS) {
        const int A = a.strips[2 * s], B = a.strips[2 * s + 1];
        const int u = a.up, d = a.down;
        double* o = a.part + 7 * (size_t(np0) + 2 * s);
        sheet_blob(a.core, X(u, A), X(d, A), X(u, B), M(u, A), M(d, A), M(u, B), o);
        sheet_blob(a.core, X(d, A), X(d, B), X(u, B), M(d, A), M(d, B), M(u, B), o + 7);
        const int k = a.merge ? a.merge[s] : 1;
        for (int h = 0; h < 2; ++h) {
            int tg = 0;
            signed char gr = 0;
            if (k > 1) {
                const int mrow = k - a.brows[s];
                const double uu = h == 0 ? 1.0 / 3 : 2.0 / 3, vv = uu;
                tg = s + 1;
                gr = uu + (mrow - 1 + vv) / k < 1 ? 1 : 2;
            }
            a.tag[np0 + 2 * s + h] = tg;
            a.group[np0 + 2 * s + h] = gr;
        }
        if (k > 1) {
            a.brows[s] += 1;
            a.blen[s] += (vnorm(X(d, A) - X(u, A)) + vnorm(X(d, B) - X(u, B))) / 2;
            a.bwid[s] = vnorm(X(u, B) - X(u, A));
        }
    }
    // tip sides: first nodes upstream (down -> up), last nodes downstream (up -> down)
    for (int k = threadIdx.x; k < ntip; k += BK_THREADS) {
        double* o = a.part + 7 * (size_t(np0) + 2 * a.nstrip + 2 * k);
        if (k < a.nfirst) {
            const int nd = a.first[k];
            segment_blob_pair(a.core, X(a.down, nd), X(a.up, nd), M(a.down, nd), M(a.up, nd), o);
        } else {
            const int nd = a.last[k - a.nfirst];
            segment_blob_pair(a.core, X(a.up, nd), X(a.down, nd), M(a.up, nd), M(a.down, nd), o);
        }
        for (int h = 0; h < 2; ++h) {
            a.tag[np0 + 2 * a.nstrip + 2 * k + h] = 0;
            a.group[np0 + 2 * a.nstrip + 2 * k + h] = 0;
        }
    }
    // far end, B -> A, the strips with a strength in strip order (an exclusive scan gives each its place)
    int base = 0;
    for (int c0 = 0; c0 < a.nstrip; c0 += BK_THREADS) {
        const int s = c0 + threadIdx.x;
        int f = 0;
        double gA = 0, gB = 0;
        int A = 0, B = 0;
        if (s < a.nstrip) {
            A = a.strips[2 * s], B = a.strips[2 * s + 1];
            gA = M(a.down, A) - a.mul[A];
            gB = M(a.down, B) - a.mul[B];
            f = (gA != 0.0 || gB != 0.0) ? 1 : 0;
        }
        s_scan[threadIdx.x] = f;
        __syncthreads();
        for (int o = 1; o < BK_THREADS; o <<= 1) {
            const int v = threadIdx.x >= o ? s_scan[threadIdx.x - o] : 0;
            __syncthreads();
            s_scan[threadIdx.x] += v;
            __syncthreads();
        }
        if (f) {
            const int pos = np0 + 2 * a.nstrip + 2 * ntip + 2 * (base + s_scan[threadIdx.x] - 1);
            segment_blob_pair(a.core, X(a.down, B), X(a.down, A), gB, gA, a.part + 7 * size_t(pos));
            for (int h = 0; h < 2; ++h) {
                a.tag[pos + h] = 0;
                a.group[pos + h] = 0;
            }
        }
        __syncthreads();
        base += s_scan[BK_THREADS - 1];
        __syncthreads();
    }
    // mu_line takes the converted row's upstream doublets
    for (int k = threadIdx.x; k < a.nte; k += BK_THREADS) a.mul[k] = M(a.up, k);
    __syncthreads();
    if (threadIdx.x == 0) *a.np = np0 + total;
    __syncthreads();
    if (a.merge)
        for (int s = 0; s < a.nstrip; ++s)
            if (a.merge[s] > 1 && a.brows[s] >= a.merge[s]) merge_strip(a, s);
}

// delete_far! (step.jl:190-195): the particles beyond the limit downstream of the trailing edge
__global__ void __launch_bounds__(BK_THREADS) delete_far_kernel(BookArgs a) {
    const int n = *a.np;
    const int m = compact(a, n, [&](int i) {
        const double* p = a.part + 7 * size_t(i);
        return !(p[0] * a.d[0] + p[1] * a.d[1] + p[2] * a.d[2] <= a.delete_limit);
    });
    if (threadIdx.x == 0) *a.np = m;
}

template <class T>
void free_all(T& v) {
    for (void* p : v) cudaFree(p);
    v.clear();
}

}  // namespace

// ---------------------------------------------------------------------------------------------------------------------

struct vp_freewake {
    vp_ctx* ctx = nullptr;
    vp_freewake_setup s{};  // scalars of the set-up (its pointers are not kept)
    const vp_factor* F = nullptr;
    CoreDev core{};
    int R = 0;  // ring rows
    int ntri = 0, nslot = 0, nq = 0, nte = 0, nstrip = 0, nfirst = 0, nlast = 0, npt = 0, npf = 0, nteseg = 0;
    double V[3] = {0, 0, 0}, d[3] = {0, 0, 0};
    std::vector<void*> owned;
    // body and maps
    TriGeo* tg = nullptr;
    BodySrc* bs = nullptr;
    double *corners = nullptr, *b0 = nullptr;
    int *slot = nullptr, *sg_ptr = nullptr, *sg_ent = nullptr;
    int *Cp = nullptr, *Ci = nullptr, *Kp = nullptr, *Ki = nullptr;
    double *Cv = nullptr, *Kv = nullptr;
    double* tex = nullptr;
    int* teseg = nullptr;
    int *strips = nullptr, *first = nullptr, *last = nullptr, *merge = nullptr;
    double* edge = nullptr;
    double* pwx = nullptr;
    int *pwte = nullptr, *pt = nullptr, *pf = nullptr;
    RulePt* rule[5] = {};
    float4* rulef[5] = {};
    int nrule[5] = {};
    // state
    double *rx = nullptr, *rmu = nullptr, *mul = nullptr;
    int head = 0, nrows = 0, conversions = 0, n = 0, np = 0;
    double t = 0;
    int cap = 0;
    double* part = nullptr;
    int* tag = nullptr;
    signed char* group = nullptr;
    int* brows = nullptr;
    double *blen = nullptr, *bwid = nullptr;
    int* d_np = nullptr;
    int* d_err = nullptr;
    // per-step work
    int ns_cap = 0, nsg_cap = 0, nteblob = 0;
    TriGeo* sheet = nullptr;
    double *sheet_G = nullptr, *seg = nullptr;
    int* sheet_ok = nullptr;
    double *blobs = nullptr, *X = nullptr, *ub = nullptr, *uw = nullptr, *umax_part = nullptr;
    double *trow = nullptr, *rhs = nullptr, *x = nullptr, *mu = nullptr, *mu_prev = nullptr, *dmu = nullptr;
    double *cp = nullptr, *surf_part = nullptr, *mom_part = nullptr, *rec = nullptr;
    // the mixed path's FP32 N-body kernels: the particles as FP32 splits, the chunks' partial sums, the body sources
    float4 *ph = nullptr, *pl = nullptr, *pa = nullptr;
    double *prhs = nullptr, *bvel = nullptr;
    float* src32 = nullptr;  // rec: the record (see step)
    SolveWork sw;
    double I_prev[3] = {0, 0, 0};
    std::vector<double> h_rec;
};

namespace {

template <class T>
int own_alloc(vp_freewake* fw, T** p, size_t n) {
    int r = vp_alloc(fw->ctx, p, n);
    if (!r) fw->owned.push_back((void*)*p);
    return r;
}

template <class T>
int own_up(vp_freewake* fw, T** p, const T* h, size_t n) {
    int r = vp_upload(fw->ctx, p, h, n);
    if (!r) fw->owned.push_back((void*)*p);
    return r;
}

// the blob list's and the point list's sizes for a particle capacity
size_t blob_cap(const vp_freewake* fw, int cap) {
    return size_t(fw->nteblob) + size_t(fw->ns_cap) + 2 * size_t(fw->nsg_cap) + size_t(cap);
}
size_t point_cap(const vp_freewake* fw, int cap) { return size_t(fw->R) * fw->nte + size_t(cap); }

void release(void* p, std::vector<void*>& owned) {
    for (auto& q : owned)
        if (q == p) {
            cudaFree(q);
            q = nullptr;
        }
}

// grow the particle arrays (and the lists sized by them) to hold at least `need` particles
int ensure_capacity(vp_freewake* fw, int need) {
    if (need <= fw->cap) return VP_OK;
    vp_ctx* ctx = fw->ctx;
    const int cap = std::max(need, 2 * fw->cap);
    double *part, *blobs, *X, *ub, *uw, *umax_part, *mom_part, *prhs, *bvel;
    float4 *ph, *pl, *pa;
    int* tag;
    signed char* group;
    int r;
    const size_t nb = blob_cap(fw, cap), npnt = point_cap(fw, cap);
    const size_t pchunks = (size_t(cap) + NB_CHUNK - 1) / NB_CHUNK, bchunks = (size_t(fw->ntri) + NB_CHUNK - 1) / NB_CHUNK;
    if ((r = own_alloc(fw, &part, 7 * size_t(cap))) || (r = own_alloc(fw, &tag, size_t(cap))) ||
        (r = own_alloc(fw, &group, size_t(cap))) || (r = own_alloc(fw, &blobs, 7 * nb)) ||
        (r = own_alloc(fw, &X, 3 * npnt)) || (r = own_alloc(fw, &ub, 3 * npnt)) || (r = own_alloc(fw, &uw, 3 * npnt)) ||
        (r = own_alloc(fw, &umax_part, (npnt + 255) / 256 + 1)) ||
        (r = own_alloc(fw, &mom_part, 6 * ((size_t(fw->ntri) + nb + 255) / 256 + 1))) ||
        (r = own_alloc(fw, &ph, size_t(cap))) || (r = own_alloc(fw, &pl, size_t(cap))) ||
        (r = own_alloc(fw, &pa, size_t(cap))) || (r = own_alloc(fw, &prhs, pchunks * fw->ntri * 3)) ||
        (r = own_alloc(fw, &bvel, bchunks * npnt * 3)))
        return r;
    if (fw->np > 0) {
        VP_CUDA(ctx, cudaMemcpyAsync(part, fw->part, sizeof(double) * 7 * fw->np, cudaMemcpyDeviceToDevice, ctx->stream));
        VP_CUDA(ctx, cudaMemcpyAsync(tag, fw->tag, sizeof(int) * fw->np, cudaMemcpyDeviceToDevice, ctx->stream));
        VP_CUDA(ctx, cudaMemcpyAsync(group, fw->group, fw->np, cudaMemcpyDeviceToDevice, ctx->stream));
    }
    VP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    for (void* p : {(void*)fw->part, (void*)fw->tag, (void*)fw->group, (void*)fw->blobs, (void*)fw->X, (void*)fw->ub,
                    (void*)fw->uw, (void*)fw->umax_part, (void*)fw->mom_part, (void*)fw->ph, (void*)fw->pl,
                    (void*)fw->pa, (void*)fw->prhs, (void*)fw->bvel})
        if (p) release(p, fw->owned);
    fw->part = part, fw->tag = tag, fw->group = group, fw->blobs = blobs, fw->X = X, fw->ub = ub, fw->uw = uw;
    fw->umax_part = umax_part, fw->mom_part = mom_part, fw->ph = ph, fw->pl = pl, fw->pa = pa, fw->prhs = prhs;
    fw->bvel = bvel;
    fw->cap = cap;
    return VP_OK;
}

int csr_check(int nrow, int ncol, const int* p, const int* c, const double* v) {
    if (!p || !v || p[0] != 0) return 0;
    for (int i = 0; i < nrow; ++i)
        if (p[i + 1] < p[i]) return 0;
    for (int k = 0; k < p[nrow]; ++k)
        if (!c || c[k] < 0 || c[k] >= ncol) return 0;
    return 1;
}

NearArgs wake_near_args(const vp_freewake* fw, const vp_assembly_options& o) {
    NearArgs na{};
    na.tri = fw->tg;
    na.wtri = fw->sheet;
    na.ntri = fw->ntri;
    na.nslot = fw->nslot;
    for (int k = 0; k < 5; ++k) {
        na.rule[k] = fw->rule[k];
        na.rulef[k] = fw->rulef[k];
        na.nrule[k] = fw->nrule[k];
    }
    na.test_mode = o.test;
    na.near_depth = o.near_depth;
    na.mixed = o.precision == VP_MIXED ? 1 : 0;
    na.far_ratio = o.far_ratio;
    na.near_ratio = o.near_ratio;
    na.corner_angle = o.corner_angle;
    na.contact_rel = o.contact_rel;
    na.kernel_far = o.kernel_far;
    na.kernel_far32 = float(o.kernel_far);
    for (int k = 0; k < 3; ++k) {
        na.vinf[k] = fw->V[k];
        na.tint[k] = o.test == 1 ? 1.0 : 1.0 / 3;
    }
    return na;
}

}  // namespace

extern "C" void vp_freewake_free(vp_freewake* fw) {
    if (!fw) return;
    if (fw->ctx) {
        cudaSetDevice(fw->ctx->device);
        cudaStreamSynchronize(fw->ctx->stream);
    }
    free_all(fw->owned);
    vp_solve_work_free(&fw->sw);
    delete fw;
}

extern "C" int vp_freewake_create(vp_ctx* ctx, const vp_freewake_setup* s, vp_freewake** out) {
    if (!ctx || !s || !out) return vp_fail(ctx, VP_ERR_ARG, "null argument");
    *out = nullptr;
    const vp_assembly_options& o = s->assembly;
    if (!(s->dt > 0) || s->keep_rows < 0 || s->core_mode < 0 || s->core_mode > 2 || !(s->overlap > 0) ||
        !(s->core_factor > 0) || (s->core_mode == 2 && !(s->core_value > 0)) || (s->advection != 0 && s->advection != 1))
        return vp_fail(ctx, VP_ERR_ARG, "free wake option out of range");
    if (o.precision != VP_FP64 && o.precision != VP_MIXED) return vp_fail(ctx, VP_ERR_ARG, "unknown precision");
    if (o.test < 0 || o.test > 2 || !(o.far_ratio > 0) || !(o.kernel_far > 0) || o.near_depth < 0 || o.near_depth > 9)
        return vp_fail(ctx, VP_ERR_ARG, "assembly option out of range");
    if (!s->factor || !s->b0 || !s->x || !s->tris || !s->corner_slot || !s->sigma || !s->vinf || !s->edge ||
        s->ntri <= 0 || s->nslot <= 0 || s->nnode <= 0 || s->nq <= 0 || s->nte <= 0 || s->nstrip <= 0 ||
        s->nfirst < 0 || s->nlast < 0 || s->npw < 0 || s->npt < 0 || s->npf < 0 || s->nline < 0 ||
        (s->nstrip > 0 && !s->strips) || (s->nfirst > 0 && !s->first_nodes) || (s->nlast > 0 && !s->last_nodes) ||
        (s->npw > 0 && (!s->pw_x || !s->pw_te)) || (s->npt > 0 && !s->pt_tris) || (s->npf > 0 && !s->pf) ||
        !s->te_x || (s->nline > 0 && (!s->line_ptr || !s->line_nodes || !s->line_closed)))
        return vp_fail(ctx, VP_ERR_ARG, "bad argument");
    const vp_factor* F = s->factor;
    if (F->nslot != s->nslot || F->nq != s->nq) return vp_fail(ctx, VP_ERR_ARG, "factorization does not match the slots");
    for (int i = 0; i < 3 * s->ntri; ++i)
        if (s->tris[i] < 0 || s->tris[i] >= s->nnode || s->corner_slot[i] < 0 || s->corner_slot[i] >= s->nslot)
            return vp_fail(ctx, VP_ERR_ARG, "triangle node or slot out of range");
    if (!csr_check(s->nslot, s->nq, s->C_rowptr, s->C_col, s->C_val) ||
        !csr_check(s->nte, s->nq, s->K_rowptr, s->K_col, s->K_val))
        return vp_fail(ctx, VP_ERR_ARG, "C or K is not a valid CSR matrix");
    for (int i = 0; i < 2 * s->nstrip; ++i)
        if (s->strips[i] < 0 || s->strips[i] >= s->nte) return vp_fail(ctx, VP_ERR_ARG, "strip node out of range");
    for (int i = 0; i < s->nfirst; ++i)
        if (s->first_nodes[i] < 0 || s->first_nodes[i] >= s->nte) return vp_fail(ctx, VP_ERR_ARG, "tip node out of range");
    for (int i = 0; i < s->nlast; ++i)
        if (s->last_nodes[i] < 0 || s->last_nodes[i] >= s->nte) return vp_fail(ctx, VP_ERR_ARG, "tip node out of range");
    for (int i = 0; i < s->npw; ++i)
        if (s->pw_te[i] < 0 || s->pw_te[i] >= s->nte) return vp_fail(ctx, VP_ERR_ARG, "panel node out of range");
    for (int i = 0; i < 3 * s->npt; ++i)
        if (s->pt_tris[i] < 0 || s->pt_tris[i] >= s->npw) return vp_fail(ctx, VP_ERR_ARG, "panel triangle out of range");
    for (int i = 0; i < 2 * s->npf; ++i)
        if (s->pf[i] < 0 || s->pf[i] >= s->npw) return vp_fail(ctx, VP_ERR_ARG, "panel filament out of range");
    if (s->merge)
        for (int i = 0; i < s->nstrip; ++i)
            if (s->merge[i] < 1) return vp_fail(ctx, VP_ERR_ARG, "merge rows must be at least 1");
    const double V2 = s->vinf[0] * s->vinf[0] + s->vinf[1] * s->vinf[1] + s->vinf[2] * s->vinf[2];
    if (!(V2 > 0)) return vp_fail(ctx, VP_ERR_ARG, "V∞ must not be zero");
    DeviceGuard dg;
    if (dg.set(ctx->device) != cudaSuccess) return vp_fail(ctx, VP_ERR_CUDA, "cudaSetDevice");

    vp_freewake* fw = new vp_freewake();
    fw->ctx = ctx;
    fw->s = *s;
    fw->F = F;
    fw->core = CoreDev{s->core_mode, s->overlap, s->core_factor, s->core_floor, s->core_value};
    fw->R = s->keep_rows + 2;
    fw->ntri = s->ntri, fw->nslot = s->nslot, fw->nq = s->nq, fw->nte = s->nte, fw->nstrip = s->nstrip;
    fw->nfirst = s->nfirst, fw->nlast = s->nlast, fw->npt = s->npt, fw->npf = s->npf;
    for (int z = 0; z < 3; ++z) {
        fw->V[z] = s->vinf[z];
        fw->d[z] = s->vinf[z] / std::sqrt(V2);
    }
    auto fail = [&](int r) {
        vp_freewake_free(fw);
        return r;
    };
    int r;
    // body element data, the body-velocity sources, corners, slots and each slot's corners (a fixed order)
    std::vector<TriGeo> tg(s->ntri);
    std::vector<BodySrc> bs(s->ntri);
    std::vector<double> corners(9 * size_t(s->ntri));
    for (int t = 0; t < s->ntri; ++t) {
        const int* tr = s->tris + 3 * t;
        if (!make_tri(s->x + 3 * tr[0], s->x + 3 * tr[1], s->x + 3 * tr[2], tg[t]))
            return fail(vp_fail(ctx, VP_ERR_DEGENERATE, "degenerate triangle " + std::to_string(t)));
        for (int k = 0; k < 3; ++k) {
            tg[t].node[k] = tr[k];
            tg[t].slot[k] = s->corner_slot[3 * t + k];
        }
        tg[t].sigma = s->sigma[t];
        BodySrc& b = bs[t];
        for (int k = 0; k < 3; ++k) {
            b.c[k] = tg[t].c[k];
            b.len[k] = tg[t].len[k];
            b.n[k] = tg[t].n[k];
            b.gam[k] = 0.0;
        }
        for (int k = 0; k < 9; ++k) {
            b.d[k] = tg[t].x[k] - tg[t].c[k % 3];
            b.nu[k] = tg[t].nu[k];
            corners[9 * size_t(t) + k] = tg[t].x[k];
        }
        b.area = tg[t].area;
        b.diam = tg[t].diam;
        b.sigma = s->sigma[t];
    }
    std::vector<int> sp(s->nslot + 1, 0), se(3 * size_t(s->ntri));
    for (int i = 0; i < 3 * s->ntri; ++i) sp[s->corner_slot[i] + 1]++;
    for (int k = 0; k < s->nslot; ++k) sp[k + 1] += sp[k];
    {
        std::vector<int> fill(sp.begin(), sp.end() - 1);
        for (int i = 0; i < 3 * s->ntri; ++i) se[fill[s->corner_slot[i]]++] = i;
    }
    // the trailing edge lines' segments (Kutta-Joukowski)
    std::vector<int> teseg;
    for (int L = 0; L < s->nline; ++L) {
        const int p0 = s->line_ptr[L], m = s->line_ptr[L + 1] - p0;
        for (int i = 0; i < m; ++i)
            if (s->line_nodes[p0 + i] < 0 || s->line_nodes[p0 + i] >= s->nte)
                return fail(vp_fail(ctx, VP_ERR_ARG, "trailing edge line node out of range"));
        const int nseg = s->line_closed[L] ? m : m - 1;
        for (int i = 0; i < nseg; ++i) {
            teseg.push_back(s->line_nodes[p0 + i]);
            teseg.push_back(s->line_nodes[p0 + (i + 1) % m]);
        }
    }
    fw->nteseg = int(teseg.size() / 2);
    if (teseg.empty()) teseg = {0, 0};
    // rules (rules.jl), as the assembly builds them
    std::vector<RulePt> rl[5] = {triangle_rule(o.near_points), {}, edge_rule(o.touch_levels, o.touch_ratio, o.touch_order),
                                 vertex_rule_base(o.touch_levels, o.touch_ratio, o.touch_order), triangle_rule(o.far_points)};
    rl[R_SELF] = self_rule(rl[R_EDGE]);
    const int nnz_c = s->C_rowptr[s->nslot], nnz_k = s->K_rowptr[s->nte];
    std::vector<int> Ci(s->C_col, s->C_col + std::max(nnz_c, 1) * (nnz_c > 0)), Ki(s->K_col, s->K_col + nnz_k);
    if (Ci.empty()) Ci = {0};
    if (Ki.empty()) Ki = {0};
    std::vector<double> Cv(s->C_val, s->C_val + nnz_c), Kv(s->K_val, s->K_val + nnz_k);
    if (Cv.empty()) Cv = {0.0};
    if (Kv.empty()) Kv = {0.0};
    std::vector<int> strips(s->strips, s->strips + 2 * s->nstrip);
    std::vector<int> first(s->first_nodes ? s->first_nodes : strips.data(),
                           (s->first_nodes ? s->first_nodes : strips.data()) + std::max(s->nfirst, 1));
    std::vector<int> last(s->last_nodes ? s->last_nodes : strips.data(),
                          (s->last_nodes ? s->last_nodes : strips.data()) + std::max(s->nlast, 1));
    std::vector<double> pwx(s->npw ? s->pw_x : s->edge, (s->npw ? s->pw_x : s->edge) + 3 * std::max(s->npw, 1));
    std::vector<int> pwte(std::max(s->npw, 1), 0), pt(3 * std::max(s->npt, 1), 0), pf(2 * std::max(s->npf, 1), 0);
    std::copy(s->pw_te, s->pw_te + s->npw, pwte.begin());
    std::copy(s->pt_tris, s->pt_tris + 3 * s->npt, pt.begin());
    std::copy(s->pf, s->pf + 2 * s->npf, pf.begin());
    if ((r = own_up(fw, &fw->tg, tg.data(), tg.size())) || (r = own_up(fw, &fw->bs, bs.data(), bs.size())) ||
        (r = own_up(fw, &fw->corners, corners.data(), corners.size())) ||
        (r = own_up(fw, &fw->slot, s->corner_slot, 3 * size_t(s->ntri))) ||
        (r = own_up(fw, &fw->sg_ptr, sp.data(), sp.size())) || (r = own_up(fw, &fw->sg_ent, se.data(), se.size())) ||
        (r = own_up(fw, &fw->b0, s->b0, size_t(s->nslot))) ||
        (r = own_up(fw, &fw->Cp, s->C_rowptr, size_t(s->nslot) + 1)) || (r = own_up(fw, &fw->Ci, Ci.data(), Ci.size())) ||
        (r = own_up(fw, &fw->Cv, Cv.data(), Cv.size())) || (r = own_up(fw, &fw->Kp, s->K_rowptr, size_t(s->nte) + 1)) ||
        (r = own_up(fw, &fw->Ki, Ki.data(), Ki.size())) || (r = own_up(fw, &fw->Kv, Kv.data(), Kv.size())) ||
        (r = own_up(fw, &fw->tex, s->te_x, 3 * size_t(s->nte))) ||
        (r = own_up(fw, &fw->teseg, teseg.data(), teseg.size())) ||
        (r = own_up(fw, &fw->strips, strips.data(), strips.size())) ||
        (r = own_up(fw, &fw->first, first.data(), first.size())) || (r = own_up(fw, &fw->last, last.data(), last.size())) ||
        (r = own_up(fw, &fw->edge, s->edge, 3 * size_t(s->nte))) || (r = own_up(fw, &fw->pwx, pwx.data(), pwx.size())) ||
        (r = own_up(fw, &fw->pwte, pwte.data(), pwte.size())) || (r = own_up(fw, &fw->pt, pt.data(), pt.size())) ||
        (r = own_up(fw, &fw->pf, pf.data(), pf.size())))
        return fail(r);
    if (s->merge && (r = own_up(fw, &fw->merge, s->merge, size_t(s->nstrip)))) return fail(r);
    for (int k = 0; k < 5; ++k) {
        if (rl[k].empty()) rl[k].push_back(RulePt{1.0 / 3, 1.0 / 3, 1.0 / 3, 0.0});
        std::vector<float4> f(rl[k].size());
        for (size_t i = 0; i < rl[k].size(); ++i)
            f[i] = make_float4(float(rl[k][i].l0), float(rl[k][i].l1), float(rl[k][i].l2), float(rl[k][i].w));
        if ((r = own_up(fw, &fw->rule[k], rl[k].data(), rl[k].size())) || (r = own_up(fw, &fw->rulef[k], f.data(), f.size())))
            return fail(r);
        fw->nrule[k] = int(rl[k].size());
    }
    // state and work arrays at their capacities
    const int R = fw->R, nte = s->nte;
    fw->ns_cap = 2 * s->nstrip * (R - 1);
    fw->nsg_cap = (s->nfirst + s->nlast) * (R - 1) + 2 * s->nstrip;
    fw->nteblob = s->npt + 2 * s->npf;
    if ((r = own_alloc(fw, &fw->rx, size_t(R) * nte * 3)) || (r = own_alloc(fw, &fw->rmu, size_t(R) * nte)) ||
        (r = own_alloc(fw, &fw->mul, size_t(nte))) || (r = own_alloc(fw, &fw->brows, size_t(s->nstrip))) ||
        (r = own_alloc(fw, &fw->blen, size_t(s->nstrip))) || (r = own_alloc(fw, &fw->bwid, size_t(s->nstrip))) ||
        (r = own_alloc(fw, &fw->d_np, 1)) || (r = own_alloc(fw, &fw->d_err, 1)) ||
        (r = own_alloc(fw, &fw->sheet, size_t(std::max(fw->ns_cap, 1)))) ||
        (r = own_alloc(fw, &fw->sheet_G, 3 * size_t(std::max(fw->ns_cap, 1)))) ||
        (r = own_alloc(fw, &fw->sheet_ok, size_t(std::max(fw->ns_cap, 1)))) ||
        (r = own_alloc(fw, &fw->seg, 8 * size_t(fw->nsg_cap))) || (r = own_alloc(fw, &fw->trow, 3 * size_t(s->ntri))) ||
        (r = own_alloc(fw, &fw->rhs, size_t(s->nslot))) || (r = own_alloc(fw, &fw->x, size_t(F->n))) ||
        (r = own_alloc(fw, &fw->mu, size_t(s->nslot))) || (r = own_alloc(fw, &fw->mu_prev, size_t(s->nslot))) ||
        (r = own_alloc(fw, &fw->dmu, size_t(s->nslot))) || (r = own_alloc(fw, &fw->cp, size_t(s->ntri))) ||
        (r = own_alloc(fw, &fw->surf_part, 6 * size_t((s->ntri + 255) / 256 + 1))) ||
        (r = own_alloc(fw, &fw->rec, 32 + size_t(nte))) || (r = own_alloc(fw, &fw->src32, size_t(BS32) * s->ntri)))
        return fail(r);
    if ((r = vp_solve_work_alloc(ctx, F, &fw->sw))) return fail(r);
    VP_CUDA(ctx, cudaMemsetAsync(fw->mul, 0, sizeof(double) * nte, ctx->stream));
    VP_CUDA(ctx, cudaMemsetAsync(fw->brows, 0, sizeof(int) * s->nstrip, ctx->stream));
    VP_CUDA(ctx, cudaMemsetAsync(fw->blen, 0, sizeof(double) * s->nstrip, ctx->stream));
    VP_CUDA(ctx, cudaMemsetAsync(fw->bwid, 0, sizeof(double) * s->nstrip, ctx->stream));
    VP_CUDA(ctx, cudaMemsetAsync(fw->d_np, 0, sizeof(int), ctx->stream));
    VP_CUDA(ctx, cudaMemsetAsync(fw->d_err, 0, sizeof(int), ctx->stream));
    VP_CUDA(ctx, cudaMemsetAsync(fw->mu_prev, 0, sizeof(double) * s->nslot, ctx->stream));
    VP_CUDA(ctx, cudaMemsetAsync(fw->cp, 0, sizeof(double) * s->ntri, ctx->stream));
    if ((r = ensure_capacity(fw, std::max(s->particle_capacity, 1)))) return fail(r);
    fw->h_rec.resize(32 + size_t(nte));
    VP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    *out = fw;
    return VP_OK;
}

// the particles a step can add at most (its conversions' sheets, tip sides and far end)
static int step_new_particles(const vp_freewake* fw) {
    const int nr_after = (fw->nrows == 0 ? 1 : fw->nrows) + 1;
    const int conv = std::max(0, nr_after - 1 - fw->s.keep_rows);
    return conv * (4 * fw->nstrip + 2 * (fw->nfirst + fw->nlast));
}

extern "C" int vp_freewake_step(vp_freewake* fw, vp_freewake_record* rec) {
    if (!fw) return VP_ERR_ARG;
    vp_ctx* ctx = fw->ctx;
    DeviceGuard dg;
    if (dg.set(ctx->device) != cudaSuccess) return vp_fail(ctx, VP_ERR_CUDA, "cudaSetDevice");
    int r;
    if ((r = ensure_capacity(fw, fw->np + step_new_particles(fw)))) return r;
    const vp_freewake_setup& s = fw->s;
    const vp_assembly_options& o = s.assembly;
    const bool mixed = o.precision == VP_MIXED;
    const int nte = fw->nte, R = fw->R, ntri = fw->ntri, nslot = fw->nslot;
    vp_phase_begin(ctx, PH_WAKE);
    // 1. the free wake's elements and their blobs; the trailing edge panel's blobs come after the solve (mu_w)
    const int nr = fw->nrows;
    const int nsh = 2 * fw->nstrip * std::max(nr - 1, 0);
    const int nsg = (fw->nfirst + fw->nlast) * std::max(nr - 1, 0) + (nr >= 1 ? 2 * fw->nstrip : 0);
    double* wblobs = fw->blobs + 7 * size_t(fw->nteblob);  // the elements' blobs follow the panel's
    if (nsh + nsg > 0) {
        ElemArgs ea{};
        ea.nr = nr, ea.head = fw->head, ea.R = R, ea.nte = nte, ea.rx = fw->rx, ea.rmu = fw->rmu, ea.mul = fw->mul;
        ea.nstrip = fw->nstrip, ea.nfirst = fw->nfirst, ea.nlast = fw->nlast;
        ea.strips = fw->strips, ea.first = fw->first, ea.last = fw->last, ea.core = fw->core;
        ea.nsh = nsh, ea.nsg = nsg, ea.sheet = fw->sheet, ea.sheet_G = fw->sheet_G, ea.sheet_ok = fw->sheet_ok;
        ea.seg = fw->seg, ea.blobs = wblobs;
        elements_kernel<<<(nsh + nsg + ELEM_THREADS - 1) / ELEM_THREADS, ELEM_THREADS, 0, ctx->stream>>>(ea);
        ctx->launches++;
    }
    const int nwblob = nsh + 2 * nsg;
    // the particles follow the elements' blobs in the blob list; they are read in place from there
    double* pblobs = wblobs + 7 * size_t(nwblob);
    if (fw->np > 0)
        VP_CUDA(ctx, cudaMemcpyAsync(pblobs, fw->part, sizeof(double) * 7 * fw->np, cudaMemcpyDeviceToDevice, ctx->stream));
    // 2. the explicit right hand side and the solve
    {
        RhsArgs ra{};
        ra.na = wake_near_args(fw, o);
        // mixed: the particles go to the FP32 N-body kernel below; FP64: they stay in the warp kernel
        ra.sheet_G = fw->sheet_G, ra.sheet_ok = fw->sheet_ok, ra.nsh = nsh, ra.nsg = nsg, ra.npart = mixed ? 0 : fw->np;
        ra.seg = fw->seg, ra.part = fw->part, ra.trow = fw->trow;
        ra.pr.rfar = fw->rule[R_FAR], ra.pr.nfar = fw->nrule[R_FAR], ra.pr.rnear = fw->rule[R_NEAR];
        ra.pr.nnear = fw->nrule[R_NEAR], ra.pr.test_mode = o.test, ra.pr.near_depth = o.near_depth;
        ra.pr.far_ratio = o.far_ratio, ra.pr.near_ratio = o.near_ratio;
        const int nb = (ntri + RHS_WARPS - 1) / RHS_WARPS;
        vp_phase_end(ctx);
        vp_phase_begin(ctx, PH_WAKE_RHS);
        if (mixed)
            wake_rhs_kernel<float><<<nb, 32 * RHS_WARPS, 0, ctx->stream>>>(ra);
        else
            wake_rhs_kernel<double><<<nb, 32 * RHS_WARPS, 0, ctx->stream>>>(ra);
        if (mixed && fw->np > 0) {
            particle_prep_kernel<<<(fw->np + 255) / 256, 256, 0, ctx->stream>>>(fw->np, fw->part, fw->ph, fw->pl, fw->pa);
            PRhsArgs pa{};
            pa.ntri = ntri, pa.npart = fw->np, pa.nchunk = (fw->np + NB_CHUNK - 1) / NB_CHUNK;
            pa.tri = fw->tg, pa.part = fw->part, pa.ph = fw->ph, pa.pl = fw->pl, pa.pa = fw->pa, pa.pr = ra.pr;
            pa.out = fw->prhs;
            particle_rhs_kernel<<<dim3((ntri + NB_TPB - 1) / NB_TPB, pa.nchunk), NB_TPB, 0, ctx->stream>>>(pa);
            add_chunks_kernel<<<(3 * ntri + 255) / 256, 256, 0, ctx->stream>>>(3 * ntri, pa.nchunk, fw->prhs, fw->trow);
            ctx->launches += 3;
        }
        vp_phase_end(ctx);
        vp_phase_begin(ctx, PH_WAKE);
        slot_gather_kernel<<<(nslot + 255) / 256, 256, 0, ctx->stream>>>(nslot, fw->sg_ptr, fw->sg_ent, fw->trow, fw->b0,
                                                                          fw->rhs);
        ctx->launches += 2;
        VP_CUDA(ctx, cudaGetLastError());
    }
    vp_phase_end(ctx);
    vp_phase_begin(ctx, PH_SOLVE);
    r = vp_solve_dev(ctx, fw->F, fw->rhs, fw->x, &fw->sw);
    vp_phase_end(ctx);
    if (r) return r;
    vp_phase_begin(ctx, PH_WAKE);
    double* muw = fw->rec + 32;  // mu_w sits in the record, after its 32 scalars
    csr_mv_kernel<<<(nslot + 255) / 256, 256, 0, ctx->stream>>>(nslot, fw->Cp, fw->Ci, fw->Cv, fw->x, fw->mu);
    csr_mv_kernel<<<(nte + 255) / 256, 256, 0, ctx->stream>>>(nte, fw->Kp, fw->Ki, fw->Kv, fw->x, muw);
    // 3. loads: Cp with dmu/dt, pressure force and moment; blobs of the panel; moments; Kutta-Joukowski
    body_state_kernel<<<(std::max(ntri, nslot) + 255) / 256, 256, 0, ctx->stream>>>(
        ntri, nslot, fw->tg, fw->mu, fw->mu_prev, 1.0 / s.dt, fw->n == 0 ? 1 : 0, fw->dmu, fw->bs);
    ctx->launches += 3;
    if ((r = vp_post_surface_launch(ctx, ntri, fw->corners, fw->slot, fw->mu, fw->dmu, fw->V, nullptr, nullptr, fw->cp,
                                    fw->surf_part, fw->rec)))
        return r;
    if (fw->nteblob > 0) {
        TeBlobArgs ta{fw->npt, fw->npf, fw->pwx, fw->pwte, fw->pt, fw->pf, muw, fw->core, fw->blobs};
        te_blobs_kernel<<<(fw->nteblob + 127) / 128, 128, 0, ctx->stream>>>(ta);
        ctx->launches++;
    }
    const int nblob = fw->nteblob + nwblob + fw->np;
    const int nmb = (ntri + nblob + 255) / 256;
    moments_kernel<<<nmb, 256, 0, ctx->stream>>>(ntri, fw->tg, fw->bs, nblob, fw->blobs, fw->mom_part);
    finish_loads_kernel<<<1, 32, 0, ctx->stream>>>(nmb, fw->mom_part, fw->nteseg, fw->teseg, fw->tex, muw, fw->rec + 6);
    ctx->launches += 2;
    // 4. the first step sheds R0 first, so that it is advected; velocities and forward Euler
    int nrows = nr, head = fw->head;
    if (nrows == 0) {
        head = (head + R - 1) % R;
        shed_kernel<<<(nte + 127) / 128, 128, 0, ctx->stream>>>(nte, head, fw->edge, muw, fw->rx, fw->rmu);
        ctx->launches++;
        nrows = 1;
    }
    PointArgs pa{nrows, head, R, nte, fw->np, fw->rx, fw->part, fw->X};
    const int npts = nrows * nte + fw->np;
    gather_points_kernel<<<(npts + 255) / 256, 256, 0, ctx->stream>>>(pa);
    ctx->launches++;
    const bool freestream = s.advection == 1;
    vp_phase_end(ctx);
    vp_phase_begin(ctx, PH_WAKE_VEL);
    if (!freestream) {
        if (mixed) {
            body_src32_kernel<<<(ntri + 255) / 256, 256, 0, ctx->stream>>>(ntri, fw->bs, fw->src32);
            BVelArgs ba{};
            ba.ntri = ntri, ba.npts = npts, ba.nchunk = (ntri + NB_CHUNK - 1) / NB_CHUNK, ba.src32 = fw->src32;
            ba.src64 = fw->bs, ba.X = fw->X, ba.kernel_far = o.kernel_far, ba.out = fw->bvel;
            body_vel_kernel<<<dim3((npts + NB_TPB - 1) / NB_TPB, ba.nchunk), NB_TPB, 0, ctx->stream>>>(ba);
            VP_CUDA(ctx, cudaMemsetAsync(fw->ub, 0, sizeof(double) * 3 * npts, ctx->stream));
            add_chunks_kernel<<<(3 * npts + 255) / 256, 256, 0, ctx->stream>>>(3 * npts, ba.nchunk, fw->bvel, fw->ub);
            ctx->launches += 3;
            if (nblob > 0)
                blob_kernel<float><<<(npts + NB_THREADS * NB_PTS - 1) / (NB_THREADS * NB_PTS), NB_THREADS, 0,
                                     ctx->stream>>>(nblob, fw->blobs, npts, fw->X, fw->uw);
        } else {
            body_kernel<double><<<(npts + NB_THREADS - 1) / NB_THREADS, NB_THREADS, 0, ctx->stream>>>(
                ntri, fw->bs, o.kernel_far, npts, fw->X, fw->ub);
            if (nblob > 0)
                blob_kernel<double><<<(npts + NB_THREADS - 1) / NB_THREADS, NB_THREADS, 0, ctx->stream>>>(
                    nblob, fw->blobs, npts, fw->X, fw->uw);
        }
        if (nblob == 0) VP_CUDA(ctx, cudaMemsetAsync(fw->uw, 0, sizeof(double) * 3 * npts, ctx->stream));
        ctx->launches += 2;
    }
    vp_phase_end(ctx);
    vp_phase_begin(ctx, PH_WAKE);
    const int nub = (npts + 255) / 256;
    advect_kernel<<<nub, 256, 0, ctx->stream>>>(pa, fw->V[0], fw->V[1], fw->V[2], freestream ? 1 : 0, s.dt, fw->ub,
                                                 fw->uw, fw->umax_part);
    max_parts_kernel<<<1, 32, 0, ctx->stream>>>(nub, fw->umax_part, fw->rec + 15);
    ctx->launches += 2;
    // 5. a new R0; conversions while more than keep_rows panel rows remain; deletion
    head = (head + R - 1) % R;
    shed_kernel<<<(nte + 127) / 128, 128, 0, ctx->stream>>>(nte, head, fw->edge, muw, fw->rx, fw->rmu);
    ctx->launches++;
    nrows += 1;
    BookArgs ba{};
    ba.nte = nte, ba.R = R, ba.rx = fw->rx, ba.rmu = fw->rmu, ba.mul = fw->mul;
    ba.nstrip = fw->nstrip, ba.nfirst = fw->nfirst, ba.nlast = fw->nlast;
    ba.strips = fw->strips, ba.first = fw->first, ba.last = fw->last, ba.merge = fw->merge, ba.core = fw->core;
    ba.cap = fw->cap, ba.np = fw->d_np, ba.part = fw->part, ba.tag = fw->tag, ba.group = fw->group;
    ba.brows = fw->brows, ba.blen = fw->blen, ba.bwid = fw->bwid, ba.err = fw->d_err;
    ba.delete_limit = s.delete_limit;
    for (int z = 0; z < 3; ++z) ba.d[z] = fw->d[z];
    int conv = 0;
    while (nrows - 1 > s.keep_rows) {
        ba.up = (head + nrows - 2) % R;
        ba.down = (head + nrows - 1) % R;
        convert_kernel<<<1, BK_THREADS, 0, ctx->stream>>>(ba);
        ctx->launches++;
        nrows -= 1;
        ++conv;
    }
    if (std::isfinite(s.delete_limit)) {
        delete_far_kernel<<<1, BK_THREADS, 0, ctx->stream>>>(ba);
        ctx->launches++;
    }
    VP_CUDA(ctx, cudaGetLastError());
    // the record: F and M (0-5), Omega and I (6-11), the Kutta-Joukowski circulation vector (12-14), max |U| (15),
    // the first border unknown (16), the particle count (17) and the overflow flag (18); mu_w from 32 on
    VP_CUDA(ctx, cudaMemcpyAsync(fw->rec + 16, fw->x + fw->nq, sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
    VP_CUDA(ctx, cudaMemcpyAsync(fw->rec + 17, fw->d_np, sizeof(int), cudaMemcpyDeviceToDevice, ctx->stream));
    VP_CUDA(ctx, cudaMemcpyAsync(fw->rec + 18, fw->d_err, sizeof(int), cudaMemcpyDeviceToDevice, ctx->stream));
    VP_CUDA(ctx, cudaMemcpyAsync(fw->mu_prev, fw->mu, sizeof(double) * nslot, cudaMemcpyDeviceToDevice, ctx->stream));
    vp_phase_end(ctx);
    VP_CUDA(ctx, vp_d2h(ctx, fw->h_rec.data(), fw->rec, sizeof(double) * (32 + size_t(nte))));
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return vp_fail(ctx, VP_ERR_CUDA, std::string("free wake step: ") + cudaGetErrorString(e));
    const double* h = fw->h_rec.data();
    int np_new = 0, err = 0;
    std::memcpy(&np_new, h + 17, sizeof(int));
    std::memcpy(&err, h + 18, sizeof(int));
    if (err) return vp_fail(ctx, VP_ERR_ARG, "free wake: particle capacity exceeded");
    const double V2 = fw->V[0] * fw->V[0] + fw->V[1] * fw->V[1] + fw->V[2] * fw->V[2];
    if (rec) {
        rec->n = fw->n;
        rec->t = fw->t;
        const double* G = h + 12;
        const double* I = h + 9;
        for (int z = 0; z < 3; ++z) {
            rec->F_pressure[z] = h[z];
            rec->M_pressure[z] = h[3 + z];
            rec->Omega[z] = h[6 + z];
            rec->I[z] = I[z];
            rec->F_impulse[z] = fw->n == 0 ? std::numeric_limits<double>::quiet_NaN()
                                           : -(2.0 / V2) * (I[z] - fw->I_prev[z]) / s.dt;
        }
        rec->F_kj[0] = 2.0 / V2 * (fw->V[1] * G[2] - fw->V[2] * G[1]);
        rec->F_kj[1] = 2.0 / V2 * (fw->V[2] * G[0] - fw->V[0] * G[2]);
        rec->F_kj[2] = 2.0 / V2 * (fw->V[0] * G[1] - fw->V[1] * G[0]);
        rec->rows = nrows - 1;
        rec->particles = np_new;
        rec->lambda = fw->F->nb > 0 ? fw->F->h_se[0] * h[16] : 0.0;
        rec->umax = h[15];
    }
    for (int z = 0; z < 3; ++z) fw->I_prev[z] = h[9 + z];
    fw->head = head;
    fw->nrows = nrows;
    fw->np = np_new;
    fw->conversions += conv;
    fw->n += 1;
    fw->t += s.dt;
    return VP_OK;
}

extern "C" int vp_freewake_info(const vp_freewake* fw, vp_freewake_counts* c) {
    if (!fw || !c) return VP_ERR_ARG;
    c->n = fw->n;
    c->t = fw->t;
    c->nrows = fw->nrows;
    c->nparticles = fw->np;
    c->conversions = fw->conversions;
    for (int z = 0; z < 3; ++z) c->I_prev[z] = fw->I_prev[z];
    return VP_OK;
}

extern "C" int vp_freewake_get_state(const vp_freewake* fw, double* rows_x, double* rows_mu, double* mu_line,
                                     double* particles, int* tag, signed char* group, int* batch_rows,
                                     double* batch_length, double* batch_width, double* mu, double* mu_w, double* cp) {
    if (!fw) return VP_ERR_ARG;
    vp_ctx* ctx = fw->ctx;
    DeviceGuard dg;
    if (dg.set(ctx->device) != cudaSuccess) return vp_fail(ctx, VP_ERR_CUDA, "cudaSetDevice");
    const int nte = fw->nte;
    for (int i = 0; i < fw->nrows; ++i) {
        const int pr = (fw->head + i) % fw->R;
        if (rows_x)
            VP_CUDA(ctx, vp_d2h(ctx, rows_x + size_t(i) * nte * 3, fw->rx + size_t(pr) * nte * 3, sizeof(double) * nte * 3));
        if (rows_mu) VP_CUDA(ctx, vp_d2h(ctx, rows_mu + size_t(i) * nte, fw->rmu + size_t(pr) * nte, sizeof(double) * nte));
    }
    if (mu_line) VP_CUDA(ctx, vp_d2h(ctx, mu_line, fw->mul, sizeof(double) * nte));
    if (fw->np > 0) {
        if (particles) VP_CUDA(ctx, vp_d2h(ctx, particles, fw->part, sizeof(double) * 7 * fw->np));
        if (tag) VP_CUDA(ctx, vp_d2h(ctx, tag, fw->tag, sizeof(int) * fw->np));
        if (group) VP_CUDA(ctx, vp_d2h(ctx, group, fw->group, size_t(fw->np)));
    }
    if (batch_rows) VP_CUDA(ctx, vp_d2h(ctx, batch_rows, fw->brows, sizeof(int) * fw->nstrip));
    if (batch_length) VP_CUDA(ctx, vp_d2h(ctx, batch_length, fw->blen, sizeof(double) * fw->nstrip));
    if (batch_width) VP_CUDA(ctx, vp_d2h(ctx, batch_width, fw->bwid, sizeof(double) * fw->nstrip));
    if (mu) VP_CUDA(ctx, vp_d2h(ctx, mu, fw->mu_prev, sizeof(double) * fw->nslot));
    if (cp) VP_CUDA(ctx, vp_d2h(ctx, cp, fw->cp, sizeof(double) * fw->ntri));
    VP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (mu_w)
        for (int k = 0; k < nte; ++k) mu_w[k] = fw->n > 0 ? fw->h_rec[32 + k] : 0.0;
    return VP_OK;
}

extern "C" int vp_freewake_set_state(vp_freewake* fw, const vp_freewake_counts* c, const double* rows_x,
                                     const double* rows_mu, const double* mu_line, const double* particles,
                                     const int* tag, const signed char* group, const int* batch_rows,
                                     const double* batch_length, const double* batch_width, const double* mu,
                                     const double* mu_w, const double* cp) {
    if (!fw || !c || !rows_x || !rows_mu || !mu_line || !batch_rows || !batch_length || !batch_width || !mu || !mu_w ||
        !cp || (c->nparticles > 0 && (!particles || !tag || !group)))
        return vp_fail(fw ? fw->ctx : nullptr, VP_ERR_ARG, "null argument");
    vp_ctx* ctx = fw->ctx;
    if (c->nrows < 0 || c->nrows > fw->R - 1 || c->nparticles < 0 || c->n < 0 || c->conversions < 0)
        return vp_fail(ctx, VP_ERR_ARG, "state sizes out of range for this simulation");
    for (int i = 0; i < c->nparticles; ++i)
        if (tag[i] < 0 || tag[i] > fw->nstrip || group[i] < 0 || group[i] > 2)
            return vp_fail(ctx, VP_ERR_ARG, "particle merge tag out of range");
    DeviceGuard dg;
    if (dg.set(ctx->device) != cudaSuccess) return vp_fail(ctx, VP_ERR_CUDA, "cudaSetDevice");
    int r;
    if ((r = ensure_capacity(fw, c->nparticles))) return r;
    const int nte = fw->nte;
    fw->head = 0;
    VP_CUDA(ctx, vp_h2d(ctx, fw->rx, rows_x, sizeof(double) * size_t(c->nrows) * nte * 3));
    VP_CUDA(ctx, vp_h2d(ctx, fw->rmu, rows_mu, sizeof(double) * size_t(c->nrows) * nte));
    VP_CUDA(ctx, vp_h2d(ctx, fw->mul, mu_line, sizeof(double) * nte));
    if (c->nparticles > 0) {
        VP_CUDA(ctx, vp_h2d(ctx, fw->part, particles, sizeof(double) * 7 * size_t(c->nparticles)));
        VP_CUDA(ctx, vp_h2d(ctx, fw->tag, tag, sizeof(int) * size_t(c->nparticles)));
        VP_CUDA(ctx, vp_h2d(ctx, fw->group, group, size_t(c->nparticles)));
    }
    VP_CUDA(ctx, vp_h2d(ctx, fw->d_np, &c->nparticles, sizeof(int)));
    VP_CUDA(ctx, vp_h2d(ctx, fw->brows, batch_rows, sizeof(int) * fw->nstrip));
    VP_CUDA(ctx, vp_h2d(ctx, fw->blen, batch_length, sizeof(double) * fw->nstrip));
    VP_CUDA(ctx, vp_h2d(ctx, fw->bwid, batch_width, sizeof(double) * fw->nstrip));
    VP_CUDA(ctx, vp_h2d(ctx, fw->mu_prev, mu, sizeof(double) * fw->nslot));
    VP_CUDA(ctx, vp_h2d(ctx, fw->cp, cp, sizeof(double) * fw->ntri));
    VP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    for (int k = 0; k < nte; ++k) fw->h_rec[32 + k] = mu_w[k];
    fw->nrows = c->nrows;
    fw->np = c->nparticles;
    fw->n = c->n;
    fw->t = c->t;
    fw->conversions = c->conversions;
    for (int z = 0; z < 3; ++z) fw->I_prev[z] = c->I_prev[z];
    return VP_OK;
}
