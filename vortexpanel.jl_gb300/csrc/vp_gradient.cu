// The adjoint pair derivatives: for fixed adjoint values nu (one per row slot) and unknowns mu (one per column), the
// derivative of F = nu' (A(x) mu - b(x)) with respect to the body nodes, the wake nodes and the angle of attack
// (through V∞(alpha) and sigma = -V∞·n), with the quadrature of the assembly kept fixed. With the adjoint solution
// nu = C xi of the transposed bordered system, dJ/dx = dJ/dx|_q - dF/dx (src/assembly/assemble.jl:377-447 is the
// forward map; the reference differentiates it with ForwardDiff duals through the same pair rules).
//
// A pair (T, S) contributes f = sum_q W_q nu(q) w_S(x_q)·m, m = n_T x Gamma_S + sigma_S n_T, where nu(q) = sum_a
// nu_a psi_a(q) and Gamma_S = sum_b mu_b gamma_b; the freestream adds (V∞·n_T A_T) sum_a nu_a ti_a. Per point the
// kernels evaluate s = w·m with its reverse-mode derivatives (vp_adjoint.cuh) and collect:
//   - on the test side, per test triangle (TA, 13 doubles): the derivative with respect to the points' positions by
//     corner (9), with respect to n_T (3) and f itself (for the area);
//   - on the source side, per source triangle (SA, 41 doubles): the sums of SrcAdj (vp_adjoint_common.cuh), which
//     a last kernel turns into derivatives with respect to the source's corners once per source.
// Kernels (one CUDA stream):
//   1. far tier: one CTA per (128-source tile, chunk of test tiles), one thread per source keeping its sums in
//      registers across the chunk; test-side sums reduced over the CTA per test and added to fixed-point
//      accumulators (vp_fixed.cuh), whose totals do not depend on the order of the additions;
//   2. non-far pairs: one warp per test triangle, every pair's rule built and walked as in the assembly (the same
//      templates with the adjoint accumulator), per-pair warp sums, test side in registers, source side added to SA;
//      the tip filaments and the freestream term;
//   3. finish: one thread per triangle turns TA and SA into node derivatives.
#include "vp_pairs.cuh"
#include "vp_fixed.cuh"

namespace {

constexpr int NSA = 41;  // SrcAdj fields
constexpr int NTA = 13;  // test side: Xg (9), U (3), f (1)

// SrcAdj in a flat order: Gr (9), Lm (9), Om (3), Grf (3), Gd (9), Gb (3), Nm (3), A, Sb
template <class T>
__device__ __forceinline__ void sa_flat(const SrcAdj<T>& s, T* f) {
    for (int k = 0; k < 3; ++k) {
        f[3 * k] = s.Gr[k].x; f[3 * k + 1] = s.Gr[k].y; f[3 * k + 2] = s.Gr[k].z;
        f[9 + 3 * k] = s.Lm[k].x; f[10 + 3 * k] = s.Lm[k].y; f[11 + 3 * k] = s.Lm[k].z;
        f[24 + 3 * k] = s.Gd[k].x; f[25 + 3 * k] = s.Gd[k].y; f[26 + 3 * k] = s.Gd[k].z;
        f[36 + k] = s.Nm[k];
    }
    f[18] = s.Om.x; f[19] = s.Om.y; f[20] = s.Om.z;
    f[21] = s.Grf.x; f[22] = s.Grf.y; f[23] = s.Grf.z;
    f[33] = s.Gb.x; f[34] = s.Gb.y; f[35] = s.Gb.z;
    f[39] = s.A;
    f[40] = s.Sb;
}

__device__ __forceinline__ SrcAdj<double> sa_unflat(const vp_fx* x) {
    double f[NSA];
    for (int k = 0; k < NSA; ++k) f[k] = fx_get(x[k]);
    SrcAdj<double> s;
    for (int k = 0; k < 3; ++k) {
        s.Gr[k] = mk3(f[3 * k], f[3 * k + 1], f[3 * k + 2]);
        s.Lm[k] = mk3(f[9 + 3 * k], f[10 + 3 * k], f[11 + 3 * k]);
        s.Gd[k] = mk3(f[24 + 3 * k], f[25 + 3 * k], f[26 + 3 * k]);
        s.Nm[k] = f[36 + k];
    }
    s.Om = mk3(f[18], f[19], f[20]);
    s.Grf = mk3(f[21], f[22], f[23]);
    s.Gb = mk3(f[33], f[34], f[35]);
    s.A = f[39];
    s.Sb = f[40];
    return s;
}

// ------------------------------------------------------------------------------------------------------------------
// far tier

struct AdjFarArgs {
    int ntest, nq, ntiles_test, tiles_per_chunk;
    const double* tq;    // test far points (ntest x NQMAX x 3)
    const double* tw;    // w_q A_T psi_a (ntest x NQMAX x 3)
    const TriGeo* tgeo;
    const CentF* tcent;
    const double* lam;   // far rule barycentrics (nq x 3)
    const double* nu[ADJ_MAX];  // row slot values, per adjoint vector of the pass
    int nset;
    int nsrc[2], ntile[2];
    const void* soa[2];  // NFIELD x pad (T), as the assembly's far kernel
    const void* gam[2];  // Gamma_S, 3 x pad (T)
    int pad[2];
    const CentF* scent[2];
    const TriGeo* sgeo[2];
    vp_fx* SA[ADJ_MAX][2];
    vp_fx* TA[ADJ_MAX];
    float ratio32;
    double ratio, kernel_far;
};

template <class T>
struct AdjFarTest {
    T xh[NQMAX][3], xl[NQMAX][3];
    T Wn[ADJ_MAX][NQMAX];  // w_q A_T nu(q), per adjoint vector
    T n[3];
    CentF cf;
    double c64[3];
    double diam64;
    int t;  // -1: past the end
};

// K adjoint vectors in one pass (their weights differ, the kernel values and derivatives are shared)
template <class T, int TT, int K>
__global__ void __launch_bounds__(FAR_NT) adj_far_kernel(AdjFarArgs a) {
    __shared__ AdjFarTest<T> ts[TT];
    __shared__ T lam[NQMAX][3];
    __shared__ T red[TT][FAR_NT / 32][K * NTA];
    const T i4pi = T(1) / (T(4) * vp_pi<T>());
    int bx = blockIdx.x, set = 0;
    if (bx >= a.ntile[0]) {
        set = 1;
        bx -= a.ntile[0];
    }
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int s = bx * FAR_NT + tid;
    const bool sv = s < a.nsrc[set];
    const T* soa = (const T*)a.soa[set];
    const int pad = a.pad[set];
    SrcKern<T> S;
    v3<T> ch = mk3(T(0), T(0), T(0)), cl = ch, G = ch;
    T sig = T(0);
    CentF scf{};
    if (sv) {
#define F(f) soa[size_t(f) * pad + s]
        ch = mk3(F(0), F(1), F(2));
        cl = mk3(F(3), F(4), F(5));
        S.diam = F(6);
        S.area = F(7);
        sig = F(8);
        for (int k = 0; k < 3; ++k) {
            S.d[k] = mk3(F(9 + 3 * k), F(10 + 3 * k), F(11 + 3 * k));
            S.nu[k] = mk3(F(18 + 3 * k), F(19 + 3 * k), F(20 + 3 * k));
            S.len[k] = F(27 + k);
        }
        S.n = mk3(F(30), F(31), F(32));
#undef F
        const T* g = (const T*)a.gam[set];
        G = mk3(g[s], g[size_t(pad) + s], g[2 * size_t(pad) + s]);
        scf = a.scent[set][s];
    }
    SrcAdj<T> acc[K];
#pragma unroll
    for (int j = 0; j < K; ++j) src_zero(acc[j]);
    if (tid < 3 * a.nq) lam[tid / 3][tid % 3] = T(a.lam[tid]);
    const T fd = T(a.kernel_far) * (sv ? S.diam : T(0));
    const int tile0 = blockIdx.y * a.tiles_per_chunk;
    const int tile1 = min(tile0 + a.tiles_per_chunk, a.ntiles_test);
    for (int tile = tile0; tile < tile1; ++tile) {
        __syncthreads();
        for (int i = tid; i < TT; i += FAR_NT) {
            const int t = tile * TT + i;
            AdjFarTest<T>& q = ts[i];
            q.t = t < a.ntest ? t : -1;
            if (q.t >= 0) {
                const TriGeo& g = a.tgeo[t];
                for (int p = 0; p < a.nq; ++p) {
                    const double* tq = a.tq + (size_t(t) * NQMAX + p) * 3;
                    const double* tw = a.tw + (size_t(t) * NQMAX + p) * 3;
                    for (int k = 0; k < 3; ++k) {
                        T h = T(tq[k]);
                        q.xh[p][k] = h;
                        q.xl[p][k] = T(tq[k] - double(h));
                    }
                    for (int j = 0; j < K; ++j) {
                        const double* nu = a.nu[j];
                        q.Wn[j][p] = T(nu[g.slot[0]] * tw[0] + nu[g.slot[1]] * tw[1] + nu[g.slot[2]] * tw[2]);
                    }
                }
                for (int k = 0; k < 3; ++k) {
                    q.n[k] = T(g.n[k]);
                    q.c64[k] = g.c[k];
                }
                q.diam64 = g.diam;
                q.cf = a.tcent[t];
            }
        }
        __syncthreads();
#pragma unroll 1
        for (int i = 0; i < TT; ++i) {
            const AdjFarTest<T>& q = ts[i];
            bool far = false;
            if (sv && q.t >= 0) {
                if (sizeof(T) == 8) {
                    far = far_exact64(q.c64, q.diam64, a.sgeo[set][s].c, a.sgeo[set][s].diam, a.ratio);
                } else {
                    int f = far_test32(q.cf, scf, a.ratio32);
                    if (f < 0) f = far_exact64(q.c64, q.diam64, a.sgeo[set][s].c, a.sgeo[set][s].diam, a.ratio);
                    far = f == 1;
                }
            }
            v3<T> Xg[K][3], U[K];
            T fs[K];
#pragma unroll
            for (int j = 0; j < K; ++j) {
                Xg[j][0] = Xg[j][1] = Xg[j][2] = U[j] = mk3(T(0), T(0), T(0));
                fs[j] = T(0);
            }
            if (far) {
                const v3<T> nT = mk3(q.n[0], q.n[1], q.n[2]);
                const v3<T> m = cross(nT, G) + sig * nT;
                for (int p = 0; p < a.nq; ++p) {
                    v3<T> r = mk3((q.xh[p][0] - ch.x) + (q.xl[p][0] - cl.x), (q.xh[p][1] - ch.y) + (q.xl[p][1] - cl.y),
                                  (q.xh[p][2] - ch.z) + (q.xl[p][2] - cl.z));
                    v3<T> w, gx;
                    T sval;
                    if (dot(r, r) > fd * fd) {
                        v3<T> gr, gd[3];
                        T ga;
                        sval = sv_far_vjp(S, r, m, gr, gd, ga);
                        w = sv_far(S, r);
#pragma unroll
                        for (int j = 0; j < K; ++j) {
                            const T Wn = q.Wn[j][p];
                            acc[j].Grf += Wn * gr;
                            for (int k = 0; k < 3; ++k) acc[j].Gd[k] += Wn * gd[k];
                            acc[j].A += Wn * ga;
                        }
                        gx = gr;
                    } else {
                        v3<T> g0, g1, g2;
                        ExactShape<T> sh;
                        sval = sv_exact_vjp(S, r - S.d[0], r - S.d[1], r - S.d[2], r, m, 0, T(1e-12), g0, g1, g2, sh);
                        w = (sh.L[0] * S.nu[0] + sh.L[1] * S.nu[1] + sh.L[2] * S.nu[2] + sh.Om * S.n) * i4pi;
#pragma unroll
                        for (int j = 0; j < K; ++j) {
                            const T Wn = q.Wn[j][p];
                            acc[j].Gr[0] += Wn * g0;
                            acc[j].Gr[1] += Wn * g1;
                            acc[j].Gr[2] += Wn * g2;
                            for (int e = 0; e < 3; ++e) {
                                acc[j].Lm[e] += (Wn * sh.L[e]) * m;
                                acc[j].Nm[e] += Wn * sh.dLdlen[e] * dot(S.nu[e], m);
                            }
                            acc[j].Om += (Wn * sh.Om) * m;
                        }
                        gx = g0 + g1 + g2;
                    }
                    const v3<T> wxn = cross(w, nT), uw = cross(G, w) + sig * w;
                    const T wn = dot(w, nT);
#pragma unroll
                    for (int j = 0; j < K; ++j) {
                        const T Wn = q.Wn[j][p];
                        acc[j].Gb += Wn * wxn;
                        acc[j].Sb += Wn * wn;
                        for (int k = 0; k < 3; ++k) Xg[j][k] += (Wn * lam[p][k]) * gx;
                        U[j] += Wn * uw;
                        fs[j] += Wn * sval;
                    }
                }
            }
            // the test side of this test: sum over the warp, then over the CTA's warps below
            const bool anyfar = __any_sync(0xffffffffu, far);
#pragma unroll
            for (int j = 0; j < K; ++j) {
                T v[NTA] = {Xg[j][0].x, Xg[j][0].y, Xg[j][0].z, Xg[j][1].x, Xg[j][1].y, Xg[j][1].z,
                            Xg[j][2].x, Xg[j][2].y, Xg[j][2].z, U[j].x,     U[j].y,     U[j].z,     fs[j]};
                if (anyfar) {
#pragma unroll
                    for (int k = 0; k < NTA; ++k)
#pragma unroll
                        for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
                }
                if (lane == 0)
#pragma unroll
                    for (int k = 0; k < NTA; ++k) red[i][wid][j * NTA + k] = v[k];
            }
        }
        __syncthreads();
        for (int k = tid; k < TT * K * NTA; k += FAR_NT) {
            const int i = k / (K * NTA), jf = k - i * (K * NTA), j = jf / NTA, f = jf - j * NTA;
            if (ts[i].t < 0) continue;
            T v = T(0);
            for (int w = 0; w < FAR_NT / 32; ++w) v += red[i][w][jf];
            if (v != T(0)) fx_add(a.TA[j] + size_t(ts[i].t) * NTA + f, double(v));
        }
    }
    if (sv) {
#pragma unroll
        for (int j = 0; j < K; ++j) {
            T f[NSA];
            sa_flat(acc[j], f);
            vp_fx* dst = a.SA[j][set] + size_t(s) * NSA;
#pragma unroll
            for (int k = 0; k < NSA; ++k)
                if (f[k] != T(0)) fx_add(dst + k, double(f[k]));
        }
    }
}

struct AdjExtra {
    const double* nu;     // row slot values
    const double* mu;     // column values (body slots, then wake nodes)
    const double* gam_b;  // Gamma_S of the body triangles (3 each)
    const double* gam_w;  // and of the wake triangles
    double V[3], dV[3];
    // the sums, in order-independent fixed point (vp_fixed.cuh): the gradients are the same from run to run
    vp_fx* SA[2];
    vp_fx* TA;
    vp_fx* gx;            // body node derivatives (3 each)
    vp_fx* gwx;           // wake node derivatives (3 each)
    vp_fx* dal;
};

// ------------------------------------------------------------------------------------------------------------------
// near-tier pairs, one per lane: the plan of the assembly's lanes kernel (tiers and quadtree leaves), every leaf point
// of a chunk of 32 pairs evaluated across the lanes (FP32 under the adjoint's guard, or queued for FP64), per-pair
// segmented sums, and each lane finishing its own pair: the source side added to SA, the test side summed over the
// warp once per test triangle. The pairs of the other tiers are listed for adj_pairs_kernel.

constexpr int NSUM = 41;  // AdjSums: Q (3), Xg (9), Gr (9), Grf (3), Gd (9), L (3), N (3), O, A

template <class T>
__device__ __forceinline__ void sums_flat(const AdjSums<T>& a, T* f) {
    f[0] = a.Q.x; f[1] = a.Q.y; f[2] = a.Q.z;
    for (int k = 0; k < 3; ++k) {
        f[3 + 3 * k] = a.Xg[k].x; f[4 + 3 * k] = a.Xg[k].y; f[5 + 3 * k] = a.Xg[k].z;
        f[12 + 3 * k] = a.Gr[k].x; f[13 + 3 * k] = a.Gr[k].y; f[14 + 3 * k] = a.Gr[k].z;
        f[24 + 3 * k] = a.Gd[k].x; f[25 + 3 * k] = a.Gd[k].y; f[26 + 3 * k] = a.Gd[k].z;
        f[33 + k] = a.L[k];
        f[36 + k] = a.N[k];
    }
    f[21] = a.Grf.x; f[22] = a.Grf.y; f[23] = a.Grf.z;
    f[39] = a.O;
    f[40] = a.A;
}

__device__ __forceinline__ AdjSums<double> sums_unflat(const double* f) {
    AdjSums<double> a;
    a.Q = mk3(f[0], f[1], f[2]);
    for (int k = 0; k < 3; ++k) {
        a.Xg[k] = mk3(f[3 + 3 * k], f[4 + 3 * k], f[5 + 3 * k]);
        a.Gr[k] = mk3(f[12 + 3 * k], f[13 + 3 * k], f[14 + 3 * k]);
        a.Gd[k] = mk3(f[24 + 3 * k], f[25 + 3 * k], f[26 + 3 * k]);
        a.L[k] = f[33 + k];
        a.N[k] = f[36 + k];
    }
    a.Grf = mk3(f[21], f[22], f[23]);
    a.O = f[39];
    a.A = f[40];
    return a;
}

// the adjoint vectors of one pass of the warp-cooperative kernels, each with its outputs
struct AdjMulti {
    AdjExtra x[ADJ_MAX];
    int nadj;
};

struct AdjChunkSh {
    NearPlanSh pl;
    float accf[ADJ_MAX][32][NSUM];  // per adjoint vector and pair: the sums of the pair's points
    double m64[32][3];              // the pair's direction m
    int off[33];                    // points before each pair
    int qp[64], qk[64];             // queued FP64 points: pair, point within the pair
};

// the FP64 adjoint evaluation of point k of pair p (queued by the FP32 guard) for the K vectors with test-corner
// values nu[j]: the kernel and its derivatives once, each vector's sums in v[j] (in the AdjSums field order)
__device__ void adj_point64(const NearArgs& a, const TriGeo& T, const TriGeo& S, const AdjChunkSh& ns,
                            const double (*nu)[3], int K, int p, int k, float (*v)[NSUM]) {
    const int nr = a.nrule[R_NEAR];
    int leaf = k / nr, q = k - leaf * nr;
    float bf[9];
    leaf_corners32(ns.pl.leaf[p][leaf], bf);
    double b[9];
    for (int z = 0; z < 9; ++z) b[z] = double(bf[z]);
    RulePt m = a.rule[R_NEAR][q];
    double l0 = m.l0 * b[0] + m.l1 * b[3] + m.l2 * b[6];
    double l1 = m.l0 * b[1] + m.l1 * b[4] + m.l2 * b[7];
    double l2 = m.l0 * b[2] + m.l1 * b[5] + m.l2 * b[8];
    int level = ns.pl.leaf[p][leaf] >> 6;
    double W = (m.w * ldexp(1.0, -2 * level)) * T.area;
    v3<double> psi = test_weights(a.test_mode, l0, l1, l2);
    double Wn[ADJ_MAX];
    for (int j = 0; j < ADJ_MAX; ++j) Wn[j] = W * (nu[j][0] * psi.x + nu[j][1] * psi.y + nu[j][2] * psi.z);
    v3<double> R[3];
    for (int c = 0; c < 3; ++c)
        R[c] = mk3(l0 * (T.x[0] - S.x[3 * c]) + l1 * (T.x[3] - S.x[3 * c]) + l2 * (T.x[6] - S.x[3 * c]),
                   l0 * (T.x[1] - S.x[3 * c + 1]) + l1 * (T.x[4] - S.x[3 * c + 1]) + l2 * (T.x[7] - S.x[3 * c + 1]),
                   l0 * (T.x[2] - S.x[3 * c + 2]) + l1 * (T.x[5] - S.x[3 * c + 2]) + l2 * (T.x[8] - S.x[3 * c + 2]));
    v3<double> x = mk3(l0 * T.x[0] + l1 * T.x[3] + l2 * T.x[6], l0 * T.x[1] + l1 * T.x[4] + l2 * T.x[7],
                       l0 * T.x[2] + l1 * T.x[5] + l2 * T.x[8]);
    v3<double> r = x - ld3(S.c);
    SrcKern<double> Kd;
    for (int z = 0; z < 3; ++z) {
        Kd.d[z] = mk3(S.x[3 * z] - S.c[0], S.x[3 * z + 1] - S.c[1], S.x[3 * z + 2] - S.c[2]);
        Kd.nu[z] = ld3(S.nu + 3 * z);
        Kd.len[z] = S.len[z];
    }
    Kd.n = ld3(S.n);
    Kd.area = S.area;
    Kd.diam = S.diam;
    const v3<double> mm = mk3(ns.m64[p][0], ns.m64[p][1], ns.m64[p][2]);
    AdjSums<double> as[ADJ_MAX];
    for (int j = 0; j < ADJ_MAX; ++j) adj_zero(as[j]);
    v3<double> gx;
    double fd = a.kernel_far * Kd.diam;
    if (dot(r, r) > fd * fd)
        adj_point_far_multi(as, K, Wn, Kd, l0, l1, l2, r, mm, gx);
    else
        adj_point_exact_multi(as, K, Wn, Kd, l0, l1, l2, R[0], R[1], R[2], r, mm, 0, 1e-12, gx);
#pragma unroll
    for (int j = 0; j < ADJ_MAX; ++j) {
        if (j >= K) break;
        double f[NSUM];
        sums_flat(as[j], f);
        for (int z = 0; z < NSUM; ++z) v[j][z] = float(f[z]);
    }
}

// one chunk of up to 32 sources of test t, for every adjoint vector of mx at once (the plan and each point's kernel
// once); returns the lanes whose pairs are not in the near tier. Xg, U, fs: this lane's test-side sums per vector.
__device__ unsigned adj_chunk(PairCtx& pc, AdjChunkSh& ns, const AdjMulti& mx, int t, const int* list, int cnt,
                              bool wake, v3<double> (*Xg)[3], v3<double>* U, double* fs, unsigned long long* P,
                              unsigned long long* Q, unsigned long long& Q64) {
    const NearArgs& a = *pc.a;
    const TriGeo& T = *pc.T;
    const int lane = pc.lane;
    const int K = mx.nadj;
    const unsigned FULL = 0xffffffffu;
    const bool valid = lane < cnt;
    const int s = valid ? list[lane] : 0;
    const TriGeo& S = wake ? a.wtri[s] : a.tri[s];
    int nleaf = 0;
    bool near = near_plan(pc, ns.pl, t, S, s, valid, wake, nleaf);
    const v3<double> nT = ld3(T.n);
    v3<double> G = mk3(0.0, 0.0, 0.0);
    double sig = 0;
    if (near) {
        const double* gp = (wake ? mx.x[0].gam_w : mx.x[0].gam_b) + 3 * size_t(s);
        G = mk3(gp[0], gp[1], gp[2]);
        sig = wake ? 0.0 : S.sigma;
        v3<double> m = cross(nT, G) + sig * nT;
        ns.m64[lane][0] = m.x;
        ns.m64[lane][1] = m.y;
        ns.m64[lane][2] = m.z;
    }
    for (int j = 0; j < ADJ_MAX; ++j)
        for (int k = 0; k < NSUM; ++k) ns.accf[j][lane][k] = 0.f;
    const int nr = a.nrule[R_NEAR];
    int incl = near ? nleaf * nr : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(FULL, incl, o);
        if (lane >= o) incl += y;
    }
    ns.off[lane + 1] = incl;
    if (lane == 0) ns.off[0] = 0;
    const int total = __shfl_sync(FULL, incl, 31);
    const unsigned nearmask = __ballot_sync(FULL, near);
    __syncwarp();
    const float kf = float(a.kernel_far), areaT = float(T.area);
    float nuf[ADJ_MAX][3];
    for (int j = 0; j < ADJ_MAX; ++j)
        for (int c = 0; c < 3; ++c) nuf[j][c] = float(pc.nuk[j][c]);
    int nq = 0;
    unsigned long long n64 = 0;
    for (int i0 = 0; i0 < total; i0 += 32) {
        const int i = i0 + lane;
        const bool v = i < total;
        int p = 32 + lane, k = 0;
        AdjSums<float> as[ADJ_MAX];
        for (int j = 0; j < ADJ_MAX; ++j) adj_zero(as[j]);
        bool need = false;
        if (v) {
            int lo = 0, hi = 31;
            while (lo < hi) {
                int mid = (lo + hi + 1) >> 1;
                if (ns.off[mid] <= i) lo = mid;
                else hi = mid - 1;
            }
            p = lo;
            k = i - ns.off[p];
            need = !a.mixed;
        }
        if (v && a.mixed) {
            int leaf = k / nr, q = k - leaf * nr;
            int code = ns.pl.leaf[p][leaf];
            float b[9];
            leaf_corners32(code, b);
            float4 m = a.rulef[R_NEAR][q];
            float l0 = m.x * b[0] + m.y * b[3] + m.z * b[6];
            float l1 = m.x * b[1] + m.y * b[4] + m.z * b[7];
            float l2 = m.x * b[2] + m.y * b[5] + m.z * b[8];
            float W = m.w * ldexpf(1.f, -2 * (code >> 6)) * areaT;
            float Wn[ADJ_MAX];
            for (int j = 0; j < ADJ_MAX; ++j)
                Wn[j] = W * (a.test_mode == 0 ? nuf[j][0] * l0 + nuf[j][1] * l1 + nuf[j][2] * l2
                                              : nuf[j][0] + nuf[j][1] + nuf[j][2]);
            const float* E = ns.pl.E32[p];
            const float* Dp = ns.pl.D32[p];
            const float* Sf = ns.pl.S32[p];
            SrcKern<float> Kf;
            for (int z = 0; z < 3; ++z) {
                Kf.d[z] = mk3(Sf[3 * z], Sf[3 * z + 1], Sf[3 * z + 2]);
                Kf.nu[z] = mk3(Sf[9 + 3 * z], Sf[10 + 3 * z], Sf[11 + 3 * z]);
                Kf.len[z] = Sf[18 + z];
            }
            Kf.n = mk3(Sf[21], Sf[22], Sf[23]);
            Kf.area = Sf[24];
            Kf.diam = Sf[25];
            const v3<float> mf = mk3(float(ns.m64[p][0]), float(ns.m64[p][1]), float(ns.m64[p][2]));
            v3<float> r = l0 * mk3(Dp[0], Dp[1], Dp[2]) + l1 * mk3(Dp[3], Dp[4], Dp[5]) + l2 * mk3(Dp[6], Dp[7], Dp[8]);
            v3<float> gx;
            float fd = kf * Kf.diam;
            if (dot(r, r) > fd * fd) {
                adj_point_far_multi(as, K, Wn, Kf, l0, l1, l2, r, mf, gx);
            } else {
                v3<float> ra = l0 * mk3(E[0], E[1], E[2]) + l1 * mk3(E[9], E[10], E[11]) + l2 * mk3(E[18], E[19], E[20]);
                v3<float> rb = l0 * mk3(E[3], E[4], E[5]) + l1 * mk3(E[12], E[13], E[14]) + l2 * mk3(E[21], E[22], E[23]);
                v3<float> rc = l0 * mk3(E[6], E[7], E[8]) + l1 * mk3(E[15], E[16], E[17]) + l2 * mk3(E[24], E[25], E[26]);
                if (fp32_guard_ok(Kf, ra, rb, rc, 0, Fp32Guard{ADJ_GUARD}))
                    adj_point_exact_multi(as, K, Wn, Kf, l0, l1, l2, ra, rb, rc, r, mf, 0, 1e-12f, gx);
                else
                    need = true;
            }
            if (need)
                for (int j = 0; j < ADJ_MAX; ++j) adj_zero(as[j]);
        }
        if (a.mixed) {
#pragma unroll
            for (int j = 0; j < ADJ_MAX; ++j)
                if (j < K)
                    seg_accumulate<NSUM>(ns.accf[j], (double (*)[NSUM])nullptr, lane, p,
                                         reinterpret_cast<float*>(&as[j]));
        }
        unsigned mq = __ballot_sync(FULL, need);
        if (mq) {
            int pos = nq + __popc(mq & ((1u << lane) - 1u));
            if (need) {
                ns.qp[pos] = p;
                ns.qk[pos] = k;
            }
            nq += __popc(mq);
            __syncwarp();
        }
        while (nq >= 32 || (nq > 0 && i0 + 32 >= total)) {
            const int take = nq < 32 ? nq : 32;
            int qpair = 32 + lane;
            float qv[ADJ_MAX][NSUM];
            for (int j = 0; j < ADJ_MAX; ++j)
                for (int z = 0; z < NSUM; ++z) qv[j][z] = 0.f;
            if (lane < take) {
                qpair = ns.qp[lane];
                const TriGeo& Sq = wake ? a.wtri[list[qpair]] : a.tri[list[qpair]];
                adj_point64(a, T, Sq, ns, pc.nuk, K, qpair, ns.qk[lane], qv);
            }
#pragma unroll
            for (int j = 0; j < ADJ_MAX; ++j)
                if (j < K) seg_accumulate<NSUM>(ns.accf[j], (double (*)[NSUM])nullptr, lane, qpair, qv[j]);
            const int rest = nq - take;
            int mp = 0, mk = 0;
            if (lane < rest) {
                mp = ns.qp[take + lane];
                mk = ns.qk[take + lane];
            }
            __syncwarp();
            if (lane < rest) {
                ns.qp[lane] = mp;
                ns.qk[lane] = mk;
            }
            __syncwarp();
            nq = rest;
            n64 += take;
        }
    }
    __syncwarp();
    // each lane finishes its own pair, for every vector
    if (near) {
        const v3<double> m = mk3(ns.m64[lane][0], ns.m64[lane][1], ns.m64[lane][2]);
        v3<double> xS[3];
        tri_corners(S, xS);
        for (int j = 0; j < K; ++j) {
            double f[NSUM];
            for (int z = 0; z < NSUM; ++z) f[z] = double(ns.accf[j][lane][z]);
            const AdjSums<double> d = sums_unflat(f);
            for (int k = 0; k < 3; ++k) Xg[j][k] += d.Xg[k];
            U[j] += cross(G, d.Q) + sig * d.Q;
            fs[j] += dot(d.Q, m);
            const SrcAdj<double> sa = src_of_pair(xS, d, m, nT);
            double g[NSA];
            sa_flat(sa, g);
            vp_fx* dst = mx.x[j].SA[wake ? 1 : 0] + size_t(s) * NSA;
            for (int z = 0; z < NSA; ++z) fx_add(dst + z, g[z]);
        }
    }
    __syncwarp();
    P[TIER_NEAR] += __popc(nearmask);
    Q[TIER_NEAR] += (unsigned long long)total;
    Q64 += n64;
    return __ballot_sync(FULL, valid && !near);
}

__global__ void __launch_bounds__(32 * NEAR_WARPS) adj_lanes_kernel(NearArgs a, AdjMulti mx) {
    extern __shared__ __align__(16) unsigned char adj_smem[];
    AdjChunkSh& ns = reinterpret_cast<AdjChunkSh*>(adj_smem)[threadIdx.x >> 5];
    const int lane = threadIdx.x & 31;
    const int idx = blockIdx.x * NEAR_WARPS + (threadIdx.x >> 5);
    if (idx >= a.ntests) return;
    const int t = a.tests[idx];
    const TriGeo& T = a.tri[t];
    const int K = mx.nadj;
    PairCtx pc;
    pc.a = &a;
    pc.T = &T;
    pc.sh = nullptr;
    pc.lane = lane;
    for (int k = 0; k < 3; ++k) {
        for (int j = 0; j < ADJ_MAX; ++j) pc.nuk[j][k] = j < K ? mx.x[j].nu[T.slot[k]] : 0.0;
        pc.nu[k] = pc.nuk[0][k];
    }
    v3<double> Xg[ADJ_MAX][3], U[ADJ_MAX];
    double fs[ADJ_MAX];
    for (int j = 0; j < ADJ_MAX; ++j) {
        for (int k = 0; k < 3; ++k) Xg[j][k] = mk3(0.0, 0.0, 0.0);
        U[j] = mk3(0.0, 0.0, 0.0);
        fs[j] = 0;
    }
    unsigned long long P[6] = {0, 0, 0, 0, 0, 0}, Q[6] = {0, 0, 0, 0, 0, 0}, Q64 = 0;
    for (int set = 0; set < 2; ++set) {
        const bool wake = set == 1;
        const long long e0 = wake ? a.wf_ptr[t] : a.nf_ptr[t];
        const long long e1 = wake ? a.wf_ptr[t + 1] : a.nf_ptr[t + 1];
        const int* src = wake ? a.wf_src : a.nf_src;
        int* rest = wake ? a.wrest_src : a.rest_src;
        int nrest = 0;
        for (long long c0 = e0; c0 < e1; c0 += 32) {
            const int cnt = int(e1 - c0 < 32 ? e1 - c0 : 32);
            unsigned m = adj_chunk(pc, ns, mx, t, src + c0, cnt, wake, Xg, U, fs, P, Q, Q64);
            if ((m >> lane) & 1u) rest[e0 + nrest + __popc(m & ((1u << lane) - 1u))] = src[c0 + lane];
            nrest += __popc(m);
        }
        if (lane == 0) a.rest_cnt[2 * t + set] = nrest;
    }
    // the test side, summed over the warp's pairs, per vector
    for (int j = 0; j < K; ++j) {
        double v[NTA] = {Xg[j][0].x, Xg[j][0].y, Xg[j][0].z, Xg[j][1].x, Xg[j][1].y, Xg[j][1].z,
                         Xg[j][2].x, Xg[j][2].y, Xg[j][2].z, U[j].x,     U[j].y,     U[j].z,     fs[j]};
#pragma unroll
        for (int k = 0; k < NTA; ++k) v[k] = warp_sum(v[k]);
        double mine = 0;
#pragma unroll
        for (int k = 0; k < NTA; ++k)
            if (k == lane) mine = v[k];
        if (lane < NTA) fx_add(mx.x[j].TA + size_t(t) * NTA + lane, mine);
    }
    for (int k = 0; k < 6; ++k) {
        unsigned long long pk = P[k], qk = Q[k];
        if (lane == 0 && pk) atomicAdd(a.stats + k, pk);
        if (lane == 0 && qk) atomicAdd(a.stats + 6 + k, qk);
    }
    if (lane == 0 && Q64) atomicAdd(a.stats + 12, Q64);
}

// ------------------------------------------------------------------------------------------------------------------
// non-far pairs, tip filaments and freestream: one warp per test triangle


// this lane's rule-geometry derivative (direction lane < 18) to the test triangle's nodes and the source's
__device__ __forceinline__ void flush_gdir(PairCtx& pc, const AdjMulti& mx, const TriGeo& T, const TriGeo* S,
                                           bool wake) {
    const int d = pc.lane;
    for (int k = 0; k < mx.nadj; ++k) {
        const AdjExtra& x = mx.x[k];
        if (d < 18 && pc.gdir[k] != 0.0) {
            if (d < 9)
                fx_add(x.gx + 3 * T.node[d / 3] + d % 3, pc.gdir[k]);
            else if (S)
                fx_add((wake ? x.gwx + 3 * S->slot[(d - 9) / 3] : x.gx + 3 * S->node[(d - 9) / 3]) + (d - 9) % 3,
                       pc.gdir[k]);
        }
        pc.gdir[k] = 0;
    }
}

// the pair's FP64 sums per adjoint vector, in every lane: FP64 lane sums added over the warp (FP64 path), or the
// warp's totals (mixed path)
__device__ __forceinline__ void pair_sums(PairCtx& pc, AdjAcc& acc, AdjSums<double>* d, int K) {
    fold32(acc);
    for (int j = 0; j < K; ++j) {
        adj_warp_sum(acc.d[j]);
        d[j] = acc.d[j];
    }
}
__device__ __forceinline__ void pair_sums(PairCtx& pc, AdjAccW& acc, AdjSums<double>* d, int K) {
    fold_w(acc, pc.lane);
    pair_totals(acc, d, K);
#pragma unroll
    for (int j = 0; j < ADJ_TSLOT; ++j) acc.tot[j] = 0;
}

__device__ __forceinline__ void acc_init(AdjAcc&, unsigned char*, int, int) {}
__device__ __forceinline__ void acc_init(AdjAccW& acc, unsigned char* smem, int w, int lane) {
    acc.lanes = reinterpret_cast<AdjLane*>(smem) + 32 * w;
    acc.me = acc.lanes + lane;
}

// the pairs the lanes kernel left (self, touching, contact), one warp per pair, for up to ADJ_MAX adjoint vectors at
// once: every point's kernel and derivatives are evaluated once, and each vector keeps its sums. A persistent grid
// whose warps take the next pair of the list from a counter, so that test triangles with many contact pairs do not
// leave the end of the launch to a few warps. The test side of a pair goes to TA, the source side to SA (atomics).
// Acc: AdjAcc (FP64 path: FP64 sums per lane) or AdjAccW (mixed path: FP32 lane partials in dynamic shared memory,
// NEAR_WARPS x 32 AdjLane, folded into the warp's FP64 totals).
template <class Acc>
__global__ void __launch_bounds__(32 * NEAR_WARPS) adj_pairs_kernel(NearArgs a, AdjMulti mx) {
    __shared__ WarpSh shm[NEAR_WARPS];
    extern __shared__ __align__(16) unsigned char adjw_smem[];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if constexpr (std::is_same<Acc, AdjAccW>::value) {
        float* mine = reinterpret_cast<float*>(reinterpret_cast<AdjLane*>(adjw_smem) + threadIdx.x);
        for (int z = 0; z < ADJ_LSTRIDE; ++z) mine[z] = 0.f;
        __syncwarp();
    }
    const int n = 2 * a.ntri;
    const long long total = a.rest_off[n];
    const int K = mx.nadj;
    PairCtx pc;
    pc.a = &a;
    pc.sh = &shm[w];
    pc.lane = lane;
    pc.nleaf = 0;
    pc.nq64 = 0;
    pc.fp32 = 0;
    pc.nadj = K;
    pc.dep = 0;
    for (int j = 0; j < ADJ_MAX; ++j) pc.gdir[j] = 0;
    unsigned long long P[6] = {0, 0, 0, 0, 0, 0}, Q[6] = {0, 0, 0, 0, 0, 0}, Q64 = 0;
    for (;;) {
        const long long idx = next_rest_pair(a.next, lane);
        if (idx >= total) break;
        const int g = rest_entry(a.rest_off, n, idx);
        const int t = g >> 1;
        const int set = g & 1;
        const bool wake = set == 1;
        const long long e0 = wake ? a.wf_ptr[t] : a.nf_ptr[t];
        const int s = (wake ? a.wrest_src : a.rest_src)[e0 + (idx - a.rest_off[g])];
        const TriGeo& T = a.tri[t];
        pc.T = &T;
        for (int k = 0; k < 3; ++k) {
            for (int j = 0; j < ADJ_MAX; ++j) {
                pc.nuk[j][k] = j < K ? mx.x[j].nu[T.slot[k]] : 0.0;
                pc.nukf[j][k] = float(pc.nuk[j][k]);
            }
            pc.nu[k] = pc.nuk[0][k];
            pc.Xc[k] = ld3(T.x + 3 * k) - ld3(T.c);
            pc.Xcf[k] = mk3(float(pc.Xc[k].x), float(pc.Xc[k].y), float(pc.Xc[k].z));
        }
        pc.dep = 0;
        const v3<double> nT = ld3(T.n);
        const TriGeo& S = wake ? a.wtri[s] : a.tri[s];
        const double* gp = (wake ? mx.x[0].gam_w : mx.x[0].gam_b) + 3 * size_t(s);
        const v3<double> G = mk3(gp[0], gp[1], gp[2]);
        const double sig = wake ? 0.0 : S.sigma;
        pc.m = cross(nT, G) + sig * nT;
        pc.mf = mk3(float(pc.m.x), float(pc.m.y), float(pc.m.z));
        Acc acc = {};
        acc_init(acc, adjw_smem, w, lane);
        pc.kind = 0;
        pc.npts = 0;
        pc.n64 = 0;
        pc.nleaf = 0;
        pc.nq64 = 0;
        const int tier = tri_pair(pc, acc, t, s, wake);
        flush_gdir(pc, mx, T, &S, wake);
        AdjSums<double> dsum[ADJ_MAX];
        pair_sums(pc, acc, dsum, K);
        v3<double> xS[3];
        tri_corners(S, xS);
        for (int j = 0; j < K; ++j) {
            const AdjSums<double>& d = dsum[j];
            // the test side: lane k adds field k of the pair's (Xg, U, fs)
            const v3<double> U = cross(G, d.Q) + sig * d.Q;
            const double v[NTA] = {d.Xg[0].x, d.Xg[0].y, d.Xg[0].z, d.Xg[1].x, d.Xg[1].y, d.Xg[1].z,
                                   d.Xg[2].x, d.Xg[2].y, d.Xg[2].z, U.x,       U.y,       U.z,       dot(d.Q, pc.m)};
            double tmine = 0;
#pragma unroll
            for (int k = 0; k < NTA; ++k)
                if (k == lane) tmine = v[k];
            if (lane < NTA) fx_add(mx.x[j].TA + size_t(t) * NTA + lane, tmine);
            // the source side: lane k adds field k
            SrcAdj<double> sa = src_of_pair(xS, d, pc.m, nT);
            double f[NSA];
            sa_flat(sa, f);
            vp_fx* dst = mx.x[j].SA[set] + size_t(s) * NSA;
            double mine = 0, mine2 = 0;
#pragma unroll
            for (int k = 0; k < 32; ++k)
                if (k == lane) mine = f[k];
#pragma unroll
            for (int k = 32; k < NSA; ++k)
                if (k - 32 == lane) mine2 = f[k];
            fx_add(dst + lane, mine);
            if (lane < NSA - 32) fx_add(dst + 32 + lane, mine2);
        }
        __syncwarp();
        P[tier] += 1;
        Q[tier] += pc.npts;
        Q64 += pc.n64;
    }
    if (lane == 0) {
        for (int k = 0; k < 6; ++k) {
            if (P[k]) atomicAdd(a.stats + k, P[k]);
            if (Q[k]) atomicAdd(a.stats + 6 + k, Q[k]);
        }
        if (Q64) atomicAdd(a.stats + 12, Q64);
    }
}

// one far tip filament (ends ia, ib) of test triangle T, summed by one lane for every adjoint vector: the far rule's
// points of the filament's part of f = sum W nu (mu_a va + mu_b vb)·n_T (eval_point64's filament branch), added to
// the lane's test-side sums Xg, U, fs; the derivatives to the filament's end nodes go to gwx
__device__ void far_filament_adj(const NearArgs& a, const AdjMulti& mx, const PairCtx& pc, const TriGeo& T, int ia,
                                 int ib, v3<double> fa, v3<double> fb, v3<double> (*Xg)[3], v3<double>* U,
                                 double* fs) {
    const RulePt* R = a.rule[R_FAR];
    const v3<double> n = ld3(T.n);
    const double mua = mx.x[0].mu[a.nslot + ia], mub = mx.x[0].mu[a.nslot + ib];
    v3<double> Ea[3], Eb[3];
    for (int k = 0; k < 3; ++k) {
        Ea[k] = ld3(T.x + 3 * k) - fa;
        Eb[k] = ld3(T.x + 3 * k) - fb;
    }
    v3<double> Ga[ADJ_MAX], Gb[ADJ_MAX], Qs[ADJ_MAX];
    for (int j = 0; j < ADJ_MAX; ++j) Ga[j] = Gb[j] = Qs[j] = mk3(0.0, 0.0, 0.0);
    for (int i = 0; i < a.nrule[R_FAR]; ++i) {
        const RulePt m = R[i];
        const double W = m.w * T.area;
        const v3<double> psi = test_weights(a.test_mode, m.l0, m.l1, m.l2);
        const v3<double> ra = m.l0 * Ea[0] + m.l1 * Ea[1] + m.l2 * Ea[2];
        const v3<double> rb = m.l0 * Eb[0] + m.l1 * Eb[1] + m.l2 * Eb[2];
        v3<double> va, vb, ga, gb;
        segment_velocity(ra, rb, va, vb);
        seg_vjp(ra, rb, n, mua, mub, ga, gb);
        const v3<double> gx = ga + gb;
        const v3<double> q = mua * va + mub * vb;
        for (int j = 0; j < mx.nadj; ++j) {
            const double Wn = W * (pc.nuk[j][0] * psi.x + pc.nuk[j][1] * psi.y + pc.nuk[j][2] * psi.z);
            Qs[j] += Wn * q;
            Xg[j][0] += (Wn * m.l0) * gx;
            Xg[j][1] += (Wn * m.l1) * gx;
            Xg[j][2] += (Wn * m.l2) * gx;
            Ga[j] += Wn * ga;
            Gb[j] += Wn * gb;
        }
    }
    for (int j = 0; j < mx.nadj; ++j) {
        U[j] += Qs[j];
        fs[j] += dot(Qs[j], n);
        vp_fx* g = mx.x[j].gwx;
        fx_add(g + 3 * ia + 0, -Ga[j].x);
        fx_add(g + 3 * ia + 1, -Ga[j].y);
        fx_add(g + 3 * ia + 2, -Ga[j].z);
        fx_add(g + 3 * ib + 0, -Gb[j].x);
        fx_add(g + 3 * ib + 1, -Gb[j].y);
        fx_add(g + 3 * ib + 2, -Gb[j].z);
    }
}

// the tip filaments and the freestream of one test triangle (one warp each), for up to ADJ_MAX adjoint vectors
__global__ void __launch_bounds__(32 * NEAR_WARPS) adj_near_kernel(NearArgs a, AdjMulti mx) {
    __shared__ WarpSh shm[NEAR_WARPS];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int idx = blockIdx.x * NEAR_WARPS + w;
    if (idx >= a.ntests) return;
    const int t = a.tests[idx];
    const TriGeo& T = a.tri[t];
    const int K = mx.nadj;
    PairCtx pc;
    pc.a = &a;
    pc.T = &T;
    pc.sh = &shm[w];
    pc.lane = lane;
    pc.nleaf = 0;
    pc.nq64 = 0;
    pc.fp32 = 0;
    pc.nadj = K;
    for (int k = 0; k < 3; ++k) {
        for (int j = 0; j < ADJ_MAX; ++j) {
            pc.nuk[j][k] = j < K ? mx.x[j].nu[T.slot[k]] : 0.0;
            pc.nukf[j][k] = float(pc.nuk[j][k]);
        }
        pc.nu[k] = pc.nuk[0][k];
        pc.Xc[k] = ld3(T.x + 3 * k) - ld3(T.c);
        pc.Xcf[k] = mk3(float(pc.Xc[k].x), float(pc.Xc[k].y), float(pc.Xc[k].z));
    }
    pc.dep = 0;
    for (int j = 0; j < ADJ_MAX; ++j) pc.gdir[j] = 0;
    const v3<double> nT = ld3(T.n);
    v3<double> Xg[ADJ_MAX][3], U[ADJ_MAX];
    double fs[ADJ_MAX], dal[ADJ_MAX];
    for (int j = 0; j < ADJ_MAX; ++j) {
        for (int k = 0; k < 3; ++k) Xg[j][k] = mk3(0.0, 0.0, 0.0);
        U[j] = mk3(0.0, 0.0, 0.0);
        fs[j] = dal[j] = 0;
    }
    unsigned long long P[6] = {0, 0, 0, 0, 0, 0}, Q[6] = {0, 0, 0, 0, 0, 0}, Q64 = 0;
    const double corners[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    // tip filaments (assemble.jl:344-354), FP64: f = sum W nu (mu_a va + mu_b vb)·n_T. A warp takes 32 filaments at
    // once: a far one (the far rule's few points) is summed by its own lane, the others by the whole warp.
    {
        v3<double> lXg[ADJ_MAX][3], lU[ADJ_MAX];
        double lfs[ADJ_MAX];
        for (int j = 0; j < ADJ_MAX; ++j) {
            for (int k = 0; k < 3; ++k) lXg[j][k] = mk3(0.0, 0.0, 0.0);
            lU[j] = mk3(0.0, 0.0, 0.0);
            lfs[j] = 0;
        }
        for (int f0 = 0; f0 < a.nfil; f0 += 32) {
            const int cnt = a.nfil - f0 < 32 ? a.nfil - f0 : 32;
            bool mfar = false;
            if (lane < cnt) {
                const int ia = a.fil[2 * (f0 + lane)], ib = a.fil[2 * (f0 + lane) + 1];
                const v3<double> fa = ld3(a.wx + 3 * ia), fb = ld3(a.wx + 3 * ib);
                mfar = vnorm((fa + fb) / 2.0 - ld3(T.c)) > a.far_ratio * fmax(T.diam, vnorm(fb - fa));
                if (mfar)
                    far_filament_adj(a, mx, pc, T, ia, ib, fa, fb, lXg, lU, lfs);
            }
            const unsigned farmask = __ballot_sync(0xffffffffu, mfar);
            P[TIER_FAR] += __popc(farmask);
            Q[TIER_FAR] += (unsigned long long)__popc(farmask) * a.nrule[R_FAR];
            for (int q = 0; q < cnt; ++q) {
                if ((farmask >> q) & 1u) continue;
                // near and vertex filaments (segment_rule, assemble.jl:299-306), the whole warp
                const int fi = f0 + q;
                const int ia = a.fil[2 * fi], ib = a.fil[2 * fi + 1];
                v3<double> fa = ld3(a.wx + 3 * ia), fb = ld3(a.wx + 3 * ib);
                if (lane == 0) {
                    for (int k = 0; k < 3; ++k) {
                        pc.sh->E[9 * k + 0] = T.x[3 * k + 0] - fa.x;
                        pc.sh->E[9 * k + 1] = T.x[3 * k + 1] - fa.y;
                        pc.sh->E[9 * k + 2] = T.x[3 * k + 2] - fa.z;
                        pc.sh->E[9 * k + 3] = T.x[3 * k + 0] - fb.x;
                        pc.sh->E[9 * k + 4] = T.x[3 * k + 1] - fb.y;
                        pc.sh->E[9 * k + 5] = T.x[3 * k + 2] - fb.z;
                    }
                }
                __syncwarp();
                AdjAcc acc = {};
                pc.kind = 1;
                pc.npts = 0;
                pc.n64 = 0;
                pc.side = 0;
                pc.fp32 = 0;
                pc.mua = mx.x[0].mu[a.nslot + ia];
                pc.mub = mx.x[0].mu[a.nslot + ib];
                int tier, kv = -1;
                for (int k = 0; k < 3 && kv < 0; ++k)
                    if (fmin(vnorm(ld3(T.x + 3 * k) - fa), vnorm(ld3(T.x + 3 * k) - fb)) <= 1e-12 * T.diam) kv = k;
                if (kv >= 0) {
                    tier = TIER_VERTEX;
                    vertex_rule(pc, acc, kv);
                } else {
                    tier = TIER_NEAR;
                    SrcRef src{1, nullptr, fa, fb};
                    near_pieces(pc, acc, src, corners, 1.0, a.near_depth);
                    flush_leaves(pc, acc);
                }
                flush_gdir(pc, mx, T, nullptr, false);
                for (int j = 0; j < K; ++j) {
                    adj_warp_sum(acc.d[j]);
                    const AdjSums<double>& d = acc.d[j];
                    for (int k = 0; k < 3; ++k) Xg[j][k] += d.Xg[k];
                    U[j] += d.Q;
                    fs[j] += dot(d.Q, nT);
                    if (lane < 3) {
                        const double ga[3] = {d.Gr[0].x, d.Gr[0].y, d.Gr[0].z},
                                     gb[3] = {d.Gr[1].x, d.Gr[1].y, d.Gr[1].z};
                        fx_add(mx.x[j].gwx + 3 * ia + lane, -ga[lane]);
                        fx_add(mx.x[j].gwx + 3 * ib + lane, -gb[lane]);
                    }
                }
                __syncwarp();
                P[tier] += 1;
                Q[tier] += pc.npts;
                Q64 += pc.n64;
            }
        }
        // the lanes' far filaments into the warp's test-side sums
        for (int j = 0; j < K; ++j) {
            for (int k = 0; k < 3; ++k) Xg[j][k] += wsum3(lXg[j][k]);
            U[j] += wsum3(lU[j]);
            fs[j] += wsum_d(lfs[j]);
        }
    }
    // freestream (assemble.jl:422): (V·n_T) A_T sum_a nu_a ti_a, and the test side of every vector
    const v3<double> V = mk3(mx.x[0].V[0], mx.x[0].V[1], mx.x[0].V[2]);
    const v3<double> dV = mk3(mx.x[0].dV[0], mx.x[0].dV[1], mx.x[0].dV[2]);
    for (int j = 0; j < K; ++j) {
        const double c = (pc.nuk[j][0] * a.tint[0] + pc.nuk[j][1] * a.tint[1] + pc.nuk[j][2] * a.tint[2]) * T.area;
        U[j] += c * V;
        fs[j] += c * dot(V, nT);
        dal[j] += c * dot(dV, nT);
        const double v[NTA] = {Xg[j][0].x, Xg[j][0].y, Xg[j][0].z, Xg[j][1].x, Xg[j][1].y, Xg[j][1].z,
                               Xg[j][2].x, Xg[j][2].y, Xg[j][2].z, U[j].x,     U[j].y,     U[j].z,     fs[j]};
        double mine = 0;
#pragma unroll
        for (int k = 0; k < NTA; ++k)
            if (k == lane) mine = v[k];
        if (lane < NTA) fx_add(mx.x[j].TA + size_t(t) * NTA + lane, mine);
        if (lane == 0) fx_add(mx.x[j].dal, dal[j]);
    }
    if (lane == 0) {
        for (int k = 0; k < 6; ++k) {
            if (P[k]) atomicAdd(a.stats + k, P[k]);
            if (Q[k]) atomicAdd(a.stats + 6 + k, Q[k]);
        }
        if (Q64) atomicAdd(a.stats + 12, Q64);
    }
}

// ------------------------------------------------------------------------------------------------------------------
// finish: node derivatives from the per-triangle sums, one thread per triangle (body, then wake)

struct AdjFinish {
    const TriGeo* tri;
    const TriGeo* wtri;
    int ntri, nwtri, nslot;
    const vp_fx* TA;
    const vp_fx* SA[2];
    const double* mu;
    double V[3], dV[3];
    vp_fx* gx;   // body node derivatives (3 each)
    vp_fx* gwx;  // wake node derivatives
    vp_fx* dal;
};

__global__ void adj_finish_kernel(AdjFinish f) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double dal = 0;
    if (i < f.ntri + f.nwtri) {
        const bool wake = i >= f.ntri;
        const int s = wake ? i - f.ntri : i;
        const TriGeo& g = wake ? f.wtri[s] : f.tri[s];
        v3<double> v[3], gr[3] = {mk3(0.0, 0.0, 0.0), mk3(0.0, 0.0, 0.0), mk3(0.0, 0.0, 0.0)};
        tri_corners(g, v);
        if (!wake) {
            double ta[NTA];
            for (int k = 0; k < NTA; ++k) ta[k] = fx_get(f.TA[size_t(s) * NTA + k]);
            v3<double> Xg[3] = {mk3(ta[0], ta[1], ta[2]), mk3(ta[3], ta[4], ta[5]), mk3(ta[6], ta[7], ta[8])};
            test_adj_grad(v, Xg, mk3(ta[9], ta[10], ta[11]), ta[12], gr);
        }
        const SrcAdj<double> sa = sa_unflat(f.SA[wake ? 1 : 0] + size_t(s) * NSA);
        double mu[3];
        for (int k = 0; k < 3; ++k) mu[k] = f.mu[(wake ? f.nslot : 0) + g.slot[k]];
        src_adj_grad(v, sa, mu, !wake, mk3(f.V[0], f.V[1], f.V[2]), mk3(f.dV[0], f.dV[1], f.dV[2]), gr, &dal);
        vp_fx* dst = wake ? f.gwx : f.gx;
        for (int k = 0; k < 3; ++k) {
            const int node = wake ? g.slot[k] : g.node[k];
            fx_add(dst + 3 * node, gr[k].x);
            fx_add(dst + 3 * node + 1, gr[k].y);
            fx_add(dst + 3 * node + 2, gr[k].z);
        }
    }
    dal = warp_sum(dal);
    if ((threadIdx.x & 31) == 0) fx_add(f.dal, dal);
}

template <class T>
void fill_gam(const std::vector<TriGeo>& g, int n, const double* mu, int col0, int pad, std::vector<T>& out) {
    out.assign(size_t(3) * std::max(pad, 1), T(0));
    for (int s = 0; s < n; ++s)
        for (int k = 0; k < 3; ++k) {
            double v = 0;
            for (int b = 0; b < 3; ++b) v += mu[col0 + g[s].slot[b]] * g[s].gam[3 * b + k];
            out[size_t(k) * pad + s] = T(v);
        }
}

// the far tier for the adjoint vectors x[0 .. K-1] in one launch
template <class T, int TT, int K>
int run_adj_far(vp_ctx* ctx, const PairSetup& ps, const PairInput& in, const AdjExtra* x, const double* mu,
                DevList& dl) {
    AdjFarArgs fa{};
    fa.ntest = in.ntri;
    fa.nq = ps.nq;
    fa.ntiles_test = (in.ntri + TT - 1) / TT;
    fa.tq = ps.d_tq;
    fa.tw = ps.d_tw;
    fa.tgeo = ps.d_tg;
    fa.tcent = ps.d_tc;
    for (int j = 0; j < K; ++j) {
        fa.nu[j] = x[j].nu;
        fa.SA[j][0] = x[j].SA[0];
        fa.SA[j][1] = x[j].SA[1];
        fa.TA[j] = x[j].TA;
    }
    fa.nset = in.nwtri > 0 ? 2 : 1;
    fa.ratio32 = ps.ratio32;
    fa.ratio = in.o->far_ratio;
    fa.kernel_far = in.o->kernel_far;
    int r;
    {
        std::vector<double> lam(3 * NQMAX, 0.0);
        for (int p = 0; p < ps.nq; ++p) {
            lam[3 * p] = ps.rfar[p].l0;
            lam[3 * p + 1] = ps.rfar[p].l1;
            lam[3 * p + 2] = ps.rfar[p].l2;
        }
        double* d;
        if ((r = dl.up(ctx, &d, lam))) return r;
        fa.lam = d;
    }
    const std::vector<TriGeo>* sets[2] = {&ps.tg, &ps.wg};
    const int nsrc[2] = {in.ntri, in.nwtri};
    int tiles = 0;
    for (int set = 0; set < fa.nset; ++set) {
        std::vector<TriGeo> g(sets[set]->begin(), sets[set]->begin() + nsrc[set]);
        std::vector<T> soa, gam;
        fill_soa(g, soa, fa.pad[set]);
        fill_gam(g, nsrc[set], mu, set == 0 ? 0 : in.nslot, fa.pad[set], gam);
        T *d_soa, *d_gam;
        if ((r = dl.up(ctx, &d_soa, soa)) || (r = dl.up(ctx, &d_gam, gam))) return r;
        fa.soa[set] = d_soa;
        fa.gam[set] = d_gam;
        fa.nsrc[set] = nsrc[set];
        fa.ntile[set] = (nsrc[set] + FAR_NT - 1) / FAR_NT;
        fa.scent[set] = set == 0 ? ps.d_tc : ps.d_wc;
        fa.sgeo[set] = set == 0 ? ps.d_tg : ps.d_wg;
        tiles += fa.ntile[set];
    }
    // enough CTAs for a few per SM: split the test tiles into chunks
    int chunks = std::max(1, std::min(fa.ntiles_test, (6 * ctx->nsm + tiles - 1) / std::max(tiles, 1)));
    fa.tiles_per_chunk = (fa.ntiles_test + chunks - 1) / chunks;
    chunks = (fa.ntiles_test + fa.tiles_per_chunk - 1) / fa.tiles_per_chunk;
    vp_phase_begin(ctx, PH_ADJ_FAR);
    adj_far_kernel<T, TT, K><<<dim3(tiles, chunks), FAR_NT, 0, ctx->stream>>>(fa);
    vp_phase_end(ctx);
    ctx->launches++;
    VP_CUDA(ctx, cudaGetLastError());
    return VP_OK;
}

}  // namespace

int vp_adjoint_impl(vp_ctx* ctx, const vp_assembly_options* o, int nnode, const double* x, int ntri, const int* tris,
                    const int* corner_slot, int nslot, int ntouch, const int* touch_pairs, const double* sigma,
                    const double* vinf, int nwnode, const double* wx, int nwtri, const int* wtris, int nfil,
                    const int* fil, int nadj, const double* nu, const double* mu, const double* dvinf, double* grad_x,
                    double* grad_wx, double* dalpha, vp_assembly_stats* stats) {
    auto t0 = std::chrono::steady_clock::now();
    if (!nu || !mu || !dvinf || !grad_x || !dalpha || (nwnode > 0 && !grad_wx))
        return vp_fail(ctx, VP_ERR_ARG, "null argument");
    if (nadj < 1 || nadj > ADJ_MAX) return vp_fail(ctx, VP_ERR_ARG, "nadj must be 1 or 2");
    const PairInput in{o,     nnode, x,     ntri, tris,  corner_slot, nslot, ntouch, touch_pairs,
                       sigma, vinf,  nwnode, wx,  nwtri, wtris,       nfil,  fil};
    PairSetup ps;
    int r = setup_pairs(ctx, in, PH_ADJOINT, PH_ADJOINT, ps);
    if (r) return r;
    DevList& dl = ps.dl;
    const int ncols = ps.ncols;
    vp_phase_begin(ctx, PH_ADJOINT);
    double *d_mu, *d_gamb, *d_gamw;
    unsigned long long* d_stats;
    std::vector<double> hmu(mu, mu + ncols);
    std::vector<double> gamb(size_t(3) * ntri), gamw(size_t(3) * std::max(nwtri, 1), 0.0);
    for (int s = 0; s < ntri; ++s)
        for (int k = 0; k < 3; ++k) {
            double v = 0;
            for (int b = 0; b < 3; ++b) v += mu[ps.tg[s].slot[b]] * ps.tg[s].gam[3 * b + k];
            gamb[3 * size_t(s) + k] = v;
        }
    for (int s = 0; s < nwtri; ++s)
        for (int k = 0; k < 3; ++k) {
            double v = 0;
            for (int b = 0; b < 3; ++b) v += mu[nslot + ps.wg[s].slot[b]] * ps.wg[s].gam[3 * b + k];
            gamw[3 * size_t(s) + k] = v;
        }
    if ((r = dl.up(ctx, &d_mu, hmu)) || (r = dl.up(ctx, &d_gamb, gamb)) || (r = dl.up(ctx, &d_gamw, gamw)) ||
        (r = dl.alloc(ctx, &d_stats, 13)))
        return r;
    VP_CUDA(ctx, cudaMemsetAsync(d_stats, 0, sizeof(unsigned long long) * 13, ctx->stream));
    // per adjoint vector: its values and outputs
    AdjMulti mx{};
    mx.nadj = nadj;
    for (int k = 0; k < nadj; ++k) {
        AdjExtra& ex = mx.x[k];
        double* d_nu;
        vp_fx *d_SA0, *d_SA1, *d_TA, *d_gx, *d_gwx, *d_dal;
        std::vector<double> hnu(nu + size_t(k) * nslot, nu + size_t(k + 1) * nslot);
        if ((r = dl.up(ctx, &d_nu, hnu)) || (r = dl.alloc(ctx, &d_SA0, size_t(NSA) * ntri)) ||
            (r = dl.alloc(ctx, &d_SA1, size_t(NSA) * std::max(nwtri, 1))) ||
            (r = dl.alloc(ctx, &d_TA, size_t(NTA) * ntri)) || (r = dl.alloc(ctx, &d_gx, size_t(3) * nnode)) ||
            (r = dl.alloc(ctx, &d_gwx, size_t(3) * std::max(nwnode, 1))) || (r = dl.alloc(ctx, &d_dal, 1)))
            return r;
        VP_CUDA(ctx, cudaMemsetAsync(d_SA0, 0, sizeof(vp_fx) * NSA * ntri, ctx->stream));
        VP_CUDA(ctx, cudaMemsetAsync(d_SA1, 0, sizeof(vp_fx) * NSA * std::max(nwtri, 1), ctx->stream));
        VP_CUDA(ctx, cudaMemsetAsync(d_TA, 0, sizeof(vp_fx) * NTA * ntri, ctx->stream));
        VP_CUDA(ctx, cudaMemsetAsync(d_gx, 0, sizeof(vp_fx) * 3 * nnode, ctx->stream));
        VP_CUDA(ctx, cudaMemsetAsync(d_gwx, 0, sizeof(vp_fx) * 3 * std::max(nwnode, 1), ctx->stream));
        VP_CUDA(ctx, cudaMemsetAsync(d_dal, 0, sizeof(vp_fx), ctx->stream));
        ex.nu = d_nu;
        ex.mu = d_mu;
        ex.gam_b = d_gamb;
        ex.gam_w = d_gamw;
        for (int z = 0; z < 3; ++z) {
            ex.V[z] = vinf[z];
            ex.dV[z] = dvinf[z];
        }
        ex.SA[0] = d_SA0;
        ex.SA[1] = d_SA1;
        ex.TA = d_TA;
        ex.gx = d_gx;
        ex.gwx = d_gwx;
        ex.dal = d_dal;
    }
    vp_phase_end(ctx);
    // far tier, one launch per adjoint vector
    // (mixed: both vectors in one pass; FP64: a launch per vector, whose FP64 sums would not fit twice in registers)
    if (ps.mixed && nadj == 2) {
        if ((r = run_adj_far<float, 8, 2>(ctx, ps, in, mx.x, mu, dl))) return r;
    } else {
        for (int k = 0; k < nadj; ++k) {
            r = ps.mixed ? run_adj_far<float, 8, 1>(ctx, ps, in, mx.x + k, mu, dl)
                         : run_adj_far<double, 4, 1>(ctx, ps, in, mx.x + k, mu, dl);
            if (r) return r;
        }
    }
    // non-far pairs: the near tier one pair per lane (a launch per adjoint vector), then the rest with all vectors
    {
        std::vector<int> all(ntri);
        std::iota(all.begin(), all.end(), 0);
        int* d_tests;
        if ((r = dl.up(ctx, &d_tests, all))) return r;
        NearArgs na = near_args(ps, in);
        na.tests = d_tests;
        na.ntests = ntri;
        int *d_rest, *d_wrest, *d_rcnt;
        if ((r = dl.alloc(ctx, &d_rest, size_t(std::max(ps.nfptr[ntri], 1LL)))) ||
            (r = dl.alloc(ctx, &d_wrest, size_t(std::max(ps.wfptr[ntri], 1LL)))) ||
            (r = dl.alloc(ctx, &d_rcnt, size_t(2) * ntri)))
            return r;
        na.rest_src = d_rest;
        na.wrest_src = d_wrest;
        na.rest_cnt = d_rcnt;
        const size_t smem = sizeof(AdjChunkSh) * NEAR_WARPS;
        VP_CUDA(ctx, cudaFuncSetAttribute(adj_lanes_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
        const int nb = (ntri + NEAR_WARPS - 1) / NEAR_WARPS;
        vp_phase_begin(ctx, PH_ADJ_NEAR);
        na.stats = d_stats;
        adj_lanes_kernel<<<nb, 32 * NEAR_WARPS, smem, ctx->stream>>>(na, mx);  // every vector in one pass
        if ((r = rest_list(ctx, dl, na, nullptr))) return r;
        vp_phase_end(ctx);
        vp_phase_begin(ctx, PH_ADJ_PAIRS);
        if (na.mixed) {  // FP32 lane partials in shared memory, FP64 totals per warp
            const size_t wsm = sizeof(AdjLane) * 32 * NEAR_WARPS;
            VP_CUDA(ctx, cudaFuncSetAttribute(adj_pairs_kernel<AdjAccW>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              int(wsm)));
            const int npb = persistent_blocks(ctx, adj_pairs_kernel<AdjAccW>, 32 * NEAR_WARPS, wsm);
            adj_pairs_kernel<AdjAccW><<<npb, 32 * NEAR_WARPS, wsm, ctx->stream>>>(na, mx);
        } else {
            const int npb = persistent_blocks(ctx, adj_pairs_kernel<AdjAcc>, 32 * NEAR_WARPS, 0);
            adj_pairs_kernel<AdjAcc><<<npb, 32 * NEAR_WARPS, 0, ctx->stream>>>(na, mx);
        }
        vp_phase_end(ctx);
        vp_phase_begin(ctx, PH_ADJ_NEAR);
        adj_near_kernel<<<nb, 32 * NEAR_WARPS, 0, ctx->stream>>>(na, mx);
        vp_phase_end(ctx);
        ctx->launches += 3;
        VP_CUDA(ctx, cudaGetLastError());
    }
    vp_phase_begin(ctx, PH_ADJOINT);
    // node derivatives, per adjoint vector
    for (int k = 0; k < nadj; ++k) {
        const AdjExtra& ex = mx.x[k];
        AdjFinish f{};
        f.tri = ps.d_tg;
        f.wtri = ps.d_wg;
        f.ntri = ntri;
        f.nwtri = nwtri;
        f.nslot = nslot;
        f.TA = ex.TA;
        f.SA[0] = ex.SA[0];
        f.SA[1] = ex.SA[1];
        f.mu = d_mu;
        for (int z = 0; z < 3; ++z) {
            f.V[z] = vinf[z];
            f.dV[z] = dvinf[z];
        }
        f.gx = ex.gx;
        f.gwx = ex.gwx;
        f.dal = ex.dal;
        const int n = ntri + nwtri;
        adj_finish_kernel<<<(n + 127) / 128, 128, 0, ctx->stream>>>(f);
        ctx->launches++;
        VP_CUDA(ctx, cudaGetLastError());
    }
    vp_phase_end(ctx);
    unsigned long long hs[13];
    std::vector<vp_fx> hgx(size_t(nadj) * 3 * nnode), hgw(size_t(nadj) * 3 * std::max(nwnode, 1)), hdal(nadj);
    for (int k = 0; k < nadj; ++k) {
        const AdjExtra& ex = mx.x[k];
        VP_CUDA(ctx, vp_d2h(ctx, hgx.data() + size_t(k) * 3 * nnode, ex.gx, sizeof(vp_fx) * 3 * nnode));
        if (nwnode > 0)
            VP_CUDA(ctx, vp_d2h(ctx, hgw.data() + size_t(k) * 3 * nwnode, ex.gwx, sizeof(vp_fx) * 3 * nwnode));
        VP_CUDA(ctx, vp_d2h(ctx, hdal.data() + k, ex.dal, sizeof(vp_fx)));
    }
    VP_CUDA(ctx, vp_d2h(ctx, hs, d_stats, sizeof(hs)));
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return vp_fail(ctx, VP_ERR_CUDA, std::string("adjoint kernels: ") + cudaGetErrorString(e));
    for (size_t i = 0; i < size_t(nadj) * 3 * nnode; ++i) grad_x[i] = fx_get(hgx[i]);
    if (nwnode > 0)
        for (size_t i = 0; i < size_t(nadj) * 3 * nwnode; ++i) grad_wx[i] = fx_get(hgw[i]);
    for (int k = 0; k < nadj; ++k) dalpha[k] = fx_get(hdal[k]);
    if (stats) {
        const int nq = ps.nq;
        long long total = (long long)ntri * (ntri + nwtri) + (long long)ntri * nfil;
        long long nonfar = 0;
        for (int k = 0; k < 6; ++k) {
            stats->pairs[k] = (long long)hs[k];
            stats->points[k] = (long long)hs[6 + k];
            if (k != TIER_FAR) nonfar += (long long)hs[k];
        }
        long long far_fil = (long long)hs[TIER_FAR];
        long long far_tri = total - nonfar - far_fil;
        stats->pairs[TIER_FAR] = far_tri + far_fil;
        stats->points[TIER_FAR] = (long long)hs[6 + TIER_FAR] + far_tri * nq;
        stats->points_fp64 = (long long)hs[12] + (ps.mixed ? 0 : far_tri * nq);
        stats->time_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    }
    return VP_OK;
}
