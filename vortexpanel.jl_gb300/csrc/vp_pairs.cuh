// Shared by the assembly (vp_assemble.cu) and its adjoint (vp_gradient.cu): quadrature rules, element data, the far
// test and the classification kernel, the pair-rule walkers of the near, touching and contact tiers (templated on
// the per-lane accumulator: the forward block or the adjoint sums), and the host helpers for tiles and colours.
// Everything sits in an anonymous namespace: each translation unit has its own copy.
#pragma once
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <numeric>
#include <type_traits>
#include <unordered_map>

#include "vp_adjoint_common.cuh"
#include "vp_internal.h"
#include "vp_math.cuh"
namespace {

constexpr int FAR_NT = 128;  // sources per far tile (one per thread)
constexpr int NQMAX = 7;     // points of the far rule, at most
constexpr int NFIELD = 42;   // scalar fields per source in the far kernel's SoA
constexpr int NEAR_WARPS = 4;
constexpr int LEAFBUF = 32;
constexpr int ADJ_MAX = ADJ_VEC_MAX;  // adjoint vectors of one pass
// FP32 guard of the adjoint's derivative evaluations (corner, edge sin^2, plane): the forward's (the derivatives keep
// the accuracy of the values there: adjoint gradients within 3e-6 of the FP64 path's on the wings measured)
// The FP32 guard of the pair integrals (Fp32Guard: corner, edge_sin2, plane): a point goes to FP64 where it sees a
// source edge at an angle whose sine squared is below edge_sin2 from inside the edge's span, or lies within 1e-4 of
// the plane over the triangle, or within 1e-4 source diameters of a corner. Measured against FP64 on the touching and
// contact tiers of a lifting wing (offsets interpolated in FP32 as the kernels form them), the FP32 error of a value
// does not grow toward a corner, so the corner bound only keeps the offsets from vanishing; it grows as the edge angle
// closes, to ~1e-5 of the point's value at a sine squared of 1e-2 (the forward's bound). The adjoint's derivatives
// grow like 1/r toward a corner and an edge, and their FP32 sums over a piece cancel: with a corner bound of 1e-4 the
// 25k wing's mixed gradients moved from 5e-6 to 5e-5 of FP64 (6e-5 with the edge bound of 1e-2 as well), so the
// adjoint keeps 1e-2 diameters at corners and 4e-2 at edges.
#define PAIR_GUARD 1e-4f, 1e-2f, 1e-4f
#define ADJ_GUARD 1e-2f, 4e-2f, 1e-4f

// ------------------------------------------------------------------------------------------------------------------
// host: quadrature rules (src/elements/rules.jl)

struct RulePt {
    double l0, l1, l2, w;
};

void gauss_legendre(int n, std::vector<double>& x, std::vector<double>& w) {  // rules.jl:12-37
    x.assign(n, 0.0);
    w.assign(n, 0.0);
    for (int i = 1; i <= (n + 1) / 2; ++i) {
        double z = std::cos(M_PI * (i - 0.25) / (n + 0.5));
        double dp = 0;
        for (int it = 0; it < 100; ++it) {
            double p1 = 1, p2 = 0;
            for (int j = 1; j <= n; ++j) {
                double p3 = p2;
                p2 = p1;
                p1 = ((2 * j - 1) * z * p2 - (j - 1) * p3) / j;
            }
            dp = n * (z * p1 - p2) / (z * z - 1);
            double dz = p1 / dp;
            z -= dz;
            if (std::fabs(dz) < 1e-16) break;
        }
        double p1 = 1, p2 = 0;
        for (int j = 1; j <= n; ++j) {
            double p3 = p2;
            p2 = p1;
            p1 = ((2 * j - 1) * z * p2 - (j - 1) * p3) / j;
        }
        dp = n * (z * p1 - p2) / (z * z - 1);
        x[i - 1] = (1 - z) / 2;
        x[n - i] = (1 + z) / 2;
        w[i - 1] = w[n - i] = 1 / ((1 - z * z) * dp * dp);
    }
}

void graded_gauss(int levels, double ratio, int order, std::vector<double>& x, std::vector<double>& w) {  // :48-64
    std::vector<double> br{0.0};
    for (int k = levels; k >= 1; --k) br.push_back(std::pow(ratio, k));
    br.push_back(1.0);
    x.clear();
    w.clear();
    for (size_t k = 1; k < br.size(); ++k) {
        std::vector<double> xg, wg;
        gauss_legendre(order + int(k) - 1, xg, wg);
        double a = br[k - 1], b = br[k];
        for (size_t i = 0; i < xg.size(); ++i) {
            if (k == 1) {
                x.push_back(b * xg[i] * xg[i]);
                w.push_back(2 * b * xg[i] * wg[i]);
            } else {
                x.push_back(a + (b - a) * xg[i]);
                w.push_back((b - a) * wg[i]);
            }
        }
    }
}

std::vector<RulePt> triangle_rule(int n) {  // rules.jl:76-92
    std::vector<RulePt> r;
    auto perm = [&](double a, double b, double wt) {
        r.push_back({a, b, b, wt});
        r.push_back({b, a, b, wt});
        r.push_back({b, b, a, wt});
    };
    if (n == 1) {
        r.push_back({1.0 / 3, 1.0 / 3, 1.0 / 3, 1.0});
    } else if (n == 3) {
        perm(2.0 / 3, 1.0 / 6, 1.0 / 3);
    } else if (n == 6) {
        double a = 0.445948490915965, b = 0.091576213509771;
        perm(1 - 2 * a, a, 0.223381589678011);
        perm(1 - 2 * b, b, 0.109951743655322);
    } else if (n == 7) {
        double s = std::sqrt(15.0);
        double a = (6 - s) / 21, b = (6 + s) / 21;
        r.push_back({1.0 / 3, 1.0 / 3, 1.0 / 3, 9.0 / 40});
        perm(1 - 2 * a, a, (155 - s) / 1200);
        perm(1 - 2 * b, b, (155 + s) / 1200);
    }
    return r;
}

std::vector<RulePt> edge_rule(int levels, double ratio, int order) {  // rules.jl:108-118
    std::vector<double> ts, wt, s0, w0;
    graded_gauss(levels, ratio, order, ts, wt);
    graded_gauss(std::max(1, levels / 2), ratio, order, s0, w0);
    size_t m = s0.size();
    std::vector<double> ss(2 * m), ws(2 * m);  // graded_gauss_both (rules.jl:66-70)
    for (size_t i = 0; i < m; ++i) {
        ss[i] = s0[i] / 2;
        ws[i] = w0[i] / 2;
        ss[m + i] = 1 - s0[m - 1 - i] / 2;
        ws[m + i] = w0[m - 1 - i] / 2;
    }
    std::vector<RulePt> r;
    for (size_t i = 0; i < ts.size(); ++i)
        for (size_t j = 0; j < ss.size(); ++j) {
            double t = ts[i], s = ss[j];
            r.push_back({(1 - t) * (1 - s), (1 - t) * s, t, 2 * (1 - t) * wt[i] * ws[j]});
        }
    return r;
}

std::vector<RulePt> vertex_rule_base(int levels, double ratio, int order) {  // rules.jl:125-135
    std::vector<double> rs, wr, ss, ws;
    graded_gauss(levels, ratio, order, rs, wr);
    gauss_legendre(order + levels, ss, ws);
    std::vector<RulePt> r;
    for (size_t i = 0; i < rs.size(); ++i)
        for (size_t j = 0; j < ss.size(); ++j) {
            double rho = rs[i], s = ss[j];
            r.push_back({1 - rho, rho * (1 - s), rho * s, 2 * rho * wr[i] * ws[j]});
        }
    return r;
}

std::vector<RulePt> self_rule(const std::vector<RulePt>& base) {  // rules.jl:142-156
    std::vector<RulePt> r;
    for (int k = 0; k < 3; ++k)
        for (const RulePt& m : base) {
            double l[3] = {m.l2 / 3, m.l2 / 3, m.l2 / 3};
            l[k] += m.l0;
            l[(k + 1) % 3] += m.l1;
            r.push_back({l[0], l[1], l[2], m.w / 3});
        }
    return r;
}

// ------------------------------------------------------------------------------------------------------------------
// host: element data (src/elements/flat_triangle.jl:12-31, src/kernels/source_triangle.jl:8-26)

bool make_tri(const double* a, const double* b, const double* c, TriGeo& g) {
    double ab[3], ac[3], nA[3];
    for (int k = 0; k < 3; ++k) {
        ab[k] = b[k] - a[k];
        ac[k] = c[k] - a[k];
    }
    nA[0] = ab[1] * ac[2] - ab[2] * ac[1];
    nA[1] = ab[2] * ac[0] - ab[0] * ac[2];
    nA[2] = ab[0] * ac[1] - ab[1] * ac[0];
    double A2 = std::sqrt(nA[0] * nA[0] + nA[1] * nA[1] + nA[2] * nA[2]);
    if (!(A2 > 0)) return false;
    const double* v[3] = {a, b, c};
    for (int k = 0; k < 3; ++k) {
        g.x[3 * 0 + k] = a[k];
        g.x[3 * 1 + k] = b[k];
        g.x[3 * 2 + k] = c[k];
        g.n[k] = nA[k] / A2;
        g.c[k] = (a[k] + b[k] + c[k]) / 3;
    }
    g.area = A2 / 2;
    double e[3][3];
    for (int q = 0; q < 3; ++q) {
        const double *p0 = v[q], *p1 = v[(q + 1) % 3];
        for (int k = 0; k < 3; ++k) e[q][k] = p1[k] - p0[k];  // edge q: corner q -> q+1
        g.len[q] = std::sqrt(e[q][0] * e[q][0] + e[q][1] * e[q][1] + e[q][2] * e[q][2]);
        // nu_q = (edge_q x n) / len_q
        g.nu[3 * q + 0] = (e[q][1] * g.n[2] - e[q][2] * g.n[1]) / g.len[q];
        g.nu[3 * q + 1] = (e[q][2] * g.n[0] - e[q][0] * g.n[2]) / g.len[q];
        g.nu[3 * q + 2] = (e[q][0] * g.n[1] - e[q][1] * g.n[0]) / g.len[q];
    }
    g.diam = g.len[0];
    if (g.len[1] > g.diam) g.diam = g.len[1];
    if (g.len[2] > g.diam) g.diam = g.len[2];
    // gamma_b = -e_b / 2A with e_b the edge opposite corner b: (c-b, a-c, b-a) = edges 1, 2, 0
    const int opp[3] = {1, 2, 0};
    for (int bb = 0; bb < 3; ++bb)
        for (int k = 0; k < 3; ++k) g.gam[3 * bb + k] = -e[opp[bb]][k] / A2;
    double rch = 0;
    for (int q = 0; q < 3; ++q) {
        double d0 = v[q][0] - g.c[0], d1 = v[q][1] - g.c[1], d2 = v[q][2] - g.c[2];
        rch = std::max(rch, std::sqrt(d0 * d0 + d1 * d1 + d2 * d2));
    }
    g.reach = rch;
    g.sigma = 0;
    return true;
}

// ------------------------------------------------------------------------------------------------------------------
// device: far test of pair_rule (assemble.jl:269), FP32 with an exact FP64 fallback near the threshold

struct CentF {
    float hx, hy, hz, lx, ly, lz, diam, pad;
};

__device__ __forceinline__ bool far_exact64(const double* cT, double dT, const double* cS, double dS, double ratio) {
    // norm(S.c - T.c) > far_ratio * max(T.diam, S.diam), rounded as the reference (no contraction)
    double ex = __dsub_rn(cS[0], cT[0]), ey = __dsub_rn(cS[1], cT[1]), ez = __dsub_rn(cS[2], cT[2]);
    double n2 = __dadd_rn(__dadd_rn(__dmul_rn(ex, ex), __dmul_rn(ey, ey)), __dmul_rn(ez, ez));
    return __dsqrt_rn(n2) > __dmul_rn(ratio, fmax(dT, dS));
}

__device__ __forceinline__ int far_test32(const CentF& T, const CentF& S, float ratio) {
    // 1 far, 0 not far, -1 too close to the threshold to decide in FP32
    float dx = (S.hx - T.hx) + (S.lx - T.lx);
    float dy = (S.hy - T.hy) + (S.ly - T.ly);
    float dz = (S.hz - T.hz) + (S.lz - T.lz);
    float d2 = dx * dx + dy * dy + dz * dz;
    float th = ratio * fmaxf(T.diam, S.diam);
    float t2 = th * th;
    if (d2 > t2 * 1.00001f) return 1;
    if (d2 < t2 * 0.99999f) return 0;
    return -1;
}

// count (mode 0) or list (mode 1) the non-far sources of every test triangle, in source order
__global__ void classify_kernel(int mode, int ntest, const CentF* __restrict__ tc, const TriGeo* __restrict__ tgeo,
                                int nsrc, const CentF* __restrict__ sc, const TriGeo* __restrict__ sgeo, float ratio32,
                                double ratio, int* __restrict__ counts, const long long* __restrict__ offs,
                                int* __restrict__ list) {
    __shared__ int warp_tot[32];
    const int t = blockIdx.x;
    if (t >= ntest) return;
    const CentF T = tc[t];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    long long base = mode ? offs[t] : 0;
    int total = 0;
    for (int s0 = 0; s0 < nsrc; s0 += blockDim.x) {
        int s = s0 + threadIdx.x;
        bool nf = false;
        if (s < nsrc) {
            int f = far_test32(T, sc[s], ratio32);
            if (f < 0) f = far_exact64(tgeo[t].c, tgeo[t].diam, sgeo[s].c, sgeo[s].diam, ratio) ? 1 : 0;
            nf = (f == 0);
        }
        unsigned bal = __ballot_sync(0xffffffffu, nf);
        if (lane == 0) warp_tot[wid] = __popc(bal);
        __syncthreads();
        if (mode && nf) {
            int before = 0;
            for (int k = 0; k < wid; ++k) before += warp_tot[k];
            int pos = before + __popc(bal & ((1u << lane) - 1u));
            list[base + total + pos] = s;
        }
        int chunk = 0;
        for (int k = 0; k < nw; ++k) chunk += warp_tot[k];
        total += chunk;
        __syncthreads();
    }
    if (!mode && threadIdx.x == 0) counts[t] = total;
}

// ------------------------------------------------------------------------------------------------------------------
// device: the far tier

template <class T>
struct FarTest {  // a test triangle of the far kernel's tile
    T xh[NQMAX][3], xl[NQMAX][3];  // far rule points (hi + lo parts for float; lo = 0 for double)
    T wpsi[NQMAX][3];             // w_q A_T psi_a(lambda_q)
    T n[3];
    CentF cf;
    double c64[3];
    double diam64;
    int valid;
};

struct FarArgs {
    int ntest, nq, test_mode;
    const double* tq;      // test far points (ntest x NQMAX x 3)
    const double* tw;      // test weights (ntest x NQMAX x 3)
    const TriGeo* tgeo;    // test triangles
    const CentF* tcent;
    // sources: body then wake
    int nset;
    int nsrc[2], ntile[2], col_off[2];
    const void* soa[2];    // NFIELD x nsrc_pad (T)
    int pad[2];
    const CentF* scent[2];
    const TriGeo* sgeo[2];
    const int* tile_cols[2];   // ntile x 384 unique column slots
    const int* tile_ncol[2];
    const short* tile_cptr[2]; // ntile x 385 CSR over unique cols -> entries (src_local * 3 + b)
    const short* tile_cent[2]; // ntile x 384
    // test tiles: unique rows
    const int* trow;        // ntiles x 24
    const int* tnrow;
    const short* trptr;     // ntiles x 25
    const short* trent;     // ntiles x 24 (test_local * 3 + a)
    const int* tiles;       // test tiles of this launch
    double* A;
    long long lda;
    double* b;
    float ratio32;
    double ratio, kernel_far;
};

// ------------------------------------------------------------------------------------------------------------------
// device: the near, touching and contact tiers (assemble.jl:63-321), one warp per test triangle

enum { TIER_SELF = 0, TIER_EDGE = 1, TIER_VERTEX = 2, TIER_CONTACT = 3, TIER_NEAR = 4, TIER_FAR = 5 };
enum { R_NEAR = 0, R_SELF = 1, R_EDGE = 2, R_VERT = 3, R_FAR = 4 };

struct NearArgs {
    const TriGeo* tri;      // body triangles
    const TriGeo* wtri;     // wake triangles
    const double* wx;       // wake nodes (nwnode x 3)
    const int* fil;         // filaments (nfil x 2)
    int ntri, nwtri, nfil, nslot;
    const long long* nf_ptr;
    const int* nf_src;
    const long long* wf_ptr;
    const int* wf_src;
    int* rest_src;   // per test, at the offsets of nf_src: the body sources left to the warp-cooperative path
    int* wrest_src;  // the same for the wake sources
    int* rest_cnt;   // per test: counts of both (2 x ntri)
    const long long* rest_off;  // exclusive prefix sums of rest_cnt (2 x ntri + 1): a rest pair's place in the list
    double* pair_out;           // forward: per rest pair, its 3 x 3 block (row-major) and its 3 right hand side terms
    unsigned long long* next;   // work counter of the pair-parallel kernels
    const long long* touch;  // sorted keys t * ntri + s
    int ntouch;
    const RulePt* rule[5];
    const float4* rulef[5];  // the same rules in FP32 (l0, l1, l2, w)
    int nrule[5];
    double* A;
    long long lda;
    double* b;
    const int* tests;
    int ntests;
    int test_mode, near_depth, mixed;
    double far_ratio, near_ratio, corner_angle, contact_rel, kernel_far;
    float kernel_far32;  // kernel_far in FP32 (the FP32 point evaluators)
    double vinf[3];
    double tint[3];
    unsigned long long* stats;  // pairs[6], points[6], points evaluated in FP64
};

struct Bary9 {
    double v[9];  // three corners in the test triangle's barycentrics (corner j at v[3j..3j+2])
};

struct WarpSh {
    double E[27];          // E[9k+3a+z]: x_T,k - v_S,a (filament: x_T,k - a, x_T,k - b)
    double D[9];           // x_T,k - c_S
    double Sd[9], Sn[3], Snu[9], Slen[3], Sarea, Sdiam;
    float E32[27];         // E in FP32
    float D32[9];          // D in FP32
    float Sdf[9], Snf[3], Snuf[9], Slenf[3], Sareaf, Sdiamf;
    double leaf[LEAFBUF][10];
    float leaff[LEAFBUF][10];  // the leaves in FP32: corners, and frac x the test triangle's area
    int qi[64], ql[64];    // points waiting for FP64: rule point, and leaf (-1: the current piece)
};

__device__ __forceinline__ v3<double> ld3(const double* p) { return mk3(p[0], p[1], p[2]); }

__device__ __forceinline__ void seg_proj(v3<double> p, v3<double> a, v3<double> c, double& d, double& t) {
    v3<double> e = c - a;
    t = dot(p - a, e) / dot(e, e);
    t = fmin(fmax(t, 0.0), 1.0);
    d = vnorm(p - (a + t * e));
}

// distance_to (flat_triangle.jl:59-78)
__device__ double dist_tri(const double* X, v3<double> p) {
    v3<double> a = ld3(X), b = ld3(X + 3), c = ld3(X + 6);
    v3<double> ab = b - a, ac = c - a, ap = p - a;
    double d1 = dot(ab, ap), d2 = dot(ac, ap);
    if (d1 <= 0 && d2 <= 0) return vnorm(ap);
    v3<double> bp = p - b;
    double d3 = dot(ab, bp), d4 = dot(ac, bp);
    if (d3 >= 0 && d4 <= d3) return vnorm(bp);
    double vc = d1 * d4 - d3 * d2;
    if (vc <= 0 && d1 >= 0 && d3 <= 0) return vnorm(p - (a + (d1 / (d1 - d3)) * ab));
    v3<double> cp = p - c;
    double d5 = dot(ab, cp), d6 = dot(ac, cp);
    if (d6 >= 0 && d5 <= d6) return vnorm(cp);
    double vb = d5 * d2 - d1 * d6;
    if (vb <= 0 && d2 >= 0 && d6 <= 0) return vnorm(p - (a + (d2 / (d2 - d6)) * ac));
    double va = d3 * d6 - d5 * d4;
    if (va <= 0 && d4 - d3 >= 0 && d5 - d6 >= 0) return vnorm(p - (b + ((d4 - d3) / ((d4 - d3) + (d5 - d6))) * (c - b)));
    double denom = 1 / (va + vb + vc);
    return vnorm(p - (a + (vb * denom) * ab + (vc * denom) * ac));
}

// distance_to on corners a, b, c given as vectors (any frame, any precision)
template <class T>
__device__ T dist_tri_v(v3<T> a, v3<T> b, v3<T> c, v3<T> p) {
    v3<T> ab = b - a, ac = c - a, ap = p - a;
    T d1 = dot(ab, ap), d2 = dot(ac, ap);
    if (d1 <= T(0) && d2 <= T(0)) return vnorm(ap);
    v3<T> bp = p - b;
    T d3 = dot(ab, bp), d4 = dot(ac, bp);
    if (d3 >= T(0) && d4 <= d3) return vnorm(bp);
    T vc = d1 * d4 - d3 * d2;
    if (vc <= T(0) && d1 >= T(0) && d3 <= T(0)) return vnorm(p - (a + (d1 / (d1 - d3)) * ab));
    v3<T> cp = p - c;
    T d5 = dot(ab, cp), d6 = dot(ac, cp);
    if (d6 >= T(0) && d5 <= d6) return vnorm(cp);
    T vb = d5 * d2 - d1 * d6;
    if (vb <= T(0) && d2 >= T(0) && d6 <= T(0)) return vnorm(p - (a + (d2 / (d2 - d6)) * ac));
    T va = d3 * d6 - d5 * d4;
    if (va <= T(0) && d4 - d3 >= T(0) && d5 - d6 >= T(0))
        return vnorm(p - (b + ((d4 - d3) / ((d4 - d3) + (d5 - d6))) * (c - b)));
    T denom = T(1) / (va + vb + vc);
    return vnorm(p - (a + (vb * denom) * ab + (vc * denom) * ac));
}

// outcome of a comparison x < y decided in FP32 with absolute error bound e: 1 true, 0 false, -1 undecided
__device__ __forceinline__ int lt32(float x, float y, float e) { return x < y - e ? 1 : (x > y + e ? 0 : -1); }

struct SrcRef {  // a source for distance tests: a triangle (X) or a segment (a, b)
    int kind;    // 0 triangle, 1 segment
    const double* X;
    v3<double> a, b;
};

__device__ __forceinline__ double dist_src(const SrcRef& s, v3<double> p) {
    if (s.kind == 0) return dist_tri(s.X, p);
    double d, t;
    seg_proj(p, s.a, s.b, d, t);
    return d;
}

__device__ __forceinline__ v3<double> tpoint(const TriGeo& T, const double* b) {
    return mk3(b[0] * T.x[0] + b[1] * T.x[3] + b[2] * T.x[6], b[0] * T.x[1] + b[1] * T.x[4] + b[2] * T.x[7],
               b[0] * T.x[2] + b[1] * T.x[5] + b[2] * T.x[8]);
}

// per-lane accumulators of a pair (forward)
struct FwdAcc {
    v3<double> P[3];      // triangle source: sum of W psi_a w
    double ca[3], cb[3];  // filament source: the two end parts
    v3<float> Pf[3];      // FP32 partial sums, folded into P every few points
    int nf;               // points in Pf
};

struct PairCtx {
    const NearArgs* a;
    const TriGeo* T;
    WarpSh* sh;
    int lane;
    int kind;       // 0 triangle source, 1 filament
    int side;       // 1 for the self pair
    int fp32;       // evaluate in FP32 with the FP64 guard (VP_MIXED, triangle sources)
    int nleaf;      // buffered leaves (uniform)
    int nq64;       // queued FP64 points (uniform)
    long long npts; // points of this pair (uniform)
    long long n64;  // points of this pair evaluated in FP64 (uniform)
    // adjoint: the test function weights nu_a at T's corners (nadj adjoint vectors, nu = the first), the pair's
    // direction m, a filament's end values
    int nadj;
    double nu[3];
    double nuk[2][3];
    v3<double> m;
    v3<float> mf;
    double mua, mub;
    // adjoint, pieces whose corners move with the geometry (contact splits, wide-corner wedges): the current piece's
    // frac, the map of a point's barycentrics to the piece's own (binv), this lane's tangent of the piece's corners
    // (9) and frac (1) along direction `lane` (< 18: the test corners' 9 coordinates, then the source's), and this
    // lane's accumulated derivative along it; the test corners relative to the test centroid
    int dep;
    double pfrac;
    double binv[9];
    double tb[10];
    // FP32 copies, converted once (a conversion from FP64 runs on the FP64 pipe): nuk, and binv per piece
    float nukf[ADJ_MAX][3];
    float binvf[9];
    double gdir[2];
    v3<double> Xc[3];
    v3<float> Xcf[3];
};

__device__ __forceinline__ void fold32(FwdAcc& acc) {
    for (int k = 0; k < 3; ++k) {
        acc.P[k].x += double(acc.Pf[k].x);
        acc.P[k].y += double(acc.Pf[k].y);
        acc.P[k].z += double(acc.Pf[k].z);
        acc.Pf[k] = mk3(0.f, 0.f, 0.f);
    }
    acc.nf = 0;
}

// the split evaluation's fallback, out of line (rare): FP64 geometry with the FP32-based functions
__device__ __noinline__ v3<double> exact64_hyb(const SrcKern<double>& S, v3<double> ra, v3<double> rb, v3<double> rc,
                                               v3<double> r, int side) {
    return sv_exact3<double, KMathHyb>(S, ra, rb, rc, r, side, 1e-12);
}

// evaluate one point (barycentric l on T, weight W) in FP64
__device__ __noinline__ void eval_point64(const PairCtx& pc, FwdAcc& acc, double l0, double l1, double l2, double W) {
    const WarpSh& sh = *pc.sh;
    v3<double> psi = test_weights(pc.a->test_mode, l0, l1, l2);
    if (pc.kind == 0) {
        v3<double> ra = l0 * ld3(sh.E + 0) + l1 * ld3(sh.E + 9) + l2 * ld3(sh.E + 18);
        v3<double> rb = l0 * ld3(sh.E + 3) + l1 * ld3(sh.E + 12) + l2 * ld3(sh.E + 21);
        v3<double> rc = l0 * ld3(sh.E + 6) + l1 * ld3(sh.E + 15) + l2 * ld3(sh.E + 24);
        v3<double> r = l0 * ld3(sh.D) + l1 * ld3(sh.D + 3) + l2 * ld3(sh.D + 6);
        SrcKern<double> S;
        for (int k = 0; k < 3; ++k) {
            S.d[k] = ld3(sh.Sd + 3 * k);
            S.nu[k] = ld3(sh.Snu + 3 * k);
            S.len[k] = sh.Slen[k];
        }
        S.n = ld3(sh.Sn);
        S.area = sh.Sarea;
        S.diam = sh.Sdiam;
        double fd = pc.a->kernel_far * S.diam;
        // the mixed path's FP64 points (where FP32 cancels): what cancels in FP64, the functions on it in FP32
        // (sv_exact3_split), or FP64 geometry with FP32-based functions (KMathHyb) where the split leaves FP32's range
        v3<double> w;
        v3<float> wf;
        if (dot(r, r) > fd * fd)
            w = sv_far(S, r);
        else if (!pc.fp32)
            w = sv_exact3(S, ra, rb, rc, r, pc.side, 1e-12);
        else if (sv_exact3_split(S, ra, rb, rc, r, pc.side, 1e-12, wf))
            w = mk3(double(wf.x), double(wf.y), double(wf.z));
        else
            w = exact64_hyb(S, ra, rb, rc, r, pc.side);
        acc.P[0] += (W * psi.x) * w;
        acc.P[1] += (W * psi.y) * w;
        acc.P[2] += (W * psi.z) * w;
    } else {
        v3<double> ra = l0 * ld3(sh.E + 0) + l1 * ld3(sh.E + 9) + l2 * ld3(sh.E + 18);   // x - a
        v3<double> rb = l0 * ld3(sh.E + 3) + l1 * ld3(sh.E + 12) + l2 * ld3(sh.E + 21);  // x - b
        v3<double> va, vb;
        segment_velocity(ra, rb, va, vb);
        v3<double> n = ld3(pc.T->n);
        double da = dot(va, n) * W, db = dot(vb, n) * W;
        acc.ca[0] += da * psi.x;
        acc.ca[1] += da * psi.y;
        acc.ca[2] += da * psi.z;
        acc.cb[0] += db * psi.x;
        acc.cb[1] += db * psi.y;
        acc.cb[2] += db * psi.z;
    }
}

// evaluate one point in FP32 (triangle sources in VP_MIXED); false when it lies where FP32 cancels
__device__ __noinline__ bool eval_point32(const PairCtx& pc, FwdAcc& acc, float l0, float l1, float l2, float W) {
    if (pc.a->test_mode == 2) return false;  // the dual test's ties are decided in FP64
    const WarpSh& sh = *pc.sh;
    SrcKern<float> S;
    for (int k = 0; k < 3; ++k) {
        S.d[k] = mk3(sh.Sdf[3 * k], sh.Sdf[3 * k + 1], sh.Sdf[3 * k + 2]);
        S.nu[k] = mk3(sh.Snuf[3 * k], sh.Snuf[3 * k + 1], sh.Snuf[3 * k + 2]);
        S.len[k] = sh.Slenf[k];
    }
    S.n = mk3(sh.Snf[0], sh.Snf[1], sh.Snf[2]);
    S.area = sh.Sareaf;
    S.diam = sh.Sdiamf;
    v3<float> r = l0 * mk3(sh.D32[0], sh.D32[1], sh.D32[2]) + l1 * mk3(sh.D32[3], sh.D32[4], sh.D32[5]) +
                  l2 * mk3(sh.D32[6], sh.D32[7], sh.D32[8]);
    v3<float> w;
    float fd = pc.a->kernel_far32 * S.diam;
    if (dot(r, r) > fd * fd) {
        w = sv_far(S, r);
    } else {
        const float* E = sh.E32;
        v3<float> ra = l0 * mk3(E[0], E[1], E[2]) + l1 * mk3(E[9], E[10], E[11]) + l2 * mk3(E[18], E[19], E[20]);
        v3<float> rb = l0 * mk3(E[3], E[4], E[5]) + l1 * mk3(E[12], E[13], E[14]) + l2 * mk3(E[21], E[22], E[23]);
        v3<float> rc = l0 * mk3(E[6], E[7], E[8]) + l1 * mk3(E[15], E[16], E[17]) + l2 * mk3(E[24], E[25], E[26]);
        const Fp32Guard g{PAIR_GUARD};
        if (!sv_exact3_guarded(S, ra, rb, rc, pc.side, g, w)) return false;
    }
    v3<float> psi = pc.a->test_mode == 0 ? mk3(l0, l1, l2) : mk3(1.f, 1.f, 1.f);
    acc.Pf[0] += (W * psi.x) * w;
    acc.Pf[1] += (W * psi.y) * w;
    acc.Pf[2] += (W * psi.z) * w;
    if (++acc.nf == 16) fold32(acc);
    return true;
}

// ---- adjoint accumulation of a pair (warp-cooperative path) --------------------------------------------------------

struct AdjAcc {
    AdjSums<double> d[ADJ_MAX];  // FP64 sums, per adjoint vector
    AdjSums<float> f[ADJ_MAX];   // FP32 partial sums, folded into d every few points
    int nf;
    // the current dependent piece: sum W beta_j dphi/dl_k (Bb, 3 x 3) and sum W phi (Fb), phi = nu(l) s
    double Bb[ADJ_MAX][9], Fb[ADJ_MAX];
    float Bbf[ADJ_MAX][9], Fbf[ADJ_MAX];
};

template <class A, class B>
__device__ __forceinline__ void adj_add(AdjSums<A>& d, const AdjSums<B>& f) {
    auto c = [](v3<B> v) { return mk3(A(v.x), A(v.y), A(v.z)); };
    d.Q += c(f.Q);
    d.Grf += c(f.Grf);
    for (int k = 0; k < 3; ++k) {
        d.Xg[k] += c(f.Xg[k]);
        d.Gr[k] += c(f.Gr[k]);
        d.Gd[k] += c(f.Gd[k]);
        d.L[k] += A(f.L[k]);
        d.N[k] += A(f.N[k]);
    }
    d.O += A(f.O);
    d.A += A(f.A);
}

__device__ __forceinline__ void fold32(AdjAcc& acc) {
    for (int j = 0; j < ADJ_MAX; ++j) {
        adj_add(acc.d[j], acc.f[j]);
        adj_zero(acc.f[j]);
        for (int k = 0; k < 9; ++k) {
            acc.Bb[j][k] += double(acc.Bbf[j][k]);
            acc.Bbf[j][k] = 0.f;
        }
        acc.Fb[j] += double(acc.Fbf[j]);
        acc.Fbf[j] = 0.f;
    }
    acc.nf = 0;
}

// Mixed-precision adjoint sums of a pair, held by the warp. Each lane adds its points into FP32 partial sums in shared
// memory (AdjLane: both vectors' AdjSums, then the dependent piece's Bb and Fb); every ADJ_FOLD point batches the warp
// adds the 32 lanes' partials field by field, in lane order, into FP64 totals spread over the lanes (field z in lane
// z % 32, slot z / 32). The lanes keep no FP64 sums of their own, and the FP64 work per point is a few additions per
// fold instead of two per field and point.
constexpr int ADJ_NSUM = 41;                                      // fields of AdjSums
constexpr int ADJ_NFIELD = ADJ_MAX * ADJ_NSUM + ADJ_MAX * 10;     // sums, then Bb (9) per vector, then Fb per vector
constexpr int ADJ_BB0 = ADJ_MAX * ADJ_NSUM;                       // field of Bb[0][0]
constexpr int ADJ_FB0 = ADJ_BB0 + ADJ_MAX * 9;                    // field of Fb[0]
constexpr int ADJ_TSLOT = (ADJ_NFIELD + 31) / 32;
constexpr int ADJ_FOLD = 8;

struct AdjLane {
    AdjSums<float> f[ADJ_MAX];
    float Bbf[ADJ_MAX][9], Fbf[ADJ_MAX];
    float pad;  // an odd stride in words: the 32 lanes' copies of a field fall in 32 banks
};
static_assert(sizeof(AdjSums<float>) == ADJ_NSUM * sizeof(float), "AdjSums is a plain array of fields");
static_assert(sizeof(AdjLane) == (ADJ_NFIELD + 1) * sizeof(float), "AdjLane is a plain array of fields");
static_assert(sizeof(AdjSums<double>) == ADJ_NSUM * sizeof(double), "AdjSums is a plain array of fields");
constexpr int ADJ_LSTRIDE = ADJ_NFIELD + 1;

struct AdjAccW {
    AdjLane* lanes;            // the warp's 32 partials (shared memory)
    AdjLane* me;               // this lane's
    double tot[ADJ_TSLOT];     // the warp's FP64 totals of fields lane + 32 j
    int nb;                    // point batches since the last fold (warp-uniform)
};

// the warp's fold: lane z sums field z over the 32 lanes (two halves of 16, in lane order), adds it to its total and
// clears the partials it read. Called by the whole warp.
__device__ __noinline__ void fold_w(AdjAccW& acc, int lane) {
    __syncwarp();
    float* base = reinterpret_cast<float*>(acc.lanes);
#pragma unroll
    for (int j = 0; j < ADJ_TSLOT; ++j) {
        const int z = lane + 32 * j;
        if (z < ADJ_NFIELD) {
            float s0 = 0.f, s1 = 0.f;
            for (int l = 0; l < 16; ++l) {
                float* p0 = base + l * ADJ_LSTRIDE + z;
                float* p1 = base + (l + 16) * ADJ_LSTRIDE + z;
                s0 += *p0;
                s1 += *p1;
                *p0 = 0.f;
                *p1 = 0.f;
            }
            acc.tot[j] += double(s0) + double(s1);
        }
    }
    __syncwarp();
    acc.nb = 0;
}

// the fold of the dependent piece's fields only (Bb, Fb), at the end of a piece: the pair's sums stay in the partials
__device__ __noinline__ void fold_piece(AdjAccW& acc, int lane) {
    __syncwarp();
    float* base = reinterpret_cast<float*>(acc.lanes);
#pragma unroll
    for (int j = ADJ_BB0 / 32; j < ADJ_TSLOT; ++j) {
        const int z = lane + 32 * j;
        if (z >= ADJ_BB0 && z < ADJ_NFIELD) {
            float s0 = 0.f, s1 = 0.f;
            for (int l = 0; l < 16; ++l) {
                float* p0 = base + l * ADJ_LSTRIDE + z;
                float* p1 = base + (l + 16) * ADJ_LSTRIDE + z;
                s0 += *p0;
                s1 += *p1;
                *p0 = 0.f;
                *p1 = 0.f;
            }
            acc.tot[j] += double(s0) + double(s1);
        }
    }
    __syncwarp();
}

// the FP64 total of field z (a compile-time index after unrolling), in every lane
__device__ __forceinline__ double tot_field(const AdjAccW& acc, int z) {
    return __shfl_sync(0xffffffffu, acc.tot[z >> 5], z & 31);
}

// the rule-geometry sums of one point of a dependent piece: weight W, barycentrics l, value s = w·m, ds/dx
template <class T>
__device__ __forceinline__ void rule_point(const PairCtx& pc, const T* nu, const T* binv, T* Bb, T& Fb, T W, T l0, T l1,
                                           T l2, T sv, v3<T> gx, const v3<T>* Xc) {
    const T n0 = nu[0], n1 = nu[1], n2 = nu[2];
    const bool hat = pc.a->test_mode == 0;
    const T nul = hat ? n0 * l0 + n1 * l1 + n2 * l2 : (pc.a->test_mode == 1 ? n0 + n1 + n2 : T(0));
    T dphi[3];
    dphi[0] = (hat ? n0 * sv : T(0)) + nul * dot(gx, Xc[0]);
    dphi[1] = (hat ? n1 * sv : T(0)) + nul * dot(gx, Xc[1]);
    dphi[2] = (hat ? n2 * sv : T(0)) + nul * dot(gx, Xc[2]);
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        const T bj = W * (binv[3 * j] * l0 + binv[3 * j + 1] * l1 + binv[3 * j + 2] * l2);
        Bb[3 * j] += bj * dphi[0];
        Bb[3 * j + 1] += bj * dphi[1];
        Bb[3 * j + 2] += bj * dphi[2];
    }
    Fb += W * nul * sv;
}

__device__ __forceinline__ SrcKern<double> src64(const WarpSh& sh) {
    SrcKern<double> S;
    for (int k = 0; k < 3; ++k) {
        S.d[k] = ld3(sh.Sd + 3 * k);
        S.nu[k] = ld3(sh.Snu + 3 * k);
        S.len[k] = sh.Slen[k];
    }
    S.n = ld3(sh.Sn);
    S.area = sh.Sarea;
    S.diam = sh.Sdiam;
    return S;
}

__device__ __forceinline__ SrcKern<float> src32(const WarpSh& sh) {
    SrcKern<float> S;
    for (int k = 0; k < 3; ++k) {
        S.d[k] = mk3(sh.Sdf[3 * k], sh.Sdf[3 * k + 1], sh.Sdf[3 * k + 2]);
        S.nu[k] = mk3(sh.Snuf[3 * k], sh.Snuf[3 * k + 1], sh.Snuf[3 * k + 2]);
        S.len[k] = sh.Slenf[k];
    }
    S.n = mk3(sh.Snf[0], sh.Snf[1], sh.Snf[2]);
    S.area = sh.Sareaf;
    S.diam = sh.Sdiamf;
    return S;
}

// one point in FP64, adjoint: W nu(q) times s = w·m and its derivatives (source sheets), or the filament's
__device__ __noinline__ void eval_point64(const PairCtx& pc, AdjAcc& acc, double l0, double l1, double l2, double W) {
    const WarpSh& sh = *pc.sh;
    v3<double> psi = test_weights(pc.a->test_mode, l0, l1, l2);
    double Wn[ADJ_MAX];
    for (int k = 0; k < ADJ_MAX; ++k) Wn[k] = W * (pc.nuk[k][0] * psi.x + pc.nuk[k][1] * psi.y + pc.nuk[k][2] * psi.z);
    v3<double> ra = l0 * ld3(sh.E + 0) + l1 * ld3(sh.E + 9) + l2 * ld3(sh.E + 18);
    v3<double> rb = l0 * ld3(sh.E + 3) + l1 * ld3(sh.E + 12) + l2 * ld3(sh.E + 21);
    v3<double> gx;
    double sv;
    if (pc.kind == 0) {
        v3<double> rc = l0 * ld3(sh.E + 6) + l1 * ld3(sh.E + 15) + l2 * ld3(sh.E + 24);
        v3<double> r = l0 * ld3(sh.D) + l1 * ld3(sh.D + 3) + l2 * ld3(sh.D + 6);
        SrcKern<double> S = src64(sh);
        double fd = pc.a->kernel_far * S.diam;
        if (dot(r, r) > fd * fd)
            sv = adj_point_far_multi(acc.d, pc.nadj, Wn, S, l0, l1, l2, r, pc.m, gx);
        else if (pc.fp32)  // the mixed path's FP64 points: FP64 geometry and derivatives, FP32-based functions
            sv = adj_point_exact_multi<double, KMathHyb>(acc.d, pc.nadj, Wn, S, l0, l1, l2, ra, rb, rc, r, pc.m,
                                                         pc.side, 1e-12, gx);
        else
            sv = adj_point_exact_multi(acc.d, pc.nadj, Wn, S, l0, l1, l2, ra, rb, rc, r, pc.m, pc.side, 1e-12, gx);
    } else {
        v3<double> n = ld3(pc.T->n), va, vb, ga, gb;
        segment_velocity(ra, rb, va, vb);
        seg_vjp(ra, rb, n, pc.mua, pc.mub, ga, gb);
        gx = ga + gb;
        sv = pc.mua * dot(va, n) + pc.mub * dot(vb, n);
        for (int k = 0; k < pc.nadj; ++k) {
            AdjSums<double>& d = acc.d[k];
            d.Q += Wn[k] * (pc.mua * va + pc.mub * vb);
            d.Xg[0] += (Wn[k] * l0) * gx;
            d.Xg[1] += (Wn[k] * l1) * gx;
            d.Xg[2] += (Wn[k] * l2) * gx;
            d.Gr[0] += Wn[k] * ga;
            d.Gr[1] += Wn[k] * gb;
        }
    }
    if (pc.dep)
        for (int k = 0; k < pc.nadj; ++k)
            rule_point(pc, pc.nuk[k], pc.binv, acc.Bb[k], acc.Fb[k], W, l0, l1, l2, sv, gx, pc.Xc);
}

// one point in FP32 under the guard, adjoint; false when it must be evaluated in FP64
__device__ __noinline__ bool eval_point32(const PairCtx& pc, AdjAcc& acc, float l0, float l1, float l2, float W) {
    if (pc.a->test_mode == 2) return false;
    const WarpSh& sh = *pc.sh;
    SrcKern<float> S = src32(sh);
    v3<float> r = l0 * mk3(sh.D32[0], sh.D32[1], sh.D32[2]) + l1 * mk3(sh.D32[3], sh.D32[4], sh.D32[5]) +
                  l2 * mk3(sh.D32[6], sh.D32[7], sh.D32[8]);
    v3<float> psi = pc.a->test_mode == 0 ? mk3(l0, l1, l2) : mk3(1.f, 1.f, 1.f);
    float Wn[ADJ_MAX];
    for (int k = 0; k < ADJ_MAX; ++k)
        Wn[k] = W * (pc.nukf[k][0] * psi.x + pc.nukf[k][1] * psi.y + pc.nukf[k][2] * psi.z);
    float fd = pc.a->kernel_far32 * S.diam;
    v3<float> gx;
    float sv;
    if (dot(r, r) > fd * fd) {
        sv = adj_point_far_multi(acc.f, pc.nadj, Wn, S, l0, l1, l2, r, pc.mf, gx);
    } else {
        const float* E = sh.E32;
        v3<float> ra = l0 * mk3(E[0], E[1], E[2]) + l1 * mk3(E[9], E[10], E[11]) + l2 * mk3(E[18], E[19], E[20]);
        v3<float> rb = l0 * mk3(E[3], E[4], E[5]) + l1 * mk3(E[12], E[13], E[14]) + l2 * mk3(E[21], E[22], E[23]);
        v3<float> rc = l0 * mk3(E[6], E[7], E[8]) + l1 * mk3(E[15], E[16], E[17]) + l2 * mk3(E[24], E[25], E[26]);
        if (!fp32_guard_ok(S, ra, rb, rc, pc.side, Fp32Guard{ADJ_GUARD})) return false;
        // the self pair's points lie in the source's plane up to FP32 rounding: its in-plane branch (solid angle
        // side 2 pi, as the forward's FP32 kernel takes it) must not depend on the sign of that rounding
        sv = adj_point_exact_multi(acc.f, pc.nadj, Wn, S, l0, l1, l2, ra, rb, rc, r, pc.mf, pc.side,
                                   pc.side ? 1e-4f : 1e-12f, gx);
    }
    if (pc.dep)
        for (int k = 0; k < pc.nadj; ++k)
            rule_point(pc, pc.nukf[k], pc.binvf, acc.Bbf[k], acc.Fbf[k], W, l0, l1, l2, sv, gx, pc.Xcf);
    if (++acc.nf == 16) fold32(acc);
    return true;
}


// the exact kernel and its derivatives wholly in FP64 geometry (KMathHyb), added to this lane's FP32 partials: the
// split evaluation's fallback, kept out of line so that the common path's code stays small
__device__ __noinline__ double exact_vjp64_acc(const PairCtx& pc, AdjAccW& acc, const SrcKern<double>& S,
                                               v3<double> ra, v3<double> rb, v3<double> rc, v3<double> r,
                                               const float* Wn, float fl0, float fl1, float fl2, v3<double>& gx) {
    v3<double> h0, h1, h2;
    ExactShape<double> shd;
    const double sv = sv_exact_vjp<double, KMathHyb>(S, ra, rb, rc, r, pc.m, pc.side, 1e-12, h0, h1, h2, shd);
    const double i4pi = 1.0 / (4.0 * vp_pi<double>());
    const v3<double> w = (shd.L[0] * S.nu[0] + shd.L[1] * S.nu[1] + shd.L[2] * S.nu[2] + shd.Om * S.n) * i4pi;
    gx = h0 + h1 + h2;
    const float Lf[3] = {float(shd.L[0]), float(shd.L[1]), float(shd.L[2])};
    const float dLf[3] = {float(shd.dLdlen[0]), float(shd.dLdlen[1]), float(shd.dLdlen[2])};
    adj_acc_exact(acc.me->f, pc.nadj, Wn, fl0, fl1, fl2, f3(w), f3(gx), f3(h0), f3(h1), f3(h2), Lf, dLf,
                  float(shd.Om));
    return sv;
}

// the mixed path's FP64 point (a triangle source's point the FP32 guard refused), warp sums: the kernel and its
// derivatives in FP64 geometry with the FP32-based functions, added to this lane's FP32 partials
__device__ __noinline__ void eval_point64(const PairCtx& pc, AdjAccW& acc, double l0, double l1, double l2, double W) {
    const WarpSh& sh = *pc.sh;
    const v3<double> psi = test_weights(pc.a->test_mode, l0, l1, l2);
    float Wn[ADJ_MAX];
    for (int k = 0; k < ADJ_MAX; ++k)
        Wn[k] = float(W * (pc.nuk[k][0] * psi.x + pc.nuk[k][1] * psi.y + pc.nuk[k][2] * psi.z));
    const v3<double> ra = l0 * ld3(sh.E + 0) + l1 * ld3(sh.E + 9) + l2 * ld3(sh.E + 18);
    const v3<double> rb = l0 * ld3(sh.E + 3) + l1 * ld3(sh.E + 12) + l2 * ld3(sh.E + 21);
    const v3<double> rc = l0 * ld3(sh.E + 6) + l1 * ld3(sh.E + 15) + l2 * ld3(sh.E + 24);
    const v3<double> r = l0 * ld3(sh.D) + l1 * ld3(sh.D + 3) + l2 * ld3(sh.D + 6);
    const SrcKern<double> S = src64(sh);
    const float fl0 = float(l0), fl1 = float(l1), fl2 = float(l2);
    const double fd = pc.a->kernel_far * S.diam;
    v3<double> gx;
    double sv;
    if (dot(r, r) > fd * fd) {
        v3<double> gd[3];
        double ga;
        sv = sv_far_vjp(S, r, pc.m, gx, gd, ga);
        const v3<float> gdf[3] = {f3(gd[0]), f3(gd[1]), f3(gd[2])};
        adj_acc_far(acc.me->f, pc.nadj, Wn, fl0, fl1, fl2, f3(sv_far(S, r)), f3(gx), gdf, float(ga));
    } else {
        v3<float> g0, g1, g2;
        ExactShape<float> shp;
        float svf;
        if (sv_exact_vjp_split(S, ra, rb, rc, r, pc.mf, pc.side, 1e-12, svf, g0, g1, g2, shp)) {
            const float i4pi = 1.f / (4.f * vp_pi<float>());
            const v3<float> w =
                (shp.L[0] * f3(S.nu[0]) + shp.L[1] * f3(S.nu[1]) + shp.L[2] * f3(S.nu[2]) + shp.Om * f3(S.n)) * i4pi;
            const v3<float> gxf = g0 + g1 + g2;
            adj_acc_exact(acc.me->f, pc.nadj, Wn, fl0, fl1, fl2, w, gxf, g0, g1, g2, shp.L, shp.dLdlen, shp.Om);
            if (pc.dep)
                for (int k = 0; k < pc.nadj; ++k)
                    rule_point(pc, pc.nukf[k], pc.binvf, acc.me->Bbf[k], acc.me->Fbf[k], float(W), fl0, fl1, fl2,
                               svf, gxf, pc.Xcf);
            return;
        }
        // offsets outside FP32's range: all in FP64, out of line (rare)
        sv = exact_vjp64_acc(pc, acc, S, ra, rb, rc, r, Wn, fl0, fl1, fl2, gx);
    }
    if (pc.dep)
        for (int k = 0; k < pc.nadj; ++k)
            rule_point(pc, pc.nukf[k], pc.binvf, acc.me->Bbf[k], acc.me->Fbf[k], float(W), fl0, fl1, fl2, float(sv),
                       f3(gx), pc.Xcf);
}

// one point in FP32 under the guard, warp sums; false when it must be evaluated in FP64
__device__ __noinline__ bool eval_point32(const PairCtx& pc, AdjAccW& acc, float l0, float l1, float l2, float W) {
    if (pc.a->test_mode == 2) return false;
    const WarpSh& sh = *pc.sh;
    SrcKern<float> S = src32(sh);
    v3<float> r = l0 * mk3(sh.D32[0], sh.D32[1], sh.D32[2]) + l1 * mk3(sh.D32[3], sh.D32[4], sh.D32[5]) +
                  l2 * mk3(sh.D32[6], sh.D32[7], sh.D32[8]);
    v3<float> psi = pc.a->test_mode == 0 ? mk3(l0, l1, l2) : mk3(1.f, 1.f, 1.f);
    float Wn[ADJ_MAX];
    for (int k = 0; k < ADJ_MAX; ++k)
        Wn[k] = W * (pc.nukf[k][0] * psi.x + pc.nukf[k][1] * psi.y + pc.nukf[k][2] * psi.z);
    float fd = pc.a->kernel_far32 * S.diam;
    v3<float> gx;
    float sv;
    if (dot(r, r) > fd * fd) {
        sv = adj_point_far_multi(acc.me->f, pc.nadj, Wn, S, l0, l1, l2, r, pc.mf, gx);
    } else {
        const float* E = sh.E32;
        v3<float> ra = l0 * mk3(E[0], E[1], E[2]) + l1 * mk3(E[9], E[10], E[11]) + l2 * mk3(E[18], E[19], E[20]);
        v3<float> rb = l0 * mk3(E[3], E[4], E[5]) + l1 * mk3(E[12], E[13], E[14]) + l2 * mk3(E[21], E[22], E[23]);
        v3<float> rc = l0 * mk3(E[6], E[7], E[8]) + l1 * mk3(E[15], E[16], E[17]) + l2 * mk3(E[24], E[25], E[26]);
        if (!fp32_guard_ok(S, ra, rb, rc, pc.side, Fp32Guard{ADJ_GUARD})) return false;
        sv = adj_point_exact_multi(acc.me->f, pc.nadj, Wn, S, l0, l1, l2, ra, rb, rc, r, pc.mf, pc.side,
                                   pc.side ? 1e-4f : 1e-12f, gx);
    }
    if (pc.dep)
        for (int k = 0; k < pc.nadj; ++k)
            rule_point(pc, pc.nukf[k], pc.binvf, acc.me->Bbf[k], acc.me->Fbf[k], W, l0, l1, l2, sv, gx, pc.Xcf);
    return true;
}

// the warp's fold after a batch of points (one per lane), every ADJ_FOLD batches; nothing for the other accumulators
template <class Acc>
__device__ __forceinline__ void batch_done(PairCtx& pc, Acc& acc) {
    if constexpr (std::is_same<Acc, AdjAccW>::value) {
        if (++acc.nb == ADJ_FOLD) fold_w(acc, pc.lane);
    }
}

__device__ __forceinline__ double wsum_d(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ v3<double> wsum3(v3<double> v) { return mk3(wsum_d(v.x), wsum_d(v.y), wsum_d(v.z)); }

__device__ void adj_warp_sum(AdjSums<double>& a) {
    a.Q = wsum3(a.Q);
    a.Grf = wsum3(a.Grf);
    for (int k = 0; k < 3; ++k) {
        a.Xg[k] = wsum3(a.Xg[k]);
        a.Gr[k] = wsum3(a.Gr[k]);
        a.Gd[k] = wsum3(a.Gd[k]);
        a.L[k] = wsum_d(a.L[k]);
        a.N[k] = wsum_d(a.N[k]);
    }
    a.O = wsum_d(a.O);
    a.A = wsum_d(a.A);
}

__device__ __forceinline__ void tri_corners(const TriGeo& g, v3<double>* v) {
    for (int k = 0; k < 3; ++k) v[k] = ld3(g.x + 3 * k);
}

// FP64 evaluation of the queued points, 32 at a time (all of them when `all`): rule point qi of the current piece
// (corners b, fraction frac) or of buffered leaf ql
template <class Acc>
__device__ __noinline__ void drain64(PairCtx& pc, Acc& acc, bool all, int rid, const double* b, double frac) {
    const RulePt* R = pc.a->rule[rid];
    const double areaT = pc.T->area;
    while (pc.nq64 >= 32 || (all && pc.nq64 > 0)) {
        __syncwarp();
        int take = pc.nq64 < 32 ? pc.nq64 : 32;
        if (pc.lane < take) {
            int i = pc.sh->qi[pc.lane], lf = pc.sh->ql[pc.lane];
            const double* c = lf < 0 ? b : pc.sh->leaf[lf];
            double fr = lf < 0 ? frac : pc.sh->leaf[lf][9];
            RulePt m = R[i];
            double l0 = m.l0 * c[0] + m.l1 * c[3] + m.l2 * c[6];
            double l1 = m.l0 * c[1] + m.l1 * c[4] + m.l2 * c[7];
            double l2 = m.l0 * c[2] + m.l1 * c[5] + m.l2 * c[8];
            eval_point64(pc, acc, l0, l1, l2, (m.w * fr) * areaT);
        }
        batch_done(pc, acc);
        __syncwarp();
        int rest = pc.nq64 - take;
        int mi = 0, ml = 0;
        if (pc.lane < rest) {
            mi = pc.sh->qi[take + pc.lane];
            ml = pc.sh->ql[take + pc.lane];
        }
        __syncwarp();
        if (pc.lane < rest) {
            pc.sh->qi[pc.lane] = mi;
            pc.sh->ql[pc.lane] = ml;
        }
        __syncwarp();
        pc.nq64 = rest;
        pc.n64 += take;
    }
}

// one point per lane (all lanes call this together). FP64: evaluated at once from the FP64 barycentrics. FP32: the
// FP32 barycentrics are evaluated under the guard; guarded points are queued (rule point i, leaf lf) for drain64.
template <class Acc>
__device__ __forceinline__ void point_step(PairCtx& pc, Acc& acc, bool valid, int rid, int i, int lf, const double* b,
                                           const float* bf, double frac) {
    if (!std::is_same<Acc, AdjAccW>::value && !pc.fp32) {
        if (valid) {
            RulePt m = pc.a->rule[rid][i];
            double l0 = m.l0 * b[0] + m.l1 * b[3] + m.l2 * b[6];
            double l1 = m.l0 * b[1] + m.l1 * b[4] + m.l2 * b[7];
            double l2 = m.l0 * b[2] + m.l1 * b[5] + m.l2 * b[8];
            eval_point64(pc, acc, l0, l1, l2, (m.w * frac) * pc.T->area);
        }
        return;
    }
    bool need = false;
    if (valid) {
        float4 m = pc.a->rulef[rid][i];
        float l0 = m.x * bf[0] + m.y * bf[3] + m.z * bf[6];
        float l1 = m.x * bf[1] + m.y * bf[4] + m.z * bf[7];
        float l2 = m.x * bf[2] + m.y * bf[5] + m.z * bf[8];
        need = !eval_point32(pc, acc, l0, l1, l2, m.w * bf[9]);
    }
    unsigned msk = __ballot_sync(0xffffffffu, need);
    if (msk) {
        int pos = pc.nq64 + __popc(msk & ((1u << pc.lane) - 1u));
        if (need) {
            pc.sh->qi[pos] = i;
            pc.sh->ql[pos] = lf;
        }
        pc.nq64 += __popc(msk);
    }
    batch_done(pc, acc);
}

// a piece carrying a whole tabulated rule: lanes stride over its points
template <class Acc>
__device__ __noinline__ void emit_rule(PairCtx& pc, Acc& acc, int rid, const double* b, double frac) {
    const int n = pc.a->nrule[rid];
    float bf[10];
    for (int z = 0; z < 9; ++z) bf[z] = float(b[z]);
    bf[9] = float(frac * pc.T->area);
    for (int i0 = 0; i0 < n; i0 += 32) {
        int i = i0 + pc.lane;
        point_step(pc, acc, i < n, rid, i < n ? i : 0, -1, b, bf, frac);
        if (pc.nq64 >= 32) drain64(pc, acc, false, rid, b, frac);
    }
    drain64(pc, acc, true, rid, b, frac);
    pc.npts += n;
    if (!pc.fp32) pc.n64 += n;
}

template <class Acc>
__device__ __noinline__ void flush_leaves(PairCtx& pc, Acc& acc) {
    const int nl = pc.nleaf;
    if (nl == 0) return;
    __syncwarp();
    const int n = pc.a->nrule[R_NEAR];
    for (int i0 = 0; i0 < nl * n; i0 += 32) {
        int i = i0 + pc.lane;
        bool valid = i < nl * n;
        int lf = valid ? i / n : 0, q = valid ? i - lf * n : 0;
        const double* b = pc.sh->leaf[lf];
        point_step(pc, acc, valid, R_NEAR, q, lf, b, pc.sh->leaff[lf], b[9]);
        if (pc.nq64 >= 32) drain64(pc, acc, false, R_NEAR, nullptr, 0.0);
    }
    drain64(pc, acc, true, R_NEAR, nullptr, 0.0);
    pc.npts += (long long)nl * n;
    if (!pc.fp32) pc.n64 += (long long)nl * n;
    __syncwarp();
    pc.nleaf = 0;
}

template <class Acc>
__device__ void emit_leaf(PairCtx& pc, Acc& acc, const double* b, double frac) {
    if (pc.lane == 0) {
        for (int k = 0; k < 9; ++k) {
            pc.sh->leaf[pc.nleaf][k] = b[k];
            pc.sh->leaff[pc.nleaf][k] = float(b[k]);
        }
        pc.sh->leaf[pc.nleaf][9] = frac;
        pc.sh->leaff[pc.nleaf][9] = float(frac * pc.T->area);
    }
    pc.nleaf++;
    if (pc.nleaf == LEAFBUF) flush_leaves(pc, acc);
}

// ---- adjoint: pieces whose corners move with the geometry ---------------------------------------------------------
// The contact splits and the wide-corner wedges place their pieces from the pair's geometry, so the points' positions
// in the test triangle and the pieces' weights move with it. Each lane carries the tangent of the current piece along
// one geometry coordinate (lane < 18); the points of a dependent piece sum sum W beta_j dphi/dl and sum W phi
// (rule_point), and piece_end contracts those with the lanes' tangents.
template <class Acc>
constexpr bool kAdj = std::is_same<Acc, AdjAcc>::value || std::is_same<Acc, AdjAccW>::value;

__device__ __forceinline__ void piece_begin(PairCtx&, FwdAcc&, const double*, double, const double*) {}
__device__ __forceinline__ void piece_end(PairCtx&, FwdAcc&) {}

// c: the piece's corners (9, test barycentrics), frac, tan: this lane's tangent (10) or null for a fixed piece
__device__ void piece_begin(PairCtx& pc, AdjAcc& acc, const double* c, double frac, const double* tan) {
    if (pc.nleaf) flush_leaves(pc, acc);
    if (!tan) {
        pc.dep = 0;
        return;
    }
    pc.dep = 1;
    pc.pfrac = frac;
    for (int k = 0; k < 10; ++k) pc.tb[k] = tan[k];
    // binv = M^-1, M[k][j] = c[3j + k]: l = M beta
    const double a = c[0], b = c[3], cc = c[6], d = c[1], e = c[4], f = c[7], g = c[2], h = c[5], i = c[8];
    const double A = e * i - f * h, B = -(d * i - f * g), C = d * h - e * g;
    const double id = 1.0 / (a * A + b * B + cc * C);
    pc.binv[0] = A * id;
    pc.binv[1] = -(b * i - cc * h) * id;
    pc.binv[2] = (b * f - cc * e) * id;
    pc.binv[3] = B * id;
    pc.binv[4] = (a * i - cc * g) * id;
    pc.binv[5] = -(a * f - cc * d) * id;
    pc.binv[6] = C * id;
    pc.binv[7] = -(a * h - b * g) * id;
    pc.binv[8] = (a * e - b * d) * id;
    for (int k = 0; k < 9; ++k) pc.binvf[k] = float(pc.binv[k]);
}

__device__ void piece_end(PairCtx& pc, AdjAcc& acc) {
    if (!pc.dep) return;
    if (pc.nleaf) flush_leaves(pc, acc);
    fold32(acc);
    for (int j = 0; j < pc.nadj; ++j) {
        double v = 0;
        for (int k = 0; k < 9; ++k) {
            v += wsum_d(acc.Bb[j][k]) * pc.tb[k];
            acc.Bb[j][k] = 0;
        }
        v += wsum_d(acc.Fb[j]) * pc.tb[9] / pc.pfrac;
        acc.Fb[j] = 0;
        if (pc.lane < 18) pc.gdir[j] += v;
    }
    pc.dep = 0;
}

__device__ void piece_begin(PairCtx& pc, AdjAccW& acc, const double* c, double frac, const double* tan) {
    if (pc.nleaf) flush_leaves(pc, acc);
    if (!tan) {
        pc.dep = 0;
        return;
    }
    pc.dep = 1;
    pc.pfrac = frac;
    for (int k = 0; k < 10; ++k) pc.tb[k] = tan[k];
    const double a = c[0], b = c[3], cc = c[6], d = c[1], e = c[4], f = c[7], g = c[2], h = c[5], i = c[8];
    const double A = e * i - f * h, B = -(d * i - f * g), C = d * h - e * g;
    const double id = 1.0 / (a * A + b * B + cc * C);
    const double bi[9] = {A * id, -(b * i - cc * h) * id, (b * f - cc * e) * id, B * id, (a * i - cc * g) * id,
                          -(a * f - cc * d) * id, C * id, -(a * h - b * g) * id, (a * e - b * d) * id};
    for (int k = 0; k < 9; ++k) {
        pc.binv[k] = bi[k];
        pc.binvf[k] = float(bi[k]);
    }
}

// the piece's rule-geometry totals (folded first) contracted with this lane's tangent; the totals are then cleared
__device__ void piece_end(PairCtx& pc, AdjAccW& acc) {
    if (!pc.dep) return;
    if (pc.nleaf) flush_leaves(pc, acc);
    fold_piece(acc, pc.lane);
#pragma unroll
    for (int j = 0; j < ADJ_MAX; ++j) {
        if (j >= pc.nadj) break;
        double v = 0;
#pragma unroll
        for (int k = 0; k < 9; ++k) v += tot_field(acc, ADJ_BB0 + 9 * j + k) * pc.tb[k];
        v += tot_field(acc, ADJ_FB0 + j) * pc.tb[9] / pc.pfrac;
        if (pc.lane < 18) pc.gdir[j] += v;
    }
#pragma unroll
    for (int j = 0; j < ADJ_TSLOT; ++j) {
        const int z = pc.lane + 32 * j;
        if (z >= ADJ_BB0 && z < ADJ_NFIELD) acc.tot[j] = 0;
    }
    pc.dep = 0;
}

// the warp's FP64 sums of the pair's d[j], j < nadj, in every lane (after the last fold)
__device__ void pair_totals(const AdjAccW& acc, AdjSums<double>* d, int nadj) {
    double* o = reinterpret_cast<double*>(d);
#pragma unroll
    for (int z = 0; z < ADJ_BB0; ++z) o[z] = z < nadj * ADJ_NSUM ? tot_field(acc, z) : 0.0;
}

// this lane's tangent of the point with test barycentrics b (3) whose tangent is bt (3)
__device__ __forceinline__ v3<double> tan_point(const PairCtx& pc, const double* b, const double* bt) {
    v3<double> r = bt[0] * pc.Xc[0] + bt[1] * pc.Xc[1] + bt[2] * pc.Xc[2];
    if (pc.lane < 9) {
        const double s = b[pc.lane / 3];
        const int c = pc.lane % 3;
        r.x += c == 0 ? s : 0.0;
        r.y += c == 1 ? s : 0.0;
        r.z += c == 2 ? s : 0.0;
    }
    return r;
}

// this lane's tangent of source corner q
__device__ __forceinline__ v3<double> tan_source(const PairCtx& pc, int q) {
    const int d = pc.lane - 9;
    const bool on = d >= 0 && d < 9 && d / 3 == q;
    return mk3(on && d % 3 == 0 ? 1.0 : 0.0, on && d % 3 == 1 ? 1.0 : 0.0, on && d % 3 == 2 ? 1.0 : 0.0);
}

// corners (k, k+1, k+2) of piece b (and of its tangent)
__device__ __forceinline__ void rotate_corners(const double* b, int k, double* c) {
    for (int z = 0; z < 3; ++z) {
        c[z] = b[3 * k + z];
        c[3 + z] = b[3 * ((k + 1) % 3) + z];
        c[6 + z] = b[3 * ((k + 2) % 3) + z];
    }
}

__device__ __forceinline__ void bmix(double* o, const double* a, double sa, const double* b, double sb) {
    o[0] = sa * a[0] + sb * b[0];
    o[1] = sa * a[1] + sb * b[1];
    o[2] = sa * a[2] + sb * b[2];
}

// near_pieces! (assemble.jl:131-142) as a depth-first walk of the quadtree of sub-triangles
template <class Acc>
__device__ __noinline__ void near_pieces(PairCtx& pc, Acc& acc, const SrcRef& src, const double* b0, double frac0, int depth) {
    int level = 0;
    unsigned path = 0;  // base-4 digits, most significant first
    const double ratio = pc.a->near_ratio;
    for (int guard = 0; guard < (1 << 22); ++guard) {
        double b[9];
        for (int k = 0; k < 9; ++k) b[k] = b0[k];
        for (int l = 0; l < level; ++l) {
            int digit = (path >> (2 * (level - 1 - l))) & 3;
            double m12[3], m23[3], m31[3], nb[9];
            bmix(m12, b, 0.5, b + 3, 0.5);
            bmix(m23, b + 3, 0.5, b + 6, 0.5);
            bmix(m31, b + 6, 0.5, b, 0.5);
            const double *c0, *c1, *c2;  // quarters (assemble.jl:79-82)
            if (digit == 0) { c0 = b; c1 = m12; c2 = m31; }
            else if (digit == 1) { c0 = m12; c1 = b + 3; c2 = m23; }
            else if (digit == 2) { c0 = m31; c1 = m23; c2 = b + 6; }
            else { c0 = m12; c1 = m23; c2 = m31; }
            for (int k = 0; k < 3; ++k) {
                nb[k] = c0[k];
                nb[3 + k] = c1[k];
                nb[6 + k] = c2[k];
            }
            for (int k = 0; k < 9; ++k) b[k] = nb[k];
        }
        v3<double> p1 = tpoint(*pc.T, b), p2 = tpoint(*pc.T, b + 3), p3 = tpoint(*pc.T, b + 6);
        double size = fmax(vnorm(p2 - p1), fmax(vnorm(p3 - p2), vnorm(p1 - p3)));
        if (level < depth && dist_src(src, (p1 + p2 + p3) / 3.0) < ratio * size) {
            level++;
            path = path * 4;
            continue;
        }
        emit_leaf(pc, acc, b, frac0 * ldexp(1.0, -2 * level));
        while (level > 0 && (path & 3) == 3) {
            path >>= 2;
            level--;
        }
        if (level == 0) break;
        path++;
    }
}

// vertex_pieces! (assemble.jl:102-116): the vertex rule toward corner k of the piece with corners p, b; tan: this
// lane's tangent of b and frac (adjoint; null for a piece fixed in the test triangle)
template <class Acc>
__device__ __noinline__ void vertex_pieces(PairCtx& pc, Acc& acc, const v3<double>* p, int k, const double* b, double frac,
                              const double* tan) {
    int i = (k + 1) % 3, j = (k + 2) % 3;
    v3<double> u = p[i] - p[k], v = p[j] - p[k];
    double cs = dot(u, v) / (vnorm(u) * vnorm(v));
    double th = acos(fmin(fmax(cs, -1.0), 1.0));
    if (th <= vp_pi<double>() / 2) {
        double c[9];
        rotate_corners(b, k, c);
        if constexpr (kAdj<Acc>) {
            double ct[10];
            if (tan) {
                rotate_corners(tan, k, ct);
                ct[9] = tan[9];
            }
            piece_begin(pc, acc, c, frac, tan ? ct : nullptr);
        }
        emit_rule(pc, acc, R_VERT, c, frac);
        if constexpr (kAdj<Acc>) piece_end(pc, acc);
        return;
    }
    int m = int(ceil(th * (180.0 / vp_pi<double>()) / pc.a->corner_angle));  // rad2deg(θ) = θ * (180 / π), as Julia
    double nu = vnorm(u), nv = vnorm(v);
    double t0 = 0;
    // adjoint: tangents of the split parameters
    double dth = 0, dnu = 0, dnv = 0, dt0 = 0;
    const double zero10[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    const double* tp = tan ? tan : zero10;
    if constexpr (kAdj<Acc>) {
        v3<double> pk = tan_point(pc, b + 3 * k, tp + 3 * k), pi_ = tan_point(pc, b + 3 * i, tp + 3 * i),
                   pj = tan_point(pc, b + 3 * j, tp + 3 * j);
        v3<double> du = pi_ - pk, dv = pj - pk;
        dnu = dot(u, du) / nu;
        dnv = dot(v, dv) / nv;
        double dcs = (dot(du, v) + dot(u, dv)) / (nu * nv) - cs * (dnu / nu + dnv / nv);
        dth = -dcs / sqrt(fmax(1 - cs * cs, 1e-300));
    }
    for (int q = 0; q < m; ++q) {
        double t1 = 1.0, dt1 = 0;
        if (q + 1 < m) {
            double phi = th * (q + 1) / m;
            double an = nu * sin(phi), bn = nv * sin(th - phi);
            t1 = an / (an + bn);
            if constexpr (kAdj<Acc>) {
                double dphi = dth * (q + 1) / m;
                double dan = dnu * sin(phi) + nu * cos(phi) * dphi;
                double dbn = dnv * sin(th - phi) + nv * cos(th - phi) * (dth - dphi);
                dt1 = (dan * bn - an * dbn) / ((an + bn) * (an + bn));
            }
        }
        double c[9];
        for (int z = 0; z < 3; ++z) c[z] = b[3 * k + z];
        bmix(c + 3, b + 3 * i, 1 - t0, b + 3 * j, t0);
        bmix(c + 6, b + 3 * i, 1 - t1, b + 3 * j, t1);
        if constexpr (kAdj<Acc>) {
            double ct[10];
            for (int z = 0; z < 3; ++z) {
                ct[z] = tp[3 * k + z];
                ct[3 + z] = (1 - t0) * tp[3 * i + z] + t0 * tp[3 * j + z] + dt0 * (b[3 * j + z] - b[3 * i + z]);
                ct[6 + z] = (1 - t1) * tp[3 * i + z] + t1 * tp[3 * j + z] + dt1 * (b[3 * j + z] - b[3 * i + z]);
            }
            ct[9] = tp[9] * (t1 - t0) + frac * (dt1 - dt0);
            piece_begin(pc, acc, c, frac * (t1 - t0), ct);
        }
        emit_rule(pc, acc, R_VERT, c, frac * (t1 - t0));
        if constexpr (kAdj<Acc>) piece_end(pc, acc);
        t0 = t1;
        dt0 = dt1;
    }
}

__device__ __forceinline__ bool on_edge_split(v3<double> q, v3<double> a, v3<double> c, double tol, double& t) {
    double L = vnorm(c - a), d;
    seg_proj(q, a, c, d, t);
    return d <= tol && t * L > tol && (1 - t) * L > tol;
}

// contact_rule / contact_pieces! (assemble.jl:199-238) for a triangle source S; returns false without contact
template <class Acc>
__device__ __noinline__ bool contact_rule(PairCtx& pc, Acc& acc, const TriGeo& S, const bool* shared) {
    const TriGeo& T = *pc.T;
    const NearArgs& a = *pc.a;
    double tol = a.contact_rel * fmin(T.diam, S.diam);
    if (vnorm(ld3(S.c) - ld3(T.c)) > T.reach + S.reach + tol) return false;
    SrcRef src{0, S.x, {}, {}};
    bool extra = false;
    for (int k = 0; k < 3; ++k)
        if (!shared[k] && dist_tri(S.x, ld3(T.x + 3 * k)) <= tol) extra = true;
    if (!extra)
        for (int k = 0; k < 3 && !extra; ++k)
            for (int q = 0; q < 3; ++q) {
                double t;
                if (on_edge_split(ld3(S.x + 3 * q), ld3(T.x + 3 * k), ld3(T.x + 3 * ((k + 1) % 3)), tol, t)) {
                    extra = true;
                    break;
                }
            }
    if (!extra) return false;
    // explicit stack of pieces: corners (9), frac, level; adjoint: this lane's tangent of corners and frac
    double stk[16][11];
    double tstk[kAdj<Acc> ? 16 : 1][10];
    int sp = 0;
    for (int k = 0; k < 9; ++k) stk[0][k] = (k == 0 || k == 4 || k == 8) ? 1.0 : 0.0;
    stk[0][9] = 1.0;
    stk[0][10] = 0;
    if constexpr (kAdj<Acc>)
        for (int k = 0; k < 10; ++k) tstk[0][k] = 0;
    sp = 1;
    while (sp > 0) {
        --sp;
        double b[9], tb[10];
        for (int k = 0; k < 9; ++k) b[k] = stk[sp][k];
        double frac = stk[sp][9];
        int level = int(stk[sp][10]);
        if constexpr (kAdj<Acc>)
            for (int k = 0; k < 10; ++k) tb[k] = tstk[sp][k];
        v3<double> p[3] = {tpoint(T, b), tpoint(T, b + 3), tpoint(T, b + 6)};
        if (level < 4) {
            int ks = -1;
            double ts[5], dts[5] = {0, 0, 0, 0, 0};
            int tq[5] = {0, 0, 0, 0, 0};
            int nts = 0;
            for (int k = 0; k < 3 && ks < 0; ++k) {
                nts = 0;
                for (int q = 0; q < 3; ++q) {
                    double t;
                    if (on_edge_split(ld3(S.x + 3 * q), p[k], p[(k + 1) % 3], tol, t)) {
                        ts[1 + nts] = t;
                        tq[1 + nts] = q;
                        nts++;
                    }
                }
                if (nts) ks = k;
            }
            if (ks >= 0) {
                for (int x = 2; x <= nts; ++x)  // sort the split parameters
                    for (int y = x; y > 1 && ts[y] < ts[y - 1]; --y) {
                        double tmp = ts[y];
                        ts[y] = ts[y - 1];
                        ts[y - 1] = tmp;
                        int tmq = tq[y];
                        tq[y] = tq[y - 1];
                        tq[y - 1] = tmq;
                    }
                ts[0] = 0;
                ts[nts + 1] = 1;
                const int k1 = (ks + 1) % 3, ko = (ks + 2) % 3;
                const double *bk = b + 3 * ks, *bk1 = b + 3 * k1, *opp = b + 3 * ko;
                if constexpr (kAdj<Acc>) {
                    // t = ((S_q - p_k)·e) / (e·e), e = p_k1 - p_k (seg_proj)
                    v3<double> dpk = tan_point(pc, bk, tb + 3 * ks), dpk1 = tan_point(pc, bk1, tb + 3 * k1);
                    v3<double> e = p[k1] - p[ks], de = dpk1 - dpk;
                    double ee = dot(e, e);
                    for (int x = 1; x <= nts; ++x) {
                        v3<double> sq = ld3(S.x + 3 * tq[x]);
                        dts[x] = (dot(tan_source(pc, tq[x]) - dpk, e) + dot(sq - p[ks], de)) / ee -
                                 2 * ts[x] * dot(e, de) / ee;
                    }
                }
                // push in reverse so that the pieces are processed in order
                for (int i = nts; i >= 0; --i) {
                    if (sp >= 16) {
                        if (pc.lane == 0) atomicExch((int*)&pc.sh->leaf[0][0], 0);  // never: depth-bounded
                        break;
                    }
                    if constexpr (kAdj<Acc>) {
                        double* te = tstk[sp];
                        for (int z = 0; z < 3; ++z) {
                            te[z] = (1 - ts[i]) * tb[3 * ks + z] + ts[i] * tb[3 * k1 + z] + dts[i] * (bk1[z] - bk[z]);
                            te[3 + z] = (1 - ts[i + 1]) * tb[3 * ks + z] + ts[i + 1] * tb[3 * k1 + z] +
                                        dts[i + 1] * (bk1[z] - bk[z]);
                            te[6 + z] = tb[3 * ko + z];
                        }
                        te[9] = tb[9] * (ts[i + 1] - ts[i]) + frac * (dts[i + 1] - dts[i]);
                    }
                    double* e = stk[sp++];
                    bmix(e, bk, 1 - ts[i], bk1, ts[i]);
                    bmix(e + 3, bk, 1 - ts[i + 1], bk1, ts[i + 1]);
                    for (int z = 0; z < 3; ++z) e[6 + z] = opp[z];
                    e[9] = frac * (ts[i + 1] - ts[i]);
                    e[10] = level + 1;
                }
                continue;
            }
        }
        // pieces below a split move with the geometry
        const double* tan = (kAdj<Acc> && level > 0) ? tb : nullptr;
        bool on[3];
        int nc = 0;
        for (int q = 0; q < 3; ++q) {
            on[q] = dist_tri(S.x, p[q]) <= tol;
            nc += on[q];
        }
        if (nc == 2) {
            int k = !on[2] ? 0 : (!on[0] ? 1 : 2);
            if (dist_tri(S.x, (p[k] + p[(k + 1) % 3]) / 2.0) <= tol) {
                double c[9];  // rules.edge[k] on piece b: corners (b_k, b_k+1, b_k+2)
                rotate_corners(b, k, c);
                if constexpr (kAdj<Acc>) {
                    double ct[10];
                    if (tan) {
                        rotate_corners(tan, k, ct);
                        ct[9] = tan[9];
                    }
                    piece_begin(pc, acc, c, frac, tan ? ct : nullptr);
                }
                emit_rule(pc, acc, R_EDGE, c, frac);
                if constexpr (kAdj<Acc>) piece_end(pc, acc);
                continue;
            }
        }
        if (nc == 1) {
            vertex_pieces(pc, acc, p, on[0] ? 0 : (on[1] ? 1 : 2), b, frac, tan);
        } else if (nc == 0) {
            if constexpr (kAdj<Acc>) piece_begin(pc, acc, b, frac, tan);
            near_pieces(pc, acc, src, b, frac, a.near_depth);
            if constexpr (kAdj<Acc>) piece_end(pc, acc);
        } else {
            if constexpr (kAdj<Acc>) piece_begin(pc, acc, b, frac, tan);
            emit_rule(pc, acc, R_SELF, b, frac);
            if constexpr (kAdj<Acc>) piece_end(pc, acc);
        }
    }
    return true;
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ void setup_tri_source(PairCtx& pc, const TriGeo& S) {
    if (pc.lane == 0) {
        WarpSh& sh = *pc.sh;
        const TriGeo& T = *pc.T;
        for (int k = 0; k < 3; ++k)
            for (int q = 0; q < 3; ++q)
                for (int z = 0; z < 3; ++z) {
                    sh.E[9 * k + 3 * q + z] = T.x[3 * k + z] - S.x[3 * q + z];
                    sh.E32[9 * k + 3 * q + z] = float(sh.E[9 * k + 3 * q + z]);
                }
        for (int k = 0; k < 3; ++k)
            for (int z = 0; z < 3; ++z) {
                sh.D[3 * k + z] = T.x[3 * k + z] - S.c[z];
                sh.D32[3 * k + z] = float(sh.D[3 * k + z]);
            }
        for (int k = 0; k < 9; ++k) {
            sh.Sd[k] = S.x[k] - S.c[k % 3];
            sh.Snu[k] = S.nu[k];
            sh.Sdf[k] = float(sh.Sd[k]);
            sh.Snuf[k] = float(S.nu[k]);
        }
        for (int k = 0; k < 3; ++k) {
            sh.Sn[k] = S.n[k];
            sh.Slen[k] = S.len[k];
            sh.Snf[k] = float(S.n[k]);
            sh.Slenf[k] = float(S.len[k]);
        }
        sh.Sarea = S.area;
        sh.Sdiam = S.diam;
        sh.Sareaf = float(S.area);
        sh.Sdiamf = float(S.diam);
    }
    __syncwarp();
}

// the rule of one triangle pair and its evaluation; returns the tier. Sources: body (wake = 0) or wake triangle.
template <class Acc>
__device__ int tri_pair(PairCtx& pc, Acc& acc, int t, int s, bool wake) {
    const NearArgs& a = *pc.a;
    const TriGeo& T = *pc.T;
    const TriGeo& S = wake ? a.wtri[s] : a.tri[s];
    setup_tri_source(pc, S);
    const double corners[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    pc.side = (!wake && s == t) ? 1 : 0;
    pc.fp32 = a.mixed;
    if (!wake && s == t) {
        emit_rule(pc, acc, R_SELF, corners, 1.0);
        return TIER_SELF;
    }
    bool shared[3] = {false, false, false};
    int ns = 0;
    if (!wake)
        for (int k = 0; k < 3; ++k) {
            shared[k] = T.node[k] == S.node[0] || T.node[k] == S.node[1] || T.node[k] == S.node[2];
            ns += shared[k];
        }
    if (contact_rule(pc, acc, S, shared)) {
        flush_leaves(pc, acc);
        return TIER_CONTACT;
    }
    if (ns == 2) {
        int k = (shared[0] && shared[1]) ? 0 : ((shared[1] && shared[2]) ? 1 : 2);
        double c[9];
        for (int z = 0; z < 3; ++z) {
            c[z] = corners[3 * k + z];
            c[3 + z] = corners[3 * ((k + 1) % 3) + z];
            c[6 + z] = corners[3 * ((k + 2) % 3) + z];
        }
        emit_rule(pc, acc, R_EDGE, c, 1.0);
        return TIER_EDGE;
    }
    if (ns == 1) {
        int k = shared[0] ? 0 : (shared[1] ? 1 : 2);
        v3<double> p[3] = {ld3(T.x), ld3(T.x + 3), ld3(T.x + 6)};
        v3<double> u = p[(k + 1) % 3] - p[k], v = p[(k + 2) % 3] - p[k];
        if (dot(u, v) >= 0) {  // vertex_rule (assemble.jl:119-125): the stored rotation
            double c[9];
            for (int z = 0; z < 3; ++z) {
                c[z] = corners[3 * k + z];
                c[3 + z] = corners[3 * ((k + 1) % 3) + z];
                c[6 + z] = corners[3 * ((k + 2) % 3) + z];
            }
            emit_rule(pc, acc, R_VERT, c, 1.0);
        } else {
            vertex_pieces(pc, acc, p, k, corners, 1.0, nullptr);
        }
        return TIER_VERTEX;
    }
    int depth = a.near_depth;
    if (!wake && a.ntouch > 0) {
        long long key = (long long)t * a.ntri + s;
        int lo = 0, hi = a.ntouch;
        while (lo < hi) {
            int mid = (lo + hi) >> 1;
            if (a.touch[mid] < key) lo = mid + 1;
            else hi = mid;
        }
        if (lo < a.ntouch && a.touch[lo] == key) depth += 4;
    }
    SrcRef src{0, S.x, {}, {}};
    near_pieces(pc, acc, src, corners, 1.0, depth);
    flush_leaves(pc, acc);
    return TIER_NEAR;
}

// vertex_rule (assemble.jl:119-125) toward corner k of the whole test triangle
template <class Acc>
__device__ void vertex_rule(PairCtx& pc, Acc& acc, int k) {
    const TriGeo& T = *pc.T;
    const double corners[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    v3<double> p[3] = {ld3(T.x), ld3(T.x + 3), ld3(T.x + 6)};
    v3<double> u = p[(k + 1) % 3] - p[k], v = p[(k + 2) % 3] - p[k];
    if (dot(u, v) >= 0) {  // the stored rotation: corners (k, k+1, k+2)
        double c[9];
        for (int z = 0; z < 3; ++z) {
            c[z] = corners[3 * k + z];
            c[3 + z] = corners[3 * ((k + 1) % 3) + z];
            c[6 + z] = corners[3 * ((k + 2) % 3) + z];
        }
        emit_rule(pc, acc, R_VERT, c, 1.0);
    } else {
        vertex_pieces(pc, acc, p, k, corners, 1.0, nullptr);
    }
}

// ---- the near tier, one pair per lane: the plan shared by the assembly and the adjoint -------------------------------
// A warp takes up to 32 sources of its test triangle at once. Each lane decides its own pair's tier (FP32 with the
// reference's FP64 test where FP32 cannot decide, exactly as pair_rule / wake_pair_rule) and, for a pair in the near
// tier, walks near_pieces' quadtree to its leaves (assemble.jl:131-142), stored as codes, with the pair's FP32 frame.
struct NearPlanSh {
    uint8_t leaf[32][64];  // leaf codes: level << 6 | path (level base-4 digits, most significant first)
    float E32[32][27];     // x_T,k - v_S,a
    float D32[32][9];      // x_T,k - c_S
    float S32[32][26];     // d (9), nu (9), len (3), n (3), area, diam
};

__device__ __forceinline__ void leaf_corners32(int code, float* b) {
    // the corners of a quadtree node in the test triangle's barycentrics (dyadic, exact in FP32)
    int level = code >> 6, path = code & 63;
    float c[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    for (int l = 0; l < level; ++l) {
        int digit = (path >> (2 * (level - 1 - l))) & 3;
        float m12[3], m23[3], m31[3];
        for (int z = 0; z < 3; ++z) {
            m12[z] = 0.5f * (c[z] + c[3 + z]);
            m23[z] = 0.5f * (c[3 + z] + c[6 + z]);
            m31[z] = 0.5f * (c[6 + z] + c[z]);
        }
        float n[9];
        for (int z = 0; z < 3; ++z) {
            if (digit == 0) { n[z] = c[z]; n[3 + z] = m12[z]; n[6 + z] = m31[z]; }
            else if (digit == 1) { n[z] = m12[z]; n[3 + z] = c[3 + z]; n[6 + z] = m23[z]; }
            else if (digit == 2) { n[z] = m31[z]; n[3 + z] = m23[z]; n[6 + z] = c[6 + z]; }
            else { n[z] = m12[z]; n[3 + z] = m23[z]; n[6 + z] = m31[z]; }
        }
        for (int z = 0; z < 9; ++z) c[z] = n[z];
    }
    for (int z = 0; z < 9; ++z) b[z] = c[z];
}

// per-lane contributions (N values), keyed by pair (non-decreasing over the lanes, 32+ for none): segmented sums in a
// fixed order, added to the pairs' accumulators (accf for FP32 contributions, acc for FP64 ones)
template <int N, class V>
__device__ __forceinline__ void seg_accumulate(float (*accf)[N], double (*acc)[N], int lane, int key, V* v) {
    const unsigned FULL = 0xffffffffu;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int ky = __shfl_up_sync(FULL, key, o);
#pragma unroll
        for (int k = 0; k < N; ++k) {
            V y = __shfl_up_sync(FULL, v[k], o);
            if (lane >= o && ky == key) v[k] += y;
        }
    }
    int kn = __shfl_down_sync(FULL, key, 1);
    bool last = lane == 31 || kn != key;
    if (last && key < 32) {
        if (sizeof(V) == 4)
            for (int k = 0; k < N; ++k) accf[key][k] += float(v[k]);
        else
            for (int k = 0; k < N; ++k) acc[key][k] += double(v[k]);
    }
    __syncwarp();
}

// returns whether this lane's pair (source s, S; valid: the lane has one) is in the near tier; nleaf: its leaves
__device__ bool near_plan(PairCtx& pc, NearPlanSh& pl, int t, const TriGeo& S, int s, bool valid, bool wake, int& nleaf) {
    const NearArgs& a = *pc.a;
    const TriGeo& T = *pc.T;
    const int lane = pc.lane;
    // 1. the tier of this lane's pair
    bool near = valid && a.test_mode != 2 && a.near_depth <= 3 && !(!wake && s == t);
    if (near && !wake) {
        for (int k = 0; k < 3; ++k)
            if (T.node[k] == S.node[0] || T.node[k] == S.node[1] || T.node[k] == S.node[2]) near = false;
        if (near && a.ntouch > 0) {
            long long key = (long long)t * a.ntri + s;
            int lo = 0, hi = a.ntouch;
            while (lo < hi) {
                int mid = (lo + hi) >> 1;
                if (a.touch[mid] < key) lo = mid + 1;
                else hi = mid;
            }
            if (lo < a.ntouch && a.touch[lo] == key) near = false;
        }
    }
    // FP32 frame of this pair: S's corner 0 at the origin (differences taken in FP64); e32 bounds the FP32 rounding
    v3<float> sv[3], tv[3];
    float e32 = 0.f;
    if (near) {
        for (int q = 0; q < 3; ++q) {
            sv[q] = mk3(float(S.x[3 * q] - S.x[0]), float(S.x[3 * q + 1] - S.x[1]), float(S.x[3 * q + 2] - S.x[2]));
            tv[q] = mk3(float(T.x[3 * q] - S.x[0]), float(T.x[3 * q + 1] - S.x[1]), float(T.x[3 * q + 2] - S.x[2]));
            e32 = fmaxf(e32, fmaxf(vnorm(sv[q]), vnorm(tv[q])));
        }
        e32 *= 1e-4f;
    }
    if (near) {  // contact_rule (assemble.jl:199-207) finds no contact beyond shared corners
        const double tol = a.contact_rel * fmin(T.diam, S.diam);
        const float tolf = float(tol);
        // FP32 pass: 1 contact, 0 none, -1 undecided (then the FP64 test decides)
        int res;
        {
            v3<float> dc = (sv[1] + sv[2]) * (1.f / 3.f) - (tv[0] + tv[1] + tv[2]) * (1.f / 3.f);
            int far_reach = lt32(float(T.reach + S.reach + tol), vnorm(dc), e32);
            if (far_reach == 1) {
                res = 0;
            } else {
                bool any_true = false, any_undec = far_reach < 0;
                for (int k = 0; k < 3; ++k) {
                    int c = lt32(dist_tri_v(sv[0], sv[1], sv[2], tv[k]), tolf, e32);
                    if (c == 1) any_true = true;
                    else if (c < 0) any_undec = true;
                }
                for (int k = 0; k < 3 && !any_true; ++k) {
                    v3<float> ta = tv[k], tc = tv[(k + 1) % 3];
                    v3<float> ev = tc - ta;
                    float L = vnorm(ev);
                    for (int q = 0; q < 3; ++q) {
                        float t = dot(sv[q] - ta, ev) / dot(ev, ev);
                        t = fminf(fmaxf(t, 0.f), 1.f);
                        float d = vnorm(sv[q] - (ta + t * ev));
                        int c1 = lt32(d, tolf, e32) , c2 = lt32(tolf, t * L, 2.f * e32), c3 = lt32(tolf, (1.f - t) * L, 2.f * e32);
                        if (d == tolf) c1 = -1;
                        if (c1 == 1 && c2 == 1 && c3 == 1) any_true = true;
                        else if (c1 != 0 && c2 != 0 && c3 != 0) any_undec = true;
                    }
                }
                res = any_true ? 1 : (any_undec ? -1 : 0);
                if (far_reach < 0 && res == 1) res = -1;  // contact needs the reach test passed
            }
        }
        if (res < 0) {  // the reference's FP64 test
            res = 0;
            if (!(vnorm(ld3(S.c) - ld3(T.c)) > T.reach + S.reach + tol)) {
                bool extra = false;
                for (int k = 0; k < 3 && !extra; ++k)
                    if (dist_tri(S.x, ld3(T.x + 3 * k)) <= tol) extra = true;
                for (int k = 0; k < 3 && !extra; ++k)
                    for (int q = 0; q < 3 && !extra; ++q) {
                        double tt;
                        if (on_edge_split(ld3(S.x + 3 * q), ld3(T.x + 3 * k), ld3(T.x + 3 * ((k + 1) % 3)), tol, tt))
                            extra = true;
                    }
                res = extra ? 1 : 0;
            }
        }
        if (res == 1) near = false;
    }
    // 2. near_pieces' leaves (assemble.jl:131-142), decided in FP32 unless a node is too close to the threshold
    if (near) {
        const int depth = a.near_depth;
        const float ratiof = float(a.near_ratio);
        int level = 0;
        unsigned path = 0;
        for (int guard = 0; guard < 1024; ++guard) {
            float bf[9];
            leaf_corners32((level << 6) | int(path), bf);
            v3<float> p1 = bf[0] * tv[0] + bf[1] * tv[1] + bf[2] * tv[2];
            v3<float> p2 = bf[3] * tv[0] + bf[4] * tv[1] + bf[5] * tv[2];
            v3<float> p3 = bf[6] * tv[0] + bf[7] * tv[1] + bf[8] * tv[2];
            float size = fmaxf(vnorm(p2 - p1), fmaxf(vnorm(p3 - p2), vnorm(p1 - p3)));
            float d = dist_tri_v(sv[0], sv[1], sv[2], (p1 + p2 + p3) * (1.f / 3.f));
            int split = level < depth ? lt32(d, ratiof * size, 2.f * e32) : 0;
            if (split < 0) {  // the reference's FP64 test at this node
                double b[9];
                for (int z = 0; z < 9; ++z) b[z] = double(bf[z]);
                v3<double> q1 = tpoint(T, b), q2 = tpoint(T, b + 3), q3 = tpoint(T, b + 6);
                double sz = fmax(vnorm(q2 - q1), fmax(vnorm(q3 - q2), vnorm(q1 - q3)));
                split = dist_tri(S.x, (q1 + q2 + q3) / 3.0) < a.near_ratio * sz ? 1 : 0;
            }
            if (split) {
                level++;
                path *= 4;
                continue;
            }
            pl.leaf[lane][nleaf++] = uint8_t((level << 6) | path);
            while (level > 0 && (path & 3) == 3) {
                path >>= 2;
                level--;
            }
            if (level == 0) break;
            path++;
        }
        for (int k = 0; k < 3; ++k)
            for (int q = 0; q < 3; ++q)
                for (int z = 0; z < 3; ++z) pl.E32[lane][9 * k + 3 * q + z] = float(T.x[3 * k + z] - S.x[3 * q + z]);
        for (int k = 0; k < 3; ++k)
            for (int z = 0; z < 3; ++z) pl.D32[lane][3 * k + z] = float(T.x[3 * k + z] - S.c[z]);
        for (int k = 0; k < 9; ++k) {
            pl.S32[lane][k] = float(S.x[k] - S.c[k % 3]);
            pl.S32[lane][9 + k] = float(S.nu[k]);
        }
        for (int k = 0; k < 3; ++k) {
            pl.S32[lane][18 + k] = float(S.len[k]);
            pl.S32[lane][21 + k] = float(S.n[k]);
        }
        pl.S32[lane][24] = float(S.area);
        pl.S32[lane][25] = float(S.diam);
    }
    return near;
}

// ------------------------------------------------------------------------------------------------------------------
// host: tiles and colours

// greedy colouring of groups of row slots: no two groups of one colour share a slot
std::vector<std::vector<int>> colour_groups(const std::vector<std::vector<int>>& groups, int nslot) {
    std::vector<std::vector<int>> of_slot(nslot);
    for (int g = 0; g < (int)groups.size(); ++g)
        for (int s : groups[g]) of_slot[s].push_back(g);
    std::vector<int> col(groups.size(), -1);
    std::vector<int> seen;
    int ncol = 0;
    for (int g = 0; g < (int)groups.size(); ++g) {
        seen.assign(ncol + 1, 0);
        for (int s : groups[g])
            for (int h : of_slot[s])
                if (h != g && col[h] >= 0) seen[col[h]] = 1;
        int c = 0;
        while (seen[c]) ++c;
        col[g] = c;
        ncol = std::max(ncol, c + 1);
    }
    std::vector<std::vector<int>> out(ncol);
    for (int g = 0; g < (int)groups.size(); ++g) out[col[g]].push_back(g);
    return out;
}

// unique slots of a group of corners, and the CSR from each unique slot to the corners (local index) using it
void unique_map(const std::vector<int>& corner_slots, int cap, int* uniq, int& nuniq, short* ptr, short* ent) {
    std::vector<int> u;
    for (int s : corner_slots)
        if (s >= 0 && std::find(u.begin(), u.end(), s) == u.end()) u.push_back(s);
    nuniq = (int)u.size();
    std::vector<int> cnt(nuniq + 1, 0);
    for (int i = 0; i < cap; ++i) uniq[i] = i < nuniq ? u[i] : 0;
    int k = 0;
    for (int j = 0; j < nuniq; ++j) {
        ptr[j] = (short)k;
        for (int c = 0; c < (int)corner_slots.size(); ++c)
            if (corner_slots[c] == u[j]) ent[k++] = (short)c;
    }
    for (int j = nuniq; j <= cap; ++j) ptr[j] = (short)k;
    for (int j = k; j < cap; ++j) ent[j] = 0;
}

struct DevList {
    std::vector<void*> ptrs;
    ~DevList() {
        for (void* p : ptrs) cudaFree(p);
    }
    template <class T>
    int up(vp_ctx* ctx, T** d, const std::vector<T>& h) {
        int r = vp_upload(ctx, d, h.data(), h.size());
        if (!r) ptrs.push_back((void*)*d);
        return r;
    }
    template <class T>
    int alloc(vp_ctx* ctx, T** d, size_t n) {
        int r = vp_alloc(ctx, d, n);
        if (!r) ptrs.push_back((void*)*d);
        return r;
    }
};

template <class T>
void fill_soa(const std::vector<TriGeo>& g, std::vector<T>& soa, int& pad) {
    int n = (int)g.size();
    pad = std::max(1, ((n + FAR_NT - 1) / FAR_NT) * FAR_NT);
    soa.assign(size_t(NFIELD) * pad, T(0));
    for (int s = 0; s < n; ++s) {
        const TriGeo& e = g[s];
        auto put = [&](int f, double v) { soa[size_t(f) * pad + s] = T(v); };
        for (int k = 0; k < 3; ++k) {
            T h = T(e.c[k]);
            put(k, e.c[k]);
            put(3 + k, sizeof(T) == 4 ? e.c[k] - double(h) : 0.0);
        }
        put(6, e.diam);
        put(7, e.area);
        put(8, e.sigma);
        for (int q = 0; q < 3; ++q)
            for (int k = 0; k < 3; ++k) {
                put(9 + 3 * q + k, e.x[3 * q + k] - e.c[k]);
                put(18 + 3 * q + k, e.nu[3 * q + k]);
                put(33 + 3 * q + k, e.gam[3 * q + k]);
            }
        for (int k = 0; k < 3; ++k) {
            put(27 + k, e.len[k]);
            put(30 + k, e.n[k]);
        }
    }
}

CentF cent_of(const TriGeo& e) {
    CentF c;
    float hx = float(e.c[0]), hy = float(e.c[1]), hz = float(e.c[2]);
    c.hx = hx;
    c.hy = hy;
    c.hz = hz;
    c.lx = float(e.c[0] - double(hx));
    c.ly = float(e.c[1] - double(hy));
    c.lz = float(e.c[2] - double(hz));
    c.diam = float(e.diam);
    c.pad = 0;
    return c;
}

struct SrcTiles {
    int ntile = 0;
    std::vector<int> cols, ncol;
    std::vector<short> cptr, cent;
};

SrcTiles make_src_tiles(const std::vector<TriGeo>& g) {
    SrcTiles st;
    int n = (int)g.size();
    st.ntile = (n + FAR_NT - 1) / FAR_NT;
    st.cols.assign(size_t(st.ntile) * 3 * FAR_NT, 0);
    st.ncol.assign(st.ntile, 0);
    st.cptr.assign(size_t(st.ntile) * (3 * FAR_NT + 1), 0);
    st.cent.assign(size_t(st.ntile) * 3 * FAR_NT, 0);
    for (int k = 0; k < st.ntile; ++k) {
        std::vector<int> cs(3 * FAR_NT, -1);
        for (int i = 0; i < FAR_NT; ++i) {
            int s = k * FAR_NT + i;
            if (s < n)
                for (int b = 0; b < 3; ++b) cs[3 * i + b] = g[s].slot[b];
        }
        unique_map(cs, 3 * FAR_NT, &st.cols[size_t(k) * 3 * FAR_NT], st.ncol[k], &st.cptr[size_t(k) * (3 * FAR_NT + 1)],
                   &st.cent[size_t(k) * 3 * FAR_NT]);
    }
    return st;
}

// ------------------------------------------------------------------------------------------------------------------
// host: the set-up shared by the assembly and its adjoint: checks, element data, rules, far points of the test
// triangles, uploads, and the classification of every test triangle's non-far sources

struct PairInput {
    const vp_assembly_options* o;
    int nnode;
    const double* x;
    int ntri;
    const int* tris;
    const int* corner_slot;
    int nslot, ntouch;
    const int* touch_pairs;
    const double* sigma;
    const double* vinf;
    int nwnode;
    const double* wx;
    int nwtri;
    const int* wtris;
    int nfil;
    const int* fil;
    bool body_sources = true;  // false: only the wake's sheets and filaments are sources (explicit_rhs)
};

struct PairSetup {
    DevList dl;
    bool mixed = false;
    int ncols = 0, nq = 0;
    float ratio32 = 0.f;
    std::vector<TriGeo> tg, wg;  // wg holds one dummy entry when there is no wake
    std::vector<RulePt> rfar, rnear, redge, rvert, rself;
    TriGeo *d_tg = nullptr, *d_wg = nullptr;
    CentF *d_tc = nullptr, *d_wc = nullptr;
    double *d_tq = nullptr, *d_tw = nullptr, *d_wx = nullptr;
    int* d_fil = nullptr;
    RulePt* d_rule[5] = {};
    float4* d_rulef[5] = {};
    std::vector<long long> nfptr, wfptr;
    long long *d_nfptr = nullptr, *d_wfptr = nullptr;
    int *d_nf = nullptr, *d_wf = nullptr;
    std::vector<long long> touch_keys;
    long long* d_touch = nullptr;
};

int check_pair_input(vp_ctx* ctx, const PairInput& in) {
    const vp_assembly_options* o = in.o;
    if (!ctx || !o || !in.x || !in.tris || !in.corner_slot || !in.sigma || !in.vinf)
        return vp_fail(ctx, VP_ERR_ARG, "null argument");
    if (o->test < 0 || o->test > 2) return vp_fail(ctx, VP_ERR_ARG, "test must be hat, onering or dual");
    auto okpts = [](int n) { return n == 1 || n == 3 || n == 6 || n == 7; };
    if (!okpts(o->far_points) || !okpts(o->near_points))
        return vp_fail(ctx, VP_ERR_ARG, "far_points and near_points must be 1, 3, 6 or 7");
    if (o->near_depth < 0 || o->near_depth > 9 || o->touch_levels < 1 || o->touch_order < 1 || !(o->touch_ratio > 0) ||
        !(o->touch_ratio < 1) || !(o->corner_angle > 0) || !(o->far_ratio > 0) || !(o->near_ratio >= 0) ||
        !(o->contact_rel >= 0) || !(o->kernel_far > 0))
        return vp_fail(ctx, VP_ERR_ARG, "assembly option out of range");
    if (o->precision != VP_FP64 && o->precision != VP_MIXED) return vp_fail(ctx, VP_ERR_ARG, "unknown precision");
    if (in.ntri <= 0 || in.nnode <= 0 || in.nslot <= 0 || in.nwnode < 0 || in.nwtri < 0 || in.nfil < 0 || in.ntouch < 0)
        return vp_fail(ctx, VP_ERR_ARG, "sizes must be positive");
    if (in.nwnode == 0 && (in.nwtri > 0 || in.nfil > 0)) return vp_fail(ctx, VP_ERR_ARG, "wake elements without wake nodes");
    if ((in.nwtri > 0 && (!in.wx || !in.wtris)) || (in.nfil > 0 && !in.fil) || (in.ntouch > 0 && !in.touch_pairs))
        return vp_fail(ctx, VP_ERR_ARG, "null argument");
    for (int i = 0; i < 3 * in.ntri; ++i) {
        if (in.tris[i] < 0 || in.tris[i] >= in.nnode) return vp_fail(ctx, VP_ERR_ARG, "triangle node out of range");
        if (in.corner_slot[i] < 0 || in.corner_slot[i] >= in.nslot)
            return vp_fail(ctx, VP_ERR_ARG, "corner slot out of range");
    }
    for (int i = 0; i < 3 * in.nwtri; ++i)
        if (in.wtris[i] < 0 || in.wtris[i] >= in.nwnode) return vp_fail(ctx, VP_ERR_ARG, "wake triangle node out of range");
    for (int i = 0; i < 2 * in.nfil; ++i)
        if (in.fil[i] < 0 || in.fil[i] >= in.nwnode) return vp_fail(ctx, VP_ERR_ARG, "filament node out of range");
    for (int i = 0; i < 2 * in.ntouch; ++i)
        if (in.touch_pairs[i] < 0 || in.touch_pairs[i] >= in.ntri) return vp_fail(ctx, VP_ERR_ARG, "touch pair out of range");
    return VP_OK;
}

// ph_setup / ph_classify: the phases the uploads and the classification are timed under
int setup_pairs(vp_ctx* ctx, const PairInput& in, int ph_setup, int ph_classify, PairSetup& ps) {
    int r;
    if ((r = check_pair_input(ctx, in))) return r;
    const vp_assembly_options* o = in.o;
    const int ntri = in.ntri, nwtri = in.nwtri;
    ps.mixed = o->precision == VP_MIXED;
    ps.ncols = in.nslot + in.nwnode;
    // elements
    ps.tg.resize(ntri);
    ps.wg.resize(nwtri);
    for (int t = 0; t < ntri; ++t) {
        const int* tr = in.tris + 3 * t;
        if (!make_tri(in.x + 3 * tr[0], in.x + 3 * tr[1], in.x + 3 * tr[2], ps.tg[t]))
            return vp_fail(ctx, VP_ERR_DEGENERATE, "degenerate triangle " + std::to_string(t));
        ps.tg[t].sigma = in.sigma[t];
        for (int k = 0; k < 3; ++k) {
            ps.tg[t].node[k] = tr[k];
            ps.tg[t].slot[k] = in.corner_slot[3 * t + k];
        }
    }
    for (int t = 0; t < nwtri; ++t) {
        const int* tr = in.wtris + 3 * t;
        if (!make_tri(in.wx + 3 * tr[0], in.wx + 3 * tr[1], in.wx + 3 * tr[2], ps.wg[t]))
            return vp_fail(ctx, VP_ERR_DEGENERATE, "degenerate wake triangle " + std::to_string(t));
        for (int k = 0; k < 3; ++k) {
            ps.wg[t].node[k] = -1 - tr[k];
            ps.wg[t].slot[k] = tr[k];
        }
    }
    // rules
    ps.rfar = triangle_rule(o->far_points);
    ps.rnear = triangle_rule(o->near_points);
    ps.redge = edge_rule(o->touch_levels, o->touch_ratio, o->touch_order);
    ps.rvert = vertex_rule_base(o->touch_levels, o->touch_ratio, o->touch_order);
    ps.rself = self_rule(ps.redge);
    // far points and weights of every test triangle
    const int nq = ps.nq = (int)ps.rfar.size();
    std::vector<double> tq(size_t(ntri) * NQMAX * 3, 0.0), tw(size_t(ntri) * NQMAX * 3, 0.0);
    for (int t = 0; t < ntri; ++t) {
        const TriGeo& e = ps.tg[t];
        for (int p = 0; p < nq; ++p) {
            const RulePt& m = ps.rfar[p];
            double l[3] = {m.l0, m.l1, m.l2};
            for (int k = 0; k < 3; ++k)
                tq[(size_t(t) * NQMAX + p) * 3 + k] = l[0] * e.x[k] + l[1] * e.x[3 + k] + l[2] * e.x[6 + k];
            double W = m.w * e.area;
            double psi[3];
            if (o->test == 0) {
                psi[0] = l[0]; psi[1] = l[1]; psi[2] = l[2];
            } else if (o->test == 1) {
                psi[0] = psi[1] = psi[2] = 1;
            } else {
                double mx = std::max(l[0], std::max(l[1], l[2]));
                int cnt = 0;
                for (int k = 0; k < 3; ++k) cnt += std::fabs(l[k] - mx) < 1e-12;
                for (int k = 0; k < 3; ++k) psi[k] = (std::fabs(l[k] - mx) < 1e-12) ? 1.0 / cnt : 0.0;
            }
            for (int k = 0; k < 3; ++k) tw[(size_t(t) * NQMAX + p) * 3 + k] = W * psi[k];
        }
    }
    std::vector<CentF> tc(ntri), wc(std::max(nwtri, 1));
    for (int t = 0; t < ntri; ++t) tc[t] = cent_of(ps.tg[t]);
    for (int t = 0; t < nwtri; ++t) wc[t] = cent_of(ps.wg[t]);

    DevList& dl = ps.dl;
    if (ph_setup >= 0) vp_phase_begin(ctx, ph_setup);
    if (ps.wg.empty()) ps.wg.resize(1);
    if ((r = dl.up(ctx, &ps.d_tg, ps.tg)) || (r = dl.up(ctx, &ps.d_wg, ps.wg)) || (r = dl.up(ctx, &ps.d_tc, tc)) ||
        (r = dl.up(ctx, &ps.d_wc, wc)) || (r = dl.up(ctx, &ps.d_tq, tq)) || (r = dl.up(ctx, &ps.d_tw, tw)))
        return r;
    {
        const double* wx = in.wx && in.nwnode ? in.wx : in.x;
        const int* fil = in.fil && in.nfil ? in.fil : in.tris;
        std::vector<double> hwx(wx, wx + 3 * std::max(in.nwnode, 1));
        std::vector<int> hfil(fil, fil + 2 * std::max(in.nfil, 1));
        if ((r = dl.up(ctx, &ps.d_wx, hwx)) || (r = dl.up(ctx, &ps.d_fil, hfil))) return r;
    }
    {
        const std::vector<RulePt>* R[5] = {&ps.rnear, &ps.rself, &ps.redge, &ps.rvert, &ps.rfar};
        for (int k = 0; k < 5; ++k) {
            std::vector<float4> f(R[k]->size());
            for (size_t i = 0; i < f.size(); ++i)
                f[i] = make_float4(float((*R[k])[i].l0), float((*R[k])[i].l1), float((*R[k])[i].l2), float((*R[k])[i].w));
            if ((r = dl.up(ctx, &ps.d_rule[k], *R[k])) || (r = dl.up(ctx, &ps.d_rulef[k], f))) return r;
        }
    }
    // touching pairs, both orders, sorted keys t * ntri + s
    for (int i = 0; i < in.ntouch; ++i) {
        long long a0 = in.touch_pairs[2 * i], b0 = in.touch_pairs[2 * i + 1];
        ps.touch_keys.push_back(a0 * ntri + b0);
        ps.touch_keys.push_back(b0 * ntri + a0);
    }
    std::sort(ps.touch_keys.begin(), ps.touch_keys.end());
    ps.touch_keys.erase(std::unique(ps.touch_keys.begin(), ps.touch_keys.end()), ps.touch_keys.end());
    {
        std::vector<long long> keys = ps.touch_keys;
        if (keys.empty()) keys.push_back(-1);
        if ((r = dl.up(ctx, &ps.d_touch, keys))) return r;
    }
    if (ph_setup >= 0) vp_phase_end(ctx);
    // classification of the non-far sources of every test triangle
    if (ph_classify >= 0) vp_phase_begin(ctx, ph_classify);
    int* d_cnt;
    if ((r = dl.alloc(ctx, &d_cnt, size_t(ntri)))) return r;
    ps.nfptr.assign(ntri + 1, 0);
    ps.wfptr.assign(ntri + 1, 0);
    std::vector<int> cnt(ntri);
    ps.ratio32 = float(o->far_ratio);
    if (in.body_sources) {
        classify_kernel<<<ntri, 256, 0, ctx->stream>>>(0, ntri, ps.d_tc, ps.d_tg, ntri, ps.d_tc, ps.d_tg, ps.ratio32,
                                                       o->far_ratio, d_cnt, nullptr, nullptr);
        ctx->launches++;
        VP_CUDA(ctx, vp_d2h(ctx, cnt.data(), d_cnt, sizeof(int) * ntri));
        VP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        for (int t = 0; t < ntri; ++t) ps.nfptr[t + 1] = ps.nfptr[t] + cnt[t];
    }
    if (nwtri > 0) {
        classify_kernel<<<ntri, 256, 0, ctx->stream>>>(0, ntri, ps.d_tc, ps.d_tg, nwtri, ps.d_wc, ps.d_wg, ps.ratio32,
                                                       o->far_ratio, d_cnt, nullptr, nullptr);
        ctx->launches++;
        VP_CUDA(ctx, vp_d2h(ctx, cnt.data(), d_cnt, sizeof(int) * ntri));
        VP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        for (int t = 0; t < ntri; ++t) ps.wfptr[t + 1] = ps.wfptr[t] + cnt[t];
    }
    if ((r = dl.up(ctx, &ps.d_nfptr, ps.nfptr)) || (r = dl.up(ctx, &ps.d_wfptr, ps.wfptr)) ||
        (r = dl.alloc(ctx, &ps.d_nf, size_t(std::max(ps.nfptr[ntri], 1LL)))) ||
        (r = dl.alloc(ctx, &ps.d_wf, size_t(std::max(ps.wfptr[ntri], 1LL)))))
        return r;
    if (in.body_sources) {
        classify_kernel<<<ntri, 256, 0, ctx->stream>>>(1, ntri, ps.d_tc, ps.d_tg, ntri, ps.d_tc, ps.d_tg, ps.ratio32,
                                                       o->far_ratio, nullptr, ps.d_nfptr, ps.d_nf);
        ctx->launches++;
    }
    if (nwtri > 0) {
        classify_kernel<<<ntri, 256, 0, ctx->stream>>>(1, ntri, ps.d_tc, ps.d_tg, nwtri, ps.d_wc, ps.d_wg, ps.ratio32,
                                                       o->far_ratio, nullptr, ps.d_wfptr, ps.d_wf);
        ctx->launches++;
    }
    VP_CUDA(ctx, cudaGetLastError());
    if (ph_classify >= 0) vp_phase_end(ctx);
    return VP_OK;
}

// the arguments of the near, touching and contact kernels that come from the set-up (A, b, tests, stats and the
// rest lists are the caller's)
// ---- the rest pairs (self, touching, contact) as one list, for the pair-parallel kernels ---------------------------
// The lanes kernels leave, per test triangle t and source set (0 body, 1 wake), rest_cnt[2t + set] pairs at the
// start of its segment of rest_src / wrest_src. Their exclusive prefix sums number the pairs 0 .. total - 1 in the
// order (t, set, position); a warp of a pair-parallel kernel takes the next number from a counter.

constexpr int SCAN_NT = 1024;

// rest_off[i] = sum of cnt[0 .. i - 1] for i = 0 .. n (one block of SCAN_NT threads)
__global__ void __launch_bounds__(SCAN_NT) rest_scan_kernel(const int* __restrict__ cnt, int n, long long* off) {
    __shared__ long long s[SCAN_NT];
    __shared__ long long carry;
    const int i0 = threadIdx.x;
    if (i0 == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < n; base += SCAN_NT) {
        const int i = base + i0;
        const long long v = i < n ? (long long)cnt[i] : 0;
        s[i0] = v;
        __syncthreads();
        for (int o = 1; o < SCAN_NT; o <<= 1) {
            const long long u = i0 >= o ? s[i0 - o] : 0;
            __syncthreads();
            s[i0] += u;
            __syncthreads();
        }
        if (i < n) off[i] = carry + s[i0] - v;
        __syncthreads();
        if (i0 == SCAN_NT - 1) carry += s[SCAN_NT - 1];
        __syncthreads();
    }
    if (i0 == 0) off[n] = carry;
}

// the (t, set) entry g = 2 t + set of rest pair idx: the largest g with off[g] <= idx (0 <= idx < off[n], so g < n
// and off[g + 1] > idx: empty entries are skipped)
__device__ __forceinline__ int rest_entry(const long long* __restrict__ off, int n, long long idx) {
    int lo = 0, hi = n;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (off[mid] <= idx) lo = mid;
        else hi = mid;
    }
    return lo;
}

// the next rest pair of this warp (all lanes call it together)
__device__ __forceinline__ long long next_rest_pair(unsigned long long* next, int lane) {
    unsigned long long v = 0;
    if (lane == 0) v = atomicAdd(next, 1ull);
    return (long long)__shfl_sync(0xffffffffu, v, 0);
}

// the offsets of the rest pairs (after the lanes kernel) and a zeroed work counter; with `total`, the number of rest
// pairs is copied to the host (the stream is synchronised)
int rest_list(vp_ctx* ctx, DevList& dl, NearArgs& na, long long* total) {
    long long* d_off;
    unsigned long long* d_next;
    int r;
    const int n = 2 * na.ntri;
    if ((r = dl.alloc(ctx, &d_off, size_t(n) + 1)) || (r = dl.alloc(ctx, &d_next, 1))) return r;
    rest_scan_kernel<<<1, SCAN_NT, 0, ctx->stream>>>(na.rest_cnt, n, d_off);
    ctx->launches++;
    VP_CUDA(ctx, cudaGetLastError());
    VP_CUDA(ctx, cudaMemsetAsync(d_next, 0, sizeof(unsigned long long), ctx->stream));
    na.rest_off = d_off;
    na.next = d_next;
    if (total) {
        VP_CUDA(ctx, vp_d2h(ctx, total, d_off + n, sizeof(long long)));
        VP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    }
    return VP_OK;
}

// CTAs of a persistent pair-parallel kernel: as many as stay resident on every SM
template <class K>
int persistent_blocks(vp_ctx* ctx, K kernel, int threads, size_t smem) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem) != cudaSuccess || per_sm < 1)
        per_sm = 1;
    return per_sm * std::max(ctx->nsm, 1);
}

NearArgs near_args(const PairSetup& ps, const PairInput& in) {
    const vp_assembly_options* o = in.o;
    NearArgs na{};
    na.tri = ps.d_tg;
    na.wtri = ps.d_wg;
    na.wx = ps.d_wx;
    na.fil = ps.d_fil;
    na.ntri = in.ntri;
    na.nwtri = in.nwtri;
    na.nfil = in.nfil;
    na.nslot = in.nslot;
    na.nf_ptr = ps.d_nfptr;
    na.nf_src = ps.d_nf;
    na.wf_ptr = ps.d_wfptr;
    na.wf_src = ps.d_wf;
    na.touch = ps.d_touch;
    na.ntouch = (int)ps.touch_keys.size();
    const int nr[5] = {(int)ps.rnear.size(), (int)ps.rself.size(), (int)ps.redge.size(), (int)ps.rvert.size(),
                       (int)ps.rfar.size()};
    for (int k = 0; k < 5; ++k) {
        na.rule[k] = ps.d_rule[k];
        na.rulef[k] = ps.d_rulef[k];
        na.nrule[k] = nr[k];
    }
    na.lda = ps.ncols;
    na.test_mode = o->test;
    na.near_depth = o->near_depth;
    na.mixed = ps.mixed ? 1 : 0;
    na.far_ratio = o->far_ratio;
    na.near_ratio = o->near_ratio;
    na.corner_angle = o->corner_angle;
    na.contact_rel = o->contact_rel;
    na.kernel_far = o->kernel_far;
    na.kernel_far32 = float(o->kernel_far);
    for (int k = 0; k < 3; ++k) {
        na.vinf[k] = in.vinf[k];
        na.tint[k] = o->test == 1 ? 1.0 : 1.0 / 3;
    }
    return na;
}


}  // namespace
