// Galerkin assembly on the GPU: assemble(g, dm, els, σ, V∞; opts, wake) of src/assembly/assemble.jl:377-447.
//
// A_ij = ∫ψ_i n·u[φ_j] dA, b_i = -∫ψ_i n·(V∞ + u_σ) dA over all (test, source) triangle pairs, each pair's 3x3 block
// and 3-vector computed with the quadrature tier of pair_rule (assemble.jl:266-282).
//
// Pipeline (one CUDA stream):
//   1. classification: for every test triangle, the sources that are NOT in the far tier (far test of
//      assemble.jl:269, FP32 with an exact FP64 fallback near the threshold), compacted in source order;
//   2. far tier: tile kernel, one CTA per tile of TT test triangles, one thread per source of a 128-source tile;
//      the far rule's points of the test tile sit in shared memory, each thread keeps its source in registers,
//      evaluates w analytically (FP32 with double-float offsets in VP_MIXED, FP64 in VP_FP64), contracts it into
//      the 3x3 hat block and gathers the tile's blocks into the slots of A in a fixed order. Test tiles are coloured
//      so that no two tiles of one launch share a row slot: the scatter needs no atomics and A is reproducible bit
//      for bit;
//   3. near, touching and contact tiers: one warp per test triangle (triangles coloured by shared slots, one launch
//      per colour) walks its non-far sources in order, builds each pair's rule as the reference does (self, edge,
//      vertex with wide-corner wedges, contact splits, recursive near subdivision), and evaluates the rule's points
//      across its lanes: FP64 for the touching and contact tiers, FP32 or FP64 for the near tier, FP64 for the
//      wake's tip filaments.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <numeric>
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
// FP32 guard of the adjoint's derivative evaluations (corner, edge sin^2, plane): tighter than the forward's
#define ADJ_GUARD 3e-2f, 1e-1f, 1e-3f

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

template <class T, int TT>
__global__ void __launch_bounds__(FAR_NT) far_kernel(FarArgs a) {
    __shared__ FarTest<T> ts[TT];
    __shared__ T blk[TT][FAR_NT][9];
    __shared__ T rbsum[TT * 3][FAR_NT / 32];
    __shared__ int s_cols[3 * FAR_NT];
    __shared__ short s_cptr[3 * FAR_NT + 1];
    __shared__ short s_cent[3 * FAR_NT];
    __shared__ int s_rows[3 * TT];
    __shared__ short s_rptr[3 * TT + 1];
    __shared__ short s_rent[3 * TT];
    __shared__ int s_ncol, s_nrow;

    const int tile = a.tiles[blockIdx.x];
    const int tid = threadIdx.x;
    // the test tile
    for (int i = tid; i < TT; i += FAR_NT) {
        int t = tile * TT + i;
        FarTest<T>& q = ts[i];
        q.valid = t < a.ntest;
        if (q.valid) {
            const TriGeo& g = a.tgeo[t];
            for (int p = 0; p < a.nq; ++p)
                for (int k = 0; k < 3; ++k) {
                    double x = a.tq[(size_t(t) * NQMAX + p) * 3 + k];
                    T h = T(x);
                    q.xh[p][k] = h;
                    q.xl[p][k] = T(x - double(h));
                    q.wpsi[p][k] = T(a.tw[(size_t(t) * NQMAX + p) * 3 + k]);
                }
            for (int k = 0; k < 3; ++k) {
                q.n[k] = T(g.n[k]);
                q.c64[k] = g.c[k];
            }
            q.diam64 = g.diam;
            q.cf = a.tcent[t];
        }
    }
    if (tid < 3 * TT) s_rows[tid] = a.trow[size_t(tile) * 3 * TT + tid];
    if (tid <= 3 * TT) s_rptr[tid] = a.trptr[size_t(tile) * (3 * TT + 1) + tid];
    if (tid < 3 * TT) s_rent[tid] = a.trent[size_t(tile) * 3 * TT + tid];
    if (tid == 0) s_nrow = a.tnrow[tile];
    __syncthreads();

    T rb[TT][3];
#pragma unroll
    for (int i = 0; i < TT; ++i) rb[i][0] = rb[i][1] = rb[i][2] = T(0);

    for (int set = 0; set < a.nset; ++set) {
        const T* soa = (const T*)a.soa[set];
        const int pad = a.pad[set];
        for (int st = 0; st < a.ntile[set]; ++st) {
            const int s = st * FAR_NT + tid;
            const bool sv = s < a.nsrc[set];
            // the source in registers
            SrcKern<T> S;
            v3<T> ch, cl, gam[3];
            T sig = T(0);
            CentF scf;
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
                    gam[k] = mk3(F(33 + 3 * k), F(34 + 3 * k), F(35 + 3 * k));
                }
                S.n = mk3(F(30), F(31), F(32));
#undef F
                scf = a.scent[set][s];
            }
#pragma unroll
            for (int i = 0; i < TT; ++i) {
                T out[9];
#pragma unroll
                for (int k = 0; k < 9; ++k) out[k] = T(0);
                const FarTest<T>& q = ts[i];
                bool far = false;
                if (sv && q.valid) {
                    if (sizeof(T) == 8) {
                        far = far_exact64(q.c64, q.diam64, a.sgeo[set][s].c, a.sgeo[set][s].diam, a.ratio);
                    } else {
                        int f = far_test32(q.cf, scf, a.ratio32);
                        if (f < 0) f = far_exact64(q.c64, q.diam64, a.sgeo[set][s].c, a.sgeo[set][s].diam, a.ratio);
                        far = f == 1;
                    }
                }
                if (far) {
                    v3<T> P[3] = {mk3(T(0), T(0), T(0)), mk3(T(0), T(0), T(0)), mk3(T(0), T(0), T(0))};
                    for (int p = 0; p < a.nq; ++p) {
                        v3<T> r = mk3((q.xh[p][0] - ch.x) + (q.xl[p][0] - cl.x), (q.xh[p][1] - ch.y) + (q.xl[p][1] - cl.y),
                                      (q.xh[p][2] - ch.z) + (q.xl[p][2] - cl.z));
                        v3<T> w = sv_rel(S, r, 0, T(a.kernel_far), T(1e-12));
                        P[0] += q.wpsi[p][0] * w;
                        P[1] += q.wpsi[p][1] * w;
                        P[2] += q.wpsi[p][2] * w;
                    }
                    v3<T> nT = mk3(q.n[0], q.n[1], q.n[2]);
#pragma unroll
                    for (int bb = 0; bb < 3; ++bb) {
                        v3<T> m = cross(nT, gam[bb]);
                        out[0 * 3 + bb] = dot(P[0], m);
                        out[1 * 3 + bb] = dot(P[1], m);
                        out[2 * 3 + bb] = dot(P[2], m);
                    }
                    rb[i][0] -= sig * dot(P[0], nT);
                    rb[i][1] -= sig * dot(P[1], nT);
                    rb[i][2] -= sig * dot(P[2], nT);
                }
#pragma unroll
                for (int k = 0; k < 9; ++k) blk[i][tid][k] = out[k];
            }
            // the source tile's unique columns
            const size_t tb = size_t(st);
            for (int k = tid; k < 3 * FAR_NT; k += FAR_NT) {
                s_cols[k] = a.tile_cols[set][tb * 3 * FAR_NT + k];
                s_cent[k] = a.tile_cent[set][tb * 3 * FAR_NT + k];
            }
            for (int k = tid; k <= 3 * FAR_NT; k += FAR_NT) s_cptr[k] = a.tile_cptr[set][tb * (3 * FAR_NT + 1) + k];
            if (tid == 0) s_ncol = a.tile_ncol[set][tb];
            __syncthreads();
            // gather into A in a fixed order: cell (r, c) = sum over the test corners of row r and the source corners
            // of column c; rows are this CTA's alone in this launch
            const int nrow = s_nrow, ncol = s_ncol;
            for (int cell = tid; cell < nrow * ncol; cell += FAR_NT) {
                int r = cell / ncol, c = cell - r * ncol;
                double acc = 0;
                for (int u = s_rptr[r]; u < s_rptr[r + 1]; ++u) {
                    int ti = s_rent[u] / 3, ta = s_rent[u] - 3 * ti;
                    T part = T(0);
                    for (int v = s_cptr[c]; v < s_cptr[c + 1]; ++v) {
                        int sj = s_cent[v] / 3, sb = s_cent[v] - 3 * sj;
                        part += blk[ti][sj][ta * 3 + sb];
                    }
                    acc += double(part);
                }
                double* dst = a.A + size_t(s_rows[r]) * size_t(a.lda) + a.col_off[set] + s_cols[c];
                *dst += acc;
            }
            __syncthreads();
        }
    }
    // right hand side: fixed-order block reduction of the per-thread partial sums
    const int lane = tid & 31, wid = tid >> 5;
#pragma unroll
    for (int i = 0; i < TT; ++i)
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            T v = rb[i][k];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            if (lane == 0) rbsum[i * 3 + k][wid] = v;
        }
    __syncthreads();
    if (tid < s_nrow) {
        double acc = 0;
        for (int u = s_rptr[tid]; u < s_rptr[tid + 1]; ++u) {
            T v = T(0);
            for (int w = 0; w < FAR_NT / 32; ++w) v += rbsum[s_rent[u]][w];
            acc += double(v);
        }
        a.b[s_rows[tid]] += acc;
    }
}

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
    // adjoint: the test function weights nu_a at T's corners, the pair's direction m, a filament's end values
    double nu[3];
    v3<double> m;
    v3<float> mf;
    double mua, mub;
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

// evaluate one point (barycentric l on T, weight W) in FP64
__device__ __forceinline__ void eval_point64(const PairCtx& pc, FwdAcc& acc, double l0, double l1, double l2, double W) {
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
        v3<double> w = dot(r, r) > fd * fd ? sv_far(S, r) : sv_exact3(S, ra, rb, rc, r, pc.side, 1e-12);
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
__device__ __forceinline__ bool eval_point32(const PairCtx& pc, FwdAcc& acc, float l0, float l1, float l2, float W) {
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
    float fd = float(pc.a->kernel_far) * S.diam;
    if (dot(r, r) > fd * fd) {
        w = sv_far(S, r);
    } else {
        const float* E = sh.E32;
        v3<float> ra = l0 * mk3(E[0], E[1], E[2]) + l1 * mk3(E[9], E[10], E[11]) + l2 * mk3(E[18], E[19], E[20]);
        v3<float> rb = l0 * mk3(E[3], E[4], E[5]) + l1 * mk3(E[12], E[13], E[14]) + l2 * mk3(E[21], E[22], E[23]);
        v3<float> rc = l0 * mk3(E[6], E[7], E[8]) + l1 * mk3(E[15], E[16], E[17]) + l2 * mk3(E[24], E[25], E[26]);
        const Fp32Guard g{1e-2f, 4e-2f, 1e-4f};
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
    AdjSums<double> d;  // FP64 sums
    AdjSums<float> f;   // FP32 partial sums, folded into d every few points
    int nf;
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
    adj_add(acc.d, acc.f);
    adj_zero(acc.f);
    acc.nf = 0;
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
__device__ __forceinline__ void eval_point64(const PairCtx& pc, AdjAcc& acc, double l0, double l1, double l2, double W) {
    const WarpSh& sh = *pc.sh;
    v3<double> psi = test_weights(pc.a->test_mode, l0, l1, l2);
    double Wn = W * (pc.nu[0] * psi.x + pc.nu[1] * psi.y + pc.nu[2] * psi.z);
    v3<double> ra = l0 * ld3(sh.E + 0) + l1 * ld3(sh.E + 9) + l2 * ld3(sh.E + 18);
    v3<double> rb = l0 * ld3(sh.E + 3) + l1 * ld3(sh.E + 12) + l2 * ld3(sh.E + 21);
    if (pc.kind == 0) {
        v3<double> rc = l0 * ld3(sh.E + 6) + l1 * ld3(sh.E + 15) + l2 * ld3(sh.E + 24);
        v3<double> r = l0 * ld3(sh.D) + l1 * ld3(sh.D + 3) + l2 * ld3(sh.D + 6);
        SrcKern<double> S = src64(sh);
        double fd = pc.a->kernel_far * S.diam;
        if (dot(r, r) > fd * fd)
            adj_point_far(acc.d, S, Wn, l0, l1, l2, r, pc.m);
        else
            adj_point_exact(acc.d, S, Wn, l0, l1, l2, ra, rb, rc, r, pc.m, pc.side, 1e-12);
    } else {
        v3<double> n = ld3(pc.T->n), va, vb, ga, gb;
        segment_velocity(ra, rb, va, vb);
        seg_vjp(ra, rb, n, pc.mua, pc.mub, ga, gb);
        acc.d.Q += Wn * (pc.mua * va + pc.mub * vb);
        v3<double> gx = ga + gb;
        acc.d.Xg[0] += (Wn * l0) * gx;
        acc.d.Xg[1] += (Wn * l1) * gx;
        acc.d.Xg[2] += (Wn * l2) * gx;
        acc.d.Gr[0] += Wn * ga;
        acc.d.Gr[1] += Wn * gb;
    }
}

// one point in FP32 under the guard, adjoint; false when it must be evaluated in FP64
__device__ __forceinline__ bool eval_point32(const PairCtx& pc, AdjAcc& acc, float l0, float l1, float l2, float W) {
    if (pc.a->test_mode == 2) return false;
    const WarpSh& sh = *pc.sh;
    SrcKern<float> S = src32(sh);
    v3<float> r = l0 * mk3(sh.D32[0], sh.D32[1], sh.D32[2]) + l1 * mk3(sh.D32[3], sh.D32[4], sh.D32[5]) +
                  l2 * mk3(sh.D32[6], sh.D32[7], sh.D32[8]);
    v3<float> psi = pc.a->test_mode == 0 ? mk3(l0, l1, l2) : mk3(1.f, 1.f, 1.f);
    float Wn = W * (float(pc.nu[0]) * psi.x + float(pc.nu[1]) * psi.y + float(pc.nu[2]) * psi.z);
    float fd = float(pc.a->kernel_far) * S.diam;
    if (dot(r, r) > fd * fd) {
        adj_point_far(acc.f, S, Wn, l0, l1, l2, r, pc.mf);
    } else {
        const float* E = sh.E32;
        v3<float> ra = l0 * mk3(E[0], E[1], E[2]) + l1 * mk3(E[9], E[10], E[11]) + l2 * mk3(E[18], E[19], E[20]);
        v3<float> rb = l0 * mk3(E[3], E[4], E[5]) + l1 * mk3(E[12], E[13], E[14]) + l2 * mk3(E[21], E[22], E[23]);
        v3<float> rc = l0 * mk3(E[6], E[7], E[8]) + l1 * mk3(E[15], E[16], E[17]) + l2 * mk3(E[24], E[25], E[26]);
        if (!fp32_guard_ok(S, ra, rb, rc, pc.side, Fp32Guard{ADJ_GUARD})) return false;
        adj_point_exact(acc.f, S, Wn, l0, l1, l2, ra, rb, rc, r, pc.mf, pc.side, 1e-12f);
    }
    if (++acc.nf == 16) fold32(acc);
    return true;
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
__device__ void drain64(PairCtx& pc, Acc& acc, bool all, int rid, const double* b, double frac) {
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
    if (!pc.fp32) {
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
}

// a piece carrying a whole tabulated rule: lanes stride over its points
template <class Acc>
__device__ void emit_rule(PairCtx& pc, Acc& acc, int rid, const double* b, double frac) {
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
__device__ void flush_leaves(PairCtx& pc, Acc& acc) {
    const int nl = pc.nleaf;
    if (nl == 0) return;
    __syncwarp();
    const int n = pc.a->nrule[R_NEAR];
    for (int i0 = 0; i0 < nl * n; i0 += 32) {
        int i = i0 + pc.lane;
        bool valid = i < nl * n;
        int lf = valid ? i / n : 0, q = valid ? i - lf * n : 0;
        const double* b = pc.sh->leaf[lf];
        float bf[10];
        for (int z = 0; z < 9; ++z) bf[z] = float(b[z]);
        bf[9] = float(b[9] * pc.T->area);
        point_step(pc, acc, valid, R_NEAR, q, lf, b, bf, b[9]);
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
        for (int k = 0; k < 9; ++k) pc.sh->leaf[pc.nleaf][k] = b[k];
        pc.sh->leaf[pc.nleaf][9] = frac;
    }
    pc.nleaf++;
    if (pc.nleaf == LEAFBUF) flush_leaves(pc, acc);
}

__device__ __forceinline__ void bmix(double* o, const double* a, double sa, const double* b, double sb) {
    o[0] = sa * a[0] + sb * b[0];
    o[1] = sa * a[1] + sb * b[1];
    o[2] = sa * a[2] + sb * b[2];
}

// near_pieces! (assemble.jl:131-142) as a depth-first walk of the quadtree of sub-triangles
template <class Acc>
__device__ void near_pieces(PairCtx& pc, Acc& acc, const SrcRef& src, const double* b0, double frac0, int depth) {
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

// vertex_pieces! (assemble.jl:102-116): the vertex rule toward corner k of the piece with corners p, b
template <class Acc>
__device__ void vertex_pieces(PairCtx& pc, Acc& acc, const v3<double>* p, int k, const double* b, double frac) {
    int i = (k + 1) % 3, j = (k + 2) % 3;
    v3<double> u = p[i] - p[k], v = p[j] - p[k];
    double cs = dot(u, v) / (vnorm(u) * vnorm(v));
    double th = acos(fmin(fmax(cs, -1.0), 1.0));
    if (th <= vp_pi<double>() / 2) {
        double c[9];
        for (int q = 0; q < 3; ++q) {
            c[q] = b[3 * k + q];
            c[3 + q] = b[3 * i + q];
            c[6 + q] = b[3 * j + q];
        }
        emit_rule(pc, acc, R_VERT, c, frac);
        return;
    }
    int m = int(ceil(th * 180.0 / vp_pi<double>() / pc.a->corner_angle));
    double nu = vnorm(u), nv = vnorm(v);
    double t0 = 0;
    for (int q = 0; q < m; ++q) {
        double t1 = 1.0;
        if (q + 1 < m) {
            double phi = th * (q + 1) / m;
            t1 = nu * sin(phi) / (nu * sin(phi) + nv * sin(th - phi));
        }
        double c[9];
        for (int z = 0; z < 3; ++z) c[z] = b[3 * k + z];
        bmix(c + 3, b + 3 * i, 1 - t0, b + 3 * j, t0);
        bmix(c + 6, b + 3 * i, 1 - t1, b + 3 * j, t1);
        emit_rule(pc, acc, R_VERT, c, frac * (t1 - t0));
        t0 = t1;
    }
}

__device__ __forceinline__ bool on_edge_split(v3<double> q, v3<double> a, v3<double> c, double tol, double& t) {
    double L = vnorm(c - a), d;
    seg_proj(q, a, c, d, t);
    return d <= tol && t * L > tol && (1 - t) * L > tol;
}

// contact_rule / contact_pieces! (assemble.jl:199-238) for a triangle source S; returns false without contact
template <class Acc>
__device__ bool contact_rule(PairCtx& pc, Acc& acc, const TriGeo& S, const bool* shared) {
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
    // explicit stack of pieces: corners (9), frac, level
    double stk[16][11];
    int sp = 0;
    for (int k = 0; k < 9; ++k) stk[0][k] = (k == 0 || k == 4 || k == 8) ? 1.0 : 0.0;
    stk[0][9] = 1.0;
    stk[0][10] = 0;
    sp = 1;
    while (sp > 0) {
        --sp;
        double b[9];
        for (int k = 0; k < 9; ++k) b[k] = stk[sp][k];
        double frac = stk[sp][9];
        int level = int(stk[sp][10]);
        v3<double> p[3] = {tpoint(T, b), tpoint(T, b + 3), tpoint(T, b + 6)};
        if (level < 4) {
            int ks = -1;
            double ts[5];
            int nts = 0;
            for (int k = 0; k < 3 && ks < 0; ++k) {
                nts = 0;
                for (int q = 0; q < 3; ++q) {
                    double t;
                    if (on_edge_split(ld3(S.x + 3 * q), p[k], p[(k + 1) % 3], tol, t)) ts[1 + nts++] = t;
                }
                if (nts) ks = k;
            }
            if (ks >= 0) {
                for (int x = 2; x <= nts; ++x)  // sort the split parameters
                    for (int y = x; y > 1 && ts[y] < ts[y - 1]; --y) {
                        double tmp = ts[y];
                        ts[y] = ts[y - 1];
                        ts[y - 1] = tmp;
                    }
                ts[0] = 0;
                ts[nts + 1] = 1;
                const double *bk = b + 3 * ks, *bk1 = b + 3 * ((ks + 1) % 3), *opp = b + 3 * ((ks + 2) % 3);
                // push in reverse so that the pieces are processed in order
                for (int i = nts; i >= 0; --i) {
                    if (sp >= 16) {
                        if (pc.lane == 0) atomicExch((int*)&pc.sh->leaf[0][0], 0);  // never: depth-bounded
                        break;
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
                for (int z = 0; z < 3; ++z) {
                    c[z] = b[3 * k + z];
                    c[3 + z] = b[3 * ((k + 1) % 3) + z];
                    c[6 + z] = b[3 * ((k + 2) % 3) + z];
                }
                emit_rule(pc, acc, R_EDGE, c, frac);
                continue;
            }
        }
        if (nc == 1) {
            vertex_pieces(pc, acc, p, on[0] ? 0 : (on[1] ? 1 : 2), b, frac);
        } else if (nc == 0) {
            near_pieces(pc, acc, src, b, frac, a.near_depth);
        } else {
            emit_rule(pc, acc, R_SELF, b, frac);
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
            vertex_pieces(pc, acc, p, k, corners, 1.0);
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

__device__ void add_block(PairCtx& pc, FwdAcc& acc, const TriGeo& S, int col0, double* rbt, bool with_rhs) {
    // reduce the per-lane sums, contract with n_T x gamma_b and add the block to this warp's rows
    fold32(acc);
    double P[9];
    for (int a = 0; a < 3; ++a) {
        P[3 * a + 0] = warp_sum(acc.P[a].x);
        P[3 * a + 1] = warp_sum(acc.P[a].y);
        P[3 * a + 2] = warp_sum(acc.P[a].z);
    }
    const TriGeo& T = *pc.T;
    v3<double> nT = ld3(T.n);
    if (pc.lane < 9) {
        int ai = pc.lane / 3, bb = pc.lane % 3;
        v3<double> m = cross(nT, ld3(S.gam + 3 * bb));
        double v = P[3 * ai] * m.x + P[3 * ai + 1] * m.y + P[3 * ai + 2] * m.z;
        double* dst = pc.a->A + size_t(T.slot[ai]) * size_t(pc.a->lda) + col0 + S.slot[bb];
        *dst += v;
    }
    if (with_rhs)
        for (int ai = 0; ai < 3; ++ai)
            rbt[ai] -= S.sigma * (P[3 * ai] * nT.x + P[3 * ai + 1] * nT.y + P[3 * ai + 2] * nT.z);
    __syncwarp();
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
        vertex_pieces(pc, acc, p, k, corners, 1.0);
    }
}

// ---- the near tier, one pair per lane ---------------------------------------------------------------------------
// A warp takes up to 32 sources of its test triangle at once. Each lane decides its own pair's tier (FP64, exactly as
// pair_rule / wake_pair_rule) and, for a pair in the near tier, walks near_pieces' quadtree to its leaves. The
// warp then evaluates all leaves' points of the 32 pairs together, one point per lane (FP32, guarded; flagged points
// are queued and evaluated 32 at a time in FP64), reduces them per pair in a fixed order and adds the blocks to A
// pair by pair. Pairs of the other tiers are returned (a lane mask) for the warp-cooperative path.
struct NearChunkSh {
    uint8_t leaf[32][64];  // leaf codes: level << 6 | path (level base-4 digits, most significant first)
    float E32[32][27];     // x_T,k - v_S,a
    float D32[32][9];      // x_T,k - c_S
    float S32[32][26];     // d (9), nu (9), len (3), n (3), area, diam
    double acc[32][9];     // per pair: sum of W psi_a w (FP64 evaluations)
    float accf[32][9];     // per pair: the same sums of the FP32 evaluations
    int off[33];           // points before each pair
    int qp[64], qk[64];    // queued FP64 points: pair, point within the pair
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

// per-lane contributions W psi_a w_c (9 values), keyed by pair (non-decreasing over the lanes, 32+ for none):
// segmented sums in a fixed order, added to the pairs' FP64 accumulators
template <class V>
__device__ __forceinline__ void seg_accumulate(NearChunkSh& ns, int lane, int key, V* v) {
    const unsigned FULL = 0xffffffffu;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int ky = __shfl_up_sync(FULL, key, o);
#pragma unroll
        for (int k = 0; k < 9; ++k) {
            V y = __shfl_up_sync(FULL, v[k], o);
            if (lane >= o && ky == key) v[k] += y;
        }
    }
    int kn = __shfl_down_sync(FULL, key, 1);
    bool last = lane == 31 || kn != key;
    if (last && key < 32) {
        if (sizeof(V) == 4)
            for (int k = 0; k < 9; ++k) ns.accf[key][k] += float(v[k]);
        else
            for (int k = 0; k < 9; ++k) ns.acc[key][k] += double(v[k]);
    }
    __syncwarp();
}

// the FP64 evaluation of point k of pair p (queued by the FP32 guard): contributions in v
__device__ void near_point64(const NearArgs& a, const TriGeo& T, const TriGeo& S, const NearChunkSh& ns, int p, int k,
                             double* v) {
    const int nr = a.nrule[R_NEAR];
    int leaf = k / nr, q = k - leaf * nr;
    float bf[9];
    leaf_corners32(ns.leaf[p][leaf], bf);
    double b[9];
    for (int z = 0; z < 9; ++z) b[z] = double(bf[z]);
    RulePt m = a.rule[R_NEAR][q];
    double l0 = m.l0 * b[0] + m.l1 * b[3] + m.l2 * b[6];
    double l1 = m.l0 * b[1] + m.l1 * b[4] + m.l2 * b[7];
    double l2 = m.l0 * b[2] + m.l1 * b[5] + m.l2 * b[8];
    int level = ns.leaf[p][leaf] >> 6;
    double W = (m.w * ldexp(1.0, -2 * level)) * T.area;
    v3<double> x = mk3(l0 * T.x[0] + l1 * T.x[3] + l2 * T.x[6], l0 * T.x[1] + l1 * T.x[4] + l2 * T.x[7],
                       l0 * T.x[2] + l1 * T.x[5] + l2 * T.x[8]);
    v3<double> ra = mk3(l0 * (T.x[0] - S.x[0]) + l1 * (T.x[3] - S.x[0]) + l2 * (T.x[6] - S.x[0]),
                        l0 * (T.x[1] - S.x[1]) + l1 * (T.x[4] - S.x[1]) + l2 * (T.x[7] - S.x[1]),
                        l0 * (T.x[2] - S.x[2]) + l1 * (T.x[5] - S.x[2]) + l2 * (T.x[8] - S.x[2]));
    v3<double> rb = mk3(l0 * (T.x[0] - S.x[3]) + l1 * (T.x[3] - S.x[3]) + l2 * (T.x[6] - S.x[3]),
                        l0 * (T.x[1] - S.x[4]) + l1 * (T.x[4] - S.x[4]) + l2 * (T.x[7] - S.x[4]),
                        l0 * (T.x[2] - S.x[5]) + l1 * (T.x[5] - S.x[5]) + l2 * (T.x[8] - S.x[5]));
    v3<double> rc = mk3(l0 * (T.x[0] - S.x[6]) + l1 * (T.x[3] - S.x[6]) + l2 * (T.x[6] - S.x[6]),
                        l0 * (T.x[1] - S.x[7]) + l1 * (T.x[4] - S.x[7]) + l2 * (T.x[7] - S.x[7]),
                        l0 * (T.x[2] - S.x[8]) + l1 * (T.x[5] - S.x[8]) + l2 * (T.x[8] - S.x[8]));
    v3<double> r = x - ld3(S.c);
    SrcKern<double> K;
    for (int z = 0; z < 3; ++z) {
        K.d[z] = mk3(S.x[3 * z] - S.c[0], S.x[3 * z + 1] - S.c[1], S.x[3 * z + 2] - S.c[2]);
        K.nu[z] = ld3(S.nu + 3 * z);
        K.len[z] = S.len[z];
    }
    K.n = ld3(S.n);
    K.area = S.area;
    K.diam = S.diam;
    double fd = a.kernel_far * K.diam;
    v3<double> w = dot(r, r) > fd * fd ? sv_far(K, r) : sv_exact3(K, ra, rb, rc, r, 0, 1e-12);
    v3<double> psi = test_weights(a.test_mode, l0, l1, l2);
    double ps[3] = {W * psi.x, W * psi.y, W * psi.z};
    for (int ai = 0; ai < 3; ++ai) {
        v[3 * ai + 0] = ps[ai] * w.x;
        v[3 * ai + 1] = ps[ai] * w.y;
        v[3 * ai + 2] = ps[ai] * w.z;
    }
}

__device__ unsigned near_chunk(PairCtx& pc, NearChunkSh& ns, int t, const int* list, int cnt, bool wake, int col0,
                               double* rbt, unsigned long long* P, unsigned long long* Q, unsigned long long& Q64) {
    const NearArgs& a = *pc.a;
    const TriGeo& T = *pc.T;
    const int lane = pc.lane;
    const unsigned FULL = 0xffffffffu;
    const bool valid = lane < cnt;
    const int s = valid ? list[lane] : 0;
    const TriGeo& S = wake ? a.wtri[s] : a.tri[s];
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
    int nleaf = 0;
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
            ns.leaf[lane][nleaf++] = uint8_t((level << 6) | path);
            while (level > 0 && (path & 3) == 3) {
                path >>= 2;
                level--;
            }
            if (level == 0) break;
            path++;
        }
        for (int k = 0; k < 3; ++k)
            for (int q = 0; q < 3; ++q)
                for (int z = 0; z < 3; ++z) ns.E32[lane][9 * k + 3 * q + z] = float(T.x[3 * k + z] - S.x[3 * q + z]);
        for (int k = 0; k < 3; ++k)
            for (int z = 0; z < 3; ++z) ns.D32[lane][3 * k + z] = float(T.x[3 * k + z] - S.c[z]);
        for (int k = 0; k < 9; ++k) {
            ns.S32[lane][k] = float(S.x[k] - S.c[k % 3]);
            ns.S32[lane][9 + k] = float(S.nu[k]);
        }
        for (int k = 0; k < 3; ++k) {
            ns.S32[lane][18 + k] = float(S.len[k]);
            ns.S32[lane][21 + k] = float(S.n[k]);
        }
        ns.S32[lane][24] = float(S.area);
        ns.S32[lane][25] = float(S.diam);
    }
    for (int k = 0; k < 9; ++k) {
        ns.acc[lane][k] = 0.0;
        ns.accf[lane][k] = 0.f;
    }
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
    // 3. every leaf point of the chunk, one per lane
    const float kf = float(a.kernel_far), areaT = float(T.area);
    const Fp32Guard g{1e-2f, 4e-2f, 1e-4f};
    int nq = 0;
    unsigned long long n64 = 0;
    for (int i0 = 0; i0 < total; i0 += 32) {
        const int i = i0 + lane;
        const bool v = i < total;
        int p = 32 + lane, k = 0;
        float vals[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        bool need = false;
        if (v && !a.mixed) {  // FP64: every point through the FP64 queue
            int lo = 0, hi = 31;
            while (lo < hi) {
                int mid = (lo + hi + 1) >> 1;
                if (ns.off[mid] <= i) lo = mid;
                else hi = mid - 1;
            }
            p = lo;
            k = i - ns.off[p];
            need = true;
        } else if (v) {
            int lo = 0, hi = 31;
            while (lo < hi) {
                int mid = (lo + hi + 1) >> 1;
                if (ns.off[mid] <= i) lo = mid;
                else hi = mid - 1;
            }
            p = lo;
            k = i - ns.off[p];
            int leaf = k / nr, q = k - leaf * nr;
            int code = ns.leaf[p][leaf];
            float b[9];
            leaf_corners32(code, b);
            float4 m = a.rulef[R_NEAR][q];
            float l0 = m.x * b[0] + m.y * b[3] + m.z * b[6];
            float l1 = m.x * b[1] + m.y * b[4] + m.z * b[7];
            float l2 = m.x * b[2] + m.y * b[5] + m.z * b[8];
            float W = m.w * ldexpf(1.f, -2 * (code >> 6)) * areaT;
            const float* E = ns.E32[p];
            const float* Dp = ns.D32[p];
            const float* Sf = ns.S32[p];
            SrcKern<float> K;
            for (int z = 0; z < 3; ++z) {
                K.d[z] = mk3(Sf[3 * z], Sf[3 * z + 1], Sf[3 * z + 2]);
                K.nu[z] = mk3(Sf[9 + 3 * z], Sf[10 + 3 * z], Sf[11 + 3 * z]);
                K.len[z] = Sf[18 + z];
            }
            K.n = mk3(Sf[21], Sf[22], Sf[23]);
            K.area = Sf[24];
            K.diam = Sf[25];
            v3<float> r = l0 * mk3(Dp[0], Dp[1], Dp[2]) + l1 * mk3(Dp[3], Dp[4], Dp[5]) + l2 * mk3(Dp[6], Dp[7], Dp[8]);
            v3<float> w;
            float fd = kf * K.diam;
            bool ok = true;
            if (dot(r, r) > fd * fd) {
                w = sv_far(K, r);
            } else {
                v3<float> ra = l0 * mk3(E[0], E[1], E[2]) + l1 * mk3(E[9], E[10], E[11]) + l2 * mk3(E[18], E[19], E[20]);
                v3<float> rb = l0 * mk3(E[3], E[4], E[5]) + l1 * mk3(E[12], E[13], E[14]) + l2 * mk3(E[21], E[22], E[23]);
                v3<float> rc = l0 * mk3(E[6], E[7], E[8]) + l1 * mk3(E[15], E[16], E[17]) + l2 * mk3(E[24], E[25], E[26]);
                ok = sv_exact3_guarded(K, ra, rb, rc, 0, g, w);
            }
            if (ok) {
                v3<float> psi = a.test_mode == 0 ? mk3(l0, l1, l2) : mk3(1.f, 1.f, 1.f);
                float ps[3] = {W * psi.x, W * psi.y, W * psi.z};
                for (int ai = 0; ai < 3; ++ai) {
                    vals[3 * ai + 0] = ps[ai] * w.x;
                    vals[3 * ai + 1] = ps[ai] * w.y;
                    vals[3 * ai + 2] = ps[ai] * w.z;
                }
            } else {
                need = true;
            }
        }
        if (a.mixed) seg_accumulate(ns, lane, p, vals);  // flagged points add zero here, their FP64 value when drained
        unsigned m = __ballot_sync(FULL, need);
        if (m) {
            int pos = nq + __popc(m & ((1u << lane) - 1u));
            if (need) {
                ns.qp[pos] = p;
                ns.qk[pos] = k;
            }
            nq += __popc(m);
            __syncwarp();
        }
        while (nq >= 32 || (nq > 0 && i0 + 32 >= total)) {
            const int take = nq < 32 ? nq : 32;
            int qpair = 32 + lane;
            double qv[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
            if (lane < take) {
                qpair = ns.qp[lane];
                const TriGeo& Sq = wake ? a.wtri[list[qpair]] : a.tri[list[qpair]];
                near_point64(a, T, Sq, ns, qpair, ns.qk[lane], qv);
            }
            seg_accumulate(ns, lane, qpair, qv);
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
    // 4. the pairs' blocks, added pair by pair in source order
    double blk[9], rb[3] = {0, 0, 0};
    if (near) {
        double Pp[9];
        for (int k = 0; k < 9; ++k) Pp[k] = ns.acc[lane][k] + double(ns.accf[lane][k]);
        v3<double> nT = ld3(T.n);
        for (int bb = 0; bb < 3; ++bb) {
            v3<double> mv = cross(nT, ld3(S.gam + 3 * bb));
            for (int ai = 0; ai < 3; ++ai) blk[3 * ai + bb] = Pp[3 * ai] * mv.x + Pp[3 * ai + 1] * mv.y + Pp[3 * ai + 2] * mv.z;
        }
        for (int ai = 0; ai < 3; ++ai) rb[ai] = -S.sigma * (Pp[3 * ai] * nT.x + Pp[3 * ai + 1] * nT.y + Pp[3 * ai + 2] * nT.z);
    }
    for (int k = 0; k < cnt; ++k) {
        if (!((nearmask >> k) & 1u)) continue;
        double vk[9];
        for (int z = 0; z < 9; ++z) vk[z] = __shfl_sync(FULL, blk[z], k);
        if (!wake)
            for (int z = 0; z < 3; ++z) rbt[z] += __shfl_sync(FULL, rb[z], k);
        if (lane < 9) {
            int ai = lane / 3, bb = lane % 3;
            const TriGeo& Sk = wake ? a.wtri[list[k]] : a.tri[list[k]];
            double* dst = a.A + size_t(T.slot[ai]) * size_t(a.lda) + col0 + Sk.slot[bb];
            double val = vk[0];
            for (int z = 1; z < 9; ++z)
                if (z == lane) val = vk[z];
            *dst += val;
        }
        __syncwarp();
    }
    P[TIER_NEAR] += __popc(nearmask);
    Q[TIER_NEAR] += (unsigned long long)total;
    Q64 += n64;
    return __ballot_sync(FULL, valid && !near);
}

// near tier, one pair per lane; the other pairs are listed for near_kernel_rest
__global__ void __launch_bounds__(32 * NEAR_WARPS) near_kernel_lanes(NearArgs a) {
    extern __shared__ __align__(16) unsigned char near_smem[];
    NearChunkSh* shm = reinterpret_cast<NearChunkSh*>(near_smem);
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int idx = blockIdx.x * NEAR_WARPS + w;
    if (idx >= a.ntests) return;
    const int t = a.tests[idx];
    const TriGeo& T = a.tri[t];
    PairCtx pc;
    pc.a = &a;
    pc.T = &T;
    pc.sh = nullptr;
    pc.lane = lane;
    unsigned long long P[6] = {0, 0, 0, 0, 0, 0}, Q[6] = {0, 0, 0, 0, 0, 0}, Q64 = 0;
    double rbt[3] = {0, 0, 0};
    for (int set = 0; set < 2; ++set) {
        const bool wake = set == 1;
        const long long e0 = wake ? a.wf_ptr[t] : a.nf_ptr[t], e1 = wake ? a.wf_ptr[t + 1] : a.nf_ptr[t + 1];
        const int* src = wake ? a.wf_src : a.nf_src;
        int* rest = wake ? a.wrest_src : a.rest_src;
        const int col0 = wake ? a.nslot : 0;
        int nrest = 0;
        for (long long c0 = e0; c0 < e1; c0 += 32) {
            const int cnt = int(e1 - c0 < 32 ? e1 - c0 : 32);
            unsigned m = near_chunk(pc, shm[w], t, src + c0, cnt, wake, col0, rbt, P, Q, Q64);
            if ((m >> lane) & 1u) rest[e0 + nrest + __popc(m & ((1u << lane) - 1u))] = src[c0 + lane];
            nrest += __popc(m);
            __syncwarp();
        }
        if (lane == 0) a.rest_cnt[2 * t + set] = nrest;
    }
    if (lane == 0) {
        for (int k = 0; k < 3; ++k) a.b[T.slot[k]] += rbt[k];
        for (int k = 0; k < 6; ++k) {
            if (P[k]) atomicAdd(a.stats + k, P[k]);
            if (Q[k]) atomicAdd(a.stats + 6 + k, Q[k]);
        }
        if (Q64) atomicAdd(a.stats + 12, Q64);
    }
}

// the self, touching and contact pairs (one warp per test triangle), the tip filaments and the freestream
__global__ void __launch_bounds__(32 * NEAR_WARPS) near_kernel_rest(NearArgs a) {
    __shared__ WarpSh shm[NEAR_WARPS];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int idx = blockIdx.x * NEAR_WARPS + w;
    if (idx >= a.ntests) return;
    const int t = a.tests[idx];
    const TriGeo& T = a.tri[t];
    PairCtx pc;
    pc.a = &a;
    pc.T = &T;
    pc.sh = &shm[w];
    pc.lane = lane;
    pc.nleaf = 0;
    pc.nq64 = 0;
    pc.fp32 = 0;
    unsigned long long P[6] = {0, 0, 0, 0, 0, 0}, Q[6] = {0, 0, 0, 0, 0, 0}, Q64 = 0;
    double rbt[3] = {0, 0, 0};
    const double corners[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    for (int set = 0; set < 2; ++set) {
        const bool wake = set == 1;
        const long long e0 = wake ? a.wf_ptr[t] : a.nf_ptr[t];
        const int n = a.rest_cnt[2 * t + set];
        const int* rest = wake ? a.wrest_src : a.rest_src;
        const int col0 = wake ? a.nslot : 0;
        for (int e = 0; e < n; ++e) {
            const int s = rest[e0 + e];
            FwdAcc acc = {};
            pc.kind = 0;
            pc.npts = 0;
            pc.n64 = 0;
            pc.nleaf = 0;
            pc.nq64 = 0;
            int tier = tri_pair(pc, acc, t, s, wake);
            add_block(pc, acc, wake ? a.wtri[s] : a.tri[s], col0, rbt, !wake);
            P[tier] += 1;
            Q[tier] += pc.npts;
            Q64 += pc.n64;
        }
    }
    // tip filaments (assemble.jl:344-354): segment_rule (:299-306) and segment_block (:312-321), FP64
    for (int f = 0; f < a.nfil; ++f) {
        int ia = a.fil[2 * f], ib = a.fil[2 * f + 1];
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
        FwdAcc acc = {};
        pc.kind = 1;
        pc.npts = 0;
        pc.n64 = 0;
        pc.side = 0;
        pc.fp32 = 0;
        double L = vnorm(fb - fa);
        int tier;
        if (vnorm((fa + fb) / 2.0 - ld3(T.c)) > a.far_ratio * fmax(T.diam, L)) {
            tier = TIER_FAR;
            emit_rule(pc, acc, R_FAR, corners, 1.0);
        } else {
            int kv = -1;
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
        }
        double ca[3], cb[3];
        for (int k = 0; k < 3; ++k) {
            ca[k] = warp_sum(acc.ca[k]);
            cb[k] = warp_sum(acc.cb[k]);
        }
        if (lane < 3) {
            double* row = a.A + size_t(T.slot[lane]) * size_t(a.lda) + a.nslot;
            row[ia] += ca[lane];
            __syncwarp(0x7u);
            row[ib] += cb[lane];
        }
        __syncwarp();
        P[tier] += 1;
        Q[tier] += pc.npts;
        Q64 += pc.n64;
    }
    // freestream, exact (assemble.jl:422), and the rows of b
    if (lane == 0) {
        double vn = (a.vinf[0] * T.n[0] + a.vinf[1] * T.n[1] + a.vinf[2] * T.n[2]) * T.area;
        for (int k = 0; k < 3; ++k) a.b[T.slot[k]] += rbt[k] - vn * a.tint[k];
        for (int k = 0; k < 6; ++k) {
            if (P[k]) atomicAdd(a.stats + k, P[k]);
            if (Q[k]) atomicAdd(a.stats + 6 + k, Q[k]);
        }
        if (Q64) atomicAdd(a.stats + 12, Q64);
    }
}

// ------------------------------------------------------------------------------------------------------------------
// host: tiles, colours and the entry point

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

template <class T, int TT>
int run_far(vp_ctx* ctx, FarArgs fa, const std::vector<TriGeo>& tg, const std::vector<int>& cslot, int nslot,
            DevList& dl) {
    int nt = (int)tg.size();
    int ntiles = (nt + TT - 1) / TT;
    std::vector<int> trow(size_t(ntiles) * 3 * TT), tnrow(ntiles);
    std::vector<short> trptr(size_t(ntiles) * (3 * TT + 1)), trent(size_t(ntiles) * 3 * TT);
    std::vector<std::vector<int>> groups(ntiles);
    for (int k = 0; k < ntiles; ++k) {
        std::vector<int> cs(3 * TT, -1);
        for (int i = 0; i < TT; ++i) {
            int t = k * TT + i;
            if (t < nt)
                for (int a = 0; a < 3; ++a) cs[3 * i + a] = cslot[3 * t + a];
        }
        unique_map(cs, 3 * TT, &trow[size_t(k) * 3 * TT], tnrow[k], &trptr[size_t(k) * (3 * TT + 1)],
                   &trent[size_t(k) * 3 * TT]);
        for (int j = 0; j < tnrow[k]; ++j) groups[k].push_back(trow[size_t(k) * 3 * TT + j]);
    }
    auto colours = colour_groups(groups, nslot);
    int *d_trow, *d_tnrow;
    short *d_trptr, *d_trent;
    int r;
    if ((r = dl.up(ctx, &d_trow, trow)) || (r = dl.up(ctx, &d_tnrow, tnrow)) || (r = dl.up(ctx, &d_trptr, trptr)) ||
        (r = dl.up(ctx, &d_trent, trent)))
        return r;
    fa.trow = d_trow;
    fa.tnrow = d_tnrow;
    fa.trptr = d_trptr;
    fa.trent = d_trent;
    std::vector<int> all;
    std::vector<int> off{0};
    for (auto& c : colours) {
        all.insert(all.end(), c.begin(), c.end());
        off.push_back((int)all.size());
    }
    int* d_tiles;
    if ((r = dl.up(ctx, &d_tiles, all))) return r;
    for (size_t c = 0; c < colours.size(); ++c) {
        fa.tiles = d_tiles + off[c];
        int nb = off[c + 1] - off[c];
        if (nb) {
            far_kernel<T, TT><<<nb, FAR_NT, 0, ctx->stream>>>(fa);
            ctx->launches++;
        }
    }
    VP_CUDA(ctx, cudaGetLastError());
    return VP_OK;
}

}  // namespace

int vp_assemble_impl(vp_ctx* ctx, const vp_assembly_options* o, int nnode, const double* x, int ntri, const int* tris,
                     const int* corner_slot, int nslot, int ntouch, const int* touch_pairs, const double* sigma,
                     const double* vinf, int nwnode, const double* wx, int nwtri, const int* wtris, int nfil,
                     const int* fil, vp_system** out, vp_assembly_stats* stats) {
    auto t0 = std::chrono::steady_clock::now();
    if (!ctx || !o || !x || !tris || !corner_slot || !sigma || !vinf || !out) return vp_fail(ctx, VP_ERR_ARG, "null argument");
    *out = nullptr;
    if (o->test < 0 || o->test > 2) return vp_fail(ctx, VP_ERR_ARG, "test must be hat, onering or dual");
    auto okpts = [](int n) { return n == 1 || n == 3 || n == 6 || n == 7; };
    if (!okpts(o->far_points) || !okpts(o->near_points))
        return vp_fail(ctx, VP_ERR_ARG, "far_points and near_points must be 1, 3, 6 or 7");
    if (o->near_depth < 0 || o->near_depth > 9 || o->touch_levels < 1 || o->touch_order < 1 || !(o->touch_ratio > 0) ||
        !(o->touch_ratio < 1) || !(o->corner_angle > 0) || !(o->far_ratio > 0) || !(o->near_ratio >= 0) ||
        !(o->contact_rel >= 0) || !(o->kernel_far > 0))
        return vp_fail(ctx, VP_ERR_ARG, "assembly option out of range");
    if (o->precision != VP_FP64 && o->precision != VP_MIXED) return vp_fail(ctx, VP_ERR_ARG, "unknown precision");
    if (ntri <= 0 || nnode <= 0 || nslot <= 0 || nwnode < 0 || nwtri < 0 || nfil < 0 || ntouch < 0)
        return vp_fail(ctx, VP_ERR_ARG, "sizes must be positive");
    if (nwnode == 0 && (nwtri > 0 || nfil > 0)) return vp_fail(ctx, VP_ERR_ARG, "wake elements without wake nodes");
    for (int i = 0; i < 3 * ntri; ++i) {
        if (tris[i] < 0 || tris[i] >= nnode) return vp_fail(ctx, VP_ERR_ARG, "triangle node out of range");
        if (corner_slot[i] < 0 || corner_slot[i] >= nslot) return vp_fail(ctx, VP_ERR_ARG, "corner slot out of range");
    }
    for (int i = 0; i < 3 * nwtri; ++i)
        if (wtris[i] < 0 || wtris[i] >= nwnode) return vp_fail(ctx, VP_ERR_ARG, "wake triangle node out of range");
    for (int i = 0; i < 2 * nfil; ++i)
        if (fil[i] < 0 || fil[i] >= nwnode) return vp_fail(ctx, VP_ERR_ARG, "filament node out of range");
    for (int i = 0; i < 2 * ntouch; ++i)
        if (touch_pairs[i] < 0 || touch_pairs[i] >= ntri) return vp_fail(ctx, VP_ERR_ARG, "touch pair out of range");
    const bool mixed = o->precision == VP_MIXED;
    const int ncols = nslot + nwnode;

    // elements
    std::vector<TriGeo> tg(ntri), wg(nwtri);
    for (int t = 0; t < ntri; ++t) {
        if (!make_tri(x + 3 * tris[3 * t], x + 3 * tris[3 * t + 1], x + 3 * tris[3 * t + 2], tg[t]))
            return vp_fail(ctx, VP_ERR_DEGENERATE, "degenerate triangle " + std::to_string(t));
        tg[t].sigma = sigma[t];
        for (int k = 0; k < 3; ++k) {
            tg[t].node[k] = tris[3 * t + k];
            tg[t].slot[k] = corner_slot[3 * t + k];
        }
    }
    for (int t = 0; t < nwtri; ++t) {
        if (!make_tri(wx + 3 * wtris[3 * t], wx + 3 * wtris[3 * t + 1], wx + 3 * wtris[3 * t + 2], wg[t]))
            return vp_fail(ctx, VP_ERR_DEGENERATE, "degenerate wake triangle " + std::to_string(t));
        for (int k = 0; k < 3; ++k) {
            wg[t].node[k] = -1 - wtris[3 * t + k];
            wg[t].slot[k] = wtris[3 * t + k];
        }
    }
    // rules
    std::vector<RulePt> rfar = triangle_rule(o->far_points), rnear = triangle_rule(o->near_points);
    std::vector<RulePt> redge = edge_rule(o->touch_levels, o->touch_ratio, o->touch_order);
    std::vector<RulePt> rvert = vertex_rule_base(o->touch_levels, o->touch_ratio, o->touch_order);
    std::vector<RulePt> rself = self_rule(redge);
    // far points and weights of every test triangle
    const int nq = (int)rfar.size();
    std::vector<double> tq(size_t(ntri) * NQMAX * 3, 0.0), tw(size_t(ntri) * NQMAX * 3, 0.0);
    for (int t = 0; t < ntri; ++t) {
        const TriGeo& e = tg[t];
        for (int p = 0; p < nq; ++p) {
            const RulePt& m = rfar[p];
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
    for (int t = 0; t < ntri; ++t) tc[t] = cent_of(tg[t]);
    for (int t = 0; t < nwtri; ++t) wc[t] = cent_of(wg[t]);

    DevList dl;
    int r;
    vp_phase_begin(ctx, PH_SETUP);
    TriGeo *d_tg, *d_wg;
    CentF *d_tc, *d_wc;
    double *d_tq, *d_tw, *d_wx = nullptr;
    int* d_fil = nullptr;
    if (wg.empty()) wg.resize(1);
    if ((r = dl.up(ctx, &d_tg, tg)) || (r = dl.up(ctx, &d_wg, wg)) || (r = dl.up(ctx, &d_tc, tc)) ||
        (r = dl.up(ctx, &d_wc, wc)) || (r = dl.up(ctx, &d_tq, tq)) || (r = dl.up(ctx, &d_tw, tw)))
        return r;
    {
        std::vector<double> hwx(wx ? wx : x, (wx ? wx : x) + 3 * std::max(nwnode, 1));
        std::vector<int> hfil(fil && nfil ? fil : tris, (fil && nfil ? fil : tris) + 2 * std::max(nfil, 1));
        if ((r = dl.up(ctx, &d_wx, hwx)) || (r = dl.up(ctx, &d_fil, hfil))) return r;
    }
    RulePt* d_rule[5];
    float4* d_rulef[5];
    {
        const std::vector<RulePt>* R[5] = {&rnear, &rself, &redge, &rvert, &rfar};
        for (int k = 0; k < 5; ++k) {
            std::vector<float4> f(R[k]->size());
            for (size_t i = 0; i < f.size(); ++i)
                f[i] = make_float4(float((*R[k])[i].l0), float((*R[k])[i].l1), float((*R[k])[i].l2), float((*R[k])[i].w));
            if ((r = dl.up(ctx, &d_rule[k], *R[k])) || (r = dl.up(ctx, &d_rulef[k], f))) return r;
        }
    }
    vp_phase_end(ctx);
    // classification of the non-far sources of every test triangle
    vp_phase_begin(ctx, PH_CLASSIFY);
    long long *d_nfptr, *d_wfptr;
    int *d_nf, *d_wf, *d_cnt;
    if ((r = dl.alloc(ctx, &d_cnt, size_t(ntri)))) return r;
    std::vector<long long> nfptr(ntri + 1, 0), wfptr(ntri + 1, 0);
    std::vector<int> cnt(ntri);
    const float ratio32 = float(o->far_ratio);
    classify_kernel<<<ntri, 256, 0, ctx->stream>>>(0, ntri, d_tc, d_tg, ntri, d_tc, d_tg, ratio32, o->far_ratio, d_cnt,
                                                   nullptr, nullptr);
    ctx->launches++;
    VP_CUDA(ctx, vp_d2h(ctx, cnt.data(), d_cnt, sizeof(int) * ntri));
    VP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    for (int t = 0; t < ntri; ++t) nfptr[t + 1] = nfptr[t] + cnt[t];
    if (nwtri > 0) {
        classify_kernel<<<ntri, 256, 0, ctx->stream>>>(0, ntri, d_tc, d_tg, nwtri, d_wc, d_wg, ratio32, o->far_ratio,
                                                       d_cnt, nullptr, nullptr);
        ctx->launches++;
        VP_CUDA(ctx, vp_d2h(ctx, cnt.data(), d_cnt, sizeof(int) * ntri));
        VP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        for (int t = 0; t < ntri; ++t) wfptr[t + 1] = wfptr[t] + cnt[t];
    }
    if ((r = dl.up(ctx, &d_nfptr, nfptr)) || (r = dl.up(ctx, &d_wfptr, wfptr)) ||
        (r = dl.alloc(ctx, &d_nf, size_t(std::max(nfptr[ntri], 1LL)))) ||
        (r = dl.alloc(ctx, &d_wf, size_t(std::max(wfptr[ntri], 1LL)))))
        return r;
    classify_kernel<<<ntri, 256, 0, ctx->stream>>>(1, ntri, d_tc, d_tg, ntri, d_tc, d_tg, ratio32, o->far_ratio,
                                                   nullptr, d_nfptr, d_nf);
    ctx->launches++;
    if (nwtri > 0) {
        classify_kernel<<<ntri, 256, 0, ctx->stream>>>(1, ntri, d_tc, d_tg, nwtri, d_wc, d_wg, ratio32, o->far_ratio,
                                                       nullptr, d_wfptr, d_wf);
        ctx->launches++;
    }
    VP_CUDA(ctx, cudaGetLastError());
    vp_phase_end(ctx);

    // the system
    vp_system* sys = new vp_system();
    sys->nslot = nslot;
    sys->ncols = ncols;
    sys->nwnode = nwnode;
    if ((r = vp_alloc(ctx, &sys->A, size_t(nslot) * ncols)) || (r = vp_alloc(ctx, &sys->b, size_t(nslot)))) {
        vp_system_free(sys);
        return r;
    }
    VP_CUDA(ctx, cudaMemsetAsync(sys->A, 0, sizeof(double) * size_t(nslot) * ncols, ctx->stream));
    VP_CUDA(ctx, cudaMemsetAsync(sys->b, 0, sizeof(double) * nslot, ctx->stream));

    // far tier
    {
        FarArgs fa{};
        fa.ntest = ntri;
        fa.nq = nq;
        fa.test_mode = o->test;
        fa.tq = d_tq;
        fa.tw = d_tw;
        fa.tgeo = d_tg;
        fa.tcent = d_tc;
        fa.nset = nwtri > 0 ? 2 : 1;
        fa.A = sys->A;
        fa.lda = ncols;
        fa.b = sys->b;
        fa.ratio32 = ratio32;
        fa.ratio = o->far_ratio;
        fa.kernel_far = o->kernel_far;
        const std::vector<TriGeo>* sets[2] = {&tg, &wg};
        int nsrc[2] = {ntri, nwtri};
        for (int set = 0; set < fa.nset; ++set) {
            std::vector<TriGeo> g(sets[set]->begin(), sets[set]->begin() + nsrc[set]);
            SrcTiles st = make_src_tiles(g);
            int *d_cols, *d_ncol;
            short *d_cptr, *d_cent;
            if ((r = dl.up(ctx, &d_cols, st.cols)) || (r = dl.up(ctx, &d_ncol, st.ncol)) ||
                (r = dl.up(ctx, &d_cptr, st.cptr)) || (r = dl.up(ctx, &d_cent, st.cent))) {
                vp_system_free(sys);
                return r;
            }
            fa.nsrc[set] = nsrc[set];
            fa.ntile[set] = st.ntile;
            fa.col_off[set] = set == 0 ? 0 : nslot;
            fa.scent[set] = set == 0 ? d_tc : d_wc;
            fa.sgeo[set] = set == 0 ? d_tg : d_wg;
            fa.tile_cols[set] = d_cols;
            fa.tile_ncol[set] = d_ncol;
            fa.tile_cptr[set] = d_cptr;
            fa.tile_cent[set] = d_cent;
            if (mixed) {
                std::vector<float> soa;
                float* d;
                fill_soa(g, soa, fa.pad[set]);
                if ((r = dl.up(ctx, &d, soa))) { vp_system_free(sys); return r; }
                fa.soa[set] = d;
            } else {
                std::vector<double> soa;
                double* d;
                fill_soa(g, soa, fa.pad[set]);
                if ((r = dl.up(ctx, &d, soa))) { vp_system_free(sys); return r; }
                fa.soa[set] = d;
            }
        }
        std::vector<int> cs(corner_slot, corner_slot + 3 * ntri);
        vp_phase_begin(ctx, PH_FAR);
        r = mixed ? run_far<float, 8>(ctx, fa, tg, cs, nslot, dl) : run_far<double, 4>(ctx, fa, tg, cs, nslot, dl);
        vp_phase_end(ctx);
        if (r) { vp_system_free(sys); return r; }
    }

    // near, touching and contact tiers, one launch per colour of test triangles
    unsigned long long* d_stats;
    if ((r = dl.alloc(ctx, &d_stats, 13))) { vp_system_free(sys); return r; }
    VP_CUDA(ctx, cudaMemsetAsync(d_stats, 0, sizeof(unsigned long long) * 13, ctx->stream));
    {
        std::vector<std::vector<int>> groups(ntri);
        for (int t = 0; t < ntri; ++t) groups[t] = {corner_slot[3 * t], corner_slot[3 * t + 1], corner_slot[3 * t + 2]};
        auto colours = colour_groups(groups, nslot);
        std::vector<int> all;
        std::vector<int> off{0};
        for (auto& c : colours) {
            all.insert(all.end(), c.begin(), c.end());
            off.push_back((int)all.size());
        }
        int* d_tests;
        std::vector<long long> keys;
        for (int i = 0; i < ntouch; ++i) {
            long long a0 = touch_pairs[2 * i], b0 = touch_pairs[2 * i + 1];
            keys.push_back(a0 * ntri + b0);
            keys.push_back(b0 * ntri + a0);
        }
        std::sort(keys.begin(), keys.end());
        keys.erase(std::unique(keys.begin(), keys.end()), keys.end());
        if (keys.empty()) keys.push_back(-1);
        long long* d_touch;
        if ((r = dl.up(ctx, &d_tests, all)) || (r = dl.up(ctx, &d_touch, keys))) { vp_system_free(sys); return r; }
        NearArgs na{};
        na.tri = d_tg;
        na.wtri = d_wg;
        na.wx = d_wx;
        na.fil = d_fil;
        na.ntri = ntri;
        na.nwtri = nwtri;
        na.nfil = nfil;
        na.nslot = nslot;
        na.nf_ptr = d_nfptr;
        na.nf_src = d_nf;
        na.wf_ptr = d_wfptr;
        na.wf_src = d_wf;
        na.touch = d_touch;
        na.ntouch = ntouch > 0 ? (int)keys.size() : 0;
        const int nr[5] = {(int)rnear.size(), (int)rself.size(), (int)redge.size(), (int)rvert.size(), (int)rfar.size()};
        for (int k = 0; k < 5; ++k) {
            na.rule[k] = d_rule[k];
            na.rulef[k] = d_rulef[k];
            na.nrule[k] = nr[k];
        }
        na.A = sys->A;
        na.lda = ncols;
        na.b = sys->b;
        na.test_mode = o->test;
        na.near_depth = o->near_depth;
        na.mixed = mixed ? 1 : 0;
        na.far_ratio = o->far_ratio;
        na.near_ratio = o->near_ratio;
        na.corner_angle = o->corner_angle;
        na.contact_rel = o->contact_rel;
        na.kernel_far = o->kernel_far;
        for (int k = 0; k < 3; ++k) {
            na.vinf[k] = vinf[k];
            na.tint[k] = o->test == 1 ? 1.0 : 1.0 / 3;
        }
        na.stats = d_stats;
        int *d_rest, *d_wrest, *d_rcnt;
        if ((r = dl.alloc(ctx, &d_rest, size_t(std::max(nfptr[ntri], 1LL)))) ||
            (r = dl.alloc(ctx, &d_wrest, size_t(std::max(wfptr[ntri], 1LL)))) ||
            (r = dl.alloc(ctx, &d_rcnt, size_t(2) * ntri))) {
            vp_system_free(sys);
            return r;
        }
        na.rest_src = d_rest;
        na.wrest_src = d_wrest;
        na.rest_cnt = d_rcnt;
        vp_phase_begin(ctx, PH_NEAR);
        const size_t near_smem = sizeof(NearChunkSh) * NEAR_WARPS;
        VP_CUDA(ctx, cudaFuncSetAttribute(near_kernel_lanes, cudaFuncAttributeMaxDynamicSharedMemorySize, int(near_smem)));
        for (int pass = 0; pass < 2; ++pass)
            for (size_t c = 0; c < colours.size(); ++c) {
                na.tests = d_tests + off[c];
                na.ntests = off[c + 1] - off[c];
                int nb = (na.ntests + NEAR_WARPS - 1) / NEAR_WARPS;
                if (!nb) continue;
                if (pass == 0)
                    near_kernel_lanes<<<nb, 32 * NEAR_WARPS, near_smem, ctx->stream>>>(na);
                else
                    near_kernel_rest<<<nb, 32 * NEAR_WARPS, 0, ctx->stream>>>(na);
                ctx->launches++;
            }
        vp_phase_end(ctx);
        VP_CUDA(ctx, cudaGetLastError());
    }
    unsigned long long hs[13];
    VP_CUDA(ctx, vp_d2h(ctx, hs, d_stats, sizeof(hs)));
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) {
        vp_system_free(sys);
        return vp_fail(ctx, VP_ERR_CUDA, std::string("assembly kernels: ") + cudaGetErrorString(e));
    }
    if (stats) {
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
        stats->points_fp64 = (long long)hs[12] + (mixed ? 0 : far_tri * nq);
        stats->time_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    }
    *out = sys;
    return VP_OK;
}
