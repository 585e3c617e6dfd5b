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
#include <memory>
#include <numeric>
#include <unordered_map>

#include "vp_pairs.cuh"

namespace {

// ------------------------------------------------------------------------------------------------------------------
// device: the far tier
template <class T, int TT>
__device__ __forceinline__ void far_body(const FarArgs& a, const int tile) {
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

// one system: block b takes test tile a.tiles[b]
template <class T, int TT>
__global__ void __launch_bounds__(FAR_NT) far_kernel(FarArgs a) {
    far_body<T, TT>(a, a.tiles[blockIdx.x]);
}

// a batch of systems in one launch: block b takes test tile work[b].y of system work[b].x
template <class T, int TT>
__global__ void __launch_bounds__(FAR_NT) far_kernel_batch(const FarArgs* __restrict__ sys,
                                                          const int2* __restrict__ work) {
    const int2 wk = work[blockIdx.x];
    far_body<T, TT>(sys[wk.x], wk.y);
}

// ---- the near tier, one pair per lane ---------------------------------------------------------------------------
// A warp takes up to 32 sources of its test triangle at once. Each lane decides its own pair's tier (FP64, exactly as
// pair_rule / wake_pair_rule) and, for a pair in the near tier, walks near_pieces' quadtree to its leaves. The
// warp then evaluates all leaves' points of the 32 pairs together, one point per lane (FP32, guarded; flagged points
// are queued and evaluated 32 at a time in FP64), reduces them per pair in a fixed order and adds the blocks to A
// pair by pair. Pairs of the other tiers are returned (a lane mask) for the warp-cooperative path.
struct NearChunkSh {
    NearPlanSh pl;         // the pairs' leaves and FP32 frames
    double acc[32][9];     // per pair: sum of W psi_a w (FP64 evaluations)
    float accf[32][9];     // per pair: the same sums of the FP32 evaluations
    int off[33];           // points before each pair
    int qp[64], qk[64];    // queued FP64 points: pair, point within the pair
};

// the FP64 evaluation of point k of pair p (queued by the FP32 guard): contributions in v
__device__ void near_point64(const NearArgs& a, const TriGeo& T, const TriGeo& S, const NearChunkSh& ns, int p, int k,
                             double* v) {
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
    int nleaf = 0;
    bool near = near_plan(pc, ns.pl, t, S, s, valid, wake, nleaf);
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
    const Fp32Guard g{PAIR_GUARD};
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
            int code = ns.pl.leaf[p][leaf];
            float b[9];
            leaf_corners32(code, b);
            float4 m = a.rulef[R_NEAR][q];
            float l0 = m.x * b[0] + m.y * b[3] + m.z * b[6];
            float l1 = m.x * b[1] + m.y * b[4] + m.z * b[7];
            float l2 = m.x * b[2] + m.y * b[5] + m.z * b[8];
            float W = m.w * ldexpf(1.f, -2 * (code >> 6)) * areaT;
            const float* E = ns.pl.E32[p];
            const float* Dp = ns.pl.D32[p];
            const float* Sf = ns.pl.S32[p];
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
        if (a.mixed) seg_accumulate<9>(ns.accf, ns.acc, lane, p, vals);  // flagged points add zero here, their FP64 value when drained
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
            seg_accumulate<9>(ns.accf, ns.acc, lane, qpair, qv);
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

// near tier, one pair per lane; the other pairs are listed for near_kernel_pairs. One warp, test triangle t.
__device__ __forceinline__ void near_lanes_body(const NearArgs& a, const int t, NearChunkSh& sh) {
    const int lane = threadIdx.x & 31;
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
            unsigned m = near_chunk(pc, sh, t, src + c0, cnt, wake, col0, rbt, P, Q, Q64);
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

__global__ void __launch_bounds__(32 * NEAR_WARPS) near_kernel_lanes(NearArgs a) {
    extern __shared__ __align__(16) unsigned char near_smem[];
    NearChunkSh* shm = reinterpret_cast<NearChunkSh*>(near_smem);
    const int idx = blockIdx.x * NEAR_WARPS + (threadIdx.x >> 5);
    if (idx >= a.ntests) return;
    near_lanes_body(a, a.tests[idx], shm[threadIdx.x >> 5]);
}

// a batch of systems: warp i takes test triangle work[i].y of system work[i].x
__global__ void __launch_bounds__(32 * NEAR_WARPS) near_kernel_lanes_batch(const NearArgs* __restrict__ sys,
                                                                        const int2* __restrict__ work, int nwork) {
    extern __shared__ __align__(16) unsigned char near_smem[];
    NearChunkSh* shm = reinterpret_cast<NearChunkSh*>(near_smem);
    const int idx = blockIdx.x * NEAR_WARPS + (threadIdx.x >> 5);
    if (idx >= nwork) return;
    const int2 wk = work[idx];
    near_lanes_body(sys[wk.x], wk.y, shm[threadIdx.x >> 5]);
}

// the block of one pair: the per-lane sums reduced and contracted with n_T x gamma_b (9 values, row-major), and the
// source part of the right hand side sigma_S (P_a . n_T) (3 values, subtracted when the pair is added)
__device__ void pair_block_out(PairCtx& pc, FwdAcc& acc, const TriGeo& S, double* out, bool with_rhs) {
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
        out[pc.lane] = P[3 * ai] * m.x + P[3 * ai + 1] * m.y + P[3 * ai + 2] * m.z;
    } else if (pc.lane < 12) {
        int ai = pc.lane - 9;
        out[pc.lane] = with_rhs ? S.sigma * (P[3 * ai] * nT.x + P[3 * ai + 1] * nT.y + P[3 * ai + 2] * nT.z) : 0.0;
    }
    __syncwarp();
}

// the self, touching and contact pairs, one warp per pair: a persistent grid whose warps take the next pair of the
// list from a counter, so that test triangles with many contact pairs (thin panels at a sharp trailing edge) do not
// hold a launch; the blocks go to pair_out and near_kernel_rest adds them in the list's order
// rest pair idx of system a: its block to a.pair_out, its tier and points counted in P, Q, Q64
__device__ __forceinline__ void near_pair_item(const NearArgs& a, PairCtx& pc, const long long idx,
                                               unsigned long long* P, unsigned long long* Q,
                                               unsigned long long& Q64) {
        const int lane = pc.lane;
        const int n = 2 * a.ntri;
        const int g = rest_entry(a.rest_off, n, idx);
        const int t = g >> 1;
        const bool wake = (g & 1) != 0;
        const long long e0 = wake ? a.wf_ptr[t] : a.nf_ptr[t];
        const int s = (wake ? a.wrest_src : a.rest_src)[e0 + (idx - a.rest_off[g])];
        pc.T = &a.tri[t];
        FwdAcc acc = {};
        pc.kind = 0;
        pc.npts = 0;
        pc.n64 = 0;
        pc.nleaf = 0;
        pc.nq64 = 0;
        const int tier = tri_pair(pc, acc, t, s, wake);
        pair_block_out(pc, acc, wake ? a.wtri[s] : a.tri[s], a.pair_out + 12 * idx, !wake);
        P[tier] += 1;
        Q[tier] += pc.npts;
        Q64 += pc.n64;
        (void)lane;
}

__global__ void __launch_bounds__(32 * NEAR_WARPS, 3) near_kernel_pairs(NearArgs a) {
    __shared__ WarpSh shm[NEAR_WARPS];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long total = a.rest_off[2 * a.ntri];
    PairCtx pc;
    pc.a = &a;
    pc.sh = &shm[w];
    pc.lane = lane;
    unsigned long long P[6] = {0, 0, 0, 0, 0, 0}, Q[6] = {0, 0, 0, 0, 0, 0}, Q64 = 0;
    for (;;) {
        const long long idx = next_rest_pair(a.next, lane);
        if (idx >= total) break;
        near_pair_item(a, pc, idx, P, Q, Q64);
    }
    if (lane == 0) {
        for (int k = 0; k < 6; ++k) {
            if (P[k]) atomicAdd(a.stats + k, P[k]);
            if (Q[k]) atomicAdd(a.stats + 6 + k, Q[k]);
        }
        if (Q64) atomicAdd(a.stats + 12, Q64);
    }
}

// a batch of systems in one persistent launch: the systems' rest pairs in one index space (system k's pairs at
// base[k] .. base[k + 1]), taken from one counter; each pair's counts go to its own system's statistics
__global__ void __launch_bounds__(32 * NEAR_WARPS, 3) near_kernel_pairs_batch(const NearArgs* __restrict__ sys, int nsys,
                                                                           const long long* __restrict__ base,
                                                                           unsigned long long* next) {
    __shared__ WarpSh shm[NEAR_WARPS];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long total = base[nsys];
    PairCtx pc;
    pc.sh = &shm[w];
    pc.lane = lane;
    for (;;) {
        const long long idx = next_rest_pair(next, lane);
        if (idx >= total) break;
        int lo = 0, hi = nsys - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (base[mid] <= idx) lo = mid;
            else hi = mid - 1;
        }
        const NearArgs& a = sys[lo];
        pc.a = &a;
        unsigned long long P[6] = {0, 0, 0, 0, 0, 0}, Q[6] = {0, 0, 0, 0, 0, 0}, Q64 = 0;
        near_pair_item(a, pc, idx - base[lo], P, Q, Q64);
        if (lane == 0) {
            for (int k = 0; k < 6; ++k) {
                if (P[k]) atomicAdd(a.stats + k, P[k]);
                if (Q[k]) atomicAdd(a.stats + 6 + k, Q[k]);
            }
            if (Q64) atomicAdd(a.stats + 12, Q64);
        }
    }
}

// one far tip filament of test triangle T, summed by one lane: segment_block (assemble.jl:312-321) with the far rule
// (the columns of the filament's two end nodes, ca and cb, per test function)
__device__ void far_filament_fwd(const NearArgs& a, const TriGeo& T, v3<double> fa, v3<double> fb, double* ca,
                                 double* cb) {
    const RulePt* R = a.rule[R_FAR];
    const v3<double> n = ld3(T.n);
    v3<double> Ea[3], Eb[3];
    for (int k = 0; k < 3; ++k) {
        Ea[k] = ld3(T.x + 3 * k) - fa;
        Eb[k] = ld3(T.x + 3 * k) - fb;
    }
    for (int i = 0; i < a.nrule[R_FAR]; ++i) {
        const RulePt m = R[i];
        const double W = m.w * T.area;
        const v3<double> ra = m.l0 * Ea[0] + m.l1 * Ea[1] + m.l2 * Ea[2];
        const v3<double> rb = m.l0 * Eb[0] + m.l1 * Eb[1] + m.l2 * Eb[2];
        v3<double> va, vb;
        segment_velocity(ra, rb, va, vb);
        const v3<double> psi = test_weights(a.test_mode, m.l0, m.l1, m.l2);
        const double da = dot(va, n) * W, db = dot(vb, n) * W;
        ca[0] += da * psi.x;
        ca[1] += da * psi.y;
        ca[2] += da * psi.z;
        cb[0] += db * psi.x;
        cb[1] += db * psi.y;
        cb[2] += db * psi.z;
    }
}

// the blocks of the self, touching and contact pairs (from near_kernel_pairs, added in the order of the test
// triangle's list), the tip filaments and the freestream: one warp per test triangle, a launch per colour
__device__ __forceinline__ void near_rest_body(const NearArgs& a, const int t, WarpSh& wsh) {
    const int lane = threadIdx.x & 31;
    const TriGeo& T = a.tri[t];
    PairCtx pc;
    pc.a = &a;
    pc.T = &T;
    pc.sh = &wsh;
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
        const double* blk = a.pair_out + 12 * a.rest_off[2 * t + set];
        for (int e = 0; e < n; ++e) {
            const TriGeo& S = wake ? a.wtri[rest[e0 + e]] : a.tri[rest[e0 + e]];
            const double* pb = blk + 12 * e;
            if (lane < 9) {
                double* dst = a.A + size_t(T.slot[lane / 3]) * size_t(a.lda) + col0 + S.slot[lane % 3];
                *dst += pb[lane];
            }
            if (!wake)
                for (int ai = 0; ai < 3; ++ai) rbt[ai] -= pb[9 + ai];
            __syncwarp();
        }
    }
    // tip filaments (assemble.jl:344-354): segment_rule (:299-306) and segment_block (:312-321), FP64. A warp takes 32
    // filaments at once: a far one (the far rule's few points) is summed by its own lane, the others by the whole
    // warp; the columns are added in the filaments' order.
    for (int f0 = 0; f0 < a.nfil; f0 += 32) {
        const int cnt = a.nfil - f0 < 32 ? a.nfil - f0 : 32;
        int mia = 0, mib = 0;
        double mca[3] = {0, 0, 0}, mcb[3] = {0, 0, 0};
        bool mfar = false;
        if (lane < cnt) {
            mia = a.fil[2 * (f0 + lane)];
            mib = a.fil[2 * (f0 + lane) + 1];
            const v3<double> fa = ld3(a.wx + 3 * mia), fb = ld3(a.wx + 3 * mib);
            mfar = vnorm((fa + fb) / 2.0 - ld3(T.c)) > a.far_ratio * fmax(T.diam, vnorm(fb - fa));
            if (mfar) far_filament_fwd(a, T, fa, fb, mca, mcb);
        }
        const unsigned farmask = __ballot_sync(0xffffffffu, mfar);
        for (int q = 0; q < cnt; ++q) {
            const int ia = __shfl_sync(0xffffffffu, mia, q), ib = __shfl_sync(0xffffffffu, mib, q);
            if ((farmask >> q) & 1u) {
                double ca[3], cb[3];
                for (int k = 0; k < 3; ++k) {
                    ca[k] = __shfl_sync(0xffffffffu, mca[k], q);
                    cb[k] = __shfl_sync(0xffffffffu, mcb[k], q);
                }
                if (lane < 3) {
                    double* row = a.A + size_t(T.slot[lane]) * size_t(a.lda) + a.nslot;
                    row[ia] += lane == 0 ? ca[0] : (lane == 1 ? ca[1] : ca[2]);
                    __syncwarp(0x7u);
                    row[ib] += lane == 0 ? cb[0] : (lane == 1 ? cb[1] : cb[2]);
                }
                __syncwarp();
                P[TIER_FAR] += 1;
                Q[TIER_FAR] += a.nrule[R_FAR];
                continue;
            }
            // near and vertex filaments (segment_rule, assemble.jl:299-306), the whole warp
            const v3<double> fa = ld3(a.wx + 3 * ia), fb = ld3(a.wx + 3 * ib);
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

__global__ void __launch_bounds__(32 * NEAR_WARPS, 3) near_kernel_rest(NearArgs a) {
    __shared__ WarpSh shm[NEAR_WARPS];
    const int idx = blockIdx.x * NEAR_WARPS + (threadIdx.x >> 5);
    if (idx >= a.ntests) return;
    near_rest_body(a, a.tests[idx], shm[threadIdx.x >> 5]);
}

__global__ void __launch_bounds__(32 * NEAR_WARPS, 3) near_kernel_rest_batch(const NearArgs* __restrict__ sys,
                                                                          const int2* __restrict__ work, int nwork) {
    __shared__ WarpSh shm[NEAR_WARPS];
    const int idx = blockIdx.x * NEAR_WARPS + (threadIdx.x >> 5);
    if (idx >= nwork) return;
    const int2 wk = work[idx];
    near_rest_body(sys[wk.x], wk.y, shm[threadIdx.x >> 5]);
}

// ------------------------------------------------------------------------------------------------------------------
// host: one system's assembly, prepared (classification, pair lists, far tiles and their colours, near colours) and
// then launched; a batch prepares every system and launches each phase once over all of them

// the far tier's test tiles of TT triangles: their unique row slots, uploaded; the tiles grouped by colour (no two
// tiles of a colour share a row slot)
template <int TT>
int far_prepare(vp_ctx* ctx, FarArgs& fa, int nt, const int* cslot, int nslot, DevList& dl,
                std::vector<std::vector<int>>& colours) {
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
    colours = colour_groups(groups, nslot);
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
    return VP_OK;
}

// one system of an assembly between its phases
struct AsmJob {
    PairInput in;
    int tt = 8;  // test triangles per far tile
    PairSetup ps;
    vp_system* sys = nullptr;
    FarArgs fa{};
    std::vector<std::vector<int>> far_col;   // far test tiles, per colour
    std::vector<std::vector<int>> near_col;  // test triangles, per colour
    NearArgs na{};
    unsigned long long* d_stats = nullptr;
    long long nrest = 0;
    std::chrono::steady_clock::time_point t0;
    ~AsmJob() {
        if (sys) vp_system_free(sys);
    }
};

// classification, pair lists, the zeroed system, the far tier's source tiles and arrays, its test tiles and their
// colours, the near tier's colours and arguments
int job_prepare(vp_ctx* ctx, AsmJob& j) {
    j.t0 = std::chrono::steady_clock::now();
    const PairInput& in = j.in;
    const vp_assembly_options* o = in.o;
    int r = setup_pairs(ctx, in, PH_SETUP, PH_CLASSIFY, j.ps);
    if (r) return r;
    PairSetup& ps = j.ps;
    DevList& dl = ps.dl;
    const int ntri = in.ntri, nslot = in.nslot, nwtri = in.nwtri, ncols = ps.ncols;
    vp_system* sys = new vp_system();
    j.sys = sys;
    sys->nslot = nslot;
    sys->ncols = ncols;
    sys->nwnode = in.nwnode;
    if ((r = vp_alloc(ctx, &sys->A, size_t(nslot) * ncols)) || (r = vp_alloc(ctx, &sys->b, size_t(nslot)))) return r;
    VP_CUDA(ctx, cudaMemsetAsync(sys->A, 0, sizeof(double) * size_t(nslot) * ncols, ctx->stream));
    VP_CUDA(ctx, cudaMemsetAsync(sys->b, 0, sizeof(double) * nslot, ctx->stream));
    // far tier
    FarArgs& fa = j.fa;
    fa.ntest = ntri;
    fa.nq = ps.nq;
    fa.test_mode = o->test;
    fa.tq = ps.d_tq;
    fa.tw = ps.d_tw;
    fa.tgeo = ps.d_tg;
    fa.tcent = ps.d_tc;
    fa.nset = nwtri > 0 ? 2 : 1;
    fa.A = sys->A;
    fa.lda = ncols;
    fa.b = sys->b;
    fa.ratio32 = ps.ratio32;
    fa.ratio = o->far_ratio;
    fa.kernel_far = o->kernel_far;
    const std::vector<TriGeo>* sets[2] = {&ps.tg, &ps.wg};
    int nsrc[2] = {in.body_sources ? ntri : 0, nwtri};
    for (int set = 0; set < fa.nset; ++set) {
        std::vector<TriGeo> g(sets[set]->begin(), sets[set]->begin() + nsrc[set]);
        SrcTiles st = make_src_tiles(g);
        int *d_cols, *d_ncol;
        short *d_cptr, *d_cent;
        if ((r = dl.up(ctx, &d_cols, st.cols)) || (r = dl.up(ctx, &d_ncol, st.ncol)) ||
            (r = dl.up(ctx, &d_cptr, st.cptr)) || (r = dl.up(ctx, &d_cent, st.cent)))
            return r;
        fa.nsrc[set] = nsrc[set];
        fa.ntile[set] = st.ntile;
        fa.col_off[set] = set == 0 ? 0 : nslot;
        fa.scent[set] = set == 0 ? ps.d_tc : ps.d_wc;
        fa.sgeo[set] = set == 0 ? ps.d_tg : ps.d_wg;
        fa.tile_cols[set] = d_cols;
        fa.tile_ncol[set] = d_ncol;
        fa.tile_cptr[set] = d_cptr;
        fa.tile_cent[set] = d_cent;
        if (ps.mixed) {
            std::vector<float> soa;
            float* d;
            fill_soa(g, soa, fa.pad[set]);
            if ((r = dl.up(ctx, &d, soa))) return r;
            fa.soa[set] = d;
        } else {
            std::vector<double> soa;
            double* d;
            fill_soa(g, soa, fa.pad[set]);
            if ((r = dl.up(ctx, &d, soa))) return r;
            fa.soa[set] = d;
        }
    }
    j.tt = ctx->far_tile[ps.mixed ? 1 : 0];
    switch (j.tt) {
        case 1: r = far_prepare<1>(ctx, fa, ntri, in.corner_slot, nslot, dl, j.far_col); break;
        case 2: r = far_prepare<2>(ctx, fa, ntri, in.corner_slot, nslot, dl, j.far_col); break;
        case 4: r = far_prepare<4>(ctx, fa, ntri, in.corner_slot, nslot, dl, j.far_col); break;
        case 8: r = far_prepare<8>(ctx, fa, ntri, in.corner_slot, nslot, dl, j.far_col); break;
        default: return vp_fail(ctx, VP_ERR_ARG, "far tile must be 1, 2, 4 or 8 test triangles");
    }
    if (r) return r;
    // near, touching and contact tiers
    if ((r = dl.alloc(ctx, &j.d_stats, 13))) return r;
    VP_CUDA(ctx, cudaMemsetAsync(j.d_stats, 0, sizeof(unsigned long long) * 13, ctx->stream));
    std::vector<std::vector<int>> groups(ntri);
    for (int t = 0; t < ntri; ++t)
        groups[t] = {in.corner_slot[3 * t], in.corner_slot[3 * t + 1], in.corner_slot[3 * t + 2]};
    j.near_col = colour_groups(groups, nslot);
    j.na = near_args(ps, in);
    j.na.A = sys->A;
    j.na.b = sys->b;
    j.na.stats = j.d_stats;
    int *d_rest, *d_wrest, *d_rcnt;
    if ((r = dl.alloc(ctx, &d_rest, size_t(std::max(ps.nfptr[ntri], 1LL)))) ||
        (r = dl.alloc(ctx, &d_wrest, size_t(std::max(ps.wfptr[ntri], 1LL)))) ||
        (r = dl.alloc(ctx, &d_rcnt, size_t(2) * ntri)))
        return r;
    j.na.rest_src = d_rest;
    j.na.wrest_src = d_wrest;
    j.na.rest_cnt = d_rcnt;
    return VP_OK;
}

// the statistics and the system of a finished job (the stream is synchronised)
int job_finish(vp_ctx* ctx, AsmJob& j, vp_system** out, vp_assembly_stats* stats) {
    unsigned long long hs[13];
    VP_CUDA(ctx, vp_d2h(ctx, hs, j.d_stats, sizeof(hs)));
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return vp_fail(ctx, VP_ERR_CUDA, std::string("assembly kernels: ") + cudaGetErrorString(e));
    if (stats) {
        const PairInput& in = j.in;
        long long total = (long long)in.ntri * (in.ntri + in.nwtri) + (long long)in.ntri * in.nfil;
        long long nonfar = 0;
        for (int k = 0; k < 6; ++k) {
            stats->pairs[k] = (long long)hs[k];
            stats->points[k] = (long long)hs[6 + k];
            if (k != TIER_FAR) nonfar += (long long)hs[k];
        }
        long long far_fil = (long long)hs[TIER_FAR];
        long long far_tri = total - nonfar - far_fil;
        stats->pairs[TIER_FAR] = far_tri + far_fil;
        stats->points[TIER_FAR] = (long long)hs[6 + TIER_FAR] + far_tri * j.ps.nq;
        stats->points_fp64 = (long long)hs[12] + (j.ps.mixed ? 0 : far_tri * j.ps.nq);
        stats->time_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - j.t0).count();
    }
    *out = j.sys;
    j.sys = nullptr;
    return VP_OK;
}

// one system: the far tiles of a colour per launch
template <class T, int TT>
int far_launch(vp_ctx* ctx, AsmJob& j) {
    std::vector<int> all;
    std::vector<int> off{0};
    for (auto& c : j.far_col) {
        all.insert(all.end(), c.begin(), c.end());
        off.push_back((int)all.size());
    }
    int* d_tiles;
    int r;
    if ((r = j.ps.dl.up(ctx, &d_tiles, all))) return r;
    FarArgs fa = j.fa;
    vp_phase_begin(ctx, PH_FAR);
    for (size_t c = 0; c < j.far_col.size(); ++c) {
        fa.tiles = d_tiles + off[c];
        int nb = off[c + 1] - off[c];
        if (nb) {
            far_kernel<T, TT><<<nb, FAR_NT, 0, ctx->stream>>>(fa);
            ctx->launches++;
        }
    }
    vp_phase_end(ctx);
    VP_CUDA(ctx, cudaGetLastError());
    return VP_OK;
}

// a batch: colour c's far tiles of every system in one launch
template <class T, int TT>
int far_launch_batch(vp_ctx* ctx, std::vector<std::unique_ptr<AsmJob>>& jobs, DevList& dl) {
    std::vector<FarArgs> args;
    size_t ncol = 0;
    for (auto& j : jobs) {
        args.push_back(j->fa);
        ncol = std::max(ncol, j->far_col.size());
    }
    FarArgs* d_args;
    int r;
    if ((r = dl.up(ctx, &d_args, args))) return r;
    vp_phase_begin(ctx, PH_FAR);
    for (size_t c = 0; c < ncol; ++c) {
        std::vector<int2> work;
        for (size_t k = 0; k < jobs.size(); ++k)
            if (c < jobs[k]->far_col.size())
                for (int tile : jobs[k]->far_col[c]) work.push_back(make_int2(int(k), tile));
        if (work.empty()) continue;
        int2* d_work;
        if ((r = dl.up(ctx, &d_work, work))) return r;
        far_kernel_batch<T, TT><<<int(work.size()), FAR_NT, 0, ctx->stream>>>(d_args, d_work);
        ctx->launches++;
    }
    vp_phase_end(ctx);
    VP_CUDA(ctx, cudaGetLastError());
    return VP_OK;
}

// one system: the near tier's lanes per colour, the rest pairs' list, the persistent pair kernel, the rest per colour
int near_launch(vp_ctx* ctx, AsmJob& j) {
    DevList& dl = j.ps.dl;
    NearArgs& na = j.na;
    std::vector<int> all;
    std::vector<int> off{0};
    for (auto& c : j.near_col) {
        all.insert(all.end(), c.begin(), c.end());
        off.push_back((int)all.size());
    }
    int* d_tests;
    int r;
    if ((r = dl.up(ctx, &d_tests, all))) return r;
    vp_phase_begin(ctx, PH_NEAR);
    const size_t near_smem = sizeof(NearChunkSh) * NEAR_WARPS;
    VP_CUDA(ctx, cudaFuncSetAttribute(near_kernel_lanes, cudaFuncAttributeMaxDynamicSharedMemorySize, int(near_smem)));
    for (int pass = 0; pass < 2; ++pass) {
        if (pass == 1) {
            // the rest pairs as one list, evaluated pair-parallel into per-pair blocks
            long long nrest = 0;
            double* d_pairs;
            if ((r = rest_list(ctx, dl, na, &nrest)) ||
                (r = dl.alloc(ctx, &d_pairs, size_t(12) * size_t(std::max(nrest, 1LL)))))
                return r;
            na.pair_out = d_pairs;
            if (nrest > 0) {
                const int nb = persistent_blocks(ctx, near_kernel_pairs, 32 * NEAR_WARPS, 0);
                vp_phase_end(ctx);
                vp_phase_begin(ctx, PH_NEAR_PAIRS);
                near_kernel_pairs<<<nb, 32 * NEAR_WARPS, 0, ctx->stream>>>(na);
                vp_phase_end(ctx);
                vp_phase_begin(ctx, PH_NEAR);
                ctx->launches++;
            }
        }
        for (size_t c = 0; c < j.near_col.size(); ++c) {
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
    }
    vp_phase_end(ctx);
    VP_CUDA(ctx, cudaGetLastError());
    return VP_OK;
}

// a batch: the lanes kernel per colour over every system, every system's rest list, one persistent launch of the
// pair kernel over all of them, the rest kernel per colour over every system
int near_launch_batch(vp_ctx* ctx, std::vector<std::unique_ptr<AsmJob>>& jobs, DevList& dl) {
    int r;
    const int nsys = int(jobs.size());
    size_t ncol = 0;
    for (auto& j : jobs) ncol = std::max(ncol, j->near_col.size());
    auto colour_work = [&](size_t c) {
        std::vector<int2> work;
        for (int k = 0; k < nsys; ++k)
            if (c < jobs[k]->near_col.size())
                for (int t : jobs[k]->near_col[c]) work.push_back(make_int2(k, t));
        return work;
    };
    auto upload_args = [&](NearArgs** d) {
        std::vector<NearArgs> args;
        for (auto& j : jobs) args.push_back(j->na);
        return dl.up(ctx, d, args);
    };
    NearArgs* d_args;
    if ((r = upload_args(&d_args))) return r;
    vp_phase_begin(ctx, PH_NEAR);
    const size_t near_smem = sizeof(NearChunkSh) * NEAR_WARPS;
    VP_CUDA(ctx, cudaFuncSetAttribute(near_kernel_lanes_batch, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      int(near_smem)));
    for (size_t c = 0; c < ncol; ++c) {
        std::vector<int2> work = colour_work(c);
        if (work.empty()) continue;
        int2* d_work;
        if ((r = dl.up(ctx, &d_work, work))) return r;
        const int n = int(work.size());
        near_kernel_lanes_batch<<<(n + NEAR_WARPS - 1) / NEAR_WARPS, 32 * NEAR_WARPS, near_smem, ctx->stream>>>(
            d_args, d_work, n);
        ctx->launches++;
    }
    // every system's rest list and block buffer; their pairs in one index space
    std::vector<long long> base{0};
    for (auto& j : jobs) {
        if ((r = rest_list(ctx, j->ps.dl, j->na, &j->nrest))) return r;
        double* d_pairs;
        if ((r = j->ps.dl.alloc(ctx, &d_pairs, size_t(12) * size_t(std::max(j->nrest, 1LL))))) return r;
        j->na.pair_out = d_pairs;
        base.push_back(base.back() + j->nrest);
    }
    if ((r = upload_args(&d_args))) return r;
    if (base.back() > 0) {
        long long* d_base;
        unsigned long long* d_next;
        if ((r = dl.up(ctx, &d_base, base)) || (r = dl.alloc(ctx, &d_next, 1))) return r;
        VP_CUDA(ctx, cudaMemsetAsync(d_next, 0, sizeof(unsigned long long), ctx->stream));
        const int nb = persistent_blocks(ctx, near_kernel_pairs_batch, 32 * NEAR_WARPS, 0);
        vp_phase_end(ctx);
        vp_phase_begin(ctx, PH_NEAR_PAIRS);
        near_kernel_pairs_batch<<<nb, 32 * NEAR_WARPS, 0, ctx->stream>>>(d_args, nsys, d_base, d_next);
        vp_phase_end(ctx);
        vp_phase_begin(ctx, PH_NEAR);
        ctx->launches++;
    }
    for (size_t c = 0; c < ncol; ++c) {
        std::vector<int2> work = colour_work(c);
        if (work.empty()) continue;
        int2* d_work;
        if ((r = dl.up(ctx, &d_work, work))) return r;
        const int n = int(work.size());
        near_kernel_rest_batch<<<(n + NEAR_WARPS - 1) / NEAR_WARPS, 32 * NEAR_WARPS, 0, ctx->stream>>>(d_args, d_work,
                                                                                                      n);
        ctx->launches++;
    }
    vp_phase_end(ctx);
    VP_CUDA(ctx, cudaGetLastError());
    return VP_OK;
}

// the far launches of the job's precision and tile (FP64: 1, 2 or 4 test triangles per tile, mixed: 2, 4 or 8)
int far_dispatch(vp_ctx* ctx, AsmJob& j) {
    if (j.ps.mixed) {
        if (j.tt == 2) return far_launch<float, 2>(ctx, j);
        if (j.tt == 4) return far_launch<float, 4>(ctx, j);
        if (j.tt == 8) return far_launch<float, 8>(ctx, j);
    } else {
        if (j.tt == 1) return far_launch<double, 1>(ctx, j);
        if (j.tt == 2) return far_launch<double, 2>(ctx, j);
        if (j.tt == 4) return far_launch<double, 4>(ctx, j);
    }
    return vp_fail(ctx, VP_ERR_ARG, "far tile not built for this precision");
}
int far_dispatch_batch(vp_ctx* ctx, std::vector<std::unique_ptr<AsmJob>>& jobs, DevList& dl) {
    const bool mixed = jobs[0]->ps.mixed;
    const int tt = jobs[0]->tt;
    for (auto& j : jobs)
        if (j->ps.mixed != mixed) return vp_fail(ctx, VP_ERR_ARG, "one precision for the whole batch");
    if (mixed) {
        if (tt == 2) return far_launch_batch<float, 2>(ctx, jobs, dl);
        if (tt == 4) return far_launch_batch<float, 4>(ctx, jobs, dl);
        if (tt == 8) return far_launch_batch<float, 8>(ctx, jobs, dl);
    } else {
        if (tt == 1) return far_launch_batch<double, 1>(ctx, jobs, dl);
        if (tt == 2) return far_launch_batch<double, 2>(ctx, jobs, dl);
        if (tt == 4) return far_launch_batch<double, 4>(ctx, jobs, dl);
    }
    return vp_fail(ctx, VP_ERR_ARG, "far tile not built for this precision");
}

}  // namespace

// body_sources = 0: the columns of the wake's sheets and filaments alone (explicit_rhs); A's body columns stay zero
int vp_assemble_impl(vp_ctx* ctx, const vp_assembly_options* o, int nnode, const double* x, int ntri, const int* tris,
                     const int* corner_slot, int nslot, int ntouch, const int* touch_pairs, const double* sigma,
                     const double* vinf, int nwnode, const double* wx, int nwtri, const int* wtris, int nfil,
                     const int* fil, vp_system** out, vp_assembly_stats* stats, int body_sources) {
    if (!out) return vp_fail(ctx, VP_ERR_ARG, "null argument");
    *out = nullptr;
    AsmJob j;
    j.in = PairInput{o,     nnode, x,     ntri, tris,  corner_slot, nslot, ntouch, touch_pairs,
                     sigma, vinf,  nwnode, wx,  nwtri, wtris,       nfil,  fil,   body_sources != 0};
    int r;
    if ((r = job_prepare(ctx, j)) || (r = far_dispatch(ctx, j)) || (r = near_launch(ctx, j))) return r;
    return job_finish(ctx, j, out, stats);
}

// the batch: every system prepared, then each phase launched once over all of them (one precision for all)
int vp_assemble_batch_impl(vp_ctx* ctx, const vp_assembly_options* o, int nsys, const vp_assembly_input* in,
                           vp_system** out, vp_assembly_stats* stats) {
    if (!out || !in || !o || nsys < 1) return vp_fail(ctx, VP_ERR_ARG, "null argument or empty batch");
    for (int k = 0; k < nsys; ++k) out[k] = nullptr;
    std::vector<std::unique_ptr<AsmJob>> jobs;
    DevList dl;
    int r;
    for (int k = 0; k < nsys; ++k) {
        const vp_assembly_input& w = in[k];
        jobs.emplace_back(new AsmJob());
        jobs.back()->in = PairInput{o,       w.nnode,  w.x,      w.ntri,  w.tris, w.corner_slot, w.nslot,
                                    w.ntouch, w.touch_pairs, w.sigma, w.vinf, w.nwnode, w.wx, w.nwtri,
                                    w.wtris, w.nfil,   w.fil,    true};
        if ((r = job_prepare(ctx, *jobs.back()))) return r;
    }
    if ((r = far_dispatch_batch(ctx, jobs, dl)) || (r = near_launch_batch(ctx, jobs, dl))) return r;
    for (int k = 0; k < nsys; ++k)
        if ((r = job_finish(ctx, *jobs[k], &out[k], stats ? stats + k : nullptr))) {
            for (int i = 0; i < k; ++i) {
                vp_system_free(out[i]);
                out[i] = nullptr;
            }
            return r;
        }
    return VP_OK;
}
