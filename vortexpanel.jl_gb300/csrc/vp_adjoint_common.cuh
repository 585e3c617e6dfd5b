// Per-pair pieces of the adjoint: the sums a pair's quadrature points leave, and their conversion into derivatives
// with respect to the source triangle's corners (the chain rule through its edge normals, edge lengths, unit normal,
// corner offsets from the centroid and area, as the forward kernel builds them: SourceTriangle,
// src/kernels/source_triangle.jl:8-26).
#pragma once
#include "vp_adjoint.cuh"

// Sums over a pair's points of W nu(q) times: w (Q); lambda_k ds/dx (Xg); ds/dr_a at fixed shape (Gr, exact form);
// the edge logs (L), dL_e/dlen_e (N) and the solid angle (O) of the exact form; ds/dr (Grf), ds/dd_a (Gd) and
// ds/darea (A) of the multipole form.
// adjoint vectors one pass carries at most (the loops over them unroll, so that per-vector sums stay in registers)
constexpr int ADJ_VEC_MAX = 2;

template <class T>
struct AdjSums {
    v3<T> Q, Xg[3], Gr[3], Grf, Gd[3];
    T L[3], N[3], O, A;
};

template <class T>
__device__ __forceinline__ void adj_zero(AdjSums<T>& s) {
    v3<T> z = mk3(T(0), T(0), T(0));
    s.Q = z;
    s.Grf = z;
    for (int k = 0; k < 3; ++k) {
        s.Xg[k] = z;
        s.Gr[k] = z;
        s.Gd[k] = z;
        s.L[k] = T(0);
        s.N[k] = T(0);
    }
    s.O = T(0);
    s.A = T(0);
}

// add one point: weight Wn = W nu(q), barycentrics l, offsets r_a (exact) or r (multipole), direction m. Returns
// s = w·m; *gxo (if given) receives ds/dx.
template <class T>
__device__ __forceinline__ T adj_point_exact(AdjSums<T>& acc, const SrcKern<T>& S, T Wn, T l0, T l1, T l2, v3<T> r0,
                                             v3<T> r1, v3<T> r2, v3<T> r, v3<T> m, int side, T plane_tol,
                                             v3<T>* gxo = nullptr) {
    v3<T> g0, g1, g2;
    ExactShape<T> sh;
    T sv = sv_exact_vjp(S, r0, r1, r2, r, m, side, plane_tol, g0, g1, g2, sh);
    const T i4pi = T(1) / (T(4) * vp_pi<T>());
    v3<T> w = (sh.L[0] * S.nu[0] + sh.L[1] * S.nu[1] + sh.L[2] * S.nu[2] + sh.Om * S.n) * i4pi;
    acc.Q += Wn * w;
    v3<T> gx = g0 + g1 + g2;
    acc.Xg[0] += (Wn * l0) * gx;
    acc.Xg[1] += (Wn * l1) * gx;
    acc.Xg[2] += (Wn * l2) * gx;
    acc.Gr[0] += Wn * g0;
    acc.Gr[1] += Wn * g1;
    acc.Gr[2] += Wn * g2;
    for (int e = 0; e < 3; ++e) {
        acc.L[e] += Wn * sh.L[e];
        acc.N[e] += Wn * sh.dLdlen[e];
    }
    acc.O += Wn * sh.Om;
    if (gxo) *gxo = gx;
    return sv;
}

template <class T>
__device__ __forceinline__ T adj_point_far(AdjSums<T>& acc, const SrcKern<T>& S, T Wn, T l0, T l1, T l2, v3<T> r,
                                           v3<T> m, v3<T>* gxo = nullptr) {
    v3<T> gr, gd[3];
    T ga;
    T sv = sv_far_vjp(S, r, m, gr, gd, ga);
    acc.Q += Wn * sv_far(S, r);
    acc.Xg[0] += (Wn * l0) * gr;
    acc.Xg[1] += (Wn * l1) * gr;
    acc.Xg[2] += (Wn * l2) * gr;
    acc.Grf += Wn * gr;
    for (int a = 0; a < 3; ++a) acc.Gd[a] += Wn * gd[a];
    acc.A += Wn * ga;
    if (gxo) *gxo = gr;
    return sv;
}

// the sums of one exact-kernel point for nk adjoint vectors (weights Wn[k]): velocity w, ds/dx gx, ds/dr_a g_a, the
// edge logs L, their length derivatives dL and the solid angle Om. The sums may be of a narrower type than the point.
template <class T>
__device__ __forceinline__ void adj_acc_exact(AdjSums<T>* acc, int nk, const T* Wn, T l0, T l1, T l2, v3<T> w,
                                              v3<T> gx, v3<T> g0, v3<T> g1, v3<T> g2, const T* L, const T* dL, T Om) {
#pragma unroll
    for (int k = 0; k < ADJ_VEC_MAX; ++k) {
        if (k >= nk) break;
        AdjSums<T>& a = acc[k];
        const T wn = Wn[k];
        a.Q += wn * w;
        a.Xg[0] += (wn * l0) * gx;
        a.Xg[1] += (wn * l1) * gx;
        a.Xg[2] += (wn * l2) * gx;
        a.Gr[0] += wn * g0;
        a.Gr[1] += wn * g1;
        a.Gr[2] += wn * g2;
        for (int e = 0; e < 3; ++e) {
            a.L[e] += wn * L[e];
            a.N[e] += wn * dL[e];
        }
        a.O += wn * Om;
    }
}

// the sums of one multipole point: velocity w, ds/dr gx, ds/d(second moments) gd, ds/d(area) ga
template <class T>
__device__ __forceinline__ void adj_acc_far(AdjSums<T>* acc, int nk, const T* Wn, T l0, T l1, T l2, v3<T> w, v3<T> gx,
                                            const v3<T>* gd, T ga) {
#pragma unroll
    for (int k = 0; k < ADJ_VEC_MAX; ++k) {
        if (k >= nk) break;
        AdjSums<T>& a = acc[k];
        const T wn = Wn[k];
        a.Q += wn * w;
        a.Xg[0] += (wn * l0) * gx;
        a.Xg[1] += (wn * l1) * gx;
        a.Xg[2] += (wn * l2) * gx;
        a.Grf += wn * gx;
        for (int b = 0; b < 3; ++b) a.Gd[b] += wn * gd[b];
        a.A += wn * ga;
    }
}

// several adjoint vectors at once (their point weights Wn[k], k < nk): the kernel and its derivatives are evaluated
// once, and each set of sums takes its own weight
template <class T, class M = KMath<T>>
__device__ __forceinline__ T adj_point_exact_multi(AdjSums<T>* acc, int nk, const T* Wn, const SrcKern<T>& S, T l0, T l1,
                                                   T l2, v3<T> r0, v3<T> r1, v3<T> r2, v3<T> r, v3<T> m, int side,
                                                   T plane_tol, v3<T>& gx) {
    v3<T> g0, g1, g2;
    ExactShape<T> sh;
    T sv = sv_exact_vjp<T, M>(S, r0, r1, r2, r, m, side, plane_tol, g0, g1, g2, sh);
    const T i4pi = T(1) / (T(4) * vp_pi<T>());
    const v3<T> w = (sh.L[0] * S.nu[0] + sh.L[1] * S.nu[1] + sh.L[2] * S.nu[2] + sh.Om * S.n) * i4pi;
    gx = g0 + g1 + g2;
    adj_acc_exact(acc, nk, Wn, l0, l1, l2, w, gx, g0, g1, g2, sh.L, sh.dLdlen, sh.Om);
    return sv;
}

template <class T>
__device__ __forceinline__ T adj_point_far_multi(AdjSums<T>* acc, int nk, const T* Wn, const SrcKern<T>& S, T l0, T l1,
                                                 T l2, v3<T> r, v3<T> m, v3<T>& gx) {
    v3<T> gd[3];
    T ga;
    T sv = sv_far_vjp(S, r, m, gx, gd, ga);
    const v3<T> w = sv_far(S, r);
    adj_acc_far(acc, nk, Wn, l0, l1, l2, w, gx, gd, ga);
    return sv;
}

// The sums a source collects over all its (test triangle, point) evaluations, with m = n_T x Gamma_S + sigma_S n_T the
// pair's direction (Gamma_S = sum_b mu_b gamma_b the source sheet's vortex density): exact form Gr (ds/dr_a at fixed
// shape), Lm_e = sum L_e m, Nm_e = sum dL_e/dlen_e (nu_e·m), Om = sum Omega m; multipole form Grf, Gd, A (as AdjSums);
// Gb = sum w x n_T and Sb = sum w·n_T (the derivatives with respect to Gamma_S and sigma_S). Every sum carries the
// point's weight W nu(q).
template <class T>
struct SrcAdj {
    v3<T> Gr[3], Lm[3], Om, Grf, Gd[3], Gb;
    T Nm[3], A, Sb;
};

template <class T>
__device__ __forceinline__ void src_zero(SrcAdj<T>& s) {
    v3<T> z = mk3(T(0), T(0), T(0));
    for (int k = 0; k < 3; ++k) {
        s.Gr[k] = z;
        s.Lm[k] = z;
        s.Gd[k] = z;
        s.Nm[k] = T(0);
    }
    s.Om = z;
    s.Grf = z;
    s.Gb = z;
    s.A = T(0);
    s.Sb = T(0);
}

// derivative of a vector of the unit normal (nbar) and of the area (Abar) of triangle v (3) with respect to its
// corners, added to g (3)
template <class T>
__device__ inline void normal_area_grad(const v3<T>* v, v3<T> nbar, T Abar, v3<T>* g) {
    v3<T> u = v[1] - v[0], w2 = v[2] - v[0];
    v3<T> nA = cross(u, w2);
    T A2 = vnorm(nA);
    v3<T> n = nA / A2;
    v3<T> nAbar = (nbar - dot(nbar, n) * n) / A2 + (T(0.5) * Abar) * n;
    v3<T> ubar = cross(w2, nAbar), w2bar = cross(nAbar, u);
    g[1] += ubar;
    g[2] += w2bar;
    g[0] -= ubar + w2bar;
}

// derivative of (V · area vector) with weight c of triangle v: the area vector is nA / 2
template <class T>
__device__ inline void area_vector_grad(const v3<T>* v, v3<T> V, T c, v3<T>* g) {
    v3<T> u = v[1] - v[0], w2 = v[2] - v[0];
    v3<T> nAbar = (T(0.5) * c) * V;
    v3<T> ubar = cross(w2, nAbar), w2bar = cross(nAbar, u);
    g[1] += ubar;
    g[2] += w2bar;
    g[0] -= ubar + w2bar;
}

// The derivative of a source's sums a with respect to its corners v, added to gout: through the offsets to the
// corners and the centroid, the edge normals, edge lengths, unit normal and area (the shape, as SourceTriangle builds
// it: src/kernels/source_triangle.jl:8-26), through Gamma_S = -sum_b mu_b e_b / 2A (e_b the edge opposite corner b)
// and, for a body source (with_sigma), through sigma_S = -V·n_S; d/dalpha of sigma_S = -dV·n_S is added to *dal.
template <class T>
__device__ inline void src_adj_grad(const v3<T>* v, const SrcAdj<T>& a, const T* mu, bool with_sigma, v3<T> V,
                                    v3<T> dV, v3<T>* gout, T* dal) {
    const T i4pi = T(1) / (T(4) * vp_pi<T>());
    v3<T> g[3];
    // exact form: r_a = x - v_a
    for (int k = 0; k < 3; ++k) g[k] = T(-1) * a.Gr[k];
    // multipole form: r = x - c, d_b = v_b - c, c the centroid
    v3<T> sGd = a.Gd[0] + a.Gd[1] + a.Gd[2];
    for (int k = 0; k < 3; ++k) g[k] += (T(-1) / T(3)) * a.Grf + a.Gd[k] - (T(1) / T(3)) * sGd;
    // shape: edges ed_e = v_{e+1} - v_e, lengths, normals nu_e = (ed_e x n) / len_e, n = nA / |nA|, area = |nA| / 2
    v3<T> nA = cross(v[1] - v[0], v[2] - v[0]);
    T A2 = vnorm(nA);
    v3<T> n = nA / A2;
    v3<T> nbar = i4pi * a.Om;
    T Abar = a.A;
    for (int e = 0; e < 3; ++e) {
        v3<T> ed = v[(e + 1) % 3] - v[e];
        T len = vnorm(ed);
        v3<T> nu = cross(ed, n) / len;
        v3<T> nubar = i4pi * a.Lm[e];
        T lenbar = -dot(nu, nubar) / len + a.Nm[e] * i4pi;
        v3<T> ebar = cross(n, nubar) / len + (lenbar / len) * ed;
        nbar += cross(nubar, ed) / len;
        g[(e + 1) % 3] += ebar;
        g[e] -= ebar;
    }
    // Gamma_S = -Et / 2A, Et = sum_b mu_b e_b
    if (mu) {
        T AS = A2 / T(2);
        v3<T> Et = mu[0] * (v[2] - v[1]) + mu[1] * (v[0] - v[2]) + mu[2] * (v[1] - v[0]);
        v3<T> Ebar = (T(-1) / (T(2) * AS)) * a.Gb;
        Abar += dot(a.Gb, Et) / (T(2) * AS * AS);
        g[2] += mu[0] * Ebar;
        g[1] -= mu[0] * Ebar;
        g[0] += mu[1] * Ebar;
        g[2] -= mu[1] * Ebar;
        g[1] += mu[2] * Ebar;
        g[0] -= mu[2] * Ebar;
    }
    if (with_sigma) {
        nbar += (T(-1) * a.Sb) * V;
        *dal += -dot(dV, n) * a.Sb;
    }
    normal_area_grad(v, nbar, Abar, g);
    for (int k = 0; k < 3; ++k) gout[k] += g[k];
}

// a pair's AdjSums (one direction m) as a source's sums; the test normal nT gives Gb and Sb
template <class T>
__device__ inline SrcAdj<T> src_of_pair(const v3<T>* xS, const AdjSums<T>& a, v3<T> m, v3<T> nT) {
    SrcAdj<T> s;
    v3<T> nA = cross(xS[1] - xS[0], xS[2] - xS[0]);
    v3<T> n = nA / vnorm(nA);
    for (int e = 0; e < 3; ++e) {
        v3<T> ed = xS[(e + 1) % 3] - xS[e];
        v3<T> nu = cross(ed, n) / vnorm(ed);
        s.Gr[e] = a.Gr[e];
        s.Lm[e] = a.L[e] * m;
        s.Nm[e] = a.N[e] * dot(nu, m);
        s.Gd[e] = a.Gd[e];
    }
    s.Om = a.O * m;
    s.Grf = a.Grf;
    s.A = a.A;
    s.Gb = cross(a.Q, nT);
    s.Sb = dot(a.Q, nT);
    return s;
}

// the derivative of sum W nu s (at fixed m) with respect to the source's corners v (3), added to g (3)
template <class T>
__device__ inline void adj_source_shape(const v3<T>* v, const AdjSums<T>& a, v3<T> m, v3<T>* gout) {
    SrcAdj<T> s = src_of_pair(v, a, m, mk3(T(0), T(0), T(0)));
    T dal = T(0);
    src_adj_grad(v, s, (const T*)nullptr, false, m, m, gout, &dal);
}

// FP64 form on corners given as 9 doubles
__device__ inline void adj_source_shape(const double* xS, const AdjSums<double>& a, v3<double> m, double* gS) {
    v3<double> v[3] = {mk3(xS[0], xS[1], xS[2]), mk3(xS[3], xS[4], xS[5]), mk3(xS[6], xS[7], xS[8])};
    v3<double> g[3] = {mk3(0.0, 0.0, 0.0), mk3(0.0, 0.0, 0.0), mk3(0.0, 0.0, 0.0)};
    adj_source_shape(v, a, m, g);
    for (int k = 0; k < 3; ++k) {
        gS[3 * k] += g[k].x;
        gS[3 * k + 1] += g[k].y;
        gS[3 * k + 2] += g[k].z;
    }
}

// The test side of f = sum W nu s, s = w·m, m = n_T x Gamma_S + sigma_S n_T: the points' positions (Xg, by corner), the
// unit normal (U = sum W nu ds/dn_T = sum W nu (Gamma_S x w + sigma_S w)) and the area (f / A_T, W = w_q A_T)
template <class T>
__device__ inline void test_adj_grad(const v3<T>* xT, const v3<T>* Xg, v3<T> U, T f, v3<T>* gT) {
    v3<T> nA = cross(xT[1] - xT[0], xT[2] - xT[0]);
    T AT = vnorm(nA) / T(2);
    for (int k = 0; k < 3; ++k) gT[k] += Xg[k];
    normal_area_grad(xT, U, f / AT, gT);
}

// One pair's derivatives from its sums a: the test triangle's corners (gT), the source's (gS) and d/dalpha (dal),
// for a source sheet with corner values mu and Gamma_S = gam, source strength sig (body sources: with_sigma).
template <class T>
__device__ inline void adj_pair_grad(const v3<T>* xT, const v3<T>* xS, const AdjSums<T>& a, v3<T> m, v3<T> gam, T sig,
                                     const T* mu, bool with_sigma, v3<T> V, v3<T> dV, v3<T>* gT, v3<T>* gS, T* dal) {
    v3<T> nT = cross(xT[1] - xT[0], xT[2] - xT[0]);
    nT = nT / vnorm(nT);
    test_adj_grad(xT, a.Xg, cross(gam, a.Q) + sig * a.Q, dot(a.Q, m), gT);
    SrcAdj<T> s = src_of_pair(xS, a, m, nT);
    src_adj_grad(xS, s, mu, with_sigma, V, dV, gS, dal);
}
