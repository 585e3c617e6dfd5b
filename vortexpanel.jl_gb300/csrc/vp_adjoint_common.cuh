// Per-pair pieces of the adjoint: the sums a pair's quadrature points leave, and their conversion into derivatives
// with respect to the source triangle's corners (the chain rule through its edge normals, edge lengths, unit normal,
// corner offsets from the centroid and area, as the forward kernel builds them: SourceTriangle,
// src/kernels/source_triangle.jl:8-26).
#pragma once
#include "vp_adjoint.cuh"

// Sums over a pair's points of W nu(q) times: w (Q); lambda_k ds/dx (Xg); ds/dr_a at fixed shape (Gr, exact form);
// the edge logs (L), dL_e/dlen_e (N) and the solid angle (O) of the exact form; ds/dr (Grf), ds/dd_a (Gd) and
// ds/darea (A) of the multipole form.
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

// add one point: weight Wn = W nu(q), barycentrics l, offsets r_a (exact) or r (multipole), direction m
template <class T>
__device__ __forceinline__ void adj_point_exact(AdjSums<T>& acc, const SrcKern<T>& S, T Wn, T l0, T l1, T l2, v3<T> r0,
                                                v3<T> r1, v3<T> r2, v3<T> r, v3<T> m, int side, T plane_tol) {
    v3<T> g0, g1, g2;
    ExactShape<T> sh;
    sv_exact_vjp(S, r0, r1, r2, r, m, side, plane_tol, g0, g1, g2, sh);
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
}

template <class T>
__device__ __forceinline__ void adj_point_far(AdjSums<T>& acc, const SrcKern<T>& S, T Wn, T l0, T l1, T l2, v3<T> r,
                                              v3<T> m) {
    v3<T> gr, gd[3];
    T ga;
    sv_far_vjp(S, r, m, gr, gd, ga);
    acc.Q += Wn * sv_far(S, r);
    acc.Xg[0] += (Wn * l0) * gr;
    acc.Xg[1] += (Wn * l1) * gr;
    acc.Xg[2] += (Wn * l2) * gr;
    acc.Grf += Wn * gr;
    for (int a = 0; a < 3; ++a) acc.Gd[a] += Wn * gd[a];
    acc.A += Wn * ga;
}

// the derivative of sum W nu s (at fixed m) with respect to the source's corners v (3), added to g (3)
template <class T>
__device__ inline void adj_source_shape(const v3<T>* v, const AdjSums<T>& a, v3<T> m, v3<T>* gout) {
    const T i4pi = T(1) / (T(4) * vp_pi<T>());
    v3<T> g[3];
    // exact form: r_a = x - v_a
    for (int k = 0; k < 3; ++k) g[k] = T(-1) * a.Gr[k];
    // multipole form: r = x - c, d_b = v_b - c, c the centroid
    v3<T> sGd = a.Gd[0] + a.Gd[1] + a.Gd[2];
    for (int k = 0; k < 3; ++k) g[k] += (T(-1) / T(3)) * a.Grf + a.Gd[k] - (T(1) / T(3)) * sGd;
    // shape: edges e_e = v_{e+1} - v_e, lengths, normals nu_e = (e_e x n) / len_e, n = nA / |nA|, area = |nA| / 2
    v3<T> u = v[1] - v[0], w2 = v[2] - v[0];
    v3<T> nA = cross(u, w2);
    T A2 = vnorm(nA);
    v3<T> n = nA / A2;
    v3<T> nbar = (a.O * i4pi) * m;
    v3<T> ebar[3];
    for (int e = 0; e < 3; ++e) {
        v3<T> ed = v[(e + 1) % 3] - v[e];
        T len = vnorm(ed);
        v3<T> nu = cross(ed, n) / len;
        v3<T> nubar = (a.L[e] * i4pi) * m;
        T lenbar = -dot(nu, nubar) / len + a.N[e] * dot(nu, m) * i4pi;
        ebar[e] = cross(n, nubar) / len + (lenbar / len) * ed;
        nbar += cross(nubar, ed) / len;
    }
    v3<T> nAbar = (nbar - dot(nbar, n) * n) / A2 + (T(0.5) * a.A) * n;  // area = |nA| / 2
    v3<T> ubar = cross(w2, nAbar), w2bar = cross(nAbar, u);
    g[1] += ubar;
    g[2] += w2bar;
    g[0] -= ubar + w2bar;
    for (int e = 0; e < 3; ++e) {
        g[(e + 1) % 3] += ebar[e];
        g[e] -= ebar[e];
    }
    for (int k = 0; k < 3; ++k) gout[k] += g[k];
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

// The derivative of one pair's f = sum W nu w·m, m = n_T x gamma_S + sigma_S n_T, from its sums a:
// the test triangle's corners (gT), the source's (gS), and d f / d alpha through sigma_S = -V·n_S (dal), for a source
// sheet with corner values mu (gamma_S = sum_b mu_b gamma_b, gamma_b = -e_b / 2A, e_b the edge opposite corner b) and
// source strength sigma (body sources: with_sigma).
template <class T>
__device__ inline void adj_pair_grad(const v3<T>* xT, const v3<T>* xS, const AdjSums<T>& a, v3<T> m, v3<T> gam, T sig,
                                     const T* mu, bool with_sigma, v3<T> V, v3<T> eL, v3<T>* gT, v3<T>* gS, T* dal) {
    v3<T> nT = cross(xT[1] - xT[0], xT[2] - xT[0]);
    T AT = vnorm(nT) / T(2);
    nT = nT / (T(2) * AT);
    T f = dot(a.Q, m);
    for (int k = 0; k < 3; ++k) gT[k] += a.Xg[k];
    normal_area_grad(xT, cross(gam, a.Q) + sig * a.Q, f / AT, gT);
    adj_source_shape(xS, a, m, gS);
    v3<T> nA = cross(xS[1] - xS[0], xS[2] - xS[0]);
    T AS = vnorm(nA) / T(2);
    v3<T> nS = nA / (T(2) * AS);
    v3<T> gbar = cross(a.Q, nT);
    v3<T> Et = mu[0] * (xS[2] - xS[1]) + mu[1] * (xS[0] - xS[2]) + mu[2] * (xS[1] - xS[0]);
    v3<T> Ebar = (T(-1) / (T(2) * AS)) * gbar;
    T Abar = dot(gbar, Et) / (T(2) * AS * AS);
    gS[2] += mu[0] * Ebar;
    gS[1] -= mu[0] * Ebar;
    gS[0] += mu[1] * Ebar;
    gS[2] -= mu[1] * Ebar;
    gS[1] += mu[2] * Ebar;
    gS[0] -= mu[2] * Ebar;
    v3<T> nbarS = mk3(T(0), T(0), T(0));
    if (with_sigma) {
        T sbar = dot(a.Q, nT);
        nbarS = T(-1) * sbar * V;
        *dal += -dot(eL, nS) * sbar;
    }
    normal_area_grad(xS, nbarS, Abar, gS);
}
