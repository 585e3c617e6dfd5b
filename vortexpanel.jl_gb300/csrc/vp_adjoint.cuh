// Reverse-mode derivatives of the pair-integral kernels for the adjoint (templated on float / double).
//
// A quadrature point contributes W nu(q) s, s = w(x)·m, with w the unit source-triangle velocity
// (src/kernels/source_triangle.jl:75-138) and m a per-pair vector. w depends on the point only through the offsets
// r_a = x - v_a to the source's corners, and on the source's shape through its edge normals nu_e, edge lengths, unit
// normal n (exact form) or its corner offsets d_a and area (multipole form). The functions below return s, the
// derivative of s with respect to the offsets at fixed shape, and the per-point factors of the shape derivatives,
// which the caller sums over the points of a pair and turns into corner derivatives once per pair.
#pragma once
#include "vp_math.cuh"

// shape factors of one exact-kernel point: s depends on the shape through
//   sum_e L_e (nu_e·m)/4pi + Omega (n·m)/4pi, with L_e depending on the edge length through num_e = r_i + r_j + len_e
template <class T>
struct ExactShape {
    T L[3];      // edge logs
    T dLdlen[3]; // dL_e / d len_e = 2 / num_e
    T Om;        // solid angle
};

// s = w·m of the exact kernel at fixed shape (nu, len, n from the source) and ds/dr_a.
template <class T, class M = KMath<T>>
__device__ __forceinline__ T sv_exact_vjp(const SrcKern<T>& S, v3<T> r0, v3<T> r1, v3<T> r2, v3<T> r, v3<T> m,
                                          int side, T plane_tol, v3<T>& g0, v3<T>& g1, v3<T>& g2, ExactShape<T>& sh) {
    const T i4pi = T(1) / (T(4) * vp_pi<T>());
    const v3<T> R[3] = {r0, r1, r2};
    T l[3] = {M::sqrt(dot(r0, r0)), M::sqrt(dot(r1, r1)), M::sqrt(dot(r2, r2))};
    v3<T> gr[3] = {mk3(T(0), T(0), T(0)), mk3(T(0), T(0), T(0)), mk3(T(0), T(0), T(0))};
    T lbar[3] = {T(0), T(0), T(0)};
    T s = T(0);
#pragma unroll
    for (int e = 0; e < 3; ++e) {
        const int i = e, j = (e + 1) % 3;
        v3<T> ri = R[i], rj = R[j];
        T p = dot(ri, rj);
        T num = l[i] + l[j] + S.len[e];
        T L, dLdli, dLdlj, dLdp;
        v3<T> c = cross(ri, rj);
        T c2 = norm2(c);
        if (p < T(0)) {
            T den = l[i] * l[j] - p;
            T q = M::div(den, T(2) * c2);
            L = M::log(num * num * q);
            // d log q: li -> lj/den, lj -> li/den, p -> -1/den, c2 -> -1/c2
            dLdli = M::div(T(2), num) + M::div(l[j], den);
            dLdlj = M::div(T(2), num) + M::div(l[i], den);
            dLdp = M::div(-T(1), den);
            T dLdc2 = M::div(-T(1), c2);
            T coef = dot(S.nu[e], m) * i4pi;
            // c2 = |ri x rj|^2: d/dri = 2 rj x c, d/drj = 2 c x ri
            gr[i] += (coef * dLdc2 * T(2)) * cross(rj, c);
            gr[j] += (coef * dLdc2 * T(2)) * cross(c, ri);
        } else {
            T den = l[i] * l[j] + p;
            if constexpr (M::hybrid)
                L = M::log1p(M::div(S.len[e] * num, den));
            else
                L = sizeof(T) == 4 ? T(log1pf(float(S.len[e] * num / den))) : vlog(num * num / (T(2) * den));
            dLdli = M::div(T(2), num) - M::div(l[j], den);
            dLdlj = M::div(T(2), num) - M::div(l[i], den);
            dLdp = M::div(-T(1), den);
        }
        T coef = dot(S.nu[e], m) * i4pi;
        s += L * coef;
        lbar[i] += coef * dLdli;
        lbar[j] += coef * dLdlj;
        gr[i] += (coef * dLdp) * rj;
        gr[j] += (coef * dLdp) * ri;
        sh.L[e] = L;
        sh.dLdlen[e] = M::div(T(2), num);
    }
    T z = dot(r, S.n);
    T nm = dot(S.n, m) * i4pi;
    T N = dot(r0, cross(r1, r2));
    T D = l[0] * l[1] * l[2] + dot(r0, r1) * l[2] + dot(r0, r2) * l[1] + dot(r1, r2) * l[0];
    if (fabs(z) <= plane_tol * S.diam) {
        v3<T> q[3] = {-r0, -r1, -r2};
        sh.Om = side == 0 ? T(0) : T(side) * T(2) * vp_pi<T>() * inplane_fraction_rel(q, S.n, S.area, plane_tol);
    } else {
        sh.Om = T(2) * M::atan2(N, D);
    }
    // 2 atan2(N, D) is smooth across the plane away from the triangle's edges (N = 0, D != 0): in the plane its
    // derivative along the normal is the one-sided limit of the general formula, which the in-plane branch keeps
    if (N * N + D * D > T(0)) {
        T h = M::div(T(2), N * N + D * D);
        T Nb = nm * D * h, Db = -nm * N * h;
        gr[0] += Nb * cross(r1, r2);
        gr[1] += Nb * cross(r2, r0);
        gr[2] += Nb * cross(r0, r1);
        lbar[0] += Db * (l[1] * l[2] + dot(r1, r2));
        lbar[1] += Db * (l[0] * l[2] + dot(r0, r2));
        lbar[2] += Db * (l[0] * l[1] + dot(r0, r1));
        gr[0] += Db * (l[2] * r1 + l[1] * r2);
        gr[1] += Db * (l[2] * r0 + l[0] * r2);
        gr[2] += Db * (l[1] * r0 + l[0] * r1);
    }
    s += sh.Om * nm;
#pragma unroll
    for (int a = 0; a < 3; ++a) gr[a] += M::div(lbar[a], l[a]) * R[a];
    g0 = gr[0];
    g1 = gr[1];
    g2 = gr[2];
    return s;
}

// The mixed path's FP64 points (where FP32 cancels), split by what cancels: the offsets' lengths, the edges' dot and
// cross products, the stable forms l_i l_j + r_i.r_j, the solid angle's numerator and denominator and the vectors
// l_k r_j + l_j r_k are formed in FP64 (with KMathHyb's square root), and the functions and the derivative algebra on
// them run in FP32, where no difference of nearly equal terms is left. The same s, ds/dr_a and shape factors as
// sv_exact_vjp<double, KMathHyb>, at FP32 accuracy, with about a quarter of its FP64 work. Returns false, with the
// outputs unset, for a point so near a corner or an edge's line that the terms leave FP32's range (a corner offset
// under 1e-10, an edge cross product |c|^2 under 1e-30); the caller takes that point wholly in FP64.
__device__ __forceinline__ bool sv_exact_vjp_split(const SrcKern<double>& S, v3<double> r0, v3<double> r1,
                                                   v3<double> r2, v3<double> r, v3<float> m, int side, double plane_tol,
                                                   float& svo, v3<float>& g0, v3<float>& g1, v3<float>& g2,
                                                   ExactShape<float>& sh) {
    const v3<double> R[3] = {r0, r1, r2};
    double l64[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) l64[a] = KMathHyb::sqrt(dot(R[a], R[a]));
    if (!(fmin(l64[0], fmin(l64[1], l64[2])) > 1e-10)) return false;
    float l[3], p[3], s2[3], c2[3];
    v3<float> c[3], Rf[3];
#pragma unroll
    for (int e = 0; e < 3; ++e) {
        const int i = e, j = (e + 1) % 3;
        const double pe = dot(R[i], R[j]);
        const v3<double> ce = cross(R[i], R[j]);
        const double lilj = l64[i] * l64[j];
        // l_i l_j + p without cancellation: |c|^2 / (l_i l_j - p) where p < 0
        const double c2e = norm2(ce);
        if (pe < 0.0 && !(c2e > 1e-30)) return false;
        const double se = pe < 0.0 ? KMathHyb::div(c2e, lilj - pe) : lilj + pe;
        c2[e] = float(c2e);
        l[e] = float(l64[e]);
        p[e] = float(pe);
        s2[e] = float(se);
        c[e] = f3(ce);
        Rf[e] = f3(R[e]);
    }
    const double N64 = dot(r0, cross(r1, r2));
    const double D64 = l64[0] * l64[1] * l64[2] + dot(r0, r1) * l64[2] + dot(r0, r2) * l64[1] + dot(r1, r2) * l64[0];
    const v3<float> V[3] = {f3(l64[2] * r1 + l64[1] * r2), f3(l64[2] * r0 + l64[0] * r2), f3(l64[1] * r0 + l64[0] * r1)};
    const double z = dot(r, S.n);
    const float N = float(N64), D = float(D64);
    // the solid angle's derivative factors 2 (D, N) / (N^2 + D^2), formed in FP64: the squares of N and D leave
    // FP32's range where the offsets are small
    const double nd2 = N64 * N64 + D64 * D64;
    const double hnd = nd2 > 0.0 ? KMathHyb::div(2.0, nd2) : 0.0;
    const float hD = float(hnd * D64), hN = float(hnd * N64);
    // FP32 from here
    const float i4pi = 1.f / (4.f * vp_pi<float>());
    v3<float> gr[3] = {mk3(0.f, 0.f, 0.f), mk3(0.f, 0.f, 0.f), mk3(0.f, 0.f, 0.f)};
    float lbar[3] = {0.f, 0.f, 0.f};
    float sv = 0.f;
#pragma unroll
    for (int e = 0; e < 3; ++e) {
        const int i = e, j = (e + 1) % 3;
        const float len = float(S.len[e]);
        const float num = l[i] + l[j] + len;
        const v3<float> nu = f3(S.nu[e]);
        const float coef = dot(nu, m) * i4pi;
        float L, dLdli, dLdlj, dLdp;
        if (p[e] < 0.f) {
            const float den = l[i] * l[j] - p[e];
            L = logf(num * num * (den / (2.f * c2[e])));
            dLdli = 2.f / num + l[j] / den;
            dLdlj = 2.f / num + l[i] / den;
            dLdp = -1.f / den;
            const float k2 = coef * (-1.f / c2[e]) * 2.f;
            gr[i] += k2 * cross(Rf[j], c[e]);
            gr[j] += k2 * cross(c[e], Rf[i]);
        } else {
            const float den = s2[e];
            L = log1pf(len * num / den);
            dLdli = 2.f / num - l[j] / den;
            dLdlj = 2.f / num - l[i] / den;
            dLdp = -1.f / den;
        }
        sv += L * coef;
        lbar[i] += coef * dLdli;
        lbar[j] += coef * dLdlj;
        gr[i] += (coef * dLdp) * Rf[j];
        gr[j] += (coef * dLdp) * Rf[i];
        sh.L[e] = L;
        sh.dLdlen[e] = 2.f / num;
    }
    const float nm = dot(f3(S.n), m) * i4pi;
    if (fabs(z) <= plane_tol * S.diam) {
        const v3<double> q[3] = {-r0, -r1, -r2};
        sh.Om = side == 0 ? 0.f
                          : float(side) * 2.f * vp_pi<float>() *
                                float(inplane_fraction_rel(q, S.n, S.area, plane_tol));
    } else {
        sh.Om = 2.f * atan2f(N, D);
    }
    if (nd2 > 0.0) {
        const float Nb = nm * hD, Db = -nm * hN;
        gr[0] += Nb * c[1];
        gr[1] += Nb * c[2];
        gr[2] += Nb * c[0];
        lbar[0] += Db * s2[1];
        lbar[1] += Db * s2[2];
        lbar[2] += Db * s2[0];
        gr[0] += Db * V[0];
        gr[1] += Db * V[1];
        gr[2] += Db * V[2];
    }
    sv += sh.Om * nm;
#pragma unroll
    for (int a = 0; a < 3; ++a) gr[a] += (lbar[a] / l[a]) * Rf[a];
    if (!(isfinite(sv) && isfinite(gr[0].x + gr[0].y + gr[0].z + gr[1].x + gr[1].y + gr[1].z + gr[2].x + gr[2].y +
                                   gr[2].z)))
        return false;
    svo = sv;
    g0 = gr[0];
    g1 = gr[1];
    g2 = gr[2];
    return true;
}

// s = w·m of the multipole form (source_triangle.jl:100-119) and its derivatives with respect to r = x - c, to the
// corner offsets d_a (gd) and the area (ga)
template <class T>
__device__ __forceinline__ T sv_far_vjp(const SrcKern<T>& S, v3<T> r, v3<T> m, v3<T>& gr, v3<T>* gd, T& ga) {
    const T k = S.area / (T(4) * vp_pi<T>());
    T R2 = dot(r, r);
    T iR2, iR3;
    inv_r23(R2, iR2, iR3);
    T iR5 = iR3 * iR2, iR7 = iR5 * iR2, iR9 = iR7 * iR2, iR11 = iR9 * iR2;
    T rm = dot(r, m);
    // F·m = iR3 rm + sum_a g_a(dr, dd, rm, dm, R2)
    T Fm = iR3 * rm;
    v3<T> gF = iR3 * m;  // d(F·m)/dr, accumulated
    T dR2 = T(-1.5) * iR5 * rm;  // d(F·m)/dR2
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        v3<T> d = S.d[a];
        T dr = dot(d, r), dd = dot(d, d), dm = dot(d, m);
        // quad·m / 24 - oct·m / 180
        T g = (T(15) * dr * dr * iR7 * rm - T(6) * dr * iR5 * dm - T(3) * dd * iR5 * rm) / T(24) -
              (T(45) * dr * dr * iR7 * dm - T(105) * dr * dr * dr * iR9 * rm - T(9) * dd * iR5 * dm +
               T(45) * dd * dr * iR7 * rm) / T(180);
        Fm += g;
        T g_dr = (T(30) * dr * iR7 * rm - T(6) * iR5 * dm) / T(24) -
                 (T(90) * dr * iR7 * dm - T(315) * dr * dr * iR9 * rm + T(45) * dd * iR7 * rm) / T(180);
        T g_dd = (-T(3) * iR5 * rm) / T(24) - (-T(9) * iR5 * dm + T(45) * dr * iR7 * rm) / T(180);
        T g_rm = (T(15) * dr * dr * iR7 - T(3) * dd * iR5) / T(24) -
                 (-T(105) * dr * dr * dr * iR9 + T(45) * dd * dr * iR7) / T(180);
        T g_dm = (-T(6) * dr * iR5) / T(24) - (T(45) * dr * dr * iR7 - T(9) * dd * iR5) / T(180);
        // iR_k = R2^(-k/2): d/dR2 = -(k/2) iR_(k+2)
        T g_R2 = (T(15) * dr * dr * (T(-3.5) * iR9) * rm - T(6) * dr * (T(-2.5) * iR7) * dm -
                  T(3) * dd * (T(-2.5) * iR7) * rm) / T(24) -
                 (T(45) * dr * dr * (T(-3.5) * iR9) * dm - T(105) * dr * dr * dr * (T(-4.5) * iR11) * rm -
                  T(9) * dd * (T(-2.5) * iR7) * dm + T(45) * dd * dr * (T(-3.5) * iR9) * rm) / T(180);
        gF += g_dr * d + g_rm * m;
        dR2 += g_R2;
        gd[a] = k * (g_dr * r + (T(2) * g_dd) * d + g_dm * m);
    }
    gF += (T(2) * dR2) * r;
    gr = k * gF;
    ga = Fm / (T(4) * vp_pi<T>());
    return k * Fm;
}

// the two end parts of a filament (segment.jl:15-25) contracted with ca, cb: s = ca (va·n) + cb (vb·n), and its
// derivatives with respect to ra = x - a and rb = x - b
template <class T>
__device__ __forceinline__ T seg_vjp(v3<T> ra, v3<T> rb, v3<T> n, T ca, T cb, v3<T>& ga, v3<T>& gb) {
    T Ra = vnorm(ra), Rb = vnorm(rb);
    v3<T> c = cross(ra, rb);
    T p = dot(ra, rb);
    T den, c2 = norm2(c);
    bool neg = p < T(0);
    den = neg ? c2 / (Ra * Rb - p) : Ra * Rb + p;
    ga = mk3(T(0), T(0), T(0));
    gb = ga;
    if (den == T(0) || Ra == T(0) || Rb == T(0)) return T(0);
    const T i4pi = T(1) / (T(4) * vp_pi<T>());
    T cn = dot(c, n);
    T wsum = ca / Ra + cb / Rb;
    T s = cn * i4pi / den * wsum;
    // s = cn * i4pi * wsum / den
    T s_cn = i4pi * wsum / den;
    T s_den = -s / den;
    T s_Ra = -cn * i4pi / den * ca / (Ra * Ra);
    T s_Rb = -cn * i4pi / den * cb / (Rb * Rb);
    // cn = (ra x rb)·n: d/dra = rb x n, d/drb = n x ra
    ga += s_cn * cross(rb, n);
    gb += s_cn * cross(n, ra);
    if (neg) {  // den = c2 / (Ra Rb - p)
        T q = Ra * Rb - p;
        T d_c2 = T(1) / q, d_q = -c2 / (q * q);
        ga += (s_den * d_c2 * T(2)) * cross(rb, c);
        gb += (s_den * d_c2 * T(2)) * cross(c, ra);
        s_Ra += s_den * d_q * Rb;
        s_Rb += s_den * d_q * Ra;
        ga += (-s_den * d_q) * rb;
        gb += (-s_den * d_q) * ra;
    } else {  // den = Ra Rb + p
        s_Ra += s_den * Rb;
        s_Rb += s_den * Ra;
        ga += s_den * rb;
        gb += s_den * ra;
    }
    ga += (s_Ra / Ra) * ra;
    gb += (s_Rb / Rb) * rb;
    return s;
}
