// Device math of the Galerkin hot path: 3-vectors, the unit source-triangle kernel w(x) (analytic inner integral,
// src/kernels/source_triangle.jl:39-138), the linearly varying filament (src/kernels/segment.jl:15-25), the
// Rosenhead-Moore blob (src/kernels/blob.jl:21-25) and the test weights (src/assembly/assemble.jl:52-61).
// Templated on the scalar (float for the FP32 far/near tiers, double for FP64).
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

template <class T>
struct v3 {
    T x, y, z;
};

template <class T> __host__ __device__ __forceinline__ v3<T> mk3(T a, T b, T c) { return v3<T>{a, b, c}; }
template <class T> __host__ __device__ __forceinline__ v3<T> operator+(v3<T> a, v3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T> __host__ __device__ __forceinline__ v3<T> operator-(v3<T> a, v3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T> __host__ __device__ __forceinline__ v3<T> operator-(v3<T> a) { return {-a.x, -a.y, -a.z}; }
template <class T> __host__ __device__ __forceinline__ v3<T> operator*(T s, v3<T> a) { return {s * a.x, s * a.y, s * a.z}; }
template <class T> __host__ __device__ __forceinline__ v3<T> operator*(v3<T> a, T s) { return {s * a.x, s * a.y, s * a.z}; }
template <class T> __host__ __device__ __forceinline__ v3<T> operator/(v3<T> a, T s) { return {a.x / s, a.y / s, a.z / s}; }
template <class T> __host__ __device__ __forceinline__ void operator+=(v3<T>& a, v3<T> b) { a.x += b.x; a.y += b.y; a.z += b.z; }
template <class T> __host__ __device__ __forceinline__ void operator-=(v3<T>& a, v3<T> b) { a.x -= b.x; a.y -= b.y; a.z -= b.z; }
template <class T> __host__ __device__ __forceinline__ T dot(v3<T> a, v3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T> __host__ __device__ __forceinline__ v3<T> cross(v3<T> a, v3<T> b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <class T> __host__ __device__ __forceinline__ T norm2(v3<T> a) { return dot(a, a); }
__host__ __device__ __forceinline__ v3<float> f3(v3<double> v) { return v3<float>{float(v.x), float(v.y), float(v.z)}; }

__device__ __forceinline__ float vsqrt(float a) { return sqrtf(a); }
__device__ __forceinline__ double vsqrt(double a) { return sqrt(a); }
__device__ __forceinline__ float vlog(float a) { return logf(a); }
__device__ __forceinline__ double vlog(double a) { return log(a); }
__device__ __forceinline__ float vatan2(float a, float b) { return atan2f(a, b); }
__device__ __forceinline__ double vatan2(double a, double b) { return atan2(a, b); }
__device__ __forceinline__ float vacos(float a) { return acosf(a); }
__device__ __forceinline__ double vacos(double a) { return acos(a); }
template <class T> __device__ __forceinline__ T vnorm(v3<T> a) { return vsqrt(dot(a, a)); }

// 1/R^2 and 1/R^3 of the multipole forms from R^2. FP32: one reciprocal square root (rsqrtf, a few ulp, far below the
// multipole's truncation error and FP32's own rounding of the sums) instead of a square root and two IEEE divisions,
// the far tiers' special-function bound. FP64: the square root and the divisions.
__device__ __forceinline__ void inv_r23(float R2, float& iR2, float& iR3) {
    const float iR = rsqrtf(R2);
    iR2 = iR * iR;
    iR3 = iR2 * iR;
}
__device__ __forceinline__ void inv_r23(double R2, double& iR2, double& iR3) {
    const double R = sqrt(R2);
    iR2 = 1.0 / R2;
    iR3 = iR2 / R;
}

// The scalar functions of the exact kernel and its derivatives, as a policy of the evaluation.
// KMath<T>: the plain FP32 or FP64 functions.
// KMathHyb: the FP64 evaluation of the mixed-precision path, for the points that FP32 cannot take (near a source's
// corners and edges, where the offsets, cross products and the solid angle's numerator and denominator cancel).
// Those quantities stay FP64; the functions applied to them are FP32-based:
// - the square root and the reciprocal are refined by one Newton step in FP64 (relative error ~1e-14);
// - log, log1p and atan2 are the FP32 functions of the FP64-formed arguments (relative error ~1e-7, the accuracy of
//   the points evaluated in FP32).
// Arguments outside FP32's comfortable range go to the FP64 functions.
template <class T>
struct KMath {
    static constexpr bool hybrid = false;
    static __device__ __forceinline__ T sqrt(T x) { return vsqrt(x); }
    static __device__ __forceinline__ T div(T a, T b) { return a / b; }
    static __device__ __forceinline__ T log(T x) { return vlog(x); }
    static __device__ __forceinline__ T atan2(T y, T x) { return vatan2(y, x); }
};

// the FP64 functions out of line, for KMathHyb's rare out-of-range arguments (kept off the hot path's registers)
static __device__ __noinline__ double f64_sqrt(double x) { return sqrt(x); }
static __device__ __noinline__ double f64_rcp(double x) { return 1.0 / x; }
static __device__ __noinline__ double f64_log(double x) { return log(x); }
static __device__ __noinline__ double f64_log1p(double x) { return log1p(x); }
static __device__ __noinline__ double f64_atan2(double y, double x) { return atan2(y, x); }

struct KMathHyb {
    static constexpr bool hybrid = true;
    static __device__ __forceinline__ bool in_range(double m) { return m > 1e-30 && m < 1e30; }
    static __device__ __forceinline__ double sqrt(double x) {
        if (!in_range(x)) return f64_sqrt(x);
        const double y = double(rsqrtf(float(x)));
        const double r = x * y;
        return fma(0.5 * y, fma(-r, r, x), r);  // Newton: r + (x - r^2) / (2 r), with 1/r ~ y
    }
    static __device__ __forceinline__ double rcp(double x) {
        if (!in_range(fabs(x))) return f64_rcp(x);
        const double r = double(1.0f / float(x));
        return fma(r, fma(-x, r, 1.0), r);  // Newton: r (2 - x r)
    }
    static __device__ __forceinline__ double div(double a, double b) { return a * rcp(b); }
    static __device__ __forceinline__ double log(double x) {
        if (!in_range(x)) return f64_log(x);
        return double(logf(float(x)));
    }
    static __device__ __forceinline__ double log1p(double x) {
        if (!(x > -0.5 && x < 1e30)) return f64_log1p(x);
        return double(log1pf(float(x)));
    }
    static __device__ __forceinline__ double atan2(double y, double x) {
        if (!in_range(fmax(fabs(x), fabs(y)))) return f64_atan2(y, x);
        return double(atan2f(float(y), float(x)));
    }
};

template <class T> __host__ __device__ __forceinline__ T vp_pi() { return T(3.141592653589793238462643383279502884); }

// The source data the kernel needs, relative to the source centroid c (vertices v_a = c + d_a).
template <class T>
struct SrcKern {
    v3<T> d[3];   // vertex offsets from the centroid
    v3<T> n;      // unit normal
    v3<T> nu[3];  // in-plane outward unit edge normals (edge a from vertex a to a+1)
    T len[3];     // edge lengths
    T area, diam;
};

// inplane_fraction (source_triangle.jl:52-64) with the vertices given relative to the point (q_k = v_k - x)
template <class T>
__device__ T inplane_fraction_rel(const v3<T> q[3], v3<T> n, T area, T tol) {
    T A2 = T(2) * area;
    T l[3] = {dot(cross(q[1], q[2]), n) / A2, dot(cross(q[2], q[0]), n) / A2, dot(cross(q[0], q[1]), n) / A2};
    for (int k = 0; k < 3; ++k)
        if (l[k] < -tol) return T(0);
    int nzero = 0;
    for (int k = 0; k < 3; ++k)
        if (fabs(l[k]) <= tol) ++nzero;
    if (nzero == 0) return T(1);
    if (nzero == 1) return T(0.5);
    int k = 0;
    while (k < 3 && !(fabs(l[k]) > tol)) ++k;
    v3<T> e1 = q[(k + 1) % 3] - q[k], e2 = q[(k + 2) % 3] - q[k];
    T cs = dot(e1, e2) / (vnorm(e1) * vnorm(e2));
    cs = cs < T(-1) ? T(-1) : (cs > T(1) ? T(1) : cs);
    return vacos(cs) / (T(2) * vp_pi<T>());
}

// edge_log with the distances to the edge's ends given: ln((r_i + r_j + d)^2 / (2(r_i r_j + ri.rj))), the denominator
// formed without cancellation as |ri x rj|^2 / (r_i r_j - ri.rj) when ri.rj < 0 (source_triangle.jl:39-44)
// (FP32: where ri.rj >= 0 the same value as log1p(d (r_i + r_j + d) / (r_i r_j + ri.rj)), using
// (r_i + r_j)^2 - d^2 = 2 (r_i r_j + ri.rj), which keeps its accuracy at a distance where the log's argument nears 1)
template <class T, class M = KMath<T>>
__device__ __forceinline__ T edge_log_n(v3<T> ri, v3<T> rj, T li, T lj, T d) {
    T p = dot(ri, rj);
    T num = li + lj + d;
    if constexpr (M::hybrid) {
        if (p >= T(0)) return M::log1p(M::div(d * num, li * lj + p));
    } else {
        if (sizeof(T) == 4 && p >= T(0)) return T(log1pf(float(d * num / (li * lj + p))));
    }
    T q = p < T(0) ? M::div(li * lj - p, T(2) * norm2(cross(ri, rj))) : M::div(T(1), T(2) * (li * lj + p));
    return M::log(num * num * q);
}

// source_velocity_exact (source_triangle.jl:75-89) from the point's offsets to the three vertices ra, rb, rc
// (r_a = x - v_a) and to the centroid r = x - c.
template <class T, class M = KMath<T>>
__device__ __forceinline__ v3<T> sv_exact3(const SrcKern<T>& S, v3<T> ra, v3<T> rb, v3<T> rc, v3<T> r, int side,
                                           T plane_tol) {
    T la = M::sqrt(dot(ra, ra)), lb = M::sqrt(dot(rb, rb)), lc = M::sqrt(dot(rc, rc));
    v3<T> wt = edge_log_n<T, M>(ra, rb, la, lb, S.len[0]) * S.nu[0] + edge_log_n<T, M>(rb, rc, lb, lc, S.len[1]) * S.nu[1] +
               edge_log_n<T, M>(rc, ra, lc, la, S.len[2]) * S.nu[2];
    T z = dot(r, S.n);
    T Om;
    if (fabs(z) <= plane_tol * S.diam) {
        v3<T> q[3] = {-ra, -rb, -rc};
        Om = side == 0 ? T(0) : T(side) * T(2) * vp_pi<T>() * inplane_fraction_rel(q, S.n, S.area, plane_tol);
    } else {
        T N = dot(ra, cross(rb, rc));
        T D = la * lb * lc + dot(ra, rb) * lc + dot(ra, rc) * lb + dot(rb, rc) * la;
        Om = T(2) * M::atan2(N, D);
    }
    return (wt + Om * S.n) * (T(1) / (T(4) * vp_pi<T>()));
}

// The mixed path's FP64 points of the exact kernel, split by what cancels: the offsets' lengths (KMathHyb's square
// root), the edges' dot products and squared cross products, and the solid angle's numerator and denominator are
// formed in FP64; the logs, the atan2 and the sums on them run in FP32, where no difference of nearly equal terms is
// left (l_i l_j - p with p < 0 and l_i l_j + p with p >= 0 are sums of non-negative terms). The value of
// sv_exact3<double, KMathHyb> at FP32 accuracy, with about half its FP64 work. Returns false, with w unset, for a
// point so near a corner or an edge's line that the terms leave FP32's range (a corner offset under 1e-10, an edge
// cross product |c|^2 under 1e-30); the caller takes that point wholly in FP64.
__device__ __forceinline__ bool sv_exact3_split(const SrcKern<double>& S, v3<double> ra, v3<double> rb, v3<double> rc,
                                                v3<double> r, int side, double plane_tol, v3<float>& w) {
    const v3<double> R[3] = {ra, rb, rc};
    double l64[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) l64[a] = KMathHyb::sqrt(dot(R[a], R[a]));
    if (!(fmin(l64[0], fmin(l64[1], l64[2])) > 1e-10)) return false;
    v3<float> wt = mk3(0.f, 0.f, 0.f);
#pragma unroll
    for (int e = 0; e < 3; ++e) {
        const int i = e, j = (e + 1) % 3;
        const double pe = dot(R[i], R[j]);
        const float li = float(l64[i]), lj = float(l64[j]), p = float(pe), len = float(S.len[e]);
        const float num = li + lj + len;
        float L;
        if (pe < 0.0) {
            const double c2e = norm2(cross(R[i], R[j]));
            if (!(c2e > 1e-30)) return false;
            const float c2 = float(c2e);
            L = logf(num * num * ((li * lj - p) / (2.f * c2)));
        } else {
            L = log1pf(len * num / (li * lj + p));
        }
        wt += L * f3(S.nu[e]);
    }
    float Om;
    if (fabs(dot(r, S.n)) <= plane_tol * S.diam) {
        const v3<double> q[3] = {-ra, -rb, -rc};
        Om = side == 0 ? 0.f : float(side) * 2.f * vp_pi<float>() * float(inplane_fraction_rel(q, S.n, S.area, plane_tol));
    } else {
        const double N = dot(ra, cross(rb, rc));
        const double D = l64[0] * l64[1] * l64[2] + dot(ra, rb) * l64[2] + dot(ra, rc) * l64[1] + dot(rb, rc) * l64[0];
        Om = 2.f * atan2f(float(N), float(D));
    }
    w = (wt + Om * f3(S.n)) * (1.f / (4.f * vp_pi<float>()));
    return isfinite(w.x + w.y + w.z);
}

// The exact kernel in FP32 where FP32 is accurate, for a point off the source's singular set: returns false (and
// leaves w unset) when the point is near a corner, next to an edge segment (the offsets to its ends nearly
// antiparallel), or near the plane over the triangle (the branch of the solid angle), where the log/atan forms
// cancel and the point must be evaluated in FP64. side != 0 marks the self pair (coplanar, interior points).
struct Fp32Guard {
    float corner, edge_sin2, plane;
};

// the guard of sv_exact3_guarded alone: true where the FP32 exact kernel (and its derivatives) may be used
__device__ __forceinline__ bool fp32_guard_ok(const SrcKern<float>& S, v3<float> ra, v3<float> rb, v3<float> rc,
                                              int side, const Fp32Guard& g) {
    float la = vnorm(ra), lb = vnorm(rb), lc = vnorm(rc);
    if (fminf(la, fminf(lb, lc)) < g.corner * S.diam) return false;
    const v3<float> R[3] = {ra, rb, rc};
    const float L[3] = {la, lb, lc};
#pragma unroll
    for (int e = 0; e < 3; ++e) {
        v3<float> ri = R[e], rj = R[(e + 1) % 3];
        float p = dot(ri, rj);
        if (p < 0.f && norm2(cross(ri, rj)) < g.edge_sin2 * (L[e] * L[e]) * (L[(e + 1) % 3] * L[(e + 1) % 3]))
            return false;
    }
    if (side == 0) {
        float P3 = la * lb * lc;
        float N = dot(ra, cross(rb, rc));
        float D = P3 + dot(ra, rb) * lc + dot(ra, rc) * lb + dot(rb, rc) * la;
        if (fabsf(N) < g.plane * P3 && (D < 0.f || fabsf(D) < g.plane * P3)) return false;
    }
    return true;
}

__device__ __forceinline__ bool sv_exact3_guarded(const SrcKern<float>& S, v3<float> ra, v3<float> rb, v3<float> rc,
                                                  int side, const Fp32Guard& g, v3<float>& w) {
    float la = vnorm(ra), lb = vnorm(rb), lc = vnorm(rc);
    if (fminf(la, fminf(lb, lc)) < g.corner * S.diam) return false;
    const v3<float> R[3] = {ra, rb, rc};
    const float L[3] = {la, lb, lc};
    v3<float> wt = mk3(0.f, 0.f, 0.f);
#pragma unroll
    for (int e = 0; e < 3; ++e) {
        v3<float> ri = R[e], rj = R[(e + 1) % 3];
        float li = L[e], lj = L[(e + 1) % 3];
        float p = dot(ri, rj);
        float num = li + lj + S.len[e];
        float q;
        if (p < 0.f) {
            float c2 = norm2(cross(ri, rj));
            if (c2 < g.edge_sin2 * (li * li) * (lj * lj)) return false;
            q = (li * lj - p) / (2.f * c2);
            wt += logf(num * num * q) * S.nu[e];
        } else {
            wt += log1pf(S.len[e] * num / (li * lj + p)) * S.nu[e];
        }
    }
    float Om;
    if (side != 0) {
        Om = float(side) * 2.f * vp_pi<float>();
    } else {
        float P3 = la * lb * lc;
        float N = dot(ra, cross(rb, rc));
        float D = P3 + dot(ra, rb) * lc + dot(ra, rc) * lb + dot(rb, rc) * la;
        if (fabsf(N) < g.plane * P3 && (D < 0.f || fabsf(D) < g.plane * P3)) return false;
        Om = 2.f * atan2f(N, D);
    }
    w = (wt + Om * S.n) * (1.f / (4.f * vp_pi<float>()));
    return true;
}

// source_velocity_far (source_triangle.jl:100-119): monopole + quadrupole + octupole about the centroid
template <class T>
__device__ __forceinline__ v3<T> sv_far(const SrcKern<T>& S, v3<T> r) {
    T R2 = dot(r, r);
    T iR2, iR3;
    inv_r23(R2, iR2, iR3);
    T iR5 = iR3 * iR2, iR7 = iR5 * iR2, iR9 = iR7 * iR2;
    v3<T> w = iR3 * r;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        v3<T> d = S.d[a];
        T dr = dot(d, r), dd = dot(d, d);
        v3<T> quad = (T(15) * dr * dr * iR7) * r - (T(6) * dr * iR5) * d - (T(3) * dd * iR5) * r;
        v3<T> oct = (T(45) * dr * dr * iR7) * d - (T(105) * dr * dr * dr * iR9) * r - (T(9) * dd * iR5) * d +
                    (T(45) * dd * dr * iR7) * r;
        w += quad * (T(1) / T(24)) - oct * (T(1) / T(180));
    }
    return (S.area / (T(4) * vp_pi<T>())) * w;
}

// source_velocity (source_triangle.jl:134-138) at x = c + r
template <class T>
__device__ __forceinline__ v3<T> sv_rel(const SrcKern<T>& S, v3<T> r, int side, T far, T plane_tol) {
    T fd = far * S.diam;
    if (dot(r, r) > fd * fd) return sv_far(S, r);
    return sv_exact3(S, r - S.d[0], r - S.d[1], r - S.d[2], r, side, plane_tol);
}

// segment_velocity (segment.jl:15-25)
template <class T>
__device__ __forceinline__ void segment_velocity(v3<T> ra, v3<T> rb, v3<T>& va, v3<T>& vb) {
    T Ra = vnorm(ra), Rb = vnorm(rb);
    v3<T> c = cross(ra, rb);
    T p = dot(ra, rb);
    T den = p >= T(0) ? Ra * Rb + p : norm2(c) / (Ra * Rb - p);
    if (den == T(0) || Ra == T(0) || Rb == T(0)) {
        va = mk3<T>(0, 0, 0);
        vb = va;
        return;
    }
    v3<T> f = c / (T(4) * vp_pi<T>() * den);
    va = f / Ra;
    vb = f / Rb;
}

// test_weights (assemble.jl:52-58): 0 hat, 1 onering, 2 dual
template <class T>
__device__ __forceinline__ v3<T> test_weights(int test, T l0, T l1, T l2) {
    if (test == 0) return mk3(l0, l1, l2);
    if (test == 1) return mk3(T(1), T(1), T(1));
    T m = fmax(l0, fmax(l1, l2));
    T a = fabs(l0 - m) < T(1e-12) ? T(1) : T(0);
    T b = fabs(l1 - m) < T(1e-12) ? T(1) : T(0);
    T c = fabs(l2 - m) < T(1e-12) ? T(1) : T(0);
    T s = a + b + c;
    return mk3(a / s, b / s, c / s);
}
