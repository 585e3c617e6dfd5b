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

__device__ __forceinline__ float vsqrt(float a) { return sqrtf(a); }
__device__ __forceinline__ double vsqrt(double a) { return sqrt(a); }
__device__ __forceinline__ float vlog(float a) { return logf(a); }
__device__ __forceinline__ double vlog(double a) { return log(a); }
__device__ __forceinline__ float vatan2(float a, float b) { return atan2f(a, b); }
__device__ __forceinline__ double vatan2(double a, double b) { return atan2(a, b); }
__device__ __forceinline__ float vacos(float a) { return acosf(a); }
__device__ __forceinline__ double vacos(double a) { return acos(a); }
template <class T> __device__ __forceinline__ T vnorm(v3<T> a) { return vsqrt(dot(a, a)); }

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

// edge_log (source_triangle.jl:39-44): ln((r_i + r_j + d)^2 / (2(r_i r_j + ri.rj))), cancellation-free denominator
template <class T>
__device__ __forceinline__ T edge_log(v3<T> ri, v3<T> rj, T d) {
    T a = vnorm(ri), b = vnorm(rj);
    T p = dot(ri, rj);
    T s2d2 = p < T(0) ? T(2) * norm2(cross(ri, rj)) / (a * b - p) : T(2) * (a * b + p);
    T num = a + b + d;
    return vlog(num * num / s2d2);
}

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

// source_velocity_exact (source_triangle.jl:75-89) from the point's offsets to the three vertices ra, rb, rc
// (r_a = x - v_a) and to the centroid r = x - c.
template <class T>
__device__ __forceinline__ v3<T> sv_exact3(const SrcKern<T>& S, v3<T> ra, v3<T> rb, v3<T> rc, v3<T> r, int side,
                                           T plane_tol) {
    v3<T> wt = edge_log(ra, rb, S.len[0]) * S.nu[0] + edge_log(rb, rc, S.len[1]) * S.nu[1] +
               edge_log(rc, ra, S.len[2]) * S.nu[2];
    T z = dot(r, S.n);
    T Om;
    if (fabs(z) <= plane_tol * S.diam) {
        v3<T> q[3] = {-ra, -rb, -rc};
        Om = side == 0 ? T(0) : T(side) * T(2) * vp_pi<T>() * inplane_fraction_rel(q, S.n, S.area, plane_tol);
    } else {
        T la = vnorm(ra), lb = vnorm(rb), lc = vnorm(rc);
        T N = dot(ra, cross(rb, rc));
        T D = la * lb * lc + dot(ra, rb) * lc + dot(ra, rc) * lb + dot(rb, rc) * la;
        Om = T(2) * vatan2(N, D);
    }
    return (wt + Om * S.n) * (T(1) / (T(4) * vp_pi<T>()));
}

// source_velocity_far (source_triangle.jl:100-119): monopole + quadrupole + octupole about the centroid
template <class T>
__device__ __forceinline__ v3<T> sv_far(const SrcKern<T>& S, v3<T> r) {
    T R2 = dot(r, r);
    T R = vsqrt(R2);
    T iR2 = T(1) / R2, iR3 = iR2 / R, iR5 = iR3 * iR2, iR7 = iR5 * iR2, iR9 = iR7 * iR2;
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
