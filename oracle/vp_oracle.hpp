// CPU oracle of the VortexPanel.jl Galerkin hot path: a restatement, in FP64 C++, of the reference's
// source-triangle, filament and blob kernels, quadrature rules, quadrature tiers, pair blocks, assembly and
// explicit right hand side. TEST INFRASTRUCTURE ONLY: the parity tests, smoke() and the bench's CPU-baseline leg
// use it as the checker; nothing in the product links or calls it.
//
// Every function cites the reference file (paths within the VortexPanel.jl project) and lines it follows.
#pragma once
#include <array>
#include <cmath>
#include <vector>

namespace vpo {

template <class T>
struct V3 {
    T x, y, z;
    V3() : x(0), y(0), z(0) {}
    V3(T a, T b, T c) : x(a), y(b), z(c) {}
    T& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    const T& operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
template <class T> inline V3<T> operator+(const V3<T>& a, const V3<T>& b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T> inline V3<T> operator-(const V3<T>& a, const V3<T>& b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T> inline V3<T> operator-(const V3<T>& a) { return {-a.x, -a.y, -a.z}; }
template <class T> inline V3<T> operator*(const T& s, const V3<T>& a) { return {s * a.x, s * a.y, s * a.z}; }
template <class T> inline V3<T> operator*(const V3<T>& a, const T& s) { return {s * a.x, s * a.y, s * a.z}; }
template <class T> inline V3<T> operator/(const V3<T>& a, const T& s) { return {a.x / s, a.y / s, a.z / s}; }
template <class T> inline V3<T>& operator+=(V3<T>& a, const V3<T>& b) { a.x += b.x; a.y += b.y; a.z += b.z; return a; }
template <class T> inline V3<T>& operator-=(V3<T>& a, const V3<T>& b) { a.x -= b.x; a.y -= b.y; a.z -= b.z; return a; }
template <class T> inline T dot(const V3<T>& a, const V3<T>& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T> inline V3<T> cross(const V3<T>& a, const V3<T>& b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <class T> inline T norm2(const V3<T>& a) { return dot(a, a); }
template <class T> inline T norm(const V3<T>& a) { using std::sqrt; return sqrt(dot(a, a)); }

typedef V3<double> Vec;
typedef std::array<double, 3> Bary;

// ---- kernels (src/kernels/source_triangle.jl, segment.jl, blob.jl) ----

// SourceTriangle (source_triangle.jl:8-26)
template <class T>
struct SourceTri {
    V3<T> v[3], n, c;
    T area, diam;
    V3<T> nu[3];
    T len[3];
};

template <class T>
bool make_source_tri(const V3<T>& a, const V3<T>& b, const V3<T>& c, SourceTri<T>& s) {
    using std::sqrt;
    V3<T> nA = cross(b - a, c - a);
    T A2 = norm(nA);
    if (!(A2 > T(0))) return false;
    s.v[0] = a; s.v[1] = b; s.v[2] = c;
    s.n = nA / A2;
    s.len[0] = norm(b - a); s.len[1] = norm(c - b); s.len[2] = norm(a - c);
    s.nu[0] = cross(b - a, s.n) / s.len[0];
    s.nu[1] = cross(c - b, s.n) / s.len[1];
    s.nu[2] = cross(a - c, s.n) / s.len[2];
    s.c = (a + b + c) / T(3);
    s.area = A2 / T(2);
    s.diam = s.len[0];
    if (s.len[1] > s.diam) s.diam = s.len[1];
    if (s.len[2] > s.diam) s.diam = s.len[2];
    return true;
}

// edge_log (source_triangle.jl:39-44)
template <class T>
inline T edge_log(const V3<T>& ri, const V3<T>& rj, T d) {
    using std::log;
    T a = norm(ri), b = norm(rj);
    T p = dot(ri, rj);
    T s2d2 = p < T(0) ? T(2) * norm2(cross(ri, rj)) / (a * b - p) : T(2) * (a * b + p);
    T num = a + b + d;
    return log(num * num / s2d2);
}

// inplane_fraction (source_triangle.jl:52-64)
template <class T>
T inplane_fraction(const SourceTri<T>& tri, const V3<T>& x, double tol) {
    using std::acos;
    const V3<T>&a = tri.v[0], &b = tri.v[1], &c = tri.v[2];
    T A2 = T(2) * tri.area;
    T l[3] = {dot(cross(b - x, c - x), tri.n) / A2, dot(cross(c - x, a - x), tri.n) / A2,
              dot(cross(a - x, b - x), tri.n) / A2};
    for (int k = 0; k < 3; ++k)
        if (l[k] < -tol) return T(0);
    int nzero = 0;
    for (int k = 0; k < 3; ++k)
        if (std::fabs(double(l[k])) <= tol) ++nzero;
    if (nzero == 0) return T(1);
    if (nzero == 1) return T(0.5);
    int k = 0;
    while (k < 3 && !(std::fabs(double(l[k])) > tol)) ++k;
    V3<T> e1 = tri.v[(k + 1) % 3] - tri.v[k], e2 = tri.v[(k + 2) % 3] - tri.v[k];
    T cs = dot(e1, e2) / (norm(e1) * norm(e2));
    if (cs < T(-1)) cs = T(-1);
    if (cs > T(1)) cs = T(1);
    return acos(cs) / (T(2) * T(M_PI));
}

// numbers that carry derivatives (the derivative oracle's duals) take the in-plane branch's value with the
// derivatives of the off-plane solid angle: the in-plane set has measure zero, so under any move of the geometry the
// solid angle of such a point follows the off-plane formula
template <class T>
struct carries_derivatives {
    static const bool value = false;
};
template <class T>
inline T plane_limit(const T& in_plane, const T&) { return in_plane; }

// the solid angle of the triangle seen from offsets ra, rb, rc (Van Oosterom-Strackee), source_triangle.jl:85-87
template <class T>
inline T solid_angle(const V3<T>& ra, const V3<T>& rb, const V3<T>& rc) {
    using std::atan2;
    T la = norm(ra), lb = norm(rb), lc = norm(rc);
    T N = dot(ra, cross(rb, rc));
    T D = la * lb * lc + dot(ra, rb) * lc + dot(ra, rc) * lb + dot(rb, rc) * la;
    return T(2) * atan2(N, D);
}

// source_velocity_exact (source_triangle.jl:75-89)
template <class T>
V3<T> source_velocity_exact(const SourceTri<T>& tri, const V3<T>& x, int side, double plane_tol) {
    V3<T> ra = x - tri.v[0], rb = x - tri.v[1], rc = x - tri.v[2];
    V3<T> wt = edge_log(ra, rb, tri.len[0]) * tri.nu[0] + edge_log(rb, rc, tri.len[1]) * tri.nu[1] +
               edge_log(rc, ra, tri.len[2]) * tri.nu[2];
    T z = dot(x - tri.c, tri.n);
    T Om;
    if (std::fabs(double(z)) <= plane_tol * double(tri.diam)) {
        Om = T(side) * T(2) * T(M_PI) * inplane_fraction(tri, x, plane_tol);
        if (carries_derivatives<T>::value) Om = plane_limit(Om, solid_angle(ra, rb, rc));
    } else {
        Om = solid_angle(ra, rb, rc);
    }
    return (wt + Om * tri.n) / (T(4) * T(M_PI));
}

// source_velocity_far (source_triangle.jl:100-119)
template <class T>
V3<T> source_velocity_far(const SourceTri<T>& tri, const V3<T>& x) {
    using std::sqrt;
    V3<T> r = x - tri.c;
    T R2 = dot(r, r);
    T R = sqrt(R2);
    T iR2 = T(1) / R2, iR3 = iR2 / R, iR5 = iR3 * iR2, iR7 = iR5 * iR2, iR9 = iR7 * iR2;
    V3<T> w = iR3 * r;
    for (int a = 0; a < 3; ++a) {
        V3<T> d = tri.v[a] - tri.c;
        T dr = dot(d, r), dd = dot(d, d);
        V3<T> quad = (T(15) * dr * dr * iR7) * r - (T(6) * dr * iR5) * d - (T(3) * dd * iR5) * r;
        V3<T> oct = (T(45) * dr * dr * iR7) * d - (T(105) * dr * dr * dr * iR9) * r - (T(9) * dd * iR5) * d +
                    (T(45) * dd * dr * iR7) * r;
        w += quad / T(24) - oct / T(180);
    }
    return (tri.area / (T(4) * T(M_PI))) * w;
}

// source_velocity (source_triangle.jl:134-138)
template <class T>
V3<T> source_velocity(const SourceTri<T>& tri, const V3<T>& x, int side, double far, double plane_tol = 1e-12) {
    V3<T> r = x - tri.c;
    if (double(dot(r, r)) > (far * double(tri.diam)) * (far * double(tri.diam))) return source_velocity_far(tri, x);
    return source_velocity_exact(tri, x, side, plane_tol);
}

// segment_velocity (segment.jl:15-25)
template <class T>
void segment_velocity(const V3<T>& a, const V3<T>& b, const V3<T>& x, V3<T>& va, V3<T>& vb) {
    V3<T> ra = x - a, rb = x - b;
    T Ra = norm(ra), Rb = norm(rb);
    V3<T> c = cross(ra, rb);
    T p = dot(ra, rb);
    T den = p >= T(0) ? Ra * Rb + p : norm2(c) / (Ra * Rb - p);
    if (den == T(0) || Ra == T(0) || Rb == T(0)) {
        va = V3<T>();
        vb = V3<T>();
        return;
    }
    V3<T> f = c / (T(4) * T(M_PI) * den);
    va = f / Ra;
    vb = f / Rb;
}

// blob_velocity (blob.jl:21-25)
template <class T>
V3<T> blob_velocity(const V3<T>& x, const V3<T>& xp, const V3<T>& al, T delta) {
    using std::sqrt;
    V3<T> r = x - xp;
    T d2 = dot(r, r) + delta * delta;
    return cross(al, r) / (T(4) * T(M_PI) * d2 * sqrt(d2));
}

// ---- elements (src/elements/flat_triangle.jl:12-31, 59-78) ----
template <class T>
struct FlatTriT {
    V3<T> x[3], n, c;
    T area, diam;
    V3<T> gradl[3], gam[3];
    SourceTri<T> src;
};
typedef FlatTriT<double> FlatTri;
template <class T>
bool make_flat_tri(const V3<T>& a, const V3<T>& b, const V3<T>& c, FlatTriT<T>& t);
template <class T, class B>
inline V3<T> point(const FlatTriT<T>& Tr, const B& l) {
    return T(l[0]) * Tr.x[0] + T(l[1]) * Tr.x[1] + T(l[2]) * Tr.x[2];
}

template <class T>
struct SegmentT {
    V3<T> a, b;
};
typedef SegmentT<double> Segment;
struct Blob {
    Vec x, al;
    double delta;
};
double distance_to(const Blob& b, const Vec& p);

// ---- rules (src/elements/rules.jl) ----
template <class T>
using BaryT = std::array<T, 3>;
template <class T>
struct RuleT {
    std::vector<BaryT<T>> lam;
    std::vector<T> w;
    size_t size() const { return w.size(); }
    void clear() { lam.clear(); w.clear(); }
};
typedef RuleT<double> Rule;
void gauss_legendre(int n, std::vector<double>& x, std::vector<double>& w);
void graded_gauss(int levels, double ratio, int order, std::vector<double>& x, std::vector<double>& w);
void graded_gauss_both(int levels, double ratio, int order, std::vector<double>& x, std::vector<double>& w);
Rule triangle_rule(int n);
Rule rotate_rule(const Rule& r, int k);  // k = 0,1,2 (0-based corner)
Rule edge_graded_rule(int levels, double ratio, int order);
Rule vertex_graded_rule(int levels, double ratio, int order);
Rule self_rule(int levels, double ratio, int order);

struct TierRules {
    Rule far, near_, self, edge[3], vertex[3];
};

// AssemblyOptions (src/assembly/assemble.jl:26-41); test: 0 hat, 1 onering, 2 dual
struct Options {
    int test = 0;
    double far_ratio = 3.0;
    int far_points = 3;
    int near_points = 7;
    double near_ratio = 1.5;
    int near_depth = 3;
    int touch_levels = 6;
    double touch_ratio = 0.15;
    int touch_order = 3;
    double corner_angle = 75.0;
    double contact_rel = 0.1;
    double kernel_far = 10.0;
};
TierRules tier_rules(const Options& o);

enum Tier { SELF = 0, EDGE = 1, VERTEX = 2, CONTACT = 3, NEAR = 4, FAR = 5 };

}  // namespace vpo
