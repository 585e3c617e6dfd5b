// CPU oracle of the VortexPanel.jl Galerkin hot path (FP64). TEST INFRASTRUCTURE ONLY: used by tests/,
// smoke() and the bench's CPU-baseline leg as the checker, never by the product path.
//
// Restates, function by function (reference file:line in each comment):
//   src/elements/rules.jl             quadrature rules
//   src/elements/flat_triangle.jl     FlatTriangle, distance_to
//   src/assembly/assemble.jl          tiers (near/vertex/contact rules), pair_block, segment_block, assemble
//   src/assembly/explicit.jl          explicit_rhs
//   src/post/Post.jl                  body_velocity
//   src/freewake/step.jl              blob_velocities
#include "vp_oracle.hpp"
#include "vp_dual.hpp"

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <set>
#include <utility>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace vpo {

// FlatTriangle (flat_triangle.jl:12-31)
template <class T>
bool make_flat_tri(const V3<T>& a, const V3<T>& b, const V3<T>& c, FlatTriT<T>& t) {
    if (!make_source_tri(a, b, c, t.src)) return false;
    t.x[0] = a; t.x[1] = b; t.x[2] = c;
    t.n = t.src.n;
    t.area = t.src.area;
    t.c = t.src.c;
    t.diam = t.src.diam;
    T A2 = T(2) * t.area;
    V3<T> e[3] = {c - b, a - c, b - a};
    for (int k = 0; k < 3; ++k) {
        t.gradl[k] = cross(t.n, e[k]) / A2;
        t.gam[k] = -e[k] / A2;
    }
    return true;
}
template bool make_flat_tri<double>(const Vec&, const Vec&, const Vec&, FlatTri&);

// reach (flat_triangle.jl:56)
template <class T>
T reach(const FlatTriT<T>& el) {
    return std::max({norm(el.x[0] - el.c), norm(el.x[1] - el.c), norm(el.x[2] - el.c)});
}

// distance_to (flat_triangle.jl:59-78), closest point after Ericson 5.1.5
template <class T>
T distance_to(const FlatTriT<T>& el, const V3<T>& p) {
    const V3<T> &a = el.x[0], &b = el.x[1], &c = el.x[2];
    V3<T> ab = b - a, ac = c - a, ap = p - a;
    T d1 = dot(ab, ap), d2 = dot(ac, ap);
    if (d1 <= 0 && d2 <= 0) return norm(ap);
    V3<T> bp = p - b;
    T d3 = dot(ab, bp), d4 = dot(ac, bp);
    if (d3 >= 0 && d4 <= d3) return norm(bp);
    T vc = d1 * d4 - d3 * d2;
    if (vc <= 0 && d1 >= 0 && d3 <= 0) return norm(p - (a + (d1 / (d1 - d3)) * ab));
    V3<T> cp = p - c;
    T d5 = dot(ab, cp), d6 = dot(ac, cp);
    if (d6 >= 0 && d5 <= d6) return norm(cp);
    T vb = d5 * d2 - d1 * d6;
    if (vb <= 0 && d2 >= 0 && d6 <= 0) return norm(p - (a + (d2 / (d2 - d6)) * ac));
    T va = d3 * d6 - d5 * d4;
    if (va <= 0 && d4 - d3 >= 0 && d5 - d6 >= 0) return norm(p - (b + ((d4 - d3) / ((d4 - d3) + (d5 - d6))) * (c - b)));
    T denom = T(1) / (va + vb + vc);
    return norm(p - (a + (vb * denom) * ab + (vc * denom) * ac));
}

// segment_projection (assemble.jl:145-149)
template <class T>
static void segment_projection(const V3<T>& p, const V3<T>& a, const V3<T>& c, T& d, T& t) {
    V3<T> e = c - a;
    t = dot(p - a, e) / dot(e, e);
    t = std::min(std::max(t, T(0)), T(1));
    d = norm(p - (a + t * e));
}

// distance_to(::Segment) (assemble.jl:157), distance_to(::Blob) (explicit.jl:20)
template <class T>
T distance_to(const SegmentT<T>& s, const V3<T>& p) {
    T d, t;
    segment_projection(p, s.a, s.b, d, t);
    return d;
}
double distance_to(const Blob& b, const Vec& p) { return norm(p - b.x); }

// ---- rules (rules.jl) ----

// gauss_legendre (rules.jl:12-37)
void gauss_legendre(int n, std::vector<double>& x, std::vector<double>& w) {
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

// graded_gauss (rules.jl:48-64)
void graded_gauss(int levels, double ratio, int order, std::vector<double>& x, std::vector<double>& w) {
    std::vector<double> br;
    br.push_back(0.0);
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

// graded_gauss_both (rules.jl:66-70)
void graded_gauss_both(int levels, double ratio, int order, std::vector<double>& x, std::vector<double>& w) {
    std::vector<double> x0, w0;
    graded_gauss(levels, ratio, order, x0, w0);
    size_t n = x0.size();
    x.resize(2 * n);
    w.resize(2 * n);
    for (size_t i = 0; i < n; ++i) {
        x[i] = x0[i] / 2;
        w[i] = w0[i] / 2;
        x[n + i] = 1 - x0[n - 1 - i] / 2;
        w[n + i] = w0[n - 1 - i] / 2;
    }
}

// triangle_rule (rules.jl:76-92)
Rule triangle_rule(int n) {
    Rule r;
    auto perm = [&](double a, double b, double wt) {
        r.lam.push_back({a, b, b}); r.w.push_back(wt);
        r.lam.push_back({b, a, b}); r.w.push_back(wt);
        r.lam.push_back({b, b, a}); r.w.push_back(wt);
    };
    if (n == 1) {
        r.lam.push_back({1.0 / 3, 1.0 / 3, 1.0 / 3});
        r.w.push_back(1.0);
    } else if (n == 3) {
        perm(2.0 / 3, 1.0 / 6, 1.0 / 3);
    } else if (n == 6) {
        double a = 0.445948490915965, b = 0.091576213509771;
        perm(1 - 2 * a, a, 0.223381589678011);
        perm(1 - 2 * b, b, 0.109951743655322);
    } else if (n == 7) {
        double s = std::sqrt(15.0);
        double a = (6 - s) / 21, b = (6 + s) / 21;
        r.lam.push_back({1.0 / 3, 1.0 / 3, 1.0 / 3});
        r.w.push_back(9.0 / 40);
        perm(1 - 2 * a, a, (155 - s) / 1200);
        perm(1 - 2 * b, b, (155 + s) / 1200);
    }
    return r;
}

// rotate_rule (rules.jl:95-99); k is 0-based here, rotating base corner 0 to corner k
Rule rotate_rule(const Rule& r, int k) {
    if (k == 0) return r;
    Rule o;
    o.w = r.w;
    for (const Bary& l : r.lam) {
        Bary m;
        // lambda_T[(k + j) % 3] = lambda_base[j]
        for (int j = 0; j < 3; ++j) m[(k + j) % 3] = l[j];
        o.lam.push_back(m);
    }
    return o;
}

// edge_graded_rule (rules.jl:108-118)
Rule edge_graded_rule(int levels, double ratio, int order) {
    std::vector<double> ts, wt, ss, ws;
    graded_gauss(levels, ratio, order, ts, wt);
    graded_gauss_both(std::max(1, levels / 2), ratio, order, ss, ws);
    Rule r;
    for (size_t i = 0; i < ts.size(); ++i)
        for (size_t j = 0; j < ss.size(); ++j) {
            double t = ts[i], s = ss[j];
            r.lam.push_back({(1 - t) * (1 - s), (1 - t) * s, t});
            r.w.push_back(2 * (1 - t) * wt[i] * ws[j]);
        }
    return r;
}

// vertex_graded_rule (rules.jl:125-135)
Rule vertex_graded_rule(int levels, double ratio, int order) {
    std::vector<double> rs, wr, ss, ws;
    graded_gauss(levels, ratio, order, rs, wr);
    gauss_legendre(order + levels, ss, ws);
    Rule r;
    for (size_t i = 0; i < rs.size(); ++i)
        for (size_t j = 0; j < ss.size(); ++j) {
            double rho = rs[i], s = ss[j];
            r.lam.push_back({1 - rho, rho * (1 - s), rho * s});
            r.w.push_back(2 * rho * wr[i] * ws[j]);
        }
    return r;
}

// self_rule (rules.jl:142-156)
Rule self_rule(int levels, double ratio, int order) {
    Rule base = edge_graded_rule(levels, ratio, order);
    Rule r;
    for (int k = 0; k < 3; ++k)
        for (size_t i = 0; i < base.size(); ++i) {
            const Bary& m = base.lam[i];
            Bary l = {m[2] / 3, m[2] / 3, m[2] / 3};
            l[k] += m[0];
            l[(k + 1) % 3] += m[1];
            r.lam.push_back(l);
            r.w.push_back(base.w[i] / 3);
        }
    return r;
}

// TierRules (rules.jl:161-174), tier_rules (assemble.jl:48-49)
TierRules tier_rules(const Options& o) {
    TierRules t;
    t.far = triangle_rule(o.far_points);
    t.near_ = triangle_rule(o.near_points);
    t.self = self_rule(o.touch_levels, o.touch_ratio, o.touch_order);
    Rule e = edge_graded_rule(o.touch_levels, o.touch_ratio, o.touch_order);
    Rule v = vertex_graded_rule(o.touch_levels, o.touch_ratio, o.touch_order);
    for (int k = 0; k < 3; ++k) {
        t.edge[k] = rotate_rule(e, k);
        t.vertex[k] = rotate_rule(v, k);
    }
    return t;
}

// ---- tiers (assemble.jl:52-321) ----
// The pieces, rules and blocks are templates on the scalar type: double for the oracle, a forward-mode dual number
// for the derivative oracle. Decisions (tiers, splits, wedge counts) compare values; the base rules stay double.

template <class T>
inline double val(const T& x) { return double(x); }

// test_weights (assemble.jl:52-58)
template <class T>
static inline V3<T> test_weights(int test, const BaryT<T>& l) {
    if (test == 0) return V3<T>(l[0], l[1], l[2]);
    if (test == 1) return V3<T>(T(1), T(1), T(1));
    double m = std::max({val(l[0]), val(l[1]), val(l[2])});
    double is[3];
    int cnt = 0;
    for (int k = 0; k < 3; ++k) {
        is[k] = std::fabs(val(l[k]) - m) < 1e-12 ? 1.0 : 0.0;
        cnt += int(is[k]);
    }
    return V3<T>(T(is[0] / cnt), T(is[1] / cnt), T(is[2] / cnt));
}

// test_integrals (assemble.jl:61)
static inline Vec test_integrals(int test) { return test == 1 ? Vec(1, 1, 1) : Vec(1.0 / 3, 1.0 / 3, 1.0 / 3); }

template <class T>
using CornersT = std::array<BaryT<T>, 3>;
typedef CornersT<double> Corners;
template <class T>
static CornersT<T> unit_corners() {
    return {BaryT<T>{T(1), T(0), T(0)}, BaryT<T>{T(0), T(1), T(0)}, BaryT<T>{T(0), T(0), T(1)}};
}

template <class T>
static inline BaryT<T> bmix(const BaryT<T>& a, const T& sa, const BaryT<T>& b, const T& sb) {
    return {sa * a[0] + sb * b[0], sa * a[1] + sb * b[1], sa * a[2] + sb * b[2]};
}

// append_piece! (assemble.jl:85-91)
template <class T>
static void append_piece(RuleT<T>& out, const Rule& r, const CornersT<T>& b, const T& frac) {
    for (size_t i = 0; i < r.size(); ++i) {
        const Bary& m = r.lam[i];
        BaryT<T> l;
        for (int j = 0; j < 3; ++j) l[j] = T(m[0]) * b[0][j] + T(m[1]) * b[1][j] + T(m[2]) * b[2][j];
        out.lam.push_back(l);
        out.w.push_back(T(r.w[i]) * frac);
    }
}

// a stored rule as the pair's rule: itself in double, a constant copy in another scalar type
static const Rule* as_rule(const Rule& r, Rule&) { return &r; }
template <class T>
static const RuleT<T>* as_rule(const Rule& r, RuleT<T>& buf) {
    buf.clear();
    append_piece(buf, r, unit_corners<T>(), T(1));
    return &buf;
}

// quarters (assemble.jl:79-82)
template <class T>
static std::array<CornersT<T>, 4> quarters(const CornersT<T>& b) {
    const T h(0.5);
    BaryT<T> m12 = bmix(b[0], h, b[1], h), m23 = bmix(b[1], h, b[2], h), m31 = bmix(b[2], h, b[0], h);
    return {CornersT<T>{b[0], m12, m31}, CornersT<T>{m12, b[1], m23}, CornersT<T>{m31, m23, b[2]},
            CornersT<T>{m12, m23, m31}};
}

// near_pieces! (assemble.jl:131-142)
template <class T, class S>
static void near_pieces(RuleT<T>& out, const FlatTriT<T>& Tr, const S& src, const Rule& base, double ratio, int depth,
                        const CornersT<T>& b, const T& frac, int level) {
    V3<T> p1 = point(Tr, b[0]), p2 = point(Tr, b[1]), p3 = point(Tr, b[2]);
    T size = std::max({norm(p2 - p1), norm(p3 - p2), norm(p1 - p3)});
    if (level < depth && distance_to(src, (p1 + p2 + p3) / T(3)) < T(ratio) * size) {
        for (const CornersT<T>& sub : quarters(b))
            near_pieces(out, Tr, src, base, ratio, depth, sub, frac / T(4), level + 1);
    } else {
        append_piece(out, base, b, frac);
    }
}

// vertex_pieces! (assemble.jl:102-116); k 0-based
template <class T>
static void vertex_pieces(RuleT<T>& out, const V3<T> p[3], int k, const Rule& base, const CornersT<T>& b,
                          const T& frac, double corner_angle) {
    using std::acos;
    using std::sin;
    int i = (k + 1) % 3, j = (k + 2) % 3;
    V3<T> u = p[i] - p[k], v = p[j] - p[k];
    T cs = dot(u, v) / (norm(u) * norm(v));
    T th = acos(std::min(std::max(cs, T(-1.0)), T(1.0)));
    if (th <= T(M_PI / 2)) {
        append_piece(out, base, CornersT<T>{b[k], b[i], b[j]}, frac);
        return;
    }
    int m = int(std::ceil(val(th) * (180.0 / M_PI) / corner_angle));  // rad2deg(θ) = θ * (180 / π), as Julia
    std::vector<T> ts(m + 1);
    ts[0] = T(0);
    ts[m] = T(1);
    T nu = norm(u), nv = norm(v);
    for (int q = 1; q < m; ++q) {
        T phi = th * T(q) / T(m);
        ts[q] = nu * sin(phi) / (nu * sin(phi) + nv * sin(th - phi));
    }
    for (int q = 0; q < m; ++q) {
        BaryT<T> b1 = bmix(b[i], T(1) - ts[q], b[j], ts[q]), b2 = bmix(b[i], T(1) - ts[q + 1], b[j], ts[q + 1]);
        append_piece(out, base, CornersT<T>{b[k], b1, b2}, frac * (ts[q + 1] - ts[q]));
    }
}

// vertex_rule (assemble.jl:119-125); returns a pointer to the stored rule or fills `buf`
template <class T>
static const RuleT<T>* vertex_rule(const FlatTriT<T>& Tr, int k, const TierRules& rules, const Options& o,
                                   RuleT<T>& buf) {
    V3<T> u = Tr.x[(k + 1) % 3] - Tr.x[k], v = Tr.x[(k + 2) % 3] - Tr.x[k];
    if (dot(u, v) >= 0) return as_rule(rules.vertex[k], buf);
    buf.clear();
    vertex_pieces(buf, Tr.x, k, rules.vertex[0], unit_corners<T>(), T(1), o.corner_angle);
    return &buf;
}

// edge_splits / splits_an_edge (assemble.jl:160-184); S is a flat triangle
template <class T>
static void edge_splits(const V3<T> p[3], const FlatTriT<T>& S, const T& tol, std::vector<T> ts[3]) {
    for (int k = 0; k < 3; ++k) {
        ts[k].clear();
        const V3<T> &a = p[k], &c = p[(k + 1) % 3];
        T L = norm(c - a);
        for (int q = 0; q < 3; ++q) {
            T d, t;
            segment_projection(S.x[q], a, c, d, t);
            if (d <= tol && t * L > tol && (T(1) - t) * L > tol) ts[k].push_back(t);
        }
        std::sort(ts[k].begin(), ts[k].end());
    }
}
template <class T>
static bool splits_an_edge(const V3<T> p[3], const FlatTriT<T>& S, const T& tol) {
    for (int k = 0; k < 3; ++k) {
        const V3<T> &a = p[k], &c = p[(k + 1) % 3];
        T L = norm(c - a);
        for (int q = 0; q < 3; ++q) {
            T d, t;
            segment_projection(S.x[q], a, c, d, t);
            if (d <= tol && t * L > tol && (T(1) - t) * L > tol) return true;
        }
    }
    return false;
}

// contact_pieces! (assemble.jl:209-238)
template <class T>
static void contact_pieces(RuleT<T>& out, const FlatTriT<T>& Tr, const FlatTriT<T>& S, const TierRules& rules,
                           const Options& o, const T& tol, const CornersT<T>& b, const T& frac, int level) {
    V3<T> p[3] = {point(Tr, b[0]), point(Tr, b[1]), point(Tr, b[2])};
    if (level < 4) {
        std::vector<T> splits[3];
        edge_splits(p, S, tol, splits);
        int k = -1;
        for (int q = 0; q < 3; ++q)
            if (!splits[q].empty()) { k = q; break; }
        if (k >= 0) {
            std::vector<T> ts;
            ts.push_back(T(0));
            ts.insert(ts.end(), splits[k].begin(), splits[k].end());
            ts.push_back(T(1));
            const BaryT<T> &bk = b[k], &bk1 = b[(k + 1) % 3], &opp = b[(k + 2) % 3];
            for (size_t i = 0; i + 1 < ts.size(); ++i) {
                CornersT<T> piece = {bmix(bk, T(1) - ts[i], bk1, ts[i]), bmix(bk, T(1) - ts[i + 1], bk1, ts[i + 1]),
                                     opp};
                contact_pieces(out, Tr, S, rules, o, tol, piece, frac * (ts[i + 1] - ts[i]), level + 1);
            }
            return;
        }
    }
    bool on[3];
    int nc = 0;
    for (int q = 0; q < 3; ++q) {
        on[q] = distance_to(S, p[q]) <= tol;
        nc += on[q];
    }
    if (nc == 2) {
        int k = !on[2] ? 0 : (!on[0] ? 1 : 2);
        if (distance_to(S, (p[k] + p[(k + 1) % 3]) / T(2)) <= tol) {
            append_piece(out, rules.edge[k], b, frac);
            return;
        }
    }
    if (nc == 1) {
        int k = on[0] ? 0 : (on[1] ? 1 : 2);
        vertex_pieces(out, p, k, rules.vertex[0], b, frac, o.corner_angle);
    } else if (nc == 0) {
        near_pieces(out, Tr, S, rules.near_, o.near_ratio, o.near_depth, b, frac, 0);
    } else {
        append_piece(out, rules.self, b, frac);
    }
}

// contact_rule (assemble.jl:199-207); returns false when S touches T at shared corners only
template <class T>
static bool contact_rule(const FlatTriT<T>& Tr, const FlatTriT<T>& S, const bool shared[3], const TierRules& rules,
                         const Options& o, RuleT<T>& out) {
    T tol = T(o.contact_rel) * std::min(Tr.diam, S.diam);
    if (norm(S.c - Tr.c) > reach(Tr) + reach(S) + tol) return false;
    bool extra = false;
    for (int k = 0; k < 3; ++k)
        if (!shared[k] && distance_to(S, Tr.x[k]) <= tol) extra = true;
    if (!extra) extra = splits_an_edge(Tr.x, S, tol);
    if (!extra) return false;
    out.clear();
    contact_pieces(out, Tr, S, rules, o, tol, unit_corners<T>(), T(1), 0);
    return true;
}

// near_rule (assemble.jl:69-73)
template <class T, class S>
static void near_rule(RuleT<T>& out, const FlatTriT<T>& Tr, const S& src, const Rule& base, double ratio, int depth) {
    out.clear();
    near_pieces(out, Tr, src, base, ratio, depth, unit_corners<T>(), T(1), 0);
}

// pair_rule (assemble.jl:266-282)
template <class T>
static const RuleT<T>* pair_rule(const FlatTriT<T>* els, const int* tris, int t, int s, const TierRules& rules,
                                 const Options& o, const std::set<std::pair<int, int>>& touch, RuleT<T>& buf,
                                 int& tier) {
    const FlatTriT<T> &Tr = els[t], &S = els[s];
    if (s == t) { tier = SELF; return as_rule(rules.self, buf); }
    if (norm(S.c - Tr.c) > T(o.far_ratio) * std::max(Tr.diam, S.diam)) { tier = FAR; return as_rule(rules.far, buf); }
    const int* tri = tris + 3 * t;
    const int* gs = tris + 3 * s;
    bool shared[3];
    int ns = 0;
    for (int k = 0; k < 3; ++k) {
        shared[k] = tri[k] == gs[0] || tri[k] == gs[1] || tri[k] == gs[2];
        ns += shared[k];
    }
    if (contact_rule(Tr, S, shared, rules, o, buf)) { tier = CONTACT; return &buf; }
    if (ns == 2) {
        tier = EDGE;
        return as_rule(rules.edge[(shared[0] && shared[1]) ? 0 : ((shared[1] && shared[2]) ? 1 : 2)], buf);
    }
    if (ns == 1) {
        tier = VERTEX;
        int k = shared[0] ? 0 : (shared[1] ? 1 : 2);
        return vertex_rule(Tr, k, rules, o, buf);
    }
    int depth = touch.count(std::make_pair(t, s)) ? o.near_depth + 4 : o.near_depth;
    tier = NEAR;
    near_rule(buf, Tr, S, rules.near_, o.near_ratio, depth);
    return &buf;
}

// wake_pair_rule (assemble.jl:288-293)
template <class T>
static const RuleT<T>* wake_pair_rule(const FlatTriT<T>& Tr, const FlatTriT<T>& S, const TierRules& rules,
                                      const Options& o, RuleT<T>& buf, int& tier) {
    if (norm(S.c - Tr.c) > T(o.far_ratio) * std::max(Tr.diam, S.diam)) { tier = FAR; return as_rule(rules.far, buf); }
    bool none[3] = {false, false, false};
    if (contact_rule(Tr, S, none, rules, o, buf)) { tier = CONTACT; return &buf; }
    tier = NEAR;
    near_rule(buf, Tr, S, rules.near_, o.near_ratio, o.near_depth);
    return &buf;
}

// segment_rule (assemble.jl:299-306)
template <class T>
static const RuleT<T>* segment_rule(const FlatTriT<T>& Tr, const SegmentT<T>& f, const TierRules& rules,
                                    const Options& o, RuleT<T>& buf, int& tier) {
    T L = norm(f.b - f.a);
    if (norm((f.a + f.b) / T(2) - Tr.c) > T(o.far_ratio) * std::max(Tr.diam, L)) {
        tier = FAR;
        return as_rule(rules.far, buf);
    }
    for (int k = 0; k < 3; ++k)
        if (std::min(norm(Tr.x[k] - f.a), norm(Tr.x[k] - f.b)) <= T(1e-12) * Tr.diam) {
            tier = VERTEX;
            return vertex_rule(Tr, k, rules, o, buf);
        }
    tier = NEAR;
    near_rule(buf, Tr, f, rules.near_, o.near_ratio, o.near_depth);
    return &buf;
}

// pair_block (assemble.jl:245-258)
template <class T>
static void pair_block(const FlatTriT<T>& Tr, const FlatTriT<T>& S, const RuleT<T>& rule, const T& sigS, int test,
                       int side, double kernel_far, T blk[3][3], T rb[3]) {
    for (int a = 0; a < 3; ++a) {
        rb[a] = T(0);
        for (int b = 0; b < 3; ++b) blk[a][b] = T(0);
    }
    for (size_t q = 0; q < rule.size(); ++q) {
        const BaryT<T>& l = rule.lam[q];
        V3<T> w = source_velocity(S.src, point(Tr, l), side, kernel_far);
        T W = rule.w[q] * Tr.area;
        V3<T> v = cross(w, Tr.n);
        T c[3] = {dot(v, S.gam[0]), dot(v, S.gam[1]), dot(v, S.gam[2])};
        V3<T> psi = W * test_weights(test, l);
        T wn = sigS * dot(w, Tr.n);
        for (int a = 0; a < 3; ++a) {
            for (int b = 0; b < 3; ++b) blk[a][b] += psi[a] * c[b];
            rb[a] -= wn * psi[a];
        }
    }
}

// segment_block (assemble.jl:312-321)
template <class T>
static void segment_block(const FlatTriT<T>& Tr, const SegmentT<T>& f, const RuleT<T>& rule, int test, T ca[3],
                          T cb[3]) {
    for (int a = 0; a < 3; ++a) ca[a] = cb[a] = T(0);
    for (size_t q = 0; q < rule.size(); ++q) {
        V3<T> va, vb;
        segment_velocity(f.a, f.b, point(Tr, rule.lam[q]), va, vb);
        V3<T> psi = (rule.w[q] * Tr.area) * test_weights(test, rule.lam[q]);
        T da = dot(va, Tr.n), db = dot(vb, Tr.n);
        for (int a = 0; a < 3; ++a) {
            ca[a] += da * psi[a];
            cb[a] += db * psi[a];
        }
    }
}

static inline Vec vec_at(const double* x, int i) { return Vec(x[3 * i], x[3 * i + 1], x[3 * i + 2]); }

template <class T>
static bool build_elements(int ntri, const V3<T>* X, const int* tris, std::vector<FlatTriT<T>>& els) {
    els.resize(ntri);
    for (int t = 0; t < ntri; ++t)
        if (!make_flat_tri(X[tris[3 * t]], X[tris[3 * t + 1]], X[tris[3 * t + 2]], els[t])) return false;
    return true;
}

static bool build_elements(int ntri, const double* x, const int* tris, std::vector<FlatTri>& els) {
    els.resize(ntri);
    for (int t = 0; t < ntri; ++t)
        if (!make_flat_tri(vec_at(x, tris[3 * t]), vec_at(x, tris[3 * t + 1]), vec_at(x, tris[3 * t + 2]), els[t]))
            return false;
    return true;
}

}  // namespace vpo

using namespace vpo;

// ---- C ABI for the Python test harness (oracle/oracle.py) ----
extern "C" {

struct vpo_options {
    int test;
    double far_ratio;
    int far_points;
    int near_points;
    double near_ratio;
    int near_depth;
    int touch_levels;
    double touch_ratio;
    int touch_order;
    double corner_angle;
    double contact_rel;
    double kernel_far;
};

static Options to_opts(const vpo_options* p) {
    Options o;
    if (!p) return o;
    o.test = p->test;
    o.far_ratio = p->far_ratio;
    o.far_points = p->far_points;
    o.near_points = p->near_points;
    o.near_ratio = p->near_ratio;
    o.near_depth = p->near_depth;
    o.touch_levels = p->touch_levels;
    o.touch_ratio = p->touch_ratio;
    o.touch_order = p->touch_order;
    o.corner_angle = p->corner_angle;
    o.contact_rel = p->contact_rel;
    o.kernel_far = p->kernel_far;
    return o;
}

int vpo_version(void) { return 1; }

// source_velocity of the triangle abc (9 doubles) at x; far = kernel far switch (inf disables)
int vpo_source_velocity(const double* abc, const double* x, int side, double far, double plane_tol, double* w) {
    SourceTri<double> s;
    if (!make_source_tri(vec_at(abc, 0), vec_at(abc, 1), vec_at(abc, 2), s)) return -1;
    Vec r = source_velocity(s, vec_at(x, 0), side, far, plane_tol);
    w[0] = r.x; w[1] = r.y; w[2] = r.z;
    return 0;
}

int vpo_source_velocity_parts(const double* abc, const double* x, int which, double* w) {
    SourceTri<double> s;
    if (!make_source_tri(vec_at(abc, 0), vec_at(abc, 1), vec_at(abc, 2), s)) return -1;
    Vec r = which == 0 ? source_velocity_exact(s, vec_at(x, 0), 0, 1e-12) : source_velocity_far(s, vec_at(x, 0));
    w[0] = r.x; w[1] = r.y; w[2] = r.z;
    return 0;
}

double vpo_inplane_fraction(const double* abc, const double* x, double tol) {
    SourceTri<double> s;
    if (!make_source_tri(vec_at(abc, 0), vec_at(abc, 1), vec_at(abc, 2), s)) return -1;
    return inplane_fraction(s, vec_at(x, 0), tol);
}

void vpo_segment_velocity(const double* a, const double* b, const double* x, double* va, double* vb) {
    Vec A, B;
    segment_velocity(vec_at(a, 0), vec_at(b, 0), vec_at(x, 0), A, B);
    va[0] = A.x; va[1] = A.y; va[2] = A.z;
    vb[0] = B.x; vb[1] = B.y; vb[2] = B.z;
}

void vpo_blob_velocity(const double* x, const double* xp, const double* al, double delta, double* u) {
    Vec r = blob_velocity(vec_at(x, 0), vec_at(xp, 0), vec_at(al, 0), delta);
    u[0] = r.x; u[1] = r.y; u[2] = r.z;
}

// kind: 0 triangle_rule(n), 1 edge_graded_rule, 2 vertex_graded_rule, 3 self_rule; k rotates to corner k (0-based)
int vpo_rule(int kind, int n, int levels, double ratio, int order, int k, double* lam, double* w, int cap) {
    Rule r;
    if (kind == 0) r = triangle_rule(n);
    else if (kind == 1) r = edge_graded_rule(levels, ratio, order);
    else if (kind == 2) r = vertex_graded_rule(levels, ratio, order);
    else if (kind == 3) r = self_rule(levels, ratio, order);
    else return -1;
    if (k) r = rotate_rule(r, k);
    int m = int(r.size());
    if (lam && w && m <= cap)
        for (int i = 0; i < m; ++i) {
            for (int j = 0; j < 3; ++j) lam[3 * i + j] = r.lam[i][j];
            w[i] = r.w[i];
        }
    return m;
}

// 1-D rules on [0,1]: kind 0 gauss_legendre(n), 1 graded_gauss, 2 graded_gauss_both
int vpo_rule1d(int kind, int n, int levels, double ratio, int order, double* x, double* w, int cap) {
    std::vector<double> xs, ws;
    if (kind == 0) gauss_legendre(n, xs, ws);
    else if (kind == 1) graded_gauss(levels, ratio, order, xs, ws);
    else graded_gauss_both(levels, ratio, order, xs, ws);
    int m = int(xs.size());
    if (x && w && m <= cap)
        for (int i = 0; i < m; ++i) { x[i] = xs[i]; w[i] = ws[i]; }
    return m;
}

// The rule pair_rule picks for test triangle T (9 doubles) and source S, sharing corners by `shared` (3 ints).
// mode 0: body pair (self when same != 0); 1: wake triangle source; 2: filament segment source (S = a, b).
int vpo_pair_rule(const vpo_options* po, const double* Tx, const double* Sx, const int* shared, int same, int mode,
                  int depth_extra, double* lam, double* w, int cap, int* tier_out) {
    Options o = to_opts(po);
    TierRules rules = tier_rules(o);
    FlatTri T;
    if (!make_flat_tri(vec_at(Tx, 0), vec_at(Tx, 1), vec_at(Tx, 2), T)) return -1;
    Rule buf;
    const Rule* r = nullptr;
    int tier = -1;
    if (mode == 2) {
        Segment f{vec_at(Sx, 0), vec_at(Sx, 1)};
        r = segment_rule(T, f, rules, o, buf, tier);
    } else {
        FlatTri S;
        if (!make_flat_tri(vec_at(Sx, 0), vec_at(Sx, 1), vec_at(Sx, 2), S)) return -1;
        if (mode == 1) {
            r = wake_pair_rule(T, S, rules, o, buf, tier);
        } else if (same) {
            tier = SELF;
            r = &rules.self;
        } else if (norm(S.c - T.c) > o.far_ratio * std::max(T.diam, S.diam)) {
            tier = FAR;
            r = &rules.far;
        } else {
            bool sh[3] = {shared[0] != 0, shared[1] != 0, shared[2] != 0};
            int ns = sh[0] + sh[1] + sh[2];
            if (contact_rule(T, S, sh, rules, o, buf)) {
                tier = CONTACT;
                r = &buf;
            } else if (ns == 2) {
                tier = EDGE;
                r = &rules.edge[(sh[0] && sh[1]) ? 0 : ((sh[1] && sh[2]) ? 1 : 2)];
            } else if (ns == 1) {
                tier = VERTEX;
                r = vertex_rule(T, sh[0] ? 0 : (sh[1] ? 1 : 2), rules, o, buf);
            } else {
                tier = NEAR;
                near_rule(buf, T, S, rules.near_, o.near_ratio, o.near_depth + depth_extra);
                r = &buf;
            }
        }
    }
    *tier_out = tier;
    int m = int(r->size());
    if (lam && w && m <= cap)
        for (int i = 0; i < m; ++i) {
            for (int j = 0; j < 3; ++j) lam[3 * i + j] = r->lam[i][j];
            w[i] = r->w[i];
        }
    return m;
}

// pair_block of test T and source S (9 doubles each) with the given rule
int vpo_pair_block(const double* Tx, const double* Sx, const double* lam, const double* w, int n, double sigS,
                   int test, int side, double kernel_far, double* blk, double* rb) {
    FlatTri T, S;
    if (!make_flat_tri(vec_at(Tx, 0), vec_at(Tx, 1), vec_at(Tx, 2), T)) return -1;
    if (!make_flat_tri(vec_at(Sx, 0), vec_at(Sx, 1), vec_at(Sx, 2), S)) return -1;
    Rule r;
    for (int i = 0; i < n; ++i) {
        r.lam.push_back({lam[3 * i], lam[3 * i + 1], lam[3 * i + 2]});
        r.w.push_back(w[i]);
    }
    double B[3][3], R[3];
    pair_block(T, S, r, sigS, test, side, kernel_far, B, R);
    for (int a = 0; a < 3; ++a) {
        rb[a] = R[a];
        for (int b = 0; b < 3; ++b) blk[3 * a + b] = B[a][b];
    }
    return 0;
}

// assemble (assemble.jl:377-447) over the test triangles [t0, t1): rows of A (nslot x (nslot + nwnode), row-major)
// and b are accumulated (the caller zeroes them). pairs/points: 6 counters per tier (self, edge, vertex, contact,
// near, far). Returns 0, or -1 for a degenerate triangle.
static int assemble_tests(const vpo_options* po, int ntri, const double* x, const int* tris, const int* corner_slot,
                          int nslot, int ntouch, const int* touch_pairs, const double* sigma, const double* V,
                          int nwnode, const double* wx, int nwtri, const int* wtris, int nfil, const int* fil, int t0,
                          int t1, const int* tlist, double* A, double* b, long long* pairs, long long* points,
                          int nthreads);

int vpo_assemble(const vpo_options* po, int nnode, const double* x, int ntri, const int* tris, const int* corner_slot,
                 int nslot, int ntouch, const int* touch_pairs, const double* sigma, const double* V, int nwnode,
                 const double* wx, int nwtri, const int* wtris, int nfil, const int* fil, int t0, int t1, double* A,
                 double* b, long long* pairs, long long* points, int nthreads) {
    (void)nnode;
    return assemble_tests(po, ntri, x, tris, corner_slot, nslot, ntouch, touch_pairs, sigma, V, nwnode, wx, nwtri,
                          wtris, nfil, fil, t0, t1, nullptr, A, b, pairs, points, nthreads);
}

// assemble over the test triangles tlist[0 .. ntest): the rows of every slot whose one-ring lies in the list are
// complete (a sample of rows anywhere on a large mesh)
int vpo_assemble_list(const vpo_options* po, int nnode, const double* x, int ntri, const int* tris,
                      const int* corner_slot, int nslot, int ntouch, const int* touch_pairs, const double* sigma,
                      const double* V, int nwnode, const double* wx, int nwtri, const int* wtris, int nfil,
                      const int* fil, int ntest, const int* tlist, double* A, double* b, long long* pairs,
                      long long* points, int nthreads) {
    (void)nnode;
    for (int k = 0; k < ntest; ++k)
        if (tlist[k] < 0 || tlist[k] >= ntri) return -2;
    return assemble_tests(po, ntri, x, tris, corner_slot, nslot, ntouch, touch_pairs, sigma, V, nwnode, wx, nwtri,
                          wtris, nfil, fil, 0, ntest, tlist, A, b, pairs, points, nthreads);
}

}  // extern "C"

namespace vpo {

// the rows of test triangles t0..t1-1 (or tlist[t0..t1)) of assemble (assemble.jl:377-447) over built elements:
// body pairs, wake sheets (add_wake!, :333-356), filaments and the exact freestream term (:422). A (nslot x ncols)
// and b are accumulated; per-tier pair and point counts go to P, Q.
template <class T>
static void assemble_core(const Options& o, const TierRules& rules, const std::vector<FlatTriT<T>>& els,
                          const int* tris, const int* corner_slot, int nslot, const std::set<std::pair<int, int>>& touch,
                          const T* sigma, const V3<T>& Vinf, int nwnode, const std::vector<FlatTriT<T>>& wels,
                          const int* wtris, const std::vector<SegmentT<T>>& segs, const int* fil, int t0, int t1,
                          const int* tlist, T* A, T* b, long long* P, long long* Q, int nthreads) {
    const int ntri = int(els.size()), nwtri = int(wels.size()), nfil = int(segs.size());
    const int ncols = nslot + nwnode;
    const Vec ti = test_integrals(o.test);
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
#pragma omp parallel
    {
        std::vector<T> buf(size_t(3) * ncols);
        RuleT<T> rbuf;
        long long myP[6] = {0}, myQ[6] = {0};
#pragma omp for schedule(dynamic, 4)
        for (int it = t0; it < t1; ++it) {
            const int t = tlist ? tlist[it] : it;
            const FlatTriT<T>& Tr = els[t];
            std::fill(buf.begin(), buf.end(), T(0));
            T rows[3] = {T(0), T(0), T(0)};
            for (int s = 0; s < ntri; ++s) {
                int tier;
                const RuleT<T>* rule = pair_rule(els.data(), tris, t, s, rules, o, touch, rbuf, tier);
                T blk[3][3], rb[3];
                pair_block(Tr, els[s], *rule, sigma[s], o.test, s == t ? 1 : 0, o.kernel_far, blk, rb);
                const int* cs = corner_slot + 3 * s;
                for (int bb = 0; bb < 3; ++bb)
                    for (int a = 0; a < 3; ++a) buf[size_t(a) * ncols + cs[bb]] += blk[a][bb];
                for (int a = 0; a < 3; ++a) rows[a] += rb[a];
                myP[tier] += 1;
                myQ[tier] += (long long)rule->size();
            }
            // add_wake! (assemble.jl:333-356)
            for (int s = 0; s < nwtri; ++s) {
                int tier;
                const RuleT<T>* rule = wake_pair_rule(Tr, wels[s], rules, o, rbuf, tier);
                T blk[3][3], rb[3];
                pair_block(Tr, wels[s], *rule, T(0), o.test, 0, o.kernel_far, blk, rb);
                const int* c = wtris + 3 * s;
                for (int bb = 0; bb < 3; ++bb)
                    for (int a = 0; a < 3; ++a) buf[size_t(a) * ncols + nslot + c[bb]] += blk[a][bb];
                myP[tier] += 1;
                myQ[tier] += (long long)rule->size();
            }
            for (int f = 0; f < nfil; ++f) {
                int tier;
                const RuleT<T>* rule = segment_rule(Tr, segs[f], rules, o, rbuf, tier);
                T ca[3], cb[3];
                segment_block(Tr, segs[f], *rule, o.test, ca, cb);
                int ia = fil[2 * f], ib = fil[2 * f + 1];
                for (int a = 0; a < 3; ++a) {
                    buf[size_t(a) * ncols + nslot + ia] += ca[a];
                    buf[size_t(a) * ncols + nslot + ib] += cb[a];
                }
                myP[tier] += 1;
                myQ[tier] += (long long)rule->size();
            }
            // freestream (exact), assemble.jl:422
            T vn = dot(Vinf, Tr.n) * Tr.area;
            for (int a = 0; a < 3; ++a) rows[a] -= vn * T(ti[a]);
            const int* ct = corner_slot + 3 * t;
#pragma omp critical(vpo_scatter)
            {
                for (int a = 0; a < 3; ++a) {
                    T* Arow = A + size_t(ct[a]) * ncols;
                    const T* src = buf.data() + size_t(a) * ncols;
                    for (int j = 0; j < ncols; ++j) Arow[j] += src[j];
                    b[ct[a]] += rows[a];
                }
            }
        }
#pragma omp critical(vpo_stats)
        for (int k = 0; k < 6; ++k) {
            P[k] += myP[k];
            Q[k] += myQ[k];
        }
    }
}

static std::set<std::pair<int, int>> touch_set(int ntouch, const int* touch_pairs) {
    std::set<std::pair<int, int>> touch;
    for (int i = 0; i < ntouch; ++i) {
        touch.insert({touch_pairs[2 * i], touch_pairs[2 * i + 1]});
        touch.insert({touch_pairs[2 * i + 1], touch_pairs[2 * i]});
    }
    return touch;
}

}  // namespace vpo

extern "C" {

static int assemble_tests(const vpo_options* po, int ntri, const double* x, const int* tris, const int* corner_slot,
                          int nslot, int ntouch, const int* touch_pairs, const double* sigma, const double* V,
                          int nwnode, const double* wx, int nwtri, const int* wtris, int nfil, const int* fil, int t0,
                          int t1, const int* tlist, double* A, double* b, long long* pairs, long long* points,
                          int nthreads) {
    Options o = to_opts(po);
    TierRules rules = tier_rules(o);
    std::vector<FlatTri> els, wels;
    if (!build_elements(ntri, x, tris, els)) return -1;
    if (nwtri > 0 && !build_elements(nwtri, wx, wtris, wels)) return -1;
    std::vector<Segment> segs(nfil);
    for (int f = 0; f < nfil; ++f) segs[f] = Segment{vec_at(wx, fil[2 * f]), vec_at(wx, fil[2 * f + 1])};
    if (t0 < 0) t0 = 0;
    if (!tlist && t1 > ntri) t1 = ntri;
    long long P[6] = {0}, Q[6] = {0};
    assemble_core(o, rules, els, tris, corner_slot, nslot, touch_set(ntouch, touch_pairs), sigma, vec_at(V, 0), nwnode,
                  wels, wtris, segs, fil, t0, t1, tlist, A, b, P, Q, nthreads);
    for (int k = 0; k < 6; ++k) {
        pairs[k] += P[k];
        points[k] += Q[k];
    }
    return 0;
}

// ---- the derivative oracle: the assembly in forward-mode dual numbers ----

// directions one dual pass carries
int vpo_dual_nd(void) { return VPO_ND; }

// A and b of assemble (assemble.jl:377-447) with their derivatives along nd <= VPO_ND directions. Node positions x
// (nnode x 3) with tangents dx (nd x nnode x 3); the wake's nodes wx (nwnode x 3) with dwx (nd x nwnode x 3); the
// freestream V with dV (nd x 3). sigma = -n.V (assemble.jl:364) is formed from the dual normals and V. Out, each
// with (1 + nd) layers (value, then the nd derivatives): A (nslot x (nslot + nwnode)), b (nslot), and per body
// triangle its area, normal (3) and barycentric gradients gradl (9) (flat_triangle.jl:12-31), 13 values.
int vpo_dual_assemble(const vpo_options* po, int nnode, const double* x, const double* dx, int ntri, const int* tris,
                      const int* corner_slot, int nslot, int ntouch, const int* touch_pairs, const double* V,
                      const double* dV, int nwnode, const double* wx, const double* dwx, int nwtri, const int* wtris,
                      int nfil, const int* fil, int nd, double* A, double* b, double* elem, long long* pairs,
                      long long* points, int nthreads) {
    typedef Dual<VPO_ND> D;
    if (nd < 0 || nd > VPO_ND) return -2;
    auto dual_points = [nd](int n, const double* p, const double* dp) {
        std::vector<V3<D>> X(n);
        for (int i = 0; i < n; ++i)
            for (int c = 0; c < 3; ++c) {
                D v(p[3 * i + c]);
                for (int k = 0; k < nd; ++k) v.d[k] = dp[(size_t(k) * n + i) * 3 + c];
                X[i][c] = v;
            }
        return X;
    };
    const std::vector<V3<D>> X = dual_points(nnode, x, dx), WX = dual_points(nwnode, wx, dwx);
    const V3<D> Vd = dual_points(1, V, dV)[0];
    Options o = to_opts(po);
    TierRules rules = tier_rules(o);
    std::vector<FlatTriT<D>> els, wels;
    if (!build_elements(ntri, X.data(), tris, els)) return -1;
    if (nwtri > 0 && !build_elements(nwtri, WX.data(), wtris, wels)) return -1;
    std::vector<SegmentT<D>> segs(nfil);
    for (int f = 0; f < nfil; ++f) segs[f] = SegmentT<D>{WX[fil[2 * f]], WX[fil[2 * f + 1]]};
    std::vector<D> sigma(ntri);
    for (int t = 0; t < ntri; ++t) sigma[t] = -dot(els[t].n, Vd);
    const int ncols = nslot + nwnode;
    std::vector<D> Ad(size_t(nslot) * ncols), bd(nslot);
    long long P[6] = {0}, Q[6] = {0};
    assemble_core(o, rules, els, tris, corner_slot, nslot, touch_set(ntouch, touch_pairs), sigma.data(), Vd, nwnode,
                  wels, wtris, segs, fil, 0, ntri, nullptr, Ad.data(), bd.data(), P, Q, nthreads);
    const size_t na = Ad.size();
    for (int k = 0; k <= nd; ++k) {
        auto pick = [k](const D& v) { return k == 0 ? v.v : v.d[k - 1]; };
        for (size_t i = 0; i < na; ++i) A[k * na + i] = pick(Ad[i]);
        for (int i = 0; i < nslot; ++i) b[size_t(k) * nslot + i] = pick(bd[i]);
        for (int t = 0; t < ntri; ++t) {
            double* e = elem + (size_t(k) * ntri + t) * 13;
            const FlatTriT<D>& el = els[t];
            e[0] = pick(el.area);
            for (int c = 0; c < 3; ++c) e[1 + c] = pick(el.n[c]);
            for (int j = 0; j < 3; ++j)
                for (int c = 0; c < 3; ++c) e[4 + 3 * j + c] = pick(el.gradl[j][c]);
        }
    }
    for (int k = 0; k < 6; ++k) {
        pairs[k] += P[k];
        points[k] += Q[k];
    }
    return 0;
}

// source_velocity (source_triangle.jl:134-138) of triangle abc at x with its Jacobian J (3 x 3, row = component of
// w, column = direction): wrt = 0 the point x, wrt = 1 the vertex a
int vpo_dual_source_velocity(const double* abc, const double* x, int wrt, double far, double* w, double* J) {
    typedef Dual<VPO_ND> D;
    V3<D> v[3], xd;
    for (int i = 0; i < 3; ++i)
        for (int c = 0; c < 3; ++c) v[i][c] = D(abc[3 * i + c]);
    for (int c = 0; c < 3; ++c) xd[c] = D(x[c]);
    for (int c = 0; c < 3; ++c) (wrt == 0 ? xd : v[0])[c].d[c] = 1.0;
    SourceTri<D> s;
    if (!make_source_tri(v[0], v[1], v[2], s)) return -1;
    const V3<D> r = source_velocity(s, xd, 0, far);
    for (int i = 0; i < 3; ++i) {
        w[i] = r[i].v;
        for (int c = 0; c < 3; ++c) J[3 * i + c] = r[i].d[c];
    }
    return 0;
}

}  // extern "C"

// ---- the free wake's kernels (src/assembly/explicit.jl, src/post/Post.jl, src/freewake/step.jl) ----
extern "C" {

// explicit_rhs (explicit.jl:31-85): -int psi_i n.u_src dA per slot of known sheets (nsheet x 9 corners, sheet_mu
// nsheet x 3), filaments (nseg x 6 ends, seg_g nseg x 2) and particles (nblob x 7: x, alpha, delta). rhs (nslot) is
// accumulated (the caller zeroes it). Returns -1 for a degenerate body triangle or sheet.
int vpo_explicit_rhs(const vpo_options* po, const double* x, int ntri, const int* tris, const int* corner_slot,
                     int nsheet, const double* sheet_x, const double* sheet_mu, int nseg, const double* seg_x,
                     const double* seg_g, int nblob, const double* blobs, double* rhs, int nthreads) {
    Options o = to_opts(po);
    TierRules rules = tier_rules(o);
    std::vector<FlatTri> els;
    if (!build_elements(ntri, x, tris, els)) return -1;
    std::vector<FlatTri> sheets(nsheet);
    for (int s = 0; s < nsheet; ++s)
        if (!make_flat_tri(vec_at(sheet_x + 9 * s, 0), vec_at(sheet_x + 9 * s, 1), vec_at(sheet_x + 9 * s, 2), sheets[s]))
            return -1;
    std::vector<Segment> segs(nseg);
    for (int f = 0; f < nseg; ++f) segs[f] = Segment{vec_at(seg_x + 6 * f, 0), vec_at(seg_x + 6 * f, 1)};
    std::vector<Blob> bl(nblob);
    for (int k = 0; k < nblob; ++k) bl[k] = Blob{vec_at(blobs + 7 * k, 0), vec_at(blobs + 7 * k + 3, 0), blobs[7 * k + 6]};
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
#pragma omp parallel
    {
        Rule rbuf;
        std::vector<Vec> ufar(rules.far.size());
#pragma omp for schedule(dynamic, 4)
        for (int t = 0; t < ntri; ++t) {
            const FlatTri& T = els[t];
            double rows[3] = {0, 0, 0};
            for (int s = 0; s < nsheet; ++s) {
                int tier;
                const Rule* rule = wake_pair_rule(T, sheets[s], rules, o, rbuf, tier);
                double blk[3][3], rb[3];
                pair_block(T, sheets[s], *rule, 0.0, o.test, 0, o.kernel_far, blk, rb);
                const double* m = sheet_mu + 3 * s;
                for (int a = 0; a < 3; ++a) rows[a] -= blk[a][0] * m[0] + blk[a][1] * m[1] + blk[a][2] * m[2];
            }
            for (int f = 0; f < nseg; ++f) {
                int tier;
                const Rule* rule = segment_rule(T, segs[f], rules, o, rbuf, tier);
                double ca[3], cb[3];
                segment_block(T, segs[f], *rule, o.test, ca, cb);
                for (int a = 0; a < 3; ++a) rows[a] -= ca[a] * seg_g[2 * f] + cb[a] * seg_g[2 * f + 1];
            }
            for (auto& u : ufar) u = Vec();
            for (int k = 0; k < nblob; ++k) {
                const Blob& b = bl[k];
                if (norm(b.x - T.c) > o.far_ratio * std::max(T.diam, b.delta)) {
                    for (size_t q = 0; q < rules.far.size(); ++q)
                        ufar[q] += blob_velocity(point(T, rules.far.lam[q]), b.x, b.al, b.delta);
                } else {
                    near_rule(rbuf, T, b, rules.near_, o.near_ratio, o.near_depth);
                    for (size_t q = 0; q < rbuf.size(); ++q) {
                        const Bary& l = rbuf.lam[q];
                        double un = rbuf.w[q] * T.area * dot(blob_velocity(point(T, l), b.x, b.al, b.delta), T.n);
                        Vec psi = test_weights(o.test, l);
                        for (int a = 0; a < 3; ++a) rows[a] -= un * psi[a];
                    }
                }
            }
            if (nblob > 0)
                for (size_t q = 0; q < rules.far.size(); ++q) {
                    double un = rules.far.w[q] * T.area * dot(ufar[q], T.n);
                    Vec psi = test_weights(o.test, rules.far.lam[q]);
                    for (int a = 0; a < 3; ++a) rows[a] -= un * psi[a];
                }
            const int* ct = corner_slot + 3 * t;
#pragma omp critical(vpo_rhs)
            for (int a = 0; a < 3; ++a) rhs[ct[a]] += rows[a];
        }
    }
    return 0;
}

// body_velocity (Post.jl:92-112): sum over the triangles of sigma_s w_s + gamma_s x w_s at the points X (npts x 3)
int vpo_body_velocity(const double* corners, int ntri, const double* sigma, const double* gamma, double kernel_far,
                      int npts, const double* X, double* U, int nthreads) {
    std::vector<SourceTri<double>> src(ntri);
    for (int t = 0; t < ntri; ++t)
        if (!make_source_tri(vec_at(corners + 9 * t, 0), vec_at(corners + 9 * t, 1), vec_at(corners + 9 * t, 2), src[t]))
            return -1;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
#pragma omp parallel for schedule(dynamic, 16)
    for (int i = 0; i < npts; ++i) {
        const Vec x = vec_at(X, i);
        Vec acc;
        for (int t = 0; t < ntri; ++t) {
            Vec w = source_velocity(src[t], x, 0, kernel_far);
            acc += sigma[t] * w + cross(vec_at(gamma, t), w);
        }
        U[3 * i] = acc.x;
        U[3 * i + 1] = acc.y;
        U[3 * i + 2] = acc.z;
    }
    return 0;
}

// blob_velocities (step.jl:176-187): the direct sum of every blob (nblob x 7) at every point
void vpo_blob_velocities(int nblob, const double* blobs, int npts, const double* X, double* U, int nthreads) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
#pragma omp parallel for schedule(static)
    for (int i = 0; i < npts; ++i) {
        const Vec x = vec_at(X, i);
        Vec acc;
        for (int k = 0; k < nblob; ++k)
            acc += blob_velocity(x, vec_at(blobs + 7 * k, 0), vec_at(blobs + 7 * k + 3, 0), blobs[7 * k + 6]);
        U[3 * i] = acc.x;
        U[3 * i + 1] = acc.y;
        U[3 * i + 2] = acc.z;
    }
}

}  // extern "C"
