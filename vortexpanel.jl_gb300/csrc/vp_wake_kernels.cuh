// The free wake's point kernels, shared by the one-shot entry points (vp_freewake.cu) and the device-resident
// simulation (vp_wake.cu):
//   - blob_kernel: the Rosenhead-Moore N-body sum (blob_velocity, src/kernels/blob.jl:21-25) of every blob at every
//     point (blob_velocities, src/freewake/step.jl:176-187), one thread per point over shared-memory tiles of blobs;
//   - body_kernel: sigma_s w_s + gamma_s x w_s of every body triangle at every point (body_velocity,
//     src/post/Post.jl:92-112), the exact kernel within kernel_far diameters and the multipole beyond.
// Include after vp_pairs.cuh; everything sits in an anonymous namespace (one copy per translation unit).
#pragma once
#include "vp_pairs.cuh"

namespace {

constexpr int NB_THREADS = 256;  // points per CTA of the N-body and body-velocity kernels
constexpr int NB_TILE = 256;     // blobs per shared-memory tile

// blob_velocity (blob.jl:21-25): (1/4pi) alpha x r / (|r|^2 + delta^2)^(3/2), r = x - xp
template <class T>
__device__ __forceinline__ v3<T> blob_vel(v3<T> r, v3<T> al, T d2core) {
    T d2 = dot(r, r) + d2core;
    T s = T(1) / (T(4) * vp_pi<T>() * d2 * vsqrt(d2));
    return s * cross(al, r);
}

// blobs: x (3), alpha (3), delta (1) per blob. FP64: the plain sum. FP32 (float specialisation below): two points
// per thread, the tile's blobs as float4 pairs (x, delta^2) and (alpha / 4 pi), 1/d^3 by a reciprocal square root,
// every tile summed in FP32 and the tiles in FP64.
template <class T>
__global__ void __launch_bounds__(NB_THREADS) blob_kernel(int nblob, const double* __restrict__ blobs, int npts,
                                                        const double* __restrict__ X, double* __restrict__ U) {
    __shared__ T sb[NB_TILE][8];
    const int i = blockIdx.x * NB_THREADS + threadIdx.x;
    const bool valid = i < npts;
    v3<double> x = valid ? mk3(X[3 * i], X[3 * i + 1], X[3 * i + 2]) : mk3(0.0, 0.0, 0.0);
    const v3<T> xt = mk3(T(x.x), T(x.y), T(x.z));
    v3<double> acc = mk3(0.0, 0.0, 0.0);
    for (int b0 = 0; b0 < nblob; b0 += NB_TILE) {
        const int nb = min(NB_TILE, nblob - b0);
        __syncthreads();
        for (int k = threadIdx.x; k < nb; k += NB_THREADS) {
            const double* p = blobs + 7 * size_t(b0 + k);
            for (int z = 0; z < 6; ++z) sb[k][z] = T(p[z]);
            sb[k][6] = T(p[6] * p[6]);
        }
        __syncthreads();
        v3<T> part = mk3(T(0), T(0), T(0));
        for (int k = 0; k < nb; ++k) {
            v3<T> r = xt - mk3(sb[k][0], sb[k][1], sb[k][2]);
            part += blob_vel(r, mk3(sb[k][3], sb[k][4], sb[k][5]), sb[k][6]);
        }
        acc += mk3(double(part.x), double(part.y), double(part.z));
    }
    if (valid) {
        U[3 * i] = acc.x;
        U[3 * i + 1] = acc.y;
        U[3 * i + 2] = acc.z;
    }
}

constexpr int NB_PTS = 2;  // points per thread of the FP32 kernel

template <>
__global__ void __launch_bounds__(NB_THREADS) blob_kernel<float>(int nblob, const double* __restrict__ blobs, int npts,
                                                               const double* __restrict__ X, double* __restrict__ U) {
    __shared__ float4 sx[NB_TILE], sa[NB_TILE];
    const float i4pi = 1.f / (4.f * vp_pi<float>());
    const int i0 = blockIdx.x * NB_THREADS * NB_PTS + threadIdx.x;
    float px[NB_PTS], py[NB_PTS], pz[NB_PTS];
    double ax[NB_PTS], ay[NB_PTS], az[NB_PTS];
#pragma unroll
    for (int j = 0; j < NB_PTS; ++j) {
        const int i = i0 + j * NB_THREADS;
        const bool v = i < npts;
        px[j] = v ? float(X[3 * i]) : 0.f;
        py[j] = v ? float(X[3 * i + 1]) : 0.f;
        pz[j] = v ? float(X[3 * i + 2]) : 0.f;
        ax[j] = ay[j] = az[j] = 0.0;
    }
    for (int b0 = 0; b0 < nblob; b0 += NB_TILE) {
        const int nb = min(NB_TILE, nblob - b0);
        __syncthreads();
        for (int k = threadIdx.x; k < NB_TILE; k += NB_THREADS) {
            if (k < nb) {
                const double* p = blobs + 7 * size_t(b0 + k);
                sx[k] = make_float4(float(p[0]), float(p[1]), float(p[2]), float(p[6] * p[6]));
                sa[k] = make_float4(float(p[3]) * i4pi, float(p[4]) * i4pi, float(p[5]) * i4pi, 0.f);
            } else {  // padding: a blob of zero strength far away
                sx[k] = make_float4(0.f, 0.f, 0.f, 1.f);
                sa[k] = make_float4(0.f, 0.f, 0.f, 0.f);
            }
        }
        __syncthreads();
        float ux[NB_PTS], uy[NB_PTS], uz[NB_PTS];
#pragma unroll
        for (int j = 0; j < NB_PTS; ++j) ux[j] = uy[j] = uz[j] = 0.f;
#pragma unroll 8
        for (int k = 0; k < NB_TILE; ++k) {
            const float4 b = sx[k], al = sa[k];
#pragma unroll
            for (int j = 0; j < NB_PTS; ++j) {
                const float rx = px[j] - b.x, ry = py[j] - b.y, rz = pz[j] - b.z;
                const float d2 = fmaf(rx, rx, fmaf(ry, ry, fmaf(rz, rz, b.w)));
                const float inv = rsqrtf(d2);
                const float s = inv * inv * inv;
                ux[j] = fmaf(s, al.y * rz - al.z * ry, ux[j]);
                uy[j] = fmaf(s, al.z * rx - al.x * rz, uy[j]);
                uz[j] = fmaf(s, al.x * ry - al.y * rx, uz[j]);
            }
        }
#pragma unroll
        for (int j = 0; j < NB_PTS; ++j) {
            ax[j] += double(ux[j]);
            ay[j] += double(uy[j]);
            az[j] += double(uz[j]);
        }
    }
#pragma unroll
    for (int j = 0; j < NB_PTS; ++j) {
        const int i = i0 + j * NB_THREADS;
        if (i < npts) {
            U[3 * i] = ax[j];
            U[3 * i + 1] = ay[j];
            U[3 * i + 2] = az[j];
        }
    }
}

// body triangles as sources: corners (9), sigma, gamma (3) -> the kernel's data in FP64
struct BodySrc {
    double c[3], d[9], nu[9], len[3], n[3], area, diam, sigma, gam[3];
};

template <class T>
__device__ __forceinline__ SrcKern<T> kern_from(const BodySrc& s) {
    SrcKern<T> K;
    for (int k = 0; k < 3; ++k) {
        K.d[k] = mk3(T(s.d[3 * k]), T(s.d[3 * k + 1]), T(s.d[3 * k + 2]));
        K.nu[k] = mk3(T(s.nu[3 * k]), T(s.nu[3 * k + 1]), T(s.nu[3 * k + 2]));
        K.len[k] = T(s.len[k]);
    }
    K.n = mk3(T(s.n[0]), T(s.n[1]), T(s.n[2]));
    K.area = T(s.area);
    K.diam = T(s.diam);
    return K;
}

// source_velocity (source_triangle.jl:134-138) off the body: exact within kernel_far diameters, multipole beyond.
// FP32 (mixed): the exact form under the FP32 guard, FP64 where the guard refuses.
template <class T>
__global__ void __launch_bounds__(NB_THREADS) body_kernel(int nsrc, const BodySrc* __restrict__ src, double kernel_far,
                                                        int npts, const double* __restrict__ X, double* __restrict__ U) {
    __shared__ BodySrc ss[32];
    const int i = blockIdx.x * NB_THREADS + threadIdx.x;
    const bool valid = i < npts;
    const v3<double> x = valid ? mk3(X[3 * i], X[3 * i + 1], X[3 * i + 2]) : mk3(0.0, 0.0, 0.0);
    v3<double> acc = mk3(0.0, 0.0, 0.0);
    const Fp32Guard g{PAIR_GUARD};
    for (int s0 = 0; s0 < nsrc; s0 += 32) {
        const int ns = min(32, nsrc - s0);
        __syncthreads();
        for (int k = threadIdx.x; k < ns * int(sizeof(BodySrc) / 8); k += NB_THREADS)
            reinterpret_cast<double*>(ss)[k] = reinterpret_cast<const double*>(src + s0)[k];
        __syncthreads();
        if (!valid) continue;
        for (int k = 0; k < ns; ++k) {
            const BodySrc& s = ss[k];
            const v3<double> r64 = x - mk3(s.c[0], s.c[1], s.c[2]);
            const double fd = kernel_far * s.diam;
            v3<double> w;
            bool done = false;
            if (sizeof(T) == 4) {
                const SrcKern<float> K = kern_from<float>(s);
                const v3<float> r = mk3(float(r64.x), float(r64.y), float(r64.z));
                v3<float> wf;
                if (dot(r64, r64) > fd * fd) {
                    wf = sv_far(K, r);
                    done = true;
                } else {
                    done = sv_exact3_guarded(K, r - K.d[0], r - K.d[1], r - K.d[2], 0, g, wf);
                }
                if (done) w = mk3(double(wf.x), double(wf.y), double(wf.z));
            }
            if (!done) {
                const SrcKern<double> K = kern_from<double>(s);
                w = sv_rel(K, r64, 0, kernel_far, 1e-12);
            }
            acc += s.sigma * w + cross(mk3(s.gam[0], s.gam[1], s.gam[2]), w);
        }
    }
    if (valid) {
        U[3 * i] = acc.x;
        U[3 * i + 1] = acc.y;
        U[3 * i + 2] = acc.z;
    }
}

// the rule data of the particles' rows of explicit_rhs (explicit.jl:63-76)
struct ParticleRule {
    const RulePt* rfar;
    int nfar;
    const RulePt* rnear;
    int nnear;
    int test_mode, near_depth;
    double far_ratio, near_ratio;
};

template <class T>
__device__ __forceinline__ void particle_point(const ParticleRule& a, const TriGeo& Tr, double l0, double l1, double l2,
                                               double W, const double* bl, double* rows) {
    v3<double> x = mk3(l0 * Tr.x[0] + l1 * Tr.x[3] + l2 * Tr.x[6], l0 * Tr.x[1] + l1 * Tr.x[4] + l2 * Tr.x[7],
                       l0 * Tr.x[2] + l1 * Tr.x[5] + l2 * Tr.x[8]);
    v3<double> r = x - mk3(bl[0], bl[1], bl[2]);
    v3<T> u = blob_vel(mk3(T(r.x), T(r.y), T(r.z)), mk3(T(bl[3]), T(bl[4]), T(bl[5])), T(bl[6] * bl[6]));
    double un = (double(u.x) * Tr.n[0] + double(u.y) * Tr.n[1] + double(u.z) * Tr.n[2]) * W;
    v3<double> psi = test_weights(a.test_mode, l0, l1, l2);
    rows[0] -= un * psi.x;
    rows[1] -= un * psi.y;
    rows[2] -= un * psi.z;
}

// -∫ψ_a n·u dA of the particle bl (x, alpha, delta) on test triangle Tr, added to rows: the far rule's points when it
// lies more than far_ratio max(diam, delta) from the centroid, else near_rule's quadtree about the particle
// (assemble.jl:69-91 with distance_to(b, p) = |p - x_b|, explicit.jl:63-76), walked depth-first
template <class T>
__device__ void particle_rows(const ParticleRule& a, const TriGeo& Tr, const double* bl, double* rows) {
    const double dx = bl[0] - Tr.c[0], dy = bl[1] - Tr.c[1], dz = bl[2] - Tr.c[2];
    if (sqrt(dx * dx + dy * dy + dz * dz) > a.far_ratio * fmax(Tr.diam, bl[6])) {
        for (int q = 0; q < a.nfar; ++q) {
            const RulePt& m = a.rfar[q];
            particle_point<T>(a, Tr, m.l0, m.l1, m.l2, m.w * Tr.area, bl, rows);
        }
        return;
    }
    int level = 0;
    unsigned path = 0;
    for (int guard = 0; guard < (1 << 20); ++guard) {
        double c[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
        for (int l = 0; l < level; ++l) {
            int digit = (path >> (2 * (level - 1 - l))) & 3;
            double m12[3], m23[3], m31[3], nb[9];
            for (int z = 0; z < 3; ++z) {
                m12[z] = 0.5 * (c[z] + c[3 + z]);
                m23[z] = 0.5 * (c[3 + z] + c[6 + z]);
                m31[z] = 0.5 * (c[6 + z] + c[z]);
            }
            for (int z = 0; z < 3; ++z) {
                if (digit == 0) { nb[z] = c[z]; nb[3 + z] = m12[z]; nb[6 + z] = m31[z]; }
                else if (digit == 1) { nb[z] = m12[z]; nb[3 + z] = c[3 + z]; nb[6 + z] = m23[z]; }
                else if (digit == 2) { nb[z] = m31[z]; nb[3 + z] = m23[z]; nb[6 + z] = c[6 + z]; }
                else { nb[z] = m12[z]; nb[3 + z] = m23[z]; nb[6 + z] = m31[z]; }
            }
            for (int z = 0; z < 9; ++z) c[z] = nb[z];
        }
        v3<double> p1 = tpoint(Tr, c), p2 = tpoint(Tr, c + 3), p3 = tpoint(Tr, c + 6);
        double size = fmax(vnorm(p2 - p1), fmax(vnorm(p3 - p2), vnorm(p1 - p3)));
        v3<double> pc = (p1 + p2 + p3) / 3.0 - mk3(bl[0], bl[1], bl[2]);
        if (level < a.near_depth && vnorm(pc) < a.near_ratio * size) {
            level++;
            path *= 4;
            continue;
        }
        const double frac = ldexp(1.0, -2 * level);
        for (int q = 0; q < a.nnear; ++q) {
            const RulePt& m = a.rnear[q];
            double l0 = m.l0 * c[0] + m.l1 * c[3] + m.l2 * c[6];
            double l1 = m.l0 * c[1] + m.l1 * c[4] + m.l2 * c[7];
            double l2 = m.l0 * c[2] + m.l1 * c[5] + m.l2 * c[8];
            particle_point<T>(a, Tr, l0, l1, l2, m.w * frac * Tr.area, bl, rows);
        }
        while (level > 0 && (path & 3) == 3) {
            path >>= 2;
            level--;
        }
        if (level == 0) break;
        path++;
    }
}

}  // namespace
