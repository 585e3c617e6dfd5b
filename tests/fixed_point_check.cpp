// Host check of the order-independent fixed-point sums (vortexpanel.jl_gb300/csrc/vp_fixed.cuh). Reads a count and
// that many doubles from stdin, adds them to one accumulator (1) in input order, (2) in several shuffled orders and
// (3) from several threads at once, each thread adding its share with relaxed atomic adds on the same words, as the
// device's atomics do; prints one line per run: the six digit words, the flag word and the value read back.
#define __host__
#define __device__
#include "vp_fixed.cuh"

#include <algorithm>
#include <cstdio>
#include <random>
#include <thread>
#include <vector>

static void plain_add(long long* p, long long x) { *p += x; }

static void atomic_add(long long* p, long long x) { __atomic_fetch_add(p, x, __ATOMIC_RELAXED); }

static void print(const vp_fx& a) {
    for (int k = 0; k < 6; ++k) std::printf("%lld ", a.d[k]);
    std::printf("%llu %.17g\n", a.flag, fx_get(a));
}

int main() {
    size_t n = 0;
    if (std::scanf("%zu", &n) != 1) return 1;
    std::vector<double> v(n);
    for (auto& x : v)
        if (std::scanf("%lf", &x) != 1) return 1;
    vp_fx a{};
    for (double x : v) fx_accumulate(&a, x, plain_add);
    print(a);
    std::mt19937_64 rng(12345);
    for (int rep = 0; rep < 3; ++rep) {
        std::vector<double> u = v;
        std::shuffle(u.begin(), u.end(), rng);
        vp_fx b{};
        for (double x : u) fx_accumulate(&b, x, plain_add);
        print(b);
    }
    for (int nt : {2, 4, 8}) {
        std::vector<double> u = v;
        std::shuffle(u.begin(), u.end(), rng);
        vp_fx c{};
        std::vector<std::thread> th;
        for (int t = 0; t < nt; ++t)
            th.emplace_back([&, t] {
                for (size_t i = t; i < u.size(); i += nt) fx_accumulate(&c, u[i], atomic_add);
            });
        for (auto& x : th) x.join();
        print(c);
    }
    return 0;
}
