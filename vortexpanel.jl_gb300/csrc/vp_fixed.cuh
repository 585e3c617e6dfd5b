// Order-independent FP64 sums: a fixed-point accumulator (least significant bit 2^-130, range +-2^61) updated by
// integer atomics. Each added double is rounded once to the accumulator's grid (an absolute 2^-131 at most, below
// 1e-39); after that every update is an exact integer addition, so the total does not depend on the order in which
// the atomics land and a sum scattered from many threads is the same bit for bit from run to run. A non-finite or
// out-of-range addend sets a flag word that makes the value read back NaN.
//
// Carry-save layout: the 192-bit value is six 32-bit digits, each held in its own signed 64-bit word. An addend's
// 53-bit significand covers at most three adjacent digits; it adds its digits (negated for a negative addend) to
// those words with atomics whose results are not needed, so no thread waits on a returned value. A word has 31 bits
// of headroom, room for 2^31 additions of full digits. The carries between digits are resolved only when the value
// is read (fx_get).
#pragma once
#include <cmath>
#include <cstring>

struct vp_fx {
    long long d[6];           // digit k weighs 2^(32 k - 130)
    unsigned long long flag;  // non-finite or out-of-range addend
    unsigned long long pad;
};

// a double's digits on the accumulator's grid: round(|v| 2^130) = (d0 + d1 2^32 + d2 2^64) 2^(32 k), negated for a
// negative v (false for a non-finite v or |v| >= 2^61, outside the range)
__host__ __device__ inline bool fx_digits(double v, int& k, long long& d0, long long& d1, long long& d2) {
    unsigned long long bits;
    memcpy(&bits, &v, sizeof bits);
    int e = int((bits >> 52) & 0x7ff);
    if (e == 0x7ff) return false;
    unsigned long long m = bits & ((1ull << 52) - 1);
    if (e)
        m |= 1ull << 52;
    else
        e = 1;
    // |v| = m 2^(e - 1075) = m 2^sh units of 2^-130
    int sh = e - 945;
    if (sh > 138) return false;
    if (sh < 0) {
        m = sh < -54 ? 0 : (m + (1ull << (-sh - 1))) >> (-sh);  // round half up
        sh = 0;
    }
    k = sh >> 5;
    const int r = sh & 31;
    const unsigned long long lo = m << r, hi = r ? m >> (64 - r) : 0;  // m 2^r, bits 0-63 and 64-84
    d0 = (long long)(lo & 0xffffffffull);
    d1 = (long long)(lo >> 32);
    d2 = (long long)hi;
    if (bits >> 63) {
        d0 = -d0;
        d1 = -d1;
        d2 = -d2;
    }
    return true;
}

// a += v, with add(word, x) adding x to one word (an atomic on the device)
template <class Add>
__host__ __device__ inline void fx_accumulate(vp_fx* a, double v, Add add) {
    if (v == 0.0) return;
    int k;
    long long d0, d1, d2;
    if (!fx_digits(v, k, d0, d1, d2)) {
        a->flag = 1;  // a flag only ever set: a plain store is race-free in effect
        return;
    }
    // k <= 4, and d2 != 0 only where k <= 3: sh <= 138 puts the significand's top bit at most at bit 190
    if (d0) add(&a->d[k], d0);
    if (d1) add(&a->d[k + 1], d1);
    if (d2) add(&a->d[k + 2], d2);
}

#ifdef __CUDACC__
__device__ __forceinline__ void fx_add(vp_fx* a, double v) {
    fx_accumulate(a, v, [](long long* p, long long x) {
        atomicAdd(reinterpret_cast<unsigned long long*>(p), (unsigned long long)x);  // two's complement, mod 2^64
    });
}
#endif

// the accumulated value, rounded to double (NaN if a non-finite or out-of-range value was added)
__host__ __device__ inline double fx_get(const vp_fx& a) {
    if (a.flag) return NAN;
    // resolve the carries: X = c 2^192 + sum_k u_k 2^(32 k) with digits u_k in [0, 2^32)
    unsigned long long u[6];
    long long c = 0;
    for (int k = 0; k < 6; ++k) {
        const long long t = a.d[k] + c;
        u[k] = (unsigned long long)t & 0xffffffffull;
        c = t >> 32;  // arithmetic shift: the floor of t / 2^32
    }
    if (c != 0 && c != -1) return NAN;  // beyond the range
    unsigned long long w0 = u[0] | (u[1] << 32), w1 = u[2] | (u[3] << 32), w2 = u[4] | (u[5] << 32);
    const bool neg = c < 0;
    if (neg) {  // |X| = 2^192 - (w0, w1, w2)
        w0 = ~w0 + 1;
        const unsigned long long c0 = w0 == 0;
        w1 = ~w1 + c0;
        const unsigned long long c1 = c0 & (w1 == 0);
        w2 = ~w2 + c1;
    }
    // non-negative words, each converted with one rounding and scaled exactly; summed smallest first
    const double r = (double(w0) * 0x1p-130 + double(w1) * 0x1p-66) + double(w2) * 0x1p-2;
    return neg ? -r : r;
}
