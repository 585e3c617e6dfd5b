// Order-independent FP64 sums: a 192-bit two's-complement fixed-point accumulator (least significant bit 2^-130,
// range +-2^61) updated by integer atomics. Each added double is rounded once to the accumulator's grid (an absolute
// 2^-131 at most, below 1e-39); after that every update is an exact integer addition modulo 2^192, so the total does
// not depend on the order in which the atomics land and a sum scattered from many threads is the same bit for bit
// from run to run. A non-finite addend sets a flag word that makes the value read back NaN.
//
// Addition of X = w0 + 2^64 w1 + 2^128 w2 with three 64-bit atomics: the carry out of each word's atomic, seen in the
// value it returned, goes into the next word's addend. Summed over every update, the carries add up to the exact
// total's carries, whatever the interleaving.
#pragma once
#include <cmath>
#include <cstring>

struct vp_fx {
    unsigned long long w[4];  // w[0..2] the value, least significant word first; w[3] non-finite flag
};

// a double on the accumulator's grid: the three words of round(v 2^130) in two's complement (false for a non-finite v
// or |v| >= 2^61, outside the range)
__host__ __device__ inline bool fx_words(double v, unsigned long long& w0, unsigned long long& w1,
                                         unsigned long long& w2) {
    w0 = w1 = w2 = 0;
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
    const int sh = e - 945;
    if (sh < -54) return true;  // below half a unit
    if (sh < 0)
        w0 = (m + (1ull << (-sh - 1))) >> (-sh);  // round half up
    else if (sh < 64) {
        w0 = m << sh;
        w1 = sh ? m >> (64 - sh) : 0;
    } else if (sh < 128) {
        const int s = sh - 64;
        w1 = m << s;
        w2 = s ? m >> (64 - s) : 0;
    } else if (sh <= 138) {
        w2 = m << (sh - 128);
    } else {
        return false;
    }
    if (bits >> 63) {  // negate: ~X + 1
        w0 = ~w0 + 1;
        const unsigned long long c0 = w0 == 0;
        w1 = ~w1 + c0;
        const unsigned long long c1 = c0 & (w1 == 0);
        w2 = ~w2 + c1;
    }
    return true;
}

// a += v, with add(word, x) adding x to one word and returning the word's previous value (an atomic on the device)
template <class Add>
__host__ __device__ inline void fx_accumulate(vp_fx* a, double v, Add add) {
    if (v == 0.0) return;
    unsigned long long w0, w1, w2;
    if (!fx_words(v, w0, w1, w2)) {
        a->w[3] = 1;  // a flag only ever set: a plain store is race-free in effect
        return;
    }
    unsigned long long c0 = 0;
    if (w0) {
        const unsigned long long o0 = add(&a->w[0], w0);
        c0 = o0 + w0 < o0;
    }
    const unsigned long long t1 = w1 + c0;
    unsigned long long c1 = t1 < w1;  // w1 = 2^64 - 1 and a carry in
    if (t1) {
        const unsigned long long o1 = add(&a->w[1], t1);
        c1 += o1 + t1 < o1;
    }
    const unsigned long long t2 = w2 + c1;
    if (t2) add(&a->w[2], t2);
}

#ifdef __CUDACC__
__device__ __forceinline__ void fx_add(vp_fx* a, double v) {
    fx_accumulate(a, v, [](unsigned long long* p, unsigned long long x) { return atomicAdd(p, x); });
}
#endif

// the accumulated value, rounded to double (NaN if a non-finite value was added)
__host__ __device__ inline double fx_get(const vp_fx& a) {
    if (a.w[3]) return NAN;
    unsigned long long w0 = a.w[0], w1 = a.w[1], w2 = a.w[2];
    const bool neg = (long long)w2 < 0;
    if (neg) {
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
