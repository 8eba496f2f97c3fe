// Exact sums of pole rings (update_poles, drainage.rs:480-503) in 256-bit fixed point.
//
// Every f32 word (the thickness, and its low word in the compensated storage) is converted to a
// two's-complement integer in units of 2^-96 m, truncated toward zero, and added with integer
// arithmetic. Integer addition is associative, so a ring's total is the same whichever way its
// cells are grouped - per lane, per warp, per block or over a strip of blocks - and the kernels and
// the oracle agree bit for bit by construction. The total converts to the correctly rounded double;
// the mean is that double divided by the ring length.
//
// Range: any finite f32 (< 2^128 m) times 2^96 fits in 224 bits, and 2^16 of them in 240, so four
// 64-bit limbs hold every sum exactly (the unstable polar rows of a coarse time step do reach
// kilometres before they collapse). Resolution: 2^-96 m per word, far below the lowest bit of any
// low word of a film thicker than 1e-20 m. An infinite or NaN word makes the mean NaN.
//
// Why not floating point: GB300 issues FP64 at a small fraction of its FP32 rate, and the
// compensated double sums this replaces cost ~2,000 SM cycles per warp and ring; a polar strip
// whose warps share a few SMs waited on them for ~10 us per pole step. The integer form costs a
// few dozen integer instructions per word.
#pragma once

#include <cuda_runtime.h>

namespace sbs {

constexpr int kFixShift = 96;  // units: 2^-96 m

struct FixSum {
    unsigned long long w0, w1, w2, w3;  // two's complement, little-endian limbs
    unsigned bad;                       // nonzero: a word was infinite or NaN
    unsigned pad;
};

__host__ __device__ inline FixSum fix_zero() { return FixSum{0ull, 0ull, 0ull, 0ull, 0u, 0u}; }

// a += (b0, b1, b2, b3) with carries
__host__ __device__ inline void fix_add_limbs(FixSum &a, unsigned long long b0, unsigned long long b1,
                                              unsigned long long b2, unsigned long long b3) {
    const unsigned long long s0 = a.w0 + b0;
    unsigned long long c = s0 < b0 ? 1ull : 0ull;
    unsigned long long s1 = a.w1 + b1;
    unsigned long long c1 = s1 < b1 ? 1ull : 0ull;
    s1 += c;
    c1 |= (s1 < c) ? 1ull : 0ull;
    unsigned long long s2 = a.w2 + b2;
    unsigned long long c2 = s2 < b2 ? 1ull : 0ull;
    s2 += c1;
    c2 |= (s2 < c1) ? 1ull : 0ull;
    a.w0 = s0;
    a.w1 = s1;
    a.w2 = s2;
    a.w3 = a.w3 + b3 + c2;
}

__host__ __device__ inline void fix_add(FixSum &a, const FixSum &b) {
    fix_add_limbs(a, b.w0, b.w1, b.w2, b.w3);
    a.bad |= b.bad;
}

__host__ __device__ inline void fix_negate(unsigned long long &w0, unsigned long long &w1, unsigned long long &w2,
                                           unsigned long long &w3) {
    w0 = ~w0 + 1ull;
    unsigned long long c = w0 == 0ull ? 1ull : 0ull;
    w1 = ~w1 + c;
    c = (c && w1 == 0ull) ? 1ull : 0ull;
    w2 = ~w2 + c;
    c = (c && w2 == 0ull) ? 1ull : 0ull;
    w3 = ~w3 + c;
}

// a += x, exactly (x truncated toward zero to a multiple of 2^-96).
__host__ __device__ inline void fix_add_float(FixSum &a, float x) {
    unsigned u;
#ifdef __CUDA_ARCH__
    u = __float_as_uint(x);
#else
    __builtin_memcpy(&u, &x, 4);
#endif
    const unsigned E = (u >> 23) & 0xffu, M = u & 0x7fffffu;
    if (E == 0xffu) {  // infinity or NaN
        a.bad = 1u;
        return;
    }
    const unsigned long long m = E ? (unsigned long long)(M | 0x800000u) : (unsigned long long)M;
    if (m == 0ull) return;
    const int sh = (E ? (int)E : 1) - 150 + kFixShift;  // x = m 2^(sh - 96), sh in [-53, 200]
    unsigned long long w0 = 0ull, w1 = 0ull, w2 = 0ull, w3 = 0ull;
    if (sh < 0) {
        w0 = sh > -24 ? m >> -sh : 0ull;
    } else {
        const int q = sh >> 6, r = sh & 63;
        const unsigned long long low = m << r, high = r > 40 ? m >> (64 - r) : 0ull;  // m spans limbs q, q + 1
        w0 = q == 0 ? low : 0ull;
        w1 = q == 1 ? low : (q == 0 ? high : 0ull);
        w2 = q == 2 ? low : (q == 1 ? high : 0ull);
        w3 = q == 3 ? low : (q == 2 ? high : 0ull);
    }
    if (u >> 31) fix_negate(w0, w1, w2, w3);
    fix_add_limbs(a, w0, w1, w2, w3);
}

__host__ __device__ inline int fix_clz64(unsigned long long v) {
#ifdef __CUDA_ARCH__
    return __clzll((long long)v);
#else
    return __builtin_clzll(v);
#endif
}

// The correctly rounded double of the exact total (NaN if a word was not finite).
__host__ __device__ inline double fix_to_double(const FixSum &a) {
    if (a.bad) {
#ifdef __CUDA_ARCH__
        return __longlong_as_double(0x7ff8000000000000ll);
#else
        return __builtin_nan("");
#endif
    }
    unsigned long long w0 = a.w0, w1 = a.w1, w2 = a.w2, w3 = a.w3;
    const bool neg = (w3 >> 63) != 0ull;
    if (neg) fix_negate(w0, w1, w2, w3);
    // bit length of the magnitude
    int bits = 0;
    if (w3)
        bits = 256 - fix_clz64(w3);
    else if (w2)
        bits = 192 - fix_clz64(w2);
    else if (w1)
        bits = 128 - fix_clz64(w1);
    else if (w0)
        bits = 64 - fix_clz64(w0);
    double d;
    int scale = -kFixShift;
    if (bits <= 64) {
        d = (double)w0;  // round to nearest even
    } else {
        // the top 64 bits (value >> sh) plus a sticky bit for everything below them
        const int sh = bits - 64, q = sh >> 6, r = sh & 63;
        const unsigned long long lq = q == 0 ? w0 : q == 1 ? w1 : q == 2 ? w2 : w3;
        const unsigned long long lq1 = q == 0 ? w1 : q == 1 ? w2 : q == 2 ? w3 : 0ull;
        unsigned long long top = r ? (lq >> r) | (lq1 << (64 - r)) : lq;
        bool sticky = r ? (lq << (64 - r)) != 0ull : false;
        sticky = sticky || (q >= 1 && w0) || (q >= 2 && w1) || (q >= 3 && w2);
        top |= sticky ? 1ull : 0ull;
        d = (double)top;
        scale += sh;
    }
    // exact scaling by a power of two (scale in [-96, 96])
    const unsigned long long pbits = (unsigned long long)(1023 + scale) << 52;
    double p;
#ifdef __CUDA_ARCH__
    p = __longlong_as_double((long long)pbits);
#else
    __builtin_memcpy(&p, &pbits, 8);
#endif
    d *= p;
    return neg ? -d : d;
}

#ifdef __CUDACC__
__device__ __forceinline__ FixSum fix_shfl_xor(const FixSum &a, int o) {
    FixSum b;
    b.w0 = __shfl_xor_sync(0xffffffffu, a.w0, o);
    b.w1 = __shfl_xor_sync(0xffffffffu, a.w1, o);
    b.w2 = __shfl_xor_sync(0xffffffffu, a.w2, o);
    b.w3 = __shfl_xor_sync(0xffffffffu, a.w3, o);
    b.bad = __shfl_xor_sync(0xffffffffu, a.bad, o);
    b.pad = 0u;
    return b;
}

// Butterfly over the warp: every lane ends with the warp's total.
__device__ __forceinline__ void fix_warp(FixSum &a) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) fix_add(a, fix_shfl_xor(a, o));
}

// A partial written by another block (read through L2).
__device__ __forceinline__ FixSum fix_ldcg(const FixSum *p) {
    FixSum v;
    v.w0 = __ldcg(&p->w0);
    v.w1 = __ldcg(&p->w1);
    v.w2 = __ldcg(&p->w2);
    v.w3 = __ldcg(&p->w3);
    v.bad = __ldcg(&p->bad);
    v.pad = 0u;
    return v;
}
#endif

}  // namespace sbs
