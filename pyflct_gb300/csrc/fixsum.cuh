// fixsum.cuh -- exact box sums of doubles in 128-bit fixed point.
//
// The local means of the reference are FP64 box sums (source/flct.c:815-827).
// GB300's FP64 pipe is narrow, and sliding FP64 sums round differently for
// every run partition.  Here the doubles of a span of one row become
// two's-complement 128-bit integers in units of 2^(e - 1137), e = the span's
// largest biased exponent over its finite values (max(e, 1) for
// subnormals): a 53-bit significand lands at or below bit 114, so the sum
// of up to 4096 of them (a 64 x 64 box) stays below 2^127.  Bits below the
// unit are dropped, which touches only values 2^62 times smaller than the
// span's largest.  Row sums carry their span's exponent; a run of box sums
// down a grid column takes the largest exponent of the row sums it reads
// and shifts the others down to it (again dropping only bits 2^62 below the
// largest).  Spans and runs are fixed by the frame geometry alone, and
// integer sums are exact, so every box sum is the same for any order, run
// length or band split, and is rounded once when it becomes a double.
// Non-finite inputs are counted instead (NaN, +inf and -inf in 16-bit
// fields) and give the value a sequential double sum would have: NaN with
// any NaN or with both infinities, else the infinity present.
#pragma once
#include <cuda_runtime.h>

namespace flct {

struct BoxSum {
    unsigned long long lo, hi;  // fixed-point sum
    unsigned long long cnt;     // NaN | +inf << 16 | -inf << 32 counts
    unsigned long long e;       // the unit's exponent (the sum is in units of 2^(e - 1137))
};

__device__ __forceinline__ void add128(unsigned long long& lo, unsigned long long& hi, unsigned long long bl,
                                       unsigned long long bh) {
    asm("add.cc.u64 %0, %0, %2;\n\taddc.u64 %1, %1, %3;" : "+l"(lo), "+l"(hi) : "l"(bl), "l"(bh));
}
__device__ __forceinline__ void sub128(unsigned long long& lo, unsigned long long& hi, unsigned long long bl,
                                       unsigned long long bh) {
    asm("sub.cc.u64 %0, %0, %2;\n\tsubc.u64 %1, %1, %3;" : "+l"(lo), "+l"(hi) : "l"(bl), "l"(bh));
}

// Arithmetic right shift of a two's-complement 128-bit value by d >= 0
// (d >= 127 leaves the sign).
__device__ __forceinline__ void sar128(unsigned long long& lo, unsigned long long& hi, int d) {
    if (d >= 127) {
        lo = hi = (unsigned long long)((long long)hi >> 63);
    } else if (d >= 64) {
        lo = (unsigned long long)((long long)hi >> (d - 64));
        hi = (unsigned long long)((long long)hi >> 63);
    } else if (d > 0) {
        lo = (lo >> d) | (hi << (64 - d));
        hi = (unsigned long long)((long long)hi >> d);
    }
}

// acc (four 32-bit words, two's complement) += x in units of 2^(ee - 1137);
// a non-finite x adds to the packed count instead (NaN | +inf << 10 |
// -inf << 20, for at most 1023 values).  The 53-bit significand is placed
// with three funnel shifts in a 192-bit window whose top 128 bits hold the
// value; the sign enters as (w ^ s) + (s & 1).
__device__ __forceinline__ void fx_accum(double x, int ee, unsigned (&acc)[4], unsigned& cnt) {
    const unsigned bl = (unsigned)__double2loint(x), bh = (unsigned)__double2hiint(x);
    const int e = (int)((bh >> 20) & 0x7ffu);
    const bool nf = e == 0x7ff;
    const unsigned mh = (bh & 0xfffffu) | (e ? 0x100000u : 0u);
    int t = min((e ? e : 1) - ee + 126, 126);  // shift in the window; < 0: below the unit
    if (nf) t = -1;
    const int q = t >> 5;  // -1 .. 3
    const unsigned r = (unsigned)t & 31u;
    const unsigned t0 = bl << r, t1 = __funnelshift_l(bl, mh, r), t2 = __funnelshift_l(mh, 0u, r);
    // t0, t1, t2 sit at window words q, q + 1, q + 2; the value is words 2..5
    const bool q3 = q == 3, q2 = q == 2, q1 = q == 1, q0 = q == 0;
    unsigned w[4];
    w[0] = q2 ? t0 : q1 ? t1 : q0 ? t2 : 0u;
    w[1] = q3 ? t0 : q2 ? t1 : q1 ? t2 : 0u;
    w[2] = q3 ? t1 : q2 ? t2 : 0u;
    w[3] = q3 ? t2 : 0u;
    const unsigned sg = (unsigned)((int)bh >> 31);
    asm("{\n.reg .u32 c;\n"
        "add.cc.u32 c, %4, 0xffffffff;\n"
        "addc.cc.u32 %0, %0, %5;\n"
        "addc.cc.u32 %1, %1, %6;\n"
        "addc.cc.u32 %2, %2, %7;\n"
        "addc.u32 %3, %3, %8;\n}"
        : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3])
        : "r"(sg & 1u), "r"(w[0] ^ sg), "r"(w[1] ^ sg), "r"(w[2] ^ sg), "r"(w[3] ^ sg));
    if (nf) cnt += (bl | (bh & 0xfffffu)) ? 1u : (sg ? (1u << 20) : (1u << 10));
}

// a += b, a -= b on four-word values.
__device__ __forceinline__ void add4(unsigned (&a)[4], const unsigned (&b)[4]) {
    asm("add.cc.u32 %0, %0, %4;\n\taddc.cc.u32 %1, %1, %5;\n\taddc.cc.u32 %2, %2, %6;\n\taddc.u32 %3, %3, %7;"
        : "+r"(a[0]), "+r"(a[1]), "+r"(a[2]), "+r"(a[3])
        : "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]));
}
__device__ __forceinline__ void sub4(unsigned (&a)[4], const unsigned (&b)[4]) {
    asm("sub.cc.u32 %0, %0, %4;\n\tsubc.cc.u32 %1, %1, %5;\n\tsubc.cc.u32 %2, %2, %6;\n\tsubc.u32 %3, %3, %7;"
        : "+r"(a[0]), "+r"(a[1]), "+r"(a[2]), "+r"(a[3])
        : "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]));
}

// The packed 10-bit counts of fx_accum as BoxSum's 16-bit fields.
__device__ __forceinline__ unsigned long long cnt_wide(unsigned c) {
    return (unsigned long long)(c & 0x3ffu) | ((unsigned long long)((c >> 10) & 0x3ffu) << 16) |
           ((unsigned long long)((c >> 20) & 0x3ffu) << 32);
}

// The double nearest to s (units of 2^(ee - 1137)), or the non-finite value
// its counts give.
__device__ __forceinline__ double fx_to_double(const BoxSum& s, int ee) {
    const unsigned nan = (unsigned)(s.cnt & 0xffff), pinf = (unsigned)((s.cnt >> 16) & 0xffff),
                   ninf = (unsigned)((s.cnt >> 32) & 0xffff);
    if (nan || (pinf && ninf)) return __longlong_as_double(0x7ff8000000000000ll);
    if (pinf) return __longlong_as_double(0x7ff0000000000000ll);
    if (ninf) return __longlong_as_double((long long)0xfff0000000000000ull);
    unsigned long long lo = s.lo, hi = s.hi;
    const bool neg = (long long)hi < 0;
    if (neg) {
        lo = ~lo + 1ull;
        hi = ~hi + (lo == 0ull ? 1ull : 0ull);
    }
    if (!hi && !lo) return 0.0;
    const int lz = hi ? __clzll((long long)hi) : 64 + __clzll((long long)lo);
    unsigned long long th, tl;  // the magnitude shifted so that its leading 1 is bit 127
    if (lz >= 64) {
        th = lo << (lz - 64);
        tl = 0ull;
    } else if (lz > 0) {
        th = (hi << lz) | (lo >> (64 - lz));
        tl = lo << lz;
    } else {
        th = hi;
        tl = lo;
    }
    unsigned long long mant = th >> 11;  // 53 bits
    const bool rnd = (th >> 10) & 1ull, sticky = ((th & 0x3ffull) | tl) != 0ull;
    int p = 127 - lz;  // unit exponent of the leading bit
    if (rnd && (sticky || (mant & 1ull))) {  // to nearest, ties to even
        ++mant;
        if (mant >> 53) {
            mant >>= 1;
            ++p;
        }
    }
    // mant * 2^(p - 52) units of 2^(ee - 1137): biased exponent p + ee - 114
    const int E = p + ee - 114;
    double d;
    if (E >= 1 && E <= 2046)
        d = __longlong_as_double((long long)(((unsigned long long)E << 52) | (mant & 0xfffffffffffffull)));
    else
        d = scalbn((double)mant, p - 52 + ee - 1137);  // subnormal or beyond the double range
    return neg ? -d : d;
}

}  // namespace flct
