// fft_reg.cuh -- register-resident mixed-radix FFT for one thread.
//
// A length-L complex transform of an array held in a thread's registers,
// fully unrolled at compile time: decimation in time, L = R * M with R in
// {4, 2, 3, 5, 7, ...} (a prime R > 5 uses the symmetric-pair DFT), so every
// box size the sliding window can take (n = 2*nsize, a multiple of 4) has a
// kernel.  Input n sits in register dit_in<L>(n) (a digit reversal), output
// frequency k in register k; every index is a compile-time constant, so the
// permutation costs nothing.  The combining butterflies of radix 4 and 2
// fuse their twiddle products into their sums with FMAs (a + w b in four
// FMAs, a - w b = 2a - (a + w b) in two), ~8% fewer FP32 operations than
// twiddling after the butterflies.
//
// Twiddles are compile-time constants: the angle 2*pi*k/L is reduced exactly
// with integer arithmetic to the first octant and evaluated by a Taylor
// series in double inside constexpr functions (written for this project),
// then rounded once to float.
#pragma once
#include <cuda_runtime.h>
#include <type_traits>

#define FLCT_HD __host__ __device__ __forceinline__

namespace flct {

// ------------------------------------------------ compile-time helpers --

template <int B, int E, class F>
FLCT_HD void sfor(F&& f) {
    if constexpr (B < E) {
        f(std::integral_constant<int, B>{});
        sfor<B + 1, E>(f);
    }
}

constexpr double kPi = 3.14159265358979323846264338327950288;

constexpr double taylor_sin(double y) {
    double term = y, sum = y, y2 = y * y;
    for (int k = 1; k < 14; ++k) {
        term *= -y2 / ((2.0 * k) * (2.0 * k + 1.0));
        sum += term;
    }
    return sum;
}

constexpr double taylor_cos(double y) {
    double term = 1.0, sum = 1.0, y2 = y * y;
    for (int k = 1; k < 14; ++k) {
        term *= -y2 / ((2.0 * k - 1.0) * (2.0 * k));
        sum += term;
    }
    return sum;
}

// cos and sin of 2*pi*num/den, with the angle reduced exactly to
// [-pi/4, pi/4] plus a whole number of quarter turns.
struct CS {
    double c, s;
};
constexpr CS ct_cossin(long num, long den) {
    long r = ((num % den) + den) % den;            // [0, den)
    long q = (8 * r + den) / (2 * den);            // nearest quarter turn, 0..4
    long rem = 4 * r - q * den;                    // angle = 2pi*(q/4 + rem/(4den))
    double y = 2.0 * kPi * (double)rem / (4.0 * (double)den);
    double c = taylor_cos(y), s = taylor_sin(y);
    switch (q % 4) {
        case 0: return {c, s};
        case 1: return {-s, c};
        case 2: return {-c, -s};
        default: return {s, -c};
    }
}

template <int L>
constexpr int radix_of() {
    if constexpr (L % 4 == 0) return 4;
    else if constexpr (L % 2 == 0) return 2;
    else if constexpr (L % 3 == 0) return 3;
    else if constexpr (L % 5 == 0) return 5;
    else if constexpr (L % 7 == 0) return 7;
    else if constexpr (L % 11 == 0) return 11;
    else if constexpr (L % 13 == 0) return 13;
    else return L;
}

// ------------------------------------------------------ complex helpers --

// Complex add / subtract / scale-and-add on the packed FP32 pipe: one
// add.f32x2 (sub, fma) instruction for the (re, im) pair instead of two
// scalar ones.  The FFTs are issue-bound, and these are most of their work.
#if defined(__CUDA_ARCH__)
#define FLCT_PACKED_OP(OP)                                                                   \
    float2 r;                                                                                \
    asm("{\n.reg .b64 ra, rb, rd;\nmov.b64 ra, {%2, %3};\nmov.b64 rb, {%4, %5};\n" OP   \
        " rd, ra, rb;\nmov.b64 {%0, %1}, rd;\n}"                                             \
        : "=f"(r.x), "=f"(r.y)                                                               \
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));                                           \
    return r;
FLCT_HD float2 cadd(float2 a, float2 b) { FLCT_PACKED_OP("add.rn.f32x2") }
FLCT_HD float2 csub(float2 a, float2 b) { FLCT_PACKED_OP("sub.rn.f32x2") }
// element-wise product (a.x * b.x, a.y * b.y)
FLCT_HD float2 emul(float2 a, float2 b) { FLCT_PACKED_OP("mul.rn.f32x2") }
// a * k for a real k
FLCT_HD float2 cscale(float2 a, float k) {
    float2 r;
    asm("{\n.reg .b64 ra, rk, rd;\nmov.b64 ra, {%2, %3};\nmov.b64 rk, {%4, %4};\n"
        "mul.rn.f32x2 rd, ra, rk;\nmov.b64 {%0, %1}, rd;\n}"
        : "=f"(r.x), "=f"(r.y)
        : "f"(a.x), "f"(a.y), "f"(k));
    return r;
}
// a * k + b for a real k
FLCT_HD float2 cfma(float2 a, float k, float2 b) {
    float2 r;
    asm("{\n.reg .b64 ra, rk, rb, rd;\nmov.b64 ra, {%2, %3};\nmov.b64 rk, {%4, %4};\nmov.b64 rb, {%5, %6};\n"
        "fma.rn.f32x2 rd, ra, rk, rb;\nmov.b64 {%0, %1}, rd;\n}"
        : "=f"(r.x), "=f"(r.y)
        : "f"(a.x), "f"(a.y), "f"(k), "f"(b.x), "f"(b.y));
    return r;
}
#undef FLCT_PACKED_OP
#else
FLCT_HD float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
FLCT_HD float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
FLCT_HD float2 cfma(float2 a, float k, float2 b) { return make_float2(fmaf(a.x, k, b.x), fmaf(a.y, k, b.y)); }
FLCT_HD float2 cscale(float2 a, float k) { return make_float2(a.x * k, a.y * k); }
FLCT_HD float2 emul(float2 a, float2 b) { return make_float2(a.x * b.x, a.y * b.y); }
#endif
// Scalar forms, for operands that are swapped or negated halves of a pair
// (a packed instruction would first need them moved into a register pair).
FLCT_HD float2 cadd_s(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
FLCT_HD float2 csub_s(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
// multiply by DIR*i
template <int DIR>
FLCT_HD float2 mul_i(float2 a) {
    if constexpr (DIR < 0) return make_float2(a.y, -a.x);
    else return make_float2(-a.y, a.x);
}

// a * exp(DIR * 2*pi*i * NUM/DEN), specialised for the exact cases.
template <int DIR, long NUM, long DEN>
FLCT_HD float2 twmul(float2 a) {
    constexpr long r = ((NUM % DEN) + DEN) % DEN;
    if constexpr (r == 0) {
        return a;
    } else if constexpr (4 * r == DEN) {
        return mul_i<DIR>(a);
    } else if constexpr (2 * r == DEN) {
        return make_float2(-a.x, -a.y);
    } else if constexpr (4 * r == 3 * DEN) {
        return mul_i<-DIR>(a);
    } else if constexpr (8 * r == DEN || 8 * r == 3 * DEN || 8 * r == 5 * DEN || 8 * r == 7 * DEN) {
        constexpr CS w = ct_cossin(r, DEN);
        constexpr float c = (float)w.c, s = (float)(DIR * w.s);
        // |c| == |s| at odd multiples of pi/4
        constexpr float h = c;
        if constexpr ((c > 0) == (s > 0)) {
            return make_float2(h * (a.x - a.y), h * (a.x + a.y));
        } else {
            return make_float2(h * (a.x + a.y), h * (a.y - a.x));
        }
    } else {
        constexpr CS w = ct_cossin(r, DEN);
        constexpr float c = (float)w.c, s = (float)(DIR * w.s);
        return make_float2(a.x * c - a.y * s, a.x * s + a.y * c);
    }
}

// ----------------------------------------------------------- butterflies --

template <int R, int DIR>
FLCT_HD void small_dft(float2* t) {
    if constexpr (R == 2) {
        float2 a = t[0], b = t[1];
        t[0] = cadd(a, b);
        t[1] = csub(a, b);
    } else if constexpr (R == 4) {
        float2 s0 = cadd(t[0], t[2]), s1 = csub(t[0], t[2]);
        float2 s2 = cadd(t[1], t[3]), s3 = mul_i<DIR>(csub(t[1], t[3]));
        t[0] = cadd(s0, s2);
        t[2] = csub(s0, s2);
        t[1] = cadd_s(s1, s3);
        t[3] = csub_s(s1, s3);
    } else if constexpr (R == 3) {
        constexpr float h = 0.866025403784438646763723170752936183f;
        float2 p = cadd(t[1], t[2]), m = csub(t[1], t[2]);
        float2 a = t[0];
        float2 u = cfma(p, -0.5f, a);
        float2 v = mul_i<DIR>(make_float2(h * m.x, h * m.y));
        t[0] = cadd(a, p);
        t[1] = cadd(u, v);
        t[2] = csub(u, v);
    } else if constexpr (R == 5) {
        constexpr CS w1 = ct_cossin(1, 5), w2 = ct_cossin(2, 5);
        constexpr float c1 = (float)w1.c, c2 = (float)w2.c, s1 = (float)w1.s, s2 = (float)w2.s;
        float2 x0 = t[0];
        float2 a1 = cadd(t[1], t[4]), a2 = cadd(t[2], t[3]);
        float2 b1 = csub(t[1], t[4]), b2 = csub(t[2], t[3]);
        float2 t1 = cfma(a2, c2, cfma(a1, c1, x0));
        float2 t2 = cfma(a2, c1, cfma(a1, c2, x0));
        float2 u1 = mul_i<DIR>(make_float2(s1 * b1.x + s2 * b2.x, s1 * b1.y + s2 * b2.y));
        float2 u2 = mul_i<DIR>(make_float2(s2 * b1.x - s1 * b2.x, s2 * b1.y - s1 * b2.y));
        t[0] = cadd(cadd(x0, a1), a2);
        t[1] = cadd(t1, u1);
        t[4] = csub(t1, u1);
        t[2] = cadd(t2, u2);
        t[3] = csub(t2, u2);
    } else {
        // odd prime R by symmetric pairs: with a_k = t[k] + t[R-k] and
        // b_k = t[k] - t[R-k] (k = 1..H, H = (R-1)/2),
        //   X[s]   = t[0] + sum_k a_k cos(2 pi k s / R) + DIR i sum_k b_k sin(2 pi k s / R)
        //   X[R-s] = the same with - DIR i,
        // real coefficients on packed FMAs: 2H^2 + O(H) operations instead
        // of the (R-1)^2 complex products of a direct DFT
        static_assert(R % 2 == 1, "symmetric DFT needs an odd length");
        constexpr int H = (R - 1) / 2;
        float2 a[H + 1], b[H + 1];
        sfor<1, H + 1>([&](auto kc) {
            constexpr int k = decltype(kc)::value;
            a[k] = cadd(t[k], t[R - k]);
            b[k] = csub(t[k], t[R - k]);
        });
        const float2 x0 = t[0];
        float2 sum = x0;
        sfor<1, H + 1>([&](auto kc) { sum = cadd(sum, a[decltype(kc)::value]); });
        sfor<1, H + 1>([&](auto sc) {
            constexpr int sidx = decltype(sc)::value;
            float2 tr = x0, ui = make_float2(0.f, 0.f);
            sfor<1, H + 1>([&](auto kc) {
                constexpr int k = decltype(kc)::value;
                constexpr CS w = ct_cossin((long)k * sidx, R);
                tr = cfma(a[k], (float)w.c, tr);
                ui = cfma(b[k], (float)w.s, ui);
            });
            const float2 v = mul_i<DIR>(ui);
            t[sidx] = cadd_s(tr, v);
            t[R - sidx] = csub_s(tr, v);
        });
        t[0] = sum;
    }
}

// ------------------------------------------------- DIT, fused twiddles --

// a + b w, w = exp(DIR * 2*pi*i * NUM/DEN), with the product fused into
// the sum: FMAs for a general twiddle, two adds and two FMAs at odd
// multiples of pi/4, a packed add or a swap for the exact cases.
template <int DIR, long NUM, long DEN>
FLCT_HD float2 tw_fma_add(float2 a, float2 b) {
    constexpr long r = ((NUM % DEN) + DEN) % DEN;
    if constexpr (r == 0) {
        return cadd(a, b);
    } else if constexpr ((4 * r) % DEN == 0) {
        return cadd_s(a, twmul<DIR, NUM, DEN>(b));
    } else if constexpr (8 * r == DEN || 8 * r == 3 * DEN || 8 * r == 5 * DEN || 8 * r == 7 * DEN) {
        constexpr CS w = ct_cossin(r, DEN);
        constexpr float c = (float)w.c, s = (float)(DIR * w.s);
        constexpr float h = c;
        if constexpr ((c > 0) == (s > 0)) {
            return make_float2(fmaf(h, b.x - b.y, a.x), fmaf(h, b.x + b.y, a.y));
        } else {
            return make_float2(fmaf(h, b.x + b.y, a.x), fmaf(h, b.y - b.x, a.y));
        }
    } else {
        constexpr CS w = ct_cossin(r, DEN);
        constexpr float c = (float)w.c, s = (float)(DIR * w.s);
        return make_float2(fmaf(c, b.x, fmaf(-s, b.y, a.x)), fmaf(c, b.y, fmaf(s, b.x, a.y)));
    }
}

// p = a + b w, m = a - b w; with a non-trivial twiddle m = 2a - p (one
// FMA per component instead of a second product).
template <int DIR, long NUM, long DEN>
FLCT_HD void tw_pair(float2 a, float2 b, float2& p, float2& m) {
    constexpr long r = ((NUM % DEN) + DEN) % DEN;
    if constexpr (r == 0) {
        p = cadd(a, b);
        m = csub(a, b);
    } else if constexpr ((4 * r) % DEN == 0) {
        const float2 tb = twmul<DIR, NUM, DEN>(b);
        p = cadd_s(a, tb);
        m = csub_s(a, tb);
    } else {
        p = tw_fma_add<DIR, NUM, DEN>(a, b);
        m = make_float2(fmaf(2.0f, a.x, -p.x), fmaf(2.0f, a.y, -p.y));
    }
}

// Register position of input n for dit<L>: the mixed-radix digit reversal
// (input r + R m of a level goes to sub-transform r, position m).
template <int L>
constexpr int dit_in(int n) {
    if constexpr (L == 1) {
        return 0;
    } else {
        constexpr int R = radix_of<L>(), M = L / R;
        return (n % R) * M + dit_in<M>(n / R);
    }
}

// In-place decimation-in-time transform of x[OFF .. OFF+L): input n at
// x[OFF + dit_in<L>(n)], output k at x[OFF + k].  The R sub-transforms of
// length M = L/R come first; the combining butterflies take their inputs
// times the twiddles w_L^(r k), fused into the butterflies' sums for
// radix 4 and 2.  DIR = -1 forward, +1 backward; unnormalised.
template <int L, int OFF, int DIR>
FLCT_HD void dit(float2* x) {
    if constexpr (L > 1) {
        constexpr int R = radix_of<L>(), M = L / R;
        sfor<0, R>([&](auto rc) {
            constexpr int r = decltype(rc)::value;
            dit<M, OFF + r * M, DIR>(x);
        });
        sfor<0, M>([&](auto kc) {
            constexpr int k = decltype(kc)::value;
            if constexpr (R == 4) {
                float2 t0, t1, t2, t3;
                tw_pair<DIR, 2L * k, L>(x[OFF + k], x[OFF + k + 2 * M], t0, t1);
                const float2 a1 = twmul<DIR, (long)k, L>(x[OFF + k + M]);
                tw_pair<DIR, 3L * k, L>(a1, x[OFF + k + 3 * M], t2, t3);
                const float2 r3 = mul_i<DIR>(t3);
                x[OFF + k] = cadd(t0, t2);
                x[OFF + k + 2 * M] = csub(t0, t2);
                x[OFF + k + M] = cadd_s(t1, r3);
                x[OFF + k + 3 * M] = csub_s(t1, r3);
            } else if constexpr (R == 2) {
                float2 t0, t1;
                tw_pair<DIR, (long)k, L>(x[OFF + k], x[OFF + k + M], t0, t1);
                x[OFF + k] = t0;
                x[OFF + k + M] = t1;
            } else {
                float2 t[R];
                t[0] = x[OFF + k];
                sfor<1, R>([&](auto rc) {
                    constexpr int r = decltype(rc)::value;
                    t[r] = twmul<DIR, (long)r * k, L>(x[OFF + k + r * M]);
                });
                small_dft<R, DIR>(t);
                sfor<0, R>([&](auto sc) {
                    constexpr int s = decltype(sc)::value;
                    x[OFF + k + s * M] = t[s];
                });
            }
        });
    }
}

// The transform the window kernel uses: input n at x[fft_in<L>(n)], output
// k at x[fft_out<L>(k)].
template <int L>
constexpr int fft_in(int n) { return dit_in<L>(n); }
template <int L>
constexpr int fft_out(int k) { return k; }
template <int L, int OFF, int DIR>
FLCT_HD void fft(float2* x) { dit<L, OFF, DIR>(x); }

}  // namespace flct
