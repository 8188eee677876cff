// prepass.cu -- the passes before and after the window kernel.
//
//   k_absmax / k_thresh_final   relative threshold (flct.c:594-629)
//   k_classify                  threshold test, skip grid, work list, the
//                               float hi+lo split of both frames, and the
//                               final values of pixels without a window
//                               (flct.c:721-755, 918-930, 1125-1133)
//   k_rowsum / k_colsum         FP64 box sums for the local means
//                               (flct.c:815-827) as sliding sums
//   k_interp                    skip-grid cubic-convolution interpolation
//                               (flct.c:958-1120 with interpcc2d,
//                               flct.c:2226-2463) and the xmiss reset
#include "prepass.cuh"

namespace flct {

// ------------------------------------------------------- threshold ----

__device__ __forceinline__ unsigned long long warp_max_u64(unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
        v = w > v ? w : v;
    }
    return v;
}

// max(|f|) over non-NaN elements of both frames, as IEEE bit patterns
// (for non-negative doubles the bit order is the numeric order).
__global__ void k_absmax(const double* __restrict__ f1, const double* __restrict__ f2, long n,
                         unsigned long long* __restrict__ out) {
    unsigned long long m1 = 0ull, m2 = 0ull;
    const unsigned long long kAbs = 0x7fffffffffffffffull, kInf = 0x7ff0000000000000ull;
    for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) {
        unsigned long long a = (unsigned long long)__double_as_longlong(f1[k]) & kAbs;
        unsigned long long b = (unsigned long long)__double_as_longlong(f2[k]) & kAbs;
        if (a <= kInf && a > m1) m1 = a;
        if (b <= kInf && b > m2) m2 = b;
    }
    m1 = warp_max_u64(m1);
    m2 = warp_max_u64(m2);
    if ((threadIdx.x & 31) == 0) {
        atomicMax(out, m1);
        atomicMax(out + 1, m2);
    }
}

// thresh *= max(f1max, f2max), where fNmax follows maxloc's sequential scan:
// a NaN first element is never replaced (flct.c:608-621, 2142-2161).
__global__ void k_thresh_final(const double* __restrict__ f1, const double* __restrict__ f2,
                               const unsigned long long* __restrict__ mx, double thresh,
                               double* __restrict__ thr) {
    double a1 = fabs(f1[0]), a2 = fabs(f2[0]);
    double m1 = (a1 != a1) ? a1 : __longlong_as_double((long long)mx[0]);
    double m2 = (a2 != a2) ? a2 : __longlong_as_double((long long)mx[1]);
    double fmax = (m1 > m2) ? m1 : m2;
    *thr = __dmul_rn(thresh, fmax);
}

// ------------------------------------------------------- classify ----

__global__ void k_classify(ClassifyArgs a) {
    const long n = (long)a.nx * a.ny;
    const double thr = a.thr_ptr ? *a.thr_ptr : a.thr_val;
    const int lane = threadIdx.x & 31;
    const long stride = (long)gridDim.x * blockDim.x;
    // whole warps iterate together so the ballot sees every lane
    for (long base = blockIdx.x * (long)blockDim.x + (threadIdx.x & ~31); base < n; base += stride) {
        const long k = base + lane;
        const bool act = k < n;
        bool comp = false, grid = false;
        int i = 0, j = 0;
        if (act) {
            const double fa = a.f1[k], fb = a.f2[k];
            const float2 sa = split_double(fa), sb = split_double(fb);
            a.s1[k] = sa;
            a.s2[k] = sb;
            if ((isinf(sa.x) && !isinf(fa)) || (isinf(sb.x) && !isinf(fb))) atomicOr(a.status, kStatusRange);
            i = (int)(k / a.ny);
            j = (int)(k - (long)i * a.ny);
            // 0.5*|f1+f2| < thresh in FP64 (flct.c:721-722)
            const bool below = __dmul_rn(0.5, fabs(__dadd_rn(fa, fb))) < thr;
            grid = (a.skip > 0) ? (!((i - a.xoff) % a.skip) && !((j - a.yoff) % a.skip)) : true;
            comp = !below && grid;
        }
        const unsigned m = __ballot_sync(0xffffffffu, comp);
        int slot = 0;
        if (lane == 0 && m) slot = atomicAdd(a.nwork, __popc(m));
        slot = __shfl_sync(0xffffffffu, slot, 0);
        if (comp) {
            a.work[slot + __popc(m & ((1u << lane) - 1u))] = (int)k;
        } else if (act) {
            // pixels without a window: (xmiss, xmiss, 0) then the reset gives
            // (0, 0, 0); skipped pixels that will be interpolated are left to
            // k_interp.
            if (grid) {
                a.vx[k] = 0.;
                a.vy[k] = 0.;
                a.vm[k] = 0.;
                if (a.gvx) {
                    const int ic = (i - a.xoff) / a.skip, jc = (j - a.yoff) / a.skip;
                    a.gvx[(size_t)ic * a.jcnt + jc] = kXmiss;
                    a.gvy[(size_t)ic * a.jcnt + jc] = kXmiss;
                }
            } else if (!a.interpolate) {
                a.vx[k] = 0.;
                a.vy[k] = 0.;
                a.vm[k] = 0.;
            }
        }
    }
}

// ------------------------------------------------------- box sums ----

// Finite test on the bit pattern (integer ops only).
__device__ __forceinline__ bool finite_bits(double x) {
    return ((__double_as_longlong(x) >> 52) & 0x7ff) != 0x7ff;
}

// Running-sum step with the reference's direct-sum semantics for NaN and
// infinities: whenever a non-finite value enters, leaves, or is in the sum,
// the box is summed again directly, so a NaN taints only boxes holding it.
template <class Get>
__device__ __forceinline__ double slide(double sum, double in, double out, int n, Get get) {
    if (finite_bits(sum) && finite_bits(in) && finite_bits(out)) return __dsub_rn(__dadd_rn(sum, in), out);
    double t = 0.;
    for (int q = 0; q < n; ++q) t = __dadd_rn(t, get(q));
    return t;
}

// R[i][s] = sum_{jj<n} f[i][s+jj] for s in [0, ny-n]; one thread per row
// segment of kSeg outputs: n adds to start, then two per step.
__global__ void k_rowsum(const double* __restrict__ f1, const double* __restrict__ f2, int nx,
                         int ny, int n, double* __restrict__ r1, double* __restrict__ r2) {
    const int W = ny - n + 1;
    const int nseg = (W + kSeg - 1) / kSeg;
    const long idx = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (idx >= (long)nx * nseg) return;
    const int i = (int)(idx / nseg);
    const int s0 = (int)(idx - (long)i * nseg) * kSeg;
    const int s1 = min(s0 + kSeg, W);
    const double* a = f1 + (size_t)i * ny;
    const double* b = f2 + (size_t)i * ny;
    double sa = 0., sb = 0.;
    for (int jj = 0; jj < n; ++jj) {
        sa = __dadd_rn(sa, a[s0 + jj]);
        sb = __dadd_rn(sb, b[s0 + jj]);
    }
    r1[(size_t)i * W + s0] = sa;
    r2[(size_t)i * W + s0] = sb;
    for (int s = s0 + 1; s < s1; ++s) {
        sa = slide(sa, a[s + n - 1], a[s - 1], n, [&](int q) { return a[s + q]; });
        sb = slide(sb, b[s + n - 1], b[s - 1], n, [&](int q) { return b[s + q]; });
        r1[(size_t)i * W + s] = sa;
        r2[(size_t)i * W + s] = sb;
    }
}

// S[t][s] = sum_{ii<n} R[t+ii][s] for t in [0, nx-n]; consecutive threads
// take consecutive columns s (coalesced), each a segment of kSeg rows.
__global__ void k_colsum(const double* __restrict__ r1, const double* __restrict__ r2, int nx,
                         int W, int n, double* __restrict__ b1, double* __restrict__ b2) {
    const int H = nx - n + 1;
    const int nseg = (H + kSeg - 1) / kSeg;
    const long idx = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (idx >= (long)W * nseg) return;
    const int seg = (int)(idx / W);
    const int s = (int)(idx - (long)seg * W);
    const int t0 = seg * kSeg, t1 = min(t0 + kSeg, H);
    double sa = 0., sb = 0.;
    for (int ii = 0; ii < n; ++ii) {
        sa = __dadd_rn(sa, r1[(size_t)(t0 + ii) * W + s]);
        sb = __dadd_rn(sb, r2[(size_t)(t0 + ii) * W + s]);
    }
    b1[(size_t)t0 * W + s] = sa;
    b2[(size_t)t0 * W + s] = sb;
    for (int t = t0 + 1; t < t1; ++t) {
        sa = slide(sa, r1[(size_t)(t + n - 1) * W + s], r1[(size_t)(t - 1) * W + s], n,
                   [&](int q) { return r1[(size_t)(t + q) * W + s]; });
        sb = slide(sb, r2[(size_t)(t + n - 1) * W + s], r2[(size_t)(t - 1) * W + s], n,
                   [&](int q) { return r2[(size_t)(t + q) * W + s]; });
        b1[(size_t)t * W + s] = sa;
        b2[(size_t)t * W + s] = sb;
    }
}

// --------------------------------------------------- interpolation ----

// Keys cubic-convolution kernel, a = -0.5, in the reference's operation
// order (flct.c:2398-2419).
__device__ __forceinline__ double keys_r(double t) {
    return (t >= 1.0) ? __dadd_rn(__dmul_rn(__dsub_rn(__dmul_rn(__dadd_rn(__dmul_rn(-0.5, t), 2.5), t), 4.), t), 2.)
                      : __dadd_rn(__dmul_rn(__dmul_rn(__dsub_rn(__dmul_rn(1.5, t), 2.5), t), t), 1.);
}

// Value of the border-extended grid cdata[a][b], a in [0, gx+1], b in
// [0, gy+1] (flct.c:2257-2336): interior copies, one-cell borders
// extrapolated as 3 f0 - 3 f1 + f2, corners from their border column/row.
__device__ __forceinline__ double cdata_at(const double* __restrict__ f, int gx, int gy, int a, int b) {
#define F(p, q) f[(size_t)(p) * gy + (q)]
    auto row_edge = [&](int p, int q) -> double {
        // p in [0, gx-1] interior row; q in {0, gy+1} border column
        if (q == 0) return __dadd_rn(__dsub_rn(F(p, 2), __dmul_rn(3., F(p, 1))), __dmul_rn(3., F(p, 0)));
        return __dadd_rn(__dsub_rn(F(p, gy - 3), __dmul_rn(3., F(p, gy - 2))), __dmul_rn(3., F(p, gy - 1)));
    };
    auto col_edge = [&](int p, int q) -> double {
        // p in {0, gx+1} border row; q in [0, gy-1] interior column
        if (p == 0) return __dadd_rn(__dsub_rn(F(2, q), __dmul_rn(3., F(1, q))), __dmul_rn(3., F(0, q)));
        return __dadd_rn(__dsub_rn(F(gx - 3, q), __dmul_rn(3., F(gx - 2, q))), __dmul_rn(3., F(gx - 1, q)));
    };
    const bool ra = (a >= 1 && a <= gx), rb = (b >= 1 && b <= gy);
    if (ra && rb) return F(a - 1, b - 1);
    if (ra) return row_edge(a - 1, b);
    if (rb) return col_edge(a, b - 1);
    // corners: cdata(0,0) from the left border column (rows 1,2,3), etc.
    auto cd = [&](int p, int q) -> double {  // p interior (1..gx) or border; q border
        return row_edge(p - 1, q);
    };
    auto cr = [&](int p, int q) -> double {  // p border row; q interior (1..gy)
        return col_edge(p, q - 1);
    };
    if (a == 0 && b == 0)
        return __dadd_rn(__dsub_rn(__dmul_rn(3., cd(1, 0)), __dmul_rn(3., cd(2, 0))), cd(3, 0));
    if (a == gx + 1 && b == 0)
        return __dadd_rn(__dsub_rn(__dmul_rn(3., cd(gx, 0)), __dmul_rn(3., cd(gx - 1, 0))), cd(gx - 2, 0));
    if (a == 0 && b == gy + 1)
        return __dadd_rn(__dsub_rn(__dmul_rn(3., cr(0, gy)), __dmul_rn(3., cr(0, gy - 1))), cr(0, gy - 2));
    return __dadd_rn(__dsub_rn(__dmul_rn(3., cd(gx, gy + 1)), __dmul_rn(3., cd(gx - 1, gy + 1))),
                     cd(gx - 2, gy + 1));
#undef F
}

// Per-axis interpolation setup: izero (clamped), the 4 kernel weights of
// the stencil rows izero-1..izero+2, and whether the target is in range.
__global__ void k_interp_axis(int n, int gcount, int off, int skip, const double* __restrict__ want,
                              int* __restrict__ zero, double* __restrict__ wts, unsigned char* __restrict__ ok) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    // xwant = (i - offset)/skip (flct.c:1037-1071), or a caller's table
    const double x = want ? want[t] : ((double)(t - off)) / (double)(skip);
    const int it = ((int)x > 0) ? (int)x : 0;
    const int z = (it < (gcount - 2)) ? it : gcount - 2;
    zero[t] = z;
    ok[t] = !((x < 0.) || (x > (double)(gcount - 1)));
#pragma unroll
    for (int q = -1; q < 3; ++q) wts[(size_t)t * 4 + (q + 1)] = keys_r(fabs(__dsub_rn(x, (double)(z + q))));
}

// One output per thread: the 4x4 cubic convolution of the border-extended
// grid in the reference's summation order; xmiss if out of range or if any
// stencil value equals xmiss (flct.c:2373-2455).
__device__ __forceinline__ double interp_one(const double* __restrict__ g, int gx, int gy, double xmiss,
                                             int iz, const double* rx, int jz, const double* ry) {
    double acc = 0.;
    bool bad = false;
#pragma unroll
    for (int p = 0; p < 4; ++p) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int a = iz + p, b = jz + q;  // cdata indices (izero+1+ii with ii=p-1)
            double cv;
            if (a >= 1 && a <= gx && b >= 1 && b <= gy) cv = g[(size_t)(a - 1) * gy + (b - 1)];
            else cv = cdata_at(g, gx, gy, a, b);
            acc = __dadd_rn(acc, __dmul_rn(__dmul_rn(cv, rx[p]), ry[q]));
            bad |= (cv == xmiss);
        }
    }
    return bad ? xmiss : acc;
}

// Separable form of the velocity pipeline's interpolation.  Every output in
// column j contracts the same cdata rows with the same ry weights, so
//   H[a][j] = sum_q cdata[a][jz(j)+q] ry_j[q]      (k_interp_rows, once)
//   out[i][j] = sum_p rx_i[p] H[iz(i)+p][j]          (k_interp, per pixel)
// which is the reference's 4x4 sum regrouped (equal up to the last bits of
// the FP64 rounding); the xmiss test is the same set of 16 comparisons,
// split the same way, so the mask is exact.
__global__ void k_interp_rows(InterpArgs a) {
    const long n = (long)(a.gx + 2) * a.ny;
    for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) {
        const int r = (int)(k / a.ny), j = (int)(k - (long)(k / a.ny) * a.ny);
        if (!a.oky[j]) continue;  // out of range: every output of column j is xmiss
        const int jz = a.zy[j];
        double hx = 0., hy = 0.;
        unsigned char bad = 0;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const double ry = a.wy[(size_t)j * 4 + q];
            const int b = jz + q;
            double cx, cy;
            if (r >= 1 && r <= a.gx && b >= 1 && b <= a.gy) {
                cx = a.gvx[(size_t)(r - 1) * a.gy + (b - 1)];
                cy = a.gvy[(size_t)(r - 1) * a.gy + (b - 1)];
            } else {
                cx = cdata_at(a.gvx, a.gx, a.gy, r, b);
                cy = cdata_at(a.gvy, a.gx, a.gy, r, b);
            }
            hx = fma(cx, ry, hx);
            hy = fma(cy, ry, hy);
            bad |= (cx == kXmiss ? 1 : 0) | (cy == kXmiss ? 2 : 0);
        }
        a.hx[k] = hx;
        a.hy[k] = hy;
        a.hbad[k] = bad;
    }
}

__global__ void k_interp(InterpArgs a) {
    const long n = (long)a.nx * a.ny;
    for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) {
        const int i = (int)(k / a.ny), j = (int)(k - (long)(k / a.ny) * a.ny);
        const bool gi = !((i - a.xoff) % a.skip), gj = !((j - a.yoff) % a.skip);
        if (gi && gj) continue;  // grid points keep their computed value
        double vx = kXmiss, vy = kXmiss;
        if (a.okx[i] && a.oky[j]) {
            const int iz = a.zx[i];
            double sx = 0., sy = 0.;
            unsigned char bad = 0;
#pragma unroll
            for (int p = 0; p < 4; ++p) {
                const double rx = a.wx[(size_t)i * 4 + p];
                const size_t h = (size_t)(iz + p) * a.ny + j;
                sx = fma(rx, a.hx[h], sx);
                sy = fma(rx, a.hy[h], sy);
                bad |= a.hbad[h];
            }
            vx = (bad & 1) ? kXmiss : sx;
            vy = (bad & 2) ? kXmiss : sy;
        }
        double vm = 0.5;
        // the final xmiss reset (flct.c:1125-1133)
        if (vx == kXmiss) {
            vm = 0.;
            vx = 0.;
        }
        if (vy == kXmiss) vy = 0.;
        a.vx[k] = vx;
        a.vy[k] = vy;
        a.vm[k] = vm;
    }
}

// interpcc2d on caller arrays (the standalone entry point).
__global__ void k_interp_general(const double* __restrict__ f, int gx, int gy, double xmiss,
                                 const int* __restrict__ zx, const double* __restrict__ wx,
                                 const unsigned char* __restrict__ okx, int nxi, const int* __restrict__ zy,
                                 const double* __restrict__ wy, const unsigned char* __restrict__ oky, int nyi,
                                 double* __restrict__ out) {
    const long n = (long)nxi * nyi;
    for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) {
        const int i = (int)(k / nyi), j = (int)(k - (long)(k / nyi) * nyi);
        if (!(okx[i] && oky[j])) {
            out[k] = xmiss;
            continue;
        }
        double rx[4], ry[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            rx[q] = wx[(size_t)i * 4 + q];
            ry[q] = wy[(size_t)j * 4 + q];
        }
        out[k] = interp_one(f, gx, gy, xmiss, zx[i], rx, zy[j], ry);
    }
}

}  // namespace flct
