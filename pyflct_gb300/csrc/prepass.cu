// prepass.cu -- the passes before and after the window kernel.
//
//   k_absmax / k_thresh_final   relative threshold (flct.c:594-629)
//   k_classify                  threshold test, skip grid, work list, the
//                               float hi+lo split of both frames, and the
//                               final values of pixels without a window
//                               (flct.c:721-755, 918-930, 1125-1133)
//   k_box_rows / k_box_cols     FP64 box sums for the local means
//                               (flct.c:815-827) as sliding sums, at the
//                               boxes the skip grid needs
//   k_interp_grid               skip-grid cubic-convolution interpolation
//                               (flct.c:958-1120 with interpcc2d,
//                               flct.c:2226-2463) and the xmiss reset
//   k_interp_axis / k_interp_general   interpcc2d itself (FP64, reference
//                               order) for the standalone entry points
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

// One tile = 256 consecutive pixels of one row, one per thread.  The work
// list grows by one atomic per tile (block-wide ballot counts); the float
// split of both frames uses integer operations, and the threshold test
// 0.5*|f1+f2| < thresh (flct.c:721-722) needs one FP64 add only when the
// threshold is positive (otherwise no pixel is below it).
__global__ void __launch_bounds__(256) k_classify(ClassifyArgs a) {
    __shared__ int s_cnt[8];
    __shared__ int s_base;
    const double thr = a.thr_ptr ? *a.thr_ptr : a.thr_val;
    const unsigned long long tb = (unsigned long long)__double_as_longlong(thr);
    // thr in (0, +inf]: compare |s|/2 with it as bit patterns
    const bool thr_pos = (long long)tb > 0ll && tb <= 0x7ff0000000000000ull;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int tpr = (a.ny + 255) >> 8;  // tiles per row
    const long ntile = (long)a.nx * tpr;
    for (long t = blockIdx.x; t < ntile; t += gridDim.x) {
        const int i = (int)(t / tpr);
        const int j = (int)(t - (long)i * tpr) * 256 + threadIdx.x;
        const bool act = j < a.ny;
        const size_t k = (size_t)i * a.ny + j;
        bool comp = false, grid = false;
        if (act) {
            const double fa = a.f1[k], fb = a.f2[k];
            const float2 sa = split_double_fast(fa), sb = split_double_fast(fb);
            a.s1[k] = sa;
            a.s2[k] = sb;
            if ((isinf(sa.x) && !isinf(fa)) || (isinf(sb.x) && !isinf(fb))) atomicOr(a.status, kStatusRange);
            bool below = false;
            if (thr_pos) {
                const unsigned long long sb2 =
                    (unsigned long long)__double_as_longlong(__dadd_rn(fa, fb)) & 0x7fffffffffffffffull;
                const unsigned E = (unsigned)(sb2 >> 52);
                if (E >= 2u && E < 0x7ffu) below = (sb2 - (1ull << 52)) < tb;  // exact halving
                else if (E == 0x7ffu) below = sb2 < tb;                         // inf / NaN
                else below = __dmul_rn(0.5, __longlong_as_double((long long)sb2)) < thr;
            }
            grid = (a.skip > 0) ? (!((i - a.xoff) % a.skip) && !((j - a.yoff) % a.skip)) : true;
            comp = !below && grid;
        }
        const unsigned m = __ballot_sync(0xffffffffu, comp);
        if (lane == 0) s_cnt[warp] = __popc(m);
        __syncthreads();
        if (threadIdx.x == 0) {
            int tot = 0;
#pragma unroll
            for (int w = 0; w < 8; ++w) {
                const int c = s_cnt[w];
                s_cnt[w] = tot;
                tot += c;
            }
            s_base = tot ? atomicAdd(a.nwork, tot) : 0;
        }
        __syncthreads();
        if (comp) {
            a.work[s_base + s_cnt[warp] + __popc(m & ((1u << lane) - 1u))] = (int)k;
        } else if (act) {
            // pixels without a window: (xmiss, xmiss, 0) then the reset gives
            // (0, 0, 0); skipped pixels that will be interpolated are left to
            // the interpolation.
            if (grid) {
                a.vx[k] = 0.;
                a.vy[k] = 0.;
                a.vm[k] = 0.;
                if (a.grid) {
                    const int ic = (i - a.xoff) / a.skip, jc = (j - a.yoff) / a.skip;
                    a.grid[(size_t)ic * a.jcnt + jc] = make_float2(kXmissF, kXmissF);
                }
            } else if (!a.interpolate) {
                a.vx[k] = 0.;
                a.vy[k] = 0.;
                a.vm[k] = 0.;
            }
        }
        __syncthreads();  // s_cnt / s_base are rewritten by the next tile
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

// Row sums RT[m][i] = sum_{jj<n} f[i][s_m + jj] at the grid's box columns
// s_m = box_start(yo + m gs).  One thread per (row, run of `seg` grid
// columns): n adds for the first box, then one column step (an add and a
// subtract) per column between consecutive boxes.  Consecutive threads take
// consecutive rows, so the transposed stores are coalesced.
__global__ void k_box_rows(BoxArgs a) {
    const int nseg = (a.gj + a.seg - 1) / a.seg;
    const long idx = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (idx >= (long)a.nx * nseg) return;
    const int sg = (int)(idx / a.nx);
    const int i = (int)(idx - (long)sg * a.nx);
    const int m0 = sg * a.seg, m1 = min(m0 + a.seg, a.gj);
    const double* f = a.f1 + (size_t)i * a.ny;
    const double* g = a.f2 + (size_t)i * a.ny;
    int s = box_start(a.yo + m0 * a.gs, a.ny, a.nsize);
    double sa = 0., sb = 0.;
    for (int jj = 0; jj < a.n; ++jj) {
        sa = __dadd_rn(sa, f[s + jj]);
        sb = __dadd_rn(sb, g[s + jj]);
    }
    a.rt1[(size_t)m0 * a.nx + i] = sa;
    a.rt2[(size_t)m0 * a.nx + i] = sb;
    for (int m = m0 + 1; m < m1; ++m) {
        const int s1 = box_start(a.yo + m * a.gs, a.ny, a.nsize);
        for (; s < s1; ++s) {
            sa = slide(sa, f[s + a.n], f[s], a.n, [&](int q) { return f[s + 1 + q]; });
            sb = slide(sb, g[s + a.n], g[s], a.n, [&](int q) { return g[s + 1 + q]; });
        }
        a.rt1[(size_t)m * a.nx + i] = sa;
        a.rt2[(size_t)m * a.nx + i] = sb;
    }
}

// Box sums B[q][m] = sum_{ii<n} RT[m][t_q + ii] at the grid's box rows
// t_q = box_start(xo + q gs); one thread per (grid column, run of `seg`
// grid rows), consecutive threads on consecutive columns.
__global__ void k_box_cols(BoxArgs a) {
    const int nseg = (a.gi + a.seg - 1) / a.seg;
    const long idx = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (idx >= (long)a.gj * nseg) return;
    const int sg = (int)(idx / a.gj);
    const int m = (int)(idx - (long)sg * a.gj);
    const int q0 = sg * a.seg, q1 = min(q0 + a.seg, a.gi);
    const double* r = a.rt1 + (size_t)m * a.nx;
    const double* u = a.rt2 + (size_t)m * a.nx;
    int t = box_start(a.xo + q0 * a.gs, a.nx, a.nsize);
    double sa = 0., sb = 0.;
    for (int ii = 0; ii < a.n; ++ii) {
        sa = __dadd_rn(sa, r[t + ii]);
        sb = __dadd_rn(sb, u[t + ii]);
    }
    a.b1[(size_t)q0 * a.gj + m] = sa;
    a.b2[(size_t)q0 * a.gj + m] = sb;
    for (int q = q0 + 1; q < q1; ++q) {
        const int t1 = box_start(a.xo + q * a.gs, a.nx, a.nsize);
        for (; t < t1; ++t) {
            sa = slide(sa, r[t + a.n], r[t], a.n, [&](int k) { return r[t + 1 + k]; });
            sb = slide(sb, u[t + a.n], u[t], a.n, [&](int k) { return u[t + 1 + k]; });
        }
        a.b1[(size_t)q * a.gj + m] = sa;
        a.b2[(size_t)q * a.gj + m] = sb;
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

// The velocity pipeline's interpolation of the skip grid onto the skipped
// pixels (flct.c:958-1120 with interpcc2d, flct.c:2226-2463), the mask 0.5
// and the final xmiss reset (flct.c:1125-1133), fused in one pass with FP32
// arithmetic (velocities interpolate to ~1e-7 relative; the FP64 reference
// order is kept by the standalone interpcc2d entry point instead).
//
// The range test and izero come from integer arithmetic on (i - offset)
// and skip, exactly as the reference's xwant = (i - offset)/skip gives
// them; a stencil holding xmiss yields xmiss (so the mask is exact).

// Keys kernel, a = -0.5 (flct.c:2398-2419).
__device__ __forceinline__ float keys_f(float t) {
    return (t >= 1.0f) ? ((-0.5f * t + 2.5f) * t - 4.0f) * t + 2.0f : (1.5f * t - 2.5f) * t * t + 1.0f;
}

// cdata[a][b] of the border-extended grid (flct.c:2257-2336) for one of the
// two components (c = 0: vx, 1: vy).
__device__ __forceinline__ float cdata_f(const float2* __restrict__ g, int gx, int gy, int a, int b, int c) {
    auto F = [&](int p, int q) -> float {
        const float2 v = g[(size_t)p * gy + q];
        return c ? v.y : v.x;
    };
    auto row_edge = [&](int p, int q) -> float {  // interior row p, border column q
        if (q == 0) return (F(p, 2) - 3.f * F(p, 1)) + 3.f * F(p, 0);
        return (F(p, gy - 3) - 3.f * F(p, gy - 2)) + 3.f * F(p, gy - 1);
    };
    auto col_edge = [&](int p, int q) -> float {  // border row p, interior column q
        if (p == 0) return (F(2, q) - 3.f * F(1, q)) + 3.f * F(0, q);
        return (F(gx - 3, q) - 3.f * F(gx - 2, q)) + 3.f * F(gx - 1, q);
    };
    const bool ra = (a >= 1 && a <= gx), rb = (b >= 1 && b <= gy);
    if (ra && rb) return F(a - 1, b - 1);
    if (ra) return row_edge(a - 1, b);
    if (rb) return col_edge(a, b - 1);
    // corners: (0, gy+1) from the top border row, the others from the
    // border columns, as the reference extrapolates them
    if (a == 0 && b == gy + 1)
        return (3.f * col_edge(0, gy - 1) - 3.f * col_edge(0, gy - 2)) + col_edge(0, gy - 3);
    const int qb = (b == 0) ? 0 : gy + 1;
    const int p0 = (a == 0) ? 1 : gx, p1 = (a == 0) ? 2 : gx - 1, p2 = (a == 0) ? 3 : gx - 2;
    return (3.f * row_edge(p0 - 1, qb) - 3.f * row_edge(p1 - 1, qb)) + row_edge(p2 - 1, qb);
}

__global__ void __launch_bounds__(256) k_interp_grid(InterpArgs a) {
    for (int i = blockIdx.y; i < a.nx; i += gridDim.y) {
        const int di = i - a.xoff;
        const bool gi = (di % a.skip) == 0;
        // xwant = di / skip in [0, gx - 1], izero = min((int)xwant, gx - 2)
        const bool okx = di >= 0 && di <= (a.gx - 1) * a.skip;
        int iz = 0;
        float rx[4] = {0.f, 0.f, 0.f, 0.f};
        if (okx) {
            iz = min(di / a.skip, a.gx - 2);
#pragma unroll
            for (int p = 0; p < 4; ++p)
                rx[p] = keys_f(fabsf((float)(di - (iz + p - 1) * a.skip) / (float)a.skip));
        }
        for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < a.ny; j += gridDim.x * blockDim.x) {
            const int dj = j - a.yoff;
            if (gi && (dj % a.skip) == 0) continue;  // grid points keep their computed value
            const bool ok = okx && dj >= 0 && dj <= (a.gy - 1) * a.skip;
            bool badx = true, bady = true;
            float sx = 0.f, sy = 0.f;
            if (ok) {
                const int jz = min(dj / a.skip, a.gy - 2);
                float ry[4];
#pragma unroll
                for (int q = 0; q < 4; ++q)
                    ry[q] = keys_f(fabsf((float)(dj - (jz + q - 1) * a.skip) / (float)a.skip));
                badx = bady = false;
                // cdata rows iz..iz+3, columns jz..jz+3 (cdata index = grid index + 1)
                const bool inner = iz >= 1 && iz + 3 <= a.gx && jz >= 1 && jz + 3 <= a.gy;
#pragma unroll
                for (int p = 0; p < 4; ++p) {
                    float hx = 0.f, hy = 0.f;
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        float cx, cy;
                        if (inner) {
                            const float2 v = __ldg(a.grid + (size_t)(iz + p - 1) * a.gy + (jz + q - 1));
                            cx = v.x;
                            cy = v.y;
                        } else {
                            cx = cdata_f(a.grid, a.gx, a.gy, iz + p, jz + q, 0);
                            cy = cdata_f(a.grid, a.gx, a.gy, iz + p, jz + q, 1);
                        }
                        badx |= cx == kXmissF;
                        bady |= cy == kXmissF;
                        hx = fmaf(cx, ry[q], hx);
                        hy = fmaf(cy, ry[q], hy);
                    }
                    sx = fmaf(rx[p], hx, sx);
                    sy = fmaf(rx[p], hy, sy);
                }
            }
            const size_t k = (size_t)i * a.ny + j;
            // xmiss reset: a missing vx clears the mask, a missing vy only vy
            a.vx[k] = badx ? 0. : f2d(sx);
            a.vy[k] = bady ? 0. : f2d(sy);
            a.vm[k] = badx ? 0. : 0.5;
        }
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
