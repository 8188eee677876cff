// prepass.cu -- the passes before and after the window kernel.
//
//   k_absmax / k_thresh_final   relative threshold (flct.c:594-629)
//   k_classify                  threshold test, skip grid, work list, the
//                               float hi+lo split of both frames, and the
//                               final values of pixels without a window
//                               (flct.c:721-755, 918-930, 1125-1133)
//   k_box_rows / k_box_cols     the local means (flct.c:815-827) from
//                               exact box sums (fixsum.cuh) as sliding
//                               sums, at the boxes the skip grid needs
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
__device__ __forceinline__ void k_absmax_body(const AbsmaxArgs& a, const int vb, const int vg) {
    unsigned long long m1 = 0ull, m2 = 0ull;
    const unsigned long long kAbs = 0x7fffffffffffffffull, kInf = 0x7ff0000000000000ull;
    for (long k = vb * (long)blockDim.x + threadIdx.x; k < a.n; k += (long)vg * blockDim.x) {
        unsigned long long x = (unsigned long long)__double_as_longlong(a.f1[k]) & kAbs;
        unsigned long long y = (unsigned long long)__double_as_longlong(a.f2[k]) & kAbs;
        if (x <= kInf && x > m1) m1 = x;
        if (y <= kInf && y > m2) m2 = y;
    }
    m1 = warp_max_u64(m1);
    m2 = warp_max_u64(m2);
    if ((threadIdx.x & 31) == 0) {
        atomicMax(a.out, m1);
        atomicMax(a.out + 1, m2);
    }
}
FLCT_MULTI_KERNEL(, k_absmax, AbsmaxArgs)

// thresh *= max(f1max, f2max), where fNmax follows maxloc's sequential scan:
// a NaN first element is never replaced (flct.c:608-621, 2142-2161).
__device__ __forceinline__ void k_thresh_final_body(const ThreshArgs& a, const int, const int) {
    if (threadIdx.x != 0) return;
    double a1 = fabs(a.f1[0]), a2 = fabs(a.f2[0]);
    double m1 = (a1 != a1) ? a1 : __longlong_as_double((long long)a.mx[0]);
    double m2 = (a2 != a2) ? a2 : __longlong_as_double((long long)a.mx[1]);
    double fmax = (m1 > m2) ? m1 : m2;
    *a.thr = __dmul_rn(a.thresh, fmax);
}
FLCT_MULTI_KERNEL(, k_thresh_final, ThreshArgs)

// ------------------------------------------------------- classify ----

// Finite test on the bit pattern (integer ops only).
__device__ __forceinline__ bool finite_bits(double x) {
    return ((__double_as_longlong(x) >> 52) & 0x7ff) != 0x7ff;
}


// One tile = kClassPix consecutive pixels of one row, kClassPpt per thread
// (thread t owns pixels t * kClassPpt ...).  The work list grows by one
// atomic per tile (block-wide ballot counts); the float split of both
// frames uses integer operations, and the threshold test 0.5*|f1+f2| <
// thresh (flct.c:721-722) needs one FP64 add only when the threshold is
// positive (otherwise no pixel is below it).  The row's grid test is one
// division per tile, the column's one per thread, then stepped per pixel.
__device__ __forceinline__ void k_classify_body(const ClassifyArgs& a, const int vb, const int vg) {
    constexpr int P = kClassPpt;
    __shared__ int s_cnt[8];
    __shared__ int s_base;
    const double thr = a.thr_ptr ? *a.thr_ptr : a.thr_val;
    const unsigned long long tb = (unsigned long long)__double_as_longlong(thr);
    // thr in (0, +inf]: compare |s|/2 with it as bit patterns
    const bool thr_pos = (long long)tb > 0ll && tb <= 0x7ff0000000000000ull;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int tpr = (a.ny + kClassPix - 1) / kClassPix;  // tiles per row
    const int ntile = (a.r1 - a.r0) * tpr;               // < 2^31: sides are limited to 2^31 pixels
    const int sk = a.skip > 0 ? a.skip : 1;
    auto pixel = [&](int t, int& i, int& j0) {
        const int ti = t / tpr;
        i = a.r0 + ti;
        j0 = (t - ti * tpr) * kClassPix + (int)threadIdx.x * P;  // this thread's first pixel
    };
    double fa[P], fb[P];
    auto load = [&](int t, double (&x)[P], double (&y)[P]) {
        int i, j0;
        pixel(t, i, j0);
        const size_t o = (size_t)i * a.ny + j0;
#pragma unroll
        for (int q = 0; q < P; ++q) {
            const bool in = j0 + q < a.ny;
            x[q] = in ? a.f1[o + q] : 0.;
            y[q] = in ? a.f2[o + q] : 0.;
        }
    };
    if (vb < ntile) load(vb, fa, fb);
    for (int t = vb; t < ntile; t += vg) {
        int i, j0;
        pixel(t, i, j0);
        double na[P], nb[P];
        if (t + vg < ntile) load(t + vg, na, nb);
        // the reference's C test !((i-xoff)%skip) && !((j-yoff)%skip): an
        // offset pixel (j < yoff) has a nonzero C remainder
        const bool grid_row = (a.skip > 0) ? !((i - a.xoff) % a.skip) : true;
        int rj = ((j0 - a.yoff) % sk + sk) % sk;  // (j - yoff) mod skip of the first pixel
        const size_t k0 = (size_t)i * a.ny + j0;
        bool comp[P], grid[P];
        unsigned range = 0u;
#pragma unroll
        for (int q = 0; q < P; ++q) {
            const int j = j0 + q;
            comp[q] = grid[q] = false;
            if (j < a.ny) {
                const float2 sa = split_double_fast(fa[q]), sb = split_double_fast(fb[q]);
                a.s12[k0 + q] = make_float4(sa.x, sb.x, sa.y, sb.y);
                // a finite value beyond the FP32 range (integer tests on the bits)
                if (((__float_as_uint(sa.x) & 0x7fffffffu) == 0x7f800000u && finite_bits(fa[q])) ||
                    ((__float_as_uint(sb.x) & 0x7fffffffu) == 0x7f800000u && finite_bits(fb[q])))
                    range = kStatusRange;
                bool below = false;
                if (thr_pos) {
                    const unsigned long long sb2 =
                        (unsigned long long)__double_as_longlong(__dadd_rn(fa[q], fb[q])) & 0x7fffffffffffffffull;
                    const unsigned E = (unsigned)(sb2 >> 52);
                    if (E >= 2u && E < 0x7ffu) below = (sb2 - (1ull << 52)) < tb;  // exact halving
                    else if (E == 0x7ffu) below = sb2 < tb;                         // inf / NaN
                    else below = __dmul_rn(0.5, __longlong_as_double((long long)sb2)) < thr;
                }
                grid[q] = (a.skip > 0) ? (grid_row && j >= a.yoff && rj == 0) : true;
                comp[q] = !below && grid[q];
            }
            rj = (rj + 1 == sk) ? 0 : rj + 1;
        }
        if (range) atomicOr(a.status, range);
        unsigned m[P];
        int wc = 0;
#pragma unroll
        for (int q = 0; q < P; ++q) {
            m[q] = __ballot_sync(0xffffffffu, comp[q]);
            wc += __popc(m[q]);
        }
        if (lane == 0) s_cnt[warp] = wc;
        // a tile is one row: its windows go to one list
        const bool second = a.work2 && i >= a.rsplit;
        int* const wl = second ? a.work2 : a.work;
        __syncthreads();
        if (threadIdx.x == 0) {
            int tot = 0;
#pragma unroll
            for (int w = 0; w < 8; ++w) {
                const int c = s_cnt[w];
                s_cnt[w] = tot;
                tot += c;
            }
            s_base = tot ? atomicAdd(second ? a.nwork2 : a.nwork, tot) : 0;
        }
        __syncthreads();
        int pos = s_base + s_cnt[warp];
        const unsigned below_me = (1u << lane) - 1u;
#pragma unroll
        for (int q = 0; q < P; ++q) {
            const int j = j0 + q;
            const size_t k = k0 + q;
            if (comp[q]) {
                wl[pos + __popc(m[q] & below_me)] = (int)k;
            } else if (j < a.ny) {
                // pixels without a window: (xmiss, xmiss, 0) then the reset gives
                // (0, 0, 0); skipped pixels that will be interpolated are left to
                // the interpolation.
                if (grid[q]) {
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
            pos += __popc(m[q]);
        }
        __syncthreads();  // s_cnt / s_base are rewritten by the next tile
#pragma unroll
        for (int q = 0; q < P; ++q) {
            fa[q] = na[q];
            fb[q] = nb[q];
        }
    }
}
FLCT_MULTI_KERNEL(__launch_bounds__(256), k_classify, ClassifyArgs)

// ------------------------------------------------------- box sums ----

// Row sums RT[i][m] = sum_{jj<n} f[i][s_m + jj] at the grid's box columns
// s_m = box_start(yo + m gs), exact (fixsum.cuh).  A warp takes one line
// (frame, row) and a pass of grid columns whose input span fits kRowSpan;
// the span's largest finite exponent sets its unit (fixsum.cuh).  Lane L
// converts the span's elements [L C, L C + C) (C odd, so the lanes'
// shared-memory words fall in distinct banks) into running sums, an
// exclusive warp scan of the lane totals gives each chunk's offset, and
// lane L then takes grid columns M + L, M + L + 32, ...: a box sum is the
// difference of two prefix sums, stored coalesced.
__device__ __forceinline__ void k_box_rows_body(const BoxArgs& a, const int vb, const int vg) {
    extern __shared__ unsigned s_rw[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    constexpr int SW = kRowSpan + 64;  // staged words per array (chunks of up to C <= kRowSpan / 32 + 2)
    unsigned* sw = s_rw + (size_t)warp * (5 * SW + 5 * 32);  // w0..w3, count; then lane offsets
    unsigned* so = sw + 5 * SW;
    const int rows = a.r1 - a.r0, lines = 2 * rows;
    const int P = a.pass_r;
    const int passes = (a.gj + P - 1) / P;
    for (long task = (long)vb * kBoxWarps + warp; task < (long)lines * passes;
         task += (long)vg * kBoxWarps) {
        const int lam = (int)(task / passes), pass = (int)(task - (long)lam * passes);
        const int img = lam >= rows, i = a.r0 + lam - img * rows;
        const double* __restrict__ v = (img ? a.f2 : a.f1) + (size_t)i * a.ny;
        BoxSum* __restrict__ o = (img ? a.rt2 : a.rt1) + (size_t)i * a.gj;
        int* __restrict__ oe = (img ? a.re2 : a.re1) + (size_t)i * a.gj;
        const int M = pass * P, Mend = min(M + P, a.gj);
        const int base = box_start(a.yo + M * a.gs, a.ny, a.nsize);
        const int span = box_start(a.yo + (Mend - 1) * a.gs, a.ny, a.nsize) + a.n - base;  // <= kRowSpan
        const int C = max(3, ((span + 31) >> 5) | 1);  // odd, >= 3: the division below is exact
        const int e0 = min(lane * C, span), e1 = min(e0 + C, span);
        // the span's doubles into words 0 and 1 of the stage (coalesced, all
        // loads in flight at once), and its largest finite exponent (its unit)
        unsigned em = 0u;
        {
            constexpr int KL = (kRowSpan + 31) / 32;
            double x[KL];
#pragma unroll
            for (int k = 0; k < KL; ++k) x[k] = (lane + 32 * k < span) ? v[base + lane + 32 * k] : 0.0;
#pragma unroll
            for (int k = 0; k < KL; ++k) {
                const int e = lane + 32 * k;
                if (e < span) {
                    const unsigned hw = (unsigned)__double2hiint(x[k]), xe = (hw >> 20) & 0x7ffu;
                    em = (xe != 0x7ffu && xe > em) ? xe : em;
                    sw[e] = (unsigned)__double2loint(x[k]);
                    sw[SW + e] = hw;
                }
            }
        }
        __syncwarp();  // lanes read each other's staged words below
        const int ee = max((int)__reduce_max_sync(0xffffffffu, em), 1);
        // running sums of the chunk, in place
        unsigned acc[4] = {0u, 0u, 0u, 0u}, cnt = 0u;
        for (int e = e0; e < e1; ++e) {
            fx_accum(__hiloint2double((int)sw[SW + e], (int)sw[e]), ee, acc, cnt);
#pragma unroll
            for (int k = 0; k < 4; ++k) sw[k * SW + e] = acc[k];
            sw[4 * SW + e] = cnt;
        }
        // exclusive scan of the lane totals
        unsigned t[5] = {acc[0], acc[1], acc[2], acc[3], cnt};
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            unsigned y[4], yc;
#pragma unroll
            for (int k = 0; k < 4; ++k) y[k] = __shfl_up_sync(0xffffffffu, t[k], d);
            yc = __shfl_up_sync(0xffffffffu, t[4], d);
            if (lane >= d) {
                unsigned z[4] = {t[0], t[1], t[2], t[3]};
                add4(z, y);
#pragma unroll
                for (int k = 0; k < 4; ++k) t[k] = z[k];
                t[4] += yc;
            }
        }
#pragma unroll
        for (int k = 0; k < 5; ++k) {
            const unsigned ex = __shfl_up_sync(0xffffffffu, t[k], 1);
            so[k * 32 + lane] = lane ? ex : 0u;
        }
        __syncwarp();
        const unsigned magic = 0xffffffffu / (unsigned)C + 1u;  // ceil(2^32 / C): e / C = umulhi(e, magic)
        auto prefix = [&](int e, unsigned (&p)[4], unsigned& pc) {
            const int L = (int)__umulhi((unsigned)e, magic);
#pragma unroll
            for (int k = 0; k < 4; ++k) p[k] = sw[k * SW + e];
            pc = sw[4 * SW + e] + so[4 * 32 + L];
            const unsigned off[4] = {so[L], so[32 + L], so[64 + L], so[96 + L]};
            add4(p, off);
        };
        for (int m = M + lane; m < Mend; m += 32) {
            const int sb = box_start(a.yo + m * a.gs, a.ny, a.nsize) - base;
            unsigned hiw[4], hc;
            prefix(sb + a.n - 1, hiw, hc);
            if (sb > 0) {
                unsigned low[4], lc;
                prefix(sb - 1, low, lc);
                sub4(hiw, low);
                hc -= lc;
            }
            o[m] = BoxSum{(unsigned long long)hiw[0] | ((unsigned long long)hiw[1] << 32),
                          (unsigned long long)hiw[2] | ((unsigned long long)hiw[3] << 32), cnt_wide(hc),
                          (unsigned long long)ee};
            oe[m] = ee;
        }
        __syncwarp();  // the next pass overwrites the stage
    }
}
FLCT_MULTI_KERNEL(__launch_bounds__(kBoxWarps * 32), k_box_rows, BoxArgs)

// Box sums B[q][m] = sum_{ii<n} RT[t_q + ii][m] at the grid's box rows
// t_q = box_start(xo + q gs), exact.  kColLanes consecutive lanes take one
// line (frame, grid column) and a run of kColRun grid rows starting at a
// multiple of kColRun; lane p reads the run's rows r with r - t = p mod
// kColLanes, and the lanes' partial sums meet by shuffles (integer sums:
// the order does not matter).  The run's unit is the largest of the row
// sums' units it reads.  A warp's loads cover 32 / kColLanes consecutive
// columns of kColLanes rows.  Each box sum becomes the grid point's FP64
// local mean, rounded once, and is stored as its float hi + lo split (the
// form the window kernels subtract): lane 0 of the group writes this
// frame's half of the grid point's float4.
__device__ __forceinline__ void col_reduce(unsigned long long& lo, unsigned long long& hi,
                                           unsigned long long& cnt) {
#pragma unroll
    for (int o = 1; o < kColLanes; o <<= 1) {
        const unsigned long long l2 = __shfl_xor_sync(0xffffffffu, lo, o, kColLanes);
        const unsigned long long h2 = __shfl_xor_sync(0xffffffffu, hi, o, kColLanes);
        cnt += __shfl_xor_sync(0xffffffffu, cnt, o, kColLanes);
        add128(lo, hi, l2, h2);
    }
}

__device__ __forceinline__ void k_box_cols_body(const BoxArgs& a, const int vb, const int vg) {
    grid_dep_wait();  // the row sums come from the kernel before
    const int lines = 2 * a.gj;
    const int runs = (a.q1 - a.q0 + kColRun - 1) / kColRun;
    const long gid = vb * (long)blockDim.x + threadIdx.x;
    const int p = (int)(gid & (kColLanes - 1));
    long idx = gid / kColLanes;
    // a group past the end repeats the last line (every lane of the warp
    // takes part in the shuffles) and stores nothing
    const bool act = idx < (long)lines * runs;
    if (!act) idx = (long)lines * runs - 1;
    const int run = (int)(idx / lines), lam = (int)(idx - (long)run * lines);
    const int img = lam >= a.gj, m = lam - img * a.gj;
    const BoxSum* __restrict__ v = (img ? a.rt2 : a.rt1) + m;  // row r at v[r * gj]
    const int* __restrict__ ve = (img ? a.re2 : a.re1) + m;
    // this line's hi and lo in the grid points' float4 means (f1 hi, f2 hi,
    // f1 lo, f2 lo): floats img and 2 + img
    float* __restrict__ o = reinterpret_cast<float*>(a.means + m) + img;
    const size_t gj = (size_t)a.gj;
    const int q0 = a.q0 + run * kColRun, q1 = min(q0 + kColRun, a.q1);
    int t = box_start(a.xo + q0 * a.gs, a.nx, a.nsize);
    const int tend = box_start(a.xo + (q1 - 1) * a.gs, a.nx, a.nsize) + a.n;
    int eb = 1;
#pragma unroll 4
    for (int r = t + p; r < tend; r += kColLanes) eb = max(eb, __ldg(ve + r * gj));
#pragma unroll
    for (int k = 1; k < kColLanes; k <<= 1) eb = max(eb, __shfl_xor_sync(0xffffffffu, eb, k, kColLanes));
    unsigned long long lo = 0ull, hi = 0ull, cnt = 0ull;
#pragma unroll 8
    for (int r = t + p; r < t + a.n; r += kColLanes) {
        BoxSum x = v[r * gj];
        sar128(x.lo, x.hi, eb - (int)x.e);
        add128(lo, hi, x.lo, x.hi);
        cnt += x.cnt;
    }
    col_reduce(lo, hi, cnt);
    for (int q = q0;;) {
        if (act && p == 0) {
            // the FP64 mean (flct.c:815-827), rounded once from the exact sum
            const BoxSum bs{lo, hi, cnt, (unsigned long long)eb};
            const float2 mhl = split_double_fast(__dmul_rn(fx_to_double(bs, eb), a.inv_n2));
            o[(size_t)q * gj * 4] = mhl.x;
            o[(size_t)q * gj * 4 + 2] = mhl.y;
        }
        if (++q >= q1) break;
        // slide down to the next grid row's box: rows [t, tn) leave, rows
        // [t + n, tn + n) enter
        const int tn = box_start(a.xo + q * a.gs, a.nx, a.nsize);
        unsigned long long dl = 0ull, dh = 0ull, dc = 0ull;
#pragma unroll 2
        for (int r = t + p; r < tn; r += kColLanes) {
            BoxSum in = v[(r + a.n) * gj], out = v[r * gj];
            sar128(in.lo, in.hi, eb - (int)in.e);
            sar128(out.lo, out.hi, eb - (int)out.e);
            add128(dl, dh, in.lo, in.hi);
            sub128(dl, dh, out.lo, out.hi);
            dc += in.cnt - out.cnt;
        }
        col_reduce(dl, dh, dc);
        add128(lo, hi, dl, dh);
        cnt += dc;
        t = tn;
    }
}
FLCT_MULTI_KERNEL(__launch_bounds__(128), k_box_cols, BoxArgs)

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

// cdata[a][b] of the border-extended grid (flct.c:2257-2336), both
// components.  Out of line: only stencils at the grid's border use it.
__device__ __noinline__ float2 cdata_f(const float2* __restrict__ g, int gx, int gy, int a, int b) {
    auto F = [&](int p, int q) -> float2 { return g[(size_t)p * gy + q]; };
    auto ext = [](float2 f0, float2 f1, float2 f2) -> float2 {  // 3 f0 - 3 f1 + f2 in the reference's order
        return make_float2((f2.x - 3.f * f1.x) + 3.f * f0.x, (f2.y - 3.f * f1.y) + 3.f * f0.y);
    };
    auto ext3 = [](float2 f0, float2 f1, float2 f2) -> float2 {  // corners: 3 c0 - 3 c1 + c2
        return make_float2((3.f * f0.x - 3.f * f1.x) + f2.x, (3.f * f0.y - 3.f * f1.y) + f2.y);
    };
    auto row_edge = [&](int p, int q) -> float2 {  // interior row p, border column q
        if (q == 0) return ext(F(p, 0), F(p, 1), F(p, 2));
        return ext(F(p, gy - 1), F(p, gy - 2), F(p, gy - 3));
    };
    auto col_edge = [&](int p, int q) -> float2 {  // border row p, interior column q
        if (p == 0) return ext(F(0, q), F(1, q), F(2, q));
        return ext(F(gx - 1, q), F(gx - 2, q), F(gx - 3, q));
    };
    const bool ra = (a >= 1 && a <= gx), rb = (b >= 1 && b <= gy);
    if (ra && rb) return F(a - 1, b - 1);
    if (ra) return row_edge(a - 1, b);
    if (rb) return col_edge(a, b - 1);
    // corners: (0, gy+1) from the top border row, the others from the
    // border columns, as the reference extrapolates them
    if (a == 0 && b == gy + 1) return ext3(col_edge(0, gy - 1), col_edge(0, gy - 2), col_edge(0, gy - 3));
    const int qb = (b == 0) ? 0 : gy + 1;
    if (a == 0) return ext3(row_edge(0, qb), row_edge(1, qb), row_edge(2, qb));
    return ext3(row_edge(gx - 1, qb), row_edge(gx - 2, qb), row_edge(gx - 3, qb));
}

// A block interpolates a tile of kTileR x kTileC pixels in three steps
// separated by barriers: stage the cdata patch the tile's stencils touch
// (interior grid values, and the border extrapolations where the tile
// reaches the grid's edge) in shared memory; contract the patch along x for
// every tile row, V[r][b] = sum_p rx_r[p] patch[izr + p][b] (with per-column
// y stencils tabulated alongside); then each pixel contracts four V values
// with its y weights.  xmiss flags travel with the values (bit 0: vx,
// bit 1: vy).  The patch and V items are spread over all threads (row =
// item / width by a multiply-high); a thread writes two adjacent pixels,
// as 16-byte stores when the rows allow.
constexpr int kPatchR = kTileR + 4, kPatchC = kTileC + 4;  // cdata rows / columns at skip 1
constexpr int kPairCols = kTileC / 2;                       // threads per tile row in the output step
constexpr int kPairRows = kInterpThreads / kPairCols;       // tile rows per output pass

__device__ __forceinline__ void k_interp_grid_body(const InterpArgs& a, const int vb, const int vg) {
    __shared__ float2 s_p[kPatchR * kPatchC];
    __shared__ unsigned char s_pb[kPatchR * kPatchC];
    __shared__ float2 s_v[kTileR * kPatchC];
    __shared__ unsigned char s_vb[kTileR * kPatchC];
    __shared__ float s_ry[kTileC][4];
    __shared__ float s_rx[kTileR][4];
    __shared__ int s_jz[kTileC];            // izero along y, -1 out of range
    __shared__ int s_iz[kTileR];            // izero along x, -1 out of range (or past i1)
    __shared__ unsigned char s_gj[kTileC];  // grid column
    __shared__ unsigned char s_gi[kTileR];  // grid row
    const int ntc = (a.ny + kTileC - 1) / kTileC;
    const int ntr = (a.i1 - a.i0 + kTileR - 1) / kTileR;
    const float inv = 1.0f / (float)a.skip;
    const int imax = (a.gx - 1) * a.skip, jmax = (a.gy - 1) * a.skip;
    const int tc = (threadIdx.x % kPairCols) * 2, tr = threadIdx.x / kPairCols;
    grid_dep_wait();
    publish_counters(a.pub_src, a.pub_dst);
    for (int tile = vb; tile < ntr * ntc; tile += vg) {
        const int i0 = a.i0 + (tile / ntc) * kTileR, j0 = (tile - (tile / ntc) * ntc) * kTileC;
        // cdata rows / columns the tile's in-range pixels use
        const int dlo = max(i0 - a.xoff, 0), dhi = min(min(i0 + kTileR, a.i1) - 1 - a.xoff, imax);
        const int elo = max(j0 - a.yoff, 0), ehi = min(min(j0 + kTileC, a.ny) - 1 - a.yoff, jmax);
        const bool any = dlo <= dhi && elo <= ehi;
        const int r0 = any ? min(dlo / a.skip, a.gx - 2) : 0, r1 = any ? min(dhi / a.skip, a.gx - 2) + 3 : -1;
        const int c0 = any ? min(elo / a.skip, a.gy - 2) : 0, c1 = any ? min(ehi / a.skip, a.gy - 2) + 3 : -1;
        const int pw = c1 - c0 + 1, ph = r1 - r0 + 1;  // pw >= 4 when any
        // item / pw = umulhi(item, ceil(2^32 / pw)), exact for items below 2^32 / pw
        const unsigned mpw = 0xffffffffu / (unsigned)max(pw, 1) + 1u;
        __syncthreads();  // the previous tile's tables are consumed
        int tb = 0;       // this thread's patch values hold an xmiss
        for (int e = threadIdx.x; e < ph * pw; e += kInterpThreads) {
            const int pr = (int)__umulhi((unsigned)e, mpw), pc = e - pr * pw;
            const int ra = r0 + pr, cb = c0 + pc;
            const float2 v = (ra >= 1 && ra <= a.gx && cb >= 1 && cb <= a.gy)
                                 ? __ldg(a.grid + (size_t)(ra - 1) * a.gy + (cb - 1))
                                 : cdata_f(a.grid, a.gx, a.gy, ra, cb);
            const int pe = pr * kPatchC + pc;
            s_p[pe] = v;
            const unsigned char f = (v.x == kXmissF ? 1 : 0) | (v.y == kXmissF ? 2 : 0);
            s_pb[pe] = f;
            tb |= f;
        }
        // per-column and per-row stencil tables
        if (threadIdx.x < kTileC) {
            const int dj = j0 + threadIdx.x - a.yoff;
            const bool okj = dj >= 0 && dj <= jmax;
            const int jz = okj ? min(dj / a.skip, a.gy - 2) : -1;
            s_jz[threadIdx.x] = jz;
            s_gj[threadIdx.x] = (dj % a.skip) == 0;
#pragma unroll
            for (int q = 0; q < 4; ++q)
                s_ry[threadIdx.x][q] = okj ? keys_f(fabsf((float)(dj - (jz + q - 1) * a.skip) * inv)) : 0.f;
        } else if (threadIdx.x < kTileC + kTileR) {  // kTileC + kTileR <= kInterpThreads
            const int r = threadIdx.x - kTileC;
            const int di = i0 + r - a.xoff;
            const bool oki = i0 + r < a.i1 && di >= 0 && di <= imax;
            const int iz = oki ? min(di / a.skip, a.gx - 2) : -1;
            s_iz[r] = iz;
            s_gi[r] = (di % a.skip) == 0;
#pragma unroll
            for (int p = 0; p < 4; ++p)
                s_rx[r][p] = oki ? keys_f(fabsf((float)(di - (iz + p - 1) * a.skip) * inv)) : 0.f;
        }
        // a tile whose patch holds no xmiss (the usual case) skips the flags
        const int tile_bad = __syncthreads_or(tb);
        // V[r][b] = sum_p rx[r][p] patch[iz_r - r0 + p][b]
        for (int e = threadIdx.x; e < kTileR * pw; e += kInterpThreads) {
            const int r = (int)__umulhi((unsigned)e, mpw), b = e - r * pw;
            const int iz = s_iz[r];
            float2 v = make_float2(0.f, 0.f);
            unsigned char bad = 3;
            if (iz >= 0) {
                bad = 0;
#pragma unroll
                for (int p = 0; p < 4; ++p) {
                    const float rx = s_rx[r][p];
                    const int pe = (iz - r0 + p) * kPatchC + b;
                    const float2 c = s_p[pe];
                    if (tile_bad) bad |= s_pb[pe];
                    v.x = fmaf(rx, c.x, v.x);
                    v.y = fmaf(rx, c.y, v.y);
                }
            }
            s_v[r * kPatchC + b] = v;
            s_vb[r * kPatchC + b] = bad;
        }
        __syncthreads();
        // pixels (i, j) and (i, j + 1); a column past ny has jz = -1
        const int j = j0 + tc;
        if (j >= a.ny) continue;
        const bool two = j + 1 < a.ny;
        int jz[2];
        bool gj[2];
        float ry[2][4];
#pragma unroll
        for (int c = 0; c < 2; ++c) {
            jz[c] = s_jz[tc + c];
            gj[c] = s_gj[tc + c];
#pragma unroll
            for (int q = 0; q < 4; ++q) ry[c][q] = s_ry[tc + c][q];
        }
#pragma unroll
        for (int k2 = 0; k2 < kTileR / kPairRows; ++k2) {
            const int r = tr + kPairRows * k2, i = i0 + r;
            if (i >= a.i1) break;
            const bool gi = s_gi[r] && i - a.xoff >= 0;
            const int iz = s_iz[r];
            double ox[2], oy[2], om[2];
            bool wr[2];
#pragma unroll
            for (int c = 0; c < 2; ++c) {
                wr[c] = (c == 0 || two) && !(gj[c] && gi);  // grid points keep their computed value
                float sx = 0.f, sy = 0.f;
                unsigned bad = 3;
                if (jz[c] >= 0 && iz >= 0) {
                    bad = 0;
                    const int vb = r * kPatchC + (jz[c] - c0);
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        const float2 v = s_v[vb + q];
                        if (tile_bad) bad |= s_vb[vb + q];
                        sx = fmaf(ry[c][q], v.x, sx);
                        sy = fmaf(ry[c][q], v.y, sy);
                    }
                }
                // xmiss reset: a missing vx clears the mask, a missing vy only vy
                ox[c] = (bad & 1) ? 0. : f2d(sx);
                oy[c] = (bad & 2) ? 0. : f2d(sy);
                om[c] = (bad & 1) ? 0. : 0.5;
            }
            const size_t k = (size_t)i * a.ny + j;
            if (a.pairs && wr[0] && wr[1]) {
                *reinterpret_cast<double2*>(a.vx + k) = make_double2(ox[0], ox[1]);
                *reinterpret_cast<double2*>(a.vy + k) = make_double2(oy[0], oy[1]);
                *reinterpret_cast<double2*>(a.vm + k) = make_double2(om[0], om[1]);
            } else {
#pragma unroll
                for (int c = 0; c < 2; ++c) {
                    if (wr[c]) {
                        a.vx[k + c] = ox[c];
                        a.vy[k + c] = oy[c];
                        a.vm[k + c] = om[c];
                    }
                }
            }
        }
    }
}
FLCT_MULTI_KERNEL(__launch_bounds__(kInterpThreads), k_interp_grid, InterpArgs)

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
