// window_common.cu -- k_fit and k_fit_hires (see window_common.cuh).
#include "window_common.cuh"

namespace flct {

// Work items go to warps in 32-item chunks dealt round the blocks (chunk c
// to block c mod gridDim), so every SM gets about the same number of fits:
// the kernel is bound by each SM's FP64 pipe, and a plain grid-stride
// mapping leaves the low blocks (and the SMs holding them) with the most.
__device__ __forceinline__ void k_fit_body(const FitArgs& a, const int vb, const int vg) {
    grid_dep_wait();
    publish_counters(a.pub_src, a.pub_dst);
    const int nw = *a.nwork;
    const int lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
    for (long c = vb + (long)vg * (threadIdx.x >> 5); c * 32 < nw; c += (long)vg * wpb) {
        const int w = (int)(c * 32) + lane;
        if (w >= nw) continue;
        fit_item(a, w, a.peaks[w]);
    }
}
FLCT_MULTI_KERNEL(, k_fit, FitArgs)

// ------------------------------------------------------------- -h ------

// Keys kernel, a = -0.5 (flct.c:2398-2419), in FP32.
__device__ __forceinline__ float keys32(float t) {
    return (t >= 1.0f) ? ((-0.5f * t + 2.5f) * t - 4.0f) * t + 2.0f : (1.5f * t - 2.5f) * t * t + 1.0f;
}

// cdata of the 6x6 patch p (array rows I-2.., columns J-2..) of an n x m
// array at array coordinates (r, c) in [-1, n] x [-1, m]: interior values, or the one-cell border
// extrapolations 3 f0 - 3 f1 + f2 (corners from the border columns, the
// top-right one from the top border row), as interpcc2d builds them
// (flct.c:2257-2336).
__device__ __forceinline__ float patch_cdata(const float* p, int I, int J, int n, int m, int r, int c) {
    auto F = [&](int rr, int cc) { return p[(rr - I + 2) * kHiresPatch + (cc - J + 2)]; };
    auto ext = [](float f0, float f1, float f2) { return (f2 - 3.f * f1) + 3.f * f0; };
    auto ext3 = [](float c0, float c1, float c2) { return (3.f * c0 - 3.f * c1) + c2; };
    auto row_edge = [&](int rr, int cc) {  // interior row rr, border column cc
        return cc < 0 ? ext(F(rr, 0), F(rr, 1), F(rr, 2)) : ext(F(rr, m - 1), F(rr, m - 2), F(rr, m - 3));
    };
    auto col_edge = [&](int rr, int cc) {  // border row rr, interior column cc
        return rr < 0 ? ext(F(0, cc), F(1, cc), F(2, cc)) : ext(F(n - 1, cc), F(n - 2, cc), F(n - 3, cc));
    };
    const bool ri = r >= 0 && r < n, ci = c >= 0 && c < m;
    if (ri && ci) return F(r, c);
    if (ri) return row_edge(r, c);
    if (ci) return col_edge(r, c);
    if (r < 0 && c >= m) return ext3(col_edge(-1, m - 1), col_edge(-1, m - 2), col_edge(-1, m - 3));
    if (r < 0) return ext3(row_edge(0, c), row_edge(1, c), row_edge(2, c));
    return ext3(row_edge(n - 1, c), row_edge(n - 2, c), row_edge(n - 3, c));
}

// Float bits -> unsigned with the order of the values (NaN excluded).
__device__ __forceinline__ unsigned ordered_bits(float v) {
    const unsigned u = __float_as_uint(v);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

// -h: per work item, the reference's zoom of |c| around the integer peak
// (flct.c:1564-1635): a 21x21 cubic-convolution interpolation at 0.1 px
// (xmiss 0: out of range, or a zero in the stencil, gives 0), its first
// maximum, and the 3x3 fit there scaled by 0.1.  One warp per work item;
// lane j < 21 owns zoom column j.  The interpolation runs in FP32 on the
// FP32 |c| patch, the fit and the shift in FP64.
__device__ __forceinline__ void k_fit_hires_body(const FitArgs& a, const int vb, const int vg) {
    constexpr int NI = 21, P = kHiresPatch;
    __shared__ float s_p[4][P * P];
    __shared__ float s_h[4][P][NI];
    __shared__ unsigned char s_hb[4][P][NI];
    __shared__ float s_pk[4][NI * NI];
    __shared__ float s_rx[4][NI][4];
    __shared__ int s_iz[4][NI];
    grid_dep_wait();
    publish_counters(a.pub_src, a.pub_dst);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nw = *a.nwork;
    const int n = a.n, m = a.n1 ? a.n1 : a.n;
    for (int w = vb * 4 + warp; w < nw; w += vg * 4) {
        const PeakRecH& r = a.peaks_h[w];
        s_p[warp][lane] = r.v[lane];
        if (lane < P * P - 32) s_p[warp][32 + lane] = r.v[32 + lane];
        const unsigned meta = r.meta;
        const int I = meta_I(meta), J = meta_J(meta);
        // zoom coordinate of index t: (t * 2)/20 - 1 + peak (exact at t = 0, 10, 20)
        int jz = 0;
        bool okj = false;
        float ry[4] = {0.f, 0.f, 0.f, 0.f};
        if (lane < NI) {
            const float x = (float)(lane * 2) / 20.0f - 1.0f + (float)I;
            const float y = (float)(lane * 2) / 20.0f - 1.0f + (float)J;
            const bool okx = !(x < 0.f || x > (float)(n - 1));
            const int iz = min(max((int)x, 0), n - 2);
            s_iz[warp][lane] = okx ? iz : -1;
#pragma unroll
            for (int q = 0; q < 4; ++q) s_rx[warp][lane][q] = keys32(fabsf(x - (float)(iz + q - 1)));
            okj = !(y < 0.f || y > (float)(m - 1));
            jz = min(max((int)y, 0), m - 2);
#pragma unroll
            for (int q = 0; q < 4; ++q) ry[q] = keys32(fabsf(y - (float)(jz + q - 1)));
        }
        __syncwarp();
        // contract patch rows I-2..I+3 (and their border extrapolations) along y
        if (lane < NI && okj) {
#pragma unroll
            for (int pr = 0; pr < P; ++pr) {
                const int rr = I - 2 + pr;
                float h = 0.f;
                bool bad = false;
                if (rr >= -1 && rr <= n) {
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        const float c = patch_cdata(s_p[warp], I, J, n, m, rr, jz + q - 1);
                        bad |= c == 0.f;
                        h = fmaf(c, ry[q], h);
                    }
                }
                s_h[warp][pr][lane] = h;
                s_hb[warp][pr][lane] = bad;
            }
        }
        __syncwarp();
        // zoom column `lane`: 21 rows, first maximum as a (value, -index) key
        unsigned long long best = 0ull;
        if (lane < NI) {
            for (int i = 0; i < NI; ++i) {
                const int iz = s_iz[warp][i];
                float v = 0.f;
                if (iz >= 0 && okj) {
                    bool bad = false;
                    float acc = 0.f;
#pragma unroll
                    for (int p = 0; p < 4; ++p) {
                        const int pr = iz - 1 + p - (I - 2);
                        bad |= s_hb[warp][pr][lane] != 0;
                        acc = fmaf(s_rx[warp][i][p], s_h[warp][pr][lane], acc);
                    }
                    v = bad ? 0.f : acc;
                }
                s_pk[warp][i * NI + lane] = v;
                if (!(v != v)) {
                    const unsigned long long key =
                        ((unsigned long long)ordered_bits(v) << 32) | (0xffffffffu - (unsigned)(i * NI + lane));
                    best = key > best ? key : best;
                }
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long other = __shfl_xor_sync(0xffffffffu, best, o);
            best = other > best ? other : best;
        }
        __syncwarp();
        if (lane == 0) {
            // a NaN first element stays the maximum of a sequential scan
            const int mi = (s_pk[warp][0] != s_pk[warp][0]) ? 0 : (int)(0xffffffffu - (unsigned)(best & 0xffffffffull));
            const int ixx = mi / NI, iyy = mi - (mi / NI) * NI;
            double ssx = 0., ssy = 0.;
            if (ixx > 0 && ixx < NI - 1 && iyy > 0 && iyy < NI - 1) {
                double v[9];
#pragma unroll
                for (int k = 0; k < 9; ++k) v[k] = f2d(s_pk[warp][(ixx - 1 + k / 3) * NI + (iyy - 1 + k % 3)]);
                fit3x3(v, &ssx, &ssy);
                // times rangex / (nxinterp - 1) = 2 / 20 (flct.c:1625-1628)
                ssx = dm(ssx, 2.) / 20.;
                ssy = dm(ssy, 2.) / 20.;
            }
            const double xw = ds(dm((double)ixx, 2.) / 20., 1.) + (double)I;
            const double yw = ds(dm((double)iyy, 2.) / 20., 1.) + (double)J;
            store_shift(a, w, ds(da(xw, ssx), (double)(n / 2)), ds(da(yw, ssy), (double)(m / 2)));
        }
        __syncwarp();
    }
}
FLCT_MULTI_KERNEL(__launch_bounds__(128), k_fit_hires, FitArgs)

__global__ void k_batch_starts(const unsigned char* ctr, const int* seg_pair, const int* first, int ngroups,
                               int* start) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= ngroups) return;
    int* st = start + first[g] + g;
    int acc = 0;
    st[0] = 0;
    for (int k = first[g]; k < first[g + 1]; ++k) {
        acc += *reinterpret_cast<const int*>(ctr + 64 * (size_t)seg_pair[k]);
        st[k - first[g] + 1] = acc;
    }
}

}  // namespace flct
