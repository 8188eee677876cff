// window_fp32.cuh -- K1, the fused per-window correlation kernel (FP32 form).
//
// Replaces the per-pixel body of the reference's main loop and cross_cor
// (source/flct.c:773-942 and 1325-1649): for every pixel on the work list it
// takes the n x n box around the pixel from both frames, subtracts the FP64
// local means, applies the Gaussian centred on the pixel, transforms both
// sub-images, forms conj(A)*B (times the squared k-space filter for -k),
// transforms back, takes |c| in the half-shifted frame, finds the first
// strict maximum and refines it with the FP64 3x3 Taylor fit.
//
// Layout: a "team" of n threads owns one window; a CTA runs TEAMS teams in
// lockstep.  The two real sub-images travel as one complex array
// z = g1 + i g2 (one forward FFT for both); A and B are separated with the
// mirror Z(-k).  The 2-D transforms are register FFTs along one axis, a
// shared-memory transpose, and register FFTs along the other axis.  Each
// sub-image is scaled by an exact power of two so FP32 never over- or
// under-flows; scaling changes neither the argmax nor the fit.
#pragma once
#include "common.cuh"
#include "fft_reg.cuh"

namespace flct {

constexpr int kMaxBox = 64;  // largest box side with a compiled kernel

struct WinArgs {
    const float2* s1;     // f1 split (hi, lo) [nx*ny]
    const float2* s2;     // f2 split
    const double* bs1;    // f1 box sums [(nx-n+1) x bsw]
    const double* bs2;
    const int* work;      // pixel indices i*ny + j
    const int* nwork;     // number of work items (device)
    int nx, ny, nsize, bsw;
    double inv_n2;        // 1 / n^2
    double deltinv, deltas;
    int use_filter;       // -k given
    int direct;           // windows given directly: box w starts at row w*n, no mean, unit weights
    int interpolate, skip, xoff, yoff, jcnt;
    double *vx, *vy, *vm; // outputs [nx*ny]
    double *gvx, *gvy;    // skip-grid copies of vx, vy (interpolation) or null
    double* shx;          // optional raw shifts per work item (slow axis)
    double* shy;          // optional raw shifts per work item (fast axis)
    float gauss[2 * kMaxBox + 1];  // weight of offset d at d + n (separable Gaussian)
    float filt2[kMaxBox];          // squared k-space filter factor by frequency index
};

template <int N>
struct WinShape {
    static constexpr int TEAMS = (N <= 8) ? (128 / N) : (N <= 20) ? 8 : (N <= 40) ? 4 : 2;
    static constexpr int THREADS = N * TEAMS;
    static constexpr int BUF = N * (N + 1);  // float2 per team
    static constexpr size_t head = 32 * TEAMS + ((3 * N + 1) * 4 + 15) / 16 * 16;
    static constexpr size_t smem = head + (size_t)TEAMS * BUF * 8 + (size_t)TEAMS * N * N * 4;
};

// Reference-order FP64 helpers (no contraction into FMA).
__device__ __forceinline__ double dm(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double da(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double ds(double a, double b) { return __dsub_rn(a, b); }

// 3x3 Taylor fit (flct.c:1536-1553) on |c| values around the peak.
// v[a][b] = |c| at (I-1+a, J-1+b).
__device__ __forceinline__ void taylor_fit(const double v[3][3], double* sx, double* sy) {
    double fx = dm(0.5, ds(v[2][1], v[0][1]));
    double fy = dm(0.5, ds(v[1][2], v[1][0]));
    double fxx = ds(da(v[2][1], v[0][1]), dm(2., v[1][1]));
    double fyy = ds(da(v[1][2], v[1][0]), dm(2., v[1][1]));
    double fxy = dm(0.25, ds(ds(da(v[2][2], v[0][0]), v[2][0]), v[0][2]));
    double den = ds(dm(fxy, fxy), dm(fxx, fyy));
    *sx = ds(dm(fyy, fx), dm(fy, fxy)) / den;
    *sy = ds(dm(fxx, fy), dm(fx, fxy)) / den;
}

template <int N>
__global__ void __launch_bounds__(WinShape<N>::THREADS)
k_window_fp32(WinArgs a) {
    using S = WinShape<N>;
    constexpr int TEAMS = S::TEAMS;
    extern __shared__ __align__(16) unsigned char sm[];
    float4* s_mean = reinterpret_cast<float4*>(sm);
    unsigned long long* s_key = reinterpret_cast<unsigned long long*>(sm + 16 * TEAMS);
    unsigned* s_max = reinterpret_cast<unsigned*>(sm + 24 * TEAMS);
    float* s_g = reinterpret_cast<float*>(sm + 32 * TEAMS);
    float* s_f = s_g + (2 * N + 1);
    float2* s_buf = reinterpret_cast<float2*>(sm + S::head);
    float* s_abs = reinterpret_cast<float*>(s_buf + TEAMS * S::BUF);

    const int team = threadIdx.x / N;
    const int ln = threadIdx.x - team * N;
    for (int k = threadIdx.x; k < 2 * N + 1; k += blockDim.x) s_g[k] = a.gauss[k];
    for (int k = threadIdx.x; k < N; k += blockDim.x) s_f[k] = a.use_filter ? a.filt2[k] : 1.0f;
    float2* buf = s_buf + team * S::BUF;
    float* ab = s_abs + team * N * N;
    const int nwork = *a.nwork;
    __syncthreads();

    for (int base = blockIdx.x * TEAMS; base < nwork; base += gridDim.x * TEAMS) {
        const int w = base + team;
        const bool valid = w < nwork;
        const int pix = a.work[valid ? w : base];
        int i, j, imin, jmin;
        if (a.direct) {
            imin = pix / a.ny;
            jmin = 0;
            i = imin;
            j = 0;
        } else {
            i = pix / a.ny;
            j = pix - i * a.ny;
            imin = box_start(i, a.nx, a.nsize);
            jmin = box_start(j, a.ny, a.nsize);
        }

        // FP64 local means from the box sums, split into float hi + lo
        if (ln == 0) {
            float2 m1 = make_float2(0.f, 0.f), m2 = m1;
            if (!a.direct) {
                const size_t b = (size_t)imin * a.bsw + jmin;
                m1 = split_double(dm(a.bs1[b], a.inv_n2));
                m2 = split_double(dm(a.bs2[b], a.inv_n2));
            }
            s_mean[team] = make_float4(m1.x, m1.y, m2.x, m2.y);
            s_max[2 * team] = 0u;
            s_max[2 * team + 1] = 0u;
            s_key[team] = 0ull;
        }
        __syncthreads();

        // windowed, mean-subtracted column jj = ln of both frames: z = g1 + i g2
        float2 x[N];
        {
            const float4 mm = s_mean[team];
            const float wc = s_g[ln + jmin - j + N];
            const float2* p1 = a.s1 + (size_t)imin * a.ny + jmin + ln;
            const float2* p2 = a.s2 + (size_t)imin * a.ny + jmin + ln;
            const float* gr = s_g + (imin - i + N);
            float mx1 = 0.f, mx2 = 0.f;
#pragma unroll
            for (int ii = 0; ii < N; ++ii) {
                const float2 u = __ldg(p1 + (size_t)ii * a.ny);
                const float2 v = __ldg(p2 + (size_t)ii * a.ny);
                const float wgt = wc * gr[ii];
                const float d1 = (u.x - mm.x) + (u.y - mm.y);
                const float d2 = (v.x - mm.z) + (v.y - mm.w);
                x[ii] = make_float2(wgt * d1, wgt * d2);
                mx1 = fmaxf(mx1, fabsf(x[ii].x));
                mx2 = fmaxf(mx2, fabsf(x[ii].y));
            }
            atomicMax(&s_max[2 * team], __float_as_uint(mx1));
            atomicMax(&s_max[2 * team + 1], __float_as_uint(mx2));
        }
        __syncthreads();
        {
            const float c1 = pow2_scale(s_max[2 * team]), c2 = pow2_scale(s_max[2 * team + 1]);
#pragma unroll
            for (int ii = 0; ii < N; ++ii) x[ii] = make_float2(x[ii].x * c1, x[ii].y * c2);
        }

        // forward 2-D FFT: columns in registers, transpose, rows in registers
        dif<N, 0, -1>(x);
        sfor<0, N>([&](auto kc) {
            constexpr int k = decltype(kc)::value;
            buf[k * (N + 1) + ln] = x[dif_pos<N>(k)];
        });
        __syncthreads();
        sfor<0, N>([&](auto jc) {
            constexpr int jj = decltype(jc)::value;
            x[jj] = buf[ln * (N + 1) + jj];
        });
        __syncthreads();
        dif<N, 0, -1>(x);  // thread ln now holds Z[kx = ln][ky]
        sfor<0, N>([&](auto kc) {
            constexpr int k = decltype(kc)::value;
            buf[ln * (N + 1) + k] = x[dif_pos<N>(k)];
        });
        __syncthreads();

        // separate A, B from Z and its mirror, C = conj(A) B filt^2
        float2 y[N];
        {
            const int mr = (N - ln) % N;
            const float fr = s_f[ln];
            sfor<0, N>([&](auto kc) {
                constexpr int k = decltype(kc)::value;
                constexpr int mk = (N - k) % N;
                const float2 z = x[dif_pos<N>(k)];
                const float2 zm = buf[mr * (N + 1) + mk];
                const float ax = z.x + zm.x, ay = z.y - zm.y;  // 2 s1 A
                const float bx = z.y + zm.y, by = zm.x - z.x;  // 2 s2 B
                const float f = fr * s_f[k];
                y[k] = make_float2(f * (ax * bx + ay * by), f * (ax * by - ay * bx));
            });
        }
        // inverse: rows (ky -> j) in registers, transpose, columns (kx -> i)
        dif<N, 0, +1>(y);
        __syncthreads();
        sfor<0, N>([&](auto jc) {
            constexpr int jj = decltype(jc)::value;
            buf[ln * (N + 1) + jj] = y[dif_pos<N>(jj)];
        });
        __syncthreads();
        sfor<0, N>([&](auto kc) {
            constexpr int k = decltype(kc)::value;
            y[k] = buf[k * (N + 1) + ln];
        });
        dif<N, 0, +1>(y);  // y[dif_pos(i)].x = c[i][ln]

        // |c| in the half-shifted frame and the first strict maximum
        {
            const int J = (ln + N / 2) % N;
            unsigned long long best = 0ull;
            sfor<0, N>([&](auto Ic) {
                constexpr int I = decltype(Ic)::value;
                constexpr int ii = (I + N / 2) % N;
                const float v = fabsf(y[dif_pos<N>(ii)].x);
                ab[I * N + J] = v;
                if (!(v != v)) {
                    const unsigned long long key =
                        ((unsigned long long)__float_as_uint(v) << 32) |
                        (unsigned long long)(0xffffffffu - (unsigned)(I * N + J));
                    best = key > best ? key : best;
                }
            });
            atomicMax(&s_key[team], best);
        }
        __syncthreads();

        if (ln == 0 && valid) {
            int I, J;
            bool have;
            const float v0 = ab[0];
            if (v0 != v0) {
                // a NaN first element stays the maximum of a sequential scan
                I = 0;
                J = 0;
                have = true;
            } else {
                const unsigned long long key = s_key[team];
                const unsigned L = 0xffffffffu - (unsigned)(key & 0xffffffffull);
                have = __uint_as_float((unsigned)(key >> 32)) != 0.0f;
                I = have ? (int)(L / N) : N / 2;
                J = have ? (int)(L % N) : N / 2;
            }
            double sx = 0., sy = 0.;
            if (have && I > 0 && I < N - 1 && J > 0 && J < N - 1) {
                double v[3][3];
#pragma unroll
                for (int p = 0; p < 3; ++p)
#pragma unroll
                    for (int q = 0; q < 3; ++q) v[p][q] = (double)ab[(I - 1 + p) * N + (J - 1 + q)];
                taylor_fit(v, &sx, &sy);
            }
            const double shx = ds(da((double)I, sx), (double)(N / 2));
            const double shy = ds(da((double)J, sy), (double)(N / 2));
            if (a.shx) {
                a.shx[w] = shx;
                a.shy[w] = shy;
            }
            if (a.vx) {
                // transposed storage: vx from the fast-axis shift (flct.c:901-905)
                double vxx = dm(dm(shy, a.deltinv), a.deltas);
                double vyy = dm(dm(shx, a.deltinv), a.deltas);
                double vmm = 1.;
                if (a.gvx) {
                    const int ic = (i - a.xoff) / a.skip, jc = (j - a.yoff) / a.skip;
                    a.gvx[(size_t)ic * a.jcnt + jc] = vxx;
                    a.gvy[(size_t)ic * a.jcnt + jc] = vyy;
                }
                // the final xmiss reset (flct.c:1125-1133)
                if (vxx == kXmiss) {
                    vmm = 0.;
                    vxx = 0.;
                }
                if (vyy == kXmiss) vyy = 0.;
                a.vx[pix] = vxx;
                a.vy[pix] = vyy;
                a.vm[pix] = vmm;
            }
        }
    }
}

// Host-side launcher for one box size (defined in the per-size .cu files).
template <int N>
cudaError_t launch_window_fp32(const WinArgs& a, int grid, cudaStream_t st);
template <int N>
int window_fp32_blocks_per_sm();

}  // namespace flct
