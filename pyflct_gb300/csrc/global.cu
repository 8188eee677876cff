// global.cu -- kernels of the sigma <= 0 mode (see global.cuh).
#include "global.cuh"

namespace flct {

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Block sums of (a, b) in a fixed order: lanes, then warps.
__device__ __forceinline__ void block_sum2(double& a, double& b) {
    __shared__ double s[2][32];
    a = warp_sum_d(a);
    b = warp_sum_d(b);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    if (lane == 0) {
        s[0][warp] = a;
        s[1][warp] = b;
    }
    __syncthreads();
    if (warp == 0) {
        a = lane < nw ? s[0][lane] : 0.;
        b = lane < nw ? s[1][lane] : 0.;
        a = warp_sum_d(a);
        b = warp_sum_d(b);
    }
}

__global__ void k_gsum_part(const double* __restrict__ f1, const double* __restrict__ f2, long n,
                            double* __restrict__ part) {
    const long chunk = (n + gridDim.x - 1) / gridDim.x;
    const long b0 = blockIdx.x * chunk, b1 = min(n, b0 + chunk);
    double a = 0., b = 0.;
    for (long k = b0 + threadIdx.x; k < b1; k += blockDim.x) {
        a = __dadd_rn(a, f1[k]);
        b = __dadd_rn(b, f2[k]);
    }
    block_sum2(a, b);
    if (threadIdx.x == 0) {
        part[2 * blockIdx.x] = a;
        part[2 * blockIdx.x + 1] = b;
    }
}

__global__ void k_gsum_final(const double* __restrict__ part, int nparts, double dn, double* __restrict__ means) {
    double a = 0., b = 0.;
    for (int k = threadIdx.x; k < nparts; k += blockDim.x) {
        a = __dadd_rn(a, part[2 * k]);
        b = __dadd_rn(b, part[2 * k + 1]);
    }
    block_sum2(a, b);
    if (threadIdx.x == 0) {
        means[0] = a / dn;  // flct.c:833-834
        means[1] = b / dn;
    }
}

__global__ void k_gz(const double* __restrict__ f1, const double* __restrict__ f2, long n,
                     const double* __restrict__ means, float2* __restrict__ z, unsigned* maxbits,
                     unsigned* status) {
    const float2 m1 = split_double_fast(means[0]), m2 = split_double_fast(means[1]);
    float mx1 = 0.f, mx2 = 0.f;
    for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) {
        const double fa = f1[k], fb = f2[k];
        const float2 a = split_double_fast(fa), b = split_double_fast(fb);
        if (((__float_as_uint(a.x) & 0x7fffffffu) == 0x7f800000u && finite_d(fa)) ||
            ((__float_as_uint(b.x) & 0x7fffffffu) == 0x7f800000u && finite_d(fb)))
            atomicOr(status, kStatusRange);
        const float d1 = (a.x - m1.x) + (a.y - m1.y), d2 = (b.x - m2.x) + (b.y - m2.y);
        z[k] = make_float2(d1, d2);
        mx1 = fmaxf(mx1, fabsf(d1));
        mx2 = fmaxf(mx2, fabsf(d2));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        mx1 = fmaxf(mx1, __shfl_xor_sync(0xffffffffu, mx1, o));
        mx2 = fmaxf(mx2, __shfl_xor_sync(0xffffffffu, mx2, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMax(maxbits, __float_as_uint(mx1));
        atomicMax(maxbits + 1, __float_as_uint(mx2));
    }
}

constexpr int kDftChunk = 2048;

template <int DIR>
__global__ void __launch_bounds__(256) k_dft_rows(const float2* __restrict__ in, float2* __restrict__ out, int L,
                                                  int lines, const float2* __restrict__ tw,
                                                  const unsigned* __restrict__ scale) {
    __shared__ float2 s_x[kDftChunk];
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = k < L;
    const float c1 = scale ? pow2_scale(scale[0]) : 1.f, c2 = scale ? pow2_scale(scale[1]) : 1.f;
    for (int line = blockIdx.y; line < lines; line += gridDim.y) {
        const float2* src = in + (size_t)line * L;
        float ax = 0.f, ay = 0.f;
        for (int j0 = 0; j0 < L; j0 += kDftChunk) {
            const int cnt = min(kDftChunk, L - j0);
            __syncthreads();
            for (int t = threadIdx.x; t < cnt; t += blockDim.x) {
                const float2 v = src[j0 + t];
                s_x[t] = make_float2(v.x * c1, v.y * c2);
            }
            __syncthreads();
            if (active) {
                int idx = (int)(((long)j0 * k) % L);  // (j k) mod L, stepped by k
                for (int t = 0; t < cnt; ++t) {
                    float2 w = __ldg(tw + idx);
                    if (DIR > 0) w.y = -w.y;
                    const float2 x = s_x[t];
                    ax = fmaf(x.x, w.x, fmaf(-x.y, w.y, ax));
                    ay = fmaf(x.x, w.y, fmaf(x.y, w.x, ay));
                    idx += k;
                    if (idx >= L) idx -= L;
                }
            }
        }
        if (active) out[(size_t)line * L + k] = make_float2(ax, ay);
    }
}
cudaError_t launch_dft_rows(bool inverse, const float2* in, float2* out, int L, int lines, const float2* tw,
                            const unsigned* scale, cudaStream_t st) {
    const dim3 g((L + 255) / 256, lines < 65535 ? lines : 65535);
    if (inverse) k_dft_rows<1><<<g, 256, 0, st>>>(in, out, L, lines, tw, scale);
    else k_dft_rows<-1><<<g, 256, 0, st>>>(in, out, L, lines, tw, scale);
    return cudaGetLastError();
}

__global__ void k_transpose(const float2* __restrict__ in, float2* __restrict__ out, int R, int C) {
    __shared__ float2 t[32][33];
    const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
    for (int dy = threadIdx.y; dy < 32; dy += blockDim.y) {
        const int r = r0 + dy, c = c0 + threadIdx.x;
        if (r < R && c < C) t[dy][threadIdx.x] = in[(size_t)r * C + c];
    }
    __syncthreads();
    for (int dy = threadIdx.y; dy < 32; dy += blockDim.y) {
        const int c = c0 + dy, r = r0 + threadIdx.x;
        if (r < R && c < C) out[(size_t)c * R + r] = t[threadIdx.x][dy];
    }
}

__global__ void k_gprod(const float2* __restrict__ zt, float2* __restrict__ ct, int nx, int ny,
                        const float* __restrict__ fx2, const float* __restrict__ fy2) {
    const long n = (long)nx * ny;
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x) {
        const int ky = (int)(e / nx), kx = (int)(e - (long)ky * nx);
        const int my = ky ? ny - ky : 0, mx = kx ? nx - kx : 0;
        const float2 z = zt[e], zm = zt[(size_t)my * nx + mx];
        const float ax = z.x + zm.x, ay = z.y - zm.y;  // 2 A
        const float bx = z.y + zm.y, by = zm.x - z.x;  // 2 B
        const float f = fx2[kx] * fy2[ky];
        ct[e] = make_float2(f * (ax * bx + ay * by), f * (ax * by - ay * bx));
    }
}

__global__ void k_gpeak(const float2* __restrict__ c, int nx, int ny, unsigned long long* key) {
    const long n = (long)nx * ny;
    unsigned long long best = 0ull;
    for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x) {
        const int i = (int)(e / ny), j = (int)(e - (long)i * ny);
        const float v = fabsf(c[e].x);
        if (v != v) continue;
        const int I = (i + nx / 2) % nx, J = (j + ny / 2) % ny;  // shift2d (flct.c:1510, 2111-2140)
        const unsigned long long kk =
            ((unsigned long long)__float_as_uint(v) << 32) | (0xffffffffu - (unsigned)(I * ny + J));
        best = kk > best ? kk : best;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long other = __shfl_xor_sync(0xffffffffu, best, o);
        best = other > best ? other : best;
    }
    if ((threadIdx.x & 31) == 0 && best) atomicMax(key, best);
}

__global__ void k_gpatch(const float2* __restrict__ c, int nx, int ny, const unsigned long long* __restrict__ key,
                         PeakRec* rec, PeakRecH* rech, int* work, int* nwork) {
    // |c| at shifted coordinates (I, J)
    auto sh = [&](int I, int J) -> float {
        const int i = (I - nx / 2 + nx) % nx, j = (J - ny / 2 + ny) % ny;
        return fabsf(c[(size_t)i * ny + j].x);
    };
    __shared__ int s_I, s_J, s_have;
    if (threadIdx.x == 0) {
        int I, J;
        bool have;
        if (sh(0, 0) != sh(0, 0)) {  // a NaN first element stays the maximum (maxloc, flct.c:2142-2161)
            I = 0;
            J = 0;
            have = true;
        } else {
            const unsigned long long k = *key;
            const unsigned L = 0xffffffffu - (unsigned)(k & 0xffffffffull);
            have = __uint_as_float((unsigned)(k >> 32)) != 0.0f;
            I = have ? (int)(L / ny) : nx / 2;
            J = have ? (int)(L % ny) : ny / 2;
        }
        s_I = I;
        s_J = J;
        s_have = have;
        work[0] = 0;
        *nwork = 1;
    }
    __syncthreads();
    const int I = s_I, J = s_J;
    const bool have = s_have;
    if (rech) {
        for (int k = threadIdx.x; k < kHiresPatch * kHiresPatch; k += blockDim.x) {
            const int r = I - 2 + k / kHiresPatch, q = J - 2 + k % kHiresPatch;
            rech->v[k] = (r >= 0 && r < nx && q >= 0 && q < ny) ? sh(r, q) : 0.f;
        }
        if (threadIdx.x == 0) rech->meta = peak_meta(I, J, have);
    } else {
        const bool dofit = have && I > 0 && I < nx - 1 && J > 0 && J < ny - 1;
        if (threadIdx.x < 9) rec->v[threadIdx.x] = dofit ? sh(I - 1 + threadIdx.x / 3, J - 1 + threadIdx.x % 3) : 0.f;
        if (threadIdx.x == 0) rec->meta = peak_meta(I, J, dofit);
    }
}

}  // namespace flct
