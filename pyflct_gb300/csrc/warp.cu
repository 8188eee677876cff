// warp.cu -- the warp program's two transforms on the GPU.
//
// shift_frac2d (source/warp.c:757-881): FFT, multiply by
//   exp(i 2 pi (kx dxarg + ky dyarg)), inverse FFT, real part / N.
// The phase factor is separable, so the operation is a circulant matrix
// along each axis: out = Re(Sx . X . Sy^T) with
//   sx[d] = (1/nx) sum_kx exp(i 2 pi kx (d/nx + dxarg)).
// Power-of-two axes (64 .. kWarpMaxAxis) apply it as transforms, one CTA
// per line (k_shift_lines_fft: forward FFT, phase factors, inverse FFT,
// O(L log L) per line), the slow axis after a transpose.  Other lengths
// take two passes of k_axis_* (one per axis), O(L) per output; the
// circulant vectors are built in FP64 from the reference's phase
// expression.
//
// warp_frac2d (source/warp.c:883-1011): F = DFT2(image) (the same axis
// kernels with the DFT matrix), then for every pixel the direct spectral sum
//   out[i][j] = (1/N) sum_{ii,jj} Re(F[ii][jj] exp(i(kx_ii xarg + ky_jj yarg)))
// with xarg = 2 pi (i - shift_slow)/nx, yarg = 2 pi (j - shift_fast)/ny.
// k_warp_sum evaluates it as a tiled complex GEMM over (pixels x ii) with the
// jj contraction inner; the phase of every term is reduced to a fraction of
// a turn from an FP64 per-pixel base with float-float products (error below
// 1e-7 turn for any wavenumber), then turned into cos/sin.
//
// Arithmetic is FP32 on the CUDA cores except the FP64 phase bases and the
// circulant / twiddle tables.
#include "warp.cuh"
#include "warp_math.cuh"

#include <algorithm>

namespace flct {

constexpr double kWarpPi = 3.1415926535898;  // warp.c:768, 895

// ------------------------------------------------------------ tables ----

// exp(sign 2 pi i k / L) for k < L in FP64, rounded once to float.
__global__ void k_twiddles(int L, int sign, float2* __restrict__ tw) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= L) return;
    double s, c;
    sincospi(2.0 * (double)k / (double)L, &s, &c);
    tw[k] = make_float2((float)c, (float)(sign * s));
}

// FP64 tables for the circulant vector of the uniform shift along an axis of
// length n: roots[e] = exp(2 pi i e / n) and ph[k] = exp(i 2 pi kf darg), the
// latter with the reference's expression 2*pi*kf*darg (warp.c:818-829).
__global__ void k_shift_tables(int n, double darg, double2* __restrict__ roots, double2* __restrict__ ph) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    double s, c;
    sincospi(2.0 * (double)k / (double)n, &s, &c);
    roots[k] = make_double2(c, s);
    const double kf = (double)freq_of(k, n);
    sincos(2. * kWarpPi * kf * darg, &s, &c);
    ph[k] = make_double2(c, s);
}

// v[d] = (1/n) sum_k exp(2 pi i k d / n) exp(i 2 pi kf darg), FP64 sums.
__global__ void k_shift_vector(int n, const double2* __restrict__ roots, const double2* __restrict__ ph,
                               float2* __restrict__ v) {
    for (int d = blockIdx.x * blockDim.x + threadIdx.x; d < n; d += gridDim.x * blockDim.x) {
        double re = 0., im = 0.;
        long long e = 0;  // k*d mod n, advanced incrementally
        for (int k = 0; k < n; ++k) {
            const double2 r = roots[e];
            const double2 p = ph[k];
            re = fma(r.x, p.x, fma(-r.y, p.y, re));
            im = fma(r.x, p.y, fma(r.y, p.x, im));
            e += d;
            if (e >= n) e -= n;
        }
        v[d] = make_float2((float)(re / n), (float)(im / n));
    }
}

// ------------------------------------------------------- axis kernels ----

// out[r][c] = sum_k in[r][k] * T(c, k) along the fast axis (length L = ny),
// T(c, k) = tab[(c - k) mod L] (circulant) or tab[(c k) mod L] (DFT).
// Tile: 16 rows x 64 columns, 256 threads (4 rows each), K chunks of 64.
template <int MODE, bool REAL_IN>
__global__ void __launch_bounds__(256) k_axis_fast(const void* __restrict__ in_, int nrows, int L,
                                                   const float2* __restrict__ tab, float2* __restrict__ out) {
    __shared__ float2 xs[16][65];
    extern __shared__ float2 ts[];  // L entries
    for (int k = threadIdx.x; k < L; k += blockDim.x) ts[k] = tab[k];
    const int c = blockIdx.x * 64 + (threadIdx.x & 63);
    const int rg = threadIdx.x >> 6;  // 0..3
    const int r0 = blockIdx.y * 16;
    float2 acc[4] = {};
    for (int k0 = 0; k0 < L; k0 += 64) {
        __syncthreads();
        for (int e = threadIdx.x; e < 16 * 64; e += blockDim.x) {
            const int rr = e >> 6, kk = e & 63;
            float2 v = make_float2(0.f, 0.f);
            if (r0 + rr < nrows && k0 + kk < L) {
                const size_t o = (size_t)(r0 + rr) * L + k0 + kk;
                if (REAL_IN) v.x = (float)static_cast<const double*>(in_)[o];
                else v = static_cast<const float2*>(in_)[o];
            }
            xs[rr][kk] = v;
        }
        __syncthreads();
        if (c < L) {
            const int kmax = min(64, L - k0);
            for (int kk = 0; kk < kmax; ++kk) {
                const int k = k0 + kk;
                int idx;
                if (MODE == 0) {
                    idx = c - k;
                    idx += (idx < 0) ? L : 0;
                } else {
                    idx = (int)(((long long)c * k) % L);
                }
                const float2 t = ts[idx];
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const float2 x = xs[rg * 4 + q][kk];
                    acc[q].x = fmaf(x.x, t.x, fmaf(-x.y, t.y, acc[q].x));
                    acc[q].y = fmaf(x.x, t.y, fmaf(x.y, t.x, acc[q].y));
                }
            }
        }
    }
    if (c < L) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int r = r0 + rg * 4 + q;
            if (r < nrows) out[(size_t)r * L + c] = acc[q];
        }
    }
}

// out[r][c] = sum_k T(r, k) * in[k][c] along the slow axis (length L = nx).
// Tile: 16 output rows x 64 columns; K chunks of 32 input rows.
template <int MODE>
__global__ void __launch_bounds__(256) k_axis_slow(const float2* __restrict__ in, int ncols, int L,
                                                   const float2* __restrict__ tab, float2* __restrict__ out) {
    __shared__ float2 xs[32][65];
    extern __shared__ float2 ts[];
    for (int k = threadIdx.x; k < L; k += blockDim.x) ts[k] = tab[k];
    const int cl = threadIdx.x & 63;
    const int c = blockIdx.x * 64 + cl;
    const int rg = threadIdx.x >> 6;
    const int r0 = blockIdx.y * 16;
    float2 acc[4] = {};
    for (int k0 = 0; k0 < L; k0 += 32) {
        __syncthreads();
        for (int e = threadIdx.x; e < 32 * 64; e += blockDim.x) {
            const int kk = e >> 6, cc = e & 63;
            float2 v = make_float2(0.f, 0.f);
            if (k0 + kk < L && blockIdx.x * 64 + cc < ncols) v = in[(size_t)(k0 + kk) * ncols + blockIdx.x * 64 + cc];
            xs[kk][cc] = v;
        }
        __syncthreads();
        const int kmax = min(32, L - k0);
        for (int kk = 0; kk < kmax; ++kk) {
            const int k = k0 + kk;
            const float2 x = xs[kk][cl];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int r = r0 + rg * 4 + q;
                int idx;
                if (MODE == 0) {
                    idx = r - k;
                    idx += (idx < 0) ? L : 0;
                    idx = (r < L) ? idx : 0;
                } else {
                    idx = (int)(((long long)r * k) % L);
                }
                const float2 t = ts[idx];
                acc[q].x = fmaf(x.x, t.x, fmaf(-x.y, t.y, acc[q].x));
                acc[q].y = fmaf(x.x, t.y, fmaf(x.y, t.x, acc[q].y));
            }
        }
    }
    if (c < ncols) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int r = r0 + rg * 4 + q;
            if (r < L) out[(size_t)r * ncols + c] = acc[q];
        }
    }
}

// --------------------------------------------------- transform path ----

// Each line of length L (a power of two): X = FFT(line) by radix-2
// decimation in time in shared memory (inputs placed at bit-reversed
// positions), X[k] *= ph[k], then the inverse by radix-2 decimation in
// frequency (natural order in, bit-reversed out), read back in natural
// order, times `scale`.  tw[t] = exp(-2 pi i t / L) (FP64, rounded once);
// ph[k] = exp(i 2 pi kf darg) in FP64 from k_shift_tables.  FWD_ONLY stops
// after the forward transform and writes X (natural order; ph and scale
// unused): warp_frac2d's spectrum.
template <bool REAL_IN, bool FWD_ONLY = false>
__global__ void __launch_bounds__(512) k_shift_lines_fft(const void* __restrict__ in_, int nlines, int L, int logL,
                                                         const float2* __restrict__ tw,
                                                         const double2* __restrict__ ph, float scale,
                                                         float2* __restrict__ out) {
    extern __shared__ float2 x[];  // L
    const int half = L >> 1;
    for (int line = blockIdx.x; line < nlines; line += gridDim.x) {
        for (int k = threadIdx.x; k < L; k += blockDim.x) {
            const size_t o = (size_t)line * L + k;
            float2 v;
            if (REAL_IN) v = make_float2((float)static_cast<const double*>(in_)[o], 0.f);
            else v = static_cast<const float2*>(in_)[o];
            x[__brev((unsigned)k) >> (32 - logL)] = v;
        }
        __syncthreads();
        for (int m = 1; m < L; m <<= 1) {  // butterflies of half-size m
            const int ts = half / m;
            for (int b = threadIdx.x; b < half; b += blockDim.x) {
                const int j = b & (m - 1), k = ((b - j) << 1) + j;
                const float2 w = __ldg(tw + j * ts);  // exp(-2 pi i j / 2m)
                const float2 u = x[k], v = x[k + m];
                const float2 t = make_float2(v.x * w.x - v.y * w.y, v.x * w.y + v.y * w.x);
                x[k] = make_float2(u.x + t.x, u.y + t.y);
                x[k + m] = make_float2(u.x - t.x, u.y - t.y);
            }
            __syncthreads();
        }
        if constexpr (FWD_ONLY) {
            for (int k = threadIdx.x; k < L; k += blockDim.x) out[(size_t)line * L + k] = x[k];
        } else {
            for (int k = threadIdx.x; k < L; k += blockDim.x) {
                const double2 p = ph[k];
                const float px = (float)p.x, py = (float)p.y;
                const float2 a = x[k];
                x[k] = make_float2(a.x * px - a.y * py, a.x * py + a.y * px);
            }
            __syncthreads();
            for (int m = half; m >= 1; m >>= 1) {
                const int ts = half / m;
                for (int b = threadIdx.x; b < half; b += blockDim.x) {
                    const int j = b & (m - 1), k = ((b - j) << 1) + j;
                    const float2 w = __ldg(tw + j * ts);
                    const float2 u = x[k], v = x[k + m];
                    const float2 d = make_float2(u.x - v.x, u.y - v.y);
                    x[k] = make_float2(u.x + v.x, u.y + v.y);
                    x[k + m] = make_float2(d.x * w.x + d.y * w.y, d.y * w.x - d.x * w.y);  // d exp(+2 pi i j / 2m)
                }
                __syncthreads();
            }
            for (int k = threadIdx.x; k < L; k += blockDim.x) {
                const float2 v = x[__brev((unsigned)k) >> (32 - logL)];
                out[(size_t)line * L + k] = make_float2(v.x * scale, v.y * scale);
            }
        }
        __syncthreads();  // the next line overwrites x
    }
}

// out[c][r] = in[r][c] (complex), 32 x 32 tiles.
__global__ void __launch_bounds__(256) k_transpose_c(const float2* __restrict__ in, int rows, int cols,
                                                     float2* __restrict__ out) {
    __shared__ float2 t[32][33];
    const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
    for (int i = threadIdx.y; i < 32; i += 8)
        if (r0 + i < rows && c0 + threadIdx.x < cols) t[i][threadIdx.x] = in[(size_t)(r0 + i) * cols + c0 + threadIdx.x];
    __syncthreads();
    for (int i = threadIdx.y; i < 32; i += 8)
        if (c0 + i < cols && r0 + threadIdx.x < rows) out[(size_t)(c0 + i) * rows + r0 + threadIdx.x] = t[threadIdx.x][i];
}

// out[c][r] = Re(in[r][c]) as double, 32 x 32 tiles.
__global__ void __launch_bounds__(256) k_transpose_re(const float2* __restrict__ in, int rows, int cols,
                                                      double* __restrict__ out) {
    __shared__ float t[32][33];
    const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
    for (int i = threadIdx.y; i < 32; i += 8)
        if (r0 + i < rows && c0 + threadIdx.x < cols) t[i][threadIdx.x] = in[(size_t)(r0 + i) * cols + c0 + threadIdx.x].x;
    __syncthreads();
    for (int i = threadIdx.y; i < 32; i += 8)
        if (c0 + i < cols && r0 + threadIdx.x < rows) out[(size_t)(c0 + i) * rows + r0 + threadIdx.x] = (double)t[threadIdx.x][i];
}

__global__ void k_real_part(const float2* __restrict__ in, long n, double* __restrict__ out) {
    for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x)
        out[k] = (double)in[k].x;
}

// --------------------------------------------------------- warp sum ----

// Per-pixel phase base in turns: ((double)idx - shift) / n, split hi + lo.
__global__ void k_warp_phase(const double* __restrict__ delx, const double* __restrict__ dely, int nx, int ny,
                             int transp, float4* __restrict__ ph) {
    const long n = (long)nx * ny;
    for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) {
        const int i = (int)(k / ny), j = (int)(k - (long)i * ny);
        // warp.c:948-959: transp swaps the roles of delx and dely
        const double sx = transp ? dely[k] : delx[k];
        const double sy = transp ? delx[k] : dely[k];
        const double tx = (((double)i) - sx) / (double)nx;  // xarg / (2 pi)
        const double ty = (((double)j) - sy) / (double)ny;
        const float txh = (float)tx, tyh = (float)ty;
        ph[k] = make_float4(txh, (float)(tx - (double)txh), tyh, (float)(ty - (double)tyh));
    }
}

// Tile: 64 pixels x 128 wavenumbers ii, contraction over jj in chunks of 16.
// 256 threads: tx = t % 16 owns ii = tx + 16 q (q < 8), ty = t / 16 owns
// pixels ty + 16 p (p < 4).
__global__ void __launch_bounds__(256) k_warp_sum(const float2* __restrict__ F, const float4* __restrict__ ph,
                                                  int nx, int ny, double normfac, double* __restrict__ out) {
    __shared__ float2 eys[64][17];   // exp(i ky_jj yarg_px)
    __shared__ float2 fs[128][17];   // F[ii][jj]
    __shared__ float4 phs[64];
    __shared__ float tot[64];
    const long npx = (long)nx * ny;
    const long p0 = (long)blockIdx.x * 64;
    const int t = threadIdx.x, tx = t & 15, ty = t >> 4;
    if (t < 64) {
        phs[t] = (p0 + t < npx) ? ph[p0 + t] : make_float4(0.f, 0.f, 0.f, 0.f);
        tot[t] = 0.f;
    }
    __syncthreads();
    for (int i0 = 0; i0 < nx; i0 += 128) {
        float2 acc[4][8] = {};
        for (int j0 = 0; j0 < ny; j0 += 16) {
            __syncthreads();
            // 64 x 16 phase factors, 4 per thread
            for (int e = t; e < 64 * 16; e += 256) {
                const int px = e >> 4, jj = e & 15;
                float2 v = make_float2(0.f, 0.f);
                if (j0 + jj < ny) {
                    const float kf = (float)freq_of(j0 + jj, ny);
                    v = turn_cs(kf, phs[px].z, phs[px].w);
                }
                eys[px][jj] = v;
            }
            for (int e = t; e < 128 * 16; e += 256) {
                const int ii = e >> 4, jj = e & 15;
                float2 v = make_float2(0.f, 0.f);
                if (i0 + ii < nx && j0 + jj < ny) v = F[(size_t)(i0 + ii) * ny + j0 + jj];
                fs[ii][jj] = v;
            }
            __syncthreads();
#pragma unroll 4
            for (int jj = 0; jj < 16; ++jj) {
                float2 a[4], b[8];
#pragma unroll
                for (int p = 0; p < 4; ++p) a[p] = eys[ty + 16 * p][jj];
#pragma unroll
                for (int q = 0; q < 8; ++q) b[q] = fs[tx + 16 * q][jj];
#pragma unroll
                for (int p = 0; p < 4; ++p)
#pragma unroll
                    for (int q = 0; q < 8; ++q) {
                        acc[p][q].x = fmaf(a[p].x, b[q].x, fmaf(-a[p].y, b[q].y, acc[p][q].x));
                        acc[p][q].y = fmaf(a[p].x, b[q].y, fmaf(a[p].y, b[q].x, acc[p][q].y));
                    }
            }
        }
        // times exp(i kx_ii xarg_px), real part, summed over this thread's ii
#pragma unroll
        for (int p = 0; p < 4; ++p) {
            const int px = ty + 16 * p;
            float s = 0.f;
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const int ii = i0 + tx + 16 * q;
                if (ii < nx) {
                    const float2 ex = turn_cs((float)freq_of(ii, nx), phs[px].x, phs[px].y);
                    s = fmaf(ex.x, acc[p][q].x, fmaf(-ex.y, acc[p][q].y, s));
                }
            }
            // reduce over the 16 tx lanes (aligned half-warp)
#pragma unroll
            for (int o = 8; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
            if (tx == 0) tot[px] += s;
        }
    }
    __syncthreads();
    if (t < 64 && p0 + t < npx) out[p0 + t] = (double)tot[t] * normfac;
}

// ------------------------------------------------------------ host ----

cudaError_t launch_axis_fast(int mode, bool real_in, const void* in, int nrows, int L, const float2* tab,
                             float2* out, cudaStream_t st) {
    dim3 g((L + 63) / 64, (nrows + 15) / 16);
    const size_t sm = (size_t)L * sizeof(float2);
    cudaError_t e = cudaSuccess;
#define FLCT_AF(M, R)                                                                                \
    e = cudaFuncSetAttribute(k_axis_fast<M, R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm); \
    if (e != cudaSuccess) return e;                                                                  \
    k_axis_fast<M, R><<<g, 256, sm, st>>>(in, nrows, L, tab, out);
    if (mode == 0 && real_in) { FLCT_AF(0, true) }
    else if (mode == 0) { FLCT_AF(0, false) }
    else if (real_in) { FLCT_AF(1, true) }
    else { FLCT_AF(1, false) }
#undef FLCT_AF
    return cudaGetLastError();
}

cudaError_t launch_axis_slow(int mode, const float2* in, int ncols, int L, const float2* tab, float2* out,
                             cudaStream_t st) {
    dim3 g((ncols + 63) / 64, (L + 15) / 16);
    const size_t sm = (size_t)L * sizeof(float2);
    cudaError_t e;
    if (mode == 0) {
        e = cudaFuncSetAttribute(k_axis_slow<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return e;
        k_axis_slow<0><<<g, 256, sm, st>>>(in, ncols, L, tab, out);
    } else {
        e = cudaFuncSetAttribute(k_axis_slow<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return e;
        k_axis_slow<1><<<g, 256, sm, st>>>(in, ncols, L, tab, out);
    }
    return cudaGetLastError();
}

cudaError_t launch_shift_vector(int n, double darg, double2* scratch, float2* v, cudaStream_t st) {
    k_shift_tables<<<(n + 127) / 128, 128, 0, st>>>(n, darg, scratch, scratch + n);
    k_shift_vector<<<(n + 63) / 64, 64, 0, st>>>(n, scratch, scratch + n, v);
    return cudaGetLastError();
}

bool shift_fft_axis(int n) { return n >= 64 && n <= kWarpMaxAxis && (n & (n - 1)) == 0; }

cudaError_t launch_shift_fft(const double* in, int nx, int ny, double dxarg, double dyarg, double2* scratch,
                             float2* tw, float2* buf1, float2* buf2, double* out, int nsm, cudaStream_t st) {
    // FP64 phase factors (and roots, unused here) of both axes, twiddles
    double2* rx = scratch;
    double2* phx = rx + nx;
    double2* ry = phx + nx;
    double2* phy = ry + ny;
    k_shift_tables<<<(nx + 127) / 128, 128, 0, st>>>(nx, dxarg, rx, phx);
    k_shift_tables<<<(ny + 127) / 128, 128, 0, st>>>(ny, dyarg, ry, phy);
    float2* twx = tw;
    float2* twy = tw + nx;
    k_twiddles<<<(nx + 255) / 256, 256, 0, st>>>(nx, -1, twx);
    k_twiddles<<<(ny + 255) / 256, 256, 0, st>>>(ny, -1, twy);
    auto log2i = [](int n) {
        int l = 0;
        while ((1 << l) < n) ++l;
        return l;
    };
    cudaError_t e;
    const size_t smy = (size_t)ny * sizeof(float2), smx = (size_t)nx * sizeof(float2);
    e = cudaFuncSetAttribute(k_shift_lines_fft<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smy);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(k_shift_lines_fft<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smx);
    if (e != cudaSuccess) return e;
    // fast axis: rows of the image, then the slow axis as rows of the transpose
    k_shift_lines_fft<true><<<std::min(nx, nsm * 4), std::min(512, ny / 2), smy, st>>>(
        in, nx, ny, log2i(ny), twy, phy, 1.0f / (float)ny, buf1);
    k_transpose_c<<<dim3((ny + 31) / 32, (nx + 31) / 32), dim3(32, 8), 0, st>>>(buf1, nx, ny, buf2);
    k_shift_lines_fft<false><<<std::min(ny, nsm * 4), std::min(512, nx / 2), smx, st>>>(
        buf2, ny, nx, log2i(nx), twx, phx, 1.0f / (float)nx, buf1);
    k_transpose_re<<<dim3((nx + 31) / 32, (ny + 31) / 32), dim3(32, 8), 0, st>>>(buf1, ny, nx, out);
    return cudaGetLastError();
}

cudaError_t launch_dft2_fft(const double* in, int nx, int ny, float2* tw, float2* buf1, float2* F, int nsm,
                           cudaStream_t st) {
    auto log2i = [](int n) {
        int l = 0;
        while ((1 << l) < n) ++l;
        return l;
    };
    float2* twx = tw;
    float2* twy = tw + nx;
    k_twiddles<<<(nx + 255) / 256, 256, 0, st>>>(nx, -1, twx);
    k_twiddles<<<(ny + 255) / 256, 256, 0, st>>>(ny, -1, twy);
    const size_t smy = (size_t)ny * sizeof(float2), smx = (size_t)nx * sizeof(float2);
    cudaError_t e;
    e = cudaFuncSetAttribute(k_shift_lines_fft<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smy);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(k_shift_lines_fft<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smx);
    if (e != cudaSuccess) return e;
    // rows (fast axis), then the slow axis as rows of the transpose, then back
    k_shift_lines_fft<true, true><<<std::min(nx, nsm * 4), std::min(512, ny / 2), smy, st>>>(
        in, nx, ny, log2i(ny), twy, nullptr, 1.0f, buf1);
    k_transpose_c<<<dim3((ny + 31) / 32, (nx + 31) / 32), dim3(32, 8), 0, st>>>(buf1, nx, ny, F);
    k_shift_lines_fft<false, true><<<std::min(ny, nsm * 4), std::min(512, nx / 2), smx, st>>>(
        F, ny, nx, log2i(nx), twx, nullptr, 1.0f, buf1);
    k_transpose_c<<<dim3((nx + 31) / 32, (ny + 31) / 32), dim3(32, 8), 0, st>>>(buf1, ny, nx, F);
    return cudaGetLastError();
}

cudaError_t launch_twiddles(int L, int sign, float2* tw, cudaStream_t st) {
    k_twiddles<<<(L + 255) / 256, 256, 0, st>>>(L, sign, tw);
    return cudaGetLastError();
}

cudaError_t launch_real_part(const float2* in, long n, double* out, cudaStream_t st) {
    k_real_part<<<(int)std::min<long>((n + 255) / 256, 4096), 256, 0, st>>>(in, n, out);
    return cudaGetLastError();
}

cudaError_t launch_warp_phase(const double* delx, const double* dely, int nx, int ny, int transp, float4* ph,
                              cudaStream_t st) {
    const long n = (long)nx * ny;
    k_warp_phase<<<(int)std::min<long>((n + 255) / 256, 4096), 256, 0, st>>>(delx, dely, nx, ny, transp, ph);
    return cudaGetLastError();
}

cudaError_t launch_warp_sum(const float2* F, const float4* ph, int nx, int ny, double* out, cudaStream_t st) {
    const long npx = (long)nx * ny;
    k_warp_sum<<<(int)((npx + 63) / 64), 256, 0, st>>>(F, ph, nx, ny, 1. / ((double)nx * ny), out);
    return cudaGetLastError();
}

}  // namespace flct
