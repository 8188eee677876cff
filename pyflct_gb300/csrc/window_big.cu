// window_big.cu -- the window-correlation kernel for boxes above 64
// (sigma >= 16), FP32 form.
//
// Same contract as k_window_fp32 (source/flct.c:829-876, 1325-1532: window,
// transforms of both sub-images, conj(A) B times the optional squared
// filter, inverse, |c| in the half-shifted frame, first strict maximum,
// peak record), for any box side n (a multiple of 4) up to kMaxBigBox.  The
// register FFTs of k_window_fp32 are compiled per box side and stop at 64;
// here one CTA of 256 threads owns one window at a time and keeps it in
// shared memory (n x (n + 1) complex values, z = g1 + i g2), and every 1-D
// transform is a direct DFT against a twiddle table (one warp per line,
// lane k sums its outputs' n terms).  That is O(n^3) work per window instead
// of O(n^2 log n), but it serves every n with one kernel, and these boxes
// are rare (the reference's own box for sigma 16 is 68 x 68).
#include <cuda_runtime.h>

#include "window_big.cuh"

namespace flct {

namespace {

constexpr int kBigThreads = 256;

__device__ __forceinline__ unsigned long long warp_max_key(unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
        v = w > v ? w : v;
    }
    return v;
}

// The n direct DFTs of length n along one axis of z (stride `ls` between
// the elements of a line, `lstride` between lines): one warp per line,
// the line staged in the warp's buffer first, so the transform is in place.
// sign -1: forward (e^{-2 pi i j k / n}), +1: inverse.  `scale` multiplies
// the inputs component-wise (the sub-images' power-of-two scales).
__device__ void dft_lines(float2* z, int n, int ls, int lstride, const float2* tw, float2* wbuf, int sign,
                          float2 scale) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float2* buf = wbuf + warp * kMaxBigBox;
    for (int line = warp; line < n; line += kBigThreads / 32) {
        float2* p = z + (size_t)line * lstride;
        for (int j = lane; j < n; j += 32) {
            const float2 v = p[(size_t)j * ls];
            buf[j] = make_float2(v.x * scale.x, v.y * scale.y);
        }
        __syncwarp();
        for (int k = lane; k < n; k += 32) {
            float sr = 0.f, si = 0.f;
            int idx = 0;  // (j k) mod n
            for (int j = 0; j < n; ++j) {
                float2 w = tw[idx];
                w.y = sign < 0 ? w.y : -w.y;  // tw holds e^{-2 pi i m / n}
                const float2 x = buf[j];
                sr = fmaf(x.x, w.x, fmaf(-x.y, w.y, sr));
                si = fmaf(x.x, w.y, fmaf(x.y, w.x, si));
                idx += k;
                idx = idx >= n ? idx - n : idx;
            }
            p[(size_t)k * ls] = make_float2(sr, si);
        }
        __syncwarp();
    }
}

}  // namespace

__global__ void __launch_bounds__(kBigThreads) k_window_big(BigArgs a) {
    const int n = a.n, H = n / 2;
    const int ld = n + 1;  // row stride of z, complex values
    extern __shared__ __align__(16) unsigned char sm[];
    float2* z = reinterpret_cast<float2*>(sm);                     // n x ld
    float2* tw = z + (size_t)n * ld;                               // n
    float2* wbuf = tw + kMaxBigBox;                                // 8 warps x kMaxBigBox
    float* s_g = reinterpret_cast<float*>(wbuf + 8 * kMaxBigBox);  // 2 n + 1
    float* s_f = s_g + 2 * kMaxBigBox + 4;                         // n
    float4* s_mean = reinterpret_cast<float4*>(s_f + kMaxBigBox);  // 16-byte aligned
    unsigned* s_max = reinterpret_cast<unsigned*>(s_mean + 1);
    unsigned long long* s_key = reinterpret_cast<unsigned long long*>(s_max + 4);
    int* s_item = reinterpret_cast<int*>(s_key + 1);  // gi, imin, jmin, gr offset, gc offset, ny
    const float4** s_src = reinterpret_cast<const float4**>(s_item + 8);

    const int t = threadIdx.x;
    for (int k = t; k < n; k += kBigThreads) {
        tw[k] = a.tw[k];
        s_f[k] = a.use_filter ? a.filt2[k] : 1.0f;
    }
    for (int k = t; k < 2 * n + 1; k += kBigThreads) s_g[k] = a.gauss[k];
    grid_dep_wait();
    const int nwork = *a.nwork;
    __syncthreads();

    for (int w = blockIdx.x; w < nwork; w += gridDim.x) {
        if (t == 0) {
            int gi = w;
            const float4* f12 = a.s12;
            int nx = a.nx, ny = a.ny;
            const float4* mp = a.means;
            MeanGrid mg = a.mg;
            if (a.nseg > 0) {
                const int k = seg_find(a.seg_start, a.nseg, gi);
                const WinSeg sg = a.segs[k];
                f12 = sg.s12;
                nx = sg.nx;
                ny = sg.ny;
                if (mp) mp += sg.base;
                mg = sg.mg;
                gi = sg.base + (gi - __ldg(a.seg_start + k));
            }
            const int pix = a.work[gi];
            int ic, jc, imin, jmin;
            if (a.direct) {
                imin = pix / ny;
                jmin = 0;
                ic = imin;
                jc = 0;
            } else {
                ic = pix / ny;
                jc = pix - ic * ny;
                imin = box_start(ic, nx, a.nsize);
                jmin = box_start(jc, ny, a.nsize);
            }
            s_item[0] = gi;
            s_item[1] = imin;
            s_item[2] = jmin;
            s_item[3] = imin - ic + n;
            s_item[4] = jmin - jc + n;
            s_item[5] = ny;
            s_src[0] = f12 + (size_t)imin * ny + jmin;
            *s_mean = (mp && !a.direct) ? mp[mean_slot(mg, ic, jc)] : make_float4(0.f, 0.f, 0.f, 0.f);
            s_max[0] = 0u;
            s_max[1] = 0u;
            *s_key = 0ull;
        }
        __syncthreads();
        const int gi = s_item[0];
        const int gro = s_item[3], gco = s_item[4], ny = s_item[5];
        const float4 mm = *s_mean;
        const float2 m1 = make_float2(mm.x, mm.z), m2 = make_float2(mm.y, mm.w);  // (hi, lo) per frame

        // windowed, mean-subtracted sub-images, z = g1 + i g2
        float mx1 = 0.f, mx2 = 0.f;
        for (int p = t; p < n * n; p += kBigThreads) {
            const int i = p / n, j = p - i * n;
            const float4 q = s_src[0][(size_t)i * ny + j];
            const float2 u = make_float2(q.x, q.z), v = make_float2(q.y, q.w);  // (hi, lo) per frame
            const float wgt = s_g[gco + j] * s_g[gro + i];
            const float2 zz = make_float2(wgt * ((u.x - m1.x) + (u.y - m1.y)), wgt * ((v.x - m2.x) + (v.y - m2.y)));
            z[(size_t)i * ld + j] = zz;
            mx1 = fmaxf(mx1, fabsf(zz.x));
            mx2 = fmaxf(mx2, fabsf(zz.y));
        }
        const unsigned b1 = __reduce_max_sync(0xffffffffu, __float_as_uint(mx1));
        const unsigned b2 = __reduce_max_sync(0xffffffffu, __float_as_uint(mx2));
        if ((t & 31) == 0) {
            atomicMax(s_max, b1);
            atomicMax(s_max + 1, b2);
        }
        __syncthreads();
        const float2 cs = make_float2(pow2_scale(s_max[0]), pow2_scale(s_max[1]));

        // forward 2-D DFT: rows (along j), then columns (along i)
        dft_lines(z, n, 1, ld, tw, wbuf, -1, cs);
        __syncthreads();
        dft_lines(z, n, ld, 1, tw, wbuf, -1, make_float2(1.f, 1.f));
        __syncthreads();

        // C = conj(A) B filt^2 with A, B separated from Z(k) and Z(-k):
        // A = (Z(k) + conj Z(-k)) / 2, B = (Z(k) - conj Z(-k)) / 2i.  C is
        // Hermitian (the spectrum of a real image), so one thread forms
        // C(k) and stores conj C(k) at -k (filt2 is even in k)
        for (int p = t; p < n * n; p += kBigThreads) {
            const int kx = p / n, ky = p - kx * n;
            const int mx = kx ? n - kx : 0, my = ky ? n - ky : 0;
            const int q = mx * n + my;
            if (q < p) continue;  // the pair is done from the other end
            const float2 Z = z[(size_t)kx * ld + ky];
            const float2 Zm = z[(size_t)mx * ld + my];
            const float2 A = make_float2(0.5f * (Z.x + Zm.x), 0.5f * (Z.y - Zm.y));
            const float2 B = make_float2(0.5f * (Z.y + Zm.y), 0.5f * (Zm.x - Z.x));
            const float f = s_f[kx] * s_f[ky];
            const float2 Cc = make_float2(f * (A.x * B.x + A.y * B.y), f * (A.x * B.y - A.y * B.x));
            z[(size_t)kx * ld + ky] = Cc;
            z[(size_t)mx * ld + my] = make_float2(Cc.x, -Cc.y);
        }
        __syncthreads();

        // inverse 2-D DFT: columns, then rows; c is real
        dft_lines(z, n, ld, 1, tw, wbuf, +1, make_float2(1.f, 1.f));
        __syncthreads();
        dft_lines(z, n, 1, ld, tw, wbuf, +1, make_float2(1.f, 1.f));
        __syncthreads();

        // first strict maximum of |c| in the half-shifted frame: the largest
        // (value, -index) key; NaN skipped (a NaN first element wins below)
        unsigned long long best = 0ull;
        for (int L = t; L < n * n; L += kBigThreads) {
            const int I = L / n, J = L - I * n;
            const int i = I + H < n ? I + H : I - H, j = J + H < n ? J + H : J - H;
            const float v = fabsf(z[(size_t)i * ld + j].x);
            if (!(v != v)) {
                const unsigned long long key =
                    ((unsigned long long)__float_as_uint(v) << 32) | (unsigned long long)(0xffffffffu - (unsigned)L);
                best = key > best ? key : best;
            }
        }
        best = warp_max_key(best);
        if ((t & 31) == 0) atomicMax(s_key, best);
        __syncthreads();
        int I, J;
        bool have;
        const float v0 = z[(size_t)H * ld + H].x;  // shifted (0, 0)
        if (v0 != v0) {
            I = 0;
            J = 0;
            have = true;
        } else {
            const unsigned long long key = *s_key;
            const unsigned L = 0xffffffffu - (unsigned)(key & 0xffffffffull);
            have = __uint_as_float((unsigned)(key >> 32)) != 0.0f;
            I = have ? (int)(L / n) : H;
            J = have ? (int)(L % n) : H;
        }
        auto shifted = [&](int r, int c) {
            const int i = r + H < n ? r + H : r - H, j = c + H < n ? c + H : c - H;
            return fabsf(z[(size_t)i * ld + j].x);
        };
        if (a.peaks_h) {
            if (t < kHiresPatch * kHiresPatch + 1) {
                float* rec = reinterpret_cast<float*>(a.peaks_h + gi);
                if (t < kHiresPatch * kHiresPatch) {
                    const int r = I - 2 + t / kHiresPatch, c = J - 2 + t % kHiresPatch;
                    rec[t] = (r >= 0 && r < n && c >= 0 && c < n) ? shifted(r, c) : 0.f;
                } else {
                    rec[t] = __uint_as_float(peak_meta(I, J, have));
                }
            }
        } else if (t < 10) {
            const bool dofit = have && I > 0 && I < n - 1 && J > 0 && J < n - 1;
            float* rec = reinterpret_cast<float*>(a.peaks + gi);
            if (t < 9)
                rec[t] = dofit ? shifted(I - 1 + t / 3, J - 1 + t % 3) : 0.f;
            else
                rec[9] = __uint_as_float(peak_meta(I, J, dofit));
        }
        __syncthreads();
    }
}

size_t window_big_smem(int n) {
    return (size_t)n * (n + 1) * sizeof(float2) + (size_t)kMaxBigBox * sizeof(float2) +
           (size_t)8 * kMaxBigBox * sizeof(float2) + (2 * kMaxBigBox + 4 + kMaxBigBox) * sizeof(float) + 256;
}

cudaError_t launch_window_big(const BigArgs& a, int grid, cudaStream_t st, bool pdl) {
    const size_t smem = window_big_smem(a.n);
    cudaError_t e = cudaFuncSetAttribute(k_window_big, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    return launch_kernel(k_window_big, dim3(grid), dim3(kBigThreads), smem, st, pdl, a);
}

int window_big_blocks_per_sm(int n) {
    const size_t smem = window_big_smem(n);
    int nb = 0;
    if (cudaFuncSetAttribute(k_window_big, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_window_big, kBigThreads, smem) != cudaSuccess) return 0;
    return nb;
}

}  // namespace flct
