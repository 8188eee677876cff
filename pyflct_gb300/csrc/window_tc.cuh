// window_tc.cuh -- the tensor-core window-correlation kernel (DFT-matrix
// form, split precision) for 32 x 32 boxes.
//
// Same contract as k_window_fp32 (source/flct.c:829-876, 1325-1532: window,
// transforms, conj product with the optional filter, inverse, |c| in the
// half-shifted frame, first strict maximum), but every transform is a dense
// DFT-matrix product on tcgen05 tensor cores.  Operands are split into a
// 16-bit high part and a 16-bit remainder (FP16 or BF16); each product is
// hi*hi + hi*lo + lo*hi accumulated in FP32 in tensor memory, which keeps
// ~21 significant bits (FP16) of each 16-bit-by-16-bit product.
//
// Eight windows per CTA iteration, 128 threads (4 warps), four GEMM stages,
// each M = 128 (rows of data), B = a constant DFT matrix in shared memory:
//   S1  along j, real input -> half spectrum T[i][c]:
//       c = 0..16 real parts (ky = c), c = 17..31 imaginary parts (ky = c-16)
//       rows (window, image, i), K = j (32), N = c (32)            4 tiles
//   S2  along i on 16 packed complex columns per image:
//       column 0 = T[:,0] + i T[:,16] (separated later by Hermitian symmetry),
//       column kc = T[:,kc] (kc = 1..15); rows (window, image, kc),
//       K = (re/im, i) (64), N = (re/im, kx) (64)                   2 tiles
//   product conj(A) B filt^2 per (kx, ky), images exchanged between lanes
//   S3  inverse along kx on 16 packed columns per window (ky = 0 and 16
//       share column 0: both inverse transforms are real),
//       rows (window, kc), K = (re/im, kx), N = (re/im, i)          1 tile
//   S4  complex-to-real along ky: rows (window, i), K = 32 spectral terms
//       (weights 1 or 2 folded into the data), N = j               2 tiles
// S3 reuses S2's matrix and S4 reuses S1's, transposed through the
// descriptors' MN-major mode.  The transposes between stages are free: each
// thread writes its TMEM row straight into the next stage's operand layout
// (MN-major where the contraction index changes).
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "common.cuh"
#include "tc_ptx.cuh"
#include "window_common.cuh"

namespace flct {

struct TcArgs {
    const float2* s1;
    const float2* s2;
    const float4* means;  // per work item, or null (direct windows)
    const int* work;
    const int* nwork;
    int nx, ny, nsize;
    int direct;
    int use_filter;
    PeakRec* peaks;
    const float* b1;      // [c][j] 32 x 32: S1 matrix, row = output column c
    const float* b2;      // [n][k] 64 x 64: S2 matrix, n = (re/im, kx), k = (re/im, i)
    unsigned* status;
    float gauss[2 * kMaxBox + 1];
    float filt2[kMaxBox];
};

template <typename T>
struct Split16;
template <>
struct Split16<__half> {
    static constexpr int fmt = 0;
    // 8 floats -> 8 hi and 8 lo halves packed in uint4
    __device__ static __forceinline__ void run(const float* v, uint4& hi, uint4& lo) {
        uint32_t h[4], l[4];
#pragma unroll
        for (int p = 0; p < 4; ++p) {
            const __half2 a = __floats2half2_rn(v[2 * p], v[2 * p + 1]);
            const float2 b = __half22float2(a);
            const __half2 c = __floats2half2_rn(v[2 * p] - b.x, v[2 * p + 1] - b.y);
            h[p] = *reinterpret_cast<const uint32_t*>(&a);
            l[p] = *reinterpret_cast<const uint32_t*>(&c);
        }
        hi = make_uint4(h[0], h[1], h[2], h[3]);
        lo = make_uint4(l[0], l[1], l[2], l[3]);
    }
};
template <>
struct Split16<__nv_bfloat16> {
    static constexpr int fmt = 1;
    __device__ static __forceinline__ void run(const float* v, uint4& hi, uint4& lo) {
        uint32_t h[4], l[4];
#pragma unroll
        for (int p = 0; p < 4; ++p) {
            const __nv_bfloat162 a = __floats2bfloat162_rn(v[2 * p], v[2 * p + 1]);
            const float2 b = __bfloat1622float2(a);
            const __nv_bfloat162 c = __floats2bfloat162_rn(v[2 * p] - b.x, v[2 * p + 1] - b.y);
            h[p] = *reinterpret_cast<const uint32_t*>(&a);
            l[p] = *reinterpret_cast<const uint32_t*>(&c);
        }
        hi = make_uint4(h[0], h[1], h[2], h[3]);
        lo = make_uint4(l[0], l[1], l[2], l[3]);
    }
};

struct TcSmem {
    static constexpr int A = 32768;            // per hi / lo
    static constexpr int B1 = 2048;            // 32 x 32 x 2 B
    static constexpr int B2 = 8192;            // 64 x 64 x 2 B
    static constexpr int off_ahi = 0;
    static constexpr int off_alo = A;
    static constexpr int off_b1hi = 2 * A;
    static constexpr int off_b1lo = off_b1hi + B1;
    static constexpr int off_b2hi = off_b1lo + B1;
    static constexpr int off_b2lo = off_b2hi + B2;
    static constexpr int off_misc = off_b2lo + B2;  // 86016
    static constexpr int misc = 1024;
    // + 1024 for aligning the base; + 16 KB so that descriptor reads stay
    // inside the allocation under any stride interpretation
    static constexpr int bytes = off_misc + misc + 1024 + 16384;
};

__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

__device__ __forceinline__ unsigned long long warp_max_key(unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
        v = w > v ? w : v;
    }
    return v;
}

template <typename T>
__global__ void __launch_bounds__(128) k_window_tc32(TcArgs a) {
    constexpr int N = 32, H = 16, WIT = 8;
    constexpr uint64_t kLimit = 2000000000ull;  // 2 s per wait
    using SP = Split16<T>;
    extern __shared__ unsigned char sm_raw[];
    // 1024-byte aligned base for the operand buffers
    unsigned char* sm = reinterpret_cast<unsigned char*>(
        (reinterpret_cast<uintptr_t>(sm_raw) + 1023) & ~static_cast<uintptr_t>(1023));
    unsigned char* Ahi = sm + TcSmem::off_ahi;
    unsigned char* Alo = sm + TcSmem::off_alo;
    unsigned char* B1hi = sm + TcSmem::off_b1hi;
    unsigned char* B1lo = sm + TcSmem::off_b1lo;
    unsigned char* B2hi = sm + TcSmem::off_b2hi;
    unsigned char* B2lo = sm + TcSmem::off_b2lo;
    float* s_g = reinterpret_cast<float*>(sm + TcSmem::off_misc);  // 65 (+pad)
    float* s_f = s_g + 80;                                         // 32
    int* s_pix = reinterpret_cast<int*>(s_f + 32);                 // 8
    float4* s_mean = reinterpret_cast<float4*>(sm + TcSmem::off_misc + 512);  // 8
    uint64_t* s_mbar = reinterpret_cast<uint64_t*>(sm + TcSmem::off_misc + 640);
    uint32_t* s_tmem = reinterpret_cast<uint32_t*>(sm + TcSmem::off_misc + 648);

    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;

    // ---- constant DFT matrices, split, K-major (n, k) layout --------------
    for (int e = t; e < 32 * 32 / 8; e += 128) {  // B1: n = c, k = j; 8 k per store
        const int n = e / 4, kc = e % 4;
        float v[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) v[q] = a.b1[n * 32 + kc * 8 + q];
        uint4 hi, lo;
        SP::run(v, hi, lo);
        const int off = (n % 8) * 16 + (n / 8) * 512 + kc * 128;
        *reinterpret_cast<uint4*>(B1hi + off) = hi;
        *reinterpret_cast<uint4*>(B1lo + off) = lo;
    }
    for (int e = t; e < 64 * 64 / 8; e += 128) {  // B2: n = (p', kx), k = (p, i)
        const int n = e / 8, kc = e % 8;
        float v[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) v[q] = a.b2[n * 64 + kc * 8 + q];
        uint4 hi, lo;
        SP::run(v, hi, lo);
        const int off = (n % 8) * 16 + (n / 8) * 1024 + kc * 128;
        *reinterpret_cast<uint4*>(B2hi + off) = hi;
        *reinterpret_cast<uint4*>(B2lo + off) = lo;
    }
    for (int k = t; k < 2 * N + 1; k += 128) s_g[k] = a.gauss[k];
    for (int k = t; k < N; k += 128) s_f[k] = a.use_filter ? a.filt2[k] : 1.0f;
    if (warp == 0) tc::tmem_alloc(s_tmem, 256);
    if (t == 0) tc::mbar_init(s_mbar, 1);
    tc::fence_async_smem();
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = *s_tmem;
    const uint32_t lane_base = (uint32_t)(warp * 32) << 16;

    constexpr uint32_t id1 = tc::idesc(SP::fmt, 128, 32, false, false);
    constexpr uint32_t id2 = tc::idesc(SP::fmt, 128, 64, true, false);
    constexpr uint32_t id3 = tc::idesc(SP::fmt, 128, 64, false, true);
    constexpr uint32_t id4 = tc::idesc(SP::fmt, 128, 32, true, true);
    const uint32_t ahi = tc::smem_u32(Ahi), alo = tc::smem_u32(Alo);
    const uint32_t b1hi = tc::smem_u32(B1hi), b1lo = tc::smem_u32(B1lo);
    const uint32_t b2hi = tc::smem_u32(B2hi), b2lo = tc::smem_u32(B2lo);

    const int nwork = *a.nwork;
    uint32_t phase = 0;
    bool ok = true;

    // issue hi*hi + hi*lo + lo*hi for one K step of 16
    auto mma3 = [&](uint32_t d, uint64_t ah, uint64_t al, uint64_t bh, uint64_t bl, uint32_t id, uint32_t acc) {
        tc::mma(d, ah, bh, id, acc);
        tc::mma(d, ah, bl, id, 1u);
        tc::mma(d, al, bh, id, 1u);
    };
    // all threads: wait for the stage's MMAs; any timeout stops the kernel
    auto wait_stage = [&]() -> bool {
        const bool done = tc::mbar_wait(s_mbar, phase, kLimit);
        phase ^= 1u;
        tc::fence_after();
        return __syncthreads_and(done ? 1 : 0) != 0;
    };
    auto to_mma = [&]() {
        tc::fence_async_smem();
        tc::fence_before();
        __syncthreads();
        tc::fence_after();
    };

    for (int base = blockIdx.x * WIT; base < nwork && ok; base += gridDim.x * WIT) {
        if (t < WIT) {
            const int w = min(base + t, nwork - 1);
            s_pix[t] = a.work[w];
            s_mean[t] = a.means ? a.means[w] : make_float4(0.f, 0.f, 0.f, 0.f);
        }
        __syncthreads();

        // ---- phase 0: windows -> A1 (K-major, 4 tiles of 128 rows) -------
        {
            const int wl = t >> 6, img = (t >> 5) & 1, i = t & 31;
#pragma unroll 1
            for (int tile = 0; tile < 4; ++tile) {
                const int w = 2 * tile + wl;
                const int pix = s_pix[w];
                int ic, jc, imin, jmin;
                if (a.direct) {
                    imin = pix / a.ny;
                    jmin = 0;
                    ic = imin;
                    jc = 0;
                } else {
                    ic = pix / a.ny;
                    jc = pix - ic * a.ny;
                    imin = box_start(ic, a.nx, a.nsize);
                    jmin = box_start(jc, a.ny, a.nsize);
                }
                const float4 mm = s_mean[w];
                const float mh = img ? mm.z : mm.x, ml = img ? mm.w : mm.y;
                const float2* src = (img ? a.s2 : a.s1) + (size_t)(imin + i) * a.ny + jmin;
                const float gr = s_g[i + imin - ic + N];
                const float* gc = s_g + (jmin - jc + N);
                float x[32];
                float mx = 0.f;
#pragma unroll
                for (int j = 0; j < 32; ++j) {
                    const float2 u = __ldg(src + j);
                    x[j] = ((u.x - mh) + (u.y - ml)) * (gr * gc[j]);
                    mx = fmaxf(mx, fabsf(x[j]));
                }
                const float sc = pow2_scale(__float_as_uint(warp_max(mx)));
#pragma unroll
                for (int j = 0; j < 32; ++j) x[j] *= sc;
                const int rowoff = tile * 8192 + (t % 8) * 16 + (t / 8) * 512;
#pragma unroll
                for (int kc = 0; kc < 4; ++kc) {
                    uint4 hi, lo;
                    SP::run(x + 8 * kc, hi, lo);
                    *reinterpret_cast<uint4*>(Ahi + rowoff + kc * 128) = hi;
                    *reinterpret_cast<uint4*>(Alo + rowoff + kc * 128) = lo;
                }
            }
        }
        to_mma();
        if (t == 0) {
            for (int tile = 0; tile < 4; ++tile)
                for (int s = 0; s < 2; ++s)
                    mma3(tmem + 32 * tile, tc::desc(ahi + tile * 8192 + s * 256, 128, 512),
                         tc::desc(alo + tile * 8192 + s * 256, 128, 512), tc::desc(b1hi + s * 256, 128, 512),
                         tc::desc(b1lo + s * 256, 128, 512), id1, s > 0);
            tc::commit(s_mbar);
        }
        if (!wait_stage()) {
            ok = false;
            break;
        }

        // ---- phase 1: D1 rows -> A2 (MN-major, 2 tiles) ---------------------
        {
            const int wl = t >> 6, img = (t >> 5) & 1, i = t & 31;
#pragma unroll 1
            for (int tile = 0; tile < 4; ++tile) {
                float d[32];
                tc::tmem_ld32(tmem + lane_base + 32 * tile, d);
                const int w = 2 * tile + wl;
                const int t2 = w >> 2, wl2 = w & 3;
                const int mcore = (wl2 * 32 + img * 16) / 8;  // first of two m-cores
                const int base2 = t2 * 16384 + mcore * 128 + (i % 8) * 16;
#pragma unroll
                for (int part = 0; part < 2; ++part) {
                    const int off = base2 + (part * 4 + i / 8) * 2048;
                    uint4 hi, lo;
                    SP::run(d + 16 * part, hi, lo);
                    *reinterpret_cast<uint4*>(Ahi + off) = hi;
                    *reinterpret_cast<uint4*>(Alo + off) = lo;
                    SP::run(d + 16 * part + 8, hi, lo);
                    *reinterpret_cast<uint4*>(Ahi + off + 128) = hi;
                    *reinterpret_cast<uint4*>(Alo + off + 128) = lo;
                }
            }
        }
        tc::fence_before();
        to_mma();
        if (t == 0) {
            for (int t2 = 0; t2 < 2; ++t2)
                for (int s = 0; s < 4; ++s)
                    mma3(tmem + 128 + 64 * t2, tc::desc(ahi + t2 * 16384 + s * 4096, 2048, 128),
                         tc::desc(alo + t2 * 16384 + s * 4096, 2048, 128), tc::desc(b2hi + s * 256, 128, 1024),
                         tc::desc(b2lo + s * 256, 128, 1024), id2, s > 0);
            tc::commit(s_mbar);
        }
        if (!wait_stage()) {
            ok = false;
            break;
        }

        // ---- phase 2: spectra -> conj(A) B filt^2 -> A3 (K-major) --------
        {
            const int img = lane >> 4, kc = lane & 15;
#pragma unroll 1
            for (int t2 = 0; t2 < 2; ++t2) {
                float zr[32], zi[32];
                tc::tmem_ld32(tmem + lane_base + 128 + 64 * t2, zr);
                tc::tmem_ld32(tmem + lane_base + 128 + 64 * t2 + 32, zi);
                float pr[32], pi[32];
#pragma unroll
                for (int k = 0; k < 32; ++k) {
                    pr[k] = __shfl_xor_sync(0xffffffffu, zr[k], 16);
                    pi[k] = __shfl_xor_sync(0xffffffffu, zi[k], 16);
                }
                // A = image 1 spectrum, B = image 2; this lane handles kx in
                // [16 img, 16 img + 16) (static register indices via selects)
                float ur[16], ui[16];
                const float fk = s_f[kc];
#pragma unroll
                for (int q = 0; q < 16; ++q) {
                    const int k0 = q, k1 = q + 16;               // kx for img 0 / img 1
                    const int m0 = (32 - k0) & 31, m1 = (32 - k1) & 31;  // -kx
                    const float ar = img ? pr[k1] : zr[k0], ai = img ? pi[k1] : zi[k0];
                    const float br = img ? zr[k1] : pr[k0], bi = img ? zi[k1] : pi[k0];
                    const int kx = img ? k1 : k0;
                    const float fx = s_f[kx];
                    if (kc != 0) {
                        const float f = fx * fk;
                        ur[q] = f * (ar * br + ai * bi);
                        ui[q] = f * (ar * bi - ai * br);
                    } else {
                        // column 0 carries ky = 0 (real part) and ky = 16 (imag
                        // part): P = Y0 + i Y16 with Y0, Y16 Hermitian in kx
                        const float amr = img ? pr[m1] : zr[m0], ami = img ? pi[m1] : zi[m0];
                        const float bmr = img ? zr[m1] : pr[m0], bmi = img ? zi[m1] : pi[m0];
                        // Y0 = (P + conj(P-))/2, Y16 = (P - conj(P-))/(2i)
                        const float a0r = 0.5f * (ar + amr), a0i = 0.5f * (ai - ami);
                        const float a6r = 0.5f * (ai + ami), a6i = -0.5f * (ar - amr);
                        const float b0r = 0.5f * (br + bmr), b0i = 0.5f * (bi - bmi);
                        const float b6r = 0.5f * (bi + bmi), b6i = -0.5f * (br - bmr);
                        const float f0 = fx * s_f[0], f6 = fx * s_f[H];
                        const float c0r = f0 * (a0r * b0r + a0i * b0i), c0i = f0 * (a0r * b0i - a0i * b0r);
                        const float c6r = f6 * (a6r * b6r + a6i * b6i), c6i = f6 * (a6r * b6i - a6i * b6r);
                        // pack u = C0 + i C16 (both inverse transforms are real)
                        ur[q] = c0r - c6i;
                        ui[q] = c0i + c6r;
                    }
                }
                float mx = 0.f;
#pragma unroll
                for (int q = 0; q < 16; ++q) mx = fmaxf(mx, fmaxf(fabsf(ur[q]), fabsf(ui[q])));
                const float sc = pow2_scale(__float_as_uint(warp_max(mx)));
#pragma unroll
                for (int q = 0; q < 16; ++q) {
                    ur[q] *= sc;
                    ui[q] *= sc;
                }
                const int wg = 4 * t2 + warp;
                const int r3 = wg * 16 + kc;
                const int rowoff = (r3 % 8) * 16 + (r3 / 8) * 1024;
#pragma unroll
                for (int part = 0; part < 2; ++part) {
                    const float* src = part ? ui : ur;
#pragma unroll
                    for (int c = 0; c < 2; ++c) {
                        const int k = part * 32 + img * 16 + 8 * c;
                        uint4 hi, lo;
                        SP::run(src + 8 * c, hi, lo);
                        *reinterpret_cast<uint4*>(Ahi + rowoff + (k / 8) * 128) = hi;
                        *reinterpret_cast<uint4*>(Alo + rowoff + (k / 8) * 128) = lo;
                    }
                }
            }
        }
        tc::fence_before();
        to_mma();
        if (t == 0) {
            for (int s = 0; s < 4; ++s)
                mma3(tmem, tc::desc(ahi + s * 256, 128, 1024), tc::desc(alo + s * 256, 128, 1024),
                     tc::desc(b2hi + s * 2048, 1024, 128), tc::desc(b2lo + s * 2048, 1024, 128), id3, s > 0);
            tc::commit(s_mbar);
        }
        if (!wait_stage()) {
            ok = false;
            break;
        }

        // ---- phase 3: D3 rows -> A4 (MN-major, 2 tiles) ---------------------
        {
            const int wg = t >> 4, kc = t & 15;
            float ur[32], ui[32];
            tc::tmem_ld32(tmem + lane_base, ur);
            tc::tmem_ld32(tmem + lane_base + 32, ui);
            const float wgt = kc ? 2.0f : 1.0f;  // c2r weights of ky = 1..15
#pragma unroll
            for (int q = 0; q < 32; ++q) {
                ur[q] *= wgt;
                ui[q] *= wgt;
            }
            const int t4 = wg >> 2, wl4 = wg & 3;
#pragma unroll
            for (int part = 0; part < 2; ++part) {
                const int k = part * 16 + kc;
                const float* src = part ? ui : ur;
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    const int off = t4 * 8192 + (wl4 * 4 + c) * 128 + (k % 8) * 16 + (k / 8) * 2048;
                    uint4 hi, lo;
                    SP::run(src + 8 * c, hi, lo);
                    *reinterpret_cast<uint4*>(Ahi + off) = hi;
                    *reinterpret_cast<uint4*>(Alo + off) = lo;
                }
            }
        }
        tc::fence_before();
        to_mma();
        if (t == 0) {
            for (int t4 = 0; t4 < 2; ++t4)
                for (int s = 0; s < 2; ++s)
                    mma3(tmem + 128 + 32 * t4, tc::desc(ahi + t4 * 8192 + s * 4096, 2048, 128),
                         tc::desc(alo + t4 * 8192 + s * 4096, 2048, 128), tc::desc(b1hi + s * 1024, 512, 128),
                         tc::desc(b1lo + s * 1024, 512, 128), id4, s > 0);
            tc::commit(s_mbar);
        }
        if (!wait_stage()) {
            ok = false;
            break;
        }

        // ---- phase 4: |c|, first strict maximum, peak record -----------------
        {
            float* stage = reinterpret_cast<float*>(Ahi) + warp * 32 * 33;  // 32 x 32 per warp, row stride 33
#pragma unroll 1
            for (int t4 = 0; t4 < 2; ++t4) {
                float c[32];
                tc::tmem_ld32(tmem + lane_base + 128 + 32 * t4, c);
                const int i = lane;
                const int I = (i + H) & 31;
                unsigned long long best = 0ull;
#pragma unroll
                for (int j = 0; j < 32; ++j) {
                    const int J = (j + H) & 31;
                    const float v = fabsf(c[j]);
                    stage[I * 33 + J] = v;
                    if (!(v != v)) {
                        const unsigned long long key = ((unsigned long long)__float_as_uint(v) << 32) |
                                                       (unsigned long long)(0xffffffffu - (unsigned)(I * 32 + J));
                        best = key > best ? key : best;
                    }
                }
                best = warp_max_key(best);
                __syncwarp();
                const int wg = 4 * t4 + warp;
                const bool valid = base + wg < nwork;
                int Ip, Jp;
                bool have;
                const float v0 = stage[0];
                if (v0 != v0) {
                    Ip = 0;
                    Jp = 0;
                    have = true;
                } else {
                    const unsigned L = 0xffffffffu - (unsigned)(best & 0xffffffffull);
                    have = __uint_as_float((unsigned)(best >> 32)) != 0.0f;
                    Ip = have ? (int)(L / 32) : H;
                    Jp = have ? (int)(L % 32) : H;
                }
                const bool dofit = have && Ip > 0 && Ip < N - 1 && Jp > 0 && Jp < N - 1;
                if (valid && lane < 10) {
                    float* rec = reinterpret_cast<float*>(a.peaks + base + wg);
                    if (lane < 9)
                        rec[lane] = dofit ? stage[(Ip - 1 + lane / 3) * 33 + (Jp - 1 + lane % 3)] : 0.f;
                    else
                        rec[9] = __uint_as_float(peak_meta(Ip, Jp, dofit));
                }
                __syncwarp();
            }
        }
        tc::fence_before();
        __syncthreads();
        tc::fence_after();
    }

    if (!ok) {
        if (t == 0) atomicOr(a.status, kStatusTimeout);
        // let any MMA still in flight finish (bounded) before freeing TMEM
        tc::mbar_wait(s_mbar, phase ^ 1u, kLimit);
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    if (warp == 0) tc::tmem_dealloc(tmem, 256);
}

template <typename T>
cudaError_t launch_window_tc32(const TcArgs& a, int grid, cudaStream_t st);
template <typename T>
int window_tc32_blocks_per_sm();

}  // namespace flct
