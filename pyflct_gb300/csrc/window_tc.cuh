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
//       column kc = T[:,kc] (kc = 1..15); rows (window, kc), one N = 64 GEMM
//       per image into adjacent TMEM columns, K = (re/im, i) (64),
//       N = (re/im, kx) (64)                                        1 tile
//   product conj(A) B filt^2 per (kx, ky): one lane holds both images'
//       spectra of its (window, kc) row
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
#include "fft_reg.cuh"
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
    PeakRecH* peaks_h;    // -h patch records, else null
    const WinSeg* segs;   // batched launch (see WinArgs), else null
    const int* seg_start;
    int nseg;
    const float* b1;      // [c][j] 32 x 32: S1 matrix, row = output column c
    const float* b2;      // [n][k] 64 x 64: S2 matrix, n = (re/im, q), k = (re/im, i), kx = tc_kx(q)
    unsigned* status;
    // failure-path test hook: when nonzero, every stage waits this many ns
    // on a barrier that nothing completes (instead of the MMA barrier), so
    // that the wait runs out; the exit path still waits for the real MMAs
    unsigned long long stall_ns;
    float gauss[2 * kMaxBox + 1];
    float filt2[kMaxBox];
};

// Column order of S2's output (and S3's input): kx and -kx adjacent, so each
// half of a spectrum row holds complete mirror pairs:
//   q = 0 -> kx 0, q = 1 -> kx 16, q = 2j -> kx j, q = 2j+1 -> kx 32-j.
__host__ __device__ constexpr int tc_kx(int q) {
    return q == 0 ? 0 : (q == 1 ? 16 : ((q % 2 == 0) ? q / 2 : 32 - q / 2));
}
// Position of -kx for the column at position q.
__host__ __device__ constexpr int tc_mirror(int q) { return q < 2 ? q : ((q % 2 == 0) ? q + 1 : q - 1); }

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
    __device__ static __forceinline__ void pair(float v0, float v1, uint32_t& hi, uint32_t& lo) {
        const __half2 a = __floats2half2_rn(v0, v1);
        const float2 b = __half22float2(a);
        const __half2 c = __floats2half2_rn(v0 - b.x, v1 - b.y);
        hi = *reinterpret_cast<const uint32_t*>(&a);
        lo = *reinterpret_cast<const uint32_t*>(&c);
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
    __device__ static __forceinline__ void pair(float v0, float v1, uint32_t& hi, uint32_t& lo) {
        const __nv_bfloat162 a = __floats2bfloat162_rn(v0, v1);
        const float2 b = __bfloat1622float2(a);
        const __nv_bfloat162 c = __floats2bfloat162_rn(v0 - b.x, v1 - b.y);
        hi = *reinterpret_cast<const uint32_t*>(&a);
        lo = *reinterpret_cast<const uint32_t*>(&c);
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
    // + 1024 for aligning the base
    static constexpr int bytes = off_misc + misc + 1024;
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
    uint64_t* s_never = reinterpret_cast<uint64_t*>(sm + TcSmem::off_misc + 696);  // test hook only
    int* s_gi = reinterpret_cast<int*>(sm + TcSmem::off_misc + 656);                    // 8
    const float2** s_src = reinterpret_cast<const float2**>(sm + TcSmem::off_misc + 704);  // 8 x 2
    int2* s_dim = reinterpret_cast<int2*>(sm + TcSmem::off_misc + 832);                 // 8

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
    if (t == 0) {
        tc::mbar_init(s_mbar, 1);
        tc::mbar_init(s_never, 1);
    }
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
        const bool done =
            a.stall_ns ? tc::mbar_wait(s_never, 0u, a.stall_ns) : tc::mbar_wait(s_mbar, phase, kLimit);
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
            int w = min(base + t, nwork - 1);
            const float2* f1s = a.s1;
            const float2* f2s = a.s2;
            int2 dim = make_int2(a.nx, a.ny);
            if (a.nseg > 0) {
                const int k = seg_find(a.seg_start, a.nseg, w);
                const WinSeg sg = a.segs[k];
                f1s = sg.s1;
                f2s = sg.s2;
                dim = make_int2(sg.nx, sg.ny);
                w = sg.base + (w - __ldg(a.seg_start + k));
            }
            s_gi[t] = w;
            s_src[2 * t] = f1s;
            s_src[2 * t + 1] = f2s;
            s_dim[t] = dim;
            s_pix[t] = a.work[w];
            s_mean[t] = a.means ? a.means[w] : make_float4(0.f, 0.f, 0.f, 0.f);
        }
        __syncthreads();

        // ---- phase 0: windows -> A1 (K-major, 4 tiles of 128 rows) -------
        {
            // warp (wl, img) of each tile; lane = column j, rows read
            // cooperatively (coalesced), values scattered into the K-major rows
            const int wl = warp >> 1, img = warp & 1;
#pragma unroll 1
            for (int tile = 0; tile < 4; ++tile) {
                const int w = 2 * tile + wl;
                const int pix = s_pix[w];
                const int2 dim = s_dim[w];
                int ic, jc, imin, jmin;
                if (a.direct) {
                    imin = pix / dim.y;
                    jmin = 0;
                    ic = imin;
                    jc = 0;
                } else {
                    ic = pix / dim.y;
                    jc = pix - ic * dim.y;
                    imin = box_start(ic, dim.x, a.nsize);
                    jmin = box_start(jc, dim.y, a.nsize);
                }
                const float4 mm = s_mean[w];
                const float mh = img ? mm.z : mm.x, ml = img ? mm.w : mm.y;
                const float2* src = s_src[2 * w + img] + (size_t)imin * dim.y + jmin + lane;
                const float* gr = s_g + (imin - ic + N);
                const float gc = s_g[lane + jmin - jc + N];
                float x[32];
                float mx = 0.f;
#pragma unroll
                for (int i = 0; i < 32; ++i) {
                    const float2 u = __ldg(src + (size_t)i * dim.y);
                    x[i] = ((u.x - mh) + (u.y - ml)) * (gr[i] * gc);
                    mx = fmaxf(mx, fabsf(x[i]));
                }
                const float sc = pow2_scale(__float_as_uint(warp_max(mx)));
                // even lanes store (j, j+1) as one 32-bit hi and one lo word
                const int rowbase = tile * 8192 + (wl * 64 + img * 32) / 8 * 512 + (lane % 8) * 2 + (lane / 8) * 128;
#pragma unroll
                for (int i = 0; i < 32; ++i) {
                    const float v = x[i] * sc;
                    const float vn = __shfl_down_sync(0xffffffffu, v, 1);
                    if ((lane & 1) == 0) {
                        uint32_t hi, lo;
                        SP::pair(v, vn, hi, lo);
                        const int off = rowbase + (i % 8) * 16 + (i / 8) * 512;
                        *reinterpret_cast<uint32_t*>(Ahi + off) = hi;
                        *reinterpret_cast<uint32_t*>(Alo + off) = lo;
                    }
                }
            }
        }
        to_mma();
        if (t == 0) {
            // consecutive MMAs go to different accumulators (tiles) so that
            // the tensor pipe can overlap them
            for (int s = 0; s < 2; ++s)
                for (int tile = 0; tile < 4; ++tile)
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
                // rows m = w*16 + kc (two m-cores), K block of this image
                const int base2 = img * 16384 + (2 * w) * 128 + (i % 8) * 16;
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
            for (int s = 0; s < 4; ++s)
                for (int img = 0; img < 2; ++img)
                    mma3(tmem + 128 + 64 * img, tc::desc(ahi + img * 16384 + s * 4096, 2048, 128),
                         tc::desc(alo + img * 16384 + s * 4096, 2048, 128), tc::desc(b2hi + s * 256, 128, 1024),
                         tc::desc(b2lo + s * 256, 128, 1024), id2, s > 0);
            tc::commit(s_mbar);
        }
        if (!wait_stage()) {
            ok = false;
            break;
        }

        // ---- phase 2: spectra -> conj(A) B filt^2 -> A3 (K-major) --------
        {
            // row t = (window w, packed column kc); both images in one lane
            const int kc = t & 15;
            const float h0 = kc ? 1.0f : 0.5f, z6 = kc ? 0.0f : 0.5f;
            const float fk0 = kc ? s_f[kc] : s_f[0], fk6 = s_f[H];
            float ur[32], ui[32];
            float mx = 0.f;
            sfor<0, 2>([&](auto hc) {
                constexpr int half = decltype(hc)::value;
                // columns q in [16 half, 16 half + 16): complete (kx, -kx) pairs
                float ar[16], ai[16], br[16], bi[16];
                tc::tmem_ld16(tmem + lane_base + 128 + 16 * half, ar);
                tc::tmem_ld16(tmem + lane_base + 160 + 16 * half, ai);
                tc::tmem_ld16(tmem + lane_base + 192 + 16 * half, br);
                tc::tmem_ld16(tmem + lane_base + 224 + 16 * half, bi);
                sfor<0, 16>([&](auto qc) {
                    constexpr int qq = decltype(qc)::value;
                    constexpr int q = 16 * half + qq;
                    constexpr int mq = tc_mirror(q) - 16 * half;  // mirror within this half
                    const float Ar = ar[qq], Ai = ai[qq], Br = br[qq], Bi = bi[qq];
                    const float sr = kc ? 0.0f : ar[mq], si = kc ? 0.0f : ai[mq];
                    const float tr = kc ? 0.0f : br[mq], ti = kc ? 0.0f : bi[mq];
                    const float a0r = h0 * (Ar + sr), a0i = h0 * (Ai - si);
                    const float a6r = z6 * (Ai + si), a6i = z6 * (sr - Ar);
                    const float b0r = h0 * (Br + tr), b0i = h0 * (Bi - ti);
                    const float b6r = z6 * (Bi + ti), b6i = z6 * (tr - Br);
                    const float fx = s_f[tc_kx(q)];
                    const float f0 = fx * fk0, f6 = fx * fk6;
                    const float c0r = f0 * (a0r * b0r + a0i * b0i), c0i = f0 * (a0r * b0i - a0i * b0r);
                    const float c6r = f6 * (a6r * b6r + a6i * b6i), c6i = f6 * (a6r * b6i - a6i * b6r);
                    ur[q] = c0r - c6i;  // u = C0 + i C16 (C16 = 0 for kc > 0)
                    ui[q] = c0i + c6r;
                    mx = fmaxf(mx, fmaxf(fabsf(ur[q]), fabsf(ui[q])));
                });
            });
#pragma unroll
            for (int o = 8; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
            const float sc = pow2_scale(__float_as_uint(mx));
#pragma unroll
            for (int q = 0; q < 32; ++q) {
                ur[q] *= sc;
                ui[q] *= sc;
            }
            const int rowoff = (t % 8) * 16 + (t / 8) * 1024;
#pragma unroll
            for (int part = 0; part < 2; ++part) {
                const float* src = part ? ui : ur;
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    uint4 hi, lo;
                    SP::run(src + 8 * c, hi, lo);
                    const int kcore = part * 4 + c;
                    *reinterpret_cast<uint4*>(Ahi + rowoff + kcore * 128) = hi;
                    *reinterpret_cast<uint4*>(Alo + rowoff + kcore * 128) = lo;
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
            for (int s = 0; s < 2; ++s)
                for (int t4 = 0; t4 < 2; ++t4)
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
                if (valid && a.peaks_h) {
                    // -h: the 6x6 patch around the peak, 37 words
                    float* rec = reinterpret_cast<float*>(a.peaks_h + s_gi[wg]);
                    for (int k = lane; k < kHiresPatch * kHiresPatch + 1; k += 32) {
                        if (k < kHiresPatch * kHiresPatch) {
                            const int r = Ip - 2 + k / kHiresPatch, cc = Jp - 2 + k % kHiresPatch;
                            rec[k] = (r >= 0 && r < N && cc >= 0 && cc < N) ? stage[r * 33 + cc] : 0.f;
                        } else {
                            rec[k] = __uint_as_float(peak_meta(Ip, Jp, have));
                        }
                    }
                } else if (valid && lane < 10) {
                    float* rec = reinterpret_cast<float*>(a.peaks + s_gi[wg]);
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
