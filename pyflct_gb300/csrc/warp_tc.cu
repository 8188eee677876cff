// warp_tc.cu -- warp_frac2d's spectral sum on the tcgen05 tensor cores.
//
// The reference evaluates, for every pixel p (source/warp.c:940-1000),
//   out[p] = (1/N) sum_{ii,jj} Re(F[ii][jj] exp(2 pi i (kx_ii tx_p + ky_jj ty_p)))
// with F the DFT of the image and tx, ty the pixel's position minus its
// shift in turns of each axis.
//
// Half spectrum.  The image is real, so F[-ii][-jj] = conj(F[ii][jj]) and
// the terms (ii, jj) and (-ii, -jj) have equal real parts whenever
// kx_{-ii} = -kx_ii and ky_{-jj} = -ky_jj.  The sum therefore runs over the
// columns jj = 0 .. ny/2 only: columns 0 and ny/2 (even ny; their partner
// column is themselves) with weight 1, the others with weight 2.  The one
// exception is the Nyquist row ii = nx/2 of an even nx, whose kx is its own
// partner: there the pair gives 2 cos(kx tx) Re(F ey) instead, so that row
// keeps weight 1 in every column and the epilogue forms
//   Re(ex A0) + 2 cos(kx tx) (Re G - Re A0),  A0 = F[N][0] + F[N][ny/2] ey_{ny/2}.
//
// GEMM.  For a tile of 128 pixels, G[p][ii] = sum_jj H[ii][jj] ey_jj(p) is a
// complex product, written as a real one with K = (re, im) of 16 columns per
// stage and N = (Re G, Im G) of 128 rows per chunk:
//   A[p][k]  = (Re ey_c, Im ey_c)                       generated per stage
//   B[n][k]  = (Re H, -Im H) for Re G rows, (Im H, Re H) for Im G rows
// then out[p] += sum_ii Re(ex_ii(p) G[p][ii]) in the epilogue.  Both
// operands are split into an FP16 high part and an FP16 remainder and each
// product is hi*hi + hi*lo + lo*hi in FP32 (tensor memory): ~22 significant
// bits per product.  H is scaled by a power of two so that its largest
// |value| sits below 2^14 (FP16 holds it); the epilogue divides it out.
// The tensor cores' FP32 accumulation truncates every partial sum, so the
// order is chosen to keep large partial sums out of most of the chain: the
// stages of a chunk run from the highest columns down, each K step adds the
// two cross products before hi*hi, and the DC term F[0][0] (the largest)
// bypasses the GEMM and is added in FP64; the epilogue sums each 8-row
// group in FP32 and the groups in FP64.
//
// CTA: 256 pixels (two 128-lane accumulators of 256 columns each, all 512
// TMEM columns), 17 warps: warps 0-15 generate the A stages (two threads
// per pixel, 8 columns each: exp(2 pi i c ty) as base(16 kc) x step(j),
// both from exact float-float turn reductions), warps 0-7 also run the
// epilogue of their own TMEM lane (row phases likewise as base x step per
// 8 rows); lane 0 of warp 16 copies the pre-split B stages (one 32 KB bulk
// copy each) and issues the MMAs.  Three 64 KB stages in shared memory.  Every wait is
// bounded (2 s); a wait that runs out sets the status word's timeout bit,
// the CTA drains its own copies and MMAs (bounded), frees its tensor memory
// and returns.
#include <cuda_fp16.h>

#include <algorithm>

#include "common.cuh"
#include "tc_ptx.cuh"
#include "warp.cuh"
#include "warp_math.cuh"

namespace flct {
namespace {

constexpr int kWtPx = 256;                       // pixels per CTA
constexpr int kWtGen = 16;                       // generator warps: two threads per pixel
constexpr int kWtThreads = 32 * (kWtGen + 1);    // + the copy / MMA warp
constexpr int kWtStages = 3;
constexpr int kWtAT = 128 * 32 * 2;              // one 128-pixel A tile (hi or lo), bytes
constexpr int kWtBH = 256 * 32 * 2;              // the B tile's hi (or lo) half, bytes
constexpr int kWtStage = 4 * kWtAT + 2 * kWtBH;  // A hi x2, A lo x2, B hi, B lo: 64 KB
constexpr int kWtSmem = kWtStages * kWtStage + 1024;
constexpr uint64_t kWtLimit = 2000000000ull;     // 2 s per wait

// Byte offset of element (row, k) of a K-major tile with 32 K (8 x 16-byte
// core matrices, no swizzle: LBO 128 between K groups, SBO 512 between row groups).
__host__ __device__ constexpr int kmaj_off(int row, int k) {
    return (row & 7) * 16 + (row >> 3) * 512 + (k & 7) * 2 + (k >> 3) * 128;
}

// Power-of-two scale that brings 2 max|F| (the weight-2 columns) below 2^14.
__device__ __forceinline__ float wt_scale(unsigned maxbits) {
    const float m = 2.0f * __uint_as_float(maxbits);
    if (!(m > 0.0f) || !(m < 3.0e38f)) return 1.0f;  // zero or non-finite spectrum: unscaled
    int e;
    frexpf(m, &e);  // m < 2^e
    return ldexpf(1.0f, max(-120, min(120, 14 - e)));
}

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}

__device__ __forceinline__ unsigned h2_bits(__half2 h) {
    return (unsigned)__half_as_ushort(__low2half(h)) | ((unsigned)__half_as_ushort(__high2half(h)) << 16);
}

// hi / lo FP16 halves of two values, packed (first value in the low half)
__device__ __forceinline__ void split2(float v0, float v1, unsigned& hi, unsigned& lo) {
    const __half2 h = __floats2half2_rn(v0, v1);
    const float2 f = __half22float2(h);
    hi = h2_bits(h);
    lo = h2_bits(__floats2half2_rn(v0 - f.x, v1 - f.y));
}

__device__ __forceinline__ void mbar_arrive(uint64_t* b) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(tc::smem_u32(b)) : "memory");
}

// max |component| of the spectrum, as the bits of a non-negative float
__global__ void k_wt_absmax(const float* __restrict__ f, long n, unsigned* __restrict__ mx) {
    float m = 0.0f;
    for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x)
        m = fmaxf(m, fabsf(f[k]));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(mx, __float_as_uint(m));
}

// The B stages: block (q, kc) holds rows ii = 128 q .. +127 and columns
// c = 16 kc .. +15 as a 256 x 32 K-major tile, hi half then lo half (32 KB).
// One thread per 16-byte unit (8 K-consecutive values of one tile row),
// ordered so that 8 consecutive threads write one 128-byte core matrix.
__global__ void k_wt_hsplit(const float2* __restrict__ F, int nx, int ny, int nkc, long nunits,
                            const unsigned* __restrict__ mx, uint4* __restrict__ hs) {
    const float sc = wt_scale(*mx);
    const int ncol = ny / 2 + 1;
    const int nyq_row = (nx % 2 == 0) ? nx / 2 : -1;
    const int nyq_col = (ny % 2 == 0) ? ny / 2 : -1;
    for (long u = blockIdx.x * (long)blockDim.x + threadIdx.x; u < nunits; u += (long)gridDim.x * blockDim.x) {
        const int n = (int)(((u >> 5) & 31) * 8 + (u & 7));
        const int kg = (int)((u >> 3) & 3);
        const long blk = u >> 10;
        const int q = (int)(blk / nkc), kc = (int)(blk - (long)q * nkc);
        const int part = n >> 7, ii = q * 128 + (n & 127);
        const bool ims = kg >= 2;
        const int c0 = kc * 16 + (kg & 1) * 8;
        unsigned hw[4], lw[4];
#pragma unroll
        for (int e = 0; e < 8; e += 2) {
            float v[2];
#pragma unroll
            for (int d = 0; d < 2; ++d) {
                const int c = c0 + e + d;
                float2 f = make_float2(0.0f, 0.0f);
                if (ii < nx && c < ncol && (ii | c) != 0) {  // the DC term is added exactly by the epilogue
                    f = F[(size_t)ii * ny + c];
                    const float w = (ii == nyq_row || c == 0 || c == nyq_col) ? sc : 2.0f * sc;
                    f.x *= w;
                    f.y *= w;
                }
                v[d] = part == 0 ? (ims ? -f.y : f.x) : (ims ? f.x : f.y);
            }
            split2(v[0], v[1], hw[e / 2], lw[e / 2]);
        }
        const size_t o = ((size_t)blk * (2 * kWtBH) + (size_t)kmaj_off(n, kg * 8)) / 16;
        hs[o] = make_uint4(hw[0], hw[1], hw[2], hw[3]);
        hs[o + kWtBH / 16] = make_uint4(lw[0], lw[1], lw[2], lw[3]);
    }
}

__global__ void __launch_bounds__(kWtThreads, 1)
    k_wt_sum(const unsigned char* __restrict__ hs, const float4* __restrict__ ph, const float2* __restrict__ F,
             const unsigned* __restrict__ mx, int nx, int ny, int nq, int nkc, double normfac,
             double* __restrict__ out, unsigned* __restrict__ status, unsigned long long stall_ns) {
    extern __shared__ unsigned char wt_raw[];
    unsigned char* sm = reinterpret_cast<unsigned char*>(
        (reinterpret_cast<uintptr_t>(wt_raw) + 1023) & ~static_cast<uintptr_t>(1023));
    __shared__ __align__(8) uint64_t s_fa[kWtStages], s_fb[kWtStages], s_em[kWtStages];
    __shared__ __align__(8) uint64_t s_accf, s_acce, s_fin, s_never;  // s_never: test hook only
    __shared__ uint32_t s_tmem;
    __shared__ volatile int s_abort;

    const int t = threadIdx.x, w = t >> 5, lane = t & 31;
    if (t == 0) {
        for (int s = 0; s < kWtStages; ++s) {
            tc::mbar_init(&s_fa[s], kWtGen);
            tc::mbar_init(&s_fb[s], 1);
            tc::mbar_init(&s_em[s], 1);
        }
        tc::mbar_init(&s_accf, 1);
        tc::mbar_init(&s_acce, 8);
        tc::mbar_init(&s_fin, 1);
        tc::mbar_init(&s_never, 1);
        s_abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (w == kWtGen) tc::tmem_alloc(&s_tmem, 512);
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = s_tmem;
    const uint32_t sbase = tc::smem_u32(sm);
    const int total = nq * nkc;

    // bounded wait; also gives up once another thread of the CTA has
    auto wait = [&](uint64_t* b, uint32_t par) -> bool {
        const uint32_t a = tc::smem_u32(b);
        const uint64_t t0 = tc::globaltimer();
        while (true) {
            uint32_t done;
            asm volatile(
                "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
                "selp.u32 %0, 1, 0, p;\n}\n"
                : "=r"(done)
                : "r"(a), "r"(par)
                : "memory");
            if (done) return true;
            if (s_abort) return false;
            if (tc::globaltimer() - t0 > kWtLimit) {
                s_abort = 1;
                return false;
            }
        }
    };

    if (w == kWtGen) {
        if (lane == 0) {
            bool ok = true;
            int gc = 0, gm = 0;  // stages copied, stages consumed
            auto copy = [&](int g) -> bool {
                const int s = g % kWtStages, u = g / kWtStages;
                if (u > 0 && !wait(&s_em[s], (uint32_t)((u - 1) & 1))) return false;
                tc::mbar_expect_tx(&s_fb[s], 2 * kWtBH);
                const int q = g / nkc, kc = nkc - 1 - (g - q * nkc);
                tc::bulk_g2s(sm + s * kWtStage + 4 * kWtAT, hs + ((size_t)q * nkc + kc) * (2 * kWtBH), 2 * kWtBH,
                             &s_fb[s]);
                return true;
            };
            while (ok && gc < (total < 2 ? total : 2)) {
                ok = copy(gc);
                if (ok) ++gc;
            }
            constexpr uint32_t id = tc::idesc(0, 128, 256, false, false);
            // test hook: a first wait on a barrier nothing completes, with a
            // short limit, takes the timeout path without a fault
            if (ok && stall_ns && !tc::mbar_wait(&s_never, 0u, stall_ns)) {
                s_abort = 1;
                ok = false;
            }
            for (int q = 0; q < nq && ok; ++q) {
                if (q > 0) {
                    ok = wait(&s_acce, (uint32_t)((q - 1) & 1));
                    if (!ok) break;
                    tc::fence_after();
                }
                for (int kc = 0; kc < nkc && ok; ++kc) {
                    const int g = q * nkc + kc, s = g % kWtStages;
                    const uint32_t par = (uint32_t)((g / kWtStages) & 1);
                    ok = wait(&s_fa[s], par) && wait(&s_fb[s], par);
                    if (!ok) break;
                    gm = g + 1;
                    tc::fence_after();
                    const uint32_t st = sbase + (uint32_t)(s * kWtStage);
#pragma unroll
                    for (int T = 0; T < 2; ++T)
#pragma unroll
                        for (int ks = 0; ks < 2; ++ks) {
                            const uint64_t ah = tc::desc(st + T * kWtAT + ks * 256, 128, 512);
                            const uint64_t al = tc::desc(st + (2 + T) * kWtAT + ks * 256, 128, 512);
                            const uint64_t bh = tc::desc(st + 4 * kWtAT + ks * 256, 128, 512);
                            const uint64_t bl = tc::desc(st + 4 * kWtAT + kWtBH + ks * 256, 128, 512);
                            const uint32_t d = tmem + (uint32_t)(T * 256);
                            // the small cross products first, the large hi*hi last
                            tc::mma(d, ah, bl, id, (kc | ks) ? 1u : 0u);
                            tc::mma(d, al, bh, id, 1u);
                            tc::mma(d, ah, bh, id, 1u);
                        }
                    tc::commit(&s_em[s]);
                    if (kc == nkc - 1) tc::commit(&s_accf);
                    if (gc < total) {
                        ok = copy(gc);
                        if (ok) ++gc;
                    }
                }
            }
            // drain: every MMA this thread issued, every copy not consumed
            tc::commit(&s_fin);
            tc::mbar_wait(&s_fin, 0u, kWtLimit);
            for (int g = gm; g < gc; ++g) tc::mbar_wait(&s_fb[g % kWtStages], (uint32_t)((g / kWtStages) & 1), kWtLimit);
            if (!ok) atomicOr(status, kStatusTimeout);
        }
        __syncwarp();
    } else {
        // pixel t % 256 of the CTA; half h generates columns 8h .. 8h+7 of
        // every stage; the threads of half 0 also run the epilogue (their
        // warp w < 8 reads TMEM lane quadrant w % 4 of tile w / 4)
        const int pix = t & (kWtPx - 1), h = t / kWtPx;
        const int T = pix >> 7, m = pix & 127;
        const long npx = (long)nx * ny;
        const long p = (long)blockIdx.x * kWtPx + pix;
        const bool live = p < npx;
        const float4 pb = live ? ph[p] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        const float sc = wt_scale(*mx);
        float2 S[8];  // exp(2 pi i (8h + j) ty), j < 8
#pragma unroll
        for (int j = 0; j < 8; ++j) S[j] = turn_cs((float)(8 * h + j), pb.z, pb.w);
        double acc = 0.0;
        bool ok = true;
        unsigned char* arow = sm + T * kWtAT + kmaj_off(m, 0);
        const uint32_t lane_base = (uint32_t)(32 * (w & 3)) << 16;

        auto epilogue = [&](int q) -> bool {
            int done = 1;
            if (lane == 0) done = wait(&s_accf, (uint32_t)(q & 1)) ? 1 : 0;
            if (!__shfl_sync(0xffffffffu, done, 0)) return false;
            tc::fence_after();
            const uint32_t tb = tmem + lane_base + (uint32_t)(T * 256);
            float2 Sx[8];  // exp(2 pi i j tx), j < 8
#pragma unroll
            for (int j = 0; j < 8; ++j) Sx[j] = turn_cs((float)j, pb.x, pb.y);
#pragma unroll 1
            for (int r0 = 0; r0 < 128; r0 += 8) {
                const int i0 = q * 128 + r0;
                if (i0 >= nx) break;
                // rows i0 .. i0+7 have wavenumbers kx(i0) + j unless the
                // wrap to negative wavenumbers falls inside the group
                const bool run = i0 + 7 <= nx / 2 || i0 > nx / 2;
                const float2 xb = turn_cs((float)freq_of(i0, nx), pb.x, pb.y);
                float gr[8], gi[8];
                tc::tmem_ld<8>(tb + r0, gr);
                tc::tmem_ld<8>(tb + 128 + r0, gi);
                float part = 0.0f;
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    const int ii = i0 + j;
                    if (ii < nx) {
                        const float2 ex = run ? cmul(xb, Sx[j]) : turn_cs((float)freq_of(ii, nx), pb.x, pb.y);
                        if (2 * ii == nx) {
                            // the Nyquist row (weight 1 in every column)
                            float2 a0 = F[(size_t)ii * ny];
                            if (ny % 2 == 0) {
                                const float2 v = cmul(F[(size_t)ii * ny + ny / 2],
                                                      turn_cs((float)(ny / 2), pb.z, pb.w));
                                a0.x += v.x;
                                a0.y += v.y;
                            }
                            a0.x *= sc;
                            a0.y *= sc;
                            part += fmaf(ex.x, a0.x, -ex.y * a0.y) + 2.0f * ex.x * (gr[j] - a0.x);
                        } else {
                            part = fmaf(ex.x, gr[j], fmaf(-ex.y, gi[j], part));
                        }
                    }
                }
                acc += (double)part;
            }
            tc::fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&s_acce);
            return true;
        };

        for (int q = 0; q < nq && ok; ++q) {
            for (int kc = 0; kc < nkc && ok; ++kc) {
                const int g = q * nkc + kc, s = g % kWtStages, u = g / kWtStages;
                if (u > 0) {
                    int done = 1;
                    if (lane == 0) done = wait(&s_em[s], (uint32_t)((u - 1) & 1)) ? 1 : 0;
                    ok = __shfl_sync(0xffffffffu, done, 0) != 0;
                    if (!ok) break;
                }
                // stage kc of a chunk holds columns 16 (nkc - 1 - kc) .. +15
                const float2 base = turn_cs((float)((nkc - 1 - kc) * 16), pb.z, pb.w);
                unsigned char* dst = arow + s * kWtStage;
                unsigned rh[4], rl[4], ih[4], il[4];
#pragma unroll
                for (int e = 0; e < 8; e += 2) {
                    const float2 v0 = cmul(base, S[e]);
                    const float2 v1 = cmul(base, S[e + 1]);
                    split2(v0.x, v1.x, rh[e / 2], rl[e / 2]);
                    split2(v0.y, v1.y, ih[e / 2], il[e / 2]);
                }
                *reinterpret_cast<uint4*>(dst + h * 128) = make_uint4(rh[0], rh[1], rh[2], rh[3]);
                *reinterpret_cast<uint4*>(dst + (2 + h) * 128) = make_uint4(ih[0], ih[1], ih[2], ih[3]);
                *reinterpret_cast<uint4*>(dst + 2 * kWtAT + h * 128) = make_uint4(rl[0], rl[1], rl[2], rl[3]);
                *reinterpret_cast<uint4*>(dst + 2 * kWtAT + (2 + h) * 128) = make_uint4(il[0], il[1], il[2], il[3]);
                tc::fence_async_smem();
                __syncwarp();
                if (lane == 0) mbar_arrive(&s_fa[s]);
                // the previous chunk's epilogue, once this chunk's first
                // stages are queued for the tensor cores
                if (h == 0 && q > 0 && kc == (nkc > 1 ? 1 : 0)) ok = epilogue(q - 1);
            }
        }
        if (ok && h == 0) ok = epilogue(nq - 1);
        if (ok && live && h == 0) out[p] = acc * (normfac / (double)sc) + (double)F[0].x * normfac;
        if (!ok && lane == 0) atomicOr(status, kStatusTimeout);
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    if (w == kWtGen) tc::tmem_dealloc(tmem, 512);
}

}  // namespace

size_t warp_tc_split_bytes(int nx, int ny) {
    const size_t nq = (size_t)(nx + 127) / 128, nkc = (size_t)(ny / 2 + 1 + 15) / 16;
    return nq * nkc * (size_t)(2 * kWtBH);
}

cudaError_t launch_warp_sum_tc(const float2* F, const float4* ph, int nx, int ny, void* hs, unsigned* misc,
                               double* out, cudaStream_t st, unsigned long long stall_ns) {
    const int nq = (nx + 127) / 128, nkc = (ny / 2 + 1 + 15) / 16;
    const long npx = (long)nx * ny;
    cudaError_t e = cudaMemsetAsync(misc, 0, 2 * sizeof(unsigned), st);
    if (e != cudaSuccess) return e;
    const long nf = 2 * npx;
    k_wt_absmax<<<(int)std::min<long>((nf + 255) / 256, 2048), 256, 0, st>>>(reinterpret_cast<const float*>(F), nf,
                                                                             misc);
    const long nunits = (long)nq * nkc * 1024;
    k_wt_hsplit<<<(int)std::min<long>((nunits + 255) / 256, 65536), 256, 0, st>>>(F, nx, ny, nkc, nunits, misc,
                                                                                   reinterpret_cast<uint4*>(hs));
    e = cudaFuncSetAttribute(k_wt_sum, cudaFuncAttributeMaxDynamicSharedMemorySize, kWtSmem);
    if (e != cudaSuccess) return e;
    k_wt_sum<<<(unsigned)((npx + kWtPx - 1) / kWtPx), kWtThreads, kWtSmem, st>>>(
        reinterpret_cast<const unsigned char*>(hs), ph, F, misc, nx, ny, nq, nkc, 1.0 / (double)npx, out, misc + 1,
        stall_ns);
    return cudaGetLastError();
}

}  // namespace flct
