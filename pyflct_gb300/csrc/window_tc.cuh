// window_tc.cuh -- the tensor-core window-correlation kernel (DFT-matrix
// form, split precision) for every box size n = 4..64 (multiples of 4).
//
// Same contract as k_window_fp32 (source/flct.c:829-876, 1325-1532: window,
// transforms, conj product with the optional filter, inverse, |c| in the
// half-shifted frame, first strict maximum), but every transform is a dense
// DFT-matrix product on the tcgen05 tensor cores.  Operands are split into a
// 16-bit high part and a 16-bit remainder (FP16 or BF16); each product is
// hi*hi + hi*lo + lo*hi accumulated in FP32 in tensor memory, which keeps
// ~21 significant bits (FP16) of every 16-bit-by-16-bit product.
//
// A CTA of 256 threads (8 warps) runs WIT windows per iteration through four
// GEMM stages, each M = 128 rows of data against a constant DFT matrix held
// in shared memory (H = n/2, n8 = n rounded up to 8, k1 = n rounded up to 16):
//   S1  along j, real input -> real-form half spectrum T[i][c]
//       (c = 0..H: cosine sums, ky = c; c = H+1..n-1: minus sine sums,
//       ky = c - H); rows (window, image, i), n8 rows per sub-image,
//       A MN-major (the box columns are loaded coalesced, one per lane),
//       K = j (k1), N = c (k1)                                      T1 tiles
//   S2  complex DFT along i: rows (window, ky), one row per complex column
//       of the half spectrum, A MN-major, K = (re/im, i) (2 n8),
//       N = (re/im, kx) (2 n8), both images into adjacent TMEM columns
//   product C = conj(A) B filt^2 per (kx, ky) in the row's lane: both
//       images' spectra sit in the same TMEM lane
//   S3  inverse complex DFT along kx: rows (window, ky), A K-major,
//       K = (re/im, kx), N = (re/im, i)               (S2's matrix, transposed)
//   S4  complex-to-real along ky: rows (window, i), A MN-major, K = the
//       spectral terms (weights 1 or 2 folded into the data), N = j
//                                                 (S1's matrix, transposed)
// then |c| in the half-shifted frame, the first strict maximum, the peak
// record.  S3 reuses S2's matrix and S4 reuses S1's through the descriptors'
// MN-major mode, so each stage's transpose is free: each thread writes its
// TMEM row straight into the next stage's operand layout, in 16-byte chunks.
//
// Half-spectrum columns: with H a multiple of 8 (n = 16, 32, 48, 64) the two
// real columns ky = 0 and ky = H share one complex row ("packed": T[:,0] +
// i T[:,H]) and the product separates them by Hermitian symmetry; otherwise
// the rows per window are padded to a multiple of 8 anyway and ky = H gets a
// row of its own.  In packed mode the S2 output columns hold kx and -kx next
// to each other (tc_kx order) so a lane has both halves of every mirror pair.
//
// Scaling: each sub-image is scaled by an exact power of two that brings its
// largest |value| into [1, 4) (FP16 holds it without overflow); the
// conj(A) B product and the inverse along kx by fixed powers of two from
// a-priori bounds (|C| <= 16 n^4, |u| <= n max |C|), so no FP16 operand can
// overflow; none of these changes the argmax or the fit.
//
// Every wait on the tensor cores is bounded (2 s); a wait that runs out
// sets the status word's timeout bit, the CTA waits (bounded) for its own
// MMAs, frees its tensor memory and returns.
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <type_traits>
#include <vector>

#include "common.cuh"
#include "fft_reg.cuh"
#include "tc_ptx.cuh"
#include "window_common.cuh"

namespace flct {

struct TcArgs {
    const float4* s12;    // both frames split per pixel (WinArgs::s12: f1 hi, f2 hi, f1 lo, f2 lo)
    const float4* means;  // per grid point at mean_slot(mg, i, j), or null (direct windows)
    MeanGrid mg;
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
    // the DFT matrices as split 16-bit hi / lo halves, already in their
    // shared-memory layouts: B1 hi, B1 lo, B2 hi, B2 lo (TcCfg<n>::BB bytes)
    const uint16_t* bmat;
    unsigned* status;
    // failure-path test hook: when nonzero, every stage waits this many ns
    // on a barrier that nothing completes (instead of the MMA barrier), so
    // that the wait runs out; the exit path still waits for the real MMAs
    unsigned long long stall_ns;
    float gauss[2 * kMaxBox + 1];
    float filt2[kMaxBox];
};

__host__ __device__ constexpr int tc_r8(int x) { return (x + 7) / 8 * 8; }
__host__ __device__ constexpr int tc_r16(int x) { return (x + 15) / 16 * 16; }
__host__ __device__ constexpr int tc_max(int a, int b) { return a > b ? a : b; }
__host__ __device__ constexpr int tc_pow2(int x) { return x <= 32 ? 32 : x <= 64 ? 64 : x <= 128 ? 128 : x <= 256 ? 256 : 512; }

// Compile-time geometry of the tensor-core form for box side N.
template <int N>
struct TcCfg {
    static_assert(N % 4 == 0 && N >= 4 && N <= kMaxBox, "box side");
    static constexpr int H = N / 2;
    static constexpr bool PACK = (H % 8) == 0;
    static constexpr int KYN = PACK ? H : H + 1;              // spectrum rows per window
    static constexpr int R2 = PACK ? H : tc_r8(H + 1);        // S2 / S3 rows per window
    static constexpr int G2 = R2 / 8;                         // 8-row groups per window
    static constexpr int WIT = 128 / R2;                      // windows per CTA iteration
    static constexpr int N8 = tc_r8(N);
    static constexpr int K1 = tc_r16(N);                      // S1 K and N, S4 K and N
    static constexpr int K2 = 2 * N8;                         // S2 K and N, S3 K and N
    static constexpr int SUBS = 2 * WIT;                      // sub-images per iteration
    static constexpr int T1 = (SUBS * N8 + 127) / 128;        // S1 tiles
    static constexpr int T4 = (WIT * N8 + 127) / 128;         // S4 tiles
    static constexpr int LW = K1 <= 16 ? 16 : 32;             // lanes per sub-image column block
    static constexpr int SPW = 32 / LW;                       // sub-images per warp pass
    static constexpr int CB = (K1 + 31) / 32;                 // column blocks (K1 > 32)
    static constexpr int QC = N8 / 8;                         // 8-column chunks of a spectrum row
    // shared memory, bytes (each operand as hi then lo)
    static constexpr int A1B = T1 * 128 * K1 * 2;
    static constexpr int A2B = 128 * K2 * 2;                  // per image
    static constexpr int A3B = 128 * K2 * 2;
    static constexpr int A4B = T4 * 128 * K1 * 2;
    // staged correlation rows: vectors of SV floats, row stride SROW floats
    // (16 bytes past a multiple of 128: 16-byte stores of 8 rows hit
    // distinct banks)
    static constexpr int SV = (H % 4 == 0) ? 4 : 2;
    static constexpr int SROW = N + SV;
    static constexpr int STGB = WIT * N * SROW * 4;
    static constexpr int AREG =
        (tc_max(tc_max(2 * A1B, 4 * A2B), tc_max(tc_max(2 * A3B, 2 * A4B), STGB)) + 1023) / 1024 * 1024;
    static constexpr int B1B = K1 * K1 * 2;
    static constexpr int B2B = K2 * K2 * 2;
    static constexpr int BB = 2 * B1B + 2 * B2B;
    static constexpr int MISC = 2048;
    static constexpr int SMEM = AREG + BB + MISC + 1024;      // + 1024 to align the base
    static constexpr int TCOLS = tc_pow2(tc_max(tc_max(T1 * K1, 2 * K2), tc_max(K2, T4 * K1)));
    static constexpr int MINB = N <= 32 ? 2 : 1;
    // fixed power-of-two scales: sub-images are scaled into |x| < 4, so
    // |A|, |B| <= 4 n^2 and |C| <= 16 n^4; 2^-CSH1 brings that bound to
    // 2^15 (below the FP16 maximum).  The inverse along kx sums n of those
    // and the c2r weight doubles it: 2^-CSH2 brings 2 n 2^15 back to 2^15.
    static constexpr int LOG2N = N <= 4 ? 2 : N <= 8 ? 3 : N <= 16 ? 4 : N <= 32 ? 5 : 6;
    static constexpr int CSH1 = 4 * LOG2N + 4 - 15;
    static constexpr int CSH2 = LOG2N + 1;
    static_assert(SMEM <= 232448, "shared memory");
    static_assert(BB % 16 == 0 && B1B % 16 == 0, "bulk copy granularity");
};

// S2 output column q of a packed spectrum row holds wavenumber tc_kx(q):
// kx and -kx adjacent, q = 0 -> 0, q = 1 -> H, q = 2j -> j, q = 2j+1 -> N - j.
__host__ __device__ constexpr int tc_kx(int q, int n) {
    return q == 0 ? 0 : (q == 1 ? n / 2 : ((q % 2 == 0) ? q / 2 : n - q / 2));
}
__host__ __device__ constexpr int tc_mirror(int q) { return q < 2 ? q : ((q % 2 == 0) ? q + 1 : q - 1); }
// Column order of S2's output: tc_kx order in packed mode, natural otherwise.
template <int N>
__host__ __device__ constexpr int tc_kxq(int q) {
    return TcCfg<N>::PACK ? tc_kx(q, N) : q;
}

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
            const float2 d = csub(make_float2(v[2 * p], v[2 * p + 1]), __half22float2(a));
            const __half2 c = __floats2half2_rn(d.x, d.y);
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
            const float2 d = csub(make_float2(v[2 * p], v[2 * p + 1]), __bfloat1622float2(a));
            const __nv_bfloat162 c = __floats2bfloat162_rn(d.x, d.y);
            h[p] = *reinterpret_cast<const uint32_t*>(&a);
            l[p] = *reinterpret_cast<const uint32_t*>(&c);
        }
        hi = make_uint4(h[0], h[1], h[2], h[3]);
        lo = make_uint4(l[0], l[1], l[2], l[3]);
    }
};

// Split 8 floats (times `s`) and store the hi / lo chunks at byte offset
// `off` of the hi and lo planes.
template <typename T>
__device__ __forceinline__ void tc_put8(unsigned char* hi_plane, unsigned char* lo_plane, int off, const float* v,
                                        float s) {
    float w[8];
#pragma unroll
    for (int k = 0; k < 8; k += 2) {
        const float2 m = emul(make_float2(v[k], v[k + 1]), make_float2(s, s));
        w[k] = m.x;
        w[k + 1] = m.y;
    }
    uint4 hi, lo;
    Split16<T>::run(w, hi, lo);
    *reinterpret_cast<uint4*>(hi_plane + off) = hi;
    *reinterpret_cast<uint4*>(lo_plane + off) = lo;
}

#ifdef FLCT_TC_PROFILE
// Per-stage clock sums of thread 0 of every CTA (profiling builds only).
static __device__ unsigned long long g_tc_stage_clk[12];
#define FLCT_TC_STAMP(k)                                                     \
    do {                                                                     \
        if (t == 0) {                                                        \
            const long long c_ = clock64();                                  \
            atomicAdd(&g_tc_stage_clk[k], (unsigned long long)(c_ - clk0_)); \
            clk0_ = c_;                                                      \
        }                                                                    \
    } while (0)
#else
#define FLCT_TC_STAMP(k) \
    do {                 \
    } while (0)
#endif

template <int N, typename T>
__global__ void __launch_bounds__(256, TcCfg<N>::MINB) k_window_tc(TcArgs a) {
    using C = TcCfg<N>;
    constexpr int H = C::H, N8 = C::N8, K1 = C::K1, K2 = C::K2, WIT = C::WIT;
    constexpr uint64_t kLimit = 2000000000ull;  // 2 s per wait
    extern __shared__ unsigned char sm_raw[];
    unsigned char* sm = reinterpret_cast<unsigned char*>(
        (reinterpret_cast<uintptr_t>(sm_raw) + 1023) & ~static_cast<uintptr_t>(1023));
    unsigned char* Ahi = sm;
    unsigned char* Bm = sm + C::AREG;  // B1 hi, B1 lo, B2 hi, B2 lo
    unsigned char* B1hi = Bm;
    unsigned char* B1lo = Bm + C::B1B;
    unsigned char* B2hi = Bm + 2 * C::B1B;
    unsigned char* B2lo = B2hi + C::B2B;
    unsigned char* misc = Bm + C::BB;
    float* s_g = reinterpret_cast<float*>(misc);                            // 2 kMaxBox + 1
    float* s_f = s_g + 2 * kMaxBox + 4;                                      // kMaxBox
    uint64_t* s_mbar = reinterpret_cast<uint64_t*>(misc + 800);             // MMA completion
    uint64_t* s_never = s_mbar + 1;                                          // test hook only
    uint64_t* s_bbar = s_mbar + 2;                                           // matrix copy
    uint32_t* s_tmem = reinterpret_cast<uint32_t*>(misc + 832);
    int* s_gi = reinterpret_cast<int*>(misc + 848);                          // WIT
    int4* s_geo = reinterpret_cast<int4*>(misc + 912);                       // WIT: imin, jmin, gr off, gc off
    float4* s_mean = reinterpret_cast<float4*>(misc + 1168);                 // WIT
    const float4** s_src = reinterpret_cast<const float4**>(misc + 1424);   // WIT box origins (2 WIT slots)
    int* s_ny = reinterpret_cast<int*>(misc + 1680);                         // WIT
    unsigned* s_wmax = reinterpret_cast<unsigned*>(misc + 1744);             // WIT
    int* s_widx = reinterpret_cast<int*>(misc + 1808);                       // WIT
    int* s_wnan = reinterpret_cast<int*>(misc + 1872);                       // WIT
    int* s_valid = reinterpret_cast<int*>(misc + 1936);                      // WIT
    static_assert(WIT <= 16, "window slots in the misc region");

    const int t = threadIdx.x, wp = t >> 5, lane = t & 31;
    const int qd = wp & 3, hf = wp >> 2;  // TMEM lane quadrant, half of the stage's columns
    const uint32_t lane_base = (uint32_t)(qd * 32) << 16;

    for (int k = t; k < 2 * kMaxBox + 1; k += 256) s_g[k] = a.gauss[k];
    for (int k = t; k < kMaxBox; k += 256) s_f[k] = a.use_filter ? a.filt2[k] : 1.0f;
    if (wp == 0) tc::tmem_alloc(s_tmem, C::TCOLS);
    if (t == 0) {
        tc::mbar_init(s_mbar, 1);
        tc::mbar_init(s_never, 1);
        tc::mbar_init(s_bbar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    // the constant matrices: two bulk copies by the TMA engine
    if (t == 0) {
        tc::mbar_expect_tx(s_bbar, (uint32_t)C::BB);
        tc::bulk_g2s(Bm, a.bmat, (uint32_t)(2 * C::B1B), s_bbar);
        tc::bulk_g2s(Bm + 2 * C::B1B, reinterpret_cast<const unsigned char*>(a.bmat) + 2 * C::B1B,
                     (uint32_t)(2 * C::B2B), s_bbar);
    }
    const bool bok = tc::mbar_wait(s_bbar, 0u, kLimit);
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = *s_tmem;

    constexpr uint32_t id1 = tc::idesc(Split16<T>::fmt, 128, K1, true, false);
    constexpr uint32_t id2 = tc::idesc(Split16<T>::fmt, 128, K2, true, false);
    constexpr uint32_t id3 = tc::idesc(Split16<T>::fmt, 128, K2, false, true);
    constexpr uint32_t id4 = tc::idesc(Split16<T>::fmt, 128, K1, true, true);
    const uint32_t ahi = tc::smem_u32(Ahi);
    const uint32_t b1hi = tc::smem_u32(B1hi);
    const uint32_t b2hi = tc::smem_u32(B2hi);
    // base descriptors of every operand layout; a tile or K step adds its
    // byte offset / 16 to the start-address field (all offsets stay inside
    // the 256 KB shared window, so the field never carries)
    const uint64_t dA_mn = tc::desc(ahi, 2048, 128);     // A1, A2, A4 (MN-major, 128 rows)
    const uint64_t dA3 = tc::desc(ahi, 128, K2 * 16);    // A3 (K-major)
    const uint64_t dB1k = tc::desc(b1hi, 128, K1 * 16);  // B1 K-major (S1)
    const uint64_t dB1m = tc::desc(b1hi, K1 * 16, 128);  // B1 MN-major (S4)
    const uint64_t dB2k = tc::desc(b2hi, 128, K2 * 16);  // B2 K-major (S2)
    const uint64_t dB2m = tc::desc(b2hi, K2 * 16, 128);  // B2 MN-major (S3)
    constexpr uint64_t oB1lo = (uint64_t)(C::B1B >> 4), oB2lo = (uint64_t)(C::B2B >> 4);

    grid_dep_wait();  // work list, means and counters come from earlier kernels
    const int nwork = *a.nwork;
    uint32_t phase = 0;
    bool ok = __syncthreads_and(bok ? 1 : 0) != 0;

    auto mma3 = [&](uint32_t d, uint64_t ah, uint64_t al, uint64_t bh, uint64_t bl, uint32_t id, uint32_t acc) {
        tc::mma(d, ah, bh, id, acc);
        tc::mma(d, ah, bl, id, 1u);
        tc::mma(d, al, bh, id, 1u);
    };
    // one thread polls the MMA barrier, the others wait at the CTA barrier
    // (a barrier wait takes no issue slots from the other CTA on the SM)
    auto wait_stage = [&]() -> bool {
        bool done = true;
        if (t == 0)
            done = a.stall_ns ? tc::mbar_wait(s_never, 0u, a.stall_ns) : tc::mbar_wait_nap(s_mbar, phase, kLimit, 64);
        phase ^= 1u;
        const bool all = __syncthreads_and(done ? 1 : 0) != 0;
        tc::fence_after();
        return all;
    };
    auto to_mma = [&]() {
        tc::fence_async_smem();
        tc::fence_before();
        __syncthreads();
        tc::fence_after();
    };

    // The work items of an iteration, fetched one iteration ahead by the
    // threads t < WIT (their global-load latency then overlaps the previous
    // iteration's tensor-core stages).
    struct Fetch {
        const float4* f12;
        float4 mean;
        int gi, pix, nx, ny, valid;
    };
    auto fetch = [&](int b) {
        Fetch f;
        f.valid = b + t < nwork;
        int w = f.valid ? b + t : nwork - 1;
        f.f12 = a.s12;
        f.nx = a.nx;
        f.ny = a.ny;
        const float4* mp = a.means;
        MeanGrid mg = a.mg;
        if (a.nseg > 0) {
            const int k = seg_find(a.seg_start, a.nseg, w);
            const WinSeg sg = a.segs[k];
            f.f12 = sg.s12;
            f.nx = sg.nx;
            f.ny = sg.ny;
            if (mp) mp += sg.base;
            mg = sg.mg;
            w = sg.base + (w - __ldg(a.seg_start + k));
        }
        f.gi = w;
        f.pix = a.work[w];
        if (mp && !a.direct) {
            const int i = f.pix / f.ny;
            f.mean = mp[mean_slot(mg, i, f.pix - i * f.ny)];
        } else {
            f.mean = make_float4(0.f, 0.f, 0.f, 0.f);
        }
        return f;
    };
    Fetch nxt{};
    if (t < WIT && blockIdx.x * WIT < nwork) nxt = fetch(blockIdx.x * WIT);
#ifdef FLCT_TC_PROFILE
    long long clk0_ = clock64();
#endif
    for (int base = blockIdx.x * WIT; base < nwork && ok; base += gridDim.x * WIT) {
        // ---- window table (from the prefetched items) ------------------------
        if (t < WIT) {
            int ic, jc, imin, jmin;
            if (a.direct) {
                imin = nxt.pix / nxt.ny;
                jmin = 0;
                ic = imin;
                jc = 0;
            } else {
                ic = nxt.pix / nxt.ny;
                jc = nxt.pix - ic * nxt.ny;
                imin = box_start(ic, nxt.nx, a.nsize);
                jmin = box_start(jc, nxt.ny, a.nsize);
            }
            s_gi[t] = nxt.gi;
            s_valid[t] = nxt.valid;
            s_geo[t] = make_int4(imin, jmin, imin - ic + N, jmin - jc + N);
            s_src[t] = nxt.f12 + (size_t)imin * nxt.ny + jmin;
            s_ny[t] = nxt.ny;
            s_mean[t] = nxt.mean;
            s_wmax[t] = 0u;
            s_widx[t] = 0x7fffffff;
            s_wnan[t] = 0;
        }
        __syncthreads();
        FLCT_TC_STAMP(0);

        // ---- stage 0: boxes -> A1 (MN-major; lane = box column) ------------
        {
            unsigned char* A1lo = Ahi + C::A1B;
            // a warp's passes over sub-images, PJ of them at once when their
            // values fit in registers (more loads in flight per lane)
            constexpr int NPASS = (C::SUBS + 8 * C::SPW - 1) / (8 * C::SPW);
            constexpr int PJ = (C::CB * N8 <= 32 && NPASS >= 2) ? 2 : 1;
#pragma unroll 1
            for (int p0 = 0; p0 < NPASS; p0 += PJ) {
                float x[PJ][C::CB][N8];
                float gcol[PJ][C::CB];
                float mx[PJ];
                int sub[PJ];
                const int jl = lane % C::LW;
                // one sub-image per warp pass and two passes at once: the
                // warp takes both images of one window, so a 16-byte load
                // gives both frames' (hi, lo) of a pixel
                constexpr bool kPair = C::SPW == 1 && PJ == 2 && NPASS == 2;
                if constexpr (kPair) {
                    const int w = wp;  // sub-images 2 wp (f1) and 2 wp + 1 (f2)
                    const bool sval = 2 * w + 1 < C::SUBS;
                    sub[0] = sval ? 2 * w : -1;
                    sub[1] = sval ? 2 * w + 1 : -1;
                    const int wv = sval ? w : 0;
                    const int4 geo = s_geo[wv];
                    const int ny = s_ny[wv];
                    const float4 mm = s_mean[wv];
                    const float4* src = s_src[wv];
                    const float* gr = s_g + geo.z;
                    mx[0] = mx[1] = 0.f;
#pragma unroll
                    for (int cb = 0; cb < C::CB; ++cb) {
                        const int j = cb * 32 + jl;
                        const bool jv = sval && j < N;
                        const float gc = jv ? s_g[geo.w + j] : 0.f;
                        gcol[0][cb] = gcol[1][cb] = gc;
                        float m0 = 0.f, m1 = 0.f;
                        if (jv) {
                            const float4* col = src + j;
#pragma unroll
                            for (int i = 0; i < N8; ++i) {
                                if (i < N) {
                                    // (f1, f2): (hi - mean hi) + (lo - mean lo)
                                    const float4 q = __ldg(col + (size_t)i * ny);
                                    x[0][cb][i] = ((q.x - mm.x) + (q.z - mm.z)) * gr[i];
                                    x[1][cb][i] = ((q.y - mm.y) + (q.w - mm.w)) * gr[i];
                                    m0 = fmaxf(m0, fabsf(x[0][cb][i]));
                                    m1 = fmaxf(m1, fabsf(x[1][cb][i]));
                                } else {
                                    x[0][cb][i] = x[1][cb][i] = 0.f;
                                }
                            }
                        } else {
#pragma unroll
                            for (int i = 0; i < N8; ++i) x[0][cb][i] = x[1][cb][i] = 0.f;
                        }
                        mx[0] = fmaxf(mx[0], m0 * gc);
                        mx[1] = fmaxf(mx[1], m1 * gc);
                    }
                } else {
#pragma unroll
                for (int pj = 0; pj < PJ; ++pj) {
                    const int s = (p0 + pj) * 8 * C::SPW + wp * C::SPW + lane / C::LW;
                    const bool sval = p0 + pj < NPASS && s < C::SUBS;
                    sub[pj] = sval ? s : -1;
                    const int w = sval ? (s >> 1) : 0, img = s & 1;
                    const int4 geo = s_geo[w];
                    const int ny = s_ny[w];
                    const float4 mm = s_mean[w];
                    // x = (f - mean) g_r(i): the column weight g_c(j) >= 0 is
                    // folded into the lane's final scale
                    // this image's (hi, lo) mean: floats img and 2 + img of the float4
                    const float2 mhl = img ? make_float2(mm.y, mm.w) : make_float2(mm.x, mm.z);
                    const float4* src = s_src[w];
                    const float* gr = s_g + geo.z;
                    mx[pj] = 0.f;
#pragma unroll
                    for (int cb = 0; cb < C::CB; ++cb) {
                        const int j = cb * 32 + jl;
                        const bool jv = sval && j < N;
                        gcol[pj][cb] = jv ? s_g[geo.w + j] : 0.f;
                        float mc = 0.f;
                        if (jv) {
                            // this image's hi and lo: floats img and 2 + img of each pixel's float4
                            const float* col = reinterpret_cast<const float*>(src + j) + img;
                            const int ld = 4 * ny;  // floats per row of the interleaved split
#pragma unroll
                            for (int i = 0; i < N8; ++i) {
                                if (i < N) {
                                    const float2 d = make_float2(__ldg(col + (size_t)i * ld) - mhl.x,
                                                                 __ldg(col + (size_t)i * ld + 2) - mhl.y);
                                    x[pj][cb][i] = (d.x + d.y) * gr[i];
                                    mc = fmaxf(mc, fabsf(x[pj][cb][i]));
                                } else {
                                    x[pj][cb][i] = 0.f;
                                }
                            }
                        } else {
#pragma unroll
                            for (int i = 0; i < N8; ++i) x[pj][cb][i] = 0.f;
                        }
                        mx[pj] = fmaxf(mx[pj], mc * gcol[pj][cb]);
                    }
                }
                }
#pragma unroll
                for (int pj = 0; pj < PJ; ++pj) {
#pragma unroll
                    for (int o = C::LW / 2; o > 0; o >>= 1)
                        mx[pj] = fmaxf(mx[pj], __shfl_xor_sync(0xffffffffu, mx[pj], o));
                    const float sc = pow2_scale(__float_as_uint(mx[pj]));
                    const int s = sub[pj];
                    if (s >= 0) {
#pragma unroll
                        for (int cb = 0; cb < C::CB; ++cb) {
                            const int j = cb * 32 + jl;
                            if (j < K1) {
                                const float sj = sc * gcol[pj][cb];
#pragma unroll
                                for (int g = 0; g < N8 / 8; ++g) {
                                    const int row = s * N8 + 8 * g;
                                    const int off = (row >> 7) * (128 * K1 * 2) + ((row & 127) >> 3) * 128 +
                                                    (j & 7) * 16 + (j >> 3) * 2048;
                                    tc_put8<T>(Ahi, A1lo, off, &x[pj][cb][8 * g], sj);
                                }
                            }
                        }
                    }
                }
            }
        }
        to_mma();
        FLCT_TC_STAMP(1);
        if (t == 0) {
            // consecutive MMAs go to different accumulators (tiles) so that
            // the tensor pipe can overlap them
#pragma unroll
            for (int s = 0; s < K1 / 16; ++s)
#pragma unroll
                for (int tl = 0; tl < C::T1; ++tl)
                    mma3(tmem + tl * K1, dA_mn + ((tl * (128 * K1 * 2) + s * 4096) >> 4),
                         dA_mn + ((C::A1B + tl * (128 * K1 * 2) + s * 4096) >> 4), dB1k + (s * 256 >> 4),
                         dB1k + oB1lo + (s * 256 >> 4), id1, s > 0);
            tc::commit(s_mbar);
        }
        if (t < WIT && base + (int)gridDim.x * WIT < nwork) nxt = fetch(base + gridDim.x * WIT);
        if (!wait_stage()) {
            ok = false;
            break;
        }
        FLCT_TC_STAMP(2);

        // ---- stage 1: T rows -> A2 (MN-major rows (ky group, window, ky lo)) --
        {
            unsigned char* A2lo = Ahi + 2 * C::A2B;
#pragma unroll 1
            for (int tl = 0; tl < C::T1; ++tl) {
                const int g = tl * 128 + qd * 32 + lane;  // S1 row
                const int s = g / N8, i = g - s * N8;
                float v[K1];
                tc::tmem_ld<K1>(tmem + lane_base + tl * K1, v);
                if (s < C::SUBS) {
                    const int w = s >> 1, img = s & 1;
                    sfor<0, 2 * C::G2>([&](auto chc) {
                        constexpr int ch = decltype(chc)::value;
                        constexpr int p = ch / C::G2, g2 = ch % C::G2;
                        if ((ch & 1) == hf) {
                            float c8[8];
                            sfor<0, 8>([&](auto kc) {
                                constexpr int kk = decltype(kc)::value;
                                constexpr int ky = 8 * g2 + kk;
                                if constexpr (p == 0) {
                                    c8[kk] = (ky <= H) ? v[ky <= H ? ky : 0] : 0.f;
                                } else if constexpr (C::PACK) {
                                    c8[kk] = v[ky == 0 ? H : H + ky];
                                } else {
                                    c8[kk] = (ky > 0 && ky < H) ? v[(ky > 0 && ky < H) ? H + ky : 0] : 0.f;
                                }
                            });
                            const int mn = (g2 * WIT + w) * 8;
                            const int k = p * N8 + i;
                            const int off = img * C::A2B + (mn >> 3) * 128 + (k & 7) * 16 + (k >> 3) * 2048;
                            tc_put8<T>(Ahi, A2lo, off, c8, 1.0f);
                        }
                    });
                }
            }
        }
        tc::fence_before();
        to_mma();
        FLCT_TC_STAMP(3);
        if (t == 0) {
#pragma unroll
            for (int s = 0; s < K2 / 16; ++s)
#pragma unroll
                for (int img = 0; img < 2; ++img)
                    mma3(tmem + img * K2, dA_mn + ((img * C::A2B + s * 4096) >> 4),
                         dA_mn + ((2 * C::A2B + img * C::A2B + s * 4096) >> 4), dB2k + (s * 256 >> 4),
                         dB2k + oB2lo + (s * 256 >> 4), id2, s > 0);
            tc::commit(s_mbar);
        }
        if (!wait_stage()) {
            ok = false;
            break;
        }
        FLCT_TC_STAMP(4);

        // ---- stage 2: spectra -> conj(A) B filt^2 -> A3 (K-major) ----------
        {
            unsigned char* A3lo = Ahi + C::A3B;
            const int mn = qd * 32 + lane;  // S2 row
            const int g2 = (mn >> 3) / WIT;
            const int ky = g2 * 8 + (mn & 7);
            const bool valid = g2 < C::G2 && ky < C::KYN;
            const bool special = C::PACK && ky == 0;  // packed ky = 0 / H row
            const float cs = __uint_as_float((uint32_t)(127 - C::CSH1) << 23) * (special ? 0.25f : 1.0f);
            const float fk = s_f[valid ? ky : 0];
            const float f0 = s_f[0], fH = s_f[H];
#pragma unroll 1
            for (int qc = hf; qc < C::QC; qc += 2) {
                float yr1[8], yi1[8], yr2[8], yi2[8];
                {
                    uint32_t r0[8], r1[8], r2[8], r3[8];
                    const uint32_t tb = tmem + lane_base + 8 * qc;
                    tc::tmem_ld8_nw(tb, r0);
                    tc::tmem_ld8_nw(tb + N8, r1);
                    tc::tmem_ld8_nw(tb + K2, r2);
                    tc::tmem_ld8_nw(tb + K2 + N8, r3);
                    tc::tmem_wait_ld();
#pragma unroll
                    for (int k = 0; k < 8; ++k) {
                        yr1[k] = __uint_as_float(r0[k]);
                        yi1[k] = __uint_as_float(r1[k]);
                        yr2[k] = __uint_as_float(r2[k]);
                        yi2[k] = __uint_as_float(r3[k]);
                    }
                }
                if (!valid) continue;
                float ur[8], ui[8];
                if (!special) {
#pragma unroll
                    for (int k = 0; k < 8; ++k) {
                        ur[k] = yr1[k] * yr2[k] + yi1[k] * yi2[k];
                        ui[k] = yr1[k] * yi2[k] - yi1[k] * yr2[k];
                    }
                    if (a.use_filter) {
                        sfor<0, 8>([&](auto kc) {
                            constexpr int k = decltype(kc)::value;
                            // wavenumber of column 8 qc + k (qc is the loop's
                            // runtime index; the table is read by column)
                            const int q = 8 * qc + k;
                            const int kx = C::PACK ? tc_kx(q, N) : q;
                            const float f = s_f[kx < N ? kx : 0] * fk;
                            ur[k] *= f;
                            ui[k] *= f;
                        });
                    }
                } else {
                    // packed row: Y = A0 + i AH and Z = B0 + i BH with A0, AH,
                    // B0, BH the (Hermitian) spectra of the real columns ky = 0
                    // and ky = H: 2 A0 = Y + Ym, 2i AH = Y - Ym (Ym = conj Y(-kx));
                    // u = f0 conj(A0) B0 + i fH conj(AH) BH (the 1/4 is in cs)
                    sfor<0, 8>([&](auto kc) {
                        constexpr int k = decltype(kc)::value;
                        // chunks hold whole mirror pairs: columns 0 and 1 of
                        // the first chunk are their own mirrors (kx = 0, H),
                        // every other column pairs with its neighbour
                        const bool self = qc == 0 && k < 2;
                        const float mr1 = self ? yr1[k] : yr1[k ^ 1], mi1 = self ? yi1[k] : yi1[k ^ 1];
                        const float mr2 = self ? yr2[k] : yr2[k ^ 1], mi2 = self ? yi2[k] : yi2[k ^ 1];
                        const float syr = yr1[k] + mr1, syi = yi1[k] - mi1;
                        const float dyr = yr1[k] - mr1, dyi = yi1[k] + mi1;
                        const float szr = yr2[k] + mr2, szi = yi2[k] - mi2;
                        const float dzr = yr2[k] - mr2, dzi = yi2[k] + mi2;
                        const float c0r = syr * szr + syi * szi, c0i = syr * szi - syi * szr;
                        const float chr = dyr * dzr + dyi * dzi, chi = dyr * dzi - dyi * dzr;
                        float fx = 1.0f, a0 = 1.0f, aH = 1.0f;
                        if (a.use_filter) {
                            const int q = 8 * qc + k;
                            fx = s_f[tc_kx(q, N)];
                            a0 = f0;
                            aH = fH;
                        }
                        ur[k] = fx * (a0 * c0r - aH * chi);
                        ui[k] = fx * (a0 * c0i + aH * chr);
                    });
                }
                const int k0 = 8 * qc;
                const int rowoff = (mn & 7) * 16 + (mn >> 3) * (K2 * 16);
                tc_put8<T>(Ahi, A3lo, rowoff + (k0 >> 3) * 128, ur, cs);
                tc_put8<T>(Ahi, A3lo, rowoff + ((N8 + k0) >> 3) * 128, ui, cs);
            }
        }
        tc::fence_before();
        to_mma();
        FLCT_TC_STAMP(5);
        if (t == 0) {
#pragma unroll
            for (int s = 0; s < K2 / 16; ++s)
                mma3(tmem, dA3 + (s * 256 >> 4), dA3 + ((C::A3B + s * 256) >> 4),
                     dB2m + (s * 2 * (K2 * 16) >> 4), dB2m + oB2lo + (s * 2 * (K2 * 16) >> 4), id3, s > 0);
            tc::commit(s_mbar);
        }
        if (!wait_stage()) {
            ok = false;
            break;
        }
        FLCT_TC_STAMP(6);

        // ---- stage 3: U rows -> A4 (MN-major rows (window, i)) -------------
        {
            unsigned char* A4lo = Ahi + C::A4B;
            const int mn = qd * 32 + lane;
            const int grp = mn >> 3, g2 = grp / WIT, w = grp - g2 * WIT;
            const int ky = g2 * 8 + (mn & 7);
            const bool valid = g2 < C::G2 && ky < C::KYN;
            // spectral term rows k4 of S4 (ky = 0 -> 0, ky = H -> H, else
            // ky and H + ky) and the c2r weights
            int kre, kim;
            float wgt;
            constexpr float s2 = 1.0f / (float)(1 << C::CSH2);
            if (C::PACK) {
                kre = ky;
                kim = ky == 0 ? H : H + ky;
                wgt = ky == 0 ? s2 : 2.0f * s2;
            } else {
                kre = ky;
                kim = (ky > 0 && ky < H) ? H + ky : -1;
                wgt = (ky > 0 && ky < H) ? 2.0f * s2 : s2;
            }
            // zero the spectral-term columns k4 in [N, K1) (no row writes them)
            if constexpr (K1 > N) {
                for (int e = t; e < C::T4 * 16 * (K1 - N); e += 256) {
                    const int k4 = N + e % (K1 - N), rg = e / (K1 - N);  // rg: tile * 16 + row group
                    const int off = (rg >> 4) * (128 * K1 * 2) + (rg & 15) * 128 + (k4 & 7) * 16 + (k4 >> 3) * 2048;
                    *reinterpret_cast<uint4*>(Ahi + off) = make_uint4(0u, 0u, 0u, 0u);
                    *reinterpret_cast<uint4*>(A4lo + off) = make_uint4(0u, 0u, 0u, 0u);
                }
            }
            sfor<0, 2>([&](auto pc) {
                constexpr int p = decltype(pc)::value;
                float u[N8];
                tc::tmem_ld<N8>(tmem + lane_base + p * N8, u);
                const int k4 = p ? kim : kre;
                if (valid && k4 >= 0) {
#pragma unroll
                    for (int ic = 0; ic < N8 / 8; ++ic) {
                        if ((ic & 1) != hf) continue;
                        const int row = w * N8 + 8 * ic;
                        const int off = (row >> 7) * (128 * K1 * 2) + ((row & 127) >> 3) * 128 + (k4 & 7) * 16 +
                                        (k4 >> 3) * 2048;
                        tc_put8<T>(Ahi, A4lo, off, &u[8 * ic], wgt);
                    }
                }
            });
        }
        tc::fence_before();
        to_mma();
        FLCT_TC_STAMP(7);
        if (t == 0) {
#pragma unroll
            for (int s = 0; s < K1 / 16; ++s)
#pragma unroll
                for (int tl = 0; tl < C::T4; ++tl)
                    mma3(tmem + tl * K1, dA_mn + ((tl * (128 * K1 * 2) + s * 4096) >> 4),
                         dA_mn + ((C::A4B + tl * (128 * K1 * 2) + s * 4096) >> 4),
                         dB1m + (s * 2 * (K1 * 16) >> 4), dB1m + oB1lo + (s * 2 * (K1 * 16) >> 4), id4, s > 0);
            tc::commit(s_mbar);
        }
        if (!wait_stage()) {
            ok = false;
            break;
        }
        FLCT_TC_STAMP(8);

        // ---- stage 4: |c|, first strict maximum, peak record ---------------
        if constexpr (32 % N8 == 0) {
            // every window's rows lie in one warp: maximum, first maximum and
            // record without CTA barriers (warp h of a quadrant takes tile h)
            float* stg = reinterpret_cast<float*>(Ahi);
            constexpr int G = N8;  // lanes per window
            const int gbase = lane & ~(G - 1);
            const unsigned gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << gbase);
#pragma unroll 1
            for (int tl = hf; tl < C::T4; tl += 2) {
                const int r4 = tl * 128 + qd * 32 + lane;
                const int w = r4 / N8, i = r4 - w * N8;
                float c[K1];
                tc::tmem_ld<K1>(tmem + lane_base + tl * K1, c);
                const bool rv = w < WIT && i < N;
                const int I = (i + H) % N;
                float m = 0.f;
                if (rv) {
                    float* dst = stg + (w * N + I) * C::SROW;
#pragma unroll
                    for (int j = 0; j < N; ++j) m = fmaxf(m, fabsf(c[j]));
                    // J = j - H (mod N): the row's two halves, swapped
                    if constexpr (C::SV == 4) {
#pragma unroll
                        for (int jj = 0; jj < H; jj += 4) {
                            *reinterpret_cast<float4*>(dst + jj) =
                                make_float4(c[H + jj], c[H + jj + 1], c[H + jj + 2], c[H + jj + 3]);
                            *reinterpret_cast<float4*>(dst + H + jj) =
                                make_float4(c[jj], c[jj + 1], c[jj + 2], c[jj + 3]);
                        }
                    } else {
#pragma unroll
                        for (int jj = 0; jj < H; jj += 2) {
                            *reinterpret_cast<float2*>(dst + jj) = make_float2(c[H + jj], c[H + jj + 1]);
                            *reinterpret_cast<float2*>(dst + H + jj) = make_float2(c[jj], c[jj + 1]);
                        }
                    }
                }
                // window maximum over its lanes (pad rows and absent
                // windows add 0)
                float wm = m;
#pragma unroll
                for (int o = G / 2; o > 0; o >>= 1) wm = fmaxf(wm, __shfl_xor_sync(0xffffffffu, wm, o));
                const bool nan0 = rv && I == 0 && c[H] != c[H];
                const bool wnan = (__ballot_sync(0xffffffffu, nan0) & gmask) != 0u;
                // the first row (in I order) holding the maximum, then its
                // first column (in J order)
                int key = (rv && wm != 0.f && m == wm) ? I : 0x7fffffff;
#pragma unroll
                for (int o = G / 2; o > 0; o >>= 1) key = min(key, __shfl_xor_sync(0xffffffffu, key, o));
                int Jl = 0;
                if (rv && key == I) {
                    bool found = false;
#pragma unroll
                    for (int J = 0; J < N; ++J) {
                        const int j = (J + H) % N;
                        if (!found && fabsf(c[j]) == wm) {
                            Jl = J;
                            found = true;
                        }
                    }
                }
                const int win_lane = gbase + ((key == 0x7fffffff ? 0 : key) + H) % N;
                const int Jw = __shfl_sync(0xffffffffu, Jl, win_lane);
                __syncwarp();
                if (w < WIT && s_valid[w]) {
                    int Ip, Jp;
                    bool have;
                    if (wnan) {
                        Ip = 0;
                        Jp = 0;
                        have = true;
                    } else {
                        have = wm != 0.f;
                        Ip = have ? key : H;
                        Jp = have ? Jw : H;
                    }
                    const float* sw = stg + w * N * C::SROW;
                    const int kl = lane - gbase;
                    if (a.peaks_h) {
                        float* rec = reinterpret_cast<float*>(a.peaks_h + s_gi[w]);
                        for (int k = kl; k < kHiresPatch * kHiresPatch + 1; k += G) {
                            if (k < kHiresPatch * kHiresPatch) {
                                const int r = Ip - 2 + k / kHiresPatch, cc = Jp - 2 + k % kHiresPatch;
                                rec[k] = (r >= 0 && r < N && cc >= 0 && cc < N) ? fabsf(sw[r * C::SROW + cc]) : 0.f;
                            } else {
                                rec[k] = __uint_as_float(peak_meta(Ip, Jp, have));
                            }
                        }
                    } else {
                        const bool dofit = have && Ip > 0 && Ip < N - 1 && Jp > 0 && Jp < N - 1;
                        float* rec = reinterpret_cast<float*>(a.peaks + s_gi[w]);
                        for (int k = kl; k < 10; k += G) {
                            if (k < 9)
                                rec[k] = dofit ? fabsf(sw[(Ip - 1 + k / 3) * C::SROW + (Jp - 1 + k % 3)]) : 0.f;
                            else
                                rec[9] = __uint_as_float(peak_meta(Ip, Jp, dofit));
                        }
                    }
                }
                __syncwarp();
            }
        } else {
            float* stg = reinterpret_cast<float*>(Ahi);
            // rows of both halves: J in [0, H) <- j in [H, N); J in [H, N) <- j in [0, H)
            auto row_pass = [&](auto jbc) {
                constexpr int jb = decltype(jbc)::value;  // first j of this half
                constexpr int Jb = jb ? 0 : H;             // its first J
#pragma unroll 1
                for (int tl = 0; tl < C::T4; ++tl) {
                    const int r4 = tl * 128 + qd * 32 + lane;
                    const int w = r4 / N8, i = r4 - w * N8;
                    float c[K1];
                    tc::tmem_ld<K1>(tmem + lane_base + tl * K1, c);
                    float m_row = 0.f;
                    if (w < WIT && i < N) {
                        const int I = (i + H) % N;
                        float* dst = stg + (w * N + I) * C::SROW + Jb;
#pragma unroll
                        for (int jj = 0; jj < H; ++jj) m_row = fmaxf(m_row, fabsf(c[jb + jj]));
                        if constexpr (C::SV == 4) {
#pragma unroll
                            for (int jj = 0; jj < H; jj += 4)
                                *reinterpret_cast<float4*>(dst + jj) =
                                    make_float4(c[jb + jj], c[jb + jj + 1], c[jb + jj + 2], c[jb + jj + 3]);
                        } else {
#pragma unroll
                            for (int jj = 0; jj < H; jj += 2)
                                *reinterpret_cast<float2*>(dst + jj) = make_float2(c[jb + jj], c[jb + jj + 1]);
                        }
                        if (jb == H && I == 0 && c[H] != c[H]) s_wnan[w] = 1;
                    }
                    // window maximum: lanes of one window reduce, one of them
                    // updates the shared slot
                    const bool rv = w < WIT && i < N;
                    const unsigned same = __match_any_sync(0xffffffffu, rv ? w : -1);
                    if (rv) {
                        const unsigned mb = __reduce_max_sync(same, __float_as_uint(m_row));
                        if ((int)(__ffs(same) - 1) == lane) atomicMax(s_wmax + w, mb);
                    }
                }
            };
            if (hf == 0) row_pass(std::integral_constant<int, H>{});
            else row_pass(std::integral_constant<int, 0>{});
            __syncthreads();
            // candidates: rows whose half holds the window maximum
#pragma unroll 1
            for (int tl = 0; tl < C::T4; ++tl) {
                const int r4 = tl * 128 + qd * 32 + lane;
                const int w = r4 / N8, i = r4 - w * N8;
                if (w < WIT && i < N) {
                    const unsigned wm = s_wmax[w];
                    const int I = (i + H) % N;
                    const int Jb = hf ? H : 0;
                    const float* row = stg + (w * N + I) * C::SROW + Jb;
                    if (wm != 0u) {
                        const float fm = __uint_as_float(wm);
                        for (int jj = 0; jj < H; ++jj) {
                            if (fabsf(row[jj]) == fm) {
                                atomicMin(s_widx + w, I * N + Jb + jj);
                                break;
                            }
                        }
                    }
                }
            }
            __syncthreads();
            // peak records: one window per group of 64 threads
            for (int e = t; e < WIT * 64; e += 256) {
                const int w = e >> 6, k = e & 63;
                if (!s_valid[w]) continue;
                int Ip, Jp;
                bool have;
                if (s_wnan[w]) {
                    Ip = 0;
                    Jp = 0;
                    have = true;
                } else {
                    have = s_wmax[w] != 0u;
                    const int idx = s_widx[w];
                    Ip = have ? idx / N : H;
                    Jp = have ? idx - (idx / N) * N : H;
                }
                const float* sw = stg + w * N * C::SROW;
                if (a.peaks_h) {
                    if (k < kHiresPatch * kHiresPatch + 1) {
                        float* rec = reinterpret_cast<float*>(a.peaks_h + s_gi[w]);
                        if (k < kHiresPatch * kHiresPatch) {
                            const int r = Ip - 2 + k / kHiresPatch, cc = Jp - 2 + k % kHiresPatch;
                            rec[k] = (r >= 0 && r < N && cc >= 0 && cc < N) ? fabsf(sw[r * C::SROW + cc]) : 0.f;
                        } else {
                            rec[k] = __uint_as_float(peak_meta(Ip, Jp, have));
                        }
                    }
                } else if (k < 10) {
                    const bool dofit = have && Ip > 0 && Ip < N - 1 && Jp > 0 && Jp < N - 1;
                    float* rec = reinterpret_cast<float*>(a.peaks + s_gi[w]);
                    if (k < 9)
                        rec[k] = dofit ? fabsf(sw[(Ip - 1 + k / 3) * C::SROW + (Jp - 1 + k % 3)]) : 0.f;
                    else
                        rec[9] = __uint_as_float(peak_meta(Ip, Jp, dofit));
                }
            }
                }
        tc::fence_before();
        __syncthreads();
        tc::fence_after();
        FLCT_TC_STAMP(9);
    }

    if (!ok) {
        if (t == 0) atomicOr(a.status, kStatusTimeout);
        // let any MMA still in flight finish (bounded) before freeing TMEM
        tc::mbar_wait(s_mbar, phase ^ 1u, kLimit);
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    if (wp == 0) tc::tmem_dealloc(tmem, C::TCOLS);
}

template <int N, typename T>
cudaError_t launch_window_tc(const TcArgs& a, int grid, cudaStream_t st, bool pdl);
template <int N, typename T>
int window_tc_blocks_per_sm();

// Host-side construction of the split DFT matrices in their shared-memory
// layouts (TcArgs::bmat, TcCfg<n>::BB bytes): fmt 0 = FP16, 1 = BF16.
void tc_build_bmat(int n, int fmt, std::vector<uint16_t>* out);
int tc_bmat_bytes(int n);

}  // namespace flct
