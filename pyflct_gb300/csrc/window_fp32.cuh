// window_fp32.cuh -- K1, the fused per-window correlation kernel (FP32 form).
//
// Replaces the per-pixel body of the reference's main loop and cross_cor
// (source/flct.c:773-942 and 1325-1649): for every pixel on the work list it
// takes the n x n box around the pixel from both frames, subtracts the FP64
// local means, applies the Gaussian centred on the pixel, transforms both
// sub-images, forms conj(A)*B (times the squared k-space filter for -k),
// transforms back, takes |c| in the half-shifted frame and finds the first
// strict maximum.  The FP64 parts run with one window per lane
// (window_common.cuh): the local means in the box-sum column pass before,
// and k_fit (3x3 Taylor fit, velocity, mask) after; this kernel does no
// FP64 arithmetic.  (The fit run inside this kernel instead, one warp
// fitting each 32 finished windows of its CTA, made the kernel 25 us slower
// at 1024^2, sigma 8, -s 4i than k_fit takes on its own: measured.)
//
// Layout: a "team" of n threads owns one window; a CTA runs TEAMS teams
// (teams that tile whole warps synchronise per warp).  The two real
// sub-images travel as one complex array z = g1 + i g2 (one forward FFT for
// both); A and B are separated with the mirror Z(-k).  The forward 2-D
// transform is register FFTs along one axis, a shared-memory transpose, and
// register FFTs along the other axis.  The correlation image is real, so the
// inverse runs as one complex n x n/2 transform (even and odd output columns
// as real and imaginary parts), half the work of a complex n x n one.  The
// register transforms run by decimation in time with the twiddle products
// fused into the butterflies' sums, exact adds on the packed FP32 pipe
// (fft_reg.cuh), and C is formed for half the frequencies, the rest taken
// from the mirror lane (C of a real image is Hermitian).  A
// sub-image whose maximum is far from 1 is scaled by an exact power of two
// so FP32 never over- or under-flows; scaling changes neither the argmax
// nor the fit.
#pragma once
#include "common.cuh"
#include "fft_reg.cuh"
#include "window_common.cuh"

namespace flct {

struct WinArgs {
    const float4* s12;    // both frames split per pixel: (f1 hi, f2 hi, f1 lo, f2 lo) [nx*ny]
    const float4* means;  // per grid point at mean_slot(mg, i, j), or null: zero means
    MeanGrid mg;
    const int* work;      // pixel indices i*ny + j
    const int* nwork;     // number of work items (device)
    int nx, ny, nsize;
    int use_filter;       // -k given
    int direct;           // windows given directly: box w starts at row w*n, unit weights
    PeakRec* peaks;       // per work item: integer peak and its 3x3 |c| stencil
    PeakRecH* peaks_h;    // -h: the 6x6 patch records instead (null otherwise)
    const WinSeg* segs;   // batched launch: the pairs (s1, s2, nx, ny unused), else null
    const int* seg_start; // batched launch: [nseg + 1] item prefix sums; nwork = seg_start + nseg
    int nseg;
    float gauss[2 * kMaxBox + 1];  // weight of offset d at d + n (separable Gaussian)
    float filt2[kMaxBox];          // squared k-space filter factor by frequency index
    // boxes above kMaxBox: the big-box kernel builds its own tables from these
    double sigma, kr;
};

// Launch shape of the box-N kernel.  Variant V = 0 is the default; V = 1
// is the autotuner's alternative: twice the teams per CTA where that CTA
// still fits twice per SM in shared memory and has at most 512 threads,
// else half the teams, with no register cap.  A window's arithmetic is the
// same in both; only the windows per CTA and the occupancy differ.
template <int N>
constexpr int win_teams0() { return (N <= 8) ? (128 / N) : (N <= 20 || N == 32) ? 8 : (N <= 40) ? 4 : 2; }
template <int N>
constexpr size_t win_smem(int teams) {
    return 32 * teams + ((3 * N + 1) * 4 + 15) / 16 * 16 + (size_t)N * 8 + (size_t)teams * N * (N + 1) * 8;
}
template <int N>
constexpr int win_teams_alt() {
    constexpr int t = win_teams0<N>();
    return (2 * t * N <= 512 && 2 * win_smem<N>(2 * t) <= 227 * 1024) ? 2 * t : (t > 1 ? t / 2 : 1);
}

template <int N, int V = 0>
struct WinShape {
    static constexpr int TEAMS = V == 0 ? win_teams0<N>() : win_teams_alt<N>();
    static constexpr int THREADS = N * TEAMS;
    static constexpr int BUF = N * (N + 1);  // float2 per team
    static constexpr size_t tw_off = 32 * TEAMS + ((3 * N + 1) * 4 + 15) / 16 * 16;
    static constexpr size_t head = tw_off + (size_t)N * 8;
    static constexpr size_t smem = head + (size_t)TEAMS * BUF * 8;  // |c| reuses the buffer
    static_assert(smem == win_smem<N>(TEAMS), "shared-memory layout");
    // CTAs per SM the register allocation is held to (0: no constraint).
    // Box 32: 2 CTAs of 8 teams at 128 registers, no spills, beat 5 CTAs of
    // 4 teams at 96 registers with 12 bytes spilled (175.8 against 181.9 us
    // for 65,536 windows; 4 CTAs of 4 teams at 128 registers: 179.9 us;
    // measured).
    static constexpr int MINB = (V == 0 && N == 32) ? 2 : 0;
};

template <int N, int V>
__global__ void __launch_bounds__(WinShape<N, V>::THREADS, WinShape<N, V>::MINB)
k_window_fp32(WinArgs a) {
    using S = WinShape<N, V>;
    constexpr int TEAMS = S::TEAMS;
    extern __shared__ __align__(16) unsigned char sm[];
    unsigned long long* s_key = reinterpret_cast<unsigned long long*>(sm + 16 * TEAMS);
    unsigned* s_max = reinterpret_cast<unsigned*>(sm + 24 * TEAMS);
    float* s_g = reinterpret_cast<float*>(sm + 32 * TEAMS);
    float* s_f = s_g + (2 * N + 1);
    float2* s_tw = reinterpret_cast<float2*>(sm + S::tw_off);  // e^{2 pi i k / N}
    float2* s_buf = reinterpret_cast<float2*>(sm + S::head);

    const int team = threadIdx.x / N;
    const int ln = threadIdx.x - team * N;
    // Teams that tile whole warps (n = 4, 8, 16, 32) synchronise per warp,
    // reduce with warp reductions and exchange the mirror spectrum by
    // shuffles; other team widths share warps and go through shared memory
    // and the CTA barrier.
    constexpr bool kWarp = (32 % N == 0);
    const unsigned tmask =
        (N == 32) ? 0xffffffffu : (((1u << (N & 31)) - 1u) << ((threadIdx.x & 31) & ~(unsigned)(N - 1)));
    auto team_sync = [] {
        if constexpr (kWarp) __syncwarp();
        else __syncthreads();
    };
    for (int k = threadIdx.x; k < 2 * N + 1; k += blockDim.x) s_g[k] = a.gauss[k];
    for (int k = threadIdx.x; k < N; k += blockDim.x) s_f[k] = a.use_filter ? a.filt2[k] : 1.0f;
    if (threadIdx.x == 0) {
        sfor<0, N>([&](auto kc) {
            constexpr int k = decltype(kc)::value;
            constexpr CS w = ct_cossin(k, N);
            s_tw[k] = make_float2((float)w.c, (float)w.s);
        });
    }
    float2* buf = s_buf + team * S::BUF;
    float* ab = reinterpret_cast<float*>(buf);  // |c|, after the last transform
    grid_dep_wait();  // the tables above come from the kernel's arguments
    const int nwork = *a.nwork;
    if (ln == 0) {
        s_max[2 * team] = 0u;
        s_max[2 * team + 1] = 0u;
        s_key[team] = 0ull;
    }
    __syncthreads();

    for (int base = blockIdx.x * TEAMS; base < nwork; base += gridDim.x * TEAMS) {
        const int w = base + team;
        const bool valid = w < nwork;
        int gi = valid ? w : base;  // item index into work / peaks
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
        int i, j, imin, jmin;
        if (a.direct) {
            imin = pix / ny;
            jmin = 0;
            i = imin;
            j = 0;
        } else {
            i = pix / ny;
            j = pix - i * ny;
            imin = box_start(i, nx, a.nsize);
            jmin = box_start(j, ny, a.nsize);
        }

        // windowed, mean-subtracted column jj = ln of both frames: z = g1 + i g2
        float2 x[N];
        {
            const float4 mm =
                (mp && !a.direct) ? __ldg(mp + mean_slot(mg, i, j)) : make_float4(0.f, 0.f, 0.f, 0.f);
            const float2 mh = make_float2(mm.x, mm.y), ml = make_float2(mm.z, mm.w);  // (f1, f2) hi, lo
            const float wc = s_g[ln + jmin - j + N];
            const float4* p12 = f12 + (size_t)imin * ny + jmin + ln;
            const float* gr = a.gauss + (imin - i + N);  // row weights: uniform, from the parameter bank
            float mx1 = 0.f, mx2 = 0.f;
            sfor<0, N>([&](auto ic) {
                constexpr int ii = decltype(ic)::value;
                // (hi - mean hi) + (lo - mean lo) for both frames at once
                // (packed f1/f2 pairs), both frames' pixel in one 16-byte load
                const float4 q = __ldg(p12 + (size_t)ii * ny);
                const float2 dh = csub(make_float2(q.x, q.y), mh);
                const float2 dl = csub(make_float2(q.z, q.w), ml);
                const float wgt = wc * gr[ii];
                const float2 z = cscale(cadd(dh, dl), wgt);
                x[fft_in<N>(ii)] = z;  // row ii where the column transform takes it
                mx1 = fmaxf(mx1, fabsf(z.x));
                mx2 = fmaxf(mx2, fabsf(z.y));
            });
            unsigned b1, b2;
            if constexpr (kWarp) {
                b1 = __reduce_max_sync(tmask, __float_as_uint(mx1));
                b2 = __reduce_max_sync(tmask, __float_as_uint(mx2));
                team_sync();  // the previous window's |c| reads are done
            } else {
                atomicMax(&s_max[2 * team], __float_as_uint(mx1));
                atomicMax(&s_max[2 * team + 1], __float_as_uint(mx2));
                team_sync();
                b1 = s_max[2 * team];
                b2 = s_max[2 * team + 1];
            }
            // maxima within 2^+-40 of 1 need no scaling: every value of the
            // transforms then stays inside FP32's normal range
            auto near1 = [](unsigned b) { return b == 0u || (b >> 23) - 87u <= 80u; };
            if (!(near1(b1) && near1(b2))) {
                const float2 cs = make_float2(pow2_scale(b1), pow2_scale(b2));
#pragma unroll
                for (int ii = 0; ii < N; ++ii) x[ii] = emul(x[ii], cs);
            }
        }

        // forward 2-D FFT: columns in registers, transpose, rows in registers
        fft<N, 0, -1>(x);
        sfor<0, N>([&](auto kc) {
            constexpr int k = decltype(kc)::value;
            buf[k * (N + 1) + ln] = x[fft_out<N>(k)];
        });
        team_sync();
        if constexpr (!kWarp) {
            // every lane has read this window's scale factors and the
            // previous window's peak key: clear both for the next use
            if (ln == 0) {
                s_max[2 * team] = 0u;
                s_max[2 * team + 1] = 0u;
                s_key[team] = 0ull;
            }
        }
        sfor<0, N>([&](auto jc) {
            constexpr int jj = decltype(jc)::value;
            x[fft_in<N>(jj)] = buf[ln * (N + 1) + jj];
        });
        if constexpr (!kWarp) team_sync();
        fft<N, 0, -1>(x);  // thread ln now holds Z[kx = ln][ky] at x[fft_out<N>(ky)]
        if constexpr (!kWarp) {
            sfor<0, N>([&](auto kc) {
                constexpr int k = decltype(kc)::value;
                buf[ln * (N + 1) + k] = x[fft_out<N>(k)];
            });
            team_sync();
        }

        // separate A, B from Z and its mirror, C = conj(A) B filt^2.  C is
        // the spectrum of a real image, C[-kx][-ky] = conj(C[kx][ky]), and
        // the products below give exactly that (the mirror lane's operands
        // are the same values with negated imaginary parts, and filt2 is even
        // in k), so a lane forms columns 0..N/2 and takes the rest from the
        // mirror lane: by shuffles in whole-warp teams, else through the
        // buffer's columns 1..N/2-1, which no lane reads for its mirror Z
        // (for n >= 24; below that the extra barrier costs more than the
        // products it saves, measured).
        constexpr int H = N / 2;
        constexpr bool kMirror = kWarp || N >= 24;
        constexpr int KC = kMirror ? H + 1 : N;
        float2 y[N];
        {
            const int mr = (N - ln) % N;
            sfor<0, KC>([&](auto kc) {
                constexpr int k = decltype(kc)::value;
                constexpr int mk = (N - k) % N;
                const float2 z = x[fft_out<N>(k)];
                float2 zm;
                if constexpr (kWarp) {
                    zm.x = __shfl_sync(tmask, x[fft_out<N>(mk)].x, mr, N);
                    zm.y = __shfl_sync(tmask, x[fft_out<N>(mk)].y, mr, N);
                } else {
                    zm = buf[mr * (N + 1) + mk];
                }
                const float ax = z.x + zm.x, ay = z.y - zm.y;  // 2 s1 A
                const float bx = z.y + zm.y, by = zm.x - z.x;  // 2 s2 B
                y[k] = make_float2(ax * bx + ay * by, ax * by - ay * bx);
            });
            if (a.use_filter) {
                const float fr = s_f[ln];
                sfor<0, KC>([&](auto kc) {
                    constexpr int k = decltype(kc)::value;
                    const float f = fr * s_f[k];
                    y[k] = make_float2(f * y[k].x, f * y[k].y);
                });
            }
            if constexpr (kWarp) {
                sfor<KC, N>([&](auto kc) {
                    constexpr int k = decltype(kc)::value;
                    y[k].x = __shfl_sync(tmask, y[N - k].x, mr, N);
                    y[k].y = -__shfl_sync(tmask, y[N - k].y, mr, N);
                });
            } else if constexpr (kMirror) {
                sfor<1, H>([&](auto kc) {
                    constexpr int k = decltype(kc)::value;
                    buf[ln * (N + 1) + k] = y[k];
                });
                team_sync();
                sfor<KC, N>([&](auto kc) {
                    constexpr int k = decltype(kc)::value;
                    const float2 c = buf[mr * (N + 1) + (N - k)];
                    y[k] = make_float2(c.x, -c.y);
                });
            }
        }

        // Inverse transform of a spectrum whose image is real, at half the
        // work of a complex N x N transform.  Along ky, the even and odd
        // output columns come from a_k = C[k] + C[k+H] and
        // b_k = (C[k] - C[k+H]) w^k (w = e^{2 pi i / N}); both halves have real
        // images, so one complex N x H transform of a + i b yields
        // c[i][2m] + i c[i][2m+1].  Rows: H-point transforms in registers.
        float2 u[H];
        sfor<0, H>([&](auto kc) {
            constexpr int k = decltype(kc)::value;
            const float2 ak = cadd(y[k], y[k + H]);
            const float2 dk = csub(y[k], y[k + H]);
            // + i w^k dk = dk e^{2 pi i (4k + N) / 4N}
            u[fft_in<H>(k)] = tw_fma_add<+1, 4L * k + N, 4L * N>(ak, dk);
        });
        fft<H, 0, +1>(u);  // u[fft_out<H>(m)] = row kx = ln, column m
        // Columns (kx -> i), split by the parity h of i over two lanes: with
        // P0 = Y and P1 = Y w^kx stored side by side, lane (m, h) transforms
        // P_h[kx'] + P_h[kx' + H] (kx' < H), which is the first radix-2 stage
        // of the length-N column transform for outputs i = 2 i' + h.
        team_sync();
        {
            const float2 tw = s_tw[ln];
            sfor<0, H>([&](auto mc) {
                constexpr int m = decltype(mc)::value;
                const float2 v = u[fft_out<H>(m)];
                buf[ln * (N + 1) + m] = v;
                buf[ln * (N + 1) + H + m] = make_float2(v.x * tw.x - v.y * tw.y, v.x * tw.y + v.y * tw.x);
            });
        }
        team_sync();
        const int cm = ln % H, ch = ln / H;
        sfor<0, H>([&](auto kc) {
            constexpr int k = decltype(kc)::value;
            u[fft_in<H>(k)] = cadd(buf[k * (N + 1) + ch * H + cm], buf[(k + H) * (N + 1) + ch * H + cm]);
        });
        fft<H, 0, +1>(u);  // u[fft_out<H>(i')] = c[2i'+h][2m] + i c[2i'+h][2m+1]
        team_sync();  // |c| overwrites the transform buffer

        unsigned long long key;  // max over the team of (|c|, -index)
        // |c| in the half-shifted frame and the first strict maximum.  H is
        // even, so the shifted row I = 2 I'' + h keeps the parity of i; a
        // lane visits its values in increasing row-major order.
        {
            const int J = (2 * cm + H) % N;
            float bv = -1.0f;  // below every |c|; NaN never compares greater
            int bi = 0;        // row-major index of bv less ch * N + J
            sfor<0, H>([&](auto Ic) {
                constexpr int I2 = decltype(Ic)::value;
                constexpr int ip = (I2 + H / 2) % H;
                const float2 c = u[fft_out<H>(ip)];
                const float v0 = fabsf(c.x), v1 = fabsf(c.y);
                *reinterpret_cast<float2*>(ab + (2 * I2 + ch) * N + J) = make_float2(v0, v1);
                if (v0 > bv) {
                    bv = v0;
                    bi = 2 * I2 * N;
                }
                if (v1 > bv) {
                    bv = v1;
                    bi = 2 * I2 * N + 1;
                }
            });
            // the team's maximum of (|c|, -index): the first strict maximum
            const unsigned idx = (unsigned)(bi + ch * N + J);
            const unsigned khi = bv >= 0.0f ? __float_as_uint(bv) : 0u;
            const unsigned klo = bv >= 0.0f ? 0xffffffffu - idx : 0u;
            if constexpr (kWarp) {
                const unsigned mhi = __reduce_max_sync(tmask, khi);
                key = ((unsigned long long)mhi << 32) | __reduce_max_sync(tmask, khi == mhi ? klo : 0u);
                team_sync();
            } else {
                atomicMax(&s_key[team], ((unsigned long long)khi << 32) | klo);
                team_sync();
                key = s_key[team];
            }
        }

        // integer peak (all lanes decode the same key), then the team stores
        // the peak record for k_fit
        {
            int I, J;
            bool have;
            const float v0 = ab[0];
            if (v0 != v0) {
                // a NaN first element stays the maximum of a sequential scan
                I = 0;
                J = 0;
                have = true;
            } else {
                const unsigned L = 0xffffffffu - (unsigned)(key & 0xffffffffull);
                have = __uint_as_float((unsigned)(key >> 32)) != 0.0f;
                I = have ? (int)(L / N) : N / 2;
                J = have ? (int)(L % N) : N / 2;
            }
            const bool dofit = have && I > 0 && I < N - 1 && J > 0 && J < N - 1;
            if (valid && a.peaks_h) {
                // -h: the 6x6 patch around the peak, 37 words
                float* rec = reinterpret_cast<float*>(a.peaks_h + gi);
                for (int k = ln; k < kHiresPatch * kHiresPatch + 1; k += N) {
                    if (k < kHiresPatch * kHiresPatch) {
                        const int r = I - 2 + k / kHiresPatch, c = J - 2 + k % kHiresPatch;
                        rec[k] = (r >= 0 && r < N && c >= 0 && c < N) ? ab[r * N + c] : 0.f;
                    } else {
                        rec[k] = __uint_as_float(peak_meta(I, J, have));
                    }
                }
            } else if (valid) {
                // 10 words per record; teams narrower than 10 lanes loop
                float* rec = reinterpret_cast<float*>(a.peaks + gi);
                for (int k = ln; k < 10; k += N) {
                    if (k < 9) {
                        rec[k] = dofit ? ab[(I - 1 + k / 3) * N + (J - 1 + k % 3)] : 0.f;
                    } else {
                        rec[9] = __uint_as_float(peak_meta(I, J, dofit));
                    }
                }
            }
        }
    }
}

// Host-side launcher for one box size and shape variant (defined in the
// per-size .cu files); pdl: launch as a programmatic dependent of the
// stream's previous kernel.
template <int N, int V>
cudaError_t launch_window_fp32(const WinArgs& a, int grid, cudaStream_t st, bool pdl);
template <int N, int V>
int window_fp32_blocks_per_sm();

}  // namespace flct
