// flct_gpu.cu -- the C ABI (include/flct_gpu.h) and its host driver.
//
// Host side of the reference's flct main() (source/flct.c:535-1133): the
// parameter derivation is done here on the host exactly as the reference
// does it, everything per pixel runs as CUDA kernels on the context's (or
// the caller's) stream.  No entry point falls back to the CPU.
#include "flct_gpu.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

#include "prepass.cuh"
#include "warp.cuh"
#include "window_fp32.cuh"
#include "window_tc.cuh"

using namespace flct;

namespace {

constexpr double kTol = 1e-2;  // flct.c:278

// ------------------------------------------------------ window kernels --

struct WinEntry {
    int n;
    cudaError_t (*launch)(const WinArgs&, int, cudaStream_t);
    int (*bps)();
};

#define FLCT_WIN(N) {N, &launch_window_fp32<N>, &window_fp32_blocks_per_sm<N>}
const WinEntry kWin[] = {FLCT_WIN(4),  FLCT_WIN(8),  FLCT_WIN(12), FLCT_WIN(16),
                         FLCT_WIN(20), FLCT_WIN(24), FLCT_WIN(28), FLCT_WIN(32),
                         FLCT_WIN(36), FLCT_WIN(40), FLCT_WIN(44), FLCT_WIN(48),
                         FLCT_WIN(52), FLCT_WIN(56), FLCT_WIN(60), FLCT_WIN(64)};
#undef FLCT_WIN

const WinEntry* find_win(int n) {
    for (const auto& e : kWin)
        if (e.n == n) return &e;
    return nullptr;
}

// ------------------------------------------------ parameter derivation --

struct Derived {
    int nsize = 0, n = 0;
    int xoff = 0, yoff = 0;
    int skip = 0;
    bool global = false;
    bool rel_thresh = false;
    int icnt = 0, jcnt = 0;
};

int grid_count(int len, int off, int skip) {
    int c = 0;
    for (int i = 0; i < len; ++i) c += !((i - off) % skip);
    return c;
}

}  // namespace

struct flct_ctx {
    int device = 0;
    int nsm = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev[8] = {};
    char err[512] = {0};
    flct_timing timing{};
    // grow-only device workspace
    struct Buf {
        void* p = nullptr;
        size_t n = 0;
    };
    Buf b_s1, b_s2, b_work, b_ctr, b_r1, b_r2, b_b1, b_b2, b_gvx, b_gvy, b_ix, b_iy;
    Buf b_f1, b_f2, b_vx, b_vy, b_vm, b_aux1, b_aux2, b_means, b_peaks, b_hrow;
    std::vector<Buf*> all() {
        return {&b_s1, &b_s2, &b_work, &b_ctr, &b_r1, &b_r2, &b_b1, &b_b2, &b_gvx, &b_gvy, &b_ix,
                &b_iy, &b_f1, &b_f2, &b_vx, &b_vy, &b_vm, &b_aux1, &b_aux2, &b_means, &b_peaks, &b_hrow, &b_tc};
    }
    int bps[sizeof(kWin) / sizeof(kWin[0])] = {0};
    int bps_tc[2] = {0, 0};
    Buf b_tc;              // tensor-core DFT matrices (b1 32x32, b2 64x64 floats)
    bool tc_ready = false;
    bool pending = false;  // a velocity call's events await collection
};

namespace {

flct_status fail(flct_ctx* c, flct_status s, const char* fmt, ...) {
    if (c) {
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(c->err, sizeof(c->err), fmt, ap);
        va_end(ap);
    }
    return s;
}

#define CK(call)                                                                          \
    do {                                                                                  \
        cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess)                                                            \
            return fail(ctx, e_ == cudaErrorMemoryAllocation ? FLCT_ERR_ALLOC : FLCT_ERR_CUDA, \
                        "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
    } while (0)

flct_status ensure(flct_ctx* ctx, flct_ctx::Buf& b, size_t bytes) {
    if (bytes == 0) bytes = 16;
    if (b.n >= bytes) return FLCT_OK;
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.n = 0;
    CK(cudaMalloc(&b.p, bytes));
    b.n = bytes;
    return FLCT_OK;
}

#define ENSURE(buf, bytes)                                      \
    do {                                                        \
        flct_status s_ = ensure(ctx, (buf), (bytes));           \
        if (s_ != FLCT_OK) return s_;                           \
    } while (0)

flct_status derive(flct_ctx* ctx, const flct_params* p, int nx, int ny, Derived* d) {
    // -s checks at parse time (flct.c:433-452); skip == 0 means no -s
    if (p->skip < 0) return fail(ctx, FLCT_ERR_SKIP_NONPOSITIVE, "flct: skip =%d is zero or negative, fatal", p->skip);
    int pp = p->poffset, qq = p->qoffset;
    if (p->skip > 0 && (std::abs(pp) >= p->skip || std::abs(qq) >= p->skip))
        return fail(ctx, FLCT_ERR_SKIP_OFFSET, "flct: p=%d,q=%d, abs(p) or abs(q) >= skip=%d", pp, qq, p->skip);
    if (pp < 0) pp = p->skip - std::abs(pp);  // flct.c:535-538
    if (qq < 0) qq = p->skip - std::abs(qq);
    d->xoff = qq;  // transposed storage (flct.c:736-745)
    d->yoff = pp;
    d->skip = p->skip;
    if (p->skip >= nx || p->skip >= ny)  // flct.c:559-563
        return fail(ctx, FLCT_ERR_SKIP_TOO_BIG, "flct: skip = %d is too big compared to nx or ny, fatal", p->skip);
    d->global = !(p->sigma > 0.);
    if (!d->global) {
        // sliding box (flct.c:567-580)
        int nt = (int)((int)p->sigma * std::sqrt(std::log(1. / kTol)));
        int ndmin = (nx < ny) ? (((nx / 3) / 2)) * 2 : (((ny / 3) / 2)) * 2;
        d->nsize = ((nt / 2) * 2 < ndmin) ? (nt / 2) * 2 : ndmin;
        if (d->nsize <= 0) return fail(ctx, FLCT_ERR_BOX_SIZE, "flct: error - illegal box size, exiting");
        d->n = 2 * d->nsize;
    }
    d->rel_thresh = !d->global && p->thresh > 0. && p->thresh < 1. && !p->thresh_abs;
    if (p->skip > 0 && p->interpolate) {
        d->icnt = grid_count(d->global ? 1 : nx, d->xoff, p->skip);
        d->jcnt = grid_count(d->global ? 1 : ny, d->yoff, p->skip);
        // interpcc2d reads three grid points per axis; the reference reads
        // outside its arrays for smaller grids, this library refuses them
        if (d->icnt < 3 || d->jcnt < 3)
            return fail(ctx, FLCT_ERR_GRID_TOO_SMALL,
                        "interpolation grid %dx%d is smaller than the 3x3 cubic-convolution stencil",
                        d->icnt, d->jcnt);
    }
    return FLCT_OK;
}

void fill_tables(const flct_params* p, int n, float* gauss, float* filt2) {
    // Gaussian weight by offset d in [-n, n] (flct.c:652-665), separable
    const double sigminv = 1. / p->sigma;
    for (int d = -n; d <= n; ++d) {
        const double ax = sigminv * (double)d;
        gauss[d + n] = (float)std::exp(-ax * ax);
    }
    if (p->filter) {
        // gaussfilt with make_freq wavenumbers (flct.c:1651-1715), squared
        // because the filter multiplies both spectra before conj(A) B
        const double kroll = p->kr * (double)(n / 2);
        for (int k = 0; k < n; ++k) {
            const int kk = (k <= n / 2) ? k : k - n;
            const double ax = (double)kk / kroll;
            filt2[k] = (float)std::exp(-2.0 * ax * ax);
        }
    }
}

float ev_ms(cudaEvent_t a, cudaEvent_t b) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, a, b) != cudaSuccess) ms = 0.f;
    return ms;
}

int win_index(int n) {
    for (size_t k = 0; k < sizeof(kWin) / sizeof(kWin[0]); ++k)
        if (kWin[k].n == n) return (int)k;
    return -1;
}

int win_grid(flct_ctx* ctx, int n) {
    int k = win_index(n);
    if (k < 0) return 0;
    if (ctx->bps[k] == 0) ctx->bps[k] = std::max(1, kWin[k].bps());
    return ctx->nsm * ctx->bps[k];
}

// The tensor-core form's constant matrices, built once per context in FP64:
// b1[c][j] (S1: real input -> half spectrum columns) and b2[n][k] (S2:
// complex DFT along the other axis, re/im by halves, columns in tc_kx order).
flct_status ensure_tc_tables(flct_ctx* ctx) {
    if (ctx->tc_ready) return FLCT_OK;
    ENSURE(ctx->b_tc, (32 * 32 + 64 * 64) * sizeof(float));
    std::vector<float> t(32 * 32 + 64 * 64);
    const double tw = 2.0 * 3.14159265358979323846 / 32.0;
    for (int c = 0; c < 32; ++c)
        for (int j = 0; j < 32; ++j) {
            const double v = (c <= 16) ? std::cos(tw * ((c * j) % 32)) : -std::sin(tw * (((c - 16) * j) % 32));
            t[c * 32 + j] = (float)v;
        }
    float* b2 = t.data() + 32 * 32;
    for (int n = 0; n < 64; ++n)
        for (int k = 0; k < 64; ++k) {
            // output column q holds wavenumber tc_kx(q): mirror pairs adjacent
            const int pp = n / 32, kx = tc_kx(n % 32), pk = k / 32, i = k % 32;
            const double th = tw * ((kx * i) % 32);
            double v;
            if (pk == 0 && pp == 0) v = std::cos(th);
            else if (pk == 1 && pp == 0) v = std::sin(th);
            else if (pk == 0 && pp == 1) v = -std::sin(th);
            else v = std::cos(th);
            b2[n * 64 + k] = (float)v;
        }
    CK(cudaMemcpy(ctx->b_tc.p, t.data(), t.size() * sizeof(float), cudaMemcpyHostToDevice));
    ctx->tc_ready = true;
    return FLCT_OK;
}

// Resolve FLCT_FORM_AUTO and check that the form exists for box size n.
flct_status pick_form(flct_ctx* ctx, int requested, int n, int* form) {
    int f = requested;
    if (f == FLCT_FORM_AUTO) f = (n == 32) ? FLCT_FORM_TC_FP16 : FLCT_FORM_FP32;
    if ((f == FLCT_FORM_TC_FP16 || f == FLCT_FORM_TC_BF16) && n != 32)
        return fail(ctx, FLCT_ERR_UNSUPPORTED, "the tensor-core form is built for 32x32 boxes (sigma 8); box %d", n);
    if (f < 0 || f > FLCT_FORM_TC_BF16) return fail(ctx, FLCT_ERR_ARG, "unknown window form %d", requested);
    *form = f;
    return FLCT_OK;
}

// Launch the window kernel of the chosen form on the prepared work list.
flct_status launch_windows(flct_ctx* ctx, int form, const WinEntry* we, int n, const WinArgs& wa, unsigned* status,
                           cudaStream_t st) {
    if (form == FLCT_FORM_FP32) {
        CK(we->launch(wa, win_grid(ctx, n), st));
        return FLCT_OK;
    }
    flct_status s = ensure_tc_tables(ctx);
    if (s != FLCT_OK) return s;
    TcArgs ta{};
    ta.s1 = wa.s1;
    ta.s2 = wa.s2;
    ta.means = wa.means;
    ta.work = wa.work;
    ta.nwork = wa.nwork;
    ta.nx = wa.nx;
    ta.ny = wa.ny;
    ta.nsize = wa.nsize;
    ta.direct = wa.direct;
    ta.use_filter = wa.use_filter;
    ta.peaks = wa.peaks;
    ta.b1 = (const float*)ctx->b_tc.p;
    ta.b2 = (const float*)ctx->b_tc.p + 32 * 32;
    ta.status = status;
    for (int k = 0; k < 2 * kMaxBox + 1; ++k) ta.gauss[k] = wa.gauss[k];
    for (int k = 0; k < kMaxBox; ++k) ta.filt2[k] = wa.filt2[k];
    const int which = (form == FLCT_FORM_TC_BF16) ? 1 : 0;
    if (ctx->bps_tc[which] == 0)
        ctx->bps_tc[which] = std::max(1, which ? window_tc32_blocks_per_sm<__nv_bfloat16>()
                                               : window_tc32_blocks_per_sm<__half>());
    const int grid = ctx->nsm * ctx->bps_tc[which];
    if (which) CK(launch_window_tc32<__nv_bfloat16>(ta, grid, st));
    else CK(launch_window_tc32<__half>(ta, grid, st));
    return FLCT_OK;
}

}  // namespace

// ===================================================================== ABI

extern "C" {

const char* flct_gpu_version(void) { return "0.1.0 sm_103a"; }

const char* flct_gpu_status_string(flct_status s) {
    switch (s) {
        case FLCT_OK: return "ok";
        case FLCT_ERR_ARG: return "invalid argument";
        case FLCT_ERR_SKIP_NONPOSITIVE: return "skip is zero or negative";
        case FLCT_ERR_SKIP_OFFSET: return "abs(p) or abs(q) >= skip";
        case FLCT_ERR_SKIP_TOO_BIG: return "skip is too big compared to nx or ny";
        case FLCT_ERR_BOX_SIZE: return "illegal box size";
        case FLCT_ERR_GRID_TOO_SMALL: return "interpolation grid smaller than 3x3";
        case FLCT_ERR_NO_DEVICE: return "no usable CUDA device";
        case FLCT_ERR_CUDA: return "CUDA error";
        case FLCT_ERR_ALLOC: return "allocation failed";
        case FLCT_ERR_UNSUPPORTED: return "not supported on the GPU path";
        case FLCT_ERR_WARP_DIMS: return "bad shift arrays";
        case FLCT_ERR_TIMEOUT: return "device wait timed out";
    }
    return "unknown status";
}

flct_status flct_gpu_create(int device, flct_ctx** out) {
    if (!out) return FLCT_ERR_ARG;
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count <= 0 || device < 0 || device >= count) {
        cudaGetLastError();
        return FLCT_ERR_NO_DEVICE;
    }
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return FLCT_ERR_NO_DEVICE;
    // the kernels are compiled for sm_103a only
    if (!(prop.major == 10 && prop.minor == 3)) return FLCT_ERR_NO_DEVICE;
    flct_ctx* ctx = new (std::nothrow) flct_ctx();
    if (!ctx) return FLCT_ERR_ALLOC;
    ctx->device = device;
    ctx->nsm = prop.multiProcessorCount;
    if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete ctx;
        return FLCT_ERR_CUDA;
    }
    for (auto& e : ctx->ev)
        if (cudaEventCreate(&e) != cudaSuccess) {
            flct_gpu_destroy(ctx);
            return FLCT_ERR_CUDA;
        }
    *out = ctx;
    return FLCT_OK;
}

void flct_gpu_destroy(flct_ctx* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    for (auto* b : ctx->all())
        if (b->p) cudaFree(b->p);
    for (auto& e : ctx->ev)
        if (e) cudaEventDestroy(e);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

const char* flct_gpu_last_error(const flct_ctx* ctx) { return ctx ? ctx->err : "no context"; }

static flct_status collect_timing(flct_ctx* ctx);

flct_status flct_gpu_last_timing(const flct_ctx* cctx, flct_timing* t) {
    if (!cctx || !t) return FLCT_ERR_ARG;
    flct_ctx* ctx = const_cast<flct_ctx*>(cctx);
    flct_status s = FLCT_OK;
    if (ctx->pending) s = collect_timing(ctx);
    *t = ctx->timing;
    return s;
}

long long flct_gpu_output_len(const flct_params* p, int nx, int ny) {
    if (!p || nx < 1 || ny < 1) return 0;
    return (p->sigma > 0.) ? (long long)nx * ny : 1;
}

flct_status flct_gpu_velocity_device(flct_ctx* ctx, const flct_params* p, const double* d_f1,
                                     const double* d_f2, int nx, int ny, double* d_vx, double* d_vy,
                                     double* d_vm, void* stream) {
    if (!ctx) return FLCT_ERR_ARG;
    if (!p || !d_f1 || !d_f2 || !d_vx || !d_vy || !d_vm || nx < 1 || ny < 1)
        return fail(ctx, FLCT_ERR_ARG, "null pointer or empty image (%d x %d)", nx, ny);
    if ((long long)nx * ny >= (1ll << 31)) return fail(ctx, FLCT_ERR_UNSUPPORTED, "image larger than 2^31 pixels");
    CK(cudaSetDevice(ctx->device));
    cudaStream_t st = (cudaStream_t)stream;  // NULL: the CUDA default stream
    Derived d;
    flct_status s = derive(ctx, p, nx, ny, &d);
    if (s != FLCT_OK) return s;
    if (d.global) return fail(ctx, FLCT_ERR_UNSUPPORTED, "sigma <= 0 (global-shift mode) is not available on the GPU path yet");
    if (p->hires) return fail(ctx, FLCT_ERR_UNSUPPORTED, "-h (hires) is not available on the GPU path yet");
    if (p->filter && !(p->kr > 0.)) return fail(ctx, FLCT_ERR_UNSUPPORTED, "-k with kr <= 0 is not available on the GPU path");
    const int n = d.n;
    const WinEntry* we = find_win(n);
    if (!we) return fail(ctx, FLCT_ERR_UNSUPPORTED, "box size %d (sigma %g) has no GPU kernel", n, p->sigma);
    int form = FLCT_FORM_FP32;
    s = pick_form(ctx, p->form, n, &form);
    if (s != FLCT_OK) return s;

    const size_t npx = (size_t)nx * ny;
    const int W = ny - n + 1, H = nx - n + 1;
    ENSURE(ctx->b_s1, npx * sizeof(float2));
    ENSURE(ctx->b_s2, npx * sizeof(float2));
    ENSURE(ctx->b_work, npx * sizeof(int));
    ENSURE(ctx->b_ctr, 64);
    ENSURE(ctx->b_r1, (size_t)nx * W * sizeof(double));
    ENSURE(ctx->b_r2, (size_t)nx * W * sizeof(double));
    ENSURE(ctx->b_b1, (size_t)H * W * sizeof(double));
    ENSURE(ctx->b_b2, (size_t)H * W * sizeof(double));
    ENSURE(ctx->b_means, npx * sizeof(float4));
    ENSURE(ctx->b_peaks, npx * sizeof(PeakRec));
    const bool interp = d.skip > 0 && p->interpolate;
    if (interp) {
        ENSURE(ctx->b_hrow, (size_t)(d.icnt + 2) * ny * (2 * sizeof(double) + 1));
        ENSURE(ctx->b_gvx, (size_t)d.icnt * d.jcnt * sizeof(double));
        ENSURE(ctx->b_gvy, (size_t)d.icnt * d.jcnt * sizeof(double));
        ENSURE(ctx->b_ix, (size_t)nx * (4 * sizeof(double) + sizeof(int) + 1) + 64);
        ENSURE(ctx->b_iy, (size_t)ny * (4 * sizeof(double) + sizeof(int) + 1) + 64);
    }
    // counters: [0] nwork (int), [1] status (u32), [8..23] absmax (2 x u64), [24..31] thresh
    unsigned char* ctr = (unsigned char*)ctx->b_ctr.p;
    int* d_nwork = (int*)ctr;
    unsigned* d_status = (unsigned*)(ctr + 4);
    unsigned long long* d_absmax = (unsigned long long*)(ctr + 8);
    double* d_thr = (double*)(ctr + 24);

    int launches = 0;
    CK(cudaEventRecord(ctx->ev[0], st));
    CK(cudaMemsetAsync(ctr, 0, 32, st));
    if (d.rel_thresh) {
        k_absmax<<<ctx->nsm * 4, 256, 0, st>>>(d_f1, d_f2, (long)npx, d_absmax);
        k_thresh_final<<<1, 1, 0, st>>>(d_f1, d_f2, d_absmax, p->thresh, d_thr);
        launches += 2;
    }
    ClassifyArgs ca{};
    ca.f1 = d_f1;
    ca.f2 = d_f2;
    ca.nx = nx;
    ca.ny = ny;
    ca.thr_val = p->thresh;
    ca.thr_ptr = d.rel_thresh ? d_thr : nullptr;
    ca.skip = d.skip;
    ca.xoff = d.xoff;
    ca.yoff = d.yoff;
    ca.interpolate = interp;
    ca.jcnt = d.jcnt;
    ca.s1 = (float2*)ctx->b_s1.p;
    ca.s2 = (float2*)ctx->b_s2.p;
    ca.work = (int*)ctx->b_work.p;
    ca.nwork = d_nwork;
    ca.vx = d_vx;
    ca.vy = d_vy;
    ca.vm = d_vm;
    ca.gvx = interp ? (double*)ctx->b_gvx.p : nullptr;
    ca.gvy = interp ? (double*)ctx->b_gvy.p : nullptr;
    ca.status = d_status;
    {
        long blocks = std::min<long>((long)(npx + 255) / 256, (long)ctx->nsm * 8);
        k_classify<<<(int)std::max(1l, blocks), 256, 0, st>>>(ca);
        ++launches;
    }
    {
        const int nseg = (W + kSeg - 1) / kSeg;
        long t = (long)nx * nseg;
        k_rowsum<<<(int)((t + 127) / 128), 128, 0, st>>>(d_f1, d_f2, nx, ny, n, (double*)ctx->b_r1.p,
                                                         (double*)ctx->b_r2.p);
        const int hseg = (H + kSeg - 1) / kSeg;
        t = (long)W * hseg;
        k_colsum<<<(int)((t + 127) / 128), 128, 0, st>>>((double*)ctx->b_r1.p, (double*)ctx->b_r2.p, nx, W, n,
                                                         (double*)ctx->b_b1.p, (double*)ctx->b_b2.p);
        launches += 2;
    }
    {
        // FP64 local means per work item, one window per lane
        MeansArgs ma{};
        ma.work = (const int*)ctx->b_work.p;
        ma.nwork = d_nwork;
        ma.nx = nx;
        ma.ny = ny;
        ma.nsize = d.nsize;
        ma.bsw = W;
        ma.bs1 = (const double*)ctx->b_b1.p;
        ma.bs2 = (const double*)ctx->b_b2.p;
        ma.inv_n2 = 1. / ((double)n * n);
        ma.means = (float4*)ctx->b_means.p;
        long blocks = std::min<long>((long)(npx + 255) / 256, (long)ctx->nsm * 8);
        k_means<<<(int)std::max(1l, blocks), 256, 0, st>>>(ma);
        ++launches;
    }
    CK(cudaGetLastError());
    CK(cudaEventRecord(ctx->ev[1], st));

    WinArgs wa{};
    fill_tables(p, n, wa.gauss, wa.filt2);
    wa.use_filter = p->filter;
    wa.s1 = (const float2*)ctx->b_s1.p;
    wa.s2 = (const float2*)ctx->b_s2.p;
    wa.means = (const float4*)ctx->b_means.p;
    wa.work = (const int*)ctx->b_work.p;
    wa.nwork = d_nwork;
    wa.nx = nx;
    wa.ny = ny;
    wa.nsize = d.nsize;
    wa.peaks = (PeakRec*)ctx->b_peaks.p;
    s = launch_windows(ctx, form, we, n, wa, d_status, st);
    if (s != FLCT_OK) return s;
    ++launches;
    CK(cudaEventRecord(ctx->ev[2], st));
    {
        FitArgs fa{};
        fa.work = (const int*)ctx->b_work.p;
        fa.nwork = d_nwork;
        fa.peaks = (const PeakRec*)ctx->b_peaks.p;
        fa.n = n;
        fa.ny = ny;
        fa.deltinv = 1. / p->deltat;  // flct.c:343
        fa.deltas = p->deltas;
        fa.skip = d.skip > 0 ? d.skip : 1;
        fa.xoff = d.xoff;
        fa.yoff = d.yoff;
        fa.jcnt = d.jcnt;
        fa.vx = d_vx;
        fa.vy = d_vy;
        fa.vm = d_vm;
        fa.gvx = ca.gvx;
        fa.gvy = ca.gvy;
        long blocks = std::min<long>((long)(npx + 127) / 128, (long)ctx->nsm * 8);
        k_fit<<<(int)std::max(1l, blocks), 128, 0, st>>>(fa);
        ++launches;
    }
    CK(cudaGetLastError());
    CK(cudaEventRecord(ctx->ev[7], st));

    if (interp) {
        unsigned char* ix = (unsigned char*)ctx->b_ix.p;
        unsigned char* iy = (unsigned char*)ctx->b_iy.p;
        double* wx = (double*)ix;
        int* zx = (int*)(ix + (size_t)nx * 4 * sizeof(double));
        unsigned char* okx = ix + (size_t)nx * (4 * sizeof(double) + sizeof(int));
        double* wy = (double*)iy;
        int* zy = (int*)(iy + (size_t)ny * 4 * sizeof(double));
        unsigned char* oky = iy + (size_t)ny * (4 * sizeof(double) + sizeof(int));
        k_interp_axis<<<(nx + 127) / 128, 128, 0, st>>>(nx, d.icnt, d.xoff, d.skip, nullptr, zx, wx, okx);
        k_interp_axis<<<(ny + 127) / 128, 128, 0, st>>>(ny, d.jcnt, d.yoff, d.skip, nullptr, zy, wy, oky);
        InterpArgs ia{};
        ia.nx = nx;
        ia.ny = ny;
        ia.skip = d.skip;
        ia.xoff = d.xoff;
        ia.yoff = d.yoff;
        ia.gx = d.icnt;
        ia.gy = d.jcnt;
        ia.gvx = ca.gvx;
        ia.gvy = ca.gvy;
        ia.zx = zx;
        ia.wx = wx;
        ia.okx = okx;
        ia.zy = zy;
        ia.wy = wy;
        ia.oky = oky;
        const size_t hn = (size_t)(d.icnt + 2) * ny;
        ia.hx = (double*)ctx->b_hrow.p;
        ia.hy = ia.hx + hn;
        ia.hbad = (unsigned char*)(ia.hy + hn);
        ia.vx = d_vx;
        ia.vy = d_vy;
        ia.vm = d_vm;
        long rblocks = std::min<long>((long)(hn + 255) / 256, (long)ctx->nsm * 8);
        k_interp_rows<<<(int)std::max(1l, rblocks), 256, 0, st>>>(ia);
        long blocks = std::min<long>((long)(npx + 255) / 256, (long)ctx->nsm * 16);
        k_interp<<<(int)std::max(1l, blocks), 256, 0, st>>>(ia);
        launches += 4;
        CK(cudaGetLastError());
    }
    CK(cudaEventRecord(ctx->ev[3], st));
    ctx->timing = flct_timing{};
    ctx->timing.launches = launches;
    ctx->timing.box = n;
    ctx->timing.form = form;
    ctx->pending = true;
    return FLCT_OK;
}

// Waits for the last velocity call's final event, then fills ctx->timing
// (event times, windows computed) and reports device-side status bits.
static flct_status collect_timing(flct_ctx* ctx) {
    ctx->pending = false;
    CK(cudaEventSynchronize(ctx->ev[3]));
    unsigned char* ctr = (unsigned char*)ctx->b_ctr.p;
    int nwork = 0;
    unsigned status = 0;
    CK(cudaMemcpy(&nwork, ctr, sizeof(int), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(&status, ctr + 4, sizeof(unsigned), cudaMemcpyDeviceToHost));
    ctx->timing.windows = nwork;
    ctx->timing.ms_prepass = ev_ms(ctx->ev[0], ctx->ev[1]);
    ctx->timing.ms_window = ev_ms(ctx->ev[1], ctx->ev[2]);
    ctx->timing.ms_fit = ev_ms(ctx->ev[2], ctx->ev[7]);
    ctx->timing.ms_interp = ev_ms(ctx->ev[7], ctx->ev[3]);
    ctx->timing.ms_total = ev_ms(ctx->ev[0], ctx->ev[3]);
    if (status & kStatusRange)
        return fail(ctx, FLCT_ERR_UNSUPPORTED, "an input magnitude exceeds the FP32 range of the GPU kernels");
    if (status & kStatusTimeout)
        return fail(ctx, FLCT_ERR_TIMEOUT, "a tensor-core stage did not complete within its wait limit");
    return FLCT_OK;
}

flct_status flct_gpu_velocity(flct_ctx* ctx, const flct_params* p, const double* f1, const double* f2,
                              int nx, int ny, double* vx, double* vy, double* vm) {
    if (!ctx) return FLCT_ERR_ARG;
    if (!p || !f1 || !f2 || !vx || !vy || !vm || nx < 1 || ny < 1)
        return fail(ctx, FLCT_ERR_ARG, "null pointer or empty image (%d x %d)", nx, ny);
    CK(cudaSetDevice(ctx->device));
    const size_t npx = (size_t)nx * ny;
    const long long nout = flct_gpu_output_len(p, nx, ny);
    ENSURE(ctx->b_f1, npx * sizeof(double));
    ENSURE(ctx->b_f2, npx * sizeof(double));
    ENSURE(ctx->b_vx, npx * sizeof(double));
    ENSURE(ctx->b_vy, npx * sizeof(double));
    ENSURE(ctx->b_vm, npx * sizeof(double));
    cudaStream_t st = ctx->stream;
    CK(cudaEventRecord(ctx->ev[4], st));
    CK(cudaMemcpyAsync(ctx->b_f1.p, f1, npx * sizeof(double), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(ctx->b_f2.p, f2, npx * sizeof(double), cudaMemcpyHostToDevice, st));
    CK(cudaEventRecord(ctx->ev[5], st));
    flct_status s = flct_gpu_velocity_device(ctx, p, (const double*)ctx->b_f1.p, (const double*)ctx->b_f2.p,
                                             nx, ny, (double*)ctx->b_vx.p, (double*)ctx->b_vy.p,
                                             (double*)ctx->b_vm.p, st);
    if (s != FLCT_OK) {
        cudaStreamSynchronize(st);
        return s;
    }
    CK(cudaMemcpyAsync(vx, ctx->b_vx.p, nout * sizeof(double), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(vy, ctx->b_vy.p, nout * sizeof(double), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(vm, ctx->b_vm.p, nout * sizeof(double), cudaMemcpyDeviceToHost, st));
    CK(cudaEventRecord(ctx->ev[6], st));
    CK(cudaStreamSynchronize(st));
    s = collect_timing(ctx);
    ctx->timing.ms_h2d = ev_ms(ctx->ev[4], ctx->ev[5]);
    ctx->timing.ms_d2h = ev_ms(ctx->ev[3], ctx->ev[6]);
    return s;
}

flct_status flct_gpu_cross_cor_batch(flct_ctx* ctx, const double* g1, const double* g2, int n, int nwin,
                                     int filter, double kr, int form, double* shiftx, double* shifty) {
    if (!ctx) return FLCT_ERR_ARG;
    if (!g1 || !g2 || !shiftx || !shifty || nwin < 0 || n < 1)
        return fail(ctx, FLCT_ERR_ARG, "null pointer or bad window size");
    if (nwin == 0) return FLCT_OK;
    const WinEntry* we = find_win(n);
    if (!we) return fail(ctx, FLCT_ERR_UNSUPPORTED, "window size %d has no GPU kernel", n);
    int fsel = FLCT_FORM_FP32;
    {
        flct_status fs = pick_form(ctx, form, n, &fsel);
        if (fs != FLCT_OK) return fs;
    }
    if (filter && !(kr > 0.)) return fail(ctx, FLCT_ERR_UNSUPPORTED, "-k with kr <= 0 is not available on the GPU path");
    if ((long long)nwin * n * n >= (1ll << 31)) return fail(ctx, FLCT_ERR_UNSUPPORTED, "too many windows in one batch");
    CK(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    const size_t npx = (size_t)nwin * n * n;
    // the stacked windows form an (nwin*n) x n "image"; each window is its
    // own box with zero mean and unit Gaussian
    ENSURE(ctx->b_f1, npx * sizeof(double));
    ENSURE(ctx->b_f2, npx * sizeof(double));
    ENSURE(ctx->b_s1, npx * sizeof(float2));
    ENSURE(ctx->b_s2, npx * sizeof(float2));
    ENSURE(ctx->b_work, (size_t)nwin * sizeof(int));
    ENSURE(ctx->b_ctr, 64);
    ENSURE(ctx->b_vx, (size_t)nwin * sizeof(double));
    ENSURE(ctx->b_vy, (size_t)nwin * sizeof(double));
    CK(cudaMemcpyAsync(ctx->b_f1.p, g1, npx * sizeof(double), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(ctx->b_f2.p, g2, npx * sizeof(double), cudaMemcpyHostToDevice, st));
    // all pixels are "computed": classify with a -inf threshold builds the
    // split arrays; the work list is then overwritten by the window indices
    std::vector<int> idx(nwin);
    for (int w = 0; w < nwin; ++w) idx[w] = w * n * n;  // pixel (w*n, 0)
    CK(cudaMemcpyAsync(ctx->b_work.p, idx.data(), nwin * sizeof(int), cudaMemcpyHostToDevice, st));
    unsigned char* ctr = (unsigned char*)ctx->b_ctr.p;
    CK(cudaMemsetAsync(ctr, 0, 64, st));  // includes the discarded list's counter at +32
    ClassifyArgs ca{};
    ca.f1 = (const double*)ctx->b_f1.p;
    ca.f2 = (const double*)ctx->b_f2.p;
    ca.nx = nwin * n;
    ca.ny = n;
    ca.thr_val = -INFINITY;
    ca.s1 = (float2*)ctx->b_s1.p;
    ca.s2 = (float2*)ctx->b_s2.p;
    ENSURE(ctx->b_aux2, npx * sizeof(int) + 64);
    ca.work = (int*)ctx->b_aux2.p;  // discarded list
    ca.nwork = (int*)(ctr + 32);
    ca.vx = ca.vy = ca.vm = nullptr;
    ca.status = (unsigned*)(ctr + 4);
    CK(cudaEventRecord(ctx->ev[0], st));
    k_classify<<<ctx->nsm * 8, 256, 0, st>>>(ca);
    CK(cudaMemcpyAsync(ctr, &nwin, sizeof(int), cudaMemcpyHostToDevice, st));
    CK(cudaGetLastError());
    CK(cudaEventRecord(ctx->ev[1], st));
    WinArgs wa{};
    if (filter) {
        flct_params fp{};
        fp.filter = 1;
        fp.kr = kr;
        fp.sigma = 1.0;
        fill_tables(&fp, n, wa.gauss, wa.filt2);
    }
    for (int k = 0; k <= 2 * n; ++k) wa.gauss[k] = 1.0f;
    wa.use_filter = filter;
    wa.s1 = (const float2*)ctx->b_s1.p;
    wa.s2 = (const float2*)ctx->b_s2.p;
    wa.means = nullptr;
    wa.work = (const int*)ctx->b_work.p;
    wa.nwork = (const int*)ctr;
    wa.nx = nwin * n;
    wa.ny = n;
    wa.nsize = n / 2;
    wa.direct = 1;
    ENSURE(ctx->b_peaks, (size_t)nwin * sizeof(PeakRec));
    wa.peaks = (PeakRec*)ctx->b_peaks.p;
    {
        flct_status ls = launch_windows(ctx, fsel, we, n, wa, (unsigned*)(ctr + 4), st);
        if (ls != FLCT_OK) return ls;
    }
    CK(cudaEventRecord(ctx->ev[2], st));
    FitArgs fa{};
    fa.work = (const int*)ctx->b_work.p;
    fa.nwork = (const int*)ctr;
    fa.peaks = (const PeakRec*)ctx->b_peaks.p;
    fa.n = n;
    fa.ny = n;
    fa.skip = 1;
    fa.shx = (double*)ctx->b_vx.p;
    fa.shy = (double*)ctx->b_vy.p;
    k_fit<<<(int)std::max(1, std::min((nwin + 127) / 128, ctx->nsm * 8)), 128, 0, st>>>(fa);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(shiftx, ctx->b_vx.p, nwin * sizeof(double), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(shifty, ctx->b_vy.p, nwin * sizeof(double), cudaMemcpyDeviceToHost, st));
    CK(cudaEventRecord(ctx->ev[3], st));
    CK(cudaStreamSynchronize(st));
    ctx->timing = flct_timing{};
    ctx->timing.windows = nwin;
    ctx->timing.launches = 3;
    ctx->timing.box = n;
    ctx->timing.form = fsel;
    ctx->timing.ms_window = ev_ms(ctx->ev[1], ctx->ev[2]);
    {
        unsigned status = 0;
        CK(cudaMemcpy(&status, ctr + 4, sizeof(unsigned), cudaMemcpyDeviceToHost));
        if (status & kStatusTimeout)
            return fail(ctx, FLCT_ERR_TIMEOUT, "a tensor-core stage did not complete within its wait limit");
    }
    ctx->timing.ms_total = ev_ms(ctx->ev[0], ctx->ev[2]);
    return FLCT_OK;
}

flct_status flct_gpu_interpcc2d(flct_ctx* ctx, const double* fdata, double xmiss, int nx, int ny,
                                const double* xwant, int nxi, const double* ywant, int nyi, double* out) {
    if (!ctx) return FLCT_ERR_ARG;
    if (!fdata || !xwant || !ywant || !out || nxi < 0 || nyi < 0)
        return fail(ctx, FLCT_ERR_ARG, "null pointer or negative size");
    if (nx < 3 || ny < 3)
        return fail(ctx, FLCT_ERR_GRID_TOO_SMALL, "interpcc2d needs at least 3x3 data points (got %dx%d)", nx, ny);
    if (nxi == 0 || nyi == 0) return FLCT_OK;
    CK(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    const size_t nf = (size_t)nx * ny, no = (size_t)nxi * nyi;
    ENSURE(ctx->b_gvx, nf * sizeof(double));
    ENSURE(ctx->b_vx, no * sizeof(double));
    ENSURE(ctx->b_ix, (size_t)nxi * (4 * sizeof(double) + sizeof(int) + 1 + sizeof(double)) + 64);
    ENSURE(ctx->b_iy, (size_t)nyi * (4 * sizeof(double) + sizeof(int) + 1 + sizeof(double)) + 64);
    unsigned char* ix = (unsigned char*)ctx->b_ix.p;
    unsigned char* iy = (unsigned char*)ctx->b_iy.p;
    double* xw = (double*)ix;
    double* wx = xw + nxi;
    int* zx = (int*)(wx + (size_t)nxi * 4);
    unsigned char* okx = (unsigned char*)(zx + nxi);
    double* yw = (double*)iy;
    double* wy = yw + nyi;
    int* zy = (int*)(wy + (size_t)nyi * 4);
    unsigned char* oky = (unsigned char*)(zy + nyi);
    CK(cudaMemcpyAsync(ctx->b_gvx.p, fdata, nf * sizeof(double), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(xw, xwant, nxi * sizeof(double), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(yw, ywant, nyi * sizeof(double), cudaMemcpyHostToDevice, st));
    CK(cudaEventRecord(ctx->ev[0], st));
    k_interp_axis<<<(nxi + 127) / 128, 128, 0, st>>>(nxi, nx, 0, 1, xw, zx, wx, okx);
    k_interp_axis<<<(nyi + 127) / 128, 128, 0, st>>>(nyi, ny, 0, 1, yw, zy, wy, oky);
    long blocks = std::min<long>((long)(no + 255) / 256, (long)ctx->nsm * 16);
    k_interp_general<<<(int)std::max(1l, blocks), 256, 0, st>>>((const double*)ctx->b_gvx.p, nx, ny, xmiss, zx, wx,
                                                                okx, nxi, zy, wy, oky, nyi, (double*)ctx->b_vx.p);
    CK(cudaGetLastError());
    CK(cudaEventRecord(ctx->ev[1], st));
    CK(cudaMemcpyAsync(out, ctx->b_vx.p, no * sizeof(double), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    ctx->timing = flct_timing{};
    ctx->timing.launches = 3;
    ctx->timing.ms_interp = ev_ms(ctx->ev[0], ctx->ev[1]);
    ctx->timing.ms_total = ctx->timing.ms_interp;
    return FLCT_OK;
}

static flct_status warp_check(flct_ctx* ctx, const double* arr, const double* out, int nx, int ny) {
    if (!arr || !out || nx < 1 || ny < 1) return fail(ctx, FLCT_ERR_ARG, "null pointer or empty image");
    if (nx > kWarpMaxAxis || ny > kWarpMaxAxis)
        return fail(ctx, FLCT_ERR_UNSUPPORTED, "warp axes are limited to %d points", kWarpMaxAxis);
    if ((long long)nx * ny >= (1ll << 31)) return fail(ctx, FLCT_ERR_UNSUPPORTED, "image larger than 2^31 pixels");
    return FLCT_OK;
}

flct_status flct_gpu_shift_frac2d(flct_ctx* ctx, const double* arr, double delx, double dely, double* out,
                                  int nx, int ny, int transp) {
    if (!ctx) return FLCT_ERR_ARG;
    flct_status s = warp_check(ctx, arr, out, nx, ny);
    if (s != FLCT_OK) return s;
    CK(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    const size_t n = (size_t)nx * ny;
    ENSURE(ctx->b_f1, n * sizeof(double));
    ENSURE(ctx->b_vx, n * sizeof(double));
    ENSURE(ctx->b_s1, n * sizeof(float2));
    ENSURE(ctx->b_s2, n * sizeof(float2));
    ENSURE(ctx->b_aux1, (size_t)(nx + ny) * sizeof(float2) + 64);
    ENSURE(ctx->b_aux2, (size_t)2 * std::max(nx, ny) * sizeof(double2));
    float2* sx = (float2*)ctx->b_aux1.p;
    float2* sy = sx + nx;
    // warp.c:811-820: shifts normalised by the axis lengths; transp swaps them
    const double dxarg = transp ? -dely / ((double)nx) : -delx / ((double)nx);
    const double dyarg = transp ? -delx / ((double)ny) : -dely / ((double)ny);
    CK(cudaMemcpyAsync(ctx->b_f1.p, arr, n * sizeof(double), cudaMemcpyHostToDevice, st));
    CK(cudaEventRecord(ctx->ev[0], st));
    CK(launch_shift_vector(nx, dxarg, (double2*)ctx->b_aux2.p, sx, st));
    CK(launch_shift_vector(ny, dyarg, (double2*)ctx->b_aux2.p, sy, st));
    CK(launch_axis_fast(0, true, ctx->b_f1.p, nx, ny, sy, (float2*)ctx->b_s1.p, st));
    CK(launch_axis_slow(0, (const float2*)ctx->b_s1.p, ny, nx, sx, (float2*)ctx->b_s2.p, st));
    CK(launch_real_part((const float2*)ctx->b_s2.p, (long)n, (double*)ctx->b_vx.p, st));
    CK(cudaEventRecord(ctx->ev[1], st));
    CK(cudaMemcpyAsync(out, ctx->b_vx.p, n * sizeof(double), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    ctx->timing = flct_timing{};
    ctx->timing.launches = 7;
    ctx->timing.ms_total = ev_ms(ctx->ev[0], ctx->ev[1]);
    return FLCT_OK;
}

flct_status flct_gpu_warp_frac2d(flct_ctx* ctx, const double* arr, const double* delx, const double* dely,
                                 double* out, int nx, int ny, int transp) {
    if (!ctx) return FLCT_ERR_ARG;
    flct_status s = warp_check(ctx, arr, out, nx, ny);
    if (s != FLCT_OK) return s;
    if (!delx || !dely) return fail(ctx, FLCT_ERR_ARG, "null shift array");
    CK(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    const size_t n = (size_t)nx * ny;
    ENSURE(ctx->b_f1, n * sizeof(double));
    ENSURE(ctx->b_f2, n * sizeof(double));
    ENSURE(ctx->b_vy, n * sizeof(double));
    ENSURE(ctx->b_vx, n * sizeof(double));
    ENSURE(ctx->b_s1, n * sizeof(float2));
    ENSURE(ctx->b_s2, n * sizeof(float2));
    ENSURE(ctx->b_means, n * sizeof(float4));
    ENSURE(ctx->b_aux1, (size_t)(nx + ny) * sizeof(float2) + 64);
    float2* twx = (float2*)ctx->b_aux1.p;
    float2* twy = twx + nx;
    CK(cudaMemcpyAsync(ctx->b_f1.p, arr, n * sizeof(double), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(ctx->b_f2.p, delx, n * sizeof(double), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(ctx->b_vy.p, dely, n * sizeof(double), cudaMemcpyHostToDevice, st));
    CK(cudaEventRecord(ctx->ev[0], st));
    // F = forward DFT of the image (warp.c:899-934)
    CK(launch_twiddles(nx, -1, twx, st));
    CK(launch_twiddles(ny, -1, twy, st));
    CK(launch_axis_fast(1, true, ctx->b_f1.p, nx, ny, twy, (float2*)ctx->b_s1.p, st));
    CK(launch_axis_slow(1, (const float2*)ctx->b_s1.p, ny, nx, twx, (float2*)ctx->b_s2.p, st));
    CK(launch_warp_phase((const double*)ctx->b_f2.p, (const double*)ctx->b_vy.p, nx, ny, transp,
                         (float4*)ctx->b_means.p, st));
    CK(cudaEventRecord(ctx->ev[1], st));
    CK(launch_warp_sum((const float2*)ctx->b_s2.p, (const float4*)ctx->b_means.p, nx, ny, (double*)ctx->b_vx.p, st));
    CK(cudaEventRecord(ctx->ev[2], st));
    CK(cudaMemcpyAsync(out, ctx->b_vx.p, n * sizeof(double), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    ctx->timing = flct_timing{};
    ctx->timing.launches = 6;
    ctx->timing.ms_prepass = ev_ms(ctx->ev[0], ctx->ev[1]);
    ctx->timing.ms_window = ev_ms(ctx->ev[1], ctx->ev[2]);
    ctx->timing.ms_total = ev_ms(ctx->ev[0], ctx->ev[2]);
    return FLCT_OK;
}

flct_status flct_gpu_velocity_batch(flct_ctx* ctx, int npairs, const flct_pair* pairs, void* stream) {
    (void)npairs; (void)pairs; (void)stream;
    if (!ctx) return FLCT_ERR_ARG;
    return fail(ctx, FLCT_ERR_UNSUPPORTED, "batched velocity is not available yet");
}

}  // extern "C"
