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
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <type_traits>
#include <vector>

#include "global.cuh"
#include "prepass.cuh"
#include "warp.cuh"
#include "window_fp32.cuh"
#include "window_big.cuh"
#include "window_tc.cuh"

using namespace flct;

namespace {

constexpr double kTol = 1e-2;  // flct.c:278

// ------------------------------------------------------ window kernels --

// The FP32 form per box size: launchers, occupancy and windows per CTA
// iteration of its two launch shapes (WinShape<N, V>, V = 0 default).
struct WinEntry {
    int n;
    cudaError_t (*launch[2])(const WinArgs&, int, cudaStream_t, bool);
    int (*bps[2])();
    int teams[2];
};

#define FLCT_WIN(N)                                                                  \
    {N,                                                                              \
     {&launch_window_fp32<N, 0>, &launch_window_fp32<N, 1>},                         \
     {&window_fp32_blocks_per_sm<N, 0>, &window_fp32_blocks_per_sm<N, 1>},           \
     {WinShape<N, 0>::TEAMS, WinShape<N, 1>::TEAMS}}
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

// The tensor-core form per box size: launchers and occupancy per split type
// (0 = FP16, 1 = BF16).
struct TcEntry {
    int n;
    cudaError_t (*launch[2])(const TcArgs&, int, cudaStream_t, bool);
    int (*bps[2])();
    int wit;  // windows per CTA iteration
};

#define FLCT_TC(N)                                                                          \
    {N,                                                                                     \
     {&launch_window_tc<N, __half>, &launch_window_tc<N, __nv_bfloat16>},                   \
     {&window_tc_blocks_per_sm<N, __half>, &window_tc_blocks_per_sm<N, __nv_bfloat16>},     \
     TcCfg<N>::WIT}
const TcEntry kTc[] = {FLCT_TC(4),  FLCT_TC(8),  FLCT_TC(12), FLCT_TC(16), FLCT_TC(20), FLCT_TC(24),
                       FLCT_TC(28), FLCT_TC(32), FLCT_TC(36), FLCT_TC(40), FLCT_TC(44), FLCT_TC(48),
                       FLCT_TC(52), FLCT_TC(56), FLCT_TC(60), FLCT_TC(64)};
#undef FLCT_TC
constexpr int kNumTc = sizeof(kTc) / sizeof(kTc[0]);

int tc_index(int n) {
    for (int k = 0; k < kNumTc; ++k)
        if (kTc[k].n == n) return k;
    return -1;
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
    cudaEvent_t tev[2] = {};  // autotuner
    char err[512] = {0};
    flct_timing timing{};
    // grow-only device workspace
    struct Buf {
        void* p = nullptr;
        size_t n = 0;
    };
    Buf b_s1, b_s2, b_work, b_ctr, b_r1, b_r2, b_b1, b_b2, b_gvx, b_gvy, b_ix, b_iy;
    Buf b_f1, b_f2, b_vx, b_vy, b_vm, b_aux1, b_aux2, b_means, b_peaks, b_grid, b_peaks_h, b_re1, b_re2;
    Buf b_whs, b_wmisc;  // warp_frac2d on the tensor cores: split spectrum stages, scale + status words
    std::vector<Buf*> all() {
        return {&b_s1,   &b_s2,   &b_work,   &b_ctr,    &b_r1,     &b_r2,     &b_b1,     &b_b2,
                &b_gvx,  &b_gvy,  &b_ix,     &b_iy,     &b_f1,     &b_f2,     &b_vx,     &b_vy,
                &b_vm,   &b_aux1, &b_aux2,   &b_means,  &b_peaks,  &b_grid,   &b_tc,     &bb_arena,
                &bb_work, &bb_means, &bb_peaks, &bb_ctr, &bb_meta, &b_peaks_h, &bb_peaks_h, &b_re1, &b_re2,
                &bb_multi, &b_whs,  &b_wmisc};
    }
    int bps[sizeof(kWin) / sizeof(kWin[0])][2] = {};
    int bps_tc[kNumTc][2] = {};
    int bps_big = 0;
    Buf b_tc;              // tensor-core DFT matrices of every box size and split type
    size_t tc_off[kNumTc][2] = {};
    bool tc_ready = false;
    bool box_attr = false;  // k_box_rows' shared-memory size is set
    bool pending = false;  // a velocity call's events await collection
    // autotuner: the fastest window configuration per box size
    struct Tune {
        int form = FLCT_FORM_FP32;
        int grid_div = 1;        // CTAs per SM = occupancy limit / grid_div
        int variant = 0;         // FP32 form: launch shape WinShape<n, variant>
        float ns_per_window = 0.f;
    };
    std::map<int, Tune> tune;
    std::string tune_path;       // JSON cache (FLCT_AUTOTUNE_CACHE), empty: none
    std::string device_name;
    // heterogeneous batches: own workspace (a batch's graph keeps pointing
    // at it), branch streams of the captured graph, the instantiated graph
    // of the last batch and the pairs it was built for
    static constexpr int kBranches = 8;
    Buf bb_arena, bb_work, bb_means, bb_peaks, bb_peaks_h, bb_ctr, bb_meta, bb_multi;
    cudaStream_t bstream[kBranches] = {};
    cudaEvent_t bev[kBranches + 1] = {};
    cudaEvent_t bdone = nullptr;  // recorded after each batch launch
    cudaGraphExec_t gexec = nullptr;
    std::vector<unsigned char> gkey;
    int batch_pending = 0;        // pairs of the batch whose timing awaits collection
    int batch_launches = 0;
    int batch_box = 0, batch_form = 0;
    unsigned char* hctr = nullptr;  // page-locked copies of a call's work counts and status words
    unsigned* hctr_dev = nullptr;   // the same memory, mapped: the last kernel of a call writes it
    // host-buffer calls in row bands, so that the copies overlap the
    // computation: copy-in and copy-out streams, per-band events
    static constexpr int kMaxBands = 8;
    int host_bands_max = 5;        // FLCT_HOST_BANDS (0 or 1: one band)
    int host_bands = 0;            // bands of the pending host call (0: not banded)
    cudaStream_t cstream[2] = {};  // copy-in, copy-out
    // the prepass (highest priority) on three streams, classification, row
    // sums and column sums, so that they overlap each other; then per-band
    // compute streams in falling priority: a band's windows fill the SMs the
    // band before leaves idle at its tail, and a band's small kernels go
    // ahead of the next band's windows
    static constexpr int kPre = 3;
    cudaStream_t prestream[kPre] = {};
    cudaStream_t bandstream[kMaxBands] = {};
    // band b copied in: [b]; finished rows ready for copy-out: [kMaxBands + b];
    // fitted: [2 kMaxBands + b]; box sums ready: [3 kMaxBands + b];
    // classified: [4 kMaxBands + b]; row sums ready: [5 kMaxBands + b];
    // start (fork): [6 kMaxBands]; join: [6 kMaxBands + 1]
    cudaEvent_t hev[6 * kMaxBands + 2] = {};
    // the device call's classification fork and join
    cudaEvent_t pev[2] = {};
    // the captured device call's stage events branch off its kernel chain
    // on this stream (fork and join events)
    cudaStream_t tstream = nullptr;
    cudaEvent_t tfork = nullptr, tjoin = nullptr;
    // the last banded call with page-locked buffers, captured as a graph
    cudaGraphExec_t hexec = nullptr;
    std::vector<unsigned char> hkey;
    int hlaunches = 0;
    // device-buffer calls: the last call's key, and the graph of a call
    // made twice in a row (replayed while the key repeats)
    cudaGraphExec_t dexec = nullptr;
    std::vector<unsigned char> dkey, dlast;
    int dlaunches = 0;
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
    if (n > kMaxBox) return;  // the big-box kernel builds its own (launch_windows)
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

// How a window launch is shaped: CTAs per SM = occupancy limit / grid_div,
// and for the FP32 form the launch shape WinShape<n, variant>.
struct WinCfg {
    int grid_div = 1;
    int variant = 0;
};

int win_grid(flct_ctx* ctx, int n, int v = 0) {
    int k = win_index(n);
    if (k < 0) return 0;
    if (ctx->bps[k][v] == 0) ctx->bps[k][v] = std::max(1, kWin[k].bps[v]());
    return ctx->nsm * ctx->bps[k][v];
}

// The tensor-core form's constant matrices, built once per context in FP64
// and split into 16-bit hi / lo halves in their shared-memory layouts, for
// every box size and both split types at once (one allocation that never
// moves, so captured graphs keep pointing at valid tables).
flct_status ensure_tc_tables(flct_ctx* ctx) {
    if (ctx->tc_ready) return FLCT_OK;
    size_t total = 0;
    for (int k = 0; k < kNumTc; ++k)
        for (int f = 0; f < 2; ++f) {
            ctx->tc_off[k][f] = total;
            total += ((size_t)tc_bmat_bytes(kTc[k].n) + 255) & ~(size_t)255;
        }
    ENSURE(ctx->b_tc, total);
    std::vector<unsigned char> host(total, 0);
    std::vector<uint16_t> m;
    for (int k = 0; k < kNumTc; ++k)
        for (int f = 0; f < 2; ++f) {
            tc_build_bmat(kTc[k].n, f, &m);
            memcpy(host.data() + ctx->tc_off[k][f], m.data(), m.size() * sizeof(uint16_t));
        }
    CK(cudaMemcpy(ctx->b_tc.p, host.data(), total, cudaMemcpyHostToDevice));
    ctx->tc_ready = true;
    return FLCT_OK;
}

// CTAs per SM of the tensor-core form for box size n (index k of kTc).
int tc_bps(flct_ctx* ctx, int k, int which) {
    if (ctx->bps_tc[k][which] == 0) ctx->bps_tc[k][which] = std::max(1, kTc[k].bps[which]());
    return ctx->bps_tc[k][which];
}

// Resolve FLCT_FORM_AUTO (the autotuner's choice once it has measured box
// size n, else the FP32 form) and check that the form exists for n.
flct_status pick_form(flct_ctx* ctx, int requested, int n, int* form) {
    int f = requested;
    if (f == FLCT_FORM_AUTO) {
        auto it = ctx->tune.find(n);
        f = (it != ctx->tune.end()) ? it->second.form : FLCT_FORM_FP32;
    }
    if ((f == FLCT_FORM_TC_FP16 || f == FLCT_FORM_TC_BF16) && tc_index(n) < 0)
        return fail(ctx, FLCT_ERR_UNSUPPORTED, "the tensor-core form has no kernel for box %d", n);
    if (f < 0 || f > FLCT_FORM_TC_BF16) return fail(ctx, FLCT_ERR_ARG, "unknown window form %d", requested);
    *form = f;
    return FLCT_OK;
}

// Launch the window kernel of the chosen form on the prepared work list.
// max_items >= 0: one CTA per group of windows up to that many items
// instead of a persistent grid, so that CTAs retire often and kernels of
// higher-priority streams get SMs in between (banded host calls).
flct_status launch_windows(flct_ctx* ctx, int form, const WinEntry* we, int n, const WinArgs& wa, unsigned* status,
                           cudaStream_t st, WinCfg cfg = {}, long max_items = -1, bool pdl = false) {
    const int grid_div = std::max(1, cfg.grid_div), v = cfg.variant ? 1 : 0;
    if (n > kMaxBox) {
        // boxes above 64: the big-box FP32 kernel, one window per CTA
        if (form != FLCT_FORM_FP32 || n > kMaxBigBox)
            return fail(ctx, FLCT_ERR_UNSUPPORTED, "box %d has no kernel of this form", n);
        BigArgs ba{};
        ba.s12 = wa.s12;
        ba.means = wa.means;
        ba.mg = wa.mg;
        ba.work = wa.work;
        ba.nwork = wa.nwork;
        ba.nx = wa.nx;
        ba.ny = wa.ny;
        ba.nsize = wa.nsize;
        ba.n = n;
        ba.use_filter = wa.use_filter;
        ba.direct = wa.direct;
        ba.peaks = wa.peaks;
        ba.peaks_h = wa.peaks_h;
        ba.segs = wa.segs;
        ba.seg_start = wa.seg_start;
        ba.nseg = wa.nseg;
        const double tw = 2.0 * 3.14159265358979323846 / n;
        for (int m = 0; m < n; ++m) ba.tw[m] = make_float2((float)std::cos(tw * m), (float)-std::sin(tw * m));
        // the same tables as fill_tables: Gaussian by offset (unit weights
        // for direct windows) and the squared filter by frequency index
        for (int d = -n; d <= n; ++d) {
            const double ax = (double)d / wa.sigma;
            ba.gauss[d + n] = wa.direct ? 1.0f : (float)std::exp(-ax * ax);
        }
        if (wa.use_filter) {
            const double kroll = wa.kr * (double)(n / 2);
            for (int k = 0; k < n; ++k) {
                const int kk = (k <= n / 2) ? k : k - n;
                const double ax = (double)kk / kroll;
                ba.filt2[k] = (float)std::exp(-2.0 * ax * ax);
            }
        }
        if (ctx->bps_big == 0) ctx->bps_big = std::max(1, window_big_blocks_per_sm(kMaxBigBox));
        int grid = std::max(ctx->nsm, ctx->nsm * ctx->bps_big / grid_div);
        if (max_items >= 0) grid = (int)std::max<long>(1, max_items);
        CK(launch_window_big(ba, grid, st, pdl));
        return FLCT_OK;
    }
    if (form == FLCT_FORM_FP32) {
        int grid = std::max(ctx->nsm, win_grid(ctx, n, v) / grid_div);
        if (max_items >= 0) grid = (int)std::max<long>(1, (max_items + we->teams[v] - 1) / we->teams[v]);
        CK(we->launch[v](wa, grid, st, pdl));
        return FLCT_OK;
    }
    flct_status s = ensure_tc_tables(ctx);
    if (s != FLCT_OK) return s;
    const int k = tc_index(n);
    if (k < 0) return fail(ctx, FLCT_ERR_UNSUPPORTED, "the tensor-core form has no kernel for box %d", n);
    TcArgs ta{};
    ta.s12 = wa.s12;
    ta.means = wa.means;
    ta.mg = wa.mg;
    ta.work = wa.work;
    ta.nwork = wa.nwork;
    ta.nx = wa.nx;
    ta.ny = wa.ny;
    ta.nsize = wa.nsize;
    ta.direct = wa.direct;
    ta.use_filter = wa.use_filter;
    ta.peaks = wa.peaks;
    ta.peaks_h = wa.peaks_h;
    ta.segs = wa.segs;
    ta.seg_start = wa.seg_start;
    ta.nseg = wa.nseg;
    const int which = (form == FLCT_FORM_TC_BF16) ? 1 : 0;
    ta.bmat = reinterpret_cast<const uint16_t*>(static_cast<const unsigned char*>(ctx->b_tc.p) + ctx->tc_off[k][which]);
    ta.status = status;
    // failure-path test hook: stage waits that run out after this many ns
    if (const char* w = getenv("FLCT_TEST_TC_STALL_NS")) ta.stall_ns = strtoull(w, nullptr, 10);
    for (int q = 0; q < 2 * kMaxBox + 1; ++q) ta.gauss[q] = wa.gauss[q];
    for (int q = 0; q < kMaxBox; ++q) ta.filt2[q] = wa.filt2[q];
    int grid = std::max(ctx->nsm, ctx->nsm * tc_bps(ctx, k, which) / grid_div);
    if (max_items >= 0) grid = (int)std::max<long>(1, (max_items + kTc[k].wit - 1) / kTc[k].wit);
    CK(kTc[k].launch[which](ta, grid, st, pdl));
    return FLCT_OK;
}

// ---------------------------------------------------------- autotuner --

void tune_save(flct_ctx* ctx) {
    if (ctx->tune_path.empty()) return;
    FILE* f = fopen(ctx->tune_path.c_str(), "w");
    if (!f) return;
    fprintf(f, "{\"device\": \"%s\", \"entries\": [\n", ctx->device_name.c_str());
    size_t k = 0;
    for (const auto& e : ctx->tune) {
        fprintf(f, "  {\"box\": %d, \"form\": %d, \"grid_div\": %d, \"ns_per_window\": %.4f, \"variant\": %d}%s\n",
                e.first, e.second.form, e.second.grid_div, e.second.ns_per_window, e.second.variant,
                (++k < ctx->tune.size()) ? "," : "");
    }
    fprintf(f, "]}\n");
    fclose(f);
}

// Reads entries written by tune_save (one per line) for this device name.
void tune_load(flct_ctx* ctx) {
    if (ctx->tune_path.empty()) return;
    FILE* f = fopen(ctx->tune_path.c_str(), "r");
    if (!f) return;
    char line[512];
    bool same_device = false;
    while (fgets(line, sizeof(line), f)) {
        if (strstr(line, "\"device\"")) same_device = strstr(line, ctx->device_name.c_str()) != nullptr;
        int box, form, gd;
        float ns;
        const char* q = strstr(line, "\"box\"");
        if (same_device && q &&
            sscanf(q, "\"box\": %d, \"form\": %d, \"grid_div\": %d, \"ns_per_window\": %f", &box, &form, &gd,
                   &ns) == 4 &&
            form >= FLCT_FORM_FP32 && form <= FLCT_FORM_TC_BF16 && gd >= 1 && gd <= 8) {
            flct_ctx::Tune t;
            t.form = form;
            t.grid_div = gd;
            t.ns_per_window = ns;
            // entries written before the shape variants existed have none: 0
            int v = 0;
            const char* qv = strstr(q, "\"variant\"");
            if (qv && sscanf(qv, "\"variant\": %d", &v) == 1 && (v == 0 || v == 1)) t.variant = v;
            ctx->tune[box] = t;
        }
    }
    fclose(f);
}

// Times every candidate configuration of the window kernel for box size n
// on the work list already prepared on `st` and keeps the fastest.  Needs
// a synchronising stream, so it never runs inside a stream capture.
flct_status tune_windows(flct_ctx* ctx, const WinEntry* we, int n, const WinArgs& wa, unsigned* status,
                         const int* d_nwork, cudaStream_t st) {
    struct Cand {
        int form;
        WinCfg cfg;
    };
    // FLCT_FORM_AUTO chooses among the forms whose error is FP32-like: the
    // radix form (both launch shapes: windows per CTA) and the split-FP16
    // tensor-core form (the BF16 split keeps fewer mantissa bits and is only
    // used when asked for), each at its occupancy limit or half of it
    std::vector<Cand> cands = {{FLCT_FORM_FP32, {1, 0}}, {FLCT_FORM_FP32, {2, 0}}, {FLCT_FORM_FP32, {1, 1}},
                               {FLCT_FORM_FP32, {2, 1}}};
    if (tc_index(n) >= 0) {
        cands.push_back({FLCT_FORM_TC_FP16, {1, 0}});
        if (tc_bps(ctx, tc_index(n), 0) > 1) cands.push_back({FLCT_FORM_TC_FP16, {2, 0}});
    }
    int nwork = 0;
    CK(cudaMemcpyAsync(&nwork, d_nwork, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (nwork <= 0) return FLCT_OK;  // nothing to measure yet
    float best = 1e30f;
    flct_ctx::Tune bt;
    for (const auto& c : cands) {
        float ms = 1e30f;
        for (int rep = 0; rep < 3; ++rep) {
            CK(cudaEventRecord(ctx->tev[0], st));
            flct_status s = launch_windows(ctx, c.form, we, n, wa, status, st, c.cfg);
            if (s != FLCT_OK) return s;
            CK(cudaEventRecord(ctx->tev[1], st));
            CK(cudaEventSynchronize(ctx->tev[1]));
            if (rep > 0) ms = std::min(ms, ev_ms(ctx->tev[0], ctx->tev[1]));
        }
        if (ms < best) {
            best = ms;
            bt.form = c.form;
            bt.grid_div = c.cfg.grid_div;
            bt.variant = c.cfg.variant;
        }
    }
    bt.ns_per_window = best * 1e6f / (float)nwork;
    ctx->tune[n] = bt;
    tune_save(ctx);
    return FLCT_OK;
}

// ------------------------------------------------- velocity pipeline --

bool capturing(cudaStream_t st) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cs) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return cs != cudaStreamCaptureStatusNone;
}

// One image pair's velocity job after the host-side checks and parameter
// derivation (flct.c:337-487, 535-745).
struct Job {
    const flct_params* p = nullptr;
    const double* f1 = nullptr;
    const double* f2 = nullptr;
    double* vx = nullptr;
    double* vy = nullptr;
    double* vm = nullptr;
    int nx = 0, ny = 0;
    Derived d;
    int n = 0;
    const WinEntry* we = nullptr;
    bool interp = false;
    // window grid: pixel (xo + q gs, yo + m gs), q < gi, m < gj (every
    // pixel without -s)
    int gs = 1, xo = 0, yo = 0, gi = 0, gj = 0;
};

flct_status plan_job(flct_ctx* ctx, const flct_params* p, const double* f1, const double* f2, int nx, int ny,
                     double* vx, double* vy, double* vm, Job* j) {
    if (!p || !f1 || !f2 || !vx || !vy || !vm || nx < 1 || ny < 1)
        return fail(ctx, FLCT_ERR_ARG, "null pointer or empty image (%d x %d)", nx, ny);
    if ((long long)nx * ny >= (1ll << 31)) return fail(ctx, FLCT_ERR_UNSUPPORTED, "image larger than 2^31 pixels");
    flct_status s = derive(ctx, p, nx, ny, &j->d);
    if (s != FLCT_OK) return s;
    if (j->d.global && (nx > kMaxGlobalAxis || ny > kMaxGlobalAxis))
        return fail(ctx, FLCT_ERR_UNSUPPORTED, "sigma <= 0 correlates whole frames of at most %d per side",
                    kMaxGlobalAxis);
    if (j->d.global && p->hires && (nx < 3 || ny < 3))
        return fail(ctx, FLCT_ERR_UNSUPPORTED, "sigma <= 0 with -h needs frames of at least 3 x 3");
    if (j->d.global && p->filter && (nx < 2 || ny < 2))
        return fail(ctx, FLCT_ERR_UNSUPPORTED, "sigma <= 0 with -k needs frames of at least 2 x 2");
    if (p->filter && !(p->kr > 0.))
        return fail(ctx, FLCT_ERR_UNSUPPORTED, "-k with kr <= 0 is not available on the GPU path");
    j->n = j->d.n;
    j->we = j->d.global ? nullptr : find_win(j->n);
    if (!j->d.global && !j->we && j->n > kMaxBigBox)
        return fail(ctx, FLCT_ERR_UNSUPPORTED, "box size %d (sigma %g) has no GPU kernel", j->n, p->sigma);
    j->p = p;
    j->f1 = f1;
    j->f2 = f2;
    j->vx = vx;
    j->vy = vy;
    j->vm = vm;
    j->nx = nx;
    j->ny = ny;
    j->interp = j->d.skip > 0 && p->interpolate;
    if (j->d.skip > 0) {
        j->gs = j->d.skip;
        j->xo = j->d.xoff;
        j->yo = j->d.yoff;
        j->gi = grid_count(nx, j->xo, j->gs);
        j->gj = grid_count(ny, j->yo, j->gs);
    } else {
        j->gi = nx;
        j->gj = ny;
    }
    return FLCT_OK;
}

// Device workspace of one job: the context's single-call buffers, or a
// slice of a batch's buffers.
struct JobBufs {
    float4* s12 = nullptr;  // both frames' float split per pixel
    int* work = nullptr;
    float4* means = nullptr;  // local means [gi][gj] (MeanGrid)
    PeakRec* peaks = nullptr;
    PeakRecH* peaks_h = nullptr;  // -h only
    BoxSum* r1 = nullptr;  // exact row sums [nx][gj]
    BoxSum* r2 = nullptr;
    int* re1 = nullptr;    // the row sums' exponents [nx][gj]
    int* re2 = nullptr;
    // 64 bytes: [0] work count (int), [4] status bits, [8..23] |f1|,|f2|
    // maxima, [24..31] relative threshold
    unsigned char* ctr = nullptr;
    float2* grid = nullptr;  // skip-grid (vx, vy) [gi][gj] for the interpolation
};

// Bytes of each workspace region of a job.
struct JobSizes {
    size_t s = 0, work = 0, means = 0, peaks = 0, peaks_h = 0, r = 0, re = 0, grid = 0;
};

JobSizes job_sizes(const Job& j) {
    const size_t npx = (size_t)j.nx * j.ny;
    JobSizes z;
    z.s = npx * sizeof(float4);
    z.work = npx * sizeof(int);
    z.means = (size_t)j.gi * j.gj * sizeof(float4);
    z.peaks = npx * sizeof(PeakRec);
    if (j.p->hires) z.peaks_h = npx * sizeof(PeakRecH);
    z.r = (size_t)j.gj * j.nx * sizeof(BoxSum);
    z.re = (size_t)j.gj * j.nx * sizeof(int);
    if (j.interp) z.grid = (size_t)j.gi * j.gj * sizeof(float2);
    return z;
}

// Classification of frame rows [r0, r1): threshold test, skip grid, the
// float split, the work list (b.work / b.ctr: the windows of those rows)
// and the final values of pixels without a window (flct.c:684-755).
ClassifyArgs classify_args(const Job& j, const JobBufs& b, int r0, int r1, const double* d_thr) {
    ClassifyArgs ca{};
    ca.f1 = j.f1;
    ca.f2 = j.f2;
    ca.nx = j.nx;
    ca.ny = j.ny;
    ca.thr_val = j.p->thresh;
    ca.thr_ptr = d_thr;
    ca.skip = j.d.skip;
    ca.xoff = j.d.xoff;
    ca.yoff = j.d.yoff;
    ca.interpolate = j.interp;
    ca.jcnt = j.d.jcnt;
    ca.s12 = b.s12;
    ca.work = b.work;
    ca.nwork = (int*)b.ctr;
    ca.vx = j.vx;
    ca.vy = j.vy;
    ca.vm = j.vm;
    ca.grid = j.interp ? b.grid : nullptr;
    ca.status = (unsigned*)(b.ctr + 4);
    ca.r0 = r0;
    ca.r1 = r1;
    return ca;
}

flct_status enqueue_classify(flct_ctx* ctx, const Job& j, const JobBufs& b, int r0, int r1, const double* d_thr,
                             cudaStream_t st, int* launches, int blocks_per_sm = 8, const JobBufs* b2 = nullptr,
                             int rsplit = 0) {
    ClassifyArgs ca = classify_args(j, b, r0, r1, d_thr);
    if (b2) {  // windows of rows >= rsplit to b2's list
        ca.work2 = b2->work;
        ca.nwork2 = (int*)b2->ctr;
        ca.rsplit = rsplit;
    }
    const long tiles = (long)(r1 - r0) * ((j.ny + kClassPix - 1) / kClassPix);
    k_classify<<<(int)std::max(1l, std::min<long>(tiles, (long)ctx->nsm * blocks_per_sm)), 256, 0, st>>>(ca);
    ++*launches;
    CK(cudaGetLastError());
    return FLCT_OK;
}

BoxArgs box_args(const Job& j, const JobBufs& b) {
    BoxArgs ba{};
    ba.f1 = j.f1;
    ba.f2 = j.f2;
    ba.nx = j.nx;
    ba.ny = j.ny;
    ba.n = j.n;
    ba.nsize = j.d.nsize;
    ba.gs = j.gs;
    ba.xo = j.xo;
    ba.yo = j.yo;
    ba.gi = j.gi;
    ba.gj = j.gj;
    ba.rt1 = b.r1;
    ba.rt2 = b.r2;
    ba.means = b.means;
    ba.inv_n2 = 1. / ((double)j.n * j.n);
    ba.re1 = b.re1;
    ba.re2 = b.re2;
    return ba;
}

// Row pass arguments for frame rows [r0, r1), and its warp tasks.
BoxArgs box_rows_args(const Job& j, const JobBufs& b, int r0, int r1, long* tasks) {
    BoxArgs ba = box_args(j, b);
    ba.r0 = r0;
    ba.r1 = r1;
    // a warp pass covers P grid columns whose input span fits kRowSpan
    ba.pass_r = std::max(1, std::min(j.gj, (kRowSpan - j.n) / j.gs + 1));
    *tasks = 2l * (r1 - r0) * ((j.gj + ba.pass_r - 1) / ba.pass_r);
    return ba;
}

constexpr size_t kBoxRowsSmem = (size_t)kBoxWarps * (5 * (kRowSpan + 64) + 5 * 32) * sizeof(unsigned);

// Column pass arguments for grid rows [q0, q1), and its threads.
BoxArgs box_cols_args(const Job& j, const JobBufs& b, int q0, int q1, long* threads) {
    BoxArgs ba = box_args(j, b);
    ba.q0 = q0;
    ba.q1 = q1;
    *threads = 2l * j.gj * ((q1 - q0 + kColRun - 1) / kColRun) * kColLanes;
    return ba;
}

// Exact row sums of frame rows [r0, r1) at the grid's box columns.
flct_status enqueue_box_rows(flct_ctx* ctx, const Job& j, const JobBufs& b, int r0, int r1, cudaStream_t st,
                             int* launches, int blocks_per_sm = 4) {
    if (r1 <= r0) return FLCT_OK;
    long tasks = 0;
    BoxArgs ba = box_rows_args(j, b, r0, r1, &tasks);
    const size_t smem = kBoxRowsSmem;
    if (!ctx->box_attr) {
        CK(cudaFuncSetAttribute(k_box_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        CK(cudaFuncSetAttribute(k_box_rows_multi, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        ctx->box_attr = true;
    }
    const long blocks = std::min<long>((tasks + kBoxWarps - 1) / kBoxWarps, (long)ctx->nsm * blocks_per_sm);
    k_box_rows<<<(int)std::max(1l, blocks), kBoxWarps * 32, smem, st>>>(ba);
    ++*launches;
    CK(cudaGetLastError());
    return FLCT_OK;
}

// Exact box sums of grid rows [q0, q1) (their row sums must be complete; q0
// a multiple of kColRun, so the runs are those of the whole frame).
flct_status enqueue_box_cols(flct_ctx* ctx, const Job& j, const JobBufs& b, int q0, int q1, cudaStream_t st,
                             int* launches, bool pdl = false) {
    if (q1 <= q0) return FLCT_OK;
    long t = 0;
    BoxArgs ba = box_cols_args(j, b, q0, q1, &t);
    CK(launch_kernel(k_box_cols, dim3((unsigned)((t + 127) / 128)), dim3(128), 0, st, pdl, ba));
    ++*launches;
    CK(cudaGetLastError());
    return FLCT_OK;
}

// The whole-frame prepass: counters, relative threshold (flct.c:594-629),
// classification and the local means (box sums).  With a side stream the
// classification runs there, beside the box sums (both only read the
// frames), on half the blocks so that the two kernels share the SMs.
flct_status enqueue_prepass(flct_ctx* ctx, const Job& j, const JobBufs& b, cudaStream_t st, int* launches,
                            cudaStream_t side = nullptr) {
    const size_t npx = (size_t)j.nx * j.ny;
    unsigned long long* d_absmax = (unsigned long long*)(b.ctr + 8);
    double* d_thr = (double*)(b.ctr + 24);
    CK(cudaMemsetAsync(b.ctr, 0, 64, st));
    if (j.d.rel_thresh) {
        k_absmax<<<ctx->nsm * 4, 256, 0, st>>>(AbsmaxArgs{j.f1, j.f2, (long)npx, d_absmax});
        k_thresh_final<<<1, 1, 0, st>>>(ThreshArgs{j.f1, j.f2, d_absmax, j.p->thresh, d_thr});
        *launches += 2;
    }
    const double* thr = j.d.rel_thresh ? d_thr : nullptr;
    flct_status s = FLCT_OK;
    if (side) {
        CK(cudaEventRecord(ctx->pev[0], st));
        CK(cudaStreamWaitEvent(side, ctx->pev[0], 0));
        // the box sums go first: their two passes are the longer chain
        s = enqueue_box_rows(ctx, j, b, 0, j.nx, st, launches);
        if (s == FLCT_OK) s = enqueue_classify(ctx, j, b, 0, j.nx, thr, side, launches, 4);
        if (s != FLCT_OK) return s;
        CK(cudaEventRecord(ctx->pev[1], side));
        // the column pass launches as a programmatic dependent of the row pass
        s = enqueue_box_cols(ctx, j, b, 0, j.gi, st, launches, true);
        CK(cudaStreamWaitEvent(st, ctx->pev[1], 0));
    } else {
        s = enqueue_classify(ctx, j, b, 0, j.nx, thr, st, launches);
        if (s == FLCT_OK) s = enqueue_box_rows(ctx, j, b, 0, j.nx, st, launches);
        if (s == FLCT_OK) s = enqueue_box_cols(ctx, j, b, 0, j.gi, st, launches);
    }
    // device calls (with a side stream) launch the window kernel next as a
    // programmatic dependent; the operation just before it on st is the wait
    // for the classification, and the window kernels' grid_dep_wait (before
    // any global access) keeps both the column sums and that join ordered,
    // eager and captured
    return s;
}

void make_wargs(const Job& j, const JobBufs& b, WinArgs* wa) {
    *wa = WinArgs{};
    fill_tables(j.p, j.n, wa->gauss, wa->filt2);
    wa->sigma = j.p->sigma;
    wa->kr = j.p->kr;
    wa->use_filter = j.p->filter;
    wa->s12 = b.s12;
    wa->means = b.means;
    wa->mg = MeanGrid{j.gs, j.xo, j.yo, j.gj};
    wa->work = b.work;
    wa->nwork = (const int*)b.ctr;
    wa->nx = j.nx;
    wa->ny = j.ny;
    wa->nsize = j.d.nsize;
    wa->peaks = b.peaks;
    wa->peaks_h = j.p->hires ? b.peaks_h : nullptr;
}

// 3x3 fit, velocity, mask and skip-grid copy per work item (flct.c:901-942).
// Where the last kernel of a call copies the call's counters (none: null).
struct Pub {
    const unsigned* src = nullptr;
    unsigned* dst = nullptr;
};

FitArgs fit_args(const Job& j, const JobBufs& b, Pub pub) {
    FitArgs fa{};
    fa.pub_src = pub.src;
    fa.pub_dst = pub.dst;
    fa.work = b.work;
    fa.nwork = (const int*)b.ctr;
    fa.peaks = b.peaks;
    fa.n = j.n;
    fa.ny = j.ny;
    fa.vscale = (1. / j.p->deltat) * j.p->deltas;  // flct.c:343, 901-905
    fa.skip = j.d.skip > 0 ? j.d.skip : 1;
    fa.xoff = j.d.xoff;
    fa.yoff = j.d.yoff;
    fa.jcnt = j.d.jcnt;
    fa.vx = j.vx;
    fa.vy = j.vy;
    fa.vm = j.vm;
    fa.grid = j.interp ? b.grid : nullptr;
    if (j.p->hires) fa.peaks_h = b.peaks_h;
    return fa;
}

flct_status enqueue_fit(flct_ctx* ctx, const Job& j, const JobBufs& b, cudaStream_t st, int* launches,
                        long max_items = -1, Pub pub = Pub{}, bool pdl = false) {
    const FitArgs fa = fit_args(j, b, pub);
    const size_t npx = max_items >= 0 ? (size_t)max_items : (size_t)j.nx * j.ny;
    if (j.p->hires) {
        long blocks = std::min<long>((long)(npx + 3) / 4, (long)ctx->nsm * 16);
        CK(launch_kernel(k_fit_hires, dim3((unsigned)std::max(1l, blocks)), dim3(128), 0, st, pdl, fa));
    } else {
        long blocks = std::min<long>((long)(npx + 127) / 128, (long)ctx->nsm * 8);
        CK(launch_kernel(k_fit, dim3((unsigned)std::max(1l, blocks)), dim3(128), 0, st, pdl, fa));
    }
    ++*launches;
    CK(cudaGetLastError());
    return FLCT_OK;
}

// Cubic-convolution interpolation of the skip grid onto the skipped pixels,
// mask and xmiss reset (flct.c:958-1133).
InterpArgs interp_args(const Job& j, const JobBufs& b, int i0, int i1, Pub pub) {
    InterpArgs ia{};
    ia.pub_src = pub.src;
    ia.pub_dst = pub.dst;
    ia.nx = j.nx;
    ia.ny = j.ny;
    ia.skip = j.d.skip;
    ia.xoff = j.d.xoff;
    ia.yoff = j.d.yoff;
    ia.gx = j.d.icnt;
    ia.gy = j.d.jcnt;
    ia.grid = b.grid;
    ia.vx = j.vx;
    ia.vy = j.vy;
    ia.vm = j.vm;
    ia.i0 = i0;
    ia.i1 = i1;
    // pixel pairs (j even) start on 16-byte boundaries when ny is even
    ia.pairs = (j.ny % 2 == 0) && ((((uintptr_t)j.vx) | ((uintptr_t)j.vy) | ((uintptr_t)j.vm)) & 15u) == 0u;
    return ia;
}

flct_status enqueue_interp(flct_ctx* ctx, const Job& j, const JobBufs& b, cudaStream_t st, int* launches,
                           int i0 = 0, int i1 = -1, Pub pub = Pub{}, bool pdl = false) {
    if (i1 < 0) i1 = j.nx;
    if (i1 <= i0) return FLCT_OK;
    const InterpArgs ia = interp_args(j, b, i0, i1, pub);
    const long tiles = (long)((i1 - i0 + kTileR - 1) / kTileR) * ((j.ny + kTileC - 1) / kTileC);
    CK(launch_kernel(k_interp_grid, dim3((unsigned)std::max(1l, std::min<long>(tiles, (long)ctx->nsm * 8))),
                     dim3(kInterpThreads), 0, st, pdl, ia));
    ++*launches;
    CK(cudaGetLastError());
    return FLCT_OK;
}

// Occupancy queries and the tensor-core tables need the host; done before
// a stream capture so the captured launches make none of these calls.
flct_status prime_form(flct_ctx* ctx, int form, int n) {
    if (form == FLCT_FORM_FP32 && n > kMaxBox) {
        if (ctx->bps_big == 0) ctx->bps_big = std::max(1, window_big_blocks_per_sm(kMaxBigBox));
        return FLCT_OK;
    }
    if (form == FLCT_FORM_FP32) {
        if (win_grid(ctx, n, 0) <= 0 || win_grid(ctx, n, 1) <= 0)
            return fail(ctx, FLCT_ERR_CUDA, "no occupancy for the box-%d window kernel", n);
        return FLCT_OK;
    }
    flct_status s = ensure_tc_tables(ctx);
    if (s != FLCT_OK) return s;
    const int k = tc_index(n);
    if (k < 0) return fail(ctx, FLCT_ERR_UNSUPPORTED, "the tensor-core form has no kernel for box %d", n);
    tc_bps(ctx, k, (form == FLCT_FORM_TC_BF16) ? 1 : 0);
    return FLCT_OK;
}

// Form, CTAs-per-SM divisor and launch shape for box size n: the request
// (default shape), or for FLCT_FORM_AUTO the autotuner's measured choice.
void resolved_config(flct_ctx* ctx, int requested, int n, int* form, WinCfg* cfg) {
    *cfg = WinCfg{};
    if (requested != FLCT_FORM_AUTO) {
        *form = requested;
        return;
    }
    auto it = ctx->tune.find(n);
    if (it == ctx->tune.end()) {
        *form = FLCT_FORM_FP32;
        return;
    }
    *form = it->second.form;
    cfg->grid_div = it->second.grid_div;
    cfg->variant = it->second.variant;
}

// ------------------------------------------------------ sigma <= 0 --

// make_freq (flct.c:1651-1690): 0..n/2-1, n/2 (and -n/2 for odd n), then
// the negative frequencies.
std::vector<double> make_freq(int n) {
    std::vector<double> k(n);
    const int n21 = n / 2 - 1;
    int i = 0;
    for (; i < n21 + 1; ++i) k[i] = (double)i;
    int inext = n21 + 1;
    if ((n / 2) * 2 != n) {
        if (inext < n) k[inext] = (double)(n / 2);
        ++inext;
        if (inext < n) k[inext] = -(double)(n / 2);
        ++inext;
    } else {
        if (inext < n) k[inext] = (double)(n / 2);
        ++inext;
    }
    for (i = inext; i < n; ++i) k[i] = -(double)(n21 - (i - inext));
    return k;
}

// The whole-frame correlation of the sigma <= 0 mode: FP64 means, FP32
// batched DFTs, the same fits as the sliding windows (flct.c:802-942 with
// init = 2).  Output: one (vx, vy, vm).
flct_status velocity_global(flct_ctx* ctx, const Job& j, cudaStream_t st) {
    const flct_params* p = j.p;
    const int nx = j.nx, ny = j.ny;
    const long n = (long)nx * ny;
    ENSURE(ctx->b_s1, (size_t)n * sizeof(float2));
    ENSURE(ctx->b_s2, (size_t)n * sizeof(float2));
    ENSURE(ctx->b_ctr, 64);
    ENSURE(ctx->b_aux2, (size_t)kGsumBlocks * 2 * sizeof(double));
    ENSURE(ctx->b_b1, (size_t)(nx + ny) * (sizeof(float2) + sizeof(float)) + 64);
    ENSURE(ctx->b_work, 64);
    ENSURE(ctx->b_peaks, sizeof(PeakRec));
    if (p->hires) ENSURE(ctx->b_peaks_h, sizeof(PeakRecH));
    // twiddles e^{-2 pi i m / L} per axis and the squared -k filter factors
    // exp(-2 (k / (kr k[L/2]))^2) (flct.c:1694-1715, applied to both spectra)
    std::vector<unsigned char> tab((size_t)(nx + ny) * (sizeof(float2) + sizeof(float)));
    float2* twx = (float2*)tab.data();
    float2* twy = twx + nx;
    float* fx2 = (float*)(twy + ny);
    float* fy2 = fx2 + nx;
    auto fill = [&](int L, float2* tw, float* f2) {
        for (int m = 0; m < L; ++m) {
            const double a = 2.0 * 3.14159265358979323846 * (double)m / (double)L;
            tw[m] = make_float2((float)std::cos(a), (float)-std::sin(a));
        }
        const std::vector<double> k = make_freq(L);
        const double roll = p->kr * k[L / 2];
        for (int m = 0; m < L; ++m) {
            const double ax = k[m] / roll;
            f2[m] = p->filter ? (float)std::exp(-2.0 * ax * ax) : 1.0f;
        }
    };
    fill(nx, twx, fx2);
    fill(ny, twy, fy2);
    unsigned char* dtab = (unsigned char*)ctx->b_b1.p;
    CK(cudaMemcpyAsync(dtab, tab.data(), tab.size(), cudaMemcpyHostToDevice, st));
    const float2* d_twx = (const float2*)dtab;
    const float2* d_twy = d_twx + nx;
    const float* d_fx2 = (const float*)(d_twy + ny);
    const float* d_fy2 = d_fx2 + nx;
    // counters: [0] nwork, [4] status, [8] peak key, [16] |g| maxima, [24] means
    unsigned char* ctr = (unsigned char*)ctx->b_ctr.p;
    int* d_nwork = (int*)ctr;
    unsigned* d_status = (unsigned*)(ctr + 4);
    unsigned long long* d_key = (unsigned long long*)(ctr + 8);
    unsigned* d_max = (unsigned*)(ctr + 16);
    double* d_means = (double*)(ctr + 24);
    float2* A = (float2*)ctx->b_s1.p;
    float2* B = (float2*)ctx->b_s2.p;
    int launches = 0;
    ctx->batch_pending = 0;
    CK(cudaEventRecord(ctx->ev[0], st));
    CK(cudaMemsetAsync(ctr, 0, 64, st));
    k_gsum_part<<<kGsumBlocks, 256, 0, st>>>(j.f1, j.f2, n, (double*)ctx->b_aux2.p);
    k_gsum_final<<<1, 256, 0, st>>>((const double*)ctx->b_aux2.p, kGsumBlocks, (double)nx * ny, d_means);
    const int eblocks = (int)std::min<long>((n + 255) / 256, (long)ctx->nsm * 8);
    k_gz<<<eblocks, 256, 0, st>>>(j.f1, j.f2, n, d_means, A, d_max, d_status);
    launches += 3;
    CK(cudaGetLastError());
    CK(cudaEventRecord(ctx->ev[1], st));
    auto dft = [&](bool inverse, const float2* in, float2* out, int L, int lines, const float2* tw,
                   const unsigned* sc) {
        launch_dft_rows(inverse, in, out, L, lines, tw, sc, st);
        ++launches;
    };
    auto transpose = [&](const float2* in, float2* out, int R, int C) {
        k_transpose<<<dim3((C + 31) / 32, (R + 31) / 32), dim3(32, 8), 0, st>>>(in, out, R, C);
        ++launches;
    };
    dft(false, A, B, ny, nx, d_twy, d_max);  // along the fast axis, with the power-of-two scales
    transpose(B, A, nx, ny);                 // [ky][i]
    dft(false, A, B, nx, ny, d_twx, nullptr);  // Zt[ky][kx]
    k_gprod<<<eblocks, 256, 0, st>>>(B, A, nx, ny, d_fx2, d_fy2);
    ++launches;
    dft(true, A, B, nx, ny, d_twx, nullptr);
    transpose(B, A, ny, nx);
    dft(true, A, B, ny, nx, d_twy, nullptr);  // c[i][j] (real part)
    k_gpeak<<<eblocks, 256, 0, st>>>(B, nx, ny, d_key);
    PeakRec* rec = (PeakRec*)ctx->b_peaks.p;
    PeakRecH* rech = p->hires ? (PeakRecH*)ctx->b_peaks_h.p : nullptr;
    k_gpatch<<<1, 64, 0, st>>>(B, nx, ny, d_key, rec, rech, (int*)ctx->b_work.p, d_nwork);
    launches += 2;
    CK(cudaGetLastError());
    CK(cudaEventRecord(ctx->ev[2], st));
    FitArgs fa{};
    fa.work = (const int*)ctx->b_work.p;
    fa.nwork = d_nwork;
    fa.peaks = rec;
    fa.peaks_h = rech;
    fa.n = nx;
    fa.n1 = ny;
    fa.ny = 1;
    fa.vscale = (1. / p->deltat) * p->deltas;  // flct.c:343, 901-905
    fa.skip = 1;
    fa.vx = j.vx;
    fa.vy = j.vy;
    fa.vm = j.vm;
    if (rech) k_fit_hires<<<1, 128, 0, st>>>(fa);
    else k_fit<<<1, 32, 0, st>>>(fa);
    ++launches;
    CK(cudaGetLastError());
    CK(cudaEventRecord(ctx->ev[7], st));
    CK(cudaMemcpyAsync(ctx->hctr, ctr, 8, cudaMemcpyDeviceToHost, st));
    CK(cudaEventRecord(ctx->ev[3], st));
    ctx->timing = flct_timing{};
    ctx->timing.launches = launches;
    ctx->timing.box = 0;
    ctx->timing.form = FLCT_FORM_FP32;
    ctx->pending = true;
    return FLCT_OK;
}

// ------------------------------------------------------------- batches --

// Pairs sharing a box size, requested form and window tables run through
// one persistent window-kernel launch.
struct BatchGroup {
    int n = 0;
    int req_form = 0;
    int use_filter = 0;
    int hires = 0;
    float gauss[2 * kMaxBox + 1] = {};
    float filt2[kMaxBox] = {};
    double sigma = 0., kr = 0.;
    std::vector<int> pairs;
    int form = FLCT_FORM_FP32;
    WinCfg cfg;
};

// One kernel's launches for many pairs merged into one grid: the per-pair
// argument structs and block prefix sums in the batch's device tables.
struct MultiSet {
    size_t args = 0, start = 0;  // byte offsets in bb_multi
    int npairs = 0, blocks = 0;
};

struct BatchPlan {
    std::vector<Job> jobs;
    std::vector<JobBufs> bufs;
    std::vector<BatchGroup> groups;
    MultiSet m_abs, m_thr, m_cls, m_rows, m_cols, m_fit, m_fith, m_interp;
    WinSeg* segs = nullptr;  // device, group-major
    int* starts = nullptr;   // device, per group nseg + 1 entries
    int* seg_pair = nullptr; // device
    int* first = nullptr;    // device, ngroups + 1
    std::vector<int> h_first;
};

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// The fields of a pair list that a captured batch depends on.
std::vector<unsigned char> batch_key(int npairs, const flct_pair* pairs) {
    std::vector<unsigned char> key;
    auto put = [&key](const void* v, size_t n) {
        const unsigned char* c = (const unsigned char*)v;
        key.insert(key.end(), c, c + n);
    };
    for (int k = 0; k < npairs; ++k) {
        const flct_pair& q = pairs[k];
        const flct_params& p = q.params;
        put(&q.f1, sizeof(q.f1));
        put(&q.f2, sizeof(q.f2));
        put(&q.vx, sizeof(q.vx));
        put(&q.vy, sizeof(q.vy));
        put(&q.vm, sizeof(q.vm));
        const int ints[] = {q.nx, q.ny, p.thresh_abs, p.skip, p.poffset, p.qoffset, p.interpolate, p.filter,
                            p.hires, p.form};
        const double dbl[] = {p.deltat, p.deltas, p.sigma, p.thresh, p.kr};
        put(ints, sizeof(ints));
        put(dbl, sizeof(dbl));
    }
    return key;
}

flct_status pair_fail(flct_ctx* ctx, flct_status s, int k) {
    char msg[sizeof(ctx->err)];
    snprintf(msg, sizeof(msg), "pair %d: %.480s", k, ctx->err);
    memcpy(ctx->err, msg, sizeof(msg));
    return s;
}

// The merged launches of a batch's per-pair kernels: every pair's prepass
// kernels, fit and interpolation as one grid each, with the same argument
// structs the single-pair calls use and as many blocks per pair as the
// pair's work (the kernels' loops are strided over the pair's own blocks).
flct_status plan_multi(flct_ctx* ctx, BatchPlan* bp) {
    const int np = (int)bp->jobs.size();
    std::vector<unsigned char> host;
    auto add = [&host](const void* p, size_t bytes) {
        const size_t o = host.size();
        host.resize(align256(o + bytes));
        memcpy(host.data() + o, p, bytes);
        return o;
    };
    // args and per-pair blocks -> a MultiSet (pairs with 0 blocks left out)
    auto pack = [&](auto& args, const std::vector<long>& blocks, MultiSet* m) {
        using A = typename std::decay_t<decltype(args)>::value_type;
        std::vector<A> used;
        std::vector<int> start(1, 0);
        for (size_t k = 0; k < args.size(); ++k) {
            if (blocks[k] <= 0) continue;
            used.push_back(args[k]);
            start.push_back(start.back() + (int)blocks[k]);
        }
        m->npairs = (int)used.size();
        m->blocks = start.back();
        if (!used.empty()) {
            m->args = add(used.data(), used.size() * sizeof(A));
            m->start = add(start.data(), start.size() * sizeof(int));
        }
    };
    std::vector<AbsmaxArgs> abs;
    std::vector<ThreshArgs> thr;
    std::vector<ClassifyArgs> cls;
    std::vector<BoxArgs> rows, cols;
    std::vector<FitArgs> fit, fith;
    std::vector<InterpArgs> ia;
    std::vector<long> babs, bthr, bcls, brows, bcols, bfit, bfith, bia;
    for (int k = 0; k < np; ++k) {
        const Job& j = bp->jobs[k];
        const JobBufs& b = bp->bufs[k];
        const long npx = (long)j.nx * j.ny;
        unsigned long long* d_absmax = (unsigned long long*)(b.ctr + 8);
        double* d_thr = (double*)(b.ctr + 24);
        abs.push_back(AbsmaxArgs{j.f1, j.f2, npx, d_absmax});
        babs.push_back(j.d.rel_thresh ? std::max(1l, std::min<long>((npx + 1023) / 1024, ctx->nsm)) : 0);
        thr.push_back(ThreshArgs{j.f1, j.f2, d_absmax, j.p->thresh, d_thr});
        bthr.push_back(j.d.rel_thresh ? 1 : 0);
        cls.push_back(classify_args(j, b, 0, j.nx, j.d.rel_thresh ? d_thr : nullptr));
        bcls.push_back((long)j.nx * ((j.ny + kClassPix - 1) / kClassPix));
        long tasks = 0, threads = 0;
        rows.push_back(box_rows_args(j, b, 0, j.nx, &tasks));
        brows.push_back((tasks + kBoxWarps - 1) / kBoxWarps);
        cols.push_back(box_cols_args(j, b, 0, j.gi, &threads));
        bcols.push_back((threads + 127) / 128);
        const FitArgs fa = fit_args(j, b, Pub{});
        fit.push_back(fa);
        fith.push_back(fa);
        bfit.push_back(j.p->hires ? 0 : std::max(1l, (npx + 127) / 128));
        bfith.push_back(j.p->hires ? std::max(1l, (npx + 3) / 4) : 0);
        ia.push_back(interp_args(j, b, 0, j.nx, Pub{}));
        bia.push_back(j.interp ? (long)((j.nx + kTileR - 1) / kTileR) * ((j.ny + kTileC - 1) / kTileC) : 0);
    }
    for (const auto* v : {&babs, &bthr, &bcls, &brows, &bcols, &bfit, &bfith, &bia}) {
        long tot = 0;
        for (long x : *v) tot += x;
        if (tot >= (1l << 31)) return fail(ctx, FLCT_ERR_UNSUPPORTED, "batch needs more than 2^31 blocks");
    }
    pack(abs, babs, &bp->m_abs);
    pack(thr, bthr, &bp->m_thr);
    pack(cls, bcls, &bp->m_cls);
    pack(rows, brows, &bp->m_rows);
    pack(cols, bcols, &bp->m_cols);
    pack(fit, bfit, &bp->m_fit);
    pack(fith, bfith, &bp->m_fith);
    pack(ia, bia, &bp->m_interp);
    ENSURE(ctx->bb_multi, std::max<size_t>(host.size(), 256));
    CK(cudaMemcpy(ctx->bb_multi.p, host.data(), host.size(), cudaMemcpyHostToDevice));
    return FLCT_OK;
}

// Launch a merged kernel of the batch (nothing when no pair has blocks).
template <class A>
cudaError_t launch_multi(flct_ctx* ctx, void (*kern)(MultiArgs<A>), const MultiSet& m, int threads, size_t smem,
                         cudaStream_t st, int* launches) {
    if (m.npairs == 0) return cudaSuccess;
    const unsigned char* M = (const unsigned char*)ctx->bb_multi.p;
    MultiArgs<A> ma{(const A*)(M + m.args), (const int*)(M + m.start), m.npairs};
    kern<<<m.blocks, threads, smem, st>>>(ma);
    ++*launches;
    return cudaGetLastError();
}

// Checks every pair, groups the pairs, lays out and allocates the batch
// workspace and uploads the segment tables.
flct_status plan_batch(flct_ctx* ctx, int npairs, const flct_pair* pairs, BatchPlan* bp) {
    bp->jobs.assign(npairs, Job{});
    for (int k = 0; k < npairs; ++k) {
        const flct_pair& q = pairs[k];
        flct_status s = plan_job(ctx, &q.params, q.f1, q.f2, q.nx, q.ny, q.vx, q.vy, q.vm, &bp->jobs[k]);
        if (s != FLCT_OK) return pair_fail(ctx, s, k);
        if (bp->jobs[k].d.global)
            return pair_fail(ctx, fail(ctx, FLCT_ERR_UNSUPPORTED, "sigma <= 0 frames are not batched"), k);
        int form = 0;
        s = pick_form(ctx, q.params.form, bp->jobs[k].n, &form);  // rejects forms without a kernel for n
        if (s != FLCT_OK) return pair_fail(ctx, s, k);
    }
    // groups: same box, requested form and window tables
    for (int k = 0; k < npairs; ++k) {
        const Job& j = bp->jobs[k];
        BatchGroup g;
        g.n = j.n;
        g.req_form = j.p->form;
        g.use_filter = j.p->filter ? 1 : 0;
        g.hires = j.p->hires ? 1 : 0;
        fill_tables(j.p, j.n, g.gauss, g.filt2);
        g.sigma = j.p->sigma;
        g.kr = j.p->filter ? j.p->kr : 0.;
        bool found = false;
        for (auto& G : bp->groups)
            if (G.n == g.n && G.req_form == g.req_form && G.use_filter == g.use_filter && G.hires == g.hires &&
                (g.n <= kMaxBox || (G.sigma == g.sigma && G.kr == g.kr)) &&
                !memcmp(G.gauss, g.gauss, sizeof(g.gauss)) && !memcmp(G.filt2, g.filt2, sizeof(g.filt2))) {
                G.pairs.push_back(k);
                found = true;
                break;
            }
        if (!found) {
            g.pairs.push_back(k);
            bp->groups.push_back(g);
        }
    }
    // workspace: per-pair arena slices, item-indexed arrays shared by all pairs
    struct Off {
        size_t s12, r1, r2, re1, re2, grid;
        long long base;
    };
    std::vector<Off> off(npairs);
    size_t arena = 0;
    long long items = 0;
    auto take = [&arena](size_t bytes) {
        const size_t o = arena;
        arena += align256(bytes);
        return o;
    };
    for (int k = 0; k < npairs; ++k) {
        const JobSizes z = job_sizes(bp->jobs[k]);
        Off& o = off[k];
        o.s12 = take(z.s);
        o.r1 = take(z.r);
        o.r2 = take(z.r);
        o.re1 = take(z.re);
        o.re2 = take(z.re);
        o.grid = take(z.grid);
        o.base = items;
        items += (long long)bp->jobs[k].nx * bp->jobs[k].ny;
    }
    if (items >= (1ll << 31)) return fail(ctx, FLCT_ERR_UNSUPPORTED, "batch larger than 2^31 pixels in total");
    const int ng = (int)bp->groups.size();
    const size_t seg_bytes = align256((size_t)npairs * sizeof(WinSeg));
    const size_t start_bytes = align256((size_t)(npairs + ng) * sizeof(int));
    const size_t pair_bytes = align256((size_t)npairs * sizeof(int));
    const size_t first_bytes = align256((size_t)(ng + 1) * sizeof(int));
    ENSURE(ctx->bb_arena, arena);
    ENSURE(ctx->bb_work, (size_t)items * sizeof(int));
    ENSURE(ctx->bb_means, (size_t)items * sizeof(float4));  // a pair's grid has at most its pixels
    ENSURE(ctx->bb_peaks, (size_t)items * sizeof(PeakRec));
    bool any_hires = false;
    for (const auto& G : bp->groups) any_hires |= G.hires != 0;
    if (any_hires) ENSURE(ctx->bb_peaks_h, (size_t)items * sizeof(PeakRecH));
    ENSURE(ctx->bb_ctr, (size_t)npairs * 64);
    ENSURE(ctx->bb_meta, seg_bytes + start_bytes + pair_bytes + first_bytes);
    unsigned char* A = (unsigned char*)ctx->bb_arena.p;
    bp->bufs.assign(npairs, JobBufs{});
    for (int k = 0; k < npairs; ++k) {
        const Off& o = off[k];
        JobBufs& b = bp->bufs[k];
        b.s12 = (float4*)(A + o.s12);
        b.r1 = (BoxSum*)(A + o.r1);
        b.r2 = (BoxSum*)(A + o.r2);
        b.re1 = (int*)(A + o.re1);
        b.re2 = (int*)(A + o.re2);
        b.grid = (float2*)(A + o.grid);
        b.work = (int*)ctx->bb_work.p + o.base;
        b.means = (float4*)ctx->bb_means.p + o.base;
        b.peaks = (PeakRec*)ctx->bb_peaks.p + o.base;
        b.peaks_h = any_hires ? (PeakRecH*)ctx->bb_peaks_h.p + o.base : nullptr;
        b.ctr = (unsigned char*)ctx->bb_ctr.p + 64 * (size_t)k;
    }
    // segment tables, group-major
    std::vector<unsigned char> meta(seg_bytes + start_bytes + pair_bytes + first_bytes, 0);
    WinSeg* hs = (WinSeg*)meta.data();
    int* hpair = (int*)(meta.data() + seg_bytes + start_bytes);
    int* hfirst = (int*)(meta.data() + seg_bytes + start_bytes + pair_bytes);
    int e = 0;
    for (int g = 0; g < ng; ++g) {
        hfirst[g] = e;
        for (int k : bp->groups[g].pairs) {
            WinSeg sg{};
            sg.s12 = bp->bufs[k].s12;
            sg.nx = bp->jobs[k].nx;
            sg.ny = bp->jobs[k].ny;
            sg.base = (int)off[k].base;
            sg.mg = MeanGrid{bp->jobs[k].gs, bp->jobs[k].xo, bp->jobs[k].yo, bp->jobs[k].gj};
            hs[e] = sg;
            hpair[e] = k;
            ++e;
        }
    }
    hfirst[ng] = e;
    bp->h_first.assign(hfirst, hfirst + ng + 1);
    unsigned char* M = (unsigned char*)ctx->bb_meta.p;
    CK(cudaMemcpy(M, meta.data(), meta.size(), cudaMemcpyHostToDevice));
    bp->segs = (WinSeg*)M;
    bp->starts = (int*)(M + seg_bytes);
    bp->seg_pair = (int*)(M + seg_bytes + start_bytes);
    bp->first = (int*)(M + seg_bytes + start_bytes + pair_bytes);
    return plan_multi(ctx, bp);
}

// Window-kernel arguments of group g (all its pairs in one launch).
void group_wargs(flct_ctx* ctx, const BatchPlan& bp, int g, WinArgs* wa) {
    const BatchGroup& G = bp.groups[g];
    *wa = WinArgs{};
    memcpy(wa->gauss, G.gauss, sizeof(G.gauss));
    memcpy(wa->filt2, G.filt2, sizeof(G.filt2));
    wa->sigma = G.sigma;
    wa->kr = G.kr;
    wa->use_filter = G.use_filter;
    wa->means = (const float4*)ctx->bb_means.p;
    wa->work = (const int*)ctx->bb_work.p;
    wa->peaks = (PeakRec*)ctx->bb_peaks.p;
    wa->peaks_h = G.hires ? (PeakRecH*)ctx->bb_peaks_h.p : nullptr;
    wa->nsize = G.n / 2;
    wa->nseg = bp.h_first[g + 1] - bp.h_first[g];
    wa->segs = bp.segs + bp.h_first[g];
    wa->seg_start = bp.starts + bp.h_first[g] + g;
    wa->nwork = wa->seg_start + wa->nseg;
}

// The prepass of every pair of a batch as merged launches: one counter
// memset, the relative thresholds, the classification (on a side stream,
// beside the box sums: all three only read the frames), row and column box
// sums with the means, then the per-group prefix sums of the work counts.  With
// `side` null everything runs on bs.
flct_status enqueue_batch_prepass(flct_ctx* ctx, BatchPlan& bp, cudaStream_t bs, cudaStream_t side, int* launches) {
    const int np = (int)bp.jobs.size();
    const int ng = (int)bp.groups.size();
    CK(cudaMemsetAsync(ctx->bb_ctr.p, 0, (size_t)np * 64, bs));
    CK(launch_multi(ctx, k_absmax_multi, bp.m_abs, 256, 0, bs, launches));
    CK(launch_multi(ctx, k_thresh_final_multi, bp.m_thr, 32, 0, bs, launches));
    cudaStream_t cs = side ? side : bs;
    if (side) {
        CK(cudaEventRecord(ctx->bev[0], bs));
        CK(cudaStreamWaitEvent(side, ctx->bev[0], 0));
    }
    if (!ctx->box_attr) {
        CK(cudaFuncSetAttribute(k_box_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kBoxRowsSmem));
        CK(cudaFuncSetAttribute(k_box_rows_multi, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kBoxRowsSmem));
        ctx->box_attr = true;
    }
    CK(launch_multi(ctx, k_box_rows_multi, bp.m_rows, kBoxWarps * 32, kBoxRowsSmem, bs, launches));
    CK(launch_multi(ctx, k_classify_multi, bp.m_cls, 256, 0, cs, launches));
    CK(launch_multi(ctx, k_box_cols_multi, bp.m_cols, 128, 0, bs, launches));
    if (side) {
        CK(cudaEventRecord(ctx->bev[1], side));
        CK(cudaStreamWaitEvent(bs, ctx->bev[1], 0));
    }
    k_batch_starts<<<(ng + 31) / 32, 32, 0, bs>>>((const unsigned char*)ctx->bb_ctr.p, bp.seg_pair, bp.first, ng,
                                                   bp.starts);
    ++*launches;
    CK(cudaGetLastError());
    return FLCT_OK;
}

// Enqueues a planned batch on `bs`: the merged prepass, one persistent
// window launch per group (groups on the context's branch streams, so that
// a stream capture makes them parallel graph branches), then the merged
// fit and interpolation of every pair.
flct_status enqueue_batch(flct_ctx* ctx, BatchPlan& bp, cudaStream_t bs, bool branches, int* launches) {
    const int np = (int)bp.jobs.size();
    const int ng = (int)bp.groups.size();
    const int nb = branches ? std::min(std::max(ng, 1), flct_ctx::kBranches) : 0;
    flct_status s = enqueue_batch_prepass(ctx, bp, bs, branches ? ctx->bstream[0] : nullptr, launches);
    if (s != FLCT_OK) return s;
    if (nb) {
        CK(cudaEventRecord(ctx->bev[0], bs));
        for (int k = 0; k < nb; ++k) CK(cudaStreamWaitEvent(ctx->bstream[k], ctx->bev[0], 0));
    }
    auto lane = [&](int i) { return nb ? ctx->bstream[i % nb] : bs; };
    for (int g = 0; g < ng && s == FLCT_OK; ++g) {
        const BatchGroup& G = bp.groups[g];
        WinArgs wa;
        group_wargs(ctx, bp, g, &wa);
        unsigned* status = (unsigned*)(bp.bufs[G.pairs[0]].ctr + 4);
        s = launch_windows(ctx, G.form, find_win(G.n), G.n, wa, status, lane(g), G.cfg);
        ++*launches;
    }
    if (s != FLCT_OK) return s;
    for (int k = 0; k < nb; ++k) {
        CK(cudaEventRecord(ctx->bev[1 + k], ctx->bstream[k]));
        CK(cudaStreamWaitEvent(bs, ctx->bev[1 + k], 0));
    }
    CK(launch_multi(ctx, k_fit_multi, bp.m_fit, 128, 0, bs, launches));
    CK(launch_multi(ctx, k_fit_hires_multi, bp.m_fith, 128, 0, bs, launches));
    CK(launch_multi(ctx, k_interp_grid_multi, bp.m_interp, kInterpThreads, 0, bs, launches));
    (void)np;
    return FLCT_OK;
}

// Autotunes every FLCT_FORM_AUTO group whose box size has no measurement
// yet, on the batch's own work lists (runs the prepasses eagerly, syncs).
flct_status tune_batch(flct_ctx* ctx, BatchPlan& bp, cudaStream_t bs) {
    bool any = false;
    for (const auto& G : bp.groups) any |= G.req_form == FLCT_FORM_AUTO && !ctx->tune.count(G.n);
    if (!any) return FLCT_OK;
    int launches = 0;
    flct_status ps = enqueue_batch_prepass(ctx, bp, bs, nullptr, &launches);
    if (ps != FLCT_OK) return ps;
    const int ng = (int)bp.groups.size();
    for (int g = 0; g < ng; ++g) {
        const BatchGroup& G = bp.groups[g];
        if (G.req_form != FLCT_FORM_AUTO || ctx->tune.count(G.n)) continue;
        WinArgs wa;
        group_wargs(ctx, bp, g, &wa);
        unsigned* status = (unsigned*)(bp.bufs[G.pairs[0]].ctr + 4);
        for (int f : {FLCT_FORM_FP32, FLCT_FORM_TC_FP16}) {
            if (f != FLCT_FORM_FP32 && tc_index(G.n) < 0) continue;
            flct_status s = prime_form(ctx, f, G.n);
            if (s != FLCT_OK) return s;
        }
        flct_status s = tune_windows(ctx, find_win(G.n), G.n, wa, status, wa.nwork, bs);
        if (s != FLCT_OK) return s;
    }
    CK(cudaStreamSynchronize(bs));
    return FLCT_OK;
}

// Plans the batch, tunes what needs tuning, captures the whole batch as one
// CUDA graph and instantiates it.
flct_status rebuild_batch(flct_ctx* ctx, int npairs, const flct_pair* pairs, cudaStream_t st) {
    // the previous batch's graph may still be running on the workspace
    if (ctx->bdone) CK(cudaEventSynchronize(ctx->bdone));
    if (ctx->gexec) {
        cudaGraphExecDestroy(ctx->gexec);
        ctx->gexec = nullptr;
    }
    ctx->gkey.clear();
    for (int k = 0; k < flct_ctx::kBranches; ++k)
        if (!ctx->bstream[k]) CK(cudaStreamCreateWithFlags(&ctx->bstream[k], cudaStreamNonBlocking));
    for (auto& e : ctx->bev)
        if (!e) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    if (!ctx->bdone) CK(cudaEventCreateWithFlags(&ctx->bdone, cudaEventDisableTiming));
    BatchPlan bp;
    flct_status s = plan_batch(ctx, npairs, pairs, &bp);
    if (s != FLCT_OK) return s;
    cudaStream_t bs = ctx->stream;
    // the internal stream sees the caller's inputs before the tuning pass
    CK(cudaEventRecord(ctx->bev[0], st));
    CK(cudaStreamWaitEvent(bs, ctx->bev[0], 0));
    s = tune_batch(ctx, bp, bs);
    if (s != FLCT_OK) return s;
    for (auto& G : bp.groups) {
        resolved_config(ctx, G.req_form, G.n, &G.form, &G.cfg);
        s = prime_form(ctx, G.form, G.n);
        if (s != FLCT_OK) return s;
    }
    CK(cudaStreamBeginCapture(bs, cudaStreamCaptureModeRelaxed));
    int launches = 0;
    s = enqueue_batch(ctx, bp, bs, true, &launches);
    cudaGraph_t graph = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(bs, &graph);
    if (s != FLCT_OK || ec != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        cudaGetLastError();
        if (s != FLCT_OK) return s;
        return fail(ctx, FLCT_ERR_CUDA, "capturing the batch failed: %s", cudaGetErrorString(ec));
    }
    const cudaError_t ei = cudaGraphInstantiate(&ctx->gexec, graph, 0);
    cudaGraphDestroy(graph);
    if (ei != cudaSuccess) {
        ctx->gexec = nullptr;
        return fail(ctx, FLCT_ERR_CUDA, "instantiating the batch graph failed: %s", cudaGetErrorString(ei));
    }
    ctx->gkey = batch_key(npairs, pairs);
    ctx->batch_launches = launches;
    ctx->batch_box = bp.groups.size() == 1 ? bp.groups[0].n : 0;
    ctx->batch_form = bp.groups[0].form;
    return FLCT_OK;
}

// The device call's kernels after the tuning point (from_start: also the
// prepass): stage events for flct_gpu_last_timing (recorded as graph nodes
// when capturing), windows, fit, interpolation and the counters' copy to
// page-locked memory.
flct_status enqueue_device_tail(flct_ctx* ctx, const Job& j, const JobBufs& b, int form, WinCfg cfg,
                                cudaStream_t st, bool graph, int* launches, bool from_start = false) {
    // Stage events.  Eager: plain records.  Captured: ev[0] and ev[3] are
    // recorded on the caller's stream around the graph launch, and the
    // others become external event nodes on a side branch off the kernel
    // chain (a node inside the chain would delay the next kernel by its own
    // latency, ~2 us each).
    auto stamp = [&](cudaEvent_t ev) -> cudaError_t {
        if (!graph) return cudaEventRecord(ev, st);
        cudaError_t e = cudaEventRecord(ctx->tfork, st);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(ctx->tstream, ctx->tfork, 0);
        if (e == cudaSuccess) e = cudaEventRecordWithFlags(ev, ctx->tstream, cudaEventRecordExternal);
        return e;
    };
    flct_status s = FLCT_OK;
    if (from_start) {
        if (!graph) CK(cudaEventRecord(ctx->ev[0], st));
        s = enqueue_prepass(ctx, j, b, st, launches, ctx->prestream[0]);
        if (s != FLCT_OK) return s;
    }
    // the last kernel copies the work count and status to page-locked
    // memory; they are there once ev[3] completes
    const Pub pub{(const unsigned*)b.ctr, ctx->hctr_dev};
    WinArgs wa;
    make_wargs(j, b, &wa);
    CK(stamp(ctx->ev[1]));
    // the window, fit and interpolation kernels launch as programmatic
    // dependents: each one's launch overlaps the tail of the kernel before it
    s = launch_windows(ctx, form, j.we, j.n, wa, (unsigned*)(b.ctr + 4), st, cfg, -1, true);
    if (s != FLCT_OK) return s;
    ++*launches;
    CK(stamp(ctx->ev[2]));
    s = enqueue_fit(ctx, j, b, st, launches, -1, j.interp ? Pub{} : pub, true);
    if (s != FLCT_OK) return s;
    CK(stamp(ctx->ev[7]));
    if (j.interp) {
        s = enqueue_interp(ctx, j, b, st, launches, 0, -1, pub, true);
        if (s != FLCT_OK) return s;
    }
    if (graph) {  // the side branch joins the chain's end
        CK(cudaEventRecord(ctx->tjoin, ctx->tstream));
        CK(cudaStreamWaitEvent(st, ctx->tjoin, 0));
    } else {
        CK(cudaEventRecord(ctx->ev[3], st));
    }
    return FLCT_OK;
}

// ------------------------------------------------ banded host calls --

// Row bands of a host-buffer call.  Band b owns pixel rows [R[b], R[b+1])
// (its windows are the grid rows [Q[b], Q[b+1])) and completes output rows
// [O[b], O[b+1]).  Its box sums and windows read input rows up to C[b+1],
// the end of its last grid row's box, so the input is copied, classified
// and row-summed in chunks [C[b], C[b+1]): band b can start as soon as
// chunk b has arrived.  A chunk's windows go to the work list of the band
// that owns their row (chunk b spans bands b and b + 1), so a band must be
// taller than a box; the interpolation of an output row reads two grid
// rows below it, so O[b+1] trails Q[b+1] by two.
struct Bands {
    int nb = 0;
    int R[flct_ctx::kMaxBands + 1], Q[flct_ctx::kMaxBands + 1], O[flct_ctx::kMaxBands + 1];
    int C[flct_ctx::kMaxBands + 1];
};

bool plan_bands(const flct_ctx* ctx, const Job& j, Bands* bd) {
    if (j.d.global || j.d.rel_thresh || j.gi < 1) return false;
    for (int nb = std::min(ctx->host_bands_max, j.gi / (2 * kColRun)); nb >= 2; --nb) {
        bool ok = true;
        // band starts at multiples of the column pass's run
        for (int b = 0; b <= nb; ++b)
            bd->Q[b] = (b == nb) ? j.gi : (int)((long)j.gi * b / nb) / kColRun * kColRun;
        for (int b = 0; b <= nb; ++b) bd->R[b] = (b == 0) ? 0 : (b == nb) ? j.nx : j.xo + bd->Q[b] * j.gs;
        bd->O[0] = 0;
        bd->O[nb] = j.nx;
        for (int b = 1; b < nb; ++b)
            bd->O[b] = j.interp ? std::min(std::max(j.xo + (bd->Q[b] - 2) * j.gs, bd->O[b - 1]), j.nx) : bd->R[b];
        bd->C[0] = 0;
        bd->C[nb] = j.nx;
        for (int b = 0; b < nb && ok; ++b) {
            if (bd->Q[b + 1] <= bd->Q[b]) ok = false;
            // input rows the band's box sums and windows read lie in bands <= b + 1
            const int last = j.xo + (bd->Q[b + 1] - 1) * j.gs;
            const int need = box_start(last, j.nx, j.d.nsize) + j.n;
            if (b + 2 <= nb && need > bd->R[b + 2]) ok = false;
            if (b + 1 < nb) bd->C[b + 1] = std::min(std::max(need, bd->R[b + 1]), j.nx);
        }
        if (ok) {
            bd->nb = nb;
            return true;
        }
    }
    return false;
}

// Workspace of a banded call.
flct_status banded_buffers(flct_ctx* ctx, const Job& j) {
    const JobSizes z = job_sizes(j);
    ENSURE(ctx->b_s1, z.s);
    ENSURE(ctx->b_work, z.work);
    ENSURE(ctx->b_ctr, 64 * flct_ctx::kMaxBands);
    ENSURE(ctx->b_r1, z.r);
    ENSURE(ctx->b_r2, z.r);
    ENSURE(ctx->b_re1, z.re);
    ENSURE(ctx->b_re2, z.re);
    ENSURE(ctx->b_means, z.means);
    ENSURE(ctx->b_peaks, z.peaks);
    if (z.peaks_h) ENSURE(ctx->b_peaks_h, z.peaks_h);
    if (j.interp) ENSURE(ctx->b_grid, z.grid);
    return FLCT_OK;
}

// Enqueues flct_gpu_velocity in bands (buffers from banded_buffers): each
// band's rows are classified and summed as soon as they (and a box of rows
// below them) are copied in, its windows compute while later bands are
// still copied in, and its finished output rows are copied out while later
// bands compute.  Each kernel does the same per-window and per-pixel work as
// in the one-band call, and the box sums are exact, so the results are
// identical.  Every stream joins ctx->stream at the end, so the enqueue can
// also run inside a stream capture.
flct_status enqueue_banded(flct_ctx* ctx, const Job& j, const Bands& bd, int form, WinCfg cfg, const double* f1,
                           const double* f2, double* vx, double* vy, double* vm, int* nlaunch) {
    const int nb = bd.nb;
    const size_t ny = (size_t)j.ny;
    const JobSizes z = job_sizes(j);
    JobBufs base;
    base.s12 = (float4*)ctx->b_s1.p;
    base.work = (int*)ctx->b_work.p;
    base.means = (float4*)ctx->b_means.p;
    base.peaks = (PeakRec*)ctx->b_peaks.p;
    base.peaks_h = (PeakRecH*)ctx->b_peaks_h.p;
    base.r1 = (BoxSum*)ctx->b_r1.p;
    base.r2 = (BoxSum*)ctx->b_r2.p;
    base.grid = (float2*)ctx->b_grid.p;
    base.re1 = (int*)ctx->b_re1.p;
    base.re2 = (int*)ctx->b_re2.p;
    // band b's work items and peak records start at pixel R[b] * ny (a band
    // has at most that many windows), its counters at ctr + 64 b; the means
    // are one grid-indexed array, each band's column sums fill its grid rows
    JobBufs bb[flct_ctx::kMaxBands];
    for (int b = 0; b < nb; ++b) {
        bb[b] = base;
        const size_t off = (size_t)bd.R[b] * ny;
        bb[b].work = base.work + off;
        bb[b].peaks = base.peaks + off;
        bb[b].peaks_h = z.peaks_h ? base.peaks_h + off : nullptr;
        bb[b].ctr = (unsigned char*)ctx->b_ctr.p + 64 * b;
    }
    cudaStream_t st = ctx->stream, cin = ctx->cstream[0], cout = ctx->cstream[1];
    // prepass streams: classification, row sums, column sums
    cudaStream_t pc = ctx->prestream[0], pr = ctx->prestream[1], pb = ctx->prestream[2];
    cudaStream_t* bs = ctx->bandstream;
    constexpr int kB = flct_ctx::kMaxBands, kC = kB, kF = 2 * kB, kP = 3 * kB, kK = 4 * kB, kR = 5 * kB,
                  kFork = 6 * kB, kJoin = 6 * kB + 1;
    double *d_f1 = (double*)j.f1, *d_f2 = (double*)j.f2;
    CK(cudaEventRecord(ctx->hev[kFork], st));
    for (cudaStream_t x : {cin, cout, pc, pr, pb}) CK(cudaStreamWaitEvent(x, ctx->hev[kFork], 0));
    // input chunk b = rows [C[b], C[b+1]): everything band b's box sums and
    // windows read beyond the chunks before it
    for (int b = 0; b < nb; ++b) {
        const size_t o = (size_t)bd.C[b] * ny, len = (size_t)(bd.C[b + 1] - bd.C[b]) * ny * sizeof(double);
        if (len) {
            CK(cudaMemcpyAsync(d_f1 + o, f1 + o, len, cudaMemcpyHostToDevice, cin));
            CK(cudaMemcpyAsync(d_f2 + o, f2 + o, len, cudaMemcpyHostToDevice, cin));
        }
        CK(cudaEventRecord(ctx->hev[b], cin));
    }
    int launches = 0;
    WinArgs wa;
    make_wargs(j, base, &wa);
    // the prepass follows the chunks: chunk b's classification (its windows
    // to the lists of bands b and b + 1, split at R[b+1]) and row sums as
    // soon as it arrives, then band b's column sums, whose rows are all in
    // chunks <= b
    CK(cudaMemsetAsync(ctx->b_ctr.p, 0, 64 * nb, pc));
    flct_status s = FLCT_OK;
    for (int b = 0; b < nb && s == FLCT_OK; ++b) {
        CK(cudaStreamWaitEvent(pc, ctx->hev[b], 0));
        CK(cudaStreamWaitEvent(pr, ctx->hev[b], 0));
        s = enqueue_box_rows(ctx, j, base, bd.C[b], bd.C[b + 1], pr, &launches);
        if (s == FLCT_OK && bd.C[b + 1] > bd.C[b])
            s = enqueue_classify(ctx, j, bb[b], bd.C[b], bd.C[b + 1], nullptr, pc, &launches, 8,
                                 b + 1 < nb ? &bb[b + 1] : nullptr, bd.R[b + 1]);
        if (s != FLCT_OK) break;
        CK(cudaEventRecord(ctx->hev[kR + b], pr));
        CK(cudaEventRecord(ctx->hev[kK + b], pc));
        CK(cudaStreamWaitEvent(pb, ctx->hev[kR + b], 0));
        s = enqueue_box_cols(ctx, j, base, bd.Q[b], bd.Q[b + 1], pb, &launches);
        CK(cudaEventRecord(ctx->hev[kP + b], pb));
    }
    for (int b = 0; b < nb && s == FLCT_OK; ++b) {
        cudaStream_t sb = bs[b];
        // the band's means (its column sums), its work list and the float
        // split of every row its windows read (chunks <= b's classification)
        CK(cudaStreamWaitEvent(sb, ctx->hev[kP + b], 0));
        CK(cudaStreamWaitEvent(sb, ctx->hev[kK + b], 0));
        // the band's windows: at most its grid points
        const long items = (long)(bd.Q[b + 1] - bd.Q[b]) * j.gj;
        // the band's last kernel copies its counters to page-locked memory
        const Pub pub{(const unsigned*)bb[b].ctr, ctx->hctr_dev + 16 * b};
        const bool interp = j.interp && bd.O[b + 1] > bd.O[b];
        WinArgs wb = wa;
        wb.work = bb[b].work;
        wb.nwork = (const int*)bb[b].ctr;
        wb.peaks = bb[b].peaks;
        wb.peaks_h = j.p->hires ? bb[b].peaks_h : nullptr;
        // a band's window launch: one CTA per CTA-full of windows, in the
        // FP32 form's launch shape with fewer windows per CTA (CTAs retire
        // more often, so the other streams' kernels interleave more finely:
        // 4 teams instead of 8 at n = 32 took 1.5% off a 1024^2 call)
        WinCfg bcfg = cfg;
        if (form == FLCT_FORM_FP32 && j.we) bcfg.variant = j.we->teams[1] < j.we->teams[0] ? 1 : 0;
        s = launch_windows(ctx, form, j.we, j.n, wb, (unsigned*)(bb[b].ctr + 4), sb, bcfg, items);
        ++launches;
        if (s == FLCT_OK) s = enqueue_fit(ctx, j, bb[b], sb, &launches, items, interp ? Pub{} : pub);
        if (s != FLCT_OK) break;
        CK(cudaEventRecord(ctx->hev[kF + b], sb));
        // the band's first output rows interpolate from the band before's grid
        if (b > 0) CK(cudaStreamWaitEvent(sb, ctx->hev[kF + b - 1], 0));
        if (interp) s = enqueue_interp(ctx, j, base, sb, &launches, bd.O[b], bd.O[b + 1], pub);
        if (s != FLCT_OK) break;
        CK(cudaEventRecord(ctx->hev[kC + b], sb));
        CK(cudaStreamWaitEvent(cout, ctx->hev[kC + b], 0));
        const size_t o = (size_t)bd.O[b] * ny, len = (size_t)(bd.O[b + 1] - bd.O[b]) * ny * sizeof(double);
        if (len) {
            CK(cudaMemcpyAsync(vx + o, j.vx + o, len, cudaMemcpyDeviceToHost, cout));
            CK(cudaMemcpyAsync(vy + o, j.vy + o, len, cudaMemcpyDeviceToHost, cout));
            CK(cudaMemcpyAsync(vm + o, j.vm + o, len, cudaMemcpyDeviceToHost, cout));
        }
        CK(cudaStreamWaitEvent(st, ctx->hev[kC + b], 0));
    }
    if (s != FLCT_OK) return s;
    // the copy-out, copy-in and prepass streams join the call's stream
    CK(cudaEventRecord(ctx->hev[kJoin], cout));
    CK(cudaStreamWaitEvent(st, ctx->hev[kJoin], 0));
    for (cudaStream_t x : {cin, pc, pr, pb}) {
        CK(cudaEventRecord(ctx->hev[kJoin], x));
        CK(cudaStreamWaitEvent(st, ctx->hev[kJoin], 0));
    }
    *nlaunch = launches;
    return FLCT_OK;
}

bool page_locked(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

// flct_gpu_velocity in bands (see Bands).  With page-locked host buffers the
// whole enqueue is captured once as a CUDA graph and replayed while the
// call's parameters, sizes and pointers stay the same: one launch instead
// of ~100 stream operations per call.
flct_status velocity_banded(flct_ctx* ctx, const Job& j, const Bands& bd, int form, WinCfg cfg,
                            const double* f1, const double* f2, double* vx, double* vy, double* vm) {
    flct_status s = banded_buffers(ctx, j);
    if (s != FLCT_OK) return s;
    cudaStream_t st = ctx->stream;
    int launches = 0;
    const bool graph = page_locked(f1) && page_locked(f2) && page_locked(vx) && page_locked(vy) && page_locked(vm);
    if (graph) {
        std::vector<unsigned char> key;
        auto put = [&key](const void* v, size_t n) {
            const unsigned char* c = (const unsigned char*)v;
            key.insert(key.end(), c, c + n);
        };
        const flct_params& p = *j.p;
        const int ints[] = {j.nx, j.ny, bd.nb, form, cfg.grid_div, cfg.variant, p.thresh_abs, p.skip, p.poffset, p.qoffset,
                            p.interpolate, p.filter, p.hires};
        const double dbl[] = {p.deltat, p.deltas, p.sigma, p.thresh, p.kr};
        const void* ptrs[] = {f1, f2, vx, vy, vm, ctx->b_f1.p, ctx->b_f2.p, ctx->b_vx.p, ctx->b_vy.p, ctx->b_vm.p,
                              ctx->b_s1.p, ctx->b_s2.p, ctx->b_work.p, ctx->b_ctr.p, ctx->b_r1.p, ctx->b_r2.p,
                              ctx->b_b1.p, ctx->b_b2.p, ctx->b_means.p, ctx->b_peaks.p, ctx->b_peaks_h.p,
                              ctx->b_grid.p, ctx->b_tc.p, ctx->hctr, ctx->b_re1.p, ctx->b_re2.p};
        put(ints, sizeof(ints));
        put(dbl, sizeof(dbl));
        put(ptrs, sizeof(ptrs));
        if (!ctx->hexec || key != ctx->hkey) {
            if (ctx->hexec) {
                cudaGraphExecDestroy(ctx->hexec);
                ctx->hexec = nullptr;
            }
            ctx->hkey.clear();
            CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed));
            s = enqueue_banded(ctx, j, bd, form, cfg, f1, f2, vx, vy, vm, &launches);
            cudaGraph_t g = nullptr;
            const cudaError_t ec = cudaStreamEndCapture(st, &g);
            if (s != FLCT_OK || ec != cudaSuccess) {
                if (g) cudaGraphDestroy(g);
                cudaGetLastError();
                if (s != FLCT_OK) return s;
                return fail(ctx, FLCT_ERR_CUDA, "capturing the banded call failed: %s", cudaGetErrorString(ec));
            }
            // keep the band streams' priorities inside the graph
            const cudaError_t ei =
                cudaGraphInstantiateWithFlags(&ctx->hexec, g, cudaGraphInstantiateFlagUseNodePriority);
            cudaGraphDestroy(g);
            if (ei != cudaSuccess) {
                ctx->hexec = nullptr;
                return fail(ctx, FLCT_ERR_CUDA, "instantiating the banded graph failed: %s", cudaGetErrorString(ei));
            }
            ctx->hkey = key;
            ctx->hlaunches = launches;
        }
        launches = ctx->hlaunches;
        CK(cudaEventRecord(ctx->ev[4], st));
        CK(cudaGraphLaunch(ctx->hexec, st));
    } else {
        CK(cudaEventRecord(ctx->ev[4], st));
        s = enqueue_banded(ctx, j, bd, form, cfg, f1, f2, vx, vy, vm, &launches);
        if (s != FLCT_OK) {
            cudaStreamSynchronize(st);
            return s;
        }
    }
    CK(cudaEventRecord(ctx->ev[3], st));
    CK(cudaEventRecord(ctx->ev[6], st));
    ctx->timing = flct_timing{};
    ctx->timing.launches = launches;
    ctx->timing.box = j.n;
    ctx->timing.form = form;
    ctx->host_bands = bd.nb;
    ctx->pending = true;
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
    for (auto& e : ctx->tev)
        if (cudaEventCreate(&e) != cudaSuccess) {
            flct_gpu_destroy(ctx);
            return FLCT_ERR_CUDA;
        }
    for (auto& st : ctx->cstream)
        if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) {
            st = nullptr;
            flct_gpu_destroy(ctx);
            return FLCT_ERR_CUDA;
        }
    {
        int least = 0, greatest = 0;  // numerically: greatest <= least
        if (cudaDeviceGetStreamPriorityRange(&least, &greatest) != cudaSuccess) {
            flct_gpu_destroy(ctx);
            return FLCT_ERR_CUDA;
        }
        for (auto& ps : ctx->prestream)
            if (cudaStreamCreateWithPriority(&ps, cudaStreamNonBlocking, greatest) != cudaSuccess) {
                ps = nullptr;
                flct_gpu_destroy(ctx);
                return FLCT_ERR_CUDA;
            }
        for (int b = 0; b < flct_ctx::kMaxBands; ++b)
            if (cudaStreamCreateWithPriority(&ctx->bandstream[b], cudaStreamNonBlocking,
                                             std::min(least, greatest + 1 + b)) != cudaSuccess) {
                ctx->bandstream[b] = nullptr;
                flct_gpu_destroy(ctx);
                return FLCT_ERR_CUDA;
            }
    }
    for (auto& e : ctx->hev)
        if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) {
            e = nullptr;
            flct_gpu_destroy(ctx);
            return FLCT_ERR_CUDA;
        }
    for (auto& e : ctx->pev)
        if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) {
            e = nullptr;
            flct_gpu_destroy(ctx);
            return FLCT_ERR_CUDA;
        }
    for (auto* e : {&ctx->tfork, &ctx->tjoin})
        if (cudaEventCreateWithFlags(e, cudaEventDisableTiming) != cudaSuccess) {
            *e = nullptr;
            flct_gpu_destroy(ctx);
            return FLCT_ERR_CUDA;
        }
    if (cudaStreamCreateWithFlags(&ctx->tstream, cudaStreamNonBlocking) != cudaSuccess) {
        ctx->tstream = nullptr;
        flct_gpu_destroy(ctx);
        return FLCT_ERR_CUDA;
    }
    if (const char* nb = getenv("FLCT_HOST_BANDS"))
        ctx->host_bands_max = std::max(0, std::min(flct_ctx::kMaxBands, atoi(nb)));
    if (cudaHostAlloc((void**)&ctx->hctr, 64 * flct_ctx::kMaxBands, cudaHostAllocMapped) != cudaSuccess) {
        ctx->hctr = nullptr;
        flct_gpu_destroy(ctx);
        return FLCT_ERR_ALLOC;
    }
    memset(ctx->hctr, 0, 64 * flct_ctx::kMaxBands);
    if (cudaHostGetDevicePointer((void**)&ctx->hctr_dev, ctx->hctr, 0) != cudaSuccess) {
        flct_gpu_destroy(ctx);
        return FLCT_ERR_CUDA;
    }
    ctx->device_name = prop.name;
    if (const char* path = getenv("FLCT_AUTOTUNE_CACHE")) ctx->tune_path = path;
    tune_load(ctx);
    *out = ctx;
    return FLCT_OK;
}

void flct_gpu_destroy(flct_ctx* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    for (auto& st : ctx->cstream)
        if (st) cudaStreamSynchronize(st);
    for (auto& st : ctx->bandstream)
        if (st) cudaStreamSynchronize(st);
    for (auto& st : ctx->prestream)
        if (st) cudaStreamSynchronize(st);
    if (ctx->tstream) cudaStreamSynchronize(ctx->tstream);
    for (auto& st : ctx->bstream)
        if (st) cudaStreamSynchronize(st);
    if (ctx->bdone) cudaEventSynchronize(ctx->bdone);
    if (ctx->gexec) cudaGraphExecDestroy(ctx->gexec);
    if (ctx->hexec) cudaGraphExecDestroy(ctx->hexec);
    if (ctx->dexec) cudaGraphExecDestroy(ctx->dexec);
    for (auto* b : ctx->all())
        if (b->p) cudaFree(b->p);
    for (auto& e : ctx->ev)
        if (e) cudaEventDestroy(e);
    for (auto& e : ctx->tev)
        if (e) cudaEventDestroy(e);
    for (auto& e : ctx->bev)
        if (e) cudaEventDestroy(e);
    for (auto& e : ctx->hev)
        if (e) cudaEventDestroy(e);
    for (auto& e : ctx->pev)
        if (e) cudaEventDestroy(e);
    if (ctx->tfork) cudaEventDestroy(ctx->tfork);
    if (ctx->tjoin) cudaEventDestroy(ctx->tjoin);
    if (ctx->tstream) cudaStreamDestroy(ctx->tstream);
    for (auto& st : ctx->cstream)
        if (st) cudaStreamDestroy(st);
    for (auto& st : ctx->bandstream)
        if (st) cudaStreamDestroy(st);
    for (auto& st : ctx->prestream)
        if (st) cudaStreamDestroy(st);
    if (ctx->hctr) cudaFreeHost(ctx->hctr);
    if (ctx->bdone) cudaEventDestroy(ctx->bdone);
    for (auto& st : ctx->bstream)
        if (st) cudaStreamDestroy(st);
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
    Job j;
    flct_status s = plan_job(ctx, p, d_f1, d_f2, nx, ny, d_vx, d_vy, d_vm, &j);
    if (s != FLCT_OK) return s;
    CK(cudaSetDevice(ctx->device));
    cudaStream_t st = (cudaStream_t)stream;  // NULL: the CUDA default stream
    if (j.d.global) return velocity_global(ctx, j, st);
    const int n = j.n;
    int form = FLCT_FORM_FP32;
    s = pick_form(ctx, p->form, n, &form);
    if (s != FLCT_OK) return s;

    const JobSizes z = job_sizes(j);
    ENSURE(ctx->b_s1, z.s);
    ENSURE(ctx->b_work, z.work);
    ENSURE(ctx->b_ctr, 64);
    ENSURE(ctx->b_r1, z.r);
    ENSURE(ctx->b_r2, z.r);
    ENSURE(ctx->b_re1, z.re);
    ENSURE(ctx->b_re2, z.re);
    ENSURE(ctx->b_means, z.means);
    ENSURE(ctx->b_peaks, z.peaks);
    if (z.peaks_h) ENSURE(ctx->b_peaks_h, z.peaks_h);
    if (j.interp) {
        ENSURE(ctx->b_grid, z.grid);
    }
    JobBufs b;
    b.s12 = (float4*)ctx->b_s1.p;
    b.work = (int*)ctx->b_work.p;
    b.means = (float4*)ctx->b_means.p;
    b.peaks = (PeakRec*)ctx->b_peaks.p;
    b.peaks_h = (PeakRecH*)ctx->b_peaks_h.p;
    b.r1 = (BoxSum*)ctx->b_r1.p;
    b.r2 = (BoxSum*)ctx->b_r2.p;
    b.re1 = (int*)ctx->b_re1.p;
    b.re2 = (int*)ctx->b_re2.p;
    b.ctr = (unsigned char*)ctx->b_ctr.p;
    b.grid = (float2*)ctx->b_grid.p;
    unsigned* d_status = (unsigned*)(b.ctr + 4);

    ctx->batch_pending = 0;
    int launches = 0;
    WinCfg cfg;
    // first FLCT_FORM_AUTO call for this box size: time the candidates on
    // this work list, eagerly (not possible inside a stream capture)
    if (p->form == FLCT_FORM_AUTO && !ctx->tune.count(n) && !capturing(st)) {
        CK(cudaEventRecord(ctx->ev[0], st));
        s = enqueue_prepass(ctx, j, b, st, &launches, ctx->prestream[0]);
        if (s != FLCT_OK) return s;
        WinArgs wa;
        make_wargs(j, b, &wa);
        for (int f : {FLCT_FORM_FP32, FLCT_FORM_TC_FP16}) {
            if (f != FLCT_FORM_FP32 && tc_index(n) < 0) continue;
            s = prime_form(ctx, f, n);
            if (s != FLCT_OK) return s;
        }
        s = tune_windows(ctx, j.we, n, wa, d_status, (const int*)b.ctr, st);
        if (s != FLCT_OK) return s;
        resolved_config(ctx, p->form, n, &form, &cfg);
        s = enqueue_device_tail(ctx, j, b, form, cfg, st, false, &launches);
        if (s != FLCT_OK) return s;
    } else {
        resolved_config(ctx, p->form, n, &form, &cfg);
        s = prime_form(ctx, form, n);
        if (s != FLCT_OK) return s;
        // a call repeated with the same parameters and buffers is captured
        // once as a CUDA graph and replayed (one launch instead of ~12)
        std::vector<unsigned char> key;
        if (!capturing(st)) {
            auto put = [&key](const void* v, size_t nb) {
                const unsigned char* c = (const unsigned char*)v;
                key.insert(key.end(), c, c + nb);
            };
            const int ints[] = {nx, ny, form, cfg.grid_div, cfg.variant, p->thresh_abs, p->skip, p->poffset, p->qoffset,
                                p->interpolate, p->filter, p->hires};
            const double dbl[] = {p->deltat, p->deltas, p->sigma, p->thresh, p->kr};
            const void* ptrs[] = {d_f1, d_f2, d_vx, d_vy, d_vm, ctx->b_s1.p, ctx->b_s2.p, ctx->b_work.p,
                                  ctx->b_ctr.p, ctx->b_r1.p, ctx->b_r2.p, ctx->b_re1.p, ctx->b_re2.p, ctx->b_b1.p,
                                  ctx->b_b2.p, ctx->b_means.p, ctx->b_peaks.p, ctx->b_peaks_h.p, ctx->b_grid.p,
                                  ctx->b_tc.p, ctx->hctr};
            put(ints, sizeof(ints));
            put(dbl, sizeof(dbl));
            put(ptrs, sizeof(ptrs));
        }
        if (!key.empty() && ctx->dexec && key == ctx->dkey) {
            CK(cudaEventRecord(ctx->ev[0], st));
            CK(cudaGraphLaunch(ctx->dexec, st));
            CK(cudaEventRecord(ctx->ev[3], st));
            launches = ctx->dlaunches;
        } else if (!key.empty() && key == ctx->dlast) {
            if (ctx->dexec) {
                cudaGraphExecDestroy(ctx->dexec);
                ctx->dexec = nullptr;
            }
            ctx->dkey.clear();
            cudaStream_t cs = ctx->stream;
            CK(cudaStreamBeginCapture(cs, cudaStreamCaptureModeRelaxed));
            s = enqueue_device_tail(ctx, j, b, form, cfg, cs, true, &launches, true);
            cudaGraph_t g = nullptr;
            const cudaError_t ec = cudaStreamEndCapture(cs, &g);
            if (s != FLCT_OK || ec != cudaSuccess) {
                if (g) cudaGraphDestroy(g);
                cudaGetLastError();
                if (s != FLCT_OK) return s;
                return fail(ctx, FLCT_ERR_CUDA, "capturing the velocity call failed: %s", cudaGetErrorString(ec));
            }
            const cudaError_t ei = cudaGraphInstantiate(&ctx->dexec, g, 0);
            cudaGraphDestroy(g);
            if (ei != cudaSuccess) {
                ctx->dexec = nullptr;
                return fail(ctx, FLCT_ERR_CUDA, "instantiating the velocity graph failed: %s", cudaGetErrorString(ei));
            }
            ctx->dkey = key;
            ctx->dlaunches = launches;
            CK(cudaEventRecord(ctx->ev[0], st));
            CK(cudaGraphLaunch(ctx->dexec, st));
            CK(cudaEventRecord(ctx->ev[3], st));
        } else {
            ctx->dlast = key;
            s = enqueue_device_tail(ctx, j, b, form, cfg, st, false, &launches, true);
            if (s != FLCT_OK) return s;
        }
    }
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
    long long nwork = 0;
    unsigned status = 0;
    const bool batch = ctx->batch_pending > 0;
    if (batch) {
        // a batch: every pair's counters
        std::vector<unsigned char> h((size_t)ctx->batch_pending * 64);
        ctx->batch_pending = 0;
        CK(cudaMemcpy(h.data(), ctx->bb_ctr.p, h.size(), cudaMemcpyDeviceToHost));
        for (size_t k = 0; k < h.size(); k += 64) {
            int w;
            unsigned st;
            memcpy(&w, h.data() + k, sizeof(int));
            memcpy(&st, h.data() + k + 4, sizeof(unsigned));
            nwork += w;
            status |= st;
        }
    } else {
        // one band, or each band of a banded host call
        const int nb = std::max(1, ctx->host_bands);
        for (int b = 0; b < nb; ++b) {
            int w = 0;
            unsigned sb = 0;
            memcpy(&w, ctx->hctr + 64 * b, sizeof(int));
            memcpy(&sb, ctx->hctr + 64 * b + 4, sizeof(unsigned));
            nwork += w;
            status |= sb;
        }
    }
    ctx->timing.windows = nwork;
    if (ctx->host_bands > 0) {  // stages interleave across bands: only the total
        ctx->host_bands = 0;
        ctx->timing.ms_total = ev_ms(ctx->ev[4], ctx->ev[3]);
    } else if (!batch) {  // a batch's graph has no per-stage events
        ctx->timing.ms_prepass = ev_ms(ctx->ev[0], ctx->ev[1]);
        ctx->timing.ms_window = ev_ms(ctx->ev[1], ctx->ev[2]);
        ctx->timing.ms_fit = ev_ms(ctx->ev[2], ctx->ev[7]);
        ctx->timing.ms_interp = ev_ms(ctx->ev[7], ctx->ev[3]);
        ctx->timing.ms_total = ev_ms(ctx->ev[0], ctx->ev[3]);
    } else {
        ctx->timing.ms_total = ev_ms(ctx->ev[0], ctx->ev[3]);
    }
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
    // row bands whose copies overlap the computation, once the window form
    // is settled (a first FLCT_FORM_AUTO call tunes in one band)
    {
        Job j;
        flct_status s = plan_job(ctx, p, (const double*)ctx->b_f1.p, (const double*)ctx->b_f2.p, nx, ny,
                                 (double*)ctx->b_vx.p, (double*)ctx->b_vy.p, (double*)ctx->b_vm.p, &j);
        if (s != FLCT_OK) return s;
        Bands bd;
        if (!j.d.global && (p->form != FLCT_FORM_AUTO || ctx->tune.count(j.n)) && plan_bands(ctx, j, &bd)) {
            int form = FLCT_FORM_FP32;
            WinCfg cfg;
            s = pick_form(ctx, p->form, j.n, &form);
            if (s != FLCT_OK) return s;
            resolved_config(ctx, p->form, j.n, &form, &cfg);
            s = prime_form(ctx, form, j.n);
            if (s != FLCT_OK) return s;
            ctx->batch_pending = 0;
            s = velocity_banded(ctx, j, bd, form, cfg, f1, f2, vx, vy, vm);
            if (s != FLCT_OK) return s;
            CK(cudaEventSynchronize(ctx->ev[6]));
            s = collect_timing(ctx);
            ctx->timing.ms_total = ev_ms(ctx->ev[4], ctx->ev[6]);
            return s;
        }
    }
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
    if (!we && (n > kMaxBigBox || n % 4 != 0))
        return fail(ctx, FLCT_ERR_UNSUPPORTED, "window size %d has no GPU kernel", n);
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
    ENSURE(ctx->b_s1, npx * sizeof(float4));
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
    ca.s12 = (float4*)ctx->b_s1.p;
    ENSURE(ctx->b_aux2, npx * sizeof(int) + 64);
    ca.work = (int*)ctx->b_aux2.p;  // discarded list
    ca.nwork = (int*)(ctr + 32);
    ca.vx = ca.vy = ca.vm = nullptr;
    ca.status = (unsigned*)(ctr + 4);
    ca.r0 = 0;
    ca.r1 = nwin * n;
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
    for (int k = 0; k <= 2 * n && k <= 2 * kMaxBox; ++k) wa.gauss[k] = 1.0f;
    wa.sigma = 1.0;
    wa.kr = kr;
    wa.use_filter = filter;
    wa.s12 = (const float4*)ctx->b_s1.p;
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
    ENSURE(ctx->b_aux2, (size_t)2 * (nx + ny) * sizeof(double2));
    float2* sx = (float2*)ctx->b_aux1.p;
    float2* sy = sx + nx;
    // warp.c:811-820: shifts normalised by the axis lengths; transp swaps them
    const double dxarg = transp ? -dely / ((double)nx) : -delx / ((double)nx);
    const double dyarg = transp ? -delx / ((double)ny) : -dely / ((double)ny);
    const bool fft = shift_fft_axis(nx) && shift_fft_axis(ny);
    CK(cudaMemcpyAsync(ctx->b_f1.p, arr, n * sizeof(double), cudaMemcpyHostToDevice, st));
    CK(cudaEventRecord(ctx->ev[0], st));
    if (fft) {
        // power-of-two axes: the same linear map by transforms, O(N log N)
        CK(launch_shift_fft((const double*)ctx->b_f1.p, nx, ny, dxarg, dyarg, (double2*)ctx->b_aux2.p, sx,
                            (float2*)ctx->b_s1.p, (float2*)ctx->b_s2.p, (double*)ctx->b_vx.p, ctx->nsm, st));
    } else {
        CK(launch_shift_vector(nx, dxarg, (double2*)ctx->b_aux2.p, sx, st));
        CK(launch_shift_vector(ny, dyarg, (double2*)ctx->b_aux2.p, sy, st));
        CK(launch_axis_fast(0, true, ctx->b_f1.p, nx, ny, sy, (float2*)ctx->b_s1.p, st));
        CK(launch_axis_slow(0, (const float2*)ctx->b_s1.p, ny, nx, sx, (float2*)ctx->b_s2.p, st));
        CK(launch_real_part((const float2*)ctx->b_s2.p, (long)n, (double*)ctx->b_vx.p, st));
    }
    CK(cudaEventRecord(ctx->ev[1], st));
    CK(cudaMemcpyAsync(out, ctx->b_vx.p, n * sizeof(double), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    ctx->timing = flct_timing{};
    ctx->timing.launches = fft ? 8 : 7;
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
    // F = forward DFT of the image (warp.c:899-934): FFTs along both axes
    // when both are powers of two (64 .. kWarpMaxAxis), else DFT matrices
    const bool fft = shift_fft_axis(nx) && shift_fft_axis(ny);
    if (fft) {
        CK(launch_dft2_fft((const double*)ctx->b_f1.p, nx, ny, twx, (float2*)ctx->b_s1.p, (float2*)ctx->b_s2.p,
                           ctx->nsm, st));
    } else {
        CK(launch_twiddles(nx, -1, twx, st));
        CK(launch_twiddles(ny, -1, twy, st));
        CK(launch_axis_fast(1, true, ctx->b_f1.p, nx, ny, twy, (float2*)ctx->b_s1.p, st));
        CK(launch_axis_slow(1, (const float2*)ctx->b_s1.p, ny, nx, twx, (float2*)ctx->b_s2.p, st));
    }
    CK(launch_warp_phase((const double*)ctx->b_f2.p, (const double*)ctx->b_vy.p, nx, ny, transp,
                         (float4*)ctx->b_means.p, st));
    CK(cudaEventRecord(ctx->ev[1], st));
    // the spectral sum: tensor cores (split FP16, half spectrum) unless
    // FLCT_WARP_SUM=fp32 asks for the FP32 CUDA-core kernel
    const char* form = getenv("FLCT_WARP_SUM");
    const bool tc = !(form && strcmp(form, "fp32") == 0);
    unsigned wstatus = 0;
    if (tc) {
        ENSURE(ctx->b_whs, warp_tc_split_bytes(nx, ny));
        ENSURE(ctx->b_wmisc, 64);
        unsigned long long stall_ns = 0;  // test hook: see k_wt_sum
        if (const char* w = getenv("FLCT_TEST_WARP_STALL_NS")) stall_ns = strtoull(w, nullptr, 10);
        CK(launch_warp_sum_tc((const float2*)ctx->b_s2.p, (const float4*)ctx->b_means.p, nx, ny, ctx->b_whs.p,
                              (unsigned*)ctx->b_wmisc.p, (double*)ctx->b_vx.p, st, stall_ns));
    } else {
        CK(launch_warp_sum((const float2*)ctx->b_s2.p, (const float4*)ctx->b_means.p, nx, ny, (double*)ctx->b_vx.p,
                           st));
    }
    CK(cudaEventRecord(ctx->ev[2], st));
    CK(cudaMemcpyAsync(out, ctx->b_vx.p, n * sizeof(double), cudaMemcpyDeviceToHost, st));
    if (tc) CK(cudaMemcpyAsync(&wstatus, (unsigned*)ctx->b_wmisc.p + 1, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    ctx->timing = flct_timing{};
    ctx->timing.launches = (fft ? 6 : 4) + 1 + (tc ? 3 : 1);
    ctx->timing.ms_prepass = ev_ms(ctx->ev[0], ctx->ev[1]);
    ctx->timing.ms_window = ev_ms(ctx->ev[1], ctx->ev[2]);
    ctx->timing.ms_total = ev_ms(ctx->ev[0], ctx->ev[2]);
    if (wstatus & kStatusTimeout)
        return fail(ctx, FLCT_ERR_TIMEOUT, "a tensor-core stage of the warp sum did not complete within its wait limit");
    return FLCT_OK;
}

flct_status flct_gpu_velocity_batch(flct_ctx* ctx, int npairs, const flct_pair* pairs, void* stream) {
    if (!ctx) return FLCT_ERR_ARG;
    if (npairs < 0 || (npairs > 0 && !pairs)) return fail(ctx, FLCT_ERR_ARG, "bad pair list (%d pairs)", npairs);
    CK(cudaSetDevice(ctx->device));
    cudaStream_t st = (cudaStream_t)stream;
    ctx->pending = false;
    ctx->batch_pending = 0;
    ctx->timing = flct_timing{};
    if (npairs == 0) return FLCT_OK;
    if (!ctx->gexec || ctx->gkey != batch_key(npairs, pairs)) {
        flct_status s = rebuild_batch(ctx, npairs, pairs, st);
        if (s != FLCT_OK) return s;
    }
    CK(cudaEventRecord(ctx->ev[0], st));
    CK(cudaGraphLaunch(ctx->gexec, st));
    CK(cudaEventRecord(ctx->ev[3], st));
    CK(cudaEventRecord(ctx->bdone, st));
    ctx->timing.launches = ctx->batch_launches;
    ctx->timing.box = ctx->batch_box;
    ctx->timing.form = ctx->batch_form;
    ctx->pending = true;
    ctx->batch_pending = npairs;
    return FLCT_OK;
}

}  // extern "C"
