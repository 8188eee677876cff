// noalloc.cu -- interpcc2d for callers that cannot allocate device memory.
//
// Some host programs own every byte of GPU memory themselves: a serving
// process or framework that runs its own memory pool and does not let
// libraries call cudaMalloc behind its back, or a real-time pipeline that
// fixes its device-memory budget at start-up.  Such callers cannot use
// flct_gpu_interpcc2d, which allocates its workspace on first use.  This
// entry point does the same interpolation with caller-provided device
// buffers for the data, targets and result, and keeps its only scratch (the
// per-axis stencil rows and cubic-convolution weights) in the fixed array
// below, which every GPU that loads the library holds until the process
// exits.
#include <cuda.h>
#include <cuda_runtime.h>

#include <mutex>

#include "common.cuh"
#include "flct_gpu.h"
#include "prepass.cuh"

namespace {

constexpr int kMax = FLCT_NOALLOC_MAX_AXIS;
// per axis: 4 weights (double), the clamped stencil start (int), in-range flag
constexpr size_t kWts = (size_t)kMax * 4 * sizeof(double);
constexpr size_t kZero = (size_t)kMax * sizeof(int);
constexpr size_t kOk = (size_t)kMax;
constexpr size_t kBytes = 2 * (kWts + kZero + kOk);

static __device__ __align__(256) unsigned char g_noalloc_scratch[kBytes];

// The array's device address belongs to a CUDA context, not to a device
// ordinal: a cudaDeviceReset or a caller-made context on the same device
// gives the module (and the array) a new address.  So the looked-up address
// is kept per context, keyed by the driver's unique context id.
using PfnCtxGetCurrent = CUresult (*)(CUcontext*);
using PfnCtxGetId = CUresult (*)(CUcontext, unsigned long long*);
PfnCtxGetCurrent g_get_current = nullptr;
PfnCtxGetId g_get_id = nullptr;
std::once_flag g_entry_once;

constexpr int kMaxContexts = 64;
constexpr int kMaxDevices = 64;
std::mutex g_mu;
struct CtxEntry {
    unsigned long long id;
    unsigned char* ptr;
};
CtxEntry g_cache[kMaxContexts] = {};
int g_ncache = 0;
int g_devok[kMaxDevices] = {};  // 0 unknown, 1 sm_103, -1 other

void load_entry_points() {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
        g_get_current = reinterpret_cast<PfnCtxGetCurrent>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
        g_get_id = reinterpret_cast<PfnCtxGetId>(f);
}

// Unique id of the calling thread's current context, 0 if unknown.
unsigned long long current_ctx_id() {
    if (!g_get_current || !g_get_id) return 0;
    CUcontext c = nullptr;
    unsigned long long id = 0;
    if (g_get_current(&c) != CUDA_SUCCESS || !c) return 0;
    if (g_get_id(c, &id) != CUDA_SUCCESS) return 0;
    return id;
}

// Device address of the scratch array in the current context: looked up
// with cudaGetSymbolAddress the first time a context calls (host code cannot
// use the array's name as a device pointer), then taken from the cache.
// Returns the CUDA error of a failed lookup in *err.
flct_status scratch_in_current_context(unsigned char** out, cudaError_t* err) {
    *err = cudaSuccess;
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return FLCT_ERR_NO_DEVICE;
    std::call_once(g_entry_once, load_entry_points);
    {
        std::lock_guard<std::mutex> lk(g_mu);
        if (g_devok[dev] == 0) {
            int major = 0, minor = 0;
            if (cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev) != cudaSuccess ||
                cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev) != cudaSuccess)
                return FLCT_ERR_NO_DEVICE;
            // the kernels are compiled for sm_103a only
            g_devok[dev] = (major == 10 && minor == 3) ? 1 : -1;
        }
        if (g_devok[dev] < 0) return FLCT_ERR_NO_DEVICE;
    }
    unsigned long long id = current_ctx_id();
    std::lock_guard<std::mutex> lk(g_mu);
    if (id != 0)
        for (int k = 0; k < g_ncache; ++k)
            if (g_cache[k].id == id) {
                *out = g_cache[k].ptr;
                return FLCT_OK;
            }
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
        *err = (e != cudaSuccess) ? e : cudaErrorInvalidSymbol;
        return FLCT_ERR_CUDA;
    }
    // the lookup binds the runtime's context on a thread that had none
    if (id == 0) id = current_ctx_id();
    if (id != 0) {
        if (g_ncache == kMaxContexts) g_ncache = 0;  // many contexts: start the cache over
        g_cache[g_ncache++] = {id, static_cast<unsigned char*>(p)};
    }
    *out = static_cast<unsigned char*>(p);
    return FLCT_OK;
}

// A device pointer of another device than the current one (the caller has
// the wrong device current) is refused; host, managed and system memory
// the GPU can reach are left to the caller.
bool on_other_device(const void* p, int dev) {
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) return false;
    return at.type == cudaMemoryTypeDevice && at.device != dev;
}

}  // namespace

extern "C" FLCT_API flct_status flct_gpu_interpcc2d_noalloc(const double* d_fdata, double xmiss, int nx,
                                                            int ny, const double* d_xwant, int nxi,
                                                            const double* d_ywant, int nyi, double* d_out,
                                                            void* stream) {
    if (!d_fdata || !d_xwant || !d_ywant || !d_out || nxi < 0 || nyi < 0) return FLCT_ERR_ARG;
    if (nx < 3 || ny < 3) return FLCT_ERR_GRID_TOO_SMALL;
    if (nxi > kMax || nyi > kMax) return FLCT_ERR_UNSUPPORTED;
    if (nxi == 0 || nyi == 0) return FLCT_OK;
    // An error some earlier work of the caller left pending stays the
    // caller's: this call only clears errors it raised itself, and only
    // when none was pending before it.
    const bool clean_before = cudaPeekAtLastError() == cudaSuccess;
    auto own_error = [&](flct_status s) {
        if (clean_before) cudaGetLastError();
        return s;
    };
    unsigned char* base = nullptr;
    cudaError_t lookup_err = cudaSuccess;
    flct_status s = scratch_in_current_context(&base, &lookup_err);
    if (s != FLCT_OK) return own_error(s);
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) return own_error(FLCT_ERR_NO_DEVICE);
    if (on_other_device(d_fdata, dev) || on_other_device(d_xwant, dev) || on_other_device(d_ywant, dev) ||
        on_other_device(d_out, dev))
        return own_error(FLCT_ERR_ARG);
    if (clean_before) cudaGetLastError();  // pointer queries of host memory may leave an error behind
    double* wx = reinterpret_cast<double*>(base);
    double* wy = reinterpret_cast<double*>(base + kWts);
    int* zx = reinterpret_cast<int*>(base + 2 * kWts);
    int* zy = reinterpret_cast<int*>(base + 2 * kWts + kZero);
    unsigned char* okx = base + 2 * kWts + 2 * kZero;
    unsigned char* oky = okx + kOk;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // every table entry a call reads is written by that call first, so no
    // part of the shared array needs clearing between calls
    const double* wantx = d_xwant;
    const double* wanty = d_ywant;
    const double* fdata = d_fdata;
    if (flct::launch_kernel(flct::k_interp_axis, dim3((nxi + 127) / 128), dim3(128), 0, st, false, nxi, nx, 0, 1,
                            wantx, zx, wx, okx) != cudaSuccess ||
        flct::launch_kernel(flct::k_interp_axis, dim3((nyi + 127) / 128), dim3(128), 0, st, false, nyi, ny, 0, 1,
                            wanty, zy, wy, oky) != cudaSuccess)
        return own_error(FLCT_ERR_CUDA);
    const long n = (long)nxi * nyi;
    long blocks = (n + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    const int* czx = zx;
    const int* czy = zy;
    const double* cwx = wx;
    const double* cwy = wy;
    const unsigned char* cokx = okx;
    const unsigned char* coky = oky;
    if (flct::launch_kernel(flct::k_interp_general, dim3((unsigned)blocks), dim3(256), 0, st, false, fdata, nx, ny,
                            xmiss, czx, cwx, cokx, nxi, czy, cwy, coky, nyi, d_out) != cudaSuccess)
        return own_error(FLCT_ERR_CUDA);
    return FLCT_OK;
}
