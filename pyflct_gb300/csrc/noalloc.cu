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
#include <cuda_runtime.h>

#include <mutex>

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

constexpr int kMaxDevices = 64;
std::mutex g_mu;
unsigned char* g_ptr[kMaxDevices] = {};

// Device address of the scratch array on the current device, looked up once
// per device (host code cannot use the array's name as a device pointer).
flct_status scratch_on_current_device(unsigned char** out) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return FLCT_ERR_NO_DEVICE;
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_ptr[dev]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) {
            cudaGetLastError();
            return FLCT_ERR_CUDA;
        }
        g_ptr[dev] = static_cast<unsigned char*>(p);
    }
    *out = g_ptr[dev];
    return FLCT_OK;
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
    unsigned char* base = nullptr;
    flct_status s = scratch_on_current_device(&base);
    if (s != FLCT_OK) return s;
    double* wx = reinterpret_cast<double*>(base);
    double* wy = reinterpret_cast<double*>(base + kWts);
    int* zx = reinterpret_cast<int*>(base + 2 * kWts);
    int* zy = reinterpret_cast<int*>(base + 2 * kWts + kZero);
    unsigned char* okx = base + 2 * kWts + 2 * kZero;
    unsigned char* oky = okx + kOk;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // every table entry a call reads is written by that call first, so no
    // part of the shared array needs clearing between calls
    flct::k_interp_axis<<<(nxi + 127) / 128, 128, 0, st>>>(nxi, nx, 0, 1, d_xwant, zx, wx, okx);
    flct::k_interp_axis<<<(nyi + 127) / 128, 128, 0, st>>>(nyi, ny, 0, 1, d_ywant, zy, wy, oky);
    const long n = (long)nxi * nyi;
    long blocks = (n + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    flct::k_interp_general<<<(int)blocks, 256, 0, st>>>(d_fdata, nx, ny, xmiss, zx, wx, okx, nxi, zy, wy, oky,
                                                         nyi, d_out);
    return cudaGetLastError() == cudaSuccess ? FLCT_OK : FLCT_ERR_CUDA;
}
