// prepass.cuh -- argument structs and launch helpers for prepass.cu.
#pragma once
#include "common.cuh"

namespace flct {

constexpr int kSeg = 32;  // outputs per thread in the sliding box sums

struct ClassifyArgs {
    const double* f1;
    const double* f2;
    int nx, ny;
    double thr_val;           // absolute threshold, used when thr_ptr is null
    const double* thr_ptr;    // device threshold from k_thresh_final
    int skip, xoff, yoff, interpolate, jcnt;
    float2* s1;
    float2* s2;
    int* work;
    int* nwork;
    double *vx, *vy, *vm;
    double *gvx, *gvy;
    unsigned* status;
};

struct InterpArgs {
    int nx, ny, skip, xoff, yoff;
    int gx, gy;               // grid counts along the slow / fast axis
    const double* gvx;
    const double* gvy;
    const int* zx;
    const double* wx;
    const unsigned char* okx;
    const int* zy;
    const double* wy;
    const unsigned char* oky;
    double *hx, *hy;          // row contractions [(gx+2) x ny]
    unsigned char* hbad;      // xmiss flags of those rows (bit 0: vx, bit 1: vy)
    double *vx, *vy, *vm;
};

__global__ void k_absmax(const double* f1, const double* f2, long n, unsigned long long* out);
__global__ void k_thresh_final(const double* f1, const double* f2, const unsigned long long* mx,
                               double thresh, double* thr);
__global__ void k_classify(ClassifyArgs a);
__global__ void k_rowsum(const double* f1, const double* f2, int nx, int ny, int n, double* r1, double* r2);
__global__ void k_colsum(const double* r1, const double* r2, int nx, int W, int n, double* b1, double* b2);
__global__ void k_interp_axis(int n, int gcount, int off, int skip, const double* want, int* zero,
                              double* wts, unsigned char* ok);
__global__ void k_interp_rows(InterpArgs a);
__global__ void k_interp(InterpArgs a);
__global__ void k_interp_general(const double* f, int gx, int gy, double xmiss, const int* zx,
                                 const double* wx, const unsigned char* okx, int nxi, const int* zy,
                                 const double* wy, const unsigned char* oky, int nyi, double* out);

}  // namespace flct
