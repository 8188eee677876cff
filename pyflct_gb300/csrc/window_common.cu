// window_common.cu -- k_means and k_fit (see window_common.cuh).
#include "window_common.cuh"

namespace flct {

__device__ __forceinline__ double dm(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double da(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double ds(double a, double b) { return __dsub_rn(a, b); }

__global__ void k_means(MeansArgs a) {
    const int nw = *a.nwork;
    for (int w = blockIdx.x * blockDim.x + threadIdx.x; w < nw; w += gridDim.x * blockDim.x) {
        const int pix = a.work[w];
        const int i = pix / a.ny, j = pix - (pix / a.ny) * a.ny;
        const size_t b = (size_t)((i - a.xo) / a.gs) * a.gj + (j - a.yo) / a.gs;
        const float2 m1 = split_double_fast(dm(a.bs1[b], a.inv_n2));
        const float2 m2 = split_double_fast(dm(a.bs2[b], a.inv_n2));
        a.means[w] = make_float4(m1.x, m1.y, m2.x, m2.y);
    }
}

// In the reference's operation order, without FMA contraction, so that the
// fit of identical |c| values rounds exactly like the reference's.
__global__ void k_fit(FitArgs a) {
    const int nw = *a.nwork;
    const int half = a.n / 2;
    for (int w = blockIdx.x * blockDim.x + threadIdx.x; w < nw; w += gridDim.x * blockDim.x) {
        const PeakRec r = a.peaks[w];
        const int I = (int)(r.meta & 0xffu), J = (int)((r.meta >> 8) & 0xffu);
        double sx = 0., sy = 0.;
        if (r.meta >> 16) {
            double v[9];
#pragma unroll
            for (int k = 0; k < 9; ++k) v[k] = f2d(r.v[k]);
            // v[3p+q] = |c| at (I-1+p, J-1+q)
            const double fx = dm(0.5, ds(v[7], v[1]));
            const double fy = dm(0.5, ds(v[5], v[3]));
            const double fxx = ds(da(v[7], v[1]), dm(2., v[4]));
            const double fyy = ds(da(v[5], v[3]), dm(2., v[4]));
            const double fxy = dm(0.25, ds(ds(da(v[8], v[0]), v[6]), v[2]));
            const double den = ds(dm(fxy, fxy), dm(fxx, fyy));
            sx = ds(dm(fyy, fx), dm(fy, fxy)) / den;
            sy = ds(dm(fxx, fy), dm(fx, fxy)) / den;
        }
        const double shx = ds(da((double)I, sx), (double)half);
        const double shy = ds(da((double)J, sy), (double)half);
        if (a.shx) {
            a.shx[w] = shx;
            a.shy[w] = shy;
        }
        if (a.vx) {
            const int pix = a.work[w];
            const int i = pix / a.ny, j = pix - (pix / a.ny) * a.ny;
            // transposed storage: vx from the fast-axis shift (flct.c:901-905)
            double vxx = dm(dm(shy, a.deltinv), a.deltas);
            double vyy = dm(dm(shx, a.deltinv), a.deltas);
            double vmm = 1.;
            if (a.grid) {
                const int ic = (i - a.xoff) / a.skip, jc = (j - a.yoff) / a.skip;
                a.grid[(size_t)ic * a.jcnt + jc] = make_float2((float)vxx, (float)vyy);
            }
            if (vxx == kXmiss) {
                vmm = 0.;
                vxx = 0.;
            }
            if (vyy == kXmiss) vyy = 0.;
            a.vx[pix] = vxx;
            a.vy[pix] = vyy;
            a.vm[pix] = vmm;
        }
    }
}

__global__ void k_batch_starts(const unsigned char* ctr, const int* seg_pair, const int* first, int ngroups,
                               int* start) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= ngroups) return;
    int* st = start + first[g] + g;
    int acc = 0;
    st[0] = 0;
    for (int k = first[g]; k < first[g + 1]; ++k) {
        acc += *reinterpret_cast<const int*>(ctr + 64 * (size_t)seg_pair[k]);
        st[k - first[g] + 1] = acc;
    }
}

}  // namespace flct
