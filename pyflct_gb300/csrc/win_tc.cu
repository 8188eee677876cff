// Host side of the tensor-core window form: the split DFT matrices in their
// shared-memory layouts, and the per-size launchers (instantiated in
// win_tc_<n>.cu so the sizes compile in parallel).
#include <cmath>
#include <vector>

#include "window_tc.cuh"

namespace flct {

namespace {

struct TcGeom {
    int n, H, N8, K1, K2;
    bool pack;
};

TcGeom tc_geom(int n) {
    TcGeom g;
    g.n = n;
    g.H = n / 2;
    g.pack = (g.H % 8) == 0;
    g.N8 = tc_r8(n);
    g.K1 = tc_r16(n);
    g.K2 = 2 * g.N8;
    return g;
}

// hi = nearest 16-bit value, lo = nearest 16-bit value to the remainder
void split16(double v, int fmt, uint16_t* hi, uint16_t* lo) {
    if (fmt == 0) {
        const __half h = __double2half(v);
        const __half l = __double2half(v - (double)__half2float(h));
        *hi = __half_as_ushort(h);
        *lo = __half_as_ushort(l);
    } else {
        const __nv_bfloat16 h = __double2bfloat16(v);
        const __nv_bfloat16 l = __double2bfloat16(v - (double)__bfloat162float(h));
        *hi = __bfloat16_as_ushort(h);
        *lo = __bfloat16_as_ushort(l);
    }
}

// byte offset of element (row r, k) of a K-major operand with K columns
size_t kmajor(int r, int k, int K) { return (size_t)(r % 8) * 16 + (size_t)(r / 8) * K * 16 + (k % 8) * 2 + (k / 8) * 128; }

}  // namespace

int tc_bmat_bytes(int n) {
    const TcGeom g = tc_geom(n);
    return 2 * (g.K1 * g.K1 * 2) + 2 * (g.K2 * g.K2 * 2);
}

// B1[c][j] (K-major, c rows): c <= H cos(2 pi c j / n); H < c < n
// -sin(2 pi (c - H) j / n); zero outside n x n.  B2[n2][k2] (K-major):
// n2 = (p', q), k2 = (p, i) with blocks of n8; the complex DFT in real form,
// wavenumber of output column q in tc_kx order when packed.
void tc_build_bmat(int n, int fmt, std::vector<uint16_t>* out) {
    const TcGeom g = tc_geom(n);
    const double tw = 2.0 * 3.14159265358979323846 / n;
    const size_t b1 = (size_t)g.K1 * g.K1 * 2, b2 = (size_t)g.K2 * g.K2 * 2;
    std::vector<uint16_t> v((2 * b1 + 2 * b2) / 2, 0);
    uint16_t* B1hi = v.data();
    uint16_t* B1lo = B1hi + b1 / 2;
    uint16_t* B2hi = B1lo + b1 / 2;
    uint16_t* B2lo = B2hi + b2 / 2;
    for (int c = 0; c < n; ++c)
        for (int j = 0; j < n; ++j) {
            const double x = (c <= g.H) ? std::cos(tw * ((long)c * j % n)) : -std::sin(tw * ((long)(c - g.H) * j % n));
            const size_t o = kmajor(c, j, g.K1) / 2;
            split16(x, fmt, B1hi + o, B1lo + o);
        }
    for (int pp = 0; pp < 2; ++pp)
        for (int q = 0; q < n; ++q)
            for (int pk = 0; pk < 2; ++pk)
                for (int i = 0; i < n; ++i) {
                    const int kx = g.pack ? tc_kx(q, n) : q;
                    const double th = tw * ((long)kx * i % n);
                    double x;
                    if (pk == 0 && pp == 0) x = std::cos(th);
                    else if (pk == 1 && pp == 0) x = std::sin(th);
                    else if (pk == 0 && pp == 1) x = -std::sin(th);
                    else x = std::cos(th);
                    const size_t o = kmajor(pp * g.N8 + q, pk * g.N8 + i, g.K2) / 2;
                    split16(x, fmt, B2hi + o, B2lo + o);
                }
    out->swap(v);
}

}  // namespace flct
