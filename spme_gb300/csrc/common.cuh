// Shared device-side definitions for the GB300 SPME-RPY operator (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace spme {

constexpr int kMaxP = 8;         // largest B-spline order instantiated
constexpr int kMaxTile = 16;     // largest mesh-tile edge

// Mesh geometry shared by the P-build, spread and interpolation kernels.
struct MeshGeom {
    int K;                 // mesh points per axis
    int p;                 // B-spline order
    int tx, ty, tz;        // tile edge per axis
    int ntx, nty, ntz;     // tiles per axis (last one may be short)
    double L;              // box edge
    double invL;           // 1 / L
};

// Record width (elements of T) for p weights per axis, padded so each
// record starts on a 16-byte boundary.
template <typename T, int P>
struct RecordWidth {
    static constexpr int raw = 3 * P;
    static constexpr int per16 = 16 / (int)sizeof(T);
    static constexpr int value = (raw + per16 - 1) / per16 * per16;
};

__host__ __device__ inline int pmod(int x, int m) {
    int r = x % m;
    return r < 0 ? r + m : r;
}

// Cardinal B-spline weights of order P at fractional coordinate w in [0,1):
// out[j] = M_P(w + P - 1 - j), the weight of mesh point start + j.
// Cox-de Boor recursion M_n(x) = [x M_{n-1}(x) + (n - x) M_{n-1}(x-1)]/(n-1),
// the same polynomials the reference tabulates in monomial form
// (old-version/spme.c:25-40, evaluated at :258-279).
template <typename T, int P>
__device__ __forceinline__ void bspline_weights(T w, T (&out)[P]) {
    T a[P];
    a[0] = w;
    a[1] = T(1) - w;
#pragma unroll
    for (int n = 3; n <= P; n++) {
        const T inv = T(1) / T(n - 1);
        a[n - 1] = T(0);
#pragma unroll
        for (int k = n - 1; k >= 1; k--)
            a[k] = ((w + T(k)) * a[k] + (T(n) - w - T(k)) * a[k - 1]) * inv;
        a[0] = w * a[0] * inv;
    }
#pragma unroll
    for (int k = 0; k < P; k++) out[k] = a[P - 1 - k];
}

// Fractional mesh coordinate of position x (wrapped into [0, L)), following
// old-version/spme.c:235-256: c = x/L*K, start = floor(c) - p/2 + 1 (mod K).
// Multiplies by 1/L (FP64 division is slow); every kernel that needs a
// particle's stencil start calls this same function, so sort keys and records
// agree.
__device__ __forceinline__ double wrap_coord(double x, double L, double invL) {
    return x - L * floor(x * invL);
}
// ... of a coordinate xw already wrapped into [0, L)
__device__ __forceinline__ void mesh_coord_w(double xw, double invL, int K, int p, int &start,
                                             double &frac) {
    double c = xw * invL * (double)K;
    double fl = floor(c);
    frac = c - fl;
    int s = (int)fl - p / 2 + 1;
    start = pmod(s, K);
}
__device__ __forceinline__ void mesh_coord(double x, double L, double invL, int K, int p,
                                           int &start, double &frac) {
    mesh_coord_w(wrap_coord(x, L, invL), invL, K, p, start, frac);
}

// Real-space cell (nc cells of edge L/nc per axis) of coordinate x, and x
// wrapped into [0, L); shared by the cell keys and the cell-relative positions.
__device__ __forceinline__ int cell_coord_w(double xw, double invL, int nc) {
    const int v = (int)(xw * invL * (double)nc);
    return v >= nc ? nc - 1 : (v < 0 ? 0 : v);
}
__device__ __forceinline__ int cell_coord(double x, double L, double invL, int nc, double &xw) {
    xw = wrap_coord(x, L, invL);
    return cell_coord_w(xw, invL, nc);
}

__device__ __forceinline__ uint32_t pack_start(int sx, int sy, int sz) {
    return (uint32_t)sx | ((uint32_t)sy << 10) | ((uint32_t)sz << 20);
}
__device__ __forceinline__ void unpack_start(uint32_t v, int &sx, int &sy, int &sz) {
    sx = (int)(v & 1023u);
    sy = (int)((v >> 10) & 1023u);
    sz = (int)((v >> 20) & 1023u);
}

// q / d and q % d for 0 <= q < 2^22, 0 < d < 2^10 via a float reciprocal
// (exact after one correction step).
struct DivMod {
    int d;
    float inv;
    __device__ __forceinline__ void init(int dd) {
        d = dd;
        inv = 1.0f / (float)dd;
    }
    __device__ __forceinline__ int div(int q, int &rem) const {
        int qd = (int)((float)q * inv);
        int r = q - qd * d;
        if (r < 0) { qd--; r += d; }
        if (r >= d) { qd++; r -= d; }
        rem = r;
        return qd;
    }
};

// The system of work item w in a batched launch: prefix[k] <= w < prefix[k + 1]
// (prefix has nsys + 1 entries).
__device__ __forceinline__ int batch_find(const int *__restrict__ prefix, int nsys, int w) {
    int a = 0, b = nsys;
    while (b - a > 1) {
        const int m = (a + b) >> 1;
        if (__ldg(prefix + m) <= w) a = m; else b = m;
    }
    return a;
}

template <typename T> struct Vec2;
template <> struct Vec2<float> { using type = float2; };
template <> struct Vec2<double> { using type = double2; };

}  // namespace spme
