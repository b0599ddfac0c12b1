// k-space RPY influence (restates old-version/spme_kernel.c:73-228 with the
// table of old-version/spme.c:129-150): on the half spectrum,
//   g(k) <- S(|k|) |b_x b_y b_z|^2 (I - k k^T / |k|^2) g(k),   g(0) = 0,
// the same real 3x3 matrix applied to re and im, one fused streaming pass
// over all 3R components.  The reference's 1/K^3 backward scale and its
// alpha*K^3/L^3 factor (old-version/spme.c:408-409,699) fold into the table
// as 1/V.
//
// Wavenumbers follow the reference's map (old-version/spme.c:96-107):
// index m <= K/2 maps to +2 pi m / L, so for even K the Nyquist index K/2 is
// +pi K / L on every axis.  On the x = 0 and (even K) x = K/2 planes that
// convention makes the result non-Hermitian; the reference's complex-to-real
// transform then keeps the real part of the inverse transform along y and z.
// This kernel produces the Hermitian part directly (pairing (y,z) with
// (-y,-z)), which gives any C2R implementation the same result.
//
// Layout: component-major half spectrum G[c][(z*K + y)*Kh + kx], c = 3r + d,
// the contiguous batched layout of the cuFFT R2C/C2R plans.
#include "kernels.h"

namespace spme {

namespace {

__device__ __forceinline__ double wavenumber(int m, int K, double twopi_L) {
    return (double)(m <= K / 2 ? m : m - K) * twopi_L;
}

// old-version/spme.c:43-60 with aa = ab = a.
__device__ __forceinline__ double scalar_recip(double k, double xi, double a) {
    double kx = k / xi, kx2 = kx * kx, k2 = k * k;
    return 6.0 * M_PI * exp(-kx2 / 4.0) * (1.0 - k2 * (2.0 * a * a) / 6.0) / k2 *
           (1.0 + kx2 * (1.0 / 4.0 + kx2 / 8.0));
}

template <typename T>
__global__ void k_table(T *__restrict__ tab2, const double *__restrict__ bmod2, int K, double L,
                        double xi, double a) {
    const int Kh = K / 2 + 1;
    const size_t Kc = (size_t)K * K * Kh;
    const double twopi_L = 2.0 * M_PI / L, invV = 1.0 / (L * L * L);
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < Kc;
         t += (size_t)gridDim.x * blockDim.x) {
        int x = (int)(t % Kh);
        size_t r = t / Kh;
        int y = (int)(r % K), z = (int)(r / K);
        double kx = wavenumber(x, K, twopi_L), ky = wavenumber(y, K, twopi_L),
               kz = wavenumber(z, K, twopi_L);
        double k2 = kx * kx + ky * ky + kz * kz;
        double m2 = 0.0, c = 0.0;
        if (k2 > 0.0) {
            m2 = scalar_recip(sqrt(k2), xi, a) * bmod2[x] * bmod2[y] * bmod2[z] * invV;
            c = m2 / k2;
        }
        tab2[2 * t] = (T)m2;
        tab2[2 * t + 1] = (T)c;
    }
}

template <typename T>
struct Cx {
    T re, im;
};

// out = B(k) g for the three Cartesian components of one right-hand side.
template <typename T>
__device__ __forceinline__ void apply_B(T m2, T c, T kx, T ky, T kz, const Cx<T> (&g)[3],
                                        Cx<T> (&o)[3]) {
    const T b0 = m2 - c * kx * kx, b1 = -c * kx * ky, b2 = -c * kx * kz;
    const T b3 = m2 - c * ky * ky, b4 = -c * ky * kz, b5 = m2 - c * kz * kz;
    o[0].re = b0 * g[0].re + b1 * g[1].re + b2 * g[2].re;
    o[0].im = b0 * g[0].im + b1 * g[1].im + b2 * g[2].im;
    o[1].re = b1 * g[0].re + b3 * g[1].re + b4 * g[2].re;
    o[1].im = b1 * g[0].im + b3 * g[1].im + b4 * g[2].im;
    o[2].re = b2 * g[0].re + b4 * g[1].re + b5 * g[2].re;
    o[2].im = b2 * g[0].im + b4 * g[1].im + b5 * g[2].im;
}

// All planes x in [1, K/2) (even K) or [1, K/2] (odd K): independent points.
// Component-major half spectrum G[c][kidx], c = 3r + d; one thread per k-point
// reads its table entry once and streams all R right-hand sides.
template <typename T>
__global__ void __launch_bounds__(256)
k_influence(Cx<T> *__restrict__ G, const T *__restrict__ tab2, int K, T twopi_L, int R) {
    using V2 = typename Vec2<T>::type;
    const int Kh = K / 2 + 1;
    const size_t Kc = (size_t)K * K * Kh;
    for (size_t kidx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; kidx < Kc;
         kidx += (size_t)gridDim.x * blockDim.x) {
        const int x = (int)(kidx % Kh);
        if (x == 0 || (!(K & 1) && x == K / 2)) continue;
        const size_t rest = kidx / Kh;
        const int y = (int)(rest % K), z = (int)(rest / K);
        const V2 mc = reinterpret_cast<const V2 *>(tab2)[kidx];
        const T kx = (T)(x <= K / 2 ? x : x - K) * twopi_L;
        const T ky = (T)(y <= K / 2 ? y : y - K) * twopi_L;
        const T kz = (T)(z <= K / 2 ? z : z - K) * twopi_L;
        const T m2 = mc.x, c = mc.y;
        const T b0 = m2 - c * kx * kx, b1 = -c * kx * ky, b2 = -c * kx * kz;
        const T b3 = m2 - c * ky * ky, b4 = -c * ky * kz, b5 = m2 - c * kz * kz;
        Cx<T> *p = G + kidx;
#pragma unroll 4
        for (int r = 0; r < R; r++) {
            Cx<T> *q = p + (size_t)(3 * r) * Kc;
            const Cx<T> g0 = q[0], g1 = q[Kc], g2 = q[2 * Kc];
            Cx<T> o;
            o.re = b0 * g0.re + b1 * g1.re + b2 * g2.re;
            o.im = b0 * g0.im + b1 * g1.im + b2 * g2.im;
            q[0] = o;
            o.re = b1 * g0.re + b3 * g1.re + b4 * g2.re;
            o.im = b1 * g0.im + b3 * g1.im + b4 * g2.im;
            q[Kc] = o;
            o.re = b2 * g0.re + b4 * g1.re + b5 * g2.re;
            o.im = b2 * g0.im + b4 * g1.im + b5 * g2.im;
            q[2 * Kc] = o;
        }
    }
}

// Planes x = 0 and (even K) x = K/2: process (y,z) with its partner
// (-y,-z) together and write the Hermitian part of B g.
template <typename T>
__global__ void __launch_bounds__(256)
k_influence_planes(Cx<T> *__restrict__ G, const T *__restrict__ tab2, int K, T twopi_L, int R) {
    using V2 = typename Vec2<T>::type;
    const int Kh = K / 2 + 1;
    const size_t Kc = (size_t)K * K * Kh;
    const int nplanes = (K & 1) ? 1 : 2;
    const size_t total = (size_t)nplanes * K * K;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (size_t)gridDim.x * blockDim.x) {
        const size_t q = t % ((size_t)K * K);
        const int pl = (int)(t / ((size_t)K * K));
        const int x = pl == 0 ? 0 : K / 2;
        const int y = (int)(q % K), z = (int)(q / K);
        const int y2 = (K - y) % K, z2 = (K - z) % K;
        const size_t q2 = (size_t)z2 * K + y2;
        if (q > q2) continue;
        const T kx = (T)(x <= K / 2 ? x : x - K) * twopi_L;
        const size_t k1 = q * Kh + x, k2 = q2 * Kh + x;
        const V2 mc1 = reinterpret_cast<const V2 *>(tab2)[k1];
        const V2 mc2 = reinterpret_cast<const V2 *>(tab2)[k2];
        const T ky1 = (T)(y <= K / 2 ? y : y - K) * twopi_L, kz1 = (T)(z <= K / 2 ? z : z - K) * twopi_L;
        const T ky2 = (T)(y2 <= K / 2 ? y2 : y2 - K) * twopi_L, kz2 = (T)(z2 <= K / 2 ? z2 : z2 - K) * twopi_L;
        for (int r = 0; r < R; r++) {
            Cx<T> *p1 = G + (size_t)(3 * r) * Kc + k1;
            Cx<T> *p2 = G + (size_t)(3 * r) * Kc + k2;
            Cx<T> g1[3] = {p1[0], p1[Kc], p1[2 * Kc]}, o1[3];
            apply_B<T>(mc1.x, mc1.y, kx, ky1, kz1, g1, o1);
            if (q == q2) {
#pragma unroll
                for (int d = 0; d < 3; d++) {
                    o1[d].im = T(0);
                    p1[d * Kc] = o1[d];
                }
                continue;
            }
            Cx<T> g2[3] = {p2[0], p2[Kc], p2[2 * Kc]}, o2[3];
            apply_B<T>(mc2.x, mc2.y, kx, ky2, kz2, g2, o2);
#pragma unroll
            for (int d = 0; d < 3; d++) {
                Cx<T> h;
                h.re = T(0.5) * (o1[d].re + o2[d].re);
                h.im = T(0.5) * (o1[d].im - o2[d].im);
                p1[d * Kc] = h;
                h.im = -h.im;
                p2[d * Kc] = h;
            }
        }
    }
}

int grid_for(size_t work, int threads) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    size_t need = (work + threads - 1) / threads;
    size_t cap = (size_t)sms * 16;
    return (int)(need < cap ? (need > 0 ? need : 1) : cap);
}

}  // namespace

template <typename T>
void launch_influence_table(T *tab2, const double *bmod2, int K, double L, double xi, double a,
                            cudaStream_t s) {
    size_t Kc = (size_t)K * K * (K / 2 + 1);
    k_table<T><<<grid_for(Kc, 256), 256, 0, s>>>(tab2, bmod2, K, L, xi, a);
}

template <typename T>
void launch_influence(T *G, const T *tab2, int K, double L, int R, cudaStream_t s) {
    const T twopi_L = (T)(2.0 * M_PI / L);
    const size_t Kh = K / 2 + 1;
    Cx<T> *g = reinterpret_cast<Cx<T> *>(G);
    k_influence<T><<<grid_for((size_t)K * K * Kh, 256), 256, 0, s>>>(g, tab2, K, twopi_L, R);
    const int nplanes = (K & 1) ? 1 : 2;
    k_influence_planes<T><<<grid_for((size_t)nplanes * K * K, 256), 256, 0, s>>>(
        g, tab2, K, twopi_L, R);
}

template void launch_influence_table<float>(float *, const double *, int, double, double, double,
                                            cudaStream_t);
template void launch_influence_table<double>(double *, const double *, int, double, double,
                                             double, cudaStream_t);
template void launch_influence<float>(float *, const float *, int, double, int, cudaStream_t);
template void launch_influence<double>(double *, const double *, int, double, int, cudaStream_t);

}  // namespace spme
