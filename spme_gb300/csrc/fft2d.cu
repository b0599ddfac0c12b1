// One-pass 2D (y, x) real transforms of the mesh's z-planes (FP32).
//
// The 3D transforms of the mesh are split into 2D (y, x) transforms of every
// z-plane and the z transform (fused with the influence, zfft.cu).  Batched 2D
// R2C/C2R transforms of 256 x 256 planes take two HBM passes (one per axis);
// these kernels take one: a plane is cut into CS row blocks of H = K/CS rows,
// one block per CTA of a CS-CTA cluster, and the y transform's first radix-CS
// stage is done across the cluster through distributed shared memory.
//
// Forward (R2C), CTA r of the cluster holding rows y = r H + m, m < H:
//   x transform: each real row is read as M = K/2 complex values
//     z[n] = x[2n] + i x[2n+1], transformed in place (M-point DIF, digit-reversed
//     out) and split into the half spectrum X[kx], kx = 0..M:
//       E = (Z[k] + conj Z[M-k]) / 2,  O = -i (Z[k] - conj Z[M-k]) / 2,
//       X[k] = E + W_K^k O,  X[M-k] = conj(E - W_K^k O)
//     (column M, the Nyquist column, lives in the row's padding);
//   y transform, cross stage: t[m] = W_K^{m r} sum_q X_q[m] W_CS^{q r}, X_q being
//     the rows held by CTA q (radix-CS decimation in frequency: CTA r keeps the
//     output residue ky = r mod CS);
//   y transform, local: H-point DIF over m; position p holds ky = r + CS perm_H[p],
//     written straight to the half spectrum G[plane][ky][kx] (K/2+1 columns).
// Inverse (C2R): the same steps reversed: H-point DIT over the rows ky = r + CS k2
//   (read in digit-reversed order straight from G), cross stage
//   x[r H + m] = sum_q W_CS^{-r q} W_K^{-q m} t_q[m], the packing
//   Z'[k] = (X[k] + conj X[M-k]) + i W_K^{-k} (X[k] - conj X[M-k]) into
//   digit-reversed positions, and an M-point DIT whose outputs are the real row
//   (z[n] = x[2n] + i x[2n+1]) written straight to the mesh.
//
// Neither direction scales (like cuFFT).  The layouts are cuFFT's defaults:
// real plane [y][x] (K floats per row), half spectrum [ky][K/2+1], planes
// consecutive.  Pass structure per transform length N (M or H): a radix-16
// pass with span 1 and a radix-N/16 pass with span 16 (N = 64, 80, 128).
#include <cooperative_groups.h>

#include <cmath>
#include <vector>

#include "fft_small.cuh"
#include "kernels.h"

namespace cg = cooperative_groups;

namespace spme {

namespace {

constexpr int kF2Threads = 256;

// Radices of the span-16 pass of an N-point transform (the span-1 pass is 4 x 4).
template <int N>
struct Span16;
template <>
struct Span16<64> {
    static constexpr int R1 = 4, R2 = 1;
};
template <>
struct Span16<80> {
    static constexpr int R1 = 5, R2 = 1;
};
template <>
struct Span16<128> {
    static constexpr int R1 = 4, R2 = 2;
};

// Per-(K, CS) constants and the shared-memory layout: S[H][RS] complex rows
// (RS = M + 2: column M holds the Nyquist value, rows stay 16-byte aligned and
// RS = 2 mod 4 keeps 16-byte row-strided accesses conflict-free), the K-point
// twiddle table, the M-point inverse digit reversal and the H-point digit
// reversal.
template <int K, int CS>
struct F2 {
    static constexpr int M = K / 2, H = K / CS, RS = M + 2, CW = M + 1;
    static constexpr size_t s_bytes = (size_t)H * RS * 8;
    static constexpr size_t tw_off = s_bytes, ipm_off = tw_off + (size_t)K * 8,
                            ph_off = ipm_off + (size_t)M * 4, total = ph_off + (size_t)H * 4;
    // blocks per SM the shared memory allows (227 KB usable, 1 KB reserved per block)
    static constexpr int minb = (int)((227 * 1024) / (total + 1024)) > 4
                                    ? 4
                                    : (int)((227 * 1024) / (total + 1024));
};

using C32 = Cx<float>;

__device__ __forceinline__ C32 ld2(const float2 *p) {
    const float2 a = *p;
    return {a.x, a.y};
}
__device__ __forceinline__ void st2(float2 *p, C32 v) { *p = make_float2(v.re, v.im); }
__device__ __forceinline__ C32 conjc(C32 a) { return {a.re, -a.im}; }

// Root of unity W_CS^{e} (e taken mod CS) from the K-point table.
template <int K, int CS>
__device__ __forceinline__ C32 root_cs(const C32 *tw, int e) {
    return tw[(e % CS) * (K / CS)];
}

template <int K, int CS>
__device__ __forceinline__ void load_tables(unsigned char *smem, const float2 *twg,
                                            const int *ipmg, const int *phg) {
    using F = F2<K, CS>;
    C32 *tw = reinterpret_cast<C32 *>(smem + F::tw_off);
    int *ipm = reinterpret_cast<int *>(smem + F::ipm_off);
    int *ph = reinterpret_cast<int *>(smem + F::ph_off);
    for (int i = threadIdx.x; i < K; i += kF2Threads) tw[i] = ld2(twg + i);
    for (int i = threadIdx.x; i < F::M; i += kF2Threads) ipm[i] = ipmg[i];
    for (int i = threadIdx.x; i < F::H; i += kF2Threads) ph[i] = phg[i];
}

// Span-1 radix-16 pass over the rows of S (x direction), rows fastest across
// lanes; elements are 16 consecutive values, moved as 16-byte pairs.
template <int K, int CS, bool DIF>
__device__ __forceinline__ void xpass_span1(C32 *S, const C32 *tw) {
    using F = F2<K, CS>;
    constexpr int NB = F::M / 16, TASKS = F::H * NB;
    for (int t = threadIdx.x; t < TASKS; t += kF2Threads) {
        const int y = t % F::H, b = t / F::H;
        float4 *x4 = reinterpret_cast<float4 *>(S + y * F::RS + 16 * b);
        C32 v[4][4];
#pragma unroll
        for (int i = 0; i < 8; i++) {
            const float4 a = x4[i];
            v[(2 * i) / 4][(2 * i) % 4] = {a.x, a.y};
            v[(2 * i + 1) / 4][(2 * i + 1) % 4] = {a.z, a.w};
        }
        butterfly<float, 4, 4, DIF, 1, K>(v, 0, tw);
#pragma unroll
        for (int i = 0; i < 8; i++) {
            const C32 a = v[(2 * i) / 4][(2 * i) % 4], c = v[(2 * i + 1) / 4][(2 * i + 1) % 4];
            x4[i] = make_float4(a.re, a.im, c.re, c.im);
        }
    }
}

// Span-16 pass of the y transform over the CW columns of S (element stride RS),
// columns fastest across lanes.
template <int K, int CS, bool DIF>
__device__ __forceinline__ void ypass_span16(C32 *S, const C32 *tw) {
    using F = F2<K, CS>;
    using P = Span16<F::H>;
    constexpr int TASKS = F::CW * 16;
    for (int t = threadIdx.x; t < TASKS; t += kF2Threads) {
        const int kx = t % F::CW, j = t / F::CW;
        C32 *x = S + j * F::RS + kx;
        C32 v[P::R2][P::R1];
#pragma unroll
        for (int q2 = 0; q2 < P::R2; q2++)
#pragma unroll
            for (int q1 = 0; q1 < P::R1; q1++) v[q2][q1] = x[16 * (q1 + q2 * P::R1) * F::RS];
        butterfly<float, P::R1, P::R2, DIF, 16, K>(v, j, tw);
#pragma unroll
        for (int q2 = 0; q2 < P::R2; q2++)
#pragma unroll
            for (int q1 = 0; q1 < P::R1; q1++) x[16 * (q1 + q2 * P::R1) * F::RS] = v[q2][q1];
    }
}

// Cross-cluster radix-CS stage of the y transform over the CW columns of every
// row, in rounds of rows (results held in registers until every CTA of the
// cluster has read the round's rows, then written in place).
//   forward (INV false): CTA r: S[m] <- W_K^{m r} sum_q S_q[m] W_CS^{q r}
//   inverse (INV true):  CTA r: S[m] <- sum_q W_CS^{-r q} W_K^{-q m} S_q[m]
template <int K, int CS, bool INV>
__device__ __forceinline__ void cross_stage(C32 *S, const C32 *tw) {
    using F = F2<K, CS>;
    cg::cluster_group cl = cg::this_cluster();
    const int r = (int)cl.block_rank();
    const C32 *src[CS];
#pragma unroll
    for (int q = 0; q < CS; q++) src[q] = cl.map_shared_rank(S, q);
    constexpr int NBT = 8, RB = (NBT * kF2Threads) / F::CW < F::H ? (NBT * kF2Threads) / F::CW : F::H;
    constexpr int TASKS = RB * F::CW;
    cl.sync();  // every CTA's rows are complete
    for (int m0 = 0; m0 < F::H; m0 += RB) {
        C32 o[NBT];
        int at[NBT];
#pragma unroll
        for (int i = 0; i < NBT; i++) {
            const int t = threadIdx.x + i * kF2Threads;
            const int m = m0 + t / F::CW, kx = t % F::CW;
            at[i] = -1;
            if (t < TASKS && m < F::H) {
                at[i] = m * F::RS + kx;
                C32 s = {0.f, 0.f};
#pragma unroll
                for (int q = 0; q < CS; q++) {
                    C32 x = src[q][at[i]];
                    if constexpr (INV) {
                        if (q > 0) x = cmul(x, conjc(tw[q * m]));
                        if (q * r % CS) x = cmul(x, conjc(root_cs<K, CS>(tw, q * r)));
                    } else {
                        if (q * r % CS) x = cmul(x, root_cs<K, CS>(tw, q * r));
                    }
                    s = cadd(s, x);
                }
                if constexpr (!INV)
                    if (r > 0) s = cmul(s, tw[m * r]);
                o[i] = s;
            }
        }
        cl.sync();  // every CTA has read this round's rows
#pragma unroll
        for (int i = 0; i < NBT; i++)
            if (at[i] >= 0) S[at[i]] = o[i];
    }
    __syncthreads();
}

// Forward: real planes mesh[plane][K][K] -> half spectra G[plane][K][K/2+1].
template <int K, int CS>
__global__ void __cluster_dims__(CS, 1, 1) __launch_bounds__(kF2Threads, F2<K, CS>::minb)
    k_fft2d_r2c(const float *__restrict__ mesh, float2 *__restrict__ G,
                const float2 *__restrict__ twg, const int *__restrict__ ipmg,
                const int *__restrict__ phg) {
    using F = F2<K, CS>;
    constexpr int M = F::M, H = F::H, RS = F::RS, CW = F::CW;
    extern __shared__ __align__(16) unsigned char smem[];
    C32 *S = reinterpret_cast<C32 *>(smem);
    const C32 *tw = reinterpret_cast<const C32 *>(smem + F::tw_off);
    const int *ipm = reinterpret_cast<const int *>(smem + F::ipm_off);
    const int *ph = reinterpret_cast<const int *>(smem + F::ph_off);
    const int r = (int)(blockIdx.x % CS);
    const size_t plane = blockIdx.x / CS;
    load_tables<K, CS>(smem, twg, ipmg, phg);
    __syncthreads();

    // x transform, span-16 pass (DIF), straight from the real rows: element e of
    // row y is the float pair (x[2e], x[2e+1])
    {
        using P = Span16<M>;
        const float2 *src = reinterpret_cast<const float2 *>(mesh) + (plane * K + (size_t)r * H) * M;
        constexpr int TASKS = H * 16;
        static_assert(TASKS % kF2Threads == 0, "row tasks");
#pragma unroll 2
        for (int i = 0; i < TASKS / kF2Threads; i++) {
            const int t = threadIdx.x + i * kF2Threads, y = t >> 4, j = t & 15;
            const float2 *x = src + (size_t)y * M + j;
            C32 v[P::R2][P::R1];
#pragma unroll
            for (int q2 = 0; q2 < P::R2; q2++)
#pragma unroll
                for (int q1 = 0; q1 < P::R1; q1++) v[q2][q1] = ld2(x + 16 * (q1 + q2 * P::R1));
            butterfly<float, P::R1, P::R2, true, 16, K>(v, j, tw);
            C32 *o = S + y * RS + j;
#pragma unroll
            for (int q2 = 0; q2 < P::R2; q2++)
#pragma unroll
                for (int q1 = 0; q1 < P::R1; q1++) o[16 * (q1 + q2 * P::R1)] = v[q2][q1];
        }
    }
    __syncthreads();
    xpass_span1<K, CS, true>(S, tw);
    __syncthreads();

    // real split: Z (digit-reversed) -> X[0..M] (natural), in rounds of rows
    {
        constexpr int PK = M / 2 + 1, NBT = 8;
        constexpr int RB = (NBT * kF2Threads) / PK < H ? (NBT * kF2Threads) / PK : H;
        for (int y0 = 0; y0 < H; y0 += RB) {
            C32 a[NBT], c[NBT];
            int at[NBT], kk[NBT];
#pragma unroll
            for (int i = 0; i < NBT; i++) {
                const int t = threadIdx.x + i * kF2Threads, y = y0 + t / PK, k = t % PK;
                at[i] = -1;
                if (t < RB * PK && y < H) {
                    const C32 *row = S + y * RS;
                    at[i] = y * RS;
                    kk[i] = k;
                    const C32 zk = row[ipm[k]];
                    if (k == 0) {
                        a[i] = {zk.re + zk.im, 0.f};
                        c[i] = {zk.re - zk.im, 0.f};
                    } else {
                        const C32 zm = conjc(row[ipm[M - k]]);
                        const C32 e = {0.5f * (zk.re + zm.re), 0.5f * (zk.im + zm.im)};
                        // O = -i (zk - zm) / 2
                        const C32 od = {0.5f * (zk.im - zm.im), -0.5f * (zk.re - zm.re)};
                        const C32 tt = cmul(od, tw[k]);
                        a[i] = cadd(e, tt);
                        c[i] = conjc(csub(e, tt));
                    }
                }
            }
            __syncthreads();
#pragma unroll
            for (int i = 0; i < NBT; i++)
                if (at[i] >= 0) {
                    S[at[i] + kk[i]] = a[i];
                    S[at[i] + M - kk[i]] = c[i];
                }
            __syncthreads();
        }
    }

    if constexpr (CS > 1) cross_stage<K, CS, false>(S, tw);

    ypass_span16<K, CS, true>(S, tw);
    __syncthreads();

    // y transform, span-1 radix-16 pass (DIF), written to the half spectrum:
    // position p holds ky = r + CS perm_H[p]
    {
        float2 *dst = G + plane * K * CW;
        constexpr int TASKS = CW * (H / 16);
        for (int t = threadIdx.x; t < TASKS; t += kF2Threads) {
            const int kx = t % CW, b = t / CW;
            const C32 *x = S + 16 * b * RS + kx;
            C32 v[4][4];
#pragma unroll
            for (int q2 = 0; q2 < 4; q2++)
#pragma unroll
                for (int q1 = 0; q1 < 4; q1++) v[q2][q1] = x[(q1 + 4 * q2) * RS];
            butterfly<float, 4, 4, true, 1, K>(v, 0, tw);
#pragma unroll
            for (int q2 = 0; q2 < 4; q2++)
#pragma unroll
                for (int q1 = 0; q1 < 4; q1++) {
                    const int ky = r + CS * ph[16 * b + q1 + 4 * q2];
                    st2(dst + (size_t)ky * CW + kx, v[q2][q1]);
                }
        }
    }
}

// Inverse: half spectra G[plane][K][K/2+1] -> real planes mesh[plane][K][K].
// The kx = 0 and K/2 columns are taken as Hermitian in ky (their imaginary
// parts after the y transform are dropped, as a C2R transform does).
template <int K, int CS>
__global__ void __cluster_dims__(CS, 1, 1) __launch_bounds__(kF2Threads, F2<K, CS>::minb)
    k_fft2d_c2r(const float2 *__restrict__ G, float *__restrict__ mesh,
                const float2 *__restrict__ twg, const int *__restrict__ ipmg,
                const int *__restrict__ phg) {
    using F = F2<K, CS>;
    constexpr int M = F::M, H = F::H, RS = F::RS, CW = F::CW;
    extern __shared__ __align__(16) unsigned char smem[];
    C32 *S = reinterpret_cast<C32 *>(smem);
    const C32 *tw = reinterpret_cast<const C32 *>(smem + F::tw_off);
    const int *ipm = reinterpret_cast<const int *>(smem + F::ipm_off);
    const int *ph = reinterpret_cast<const int *>(smem + F::ph_off);
    const int r = (int)(blockIdx.x % CS);
    const size_t plane = blockIdx.x / CS;
    load_tables<K, CS>(smem, twg, ipmg, phg);
    __syncthreads();

    // y transform, span-1 radix-16 pass (DIT) straight from the half spectrum:
    // position p takes ky = r + CS perm_H[p]
    {
        const float2 *src = G + plane * K * CW;
        constexpr int TASKS = CW * (H / 16);
        for (int t = threadIdx.x; t < TASKS; t += kF2Threads) {
            const int kx = t % CW, b = t / CW;
            C32 v[4][4];
#pragma unroll
            for (int q2 = 0; q2 < 4; q2++)
#pragma unroll
                for (int q1 = 0; q1 < 4; q1++) {
                    const int ky = r + CS * ph[16 * b + q1 + 4 * q2];
                    v[q2][q1] = ld2(src + (size_t)ky * CW + kx);
                }
            butterfly<float, 4, 4, false, 1, K>(v, 0, tw);
            C32 *x = S + 16 * b * RS + kx;
#pragma unroll
            for (int q2 = 0; q2 < 4; q2++)
#pragma unroll
                for (int q1 = 0; q1 < 4; q1++) x[(q1 + 4 * q2) * RS] = v[q2][q1];
        }
    }
    __syncthreads();
    ypass_span16<K, CS, false>(S, tw);
    __syncthreads();

    if constexpr (CS > 1) cross_stage<K, CS, true>(S, tw);

    // packing: X[0..M] (natural) -> Z' (digit-reversed), in rounds of rows
    {
        constexpr int PK = M / 2 + 1, NBT = 8;
        constexpr int RB = (NBT * kF2Threads) / PK < H ? (NBT * kF2Threads) / PK : H;
        for (int y0 = 0; y0 < H; y0 += RB) {
            C32 a[NBT], c[NBT];
            int at[NBT], kk[NBT];
#pragma unroll
            for (int i = 0; i < NBT; i++) {
                const int t = threadIdx.x + i * kF2Threads, y = y0 + t / PK, k = t % PK;
                at[i] = -1;
                if (t < RB * PK && y < H) {
                    const C32 *row = S + y * RS;
                    at[i] = y * RS;
                    kk[i] = k;
                    C32 xk = row[k], xm = conjc(row[M - k]);  // k = 0: X[M] from column M
                    if (k == 0) {
                        xk.im = 0.f;  // X[0], X[M] are real for a Hermitian column
                        xm.im = 0.f;
                    }
                    const C32 A = cadd(xk, xm), B = csub(xk, xm);
                    const C32 u = cmul(B, conjc(tw[k]));
                    const C32 iu = {-u.im, u.re};
                    a[i] = cadd(A, iu);
                    c[i] = conjc(csub(A, iu));
                }
            }
            __syncthreads();
#pragma unroll
            for (int i = 0; i < NBT; i++)
                if (at[i] >= 0) {
                    S[at[i] + ipm[kk[i]]] = a[i];
                    if (kk[i] > 0) S[at[i] + ipm[M - kk[i]]] = c[i];
                }
            __syncthreads();
        }
    }

    xpass_span1<K, CS, false>(S, tw);
    __syncthreads();

    // x transform, span-16 pass (DIT), written as the real rows: element e of
    // row y is the float pair (x[2e], x[2e+1])
    {
        using P = Span16<M>;
        float2 *dst = reinterpret_cast<float2 *>(mesh) + (plane * K + (size_t)r * H) * M;
        constexpr int TASKS = H * 16;
#pragma unroll 2
        for (int i = 0; i < TASKS / kF2Threads; i++) {
            const int t = threadIdx.x + i * kF2Threads, y = t >> 4, j = t & 15;
            const C32 *x = S + y * RS + j;
            C32 v[P::R2][P::R1];
#pragma unroll
            for (int q2 = 0; q2 < P::R2; q2++)
#pragma unroll
                for (int q1 = 0; q1 < P::R1; q1++) v[q2][q1] = x[16 * (q1 + q2 * P::R1)];
            butterfly<float, P::R1, P::R2, false, 16, K>(v, j, tw);
            float2 *o = dst + (size_t)y * M + j;
#pragma unroll
            for (int q2 = 0; q2 < P::R2; q2++)
#pragma unroll
                for (int q1 = 0; q1 < P::R1; q1++) st2(o + 16 * (q1 + q2 * P::R1), v[q2][q1]);
        }
    }
}

constexpr int fft2d_cs(int K) { return K == 256 ? 4 : (K == 160 ? 2 : 1); }

template <int K>
cudaError_t launch_k(bool inverse, const void *in, void *out, long planes, const void *tables,
                     cudaStream_t s) {
    constexpr int CS = fft2d_cs(K);
    using F = F2<K, CS>;
    const float2 *tw = static_cast<const float2 *>(tables);
    const int *ipm = reinterpret_cast<const int *>(tw + K);
    const int *ph = ipm + F::M;
    const long blocks = planes * CS;
    if (blocks <= 0 || blocks > 0x7fffffffL) return cudaErrorInvalidValue;
    if (inverse) {
        auto kern = k_fft2d_c2r<K, CS>;
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)F::total);
        if (e != cudaSuccess) return e;
        kern<<<(unsigned)blocks, kF2Threads, F::total, s>>>(static_cast<const float2 *>(in),
                                                            static_cast<float *>(out), tw, ipm, ph);
    } else {
        auto kern = k_fft2d_r2c<K, CS>;
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)F::total);
        if (e != cudaSuccess) return e;
        kern<<<(unsigned)blocks, kF2Threads, F::total, s>>>(static_cast<const float *>(in),
                                                            static_cast<float2 *>(out), tw, ipm, ph);
    }
    return cudaGetLastError();
}

cudaError_t launch_any(int K, bool inverse, const void *in, void *out, long planes,
                       const void *tables, cudaStream_t s) {
    switch (K) {
        case 128: return launch_k<128>(inverse, in, out, planes, tables, s);
        case 160: return launch_k<160>(inverse, in, out, planes, tables, s);
        case 256: return launch_k<256>(inverse, in, out, planes, tables, s);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace

bool fft2d_ok(int K, size_t elem) { return elem == 4 && (K == 128 || K == 160 || K == 256); }

size_t fft2d_table_bytes(int K) {
    return (size_t)K * 8 + (size_t)(K / 2) * 4 + (size_t)(K / fft2d_cs(K)) * 4;
}

// Twiddles e^{-2 pi i e/K} (FP64, rounded), the inverse digit reversal of the
// K/2-point x transform and the digit reversal of the K/CS-point local y
// transform, both from the z-transform planner (whose pass sequence for these
// lengths, radix 16 with span 1 then radix N/16 with span 16, the kernels
// hard-code: checked here).
bool make_fft2d_tables(int K, std::vector<unsigned char> *out) {
    if (!fft2d_ok(K, 4)) return false;
    const int M = K / 2, H = K / fft2d_cs(K);
    ZPlan zm, zh;
    std::vector<double> twd;
    std::vector<int> pm, phv;
    if (!make_zplan(M, 4, &zm, &twd, &pm) || !make_zplan(H, 4, &zh, &twd, &phv)) return false;
    for (const ZPlan *z : {&zm, &zh}) {
        const int n16 = z->K / 16;
        const int code = n16 == 8 ? 42 : 10 * n16 + 1;
        if (z->npass != 2 || z->pcode[0] != 44 || z->pspan[0] != 1 || z->pcode[1] != code ||
            z->pspan[1] != 16)
            return false;
    }
    out->assign(fft2d_table_bytes(K), 0);
    float *tw = reinterpret_cast<float *>(out->data());
    for (int e = 0; e < K; e++) {
        const double a = -2.0 * M_PI * (double)e / (double)K;
        tw[2 * e] = (float)std::cos(a);
        tw[2 * e + 1] = (float)std::sin(a);
    }
    int *ipm = reinterpret_cast<int *>(tw + 2 * K);
    for (int p = 0; p < M; p++) ipm[pm[p]] = p;
    int *ph = ipm + M;
    for (int p = 0; p < H; p++) ph[p] = phv[p];
    return true;
}

cudaError_t launch_fft2d_r2c(int K, const float *mesh, float *G, long planes, const void *tables,
                             cudaStream_t s) {
    return launch_any(K, false, mesh, G, planes, tables, s);
}

cudaError_t launch_fft2d_c2r(int K, const float *G, float *mesh, long planes, const void *tables,
                             cudaStream_t s) {
    return launch_any(K, true, G, mesh, planes, tables, s);
}

}  // namespace spme
