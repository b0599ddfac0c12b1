// One-pass 2D (y, x) real transforms of the mesh's z-planes (FP32).
//
// The 3D transforms of the mesh are split into 2D (y, x) transforms of every
// z-plane and the z transform (fused with the influence, zfft.cu).  A batched
// 2D R2C/C2R transform takes two HBM passes (one per axis); these kernels take
// one.  A plane (K x K reals, K/2+1 complex columns) does not fit one CTA's
// shared memory, so a cluster of two CTAs shares it: each holds K/2 rows for
// the x transform, then the rows are scattered through distributed shared
// memory into K/4 whole columns per CTA for the y transform.  The kx = 0 and
// kx = K/2 columns (real along y before the y transform) travel packed as one
// complex column c = X[.][0] + i X[.][K/2], so both CTAs own exactly K/4
// columns: CTA 0 kx = 0 (packed), 1 .. K/4-1, CTA 1 kx = K/4 .. K/2-1.
// Persistent clusters loop over the planes.
//
// Forward (R2C), CTA r with rows y = r K/2 + m:
//   x: each real row is read as M = K/2 complex values z[n] = x[2n] + i x[2n+1]
//      and transformed in place (M-point DIF, digit-reversed out); the split
//        E = (Z[k] + conj Z[M-k]) / 2,  O = -i (Z[k] - conj Z[M-k]) / 2,
//        X[k] = E + W_K^k O,  X[M-k] = conj(E - W_K^k O),
//        X[0] = Re Z0 + Im Z0,  X[M] = Re Z0 - Im Z0,  X[M/2] = conj Z[M/2]
//      goes to registers, then (after a cluster barrier: every CTA has read its
//      rows) to the owners' column buffers;
//   y: K-point DIF over each column; the last pass writes the half spectrum
//      G[plane][ky][kx] directly (ky = perm_K[p] at position p), except the
//      packed column, whose C[ky] is split as X0 = (C[ky] + conj C[-ky]) / 2,
//      XM = (C[ky] - conj C[-ky]) / (2i).
// Inverse (C2R): K-point DIT over the columns read from G in digit-reversed
//   order (packed column C = G[.][0] + i G[.][K/2]), the last pass kept in
//   registers and scattered to the rows' owners, then per row the packing
//   Z'[k] = (X[k] + conj X[M-k]) + i W_K^{-k} (X[k] - conj X[M-k]) into
//   digit-reversed positions and an M-point DIT whose outputs are the real row
//   (z[n] = x[2n] + i x[2n+1]), written to the mesh.
//
// Neither direction scales (like cuFFT).  Layouts are cuFFT's defaults: real
// plane [y][x] (K floats per row), half spectrum [ky][K/2+1], planes
// consecutive.  Compiled for K = 128, 160, 256.
#include <cooperative_groups.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "fft_small.cuh"
#include "kernels.h"

namespace cg = cooperative_groups;

namespace spme {

namespace {

constexpr int kF2Threads = 512;

// Pass sequences (DIT order: codes 10 R1 + R2, spans) of the transform lengths
// used: the x transforms (M = 64, 80, 128) and the y transforms (K = 128, 160,
// 256).  The planner's sequences for these lengths are checked to match.
template <int N>
struct Seq;
template <>
struct Seq<64> {
    static constexpr int n = 2, code[2] = {44, 41}, span[2] = {1, 16};
};
template <>
struct Seq<80> {
    static constexpr int n = 2, code[2] = {44, 51}, span[2] = {1, 16};
};
template <>
struct Seq<128> {
    static constexpr int n = 2, code[2] = {44, 42}, span[2] = {1, 16};
};
template <>
struct Seq<160> {
    static constexpr int n = 3, code[3] = {44, 21, 51}, span[3] = {1, 16, 32};
};
template <>
struct Seq<256> {
    static constexpr int n = 2, code[2] = {44, 44}, span[2] = {1, 16};
};

// Sizes and the shared-memory layout: the data buffer holds either K/2 rows of
// RSX = M + 2 complex values (column M is the Nyquist value; rows stay 16-byte
// aligned) or K rows of the CTA's NCY = K/4 columns; then the K-point twiddle
// table, the M-point inverse digit reversal, the K-point digit reversal and a
// K-value scratch column for the packed column's split.
template <int K>
struct F2 {
    static constexpr int M = K / 2, H = K / 2, RSX = M + 2, NCY = K / 4, CW = M + 1;
    static constexpr size_t a_bytes = (size_t)H * RSX * 8;
    static constexpr size_t tw_off = a_bytes, ipm_off = tw_off + (size_t)K * 8,
                            pk_off = ipm_off + (size_t)M * 4, sc_off = pk_off + (size_t)K * 4,
                            total = sc_off + (size_t)K * 8;
    static_assert((size_t)K * NCY <= (size_t)H * RSX, "column layout fits the row buffer");
};

using C32 = Cx<float>;

__device__ __forceinline__ C32 ld2(const float2 *p) {
    const float2 a = *p;
    return {a.x, a.y};
}
__device__ __forceinline__ void st2(float2 *p, C32 v) { *p = make_float2(v.re, v.im); }
__device__ __forceinline__ C32 conjc(C32 a) { return {a.re, -a.im}; }

template <int K>
__device__ __forceinline__ void load_tables(unsigned char *smem, const float2 *twg,
                                            const int *ipmg, const int *pkg) {
    using F = F2<K>;
    C32 *tw = reinterpret_cast<C32 *>(smem + F::tw_off);
    int *ipm = reinterpret_cast<int *>(smem + F::ipm_off);
    int *pk = reinterpret_cast<int *>(smem + F::pk_off);
    for (int i = threadIdx.x; i < K; i += kF2Threads) tw[i] = ld2(twg + i);
    for (int i = threadIdx.x; i < F::M; i += kF2Threads) ipm[i] = ipmg[i];
    for (int i = threadIdx.x; i < K; i += kF2Threads) pk[i] = pkg[i];
}

// One radix-(R1 x R2) pass with span L of N-point transforms over NS sequences
// in shared memory (element i of sequence s at A[s SS + i SE]); tasks
// (sequence, butterfly) go sequence-fastest across lanes when SEQ_FAST.  With
// unit element stride and span 1 the butterfly's elements are contiguous and
// move as 16-byte pairs.
template <int KT, int N, int CODE, int L, bool DIF, int NS, int SS, int SE, bool SEQ_FAST>
__device__ __forceinline__ void spass(C32 *A, const C32 *tw) {
    constexpr int R1 = CODE / 10, R2 = CODE % 10;
    constexpr int NB = N / (R1 * R2), TASKS = NS * NB, L3 = L * R1 * R2;
    constexpr bool VEC = SE == 1 && L == 1 && (R1 * R2) % 2 == 0 && SS % 2 == 0;
    for (int t = threadIdx.x; t < TASKS; t += kF2Threads) {
        const int s = SEQ_FAST ? t % NS : t / NB, bi = SEQ_FAST ? t / NS : t % NB;
        const int j = bi % L, b = bi / L;
        C32 *x = A + s * SS + (b * L3 + j) * SE;
        C32 v[R2][R1];
        if constexpr (VEC) {
            const float4 *x4 = reinterpret_cast<const float4 *>(x);
#pragma unroll
            for (int i = 0; i < R1 * R2 / 2; i++) {
                const float4 a = x4[i];
                v[(2 * i) / R1][(2 * i) % R1] = {a.x, a.y};
                v[(2 * i + 1) / R1][(2 * i + 1) % R1] = {a.z, a.w};
            }
        } else {
#pragma unroll
            for (int q2 = 0; q2 < R2; q2++)
#pragma unroll
                for (int q1 = 0; q1 < R1; q1++) v[q2][q1] = x[(q1 * L + q2 * L * R1) * SE];
        }
        butterfly<float, R1, R2, DIF, L, KT>(v, j, tw);
        if constexpr (VEC) {
            float4 *x4 = reinterpret_cast<float4 *>(x);
#pragma unroll
            for (int i = 0; i < R1 * R2 / 2; i++) {
                const C32 a = v[(2 * i) / R1][(2 * i) % R1], c = v[(2 * i + 1) / R1][(2 * i + 1) % R1];
                x4[i] = make_float4(a.re, a.im, c.re, c.im);
            }
        } else {
#pragma unroll
            for (int q2 = 0; q2 < R2; q2++)
#pragma unroll
                for (int q1 = 0; q1 < R1; q1++) x[(q1 * L + q2 * L * R1) * SE] = v[q2][q1];
        }
    }
}

// Passes I0 .. I1 (inclusive, DIT indices of Seq<N>) in DIF order (I1 down to
// I0) or DIT order (I0 up to I1), with a block barrier after each.
template <int KT, int N, bool DIF, int NS, int SS, int SE, bool SEQ_FAST, int I0, int I1>
__device__ __forceinline__ void spasses(C32 *A, const C32 *tw) {
    if constexpr (I0 <= I1) {
        constexpr int I = DIF ? I1 : I0;
        spass<KT, N, Seq<N>::code[I], Seq<N>::span[I], DIF, NS, SS, SE, SEQ_FAST>(A, tw);
        __syncthreads();
        if constexpr (DIF)
            spasses<KT, N, DIF, NS, SS, SE, SEQ_FAST, I0, I1 - 1>(A, tw);
        else
            spasses<KT, N, DIF, NS, SS, SE, SEQ_FAST, I0 + 1, I1>(A, tw);
    }
}

// Forward: real planes mesh[plane][K][K] -> half spectra G[plane][K][K/2+1].
template <int K>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(kF2Threads, 1)
    k_fft2d_r2c(const float *__restrict__ mesh, float2 *__restrict__ G,
                const float2 *__restrict__ twg, const int *__restrict__ ipmg,
                const int *__restrict__ pkg, int planes) {
    using F = F2<K>;
    constexpr int M = F::M, H = F::H, RSX = F::RSX, NCY = F::NCY, CW = F::CW, PT = M / 2;
    extern __shared__ __align__(16) unsigned char smem[];
    C32 *A = reinterpret_cast<C32 *>(smem);
    const C32 *tw = reinterpret_cast<const C32 *>(smem + F::tw_off);
    const int *ipm = reinterpret_cast<const int *>(smem + F::ipm_off);
    const int *pk = reinterpret_cast<const int *>(smem + F::pk_off);
    C32 *sc = reinterpret_cast<C32 *>(smem + F::sc_off);
    cg::cluster_group cl = cg::this_cluster();
    const int r = (int)cl.block_rank();
    C32 *col[2] = {cl.map_shared_rank(A, 0), cl.map_shared_rank(A, 1)};
    load_tables<K>(smem, twg, ipmg, pkg);
    __syncthreads();
    const int ncl = (int)(gridDim.x / 2);
    for (int P = (int)(blockIdx.x / 2); P < planes; P += ncl) {
        // x: the span-16 pass (first in DIF order) straight from the real rows;
        // element e of row y is the float pair (x[2e], x[2e+1])
        {
            constexpr int I = Seq<M>::n - 1, CODE = Seq<M>::code[I];
            constexpr int R1 = CODE / 10, R2 = CODE % 10;
            static_assert(Seq<M>::span[I] == 16 && 16 * R1 * R2 == M, "x pass layout");
            constexpr int TASKS = H * 16, NI = (TASKS + kF2Threads - 1) / kF2Threads;
            const float2 *src =
                reinterpret_cast<const float2 *>(mesh) + ((size_t)P * K + (size_t)r * H) * M;
            C32 v[NI][R2][R1];
#pragma unroll
            for (int i = 0; i < NI; i++) {
                const int t = threadIdx.x + i * kF2Threads;
                if (TASKS % kF2Threads == 0 || t < TASKS) {
                    const float2 *x = src + (size_t)(t >> 4) * M + (t & 15);
#pragma unroll
                    for (int q2 = 0; q2 < R2; q2++)
#pragma unroll
                        for (int q1 = 0; q1 < R1; q1++) v[i][q2][q1] = ld2(x + 16 * (q1 + q2 * R1));
                }
            }
#pragma unroll
            for (int i = 0; i < NI; i++) {
                const int t = threadIdx.x + i * kF2Threads;
                if (TASKS % kF2Threads == 0 || t < TASKS) {
                    const int j = t & 15;
                    butterfly<float, R1, R2, true, 16, K>(v[i], j, tw);
                    C32 *o = A + (t >> 4) * RSX + j;
#pragma unroll
                    for (int q2 = 0; q2 < R2; q2++)
#pragma unroll
                        for (int q1 = 0; q1 < R1; q1++) o[16 * (q1 + q2 * R1)] = v[i][q2][q1];
                }
            }
        }
        __syncthreads();
        spasses<K, M, true, H, RSX, 1, true, 0, Seq<M>::n - 2>(A, tw);

        // split into registers, then into the owners' column buffers
        {
            constexpr int TS = H * PT, NS = (TS + kF2Threads - 1) / kF2Threads;
            C32 o0[NS], o1[NS];
#pragma unroll
            for (int i = 0; i < NS; i++) {
                const int t = threadIdx.x + i * kF2Threads;
                if (TS % kF2Threads == 0 || t < TS) {
                    const int y = t / PT, j = t % PT;
                    const C32 *row = A + y * RSX;
                    if (j == 0) {
                        const C32 z0 = row[ipm[0]], zh = row[ipm[PT]];
                        o0[i] = {z0.re + z0.im, z0.re - z0.im};  // packed X[0] + i X[M]
                        o1[i] = conjc(zh);                       // X[M/2]
                    } else {
                        const C32 zk = row[ipm[j]], zm = conjc(row[ipm[M - j]]);
                        const C32 e = {0.5f * (zk.re + zm.re), 0.5f * (zk.im + zm.im)};
                        const C32 od = {0.5f * (zk.im - zm.im), -0.5f * (zk.re - zm.re)};
                        const C32 tt = cmul(od, tw[j]);
                        o0[i] = cadd(e, tt);         // X[j]
                        o1[i] = conjc(csub(e, tt));  // X[M - j]
                    }
                }
            }
            cl.sync();  // every CTA has read its rows
#pragma unroll
            for (int i = 0; i < NS; i++) {
                const int t = threadIdx.x + i * kF2Threads;
                if (TS % kF2Threads == 0 || t < TS) {
                    const int y = t / PT, j = t % PT, yg = r * H + y;
                    col[0][yg * NCY + j] = o0[i];
                    col[1][yg * NCY + (j == 0 ? 0 : PT - j)] = o1[i];
                }
            }
            cl.sync();  // the columns are complete
        }

        // y: DIF passes but the last, then the span-1 pass to the half spectrum
        spasses<K, K, true, NCY, 1, NCY, true, 1, Seq<K>::n - 1>(A, tw);
        {
            static_assert(Seq<K>::code[0] == 44 && Seq<K>::span[0] == 1, "y pass layout");
            float2 *dst = G + (size_t)P * K * CW;
            constexpr int TASKS = NCY * (K / 16);
            for (int t = threadIdx.x; t < TASKS; t += kF2Threads) {
                const int c = t % NCY, b = t / NCY;
                const C32 *x = A + 16 * b * NCY + c;
                C32 v[4][4];
#pragma unroll
                for (int q2 = 0; q2 < 4; q2++)
#pragma unroll
                    for (int q1 = 0; q1 < 4; q1++) v[q2][q1] = x[(q1 + 4 * q2) * NCY];
                butterfly<float, 4, 4, true, 1, K>(v, 0, tw);
                if (r == 0 && c == 0) {
#pragma unroll
                    for (int q2 = 0; q2 < 4; q2++)
#pragma unroll
                        for (int q1 = 0; q1 < 4; q1++) sc[pk[16 * b + q1 + 4 * q2]] = v[q2][q1];
                } else {
                    float2 *o = dst + r * PT + c;
#pragma unroll
                    for (int q2 = 0; q2 < 4; q2++)
#pragma unroll
                        for (int q1 = 0; q1 < 4; q1++)
                            st2(o + (size_t)pk[16 * b + q1 + 4 * q2] * CW, v[q2][q1]);
                }
            }
        }
        if (r == 0) {
            // the packed column: X[.][0] and X[.][M] from C[ky] and conj C[-ky]
            __syncthreads();
            float2 *dst = G + (size_t)P * K * CW;
            for (int ky = threadIdx.x; ky < K; ky += kF2Threads) {
                const C32 a = sc[ky], b = conjc(sc[ky == 0 ? 0 : K - ky]);
                st2(dst + (size_t)ky * CW, {0.5f * (a.re + b.re), 0.5f * (a.im + b.im)});
                const C32 d = csub(a, b);
                st2(dst + (size_t)ky * CW + M, {0.5f * d.im, -0.5f * d.re});
            }
        }
        __syncthreads();  // the buffer is free for the next plane
    }
}

// Inverse: half spectra G[plane][K][K/2+1] -> real planes mesh[plane][K][K].
// The kx = 0 and K/2 columns are taken as Hermitian in ky (their imaginary
// parts after the y transform are dropped, as a C2R transform does).
template <int K>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(kF2Threads, 1)
    k_fft2d_c2r(const float2 *__restrict__ G, float *__restrict__ mesh,
                const float2 *__restrict__ twg, const int *__restrict__ ipmg,
                const int *__restrict__ pkg, int planes) {
    using F = F2<K>;
    constexpr int M = F::M, H = F::H, RSX = F::RSX, NCY = F::NCY, CW = F::CW, PT = M / 2;
    extern __shared__ __align__(16) unsigned char smem[];
    C32 *A = reinterpret_cast<C32 *>(smem);
    const C32 *tw = reinterpret_cast<const C32 *>(smem + F::tw_off);
    const int *ipm = reinterpret_cast<const int *>(smem + F::ipm_off);
    const int *pk = reinterpret_cast<const int *>(smem + F::pk_off);
    cg::cluster_group cl = cg::this_cluster();
    const int r = (int)cl.block_rank();
    C32 *rows[2] = {cl.map_shared_rank(A, 0), cl.map_shared_rank(A, 1)};
    load_tables<K>(smem, twg, ipmg, pkg);
    __syncthreads();
    const int ncl = (int)(gridDim.x / 2);
    for (int P = (int)(blockIdx.x / 2); P < planes; P += ncl) {
        // y: the span-1 pass (first in DIT order) straight from the half
        // spectrum, position p taking ky = perm_K[p]
        {
            static_assert(Seq<K>::code[0] == 44 && Seq<K>::span[0] == 1, "y pass layout");
            const float2 *src = G + (size_t)P * K * CW;
            constexpr int TASKS = NCY * (K / 16), NI = (TASKS + kF2Threads - 1) / kF2Threads;
            C32 v[NI][4][4];
#pragma unroll
            for (int i = 0; i < NI; i++) {
                const int t = threadIdx.x + i * kF2Threads;
                if (TASKS % kF2Threads == 0 || t < TASKS) {
                    const int c = t % NCY, b = t / NCY;
                    const bool packed = r == 0 && c == 0;
                    const float2 *o = src + r * PT + c;
#pragma unroll
                    for (int q2 = 0; q2 < 4; q2++)
#pragma unroll
                        for (int q1 = 0; q1 < 4; q1++) {
                            const size_t ky = pk[16 * b + q1 + 4 * q2];
                            C32 g = ld2(o + ky * CW);
                            if (packed) {
                                const C32 gm = ld2(src + ky * CW + M);
                                g = {g.re - gm.im, g.im + gm.re};  // G[.][0] + i G[.][M]
                            }
                            v[i][q2][q1] = g;
                        }
                }
            }
#pragma unroll
            for (int i = 0; i < NI; i++) {
                const int t = threadIdx.x + i * kF2Threads;
                if (TASKS % kF2Threads == 0 || t < TASKS) {
                    const int c = t % NCY, b = t / NCY;
                    butterfly<float, 4, 4, false, 1, K>(v[i], 0, tw);
                    C32 *x = A + 16 * b * NCY + c;
#pragma unroll
                    for (int q2 = 0; q2 < 4; q2++)
#pragma unroll
                        for (int q1 = 0; q1 < 4; q1++) x[(q1 + 4 * q2) * NCY] = v[i][q2][q1];
                }
            }
        }
        __syncthreads();
        spasses<K, K, false, NCY, 1, NCY, true, 1, Seq<K>::n - 2>(A, tw);

        // y: the last DIT pass into registers, then to the rows' owners
        {
            constexpr int I = Seq<K>::n - 1, CODE = Seq<K>::code[I], L = Seq<K>::span[I];
            constexpr int R1 = CODE / 10, R2 = CODE % 10, L3 = L * R1 * R2;
            constexpr int TASKS = NCY * (K / (R1 * R2)), NI = (TASKS + kF2Threads - 1) / kF2Threads;
            C32 v[NI][R2][R1];
#pragma unroll
            for (int i = 0; i < NI; i++) {
                const int t = threadIdx.x + i * kF2Threads;
                if (TASKS % kF2Threads == 0 || t < TASKS) {
                    const int c = t % NCY, bi = t / NCY, j = bi % L, b = bi / L;
                    const C32 *x = A + (b * L3 + j) * NCY + c;
#pragma unroll
                    for (int q2 = 0; q2 < R2; q2++)
#pragma unroll
                        for (int q1 = 0; q1 < R1; q1++) v[i][q2][q1] = x[(q1 * L + q2 * L * R1) * NCY];
                    butterfly<float, R1, R2, false, L, K>(v[i], j, tw);
                }
            }
            cl.sync();  // every CTA has read its columns
#pragma unroll
            for (int i = 0; i < NI; i++) {
                const int t = threadIdx.x + i * kF2Threads;
                if (TASKS % kF2Threads == 0 || t < TASKS) {
                    const int c = t % NCY, bi = t / NCY, j = bi % L, b = bi / L;
#pragma unroll
                    for (int q2 = 0; q2 < R2; q2++)
#pragma unroll
                        for (int q1 = 0; q1 < R1; q1++) {
                            const int y = b * L3 + j + q1 * L + q2 * L * R1;
                            C32 *row = rows[y / H] + (y % H) * RSX;
                            const C32 w = v[i][q2][q1];
                            if (r == 0 && c == 0) {
                                row[0] = {w.re, 0.f};  // X[y][0]
                                row[M] = {w.im, 0.f};  // X[y][M]
                            } else {
                                row[r * PT + c] = w;
                            }
                        }
                }
            }
            cl.sync();  // the rows are complete
        }

        // packing: X[0..M] (natural) -> Z' (digit-reversed), in rounds of rows
        {
            constexpr int NBT = 8;
            constexpr int RB = (NBT * kF2Threads) / PT < H ? (NBT * kF2Threads) / PT : H;
            for (int y0 = 0; y0 < H; y0 += RB) {
                C32 a[NBT], c[NBT];
                int at[NBT], pa[NBT], pc[NBT];
#pragma unroll
                for (int i = 0; i < NBT; i++) {
                    const int t = threadIdx.x + i * kF2Threads, y = y0 + t / PT, j = t % PT;
                    at[i] = -1;
                    if (t < RB * PT && y < H) {
                        const C32 *row = A + y * RSX;
                        at[i] = y * RSX;
                        if (j == 0) {
                            const float x0 = row[0].re, xm = row[M].re;
                            a[i] = {x0 + xm, x0 - xm};  // Z'[0]
                            c[i] = conjc(row[PT]);      // Z'[M/2] / 2
                            c[i].re *= 2.f;
                            c[i].im *= 2.f;
                            pa[i] = ipm[0];
                            pc[i] = ipm[PT];
                        } else {
                            const C32 xk = row[j], xm = conjc(row[M - j]);
                            const C32 s = cadd(xk, xm), d = csub(xk, xm);
                            const C32 u = cmul(d, conjc(tw[j]));
                            const C32 iu = {-u.im, u.re};
                            a[i] = cadd(s, iu);         // Z'[j]
                            c[i] = conjc(csub(s, iu));  // Z'[M - j]
                            pa[i] = ipm[j];
                            pc[i] = ipm[M - j];
                        }
                    }
                }
                __syncthreads();
#pragma unroll
                for (int i = 0; i < NBT; i++)
                    if (at[i] >= 0) {
                        A[at[i] + pa[i]] = a[i];
                        A[at[i] + pc[i]] = c[i];
                    }
                __syncthreads();
            }
        }

        // x: DIT passes but the last, then the span-16 pass to the real rows
        spasses<K, M, false, H, RSX, 1, true, 0, Seq<M>::n - 2>(A, tw);
        {
            constexpr int I = Seq<M>::n - 1, CODE = Seq<M>::code[I];
            constexpr int R1 = CODE / 10, R2 = CODE % 10;
            static_assert(Seq<M>::span[I] == 16 && 16 * R1 * R2 == M, "x pass layout");
            constexpr int TASKS = H * 16;
            float2 *dst = reinterpret_cast<float2 *>(mesh) + ((size_t)P * K + (size_t)r * H) * M;
            for (int t = threadIdx.x; t < TASKS; t += kF2Threads) {
                const int y = t >> 4, j = t & 15;
                const C32 *x = A + y * RSX + j;
                C32 v[R2][R1];
#pragma unroll
                for (int q2 = 0; q2 < R2; q2++)
#pragma unroll
                    for (int q1 = 0; q1 < R1; q1++) v[q2][q1] = x[16 * (q1 + q2 * R1)];
                butterfly<float, R1, R2, false, 16, K>(v, j, tw);
                float2 *o = dst + (size_t)y * M + j;
#pragma unroll
                for (int q2 = 0; q2 < R2; q2++)
#pragma unroll
                    for (int q1 = 0; q1 < R1; q1++) st2(o + 16 * (q1 + q2 * R1), v[q2][q1]);
            }
        }
        __syncthreads();  // the buffer is free for the next plane
    }
}

// Launch: persistent clusters, as many as can be resident at once (at most one
// per plane).
template <int K>
cudaError_t launch_k(bool inverse, const void *in, void *out, long planes, const void *tables,
                     cudaStream_t s) {
    using F = F2<K>;
    if (planes <= 0 || planes > 0x7fffffffL) return cudaErrorInvalidValue;
    const float2 *tw = static_cast<const float2 *>(tables);
    const int *ipm = reinterpret_cast<const int *>(tw + K);
    const int *pk = ipm + F::M;
    auto kr = k_fft2d_r2c<K>;
    auto kc = k_fft2d_c2r<K>;
    const void *fn = inverse ? (const void *)kc : (const void *)kr;
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)F::total);
    if (e != cudaSuccess) return e;
    static int max_clusters[2] = {0, 0};  // per direction; the same on every call
    int &mc = max_clusters[inverse ? 1 : 0];
    if (mc == 0) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(2 * 152, 1, 1);
        cfg.blockDim = dim3(kF2Threads, 1, 1);
        cfg.dynamicSmemBytes = F::total;
        cudaLaunchAttribute at;
        at.id = cudaLaunchAttributeClusterDimension;
        at.val.clusterDim.x = 2;
        at.val.clusterDim.y = 1;
        at.val.clusterDim.z = 1;
        cfg.attrs = &at;
        cfg.numAttrs = 1;
        int n = 0;
        e = cudaOccupancyMaxActiveClusters(&n, fn, &cfg);
        if (e != cudaSuccess) return e;
        mc = n > 0 ? n : 1;
    }
    const int ncl = (int)std::min<long>(mc, planes);
    if (inverse)
        kc<<<2 * ncl, kF2Threads, F::total, s>>>(static_cast<const float2 *>(in),
                                                  static_cast<float *>(out), tw, ipm, pk, (int)planes);
    else
        kr<<<2 * ncl, kF2Threads, F::total, s>>>(static_cast<const float *>(in),
                                                  static_cast<float2 *>(out), tw, ipm, pk, (int)planes);
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

template <int N>
bool seq_matches(const ZPlan &z) {
    if (z.K != N || z.npass != Seq<N>::n) return false;
    for (int i = 0; i < Seq<N>::n; i++)
        if (z.pcode[i] != Seq<N>::code[i] || z.pspan[i] != Seq<N>::span[i]) return false;
    return true;
}

template <int K>
bool plans_match(const ZPlan &zm, const ZPlan &zk) {
    return seq_matches<K / 2>(zm) && seq_matches<K>(zk);
}

}  // namespace

bool fft2d_ok(int K, size_t elem) { return elem == 4 && (K == 128 || K == 160 || K == 256); }

size_t fft2d_table_bytes(int K) { return (size_t)K * 8 + (size_t)(K / 2) * 4 + (size_t)K * 4; }

// Twiddles e^{-2 pi i e/K} (FP64, rounded), the inverse digit reversal of the
// K/2-point x transform and the digit reversal of the K-point y transform, both
// from the z-transform planner (whose pass sequences for these lengths the
// kernels hard-code: checked here).
bool make_fft2d_tables(int K, std::vector<unsigned char> *out) {
    if (!fft2d_ok(K, 4)) return false;
    const int M = K / 2;
    ZPlan zm, zk;
    std::vector<double> twd;
    std::vector<int> pm, pkv;
    if (!make_zplan(M, 4, &zm, &twd, &pm) || !make_zplan(K, 4, &zk, &twd, &pkv)) return false;
    const bool ok = K == 128 ? plans_match<128>(zm, zk)
                             : (K == 160 ? plans_match<160>(zm, zk) : plans_match<256>(zm, zk));
    if (!ok) return false;
    out->assign(fft2d_table_bytes(K), 0);
    float *tw = reinterpret_cast<float *>(out->data());
    for (int e = 0; e < K; e++) {
        const double a = -2.0 * M_PI * (double)e / (double)K;
        tw[2 * e] = (float)std::cos(a);
        tw[2 * e + 1] = (float)std::sin(a);
    }
    int *ipm = reinterpret_cast<int *>(tw + 2 * K);
    for (int p = 0; p < M; p++) ipm[pm[p]] = p;
    int *pk = ipm + M;
    for (int p = 0; p < K; p++) pk[p] = pkv[p];
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
