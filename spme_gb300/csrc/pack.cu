// Layout conversions between the reference's vector layout
// v[r*ld + 3i + d] (old-version/spme.h:95-97) and the particle-major
// component rows W[i][3R] that the spread / interpolation / real-space
// kernels read and write.  The BLAS-style combine of compute_spme
// (old-version/spme_kernel.c:28-30, alpha/beta) is fused into the unpack.
#include <cstdint>

#include "kernels.h"

namespace spme {

namespace {

template <typename T>
__global__ void k_pack(const T *__restrict__ f, long ld, int n, int R, T *__restrict__ F) {
    const size_t total = (size_t)n * 3 * R;
    const int C = 3 * R;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (size_t)gridDim.x * blockDim.x) {
        // read-major: t walks the source (r, 3i+d) contiguously
        const int r = (int)(t / ((size_t)3 * n));
        const size_t q = t - (size_t)r * 3 * n;
        const size_t i = q / 3;
        const int d = (int)(q - i * 3);
        F[i * C + 3 * r + d] = f[(size_t)r * ld + q];
    }
}

// Fs[s][c] = F[idx[s]][c]: force rows in another particle order.
template <typename T>
__global__ void k_gather_rows(const T *__restrict__ F, const int *__restrict__ idx, int n, int C,
                              T *__restrict__ Fs) {
    const size_t total = (size_t)n * C;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (size_t)gridDim.x * blockDim.x) {
        const size_t s = t / C;
        const int c = (int)(t - s * C);
        Fs[t] = F[(size_t)idx[s] * C + c];
    }
}

template <typename T>
__global__ void k_unpack(const T *__restrict__ W, int n, int R, T alpha, T beta,
                         T *__restrict__ u, long ld) {
    const size_t total = (size_t)n * 3 * R;
    const int C = 3 * R;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (size_t)gridDim.x * blockDim.x) {
        const int r = (int)(t / ((size_t)3 * n));
        const size_t q = t - (size_t)r * 3 * n;
        const size_t i = q / 3;
        const int d = (int)(q - i * 3);
        const T w = W[i * C + 3 * r + d];
        T *o = u + (size_t)r * ld + q;
        *o = beta == T(0) ? alpha * w : beta * *o + alpha * w;
    }
}

// Tiled forms: a block moves pb particles at a time (at most kPB, fewer for
// many right-hand sides so the tile stays within 48 KB) through shared memory
// so both sides are coalesced (rows of 3 pb values per right-hand side on the
// caller's side, rows of C values per particle on the packed side).  128
// measured faster than 32 for the 48-component pack/unpack at N = 1e6 (0.157 /
// 0.158 vs 0.172 / 0.178 ms).
constexpr int kPB = 128;

// FP32 tiles whose rows are 16-byte aligned on both sides (vec set by the
// launcher: ld, the base, C, 3 r0 and CP multiples of 4; np a multiple of 4 per
// tile) move 16-byte vectors and divide once per vector; other tiles move scalars.
template <typename T>
__global__ void __launch_bounds__(256)
k_pack_tiled(const T *__restrict__ f, long ld, int n, int R, int r0, int r1, int pb, int vec,
             T *__restrict__ F) {
    extern __shared__ __align__(16) unsigned char pk_raw[];
    T *tile = reinterpret_cast<T *>(pk_raw);  // [pb][CP + 1]
    const int C = 3 * R, CP = 3 * (r1 - r0), CS = CP + 1;  // row stride, columns written
    for (int i0 = blockIdx.x * pb; i0 < n; i0 += gridDim.x * pb) {
        const int np = min(pb, n - i0);
        if constexpr (sizeof(T) == 4) {
            if (vec && (np & 3) == 0) {
                const int nq4 = 3 * np / 4, nc4 = CP / 4;  // vectors per row, per particle
                DivMod dq, dc;
                dq.init(nq4);
                dc.init(nc4);
                for (int t = threadIdx.x; t < (r1 - r0) * nq4; t += blockDim.x) {
                    int q4;
                    const int r = dq.div(t, q4);
                    const float4 v = __ldg(reinterpret_cast<const float4 *>(
                        f + (size_t)(r0 + r) * ld + (size_t)3 * i0 + 4 * q4));
                    const float e[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
                    for (int j = 0; j < 4; j++) {
                        const int q = 4 * q4 + j, p = q / 3;
                        tile[p * CS + 3 * r + (q - 3 * p)] = e[j];
                    }
                }
                __syncthreads();
                for (int t = threadIdx.x; t < np * nc4; t += blockDim.x) {
                    int c4;
                    const int p = dc.div(t, c4);
                    const float *src = tile + p * CS + 4 * c4;
                    *reinterpret_cast<float4 *>(F + (size_t)(i0 + p) * C + 3 * r0 + 4 * c4) =
                        make_float4(src[0], src[1], src[2], src[3]);
                }
                __syncthreads();
                continue;
            }
        }
        for (int t = threadIdx.x; t < (r1 - r0) * 3 * np; t += blockDim.x) {
            const int r = t / (3 * np), q = t - r * 3 * np;
            const int p = q / 3, d = q - p * 3;
            tile[p * CS + 3 * r + d] = f[(size_t)(r0 + r) * ld + (size_t)3 * i0 + q];
        }
        __syncthreads();
        for (int t = threadIdx.x; t < np * CP; t += blockDim.x) {
            const int p = t / CP, c = t - p * CP;
            F[(size_t)(i0 + p) * C + 3 * r0 + c] = tile[p * CS + c];
        }
        __syncthreads();
    }
}

// u = alpha (W [+ W2]) + beta u, tiled as k_pack_tiled.
template <typename T, bool SUM>
__global__ void __launch_bounds__(256)
k_unpack_tiled(const T *__restrict__ W, const T *__restrict__ W2, int n, int R, int r0, int r1,
               int pb, int vec, T alpha, T beta, T *__restrict__ u, long ld) {
    extern __shared__ __align__(16) unsigned char pk_raw[];
    T *tile = reinterpret_cast<T *>(pk_raw);  // [pb][CP + 1]
    const int C = 3 * R, CP = 3 * (r1 - r0), CS = CP + 1;  // row stride, columns taken
    for (int i0 = blockIdx.x * pb; i0 < n; i0 += gridDim.x * pb) {
        const int np = min(pb, n - i0);
        if constexpr (sizeof(T) == 4) {
            if (vec && (np & 3) == 0) {
                const int nq4 = 3 * np / 4, nc4 = CP / 4;
                DivMod dq, dc;
                dq.init(nq4);
                dc.init(nc4);
                for (int t = threadIdx.x; t < np * nc4; t += blockDim.x) {
                    int c4;
                    const int p = dc.div(t, c4);
                    const size_t k = (size_t)(i0 + p) * C + 3 * r0 + 4 * c4;
                    float4 v = __ldg(reinterpret_cast<const float4 *>(W + k));
                    if (SUM) {
                        const float4 v2 = __ldg(reinterpret_cast<const float4 *>(W2 + k));
                        v.x += v2.x;
                        v.y += v2.y;
                        v.z += v2.z;
                        v.w += v2.w;
                    }
                    float *dst = tile + p * CS + 4 * c4;
                    dst[0] = v.x;
                    dst[1] = v.y;
                    dst[2] = v.z;
                    dst[3] = v.w;
                }
                __syncthreads();
                for (int t = threadIdx.x; t < (r1 - r0) * nq4; t += blockDim.x) {
                    int q4;
                    const int r = dq.div(t, q4);
                    float e[4];
#pragma unroll
                    for (int j = 0; j < 4; j++) {
                        const int q = 4 * q4 + j, p = q / 3;
                        e[j] = alpha * tile[p * CS + 3 * r + (q - 3 * p)];
                    }
                    float4 *o = reinterpret_cast<float4 *>(u + (size_t)(r0 + r) * ld +
                                                           (size_t)3 * i0 + 4 * q4);
                    if (beta != 0.f) {
                        const float4 b = *o;
                        e[0] += beta * b.x;
                        e[1] += beta * b.y;
                        e[2] += beta * b.z;
                        e[3] += beta * b.w;
                    }
                    *o = make_float4(e[0], e[1], e[2], e[3]);
                }
                __syncthreads();
                continue;
            }
        }
        for (int t = threadIdx.x; t < np * CP; t += blockDim.x) {
            const int p = t / CP, c = t - p * CP;
            const size_t k = (size_t)(i0 + p) * C + 3 * r0 + c;
            tile[p * CS + c] = SUM ? W[k] + W2[k] : W[k];
        }
        __syncthreads();
        for (int t = threadIdx.x; t < (r1 - r0) * 3 * np; t += blockDim.x) {
            const int r = t / (3 * np), q = t - r * 3 * np;
            const int p = q / 3, d = q - p * 3;
            const T w = tile[p * CS + 3 * r + d];
            T *o = u + (size_t)(r0 + r) * ld + (size_t)3 * i0 + q;
            *o = beta == T(0) ? alpha * w : beta * *o + alpha * w;
        }
        __syncthreads();
    }
}

template <typename T>
__global__ void k_self(const T *__restrict__ F, size_t total, T self_c, T *__restrict__ W) {
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (size_t)gridDim.x * blockDim.x)
        W[t] = self_c * F[t];
}

int blocks_for(size_t work) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    size_t need = (work + 255) / 256;
    size_t cap = (size_t)sms * 16;
    return (int)(need < cap ? (need > 0 ? need : 1) : cap);
}

}  // namespace

template <typename T>
void launch_pack(const T *f, long ld, int n, int R, T *F, cudaStream_t s) {
    size_t total = (size_t)n * 3 * R;
    if (total) k_pack<T><<<blocks_for(total), 256, 0, s>>>(f, ld, n, R, F);
}

template <typename T>
void launch_gather_rows(const T *F, const int *idx, int n, int C, T *Fs, cudaStream_t s) {
    size_t total = (size_t)n * C;
    if (total) k_gather_rows<T><<<blocks_for(total), 256, 0, s>>>(F, idx, n, C, Fs);
}

template <typename T>
void launch_unpack(const T *W, int n, int R, double alpha, double beta, T *u, long ld,
                   cudaStream_t s) {
    size_t total = (size_t)n * 3 * R;
    if (total) k_unpack<T><<<blocks_for(total), 256, 0, s>>>(W, n, R, (T)alpha, (T)beta, u, ld);
}

int tiled_blocks(int n, int pb) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int need = (n + pb - 1) / pb;
    return need < sms * 8 ? (need > 0 ? need : 1) : sms * 8;
}

int tile_particles(int R, size_t elem) {
    const size_t row = (size_t)(3 * R + 1) * elem;
    size_t pb = (size_t)48 * 1024 / row;
    pb = pb > (size_t)kPB ? kPB : pb;
    if (pb >= 4) pb &= ~(size_t)3;  // whole 16-byte vectors of 3 pb / 4 per row
    return (int)(pb < 1 ? 1 : pb);
}

template <typename T>
void launch_pack_tiled(const T *f, long ld, int n, int R, T *F, cudaStream_t s) {
    launch_pack_tiled<T>(f, ld, n, R, 0, R, F, s);
}

// 16-byte vectors on both sides of an FP32 tile: the caller's rows (ld, base) and
// the packed rows (C, the first column 3 r0, the width 3 (r1 - r0), the base)
// all 16-byte aligned, and whole tiles of a multiple of 4 particles.
template <typename T>
int vec_tiles(const T *caller, long ld, const T *packed, int R, int r0, int r1, int pb) {
    if (sizeof(T) != 4) return 0;
    return (ld % 4 == 0 && (3 * R) % 4 == 0 && (3 * r0) % 4 == 0 && (3 * (r1 - r0)) % 4 == 0 &&
            pb % 4 == 0 && (uintptr_t)caller % 16 == 0 && (uintptr_t)packed % 16 == 0)
               ? 1
               : 0;
}

template <typename T>
void launch_pack_tiled(const T *f, long ld, int n, int R, int r0, int r1, T *F, cudaStream_t s) {
    if (n <= 0 || R <= 0 || r0 < 0 || r1 > R || r0 >= r1) return;
    const int pb = tile_particles(r1 - r0, sizeof(T));
    const size_t smem = (size_t)pb * (3 * (r1 - r0) + 1) * sizeof(T);
    const int vec = vec_tiles<T>(f, ld, F, R, r0, r1, pb);
    k_pack_tiled<T><<<tiled_blocks(n, pb), 256, smem, s>>>(f, ld, n, R, r0, r1, pb, vec, F);
}

template <typename T>
void launch_unpack_tiled(const T *W, const T *W2, int n, int R, int r0, int r1, double alpha,
                         double beta, T *u, long ld, cudaStream_t s) {
    if (n <= 0 || R <= 0 || r0 < 0 || r1 > R || r0 >= r1) return;
    const int pb = tile_particles(r1 - r0, sizeof(T));
    const size_t smem = (size_t)pb * (3 * (r1 - r0) + 1) * sizeof(T);
    const int vec = vec_tiles<T>(u, ld, W, R, r0, r1, pb) &&
                    (!W2 || (uintptr_t)W2 % 16 == 0);
    if (W2)
        k_unpack_tiled<T, true><<<tiled_blocks(n, pb), 256, smem, s>>>(
            W, W2, n, R, r0, r1, pb, vec, (T)alpha, (T)beta, u, ld);
    else
        k_unpack_tiled<T, false><<<tiled_blocks(n, pb), 256, smem, s>>>(
            W, W, n, R, r0, r1, pb, vec, (T)alpha, (T)beta, u, ld);
}

template <typename T>
void launch_self(const T *F, int n, int R, double self_c, T *W, cudaStream_t s) {
    size_t total = (size_t)n * 3 * R;
    if (total) k_self<T><<<blocks_for(total), 256, 0, s>>>(F, total, (T)self_c, W);
}

template void launch_pack_tiled<float>(const float *, long, int, int, float *, cudaStream_t);
template void launch_pack_tiled<double>(const double *, long, int, int, double *, cudaStream_t);
template void launch_pack_tiled<float>(const float *, long, int, int, int, int, float *,
                                       cudaStream_t);
template void launch_pack_tiled<double>(const double *, long, int, int, int, int, double *,
                                        cudaStream_t);
template void launch_unpack_tiled<float>(const float *, const float *, int, int, int, int, double,
                                         double, float *, long, cudaStream_t);
template void launch_unpack_tiled<double>(const double *, const double *, int, int, int, int,
                                          double, double, double *, long, cudaStream_t);
template void launch_self<float>(const float *, int, int, double, float *, cudaStream_t);
template void launch_self<double>(const double *, int, int, double, double *, cudaStream_t);
template void launch_gather_rows<float>(const float *, const int *, int, int, float *,
                                        cudaStream_t);
template void launch_gather_rows<double>(const double *, const int *, int, int, double *,
                                         cudaStream_t);
template void launch_pack<float>(const float *, long, int, int, float *, cudaStream_t);
template void launch_pack<double>(const double *, long, int, int, double *, cudaStream_t);
template void launch_unpack<float>(const float *, int, int, double, double, float *, long,
                                   cudaStream_t);
template void launch_unpack<double>(const double *, int, int, double, double, double *, long,
                                    cudaStream_t);

}  // namespace spme
