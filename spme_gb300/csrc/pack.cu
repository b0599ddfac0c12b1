// Layout conversions between the reference's vector layout
// v[r*ld + 3i + d] (old-version/spme.h:95-97) and the particle-major
// component rows W[i][3R] that the spread / interpolation / real-space
// kernels read and write.  The BLAS-style combine of compute_spme
// (old-version/spme_kernel.c:28-30, alpha/beta) is fused into the unpack.
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

template <typename T>
__global__ void __launch_bounds__(256)
k_pack_tiled(const T *__restrict__ f, long ld, int n, int R, int r0, int r1, int pb,
             T *__restrict__ F) {
    extern __shared__ __align__(16) unsigned char pk_raw[];
    T *tile = reinterpret_cast<T *>(pk_raw);  // [pb][CP + 1]
    const int C = 3 * R, CP = 3 * (r1 - r0), CS = CP + 1;  // row stride, columns written
    for (int i0 = blockIdx.x * pb; i0 < n; i0 += gridDim.x * pb) {
        const int np = min(pb, n - i0);
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
               int pb, T alpha, T beta, T *__restrict__ u, long ld) {
    extern __shared__ __align__(16) unsigned char pk_raw[];
    T *tile = reinterpret_cast<T *>(pk_raw);  // [pb][CP + 1]
    const int C = 3 * R, CP = 3 * (r1 - r0), CS = CP + 1;  // row stride, columns taken
    for (int i0 = blockIdx.x * pb; i0 < n; i0 += gridDim.x * pb) {
        const int np = min(pb, n - i0);
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
    const size_t pb = (size_t)48 * 1024 / row;
    return (int)(pb < 1 ? 1 : (pb > (size_t)kPB ? kPB : pb));
}

template <typename T>
void launch_pack_tiled(const T *f, long ld, int n, int R, T *F, cudaStream_t s) {
    launch_pack_tiled<T>(f, ld, n, R, 0, R, F, s);
}

template <typename T>
void launch_pack_tiled(const T *f, long ld, int n, int R, int r0, int r1, T *F, cudaStream_t s) {
    if (n <= 0 || R <= 0 || r0 < 0 || r1 > R || r0 >= r1) return;
    const int pb = tile_particles(r1 - r0, sizeof(T));
    const size_t smem = (size_t)pb * (3 * (r1 - r0) + 1) * sizeof(T);
    k_pack_tiled<T><<<tiled_blocks(n, pb), 256, smem, s>>>(f, ld, n, R, r0, r1, pb, F);
}

template <typename T>
void launch_unpack_tiled(const T *W, const T *W2, int n, int R, int r0, int r1, double alpha,
                         double beta, T *u, long ld, cudaStream_t s) {
    if (n <= 0 || R <= 0 || r0 < 0 || r1 > R || r0 >= r1) return;
    const int pb = tile_particles(r1 - r0, sizeof(T));
    const size_t smem = (size_t)pb * (3 * (r1 - r0) + 1) * sizeof(T);
    if (W2)
        k_unpack_tiled<T, true><<<tiled_blocks(n, pb), 256, smem, s>>>(W, W2, n, R, r0, r1, pb,
                                                                        (T)alpha, (T)beta, u, ld);
    else
        k_unpack_tiled<T, false><<<tiled_blocks(n, pb), 256, smem, s>>>(W, W, n, R, r0, r1, pb,
                                                                         (T)alpha, (T)beta, u, ld);
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
