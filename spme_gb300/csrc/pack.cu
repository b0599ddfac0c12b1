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

// u = alpha (W + W2) + beta u: the real-space and mesh parts of the operator.
template <typename T>
__global__ void k_unpack_sum(const T *__restrict__ W, const T *__restrict__ W2, int n, int R,
                             T alpha, T beta, T *__restrict__ u, long ld) {
    const size_t total = (size_t)n * 3 * R;
    const int C = 3 * R;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (size_t)gridDim.x * blockDim.x) {
        const int r = (int)(t / ((size_t)3 * n));
        const size_t q = t - (size_t)r * 3 * n;
        const size_t i = q / 3;
        const int d = (int)(q - i * 3);
        const size_t k = i * C + 3 * r + d;
        const T w = W[k] + W2[k];
        T *o = u + (size_t)r * ld + q;
        *o = beta == T(0) ? alpha * w : beta * *o + alpha * w;
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

template <typename T>
void launch_unpack_sum(const T *W, const T *W2, int n, int R, double alpha, double beta, T *u,
                       long ld, cudaStream_t s) {
    size_t total = (size_t)n * 3 * R;
    if (total)
        k_unpack_sum<T><<<blocks_for(total), 256, 0, s>>>(W, W2, n, R, (T)alpha, (T)beta, u, ld);
}

template <typename T>
void launch_self(const T *F, int n, int R, double self_c, T *W, cudaStream_t s) {
    size_t total = (size_t)n * 3 * R;
    if (total) k_self<T><<<blocks_for(total), 256, 0, s>>>(F, total, (T)self_c, W);
}

template void launch_unpack_sum<float>(const float *, const float *, int, int, double, double,
                                       float *, long, cudaStream_t);
template void launch_unpack_sum<double>(const double *, const double *, int, int, double, double,
                                        double *, long, cudaStream_t);
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
