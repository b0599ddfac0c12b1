// Interpolation of the 3R mesh components back to the particles (restates
// old-version/spme_kernel.c:8-70: v_i = sum_j P_ij grid[c][ind_ij]).
//
// One warp per particle, visited in tile-sorted order so that consecutive
// warps read overlapping mesh neighbourhoods (L1/L2 reuse).  Lanes are
// (x-slot, component) pairs: each load instruction reads C-contiguous runs of
// the interleaved mesh [z][y][x][C]; the x-slots are summed with shuffles.
#include "kernels.h"

namespace spme {

namespace {

constexpr int kThreads = 256;

template <typename T, int P, int CGP, int NS>
__global__ void __launch_bounds__(kThreads)
k_interp(int n, const int *__restrict__ rec_idx, const uint32_t *__restrict__ rec_start,
         const T *__restrict__ rec_w, const T *__restrict__ mesh, int C, MeshGeom g,
         T *__restrict__ W, int accumulate) {
    constexpr int WS = RecordWidth<T, P>::value;
    constexpr int XS = 32 / CGP;
    constexpr int CC = CGP * NS;
    constexpr int XI = (P + XS - 1) / XS;  // x iterations per lane
    const int lane = threadIdx.x & 31;
    const int xs = lane / CGP, cl = lane % CGP;
    const int K = g.K;
    const long warps = (long)gridDim.x * (kThreads / 32);
    for (long s = (long)blockIdx.x * (kThreads / 32) + (threadIdx.x >> 5); s < n; s += warps) {
        const T wreg = lane < 3 * P ? rec_w[(size_t)s * WS + lane] : T(0);
        int sx, sy, sz;
        unpack_start(rec_start[s], sx, sy, sz);
        const int idx = rec_idx[s];
        // this lane's x weights and mesh x coordinates
        T wx[XI];
        int gx[XI];
#pragma unroll
        for (int k = 0; k < XI; k++) {
            const int x = xs + k * XS;
            const T v = __shfl_sync(0xffffffffu, wreg, x < P ? x : P - 1);
            wx[k] = x < P ? v : T(0);
            int c = sx + (x < P ? x : 0);
            gx[k] = c >= K ? c - K : c;
        }
        for (int cbase = 0; cbase < C; cbase += CC) {
            T acc[NS];
#pragma unroll
            for (int sl = 0; sl < NS; sl++) acc[sl] = T(0);
#pragma unroll
            for (int z = 0; z < P; z++) {
                const T wz = __shfl_sync(0xffffffffu, wreg, 2 * P + z);
                int gz = sz + z;
                gz = gz >= K ? gz - K : gz;
#pragma unroll
                for (int y = 0; y < P; y++) {
                    const T wzy = wz * __shfl_sync(0xffffffffu, wreg, P + y);
                    int gy = sy + y;
                    gy = gy >= K ? gy - K : gy;
                    const size_t row = ((size_t)gz * K + gy) * K;
#pragma unroll
                    for (int k = 0; k < XI; k++) {
                        const T w = wzy * wx[k];
                        const T *mp = mesh + (row + gx[k]) * C + cbase + cl;
#pragma unroll
                        for (int sl = 0; sl < NS; sl++)
                            if (cbase + sl * CGP + cl < C) acc[sl] += w * __ldg(mp + sl * CGP);
                    }
                }
            }
#pragma unroll
            for (int sl = 0; sl < NS; sl++)
#pragma unroll
                for (int o = CGP; o < 32; o <<= 1)
                    acc[sl] += __shfl_xor_sync(0xffffffffu, acc[sl], o);
            if (xs == 0) {
#pragma unroll
                for (int sl = 0; sl < NS; sl++) {
                    const int c = cbase + sl * CGP + cl;
                    if (c < C) {
                        T *o = W + (size_t)idx * C + c;
                        *o = accumulate ? *o + acc[sl] : acc[sl];
                    }
                }
            }
        }
    }
}

template <typename T, int P, int CGP, int NS>
cudaError_t launch_interp_t(int n, const int *rec_idx, const uint32_t *rec_start,
                            const T *rec_w, const T *mesh, int C, const MeshGeom &g, T *W,
                            int accumulate, cudaStream_t s) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    long need = ((long)n + (kThreads / 32) - 1) / (kThreads / 32);
    long cap = (long)sms * 8;
    int blocks = (int)(need < cap ? need : cap);
    if (blocks < 1) blocks = 1;
    k_interp<T, P, CGP, NS><<<blocks, kThreads, 0, s>>>(n, rec_idx, rec_start, rec_w, mesh, C,
                                                        g, W, accumulate);
    return cudaGetLastError();
}

template <typename T, int P>
cudaError_t dispatch_split(int n, const int *rec_idx, const uint32_t *rec_start,
                           const T *rec_w, const T *mesh, int C, const MeshGeom &g, T *W,
                           int accumulate, cudaStream_t s) {
    CompSplit cs = choose_comp_split(C, 1 << 30);
#define SPME_INTERP_CASE(CG, N)                                                          \
    if (cs.cgp == CG && cs.ns == N)                                                      \
        return launch_interp_t<T, P, CG, N>(n, rec_idx, rec_start, rec_w, mesh, C, g, W, \
                                            accumulate, s);
    SPME_INTERP_CASE(4, 1)
    SPME_INTERP_CASE(8, 1)
    SPME_INTERP_CASE(16, 1)
    SPME_INTERP_CASE(4, 3)
    SPME_INTERP_CASE(8, 3)
    SPME_INTERP_CASE(16, 3)
#undef SPME_INTERP_CASE
    return cudaErrorInvalidValue;
}

}  // namespace

template <typename T>
cudaError_t launch_interp(int n, const int *rec_idx, const uint32_t *rec_start,
                          const T *rec_w, const T *mesh, int C, const MeshGeom &g, T *W,
                          int accumulate, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    switch (g.p) {
        case 4: return dispatch_split<T, 4>(n, rec_idx, rec_start, rec_w, mesh, C, g, W, accumulate, s);
        case 6: return dispatch_split<T, 6>(n, rec_idx, rec_start, rec_w, mesh, C, g, W, accumulate, s);
        case 8: return dispatch_split<T, 8>(n, rec_idx, rec_start, rec_w, mesh, C, g, W, accumulate, s);
        default: return cudaErrorInvalidValue;
    }
}

template cudaError_t launch_interp<float>(int, const int *, const uint32_t *, const float *,
                                          const float *, int, const MeshGeom &, float *, int,
                                          cudaStream_t);
template cudaError_t launch_interp<double>(int, const int *, const uint32_t *, const double *,
                                           const double *, int, const MeshGeom &, double *, int,
                                           cudaStream_t);

}  // namespace spme
