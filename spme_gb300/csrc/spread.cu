// Spread of 3R force components onto the K^3 mesh (restates
// old-version/spme_kernel.c:231-312: grid[c][ind] += P * f_c).
//
// GB300 design (owner computes, register accumulation):
//   * particles are sorted by the mesh tile that holds their stencil start;
//   * one CTA owns one tile (tx x ty x tz, tz <= TZ) and a range of components;
//     every thread owns one (x, y) column of the tile for CPT components and
//     keeps all TZ planes of that column in registers;
//   * the CTA stages, in chunks, every particle whose stencil reaches the tile
//     (its own tile and the lower neighbours per axis, wrap-aware): the
//     particle's B-spline weights scattered into zero-filled tile-local x / y /
//     z rows (transposed, padded stride: conflict-free) and its forces;
//   * each thread adds w_x w_y w_z f_c for the staged particles that cover its
//     column, skipping (warp-uniformly) the planes the stencil misses, then
//     writes its column once (no zeroing, no atomics).
// Mesh layout is component-major, mesh[c][z][y][x], the contiguous batched
// layout the cuFFT plans use.
#include "kernels.h"

namespace spme {

namespace {

constexpr int kMaxSrc = 6;   // source tiles per axis; 5 suffice for tile edges >= 4, p <= 8
constexpr int kChunk = 256;  // particles staged per round

template <typename T> struct Vec16;
template <> struct Vec16<float> { using type = float4; };
template <> struct Vec16<double> { using type = double2; };

struct Segments {
    int beg[kMaxSrc * kMaxSrc * kMaxSrc];
    int pre[kMaxSrc * kMaxSrc * kMaxSrc + 1];
    int n;
};

// Tiles whose cells can hold a stencil start that reaches [org, org+ext) on
// one axis, deduplicated (the range can wrap onto itself for small K).
__device__ int source_tiles(int org, int ext, int te, int K, int P, int *out) {
    int cell = pmod(org - (P - 1), K);
    int remaining = min(ext + P - 1, K);
    int cnt = 0;
    while (remaining > 0 && cnt < kMaxSrc) {
        int tl = cell / te;
        bool dup = false;
        for (int k = 0; k < cnt; k++) dup |= (out[k] == tl);
        if (!dup) out[cnt++] = tl;
        int end = min((tl + 1) * te, K);
        remaining -= end - cell;
        cell = end % K;
    }
    return cnt;
}

__device__ void build_segments(const int *tile_off, const MeshGeom &g, const int org[3],
                               const int ext[3], int P, Segments &sg) {
    int src[3][kMaxSrc], ns[3];
    ns[0] = source_tiles(org[0], ext[0], g.tx, g.K, P, src[0]);
    ns[1] = source_tiles(org[1], ext[1], g.ty, g.K, P, src[1]);
    ns[2] = source_tiles(org[2], ext[2], g.tz, g.K, P, src[2]);
    int k = 0, pre = 0;
    for (int c = 0; c < ns[2]; c++)
        for (int b = 0; b < ns[1]; b++)
            for (int a = 0; a < ns[0]; a++) {
                int id = (src[2][c] * g.nty + src[1][b]) * g.ntx + src[0][a];
                int beg = tile_off[id], len = tile_off[id + 1] - beg;
                sg.beg[k] = beg;
                sg.pre[k] = pre;
                pre += len;
                k++;
            }
    sg.pre[k] = pre;
    sg.n = k;
}

template <typename T, int P, int CPT, int TZ>
__global__ void __launch_bounds__(256, (CPT * TZ > 96 ? 1 : 2))
k_spread(const int *__restrict__ tile_off, const int *__restrict__ rec_idx,
         const uint32_t *__restrict__ rec_start, const T *__restrict__ rec_w,
         const T *__restrict__ F, int C, MeshGeom g, T *__restrict__ mesh) {
    constexpr int WS = RecordWidth<T, P>::value;
    constexpr int KS = kChunk + 1;  // padded stride of the transposed weight rows
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ Segments sg;
    const int npt = g.tx * g.ty;
    const int ng = blockDim.x / npt;
    const int CC = ng * CPT;  // components staged per particle (this CTA's range)
    const int WL = g.tx + g.ty + TZ;
    T *fs = reinterpret_cast<T *>(smem_raw);      // [kChunk][CC] forces
    T *wl = fs + (size_t)kChunk * CC;             // [WL][KS] tile-local weights
    int *pidx = reinterpret_cast<int *>(wl + (size_t)WL * KS);  // [kChunk] particle ids

    const int tile = blockIdx.x;
    const int tix = tile % g.ntx, tiy = (tile / g.ntx) % g.nty, tiz = tile / (g.ntx * g.nty);
    const int org[3] = {tix * g.tx, tiy * g.ty, tiz * g.tz};
    const int ext[3] = {min(g.tx, g.K - org[0]), min(g.ty, g.K - org[1]), min(g.tz, g.K - org[2])};
    const int pt = threadIdx.x % npt, grp = threadIdx.x / npt;
    const int x = pt % g.tx, y = pt / g.tx;
    const int ccta = blockIdx.y * CC;  // first component of this CTA
    const int cbase = ccta + grp * CPT;
    const int ncomp = max(0, min(CPT, C - cbase));
    const int ncta = min(CC, C - ccta);
    const bool owner = x < ext[0] && y < ext[1] && ncomp > 0;

    if (threadIdx.x == 0) build_segments(tile_off, g, org, ext, P, sg);
    __syncthreads();
    const int total = sg.pre[sg.n];

    T acc[TZ][CPT];
#pragma unroll
    for (int z = 0; z < TZ; z++)
#pragma unroll
        for (int j = 0; j < CPT; j++) acc[z][j] = T(0);

    const T *wxr = wl + (size_t)x * KS;
    const T *wyr = wl + (size_t)(g.tx + y) * KS;
    const T *wzr = wl + (size_t)(g.tx + g.ty) * KS;
    for (int c0 = 0; c0 < total; c0 += kChunk) {
        const int nch = min(kChunk, total - c0);
        __syncthreads();
        for (int k = threadIdx.x; k < nch; k += blockDim.x) {
            const int q = c0 + k;
            int seg = 0;
            while (q >= sg.pre[seg + 1]) seg++;
            const int s = sg.beg[seg] + (q - sg.pre[seg]);
            for (int j = 0; j < WL; j++) wl[(size_t)j * KS + k] = T(0);
            int st[3];
            unpack_start(rec_start[s], st[0], st[1], st[2]);
            const T *rw = rec_w + (size_t)s * WS;
            const int base[3] = {0, g.tx, g.tx + g.ty};
#pragma unroll
            for (int a = 0; a < 3; a++) {
#pragma unroll
                for (int j = 0; j < P; j++) {
                    int gc = st[a] + j;
                    if (gc >= g.K) gc -= g.K;
                    const int l = gc - org[a];
                    if ((unsigned)l < (unsigned)ext[a]) wl[(size_t)(base[a] + l) * KS + k] = rw[a * P + j];
                }
            }
            pidx[k] = rec_idx[s];
        }
        __syncthreads();
        // forces of the staged particles, one element per thread (coalesced rows,
        // conflict-free shared stores)
        {
            DivMod dcc;
            dcc.init(CC);
            for (int q = threadIdx.x; q < nch * CC; q += blockDim.x) {
                int j;
                const int k = dcc.div(q, j);
                fs[q] = j < ncta ? __ldg(F + (size_t)pidx[k] * C + ccta + j) : T(0);
            }
        }
        __syncthreads();
        if (owner) {
            for (int k = 0; k < nch; k++) {
                const T wxy = wxr[k] * wyr[k];
                if (wxy == T(0)) continue;  // column not covered by this particle
                T f[CPT], wz[TZ];
                const T *fk = fs + (size_t)k * CC + grp * CPT;
                if constexpr ((CPT * sizeof(T)) % 16 == 0) {
                    // CC and CPT are multiples of 16 bytes: vector broadcast loads
                    using V = typename Vec16<T>::type;
                    constexpr int VW = 16 / sizeof(T);
#pragma unroll
                    for (int j = 0; j < CPT; j += VW)
                        *reinterpret_cast<V *>(&f[j]) = *reinterpret_cast<const V *>(fk + j);
                } else {
#pragma unroll
                    for (int j = 0; j < CPT; j++) f[j] = fk[j];
                }
#pragma unroll
                for (int z = 0; z < TZ; z++) wz[z] = wzr[(size_t)z * KS + k];
                // wz is the same for every lane (one particle per iteration), so this
                // branch is warp-uniform: planes the stencil misses cost nothing
#pragma unroll
                for (int z = 0; z < TZ; z++) {
                    if (wz[z] != T(0)) {
                        const T wv = wxy * wz[z];
#pragma unroll
                        for (int j = 0; j < CPT; j++) acc[z][j] += wv * f[j];
                    }
                }
            }
        }
    }
    if (owner) {
        const size_t K = (size_t)g.K;
        const size_t col = ((size_t)org[1] + y) * K + org[0] + x;
#pragma unroll
        for (int z = 0; z < TZ; z++) {
            if (z < ext[2]) {
#pragma unroll
                for (int j = 0; j < CPT; j++)
                    if (j < ncomp)
                        mesh[((size_t)(cbase + j) * K + org[2] + z) * K * K + col] = acc[z][j];
            }
        }
    }
}

template <int CPT>
int groups_per_cta(const MeshGeom &g, int C) {
    int npt = g.tx * g.ty;
    int need = (C + CPT - 1) / CPT;
    int cap = 256 / npt;
    if (cap < 1) cap = 1;
    return need < cap ? need : cap;
}

template <typename T, int P, int CPT, int TZ>
cudaError_t launch_spread_t(const int *tile_off, const int *rec_idx, const uint32_t *rec_start,
                            const T *rec_w, const T *F, int C, const MeshGeom &g, T *mesh,
                            cudaStream_t s) {
    const int ng = groups_per_cta<CPT>(g, C);
    const int threads = g.tx * g.ty * ng;
    const int WL = g.tx + g.ty + TZ;
    size_t smem = ((size_t)kChunk * CPT * ng + (size_t)WL * (kChunk + 1)) * sizeof(T) +
                  (size_t)kChunk * sizeof(int);
    auto kern = k_spread<T, P, CPT, TZ>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    dim3 grid(g.ntx * g.nty * g.ntz, (C + CPT * ng - 1) / (CPT * ng));
    kern<<<grid, threads, smem, s>>>(tile_off, rec_idx, rec_start, rec_w, F, C, g, mesh);
    return cudaGetLastError();
}

template <typename T, int P, int TZ>
cudaError_t dispatch_cpt(const int *tile_off, const int *rec_idx, const uint32_t *rec_start,
                         const T *rec_w, const T *F, int C, const MeshGeom &g, T *mesh,
                         cudaStream_t s) {
    // with at most 4 register planes, 24 components per thread halve the number
    // of (warp, particle) visits for many right-hand sides
    if constexpr (TZ <= 4 && sizeof(T) == 4)
        if (C >= 16)
            return launch_spread_t<T, P, 24, TZ>(tile_off, rec_idx, rec_start, rec_w, F, C, g, mesh, s);
    if (C <= 3)
        return launch_spread_t<T, P, 3, TZ>(tile_off, rec_idx, rec_start, rec_w, F, C, g, mesh, s);
    if (C <= 6)
        return launch_spread_t<T, P, 6, TZ>(tile_off, rec_idx, rec_start, rec_w, F, C, g, mesh, s);
    return launch_spread_t<T, P, 12, TZ>(tile_off, rec_idx, rec_start, rec_w, F, C, g, mesh, s);
}

template <typename T, int P>
cudaError_t dispatch_tz(const int *tile_off, const int *rec_idx, const uint32_t *rec_start,
                        const T *rec_w, const T *F, int C, const MeshGeom &g, T *mesh,
                        cudaStream_t s) {
    if (g.tz <= 4) return dispatch_cpt<T, P, 4>(tile_off, rec_idx, rec_start, rec_w, F, C, g, mesh, s);
    if (g.tz <= 8) return dispatch_cpt<T, P, 8>(tile_off, rec_idx, rec_start, rec_w, F, C, g, mesh, s);
    return cudaErrorInvalidValue;
}

}  // namespace

template <typename T>
cudaError_t launch_spread(const int *tile_off, const int *rec_idx, const uint32_t *rec_start,
                          const T *rec_w, const T *F, int C, const MeshGeom &g, T *mesh,
                          cudaStream_t s) {
    if (g.tx > 16 || g.ty > 16 || g.tz > 8) return cudaErrorInvalidValue;
    switch (g.p) {
        case 4: return dispatch_tz<T, 4>(tile_off, rec_idx, rec_start, rec_w, F, C, g, mesh, s);
        case 6: return dispatch_tz<T, 6>(tile_off, rec_idx, rec_start, rec_w, F, C, g, mesh, s);
        case 8: return dispatch_tz<T, 8>(tile_off, rec_idx, rec_start, rec_w, F, C, g, mesh, s);
        default: return cudaErrorInvalidValue;
    }
}

template cudaError_t launch_spread<float>(const int *, const int *, const uint32_t *,
                                          const float *, const float *, int, const MeshGeom &,
                                          float *, cudaStream_t);
template cudaError_t launch_spread<double>(const int *, const int *, const uint32_t *,
                                           const double *, const double *, int,
                                           const MeshGeom &, double *, cudaStream_t);

}  // namespace spme
