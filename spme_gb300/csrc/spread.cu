// Spread of 3R force components onto the K^3 mesh (restates
// old-version/spme_kernel.c:231-312: grid[c][ind] += P * f_c).
//
// GB300 design: particles are sorted by the mesh tile holding their stencil
// start.  One CTA owns one tile (and a group of components): it accumulates,
// in shared memory, the contributions of every particle whose stencil reaches
// the tile (its own tile and up to 3 lower neighbours per axis, wrap-aware),
// clipped to the tile, then writes the tile once with coalesced stores.  Every
// mesh value is written exactly once, so the mesh needs no zeroing and no
// global atomics.  Mesh layout is interleaved [z][y][x][C].
#include "kernels.h"

namespace spme {

namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kMaxSrc = 6;   // source tiles per axis; 5 suffice for tile edges >= 4, p <= 8

template <typename T, int P, int CGP, int NS>
__global__ void __launch_bounds__(kThreads)
k_spread(const int *__restrict__ tile_off, const int *__restrict__ rec_idx,
         const uint32_t *__restrict__ rec_start, const T *__restrict__ rec_w,
         const T *__restrict__ F, int C, MeshGeom g, T *__restrict__ mesh) {
    constexpr int WS = RecordWidth<T, P>::value;
    constexpr int XS = 32 / CGP;
    constexpr int CC = CGP * NS;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *acc = reinterpret_cast<T *>(smem_raw);
    __shared__ T wl[kWarps][3][P];
    __shared__ int ll[kWarps][3][P];
    __shared__ int src[3][kMaxSrc];
    __shared__ int nsrc[3];
    __shared__ int seg_beg[kMaxSrc * kMaxSrc * kMaxSrc];
    __shared__ int seg_pre[kMaxSrc * kMaxSrc * kMaxSrc + 1];
    __shared__ int nseg;

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int tile = blockIdx.x;
    const int c0 = blockIdx.y * CC;
    const int ncomp = min(CC, C - c0);
    const int ti[3] = {tile % g.ntx, (tile / g.ntx) % g.nty, tile / (g.ntx * g.nty)};
    const int te[3] = {g.tx, g.ty, g.tz};
    const int org[3] = {ti[0] * g.tx, ti[1] * g.ty, ti[2] * g.tz};
    const int ext[3] = {min(g.tx, g.K - org[0]), min(g.ty, g.K - org[1]), min(g.tz, g.K - org[2])};
    const int npts = g.tx * g.ty * g.tz;

    for (int q = threadIdx.x; q < npts * CC; q += kThreads) acc[q] = T(0);

    // tiles whose cells can hold a stencil start reaching this tile, per axis
    if (threadIdx.x < 3) {
        const int a = threadIdx.x;
        int cell = pmod(org[a] - (P - 1), g.K);
        int remaining = min(ext[a] + P - 1, g.K);
        int cnt = 0;
        while (remaining > 0 && cnt < kMaxSrc) {
            int tl = cell / te[a];
            bool dup = false;
            for (int k = 0; k < cnt; k++) dup |= (src[a][k] == tl);
            if (!dup) src[a][cnt++] = tl;
            int end = min((tl + 1) * te[a], g.K);
            remaining -= end - cell;
            cell = end % g.K;
        }
        nsrc[a] = cnt;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int k = 0, pre = 0;
        for (int c = 0; c < nsrc[2]; c++)
            for (int b = 0; b < nsrc[1]; b++)
                for (int a = 0; a < nsrc[0]; a++) {
                    int id = (src[2][c] * g.nty + src[1][b]) * g.ntx + src[0][a];
                    int beg = tile_off[id], len = tile_off[id + 1] - beg;
                    seg_beg[k] = beg;
                    seg_pre[k] = pre;
                    pre += len;
                    k++;
                }
        seg_pre[k] = pre;
        nseg = k;
    }
    __syncthreads();

    const int total = seg_pre[nseg];
    const int xs = lane / CGP, cl = lane % CGP;
    const int axis = lane / P, jj = lane - (lane / P) * P;
    int seg = 0;
    for (int q = warp; q < total; q += kWarps) {
        while (q >= seg_pre[seg + 1]) seg++;
        const int s = seg_beg[seg] + (q - seg_pre[seg]);
        const T wreg = lane < 3 * P ? rec_w[(size_t)s * WS + lane] : T(0);
        int st[3];
        unpack_start(rec_start[s], st[0], st[1], st[2]);
        const int idx = rec_idx[s];
        bool valid = false;
        int l = 0;
        if (lane < 3 * P) {
            const int sa = axis == 0 ? st[0] : (axis == 1 ? st[1] : st[2]);
            const int oa = axis == 0 ? org[0] : (axis == 1 ? org[1] : org[2]);
            const int ea = axis == 0 ? ext[0] : (axis == 1 ? ext[1] : ext[2]);
            int gc = sa + jj;
            if (gc >= g.K) gc -= g.K;
            l = gc - oa;
            valid = (unsigned)l < (unsigned)ea;
        }
        const unsigned m = __ballot_sync(0xffffffffu, valid);
        const unsigned pm = (1u << P) - 1u;
        const int nx = __popc(m & pm), ny = __popc((m >> P) & pm), nz = __popc((m >> (2 * P)) & pm);
        if (nx == 0 || ny == 0 || nz == 0) continue;  // warp-uniform
        if (valid) {
            int posn = __popc((m >> (axis * P)) & ((1u << jj) - 1u));
            wl[warp][axis][posn] = wreg;
            ll[warp][axis][posn] = l;
        }
        T fv[NS];
#pragma unroll
        for (int sl = 0; sl < NS; sl++) {
            int c = sl * CGP + cl;
            fv[sl] = c < ncomp ? F[(size_t)idx * C + c0 + c] : T(0);
        }
        __syncwarp();
        for (int iz = 0; iz < nz; iz++) {
            const T wz = wl[warp][2][iz];
            const int lz = ll[warp][2][iz];
            for (int iy = 0; iy < ny; iy++) {
                const T wzy = wz * wl[warp][1][iy];
                const int rowbase = (lz * g.ty + ll[warp][1][iy]) * g.tx;
                for (int ix = xs; ix < nx; ix += XS) {
                    const T w = wzy * wl[warp][0][ix];
                    T *a = acc + (size_t)(rowbase + ll[warp][0][ix]) * CC + cl;
#pragma unroll
                    for (int sl = 0; sl < NS; sl++)
                        if (sl * CGP + cl < ncomp) atomicAdd(a + sl * CGP, w * fv[sl]);
                }
            }
        }
        __syncwarp();
    }
    __syncthreads();

    // flush: each (point, component) of the tile written once, C-contiguous rows
    const int nvals = ext[0] * ext[1] * ext[2] * ncomp;
    for (int q = threadIdx.x; q < nvals; q += kThreads) {
        const int c = q % ncomp;
        const int pt = q / ncomp;
        const int x = pt % ext[0], y = (pt / ext[0]) % ext[1], z = pt / (ext[0] * ext[1]);
        const size_t gi = ((size_t)(org[2] + z) * g.K + (org[1] + y)) * g.K + (org[0] + x);
        mesh[gi * C + c0 + c] = acc[((z * g.ty + y) * g.tx + x) * CC + c];
    }
}

template <typename T, int P, int CGP, int NS>
cudaError_t launch_spread_t(const int *tile_off, const int *rec_idx, const uint32_t *rec_start,
                            const T *rec_w, const T *F, int C, const MeshGeom &g, T *mesh,
                            cudaStream_t s) {
    constexpr int CC = CGP * NS;
    size_t smem = (size_t)g.tx * g.ty * g.tz * CC * sizeof(T);
    auto kern = k_spread<T, P, CGP, NS>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    dim3 grid(g.ntx * g.nty * g.ntz, (C + CC - 1) / CC);
    kern<<<grid, kThreads, smem, s>>>(tile_off, rec_idx, rec_start, rec_w, F, C, g, mesh);
    return cudaGetLastError();
}

template <typename T, int P>
cudaError_t dispatch_split(const int *tile_off, const int *rec_idx, const uint32_t *rec_start,
                           const T *rec_w, const T *F, int C, const MeshGeom &g, T *mesh,
                           cudaStream_t s) {
    const int max_cc = (int)(kSpreadSmemCap / ((size_t)g.tx * g.ty * g.tz * sizeof(T)));
    CompSplit cs = choose_comp_split(C, max_cc);
#define SPME_SPREAD_CASE(CG, N)                                                          \
    if (cs.cgp == CG && cs.ns == N)                                                      \
        return launch_spread_t<T, P, CG, N>(tile_off, rec_idx, rec_start, rec_w, F, C, g, \
                                            mesh, s);
    SPME_SPREAD_CASE(4, 1)
    SPME_SPREAD_CASE(8, 1)
    SPME_SPREAD_CASE(16, 1)
    SPME_SPREAD_CASE(4, 3)
    SPME_SPREAD_CASE(8, 3)
    SPME_SPREAD_CASE(16, 3)
#undef SPME_SPREAD_CASE
    return cudaErrorInvalidValue;
}

}  // namespace

CompSplit choose_comp_split(int C, int max_cc) {
    // lanes per component group x groups per CTA; minimise idle lanes, then
    // prefer wider groups (fewer x-slots to iterate).
    static const CompSplit opts[] = {{16, 3}, {8, 3}, {4, 3}, {16, 1}, {8, 1}, {4, 1}};
    CompSplit best = {4, 1};
    double best_eff = -1.0;
    for (const CompSplit &o : opts) {
        int cc = o.cgp * o.ns;
        if (cc > max_cc && cc > 4) continue;
        int passes = (C + cc - 1) / cc;
        double eff = (double)C / (double)(passes * cc);
        // a CTA pass re-reads every source particle; penalise extra passes
        double score = eff - 0.05 * (passes - 1);
        if (score > best_eff + 1e-9) {
            best_eff = score;
            best = o;
        }
    }
    return best;
}

size_t spread_smem_bytes(const MeshGeom &g, size_t elem, CompSplit cs) {
    return (size_t)g.tx * g.ty * g.tz * cs.cgp * cs.ns * elem;
}

template <typename T>
cudaError_t launch_spread(const int *tile_off, const int *rec_idx, const uint32_t *rec_start,
                          const T *rec_w, const T *F, int C, const MeshGeom &g, T *mesh,
                          cudaStream_t s) {
    switch (g.p) {
        case 4: return dispatch_split<T, 4>(tile_off, rec_idx, rec_start, rec_w, F, C, g, mesh, s);
        case 6: return dispatch_split<T, 6>(tile_off, rec_idx, rec_start, rec_w, F, C, g, mesh, s);
        case 8: return dispatch_split<T, 8>(tile_off, rec_idx, rec_start, rec_w, F, C, g, mesh, s);
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
