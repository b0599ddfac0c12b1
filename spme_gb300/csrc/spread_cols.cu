// Spread of 3R force components onto the K^3 mesh, column-gather form
// (restates old-version/spme_kernel.c:231-312: grid[c][ind] += P * f_c).
//
// Every mesh point receives ~p^3 rho contributions (rho particles per mesh
// cell), so the useful work per point is small and any scheme that lets a
// thread visit particles that do not cover its point wastes most of its
// arithmetic.  Here:
//   * particles are counting-sorted by their stencil-start cell in (y, x, z)
//     order, z fastest: the particles whose stencil starts in start column
//     (sy, sx) and in a z range are one contiguous run, found through the
//     start-cell offsets;
//   * a warp owns two neighbouring x columns of one y row and TZ planes; half
//     warp h holds column x0 + h, its 16 lanes hold up to 16 CPL force
//     components (c = c0 + lane + 16 k) and the TZ planes of those components
//     in registers;
//   * the warp walks the p (p + 1) start columns that reach its column pair and
//     their z runs, so every particle it visits covers at least one of its two
//     columns (a half whose column is missed multiplies by a zero weight);
//   * the particle's z offset relative to the tile selects, through a
//     warp-uniform jump, straight-line code with compile-time plane indices;
//   * the block's columns are transposed through shared memory and written as
//     whole mesh rows (coalesced), once: no zeroing, no atomics.
// Mesh layout: component-major mesh[c][z][y][x] (the cuFFT batch layout).
#include "kernels.h"

namespace spme {

namespace {

template <typename T> struct V16;
template <> struct V16<float> { using type = float4; };
template <> struct V16<double> { using type = double2; };

// p weights from a 16-byte aligned address, global or shared (vector loads
// where they fit).
template <typename T, int P>
__device__ __forceinline__ void load_weights(const T *__restrict__ src, T (&w)[P]) {
    constexpr int VW = 16 / (int)sizeof(T);
    constexpr int NV = P / VW;
    using V = typename V16<T>::type;
#pragma unroll
    for (int v = 0; v < NV; v++) {
        const V q = reinterpret_cast<const V *>(src)[v];
        if constexpr (VW == 4) {
            w[4 * v] = q.x;
            w[4 * v + 1] = q.y;
            w[4 * v + 2] = q.z;
            w[4 * v + 3] = q.w;
        } else {
            w[2 * v] = q.x;
            w[2 * v + 1] = q.y;
        }
    }
#pragma unroll
    for (int j = NV * VW; j < P; j++) w[j] = src[j];
}

// acc[D + j] += wt[j] f for the planes D + j inside [0, TZ) (wt[j] = w_x w_y w_z[j]).
template <typename T, int P, int CPL, int TZ, int D>
__device__ __forceinline__ void add_planes(T (&acc)[TZ][CPL], const T (&wt)[P],
                                           const T (&f)[CPL]) {
#pragma unroll
    for (int j = 0; j < P; j++) {
        constexpr int lo = D < 0 ? -D : 0;
        if (j >= lo && D + j < TZ) {
#pragma unroll
            for (int k = 0; k < CPL; k++) acc[D + j][k] += wt[j] * f[k];
        }
    }
}

// Per-warp shared scratch: the warp's start-column table (z runs and visit
// prefix) and one batch of 32 staged particles.
template <typename T, int P>
struct WarpScratch {
    static constexpr int NQ = P * (P + 1);
    static constexpr int PW = (P * (int)sizeof(T) + 15) / 16 * 16 / (int)sizeof(T);  // padded P
    // staged visit: w_x w_y w_z[j] for the pair's two columns (16-byte rows), then
    // (z offset, row of Fs)
    __align__(16) T wt[32][2][PW];
    int2 dz_row[32];  // (z offset, force-row offset s C)
    int begA[NQ], nA[NQ], begB[NQ];
    int pre[NQ + 1];
};

template <typename T, int P, int CPL, int TZ, int NW>
__global__ void __launch_bounds__(NW * 32, (sizeof(T) == 4 ? 3 : 1))
k_spread_cols(const int *__restrict__ soff, const uint32_t *__restrict__ rec_start,
              const T *__restrict__ rec_w, const T *__restrict__ Fs, int C, int K, int nzt,
              T *__restrict__ mesh) {
    constexpr int WS = RecordWidth<T, P>::value;
    constexpr int XT = 2 * NW;          // columns per block
    constexpr int CC = 16 * CPL;        // components per block
    constexpr int NX = P + 1;           // start columns per column pair (x)
    constexpr int NQ = P * NX;          // start columns per column pair (x and y)
    // shared stride per component, padded so the two half-warps' column stores fall
    // on different banks (even / odd words in FP32)
    constexpr int ROW = TZ * XT + (sizeof(T) == 4 ? 2 : 1);
    static_assert(-(P - 1) >= -7 && TZ <= 16, "jump table covers offsets -7 .. 15");
    extern __shared__ __align__(16) unsigned char sp_raw[];
    T *tsm = reinterpret_cast<T *>(sp_raw);  // [CC][ROW] transpose buffer
    const size_t tsm_bytes = ((size_t)CC * ROW * sizeof(T) + 15) & ~(size_t)15;

    const int x0 = blockIdx.x * XT;
    const int y = blockIdx.y;
    const int zt = blockIdx.z % nzt, chunk = blockIdx.z / nzt;
    const int z0 = zt * TZ;
    const int ext = min(TZ, K - z0);
    const int cb = chunk * CC;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int half = lane >> 4, l16 = lane & 15;
    const int xa = x0 + 2 * warp;  // first column of the warp's pair
    WarpScratch<T, P> &ws = reinterpret_cast<WarpScratch<T, P> *>(sp_raw + tsm_bytes)[warp];

    T acc[TZ][CPL];
#pragma unroll
    for (int z = 0; z < TZ; z++)
#pragma unroll
        for (int k = 0; k < CPL; k++) acc[z][k] = T(0);
    // this lane's components: Fs + row offset + 16 k, valid where c < C
    const T *fbase = Fs + cb + l16;
    bool cval[CPL];
#pragma unroll
    for (int k = 0; k < CPL; k++) cval[k] = cb + l16 + 16 * k < C;

    if (xa < K) {
        // start-column table: z runs of start cells that reach [z0, z0 + ext),
        // part A [max(lo, 0), hi) and part B [lo + K, K) when lo < 0
        const int lo = z0 - (P - 1), hi = z0 + ext;
        int run = 0;
        for (int qb = 0; qb < NQ; qb += 32) {
            const int q = qb + lane;
            int cnt = 0;
            if (q < NQ) {
                const int ty = q / NX, tx = q - ty * NX;
                const int sy = pmod(y - (P - 1) + ty, K), sx = pmod(xa - (P - 1) + tx, K);
                const size_t base = ((size_t)sy * K + sx) * K;
                const int bA = __ldg(soff + base + max(lo, 0));
                const int eA = __ldg(soff + base + hi);
                int bB = 0, eB = 0;
                if (lo < 0) {
                    bB = __ldg(soff + base + lo + K);
                    eB = __ldg(soff + base + K);
                }
                ws.begA[q] = bA;
                ws.nA[q] = eA - bA;
                ws.begB[q] = bB;
                cnt = (eA - bA) + (eB - bB);
            }
            int inc = cnt;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int t = __shfl_up_sync(0xffffffffu, inc, o);
                if (lane >= o) inc += t;
            }
            if (q < NQ) ws.pre[q] = run + inc - cnt;
            run += __shfl_sync(0xffffffffu, inc, 31);
        }
        if (lane == 0) ws.pre[NQ] = run;
        __syncwarp();
        const int M = run;  // visits of this warp

        for (int vb = 0; vb < M; vb += 32) {
            const int nb = min(32, M - vb);
            // stage: lane t fetches visit vb + t
            if (lane < nb) {
                const int v = vb + lane;
                int a = 0, b = NQ;  // pre[a] <= v < pre[b]
                while (b - a > 1) {
                    const int m = (a + b) >> 1;
                    if (ws.pre[m] <= v) a = m; else b = m;
                }
                const int r = v - ws.pre[a];
                const bool partB = r >= ws.nA[a];
                const int s = partB ? ws.begB[a] + (r - ws.nA[a]) : ws.begA[a] + r;
                int sx, sy, sz;
                unpack_start(__ldg(rec_start + s), sx, sy, sz);
                int ox = xa - sx;
                if (ox < 0) ox += K;
                int oy = y - sy;
                if (oy < 0) oy += K;
                const T *rw = rec_w + (size_t)s * WS;
                const T wy = __ldg(rw + P + oy);
                // column xa covered when ox < P, column xa + 1 when ox + 1 < P
                // (or ox = K - 1: the stencil starts at xa + 1)
                const int ox1 = ox + 1 == K ? 0 : ox + 1;
                const T w0 = ox < P ? wy * __ldg(rw + ox) : T(0);
                const T w1 = (ox1 < P && xa + 1 < K) ? wy * __ldg(rw + ox1) : T(0);
                // dz in [-(P-1), ext); the visit's force row as an offset (s C < 2^31)
                ws.dz_row[lane] = make_int2(sz - (partB ? z0 + K : z0), s * C);
                T wz[P];
                load_weights<T, P>(rw + 2 * P, wz);
                // 16-byte stores (scalar stores at this lane stride conflict 16-way)
                constexpr int PW = WarpScratch<T, P>::PW, VW = 16 / (int)sizeof(T);
                using V = typename V16<T>::type;
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    const T w = h ? w1 : w0;
                    T row[PW];
#pragma unroll
                    for (int j = 0; j < PW; j++) row[j] = j < P ? w * wz[j] : T(0);
#pragma unroll
                    for (int v = 0; v < PW / VW; v++) {
                        V q;
                        if constexpr (VW == 4) {
                            q.x = row[4 * v];
                            q.y = row[4 * v + 1];
                            q.z = row[4 * v + 2];
                            q.w = row[4 * v + 3];
                        } else {
                            q.x = row[2 * v];
                            q.y = row[2 * v + 1];
                        }
                        reinterpret_cast<V *>(&ws.wt[lane][h][0])[v] = q;
                    }
                }
            }
            __syncwarp();
            // accumulate the batch (force row of the next visit prefetched)
            T fn[CPL];
            {
                const T *row = fbase + ws.dz_row[0].y;
#pragma unroll
                for (int k = 0; k < CPL; k++) fn[k] = cval[k] ? __ldg(row + 16 * k) : T(0);
            }
            for (int j = 0; j < nb; j++) {
                T f[CPL];
#pragma unroll
                for (int k = 0; k < CPL; k++) f[k] = fn[k];
                const int2 dr = ws.dz_row[j];
                if (j + 1 < nb) {
                    const T *row = fbase + ws.dz_row[j + 1].y;
#pragma unroll
                    for (int k = 0; k < CPL; k++) fn[k] = cval[k] ? __ldg(row + 16 * k) : T(0);
                }
                T wt[P];
                load_weights<T, P>(&ws.wt[j][half][0], wt);
                switch (dr.x) {
#define SPME_SPC(DD)                                                                      \
    case DD:                                                                              \
        if constexpr (DD >= -(P - 1) && DD < TZ) add_planes<T, P, CPL, TZ, DD>(acc, wt, f); \
        break;
                    SPME_SPC(-7) SPME_SPC(-6) SPME_SPC(-5) SPME_SPC(-4) SPME_SPC(-3)
                    SPME_SPC(-2) SPME_SPC(-1) SPME_SPC(0) SPME_SPC(1) SPME_SPC(2)
                    SPME_SPC(3) SPME_SPC(4) SPME_SPC(5) SPME_SPC(6) SPME_SPC(7)
                    SPME_SPC(8) SPME_SPC(9) SPME_SPC(10) SPME_SPC(11) SPME_SPC(12)
                    SPME_SPC(13) SPME_SPC(14) SPME_SPC(15)
#undef SPME_SPC
                    default: break;
                }
            }
            __syncwarp();
        }
    }

    // transpose through shared memory: tsm[c][z][x]
    const int xl = 2 * warp + half;
#pragma unroll
    for (int z = 0; z < TZ; z++)
#pragma unroll
        for (int k = 0; k < CPL; k++) tsm[(size_t)(l16 + 16 * k) * ROW + z * XT + xl] = acc[z][k];
    __syncthreads();
    // whole rows of XT columns per (component, plane): each thread keeps one
    // (plane, column) slot and walks the components with pointer increments
    static_assert((NW * 32) % (XT * TZ) == 0 || (XT * TZ) % (NW * 32) == 0, "row split");
    constexpr int SLOTS = XT * TZ;                    // (plane, column) slots of a component
    constexpr int CSTEP = (NW * 32) >= SLOTS ? (NW * 32) / SLOTS : 1;  // components per sweep
    const size_t K3 = (size_t)K * K * K;
    const int nc = min(CC, C - cb);
    for (int slot = threadIdx.x % SLOTS; slot < SLOTS; slot += NW * 32) {
        const int z = slot / XT, x = slot - z * XT;
        if (z >= ext || x0 + x >= K) continue;
        T *out = mesh + (size_t)cb * K3 + ((size_t)(z0 + z) * K + y) * K + x0 + x;
        const T *src = tsm + z * XT + x;
        for (int c = threadIdx.x / SLOTS; c < nc; c += CSTEP)
            out[(size_t)c * K3] = src[(size_t)c * ROW];
    }
}

template <typename T, int P, int CPL>
cudaError_t launch_cols(const int *soff, const uint32_t *rec_start, const T *rec_w, const T *Fs,
                        int C, const MeshGeom &g, T *mesh, cudaStream_t s) {
    constexpr int NW = 8;
    constexpr int TZ = sizeof(T) == 4 ? 16 : 8;
    constexpr int XT = 2 * NW, CC = 16 * CPL;
    const int K = g.K;
    const int nzt = (K + TZ - 1) / TZ, nchunk = (C + CC - 1) / CC;
    const size_t smem = (((size_t)CC * (TZ * XT + (sizeof(T) == 4 ? 2 : 1)) * sizeof(T) + 15) &
                         ~(size_t)15) +
                        NW * sizeof(WarpScratch<T, P>);
    auto kern = k_spread_cols<T, P, CPL, TZ, NW>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    dim3 grid((K + XT - 1) / XT, K, nzt * nchunk);
    kern<<<grid, NW * 32, smem, s>>>(soff, rec_start, rec_w, Fs, C, K, nzt, mesh);
    return cudaGetLastError();
}

template <typename T, int P>
cudaError_t dispatch_cpl(const int *soff, const uint32_t *rec_start, const T *rec_w, const T *Fs,
                         int C, const MeshGeom &g, T *mesh, cudaStream_t s) {
    // components per lane: the smallest CPL with 16 CPL >= C, at most 3
    if (C <= 16) return launch_cols<T, P, 1>(soff, rec_start, rec_w, Fs, C, g, mesh, s);
    if (C <= 32) return launch_cols<T, P, 2>(soff, rec_start, rec_w, Fs, C, g, mesh, s);
    return launch_cols<T, P, 3>(soff, rec_start, rec_w, Fs, C, g, mesh, s);
}

}  // namespace

// The z runs of one tile must not wrap onto themselves (TZ + p - 1 <= K) and
// the p + 1 start columns of a column pair must be distinct: K >= 32 covers
// both for p <= 8.  Any number of components (the cost is per visit: below 16
// components lanes idle, but the tile kernel's wasted visits cost more).
bool spread_cols_ok(int K, int C, size_t elem) {
    (void)elem;
    return K >= 32 && K <= 1024 && C >= 1;
}

template <typename T>
cudaError_t launch_spread_cols(const int *start_off, const uint32_t *rec_start, const T *rec_w,
                               const T *Fs, int C, const MeshGeom &g, T *mesh, cudaStream_t s) {
    if (!spread_cols_ok(g.K, C, sizeof(T))) return cudaErrorInvalidValue;
    switch (g.p) {
        case 4: return dispatch_cpl<T, 4>(start_off, rec_start, rec_w, Fs, C, g, mesh, s);
        case 6: return dispatch_cpl<T, 6>(start_off, rec_start, rec_w, Fs, C, g, mesh, s);
        case 8: return dispatch_cpl<T, 8>(start_off, rec_start, rec_w, Fs, C, g, mesh, s);
        default: return cudaErrorInvalidValue;
    }
}

template cudaError_t launch_spread_cols<float>(const int *, const uint32_t *, const float *,
                                               const float *, int, const MeshGeom &, float *,
                                               cudaStream_t);
template cudaError_t launch_spread_cols<double>(const int *, const uint32_t *, const double *,
                                                const double *, int, const MeshGeom &, double *,
                                                cudaStream_t);

}  // namespace spme
