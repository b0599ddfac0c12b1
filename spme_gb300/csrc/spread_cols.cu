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
//   * visits are staged in batches (one lane per visit: record, weights of
//     both columns, force-row offset) and ranked by their z offset relative to
//     the tile (a 5-bit radix rank from ballots), so the accumulation walks the
//     offsets in a compile-time sequence, each with straight-line code for its
//     planes (FP32: one body per pair of offsets): no per-visit dispatch;
//   * FP32 accumulators are pairs of planes, updated with the packed
//     two-lane FMA (fma.rn.f32x2, sm_100 and later): a visit whose first plane
//     is odd uses weights staged one plane later (0, w_0 .. w_{p-1}, 0), one
//     whose first plane is even (w_0 .. w_{p-1}, 0, 0);
//   * force rows are read as one vector per lane: the rows are gathered per
//     pass into a padded layout where each lane's CPL components are
//     contiguous (spread_cols_row_width);
//   * the block's columns are transposed through shared memory and written as
//     whole mesh rows (coalesced), once: no zeroing, no atomics.
// Mesh layout: component-major mesh[c][z][y][x] (the cuFFT batch layout).
#include <algorithm>
#include <utility>

#include "kernels.h"

namespace spme {

namespace {

// fn(std::integral_constant<int, i>) for i = 0 .. N-1, unrolled at compile time.
template <typename Fn, int... Is>
__device__ __forceinline__ void static_for_impl(Fn &&fn, std::integer_sequence<int, Is...>) {
    (fn(std::integral_constant<int, Is>{}), ...);
}
template <int N, typename Fn>
__device__ __forceinline__ void static_for(Fn &&fn) {
    static_for_impl(fn, std::make_integer_sequence<int, N>{});
}

// Asynchronous global -> shared copies (cp.async, completion tracked per thread).
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void cp_async16(void *dst, const void *src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)), "l"(src)
                 : "memory");
}
template <int B>
__device__ __forceinline__ void cp_async_small(void *dst, const void *src) {
    static_assert(B == 4 || B == 8, "4 or 8 bytes");
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2;" ::"r"(smem_u32(dst)), "l"(src),
                 "n"(B)
                 : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
    asm volatile("cp.async.wait_all;" ::: "memory");
}

template <typename T> struct V16;
template <> struct V16<float> { using type = float4; };
template <> struct V16<double> { using type = double2; };

// Components per lane for C components (chunks of 16 CPL components per block).
__host__ __device__ constexpr int cols_cpl(int C) { return C <= 16 ? 1 : (C <= 32 ? 2 : 3); }
// Padded components per lane in the gathered force rows.
__host__ __device__ constexpr int cols_pcpl(int cpl) { return cpl == 3 ? 4 : cpl; }

// n values from a 16-byte aligned address, global or shared (vector loads
// where they fit).
template <typename T, int NV>
__device__ __forceinline__ void load_vec(const T *__restrict__ src, T (&w)[NV]) {
    constexpr int VW = 16 / (int)sizeof(T);
    constexpr int NQ = NV / VW;
    using V = typename V16<T>::type;
#pragma unroll
    for (int v = 0; v < NQ; v++) {
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
    for (int j = NQ * VW; j < NV; j++) w[j] = src[j];
}

// Staged weight row length: FP32 rows hold p + 2 values (the first plane of an
// odd offset shifted by one, so pairs of planes line up), FP64 rows p; both
// padded to 16 bytes.
template <typename T, int P>
struct WRow {
    static constexpr int raw = sizeof(T) == 4 ? P + 2 : P;
    static constexpr int per16 = 16 / (int)sizeof(T);
    static constexpr int value = (raw + per16 - 1) / per16 * per16;
};

// FP32, one body for the offsets 2 M0 and 2 M0 + 1: P/2 + 1 pairs from pair M0
// (the staged weights put an odd offset's planes one slot later; an even
// offset's last pair is zero).
template <int P, int CPL, int TZ, int M0, int NW>
__device__ __forceinline__ void add_pair_run(float2 (&acc)[TZ / 2][CPL], const float (&w)[NW],
                                             const float (&f)[CPL]) {
    static_assert(NW >= P + 2, "staged row holds P + 2 weights");
    float2 fd[CPL];
#pragma unroll
    for (int k = 0; k < CPL; k++) fd[k] = make_float2(f[k], f[k]);
#pragma unroll
    for (int i = 0; i < P / 2 + 1; i++) {
        const int m = M0 + i;
        if (m >= 0 && m < TZ / 2) {
            const float2 wp = make_float2(w[2 * i], w[2 * i + 1]);
#pragma unroll
            for (int k = 0; k < CPL; k++) acc[m][k] = __ffma2_rn(wp, fd[k], acc[m][k]);
        }
    }
}

// FP64: acc[D + j][k] += w[j] f_k for the planes D + j inside [0, TZ).
template <int P, int CPL, int TZ, int D, int NW>
__device__ __forceinline__ void add_planes(double (&acc)[TZ][CPL], const double (&w)[NW],
                                           const double (&f)[CPL]) {
#pragma unroll
    for (int j = 0; j < P; j++) {
        if (D + j >= 0 && D + j < TZ) {
#pragma unroll
            for (int k = 0; k < CPL; k++) acc[D + j][k] = fma(w[j], f[k], acc[D + j][k]);
        }
    }
}

template <typename T, int TZ, int CPL> struct AccType;
template <int TZ, int CPL> struct AccType<float, TZ, CPL> { using type = float2[TZ / 2][CPL]; };
template <int TZ, int CPL> struct AccType<double, TZ, CPL> { using type = double[TZ][CPL]; };

// Per-warp shared scratch: the warp's start-column table (z runs and visit
// prefix) and one batch of 32 staged visits in offset order.
template <typename T, int P>
struct WarpScratch {
    static constexpr int NQ = P * (P + 1);
    static constexpr int WR = WRow<T, P>::value;
    __align__(16) T wt[32][2][WR];  // weights of the pair's two columns
    int row[32];                    // force-row offset (elements) of the visit
    int begA[NQ], nA[NQ], begB[NQ];
    int pre[NQ + 1];
};

// One block's work: columns [bx XT, bx XT + XT) of row y = by, z tile and
// component chunk bz (nzt z tiles per chunk).  Runs as the body of the
// single-system kernel and of the batched one.
template <typename T, int P, int CPL, int TZ, int NW>
__device__ __forceinline__ void spread_cols_body(const SpreadColsArgs<T> &A, int bx, int by,
                                                 int bz) {
    constexpr bool F32 = sizeof(T) == 4;
    constexpr int WR = WRow<T, P>::value;
    const int *__restrict__ soff = A.soff;
    const uint32_t *__restrict__ rec_start = A.rec_start;
    const T *__restrict__ rec_w = A.rec_w;
    const T *__restrict__ Fs = A.Fs;
    T *__restrict__ mesh = A.mesh;
    const int C = A.C, RW = A.RW, K = A.K, nzt = A.nzt, WS = A.ws;
    constexpr int PC = cols_pcpl(CPL);  // padded components per lane in a force row
    constexpr int XT = 2 * NW;          // columns per block
    constexpr int CC = 16 * CPL;        // components per block
    constexpr int NX = P + 1;           // start columns per column pair (x)
    constexpr int NQ = P * NX;          // start columns per column pair (x and y)
    constexpr int ND = TZ + P - 1;      // z offsets -(P-1) .. TZ-1
    static_assert(ND <= 31 && TZ % 2 == 0, "offsets rank in 5 bits; plane pairs");
    // shared stride per component, padded so the two half-warps' column stores fall
    // on different banks (even / odd words in FP32)
    constexpr int ROW = TZ * XT + (F32 ? 2 : 1);
    // a staged force row (this block's chunk: 16 lanes x PC values) and the visits
    // per batch: the batch's rows share the transpose buffer, NB rows per warp
    constexpr int LR = 16 * PC;
    constexpr int NB = (CC * ROW) / (NW * LR) < 32 ? (CC * ROW) / (NW * LR) : 32;
    static_assert(NB >= 8, "staged batch");
    extern __shared__ __align__(16) unsigned char sp_raw[];
    T *tsm = reinterpret_cast<T *>(sp_raw);  // [CC][ROW] transpose buffer
    const size_t tsm_bytes = ((size_t)CC * ROW * sizeof(T) + 15) & ~(size_t)15;

    const int x0 = bx * XT;
    const int y = by;
    const int zt = bz % nzt, chunk = bz / nzt;
    const int z0 = zt * TZ;
    const int ext = min(TZ, K - z0);
    const int cb = chunk * CC;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int half = lane >> 4, l16 = lane & 15;
    const int xa = x0 + 2 * warp;  // first column of the warp's pair
    WarpScratch<T, P> &ws = reinterpret_cast<WarpScratch<T, P> *>(sp_raw + tsm_bytes)[warp];

    typename AccType<T, TZ, CPL>::type acc;
    if constexpr (F32) {
#pragma unroll
        for (int m = 0; m < TZ / 2; m++)
#pragma unroll
            for (int k = 0; k < CPL; k++) acc[m][k] = make_float2(0.f, 0.f);
    } else {
#pragma unroll
        for (int z = 0; z < TZ; z++)
#pragma unroll
            for (int k = 0; k < CPL; k++) acc[z][k] = 0.0;
    }
    // the warp's staged force rows of one batch (in the transpose buffer, free
    // until the write-out); this lane's components of row j at j LR + l16 PC
    // (CPL = 1: component l16, present when l16 < C)
    T *fst = tsm + (size_t)warp * NB * LR;
    const bool lane_live = CPL > 1 || l16 < C;

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

        for (int vb = 0; vb < M; vb += NB) {
            const int nb = min(NB, M - vb);
            // stage: lane t fetches visit vb + t; dl = its z offset + P - 1 (31: none)
            int dl = 31, s = 0;
            uint32_t st = 0;
            if (lane < nb) {
                const int v = vb + lane;
                int a = 0, b = NQ;  // pre[a] <= v < pre[b]
                while (b - a > 1) {
                    const int m = (a + b) >> 1;
                    if (ws.pre[m] <= v) a = m; else b = m;
                }
                const int r = v - ws.pre[a];
                const bool partB = r >= ws.nA[a];
                s = partB ? ws.begB[a] + (r - ws.nA[a]) : ws.begA[a] + r;
                st = __ldg(rec_start + s);
                // dz in [-(P-1), ext)
                dl = (int)((st >> 20) & 1023u) - (partB ? z0 + K : z0) + (P - 1);
            }
            // rank by offset: lanes with a smaller offset, then equal offsets in lane order
            unsigned eq = 0xffffffffu;
            int lt = 0;
#pragma unroll
            for (int bit = 4; bit >= 0; bit--) {
                const bool one = (dl >> bit) & 1;
                const unsigned bm = __ballot_sync(0xffffffffu, one);
                if (one) {
                    lt += __popc(eq & ~bm);
                    eq &= bm;
                } else {
                    eq &= ~bm;
                }
            }
            const int pos = lt + __popc(eq & ((1u << lane) - 1u));
            if (lane < nb) {
                ws.row[pos] = s * RW;  // CPL = 1: RW = C
                int sx, sy, sz;
                unpack_start(st, sx, sy, sz);
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
                T wz[P];
                load_vec<T, P>(rw + 2 * P, wz);
                // weight rows of both columns (16-byte stores; scalar stores at this
                // lane stride conflict 16-way)
                constexpr int VW = 16 / (int)sizeof(T);
                using V = typename V16<T>::type;
                const int shift = F32 ? ((dl - (P - 1)) & 1) : 0;
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    const T w = h ? w1 : w0;
                    T row[WR];
#pragma unroll
                    for (int j = 0; j < WR; j++) {
                        // j - shift in [0, P): weight of plane j - shift of the stencil
                        const T a0 = (j < P) ? wz[j < P ? j : 0] : T(0);
                        const T a1 = (j >= 1 && j - 1 < P) ? wz[j >= 1 && j - 1 < P ? j - 1 : 0] : T(0);
                        row[j] = w * (shift ? a1 : a0);
                    }
#pragma unroll
                    for (int q = 0; q < WR / VW; q++) {
                        V qv;
                        if constexpr (VW == 4) {
                            qv.x = row[4 * q];
                            qv.y = row[4 * q + 1];
                            qv.z = row[4 * q + 2];
                            qv.w = row[4 * q + 3];
                        } else {
                            qv.x = row[2 * q];
                            qv.y = row[2 * q + 1];
                        }
                        reinterpret_cast<V *>(&ws.wt[pos][h][0])[q] = qv;
                    }
                }
            }
            __syncwarp();
            // the batch's force rows, in offset order, into shared memory: one
            // round trip per batch instead of one per visit
            if constexpr (CPL > 1) {
                constexpr int VW = 16 / (int)sizeof(T);
                constexpr int NCH = LR / VW;  // 16-byte pieces per row
                for (int t = lane; t < nb * NCH; t += 32) {
                    const int v = t / NCH, q = t - v * NCH;
                    cp_async16(fst + v * LR + q * VW, Fs + ws.row[v] + (size_t)chunk * LR + q * VW);
                }
            } else {
                for (int t = lane; t < nb * 16; t += 32) {
                    const int v = t >> 4, c = t & 15;
                    if (c < C) cp_async_small<(int)sizeof(T)>(fst + v * LR + c, Fs + ws.row[v] + c);
                }
            }
            cp_async_wait_all();
            __syncwarp();
            // accumulate in offset order
            auto visit_force = [&](int j, T (&f)[CPL]) {
                if constexpr (CPL > 1) {
                    T fv[PC];
                    load_vec<T, PC>(fst + j * LR + l16 * PC, fv);
#pragma unroll
                    for (int c = 0; c < CPL; c++) f[c] = fv[c];
                } else {
                    f[0] = lane_live ? fst[j * LR + l16] : T(0);
                }
            };
            int j = 0;
            if constexpr (F32) {
                // FP32: one bucket per first plane pair m0 = floor(offset / 2) (the
                // offsets 2 m0 and 2 m0 + 1 share one straight-line body of P/2 + 1
                // pairs; an even offset's last pair has zero weights)
                constexpr int NDP = TZ / 2 + P / 2;
                const int bl = (dl + 1) >> 1;  // m0 + P/2 (31: none)
                static_for<NDP>([&](auto bc) {
                    constexpr int M0 = decltype(bc)::value - P / 2;
                    const int cnt = __popc(__ballot_sync(0xffffffffu, bl == M0 + P / 2));
                    for (int k = 0; k < cnt; k++, j++) {
                        T f[CPL];
                        visit_force(j, f);
                        T wt[WR];
                        load_vec<T, WR>(&ws.wt[j][half][0], wt);
                        add_pair_run<P, CPL, TZ, M0, WR>(acc, wt, f);
                    }
                });
            } else {
                static_for<ND>([&](auto bc) {
                    constexpr int D = decltype(bc)::value - (P - 1);  // the bucket's z offset
                    const int cnt = __popc(__ballot_sync(0xffffffffu, dl == D + (P - 1)));
                    for (int k = 0; k < cnt; k++, j++) {
                        T f[CPL];
                        visit_force(j, f);
                        T wt[WR];
                        load_vec<T, WR>(&ws.wt[j][half][0], wt);
                        add_planes<P, CPL, TZ, D, WR>(acc, wt, f);
                    }
                });
            }
            __syncwarp();
        }
    }

    // transpose through shared memory: tsm[c][z][x] (after every warp of the
    // block is done with its staged force rows, which live in the same buffer)
    __syncthreads();
    const int xl = 2 * warp + half;
#pragma unroll
    for (int z = 0; z < TZ; z++)
#pragma unroll
        for (int k = 0; k < CPL; k++) {
            T v;
            if constexpr (F32) v = (z & 1) ? acc[z >> 1][k].y : acc[z >> 1][k].x;
            else v = acc[z][k];
            tsm[(size_t)(l16 + 16 * k) * ROW + z * XT + xl] = v;
        }
    __syncthreads();
    // whole rows of XT columns per (component, plane): each thread keeps one
    // (plane, column) slot and walks the components with pointer increments
    static_assert((NW * 32) % (XT * TZ) == 0 || (XT * TZ) % (NW * 32) == 0, "row split");
    constexpr int SLOTS = XT * TZ;                    // (plane, column) slots of a component
    constexpr int CSTEP = (NW * 32) >= SLOTS ? (NW * 32) / SLOTS : 1;  // components per sweep
    const size_t K3 = (size_t)K * K * K;
    const int nc = min(CC, C - cb);
    if constexpr (F32) {
        // even K: pairs of columns per thread (8-byte loads and stores; ROW is even)
        if ((K & 1) == 0) {
            constexpr int SL2 = XT * TZ / 2;  // (plane, column pair) slots of a component
            constexpr int CS2 = (NW * 32) >= SL2 ? (NW * 32) / SL2 : 1;
            static_assert(ROW % 2 == 0, "pair loads from the transpose buffer");
            for (int slot = threadIdx.x % SL2; slot < SL2; slot += NW * 32) {
                const int z = slot / (XT / 2), x = 2 * (slot - z * (XT / 2));
                if (z >= ext || x0 + x >= K) continue;  // K, x0 + x even: x0 + x + 1 < K
                float2 *out = reinterpret_cast<float2 *>(
                    mesh + (size_t)cb * K3 + ((size_t)(z0 + z) * K + y) * K + x0 + x);
                const float2 *src = reinterpret_cast<const float2 *>(tsm + z * XT + x);
                for (int c = threadIdx.x / SL2; c < nc; c += CS2)
                    out[(size_t)c * (K3 / 2)] = src[(size_t)c * (ROW / 2)];
            }
            return;
        }
    }
    for (int slot = threadIdx.x % SLOTS; slot < SLOTS; slot += NW * 32) {
        const int z = slot / XT, x = slot - z * XT;
        if (z >= ext || x0 + x >= K) continue;
        T *out = mesh + (size_t)cb * K3 + ((size_t)(z0 + z) * K + y) * K + x0 + x;
        const T *src = tsm + z * XT + x;
        for (int c = threadIdx.x / SLOTS; c < nc; c += CSTEP)
            out[(size_t)c * K3] = src[(size_t)c * ROW];
    }
}

template <typename T, int P, int CPL, int TZ, int NW>
__global__ void __launch_bounds__(NW * 32, (sizeof(T) == 4 ? 3 : 1))
k_spread_cols(SpreadColsArgs<T> A) {
    spread_cols_body<T, P, CPL, TZ, NW>(A, blockIdx.x, blockIdx.y, blockIdx.z);
}

// Many systems in one persistent launch: work item w (a block of one system)
// -> system k with prefix[k] <= w < prefix[k + 1]; the order p of each system
// selects the body.
template <typename T, int CPL, int TZ, int NW>
__global__ void __launch_bounds__(NW * 32, (sizeof(T) == 4 ? 3 : 1))
k_spread_cols_batch(const SpreadColsSys<T> *__restrict__ sys, const int *__restrict__ prefix,
                    int nsys, int total) {
    for (int w = blockIdx.x; w < total; w += gridDim.x) {
        const int k = batch_find(prefix, nsys, w);
        const SpreadColsSys<T> S = sys[k];
        const int local = w - prefix[k];
        const int bx = local % S.gx, rest = local / S.gx;
        const int by = rest % S.args.K, bz = rest / S.args.K;
        switch (S.p) {
            case 4: spread_cols_body<T, 4, CPL, TZ, NW>(S.args, bx, by, bz); break;
            case 6: spread_cols_body<T, 6, CPL, TZ, NW>(S.args, bx, by, bz); break;
            default: spread_cols_body<T, 8, CPL, TZ, NW>(S.args, bx, by, bz); break;
        }
        __syncthreads();  // shared memory is reused by the next work item
    }
}

// Fs[s][chunk*16*PC + l*PC + k] = F[idx[s]][chunk*16*CPL + l + 16 k] for k < CPL
// (0 where that component does not exist or k >= CPL); CPL = 1: Fs[s][c] = F[idx[s]][c].
template <typename T, int CPL>
__global__ void k_gather_cols_rows(const T *__restrict__ F, const int *__restrict__ idx, int n,
                                   int C, int RW, int nchunk, T *__restrict__ Fs) {
    // one thread per (slot, chunk, lane): the lane's CPL components (padded to PC)
    // as one vector store
    constexpr int PC = cols_pcpl(CPL);
    const size_t total = (size_t)n * nchunk * 16;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (size_t)gridDim.x * blockDim.x) {
        const int l = (int)(t & 15);
        const size_t sc = t >> 4;  // (slot, chunk)
        const size_t s = nchunk == 1 ? sc : sc / nchunk;
        const int chunk = (int)(sc - s * nchunk);
        const T *src = F + (size_t)__ldg(idx + s) * C;
        if constexpr (CPL == 1) {
            if (l < C) Fs[s * RW + l] = __ldg(src + l);
        } else {
            T v[PC];
#pragma unroll
            for (int k = 0; k < PC; k++) {
                const int c = chunk * 16 * CPL + l + 16 * k;
                v[k] = (k < CPL && c < C) ? __ldg(src + c) : T(0);
            }
            T *dst = Fs + s * RW + (size_t)chunk * 16 * PC + (size_t)l * PC;
            using V = typename V16<T>::type;  // 16 bytes: float4 or double2
            constexpr int VW = 16 / (int)sizeof(T);
            if constexpr (PC * sizeof(T) >= 16) {
#pragma unroll
                for (int q = 0; q < PC / VW; q++) {
                    V w;
                    if constexpr (VW == 4) {
                        w.x = v[4 * q];
                        w.y = v[4 * q + 1];
                        w.z = v[4 * q + 2];
                        w.w = v[4 * q + 3];
                    } else {
                        w.x = v[2 * q];
                        w.y = v[2 * q + 1];
                    }
                    reinterpret_cast<V *>(dst)[q] = w;
                }
            } else {
#pragma unroll
                for (int k = 0; k < PC; k++) dst[k] = v[k];
            }
        }
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
    SpreadColsArgs<T> A{soff, rec_start, rec_w, Fs, mesh, C, spread_cols_row_width(C), K, nzt,
                        RecordWidth<T, P>::value};
    kern<<<grid, NW * 32, smem, s>>>(A);
    return cudaGetLastError();
}

template <typename T, int CPL>
cudaError_t launch_cols_batch(const SpreadColsSys<T> *sys, const int *prefix, int nsys,
                              int total, cudaStream_t s) {
    constexpr int NW = 8;
    constexpr int TZ = sizeof(T) == 4 ? 16 : 8;
    constexpr int XT = 2 * NW, CC = 16 * CPL;
    const size_t smem = (((size_t)CC * (TZ * XT + (sizeof(T) == 4 ? 2 : 1)) * sizeof(T) + 15) &
                         ~(size_t)15) +
                        NW * sizeof(WarpScratch<T, 8>);  // the largest order's scratch
    auto kern = k_spread_cols_batch<T, CPL, TZ, NW>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, NW * 32, smem);
    const int grid = std::max(1, std::min(total, sms * std::max(per_sm, 1)));
    kern<<<grid, NW * 32, smem, s>>>(sys, prefix, nsys, total);
    return cudaGetLastError();
}

template <typename T, int P>
cudaError_t dispatch_cpl(const int *soff, const uint32_t *rec_start, const T *rec_w, const T *Fs,
                         int C, const MeshGeom &g, T *mesh, cudaStream_t s) {
    // components per lane: the smallest CPL with 16 CPL >= C, at most 3
    switch (cols_cpl(C)) {
        case 1: return launch_cols<T, P, 1>(soff, rec_start, rec_w, Fs, C, g, mesh, s);
        case 2: return launch_cols<T, P, 2>(soff, rec_start, rec_w, Fs, C, g, mesh, s);
        default: return launch_cols<T, P, 3>(soff, rec_start, rec_w, Fs, C, g, mesh, s);
    }
}

int blocks_for_rows(size_t total) {
    const size_t b = (total + 255) / 256;
    return (int)(b < 8192 ? (b > 0 ? b : 1) : 8192);
}

}  // namespace

// The z runs of one tile must not wrap onto themselves (TZ + p - 1 <= K, TZ =
// 16 planes in FP32, 8 in FP64) and the p + 1 start columns of a column pair
// must be distinct (K >= p + 1).  Any number of components (the cost is per
// visit: below 16 components lanes idle, but the tile kernel's wasted visits
// cost more).
bool spread_cols_ok(int K, int C, size_t elem, int p) {
    const int TZ = elem == 4 ? 16 : 8;
    return K >= TZ + p - 1 && K >= p + 1 && K <= 1024 && C >= 1;
}

int spread_cols_row_width(int C) {
    const int cpl = cols_cpl(C);
    if (cpl == 1) return C;
    const int nchunk = (C + 16 * cpl - 1) / (16 * cpl);
    return nchunk * 16 * cols_pcpl(cpl);
}

template <typename T>
void launch_gather_cols_rows(const T *F, const int *idx, int n, int C, T *Fs, cudaStream_t s) {
    const int RW = spread_cols_row_width(C);
    const int cpl = cols_cpl(C);
    const int nchunk = cpl == 1 ? 1 : RW / (16 * cols_pcpl(cpl));
    const size_t total = (size_t)n * nchunk * 16;  // threads: (slot, chunk, lane)
    if (n <= 0) return;
    switch (cpl) {
        case 1:
            k_gather_cols_rows<T, 1><<<blocks_for_rows(total), 256, 0, s>>>(F, idx, n, C, RW,
                                                                            nchunk, Fs);
            break;
        case 2:
            k_gather_cols_rows<T, 2><<<blocks_for_rows(total), 256, 0, s>>>(F, idx, n, C, RW,
                                                                            nchunk, Fs);
            break;
        default:
            k_gather_cols_rows<T, 3><<<blocks_for_rows(total), 256, 0, s>>>(F, idx, n, C, RW,
                                                                            nchunk, Fs);
            break;
    }
}

template <typename T>
cudaError_t launch_spread_cols(const int *start_off, const uint32_t *rec_start, const T *rec_w,
                               const T *Fs, int C, const MeshGeom &g, T *mesh, cudaStream_t s) {
    if (!spread_cols_ok(g.K, C, sizeof(T), g.p)) return cudaErrorInvalidValue;
    switch (g.p) {
        case 4: return dispatch_cpl<T, 4>(start_off, rec_start, rec_w, Fs, C, g, mesh, s);
        case 6: return dispatch_cpl<T, 6>(start_off, rec_start, rec_w, Fs, C, g, mesh, s);
        case 8: return dispatch_cpl<T, 8>(start_off, rec_start, rec_w, Fs, C, g, mesh, s);
        default: return cudaErrorInvalidValue;
    }
}

template <typename T>
cudaError_t launch_spread_cols_batch(const SpreadColsSys<T> *sys, const int *prefix, int nsys,
                                     int total, int C, cudaStream_t s) {
    if (total <= 0) return cudaSuccess;
    switch (cols_cpl(C)) {
        case 1: return launch_cols_batch<T, 1>(sys, prefix, nsys, total, s);
        case 2: return launch_cols_batch<T, 2>(sys, prefix, nsys, total, s);
        default: return launch_cols_batch<T, 3>(sys, prefix, nsys, total, s);
    }
}

int spread_cols_blocks(int K, int C, size_t elem) {
    const int TZ = elem == 4 ? 16 : 8, XT = 16, CC = 16 * cols_cpl(C);
    return ((K + XT - 1) / XT) * K * ((K + TZ - 1) / TZ) * ((C + CC - 1) / CC);
}

template cudaError_t launch_spread_cols_batch<float>(const SpreadColsSys<float> *, const int *,
                                                     int, int, int, cudaStream_t);
template cudaError_t launch_spread_cols_batch<double>(const SpreadColsSys<double> *, const int *,
                                                      int, int, int, cudaStream_t);
template void launch_gather_cols_rows<float>(const float *, const int *, int, int, float *,
                                             cudaStream_t);
template void launch_gather_cols_rows<double>(const double *, const int *, int, int, double *,
                                              cudaStream_t);
template cudaError_t launch_spread_cols<float>(const int *, const uint32_t *, const float *,
                                               const float *, int, const MeshGeom &, float *,
                                               cudaStream_t);
template cudaError_t launch_spread_cols<double>(const int *, const uint32_t *, const double *,
                                                const double *, int, const MeshGeom &, double *,
                                                cudaStream_t);

}  // namespace spme
