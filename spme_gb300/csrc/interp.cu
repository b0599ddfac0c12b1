// Interpolation of the 3R mesh components back to the particles (restates
// old-version/spme_kernel.c:8-70: v_i = sum_j P_ij grid[c][ind_ij]).
//
// One CTA per mesh tile.  For CG components at a time it stages the tile
// plus its (p-1) upper halo in shared memory as a dense box
// [CG][HZB][HYB][HX] (HX = 24 wide: every lane's x offset fits; at 16x8x4
// tiles the component-plane stride is 24 (mod 32) words, so the gather below
// is bank-conflict free):
//   * one TMA (cp.async.bulk.tensor) load per chunk, completing on an mbarrier
//     (bounded wait, error flag on timeout); for tiles whose halo wraps the
//     periodic boundary the part past K arrives as zeros and is patched with
//     16-byte vector loads (all rows with plain loads when TMA is unavailable).
// Each warp then interpolates the tile's own particles from shared memory:
// FP32 at p = 4, 6 two particles per warp with lanes = (x column pair,
// component) and two-lane FMAs (interp_pairs); otherwise one particle per warp
// with lanes = (x offset 0..7, component 0..3).  The x offsets are summed with
// shuffles.  Every particle is handled by exactly one CTA; a tile's halo is
// staged again by its neighbours (from L2 where it is still cached).
#include <algorithm>

#include "kernels.h"
#include "tma.cuh"

namespace spme {

namespace {

constexpr int kThreads = 256;
constexpr int kHX = 24;  // staged row width (elements)

template <typename T> struct Vec16;
template <> struct Vec16<float> { using type = float4; static constexpr int n = 4; };
template <> struct Vec16<double> { using type = double2; static constexpr int n = 2; };

// A half-warp's copy of one particle record for interp_pairs: lane j of the
// half holds weights j and 16 + j (the record's 3p weights: x, y, z), plus
// the stencil start; read by shuffles within the half.
struct HalfRec {
    float wa, wb;
    uint32_t st;
};

template <int P>
__device__ __forceinline__ HalfRec load_pair_rec(const InterpArgs<float> &A, int s) {
    const int j = threadIdx.x & 15;
    const float *rw = A.rec_w + (size_t)s * A.ws;
    HalfRec r;
    r.wa = j < 3 * P ? __ldg(rw + j) : 0.f;
    r.wb = j < 3 * P - 16 ? __ldg(rw + 16 + j) : 0.f;
    r.st = __ldg(A.rec_start + s);
    return r;
}

// FP32, 4-component boxes, p = 4 or 6: two particles per warp, one per
// half-warp, lanes of a half = (x pair 0..3, component 0..3).  A lane's x pair
// starts at an even box column (the particle's first column, or the one before
// it when that is odd), is read with one 8-byte load and meets its two x
// weights (times the y weight) in one two-lane FMA (fma.rn.f32x2): each load
// and FMA instruction covers two mesh points.  Columns outside the stencil
// carry zero weights (the box is 24 columns wide: a pair ends at most at
// column tx + 6).  The next pair's records are loaded while this pair is
// interpolated; rec0 is the warp's first pair, loaded once per tile.
template <int P>
__device__ __forceinline__ void interp_pairs(const float *box, int PS, int HYB,
                                             const InterpArgs<float> &A, int c0, int nc,
                                             int pbeg, int pend, int ox, int oy, int oz,
                                             HalfRec rec0) {
    constexpr int kWarps = kThreads / 32;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int h = lane >> 4, xp = (lane >> 2) & 3, cl = lane & 3;
    const int C = A.C;
    HalfRec nxt = rec0;
    for (int s0 = pbeg + 2 * warp; s0 < pend; s0 += 2 * kWarps) {
        const HalfRec r = nxt;
        if (s0 + 2 * kWarps < pend) nxt = load_pair_rec<P>(A, min(s0 + 2 * kWarps + h, pend - 1));
        // weight i of this half's particle
        auto w = [&](int i) {
            return i < 16 ? __shfl_sync(0xffffffffu, r.wa, i, 16)
                          : __shfl_sync(0xffffffffu, r.wb, i - 16, 16);
        };
        const int s = s0 + h;
        int sx, sy, sz;
        unpack_start(r.st, sx, sy, sz);
        const int lx = sx - ox, ly = sy - oy, lz = sz - oz;  // own tile: no wrap
        const int odd = lx & 1;
        const int i0 = 2 * xp - odd;  // stencil column of the pair's first point
        const float x0 = __shfl_sync(0xffffffffu, r.wa, i0 & 15, 16);
        const float x1 = __shfl_sync(0xffffffffu, r.wa, i0 + 1, 16);
        const float wx0 = i0 >= 0 && i0 < P ? x0 : 0.f;
        const float wx1 = i0 + 1 < P ? x1 : 0.f;
        float2 wxy[P];
        float wz[P];
#pragma unroll
        for (int y = 0; y < P; y++) {
            const float wy = w(P + y);
            wxy[y] = make_float2(wx0 * wy, wx1 * wy);
        }
#pragma unroll
        for (int z = 0; z < P; z++) wz[z] = w(2 * P + z);
        const float *base = box + (size_t)cl * PS + (lz * HYB + ly) * kHX + (lx - odd) + 2 * xp;
        float2 acc = make_float2(0.f, 0.f);
        // sum over y with w_x w_y first, then one w_z per plane
#pragma unroll
        for (int z = 0; z < P; z++) {
            const float *pz = base + z * HYB * kHX;
            float2 t = make_float2(0.f, 0.f);
#pragma unroll
            for (int y = 0; y < P; y++)
                t = __ffma2_rn(wxy[y], *reinterpret_cast<const float2 *>(pz + y * kHX), t);
            acc = __ffma2_rn(make_float2(wz[z], wz[z]), t, acc);
        }
        float a = acc.x + acc.y;
        a += __shfl_xor_sync(0xffffffffu, a, 4);
        a += __shfl_xor_sync(0xffffffffu, a, 8);
        if (s < pend && xp == 0 && cl < nc) {
            float *out = A.W + (size_t)__ldg(A.rec_idx + s) * C + c0 + cl;
            *out = A.accumulate ? *out + a : a;
        }
    }
}

// One tile's work (the body of the single-system kernel and of the batched
// one); tmap is read only when use_tma is set.
template <typename T, int P, int CG>
__device__ __forceinline__ void interp_body(const CUtensorMap *tmap, const InterpArgs<T> &A,
                                            int tile) {
    using V = typename Vec16<T>::type;
    constexpr int VW = Vec16<T>::n;
    constexpr int NV = kHX / VW;  // vectors per staged row
    constexpr int NG = CG / 4;    // groups of 4 components per chunk
    const int use_tma = A.use_tma;
    const int *__restrict__ tile_off = A.tile_off;
    const int *__restrict__ rec_idx = A.rec_idx;
    const uint32_t *__restrict__ rec_start = A.rec_start;
    const T *__restrict__ rec_w = A.rec_w;
    const T *__restrict__ mesh = A.mesh;
    T *__restrict__ W = A.W;
    int *__restrict__ err = A.err;
    const MeshGeom &g = A.g;
    const int C = A.C, cb = A.cb, ce = A.ce, accumulate = A.accumulate, WS = A.ws;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t bar;
    // TMA destinations must be 128-byte aligned (128 spare bytes are allocated)
    T *box = reinterpret_cast<T *>(smem_raw + ((128 - (smem_addr(smem_raw) & 127)) & 127));

    const int pbeg = tile_off[tile], pend = tile_off[tile + 1];
    if (pbeg == pend) return;
    const int K = g.K;
    const int HYB = g.ty + P - 1, HZB = g.tz + P - 1;
    const int PS = HZB * HYB * kHX;  // component-plane stride
    const int tix = tile % g.ntx, tiy = (tile / g.ntx) % g.nty, tiz = tile / (g.ntx * g.nty);
    const int ox = tix * g.tx, oy = tiy * g.ty, oz = tiz * g.tz;
    const int hx = min(g.tx, K - ox) + P - 1;
    const int hy = min(g.ty, K - oy) + P - 1;
    const int hz = min(g.tz, K - oz) + P - 1;
    // TMA: the box's innermost start coordinate times the element size must be a
    // multiple of 16 bytes.  A halo that wraps the periodic boundary is loaded by
    // TMA too (the part past K arrives as zeros) and the wrapped part patched
    // with plain loads.
    const bool wraps = ox + hx > K || oy + hy > K || oz + hz > K;
    const bool tma = use_tma && ((size_t)ox * sizeof(T)) % 16 == 0;
    const size_t K2 = (size_t)K * K, K3 = K2 * K;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int xs = lane >> 2, cl = lane & 3;

    if (tma && threadIdx.x == 0) {
        mbar_init(&bar, 1);
        mbar_fence_init();
    }
    __syncthreads();

    // rows [c][z][y][0..kHX) of the halo region with plain (wrap-aware) loads:
    // all of them, or only the elements past the periodic boundary
    auto stage_rows = [&](int c0, int nc, bool only_wrapped) {
        const bool vec = (K % VW) == 0 && (ox % VW) == 0;
        DivMod dnv, dhy, dhz;
        dnv.init(NV);
        dhy.init(hy);
        dhz.init(hz);
        const int nrow = nc * hz * hy;
        for (int q = threadIdx.x; q < nrow * NV; q += kThreads) {
            int v, y, z;
            const int row = dnv.div(q, v);
            const int cz = dhy.div(row, y);
            const int c = dhz.div(cz, z);
            int gy = oy + y, gz = oz + z;
            const bool row_wraps = gy >= K || gz >= K;
            gy -= gy >= K ? K : 0;
            gz -= gz >= K ? K : 0;
            const int x0 = ox + v * VW;
            if (only_wrapped && !row_wraps && (x0 + VW <= K || v * VW >= hx)) continue;
            const T *src = mesh + (size_t)(c0 + c) * K3 + (size_t)gz * K2 + (size_t)gy * K;
            T *dst = box + (size_t)c * PS + (z * HYB + y) * kHX + v * VW;
            if (vec) {
                *reinterpret_cast<V *>(dst) = __ldg(reinterpret_cast<const V *>(src + x0 % K));
            } else {
#pragma unroll
                for (int e = 0; e < VW; e++)
                    if (!only_wrapped || row_wraps || x0 + e >= K) dst[e] = __ldg(src + (x0 + e) % K);
            }
        }
        __syncthreads();
    };

    // FP32 p = 4, 6: two particles per warp, x columns in pairs (interp_pairs)
    constexpr bool kPairs = sizeof(T) == 4 && CG == 4 && (P == 4 || P == 6);
    // after a TMA box of a tile whose halo wraps: the elements past the periodic
    // boundary (zeros in the box) from plain loads, one thread per box row: a
    // row past K in y or z is copied whole, other rows only from column K - ox on
    const int xw0 = ox + hx > K ? (K - ox) / VW : NV;  // first vector holding a wrapped column
    const int xw1 = (hx - 1) / VW;                     // last vector of the halo
    auto patch_wrapped = [&](int c0, int nc) {
        const bool vec = (K % VW) == 0 && (ox % VW) == 0;
        DivMod dhy, dhz;
        dhy.init(hy);
        dhz.init(hz);
        const int nrow = nc * hz * hy;
        for (int row = threadIdx.x; row < nrow; row += kThreads) {
            int y, z;
            const int cz = dhy.div(row, y);
            const int c = dhz.div(cz, z);
            int gy = oy + y, gz = oz + z;
            const bool row_wraps = gy >= K || gz >= K;
            if (!row_wraps && xw0 == NV) continue;
            gy -= gy >= K ? K : 0;
            gz -= gz >= K ? K : 0;
            const T *src = mesh + (size_t)(c0 + c) * K3 + (size_t)gz * K2 + (size_t)gy * K;
            T *dst = box + (size_t)c * PS + (z * HYB + y) * kHX;
            const int v1 = row_wraps ? NV - 1 : xw1;
            for (int v = row_wraps ? 0 : xw0; v <= v1; v++) {
                const int x0 = ox + v * VW;
                if (vec) {
                    *reinterpret_cast<V *>(dst + v * VW) =
                        __ldg(reinterpret_cast<const V *>(src + x0 % K));
                } else {
#pragma unroll
                    for (int e = 0; e < VW; e++) dst[v * VW + e] = __ldg(src + (x0 + e) % K);
                }
            }
        }
        __syncthreads();
    };

    // the warp's first particle's record, the same for every component chunk:
    // loaded once, before the first box is waited for
    constexpr int kWarps = kThreads / 32;
    T wreg_0 = T(0);
    uint32_t st_0 = 0;
    int idx_0 = 0;
    HalfRec hrec_0{0.f, 0.f, 0u};
    if constexpr (kPairs) {
        if (pbeg + 2 * warp < pend)
            hrec_0 = load_pair_rec<P>(reinterpret_cast<const InterpArgs<float> &>(A),
                                      min(pbeg + 2 * warp + (lane >> 4), pend - 1));
    } else if (pbeg + warp < pend) {
        const int s = pbeg + warp;
        wreg_0 = lane < 3 * P ? __ldg(rec_w + (size_t)s * WS + lane) : T(0);
        st_0 = __ldg(rec_start + s);
        idx_0 = __ldg(rec_idx + s);
    }

    int chunk = 0;
    for (int c0 = cb; c0 < ce; c0 += CG, chunk++) {
        const int nc = min(CG, ce - c0);
        if (tma) {
            if (threadIdx.x == 0) {
                fence_proxy_async();  // order earlier generic reads of the box before the TMA write
                mbar_expect_tx(&bar, (uint32_t)((size_t)CG * PS * sizeof(T)));
                tma_load_4d(box, tmap, ox, oy, oz, c0, &bar);
            }
            const bool ok = mbar_wait(&bar, (uint32_t)(chunk & 1));
            if (!__syncthreads_and(ok)) {  // uniform decision: all threads give up together
                if (threadIdx.x == 0) atomicExch(err, 1);
                return;
            }
            if (wraps) patch_wrapped(c0, nc);
        } else {
            stage_rows(c0, nc, false);
        }
        if constexpr (kPairs) {
            interp_pairs<P>(reinterpret_cast<const float *>(box), PS, HYB,
                            reinterpret_cast<const InterpArgs<float> &>(A), c0, nc, pbeg, pend,
                            ox, oy, oz, hrec_0);
            __syncthreads();  // the box is rewritten by the next chunk
            continue;
        }
        // the next particle's record is loaded while this one is interpolated
        T wreg_n = wreg_0;
        uint32_t st_n = st_0;
        int idx_n = idx_0;
        for (int s = pbeg + warp; s < pend; s += kWarps) {
            const T wreg = wreg_n;
            const uint32_t st = st_n;
            const int idx = idx_n;
            if (s + kWarps < pend) {
                const int sn = s + kWarps;
                wreg_n = lane < 3 * P ? __ldg(rec_w + (size_t)sn * WS + lane) : T(0);
                st_n = __ldg(rec_start + sn);
                idx_n = __ldg(rec_idx + sn);
            }
            int sx, sy, sz;
            unpack_start(st, sx, sy, sz);
            const int lx = sx - ox, ly = sy - oy, lz = sz - oz;  // own tile: no wrap
            const T wxv = __shfl_sync(0xffffffffu, wreg, xs < P ? xs : P - 1);
            const T wx = xs < P ? wxv : T(0);
            T wxy[P], wz[P];
#pragma unroll
            for (int y = 0; y < P; y++) wxy[y] = wx * __shfl_sync(0xffffffffu, wreg, P + y);
#pragma unroll
            for (int z = 0; z < P; z++) wz[z] = __shfl_sync(0xffffffffu, wreg, 2 * P + z);
            T acc[NG];
#pragma unroll
            for (int k = 0; k < NG; k++) acc[k] = T(0);
            const T *base = box + (size_t)cl * PS + (lz * HYB + ly) * kHX + lx + xs;
            // sum over y with w_x w_y first, then one w_z per plane
#pragma unroll
            for (int z = 0; z < P; z++) {
                const T *pz = base + z * HYB * kHX;
                T t[NG];
#pragma unroll
                for (int k = 0; k < NG; k++) t[k] = T(0);
#pragma unroll
                for (int y = 0; y < P; y++)
#pragma unroll
                    for (int k = 0; k < NG; k++) t[k] += wxy[y] * pz[(size_t)k * 4 * PS + y * kHX];
#pragma unroll
                for (int k = 0; k < NG; k++) acc[k] += wz[z] * t[k];
            }
#pragma unroll
            for (int k = 0; k < NG; k++)
#pragma unroll
                for (int o = 4; o < 32; o <<= 1) acc[k] += __shfl_xor_sync(0xffffffffu, acc[k], o);
            if (xs == 0) {
                T *out = W + (size_t)idx * C + c0;
#pragma unroll
                for (int k = 0; k < NG; k++) {
                    const int c = 4 * k + cl;
                    if (c < nc) out[c] = accumulate ? out[c] + acc[k] : acc[k];
                }
            }
        }
        __syncthreads();  // the box is rewritten by the next chunk
    }
}

template <typename T, int P, int CG>
// blocks per SM that the 4-component box's shared memory allows (16x8x4 tiles)
__global__ void __launch_bounds__(kThreads, sizeof(T) == 4 ? 5 : 2)
k_interp(const __grid_constant__ CUtensorMap tmap, InterpArgs<T> A) {
    // tiles z fastest: blocks launched together are z neighbours, whose boxes
    // share p - 1 of their tz + p - 1 planes (read from L2 by the later ones)
    const int b = blockIdx.x, ntx = A.g.ntx, nty = A.g.nty, ntz = A.g.ntz;
    const int tiz = b % ntz, rest = b / ntz;
    interp_body<T, P, CG>(&tmap, A, (tiz * nty + rest / ntx) * ntx + rest % ntx);
}

// Many systems in one persistent launch over their tiles: each system's boxes
// by TMA through its own descriptor in the work list where its mesh rows allow
// it, by plain loads otherwise; the order p of each system selects the body
// (the batch launches one such kernel per order).
template <typename T, int CG>
__global__ void __launch_bounds__(kThreads)
k_interp_batch(const InterpSys<T> *__restrict__ sys, const int *__restrict__ prefix, int nsys,
               int total) {
    for (int w = blockIdx.x; w < total; w += gridDim.x) {
        const int k = batch_find(prefix, nsys, w);
        const InterpArgs<T> A = sys[k].args;
        // the system's TMA box stays in the global work list (a descriptor in
        // global memory; never a local copy)
        const CUtensorMap *tmap = A.use_tma ? &sys[k].tmap : nullptr;
        const int tile = w - prefix[k];
        switch (A.g.p) {
            case 4: interp_body<T, 4, CG>(tmap, A, tile); break;
            case 6: interp_body<T, 6, CG>(tmap, A, tile); break;
            default: interp_body<T, 8, CG>(tmap, A, tile); break;
        }
        __syncthreads();
    }
}

template <typename T, int P, int CG>
size_t interp_smem(const MeshGeom &g) {
    return (size_t)CG * (g.tz + P - 1) * (g.ty + P - 1) * kHX * sizeof(T) + 128;
}

template <typename T, int P, int CG>
cudaError_t launch_interp_t(const InterpMaps &maps, const int *tile_off, const int *rec_idx,
                            const uint32_t *rec_start, const T *rec_w, const T *mesh, int C,
                            int cb, int ce, const MeshGeom &g, T *W, int accumulate, int *err,
                            cudaStream_t s) {
    const size_t smem = interp_smem<T, P, CG>(g);
    auto kern = k_interp<T, P, CG>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    const bool use = maps.ok4;
    const CUtensorMap &m = maps.cg4;
    InterpArgs<T> A{tile_off, rec_idx, rec_start, rec_w, mesh, W, err, g, C, cb, ce,
                    accumulate, use ? 1 : 0, RecordWidth<T, P>::value};
    kern<<<g.ntx * g.nty * g.ntz, kThreads, smem, s>>>(m, A);
    return cudaGetLastError();
}

template <typename T, int P>
cudaError_t dispatch_cg(const InterpMaps &maps, const int *tile_off, const int *rec_idx,
                        const uint32_t *rec_start, const T *rec_w, const T *mesh, int C,
                        int cb, int ce, const MeshGeom &g, T *W, int accumulate, int *err,
                        cudaStream_t s) {
    return launch_interp_t<T, P, 4>(maps, tile_off, rec_idx, rec_start, rec_w, mesh, C, cb, ce, g,
                                    W, accumulate, err, s);
}

bool encode_box(CUtensorMap *m, const void *mesh, int K, int C, const MeshGeom &g, size_t elem,
                int CG) {
    EncodeTiledFn fn = encode_fn();
    if (!fn || (K * elem) % 16 != 0 || ((uintptr_t)mesh % 16) != 0) return false;
    const cuuint64_t dims[4] = {(cuuint64_t)K, (cuuint64_t)K, (cuuint64_t)K, (cuuint64_t)C};
    const cuuint64_t strides[3] = {(cuuint64_t)K * elem, (cuuint64_t)K * K * elem,
                                   (cuuint64_t)K * K * K * elem};
    const cuuint32_t box[4] = {(cuuint32_t)kHX, (cuuint32_t)(g.ty + g.p - 1),
                               (cuuint32_t)(g.tz + g.p - 1), (cuuint32_t)CG};
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    if (box[1] > 256 || box[2] > 256) return false;
    CUresult r = fn(m, elem == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64,
                    4, const_cast<void *>(mesh), dims, strides, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                    CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

}  // namespace

size_t interp_smem_bytes(const MeshGeom &g, size_t elem) {
    return (size_t)4 * (g.tz + g.p - 1) * (g.ty + g.p - 1) * kHX * elem + 128;
}

bool make_interp_box(CUtensorMap *map, const void *mesh, int C, const MeshGeom &g, size_t elem) {
    return encode_box(map, mesh, g.K, C, g, elem, 4);
}

bool make_interp_maps(InterpMaps *maps, const void *mesh, int C, const MeshGeom &g, size_t elem) {
    maps->ok4 = encode_box(&maps->cg4, mesh, g.K, C, g, elem, 4);
    return maps->ok4;
}

template <typename T>
cudaError_t launch_interp(const InterpMaps &maps, const int *tile_off, int n, const int *rec_idx,
                          const uint32_t *rec_start, const T *rec_w, const T *mesh, int C,
                          int cb, int ce, const MeshGeom &g, T *W, int accumulate, int *err,
                          cudaStream_t s) {
    if (n <= 0 || cb >= ce) return cudaSuccess;
    if (cb < 0 || ce > C) return cudaErrorInvalidValue;
    if (g.tx + 7 > kHX || g.tx + g.p - 1 > kHX) return cudaErrorInvalidValue;
    switch (g.p) {
        case 4: return dispatch_cg<T, 4>(maps, tile_off, rec_idx, rec_start, rec_w, mesh, C, cb, ce, g, W, accumulate, err, s);
        case 6: return dispatch_cg<T, 6>(maps, tile_off, rec_idx, rec_start, rec_w, mesh, C, cb, ce, g, W, accumulate, err, s);
        case 8: return dispatch_cg<T, 8>(maps, tile_off, rec_idx, rec_start, rec_w, mesh, C, cb, ce, g, W, accumulate, err, s);
        default: return cudaErrorInvalidValue;
    }
}

template <typename T>
cudaError_t launch_interp_batch(const InterpSys<T> *sys, const int *prefix, int nsys, int total,
                                size_t smem, cudaStream_t s, size_t smem_limit) {
    if (total <= 0) return cudaSuccess;
    auto kern = k_interp_batch<T, 4>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)std::max(smem, smem_limit));
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreads, smem);
    const int grid = std::max(1, std::min(total, sms * std::max(per_sm, 1)));
    kern<<<grid, kThreads, smem, s>>>(sys, prefix, nsys, total);
    return cudaGetLastError();
}

template cudaError_t launch_interp_batch<float>(const InterpSys<float> *, const int *, int, int,
                                                size_t, cudaStream_t, size_t);
template cudaError_t launch_interp_batch<double>(const InterpSys<double> *, const int *, int, int,
                                                 size_t, cudaStream_t, size_t);
template cudaError_t launch_interp<float>(const InterpMaps &, const int *, int, const int *,
                                          const uint32_t *, const float *, const float *, int,
                                          int, int, const MeshGeom &, float *, int, int *,
                                          cudaStream_t);
template cudaError_t launch_interp<double>(const InterpMaps &, const int *, int, const int *,
                                           const uint32_t *, const double *, const double *, int,
                                           int, int, const MeshGeom &, double *, int, int *,
                                           cudaStream_t);

}  // namespace spme
