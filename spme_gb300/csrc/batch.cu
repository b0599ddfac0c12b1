// Batches of independent systems (uneven N, L, K, p) applied together: every
// stage of the position build and of the apply is one launch over a packed
// work list covering all systems (persistent blocks walk the list), and cuFFT
// runs one batched plan per distinct mesh size.  No counterpart in the
// reference, whose compute_spme (old-version/spme.c:560-726) applies one
// system; each system's operator is the engine's full M = M_recip + M_real +
// M_self.
//
// Packing:
//   * particles of system k occupy [P_k, P_k + N_k) in every per-particle
//     array (positions, forces, results, records); the caller's vectors hold
//     system k's R right-hand sides at element offset 3 R P_k, rows of 3 N_k;
//   * sort keys of system k are offset into one key space per sort (mesh
//     tiles, stencil-start cells, real-space cells), so a single counting sort
//     over the concatenated keys leaves each system's particles in its own
//     slot range [P_k, P_k + N_k);
//   * meshes and half spectra are laid out grouped by mesh size K, so each
//     group is one batched cuFFT plan (component-major, as in the engine).
#include <cuda_runtime.h>
#include <cufft.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <new>
#include <vector>

#include "kernels.h"
#include "spme_gb300.h"

namespace spme {
namespace {

// Geometry of one system for the per-particle batched kernels.
struct BatchGeo {
    MeshGeom g;
    int nc;         // real-space cells per axis (1: one cell, minimum image)
    int p_off;      // first particle
    int tile_off;   // first mesh-tile key
    int start_off;  // first stencil-start-cell key
    int cell_off;   // first real-space cell key
};

template <typename T> struct V4T;
template <> struct V4T<float> { using type = float4; };
template <> struct V4T<double> { using type = double4_32a; };

// Sort keys (with slots from atomic counts), stencil starts, fractional mesh
// coordinates and cell-relative positions of every particle of every system
// (the engine's k_all_keys with the system looked up per particle).
template <typename T>
__global__ void k_batch_keys(const double *__restrict__ pos, int n, const int *__restrict__ sysid,
                             const BatchGeo *__restrict__ geo, int *__restrict__ key1,
                             int *__restrict__ count1, int *__restrict__ slot1,
                             int *__restrict__ key2, int *__restrict__ count2,
                             int *__restrict__ slot2, int *__restrict__ key3,
                             int *__restrict__ count3, int *__restrict__ slot3,
                             uint32_t *__restrict__ pstart, T *__restrict__ pfrac,
                             typename V4T<T>::type *__restrict__ prel) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const BatchGeo G = geo[sysid[i]];
    const MeshGeom &g = G.g;
    int s[3], cc[3];
    double fr[3], rel[3];
    const double h = g.L / G.nc;
#pragma unroll
    for (int d = 0; d < 3; d++) {
        const double xw = wrap_coord(pos[3 * i + d], g.L, g.invL);
        mesh_coord_w(xw, g.invL, g.K, g.p, s[d], fr[d]);
        cc[d] = cell_coord_w(xw, g.invL, G.nc);
        rel[d] = xw - cc[d] * h;
    }
    typename V4T<T>::type v;
    v.x = (T)rel[0];
    v.y = (T)rel[1];
    v.z = (T)rel[2];
    v.w = T(0);
    prel[i] = v;
    pstart[i] = pack_start(s[0], s[1], s[2]);
#pragma unroll
    for (int d = 0; d < 3; d++) pfrac[3 * i + d] = (T)fr[d];
    int k = G.tile_off + ((s[2] / g.tz) * g.nty + s[1] / g.ty) * g.ntx + s[0] / g.tx;
    key1[i] = k;
    slot1[i] = atomicAdd(&count1[k], 1);
    k = G.start_off + (s[1] * g.K + s[0]) * g.K + s[2];
    key2[i] = k;
    slot2[i] = atomicAdd(&count2[k], 1);
    k = G.cell_off + (cc[2] * G.nc + cc[1]) * G.nc + cc[0];
    key3[i] = k;
    slot3[i] = atomicAdd(&count3[k], 1);
}

// Records in sorted order (the engine's k_records, order p per system, one
// record stride ws for the whole batch).
template <typename T, int P>
__device__ __forceinline__ void batch_record(const T *__restrict__ pfrac, int i, int ws, T *out) {
    T w[P];
#pragma unroll
    for (int d = 0; d < 3; d++) {
        bspline_weights<T, P>(pfrac[3 * i + d], w);
#pragma unroll
        for (int j = 0; j < P; j++) out[d * P + j] = w[j];
    }
    for (int j = 3 * P; j < ws; j++) out[j] = T(0);
}

// (records assembled in shared memory, written as one contiguous run)
constexpr int kRecThreads = 128;
constexpr int kMaxWs = 24;  // record stride of order 8

template <typename T>
__global__ void __launch_bounds__(kRecThreads)
k_batch_records(const uint32_t *__restrict__ pstart, const T *__restrict__ pfrac,
                const int *__restrict__ perm, int n, const int *__restrict__ sysid,
                const BatchGeo *__restrict__ geo, int ws, int *__restrict__ rec_idx,
                uint32_t *__restrict__ rec_start, T *__restrict__ rec_w) {
    __shared__ __align__(16) T sm[kRecThreads * kMaxWs];
    const int s0 = blockIdx.x * kRecThreads;
    const int s = s0 + threadIdx.x;
    if (s < n) {
        const int i = perm[s];
        rec_idx[s] = i;
        rec_start[s] = pstart[i];
        T *out = sm + (size_t)threadIdx.x * ws;
        switch (geo[sysid[i]].g.p) {
            case 4: batch_record<T, 4>(pfrac, i, ws, out); break;
            case 6: batch_record<T, 6>(pfrac, i, ws, out); break;
            default: batch_record<T, 8>(pfrac, i, ws, out); break;
        }
    }
    __syncthreads();
    const int cnt = min(kRecThreads, n - s0);
    const int vq = ws * (int)sizeof(T) / 16;
    float4 *dst = reinterpret_cast<float4 *>(rec_w + (size_t)s0 * ws);
    const float4 *src = reinterpret_cast<const float4 *>(sm);
    for (int v = threadIdx.x; v < cnt * vq; v += kRecThreads) dst[v] = src[v];
}

// Caller layout (system k at element 3 R P_k, rows of 3 N_k) <-> packed rows
// F[i][3R]; one thread per particle (its system found once from the particle
// prefix), four right-hand sides at a time as three 16-byte vectors on the
// packed side where R is a multiple of 4 (FP32), scalars otherwise.
template <typename T>
__global__ void k_batch_pack(const T *__restrict__ f, const int *__restrict__ pref, int nsys,
                             int R, int ntot, T *__restrict__ F) {
    const int C = 3 * R;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ntot; i += gridDim.x * blockDim.x) {
        const int k = batch_find(pref, nsys, i);
        const int P0 = pref[k], nk = pref[k + 1] - P0, li = i - P0;
        const T *src = f + (size_t)C * P0 + 3 * li;
        T *dst = F + (size_t)i * C;
        int r = 0;
        if constexpr (sizeof(T) == 4) {
            if ((R & 3) == 0) {
                for (; r < R; r += 4) {
                    float v[12];
#pragma unroll
                    for (int q = 0; q < 4; q++) {
                        const T *s = src + (size_t)(r + q) * 3 * nk;
                        v[3 * q] = __ldg(s);
                        v[3 * q + 1] = __ldg(s + 1);
                        v[3 * q + 2] = __ldg(s + 2);
                    }
                    float4 *d4 = reinterpret_cast<float4 *>(dst + 3 * r);
                    d4[0] = make_float4(v[0], v[1], v[2], v[3]);
                    d4[1] = make_float4(v[4], v[5], v[6], v[7]);
                    d4[2] = make_float4(v[8], v[9], v[10], v[11]);
                }
            }
        }
        for (; r < R; r++) {
            const T *s = src + (size_t)r * 3 * nk;
            dst[3 * r] = __ldg(s);
            dst[3 * r + 1] = __ldg(s + 1);
            dst[3 * r + 2] = __ldg(s + 2);
        }
    }
}

template <typename T>
__global__ void k_batch_unpack(const T *__restrict__ W, const T *__restrict__ W2,
                               const int *__restrict__ pref, int nsys, int R, int ntot, T alpha,
                               T beta, T *__restrict__ u) {
    const int C = 3 * R;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ntot; i += gridDim.x * blockDim.x) {
        const int k = batch_find(pref, nsys, i);
        const int P0 = pref[k], nk = pref[k + 1] - P0, li = i - P0;
        T *dst = u + (size_t)C * P0 + 3 * li;
        const size_t row = (size_t)i * C;
        auto put = [&](int r, int d, T w) {
            T *o = dst + (size_t)r * 3 * nk + d;
            *o = beta == T(0) ? alpha * w : beta * *o + alpha * w;
        };
        int r = 0;
        if constexpr (sizeof(T) == 4) {
            if ((R & 3) == 0) {
                for (; r < R; r += 4) {
                    const float4 *a4 = reinterpret_cast<const float4 *>(W + row + 3 * r);
                    const float4 *b4 = reinterpret_cast<const float4 *>(W2 + row + 3 * r);
                    float v[12];
#pragma unroll
                    for (int q = 0; q < 3; q++) {
                        const float4 a = __ldg(a4 + q), bb = __ldg(b4 + q);
                        v[4 * q] = a.x + bb.x;
                        v[4 * q + 1] = a.y + bb.y;
                        v[4 * q + 2] = a.z + bb.z;
                        v[4 * q + 3] = a.w + bb.w;
                    }
#pragma unroll
                    for (int q = 0; q < 12; q++) put(r + q / 3, q % 3, v[q]);
                }
            }
        }
        for (; r < R; r++)
            for (int d = 0; d < 3; d++) put(r, d, W[row + 3 * r + d] + W2[row + 3 * r + d]);
    }
}

// Influence on every system's half spectrum (interior planes as the engine's
// k_influence, the kx = 0 and K/2 planes as k_influence_planes: the Hermitian
// part, pairing (y, z) with (-y, -z)).  Work item: a block of 256 points of
// one system, interior points first, then the points of its x = 0 / K/2
// planes.
struct InflSys {
    int K, nb_int;             // blocks over the interior points, then the plane points
    size_t spec_off, tab_off;  // complex-element offsets
    double twopi_L;
};

template <typename T>
struct Cx2 {
    T re, im;
};

template <typename T>
__device__ __forceinline__ void infl_apply(T m2, T c, T kx, T ky, T kz, const Cx2<T> (&g)[3],
                                           Cx2<T> (&o)[3]) {
    const T b0 = m2 - c * kx * kx, b1 = -c * kx * ky, b2 = -c * kx * kz;
    const T b3 = m2 - c * ky * ky, b4 = -c * ky * kz, b5 = m2 - c * kz * kz;
    o[0].re = b0 * g[0].re + b1 * g[1].re + b2 * g[2].re;
    o[0].im = b0 * g[0].im + b1 * g[1].im + b2 * g[2].im;
    o[1].re = b1 * g[0].re + b3 * g[1].re + b4 * g[2].re;
    o[1].im = b1 * g[0].im + b3 * g[1].im + b4 * g[2].im;
    o[2].re = b2 * g[0].re + b4 * g[1].re + b5 * g[2].re;
    o[2].im = b2 * g[0].im + b4 * g[1].im + b5 * g[2].im;
}

template <typename T>
__global__ void __launch_bounds__(256)
k_batch_influence(Cx2<T> *__restrict__ G_all, const T *__restrict__ tab_all,
                  const InflSys *__restrict__ sys, const int *__restrict__ prefix, int nsys,
                  int total, int R) {
    using V2 = typename Vec2<T>::type;
    for (int w = blockIdx.x; w < total; w += gridDim.x) {
        const int k = batch_find(prefix, nsys, w);
        const InflSys S = sys[k];
        const int K = S.K, Kh = K / 2 + 1;
        const size_t Kc = (size_t)K * K * Kh;
        Cx2<T> *G = G_all + S.spec_off;
        const V2 *tab = reinterpret_cast<const V2 *>(tab_all) + S.tab_off;
        const T tl = (T)S.twopi_L;
        const int local = w - prefix[k];
        if (local < S.nb_int) {
            // a system's half spectrum has fewer than 2^31 points (K <= 1024):
            // 32-bit index arithmetic
            const unsigned kidx = (unsigned)local * 256u + threadIdx.x;
            if (kidx >= (unsigned)Kc) continue;
            const unsigned rest = kidx / (unsigned)Kh;
            const int x = (int)(kidx - rest * (unsigned)Kh);
            if (x == 0 || (!(K & 1) && x == K / 2)) continue;
            const int z = (int)(rest / (unsigned)K), y = (int)(rest - (unsigned)z * (unsigned)K);
            const V2 mc = tab[kidx];
            const T kx = (T)x * tl;
            const T ky = (T)(y <= K / 2 ? y : y - K) * tl;
            const T kz = (T)(z <= K / 2 ? z : z - K) * tl;
            for (int r = 0; r < R; r++) {
                Cx2<T> *q = G + (size_t)(3 * r) * Kc + kidx;
                const Cx2<T> g[3] = {q[0], q[Kc], q[2 * Kc]};
                Cx2<T> o[3];
                infl_apply<T>(mc.x, mc.y, kx, ky, kz, g, o);
                q[0] = o[0];
                q[Kc] = o[1];
                q[2 * Kc] = o[2];
            }
        } else {
            const size_t t = (size_t)(local - S.nb_int) * 256 + threadIdx.x;
            const int nplanes = (K & 1) ? 1 : 2;
            if (t >= (size_t)nplanes * K * K) continue;
            const size_t qq = t % ((size_t)K * K);
            const int pl = (int)(t / ((size_t)K * K));
            const int x = pl == 0 ? 0 : K / 2;
            const int y = (int)(qq % K), z = (int)(qq / K);
            const int y2 = (K - y) % K, z2 = (K - z) % K;
            const size_t q2 = (size_t)z2 * K + y2;
            if (qq > q2) continue;
            const T kx = (T)x * tl;
            const size_t k1 = qq * Kh + x, k2 = q2 * Kh + x;
            const V2 mc1 = tab[k1], mc2 = tab[k2];
            const T ky1 = (T)(y <= K / 2 ? y : y - K) * tl, kz1 = (T)(z <= K / 2 ? z : z - K) * tl;
            const T ky2 = (T)(y2 <= K / 2 ? y2 : y2 - K) * tl,
                    kz2 = (T)(z2 <= K / 2 ? z2 : z2 - K) * tl;
            for (int r = 0; r < R; r++) {
                Cx2<T> *p1 = G + (size_t)(3 * r) * Kc + k1;
                Cx2<T> *p2 = G + (size_t)(3 * r) * Kc + k2;
                const Cx2<T> g1[3] = {p1[0], p1[Kc], p1[2 * Kc]};
                Cx2<T> o1[3];
                infl_apply<T>(mc1.x, mc1.y, kx, ky1, kz1, g1, o1);
                if (qq == q2) {
#pragma unroll
                    for (int d = 0; d < 3; d++) {
                        o1[d].im = T(0);
                        p1[d * Kc] = o1[d];
                    }
                    continue;
                }
                const Cx2<T> g2[3] = {p2[0], p2[Kc], p2[2 * Kc]};
                Cx2<T> o2[3];
                infl_apply<T>(mc2.x, mc2.y, kx, ky2, kz2, g2, o2);
#pragma unroll
                for (int d = 0; d < 3; d++) {
                    Cx2<T> hh;
                    hh.re = T(0.5) * (o1[d].re + o2[d].re);
                    hh.im = T(0.5) * (o1[d].im - o2[d].im);
                    p1[d * Kc] = hh;
                    hh.im = -hh.im;
                    p2[d * Kc] = hh;
                }
            }
        }
    }
}

int sm_count() {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms > 0 ? sms : 1;
}

int grid_cap(long work, int threads, int per_sm) {
    const long need = (work + threads - 1) / threads;
    const long cap = (long)sm_count() * per_sm;
    return (int)std::max(1L, std::min(need, cap));
}

int nblk(long n, int t) { return (int)((n + t - 1) / t); }

}  // namespace
}  // namespace spme

using namespace spme;

struct BatchSys {
    spme_batch_system s;
    MeshGeom g;
    int nc = 1;
    int p_off = 0, tile_off = 0, start_off = 0, cell_off = 0;
    size_t mesh_off = 0, spec_off = 0, tab_off = 0;  // elements / complex elements
};

struct FftGroup {
    int K = 0;
    size_t mesh_off = 0, spec_off = 0;  // of the group's first system
    int nsys = 0;
    cufftHandle fwd = 0, bwd = 0;
};

struct _spme_batch_t {
    int device = 0;
    int precision = SPME_FP32;
    size_t elem = 4;
    int R = 1, C = 3;
    int nsys = 0, ntot = 0;
    int ntile_keys = 0, nstart_keys = 0, ncell_keys = 0;
    int ws = 0;  // record stride (elements)
    int tile[3] = {16, 8, 4};
    std::vector<BatchSys> sys;
    std::vector<FftGroup> groups;
    cudaStream_t own_stream = nullptr, stream = nullptr;
    // concurrency inside a step: the real-space sum beside the mesh pipeline
    // (overlap bit 0), the cuFFT groups on kFftStreams streams, each with its
    // own work area (bit 1)
    static constexpr int kFftStreams = 4;
    int overlap = 0;
    cudaStream_t rs_stream = nullptr, fft_stream[kFftStreams] = {};
    cudaEvent_t ev_fork = nullptr, ev_rs_join = nullptr, ev_fft_join[kFftStreams] = {};
    void *d_works[kFftStreams] = {};
    long launches = 0;
    bool have_pos = false;
    // per-stage CUDA events of the last uncaptured step (profiling on)
    static constexpr int kStages = 9;
    bool profiling = false, stages_valid = false;
    cudaEvent_t ev[kStages + 1] = {};
    // device
    int *d_sysid = nullptr, *d_pref = nullptr;
    BatchGeo *d_geo = nullptr;
    // d_sort_tmp: scratch of the three counting sorts (the atomic slots are kept
    // in the sorts' permutation buffers until the scatter)
    int *d_key1 = nullptr, *d_key2 = nullptr, *d_key3 = nullptr, *d_sort_tmp = nullptr;
    int *d_cnt1 = nullptr, *d_off1 = nullptr, *d_cnt2 = nullptr, *d_off2 = nullptr,
        *d_cnt3 = nullptr, *d_off3 = nullptr, *d_scan_tmp = nullptr;
    int *d_perm1 = nullptr, *d_perm2 = nullptr, *d_perm3 = nullptr;
    uint32_t *d_pstart = nullptr;
    void *d_pfrac = nullptr, *d_prel = nullptr, *d_cpos = nullptr;
    int *d_ridx1 = nullptr, *d_ridx2 = nullptr;
    uint32_t *d_rst1 = nullptr, *d_rst2 = nullptr;
    void *d_rw1 = nullptr, *d_rw2 = nullptr;
    void *d_F = nullptr, *d_Fs = nullptr, *d_W = nullptr, *d_W2 = nullptr;
    void *d_mesh = nullptr, *d_spec = nullptr, *d_tab = nullptr;
    double *d_pair = nullptr;  // FP64 batches: Chebyshev tables of all systems
    int *d_err = nullptr;
    // work lists (device): per-system launch arguments and block prefixes
    void *d_spread_sys = nullptr, *d_interp_sys = nullptr, *d_real_sys = nullptr;
    InflSys *d_infl_sys = nullptr;
    int *d_pre_spread = nullptr, *d_pre_interp = nullptr, *d_pre_real = nullptr,
        *d_pre_infl = nullptr;
    int tot_spread = 0, tot_real = 0, tot_infl = 0;
    // interpolation work lists, one per B-spline order: each group is one launch
    // with its own shared-memory size (a p = 8 box would otherwise set the
    // occupancy of every system)
    struct InterpGroup {
        int first = 0, count = 0, pre_off = 0, total = 0;
        size_t smem = 0;
    };
    std::vector<InterpGroup> igroups;
    // one captured graph of set_positions + apply
    bool use_graphs = false;
    cudaGraphExec_t gexec = nullptr;
    const double *g_pos = nullptr;
    const void *g_f = nullptr;
    void *g_u = nullptr;
    double g_alpha = 0.0, g_beta = 0.0;
    cudaStream_t g_stream = nullptr;
    long g_launches = 0;
};

namespace {

int from_cuda(cudaError_t e) {
    if (e == cudaSuccess) return SPME_OK;
    cudaGetLastError();
    return e == cudaErrorMemoryAllocation ? SPME_ERR_NOMEM : SPME_ERR_CUDA;
}

#define BTRY(x)                       \
    do {                              \
        int s_ = (x);                 \
        if (s_ != SPME_OK) return s_; \
    } while (0)
#define BTRY_CUDA(x) BTRY(from_cuda(x))

template <typename P>
int balloc(P **p, size_t bytes) {
    void *q = nullptr;
    if (cudaMalloc(&q, bytes < 256 ? 256 : bytes) != cudaSuccess) {
        cudaGetLastError();
        return SPME_ERR_NOMEM;
    }
    *p = reinterpret_cast<P *>(q);
    return SPME_OK;
}

int real_cells(const spme_batch_system &s) {
    long nc = (long)std::floor(s.box_size / s.rcut);
    const long cap = std::max<long>(3, (long)std::cbrt(8.0 * s.np + 27.0));
    nc = std::min(nc, std::min(cap, 1024L));
    return nc < 3 ? 1 : (int)nc;
}

int validate_sys(const spme_batch_system &s, int precision) {
    if (s.np < 1 || s.dim < 2 || s.dim > 1024) return SPME_ERR_INVALID;
    if (s.porder != 4 && s.porder != 6 && s.porder != 8) return SPME_ERR_UNSUPPORTED;
    if (!(s.box_size > 0.0) || !(s.xi > 0.0) || !(s.radius > 0.0)) return SPME_ERR_INVALID;
    if (!(s.rcut > 0.0 && s.rcut < 0.5 * s.box_size)) return SPME_ERR_INVALID;
    // the column-gather spread's z window
    if (!spread_cols_ok(s.dim, 3, precision == SPME_FP32 ? 4 : 8, s.porder))
        return SPME_ERR_UNSUPPORTED;
    return SPME_OK;
}

void set_geo(BatchSys &b, const int tile[3]) {
    MeshGeom &g = b.g;
    g.K = b.s.dim;
    g.p = b.s.porder;
    g.L = b.s.box_size;
    g.invL = 1.0 / b.s.box_size;
    g.tx = std::min(tile[0], g.K);
    g.ty = std::min(tile[1], g.K);
    g.tz = std::min(tile[2], g.K);
    g.ntx = (g.K + g.tx - 1) / g.tx;
    g.nty = (g.K + g.ty - 1) / g.ty;
    g.ntz = (g.K + g.tz - 1) / g.tz;
}

template <typename T>
int record_stride(const _spme_batch_t *b) {
    int pmax = 4;
    for (const BatchSys &x : b->sys) pmax = std::max(pmax, x.s.porder);
    const int per16 = (int)(16 / sizeof(T));
    return (3 * pmax + per16 - 1) / per16 * per16;
}

// Tile-dependent state: tile keys, their offsets, the interpolation work list.
template <typename T>
int build_tiles(_spme_batch_t *b) {
    int off = 0;
    size_t smem = 0;
    for (BatchSys &x : b->sys) {
        set_geo(x, b->tile);
        x.tile_off = off;
        off += x.g.ntx * x.g.nty * x.g.ntz;
        smem = std::max(smem, interp_smem_bytes(x.g, sizeof(T)));
    }
    if (smem > 220 * 1024) return SPME_ERR_UNSUPPORTED;
    cudaFree(b->d_cnt1);
    cudaFree(b->d_off1);
    b->d_cnt1 = b->d_off1 = nullptr;
    b->ntile_keys = off;
    BTRY(balloc(&b->d_cnt1, sizeof(int) * off));
    BTRY(balloc(&b->d_off1, sizeof(int) * (off + 1)));
    // systems ordered by p, one work list (and prefix) per order
    std::vector<int> order(b->nsys);
    for (int k = 0; k < b->nsys; k++) order[k] = k;
    std::stable_sort(order.begin(), order.end(), [&](int i, int j) {
        return b->sys[i].s.porder < b->sys[j].s.porder;
    });
    b->igroups.clear();
    std::vector<InterpSys<T>> is(b->nsys);
    std::vector<int> pre;
    pre.reserve(b->nsys + 3);
    for (int q = 0; q < b->nsys; q++) {
        const int k = order[q];
        const BatchSys &x = b->sys[k];
        if (b->igroups.empty() || b->sys[order[q - 1]].s.porder != x.s.porder) {
            typename _spme_batch_t::InterpGroup grp;
            grp.first = q;
            grp.pre_off = (int)pre.size();
            b->igroups.push_back(grp);
            pre.push_back(0);
        }
        auto &grp = b->igroups.back();
        grp.count++;
        grp.smem = std::max(grp.smem, interp_smem_bytes(x.g, sizeof(T)));
        InterpArgs<T> &A = is[q].args;
        A.tile_off = b->d_off1 + x.tile_off;
        A.rec_idx = b->d_ridx1;
        A.rec_start = b->d_rst1;
        A.rec_w = (const T *)b->d_rw1;
        A.mesh = (const T *)b->d_mesh + x.mesh_off;
        A.W = (T *)b->d_W2;
        A.err = b->d_err;
        A.g = x.g;
        A.C = b->C;
        A.cb = 0;
        A.ce = b->C;
        A.accumulate = 0;
        // TMA boxes where the mesh rows allow them (K a multiple of 16 bytes / elem);
        // plain-load staging otherwise
        A.use_tma = make_interp_box(&is[q].tmap, A.mesh, b->C, x.g, sizeof(T)) ? 1 : 0;
        A.ws = b->ws;
        grp.total += x.g.ntx * x.g.nty * x.g.ntz;
        pre.push_back(grp.total);
    }
    // orders are 4, 6 or 8 (validate_sys): at most three groups, nsys + 3 prefix entries
    if (pre.size() > (size_t)b->nsys + 3) return SPME_ERR_INVALID;
    BTRY_CUDA(cudaMemcpy(b->d_interp_sys, is.data(), sizeof(InterpSys<T>) * b->nsys,
                         cudaMemcpyHostToDevice));
    BTRY_CUDA(cudaMemcpy(b->d_pre_interp, pre.data(), sizeof(int) * pre.size(),
                         cudaMemcpyHostToDevice));
    std::vector<BatchGeo> geo(b->nsys);
    for (int k = 0; k < b->nsys; k++) {
        const BatchSys &x = b->sys[k];
        geo[k] = BatchGeo{x.g, x.nc, x.p_off, x.tile_off, x.start_off, x.cell_off};
    }
    BTRY_CUDA(cudaMemcpy(b->d_geo, geo.data(), sizeof(BatchGeo) * b->nsys,
                         cudaMemcpyHostToDevice));
    b->have_pos = false;
    return SPME_OK;
}

template <typename T>
int create_t(_spme_batch_t *b) {
    const int n = b->ntot, C = b->C, ns = b->nsys;
    b->ws = record_stride<T>(b);
    // offsets of keys, meshes (grouped by K) and tables
    int start = 0, cell = 0;
    for (BatchSys &x : b->sys) {
        x.start_off = start;
        start += x.s.dim * x.s.dim * x.s.dim;
        x.cell_off = cell;
        cell += x.nc * x.nc * x.nc;
    }
    b->nstart_keys = start;
    b->ncell_keys = cell;
    std::map<int, std::vector<int>> byK;
    for (int k = 0; k < ns; k++) byK[b->sys[k].s.dim].push_back(k);
    size_t mesh = 0, spec = 0, tab = 0;
    for (auto &kv : byK) {
        FftGroup grp;
        grp.K = kv.first;
        grp.mesh_off = mesh;
        grp.spec_off = spec;
        grp.nsys = (int)kv.second.size();
        const size_t K = (size_t)kv.first, K3 = K * K * K, Kc = K * K * (K / 2 + 1);
        for (int k : kv.second) {
            b->sys[k].mesh_off = mesh;
            b->sys[k].spec_off = spec;
            b->sys[k].tab_off = tab;
            mesh += (size_t)C * K3;
            spec += (size_t)C * Kc;
            tab += Kc;
        }
        b->groups.push_back(grp);
    }
    // device buffers
    BTRY(balloc(&b->d_sysid, sizeof(int) * n));
    BTRY(balloc(&b->d_pref, sizeof(int) * (ns + 1)));
    BTRY(balloc(&b->d_geo, sizeof(BatchGeo) * ns));
    BTRY(balloc(&b->d_key1, sizeof(int) * n));
    BTRY(balloc(&b->d_key2, sizeof(int) * n));
    BTRY(balloc(&b->d_key3, sizeof(int) * n));
    BTRY(balloc(&b->d_sort_tmp, sizeof(int) * n));
    BTRY(balloc(&b->d_cnt2, sizeof(int) * start));
    BTRY(balloc(&b->d_off2, sizeof(int) * (start + 1)));
    BTRY(balloc(&b->d_cnt3, sizeof(int) * cell));
    BTRY(balloc(&b->d_off3, sizeof(int) * (cell + 1)));
    BTRY(balloc(&b->d_perm1, sizeof(int) * n));
    BTRY(balloc(&b->d_perm2, sizeof(int) * n));
    BTRY(balloc(&b->d_perm3, sizeof(int) * n));
    BTRY(balloc(&b->d_pstart, sizeof(uint32_t) * n));
    BTRY(balloc(&b->d_pfrac, sizeof(T) * 3 * n));
    BTRY(balloc(&b->d_prel, sizeof(typename V4T<T>::type) * n));
    BTRY(balloc(&b->d_cpos, sizeof(typename V4T<T>::type) * n));
    BTRY(balloc(&b->d_ridx1, sizeof(int) * n));
    BTRY(balloc(&b->d_ridx2, sizeof(int) * n));
    BTRY(balloc(&b->d_rst1, sizeof(uint32_t) * n));
    BTRY(balloc(&b->d_rst2, sizeof(uint32_t) * n));
    BTRY(balloc(&b->d_rw1, sizeof(T) * (size_t)b->ws * n));
    BTRY(balloc(&b->d_rw2, sizeof(T) * (size_t)b->ws * n));
    BTRY(balloc(&b->d_F, sizeof(T) * (size_t)C * n));
    BTRY(balloc(&b->d_Fs, sizeof(T) * (size_t)spread_cols_row_width(C) * n));
    BTRY(balloc(&b->d_W, sizeof(T) * (size_t)C * n));
    BTRY(balloc(&b->d_W2, sizeof(T) * (size_t)C * n));
    BTRY(balloc(&b->d_mesh, sizeof(T) * mesh));
    BTRY(balloc(&b->d_spec, 2 * sizeof(T) * spec));
    BTRY(balloc(&b->d_tab, 2 * sizeof(T) * tab));
    BTRY(balloc(&b->d_err, sizeof(int)));
    BTRY_CUDA(cudaMemset(b->d_err, 0, sizeof(int)));
    // (the tile keys, counted later, are never more than the stencil-start cells)
    BTRY(balloc(&b->d_scan_tmp, sizeof(int) * scan_tmp_elems(std::max(start, cell))));
    BTRY(balloc(&b->d_spread_sys, sizeof(SpreadColsSys<T>) * ns));
    BTRY(balloc(&b->d_interp_sys, sizeof(InterpSys<T>) * ns));
    BTRY(balloc(&b->d_real_sys, sizeof(RealArgs<T>) * ns));
    BTRY(balloc(&b->d_infl_sys, sizeof(InflSys) * ns));
    BTRY(balloc(&b->d_pre_spread, sizeof(int) * (ns + 1)));
    BTRY(balloc(&b->d_pre_interp, sizeof(int) * (ns + 3)));  // a prefix per order group
    BTRY(balloc(&b->d_pre_real, sizeof(int) * (ns + 1)));
    BTRY(balloc(&b->d_pre_infl, sizeof(int) * (ns + 1)));

    // system of every particle, particle prefix
    std::vector<int> sid(n), pref(ns + 1, 0);
    for (int k = 0; k < ns; k++) {
        pref[k + 1] = pref[k] + b->sys[k].s.np;
        std::fill(sid.begin() + pref[k], sid.begin() + pref[k + 1], k);
    }
    BTRY_CUDA(cudaMemcpy(b->d_sysid, sid.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
    BTRY_CUDA(cudaMemcpy(b->d_pref, pref.data(), sizeof(int) * (ns + 1), cudaMemcpyHostToDevice));

    // influence tables (FP64 moduli, one table per system)
    double *d_bm = nullptr;
    int Kmax = 2;
    for (const BatchSys &x : b->sys) Kmax = std::max(Kmax, x.s.dim);
    BTRY(balloc(&d_bm, sizeof(double) * Kmax));
    for (const BatchSys &x : b->sys) {
        std::vector<double> bm;
        host_moduli2(x.s.dim, x.s.porder, bm);
        cudaError_t e = cudaMemcpy(d_bm, bm.data(), sizeof(double) * x.s.dim, cudaMemcpyHostToDevice);
        if (e == cudaSuccess) {
            launch_influence_table<T>((T *)b->d_tab + 2 * x.tab_off, d_bm, x.s.dim, x.s.box_size,
                                      x.s.xi, x.s.radius, b->stream);
            b->launches++;
            e = cudaStreamSynchronize(b->stream);
        }
        if (e != cudaSuccess) {
            cudaFree(d_bm);
            return from_cuda(e);
        }
    }
    cudaFree(d_bm);

    // FP64 batches: the pair functions from per-system Chebyshev tables
    std::vector<PairTable> ptab(ns);
    if (sizeof(T) == 8) {
        std::vector<std::vector<double>> coefs(ns);
        size_t total = 0;
        std::vector<size_t> at(ns, 0);
        for (int k = 0; k < ns; k++) {
            const BatchSys &x = b->sys[k];
            if (build_pair_table(x.s.xi, x.s.radius, x.s.rcut, &coefs[k], &ptab[k])) {
                at[k] = total;
                total += coefs[k].size();
            } else {
                ptab[k] = PairTable{};
            }
        }
        if (total) {
            BTRY(balloc(&b->d_pair, sizeof(double) * total));
            for (int k = 0; k < ns; k++)
                if (!coefs[k].empty()) {
                    BTRY_CUDA(cudaMemcpy(b->d_pair + at[k], coefs[k].data(),
                                         sizeof(double) * coefs[k].size(), cudaMemcpyHostToDevice));
                    ptab[k].coef = b->d_pair + at[k];
                }
        }
    }

    // work lists that do not depend on the tile
    std::vector<SpreadColsSys<T>> ss(ns);
    std::vector<RealArgs<T>> rs(ns);
    std::vector<InflSys> fs(ns);
    std::vector<int> ps(ns + 1, 0), pr(ns + 1, 0), pf(ns + 1, 0);
    const int RW = spread_cols_row_width(C);
    for (int k = 0; k < ns; k++) {
        const BatchSys &x = b->sys[k];
        const int K = x.s.dim;
        const int TZ = sizeof(T) == 4 ? 16 : 8;
        ss[k].args = SpreadColsArgs<T>{b->d_off2 + x.start_off, b->d_rst2, (const T *)b->d_rw2,
                                       (const T *)b->d_Fs, (T *)b->d_mesh + x.mesh_off, C, RW, K,
                                       (K + TZ - 1) / TZ, b->ws};
        ss[k].p = x.s.porder;
        ss[k].gx = (K + 15) / 16;
        ps[k + 1] = ps[k] + spread_cols_blocks(K, C, sizeof(T));
        rs[k] = real_args<T>(x.nc, b->d_off3 + x.cell_off, b->d_perm3, b->d_cpos, (const T *)b->d_F,
                             b->R, x.s.box_size, x.s.rcut, x.s.xi, x.s.radius, 1, ptab[k],
                             (T *)b->d_W);
        pr[k + 1] = pr[k] + x.nc * x.nc * x.nc;
        const size_t Kc = (size_t)K * K * (K / 2 + 1);
        fs[k].K = K;
        fs[k].nb_int = (int)((Kc + 255) / 256);
        fs[k].spec_off = x.spec_off;
        fs[k].tab_off = x.tab_off;
        fs[k].twopi_L = 2.0 * M_PI / x.s.box_size;
        const int nplane = ((K & 1) ? 1 : 2) * K * K;
        pf[k + 1] = pf[k] + fs[k].nb_int + (nplane + 255) / 256;
    }
    b->tot_spread = ps[ns];
    b->tot_real = pr[ns];
    b->tot_infl = pf[ns];
    BTRY_CUDA(cudaMemcpy(b->d_spread_sys, ss.data(), sizeof(SpreadColsSys<T>) * ns, cudaMemcpyHostToDevice));
    BTRY_CUDA(cudaMemcpy(b->d_real_sys, rs.data(), sizeof(RealArgs<T>) * ns, cudaMemcpyHostToDevice));
    BTRY_CUDA(cudaMemcpy(b->d_infl_sys, fs.data(), sizeof(InflSys) * ns, cudaMemcpyHostToDevice));
    BTRY_CUDA(cudaMemcpy(b->d_pre_spread, ps.data(), sizeof(int) * (ns + 1), cudaMemcpyHostToDevice));
    BTRY_CUDA(cudaMemcpy(b->d_pre_real, pr.data(), sizeof(int) * (ns + 1), cudaMemcpyHostToDevice));
    BTRY_CUDA(cudaMemcpy(b->d_pre_infl, pf.data(), sizeof(int) * (ns + 1), cudaMemcpyHostToDevice));

    // one batched 3D plan pair per mesh size
    size_t wsz = 0;
    const cufftType tf = sizeof(T) == 4 ? CUFFT_R2C : CUFFT_D2Z;
    const cufftType tb = sizeof(T) == 4 ? CUFFT_C2R : CUFFT_Z2D;
    for (FftGroup &grp : b->groups) {
        const int K = grp.K;
        int nn[3] = {K, K, K}, re[3] = {K, K, K}, ce[3] = {K, K, K / 2 + 1};
        const int K3 = K * K * K, Kc = K * K * (K / 2 + 1);
        size_t w1 = 0, w2 = 0;
        if (cufftCreate(&grp.fwd) != CUFFT_SUCCESS || cufftCreate(&grp.bwd) != CUFFT_SUCCESS)
            return SPME_ERR_CUFFT;
        cufftSetAutoAllocation(grp.fwd, 0);
        cufftSetAutoAllocation(grp.bwd, 0);
        if (cufftMakePlanMany(grp.fwd, 3, nn, re, 1, K3, ce, 1, Kc, tf, C * grp.nsys, &w1) !=
                CUFFT_SUCCESS ||
            cufftMakePlanMany(grp.bwd, 3, nn, ce, 1, Kc, re, 1, K3, tb, C * grp.nsys, &w2) !=
                CUFFT_SUCCESS)
            return SPME_ERR_CUFFT;
        wsz = std::max({wsz, w1, w2});
    }
    for (void *&w : b->d_works) BTRY(balloc(&w, wsz));
    BTRY(build_tiles<T>(b));
    BTRY_CUDA(cudaStreamSynchronize(b->stream));
    return SPME_OK;
}

// Stage boundary k (0 .. kStages) when profiling.
void mark(_spme_batch_t *b, int k) {
    if (b->profiling) cudaEventRecord(b->ev[k], b->stream);
}

template <typename T>
int positions_body(_spme_batch_t *b, const double *pos) {
    cudaStream_t s = b->stream;
    const int n = b->ntot;
    mark(b, 0);
    BTRY_CUDA(cudaMemsetAsync(b->d_cnt1, 0, sizeof(int) * b->ntile_keys, s));
    BTRY_CUDA(cudaMemsetAsync(b->d_cnt2, 0, sizeof(int) * b->nstart_keys, s));
    BTRY_CUDA(cudaMemsetAsync(b->d_cnt3, 0, sizeof(int) * b->ncell_keys, s));
    k_batch_keys<T><<<nblk(n, 256), 256, 0, s>>>(
        pos, n, b->d_sysid, b->d_geo, b->d_key1, b->d_cnt1, b->d_perm1, b->d_key2, b->d_cnt2,
        b->d_perm2, b->d_key3, b->d_cnt3, b->d_perm3, b->d_pstart, (T *)b->d_pfrac,
        (typename V4T<T>::type *)b->d_prel);
    launch_scan(b->d_cnt1, b->ntile_keys, b->d_off1, b->d_scan_tmp, s);
    launch_scatter(b->d_key1, b->d_off1, n, b->d_perm1, b->d_sort_tmp, s);
    launch_scan(b->d_cnt2, b->nstart_keys, b->d_off2, b->d_scan_tmp, s);
    launch_scatter(b->d_key2, b->d_off2, n, b->d_perm2, b->d_sort_tmp, s);
    launch_scan(b->d_cnt3, b->ncell_keys, b->d_off3, b->d_scan_tmp, s);
    launch_scatter(b->d_key3, b->d_off3, n, b->d_perm3, b->d_sort_tmp, s);
    k_batch_records<T><<<nblk(n, kRecThreads), kRecThreads, 0, s>>>(b->d_pstart, (const T *)b->d_pfrac,
                                                    b->d_perm1, n, b->d_sysid, b->d_geo, b->ws,
                                                    b->d_ridx1, b->d_rst1, (T *)b->d_rw1);
    k_batch_records<T><<<nblk(n, kRecThreads), kRecThreads, 0, s>>>(b->d_pstart, (const T *)b->d_pfrac,
                                                    b->d_perm2, n, b->d_sysid, b->d_geo, b->ws,
                                                    b->d_ridx2, b->d_rst2, (T *)b->d_rw2);
    launch_cell_gather(b->d_prel, b->d_perm3, n, sizeof(T) == 4, b->d_cpos, s);
    b->launches += 1 + 3 * 3 + 3 * 2 + 2 + 1;
    return from_cuda(cudaGetLastError());
}

// One direction of every group's transform: groups round-robin on the FFT
// streams (forked from and joined back to the batch's stream), or all on the
// batch's stream.
template <typename T>
int run_ffts(_spme_batch_t *b, bool inverse, bool conc) {
    cudaStream_t s = b->stream;
    const int ns = conc ? _spme_batch_t::kFftStreams : 1;
    if (conc) {
        BTRY_CUDA(cudaEventRecord(b->ev_fork, s));
        for (int j = 0; j < ns; j++) BTRY_CUDA(cudaStreamWaitEvent(b->fft_stream[j], b->ev_fork, 0));
    }
    for (size_t q = 0; q < b->groups.size(); q++) {
        FftGroup &grp = b->groups[q];
        const int j = (int)(q % ns);
        cufftHandle h = inverse ? grp.bwd : grp.fwd;
        if (cufftSetStream(h, conc ? b->fft_stream[j] : s) != CUFFT_SUCCESS ||
            cufftSetWorkArea(h, b->d_works[j]) != CUFFT_SUCCESS)
            return SPME_ERR_CUFFT;
        T *mesh = (T *)b->d_mesh + grp.mesh_off, *spec = (T *)b->d_spec + 2 * grp.spec_off;
        cufftResult r;
        if (sizeof(T) == 4)
            r = inverse ? cufftExecC2R(h, (cufftComplex *)spec, (cufftReal *)mesh)
                        : cufftExecR2C(h, (cufftReal *)mesh, (cufftComplex *)spec);
        else
            r = inverse ? cufftExecZ2D(h, (cufftDoubleComplex *)spec, (cufftDoubleReal *)mesh)
                        : cufftExecD2Z(h, (cufftDoubleReal *)mesh, (cufftDoubleComplex *)spec);
        if (r != CUFFT_SUCCESS) return SPME_ERR_CUFFT;
    }
    if (conc)
        for (int j = 0; j < ns; j++) {
            BTRY_CUDA(cudaEventRecord(b->ev_fft_join[j], b->fft_stream[j]));
            BTRY_CUDA(cudaStreamWaitEvent(s, b->ev_fft_join[j], 0));
        }
    return SPME_OK;
}

template <typename T>
int apply_body(_spme_batch_t *b, double alpha, const T *f, double beta, T *u) {
    cudaStream_t s = b->stream;
    const int n = b->ntot, C = b->C;
    const long total = (long)n * C;
    mark(b, 1);  // (the position build, when it ran, ends here)
    k_batch_pack<T><<<grid_cap(n, 256, 8), 256, 0, s>>>(f, b->d_pref, b->nsys, b->R, n,
                                                       (T *)b->d_F);
    mark(b, 2);
    // the real-space sum beside the mesh pipeline when asked (serially when
    // profiling, so that every stage is timed alone)
    const bool conc = !b->profiling && (b->overlap & 1);
    cudaStream_t rss = conc ? b->rs_stream : s;
    if (conc) {
        BTRY_CUDA(cudaEventRecord(b->ev_fork, s));
        BTRY_CUDA(cudaStreamWaitEvent(rss, b->ev_fork, 0));
    }
    BTRY_CUDA(launch_realspace_batch<T>((const RealArgs<T> *)b->d_real_sys, b->d_pre_real,
                                        b->nsys, b->tot_real, rss));
    if (conc) BTRY_CUDA(cudaEventRecord(b->ev_rs_join, rss));
    mark(b, 3);
    launch_gather_cols_rows<T>((const T *)b->d_F, b->d_ridx2, n, C, (T *)b->d_Fs, s);
    BTRY_CUDA(launch_spread_cols_batch<T>((const SpreadColsSys<T> *)b->d_spread_sys,
                                          b->d_pre_spread, b->nsys, b->tot_spread, C, s));
    mark(b, 4);
    const bool fconc = !b->profiling && (b->overlap & 2);
    BTRY(run_ffts<T>(b, false, fconc));
    mark(b, 5);
    k_batch_influence<T><<<grid_cap((long)b->tot_infl * 256, 256, 8), 256, 0, s>>>(
        (Cx2<T> *)b->d_spec, (const T *)b->d_tab, b->d_infl_sys, b->d_pre_infl, b->nsys,
        b->tot_infl, b->R);
    mark(b, 6);
    BTRY(run_ffts<T>(b, true, fconc));
    mark(b, 7);
    // the kernel's shared-memory limit covers every group (a captured graph replays
    // all the launches against the limit last set)
    size_t smem_max = 0;
    for (const auto &grp : b->igroups) smem_max = std::max(smem_max, grp.smem);
    for (const auto &grp : b->igroups)
        BTRY_CUDA(launch_interp_batch<T>((const InterpSys<T> *)b->d_interp_sys + grp.first,
                                         b->d_pre_interp + grp.pre_off, grp.count, grp.total,
                                         grp.smem, s, smem_max));
    mark(b, 8);
    if (conc) BTRY_CUDA(cudaStreamWaitEvent(s, b->ev_rs_join, 0));
    k_batch_unpack<T><<<grid_cap(n, 256, 8), 256, 0, s>>>(
        (const T *)b->d_W, (const T *)b->d_W2, b->d_pref, b->nsys, b->R, n, (T)alpha,
        (T)beta, u);
    mark(b, 9);
    b->stages_valid = b->profiling;
    b->launches += 6 + (long)b->igroups.size();
    return from_cuda(cudaGetLastError());
}

int step_body(_spme_batch_t *b, const double *pos, double alpha, const void *f, double beta,
              void *u) {
    if (b->precision == SPME_FP32) {
        if (pos) BTRY(positions_body<float>(b, pos));
        return apply_body<float>(b, alpha, (const float *)f, beta, (float *)u);
    }
    if (pos) BTRY(positions_body<double>(b, pos));
    return apply_body<double>(b, alpha, (const double *)f, beta, (double *)u);
}

void drop_graph(_spme_batch_t *b) {
    if (b->gexec) cudaGraphExecDestroy(b->gexec);
    b->gexec = nullptr;
}

void destroy_b(_spme_batch_t *b) {
    if (!b) return;
    int prev = -1;
    cudaGetDevice(&prev);
    if (prev != b->device) cudaSetDevice(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->own_stream) cudaStreamSynchronize(b->own_stream);
    drop_graph(b);
    for (FftGroup &g : b->groups) {
        if (g.fwd) cufftDestroy(g.fwd);
        if (g.bwd) cufftDestroy(g.bwd);
    }
    void *bufs[] = {b->d_sysid, b->d_pref,  b->d_geo,   b->d_key1,  b->d_key2,
                    b->d_key3,  b->d_sort_tmp, b->d_cnt1,  b->d_off1,  b->d_cnt2,
                    b->d_off2,  b->d_cnt3,  b->d_off3,  b->d_scan_tmp, b->d_perm1, b->d_perm2,
                    b->d_perm3, b->d_pstart, b->d_pfrac, b->d_prel, b->d_cpos,  b->d_ridx1,
                    b->d_ridx2, b->d_rst1,  b->d_rst2,  b->d_rw1,   b->d_rw2,   b->d_F,
                    b->d_Fs,    b->d_W,     b->d_W2,    b->d_mesh,  b->d_spec,  b->d_tab,
                    b->d_pair,  b->d_err,   b->d_spread_sys, b->d_interp_sys,
                    b->d_real_sys, b->d_infl_sys, b->d_pre_spread, b->d_pre_interp,
                    b->d_pre_real, b->d_pre_infl};
    for (void *p : bufs)
        if (p) cudaFree(p);
    for (void *w : b->d_works)
        if (w) cudaFree(w);
    for (cudaEvent_t e : b->ev)
        if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : b->ev_fft_join)
        if (e) cudaEventDestroy(e);
    if (b->ev_fork) cudaEventDestroy(b->ev_fork);
    if (b->ev_rs_join) cudaEventDestroy(b->ev_rs_join);
    for (cudaStream_t x : b->fft_stream)
        if (x) cudaStreamDestroy(x);
    if (b->rs_stream) cudaStreamDestroy(b->rs_stream);
    if (b->own_stream) cudaStreamDestroy(b->own_stream);
    if (prev >= 0 && prev != b->device) cudaSetDevice(prev);
    delete b;
}

struct DevGuard {
    int prev = -1;
    explicit DevGuard(int dev) {
        if (cudaGetDevice(&prev) == cudaSuccess && prev != dev) cudaSetDevice(dev);
        else prev = -1;
    }
    ~DevGuard() {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

int create_streams(_spme_batch_t *b) {
    BTRY_CUDA(cudaStreamCreateWithFlags(&b->own_stream, cudaStreamNonBlocking));
    b->stream = b->own_stream;
    BTRY_CUDA(cudaStreamCreateWithFlags(&b->rs_stream, cudaStreamNonBlocking));
    for (int j = 0; j < _spme_batch_t::kFftStreams; j++) {
        BTRY_CUDA(cudaStreamCreateWithFlags(&b->fft_stream[j], cudaStreamNonBlocking));
        BTRY_CUDA(cudaEventCreateWithFlags(&b->ev_fft_join[j], cudaEventDisableTiming));
    }
    BTRY_CUDA(cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming));
    BTRY_CUDA(cudaEventCreateWithFlags(&b->ev_rs_join, cudaEventDisableTiming));
    for (cudaEvent_t &e : b->ev) BTRY_CUDA(cudaEventCreate(&e));
    return SPME_OK;
}

}  // namespace

extern "C" {

int spme_batch_create(const spme_batch_system *systems, int count, int nrhs, int precision,
                      spme_batch_t **out) {
    if (!out) return SPME_ERR_INVALID;
    *out = nullptr;
    if (!systems || count < 1 || nrhs < 1 || nrhs > 1024) return SPME_ERR_INVALID;
    if (precision != SPME_FP32 && precision != SPME_FP64) return SPME_ERR_INVALID;
    long long ntot = 0;
    for (int k = 0; k < count; k++) {
        BTRY(validate_sys(systems[k], precision));
        ntot += systems[k].np;
    }
    if (ntot * 3LL * nrhs >= (1LL << 31)) return SPME_ERR_UNSUPPORTED;
    _spme_batch_t *b = new (std::nothrow) _spme_batch_t();
    if (!b) return SPME_ERR_NOMEM;
    cudaGetDevice(&b->device);
    b->precision = precision;
    b->elem = precision == SPME_FP32 ? 4 : 8;
    b->R = nrhs;
    b->C = 3 * nrhs;
    b->nsys = count;
    b->ntot = (int)ntot;
    b->sys.resize(count);
    int off = 0;
    for (int k = 0; k < count; k++) {
        b->sys[k].s = systems[k];
        b->sys[k].nc = real_cells(systems[k]);
        b->sys[k].p_off = off;
        off += systems[k].np;
    }
    int st = create_streams(b);
    if (st == SPME_OK) st = precision == SPME_FP32 ? create_t<float>(b) : create_t<double>(b);
    if (st != SPME_OK) {
        destroy_b(b);
        return st;
    }
    *out = b;
    return SPME_OK;
}

int spme_batch_destroy(spme_batch_t *b) {
    destroy_b(b);
    return SPME_OK;
}

int spme_batch_set_stream(spme_batch_t *b, void *stream) {
    if (!b) return SPME_ERR_INVALID;
    b->stream = (cudaStream_t)stream;  // NULL: the legacy default stream
    return SPME_OK;
}

void *spme_batch_get_stream(const spme_batch_t *b) { return b ? (void *)b->stream : nullptr; }

int spme_batch_set_tile(spme_batch_t *b, int tx, int ty, int tz) {
    if (!b) return SPME_ERR_INVALID;
    if (tx < 4 || ty < 4 || tz < 4 || tx > kMaxTile || ty > kMaxTile || tz > 8)
        return SPME_ERR_INVALID;
    DevGuard dg(b->device);
    BTRY_CUDA(cudaStreamSynchronize(b->stream));
    drop_graph(b);
    const int old[3] = {b->tile[0], b->tile[1], b->tile[2]};
    b->tile[0] = tx;
    b->tile[1] = ty;
    b->tile[2] = tz;
    const int st = b->precision == SPME_FP32 ? build_tiles<float>(b) : build_tiles<double>(b);
    if (st != SPME_OK) {
        std::memcpy(b->tile, old, sizeof(old));
        if (b->precision == SPME_FP32) build_tiles<float>(b);
        else build_tiles<double>(b);
    }
    return st;
}

int spme_batch_set_positions(spme_batch_t *b, const double *pos) {
    if (!b || !pos) return SPME_ERR_INVALID;
    DevGuard dg(b->device);
    const int st = b->precision == SPME_FP32 ? positions_body<float>(b, pos)
                                             : positions_body<double>(b, pos);
    if (st == SPME_OK) b->have_pos = true;
    return st;
}

int spme_batch_apply(spme_batch_t *b, double alpha, const void *f, double beta, void *u) {
    if (!b || !f || !u) return SPME_ERR_INVALID;
    if (!b->have_pos) return SPME_ERR_STATE;
    DevGuard dg(b->device);
    return b->precision == SPME_FP32
               ? apply_body<float>(b, alpha, (const float *)f, beta, (float *)u)
               : apply_body<double>(b, alpha, (const double *)f, beta, (double *)u);
}

int spme_batch_step(spme_batch_t *b, const double *pos, double alpha, const void *f, double beta,
                    void *u) {
    if (!b || !pos || !f || !u) return SPME_ERR_INVALID;
    DevGuard dg(b->device);
    if (!b->use_graphs) {
        const int st = step_body(b, pos, alpha, f, beta, u);
        if (st == SPME_OK) b->have_pos = true;
        return st;
    }
    if (b->gexec && b->g_pos == pos && b->g_f == f && b->g_u == u && b->g_alpha == alpha &&
        b->g_beta == beta && b->g_stream == b->stream) {
        BTRY_CUDA(cudaGraphLaunch(b->gexec, b->stream));
        b->launches += b->g_launches;
        return SPME_OK;
    }
    // capture on the batch's stream (on a side stream, ordered after the legacy
    // default stream's earlier work, when the batch runs on that stream)
    const cudaStream_t orig = b->stream;
    cudaStream_t side = nullptr;
    if (!orig) {
        BTRY_CUDA(cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking));
        BTRY_CUDA(cudaEventRecord(b->ev_fork, nullptr));
        BTRY_CUDA(cudaStreamWaitEvent(side, b->ev_fork, 0));
        b->stream = side;
    }
    const cudaStream_t cs = b->stream;
    const long l0 = b->launches;
    const bool prof = b->profiling;
    b->profiling = false;  // no stage events inside a graph
    cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    int st = e == cudaSuccess ? step_body(b, pos, alpha, f, beta, u) : from_cuda(e);
    cudaGraph_t graph = nullptr;
    if (e == cudaSuccess) {
        e = cudaStreamEndCapture(cs, &graph);
        if (st == SPME_OK && e != cudaSuccess) st = from_cuda(e);
    }
    b->profiling = prof;
    cudaGraphExec_t exec = nullptr;
    if (st == SPME_OK) st = from_cuda(cudaGraphInstantiate(&exec, graph, 0));
    if (graph) cudaGraphDestroy(graph);
    if (st == SPME_OK) {
        drop_graph(b);
        b->gexec = exec;
        b->g_launches = b->launches - l0;
        b->g_pos = pos;
        b->g_f = f;
        b->g_u = u;
        b->g_alpha = alpha;
        b->g_beta = beta;
        b->g_stream = orig;
        st = from_cuda(cudaGraphLaunch(b->gexec, cs));
    }
    b->launches = l0;
    if (st == SPME_OK) {
        b->launches += b->g_launches;
        b->have_pos = true;
    }
    if (side) {
        // the legacy default stream waits for the replay on the side stream
        cudaEventRecord(b->ev_fork, side);
        cudaStreamWaitEvent(nullptr, b->ev_fork, 0);
        cudaStreamSynchronize(side);
        cudaStreamDestroy(side);
        b->stream = orig;
    }
    return st;
}

int spme_batch_set_graphs(spme_batch_t *b, int on) {
    if (!b) return SPME_ERR_INVALID;
    DevGuard dg(b->device);
    BTRY_CUDA(cudaStreamSynchronize(b->stream));
    drop_graph(b);
    b->use_graphs = on != 0;
    return SPME_OK;
}

int spme_batch_set_overlap(spme_batch_t *b, int mode) {
    if (!b || mode < 0 || mode > 3) return SPME_ERR_INVALID;
    DevGuard dg(b->device);
    BTRY_CUDA(cudaStreamSynchronize(b->stream));
    drop_graph(b);
    b->overlap = mode;
    return SPME_OK;
}

int spme_batch_synchronize(spme_batch_t *b) {
    if (!b) return SPME_ERR_INVALID;
    DevGuard dg(b->device);
    BTRY_CUDA(cudaStreamSynchronize(b->stream));
    int h = 0;
    BTRY_CUDA(cudaMemcpy(&h, b->d_err, sizeof(int), cudaMemcpyDeviceToHost));
    if (h) {
        cudaMemset(b->d_err, 0, sizeof(int));
        return SPME_ERR_KERNEL;
    }
    return SPME_OK;
}

long spme_batch_launch_count(const spme_batch_t *b) { return b ? b->launches : 0; }

long spme_batch_particles(const spme_batch_t *b) { return b ? (long)b->ntot : 0; }

int spme_batch_set_profiling(spme_batch_t *b, int on) {
    if (!b) return SPME_ERR_INVALID;
    b->profiling = on != 0;
    b->stages_valid = false;
    return SPME_OK;
}

int spme_batch_stage_times(const spme_batch_t *b, float *ms, int n) {
    if (!b || !ms || n < 0 || !b->stages_valid) return 0;
    DevGuard dg(b->device);
    if (cudaEventSynchronize(b->ev[_spme_batch_t::kStages]) != cudaSuccess) return 0;
    const int m = std::min(n, (int)_spme_batch_t::kStages);
    for (int k = 0; k < m; k++) {
        float t = 0.f;
        cudaEventElapsedTime(&t, b->ev[k], b->ev[k + 1]);
        ms[k] = t;
    }
    return m;
}

}  // extern "C"
