// P-build: stencil starts, tile / cell keys, counting sorts and B-spline
// records (restates old-version/spme.c:158-297 in factored form: p weights per
// axis instead of the dense p^3 P matrix and index list).
#include "kernels.h"

namespace spme {

namespace {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

__global__ void k_cell_keys(const double *__restrict__ pos, int n, double L, int nc,
                            int *__restrict__ key, int *__restrict__ count,
                            int *__restrict__ slot) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double invL = 1.0 / L;
    int c[3];
#pragma unroll
    for (int d = 0; d < 3; d++) {
        double xw;
        c[d] = cell_coord(pos[3 * i + d], L, invL, nc, xw);
    }
    int k = (c[2] * nc + c[1]) * nc + c[0];
    key[i] = k;
    slot[i] = atomicAdd(&count[k], 1);
}

// All sort keys of a position build in one pass over the positions: the mesh
// tile of the stencil start (always), the stencil-start cell (key2, when
// count2 is set) and the real-space cell (key3, when count3 is set), each with
// its slot from an atomic count.
// ... and, when the mesh keys are wanted, each particle's packed stencil start
// and fractional mesh coordinates (read by the record builds), and with the cell
// key its position relative to its cell's lower corner (gathered into cell
// order later), so the FP64 coordinate arithmetic runs once per particle.
template <typename T> struct Vec4T;
template <> struct Vec4T<float> { using type = float4; };
template <> struct Vec4T<double> { using type = double4_32a; };

template <typename T>
__global__ void k_all_keys(const double *__restrict__ pos, int n, MeshGeom g, int nc,
                           int *__restrict__ key1, int *__restrict__ count1,
                           int *__restrict__ slot1, int *__restrict__ key2,
                           int *__restrict__ count2, int *__restrict__ slot2,
                           int *__restrict__ key3, int *__restrict__ count3,
                           int *__restrict__ slot3, uint32_t *__restrict__ pstart,
                           T *__restrict__ pfrac, typename Vec4T<T>::type *__restrict__ prel) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int s[3] = {0, 0, 0}, cc[3] = {0, 0, 0};
    double fr[3] = {0.0, 0.0, 0.0}, rel[3] = {0.0, 0.0, 0.0};
    const bool mesh = count1 || count2;  // the mesh geometry is set only then
    const double h = g.L / nc;
#pragma unroll
    for (int d = 0; d < 3; d++) {
        const double xw = wrap_coord(pos[3 * i + d], g.L, g.invL);
        if (mesh) mesh_coord_w(xw, g.invL, g.K, g.p, s[d], fr[d]);
        if (count3) {
            cc[d] = cell_coord_w(xw, g.invL, nc);
            rel[d] = xw - cc[d] * h;
        }
    }
    if (count3 && prel) {
        typename Vec4T<T>::type v;
        v.x = (T)rel[0];
        v.y = (T)rel[1];
        v.z = (T)rel[2];
        v.w = T(0);
        prel[i] = v;
    }
    if (mesh && pstart) {
        pstart[i] = pack_start(s[0], s[1], s[2]);
#pragma unroll
        for (int d = 0; d < 3; d++) pfrac[3 * i + d] = (T)fr[d];
    }
    if (count1) {
        const int k = ((s[2] / g.tz) * g.nty + s[1] / g.ty) * g.ntx + s[0] / g.tx;
        key1[i] = k;
        slot1[i] = atomicAdd(&count1[k], 1);
    }
    if (count2) {
        const int k = (s[1] * g.K + s[0]) * g.K + s[2];
        key2[i] = k;
        slot2[i] = atomicAdd(&count2[k], 1);
    }
    if (count3) {
        const int k = (cc[2] * nc + cc[1]) * nc + cc[0];
        key3[i] = k;
        slot3[i] = atomicAdd(&count3[k], 1);
    }
}

// Block-wide exclusive scan of one value per thread; returns the block total.
__device__ int block_exclusive_scan(int v, int &total) {
    __shared__ int warp_tot[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int nw = blockDim.x >> 5;
        int t = lane < nw ? warp_tot[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        if (lane < nw) warp_tot[lane] = t;  // inclusive
    }
    __syncthreads();
    int before = warp > 0 ? warp_tot[warp - 1] : 0;
    total = warp_tot[(blockDim.x >> 5) - 1];
    __syncthreads();
    return before + x - v;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_reduce(const int *__restrict__ in, int n,
                                                             int *__restrict__ sums) {
    long base = (long)blockIdx.x * kScanTile + (long)threadIdx.x * kScanItems;
    int s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++)
        if (base + k < n) s += in[base + k];
    int total;
    block_exclusive_scan(s, total);
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

// Exclusive scan of sums[0..nb) in place, one block, looping with a carry.
__global__ void __launch_bounds__(kScanThreads) k_scan_sums(int *__restrict__ sums, int nb) {
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < nb; base += kScanTile) {
        int v[kScanItems];
        int s = 0;
#pragma unroll
        for (int k = 0; k < kScanItems; k++) {
            int q = base + threadIdx.x * kScanItems + k;
            v[k] = q < nb ? sums[q] : 0;
            s += v[k];
        }
        int total;
        int ex = block_exclusive_scan(s, total) + carry;
#pragma unroll
        for (int k = 0; k < kScanItems; k++) {
            int q = base + threadIdx.x * kScanItems + k;
            if (q < nb) sums[q] = ex;
            ex += v[k];
        }
        __syncthreads();
        if (threadIdx.x == 0) carry += total;
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kScanThreads) k_scan_final(const int *__restrict__ in, int n,
                                                            const int *__restrict__ sums,
                                                            int *__restrict__ out) {
    long base = (long)blockIdx.x * kScanTile + (long)threadIdx.x * kScanItems;
    int v[kScanItems];
    int s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        v[k] = base + k < n ? in[base + k] : 0;
        s += v[k];
    }
    int total;
    int ex = block_exclusive_scan(s, total) + sums[blockIdx.x];
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        if (base + k < n) out[base + k] = ex;
        ex += v[k];
    }
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == blockDim.x - 1) out[n] = ex;
}

__global__ void k_scatter(const int *__restrict__ key, const int *__restrict__ slot,
                          const int *__restrict__ off, int n, int *__restrict__ perm) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    perm[off[key[i]] + slot[i]] = i;
}

// Keys holding more particles than this keep the order of the atomic slots:
// ranking a key's particles costs (its count)^2 / 32 warp steps.
constexpr int kStableMax = 16384;

// Particle v = in[q] goes to out[b + r], r its rank by particle index among
// the particles of its key [b, e): every key's particles in increasing index,
// so a position build gives the same order (and the sums over particles the
// same rounding) on every run.  Consecutive q share a key, so the lanes of a
// warp read the same entries (broadcast loads).
__global__ void k_stable_place(const int *__restrict__ key, const int *__restrict__ off,
                               const int *__restrict__ in, int n, int *__restrict__ out) {
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    const int v = in[q];
    const int k = key[v];
    const int b = off[k], e = off[k + 1];
    int r = q - b;
    if (e - b <= kStableMax) {
        r = 0;
        for (int j = b; j < e; j++) r += in[j] < v;
    }
    out[b + r] = v;
}

// The block's records are assembled in shared memory and written as one
// contiguous run of 16-byte stores: a record is WS elements (80 bytes at p = 6
// FP32), and per-thread record stores would touch a separate sector per lane.
constexpr int kRecThreads = 128;

template <typename T, int P>
__global__ void __launch_bounds__(kRecThreads)
k_records(const uint32_t *__restrict__ pstart, const T *__restrict__ pfrac,
          const int *__restrict__ perm, int n, int *__restrict__ rec_idx,
          uint32_t *__restrict__ rec_start, T *__restrict__ rec_w) {
    constexpr int WS = RecordWidth<T, P>::value;
    constexpr int VQ = WS * (int)sizeof(T) / 16;  // 16-byte pieces per record
    __shared__ __align__(16) T sm[kRecThreads * WS];
    const int s0 = blockIdx.x * kRecThreads;
    const int s = s0 + threadIdx.x;
    if (s < n) {
        const int i = perm[s];
        T row[WS];
        T w[P];
#pragma unroll
        for (int d = 0; d < 3; d++) {
            bspline_weights<T, P>(pfrac[3 * i + d], w);
#pragma unroll
            for (int j = 0; j < P; j++) row[d * P + j] = w[j];
        }
#pragma unroll
        for (int j = 3 * P; j < WS; j++) row[j] = T(0);
        rec_idx[s] = i;
        rec_start[s] = pstart[i];
        float4 *dst = reinterpret_cast<float4 *>(sm + (size_t)threadIdx.x * WS);
#pragma unroll
        for (int q = 0; q < VQ; q++) dst[q] = reinterpret_cast<const float4 *>(row)[q];
    }
    __syncthreads();
    const int cnt = min(kRecThreads, n - s0);
    float4 *out = reinterpret_cast<float4 *>(rec_w + (size_t)s0 * WS);
    const float4 *src = reinterpret_cast<const float4 *>(sm);
    for (int v = threadIdx.x; v < cnt * VQ; v += kRecThreads) out[v] = src[v];
}

// Cell-relative positions in cell order, gathered from the keys pass's output.
template <typename G4>
__global__ void k_cell_gather(const G4 *__restrict__ prel, const int *__restrict__ perm, int n,
                              G4 *__restrict__ cpos) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < n) cpos[s] = prel[perm[s]];
}

// Positions relative to the lower corner of their real-space cell.
template <typename G4, typename G>
__global__ void k_cell_positions(const double *__restrict__ pos, const int *__restrict__ perm,
                                 int n, double L, int nc, G4 *__restrict__ cpos) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    int i = perm[s];
    const double h = L / nc, invL = 1.0 / L;
    double o[3];
#pragma unroll
    for (int d = 0; d < 3; d++) {
        double xw;
        const int c = cell_coord(pos[3 * i + d], L, invL, nc, xw);
        o[d] = xw - c * h;
    }
    G4 v;
    v.x = (G)o[0];
    v.y = (G)o[1];
    v.z = (G)o[2];
    v.w = (G)0;
    cpos[s] = v;
}

inline int nblk(long n, int t) { return (int)((n + t - 1) / t); }

}  // namespace

void launch_all_keys(const double *pos, int n, const MeshGeom &g, int nc, int *key1, int *count1,
                     int *slot1, int *key2, int *count2, int *slot2, int *key3, int *count3,
                     int *slot3, uint32_t *pstart, void *pfrac, void *prel, bool fp32,
                     cudaStream_t s) {
    if (n <= 0) return;
    if (fp32)
        k_all_keys<float><<<nblk(n, 256), 256, 0, s>>>(pos, n, g, nc, key1, count1, slot1, key2,
                                                       count2, slot2, key3, count3, slot3, pstart,
                                                       (float *)pfrac, (float4 *)prel);
    else
        k_all_keys<double><<<nblk(n, 256), 256, 0, s>>>(pos, n, g, nc, key1, count1, slot1, key2,
                                                        count2, slot2, key3, count3, slot3, pstart,
                                                        (double *)pfrac, (double4_32a *)prel);
}

void launch_cell_gather(const void *prel, const int *perm, int n, bool fp32, void *cpos,
                        cudaStream_t s) {
    if (n <= 0) return;
    if (fp32)
        k_cell_gather<float4><<<nblk(n, 256), 256, 0, s>>>((const float4 *)prel, perm, n,
                                                           (float4 *)cpos);
    else
        k_cell_gather<double4_32a><<<nblk(n, 256), 256, 0, s>>>((const double4_32a *)prel, perm, n,
                                                            (double4_32a *)cpos);
}

void launch_cell_keys(const double *pos, int n, double L, int nc, int *key, int *count,
                      int *slot, cudaStream_t s) {
    if (n > 0) k_cell_keys<<<nblk(n, 256), 256, 0, s>>>(pos, n, L, nc, key, count, slot);
}

size_t scan_tmp_elems(int nkeys) { return (size_t)nblk(nkeys, kScanTile) + 1; }

void launch_scan(const int *count, int nkeys, int *off, int *tmp, cudaStream_t s) {
    int nb = nblk(nkeys, kScanTile);
    if (nb < 1) nb = 1;
    k_scan_reduce<<<nb, kScanThreads, 0, s>>>(count, nkeys, tmp);
    k_scan_sums<<<1, kScanThreads, 0, s>>>(tmp, nb);
    k_scan_final<<<nb, kScanThreads, 0, s>>>(count, nkeys, tmp, off);
}

void launch_scatter(const int *key, const int *off, int n, int *perm, int *tmp,
                    cudaStream_t s) {
    if (n <= 0) return;
    k_scatter<<<nblk(n, 256), 256, 0, s>>>(key, perm, off, n, tmp);
    k_stable_place<<<nblk(n, 256), 256, 0, s>>>(key, off, tmp, n, perm);
}

template <typename T>
void launch_records(const uint32_t *pstart, const T *pfrac, const int *perm, int n, int p,
                    int *rec_idx, uint32_t *rec_start, T *rec_w, cudaStream_t s) {
    if (n <= 0) return;
    const int nb = nblk(n, kRecThreads);
    switch (p) {
        case 4: k_records<T, 4><<<nb, kRecThreads, 0, s>>>(pstart, pfrac, perm, n, rec_idx, rec_start, rec_w); break;
        case 6: k_records<T, 6><<<nb, kRecThreads, 0, s>>>(pstart, pfrac, perm, n, rec_idx, rec_start, rec_w); break;
        case 8: k_records<T, 8><<<nb, kRecThreads, 0, s>>>(pstart, pfrac, perm, n, rec_idx, rec_start, rec_w); break;
        default: break;
    }
}

void launch_cell_positions(const double *pos, const int *perm, int n, double L, int nc,
                           bool fp32, void *cpos, cudaStream_t s) {
    if (n <= 0) return;
    if (fp32)
        k_cell_positions<float4, float><<<nblk(n, 256), 256, 0, s>>>(pos, perm, n, L, nc,
                                                                    (float4 *)cpos);
    else
        k_cell_positions<double4_32a, double><<<nblk(n, 256), 256, 0, s>>>(pos, perm, n, L, nc,
                                                                      (double4_32a *)cpos);
}

template void launch_records<float>(const uint32_t *, const float *, const int *, int, int, int *,
                                    uint32_t *, float *, cudaStream_t);
template void launch_records<double>(const uint32_t *, const double *, const int *, int, int,
                                     int *, uint32_t *, double *, cudaStream_t);

}  // namespace spme
