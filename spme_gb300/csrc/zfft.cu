// Fused z-transform + k-space influence + inverse z-transform.
//
// The 3D R2C/C2R transforms of the mesh are split: cuFFT does the 2D (y, x)
// transforms of every z-plane, and this kernel does, for a chunk of W (y, x)
// columns of all 3R components, the forward FFT along z, the RPY influence
// g <- S|b|^2 (I - k k^T/k^2) g (the physics of influence.cu, restating
// old-version/spme_kernel.c:73-228), and the inverse FFT along z, in shared
// memory: one read and one write of the half spectrum instead of three
// streaming passes.
//
// Data movement: the half spectrum keeps cuFFT's default layout
// G[c][z][y][K/2+1] (padded rows make cuFFT's 2D transforms slower).  A z-plane
// is viewed as one flat row of K (K/2+1) columns and cut into chunks of W
// consecutive columns, so every chunk starts on a 16-byte boundary and its
// z-columns of one component are one exact TMA box {2W values, zb rows}, for
// loads and stores alike (columns of two y rows may share a chunk: the
// transforms are per column).  Two buffers per block; a dedicated warp issues
// the TMA loads and, once the compute warps hand a buffer back, its TMA store
// and the load of the next right-hand side into it.
//
// FFT along z (length K = 2^a 3^b 5^c): in-place mixed-radix Cooley-Tukey in
// shared memory, radices 4, 2, 3, 5.  The forward transform is decimation in
// frequency (natural order in, digit-reversed order out), the influence is
// applied in the digit-reversed order (position p holds frequency perm[p]),
// and the inverse is decimation in time (digit-reversed in, natural out), so
// no permutation pass is needed.  Neither direction scales (the table's 1/V
// covers it).
//
// The reference's Nyquist convention (influence.cu) needs the Hermitian part
// of the influenced spectrum on the kx = 0 and (even K) kx = K/2 planes.  The
// forward spectrum of real data is Hermitian there, and for Hermitian g the
// Hermitian part of I(k) g equals (I(k) + I(-k))/2 g: the kernel applies that
// averaged tensor on those planes (I(-k) differs from I(k) only in the sign of
// the couplings between a Nyquist and a non-Nyquist axis, which cancel).
#include <algorithm>
#include <cmath>
#include <vector>

#include "fft_small.cuh"
#include "kernels.h"
#include "tma.cuh"

namespace spme {

namespace {

constexpr int kZSmemCap = 224 * 1024;

// One pass = two consecutive radix stages (R1 with span L, then R2 with span
// L R1; R2 = 1 for a single stage) done in registers, over every column of the
// block.  Column col = (component g, column w) is fixed per thread (the CT
// compute threads are a multiple of 3W); the thread walks pass butterflies bi = bi0, bi0 + BS,
// ...  Element z of the thread's column is sb[z W].  A radix-R stage with span
// L (block span L2 = L R) is
//   DIT (inverse):  t_q = x[b L2 + j + q L] w^{q j};  x[b L2 + j + p L] = sum_q t_q W_R^{pq}
//   DIF (forward):  x[b L2 + j + q L] = (sum_p x[b L2 + j + p L] W_R^{pq}) w^{q j}
// with w = e^{-2 pi i / L2} (conjugated for the inverse) read from the K-point
// table at stride K / L2.  In a pass, element (q1, q2) sits at
// b L3 + j + q1 L + q2 L R1 (L3 = L R1 R2); the R2 stage sees span L R1 and
// offset j + q1 L.  DIT runs the R1 stage first, DIF the R2 stage first.  A
// pass with L = 1 has j = 0: its R1-stage twiddles are 1 and are skipped.
// KC, LC: K and L as compile-time constants (0: taken from the arguments).
template <typename T, int W, int CT, int R1, int R2, bool DIF, int KC = 0, int LC = 0>
__device__ __forceinline__ void zpass(Cx<T> *__restrict__ sb, int Kr, int Lr,
                                      const Cx<T> *__restrict__ tw, int bi0) {
    constexpr int BS = CT / (3 * W);
    const int K = KC ? KC : Kr, L = LC ? LC : Lr;
    const int La = L * R1, L3 = La * R2;
    const int nb = K / (R1 * R2), ts1 = K / La, ts2 = K / L3;
    const bool unit1 = L == 1;
    DivMod dl;
    if constexpr (LC == 0) dl.init(L);
#pragma unroll(KC ? 2 : 1)
    for (int bi = bi0; bi < nb; bi += BS) {
        int j, b;
        if constexpr (LC != 0) {
            b = bi / LC;  // compile-time divisor
            j = bi - b * LC;
        } else {
            b = dl.div(bi, j);
        }
        Cx<T> *x = sb + (size_t)(b * L3 + j) * W;
        Cx<T> v[R2][R1];
#pragma unroll
        for (int q2 = 0; q2 < R2; q2++)
#pragma unroll
            for (int q1 = 0; q1 < R1; q1++) v[q2][q1] = x[(q1 * L + q2 * La) * W];
        if constexpr (!DIF) {
#pragma unroll
            for (int q2 = 0; q2 < R2; q2++) {
                Cx<T> in[R1], out[R1];
#pragma unroll
                for (int q1 = 0; q1 < R1; q1++) in[q1] = v[q2][q1];
                if (!unit1) {
#pragma unroll
                    for (int q1 = 1; q1 < R1; q1++) {
                        Cx<T> w = tw[q1 * j * ts1];
                        w.im = -w.im;
                        in[q1] = cmul(in[q1], w);
                    }
                }
                dft_small<T, R1, true>(in, out);
#pragma unroll
                for (int p1 = 0; p1 < R1; p1++) v[q2][p1] = out[p1];
            }
            if constexpr (R2 > 1) {
#pragma unroll
                for (int p1 = 0; p1 < R1; p1++) {
                    Cx<T> in[R2], out[R2];
                    in[0] = v[0][p1];
#pragma unroll
                    for (int q2 = 1; q2 < R2; q2++) {
                        Cx<T> w = tw[q2 * (j + p1 * L) * ts2];
                        w.im = -w.im;
                        in[q2] = cmul(v[q2][p1], w);
                    }
                    dft_small<T, R2, true>(in, out);
#pragma unroll
                    for (int p2 = 0; p2 < R2; p2++) v[p2][p1] = out[p2];
                }
            }
        } else {
            if constexpr (R2 > 1) {
#pragma unroll
                for (int p1 = 0; p1 < R1; p1++) {
                    Cx<T> in[R2], out[R2];
#pragma unroll
                    for (int q2 = 0; q2 < R2; q2++) in[q2] = v[q2][p1];
                    dft_small<T, R2, false>(in, out);
                    v[0][p1] = out[0];
#pragma unroll
                    for (int q2 = 1; q2 < R2; q2++)
                        v[q2][p1] = cmul(out[q2], tw[q2 * (j + p1 * L) * ts2]);
                }
            }
#pragma unroll
            for (int q2 = 0; q2 < R2; q2++) {
                Cx<T> in[R1], out[R1];
#pragma unroll
                for (int p1 = 0; p1 < R1; p1++) in[p1] = v[q2][p1];
                dft_small<T, R1, false>(in, out);
#pragma unroll
                for (int q1 = 0; q1 < R1; q1++) v[q2][q1] = out[q1];
                if (!unit1) {
#pragma unroll
                    for (int q1 = 1; q1 < R1; q1++) v[q2][q1] = cmul(out[q1], tw[q1 * j * ts1]);
                }
            }
        }
#pragma unroll
        for (int q2 = 0; q2 < R2; q2++)
#pragma unroll
            for (int q1 = 0; q1 < R1; q1++) x[(q1 * L + q2 * La) * W] = v[q2][q1];
    }
}

// Pass codes: 10 * R1 + R2.
template <typename T, int W, int CT, bool DIF>
__device__ __forceinline__ void zstage(Cx<T> *sb, int K, int code, int L, const Cx<T> *tw,
                                       int bi0) {
    switch (code) {
        case 44: zpass<T, W, CT, 4, 4, DIF>(sb, K, L, tw, bi0); break;
        case 42: zpass<T, W, CT, 4, 2, DIF>(sb, K, L, tw, bi0); break;
        case 43:
            // radix-12 / radix-20 passes only in FP32 (register pressure in FP64)
            if constexpr (sizeof(T) == 4) zpass<T, W, CT, 4, 3, DIF>(sb, K, L, tw, bi0);
            break;
        case 45:
            if constexpr (sizeof(T) == 4) zpass<T, W, CT, 4, 5, DIF>(sb, K, L, tw, bi0);
            break;
        case 41: zpass<T, W, CT, 4, 1, DIF>(sb, K, L, tw, bi0); break;
        case 21: zpass<T, W, CT, 2, 1, DIF>(sb, K, L, tw, bi0); break;
        case 31: zpass<T, W, CT, 3, 1, DIF>(sb, K, L, tw, bi0); break;
        default: zpass<T, W, CT, 5, 1, DIF>(sb, K, L, tw, bi0); break;
    }
}

// Barrier over the CT compute threads only (named barrier 1; the TMA warp
// never joins it), optionally AND-reducing a predicate.
template <int CT>
__device__ __forceinline__ void compute_sync() {
    asm volatile("bar.sync 1, %0;" ::"n"(CT) : "memory");
}
template <int CT>
__device__ __forceinline__ bool compute_sync_and(bool p) {
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred q, o;\n\t"
        "setp.ne.u32 q, %1, 0;\n\t"
        "bar.red.and.pred o, 1, %2, q;\n\t"
        "selp.u32 %0, 1, 0, o;\n\t}"
        : "=r"(r)
        : "r"((uint32_t)p), "n"(CT)
        : "memory");
    return r != 0;
}

// Shared-memory layout (bytes from the 128-aligned base).  TMA boxes land at
// 128-byte aligned addresses: each component's K x W block starts on a 128-byte
// boundary (stride gs complex values), and so does every z chunk of zb rows
// (checked by zcfg_fits).  Barriers: full[b] (TMA load of buffer b landed),
// done[b] (the compute warps finished buffer b).
template <typename T>
struct ZSmem {
    int gs;            // component stride (complex values)
    size_t buf_bytes;  // one buffer: 3 components
    size_t tw_off, perm_off, bar_off, total;
    __host__ __device__ ZSmem(int K, int W) {
        const size_t comp = ((size_t)K * W * sizeof(Cx<T>) + 127) & ~(size_t)127;
        gs = (int)(comp / sizeof(Cx<T>));
        buf_bytes = 3 * comp;
        tw_off = 2 * buf_bytes;
        perm_off = tw_off + (size_t)K * sizeof(Cx<T>);
        bar_off = (perm_off + (size_t)K * sizeof(int) + 15) & ~(size_t)15;
        total = bar_off + 4 * sizeof(uint64_t);
    }
};

// Launch configurations, in order of preference: W columns per block, CT
// compute threads, MINB blocks per SM, MAXP influence points per thread
// (table values kept in registers: points p = p0 + i PS, i < MAXP, so
// K W <= MAXP CT).  Fewer transform threads with more registers each measured
// faster than more threads that spill (K = 256 FP32: 192 threads 1.88 ms,
// 288 threads 1.93 ms, 384 threads 2.51 ms).
struct ZCfg {
    int W, ct, minb, maxp;
};
constexpr ZCfg kCfg32[] = {{16, 192, 1, 24}, {8, 192, 2, 12},
                           {4, 192, 1, 24},  {2, 192, 1, 24}};
constexpr ZCfg kCfg64[] = {{8, 384, 1, 6}, {4, 192, 2, 12}, {8, 192, 1, 12},
                           {2, 192, 1, 24}, {1, 192, 1, 24}};

// One block per chunk of W consecutive (y, x) columns of the flattened z-plane
// (chunk starts are multiples of W: 16-byte aligned in the global layout), all
// 3R components.  Threads 0..CT-1 transform; the warp after them moves data: TMA loads into
// the two buffers, TMA stores of finished buffers.
// Compile-time pass sequences (codes and spans as in ZPlan, DIT order) for the
// mesh sizes used most; any other K runs the plan's passes with runtime spans.
template <int KS>
struct ZFixed {
    static constexpr int n = 0;
};
template <>
struct ZFixed<128> {
    static constexpr int n = 2;
    static constexpr int code[2] = {44, 42}, span[2] = {1, 16};
};
template <>
struct ZFixed<160> {
    static constexpr int n = 3;
    static constexpr int code[3] = {44, 21, 51}, span[3] = {1, 16, 32};
};
template <>
struct ZFixed<256> {
    static constexpr int n = 2;
    static constexpr int code[2] = {44, 44}, span[2] = {1, 16};
};

// Passes I .. (DIF: down to 0, DIT: up to n - 1) of the fixed sequence of KS.
template <typename T, int W, int CT, int KS, bool DIF, int I>
__device__ __forceinline__ void zpasses_fixed(Cx<T> *cb, const Cx<T> *tw, int bi0) {
    using Z = ZFixed<KS>;
    constexpr int CODE = Z::code[I], SPAN = Z::span[I];
    zpass<T, W, CT, CODE / 10, CODE % 10, DIF, KS, SPAN>(cb, KS, SPAN, tw, bi0);
    if constexpr (DIF) {
        compute_sync<CT>();
        if constexpr (I > 0) zpasses_fixed<T, W, CT, KS, true, I - 1>(cb, tw, bi0);
    } else if constexpr (I + 1 < Z::n) {
        compute_sync<CT>();
        zpasses_fixed<T, W, CT, KS, false, I + 1>(cb, tw, bi0);
    }
}

// The z transform's passes: forward DIF (last pass first, each followed by a
// barrier) or inverse DIT (first pass first, barriers between passes).
template <typename T, int W, int CT, int KS, bool DIF>
__device__ __forceinline__ void zpasses(Cx<T> *cb, const ZPlan &zp, const Cx<T> *tw, int bi0) {
    if constexpr (ZFixed<KS>::n > 0) {
        zpasses_fixed<T, W, CT, KS, DIF, DIF ? ZFixed<KS>::n - 1 : 0>(cb, tw, bi0);
    } else {
        if constexpr (DIF) {
            for (int i = zp.npass - 1; i >= 0; i--) {
                zstage<T, W, CT, true>(cb, zp.K, zp.pcode[i], zp.pspan[i], tw, bi0);
                compute_sync<CT>();
            }
        } else {
            for (int i = 0; i < zp.npass; i++) {
                zstage<T, W, CT, false>(cb, zp.K, zp.pcode[i], zp.pspan[i], tw, bi0);
                if (i + 1 < zp.npass) compute_sync<CT>();
            }
        }
    }
}

template <typename T, int W, int CT, int MINB, int MAXP, int KS>
__global__ void __launch_bounds__(CT + 32, MINB)
k_zfft_influence(const __grid_constant__ CUtensorMap gmap, const T *__restrict__ tab2,
                 const Cx<T> *__restrict__ tw_g, const int *__restrict__ perm_g,
                 const __grid_constant__ ZPlan zp, T twopi_L, int R, int zb,
                 int *__restrict__ err) {
    using V2 = typename Vec2<T>::type;
    constexpr int NCOL = 3 * W;
    constexpr int PS = CT / W;  // z stride of a thread's influence points
    constexpr int NT = CT + 32;
    const int K = zp.K;
    const int Kh = K / 2 + 1;
    const int plane = K * Kh;       // columns per z-plane
    const int f0 = blockIdx.x * W;  // first flat column of the chunk
    const int tid = threadIdx.x;
    extern __shared__ __align__(128) unsigned char zsm_raw[];
    // 128-byte aligned base (the launch reserves 128 bytes of slack)
    unsigned char *zsm = zsm_raw + ((128u - (smem_addr(zsm_raw) & 127u)) & 127u);
    const ZSmem<T> lay(K, W);
    const int GS = lay.gs;
    Cx<T> *const buf0 = reinterpret_cast<Cx<T> *>(zsm);
    Cx<T> *const buf1 = reinterpret_cast<Cx<T> *>(zsm + lay.buf_bytes);
    Cx<T> *tw = reinterpret_cast<Cx<T> *>(zsm + lay.tw_off);
    int *perm = reinterpret_cast<int *>(zsm + lay.perm_off);
    uint64_t *full = reinterpret_cast<uint64_t *>(zsm + lay.bar_off);
    uint64_t *done = full + 2;
    const int nzc = K / zb;

    if (tid == 0) {
        mbar_init(&full[0], 1);
        mbar_init(&full[1], 1);
        mbar_init(&done[0], CT);
        mbar_init(&done[1], CT);
        mbar_fence_init();
    }
    for (int e = tid; e < K; e += NT) {
        tw[e] = tw_g[e];
        perm[e] = perm_g[e];
    }
    __syncthreads();

    if (tid >= CT) {
        // ---- TMA warp (one lane) ----
        if (tid != CT) return;
        const uint32_t bytes = (uint32_t)(3 * nzc * 2 * W * zb * sizeof(T));
        auto issue_load = [&](int r, int b) {
            mbar_expect_tx(&full[b], bytes);
            Cx<T> *dst = b ? buf1 : buf0;
            for (int d = 0; d < 3; d++)
                for (int zc = 0; zc < nzc; zc++)
                    tma_load_3d(dst + (size_t)d * GS + (size_t)zc * zb * W, &gmap, 2 * f0,
                                zc * zb, 3 * r + d, &full[b]);
        };
        issue_load(0, 0);
        int issued = 1;
        if (R > 1) issue_load(1, 1), issued = 2;
        int r = 0;
        for (; r < R; r++) {
            const int b = r & 1;
            if (!mbar_wait(&done[b], (uint32_t)((r >> 1) & 1))) break;
            const Cx<T> *src = b ? buf1 : buf0;
            for (int d = 0; d < 3; d++)
                for (int zc = 0; zc < nzc; zc++)
                    tma_store_3d(&gmap, 2 * f0, zc * zb, 3 * r + d,
                                 src + (size_t)d * GS + (size_t)zc * zb * W);
            bulk_commit_group();
            if (r + 2 < R) {
                bulk_wait_read_all();  // buffer b is free again
                issue_load(r + 2, b);
                issued++;
            }
        }
        if (r < R) {
            atomicExch(err, 1);
            // loads of right-hand sides r .. issued-1 may still be in flight
            for (int q = r; q < issued; q++) mbar_wait(&full[q & 1], (uint32_t)((q >> 1) & 1));
        }
        bulk_wait_all();
        return;
    }

    // ---- compute warps ----
    // influence table of this thread's points, read once for all R
    const int wi = tid % W, p0 = tid / W;
    const int fl = f0 + wi;
    const bool valid = fl < plane;
    const int ky = valid ? fl / Kh : 0, kx = valid ? fl - ky * Kh : 0;
    const T kxv = (T)kx * twopi_L;  // kx <= K/2: non-negative wavenumber
    const T kyv = (T)(ky <= K / 2 ? ky : ky - K) * twopi_L;
    // kx = 0 and (even K) K/2 planes hold k and -k: there the tensor is averaged
    // with its mirror (the Hermitian part of the result):
    // with s_i = +1 for a zero or Nyquist index and -1 otherwise, the ij
    // coupling survives when s_i s_j = +1 (s_x = +1 on these planes)
    const bool xplane = valid && (kx == 0 || (!(K & 1) && kx == K / 2));
    const bool sy = ky == 0 || (!(K & 1) && ky == K / 2);
    T m2r[MAXP], cr[MAXP];
#pragma unroll
    for (int i = 0; i < MAXP; i++) {
        const int p = p0 + i * PS;
        m2r[i] = T(0);
        cr[i] = T(0);
        if (p < K && valid) {
            const V2 mc = reinterpret_cast<const V2 *>(tab2)[(size_t)perm[p] * plane + fl];
            m2r[i] = mc.x;
            cr[i] = mc.y;
        }
    }

    static_assert(CT % NCOL == 0 && CT % 32 == 0, "columns must tile the compute warps");
    const int col = tid % NCOL, bi0 = tid / NCOL;
    const int gcol = col / W, wcol = col - gcol * W;

    for (int r = 0; r < R; r++) {
        const int b = r & 1;
        const bool ok = mbar_wait(&full[b], (uint32_t)((r >> 1) & 1));
        if (!compute_sync_and<CT>(ok)) {
            if (tid == 0) atomicExch(err, 1);
            break;
        }
        Cx<T> *B = b ? buf1 : buf0;
        Cx<T> *cb = B + (size_t)gcol * GS + wcol;
        // forward DIF, passes from the last down
        zpasses<T, W, CT, KS, true>(cb, zp, tw, bi0);
        // influence, digit-reversed z order
#pragma unroll
        for (int i = 0; i < MAXP; i++) {
            const int p = p0 + i * PS;
            if (p < K) {
                const int kz = perm[p];
                const T kzv = (T)(kz <= K / 2 ? kz : kz - K) * twopi_L;
                const T m2 = m2r[i], c = cr[i];
                T b1 = -c * kxv * kyv, b2 = -c * kxv * kzv, b4 = -c * kyv * kzv;
                if (xplane) {
                    const bool sz = kz == 0 || (!(K & 1) && kz == K / 2);
                    if (!sy) b1 = T(0);
                    if (!sz) b2 = T(0);
                    if (sy != sz) b4 = T(0);
                }
                const T b0 = m2 - c * kxv * kxv, b3 = m2 - c * kyv * kyv, b5 = m2 - c * kzv * kzv;
                Cx<T> *q0 = B + (size_t)p * W + wi;
                Cx<T> *q1 = q0 + GS;
                Cx<T> *q2 = q1 + GS;
                const Cx<T> g0 = *q0, g1 = *q1, g2 = *q2;
                *q0 = {b0 * g0.re + b1 * g1.re + b2 * g2.re, b0 * g0.im + b1 * g1.im + b2 * g2.im};
                *q1 = {b1 * g0.re + b3 * g1.re + b4 * g2.re, b1 * g0.im + b3 * g1.im + b4 * g2.im};
                *q2 = {b2 * g0.re + b4 * g1.re + b5 * g2.re, b2 * g0.im + b4 * g1.im + b5 * g2.im};
            }
        }
        compute_sync<CT>();
        // inverse DIT, passes from the first up
        zpasses<T, W, CT, KS, false>(cb, zp, tw, bi0);
        // hand the buffer to the TMA warp (its store reads what this thread wrote)
        fence_proxy_async();
        mbar_arrive(&done[b]);
    }
}

}  // namespace

bool make_zplan(int K, size_t elem, ZPlan *zp, std::vector<double> *twr, std::vector<int> *perm) {
    if (K < 2 || K > 4096) return false;
    int m = K, n = 0;
    int rad[16];
    for (int r : {4, 2, 3, 5})
        while (m % r == 0 && n < 16) {
            rad[n++] = r;
            m /= r;
        }
    if (m != 1 || n > 12) return false;
    zp->K = K;
    zp->nst = n;
    int lb = 1;
    for (int s = 0; s < n; s++) {
        zp->rad[s] = rad[s];
        if (s < n - 1) lb *= rad[s];
    }
    zp->len_before_last = lb;  // L at the last stage = product of the first n-1 radices
    // passes: a radix 4 pairs with the radix after it (in FP64 only with 4 or 2)
    zp->npass = 0;
    for (int s = 0, span = 1; s < n;) {
        int r2 = (rad[s] == 4 && s + 1 < n) ? rad[s + 1] : 1;
        if (elem == 8 && r2 != 4 && r2 != 2) r2 = 1;
        const int r1 = rad[s];
        zp->pcode[zp->npass] = 10 * r1 + r2;
        zp->pspan[zp->npass] = span;
        zp->npass++;
        span *= r1 * r2;
        s += r2 > 1 ? 2 : 1;
    }
    // digit reversal: position p holds natural index perm[p] (recursive
    // decimation by the last radix first)
    std::vector<int> idx(K), tmp(K);
    for (int i = 0; i < K; i++) idx[i] = i;
    struct Rec {
        static void run(int *a, int len, const int *rs, int nr, int *scratch) {
            if (len == 1 || nr == 0) return;
            const int R = rs[nr - 1], sub = len / R;
            for (int q = 0; q < R; q++)
                for (int k = 0; k < sub; k++) scratch[q * sub + k] = a[k * R + q];
            for (int i = 0; i < len; i++) a[i] = scratch[i];
            for (int q = 0; q < R; q++) run(a + q * sub, sub, rs, nr - 1, scratch + q * sub);
        }
    };
    Rec::run(idx.data(), K, rad, n, tmp.data());
    perm->assign(idx.begin(), idx.end());
    twr->resize(2 * (size_t)K);
    for (int e = 0; e < K; e++) {
        const double a = -2.0 * M_PI * (double)e / (double)K;
        (*twr)[2 * e] = std::cos(a);
        (*twr)[2 * e + 1] = std::sin(a);
    }
    return true;
}

namespace {

template <typename T>
size_t zsmem_bytes(int K, int W) {
    return ZSmem<T>(K, W).total + 128;
}

int zchunk(int K) {
    int zb = K;
    while (zb > 256) zb /= 2;  // TMA box dimensions are at most 256
    return zb;
}

bool zcfg_fits(const ZCfg &c, int K, size_t elem) {
    if ((size_t)2 * c.W * elem % 16 != 0) return false;  // TMA inner box bytes
    const int zb = zchunk(K);
    if (K % zb != 0) return false;
    if (zb < K && ((size_t)zb * c.W * 2 * elem) % 128 != 0) return false;  // chunk alignment
    if (((size_t)K * (K / 2 + 1) * 2 * elem) % 16 != 0) return false;     // z-plane stride
    if (c.ct % (3 * c.W) != 0) return false;
    const size_t smem = elem == 4 ? zsmem_bytes<float>(K, c.W) : zsmem_bytes<double>(K, c.W);
    if (smem * c.minb > (size_t)kZSmemCap) return false;
    return (size_t)K * c.W <= (size_t)c.maxp * c.ct;
}

// Preferred configuration index for K, -1 if none fits.
int zcfg_index(int K, size_t elem) {
    const ZCfg *list = elem == 4 ? kCfg32 : kCfg64;
    const int n = elem == 4 ? (int)(sizeof(kCfg32) / sizeof(ZCfg)) : (int)(sizeof(kCfg64) / sizeof(ZCfg));
    for (int i = 0; i < n; i++)
        if (zcfg_fits(list[i], K, elem)) return i;
    return -1;
}

}  // namespace

int zfft_width(int K, size_t elem) {
    const int i = zcfg_index(K, elem);
    if (i < 0) return 0;
    return (elem == 4 ? kCfg32 : kCfg64)[i].W;
}

bool make_zfft_map(CUtensorMap *map, void *G, int K, int C, size_t elem) {
    EncodeTiledFn fn = encode_fn();
    const int W = zfft_width(K, elem);
    if (!fn || W == 0 || ((uintptr_t)G % 16) != 0) return false;
    const int zb = zchunk(K);
    const cuuint64_t plane = (cuuint64_t)K * (K / 2 + 1) * 2;  // values per z-plane
    const cuuint64_t dims[3] = {plane, (cuuint64_t)K, (cuuint64_t)C};
    const cuuint64_t strides[2] = {plane * elem, plane * K * elem};
    const cuuint32_t box[3] = {(cuuint32_t)(2 * W), (cuuint32_t)zb, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = fn(map, elem == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64,
                    3, G, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                    CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

template <int KS>
bool plan_is(const ZPlan &zp) {
    using Z = ZFixed<KS>;
    if (zp.K != KS || zp.npass != Z::n) return false;
    for (int i = 0; i < Z::n; i++)
        if (zp.pcode[i] != Z::code[i] || zp.pspan[i] != Z::span[i]) return false;
    return true;
}

template <typename T, int W, int CT, int MINB, int MAXP>
cudaError_t launch_zcfg(const CUtensorMap &map, const T *tab2, const T *tw, const int *perm,
                        const ZPlan &zp, T twopi_L, int R, int zb, int *err, cudaStream_t s) {
    // a fixed pass sequence when the plan matches one (instantiated for each
    // precision's first configuration, the one these K get)
    constexpr ZCfg first = sizeof(T) == 4 ? kCfg32[0] : kCfg64[0];
    constexpr bool fixed_ok = first.W == W && first.ct == CT && first.minb == MINB &&
                              first.maxp == MAXP;
    auto kern = k_zfft_influence<T, W, CT, MINB, MAXP, 0>;
    if constexpr (fixed_ok) {
        if (plan_is<256>(zp)) kern = k_zfft_influence<T, W, CT, MINB, MAXP, 256>;
        if (plan_is<160>(zp)) kern = k_zfft_influence<T, W, CT, MINB, MAXP, 160>;
        if (plan_is<128>(zp)) kern = k_zfft_influence<T, W, CT, MINB, MAXP, 128>;
    }
    const int K = zp.K, Kh = K / 2 + 1;
    const size_t smem = zsmem_bytes<T>(K, W);
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const int nchunk = (K * Kh + W - 1) / W;
    kern<<<nchunk, CT + 32, smem, s>>>(map, tab2, reinterpret_cast<const Cx<T> *>(tw), perm, zp,
                                         twopi_L, R, zb, err);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_zfft_influence(const CUtensorMap &map, T *G, const T *tab2, const T *tw,
                                  const int *perm, const ZPlan &zp, double L, int R, int *err,
                                  cudaStream_t s) {
    (void)G;  // addressed through the tensor map
    const int K = zp.K;
    const int ci = zcfg_index(K, sizeof(T));
    if (ci < 0) return cudaErrorInvalidValue;
    const T twopi_L = (T)(2.0 * M_PI / L);
    const int zb = zchunk(K);
    cudaError_t e = cudaErrorInvalidValue;
    const ZCfg c = (sizeof(T) == 4 ? kCfg32 : kCfg64)[ci];
#define SPME_ZCFG(WW, CC, BB, PP)                                                               \
    if (c.W == WW && c.ct == CC && c.minb == BB && c.maxp == PP)                                \
        e = launch_zcfg<T, WW, CC, BB, PP>(map, tab2, tw, perm, zp, twopi_L, R, zb, err, s);
    if constexpr (sizeof(T) == 4) {
        SPME_ZCFG(8, 192, 2, 12)
        SPME_ZCFG(16, 192, 1, 24)
        SPME_ZCFG(4, 192, 1, 24)
        SPME_ZCFG(2, 192, 1, 24)
    } else {
        SPME_ZCFG(8, 384, 1, 6)
        SPME_ZCFG(4, 192, 2, 12)
        SPME_ZCFG(8, 192, 1, 12)
        SPME_ZCFG(2, 192, 1, 24)
        SPME_ZCFG(1, 192, 1, 24)
    }
#undef SPME_ZCFG
    return e;
}

template cudaError_t launch_zfft_influence<float>(const CUtensorMap &, float *, const float *,
                                                  const float *, const int *, const ZPlan &,
                                                  double, int, int *, cudaStream_t);
template cudaError_t launch_zfft_influence<double>(const CUtensorMap &, double *, const double *,
                                                   const double *, const int *, const ZPlan &,
                                                   double, int, int *, cudaStream_t);

}  // namespace spme
