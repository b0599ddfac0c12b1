// Real-space Ewald RPY pair sum over a cell list within rc, plus the self
// term.  The reference has no real-space part (it computes only M_recip,
// old-version/spme.c:560-726); this restates Beenakker, J. Chem. Phys. 85,
// 1581 (1986), in the reference's units (mobility x 6 pi eta, matching
// scalar_recip at old-version/spme.c:43-60), with the RPY overlap form for
// pairs closer than 2a.
//
// One CTA per cell of edge >= rc; a warp per particle of the cell against the
// candidates of the 27 neighbour cells (details at the kernel below).
#include <algorithm>
#include <cmath>
#include <type_traits>
#include <vector>

#include "kernels.h"

namespace spme {

namespace {

constexpr int kThreads = 64;  // two warps per cell: ~4-5 particles each at typical densities

__device__ __forceinline__ double d_erfc(double x) { return erfc(x); }
__device__ __forceinline__ double d_exp(double x) { return exp(x); }

__device__ __forceinline__ double d_erf(double x) { return erf(x); }

// Maclaurin coefficients (without the 2/sqrt(pi) factor) of S(x) = erf(x)/x,
// (-1)^n / (n! (2n+1)), and of psi(x) = (erf(x) - 2x e^{-x^2}/sqrt(pi)) / x^3,
// (-1)^(n+1) 2n / (n! (2n+1)) for n >= 1; in x^2, ten terms (below 1e-17
// relative for x < 0.5).
__device__ __constant__ double kSerS[10] = {1.0, -1.0 / 3, 1.0 / 10, -1.0 / 42, 1.0 / 216,
                                            -1.0 / 1320, 1.0 / 9360, -1.0 / 75600,
                                            1.0 / 685440, -1.0 / 6894720};
__device__ __constant__ double kSerPsi[10] = {2.0 / 3, -2.0 / 5, 1.0 / 7, -1.0 / 27, 1.0 / 132,
                                              -1.0 / 780, 1.0 / 5400, -1.0 / 42840,
                                              1.0 / 383040, -1.0 / 3810240};

// M_real(r) = F I + G rhat rhat: Beenakker's real-space form divided by a, and
// for r < 2a plus (overlap RPY - far-field RPY).  For r < 2a the 1/r and 1/r^3
// terms of the two cancel; written with x = xi r, S(x) = erf(x)/x and psi(x)
// they cancel analytically (no loss of precision as r -> 0, finite at r = 0):
//   F = xi [-3/4 S + e (3x^2 - 9/2)/sqrt(pi)] + xi^3 a^2 [-psi/2 + e (4x^4 - 20x^2 + 14)/sqrt(pi)]
//       + (1 - 9r/(32a)) / a
//   G = xi [-3/4 S + e (3/2 - 3x^2)/sqrt(pi)] + xi^3 a^2 [3psi/2 + e (-4x^4 + 16x^2 - 2)/sqrt(pi)]
//       + 3r/(32 a^2)
// with e = exp(-x^2); S and psi from their series for x < 0.5.
template <typename T>
__device__ __forceinline__ void real_FG(T r, T xi, T a, T &F, T &G) {
    const T rsp = T(0.56418958354775628695);  // 1/sqrt(pi)
    const T x = xi * r, x2 = x * x, e = d_exp(-x2);
    if (r < T(2) * a) {
        T S, P;
        if (x < T(0.5)) {
            S = T(0);
            P = T(0);
#pragma unroll
            for (int k = 9; k >= 0; k--) {
                S = S * x2 + T(kSerS[k]);
                P = P * x2 + T(kSerPsi[k]);
            }
            S *= T(2) * rsp;
            P *= T(2) * rsp;
        } else {
            const T ef = d_erf(x);
            S = ef / x;
            P = (ef - T(2) * rsp * x * e) / (x2 * x);
        }
        const T x4 = x2 * x2, xi3a2 = xi * xi * xi * a * a;
        F = xi * (T(-0.75) * S + rsp * e * (T(3) * x2 - T(4.5))) +
            xi3a2 * (T(-0.5) * P + rsp * e * (T(4) * x4 - T(20) * x2 + T(14))) +
            (T(1) - T(9) * r / (T(32) * a)) / a;
        G = xi * (T(-0.75) * S + rsp * e * (T(1.5) - T(3) * x2)) +
            xi3a2 * (T(1.5) * P + rsp * e * (T(-4) * x4 + T(16) * x2 - T(2))) +
            T(3) * r / (T(32) * a * a);
        return;
    }
    const T ec = d_erfc(x);
    const T r2 = r * r, a3 = a * a * a, ir = T(1) / r, ir3 = ir * ir * ir, ir2 = ir * ir;
    const T xi2 = xi * xi, xi3 = xi2 * xi, xi5 = xi3 * xi2, xi7 = xi5 * xi2;
    const T f = ec * (T(0.75) * a * ir + T(0.5) * a3 * ir3) +
                e * rsp * (T(4) * xi7 * a3 * r2 * r2 + T(3) * xi3 * a * r2 - T(20) * xi5 * a3 * r2 -
                           T(4.5) * xi * a + T(14) * xi3 * a3 + xi * a3 * ir2);
    const T g = ec * (T(0.75) * a * ir - T(1.5) * a3 * ir3) +
                e * rsp * (-T(4) * xi7 * a3 * r2 * r2 - T(3) * xi3 * a * r2 + T(16) * xi5 * a3 * r2 +
                           T(1.5) * xi * a - T(2) * xi3 * a3 - T(3) * xi * a3 * ir2);
    F = f / a;
    G = g / a;
}

// FP32 engines: F, G and ir = 1/r (0 at r = 0) from r^2, with the launch's
// coefficients (RealCoef): one reciprocal square root gives r, 1/r and the
// unit vector; the far field (r >= 2a) is real_FG's far form divided through
// by a, the near field real_FG's cancellation-free form with FP32 constants.
__device__ __forceinline__ void real_FG_f32(float r2, const RealCoef &c, float &F, float &G,
                                            float &ir) {
    constexpr float rsp = 0.56418958354775628695f;  // 1/sqrt(pi)
    ir = r2 > 0.f ? rsqrtf(r2) : 0.f;
    const float r = r2 * ir;
    if (r2 < c.a2x4) {
        const float x = c.xi * r, x2 = x * x, e = expf(-x2);
        float S, P;
        if (x < 0.5f) {
            constexpr float ks[10] = {1.0f, -1.0f / 3, 1.0f / 10, -1.0f / 42, 1.0f / 216,
                                      -1.0f / 1320, 1.0f / 9360, -1.0f / 75600,
                                      1.0f / 685440, -1.0f / 6894720};
            constexpr float kp[10] = {2.0f / 3, -2.0f / 5, 1.0f / 7, -1.0f / 27, 1.0f / 132,
                                      -1.0f / 780, 1.0f / 5400, -1.0f / 42840,
                                      1.0f / 383040, -1.0f / 3810240};
            S = 0.f;
            P = 0.f;
#pragma unroll
            for (int k = 9; k >= 0; k--) {
                S = fmaf(S, x2, ks[k]);
                P = fmaf(P, x2, kp[k]);
            }
            S *= 2.f * rsp;
            P *= 2.f * rsp;
        } else {
            const float ef = erff(x), ix = 1.f / x;
            S = ef * ix;
            P = (ef - 2.f * rsp * x * e) * (ix * ix * ix);
        }
        const float x4 = x2 * x2, re = rsp * e;
        F = c.xi * (-0.75f * S + re * (3.f * x2 - 4.5f)) +
            c.xi3a2 * (-0.5f * P + re * (4.f * x4 - 20.f * x2 + 14.f)) + (c.ia - c.n1 * r);
        G = c.xi * (-0.75f * S + re * (1.5f - 3.f * x2)) +
            c.xi3a2 * (1.5f * P + re * (-4.f * x4 + 16.f * x2 - 2.f)) + c.n2 * r;
        return;
    }
    const float ec = erfcf(c.xi * r), e = expf(-c.xi2 * r2);
    const float ir2 = ir * ir, ir3 = ir2 * ir, r4 = r2 * r2;
    const float pF = fmaf(c.A4, r4, fmaf(c.A2, r2, fmaf(c.Am2, ir2, c.A0)));
    const float pG = fmaf(-c.A4, r4, fmaf(c.B2, r2, fmaf(c.Bm2, ir2, c.B0)));
    F = ec * fmaf(c.c1, ir3, 0.75f * ir) + e * pF;
    G = ec * fmaf(c.c3, ir3, 0.75f * ir) + e * pG;
}

// F and G from the per-engine Chebyshev table (FP64 engines): false when r is
// outside the table (the caller then evaluates real_FG directly).  Clenshaw
// recurrence in t in [-1, 1] on the segment holding r; F and G coefficients
// interleaved.
__device__ __forceinline__ bool table_FG(const PairTable &tb, double r, double &F, double &G) {
    if (!tb.coef || r < tb.r_lo || r > tb.r_hi) return false;
    int seg;
    double u;
    if (r < tb.r_mid) {
        u = (r - tb.r_lo) * tb.inv_h1;
        seg = min((int)u, tb.nseg1 - 1);
        u -= seg;
    } else {
        u = (r - tb.r_mid) * tb.inv_h2;
        const int s2 = min((int)u, tb.nseg2 - 1);
        u -= s2;
        seg = tb.nseg1 + s2;
    }
    const double t = 2.0 * u - 1.0;
    const double2 *c = reinterpret_cast<const double2 *>(tb.coef) + (size_t)seg * (kPairDeg + 1);
    double bF = 0.0, bF1 = 0.0, bG = 0.0, bG1 = 0.0;
#pragma unroll
    for (int k = kPairDeg; k >= 1; k--) {
        const double2 ck = __ldg(c + k);
        const double nF = 2.0 * t * bF - bF1 + ck.x, nG = 2.0 * t * bG - bG1 + ck.y;
        bF1 = bF;
        bG1 = bG;
        bF = nF;
        bG = nG;
    }
    const double2 c0 = __ldg(c);
    F = t * bF - bF1 + 0.5 * c0.x;
    G = t * bG - bG1 + 0.5 * c0.y;
    return true;
}

// Accumulator across pair batches: FP64 engines add in FP64; FP32 engines add
// in FP32 with Knuth's TwoSum error term carried alongside (the FP64 pipe is a
// small fraction of the FP32 rate on this GPU, and a handful of double adds
// per particle had become the kernel's limiter).
template <typename T>
struct PairSum {
    T s = T(0), c = T(0);
    __device__ __forceinline__ void add(T x) {
        if constexpr (sizeof(T) == 8) {
            s += x;
        } else {
            const T t = s + x, bp = t - s;
            c += (s - (t - bp)) + (x - bp);
            s = t;
        }
    }
    __device__ __forceinline__ void add(const PairSum &o) {
        add(o.s);
        c += o.c;
    }
    __device__ __forceinline__ T value() const { return s + c; }
};

template <typename T>
__device__ __forceinline__ PairSum<T> shfl_xor(const PairSum<T> &a, int o) {
    PairSum<T> b;
    b.s = __shfl_xor_sync(0xffffffffu, a.s, o);
    b.c = __shfl_xor_sync(0xffffffffu, a.c, o);
    return b;
}

template <typename G> struct Geo4;
template <> struct Geo4<float> { using type = float4; };
template <> struct Geo4<double> { using type = double4_32a; };

__device__ __forceinline__ float d_rint(float x) { return rintf(x); }
__device__ __forceinline__ double d_rint(double x) { return rint(x); }

constexpr int kWarps = kThreads / 32;
constexpr int kCap = 512;  // candidates staged in shared memory per cell

// T: pair-function type; G: pair geometry type.  Positions are stored relative
// to the corner of their cell (edge h = L/nc), so the displacement to a
// candidate in neighbour cell c_i + dc is (o_i - o_j) - dc*h, accurate in
// FP32 for any box size.
//
// One CTA per cell.  The candidates of the 27 neighbour cells are staged once
// in shared memory (positions in the frame of the CTA's cell), then each warp
// takes one of the cell's particles at a time:
//   1. lanes test 32 candidates at a time for r < rc and compact the hits
//      into a per-warp buffer (ballot + popc);
//   2. every 32 hits, lanes evaluate the 32 pair functions F, G and unit
//      vectors (all lanes busy);
//   3. lanes as (pair, right-hand side) apply the batch to the forces:
//      u_i[r] += F f_j[r] + G rhat (rhat . f_j[r]).
// Sums over one batch run in T; across batches FP64 engines add in FP64 and
// FP32 engines in compensated FP32 (TwoSum, PairSum below).  No block
// barrier after the staging.  More than kCap candidates (very dense cells)
// take a second path that reads candidates straight from global memory.
// FP32: 64 registers, 16 blocks (32 warps) per SM (measured faster than the
// unconstrained 80 registers); FP64 needs more registers.
template <typename T, typename G>
__device__ __forceinline__ void realspace_body(const RealArgs<T> &A, int cell) {
    const int nc = A.nc;
    const int *__restrict__ cell_off = A.cell_off;
    const int *__restrict__ cell_perm = A.cell_perm;
    const typename Geo4<G>::type *__restrict__ cpos =
        reinterpret_cast<const typename Geo4<G>::type *>(A.cpos);
    const T *__restrict__ F = A.F;
    T *__restrict__ W = A.W;
    const int R = A.R, with_self = A.with_self;
    constexpr bool kF32 = sizeof(T) == 4;
    // FP32: the geometry and coefficients as FP32 copies (no conversions here)
    const G L = kF32 ? (G)A.cf.L : (G)A.L, h = kF32 ? (G)A.cf.h : (G)A.h,
            rc2 = kF32 ? (G)A.cf.rc2 : (G)A.rc2;
    const T xi = kF32 ? (T)A.cf.xi : (T)A.xi, a = (T)A.a;
    const T self_c = kF32 ? (T)A.cf.self_c : (T)A.self_c;
    const PairTable &tab = A.tab;
    __shared__ int nb_beg[27], nb_pre[28], nnb;
    __shared__ G nb_shift[27][3];
    // a staged candidate: position in the CTA cell's frame and particle id in
    // one 16-byte (FP32) or 32-byte (FP64) record
    struct __align__(4 * sizeof(G)) Cand {
        G x, y, z;
        int j;
    };
    __shared__ Cand cand[kCap];
    // FP64 engines: FP32 copies for a conservative first distance test (the FP64
    // test then runs only on candidates that pass it)
    constexpr bool kPre = sizeof(G) == 8;
    __shared__ float fx[kPre ? kCap : 1], fy[kPre ? kCap : 1], fz[kPre ? kCap : 1];
    // candidates tested per lane per iteration (FP32: 2; FP64 keeps 1, its shared
    // memory is at the 8-blocks-per-SM limit)
    constexpr int kU = sizeof(T) == 4 ? 2 : 1;
    __shared__ int hits[kWarps][32 + 32 * kU];  // up to 31 carried + 32 kU new
    // one record per buffered pair: unit vector and F in one 16/32-byte vector,
    // then G and the start of the partner's force row (aligned as that vector)
    struct PairRec {
        typename Geo4<T>::type rf;  // (rhat_x, rhat_y, rhat_z, F)
        const T *frow;
        T gfac;
    };
    __shared__ PairRec prec[kWarps][32];

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int C = 3 * R;
    // neighbour table: lane k of warp 0 takes neighbour cell k (27 of them, or
    // the cell alone when nc < 3), candidate offsets by a warp scan
    if (warp == 0) {
        const int ccx = cell % nc, ccy = (cell / nc) % nc, ccz = cell / (nc * nc);
        const int nk = nc >= 3 ? 27 : 1;
        int cnt = 0;
        if (lane < nk) {
            const int dx = nk == 1 ? 0 : lane % 3 - 1, dy = nk == 1 ? 0 : (lane / 3) % 3 - 1,
                      dz = nk == 1 ? 0 : lane / 9 - 1;
            auto wrap = [nc](int v) { return v < 0 ? v + nc : (v >= nc ? v - nc : v); };
            const int c2 = (wrap(ccz + dz) * nc + wrap(ccy + dy)) * nc + wrap(ccx + dx);
            const int b = __ldg(cell_off + c2);
            cnt = __ldg(cell_off + c2 + 1) - b;
            nb_beg[lane] = b;
            nb_shift[lane][0] = (G)dx * h;
            nb_shift[lane][1] = (G)dy * h;
            nb_shift[lane][2] = (G)dz * h;
        }
        int inc = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += t;
        }
        if (lane < nk) nb_pre[lane] = inc - cnt;
        if (lane == nk - 1) {
            nb_pre[nk] = inc;
            nnb = nk;
        }
    }
    __syncthreads();
    const int ncand = nb_pre[nnb];
    const bool staged = ncand <= kCap;
    // neighbour k holding candidate q: nb_pre[k] <= q < nb_pre[k + 1]
    auto find_nb = [&](int q) {
        int lo = 0, hi = nnb;
        while (hi - lo > 1) {
            const int m = (lo + hi) >> 1;
            if (nb_pre[m] <= q) lo = m; else hi = m;
        }
        return lo;
    };
    if (staged) {
        for (int q = tid; q < ncand; q += kThreads) {
            const int k = find_nb(q);
            const int js = nb_beg[k] + (q - nb_pre[k]);
            const auto p = cpos[js];
            Cand c;
            c.x = p.x + nb_shift[k][0];
            c.y = p.y + nb_shift[k][1];
            c.z = p.z + nb_shift[k][2];
            c.j = cell_perm[js];
            cand[q] = c;
            if constexpr (kPre) {
                fx[q] = (float)c.x;
                fy[q] = (float)c.y;
                fz[q] = (float)c.z;
            }
        }
    }
    __syncthreads();
    const bool single = nc < 3;
    // the FP32 test accepts a superset of the pairs within rc: coordinates lie
    // within 3 cells, so FP32 rounding moves d^2 by far less than the margin
    const bool pre = kPre && staged && !single;
    const float pre_r2 =
        kPre ? (float)((double)rc2 * 1.0001 + 1e-5 * 9.0 * (double)h * (double)h) : 0.f;
    const G invL = G(1) / L;
    const int ib0 = cell_off[cell], ie = cell_off[cell + 1];

    // candidate q -> position in this cell's frame and particle id
    auto candidate = [&](int q, G &x, G &y, G &z, int &j) {
        if (staged) {
            const Cand c = cand[q];
            x = c.x;
            y = c.y;
            z = c.z;
            j = c.j;
        } else {
            const int k = find_nb(q);
            const int js = nb_beg[k] + (q - nb_pre[k]);
            const auto p = cpos[js];
            x = p.x + nb_shift[k][0];
            y = p.y + nb_shift[k][1];
            z = p.z + nb_shift[k][2];
            j = cell_perm[js];
        }
    };

    const int RL = R >= 32 ? 32 : (R > 16 ? 32 : (R > 8 ? 16 : (R > 4 ? 8 : (R > 2 ? 4 : (R > 1 ? 2 : 1)))));
    const int PR = 32 / RL;             // pairs applied in parallel
    const int pp = lane / RL, rl = lane % RL;

    for (int i = ib0 + warp; i < ie; i += kWarps) {
        const auto pi = cpos[i];
        const int ii = cell_perm[i];
        for (int rb = 0; rb < R; rb += RL) {
            const int r = rb + rl;
            const bool rok = r < R;
            PairSum<T> a0, a1, a2;
            int nh = 0;  // buffered hits (warp-uniform)
            // evaluate and apply `m` buffered hits; returns this lane's partial sums
            auto flush = [&](int m, T &s0, T &s1, T &s2) {
                if (lane < m) {
                    G x, y, z;
                    int j;
                    candidate(hits[warp][lane], x, y, z, j);
                    G d0 = (G)pi.x - x, d1 = (G)pi.y - y, d2 = (G)pi.z - z;
                    if (single) {
                        d0 -= L * d_rint(d0 * invL);
                        d1 -= L * d_rint(d1 * invL);
                        d2 -= L * d_rint(d2 * invL);
                    }
                    T Fv, Gv;
                    G ir;  // coincident particles (r = 0): no direction, the G term vanishes
                    if constexpr (kF32) {
                        real_FG_f32(d0 * d0 + d1 * d1 + d2 * d2, A.cf, Fv, Gv, ir);
                    } else {
                        const G rr = sqrt(d0 * d0 + d1 * d1 + d2 * d2);
                        double Fd, Gd;
                        if (table_FG(tab, (double)rr, Fd, Gd)) {
                            Fv = (T)Fd;
                            Gv = (T)Gd;
                        } else {
                            real_FG<T>((T)rr, xi, a, Fv, Gv);
                        }
                        ir = rr > G(0) ? G(1) / rr : G(0);
                    }
                    PairRec &pq = prec[warp][lane];
                    pq.rf.x = (T)(d0 * ir);
                    pq.rf.y = (T)(d1 * ir);
                    pq.rf.z = (T)(d2 * ir);
                    pq.rf.w = Fv;
                    pq.gfac = Gv;
                    pq.frow = F + (size_t)j * C;
                }
                __syncwarp();
                s0 = s1 = s2 = T(0);
                if (rok) {
#pragma unroll 4
                    for (int k = pp; k < m; k += PR) {
                        const PairRec &pq = prec[warp][k];
                        const auto rf = pq.rf;
                        const T *fj = pq.frow + 3 * r;
                        const T f0 = __ldg(fj), f1 = __ldg(fj + 1), f2 = __ldg(fj + 2);
                        const T rx = rf.x, ry = rf.y, rz = rf.z;
                        const T Fk = rf.w, Gd = pq.gfac * (rx * f0 + ry * f1 + rz * f2);
                        s0 += Fk * f0 + Gd * rx;
                        s1 += Fk * f1 + Gd * ry;
                        s2 += Fk * f2 + Gd * rz;
                    }
                }
                __syncwarp();
            };
            // candidate q within rc of particle i (and not i itself)
            auto test = [&](int q) {
                bool hit = false;
                bool maybe = q < ncand;
                if (pre && maybe) {
                    const float e0 = (float)pi.x - fx[q], e1 = (float)pi.y - fy[q],
                                e2 = (float)pi.z - fz[q];
                    maybe = e0 * e0 + e1 * e1 + e2 * e2 < pre_r2;
                }
                if (maybe) {
                    G x, y, z;
                    int j;
                    candidate(q, x, y, z, j);
                    if (j != ii) {
                        G d0 = (G)pi.x - x, d1 = (G)pi.y - y, d2 = (G)pi.z - z;
                        if (single) {
                            d0 -= L * d_rint(d0 * invL);
                            d1 -= L * d_rint(d1 * invL);
                            d2 -= L * d_rint(d2 * invL);
                        }
                        hit = d0 * d0 + d1 * d1 + d2 * d2 < rc2;
                    }
                }
                return hit;
            };
            // kU candidates per lane per iteration: hits are appended in candidate
            // order and evaluated 32 at a time
            const unsigned below = (1u << lane) - 1u;
            for (int q0 = 0; q0 < ncand; q0 += 32 * kU) {
                bool hu[kU];
#pragma unroll
                for (int v = 0; v < kU; v++) hu[v] = test(q0 + 32 * v + lane);
#pragma unroll
                for (int v = 0; v < kU; v++) {
                    const unsigned mv = __ballot_sync(0xffffffffu, hu[v]);
                    if (hu[v]) hits[warp][nh + __popc(mv & below)] = q0 + 32 * v + lane;
                    nh += __popc(mv);
                }
                __syncwarp();
                while (nh >= 32) {
                    T s0, s1, s2;
                    flush(32, s0, s1, s2);
                    a0.add(s0);
                    a1.add(s1);
                    a2.add(s2);
                    // the rest (at most 32 kU - 1 entries) moves down by 32
                    const int rest = nh - 32;
                    int e[kU];
#pragma unroll
                    for (int v = 0; v < kU; v++)
                        e[v] = lane + 32 * v < rest ? hits[warp][32 + 32 * v + lane] : 0;
                    __syncwarp();
#pragma unroll
                    for (int v = 0; v < kU; v++)
                        if (lane + 32 * v < rest) hits[warp][32 * v + lane] = e[v];
                    nh = rest;
                    __syncwarp();
                }
            }
            if (nh > 0) {
                T s0, s1, s2;
                flush(nh, s0, s1, s2);
                a0.add(s0);
                a1.add(s1);
                a2.add(s2);
            }
            // sum the PR pair slots of each right-hand side
            for (int o = RL; o < 32; o <<= 1) {
                a0.add(shfl_xor(a0, o));
                a1.add(shfl_xor(a1, o));
                a2.add(shfl_xor(a2, o));
            }
            if (pp == 0 && rok) {
                const T *fi = F + (size_t)ii * C + 3 * r;
                if (with_self) {
                    a0.add(self_c * fi[0]);
                    a1.add(self_c * fi[1]);
                    a2.add(self_c * fi[2]);
                }
                T *o = W + (size_t)ii * C + 3 * r;
                o[0] = a0.value();
                o[1] = a1.value();
                o[2] = a2.value();
            }
        }
    }
}

template <typename T, typename G>
__global__ void __launch_bounds__(kThreads, sizeof(T) == 4 ? 16 : 8) k_realspace(RealArgs<T> A) {
    realspace_body<T, G>(A, blockIdx.x);
}

// Many systems in one persistent launch over their cells.
template <typename T, typename G>
__global__ void __launch_bounds__(kThreads, sizeof(T) == 4 ? 16 : 8)
k_realspace_batch(const RealArgs<T> *__restrict__ sys, const int *__restrict__ prefix, int nsys,
                  int total) {
    for (int w = blockIdx.x; w < total; w += gridDim.x) {
        const int k = batch_find(prefix, nsys, w);
        realspace_body<T, G>(sys[k], w - prefix[k]);
        __syncthreads();
    }
}

}  // namespace

double real_self_coeff(double xi, double a) {
    const double rsp = 0.56418958354775628695;
    return (1.0 - 6.0 * xi * a * rsp + 40.0 / 3.0 * xi * xi * xi * a * a * a * rsp) / a;
}

template <typename T>
RealArgs<T> real_args(int nc, const int *cell_off, const int *cell_perm, const void *cpos,
                      const T *F, int R, double L, double rc, double xi, double a, int with_self,
                      const PairTable &tab, T *W) {
    RealArgs<T> A;
    A.nc = nc;
    A.cell_off = cell_off;
    A.cell_perm = cell_perm;
    A.cpos = cpos;
    A.F = F;
    A.W = W;
    A.R = R;
    A.with_self = with_self;
    A.L = L;
    A.h = L / nc;
    A.rc2 = rc * rc;
    A.xi = xi;
    A.a = a;
    A.self_c = real_self_coeff(xi, a);
    A.tab = tab;
    const double rsp = 0.56418958354775628695, a2 = a * a, xi2 = xi * xi, xi3 = xi2 * xi,
                 xi5 = xi3 * xi2, xi7 = xi5 * xi2;
    RealCoef &c = A.cf;
    c.xi = (float)xi;
    c.xi2 = (float)xi2;
    c.a2x4 = (float)(4.0 * a2);
    c.xi3a2 = (float)(xi3 * a2);
    c.ia = (float)(1.0 / a);
    c.n1 = (float)(9.0 / (32.0 * a2));
    c.n2 = (float)(3.0 / (32.0 * a2));
    c.A4 = (float)(4.0 * rsp * xi7 * a2);
    c.A2 = (float)(rsp * (3.0 * xi3 - 20.0 * xi5 * a2));
    c.A0 = (float)(rsp * (-4.5 * xi + 14.0 * xi3 * a2));
    c.Am2 = (float)(rsp * xi * a2);
    c.B2 = (float)(rsp * (-3.0 * xi3 + 16.0 * xi5 * a2));
    c.B0 = (float)(rsp * (1.5 * xi - 2.0 * xi3 * a2));
    c.Bm2 = (float)(-3.0 * rsp * xi * a2);
    c.c1 = (float)(0.5 * a2);
    c.c3 = (float)(-1.5 * a2);
    c.L = (float)L;
    c.h = (float)A.h;
    c.rc2 = (float)A.rc2;
    c.self_c = (float)A.self_c;
    return A;
}

template <typename T>
cudaError_t launch_realspace(int nc, const int *cell_off, const int *cell_perm, const void *cpos,
                             const T *F, int R, double L, double rc, double xi, double a,
                             int with_self, const PairTable &tab, T *W, cudaStream_t s) {
    const int ncell = nc * nc * nc;
    const RealArgs<T> A = real_args<T>(nc, cell_off, cell_perm, cpos, F, R, L, rc, xi, a,
                                       with_self, tab, W);
    if constexpr (sizeof(T) == 8)
        k_realspace<T, double><<<ncell, kThreads, 0, s>>>(A);
    else
        k_realspace<T, float><<<ncell, kThreads, 0, s>>>(A);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_realspace_batch(const RealArgs<T> *sys, const int *prefix, int nsys,
                                   int total, cudaStream_t s) {
    if (total <= 0) return cudaSuccess;
    using G = typename std::conditional<sizeof(T) == 8, double, float>::type;
    auto kern = k_realspace_batch<T, G>;
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreads, 0);
    const int grid = std::max(1, std::min(total, sms * std::max(per_sm, 1)));
    kern<<<grid, kThreads, 0, s>>>(sys, prefix, nsys, total);
    return cudaGetLastError();
}

template RealArgs<float> real_args<float>(int, const int *, const int *, const void *,
                                          const float *, int, double, double, double, double, int,
                                          const PairTable &, float *);
template RealArgs<double> real_args<double>(int, const int *, const int *, const void *,
                                            const double *, int, double, double, double, double,
                                            int, const PairTable &, double *);
template cudaError_t launch_realspace_batch<float>(const RealArgs<float> *, const int *, int, int,
                                                   cudaStream_t);
template cudaError_t launch_realspace_batch<double>(const RealArgs<double> *, const int *, int,
                                                    int, cudaStream_t);

template <typename T>
cudaError_t launch_realspace(int nc, const int *cell_off, const int *cell_perm, const void *cpos,
                             const T *F, int R, double L, double rc, double xi, double a,
                             int with_self, T *W, cudaStream_t s) {
    return launch_realspace<T>(nc, cell_off, cell_perm, cpos, F, R, L, rc, xi, a, with_self,
                               PairTable{}, W, s);
}

namespace {

// real_FG on the host (same formulas, std::erf / std::erfc / std::exp in FP64).
void host_real_FG(double r, double xi, double a, double &F, double &G) {
    static const double ser_s[10] = {1.0, -1.0 / 3, 1.0 / 10, -1.0 / 42, 1.0 / 216,
                                     -1.0 / 1320, 1.0 / 9360, -1.0 / 75600,
                                     1.0 / 685440, -1.0 / 6894720};
    static const double ser_p[10] = {2.0 / 3, -2.0 / 5, 1.0 / 7, -1.0 / 27, 1.0 / 132,
                                     -1.0 / 780, 1.0 / 5400, -1.0 / 42840,
                                     1.0 / 383040, -1.0 / 3810240};
    const double rsp = 0.56418958354775628695;
    const double x = xi * r, x2 = x * x, e = std::exp(-x2);
    if (r < 2.0 * a) {
        double S = 0.0, P = 0.0;
        if (x < 0.5) {
            for (int k = 9; k >= 0; k--) {
                S = S * x2 + ser_s[k];
                P = P * x2 + ser_p[k];
            }
            S *= 2.0 * rsp;
            P *= 2.0 * rsp;
        } else {
            const double ef = std::erf(x);
            S = ef / x;
            P = (ef - 2.0 * rsp * x * e) / (x2 * x);
        }
        const double x4 = x2 * x2, xi3a2 = xi * xi * xi * a * a;
        F = xi * (-0.75 * S + rsp * e * (3.0 * x2 - 4.5)) +
            xi3a2 * (-0.5 * P + rsp * e * (4.0 * x4 - 20.0 * x2 + 14.0)) +
            (1.0 - 9.0 * r / (32.0 * a)) / a;
        G = xi * (-0.75 * S + rsp * e * (1.5 - 3.0 * x2)) +
            xi3a2 * (1.5 * P + rsp * e * (-4.0 * x4 + 16.0 * x2 - 2.0)) + 3.0 * r / (32.0 * a * a);
        return;
    }
    const double ec = std::erfc(x);
    const double r2 = r * r, a3 = a * a * a, ir = 1.0 / r, ir3 = ir * ir * ir, ir2 = ir * ir;
    const double xi2 = xi * xi, xi3 = xi2 * xi, xi5 = xi3 * xi2, xi7 = xi5 * xi2;
    const double f = ec * (0.75 * a * ir + 0.5 * a3 * ir3) +
                     e * rsp * (4.0 * xi7 * a3 * r2 * r2 + 3.0 * xi3 * a * r2 - 20.0 * xi5 * a3 * r2 -
                                4.5 * xi * a + 14.0 * xi3 * a3 + xi * a3 * ir2);
    const double g = ec * (0.75 * a * ir - 1.5 * a3 * ir3) +
                     e * rsp * (-4.0 * xi7 * a3 * r2 * r2 - 3.0 * xi3 * a * r2 + 16.0 * xi5 * a3 * r2 +
                                1.5 * xi * a - 2.0 * xi3 * a3 - 3.0 * xi * a3 * ir2);
    F = f / a;
    G = g / a;
}

// Chebyshev coefficients (degree kPairDeg) of F and G on [x0, x0 + h],
// interleaved, from the values at the kPairDeg + 1 Chebyshev nodes.
void fit_segment(double x0, double h, double xi, double a, double *out) {
    constexpr int n = kPairDeg + 1;
    double fv[n], gv[n];
    for (int j = 0; j < n; j++) {
        const double th = M_PI * (j + 0.5) / n;
        host_real_FG(x0 + 0.5 * h * (std::cos(th) + 1.0), xi, a, fv[j], gv[j]);
    }
    for (int k = 0; k < n; k++) {
        double sf = 0.0, sg = 0.0;
        for (int j = 0; j < n; j++) {
            const double c = std::cos(M_PI * k * (j + 0.5) / n);
            sf += fv[j] * c;
            sg += gv[j] * c;
        }
        out[2 * k] = 2.0 * sf / n;
        out[2 * k + 1] = 2.0 * sg / n;
    }
}

double eval_segment(const double *c, double t, int which) {
    double b = 0.0, b1 = 0.0;
    for (int k = kPairDeg; k >= 1; k--) {
        const double nb = 2.0 * t * b - b1 + c[2 * k + which];
        b1 = b;
        b = nb;
    }
    return t * b - b1 + 0.5 * c[which];
}

}  // namespace

bool build_pair_table(double xi, double a, double rc, std::vector<double> *coef, PairTable *t) {
    // [r_lo, r_mid): overlap form (r < 2a); [r_mid, rc]: far form.  Below r_lo
    // = a/2 the closed form's cancelling 1/r^2 terms leave rounding noise above
    // 1e-13 relative that no fit reproduces: those (rare) pairs are evaluated
    // directly.
    const double r_lo = 0.5 * a, r_mid = std::min(2.0 * a, rc);
    if (rc <= r_lo) return false;
    double hmax = 0.1 * std::min(a, 1.0 / xi);
    for (int attempt = 0; attempt < 4; attempt++, hmax *= 0.5) {
        const int n1 = std::max(1, (int)std::ceil((r_mid - r_lo) / hmax));
        const int n2 = rc > r_mid ? std::max(1, (int)std::ceil((rc - r_mid) / hmax)) : 0;
        if (n1 + n2 > 4096) break;
        const double h1 = (r_mid - r_lo) / n1, h2 = n2 ? (rc - r_mid) / n2 : 1.0;
        coef->assign((size_t)(n1 + n2) * (kPairDeg + 1) * 2, 0.0);
        for (int s = 0; s < n1 + n2; s++) {
            const double x0 = s < n1 ? r_lo + s * h1 : r_mid + (s - n1) * h2;
            fit_segment(x0, s < n1 ? h1 : h2, xi, a, coef->data() + (size_t)s * (kPairDeg + 1) * 2);
        }
        // the fit between the nodes, relative to the function scale there
        bool ok = true;
        for (int s = 0; s < n1 + n2 && ok; s++) {
            const double x0 = s < n1 ? r_lo + s * h1 : r_mid + (s - n1) * h2;
            const double hh = s < n1 ? h1 : h2;
            const double *c = coef->data() + (size_t)s * (kPairDeg + 1) * 2;
            for (int q = 0; q <= 16 && ok; q++) {
                const double tt = -1.0 + q / 8.0;
                double F, G;
                host_real_FG(x0 + 0.5 * hh * (tt + 1.0), xi, a, F, G);
                const double scale = std::fabs(F) + std::fabs(G) + 1e-300;
                ok = std::fabs(eval_segment(c, tt, 0) - F) <= 2e-13 * scale &&
                     std::fabs(eval_segment(c, tt, 1) - G) <= 2e-13 * scale;
            }
        }
        if (!ok) continue;
        t->coef = nullptr;  // the caller points it at the device copy
        t->r_lo = r_lo;
        t->r_mid = r_mid;
        t->r_hi = rc;
        t->inv_h1 = 1.0 / h1;
        t->inv_h2 = 1.0 / h2;
        t->nseg1 = n1;
        t->nseg2 = n2;
        return true;
    }
    return false;
}

template cudaError_t launch_realspace<float>(int, const int *, const int *, const void *,
                                             const float *, int, double, double, double, double,
                                             int, float *, cudaStream_t);
template cudaError_t launch_realspace<double>(int, const int *, const int *, const void *,
                                              const double *, int, double, double, double,
                                              double, int, double *, cudaStream_t);
template cudaError_t launch_realspace<float>(int, const int *, const int *, const void *,
                                             const float *, int, double, double, double, double,
                                             int, const PairTable &, float *, cudaStream_t);
template cudaError_t launch_realspace<double>(int, const int *, const int *, const void *,
                                              const double *, int, double, double, double,
                                              double, int, const PairTable &, double *,
                                              cudaStream_t);

}  // namespace spme
