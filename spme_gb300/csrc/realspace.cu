// Real-space Ewald RPY pair sum over a cell list within rc, plus the self
// term.  The reference has no real-space part (it computes only M_recip,
// old-version/spme.c:560-726); this restates Beenakker, J. Chem. Phys. 85,
// 1581 (1986), in the reference's units (mobility x 6 pi eta, matching
// scalar_recip at old-version/spme.c:43-60), with the RPY overlap form for
// pairs closer than 2a.
//
// One CTA per cell: the cell's particles (chunks of ICH) against the
// candidates of the 27 neighbour cells (chunks of JCH).  Phase A evaluates each
// pair within rc once (displacement from cell-relative coordinates, the
// scalar functions in T) into per-particle shared-memory lists; phase B applies
// every listed pair tensor to all right-hand sides, one thread per
// (particle, right-hand side).  Sums over a candidate chunk run in T and are
// accumulated across chunks in FP64.
#include "kernels.h"

namespace spme {

namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ float d_erfc(float x) { return erfcf(x); }
__device__ __forceinline__ double d_erfc(double x) { return erfc(x); }
__device__ __forceinline__ float d_exp(float x) { return expf(x); }
__device__ __forceinline__ double d_exp(double x) { return exp(x); }

// M_real(r) = F I + G rhat rhat, Beenakker's form divided by a, plus
// (overlap RPY - far-field RPY) for r < 2a.
template <typename T>
__device__ __forceinline__ void real_FG(T r, T xi, T a, T &F, T &G) {
    const T rsp = T(0.56418958354775628695);  // 1/sqrt(pi)
    const T xr = xi * r, e = d_exp(-xr * xr), ec = d_erfc(xr);
    const T r2 = r * r, a3 = a * a * a, ir = T(1) / r, ir3 = ir * ir * ir, ir2 = ir * ir;
    const T xi2 = xi * xi, xi3 = xi2 * xi, xi5 = xi3 * xi2, xi7 = xi5 * xi2;
    T f = ec * (T(0.75) * a * ir + T(0.5) * a3 * ir3) +
          e * rsp * (T(4) * xi7 * a3 * r2 * r2 + T(3) * xi3 * a * r2 - T(20) * xi5 * a3 * r2 -
                     T(4.5) * xi * a + T(14) * xi3 * a3 + xi * a3 * ir2);
    T g = ec * (T(0.75) * a * ir - T(1.5) * a3 * ir3) +
          e * rsp * (-T(4) * xi7 * a3 * r2 * r2 - T(3) * xi3 * a * r2 + T(16) * xi5 * a3 * r2 +
                     T(1.5) * xi * a - T(2) * xi3 * a3 - T(3) * xi * a3 * ir2);
    if (r < T(2) * a) {
        f += (T(1) - T(9) * r / (T(32) * a)) - (T(0.75) * a * ir + T(0.5) * a3 * ir3);
        g += (T(3) * r / (T(32) * a)) - (T(0.75) * a * ir - T(1.5) * a3 * ir3);
    }
    F = f / a;
    G = g / a;
}

template <typename G> struct Geo4;
template <> struct Geo4<float> { using type = float4; };
template <> struct Geo4<double> { using type = double4; };

__device__ __forceinline__ float d_rint(float x) { return rintf(x); }
__device__ __forceinline__ double d_rint(double x) { return rint(x); }

// T: pair-function and per-chunk accumulation type; G: pair geometry type.
// Positions are stored relative to the corner of their cell (cell edge
// h = L/nc), so the displacement to a candidate in neighbour cell c_i + dc is
// (o_i - o_j) - dc*h, which is accurate in FP32 for any box size.
template <typename T, typename G, int ICH, int JCH>
__global__ void __launch_bounds__(kThreads)
k_realspace(int nc, const int *__restrict__ cell_off, const int *__restrict__ cell_perm,
            const typename Geo4<G>::type *__restrict__ cpos, const T *__restrict__ F, int R,
            G L, G h, G rc2, T xi, T a, T self_c, int with_self, T *__restrict__ W) {
    __shared__ int nb_beg[27], nb_pre[28], nnb;
    __shared__ G nb_shift[27][3];
    __shared__ G ipos[ICH][3];
    __shared__ int iidx[ICH];
    __shared__ G jpos[JCH][3];
    __shared__ int jidx[JCH];
    __shared__ int pcnt[ICH];
    __shared__ T pF[ICH][JCH], pG[ICH][JCH], pR[3][ICH][JCH];
    __shared__ int pJ[ICH][JCH];

    constexpr int RCHMAX = kThreads / ICH;
    const int tid = threadIdx.x;
    const int cell = blockIdx.x;
    const int C = 3 * R;
    if (tid == 0) {
        const int cx = cell % nc, cy = (cell / nc) % nc, cz = cell / (nc * nc);
        const int span = nc >= 3 ? 1 : 0;
        int k = 0, pre = 0;
        for (int dz = -span; dz <= span; dz++)
            for (int dy = -span; dy <= span; dy++)
                for (int dx = -span; dx <= span; dx++) {
                    int c2 = (pmod(cz + dz, nc) * nc + pmod(cy + dy, nc)) * nc + pmod(cx + dx, nc);
                    nb_beg[k] = cell_off[c2];
                    nb_pre[k] = pre;
                    nb_shift[k][0] = (G)dx * h;
                    nb_shift[k][1] = (G)dy * h;
                    nb_shift[k][2] = (G)dz * h;
                    pre += cell_off[c2 + 1] - cell_off[c2];
                    k++;
                }
        nb_pre[k] = pre;
        nnb = k;
    }
    __syncthreads();
    const int ncand = nb_pre[nnb];
    const int ib0 = cell_off[cell], ie = cell_off[cell + 1];
    const bool single = nc < 3;
    const G invL = G(1) / L;

    for (int ib = ib0; ib < ie; ib += ICH) {
        const int ni = min(ICH, ie - ib);
        __syncthreads();
        if (tid < ni) {
            const auto p = cpos[ib + tid];
            ipos[tid][0] = p.x;
            ipos[tid][1] = p.y;
            ipos[tid][2] = p.z;
            iidx[tid] = cell_perm[ib + tid];
        }
        __syncthreads();
        for (int rb = 0; rb < R; rb += RCHMAX) {
            const int rch = min(RCHMAX, R - rb);
            const int il = tid / rch, r = rb + tid % rch;
            const bool active = tid < ni * rch;
            double acc0 = 0.0, acc1 = 0.0, acc2 = 0.0;
            for (int jb = 0; jb < ncand; jb += JCH) {
                const int nj = min(JCH, ncand - jb);
                __syncthreads();
                if (tid < nj) {
                    const int cand = jb + tid;
                    int k = 0;
                    while (cand >= nb_pre[k + 1]) k++;
                    const int js = nb_beg[k] + (cand - nb_pre[k]);
                    const auto p = cpos[js];
                    // candidate position expressed in the frame of cell i
                    jpos[tid][0] = p.x + nb_shift[k][0];
                    jpos[tid][1] = p.y + nb_shift[k][1];
                    jpos[tid][2] = p.z + nb_shift[k][2];
                    jidx[tid] = cell_perm[js];
                }
                if (tid < ICH) pcnt[tid] = 0;
                __syncthreads();
                for (int w = tid; w < ni * nj; w += kThreads) {
                    const int i2 = w / nj, jl = w - (w / nj) * nj;
                    if (jidx[jl] == iidx[i2]) continue;
                    G d0 = ipos[i2][0] - jpos[jl][0];
                    G d1 = ipos[i2][1] - jpos[jl][1];
                    G d2 = ipos[i2][2] - jpos[jl][2];
                    if (single) {
                        d0 -= L * d_rint(d0 * invL);
                        d1 -= L * d_rint(d1 * invL);
                        d2 -= L * d_rint(d2 * invL);
                    }
                    const G r2 = d0 * d0 + d1 * d1 + d2 * d2;
                    if (r2 >= rc2) continue;
                    const G rr = sqrt(r2);
                    T Fv, Gv;
                    real_FG<T>((T)rr, xi, a, Fv, Gv);
                    const int slot = atomicAdd(&pcnt[i2], 1);
                    const G ir = G(1) / rr;
                    pF[i2][slot] = Fv;
                    pG[i2][slot] = Gv;
                    pR[0][i2][slot] = (T)(d0 * ir);
                    pR[1][i2][slot] = (T)(d1 * ir);
                    pR[2][i2][slot] = (T)(d2 * ir);
                    pJ[i2][slot] = jidx[jl];
                }
                __syncthreads();
                if (active) {
                    T s0 = T(0), s1 = T(0), s2 = T(0);
                    const int np_ = pcnt[il];
                    for (int k = 0; k < np_; k++) {
                        const T *fj = F + (size_t)pJ[il][k] * C + 3 * r;
                        const T f0 = fj[0], f1 = fj[1], f2 = fj[2];
                        const T rx = pR[0][il][k], ry = pR[1][il][k], rz = pR[2][il][k];
                        const T Fk = pF[il][k], Gd = pG[il][k] * (rx * f0 + ry * f1 + rz * f2);
                        s0 += Fk * f0 + Gd * rx;
                        s1 += Fk * f1 + Gd * ry;
                        s2 += Fk * f2 + Gd * rz;
                    }
                    acc0 += (double)s0;
                    acc1 += (double)s1;
                    acc2 += (double)s2;
                }
            }
            if (active) {
                const int i = iidx[il];
                const T *fi = F + (size_t)i * C + 3 * r;
                if (with_self) {
                    acc0 += (double)self_c * (double)fi[0];
                    acc1 += (double)self_c * (double)fi[1];
                    acc2 += (double)self_c * (double)fi[2];
                }
                T *o = W + (size_t)i * C + 3 * r;
                o[0] = (T)acc0;
                o[1] = (T)acc1;
                o[2] = (T)acc2;
            }
        }
    }
}

}  // namespace

template <typename T>
cudaError_t launch_realspace(int nc, const int *cell_off, const int *cell_perm, const void *cpos,
                             const T *F, int R, double L, double rc, double xi, double a,
                             int with_self, T *W, cudaStream_t s) {
    const double rsp = 0.56418958354775628695;
    const double self_c = (1.0 - 6.0 * xi * a * rsp + 40.0 / 3.0 * xi * xi * xi * a * a * a * rsp) / a;
    const int ncell = nc * nc * nc;
    const double h = L / nc;
    if (sizeof(T) == 8)
        k_realspace<T, double, 16, 64><<<ncell, kThreads, 0, s>>>(
            nc, cell_off, cell_perm, (const double4 *)cpos, F, R, L, h, rc * rc, (T)xi, (T)a,
            (T)self_c, with_self, W);
    else
        k_realspace<T, float, 16, 96><<<ncell, kThreads, 0, s>>>(
            nc, cell_off, cell_perm, (const float4 *)cpos, F, R, (float)L, (float)h,
            (float)(rc * rc), (T)xi, (T)a, (T)self_c, with_self, W);
    return cudaGetLastError();
}

template cudaError_t launch_realspace<float>(int, const int *, const int *, const void *,
                                             const float *, int, double, double, double, double,
                                             int, float *, cudaStream_t);
template cudaError_t launch_realspace<double>(int, const int *, const int *, const void *,
                                              const double *, int, double, double, double,
                                              double, int, double *, cudaStream_t);

}  // namespace spme
