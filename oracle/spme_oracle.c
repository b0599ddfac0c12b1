/*
 * TEST INFRASTRUCTURE ONLY — the oracle (see spme_oracle.h).  FP64, OpenMP.
 * Each function cites the reference lines it restates.  Nothing in the
 * product path calls this code.
 */
#include "spme_oracle.h"
#include "fft.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORACLE_MAXP 16

static int nthreads_or_all(int nthreads)
{
#ifdef _OPENMP
    return nthreads > 0 ? nthreads : omp_get_max_threads();
#else
    (void)nthreads;
    return 1;
#endif
}

static inline long pmod(long x, long m)
{
    long r = x % m;
    return r < 0 ? r + m : r;
}

/* B-spline weights.  The reference evaluates the same polynomials through the
 * monomial table tab_W (old-version/spme.c:25-40, used at :258-279 with
 * g = frac - 1/2); here they come from the Cox-de Boor recursion
 *   M_n(x) = [x M_{n-1}(x) + (n - x) M_{n-1}(x - 1)] / (n - 1),  M_2(x) = 1 - |x - 1|. */
void oracle_bspline_weights(int p, double w, double *out)
{
    double a[ORACLE_MAXP + 1];
    int n, k;
    a[0] = w;        /* M_2(w)     */
    a[1] = 1.0 - w;  /* M_2(w + 1) */
    for (n = 3; n <= p; n++) {
        a[n - 1] = 0.0;
        for (k = n - 1; k >= 1; k--)
            a[k] = ((w + k) * a[k] + ((double)n - w - k) * a[k - 1]) / (double)(n - 1);
        a[0] = w * a[0] / (double)(n - 1);
    }
    for (k = 0; k < p; k++) out[k] = a[p - 1 - k];
}

/* old-version/spme.c:96-126: map[m] = 2 pi m'/L with m' = m for m <= K/2 and
 * m - K above; b(m) = e^{i(p-1)phi} / sum_{j<p-1} M_p(j+1) e^{i j phi},
 * phi = map[m] L / K.  Only |b|^2 = 1/|den|^2 enters the influence table. */
void oracle_bspline_moduli2(int K, int p, double *bmod2)
{
    double mp[ORACLE_MAXP];
    int m, j;
    oracle_bspline_weights(p, 0.0, mp); /* mp[j] = M_p(p - 1 - j) */
    for (m = 0; m < K; m++) {
        int mm = m <= K / 2 ? m : m - K;
        double phi = 2.0 * M_PI * (double)mm / (double)K;
        double re = 0.0, im = 0.0;
        for (j = 0; j < p - 1; j++) {
            double s = mp[p - 2 - j]; /* M_p(j + 1) */
            re += s * cos(j * phi);
            im += s * sin(j * phi);
        }
        bmod2[m] = 1.0 / (re * re + im * im);
    }
}

/* old-version/spme.c:43-60 with aa = ab = a (the reference passes 1.0, 1.0 at :141). */
double oracle_scalar_recip(double k, double xi, double a)
{
    double kx = k / xi;
    double kx2 = kx * kx;
    double k2 = k * k;
    return 6.0 * M_PI * exp(-kx2 / 4.0) * (1.0 - k2 * (2.0 * a * a) / 6.0) / k2
           * (1.0 + kx2 * (1.0 / 4.0 + kx2 / 8.0));
}

static double wavenumber(int m, int K, double L)
{
    int mm = m <= K / 2 ? m : m - K;
    return 2.0 * M_PI * (double)mm / L;
}

typedef struct {
    int start[3];
    double w[3][ORACLE_MAXP];
} oracle_pstencil;

/* old-version/spme.c:235-256: c = pos/L*K, start = (floor(c) - p/2 + 1) mod K,
 * weights from frac(c). */
static void particle_stencil(const double *x, double L, int K, int p, oracle_pstencil *s)
{
    int d;
    for (d = 0; d < 3; d++) {
        double c = x[d] / L * (double)K;
        double fl = floor(c);
        s->start[d] = (int)pmod((long)fl - p / 2 + 1, K);
        oracle_bspline_weights(p, c - fl, s->w[d]);
    }
}

int oracle_recip(int np, const double *pos, double L, double xi, double a, int K, int p,
                 int nrhs, double alpha, const double *f, long ldf, double beta,
                 double *u, long ldu, int nthreads)
{
    int nt = nthreads_or_all(nthreads);
    long K3 = (long)K * K * K, Kh = K / 2 + 1, Kc = (long)K * K * Kh;
    double *map, *bmod2, *grid;
    offt_cpx *half;
    oracle_pstencil *st;
    int *slab_of, *order, *slab_start, nslab, r, i;
    double scale;

    if (np < 0 || K < 2 || p < 2 || p > ORACLE_MAXP || (p & 1) || nrhs < 0) return 1;
    if (np == 0 || nrhs == 0) {
        for (r = 0; r < nrhs; r++)
            for (i = 0; i < 3 * np; i++) u[r * ldu + i] *= beta;
        return 0;
    }
    map = (double *)malloc(sizeof(double) * K);
    bmod2 = (double *)malloc(sizeof(double) * K);
    grid = (double *)malloc(sizeof(double) * 3 * K3);
    half = (offt_cpx *)malloc(sizeof(offt_cpx) * 3 * Kc);
    st = (oracle_pstencil *)malloc(sizeof(oracle_pstencil) * np);
    slab_of = (int *)malloc(sizeof(int) * np);
    order = (int *)malloc(sizeof(int) * np);
    if (!map || !bmod2 || !grid || !half || !st || !slab_of || !order) return 2;
    for (i = 0; i < K; i++) map[i] = wavenumber(i, K, L);
    oracle_bspline_moduli2(K, p, bmod2);

    /* compute_P (old-version/spme.c:158-297), in factored form */
    #pragma omp parallel for num_threads(nt)
    for (i = 0; i < np; i++) particle_stencil(&pos[3 * i], L, K, p, &st[i]);

    /* Race-free parallel spread: group particles by z-slabs of width >= p and
     * process even then odd slabs (a particle in slab s only touches s, s+1). */
    nslab = 2 * (K / (2 * p));
    if (nslab < 2 || nt == 1) nslab = 1;
    slab_start = (int *)calloc(nslab + 1, sizeof(int));
    for (i = 0; i < np; i++) {
        int s = (int)(((long)st[i].start[2] * nslab) / K);
        slab_of[i] = s;
        slab_start[s + 1]++;
    }
    for (i = 0; i < nslab; i++) slab_start[i + 1] += slab_start[i];
    {
        int *cur = (int *)malloc(sizeof(int) * (nslab + 1));
        memcpy(cur, slab_start, sizeof(int) * (nslab + 1));
        for (i = 0; i < np; i++) order[cur[slab_of[i]]++] = i;
        free(cur);
    }

    scale = alpha * ((double)K * K * K) / (L * L * L); /* old-version/spme.c:699 */
    for (r = 0; r < nrhs; r++) {
        const double *fr = f + r * ldf;
        double *ur = u + r * ldu;
        int phase, comp;
        memset(grid, 0, sizeof(double) * 3 * K3);
        /* spread (old-version/spme_kernel.c:231-247 per particle) */
        for (phase = 0; phase < (nslab > 1 ? 2 : 1); phase++) {
            int s;
            #pragma omp parallel for num_threads(nt) schedule(dynamic)
            for (s = phase; s < nslab; s += (nslab > 1 ? 2 : 1)) {
                int k;
                for (k = slab_start[s]; k < slab_start[s + 1]; k++) {
                    int ip = order[k], x, y, z;
                    const oracle_pstencil *ps = &st[ip];
                    for (z = 0; z < p; z++) {
                        long zz = (ps->start[2] + z) % K;
                        for (y = 0; y < p; y++) {
                            long yy = (ps->start[1] + y) % K;
                            double wzy = ps->w[2][z] * ps->w[1][y];
                            for (x = 0; x < p; x++) {
                                long xx = (ps->start[0] + x) % K;
                                long idx = (zz * K + yy) * K + xx;
                                double w = wzy * ps->w[0][x];
                                grid[0 * K3 + idx] += w * fr[3 * ip + 0];
                                grid[1 * K3 + idx] += w * fr[3 * ip + 1];
                                grid[2 * K3 + idx] += w * fr[3 * ip + 2];
                            }
                        }
                    }
                }
            }
        }
        /* forward FFT (old-version/spme.c:654-656) */
        for (comp = 0; comp < 3; comp++)
            offt_r2c_3d(K, grid + comp * K3, K, (long)K * K, half + comp * Kc, Kh, K * Kh, nt);
        /* influence (old-version/spme_kernel.c:114-228 with the table of
         * old-version/spme.c:129-150): g <- S|b|^2 (I - k k^T / k^2) g on the
         * half spectrum, the same real matrix on re and im, k = 0 zeroed. */
        {
            long j;
            #pragma omp parallel for num_threads(nt)
            for (j = 0; j < (long)K * K; j++) {
                int z = (int)(j / K), y = (int)(j % K), x;
                double kz = map[z], ky = map[y], kyz = ky * ky + kz * kz;
                for (x = 0; x < Kh; x++) {
                    double kx = map[x];
                    long id = j * Kh + x;
                    offt_cpx g0 = half[id], g1 = half[Kc + id], g2 = half[2 * Kc + id];
                    double k2 = kx * kx + kyz, kk, m2, b0, b1, b2, b3, b4, b5;
                    if (k2 == 0.0) {
                        half[id].re = half[id].im = 0.0;
                        half[Kc + id].re = half[Kc + id].im = 0.0;
                        half[2 * Kc + id].re = half[2 * Kc + id].im = 0.0;
                        continue;
                    }
                    m2 = oracle_scalar_recip(sqrt(k2), xi, a) * bmod2[x] * bmod2[y] * bmod2[z];
                    kk = 1.0 / k2;
                    b0 = m2 - m2 * kx * kx * kk;
                    b1 = -m2 * kx * ky * kk;
                    b2 = -m2 * kx * kz * kk;
                    b3 = m2 - m2 * ky * ky * kk;
                    b4 = -m2 * ky * kz * kk;
                    b5 = m2 - m2 * kz * kz * kk;
                    half[id].re = b0 * g0.re + b1 * g1.re + b2 * g2.re;
                    half[id].im = b0 * g0.im + b1 * g1.im + b2 * g2.im;
                    half[Kc + id].re = b1 * g0.re + b3 * g1.re + b4 * g2.re;
                    half[Kc + id].im = b1 * g0.im + b3 * g1.im + b4 * g2.im;
                    half[2 * Kc + id].re = b2 * g0.re + b4 * g1.re + b5 * g2.re;
                    half[2 * Kc + id].im = b2 * g0.im + b4 * g1.im + b5 * g2.im;
                }
            }
        }
        /* backward FFT with 1/K^3 (old-version/spme.c:408-409,680-682) */
        for (comp = 0; comp < 3; comp++) {
            long q;
            offt_c2r_3d(K, half + comp * Kc, Kh, K * Kh, grid + comp * K3, K, (long)K * K, nt);
            for (q = 0; q < K3; q++) grid[comp * K3 + q] /= (double)K3;
        }
        /* interpolate (old-version/spme_kernel.c:8-31,34-62) */
        #pragma omp parallel for num_threads(nt) schedule(static)
        for (i = 0; i < np; i++) {
            const oracle_pstencil *ps = &st[i];
            double t0 = 0.0, t1 = 0.0, t2 = 0.0;
            int x, y, z;
            for (z = 0; z < p; z++) {
                long zz = (ps->start[2] + z) % K;
                for (y = 0; y < p; y++) {
                    long yy = (ps->start[1] + y) % K;
                    double wzy = ps->w[2][z] * ps->w[1][y];
                    for (x = 0; x < p; x++) {
                        long xx = (ps->start[0] + x) % K;
                        long idx = (zz * K + yy) * K + xx;
                        double w = wzy * ps->w[0][x];
                        t0 += grid[idx] * w;
                        t1 += grid[K3 + idx] * w;
                        t2 += grid[2 * K3 + idx] * w;
                    }
                }
            }
            ur[3 * i + 0] = beta * ur[3 * i + 0] + scale * t0;
            ur[3 * i + 1] = beta * ur[3 * i + 1] + scale * t1;
            ur[3 * i + 2] = beta * ur[3 * i + 2] + scale * t2;
        }
    }
    free(map); free(bmod2); free(grid); free(half); free(st);
    free(slab_of); free(order); free(slab_start);
    return 0;
}

/* Beenakker (1986) real-space Ewald RPY kernel, in mobility*6*pi*eta units
 * (the mu0 = 1/(6 pi eta a) form divided by a), with the RPY overlap form
 * replacing the far-field form for r < 2a. */
void oracle_real_FG(double r, double xi, double a, double *F, double *G)
{
    /* Beenakker's real-space RPY form divided by a; for r < 2a plus
     * (overlap RPY - far-field RPY), whose 1/r and 1/r^3 terms cancel: there
     * the sum is written with x = xi r, S(x) = erf(x)/x and
     * psi(x) = (erf(x) - 2x e^{-x^2}/sqrt(pi))/x^3 (Maclaurin series below
     * x = 0.5), which keeps full precision as r -> 0 and is finite at r = 0. */
    static const double ser_s[10] = {1.0, -1.0 / 3, 1.0 / 10, -1.0 / 42, 1.0 / 216,
                                     -1.0 / 1320, 1.0 / 9360, -1.0 / 75600,
                                     1.0 / 685440, -1.0 / 6894720};
    static const double ser_p[10] = {2.0 / 3, -2.0 / 5, 1.0 / 7, -1.0 / 27, 1.0 / 132,
                                     -1.0 / 780, 1.0 / 5400, -1.0 / 42840,
                                     1.0 / 383040, -1.0 / 3810240};
    const double rsp = 1.0 / sqrt(M_PI);
    double x = xi * r, x2 = x * x, e = exp(-x2);
    if (r < 2.0 * a) {
        double S = 0.0, P = 0.0, x4 = x2 * x2, xi3a2 = xi * xi * xi * a * a;
        int k;
        if (x < 0.5) {
            for (k = 9; k >= 0; k--) {
                S = S * x2 + ser_s[k];
                P = P * x2 + ser_p[k];
            }
            S *= 2.0 * rsp;
            P *= 2.0 * rsp;
        } else {
            double ef = erf(x);
            S = ef / x;
            P = (ef - 2.0 * rsp * x * e) / (x2 * x);
        }
        *F = xi * (-0.75 * S + rsp * e * (3.0 * x2 - 4.5))
             + xi3a2 * (-0.5 * P + rsp * e * (4.0 * x4 - 20.0 * x2 + 14.0))
             + (1.0 - 9.0 * r / (32.0 * a)) / a;
        *G = xi * (-0.75 * S + rsp * e * (1.5 - 3.0 * x2))
             + xi3a2 * (1.5 * P + rsp * e * (-4.0 * x4 + 16.0 * x2 - 2.0))
             + 3.0 * r / (32.0 * a * a);
        return;
    }
    {
        double ec = erfc(x);
        double r2 = r * r, a3 = a * a * a;
        double xi2 = xi * xi, xi3 = xi2 * xi, xi5 = xi3 * xi2, xi7 = xi5 * xi2;
        double f = ec * (0.75 * a / r + 0.5 * a3 / (r2 * r))
                   + e * rsp * (4.0 * xi7 * a3 * r2 * r2 + 3.0 * xi3 * a * r2 - 20.0 * xi5 * a3 * r2
                                - 4.5 * xi * a + 14.0 * xi3 * a3 + xi * a3 / r2);
        double g = ec * (0.75 * a / r - 1.5 * a3 / (r2 * r))
                   + e * rsp * (-4.0 * xi7 * a3 * r2 * r2 - 3.0 * xi3 * a * r2 + 16.0 * xi5 * a3 * r2
                                + 1.5 * xi * a - 2.0 * xi3 * a3 - 3.0 * xi * a3 / r2);
        *F = f / a;
        *G = g / a;
    }
}

double oracle_self_coeff(double xi, double a)
{
    const double rsp = 1.0 / sqrt(M_PI);
    return (1.0 - 6.0 * xi * a * rsp + 40.0 / 3.0 * xi * xi * xi * a * a * a * rsp) / a;
}

int oracle_real_self(int np, const double *pos, double L, double xi, double a, double rc,
                     int nrhs, double alpha, const double *f, long ldf, double beta,
                     double *u, long ldu, int flags, int nthreads)
{
    int nt = nthreads_or_all(nthreads);
    int nc = (int)floor(L / rc), i, r;
    int *cell_start, *cell_of, *order;
    double s0 = oracle_self_coeff(xi, a), rc2 = rc * rc;
    if (np < 0 || nrhs < 0 || !(rc > 0.0) || !(rc < 0.5 * L)) return 1;
    if (np == 0 || nrhs == 0) return 0;
    if (nc < 3) nc = 1;
    cell_start = (int *)calloc((size_t)nc * nc * nc + 1, sizeof(int));
    cell_of = (int *)malloc(sizeof(int) * np);
    order = (int *)malloc(sizeof(int) * np);
    for (i = 0; i < np; i++) {
        int c[3], d;
        for (d = 0; d < 3; d++) {
            double x = pos[3 * i + d] - L * floor(pos[3 * i + d] / L);
            c[d] = (int)(x / L * nc);
            if (c[d] >= nc) c[d] = nc - 1;
        }
        cell_of[i] = (c[2] * nc + c[1]) * nc + c[0];
        cell_start[cell_of[i] + 1]++;
    }
    for (i = 0; i < nc * nc * nc; i++) cell_start[i + 1] += cell_start[i];
    {
        int *cur = (int *)malloc(sizeof(int) * ((size_t)nc * nc * nc + 1));
        memcpy(cur, cell_start, sizeof(int) * ((size_t)nc * nc * nc + 1));
        for (i = 0; i < np; i++) order[cur[cell_of[i]]++] = i;
        free(cur);
    }
    #pragma omp parallel for num_threads(nt) schedule(dynamic, 16) private(r)
    for (i = 0; i < np; i++) {
        double acc[3 * 64];
        double *ac = nrhs <= 64 ? acc : (double *)calloc((size_t)3 * nrhs, sizeof(double));
        int ci = cell_of[i], cx = ci % nc, cy = (ci / nc) % nc, cz = ci / (nc * nc);
        int dx, dy, dz, span = nc >= 3 ? 1 : 0;
        for (r = 0; r < 3 * nrhs; r++) ac[r] = 0.0;
        if (flags & 1) {
            for (dz = -span; dz <= span; dz++)
                for (dy = -span; dy <= span; dy++)
                    for (dx = -span; dx <= span; dx++) {
                        int cc = ((int)pmod(cz + dz, nc) * nc + (int)pmod(cy + dy, nc)) * nc
                                 + (int)pmod(cx + dx, nc);
                        int k;
                        for (k = cell_start[cc]; k < cell_start[cc + 1]; k++) {
                            int j = order[k], d;
                            double dv[3], r2 = 0.0, rr, F, G;
                            if (j == i) continue;
                            for (d = 0; d < 3; d++) {
                                double q = pos[3 * i + d] - pos[3 * j + d];
                                q -= L * nearbyint(q / L);
                                dv[d] = q;
                                r2 += q * q;
                            }
                            if (r2 >= rc2) continue;
                            rr = sqrt(r2);
                            oracle_real_FG(rr, xi, a, &F, &G);
                            /* coincident particles: no direction, the G term vanishes */
                            for (d = 0; d < 3; d++) dv[d] = rr > 0.0 ? dv[d] / rr : 0.0;
                            for (r = 0; r < nrhs; r++) {
                                const double *fj = f + r * ldf + 3 * j;
                                double dot = dv[0] * fj[0] + dv[1] * fj[1] + dv[2] * fj[2];
                                ac[3 * r + 0] += F * fj[0] + G * dv[0] * dot;
                                ac[3 * r + 1] += F * fj[1] + G * dv[1] * dot;
                                ac[3 * r + 2] += F * fj[2] + G * dv[2] * dot;
                            }
                        }
                    }
        }
        for (r = 0; r < nrhs; r++) {
            int d;
            for (d = 0; d < 3; d++) {
                double v = ac[3 * r + d];
                if (flags & 2) v += s0 * f[r * ldf + 3 * i + d];
                u[r * ldu + 3 * i + d] = beta * u[r * ldu + 3 * i + d] + alpha * v;
            }
        }
        if (ac != acc) free(ac);
    }
    free(cell_start); free(cell_of); free(order);
    return 0;
}

int oracle_recip_direct(int np, const double *pos, double L, double xi, double a,
                        double kcut, int nrhs, double alpha, const double *f, long ldf,
                        double beta, double *u, long ldu, int nthreads)
{
    int nt = nthreads_or_all(nthreads);
    int nmax = (int)floor(kcut * L / (2.0 * M_PI)), i, r;
    double V = L * L * L;
    double *acc;
    if (np < 0 || nrhs < 0) return 1;
    acc = (double *)calloc((size_t)3 * np * (nrhs > 0 ? nrhs : 1), sizeof(double));
    #pragma omp parallel num_threads(nt) private(r, i)
    {
        double *loc = (double *)calloc((size_t)3 * np * (nrhs > 0 ? nrhs : 1), sizeof(double));
        double *cs = (double *)malloc(sizeof(double) * 2 * (size_t)np);
        long side = 2L * nmax + 1, t;
        #pragma omp for schedule(dynamic, 8)
        for (t = 0; t < side * side * side; t++) {
            int n0 = (int)(t % side) - nmax, n1 = (int)((t / side) % side) - nmax,
                n2 = (int)(t / (side * side)) - nmax;
            double k[3] = { 2.0 * M_PI * n0 / L, 2.0 * M_PI * n1 / L, 2.0 * M_PI * n2 / L };
            double k2 = k[0] * k[0] + k[1] * k[1] + k[2] * k[2], S, kh[3];
            if (k2 == 0.0 || k2 > kcut * kcut) continue;
            S = oracle_scalar_recip(sqrt(k2), xi, a) / V;
            for (i = 0; i < 3; i++) kh[i] = k[i] / sqrt(k2);
            for (i = 0; i < np; i++) {
                double ph = k[0] * pos[3 * i] + k[1] * pos[3 * i + 1] + k[2] * pos[3 * i + 2];
                cs[2 * i] = cos(ph);
                cs[2 * i + 1] = sin(ph);
            }
            for (r = 0; r < nrhs; r++) {
                /* F(k) = sum_j f_j e^{-i k.x_j}; projected by (I - khat khat) */
                double Fr[3] = { 0, 0, 0 }, Fi[3] = { 0, 0, 0 }, dr, di;
                int d;
                for (i = 0; i < np; i++)
                    for (d = 0; d < 3; d++) {
                        double fv = f[r * ldf + 3 * i + d];
                        Fr[d] += fv * cs[2 * i];
                        Fi[d] -= fv * cs[2 * i + 1];
                    }
                dr = kh[0] * Fr[0] + kh[1] * Fr[1] + kh[2] * Fr[2];
                di = kh[0] * Fi[0] + kh[1] * Fi[1] + kh[2] * Fi[2];
                for (d = 0; d < 3; d++) { Fr[d] -= kh[d] * dr; Fi[d] -= kh[d] * di; }
                for (i = 0; i < np; i++)
                    for (d = 0; d < 3; d++)
                        loc[(long)r * 3 * np + 3 * i + d] +=
                            S * (cs[2 * i] * Fr[d] - cs[2 * i + 1] * Fi[d]);
            }
        }
        #pragma omp critical
        {
            long q;
            for (q = 0; q < 3L * np * nrhs; q++) acc[q] += loc[q];
        }
        free(loc);
        free(cs);
    }
    for (r = 0; r < nrhs; r++)
        for (i = 0; i < 3 * np; i++)
            u[r * ldu + i] = beta * u[r * ldu + i] + alpha * acc[(long)r * 3 * np + i];
    free(acc);
    return 0;
}
