/*
 * Test infrastructure only (see fft.h): recursive mixed-radix decimation-in-
 * time complex FFT, written for the oracle from the textbook Cooley-Tukey
 * factorisation, plus 3D real transforms built from it.
 */
#include "fft.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

struct offt_plan {
    int n;
    int nf;
    int fac[64];
    offt_cpx *tw; /* tw[k] = exp(-2 pi i k / n) */
};

offt_plan *offt_plan_create(int n)
{
    offt_plan *p = (offt_plan *)calloc(1, sizeof(offt_plan));
    int m = n, k;
    if (!p || n < 1) { free(p); return NULL; }
    p->n = n;
    /* radix 4 first, then 2, 3, 5, then any remaining prime */
    while (m % 4 == 0) { p->fac[p->nf++] = 4; m /= 4; }
    while (m % 2 == 0) { p->fac[p->nf++] = 2; m /= 2; }
    for (k = 3; m > 1; k += 2) {
        while (m % k == 0) { p->fac[p->nf++] = k; m /= k; }
    }
    p->tw = (offt_cpx *)malloc(sizeof(offt_cpx) * (size_t)n);
    for (k = 0; k < n; k++) {
        double a = -2.0 * M_PI * (double)k / (double)n;
        p->tw[k].re = cos(a);
        p->tw[k].im = sin(a);
    }
    return p;
}

void offt_plan_destroy(offt_plan *p)
{
    if (p) { free(p->tw); free(p); }
}

static inline offt_cpx cmul(offt_cpx a, offt_cpx b)
{
    offt_cpx r = { a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re };
    return r;
}

static inline offt_cpx twid(const offt_plan *p, long e, int sign)
{
    offt_cpx w = p->tw[e % p->n];
    if (sign > 0) w.im = -w.im;
    return w;
}

/* out[0..n) = DFT of in[0], in[is], in[2 is], ...; twiddle step = N / n. */
static void rec(const offt_plan *p, const offt_cpx *in, long is, offt_cpx *out,
                int n, int fi, long tstep, int sign)
{
    int r, m, q, j, k;
    if (n == 1) { out[0] = in[0]; return; }
    r = p->fac[fi];
    m = n / r;
    for (q = 0; q < r; q++)
        rec(p, in + q * is, is * r, out + q * m, m, fi + 1, tstep * r, sign);
    if (r == 2) {
        for (k = 0; k < m; k++) {
            offt_cpx a = out[k];
            offt_cpx b = cmul(out[m + k], twid(p, (long)k * tstep, sign));
            out[k].re = a.re + b.re; out[k].im = a.im + b.im;
            out[m + k].re = a.re - b.re; out[m + k].im = a.im - b.im;
        }
    } else if (r == 4) {
        for (k = 0; k < m; k++) {
            offt_cpx a0 = out[k];
            offt_cpx a1 = cmul(out[m + k], twid(p, (long)k * tstep, sign));
            offt_cpx a2 = cmul(out[2 * m + k], twid(p, 2L * k * tstep, sign));
            offt_cpx a3 = cmul(out[3 * m + k], twid(p, 3L * k * tstep, sign));
            offt_cpx s02 = { a0.re + a2.re, a0.im + a2.im };
            offt_cpx d02 = { a0.re - a2.re, a0.im - a2.im };
            offt_cpx s13 = { a1.re + a3.re, a1.im + a3.im };
            offt_cpx d13 = { a1.re - a3.re, a1.im - a3.im };
            /* multiply d13 by sign*i: forward (sign<0) uses -i */
            offt_cpx jd13;
            if (sign < 0) { jd13.re = d13.im; jd13.im = -d13.re; }
            else { jd13.re = -d13.im; jd13.im = d13.re; }
            out[k].re = s02.re + s13.re; out[k].im = s02.im + s13.im;
            out[m + k].re = d02.re + jd13.re; out[m + k].im = d02.im + jd13.im;
            out[2 * m + k].re = s02.re - s13.re; out[2 * m + k].im = s02.im - s13.im;
            out[3 * m + k].re = d02.re - jd13.re; out[3 * m + k].im = d02.im - jd13.im;
        }
    } else {
        offt_cpx t[64];
        offt_cpx *tt = t;
        long rstep = (long)p->n / r;
        if (r > 64) tt = (offt_cpx *)malloc(sizeof(offt_cpx) * (size_t)r);
        for (k = 0; k < m; k++) {
            for (q = 0; q < r; q++)
                tt[q] = cmul(out[q * m + k], twid(p, (long)q * k * tstep, sign));
            for (j = 0; j < r; j++) {
                offt_cpx s = { 0.0, 0.0 };
                for (q = 0; q < r; q++) {
                    offt_cpx w = twid(p, ((long)j * q % r) * rstep, sign);
                    offt_cpx v = cmul(tt[q], w);
                    s.re += v.re; s.im += v.im;
                }
                out[j * m + k] = s;
            }
        }
        if (tt != t) free(tt);
    }
}

void offt_exec(const offt_plan *p, const offt_cpx *in, offt_cpx *out, int sign)
{
    rec(p, in, 1, out, p->n, 0, 1, sign);
}

static int nthreads_or_default(int nthreads)
{
#ifdef _OPENMP
    return nthreads > 0 ? nthreads : omp_get_max_threads();
#else
    (void)nthreads;
    return 1;
#endif
}

/* complex passes along y (stride cs1) and z (stride cs2) over kx in [0, nh) */
static void yz_passes(int n, int nh, offt_cpx *c, long cs1, long cs2, int sign,
                      const offt_plan *p, int nt)
{
    int pass;
    for (pass = 0; pass < 2; pass++) {
        long ls = pass == 0 ? cs1 : cs2;   /* stride along the transformed axis */
        long os = pass == 0 ? cs2 : cs1;   /* stride along the other axis */
        #pragma omp parallel num_threads(nt)
        {
            offt_cpx *a = (offt_cpx *)malloc(sizeof(offt_cpx) * (size_t)n * 2);
            offt_cpx *b = a + n;
            long line;
            #pragma omp for schedule(static)
            for (line = 0; line < (long)n * nh; line++) {
                long o = line / nh, kx = line % nh;
                offt_cpx *base = c + o * os + kx;
                int j;
                for (j = 0; j < n; j++) a[j] = base[j * ls];
                offt_exec(p, a, b, sign);
                for (j = 0; j < n; j++) base[j * ls] = b[j];
            }
            free(a);
        }
    }
}

void offt_r2c_3d(int n, const double *r, long rs1, long rs2,
                 offt_cpx *c, long cs1, long cs2, int nthreads)
{
    int nt = nthreads_or_default(nthreads);
    int nh = n / 2 + 1;
    offt_plan *p = offt_plan_create(n);
    #pragma omp parallel num_threads(nt)
    {
        offt_cpx *a = (offt_cpx *)malloc(sizeof(offt_cpx) * (size_t)n * 2);
        offt_cpx *b = a + n;
        long line;
        #pragma omp for schedule(static)
        for (line = 0; line < (long)n * n; line++) {
            long z = line / n, y = line % n;
            const double *rr = r + z * rs2 + y * rs1;
            offt_cpx *cc = c + z * cs2 + y * cs1;
            int j;
            for (j = 0; j < n; j++) { a[j].re = rr[j]; a[j].im = 0.0; }
            offt_exec(p, a, b, -1);
            for (j = 0; j < nh; j++) cc[j] = b[j];
        }
        free(a);
    }
    yz_passes(n, nh, c, cs1, cs2, -1, p, nt);
    offt_plan_destroy(p);
}

void offt_c2r_3d(int n, const offt_cpx *c_in, long cs1, long cs2,
                 double *r, long rs1, long rs2, int nthreads)
{
    int nt = nthreads_or_default(nthreads);
    int nh = n / 2 + 1;
    offt_cpx *c = (offt_cpx *)c_in; /* overwritten, as MKL's in-place backward does */
    offt_plan *p = offt_plan_create(n);
    yz_passes(n, nh, c, cs1, cs2, +1, p, nt);
    #pragma omp parallel num_threads(nt)
    {
        offt_cpx *a = (offt_cpx *)malloc(sizeof(offt_cpx) * (size_t)n * 2);
        offt_cpx *b = a + n;
        long line;
        #pragma omp for schedule(static)
        for (line = 0; line < (long)n * n; line++) {
            long z = line / n, y = line % n;
            const offt_cpx *cc = c + z * cs2 + y * cs1;
            double *rr = r + z * rs2 + y * rs1;
            int j;
            for (j = 0; j < nh; j++) a[j] = cc[j];
            for (j = nh; j < n; j++) { a[j].re = cc[n - j].re; a[j].im = -cc[n - j].im; }
            a[0].im = 0.0;
            if (n % 2 == 0) a[n / 2].im = 0.0;
            offt_exec(p, a, b, +1);
            for (j = 0; j < n; j++) rr[j] = b[j].re;
        }
        free(a);
    }
    offt_plan_destroy(p);
}
