/*
 * Test infrastructure only: a small mixed-radix complex FFT written for the
 * oracle.  It stands in for the FFT libraries the reference calls (Intel MKL
 * DFTI in old-version/spme.c:383-411,654-656,680-682; cuFFT D2Z/Z2D in
 * old-version/gpu_spme.cu:89-97,266-270,289-293), which are closed code and
 * absent here.  Nothing in the product links this file.
 *
 * Conventions: forward uses exp(-2 pi i j k / n), backward exp(+2 pi i j k / n);
 * neither direction scales.  The real 3D transforms follow the semantics of
 * numpy.fft.rfftn / irfftn: the inverse first runs the complex inverse along
 * z and y on the half spectrum, then a complex-to-real line transform along x
 * that uses only the real parts of the x = 0 and (even n) x = n/2 bins.
 */
#ifndef ORACLE_FFT_H
#define ORACLE_FFT_H
#ifdef __cplusplus
extern "C" {
#endif

typedef struct { double re, im; } offt_cpx;

typedef struct offt_plan offt_plan;

/* Plan for a length-n complex transform; n >= 1, any factorisation. */
offt_plan *offt_plan_create(int n);
void offt_plan_destroy(offt_plan *p);
/* out[k] = sum_j in[j] * exp(sign * 2 pi i j k / n); in and out must differ. */
void offt_exec(const offt_plan *p, const offt_cpx *in, offt_cpx *out, int sign);

/* Real 3D forward transform of an n^3 array.
 * real element (z,y,x) at r[z*rs2 + y*rs1 + x];
 * complex element (z,y,kx), kx <= n/2, at c[z*cs2 + y*cs1 + kx].
 * r and c may alias (in-place, as the reference's padded layout does). */
void offt_r2c_3d(int n, const double *r, long rs1, long rs2,
                 offt_cpx *c, long cs1, long cs2, int nthreads);
/* Inverse of the above without scaling (numpy irfftn semantics times n^3). */
void offt_c2r_3d(int n, const offt_cpx *c, long cs1, long cs2,
                 double *r, long rs1, long rs2, int nthreads);

#ifdef __cplusplus
}
#endif
#endif
