/*
 * Test infrastructure only: the DFTI subset declared in shim/mkl.h, for the
 * in-place 3D real transforms the reference configures at
 * old-version/spme.c:370-412 (cubic n^3, padded strides, CCE storage
 * "COMPLEX_COMPLEX", backward scale 1/n^3).  Backed by oracle/fft.c.
 */
#include "mkl.h"
#include "../fft.h"
#include <stdarg.h>
#include <string.h>

struct oracle_dfti_desc {
    long n[3];
    long in_str[4];
    long out_str[4];
    double bscale;
};

MKL_LONG DftiCreateDescriptor(DFTI_DESCRIPTOR_HANDLE *h, int precision, int domain,
                              MKL_LONG dimension, ...)
{
    struct oracle_dfti_desc *d;
    va_list ap;
    if (precision != DFTI_DOUBLE || domain != DFTI_REAL || dimension != 3) return 1;
    d = (struct oracle_dfti_desc *)calloc(1, sizeof(*d));
    if (!d) return 1;
    va_start(ap, dimension);
    {
        MKL_LONG *sz = va_arg(ap, MKL_LONG *);
        d->n[0] = sz[0]; d->n[1] = sz[1]; d->n[2] = sz[2];
    }
    va_end(ap);
    if (d->n[0] != d->n[1] || d->n[1] != d->n[2]) { free(d); return 1; }
    d->bscale = 1.0;
    *h = d;
    return 0;
}

MKL_LONG DftiSetValue(DFTI_DESCRIPTOR_HANDLE h, int param, ...)
{
    va_list ap;
    MKL_LONG ret = 0;
    va_start(ap, param);
    if (param == DFTI_INPUT_STRIDES || param == DFTI_OUTPUT_STRIDES) {
        MKL_LONG *s = va_arg(ap, MKL_LONG *);
        long *dst = param == DFTI_INPUT_STRIDES ? h->in_str : h->out_str;
        int i;
        for (i = 0; i < 4; i++) dst[i] = s[i];
    } else if (param == DFTI_CONJUGATE_EVEN_STORAGE) {
        int v = va_arg(ap, int);
        if (v != DFTI_COMPLEX_COMPLEX) ret = 1;
    } else if (param == DFTI_BACKWARD_SCALE) {
        h->bscale = va_arg(ap, double);
    } else {
        ret = 1;
    }
    va_end(ap);
    return ret;
}

MKL_LONG DftiCommitDescriptor(DFTI_DESCRIPTOR_HANDLE h) { return h ? 0 : 1; }

MKL_LONG DftiComputeForward(DFTI_DESCRIPTOR_HANDLE h, void *inout)
{
    /* input strides are real (doubles), output strides complex elements */
    offt_r2c_3d((int)h->n[0], (const double *)inout, h->in_str[2], h->in_str[1],
                (offt_cpx *)inout, h->out_str[2], h->out_str[1], 0);
    return 0;
}

MKL_LONG DftiComputeBackward(DFTI_DESCRIPTOR_HANDLE h, void *inout)
{
    int n = (int)h->n[0];
    long z, y, x;
    double *r = (double *)inout;
    offt_c2r_3d(n, (offt_cpx *)inout, h->in_str[2], h->in_str[1],
                r, h->out_str[2], h->out_str[1], 0);
    if (h->bscale != 1.0) {
        #pragma omp parallel for private(y, x)
        for (z = 0; z < n; z++)
            for (y = 0; y < n; y++)
                for (x = 0; x < n; x++)
                    r[z * h->out_str[1] + y * h->out_str[2] + x] *= h->bscale;
    }
    return 0;
}

MKL_LONG DftiFreeDescriptor(DFTI_DESCRIPTOR_HANDLE *h)
{
    if (h && *h) { free(*h); *h = NULL; }
    return 0;
}
