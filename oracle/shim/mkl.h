/*
 * Test infrastructure only.  A project-written stand-in for the small part of
 * Intel MKL that the reference's CPU path uses, so that old-version/spme.c and
 * old-version/spme_kernel.c compile unmodified with gcc:
 *   MKL_Complex16 (.real/.imag), MKL_LONG, _mm_malloc/_mm_free, and the DFTI
 *   subset called at old-version/spme.c:370-412,530-531,654-656,680-682.
 * The transforms run on the oracle's own FFT (oracle/fft.c); MKL itself is
 * closed code and is not used.
 */
#ifndef ORACLE_MKL_SHIM_H
#define ORACLE_MKL_SHIM_H
#include <stddef.h>
#include <stdlib.h>

typedef long MKL_LONG;
typedef struct { double real; double imag; } MKL_Complex16;

static inline void *_mm_malloc(size_t size, size_t align)
{
    void *p = NULL;
    if (align < sizeof(void *)) align = sizeof(void *);
    if (posix_memalign(&p, align, size ? size : 1) != 0) return NULL;
    return p;
}
static inline void _mm_free(void *p) { free(p); }

typedef struct oracle_dfti_desc *DFTI_DESCRIPTOR_HANDLE;

enum {
    DFTI_DOUBLE = 36,
    DFTI_REAL = 33,
    DFTI_INPUT_STRIDES = 12,
    DFTI_OUTPUT_STRIDES = 13,
    DFTI_CONJUGATE_EVEN_STORAGE = 10,
    DFTI_COMPLEX_COMPLEX = 39,
    DFTI_BACKWARD_SCALE = 5
};

MKL_LONG DftiCreateDescriptor(DFTI_DESCRIPTOR_HANDLE *h, int precision, int domain,
                              MKL_LONG dimension, ...);
MKL_LONG DftiSetValue(DFTI_DESCRIPTOR_HANDLE h, int param, ...);
MKL_LONG DftiCommitDescriptor(DFTI_DESCRIPTOR_HANDLE h);
MKL_LONG DftiComputeForward(DFTI_DESCRIPTOR_HANDLE h, void *inout);
MKL_LONG DftiComputeBackward(DFTI_DESCRIPTOR_HANDLE h, void *inout);
MKL_LONG DftiFreeDescriptor(DFTI_DESCRIPTOR_HANDLE *h);

#endif
