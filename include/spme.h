/*
 * spme.h — drop-in C ABI of the GB300 SPME-RPY mobility operator.
 *
 * Same entry points, argument order and meaning as billy-inn/SPME
 * old-version/spme.h:85-97, so a caller of the reference's CPU engine links
 * against libspme_gb300.so instead of spme.o/spme_kernel.o.  Differences a
 * caller can see:
 *   - spme_t is opaque (the reference exposes its struct, old-version/spme.h:42-82;
 *     callers only ever hold the pointer, old-version/main.c:136,215).
 *   - failures do not assert: the void entry points record a status that
 *     spme_last_error() returns (0 = success); create_spme_engine sets
 *     *_spme = NULL when it fails.
 *   - the work runs on one GPU; nthreads is accepted and ignored.
 * Like the reference, compute_spme applies only the reciprocal-space part of
 * the Ewald-split RPY mobility with particle radius 1 (old-version/spme.c:141).
 * The full operator (real space + self + reciprocal, any radius, FP32
 * batching) is in spme_gb300.h.
 */
#ifndef SPME_GB300_SPME_H
#define SPME_GB300_SPME_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct _spme_t spme_t;

/* Replaces old-version/spme.h:85-86 (declared there, never defined).
 * Returns the Ewald parameter xi for which the real-space truncation error
 * exp(-xi^2 rmax^2) equals ewald_eps (0 < ewald_eps < 1); box_size is unused
 * by this estimate and kept for the signature. */
void cutoff2xi(double rmax, double ewald_eps, double box_size, double *_xi);

/* Replaces old-version/spme.h:89-91 (old-version/spme.c:327-523).
 * dim = mesh size K (2..1024, any factorisation), porder = B-spline order p
 * (4, 6 or 8), np = number of particles, box_size = L. */
void create_spme_engine(double xi, int dim, int porder, int np, double box_size,
                        int nthreads, spme_t **_spme);

/* Replaces old-version/spme.h:93 (old-version/spme.c:526-557). Frees everything. */
void destroy_spme_engine(spme_t *spme);

/* Replaces old-version/spme.h:95-97 (old-version/spme.c:560-726).
 * Host pointers.  pos: np x 3 doubles in [0, L) (pos == NULL reuses the
 * previous positions).  For each of nrhs right-hand sides r:
 *   vec_out[r*ldout + 3i + d] = beta * vec_out[...] + alpha * (M_recip f_r)[3i + d]
 * with f_r[3i + d] = vec_in[r*ldin + 3i + d].  FP64 throughout. */
void compute_spme(spme_t *spme, double *pos, int nrhs, double alpha, double *vec_in,
                  int ldin, double beta, double *vec_out, int ldout);

/* Status of the last call on this engine (0 = success); see spme_gb300.h for codes. */
int spme_last_error(const spme_t *spme);
/* Human-readable text for a status code. */
const char *spme_error_string(int code);

/* Padding helpers callers of the reference use for leading dimensions
 * (old-version/spme.h:100-101, old-version/main.c:203). */
#define PAD_LEN(N, size) ((((N) + (64 / (size)) - 1) / (64 / (size))) * (64 / (size)))
#define PAD_FFT_LEN(N, size) (((((N) + (64 / (size)) - 1) / (64 / (size))) | 1) * (64 / (size)))

#ifdef __cplusplus
}
#endif

#endif /* SPME_GB300_SPME_H */
