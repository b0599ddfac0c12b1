/*
 * TEST INFRASTRUCTURE ONLY — the oracle.  A plain-C FP64 restatement of the
 * reference's SPME-RPY mobility apply (billy-inn/SPME, old-version/spme.c and
 * old-version/spme_kernel.c) plus the terms the reference lacks (real-space
 * Ewald sum, self term) restated from Beenakker, J. Chem. Phys. 85, 1581
 * (1986).  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
 * leg may load it, and only as the checker.  The product never links it.
 *
 * Units follow the reference's scalar_recip (old-version/spme.c:43-60): the
 * operator is the RPY mobility times 6*pi*eta, so an isolated sphere of
 * radius a has self-mobility 1/a (exactly 1 for the reference's a = 1).
 *
 * Vector layout follows compute_spme (old-version/spme.h:95-97): right-hand
 * side r of nrhs lives at vec[r*ld + 3*i + d].
 */
#ifndef SPME_ORACLE_H
#define SPME_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

/* Cardinal B-spline weights for fractional coordinate w in [0,1):
 * out[j] = M_p(w + p - 1 - j), j = 0..p-1 (weight of mesh point start + j). */
void oracle_bspline_weights(int p, double w, double *out);

/* |b(m)|^2 of the Euler exponential spline moduli, m = 0..K-1
 * (old-version/spme.c:109-126). */
void oracle_bspline_moduli2(int K, int p, double *bmod2);

/* Reference scalar_recip generalised to radius a (old-version/spme.c:43-60). */
double oracle_scalar_recip(double k, double xi, double a);

/* Reciprocal part, reference semantics (old-version/spme.c:560-726):
 * u_r = beta*u_r + alpha * M_recip f_r for each of nrhs right-hand sides.
 * Any K >= 2, even p in [2, 16]; nthreads <= 0 means all. */
int oracle_recip(int np, const double *pos, double L, double xi, double a, int K, int p,
                 int nrhs, double alpha, const double *f, long ldf, double beta,
                 double *u, long ldu, int nthreads);

/* Real-space Ewald sum over pairs with r < rc plus the self term
 * (flags bit 0: real space, bit 1: self):
 * u_r = beta*u_r + alpha * (M_real + M_self) f_r. Requires rc < L/2. */
int oracle_real_self(int np, const double *pos, double L, double xi, double a, double rc,
                     int nrhs, double alpha, const double *f, long ldf, double beta,
                     double *u, long ldu, int flags, int nthreads);

/* Mesh-free Ewald reciprocal sum over all k != 0 with |k| <= kcut:
 * u_r = beta*u_r + alpha * M_recip_exact f_r.  O(N * #k); small cases only. */
int oracle_recip_direct(int np, const double *pos, double L, double xi, double a,
                        double kcut, int nrhs, double alpha, const double *f, long ldf,
                        double beta, double *u, long ldu, int nthreads);

/* Beenakker real-space scalars: M_real(r) = F(r) I + G(r) rhat rhat (units above),
 * including the overlap correction for r < 2a. */
void oracle_real_FG(double r, double xi, double a, double *F, double *G);
double oracle_self_coeff(double xi, double a);

#ifdef __cplusplus
}
#endif
#endif
