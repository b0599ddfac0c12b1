/*
 * spme_gb300.h — extended C ABI of the GB300 SPME-RPY mobility operator.
 *
 * The reference (billy-inn/SPME) has only the spme.h entry points
 * (old-version/spme.h:85-97) and computes only the reciprocal-space part with
 * radius 1.  These entry points add what the reference's callers (block
 * Krylov / Lanczos Brownian-dynamics samplers) need around that apply:
 *   - the full Ewald-split RPY mobility  M = M_recip + M_real + M_self
 *     for any radius a and real-space cutoff rc (Beenakker 1986 splitting);
 *   - FP32 batching of R right-hand sides through one mesh pass (3R
 *     components), with FP64 kept for fractional coordinates, the moduli and
 *     influence tables, and the real-space / self accumulation;
 *   - host or device-resident vectors, and a caller-chosen CUDA stream;
 *   - integer status codes instead of the reference's asserts.
 *
 * Units follow the reference's scalar_recip (old-version/spme.c:43-60): the
 * mobility times 6*pi*eta, so an isolated sphere of radius a has
 * self-mobility 1/a.
 *
 * Vector layout everywhere is compute_spme's (old-version/spme.h:95-97):
 * right-hand side r of particle i, Cartesian d, at v[r*ld + 3*i + d].
 * Element type is double for SPME_FP64 engines and float for SPME_FP32.
 *
 * An engine is bound to the device that was current at spme_create.  It is
 * not thread-safe; separate engines may be used from separate threads.
 */
#ifndef SPME_GB300_EXT_H
#define SPME_GB300_EXT_H

#include "spme.h"

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
enum {
    SPME_OK = 0,
    SPME_ERR_INVALID = 1,     /* bad argument */
    SPME_ERR_UNSUPPORTED = 2, /* valid but outside what this build supports */
    SPME_ERR_CUDA = 3,        /* CUDA runtime error */
    SPME_ERR_CUFFT = 4,       /* cuFFT error */
    SPME_ERR_NOMEM = 5,       /* device or host allocation failed */
    SPME_ERR_STATE = 6,       /* e.g. apply before any positions were given */
    SPME_ERR_KERNEL = 7,      /* a device-side check failed (status read back) */
    SPME_ERR_TOO_LARGE = 8    /* exceeds the fixed scratch of spme_realspace_apply_noalloc */
};

enum { SPME_FP64 = 0, SPME_FP32 = 1 };

enum {
    SPME_TERM_RECIP = 1,
    SPME_TERM_REAL = 2,
    SPME_TERM_SELF = 4,
    SPME_TERM_ALL = 7
};

enum { SPME_MEM_HOST = 0, SPME_MEM_DEVICE = 1 };

typedef struct spme_params {
    int np;           /* particles, >= 0 */
    int dim;          /* mesh size K per axis, 2..1024 */
    int porder;       /* B-spline order p: 4, 6 or 8 */
    double box_size;  /* cubic periodic box edge L > 0 */
    double xi;        /* Ewald splitting parameter > 0 */
    double radius;    /* particle radius a > 0 (the reference fixes 1) */
    double rcut;      /* real-space cutoff, 0 < rc < L/2 (needed if SPME_TERM_REAL) */
    int precision;    /* SPME_FP64 or SPME_FP32 */
    int max_nrhs;     /* right-hand sides carried per mesh pass, >= 1 */
    int terms;        /* OR of SPME_TERM_* */
} spme_params;

/* Fill *p with defaults: radius 1, precision FP64, max_nrhs 1, terms RECIP
 * (the reference's operator); np/dim/porder/box_size/xi/rcut zero. */
void spme_params_init(spme_params *p);

/* Create an engine (allocates device memory, cuFFT plans, tables). */
int spme_create(const spme_params *params, spme_t **out);

/* Destroy an engine; NULL is a no-op. */
int spme_destroy(spme_t *spme);

/* Run subsequent work on `stream` (a cudaStream_t; NULL is the legacy default
 * stream).  An engine starts on a non-blocking stream of its own, which
 * spme_get_stream returns before any spme_set_stream call. */
int spme_set_stream(spme_t *spme, void *stream);
void *spme_get_stream(const spme_t *spme);

/* Load positions (np x 3 doubles; host or device per `mem`) and build the
 * B-spline records, the mesh-tile sort and the real-space cell list.
 * Positions outside [0, L) are wrapped. */
int spme_set_positions(spme_t *spme, const double *pos, int mem);

/* u_r = beta*u_r + alpha * M f_r for r < nrhs (any nrhs >= 0; passes of at
 * most max_nrhs).  f and u are host or device pointers per `mem`, element
 * type per the engine's precision, layout v[r*ld + 3*i + d], ld >= 3*np.
 * Host calls return after the result is in u; device calls are
 * stream-ordered on the engine's stream. */
int spme_apply(spme_t *spme, int nrhs, double alpha, const void *f, long ldf, double beta,
               void *u, long ldu, int mem);

/* Block until the engine's stream is idle. */
int spme_synchronize(spme_t *spme);

/* Per-stage device times (ms) of the last apply when profiling is on.
 * spme_set_profiling(spme, 1): CUDA events around each stage (with
 * spme_set_overlap on, the real-space sum still overlaps the mesh stages on its
 * own stream); level 2 always runs the real-space sum on the main stream so
 * each stage is timed alone; 0 off.
 * Stages, in order: pack, real-space, spread, forward FFT, influence,
 * backward FFT, interpolate, unpack.  Returns the number of stages written
 * (<= n). */
int spme_set_profiling(spme_t *spme, int on);
int spme_stage_times(const spme_t *spme, float *ms, int n);

/* Number of this library's kernels the engine has launched since creation
 * (cuFFT's own kernels are not included). */
long spme_launch_count(const spme_t *spme);

/* Real-space sum concurrent with the mesh pipeline (on = 1: on a second
 * stream, joined before the interpolation adds onto it) or before it on the
 * same stream (0, the default: on a full GPU the mesh kernels occupy every SM
 * and the concurrent sum only slows them down). */
int spme_set_overlap(spme_t *spme, int on);

/* Spread kernel.  1 (default): column gather where it applies (K >= 32; in
 * FP32 from 9 components on, below that the tile kernel is faster), each mesh
 * column visits only the particles whose stencil covers it, force components
 * across the lanes of a warp.  0: tile kernel always, threads own the columns
 * of a mesh tile and visit every particle staged for the tile.  Mode 1 on an
 * engine without the column-gather buffers returns SPME_ERR_UNSUPPORTED. */
int spme_set_spread_mode(spme_t *spme, int mode);

/* Transform strategy of the mesh pass.  1: cuFFT 2D (y, x) transforms of
 * every z-plane, then one fused kernel doing the z transform, the influence
 * and the inverse z transform in shared memory (one pass over the half
 * spectrum instead of three).  2: as 1 with this library's one-pass 2D
 * transforms (FP32, K = 128, 160, 256; thread-block clusters exchange the
 * row blocks of a plane).  0: cuFFT 3D transforms and a separate influence
 * kernel.  Default: 1 in FP32 when K fits the fused kernel, else 0.  Modes 1
 * and 2 on an engine they do not fit return SPME_ERR_UNSUPPORTED. */
int spme_set_fft_mode(spme_t *spme, int mode);

/* Capture each mesh pass (and each device-pointer position build) into a CUDA
 * graph the first time it is seen and replay it afterwards (on = 1).  A pass
 * is keyed by nrhs, the f/u pointers and leading dimensions, alpha, beta, the
 * profiling level and the stream; host-pointer calls capture only their
 * device work (the copies to and from the caller's memory stay outside).
 * Turning graphs on or off, or changing the tile, drops all graphs. */
int spme_set_graphs(spme_t *spme, int on);

/* Mesh-tile shape used by spread/interpolate (default 8 x 8 x 8; tx, ty in
 * 4..16, tz in 4..8).  Takes effect at the next spme_set_positions, which must
 * follow before the next apply. */
int spme_set_tile(spme_t *spme, int tx, int ty, int tz);

/* Ewald parameters for a target relative error `tol` (host only; the reference
 * declares cutoff2xi for parameter selection, old-version/spme.h:85-86, but
 * never defines it).  Error models fitted to the oracle: real space
 * exp(-x^2)(1 + x^4/3) = tol with x = xi rc; k-space tail exp(-y)(1 + y + 2y^2)
 * = tol with y = (pi K/L)^2/(4 xi^2); B-spline interpolation xi L/K <=
 * c_p tol^(1/p); p = 4 / 6 / 8 for tol >= 1e-3 / >= 1e-6 / below; K the next
 * 2^a 3^b 5^c.  rcut <= 0 picks rc = min(10 a, 0.49 L).  Fills *out, all terms. */
int spme_suggest_params(int np, double box_size, double radius, double tol, double rcut,
                        spme_params *out);
/* Smallest n' >= max(n, 2) whose prime factors are 2, 3 and 5. */
int spme_next_smooth(int n);

/* Particle files in the reference driver's .xyz format (old-version/main.c:46-127):
 * '#' comment lines, a header line "np L", then "name x y z a" per particle.
 * spme_read_xyz wraps positions into [0, L) like the driver does and returns
 * malloc'd arrays (release with spme_free); radii may be NULL. */
int spme_read_xyz(const char *path, int *np, double *box_size, double **pos, double **radii);
int spme_write_xyz(const char *path, int np, double box_size, const double *pos, double radius);
void spme_free(void *p);

/* Measured FMA throughput of the current device in FLOP/s (2 per FMA) for
 * SPME_FP32 or SPME_FP64: independent FMA chains on every SM, timed with CUDA
 * events.  The roofline denominator for the real-space sum's arithmetic.  No
 * counterpart in the reference. */
int spme_fma_peak(int precision, double *flops_per_s);

/* ---- batches of independent systems --------------------------------------
 * No counterpart in the reference (its compute_spme, old-version/spme.c:560-726,
 * applies one system).  A batch holds systems of different size N_k, box L_k,
 * mesh K_k and order p_k with the same number of right-hand sides R and
 * precision, and applies the full operator M_k = M_recip + M_real + M_self to
 * each of them; every stage (position build, spread, influence,
 * interpolation, real-space sum, layout conversions) is one launch over a
 * packed work list of all systems, and cuFFT runs one batched plan per
 * distinct K.  Device pointers only; work ordered on the batch's stream.
 *
 * Packed layouts (systems in the order given, P_k = N_0 + ... + N_{k-1}):
 *   positions: system k's N_k x 3 doubles at element 3 P_k;
 *   vectors:   system k's R right-hand sides at element 3 R P_k, right-hand
 *              side r of particle i, Cartesian d at 3 R P_k + r 3 N_k + 3 i + d
 *              (compute_spme's layout with ld = 3 N_k, per system).
 * Each system needs K >= p + 15 (FP32) or K >= p + 7 (FP64), rc < L/2. */
typedef struct spme_batch_system {
    int np;
    int dim;
    int porder;
    double box_size;
    double xi;
    double radius;
    double rcut;
} spme_batch_system;

typedef struct _spme_batch_t spme_batch_t;

int spme_batch_create(const spme_batch_system *systems, int count, int nrhs, int precision,
                      spme_batch_t **out);
int spme_batch_destroy(spme_batch_t *batch);
/* A batch starts on a non-blocking stream of its own (spme_batch_get_stream);
 * NULL selects the legacy default stream, as for spme_set_stream. */
int spme_batch_set_stream(spme_batch_t *batch, void *stream);
void *spme_batch_get_stream(const spme_batch_t *batch);
/* Interpolation tile of every system (as spme_set_tile, default 16 x 8 x 4);
 * positions must be set again. */
int spme_batch_set_tile(spme_batch_t *batch, int tx, int ty, int tz);
int spme_batch_set_positions(spme_batch_t *batch, const double *pos);
/* u = beta u + alpha M f for every system (packed layouts above). */
int spme_batch_apply(spme_batch_t *batch, double alpha, const void *f, double beta, void *u);
/* set_positions + apply; with graphs on, captured once per (pointers, alpha,
 * beta, stream) and replayed as one CUDA graph launch. */
int spme_batch_step(spme_batch_t *batch, const double *pos, double alpha, const void *f,
                    double beta, void *u);
int spme_batch_set_graphs(spme_batch_t *batch, int on);
/* Concurrency inside a step (OR of): 1 the real-space sum on a second stream
 * beside the mesh pipeline, 2 the cuFFT groups on four streams.  Default 0. */
int spme_batch_set_overlap(spme_batch_t *batch, int mode);
int spme_batch_synchronize(spme_batch_t *batch);
long spme_batch_launch_count(const spme_batch_t *batch);
long spme_batch_particles(const spme_batch_t *batch);
/* Per-stage device times (ms) of the last uncaptured step with profiling on:
 * position build, pack, real-space, spread, forward FFT, influence, backward
 * FFT, interpolate, unpack.  Returns the number written (<= n). */
int spme_batch_set_profiling(spme_batch_t *batch, int on);
int spme_batch_stage_times(const spme_batch_t *batch, float *ms, int n);

/* Real-space + self mobility apply that allocates no device memory.
 * No counterpart in the reference (which has no real-space term).  For callers
 * that cannot call cudaMalloc: applications that reserve all device memory in
 * their own pool at start-up, and time-stepping loops that must not stall
 * (cudaMalloc/cudaFree can synchronise the device).  FP64, device pointers,
 * work ordered on `stream` (NULL: the legacy default stream):
 *   u_r = beta*u_r + alpha * (M_real + M_self) f_r,  layout v[r*ld + 3i + d],
 * with the same Beenakker real-space sum and self term as spme_apply.
 * Scratch is one fixed device array inside the library (about 16 MB), so the
 * sizes are capped: np <= SPME_NOALLOC_MAX_NP, nrhs <= SPME_NOALLOC_MAX_NRHS;
 * larger requests return SPME_ERR_TOO_LARGE.  The array takes device memory on
 * a device when the first call there loads the library's code (CUDA loads it
 * lazily) and keeps it until the process exits: make one call, a zero-size one
 * (np = 0) is enough, on each device before reserving the rest of its memory
 * and before any stream capture.  Resetting the device after that call is not
 * supported.  All calls share the array: calls that overlap on the GPU race and
 * must be serialised by the caller.  A pending error of the caller's earlier
 * launches is cleared on entry; the status describes this call only. */
#define SPME_NOALLOC_MAX_NP 65536
#define SPME_NOALLOC_MAX_NRHS 4
int spme_realspace_apply_noalloc(int np, const double *pos, double box_size, double xi,
                                 double radius, double rcut, int nrhs, double alpha,
                                 const double *f, long ldf, double beta, double *u, long ldu,
                                 void *stream);

#ifdef __cplusplus
}
#endif

#endif /* SPME_GB300_EXT_H */
