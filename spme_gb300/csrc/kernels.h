// Host-side launchers for the GB300 SPME-RPY kernels (sm_103a).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include <vector>

#include "common.cuh"

namespace spme {

// ---- P-build and counting sorts (pbuild.cu) -------------------------------
// Sort keys with a slot within each key (atomic counts): the mesh tile of the
// stencil start (key1), the stencil-start cell ((sy K + sx) K + sz, K^3 keys;
// key2), the real-space cell (nc^3 cells of edge L/nc; key3), in one pass over
// the positions.  A null count skips that key.  With a mesh key, pstart (n)
// and pfrac (3n values of the engine's type: float when fp32) receive each
// particle's packed stencil start and fractional mesh coordinates; with the
// cell key, prel (n float4 / double4_32a) its position relative to its cell.
void launch_all_keys(const double *pos, int n, const MeshGeom &g, int nc, int *key1, int *count1,
                     int *slot1, int *key2, int *count2, int *slot2, int *key3, int *count3,
                     int *slot3, uint32_t *pstart, void *pfrac, void *prel, bool fp32,
                     cudaStream_t s);
// cpos[s] = prel[perm[s]] (float4 or double4_32a): cell-relative positions in cell order.
void launch_cell_gather(const void *prel, const int *perm, int n, bool fp32, void *cpos,
                        cudaStream_t s);
// Real-space cell key (nc^3 cells of edge L/nc) and slot within its cell.
void launch_cell_keys(const double *pos, int n, double L, int nc, int *key, int *count,
                      int *slot, cudaStream_t s);
// Exclusive scan of count[0..nkeys) into off[0..nkeys] (off[nkeys] = total).
// tmp must hold scan_tmp_elems(nkeys) ints.
size_t scan_tmp_elems(int nkeys);
void launch_scan(const int *count, int nkeys, int *off, int *tmp, cudaStream_t s);
// Counting-sort scatter.  On entry perm[i] is particle i's slot within its key
// (from the atomic counts, in no fixed order); on return perm[off[k] ..
// off[k + 1]) lists key k's particles in increasing index.  tmp: n ints.
void launch_scatter(const int *key, const int *off, int n, int *perm, int *tmp,
                    cudaStream_t s);
// B-spline records in sorted order (perm): rec_idx[s] = perm[s], the packed
// stencil start, and p weights per axis (record width RecordWidth<T,P>), from
// launch_all_keys' per-particle starts and fractional coordinates.
template <typename T>
void launch_records(const uint32_t *pstart, const T *pfrac, const int *perm, int n, int p,
                    int *rec_idx, uint32_t *rec_start, T *rec_w, cudaStream_t s);
// Cell-sorted positions relative to their cell's lower corner (float4 or double4_32a).
void launch_cell_positions(const double *pos, const int *perm, int n, double L, int nc,
                           bool fp32, void *cpos, cudaStream_t s);

// ---- spread / interpolate (spread.cu, interp.cu) --------------------------
template <typename T>
cudaError_t launch_spread(const int *tile_off, const int *rec_idx, const uint32_t *rec_start,
                          const T *rec_w, const T *F, int C, const MeshGeom &g, T *mesh,
                          cudaStream_t s);
// Column-gather spread (spread_cols.cu): records sorted by stencil-start cell,
// start_off[(sy K + sx) K + sz] the offsets of that order (K^3 + 1 entries),
// Fs the force rows in the same order.  Usable when spread_cols_ok(K, C, elem, p).
bool spread_cols_ok(int K, int C, size_t elem, int p);
// Row width (elements) of the force rows the column-gather spread reads: each
// lane's components contiguous and padded (C <= 16: C, unpadded).
int spread_cols_row_width(int C);
// Fs[s] = the row of F[idx[s]] (C components) in that padded layout.
template <typename T>
void launch_gather_cols_rows(const T *F, const int *idx, int n, int C, T *Fs, cudaStream_t s);
// Arguments of one system's column-gather spread: start-cell offsets of this
// system (indexed by its own (sy K + sx) K + sz), records and force rows
// indexed by sorted slot, ws the record stride (elements).
template <typename T>
struct SpreadColsArgs {
    const int *soff;
    const uint32_t *rec_start;
    const T *rec_w;
    const T *Fs;
    T *mesh;
    int C, RW, K, nzt, ws;
};
// A system of a batched launch: its arguments, order and blocks along x.
template <typename T>
struct SpreadColsSys {
    SpreadColsArgs<T> args;
    int p, gx;
};
// Blocks of one system's column-gather spread (all component chunks).
int spread_cols_blocks(int K, int C, size_t elem);
// All systems (same C) in one persistent launch; prefix[k] = the first block
// of system k (nsys + 1 entries, prefix[nsys] = total), both on the device.
template <typename T>
cudaError_t launch_spread_cols_batch(const SpreadColsSys<T> *sys, const int *prefix, int nsys,
                                     int total, int C, cudaStream_t s);
template <typename T>
cudaError_t launch_spread_cols(const int *start_off, const uint32_t *rec_start, const T *rec_w,
                               const T *Fs, int C, const MeshGeom &g, T *mesh, cudaStream_t s);
// TMA descriptor of the real mesh [C][K][K][K] for the interpolation halo
// boxes (4 components per box: more blocks per SM than 8, measured faster).
struct InterpMaps {
    CUtensorMap cg4;
    bool ok4 = false;
};
bool make_interp_maps(InterpMaps *maps, const void *mesh, int C, const MeshGeom &g, size_t elem);
// Shared memory the interpolation kernel needs (4-component boxes).
size_t interp_smem_bytes(const MeshGeom &g, size_t elem);
// Arguments of one system's interpolation (records indexed by sorted slot,
// stride ws; tile_off indexed by this system's tiles; W rows by particle).
template <typename T>
struct InterpArgs {
    const int *tile_off;
    const int *rec_idx;
    const uint32_t *rec_start;
    const T *rec_w;
    const T *mesh;
    T *W;
    int *err;
    MeshGeom g;
    int C, cb, ce, accumulate, use_tma, ws;
};
// One system of a batched interpolation: its arguments and, when args.use_tma
// is set, its 4-component TMA box over its own mesh (make_interp_box; read by
// the kernel from this global work list, 64-byte aligned).
template <typename T>
struct InterpSys {
    CUtensorMap tmap;
    InterpArgs<T> args;
};
// The 4-component TMA box of one mesh (false where TMA does not apply: K * elem
// not a multiple of 16 bytes, an unaligned mesh, or no driver entry point).
bool make_interp_box(CUtensorMap *map, const void *mesh, int C, const MeshGeom &g, size_t elem);
// All systems in one persistent launch over their tiles (prefix as for the
// spread; smem = the largest interp_smem_bytes of the systems; the kernel's
// dynamic shared-memory limit is set to max(smem, smem_limit)).
template <typename T>
cudaError_t launch_interp_batch(const InterpSys<T> *sys, const int *prefix, int nsys, int total,
                                size_t smem, cudaStream_t s, size_t smem_limit = 0);
// Components [cb, ce) of the C-component mesh (cb a multiple of 4) into
// W[n][C]; err: device flag set to 1 if a TMA wait timed out.
template <typename T>
cudaError_t launch_interp(const InterpMaps &maps, const int *tile_off, int n, const int *rec_idx,
                          const uint32_t *rec_start, const T *rec_w, const T *mesh, int C,
                          int cb, int ce, const MeshGeom &g, T *W, int accumulate, int *err,
                          cudaStream_t s);

// ---- host tables (engine.cu) ----------------------------------------------
// |b(m)|^2 = 1 / |sum_{j<p-1} M_p(j+1) e^{i j 2 pi m'/K}|^2 (old-version/spme.c:109-126).
void host_moduli2(int K, int p, std::vector<double> &out);

// ---- k-space influence (influence.cu) -------------------------------------
// tab[(z*K + y)*Kh + kx] = (S(k)|b|^2 / V, S(k)|b|^2 / (V k^2)), zero at k = 0.
template <typename T>
void launch_influence_table(T *tab2, const double *bmod2, int K, double L, double xi,
                            double a, cudaStream_t s);
// In-place influence on the component-major half spectrum G[c][(z*K+y)*Kh+kx].
template <typename T>
void launch_influence(T *G, const T *tab2, int K, double L, int R, cudaStream_t s);

// ---- fused z-FFT + influence + inverse z-FFT (zfft.cu) --------------------
struct ZPlan {
    int K;
    int nst;              // radix stages
    int rad[12];          // radices, first stage of the inverse (DIT) first
    int len_before_last;  // product of the first nst-1 radices
    int npass;            // passes of one or two stages
    int pcode[12];        // 10 * R1 + R2 (R2 = 1: single stage)
    int pspan[12];        // span of the pass's first (R1) stage in DIT order
};
// Radix plan, twiddles e^{-2 pi i e/K} (re, im pairs) and the digit-reversal
// permutation (position p holds frequency perm[p]) for length-K transforms.
bool make_zplan(int K, size_t elem, ZPlan *zp, std::vector<double> *tw, std::vector<int> *perm);
// Columns per block for K (0 if K does not fit the fused kernel).
int zfft_width(int K, size_t elem);
// One-pass 2D (y, x) transforms of the mesh's z-planes (FP32; K = 128, 160,
// 256): real planes [planes][K][K] <-> half spectra [planes][K][K/2+1], cuFFT's
// layouts and unnormalised conventions.  tables: make_fft2d_tables' bytes on
// the device.
bool fft2d_ok(int K, size_t elem);
size_t fft2d_table_bytes(int K);
bool make_fft2d_tables(int K, std::vector<unsigned char> *out);
cudaError_t launch_fft2d_r2c(int K, const float *mesh, float *G, long planes, const void *tables,
                             cudaStream_t s);
cudaError_t launch_fft2d_c2r(int K, const float *G, float *mesh, long planes, const void *tables,
                             cudaStream_t s);
// TMA descriptor over the half spectrum G[C][K][K][K/2+1] (complex of elem-byte
// reals), z-planes viewed as flat rows.
bool make_zfft_map(CUtensorMap *map, void *G, int K, int C, size_t elem);
// On the half spectrum after 2D (y, x) R2C transforms: FFT along z,
// influence (table as launch_influence), inverse FFT along z, Hermitian part of
// the kx = 0 and K/2 planes.  tw: K complex twiddles of type T; perm: K ints.
template <typename T>
cudaError_t launch_zfft_influence(const CUtensorMap &map, T *G, const T *tab2, const T *tw,
                                  const int *perm, const ZPlan &zp, double L, int R, int *err,
                                  cudaStream_t s);

// ---- real-space pair sum + self term (realspace.cu) -----------------------
// cpos: float4 for T = float, double4_32a for T = double (cell-relative).
template <typename T>
cudaError_t launch_realspace(int nc, const int *cell_off, const int *cell_perm, const void *cpos,
                             const T *F, int R, double L, double rc, double xi, double a,
                             int with_self, T *W, cudaStream_t s);
// Piecewise Chebyshev table of the real-space pair functions F(r), G(r) for FP64
// engines (xi and a fixed per engine): degree kPairDeg on nseg1 segments of
// [r_lo, r_mid) and nseg2 of [r_mid, r_hi]; coef (device) holds the F and G
// coefficients interleaved per segment.  A null coef means no table.
constexpr int kPairDeg = 10;
struct PairTable {
    const double *coef = nullptr;
    double r_lo = 0, r_mid = 0, r_hi = 0, inv_h1 = 0, inv_h2 = 0;
    int nseg1 = 0, nseg2 = 0;
};
// Fits the table on the host (checked between nodes to 2e-13 relative);
// false if no fit meets that within 4096 segments.
bool build_pair_table(double xi, double a, double rc, std::vector<double> *coef, PairTable *t);
template <typename T>
cudaError_t launch_realspace(int nc, const int *cell_off, const int *cell_perm, const void *cpos,
                             const T *F, int R, double L, double rc, double xi, double a,
                             int with_self, const PairTable &tab, T *W, cudaStream_t s);
// FP32 pair-function coefficients of one (xi, a) and the FP32 copies of the
// geometry (real_args fills them): far field (r >= 2a), with ir = 1/r,
//   F = erfc(xi r) (0.75 ir + c1 ir^3) + e^{-xi^2 r^2} (A4 r^4 + A2 r^2 + A0 + Am2 ir^2)
//   G = erfc(xi r) (0.75 ir + c3 ir^3) + e^{-xi^2 r^2} (-A4 r^4 + B2 r^2 + B0 + Bm2 ir^2)
// near field: xi, xi3a2 = xi^3 a^2, ia = 1/a, n1 = 9/(32 a^2), n2 = 3/(32 a^2).
struct RealCoef {
    float xi, xi2, a2x4, xi3a2, ia, n1, n2;
    float A4, A2, A0, Am2, B2, B0, Bm2, c1, c3;
    float L, h, rc2, self_c;
};
// Arguments of one system's real-space sum (cell_off indexed by this system's
// cells; slots, positions and rows global).
template <typename T>
struct RealArgs {
    const int *cell_off;
    const int *cell_perm;
    const void *cpos;
    const T *F;
    T *W;
    int nc, R, with_self;
    double L, h, rc2, xi, a, self_c;
    PairTable tab;
    RealCoef cf;
};
double real_self_coeff(double xi, double a);
template <typename T>
RealArgs<T> real_args(int nc, const int *cell_off, const int *cell_perm, const void *cpos,
                      const T *F, int R, double L, double rc, double xi, double a, int with_self,
                      const PairTable &tab, T *W);
// All systems in one persistent launch over their cells (prefix as for the spread).
template <typename T>
cudaError_t launch_realspace_batch(const RealArgs<T> *sys, const int *prefix, int nsys,
                                   int total, cudaStream_t s);

// ---- layout conversions (pack.cu) -----------------------------------------
// W = self_c * F (the self term alone, when no real-space sum is requested)
template <typename T>
void launch_self(const T *F, int n, int R, double self_c, T *W, cudaStream_t s);
// F[i][3R] = f[r*ld + 3i + d]
// Fs[s][c] = F[idx[s]][c] for s < n (C components per row).
template <typename T>
void launch_gather_rows(const T *F, const int *idx, int n, int C, T *Fs, cudaStream_t s);
template <typename T>
void launch_pack(const T *f, long ld, int n, int R, T *F, cudaStream_t s);
// u[r*ld + 3i + d] = beta*u + alpha*W[i][3r+d]   (u not read when beta == 0)
// Tiled (shared-memory) forms of launch_pack / launch_unpack(_sum): coalesced on
// both sides; W2 may be null (plain unpack).  Up to 48 KB of shared memory.
template <typename T>
void launch_pack_tiled(const T *f, long ld, int n, int R, T *F, cudaStream_t s);
// (right-hand sides [r0, r1) of f into their columns of F[n][3R])
template <typename T>
void launch_pack_tiled(const T *f, long ld, int n, int R, int r0, int r1, T *F, cudaStream_t s);
// (launch_unpack_tiled: right-hand sides [r0, r1) of the R in W / W2.)
template <typename T>
void launch_unpack_tiled(const T *W, const T *W2, int n, int R, int r0, int r1, double alpha,
                         double beta, T *u, long ld, cudaStream_t s);
template <typename T>
void launch_unpack(const T *W, int n, int R, double alpha, double beta, T *u, long ld,
                   cudaStream_t s);

}  // namespace spme
