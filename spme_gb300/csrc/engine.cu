// Host engine and C ABI of the GB300 SPME-RPY mobility operator.
//
// Orchestrates, per mesh pass of R right-hand sides (C = 3R components, mesh
// stored component-major so cuFFT runs contiguous batched transforms):
//   pack -> [aux stream: real-space + self] -> spread -> cuFFT R2C ->
//   influence -> cuFFT C2R -> interpolate (+ real-space result) -> unpack
// The reference's compute_spme (old-version/spme.c:560-726) runs the whole
// pipeline once per right-hand side; here one pass carries up to max_nrhs.
#include <cuda_runtime.h>
#include <cufft.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include "kernels.h"
#include "spme_gb300.h"

using spme::MeshGeom;

namespace spme {

// Host B-spline values M_p(w + p - 1 - j) (same recursion as the kernels).
void host_bspline(int p, double w, double *out) {
    double a[spme::kMaxP + 1];
    a[0] = w;
    a[1] = 1.0 - w;
    for (int n = 3; n <= p; n++) {
        a[n - 1] = 0.0;
        for (int k = n - 1; k >= 1; k--)
            a[k] = ((w + k) * a[k] + ((double)n - w - k) * a[k - 1]) / (double)(n - 1);
        a[0] = w * a[0] / (double)(n - 1);
    }
    for (int k = 0; k < p; k++) out[k] = a[p - 1 - k];
}

// |b(m)|^2 = 1/|sum_{j<p-1} M_p(j+1) e^{i j phi}|^2, phi = 2 pi m'/K
// (old-version/spme.c:109-126; only the modulus enters the table).
void host_moduli2(int K, int p, std::vector<double> &out) {
    double mp[spme::kMaxP];
    host_bspline(p, 0.0, mp);  // mp[j] = M_p(p - 1 - j)
    out.resize(K);
    for (int m = 0; m < K; m++) {
        int mm = m <= K / 2 ? m : m - K;
        double phi = 2.0 * M_PI * (double)mm / (double)K;
        double re = 0.0, im = 0.0;
        for (int j = 0; j < p - 1; j++) {
            double s = mp[p - 2 - j];
            re += s * std::cos(j * phi);
            im += s * std::sin(j * phi);
        }
        out[m] = 1.0 / (re * re + im * im);
    }
}

}  // namespace spme

using spme::host_moduli2;

namespace {

constexpr int kStages = 8;

// One captured pass (or position build) and the key it was captured for.
struct GraphEntry {
    bool valid = false;
    int R = 0, prof = 0;
    const void *f = nullptr;
    void *u = nullptr;
    long ldf = 0, ldu = 0;
    double alpha = 0.0, beta = 0.0;
    cudaStream_t stream = nullptr;
    cudaGraphExec_t exec = nullptr;
    long launches = 0;
};
constexpr int kGraphSlots = 4;

struct PlanPair {
    int C;
    cufftHandle fwd;
    cufftHandle bwd;
    cufftHandle fwd2 = 0, bwd2 = 0;  // 2D (y, x) transforms of every z-plane
    bool has2d = false;
    spme::InterpMaps maps;  // TMA boxes over the mesh for this C and tile shape
    int maps_tile[3];
};

}  // namespace

struct _spme_t {
    spme_params prm;
    int device = 0;
    int last_error = SPME_OK;
    cudaStream_t own_stream = nullptr, stream = nullptr, aux = nullptr;
    cudaStream_t cap_stream = nullptr;  // graph capture when the caller's stream is the legacy default
    // host-pointer applies: inputs copied on their own stream (overlapping work
    // already queued on the main stream, e.g. a position build)
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t ev_staged = nullptr, ev_stage_free = nullptr;
    // host-pointer applies: the result leaves in parts of right-hand sides, part k
    // complete at ev_part[k]
    static constexpr int kOutParts = 4;
    cudaEvent_t ev_part[kOutParts] = {};
    cudaEvent_t ev_in[kOutParts] = {};  // force part k uploaded
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    int profiling = 0;  // 1: stage events; 2: events + real-space serialized
    cudaEvent_t ev[kStages + 1] = {};
    cudaEvent_t ev_rs[2] = {};
    float stage_ms[kStages] = {};
    bool ran_serial = false;  // last profiled pass ran the real-space sum on the main stream
    // real-space sum concurrent with the mesh pipeline (aux stream) or before it
    int overlap = 0;
    bool stages_valid = false;
    bool ran_real = false;
    long launches = 0;
    MeshGeom g{};
    int tile[3] = {8, 8, 8};
    size_t elem = 8;
    int Cmax = 3;
    int ntiles = 0;
    int nc = 1;
    bool have_pos = false;
    // device buffers
    double *d_pos = nullptr;
    int *d_key2 = nullptr, *d_key3 = nullptr;
    uint32_t *d_pstart = nullptr;  // per-particle stencil start (mesh engines)
    void *d_pfrac = nullptr;       // per-particle fractional mesh coordinates
    // d_sort_tmp: scratch of the three counting sorts (the atomic slots are kept
    // in the sorts' permutation buffers until the scatter)
    int *d_key = nullptr, *d_sort_tmp = nullptr, *d_tcount = nullptr, *d_toff = nullptr,
        *d_tperm = nullptr, *d_scan_tmp = nullptr;
    int *d_rec_idx = nullptr;
    uint32_t *d_rec_start = nullptr;
    void *d_rec_w = nullptr;
    // column-gather spread: records sorted by stencil-start cell (K^3 keys)
    bool cols = false;
    int spread_mode = 1;  // 1: column-gather kernel where it applies, 0: tile kernel
    int *d_scount = nullptr, *d_soff = nullptr, *d_sperm = nullptr, *d_srec_idx = nullptr;
    uint32_t *d_srec_start = nullptr;
    void *d_srec_w = nullptr;
    void *d_Fs = nullptr;  // force rows in start-cell order
    int *d_ccount = nullptr, *d_coff = nullptr, *d_cperm = nullptr;
    void *d_cpos = nullptr;  // float4 (FP32 engine) or double4_32a (FP64 engine)
    void *d_prel = nullptr;  // the same in particle order (from the keys pass)
    void *d_pair = nullptr;  // Chebyshev table of the pair functions (FP64 engines)
    spme::PairTable pair;
    void *d_mesh = nullptr, *d_cmesh = nullptr, *d_tab = nullptr;
    double *d_bmod2 = nullptr;
    void *d_work = nullptr;
    size_t work_bytes = 0;
    std::vector<PlanPair> plans;
    void *d_F = nullptr, *d_W = nullptr, *d_fstage = nullptr, *d_ustage = nullptr;
    void *d_W2 = nullptr;  // mesh part of the result when the real-space part is in d_W
    int *d_err = nullptr;  // device-side error flag (TMA wait timeouts)
    // FFT mode 1: 2D cuFFT + fused z-FFT/influence kernel; 0: 3D cuFFT + influence
    int fft_mode = 1;
    spme::ZPlan zp{};
    void *d_ztw = nullptr;
    int *d_zip = nullptr;
    void *d_f2tab = nullptr;  // one-pass 2D transform tables (fft_mode 2)
    CUtensorMap zmap;  // over the half spectrum (fft_mode 1)
    size_t cap_tiles = 0;  // allocated tile-count capacity
    // CUDA graphs: passes and device-pointer position builds are captured once
    // per key and replayed (spme_set_graphs)
    bool use_graphs = false;
    GraphEntry gpass[kGraphSlots];
    int gnext = 0;
    GraphEntry gpos;
};

namespace {

struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev) {
        if (cudaGetDevice(&prev) == cudaSuccess && prev != dev) cudaSetDevice(dev);
        else prev = -1;
    }
    ~DeviceGuard() {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

int from_cuda(cudaError_t e) {
    if (e == cudaSuccess) return SPME_OK;
    if (e == cudaErrorMemoryAllocation) return SPME_ERR_NOMEM;
    return SPME_ERR_CUDA;
}

int from_cufft(cufftResult r) {
    if (r == CUFFT_SUCCESS) return SPME_OK;
    if (r == CUFFT_ALLOC_FAILED) return SPME_ERR_NOMEM;
    return SPME_ERR_CUFFT;
}

#define TRY_CUDA(x)                              \
    do {                                         \
        cudaError_t e_ = (x);                    \
        if (e_ != cudaSuccess) return from_cuda(e_); \
    } while (0)
#define TRY_FFT(x)                               \
    do {                                         \
        cufftResult r_ = (x);                    \
        if (r_ != CUFFT_SUCCESS) return from_cufft(r_); \
    } while (0)
#define TRY(x)                                   \
    do {                                         \
        int s_ = (x);                            \
        if (s_ != SPME_OK) return s_;            \
    } while (0)

template <typename P>
int dalloc(P **p, size_t bytes) {
    void *q = nullptr;
    cudaError_t e = cudaMalloc(&q, bytes < 256 ? 256 : bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return SPME_ERR_NOMEM;
    }
    *p = reinterpret_cast<P *>(q);
    return SPME_OK;
}

void dfree(void *p) {
    if (p) cudaFree(p);
}

bool is_fp32(const spme_t *e) { return e->prm.precision == SPME_FP32; }

// Beenakker's self term in mobility x 6 pi eta units: (1 - 6 xi a/sqrt(pi)
// + 40 xi^3 a^3 / (3 sqrt(pi))) / a.
double self_coeff(double xi, double a) {
    const double rsp = 0.56418958354775628695;
    return (1.0 - 6.0 * xi * a * rsp + 40.0 / 3.0 * xi * xi * xi * a * a * a * rsp) / a;
}

int validate(const spme_params &p) {
    if (p.np < 0 || p.dim < 2 || p.dim > 1024) return SPME_ERR_INVALID;
    if (p.porder != 4 && p.porder != 6 && p.porder != 8) return SPME_ERR_UNSUPPORTED;
    if (p.dim < p.porder) return SPME_ERR_UNSUPPORTED;
    if (!(p.box_size > 0.0) || !(p.xi > 0.0) || !(p.radius > 0.0)) return SPME_ERR_INVALID;
    if (p.precision != SPME_FP64 && p.precision != SPME_FP32) return SPME_ERR_INVALID;
    if (p.max_nrhs < 1 || p.max_nrhs > 1024) return SPME_ERR_INVALID;
    if (p.terms <= 0 || (p.terms & ~SPME_TERM_ALL)) return SPME_ERR_INVALID;
    if ((p.terms & SPME_TERM_REAL) && !(p.rcut > 0.0 && p.rcut < 0.5 * p.box_size))
        return SPME_ERR_INVALID;
    return SPME_OK;
}

void set_geometry(spme_t *e) {
    MeshGeom &g = e->g;
    g.K = e->prm.dim;
    g.p = e->prm.porder;
    g.L = e->prm.box_size;
    g.invL = 1.0 / e->prm.box_size;
    g.tx = std::min(e->tile[0], g.K);
    g.ty = std::min(e->tile[1], g.K);
    g.tz = std::min(e->tile[2], g.K);
    g.ntx = (g.K + g.tx - 1) / g.tx;
    g.nty = (g.K + g.ty - 1) / g.ty;
    g.ntz = (g.K + g.tz - 1) / g.tz;
    e->ntiles = g.ntx * g.nty * g.ntz;
}

int record_width(const spme_t *e) {
    int raw = 3 * e->prm.porder, per16 = (int)(16 / e->elem);
    return (raw + per16 - 1) / per16 * per16;
}

int alloc_tiles(spme_t *e) {
    size_t need = (size_t)e->ntiles;
    if (need <= e->cap_tiles && e->d_tcount) return SPME_OK;
    dfree(e->d_tcount);
    dfree(e->d_toff);
    dfree(e->d_scan_tmp);
    e->d_tcount = e->d_toff = e->d_scan_tmp = nullptr;
    size_t ncell = (size_t)e->nc * e->nc * e->nc;
    size_t nkeys = std::max(need, ncell);
    if (e->cols) nkeys = std::max(nkeys, (size_t)e->prm.dim * e->prm.dim * e->prm.dim);
    TRY(dalloc(&e->d_tcount, sizeof(int) * need));
    TRY(dalloc(&e->d_toff, sizeof(int) * (need + 1)));
    TRY(dalloc(&e->d_scan_tmp, sizeof(int) * spme::scan_tmp_elems((int)nkeys)));
    e->cap_tiles = need;
    return SPME_OK;
}

// cuFFT plan candidates: the default kernels and the patient-JIT search, which
// is faster at some sizes and slower at others on GB300 (2D transforms at
// K = 256: 2.44 vs 2.56 ms per direction; K = 160: 0.84 vs 0.80 ms).
struct PlanCand {
    cufftHandle h[2] = {0, 0};  // [patient]
    size_t ws = 0;
    void drop() {
        for (cufftHandle &x : h)
            if (x) {
                cufftDestroy(x);
                x = 0;
            }
    }
};

// Creates the candidates (patient one only when `both`); false if the default
// plan cannot be made.
bool make_cands(PlanCand &pc, int rank, int *n, int *inembed, int idist, int *onembed, int odist,
                cufftType type, int batch, bool both) {
    for (int pt = 0; pt < (both ? 2 : 1); pt++) {
        cufftHandle h = 0;
        if (cufftCreate(&h) != CUFFT_SUCCESS) continue;
        bool ok = cufftSetAutoAllocation(h, 0) == CUFFT_SUCCESS;
        if (ok && pt)
            ok = cufftSetPlanPropertyInt64(h, NVFFT_PLAN_PROPERTY_INT64_PATIENT_JIT, 1) ==
                 CUFFT_SUCCESS;
        size_t w = 0;
        if (ok)
            ok = cufftMakePlanMany(h, rank, n, inembed, 1, idist, onembed, 1, odist, type, batch,
                                   &w) == CUFFT_SUCCESS;
        if (!ok) {
            cufftDestroy(h);
            continue;
        }
        pc.h[pt] = h;
        pc.ws = std::max(pc.ws, w);
    }
    return pc.h[0] != 0;
}

// With the work area in place: times each candidate once (one warm and one
// timed run on the engine's mesh buffers, whose contents the next pass
// overwrites; not while the stream is being captured), keeps the faster.
cufftHandle pick_cand(spme_t *e, PlanCand &pc, bool inverse) {
    for (cufftHandle h : pc.h)
        if (h) {
            cufftSetWorkArea(h, e->d_work);
            cufftSetStream(h, e->stream);
        }
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(e->stream, &cs);
    auto exec = [&](cufftHandle h) {
        if (is_fp32(e))
            return inverse ? cufftExecC2R(h, (cufftComplex *)e->d_cmesh, (cufftReal *)e->d_mesh)
                           : cufftExecR2C(h, (cufftReal *)e->d_mesh, (cufftComplex *)e->d_cmesh);
        return inverse ? cufftExecZ2D(h, (cufftDoubleComplex *)e->d_cmesh, (cufftDoubleReal *)e->d_mesh)
                       : cufftExecD2Z(h, (cufftDoubleReal *)e->d_mesh, (cufftDoubleComplex *)e->d_cmesh);
    };
    auto time_ms = [&](cufftHandle h) -> float {
        if (exec(h) != CUFFT_SUCCESS) return -1.f;
        cudaEventRecord(e->ev[0], e->stream);
        if (exec(h) != CUFFT_SUCCESS) return -1.f;
        cudaEventRecord(e->ev[1], e->stream);
        float ms = -1.f;
        if (cudaEventSynchronize(e->ev[1]) != cudaSuccess ||
            cudaEventElapsedTime(&ms, e->ev[0], e->ev[1]) != cudaSuccess)
            return -1.f;
        return ms;
    };
    int k = 0;
    if (pc.h[1] && cs == cudaStreamCaptureStatusNone) {
        const float t0 = time_ms(pc.h[0]), t1 = time_ms(pc.h[1]);
        if (t1 > 0.f && t0 > 0.f && t1 < t0) k = 1;
    }
    cudaGetLastError();
    const cufftHandle h = pc.h[k];
    if (pc.h[1 - k]) cufftDestroy(pc.h[1 - k]);
    pc.h[0] = pc.h[1] = 0;
    return h;
}

int get_plans(spme_t *e, int C, PlanPair **out) {
    for (PlanPair &p : e->plans)
        if (p.C == C) {
            *out = &p;
            return SPME_OK;
        }
    const int K = e->prm.dim;
    int n[3] = {K, K, K}, re[3] = {K, K, K}, ce[3] = {K, K, K / 2 + 1};
    PlanPair pp;
    pp.C = C;
    pp.maps_tile[0] = pp.maps_tile[1] = pp.maps_tile[2] = 0;
    cufftType tf = is_fp32(e) ? CUFFT_R2C : CUFFT_D2Z;
    cufftType tb = is_fp32(e) ? CUFFT_C2R : CUFFT_Z2D;
    // component-major: batch b of the real mesh at b*K^3, of the half spectrum at b*Kc.
    // 3D plans (run in fft_mode 0, candidates timed there) and, in fft_mode 1, 2D
    // (y, x) plans of the C*K z-planes with the same memory layout
    const long long K3 = (long long)K * K * K, Kc = (long long)K * K * (K / 2 + 1);
    const bool mode0 = e->fft_mode == 0, mode1 = e->fft_mode == 1;
    PlanCand c3[2], c2[2];
    auto drop_all = [&]() {
        for (PlanCand &c : c3) c.drop();
        for (PlanCand &c : c2) c.drop();
    };
    if (!make_cands(c3[0], 3, n, re, (int)K3, ce, (int)Kc, tf, C, mode0) ||
        !make_cands(c3[1], 3, n, ce, (int)Kc, re, (int)K3, tb, C, mode0)) {
        drop_all();
        return SPME_ERR_CUDA;
    }
    const int Khp = K / 2 + 1, P2 = K * K, C2 = K * Khp;
    int n2[2] = {K, K}, re2[2] = {K, K}, ce2[2] = {K, Khp};
    if (mode1 && (!make_cands(c2[0], 2, n2, re2, P2, ce2, C2, tf, C * K, true) ||
                  !make_cands(c2[1], 2, n2, ce2, C2, re2, P2, tb, C * K, true))) {
        drop_all();
        return SPME_ERR_CUDA;
    }
    size_t ws = 0;
    for (PlanCand &c : c3) ws = std::max(ws, c.ws);
    for (PlanCand &c : c2) ws = std::max(ws, c.ws);
    if (ws > e->work_bytes) {
        dfree(e->d_work);
        e->d_work = nullptr;
        e->work_bytes = 0;
        if (dalloc(&e->d_work, ws) != SPME_OK) {
            drop_all();
            return SPME_ERR_NOMEM;
        }
        e->work_bytes = ws;
        bool ok = true;
        for (PlanPair &q : e->plans) {
            ok = ok && cufftSetWorkArea(q.fwd, e->d_work) == CUFFT_SUCCESS &&
                 cufftSetWorkArea(q.bwd, e->d_work) == CUFFT_SUCCESS;
            if (q.has2d)
                ok = ok && cufftSetWorkArea(q.fwd2, e->d_work) == CUFFT_SUCCESS &&
                     cufftSetWorkArea(q.bwd2, e->d_work) == CUFFT_SUCCESS;
        }
        if (!ok) {
            drop_all();
            return SPME_ERR_CUDA;
        }
    }
    pp.fwd = pick_cand(e, c3[0], false);
    pp.bwd = pick_cand(e, c3[1], true);
    if (mode1) {
        pp.fwd2 = pick_cand(e, c2[0], false);
        pp.bwd2 = pick_cand(e, c2[1], true);
        pp.has2d = true;
    }
    TRY_CUDA(cudaGetLastError());
    e->plans.push_back(pp);
    *out = &e->plans.back();
    return SPME_OK;
}

int create_impl(const spme_params &prm, spme_t **out) {
    TRY(validate(prm));
    spme_t *e = new (std::nothrow) _spme_t();
    if (!e) return SPME_ERR_NOMEM;
    *out = e;
    e->prm = prm;
    cudaGetDevice(&e->device);
    e->elem = is_fp32(e) ? sizeof(float) : sizeof(double);
    e->Cmax = 3 * prm.max_nrhs;
    set_geometry(e);
    if (prm.terms & SPME_TERM_REAL) {
        long nc = (long)std::floor(prm.box_size / prm.rcut);
        long cap = std::max<long>(3, (long)std::cbrt(8.0 * prm.np + 27.0));
        nc = std::min(nc, std::min(cap, 1024L));
        e->nc = nc < 3 ? 1 : (int)nc;
    }
    TRY_CUDA(cudaStreamCreateWithFlags(&e->own_stream, cudaStreamNonBlocking));
    TRY_CUDA(cudaStreamCreateWithFlags(&e->aux, cudaStreamNonBlocking));
    TRY_CUDA(cudaStreamCreateWithFlags(&e->cap_stream, cudaStreamNonBlocking));
    TRY_CUDA(cudaStreamCreateWithFlags(&e->copy_stream, cudaStreamNonBlocking));
    TRY_CUDA(cudaEventCreateWithFlags(&e->ev_staged, cudaEventDisableTiming));
    TRY_CUDA(cudaEventCreateWithFlags(&e->ev_stage_free, cudaEventDisableTiming));
    for (cudaEvent_t &ev : e->ev_part) TRY_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    for (cudaEvent_t &ev : e->ev_in) TRY_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    e->stream = e->own_stream;
    TRY_CUDA(cudaEventCreateWithFlags(&e->ev_fork, cudaEventDisableTiming));
    TRY_CUDA(cudaEventCreateWithFlags(&e->ev_join, cudaEventDisableTiming));
    for (int i = 0; i <= kStages; i++) TRY_CUDA(cudaEventCreate(&e->ev[i]));
    TRY_CUDA(cudaEventCreate(&e->ev_rs[0]));
    TRY_CUDA(cudaEventCreate(&e->ev_rs[1]));

    const size_t n = (size_t)prm.np, K = (size_t)prm.dim, Kh = K / 2 + 1;
    const size_t C = (size_t)e->Cmax;
    TRY(dalloc(&e->d_pos, sizeof(double) * 3 * n));
    TRY(dalloc(&e->d_key, sizeof(int) * n));
    TRY(dalloc(&e->d_sort_tmp, sizeof(int) * n));
    TRY(dalloc(&e->d_key3, sizeof(int) * n));
    TRY(dalloc(&e->d_tperm, sizeof(int) * n));
    if (prm.terms & SPME_TERM_RECIP) {
        TRY(dalloc(&e->d_pstart, sizeof(uint32_t) * n));
        TRY(dalloc(&e->d_pfrac, e->elem * 3 * n));
    }
    e->cols = (prm.terms & SPME_TERM_RECIP) && spme::spread_cols_ok((int)K, (int)C, e->elem, prm.porder);
    if (e->cols) {
        const size_t K3 = K * K * K;
        TRY(dalloc(&e->d_scount, sizeof(int) * K3));
        TRY(dalloc(&e->d_soff, sizeof(int) * (K3 + 1)));
        TRY(dalloc(&e->d_sperm, sizeof(int) * n));
        TRY(dalloc(&e->d_key2, sizeof(int) * n));
        TRY(dalloc(&e->d_srec_idx, sizeof(int) * n));
        TRY(dalloc(&e->d_srec_start, sizeof(uint32_t) * n));
        TRY(dalloc(&e->d_srec_w, e->elem * record_width(e) * n));
        TRY(dalloc(&e->d_Fs, e->elem * (size_t)spme::spread_cols_row_width((int)C) * n));
    }
    TRY(alloc_tiles(e));
    TRY(dalloc(&e->d_rec_idx, sizeof(int) * n));
    TRY(dalloc(&e->d_rec_start, sizeof(uint32_t) * n));
    TRY(dalloc(&e->d_rec_w, e->elem * record_width(e) * n));
    if (prm.terms & SPME_TERM_REAL) {
        size_t ncell = (size_t)e->nc * e->nc * e->nc;
        TRY(dalloc(&e->d_ccount, sizeof(int) * ncell));
        TRY(dalloc(&e->d_coff, sizeof(int) * (ncell + 1)));
        TRY(dalloc(&e->d_cperm, sizeof(int) * n));
        TRY(dalloc(&e->d_cpos, sizeof(double4_32a) * n));
        TRY(dalloc(&e->d_prel, sizeof(double4_32a) * n));
        // FP64: the pair functions from a Chebyshev table instead of erfc / exp
        std::vector<double> coef;
        if (!is_fp32(e) && spme::build_pair_table(prm.xi, prm.radius, prm.rcut, &coef, &e->pair)) {
            TRY(dalloc(&e->d_pair, sizeof(double) * coef.size()));
            TRY_CUDA(cudaMemcpy(e->d_pair, coef.data(), sizeof(double) * coef.size(),
                                cudaMemcpyHostToDevice));
            e->pair.coef = (const double *)e->d_pair;
        } else {
            e->pair = spme::PairTable{};
        }
    }
    if (prm.terms & SPME_TERM_RECIP) {
        TRY(dalloc(&e->d_mesh, e->elem * K * K * K * C));
        TRY(dalloc(&e->d_cmesh, 2 * e->elem * K * K * Kh * C));
        TRY(dalloc(&e->d_tab, 2 * e->elem * K * K * Kh));
        TRY(dalloc(&e->d_bmod2, sizeof(double) * K));
        std::vector<double> bm;
        host_moduli2((int)K, prm.porder, bm);
        TRY_CUDA(cudaMemcpyAsync(e->d_bmod2, bm.data(), sizeof(double) * K,
                                 cudaMemcpyHostToDevice, e->stream));
        if (is_fp32(e))
            spme::launch_influence_table<float>((float *)e->d_tab, e->d_bmod2, (int)K,
                                                prm.box_size, prm.xi, prm.radius, e->stream);
        else
            spme::launch_influence_table<double>((double *)e->d_tab, e->d_bmod2, (int)K,
                                                 prm.box_size, prm.xi, prm.radius, e->stream);
        e->launches++;
        TRY_CUDA(cudaGetLastError());
        std::vector<double> twd;
        std::vector<int> ip;
        if (spme::zfft_width((int)K, e->elem) > 0 && spme::make_zplan((int)K, e->elem, &e->zp, &twd, &ip) &&
            spme::make_zfft_map(&e->zmap, e->d_cmesh, (int)K, (int)C, e->elem)) {
            TRY(dalloc(&e->d_ztw, 2 * e->elem * K));
            TRY(dalloc(&e->d_zip, sizeof(int) * K));
            if (is_fp32(e)) {
                std::vector<float> twf(twd.begin(), twd.end());
                TRY_CUDA(cudaMemcpy(e->d_ztw, twf.data(), sizeof(float) * twf.size(),
                                    cudaMemcpyHostToDevice));
            } else {
                TRY_CUDA(cudaMemcpy(e->d_ztw, twd.data(), sizeof(double) * twd.size(),
                                    cudaMemcpyHostToDevice));
            }
            TRY_CUDA(cudaMemcpy(e->d_zip, ip.data(), sizeof(int) * K, cudaMemcpyHostToDevice));
            // measured on GB300 (K = 256): the fused path wins in FP32; in FP64
            // the 3D transforms + influence are as fast
            e->fft_mode = is_fp32(e) ? 1 : 0;
            // tables of the one-pass 2D transforms (fft_mode 2, opt-in: measured
            // slower than cuFFT's two-pass 2D transforms on GB300, 3.7 vs 2.55 ms
            // per direction at K = 256, 48 components)
            std::vector<unsigned char> f2;
            if (e->fft_mode == 1 && spme::fft2d_ok((int)K, e->elem) &&
                spme::make_fft2d_tables((int)K, &f2)) {
                TRY(dalloc(&e->d_f2tab, f2.size()));
                TRY_CUDA(cudaMemcpy(e->d_f2tab, f2.data(), f2.size(), cudaMemcpyHostToDevice));
            }
        } else {
            e->fft_mode = 0;
        }
        PlanPair *pp;
        TRY(get_plans(e, (int)C, &pp));
    }
    TRY(dalloc(&e->d_err, sizeof(int)));
    TRY_CUDA(cudaMemsetAsync(e->d_err, 0, sizeof(int), e->stream));
    TRY(dalloc(&e->d_F, e->elem * n * C));
    TRY(dalloc(&e->d_W, e->elem * n * C));
    if ((prm.terms & SPME_TERM_RECIP) && (prm.terms & (SPME_TERM_REAL | SPME_TERM_SELF)))
        TRY(dalloc(&e->d_W2, e->elem * n * C));
    TRY(dalloc(&e->d_fstage, e->elem * n * C));
    TRY(dalloc(&e->d_ustage, e->elem * n * C));
    TRY_CUDA(cudaStreamSynchronize(e->stream));
    return SPME_OK;
}

void drop_graph(GraphEntry &g) {
    if (g.exec) cudaGraphExecDestroy(g.exec);
    g = GraphEntry();
}

void drop_graphs(spme_t *e) {
    for (GraphEntry &g : e->gpass) drop_graph(g);
    drop_graph(e->gpos);
    e->gnext = 0;
}

// Capture `body` on the engine's stream into g (launch count of the captured
// kernels kept for the replays), then launch it.
void use_stream(spme_t *e, cudaStream_t s) {
    e->stream = s;
    for (PlanPair &p : e->plans) {
        cufftSetStream(p.fwd, s);
        cufftSetStream(p.bwd, s);
        if (p.has2d) {
            cufftSetStream(p.fwd2, s);
            cufftSetStream(p.bwd2, s);
        }
    }
}

template <typename F>
int capture_and_launch(spme_t *e, GraphEntry &g, F body) {
    const long l0 = e->launches;
    // the legacy default stream cannot be captured: capture on a side stream
    // (ordered after the default stream's earlier work) and launch there
    const cudaStream_t orig = e->stream;
    const cudaStream_t cs = orig ? orig : e->cap_stream;
    if (cs != orig) use_stream(e, cs);
    TRY_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
    int st = body();
    cudaGraph_t graph = nullptr;
    cudaError_t ce = cudaStreamEndCapture(cs, &graph);
    if (cs != orig) use_stream(e, orig);
    if (st != SPME_OK || ce != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        cudaGetLastError();
        return st != SPME_OK ? st : from_cuda(ce);
    }
    cudaGraphExec_t exec = nullptr;
    ce = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    TRY_CUDA(ce);
    drop_graph(g);
    g.exec = exec;
    g.launches = e->launches - l0;
    g.valid = true;
    e->launches = l0;
    TRY_CUDA(cudaGraphLaunch(g.exec, e->stream));
    e->launches += g.launches;
    return SPME_OK;
}

void destroy_impl(spme_t *e) {
    if (!e) return;
    DeviceGuard dg(e->device);
    if (e->stream) cudaStreamSynchronize(e->stream);
    if (e->aux) cudaStreamSynchronize(e->aux);
    drop_graphs(e);
    for (PlanPair &p : e->plans) {
        cufftDestroy(p.fwd);
        cufftDestroy(p.bwd);
        if (p.has2d) {
            cufftDestroy(p.fwd2);
            cufftDestroy(p.bwd2);
        }
    }
    void *bufs[] = {e->d_pos,    e->d_key,     e->d_sort_tmp, e->d_tcount,   e->d_toff,
                    e->d_tperm,  e->d_scan_tmp, e->d_rec_idx, e->d_rec_start, e->d_rec_w,
                    e->d_ccount, e->d_coff,    e->d_cperm, e->d_cpos,     e->d_prel, e->d_mesh,
                    e->d_cmesh,  e->d_tab,     e->d_bmod2, e->d_work,     e->d_F,
                    e->d_W,      e->d_fstage,  e->d_ustage, e->d_err,  e->d_ztw,
                    e->d_zip,    e->d_f2tab,    e->d_scount,  e->d_soff,   e->d_sperm, e->d_srec_idx,
                    e->d_srec_start, e->d_srec_w, e->d_Fs, e->d_W2, e->d_pair, e->d_key2,
                    e->d_key3,   e->d_pstart, e->d_pfrac};
    for (void *b : bufs) dfree(b);
    for (int i = 0; i <= kStages; i++)
        if (e->ev[i]) cudaEventDestroy(e->ev[i]);
    if (e->ev_rs[0]) cudaEventDestroy(e->ev_rs[0]);
    if (e->ev_rs[1]) cudaEventDestroy(e->ev_rs[1]);
    if (e->ev_fork) cudaEventDestroy(e->ev_fork);
    if (e->ev_join) cudaEventDestroy(e->ev_join);
    if (e->aux) cudaStreamDestroy(e->aux);
    if (e->cap_stream) cudaStreamDestroy(e->cap_stream);
    if (e->copy_stream) cudaStreamDestroy(e->copy_stream);
    if (e->ev_staged) cudaEventDestroy(e->ev_staged);
    if (e->ev_stage_free) cudaEventDestroy(e->ev_stage_free);
    for (cudaEvent_t ev : e->ev_part)
        if (ev) cudaEventDestroy(ev);
    for (cudaEvent_t ev : e->ev_in)
        if (ev) cudaEventDestroy(ev);
    if (e->own_stream) cudaStreamDestroy(e->own_stream);
    delete e;
}

int set_positions_body(spme_t *e, const double *pos, int mem) {
    const int n = e->prm.np;
    cudaStream_t s = e->stream;
    if (n > 0) {
        if (!pos) return SPME_ERR_INVALID;
        TRY_CUDA(cudaMemcpyAsync(e->d_pos, pos, sizeof(double) * 3 * n,
                                 mem == SPME_MEM_HOST ? cudaMemcpyHostToDevice
                                                      : cudaMemcpyDeviceToDevice,
                                 s));
    }
    const bool recip = (e->prm.terms & SPME_TERM_RECIP) != 0;  // geometry set by the caller
    const bool real = (e->prm.terms & SPME_TERM_REAL) != 0;
    const bool cols = recip && e->cols;
    const int ncell = e->nc * e->nc * e->nc;
    const int K3 = e->g.K * e->g.K * e->g.K;
    if (recip) TRY_CUDA(cudaMemsetAsync(e->d_tcount, 0, sizeof(int) * e->ntiles, s));
    if (cols) TRY_CUDA(cudaMemsetAsync(e->d_scount, 0, sizeof(int) * K3, s));
    if (real) TRY_CUDA(cudaMemsetAsync(e->d_ccount, 0, sizeof(int) * ncell, s));
    if (recip || real) {
        // one pass over the positions for every key this engine sorts by
        spme::launch_all_keys(e->d_pos, n, e->g, e->nc, e->d_key, recip ? e->d_tcount : nullptr,
                              e->d_tperm, e->d_key2, cols ? e->d_scount : nullptr, e->d_sperm,
                              e->d_key3, real ? e->d_ccount : nullptr, e->d_cperm,
                              recip ? e->d_pstart : nullptr, e->d_pfrac,
                              real ? e->d_prel : nullptr, is_fp32(e), s);
        e->launches++;
    }
    if (recip) {
        spme::launch_scan(e->d_tcount, e->ntiles, e->d_toff, e->d_scan_tmp, s);
        spme::launch_scatter(e->d_key, e->d_toff, n, e->d_tperm, e->d_sort_tmp, s);
        if (is_fp32(e))
            spme::launch_records<float>(e->d_pstart, (const float *)e->d_pfrac, e->d_tperm, n,
                                        e->g.p, e->d_rec_idx, e->d_rec_start,
                                        (float *)e->d_rec_w, s);
        else
            spme::launch_records<double>(e->d_pstart, (const double *)e->d_pfrac, e->d_tperm, n,
                                         e->g.p, e->d_rec_idx, e->d_rec_start,
                                         (double *)e->d_rec_w, s);
        e->launches += 6;
    }
    if (cols) {
        spme::launch_scan(e->d_scount, K3, e->d_soff, e->d_scan_tmp, s);
        spme::launch_scatter(e->d_key2, e->d_soff, n, e->d_sperm, e->d_sort_tmp, s);
        if (is_fp32(e))
            spme::launch_records<float>(e->d_pstart, (const float *)e->d_pfrac, e->d_sperm, n,
                                        e->g.p, e->d_srec_idx, e->d_srec_start,
                                        (float *)e->d_srec_w, s);
        else
            spme::launch_records<double>(e->d_pstart, (const double *)e->d_pfrac, e->d_sperm, n,
                                         e->g.p, e->d_srec_idx, e->d_srec_start,
                                         (double *)e->d_srec_w, s);
        e->launches += 6;
    }
    if (real) {
        spme::launch_scan(e->d_ccount, ncell, e->d_coff, e->d_scan_tmp, s);
        spme::launch_scatter(e->d_key3, e->d_coff, n, e->d_cperm, e->d_sort_tmp, s);
        spme::launch_cell_gather(e->d_prel, e->d_cperm, n, is_fp32(e), e->d_cpos, s);
        e->launches += 6;
    }
    TRY_CUDA(cudaGetLastError());
    return SPME_OK;
}

int set_positions_impl(spme_t *e, const double *pos, int mem) {
    if (e->prm.np > 0 && !pos) return SPME_ERR_INVALID;
    if (e->prm.terms & SPME_TERM_RECIP) {
        set_geometry(e);
        TRY(alloc_tiles(e));
    }
    // host positions come from pageable memory: never captured
    if (!e->use_graphs || mem != SPME_MEM_DEVICE || e->prm.np == 0) {
        TRY(set_positions_body(e, pos, mem));
    } else if (e->gpos.valid && e->gpos.f == pos && e->gpos.stream == e->stream) {
        TRY_CUDA(cudaGraphLaunch(e->gpos.exec, e->stream));
        e->launches += e->gpos.launches;
    } else {
        TRY(capture_and_launch(e, e->gpos, [&]() { return set_positions_body(e, pos, mem); }));
        e->gpos.f = pos;
        e->gpos.stream = e->stream;
    }
    e->have_pos = true;
    return SPME_OK;
}

template <typename T>
int run_pass(spme_t *e, int R, const T *f, long ldf, T *u, long ldu, double alpha, double beta,
             int rpart) {
    const int n = e->prm.np, C = 3 * R, K = e->prm.dim;
    const int terms = e->prm.terms;
    cudaStream_t s = e->stream;
    const bool rs = (terms & (SPME_TERM_REAL | SPME_TERM_SELF)) != 0;
    const bool prof = e->profiling;
    T *F = (T *)e->d_F, *W = (T *)e->d_W;
    if (prof) cudaEventRecord(e->ev[0], s);
    if (f) {  // null: F already packed (host-pointer applies pack on the copy stream)
        spme::launch_pack_tiled<T>(f, ldf, n, R, F, s);
        e->launches++;
    }
    if (prof) cudaEventRecord(e->ev[1], s);
    // the real-space sum runs before the mesh pipeline on the main stream, or
    // (overlap on) concurrently on the aux stream; at profiling level 2 always
    // on the main stream so every stage is timed alone
    const bool serial = e->profiling >= 2 || !e->overlap;
    cudaStream_t rss = serial ? s : e->aux;
    if (rs) {
        if (!serial) {
            TRY_CUDA(cudaEventRecord(e->ev_fork, s));
            TRY_CUDA(cudaStreamWaitEvent(e->aux, e->ev_fork, 0));
        }
        if (prof) cudaEventRecord(e->ev_rs[0], rss);
        if (terms & SPME_TERM_REAL) {
            if (!e->d_coff || !e->d_cperm || !e->d_cpos) return SPME_ERR_STATE;
            TRY_CUDA(spme::launch_realspace<T>(e->nc, e->d_coff, e->d_cperm, e->d_cpos, F, R,
                                               e->prm.box_size, e->prm.rcut, e->prm.xi,
                                               e->prm.radius, (terms & SPME_TERM_SELF) ? 1 : 0,
                                               e->pair, W, rss));
        } else {
            spme::launch_self<T>(F, n, R, self_coeff(e->prm.xi, e->prm.radius), W, rss);
        }
        e->launches++;
        if (prof) cudaEventRecord(e->ev_rs[1], rss);
        TRY_CUDA(cudaEventRecord(e->ev_join, rss));
        if (serial) cudaEventRecord(e->ev[1], s);
    }
    if (terms & SPME_TERM_RECIP) {
        if (!e->d_mesh || !e->d_cmesh || !e->d_tab) return SPME_ERR_STATE;
        PlanPair *pp;
        TRY(get_plans(e, C, &pp));
        // column gather where it applies; measured on GB300 (K = 256, N = 1e6): in FP64
        // it wins at every C (8.0 vs 19.6 ms at C = 3), in FP32 from C = 9 on (the
        // tile kernel's per-component cost is lower at C = 3, 6)
        // (the kernel stages force-row offsets as 32-bit integers)
        const bool use_cols = e->cols && e->spread_mode == 1 &&
                              spme::spread_cols_ok(K, C, e->elem, e->g.p) &&
                              (e->elem == 8 || C >= 9) &&
                              (long long)n * spme::spread_cols_row_width(C) < (1LL << 31);
        if (use_cols) {
            spme::launch_gather_cols_rows<T>(F, e->d_srec_idx, n, C, (T *)e->d_Fs, s);
            TRY_CUDA(spme::launch_spread_cols<T>(e->d_soff, e->d_srec_start,
                                                 (const T *)e->d_srec_w, (const T *)e->d_Fs, C,
                                                 e->g, (T *)e->d_mesh, s));
            e->launches++;
        } else
            TRY_CUDA(spme::launch_spread<T>(e->d_toff, e->d_rec_idx, e->d_rec_start,
                                            (const T *)e->d_rec_w, F, C, e->g, (T *)e->d_mesh, s));
        e->launches++;
        if (prof) cudaEventRecord(e->ev[2], s);
        // fft_mode 2: this project's one-pass 2D transforms; 1: cuFFT's 2D
        // transforms; both followed by the fused z transform + influence
        const bool own2d = e->fft_mode == 2 && e->d_f2tab;
        const bool fused = own2d || (e->fft_mode == 1 && pp->has2d);
        cufftHandle fwd = fused ? pp->fwd2 : pp->fwd, bwd = fused ? pp->bwd2 : pp->bwd;
        if (own2d) {
            TRY_CUDA(spme::launch_fft2d_r2c(K, (const float *)e->d_mesh, (float *)e->d_cmesh,
                                            (long)C * K, e->d_f2tab, s));
            e->launches++;
        } else if (sizeof(T) == 4)
            TRY_FFT(cufftExecR2C(fwd, (cufftReal *)e->d_mesh, (cufftComplex *)e->d_cmesh));
        else
            TRY_FFT(cufftExecD2Z(fwd, (cufftDoubleReal *)e->d_mesh,
                                 (cufftDoubleComplex *)e->d_cmesh));
        if (prof) cudaEventRecord(e->ev[3], s);
        if (fused) {
            TRY_CUDA(spme::launch_zfft_influence<T>(e->zmap, (T *)e->d_cmesh, (const T *)e->d_tab,
                                                    (const T *)e->d_ztw, e->d_zip, e->zp,
                                                    e->prm.box_size, R, e->d_err, s));
            e->launches++;
        } else {
            spme::launch_influence<T>((T *)e->d_cmesh, (const T *)e->d_tab, K, e->prm.box_size,
                                      R, s);
            e->launches += 2;
        }
        if (prof) cudaEventRecord(e->ev[4], s);
        if (own2d) {
            TRY_CUDA(spme::launch_fft2d_c2r(K, (const float *)e->d_cmesh, (float *)e->d_mesh,
                                            (long)C * K, e->d_f2tab, s));
            e->launches++;
        } else if (sizeof(T) == 4)
            TRY_FFT(cufftExecC2R(bwd, (cufftComplex *)e->d_cmesh, (cufftReal *)e->d_mesh));
        else
            TRY_FFT(cufftExecZ2D(bwd, (cufftDoubleComplex *)e->d_cmesh,
                                 (cufftDoubleReal *)e->d_mesh));
        if (prof) cudaEventRecord(e->ev[5], s);
        if (pp->maps_tile[0] != e->g.tx || pp->maps_tile[1] != e->g.ty ||
            pp->maps_tile[2] != e->g.tz) {
            spme::make_interp_maps(&pp->maps, e->d_mesh, C, e->g, e->elem);
            pp->maps_tile[0] = e->g.tx;
            pp->maps_tile[1] = e->g.ty;
            pp->maps_tile[2] = e->g.tz;
        }
        // the mesh part goes to its own buffer when W holds the real-space part:
        // no read-modify-write (and no wait for the real-space sum) in the
        // interpolation; the unpack adds the two
        T *Wm = rs ? (T *)e->d_W2 : W;
        if (!Wm) return SPME_ERR_STATE;
        // rpart > 0: interpolation and unpack in parts of rpart right-hand sides (a
        // multiple of 4: 12 components, whole 4-component interpolation chunks),
        // part k complete at ev_part[k], so a host copy of a part overlaps the
        // next part's interpolation
        const int rp = rpart > 0 ? rpart : R;
        for (int r0 = 0, k = 0; r0 < R; r0 += rp, k++) {
            const int r1 = std::min(R, r0 + rp);
            TRY_CUDA(spme::launch_interp<T>(pp->maps, e->d_toff, n, e->d_rec_idx,
                                            e->d_rec_start, (const T *)e->d_rec_w,
                                            (const T *)e->d_mesh, C, 3 * r0, 3 * r1, e->g, Wm, 0,
                                            e->d_err, s));
            e->launches++;
            if (prof && r1 == R) cudaEventRecord(e->ev[6], s);
            if (rs && k == 0) TRY_CUDA(cudaStreamWaitEvent(s, e->ev_join, 0));
            spme::launch_unpack_tiled<T>(W, rs ? Wm : nullptr, n, R, r0, r1, alpha, beta, u, ldu,
                                         s);
            if (r1 < R) e->launches++;
            if (rpart > 0 && k < spme_t::kOutParts) TRY_CUDA(cudaEventRecord(e->ev_part[k], s));
        }
    } else {
        TRY_CUDA(cudaStreamWaitEvent(s, e->ev_join, 0));
        if (prof)
            for (int k = 2; k <= 6; k++) cudaEventRecord(e->ev[k], s);
        spme::launch_unpack_tiled<T>(W, nullptr, n, R, 0, R, alpha, beta, u, ldu, s);
        if (rpart > 0) TRY_CUDA(cudaEventRecord(e->ev_part[0], s));
    }
    e->launches++;
    if (prof) cudaEventRecord(e->ev[7], s);
    e->ran_real = rs;
    e->ran_serial = serial;
    e->stages_valid = prof;
    return from_cuda(cudaGetLastError());
}

// A device-side check (bounded TMA wait) failed: report it once and clear.
int check_device_error(spme_t *e) {
    int h = 0;
    TRY_CUDA(cudaMemcpy(&h, e->d_err, sizeof(int), cudaMemcpyDeviceToHost));
    if (h) {
        TRY_CUDA(cudaMemset(e->d_err, 0, sizeof(int)));
        return SPME_ERR_KERNEL;
    }
    return SPME_OK;
}

int pass_body(spme_t *e, int R, const void *f, long ldf, void *u, long ldu, double alpha,
              double beta, int rpart = 0) {
    if (is_fp32(e))
        return run_pass<float>(e, R, (const float *)f, ldf, (float *)u, ldu, alpha, beta, rpart);
    return run_pass<double>(e, R, (const double *)f, ldf, (double *)u, ldu, alpha, beta, rpart);
}

// One mesh pass of R right-hand sides, replayed from a CUDA graph when graphs
// are on (key: R, pointers, leading dimensions, alpha, beta, profiling level,
// stream).
int pass(spme_t *e, int R, const void *f, long ldf, void *u, long ldu, double alpha,
         double beta) {
    if (!e->use_graphs) return pass_body(e, R, f, ldf, u, ldu, alpha, beta);
    for (GraphEntry &g : e->gpass) {
        if (g.valid && g.R == R && g.f == f && g.u == u && g.ldf == ldf && g.ldu == ldu &&
            g.alpha == alpha && g.beta == beta && g.prof == e->profiling &&
            g.stream == e->stream) {
            TRY_CUDA(cudaGraphLaunch(g.exec, e->stream));
            e->launches += g.launches;
            e->ran_real = (e->prm.terms & (SPME_TERM_REAL | SPME_TERM_SELF)) != 0;
            e->stages_valid = e->profiling > 0;
            return SPME_OK;
        }
    }
    if (e->prm.terms & SPME_TERM_RECIP) {  // plans (and their work area) before capture
        PlanPair *pp;
        TRY(get_plans(e, 3 * R, &pp));
    }
    GraphEntry &g = e->gpass[e->gnext];
    e->gnext = (e->gnext + 1) % kGraphSlots;
    TRY(capture_and_launch(e, g, [&]() { return pass_body(e, R, f, ldf, u, ldu, alpha, beta); }));
    g.R = R;
    g.f = f;
    g.u = u;
    g.ldf = ldf;
    g.ldu = ldu;
    g.alpha = alpha;
    g.beta = beta;
    g.prof = e->profiling;
    g.stream = e->stream;
    return SPME_OK;
}

int apply_impl(spme_t *e, int nrhs, double alpha, const void *f, long ldf, double beta, void *u,
               long ldu, int mem) {
    const int n = e->prm.np;
    if (nrhs < 0 || (mem != SPME_MEM_HOST && mem != SPME_MEM_DEVICE)) return SPME_ERR_INVALID;
    if (nrhs == 0 || n == 0) return SPME_OK;
    if (!f || !u || ldf < 3L * n || ldu < 3L * n) return SPME_ERR_INVALID;
    if (!e->have_pos) return SPME_ERR_STATE;
    const size_t el = e->elem, row = el * 3 * (size_t)n;
    for (int r0 = 0; r0 < nrhs; r0 += e->prm.max_nrhs) {
        const int R = std::min(e->prm.max_nrhs, nrhs - r0);
        const char *fp = (const char *)f + el * (size_t)r0 * ldf;
        char *up = (char *)u + el * (size_t)r0 * ldu;
        int st;
        if (mem == SPME_MEM_HOST) {
            // With the mesh part and 8+ right-hand sides, forces go up and the result
            // comes back in parts of rpart right-hand sides (a multiple of 4): the
            // uploads run back to back on the copy stream and each part is packed on
            // the main stream (after the position build) as it lands, and each result
            // part is copied back while the next is interpolated
            // (a direct pass: a captured graph would expose only its end; the
            // launches it saves are negligible next to a pass of this size).
            const int rpart = ((e->prm.terms & SPME_TERM_RECIP) && !e->profiling && R >= 8)
                                  ? std::max(4, (R + spme_t::kOutParts - 1) / spme_t::kOutParts + 3) / 4 * 4
                                  : 0;
            // stage the inputs on the copy stream (after the staging buffers' last
            // use), so the copy overlaps what the main stream is still running
            TRY_CUDA(cudaStreamWaitEvent(e->copy_stream, e->ev_stage_free, 0));
            if (rpart > 0) {
                for (int q0 = 0, k = 0; q0 < R; q0 += rpart, k++) {
                    const int q1 = std::min(R, q0 + rpart);
                    char *fs = (char *)e->d_fstage + row * q0;
                    TRY_CUDA(cudaMemcpy2DAsync(fs, row, fp + el * (size_t)q0 * ldf, el * ldf, row,
                                               q1 - q0, cudaMemcpyHostToDevice, e->copy_stream));
                    TRY_CUDA(cudaEventRecord(e->ev_in[k], e->copy_stream));
                }
            } else {
                TRY_CUDA(cudaMemcpy2DAsync(e->d_fstage, row, fp, el * ldf, row, R,
                                           cudaMemcpyHostToDevice, e->copy_stream));
            }
            if (beta != 0.0)
                TRY_CUDA(cudaMemcpy2DAsync(e->d_ustage, row, up, el * ldu, row, R,
                                           cudaMemcpyHostToDevice, e->copy_stream));
            TRY_CUDA(cudaEventRecord(e->ev_staged, e->copy_stream));
            if (rpart > 0) {
                for (int q0 = 0, k = 0; q0 < R; q0 += rpart, k++) {
                    const int q1 = std::min(R, q0 + rpart);
                    TRY_CUDA(cudaStreamWaitEvent(e->stream, e->ev_in[k], 0));
                    if (is_fp32(e))
                        spme::launch_pack_tiled<float>((const float *)e->d_fstage, 3L * n, n, R, q0,
                                                       q1, (float *)e->d_F, e->stream);
                    else
                        spme::launch_pack_tiled<double>((const double *)e->d_fstage, 3L * n, n, R,
                                                        q0, q1, (double *)e->d_F, e->stream);
                    e->launches++;
                }
                TRY_CUDA(cudaGetLastError());
            }
            TRY_CUDA(cudaStreamWaitEvent(e->stream, e->ev_staged, 0));
            if (rpart > 0) {
                st = pass_body(e, R, nullptr, 3L * n, e->d_ustage, 3L * n, alpha, beta, rpart);
                TRY(st);
                for (int q0 = 0, k = 0; q0 < R; q0 += rpart, k++) {
                    const int q1 = std::min(R, q0 + rpart);
                    TRY_CUDA(cudaStreamWaitEvent(e->copy_stream, e->ev_part[k], 0));
                    TRY_CUDA(cudaMemcpy2DAsync(up + el * (size_t)q0 * ldu, el * ldu,
                                               (const char *)e->d_ustage + row * q0, row, row,
                                               q1 - q0, cudaMemcpyDeviceToHost, e->copy_stream));
                }
                // the next staging waits for these copies (same stream); the main
                // stream's next pass waits for that staging
                TRY_CUDA(cudaEventRecord(e->ev_stage_free, e->copy_stream));
            } else {
                st = pass(e, R, e->d_fstage, 3L * n, e->d_ustage, 3L * n, alpha, beta);
                TRY(st);
                TRY_CUDA(cudaMemcpy2DAsync(up, el * ldu, e->d_ustage, row, row, R,
                                           cudaMemcpyDeviceToHost, e->stream));
                TRY_CUDA(cudaEventRecord(e->ev_stage_free, e->stream));
            }
        } else {
            st = pass(e, R, fp, ldf, up, ldu, alpha, beta);
            TRY(st);
        }
    }
    if (mem == SPME_MEM_HOST) {
        TRY_CUDA(cudaStreamSynchronize(e->stream));
        TRY_CUDA(cudaStreamSynchronize(e->copy_stream));
        TRY(check_device_error(e));
    }
    return SPME_OK;
}

}  // namespace

extern "C" {

void spme_params_init(spme_params *p) {
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    p->radius = 1.0;
    p->precision = SPME_FP64;
    p->max_nrhs = 1;
    p->terms = SPME_TERM_RECIP;
}

int spme_create(const spme_params *params, spme_t **out) {
    if (!params || !out) return SPME_ERR_INVALID;
    *out = nullptr;
    spme_t *e = nullptr;
    int st = create_impl(*params, &e);
    if (st != SPME_OK) {
        destroy_impl(e);
        return st;
    }
    *out = e;
    return SPME_OK;
}

int spme_destroy(spme_t *e) {
    destroy_impl(e);
    return SPME_OK;
}

void *spme_get_stream(const spme_t *e) { return e ? (void *)e->stream : nullptr; }

int spme_set_stream(spme_t *e, void *stream) {
    if (!e) return SPME_ERR_INVALID;
    DeviceGuard dg(e->device);
    use_stream(e, (cudaStream_t)stream);
    return e->last_error = SPME_OK;
}

int spme_set_positions(spme_t *e, const double *pos, int mem) {
    if (!e) return SPME_ERR_INVALID;
    if (mem != SPME_MEM_HOST && mem != SPME_MEM_DEVICE) return e->last_error = SPME_ERR_INVALID;
    DeviceGuard dg(e->device);
    return e->last_error = set_positions_impl(e, pos, mem);
}

int spme_apply(spme_t *e, int nrhs, double alpha, const void *f, long ldf, double beta, void *u,
               long ldu, int mem) {
    if (!e) return SPME_ERR_INVALID;
    DeviceGuard dg(e->device);
    return e->last_error = apply_impl(e, nrhs, alpha, f, ldf, beta, u, ldu, mem);
}

int spme_synchronize(spme_t *e) {
    if (!e) return SPME_ERR_INVALID;
    DeviceGuard dg(e->device);
    int st = from_cuda(cudaStreamSynchronize(e->stream));
    if (st == SPME_OK) st = check_device_error(e);
    return e->last_error = st;
}

int spme_set_profiling(spme_t *e, int on) {
    if (!e) return SPME_ERR_INVALID;
    e->profiling = on < 0 ? 0 : (on > 2 ? 2 : on);
    e->stages_valid = false;
    return SPME_OK;
}

int spme_stage_times(const spme_t *e, float *ms, int n) {
    if (!e || !ms || n < 0 || !e->stages_valid) return 0;
    DeviceGuard dg(e->device);
    cudaEventSynchronize(e->ev[kStages - 1]);
    float t[kStages] = {};
    // serial: ev[1] was re-recorded after the real-space sum, which starts at ev_rs[0]
    cudaEventElapsedTime(&t[0], e->ev[0], (e->ran_real && e->ran_serial) ? e->ev_rs[0] : e->ev[1]);
    if (e->ran_real) cudaEventElapsedTime(&t[1], e->ev_rs[0], e->ev_rs[1]);
    for (int k = 2; k < kStages; k++) {
        int from = k == 2 ? 1 : k - 1;
        cudaEventElapsedTime(&t[k], e->ev[from], e->ev[k]);
    }
    int m = std::min(n, kStages);
    for (int k = 0; k < m; k++) ms[k] = t[k];
    return m;
}

long spme_launch_count(const spme_t *e) { return e ? e->launches : 0; }

int spme_set_tile(spme_t *e, int tx, int ty, int tz) {
    if (!e) return SPME_ERR_INVALID;
    if (tx < 4 || ty < 4 || tz < 4 || tx > spme::kMaxTile || ty > spme::kMaxTile || tz > 8)
        return e->last_error = SPME_ERR_INVALID;
    // the interpolation kernel stages the tile plus its (p - 1) halo for at
    // least 4 components in shared memory
    MeshGeom g = e->g;
    g.tx = tx;
    g.ty = ty;
    g.tz = tz;
    if (spme::interp_smem_bytes(g, e->elem) > 220 * 1024)
        return e->last_error = SPME_ERR_UNSUPPORTED;
    e->tile[0] = tx;
    e->tile[1] = ty;
    e->tile[2] = tz;
    e->have_pos = false;
    drop_graphs(e);
    return e->last_error = SPME_OK;
}

int spme_set_overlap(spme_t *e, int on) {
    if (!e) return SPME_ERR_INVALID;
    DeviceGuard dg(e->device);
    if (e->stream) cudaStreamSynchronize(e->stream);
    drop_graphs(e);
    e->overlap = on ? 1 : 0;
    return e->last_error = SPME_OK;
}

int spme_set_spread_mode(spme_t *e, int mode) {
    if (!e || (mode != 0 && mode != 1)) return SPME_ERR_INVALID;
    DeviceGuard dg(e->device);
    if (mode == 1 && !e->cols) return e->last_error = SPME_ERR_UNSUPPORTED;
    if (e->stream) cudaStreamSynchronize(e->stream);
    drop_graphs(e);
    e->spread_mode = mode;
    return e->last_error = SPME_OK;
}

int spme_set_fft_mode(spme_t *e, int mode) {
    if (!e || mode < 0 || mode > 2) return SPME_ERR_INVALID;
    DeviceGuard dg(e->device);
    if (mode >= 1 && !e->d_ztw) return e->last_error = SPME_ERR_UNSUPPORTED;
    if (mode == 2 && !e->d_f2tab) return e->last_error = SPME_ERR_UNSUPPORTED;
    if (e->stream) cudaStreamSynchronize(e->stream);
    drop_graphs(e);
    if (mode == 1) {
        for (PlanPair &p : e->plans) {
            cufftDestroy(p.fwd);
            cufftDestroy(p.bwd);
            if (p.has2d) {
                cufftDestroy(p.fwd2);
                cufftDestroy(p.bwd2);
            }
        }
        e->plans.clear();  // rebuilt with their 2D companions on the next pass
    }
    e->fft_mode = mode;
    return e->last_error = SPME_OK;
}

int spme_set_graphs(spme_t *e, int on) {
    if (!e) return SPME_ERR_INVALID;
    DeviceGuard dg(e->device);
    if (e->stream) cudaStreamSynchronize(e->stream);
    drop_graphs(e);
    e->use_graphs = on != 0;
    return e->last_error = SPME_OK;
}

int spme_last_error(const spme_t *e) { return e ? e->last_error : SPME_ERR_INVALID; }

const char *spme_error_string(int code) {
    switch (code) {
        case SPME_OK: return "success";
        case SPME_ERR_INVALID: return "invalid argument";
        case SPME_ERR_UNSUPPORTED: return "unsupported parameters";
        case SPME_ERR_CUDA: return "CUDA runtime error";
        case SPME_ERR_CUFFT: return "cuFFT error";
        case SPME_ERR_NOMEM: return "out of memory";
        case SPME_ERR_STATE: return "engine state error (positions not set)";
        case SPME_ERR_KERNEL: return "device-side check failed";
        case SPME_ERR_TOO_LARGE:
            return "request exceeds the fixed scratch of the allocation-free entry point "
                   "(np <= SPME_NOALLOC_MAX_NP, nrhs <= SPME_NOALLOC_MAX_NRHS)";
        default: return "unknown error";
    }
}

// ---- drop-in entry points (old-version/spme.h:85-97) ----------------------

void cutoff2xi(double rmax, double ewald_eps, double box_size, double *_xi) {
    (void)box_size;
    if (!_xi) return;
    if (!(rmax > 0.0) || !(ewald_eps > 0.0 && ewald_eps < 1.0)) {
        *_xi = 0.0;
        return;
    }
    *_xi = std::sqrt(-std::log(ewald_eps)) / rmax;
}

void create_spme_engine(double xi, int dim, int porder, int np, double box_size, int nthreads,
                        spme_t **_spme) {
    (void)nthreads;
    if (!_spme) return;
    spme_params p;
    spme_params_init(&p);
    p.np = np;
    p.dim = dim;
    p.porder = porder;
    p.box_size = box_size;
    p.xi = xi;
    spme_create(&p, _spme);
}

void destroy_spme_engine(spme_t *spme) { spme_destroy(spme); }

void compute_spme(spme_t *spme, double *pos, int nrhs, double alpha, double *vec_in, int ldin,
                  double beta, double *vec_out, int ldout) {
    if (!spme) return;
    if (pos) {
        if (spme_set_positions(spme, pos, SPME_MEM_HOST) != SPME_OK) return;
    }
    spme_apply(spme, nrhs, alpha, vec_in, ldin, beta, vec_out, ldout, SPME_MEM_HOST);
}

}  // extern "C"
