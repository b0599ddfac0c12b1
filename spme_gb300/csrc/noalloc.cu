// Allocation-free real-space + self mobility apply.
//
// Some callers cannot call cudaMalloc: applications that reserve all device
// memory up front in their own pool, and time-stepping loops that must not
// stall, where cudaMalloc/cudaFree can synchronise the whole device.  This
// entry point runs the real-space Ewald RPY sum and the self term
// (realspace.cu, cell-list build of pbuild.cu) with all of its scratch in one
// file-scope device array of fixed size, so it allocates nothing.
//
// Limits (also in include/spme_gb300.h): np <= SPME_NOALLOC_MAX_NP, nrhs <=
// SPME_NOALLOC_MAX_NRHS, at most kMaxCells real-space cells (the cell count is
// capped, which only makes cells larger).
//
// When the array takes device memory: CUDA loads this file's module on a
// device lazily (the default module loading), at the first use of one of its
// kernels or symbols there, and the array (kScratchBytes) is allocated then
// and held until the process exits.  The first call on each device, a
// zero-size one included, looks up the array's address with that device
// current and so loads the module: a caller that reserves all remaining device
// memory for its own pool makes one call (np = 0 is enough) before doing so,
// and before any stream capture.  The address is kept per device for the
// process; resetting a device (cudaDeviceReset) after that first call is not
// supported.
//
// Every call shares the one array, which keeps the previous call's contents:
// the cell counts are cleared at the start of each call, everything else is
// overwritten before it is read.  Calls whose work overlaps on the GPU (two
// streams, or two host threads) race on the array and give wrong results;
// serialise them.
//
// Errors: a pending error from the caller's earlier, unrelated launches is
// cleared on entry (cudaGetLastError), so the status returned describes this
// call's own work only.

#include "kernels.h"
#include "spme_gb300.h"

namespace {

constexpr size_t kMaxNp = SPME_NOALLOC_MAX_NP;
constexpr size_t kMaxC = 3 * SPME_NOALLOC_MAX_NRHS;
constexpr int kMaxNc = 32;
constexpr size_t kMaxCells = (size_t)kMaxNc * kMaxNc * kMaxNc;

constexpr size_t align256(size_t b) { return (b + 255) / 256 * 256; }

// scratch carve-up (bytes)
constexpr size_t kOffKey = 0;
constexpr size_t kOffSlot = kOffKey + align256(sizeof(int) * kMaxNp);
constexpr size_t kOffPerm = kOffSlot + align256(sizeof(int) * kMaxNp);
constexpr size_t kOffCpos = kOffPerm + align256(sizeof(int) * kMaxNp);
constexpr size_t kOffF = kOffCpos + align256(sizeof(double4_32a) * kMaxNp);
constexpr size_t kOffW = kOffF + align256(sizeof(double) * kMaxC * kMaxNp);
constexpr size_t kOffCount = kOffW + align256(sizeof(double) * kMaxC * kMaxNp);
constexpr size_t kOffOff = kOffCount + align256(sizeof(int) * kMaxCells);
constexpr size_t kOffTmp = kOffOff + align256(sizeof(int) * (kMaxCells + 1));
constexpr size_t kScratchBytes = kOffTmp + align256(sizeof(int) * (kMaxCells / 2048 + 2));

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// Device address of the scratch array on the current device (in host code the
// array's name is only a host-side stand-in).  Looked up on every call: cheap
// once the module is loaded, legal during stream capture, and never stale
// after a device reset reloads the module at another address.
int scratch_address(unsigned char **out) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
        cudaGetLastError();
        return SPME_ERR_CUDA;
    }
    *out = static_cast<unsigned char *>(p);
    return SPME_OK;
}

}  // namespace

extern "C" int spme_realspace_apply_noalloc(int np, const double *pos, double box_size,
                                            double xi, double radius, double rcut, int nrhs,
                                            double alpha, const double *f, long ldf,
                                            double beta, double *u, long ldu, void *stream) {
    if (np < 0 || nrhs < 0 || !(box_size > 0.0) || !(xi > 0.0) || !(radius > 0.0) ||
        !(rcut > 0.0 && rcut < 0.5 * box_size))
        return SPME_ERR_INVALID;
    if ((size_t)np > kMaxNp || nrhs > SPME_NOALLOC_MAX_NRHS) return SPME_ERR_TOO_LARGE;
    // an error left pending by the caller's earlier launches is not this call's
    cudaGetLastError();
    // before the zero-size return: a zero-size first call loads the module (and
    // with it the scratch array) on this device
    unsigned char *base = nullptr;
    int st = scratch_address(&base);
    if (st != SPME_OK) return st;
    if (np == 0 || nrhs == 0) return SPME_OK;
    if (!pos || !f || !u || ldf < 3L * np || ldu < 3L * np) return SPME_ERR_INVALID;
    cudaStream_t s = static_cast<cudaStream_t>(stream);

    // cells of edge >= rc, at most kMaxNc per axis (fewer than 3 -> one cell)
    long nc = (long)(box_size / rcut);
    if (nc > kMaxNc) nc = kMaxNc;
    if (nc < 3) nc = 1;
    const int ncell = (int)(nc * nc * nc);

    int *key = reinterpret_cast<int *>(base + kOffKey);
    int *slot = reinterpret_cast<int *>(base + kOffSlot);
    int *perm = reinterpret_cast<int *>(base + kOffPerm);
    double4_32a *cpos = reinterpret_cast<double4_32a *>(base + kOffCpos);
    double *F = reinterpret_cast<double *>(base + kOffF);
    double *W = reinterpret_cast<double *>(base + kOffW);
    int *count = reinterpret_cast<int *>(base + kOffCount);
    int *off = reinterpret_cast<int *>(base + kOffOff);
    int *tmp = reinterpret_cast<int *>(base + kOffTmp);

    if (cudaMemsetAsync(count, 0, sizeof(int) * ncell, s) != cudaSuccess) {
        cudaGetLastError();
        return SPME_ERR_CUDA;
    }
    spme::launch_cell_keys(pos, np, box_size, (int)nc, key, count, perm, s);
    spme::launch_scan(count, ncell, off, tmp, s);
    spme::launch_scatter(key, off, np, perm, slot, s);
    spme::launch_cell_positions(pos, perm, np, box_size, (int)nc, false, cpos, s);
    spme::launch_pack<double>(f, ldf, np, nrhs, F, s);
    if (spme::launch_realspace<double>((int)nc, off, perm, cpos, F, nrhs, box_size, rcut, xi,
                                       radius, 1, W, s) != cudaSuccess)
        return SPME_ERR_CUDA;
    spme::launch_unpack<double>(W, np, nrhs, alpha, beta, u, ldu, s);
    return cudaGetLastError() == cudaSuccess ? SPME_OK : SPME_ERR_CUDA;
}
