// pme — command-line driver with the reference driver's semantics
// (billy-inn/SPME old-version/main.c:130-260): read an .xyz particle file
// (--xyz, main.c:46-127, positions wrapped into [0, L)), build an engine for
// mesh --dim and order --porder, and apply v = alpha M f + beta v with the
// reference's alpha = 2.1, beta = 2.2 (main.c:224-225).  It links only the C
// ABI of libspme_gb300.so.
//
// Reference options: -h/--help, -v/--version, --xyz FILE, --dim K, --porder p
// (defaults input.xyz, 64, 4; xi = 0.5, main.c:153-156,210).  The driver keeps
// the reference's "dim must be larger than 4 * porder" check (main.c:205-209).
// Extensions: --xi X, --tol T (suggest xi/K/p for a target error), --full
// (real space + self + reciprocal with --rc/--radius), --precision fp64|fp32,
// --nrhs R, --seed S, --synthetic N,L (uniform particles instead of --xyz),
// --write-xyz FILE, --out PREFIX (writes PREFIX.f, PREFIX.v0 and PREFIX.v: forces,
// initial and final velocities, one value per line), --reps N, --no-dim-check.
//
// Forces and initial velocities are N(0, 1) from a seeded generator (the
// reference's rand()*3.0 values, main.c:231-236, depend on the C library).
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "spme_gb300.h"

namespace {

const char *kVersion = "0.1.0";

void usage(const char *call) {
    std::fprintf(stderr,
                 "Usage: %s [OPTIONS]\n"
                 "Options:\n"
                 "\t-h or --help         Display this information\n"
                 "\t-v or --version      Display version information\n"
                 "\t--dim                nfft grids\n"
                 "\t--porder             interpolation order\n"
                 "\t--xyz                xyz file\n"
                 "\t--xi X --tol T --full --rc R --radius A --precision fp64|fp32\n"
                 "\t--nrhs R --seed S --synthetic N,L --write-xyz F --out F --reps N\n"
                 "\t--no-dim-check\n",
                 call);
}

// splitmix64 + Box-Muller: portable seeded N(0,1)
struct Rng {
    uint64_t s;
    explicit Rng(uint64_t seed) : s(seed) {}
    uint64_t next() {
        uint64_t z = (s += 0x9e3779b97f4a7c15ULL);
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
        return z ^ (z >> 31);
    }
    double uniform() { return ((next() >> 11) + 0.5) * (1.0 / 9007199254740992.0); }
    double normal() {
        double u1 = uniform(), u2 = uniform();
        return std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * M_PI * u2);
    }
};

bool arg(int &i, int argc, char **argv, const char *name, const char **val) {
    if (std::strcmp(argv[i], name) != 0) return false;
    if (i + 1 >= argc) {
        std::fprintf(stderr, "Option %s requires an argument.\n", name);
        std::exit(2);
    }
    *val = argv[++i];
    return true;
}

}  // namespace

int main(int argc, char **argv) {
    std::string xyz = "input.xyz", out_path, write_xyz;
    int dim = 64, porder = 4, nrhs = 1, reps = 1, np = 0;
    double xi = 0.5, tol = 0.0, rc = 10.0, radius = 1.0, L = 0.0;
    bool full = false, fp32 = false, dim_check = true, synthetic = false, xi_set = false;
    uint64_t seed = 1234;
    for (int i = 1; i < argc; i++) {
        const char *v = nullptr;
        if (!std::strcmp(argv[i], "-h") || !std::strcmp(argv[i], "--help")) {
            usage(argv[0]);
            return 0;
        } else if (!std::strcmp(argv[i], "-v") || !std::strcmp(argv[i], "--version")) {
            std::printf("%s version %s\n", argv[0], kVersion);
            return 0;
        } else if (arg(i, argc, argv, "--xyz", &v)) {
            xyz = v;
        } else if (arg(i, argc, argv, "--dim", &v)) {
            dim = std::atoi(v);
        } else if (arg(i, argc, argv, "--porder", &v)) {
            porder = std::atoi(v);
        } else if (arg(i, argc, argv, "--xi", &v)) {
            xi = std::atof(v);
            xi_set = true;
        } else if (arg(i, argc, argv, "--tol", &v)) {
            tol = std::atof(v);
        } else if (arg(i, argc, argv, "--rc", &v)) {
            rc = std::atof(v);
        } else if (arg(i, argc, argv, "--radius", &v)) {
            radius = std::atof(v);
        } else if (arg(i, argc, argv, "--precision", &v)) {
            fp32 = !std::strcmp(v, "fp32");
        } else if (arg(i, argc, argv, "--nrhs", &v)) {
            nrhs = std::atoi(v);
        } else if (arg(i, argc, argv, "--seed", &v)) {
            seed = std::strtoull(v, nullptr, 10);
        } else if (arg(i, argc, argv, "--synthetic", &v)) {
            synthetic = std::sscanf(v, "%d,%lf", &np, &L) == 2;
        } else if (arg(i, argc, argv, "--write-xyz", &v)) {
            write_xyz = v;
        } else if (arg(i, argc, argv, "--out", &v)) {
            out_path = v;
        } else if (arg(i, argc, argv, "--reps", &v)) {
            reps = std::atoi(v);
        } else if (!std::strcmp(argv[i], "--full")) {
            full = true;
        } else if (!std::strcmp(argv[i], "--no-dim-check")) {
            dim_check = false;
        } else {
            std::fprintf(stderr, "Unknown option `%s'.\n", argv[i]);
            usage(argv[0]);
            return 2;
        }
    }
    if (dim <= 0 || porder <= 0 || nrhs <= 0 || reps <= 0) {
        usage(argv[0]);
        return 2;
    }

    std::vector<double> pos;
    if (synthetic) {
        if (np <= 0 || !(L > 0.0)) {
            std::fprintf(stderr, "--synthetic wants N,L with N > 0 and L > 0\n");
            return 2;
        }
        Rng r(seed ^ 0x5eedULL);
        pos.resize((size_t)3 * np);
        for (double &x : pos) x = r.uniform() * L;
    } else {
        double *p = nullptr;
        if (spme_read_xyz(xyz.c_str(), &np, &L, &p, nullptr) != SPME_OK) {
            std::fprintf(stderr, "Can not read particles from %s\n", xyz.c_str());
            return 1;
        }
        pos.assign(p, p + (size_t)3 * np);
        spme_free(p);
    }
    std::printf("imported %d particles, L = %lf\n", np, L);
    if (!write_xyz.empty() && spme_write_xyz(write_xyz.c_str(), np, L, pos.data(), radius) != 0)
        std::fprintf(stderr, "could not write %s\n", write_xyz.c_str());

    if (tol > 0.0) {
        spme_params s;
        if (spme_suggest_params(np, L, radius, tol, full ? rc : 0.0, &s) != SPME_OK) {
            std::fprintf(stderr, "no parameters for tol %g\n", tol);
            return 1;
        }
        if (!xi_set) xi = s.xi;
        dim = s.dim;
        porder = s.porder;
        rc = s.rcut;
    }
    if (dim_check && 4 * porder >= dim) {
        std::fprintf(stderr, "dim must be larger than 4 * porder\n");
        return 1;
    }
    std::printf("SPME: xi = %lf, dim = %d, porder = %d%s\n", xi, dim, porder,
                full ? " (real space + self + reciprocal)" : "");

    const double alpha = 2.1, beta = 2.2;  // old-version/main.c:224-225
    const long ld = 3L * np;
    Rng r(seed);
    std::vector<double> f((size_t)ld * nrhs), v((size_t)ld * nrhs);
    for (size_t i = 0; i < f.size(); i++) {
        f[i] = r.normal();
        v[i] = r.normal();
    }
    const std::vector<double> v0 = v;

    int st = SPME_OK;
    spme_t *h = nullptr;
    const bool dropin = !full && !fp32;
    if (dropin) {
        create_spme_engine(xi, dim, porder, np, L, 1, &h);
        if (!h) st = SPME_ERR_INVALID;
    } else {
        spme_params p;
        spme_params_init(&p);
        p.np = np;
        p.dim = dim;
        p.porder = porder;
        p.box_size = L;
        p.xi = xi;
        p.radius = radius;
        p.rcut = rc;
        p.precision = fp32 ? SPME_FP32 : SPME_FP64;
        p.max_nrhs = nrhs;
        p.terms = full ? SPME_TERM_ALL : SPME_TERM_RECIP;
        st = spme_create(&p, &h);
    }
    if (st != SPME_OK) {
        std::fprintf(stderr, "engine creation failed: %s\n", spme_error_string(st));
        return 1;
    }
    std::vector<float> f32, v32;
    if (fp32) {
        f32.assign(f.begin(), f.end());
        v32.assign(v.begin(), v.end());
    }
    double best = 1e300;
    for (int rep = 0; rep < reps; rep++) {
        if (fp32) v32.assign(v.begin(), v.end());
        std::vector<double> vv = v;
        auto t0 = std::chrono::steady_clock::now();
        if (dropin) {
            compute_spme(h, pos.data(), nrhs, alpha, f.data(), (int)ld, beta, vv.data(), (int)ld);
            st = spme_last_error(h);
        } else {
            st = spme_set_positions(h, pos.data(), SPME_MEM_HOST);
            if (st == SPME_OK)
                st = fp32 ? spme_apply(h, nrhs, alpha, f32.data(), ld, beta, v32.data(), ld,
                                       SPME_MEM_HOST)
                          : spme_apply(h, nrhs, alpha, f.data(), ld, beta, vv.data(), ld,
                                       SPME_MEM_HOST);
        }
        auto t1 = std::chrono::steady_clock::now();
        if (st != SPME_OK) break;
        best = std::fmin(best, std::chrono::duration<double>(t1 - t0).count());
        if (rep == reps - 1) {
            if (fp32) vv.assign(v32.begin(), v32.end());
            v.swap(vv);
        }
    }
    if (st != SPME_OK) {
        std::fprintf(stderr, "compute failed: %s\n", spme_error_string(st));
        destroy_spme_engine(h);
        return 1;
    }
    double nrm = 0.0;
    for (double x : v) nrm += x * x;
    std::printf("    totally takes %.3le secs (best of %d), %.3lf ns/particle/rhs, |v| = %.17g\n",
                best, reps, best * 1e9 / ((double)np * nrhs), std::sqrt(nrm));
    if (!out_path.empty()) {
        const std::vector<double> *arrs[3] = {&f, &v0, &v};
        const char *ext[3] = {".f", ".v0", ".v"};
        for (int k = 0; k < 3; k++) {
            FILE *fp = std::fopen((out_path + ext[k]).c_str(), "w");
            if (!fp) {
                std::fprintf(stderr, "could not write %s%s\n", out_path.c_str(), ext[k]);
                continue;
            }
            for (double x : *arrs[k]) std::fprintf(fp, "%.17g\n", x);
            std::fclose(fp);
        }
    }
    destroy_spme_engine(h);
    return 0;
}
