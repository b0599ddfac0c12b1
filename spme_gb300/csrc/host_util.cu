// Host-side utilities around the operator: Ewald parameter selection from a
// target error and the reference driver's .xyz particle format.
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "spme_gb300.h"

namespace {

bool smooth235(int n) {
    for (int f : {2, 3, 5})
        while (n % f == 0) n /= f;
    return n == 1;
}

// Root of g(x) = tol for a decreasing g on [lo, hi] (bisection).
template <typename G>
double solve_decreasing(G g, double tol, double lo, double hi) {
    for (int it = 0; it < 200; it++) {
        double mid = 0.5 * (lo + hi);
        if (g(mid) > tol) lo = mid;
        else hi = mid;
    }
    return hi;
}

}  // namespace

extern "C" {

int spme_next_smooth(int n) {
    if (n < 2) n = 2;
    while (!smooth235(n)) n++;
    return n;
}

// Parameters for a target relative error `tol` of the Ewald-split mobility,
// from error models fitted to the oracle (the tails carry polynomial
// prefactors, so the bare Gaussians exp(-xi^2 rc^2), exp(-k^2/4xi^2)
// underestimate the error by one to two orders):
//   real space   exp(-x^2) (1 + x^4/3) = tol,  x = xi rc          -> xi
//   k-space tail exp(-y) (1 + y + 2 y^2) = tol, y = k_max^2/4xi^2 -> K >= k_max L / pi
//   B-splines    xi L / K <= c_p tol^(1/p), c_4 = 1.8, c_6 = 1.2, c_8 = 1.1
//   p = 4 for tol >= 1e-3, 6 for tol >= 1e-6, else 8;  K the next 2^a 3^b 5^c.
// rcut <= 0 picks rc = min(10 a, 0.49 L).  Fills *out (spme_params_init
// defaults for the other fields, all terms).
int spme_suggest_params(int np, double box_size, double radius, double tol, double rcut,
                        spme_params *out) {
    if (!out || np < 0 || !(box_size > 0.0) || !(radius > 0.0) || !(tol > 0.0 && tol < 1.0))
        return SPME_ERR_INVALID;
    double rc = rcut > 0.0 ? rcut : std::fmin(10.0 * radius, 0.49 * box_size);
    if (!(rc < 0.5 * box_size)) return SPME_ERR_INVALID;
    const double x = solve_decreasing(
        [](double v) { return std::exp(-v * v) * (1.0 + v * v * v * v / 3.0); }, tol, 1.0, 30.0);
    const double xi = x / rc;
    const double y = solve_decreasing(
        [](double v) { return std::exp(-v) * (1.0 + v + 2.0 * v * v); }, tol, 1.0, 400.0);
    const double kmax = 2.0 * xi * std::sqrt(y);
    const int p = tol >= 1e-3 ? 4 : (tol >= 1e-6 ? 6 : 8);
    const double cp = p == 4 ? 1.8 : (p == 6 ? 1.2 : 1.1);
    const double k_trunc = kmax * box_size / M_PI;
    const double k_interp = xi * box_size / (cp * std::pow(tol, 1.0 / p));
    int K = (int)std::ceil(std::fmax(k_trunc, k_interp));
    if (K < 2 * p) K = 2 * p;
    K = spme_next_smooth(K);
    if (K > 1024) return SPME_ERR_UNSUPPORTED;
    spme_params_init(out);
    out->np = np;
    out->dim = K;
    out->porder = p;
    out->box_size = box_size;
    out->xi = xi;
    out->radius = radius;
    out->rcut = rc;
    out->terms = SPME_TERM_ALL;
    return SPME_OK;
}

// .xyz as read by the reference driver (old-version/main.c:46-127): '#' lines
// are comments; the first other line is "np L"; then one line per particle
// "name x y z a".  Positions are wrapped into [0, L) (main.c:107-121).
// Returns SPME_OK and fills np / L / pos (malloc'd, caller frees with free()) and
// optionally radii (may be NULL).
int spme_read_xyz(const char *path, int *np, double *box_size, double **pos, double **radii) {
    if (!path || !np || !box_size || !pos) return SPME_ERR_INVALID;
    FILE *fp = std::fopen(path, "r");
    if (!fp) return SPME_ERR_INVALID;
    char line[1024];
    int n = 0;
    double L = 0.0;
    bool header = false;
    while (std::fgets(line, sizeof line, fp)) {
        char tok[128];
        if (std::sscanf(line, "%127s", tok) != 1 || tok[0] == '#') continue;
        if (std::sscanf(line, "%d %lf", &n, &L) == 2) header = true;
        break;
    }
    if (!header || n <= 0 || !(L > 0.0)) {
        std::fclose(fp);
        return SPME_ERR_INVALID;
    }
    std::vector<double> p;
    std::vector<double> a;
    p.reserve((size_t)3 * n);
    while (std::fgets(line, sizeof line, fp)) {
        char tok[128];
        double x, y, z, r = 1.0;
        if (std::sscanf(line, "%127s", tok) != 1 || tok[0] == '#') continue;
        int got = std::sscanf(line, "%127s %lf %lf %lf %lf", tok, &x, &y, &z, &r);
        if (got < 4) continue;
        p.push_back(x);
        p.push_back(y);
        p.push_back(z);
        a.push_back(got >= 5 ? r : 1.0);
    }
    std::fclose(fp);
    if ((int)a.size() != n) return SPME_ERR_INVALID;
    double *out = (double *)std::malloc(sizeof(double) * 3 * (size_t)n);
    if (!out) return SPME_ERR_NOMEM;
    for (size_t i = 0; i < p.size(); i++) {
        double v = std::fmod(p[i], L);
        out[i] = v >= 0.0 ? v : L + v;
    }
    *pos = out;
    if (radii) {
        double *ra = (double *)std::malloc(sizeof(double) * (size_t)n);
        if (!ra) {
            std::free(out);
            *pos = nullptr;
            return SPME_ERR_NOMEM;
        }
        std::memcpy(ra, a.data(), sizeof(double) * (size_t)n);
        *radii = ra;
    }
    *np = n;
    *box_size = L;
    return SPME_OK;
}

// Writes the same format (radius column = `radius` for every particle).
int spme_write_xyz(const char *path, int np, double box_size, const double *pos, double radius) {
    if (!path || np < 0 || (np > 0 && !pos)) return SPME_ERR_INVALID;
    FILE *fp = std::fopen(path, "w");
    if (!fp) return SPME_ERR_INVALID;
    std::fprintf(fp, "# spme_gb300 particle file: np L, then name x y z a\n%d %.17g\n", np,
                 box_size);
    for (int i = 0; i < np; i++)
        std::fprintf(fp, "P %.17g %.17g %.17g %.17g\n", pos[3 * i], pos[3 * i + 1],
                     pos[3 * i + 2], radius);
    std::fclose(fp);
    return SPME_OK;
}

void spme_free(void *p) { std::free(p); }

}  // extern "C"
