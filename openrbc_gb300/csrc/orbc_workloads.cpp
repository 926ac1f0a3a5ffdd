// Synthetic workload generators (host code): see include/orbc_workloads.h.
#include "orbc_workloads.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <tuple>
#include <vector>

#include "orbc_gen_util.h"

using namespace orbc_gen;


extern "C" {

int orbc_gen_lattice(int64_t n, int ncol, double spacing, double jitter, double tilt, double kT, uint64_t seed,
                     double *x3, double *n3, double *v3, double *o3, int *type, int *tag) {
    if (n < 1 || ncol < 1 || !x3 || !n3 || !v3 || !o3 || !type || !tag) return 1;
    Stream rs(seed, 1);
    for (int64_t k = 0; k < n; ++k) {
        const int64_t col = k % ncol, row = k / ncol;
        x3[3 * k] = col * spacing + jitter * rs.gauss();
        x3[3 * k + 1] = row * spacing + jitter * rs.gauss();
        x3[3 * k + 2] = jitter * rs.gauss();
        tilt_normal(rs, tilt, &n3[3 * k]);
        const double sv = std::sqrt(kT / kMass[0]);
        for (int d = 0; d < 3; ++d) {
            v3[3 * k + d] = sv * rs.gauss();
            o3[3 * k + d] = 0.0;
        }
        type[k] = 0;
        tag[k] = int(k + 1);
    }
    return 0;
}

int orbc_gen_vesicle_sizes(int nves, int64_t nmin, int64_t nmax, int64_t median, int64_t total, uint64_t seed,
                           int64_t *sizes) {
    if (nves < 1 || nmin < 1 || nmax < nmin || !sizes) return 1;
    Stream rs(seed, 4);
    std::vector<double> z(static_cast<size_t>(nves));
    for (int k = 0; k < nves; ++k) z[size_t(k)] = rs.gauss();
    const double mu = std::log(double(median));
    auto sum_for = [&](double sg) {
        double s = 0;
        for (int k = 0; k < nves; ++k)
            s += std::min(double(nmax), std::max(double(nmin), std::exp(mu + sg * z[size_t(k)])));
        return s;
    };
    double lo = 0.0, hi = 3.0;
    for (int it = 0; it < 100; ++it) {
        const double mid = 0.5 * (lo + hi);
        if (sum_for(mid) < double(total)) lo = mid; else hi = mid;
    }
    const double sg = 0.5 * (lo + hi);
    for (int k = 0; k < nves; ++k)
        sizes[k] = int64_t(std::llround(std::min(double(nmax), std::max(double(nmin), std::exp(mu + sg * z[size_t(k)])))));
    return 0;
}

int orbc_gen_vesicle(int64_t n, double rho, double kT, uint64_t seed, int tag0, double *x3, double *n3, double *v3,
                     double *o3, int *type, int *tag, double *radius) {
    if (n < 1 || !(rho > 0) || !x3 || !n3 || !v3 || !o3 || !type || !tag) return 1;
    const double R = std::sqrt(double(n) / (4.0 * M_PI * rho));
    if (radius) *radius = R;
    Stream rs(seed, 5);
    PointHash ph(1.0, size_t(n));
    int64_t k = 0, tries = 0;
    while (k < n) {
        const double u = 2.0 * rs.u01() - 1.0, th = 2.0 * M_PI * rs.u01();
        const double s = std::sqrt(std::max(0.0, 1.0 - u * u));
        const double p[3] = {R * s * std::cos(th), R * s * std::sin(th), R * u};
        if (++tries > 1000 * n) return 2;
        if (ph.near(p, 0.55)) continue;
        ph.insert(p);
        for (int d = 0; d < 3; ++d) {
            x3[3 * k + d] = p[d];
            n3[3 * k + d] = p[d] / R;
            v3[3 * k + d] = std::sqrt(kT / kMass[0]) * rs.gauss();
            o3[3 * k + d] = 0.0;
        }
        type[k] = 0;
        tag[k] = int(tag0 + k);
        ++k;
    }
    return 0;
}

}  // extern "C"
