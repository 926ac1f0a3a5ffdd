// Whole red-cell membrane generator (see include/orbc_workloads.h): an
// Evans-Fung biconcave surface (Evans & Fung, Microvasc. Res. 4, 1972:
// z(r) = +-R/2 sqrt(1 - (r/R)^2) (C0 + C2 (r/R)^2 + C4 (r/R)^4)), lipids placed
// uniformly by area, and a geodesic-icosahedron spectrin mesh mapped onto it.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <tuple>
#include <vector>

#include "orbc_gen_util.h"
#include "orbc_workloads.h"

using namespace orbc_gen;

namespace {

constexpr double C0 = 0.207161, C2 = 2.002558, C4 = -1.122762;

/* Upper half of the profile, parametrised by t in [0, pi/2]:
 * r = R sin t, z = R/2 cos t (C0 + C2 sin^2 t + C4 sin^4 t). */
struct Profile {
    static constexpr int K = 200001;
    double R;
    std::vector<double> t, cum;  // cumulative area of the upper half from the pole
    explicit Profile(double R_) : R(R_), t(K), cum(K) {
        double prev = 0;
        for (int k = 0; k < K; ++k) {
            t[size_t(k)] = 0.5 * M_PI * k / (K - 1);
            if (k == 0) {
                cum[0] = 0;
            } else {
                const double tm = 0.5 * (t[size_t(k)] + t[size_t(k - 1)]);
                double r, z, dr, dz;
                eval(tm, r, z, dr, dz);
                const double ds = std::sqrt(dr * dr + dz * dz) * (t[size_t(k)] - t[size_t(k - 1)]);
                prev += 2.0 * M_PI * r * ds;
                cum[size_t(k)] = prev;
            }
        }
    }
    void eval(double tt, double &r, double &z, double &dr, double &dz) const {
        const double s = std::sin(tt), c = std::cos(tt), s2 = s * s;
        const double poly = C0 + C2 * s2 + C4 * s2 * s2;
        r = R * s;
        z = 0.5 * R * c * poly;
        dr = R * c;
        dz = 0.5 * R * (-s * poly + c * (2.0 * C2 * s * c + 4.0 * C4 * s2 * s * c));
    }
    double upper_area() const { return cum.back(); }
    /* parameter t at which the area from the pole is frac * upper_area */
    double t_of(double frac) const {
        const double target = frac * cum.back();
        auto it = std::lower_bound(cum.begin(), cum.end(), target);
        size_t k = size_t(it - cum.begin());
        if (k == 0) return 0.0;
        if (k >= cum.size()) return t.back();
        const double a0 = cum[k - 1], a1 = cum[k];
        const double w = a1 > a0 ? (target - a0) / (a1 - a0) : 0.0;
        return t[k - 1] + w * (t[k] - t[k - 1]);
    }
    /* point and outward normal; lower = mirror image below z = 0 */
    void point(double tt, double phi, bool lower, double *p, double *n) const {
        double r, z, dr, dz;
        eval(tt, r, z, dr, dz);
        double nr = -dz, nz = dr;
        const double nn = std::sqrt(nr * nr + nz * nz);
        nr /= nn;
        nz /= nn;
        if (tt == 0.0) {
            nr = 0;
            nz = 1;
        }
        const double cp = std::cos(phi), sp = std::sin(phi);
        p[0] = r * cp;
        p[1] = r * sp;
        p[2] = lower ? -z : z;
        n[0] = nr * cp;
        n[1] = nr * sp;
        n[2] = lower ? -nz : nz;
    }
};

/* Geodesic icosahedron of frequency F (class I): 10 F^2 + 2 unit vectors,
 * 20 F^2 faces counter-clockwise seen from outside. */
void geodesic(int F, std::vector<double> &V, std::vector<int> &T) {
    const double g = (1 + std::sqrt(5.0)) / 2;
    double ico[12][3] = {{-1, g, 0}, {1, g, 0}, {-1, -g, 0}, {1, -g, 0}, {0, -1, g}, {0, 1, g},
                         {0, -1, -g}, {0, 1, -g}, {g, 0, -1}, {g, 0, 1}, {-g, 0, -1}, {-g, 0, 1}};
    int fc[20][3] = {{0, 11, 5}, {0, 5, 1}, {0, 1, 7}, {0, 7, 10}, {0, 10, 11}, {1, 5, 9}, {5, 11, 4},
                     {11, 10, 2}, {10, 7, 6}, {7, 1, 8}, {3, 9, 4}, {3, 4, 2}, {3, 2, 6}, {3, 6, 8},
                     {3, 8, 9}, {4, 9, 5}, {2, 4, 11}, {6, 2, 10}, {8, 6, 7}, {9, 8, 1}};
    for (auto &f : fc) {  // orient counter-clockwise from outside
        const double *a = ico[f[0]], *b = ico[f[1]], *c = ico[f[2]];
        const double u[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]}, w[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
        const double nx = u[1] * w[2] - u[2] * w[1], ny = u[2] * w[0] - u[0] * w[2], nz = u[0] * w[1] - u[1] * w[0];
        if (nx * (a[0] + b[0] + c[0]) + ny * (a[1] + b[1] + c[1]) + nz * (a[2] + b[2] + c[2]) < 0) std::swap(f[1], f[2]);
    }
    std::map<std::tuple<long long, long long, long long>, int> index;
    V.clear();
    T.clear();
    auto vid = [&](const double *p) {
        const double nn = std::sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
        const double q[3] = {p[0] / nn, p[1] / nn, p[2] / nn};
        const auto key = std::make_tuple(std::llround(q[0] * 1e9), std::llround(q[1] * 1e9), std::llround(q[2] * 1e9));
        auto it = index.find(key);
        if (it != index.end()) return it->second;
        const int id = int(V.size() / 3);
        V.insert(V.end(), q, q + 3);
        index.emplace(key, id);
        return id;
    };
    std::vector<int> grid(size_t((F + 1) * (F + 1)));
    for (auto &f : fc) {
        const double *A = ico[f[0]], *B = ico[f[1]], *Cc = ico[f[2]];
        for (int i = 0; i <= F; ++i)
            for (int j = 0; i + j <= F; ++j) {
                double p[3];
                for (int d = 0; d < 3; ++d) p[d] = A[d] + (B[d] - A[d]) * i / F + (Cc[d] - A[d]) * j / F;
                grid[size_t(i * (F + 1) + j)] = vid(p);
            }
        auto G = [&](int i, int j) { return grid[size_t(i * (F + 1) + j)]; };
        for (int i = 0; i < F; ++i)
            for (int j = 0; i + j < F; ++j) {
                T.insert(T.end(), {G(i, j), G(i + 1, j), G(i, j + 1)});
                if (i + j < F - 1) T.insert(T.end(), {G(i + 1, j), G(i + 1, j + 1), G(i, j + 1)});
            }
    }
}

}  // namespace

extern "C" {

int orbc_gen_rbc_counts(int64_t n_lipid, int freq, int64_t *n_total, int64_t *n_bonds, int64_t *n_faces) {
    if (n_lipid < 1 || freq < 1) return 1;
    const int64_t nv = 10LL * freq * freq + 2;
    if (n_total) *n_total = nv + n_lipid;
    if (n_bonds) *n_bonds = 30LL * freq * freq;
    if (n_faces) *n_faces = 20LL * freq * freq;
    return 0;
}

int orbc_gen_rbc(int64_t n_lipid, int freq, double kT, uint64_t seed, double *x3, double *n3, double *v3, double *o3,
                 int *type, int *tag, int *bonds3, double *bond_r0, int *faces3, double *radius, double *area,
                 double *volume) {
    if (n_lipid < 1 || freq < 1 || !x3 || !n3 || !v3 || !o3 || !type || !tag || !bonds3 || !bond_r0 || !faces3)
        return 1;
    const double rho = 1.05;
    const Profile unit(1.0);
    const double R = std::sqrt(double(n_lipid) / rho / (2.0 * unit.upper_area()));
    const Profile prof(R);
    if (radius) *radius = R;
    Stream rs(seed, 2);

    // spectrin mesh -> anchors
    std::vector<double> V;
    std::vector<int> T;
    geodesic(freq, V, T);
    const int64_t nv = int64_t(V.size() / 3), nf = int64_t(T.size() / 3);
    PointHash anchors(2.0, size_t(nv));
    for (int64_t k = 0; k < nv; ++k) {
        const double *q = &V[size_t(3 * k)];
        const double f = 0.5 * (1.0 - q[2]);  // sphere area fraction from the north pole
        const bool lower = f > 0.5;
        const double tt = prof.t_of(lower ? 2.0 * (1.0 - f) : 2.0 * f);
        const double phi = std::atan2(q[1], q[0]);
        prof.point(tt, phi, lower, &x3[3 * k], &n3[3 * k]);
        anchors.insert(&x3[3 * k]);
        type[k] = 3;
        tag[k] = int(k + 1);
    }
    // bonds: unique mesh edges, rest length U[0.9, 1.1] x mean edge
    std::vector<std::pair<int, int>> edges;
    edges.reserve(size_t(3 * nf));
    for (int64_t f = 0; f < nf; ++f)
        for (int c = 0; c < 3; ++c) {
            const int a = T[size_t(3 * f + c)], b = T[size_t(3 * f + (c + 1) % 3)];
            edges.emplace_back(std::min(a, b), std::max(a, b));
        }
    std::sort(edges.begin(), edges.end());
    edges.erase(std::unique(edges.begin(), edges.end()), edges.end());
    double mean = 0;
    for (auto &e : edges) {
        const double *a = &x3[3 * e.first], *b = &x3[3 * e.second];
        mean += std::sqrt((a[0] - b[0]) * (a[0] - b[0]) + (a[1] - b[1]) * (a[1] - b[1]) + (a[2] - b[2]) * (a[2] - b[2]));
    }
    mean /= double(edges.size());
    for (size_t l = 0; l < edges.size(); ++l) {
        bonds3[3 * l] = 4;
        bonds3[3 * l + 1] = edges[l].first + 1;
        bonds3[3 * l + 2] = edges[l].second + 1;
        bond_r0[l] = mean * (0.9 + 0.2 * rs.u01());
    }
    // faces and their area / enclosed volume
    double A = 0, Vol = 0;
    for (int64_t f = 0; f < nf; ++f) {
        const int a = T[size_t(3 * f)], b = T[size_t(3 * f + 1)], c = T[size_t(3 * f + 2)];
        faces3[3 * f] = a + 1;
        faces3[3 * f + 1] = b + 1;
        faces3[3 * f + 2] = c + 1;
        const double *P = &x3[3 * a], *Q = &x3[3 * b], *S = &x3[3 * c];
        const double u[3] = {Q[0] - P[0], Q[1] - P[1], Q[2] - P[2]}, w[3] = {S[0] - P[0], S[1] - P[1], S[2] - P[2]};
        const double nx = u[1] * w[2] - u[2] * w[1], ny = u[2] * w[0] - u[0] * w[2], nz = u[0] * w[1] - u[1] * w[0];
        A += 0.5 * std::sqrt(nx * nx + ny * ny + nz * nz);
        Vol += (P[0] * (Q[1] * S[2] - Q[2] * S[1]) + P[1] * (Q[2] * S[0] - Q[0] * S[2]) + P[2] * (Q[0] * S[1] - Q[1] * S[0])) / 6.0;
    }
    if (area) *area = A;
    if (volume) *volume = Vol;

    // lipids: uniform by area, 0.55 exclusion among lipids, 1.685 from anchors
    PointHash lip(1.0, size_t(n_lipid));
    int64_t k = 0, tries = 0;
    while (k < n_lipid) {
        if (++tries > 100 * n_lipid + 1000000) return 2;
        const bool lower = rs.u01() < 0.5;
        const double tt = prof.t_of(rs.u01());
        const double phi = 2.0 * M_PI * rs.u01();
        double p[3], n[3];
        prof.point(tt, phi, lower, p, n);
        if (anchors.near(p, 1.685) || lip.near(p, 0.55)) continue;
        lip.insert(p);
        const int64_t i = nv + k;
        for (int d = 0; d < 3; ++d) {
            x3[3 * i + d] = p[d];
            n3[3 * i + d] = n[d];
        }
        type[i] = 0;
        tag[i] = int(i + 1);
        ++k;
    }
    for (int64_t i = 0; i < nv + n_lipid; ++i) {
        const double sv = std::sqrt(kT / kMass[type[i]]);
        for (int d = 0; d < 3; ++d) {
            v3[3 * i + d] = sv * rs.gauss();
            o3[3 * i + d] = 0.0;
        }
    }
    return 0;
}

}  // extern "C"
