/*
 * TEST INFRASTRUCTURE ONLY -- the oracle.  CPU restatement of OpenRBC's
 * per-timestep path, used by tests/, __graft_entry__.smoke() and bench.py's
 * CPU baseline to check / time the GPU library.  The shipped package never
 * links or loads this file.
 *
 * Every routine cites the reference file:line it restates.  Arithmetic is the
 * reference's (same formulas, same operation order) in FP64 (R = double), or
 * in FP32 (R = float, the reference default, src/config_static.h:34).
 *
 * Deliberate differences from the reference, each stated where it happens:
 *  - pairs come from an exact cell list (every pair inside the cutoff), not the
 *    heuristic Voronoi stencil of src/compute_pairwise_fused.h:260-315;
 *  - each ordered pair is evaluated from its first particle's side
 *    (full list, Newton off), so no atomics are needed;
 *  - Langevin noise comes from Philox4x32-10 keyed by (seed, step, tag, system)
 *    instead of per-thread xorshift128 (src/integrate_langevin.h:116-136);
 *  - KE sums use fixed 4096-particle chunks so results do not depend on the
 *    thread count.
 */
#include "orbc_oracle.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

/* ------------------------------------------------------------------ */
/* Force field (src/forcefield_canonical.h:23-156), computed in R the  */
/* way the reference's constexpr helpers compute it.                    */
/* ------------------------------------------------------------------ */
constexpr int NT = 6;

template<class R> R POWr(R b, int e) {  // forcefield_canonical.h:24
    R p = 1;
    for (int k = 0; k < e; ++k) p = b * p;
    return p;
}
template<class R> R rep_of(R cut, R req, R eps) { return eps / POWr<R>(R(cut - req), 8); }   // :27
template<class R> R att_of(R cut, R req, R eps) {                                          // :28
    return R(-2.0 * double(eps) / double(POWr<R>(R(cut - req), 4)));
}

template<class R> struct FF {
    R mass[NT], radius[NT];
    R cutlp[NT], cutsqlp[NT], replp[NT], attlp[NT], alphalp[NT];
    R cutpp[NT * NT], cutsqpp[NT * NT], reppp[NT * NT];
    R lj_cutsq[NT * NT], lj1[NT * NT], lj2[NT * NT];
    double cut_pair[NT * NT];  // largest interaction range of a type pair
    FF() {
        const double m[NT] = {1, 4, 4, 1, 10, 10};                       // :40
        const double rad[NT] = {0.56125, 1.12375, 1.12375, 0.56125, 1.5, 0.5};  // :41
        const double cl[NT] = {2.6, 2.6, 2.6, 2.6, 0, 0};                // :52
        const double rl[NT] = {1.1225, 1.685, 1.685, 1.1225, 0, 0};     // :53
        const double el[NT] = {1.2, 1.4, 2.8, 2.8, 0, 0};                // :54
        const double al[NT] = {1.55, 5, 5, 5, 0, 0};                     // :55
        // protein-protein poly tables, rows/cols 0..3 (:57-73); zero elsewhere
        const double cp4[4][4] = {{2.6, 2.6, 2.6, 2.6}, {2.6, 2.6, 2.6, 2.6}, {2.6, 2.6, 2.6, 2.6}, {2.6, 2.6, 2.6, 2.6}};
        const double rp4[4][4] = {{1.1225, 1.685, 1.685, 1.1225}, {1.685, 2.245, 2.245, 1.685},
                                  {1.685, 2.245, 2.245, 1.685}, {1.1225, 1.685, 1.685, 1.1225}};
        const double ep4[4][4] = {{1.2, 1.4, 2.8, 2.8}, {1.4, 1, 1, 1}, {2.8, 1, 1, 1}, {2.8, 1, 1, 1}};
        // LJ tables (:76-99)
        const double lje[NT * NT] = {0, 0, 0, 0, 1, 1, 0, 0, 0, 0, 1, 1, 0, 0, 0, 0, 1, 1,
                                     0, 0, 0, 0, 0, 0, 1, 1, 1, 0, 0, 0, 1, 1, 1, 0, 0, 0};
        const double ljs[NT * NT] = {0, 0, 0, 0, 1, 1, 0, 0, 0, 0, 3.4, 3.4, 0, 0, 0, 0, 3.4, 1,
                                     0, 0, 0, 0, 0, 0, 1, 3.4, 3.4, 0, 3, 1.8, 1, 3.4, 1, 0, 1.8, 1};
        const double a = 3.4 * 1.1225;
        const double ljc[NT * NT] = {0, 0, 0, 0, 1.1225, 1.1225, 0, 0, 0, 0, a, a, 0, 0, 0, 0, a, 1.1225,
                                     0, 0, 0, 0, 0, 0, 1.1225, a, a, 0, 0, 0, 1.1225, a, 1.1225, 0, 0, 0};
        for (int t = 0; t < NT; ++t) {
            mass[t] = R(m[t]);
            radius[t] = R(rad[t]);
            cutlp[t] = R(cl[t]);
            alphalp[t] = R(al[t]);
            cutsqlp[t] = cutlp[t] * cutlp[t];  // cutsq() :25
            if (t < 4) {
                replp[t] = rep_of<R>(R(cl[t]), R(rl[t]), R(el[t]));
                attlp[t] = att_of<R>(R(cl[t]), R(rl[t]), R(el[t]));
            } else {
                replp[t] = 0;
                attlp[t] = 0;
            }
        }
        for (int k = 0; k < NT * NT; ++k) {
            int r = k / NT, c = k % NT;
            if (r < 4 && c < 4) {
                cutpp[k] = R(cp4[r][c]);
                cutsqpp[k] = cutpp[k] * cutpp[k];
                reppp[k] = rep_of<R>(R(cp4[r][c]), R(rp4[r][c]), R(ep4[r][c]));
            } else {
                cutpp[k] = cutsqpp[k] = reppp[k] = 0;
            }
            const R ljcut = R(ljc[k]);
            lj_cutsq[k] = ljcut * ljcut;                               // init() :144-148
            lj1[k] = R(48.0 * double(R(lje[k])) * std::pow(double(R(ljs[k])), 12));
            lj2[k] = R(24.0 * double(R(lje[k])) * std::pow(double(R(ljs[k])), 6));
        }
        for (int ti = 0; ti < NT; ++ti)
            for (int tj = 0; tj < NT; ++tj) {
                double c2 = 0;
                if (ti == 0 || tj == 0) {
                    int p = std::max(ti, tj);
                    c2 = std::max(double(cutsqlp[p]), double(lj_cutsq[p]));
                } else {
                    int k = ti + NT * tj;
                    c2 = std::max(double(cutsqpp[k]), double(lj_cutsq[k]));
                }
                cut_pair[ti * NT + tj] = std::sqrt(c2);
            }
    }
};

template<class R> const FF<R> &ff() {
    static const FF<R> f;
    return f;
}

template<class R> struct V3 {
    R x[3];
};
template<class R> inline R dot3(const R *a, const R *b) {  // math_vector_base.h:190-194
    R s = 0;
    for (int i = 0; i < 3; ++i) s += a[i] * b[i];
    return s;
}
template<class R> inline void cross3(const R *u, const R *v, R *w) {  // math_vector_base.h:226-233
    for (int i = 0; i < 3; ++i) w[i] = u[(i + 1) % 3] * v[(i + 2) % 3] - u[(i + 2) % 3] * v[(i + 1) % 3];
}

/* ------------------------------------------------------------------ */
/* Pair interactions, evaluated from particle i's side.                */
/* ------------------------------------------------------------------ */

/* Anisotropic poly 4-8 pair: src/pairwise_kernel.h:30-68 (lipid-lipid) and
 * src/pairwise_kernel_fused.h:22-61 (protein-lipid), same formula with the
 * lipid-protein table row of the protein type.  Adds force/torque on i and,
 * when fj is given (Newton on), the opposite force and j's torque on j. */
template<class R>
inline void aniso(const R *dx, R r_sq, const R *mu1, const R *mu2, R cut, R rep, R att, R alpha, R *f,
                  R *t, double *e, R *fj, R *tj, double *ej) {
    const R r = std::sqrt(r_sq);
    const R rinv = R(1) / r;
    R u[3];
    for (int k = 0; k < 3; ++k) u[k] = dx[k] * rinv;
    const R ninj = dot3(mu1, mu2);
    const R niu = dot3(mu1, u);
    const R nju = dot3(mu2, u);
    const R a = ninj - niu * nju;
    const R A = R(1.0) + alpha * (a - R(1.0));
    const R rc = cut - r;
    const R rc3 = rc * rc * rc;
    const R rc4 = rc * rc3;
    const R rc7 = rc3 * rc4;
    R pni[3], pnj[3];
    for (int k = 0; k < 3; ++k) {
        pni[k] = mu1[k] - niu * u[k];
        pnj[k] = mu2[k] - nju * u[k];
    }
    const R ua = att * rc4;
    const R alphaua = alpha * ua;
    const R alphauar = alphaua / r;
    const R fra = R(8.0) * rep * rc7 + A * R(4.0) * att * rc3;
    for (int k = 0; k < 3; ++k) {
        const R fk = fra * u[k] + (nju * pni[k] + niu * pnj[k]) * alphauar;
        f[k] += fk;
        t[k] -= alphaua * pnj[k];
        if (fj) {
            fj[k] -= fk;
            tj[k] -= alphaua * pni[k];
        }
    }
    const double u2 = 0.5 * (double(rep) * double(rc4) * double(rc4) + double(A) * double(att) * double(rc4));
    if (e) *e += u2;
    if (ej) *ej += u2;
}

/* Lennard-Jones (WCA cut): src/pairwise_kernel_fused.h:63-77. */
template<class R> inline void lj(const R *dx, R rsq, R lj1, R lj2, R *f, double *e, R *fj, double *ej) {
    const R r2inv = R(1) / rsq;
    const R r6inv = r2inv * r2inv * r2inv;
    const R forcelj = r6inv * (lj1 * r6inv - lj2);
    const R fpair = forcelj * r2inv;
    for (int k = 0; k < 3; ++k) {
        f[k] += dx[k] * fpair;
        if (fj) fj[k] -= dx[k] * fpair;
    }
    const double u2 = 0.5 * (double(r6inv) * (double(lj1) / 12.0 * double(r6inv) - double(lj2) / 6.0));
    if (e) *e += u2;
    if (ej) *ej += u2;
}

/* Protein-protein repulsion: src/pairwise_kernel_fused.h:79-97. */
template<class R> inline void prep(const R *dx, R r_sq, R cut, R rep, R *f, double *e, R *fj, double *ej) {
    const R r = std::sqrt(r_sq);
    R u[3];
    for (int k = 0; k < 3; ++k) u[k] = dx[k] / r;
    const R rc = cut - r;
    const R rc3 = rc * rc * rc;
    const R rc4 = rc * rc3;
    const R rc7 = rc3 * rc4;
    const R fr = R(8.0) * rep * rc7;
    for (int k = 0; k < 3; ++k) {
        f[k] += fr * u[k];
        if (fj) fj[k] -= fr * u[k];
    }
    const double u2 = 0.5 * double(rep) * double(rc4) * double(rc4);
    if (e) *e += u2;
    if (ej) *ej += u2;
}

/* Dispatch of src/compute_pairwise_fused.h:91-236: lipid-lipid
 * (:109,134), protein-lipid then LJ fallback with the protein type as the
 * table index (:168-171), protein-protein with type12 = t1 + 6 t2 (:199-203,
 * :226-230).  Returns 1 if the pair interacted. */
template<class R>
inline int pair_force(int ti, int tj, const R *dx, R r_sq, const R *mui, const R *muj, R *f, R *t, double *e,
                      R *fj = nullptr, R *tqj = nullptr, double *ej = nullptr) {
    const FF<R> &F = ff<R>();
    if (!(r_sq > R(1e-5))) return 0;
    if (ti == 0 || tj == 0) {
        const int p = ti > tj ? ti : tj;
        if (r_sq < F.cutsqlp[p]) {
            aniso<R>(dx, r_sq, mui, muj, F.cutlp[p], F.replp[p], F.attlp[p], F.alphalp[p], f, t, e, fj, tqj, ej);
            return 1;
        } else if (r_sq < F.lj_cutsq[p]) {
            lj<R>(dx, r_sq, F.lj1[p], F.lj2[p], f, e, fj, ej);
            return 1;
        }
        return 0;
    }
    const int k = ti + NT * tj;
    if (r_sq < F.cutsqpp[k]) {
        prep<R>(dx, r_sq, F.cutpp[k], F.reppp[k], f, e, fj, ej);
        return 1;
    } else if (r_sq < F.lj_cutsq[k]) {
        lj<R>(dx, r_sq, F.lj1[k], F.lj2[k], f, e, fj, ej);
        return 1;
    }
    return 0;
}

/* ------------------------------------------------------------------ */
/* Geometry helpers                                                    */
/* ------------------------------------------------------------------ */
struct Box {
    double lo[3], L[3];
    int per[3];
};
inline Box box_of(const orc_system *s) {
    Box b;
    for (int d = 0; d < 3; ++d) {
        b.lo[d] = s->lo[d];
        b.L[d] = s->hi[d] - s->lo[d];
        b.per[d] = s->periodic[d];
    }
    return b;
}
inline double min_image(double d, double L, int per) {
    if (!per) return d;
    return d - L * std::nearbyint(d / L);
}

/* Uniform cell list over the particles (periodic dims wrap, open dims span the
 * bounding box).  Used only to enumerate candidate pairs exactly. */
struct CellList {
    int nc[3];
    double lo[3], w[3];
    int per[3];
    bool brute = false;
    std::vector<int> start, idx;
    void build(const double *x, int64_t n, const Box &b, double cmax) {
        double lo_[3], hi_[3];
        for (int d = 0; d < 3; ++d) {
            per[d] = b.per[d];
            if (per[d]) {
                lo_[d] = b.lo[d];
                hi_[d] = b.lo[d] + b.L[d];
            } else {
                lo_[d] = 1e300;
                hi_[d] = -1e300;
                for (int64_t i = 0; i < n; ++i) {
                    lo_[d] = std::min(lo_[d], x[3 * i + d]);
                    hi_[d] = std::max(hi_[d], x[3 * i + d]);
                }
                if (n == 0) lo_[d] = hi_[d] = 0;
                lo_[d] -= 1e-3;
                hi_[d] += 1e-3;
            }
            double L = hi_[d] - lo_[d];
            nc[d] = std::max(1, int(std::floor(L / cmax)));
            if (per[d] && nc[d] < 3) brute = true;
            if (nc[d] > 4096) nc[d] = 4096;
            lo[d] = lo_[d];
            w[d] = L / nc[d];
        }
        const int64_t ncell = int64_t(nc[0]) * nc[1] * nc[2];
        if (ncell > (int64_t(1) << 28)) brute = true;
        if (brute) return;
        std::vector<int> cid(n);
        start.assign(ncell + 1, 0);
        for (int64_t i = 0; i < n; ++i) {
            int64_t c = cell_of(&x[3 * i]);
            cid[i] = int(c);
            start[c + 1]++;
        }
        for (int64_t c = 0; c < ncell; ++c) start[c + 1] += start[c];
        idx.resize(n);
        std::vector<int> fill(start.begin(), start.end() - 1);
        for (int64_t i = 0; i < n; ++i) idx[fill[cid[i]]++] = int(i);
    }
    int coord(double v, int d) const {
        double u = (v - lo[d]) / w[d];
        int c = int(std::floor(u));
        if (per[d]) {
            c %= nc[d];
            if (c < 0) c += nc[d];
        } else {
            c = std::min(std::max(c, 0), nc[d] - 1);
        }
        return c;
    }
    int64_t cell_of(const double *p) const {
        return coord(p[0], 0) + int64_t(nc[0]) * (coord(p[1], 1) + int64_t(nc[1]) * coord(p[2], 2));
    }
    /* visit every sorted position k2 (k2 != kself) whose particle may lie
     * within cmax of point p; positions index the cell-sorted order idx[] */
    template<class FN> void for_positions(const double *p, int64_t n, int64_t kself, FN &&fn) const {
        if (brute) {
            for (int64_t k2 = 0; k2 < n; ++k2)
                if (k2 != kself) fn(k2);
            return;
        }
        int c[3], lo3[3], hi3[3];
        for (int d = 0; d < 3; ++d) {
            c[d] = coord(p[d], d);
            lo3[d] = (per[d] || c[d] > 0) ? -1 : 0;
            hi3[d] = (per[d] || c[d] < nc[d] - 1) ? 1 : 0;
        }
        for (int dz = lo3[2]; dz <= hi3[2]; ++dz)
            for (int dy = lo3[1]; dy <= hi3[1]; ++dy)
                for (int dx = lo3[0]; dx <= hi3[0]; ++dx) {
                    int cc[3] = {c[0] + dx, c[1] + dy, c[2] + dz};
                    for (int d = 0; d < 3; ++d)
                        if (per[d]) cc[d] = (cc[d] + nc[d]) % nc[d];
                    const int64_t cell = cc[0] + int64_t(nc[0]) * (cc[1] + int64_t(nc[1]) * cc[2]);
                    for (int k2 = start[cell]; k2 < start[cell + 1]; ++k2)
                        if (k2 != kself) fn(int64_t(k2));
                }
    }
    /* visit every j that may lie within cmax of particle i (j != i) */
    template<class FN> void for_candidates(const double *x, int64_t n, int64_t i, FN &&fn) const {
        if (brute) {
            for (int64_t j = 0; j < n; ++j)
                if (j != i) fn(j);
            return;
        }
        int c[3];
        for (int d = 0; d < 3; ++d) c[d] = coord(x[3 * i + d], d);
        int lo3[3], hi3[3];
        for (int d = 0; d < 3; ++d) {
            if (per[d]) {
                lo3[d] = -1;
                hi3[d] = 1;
            } else {
                lo3[d] = c[d] > 0 ? -1 : 0;
                hi3[d] = c[d] < nc[d] - 1 ? 1 : 0;
            }
        }
        for (int dz = lo3[2]; dz <= hi3[2]; ++dz)
            for (int dy = lo3[1]; dy <= hi3[1]; ++dy)
                for (int dx = lo3[0]; dx <= hi3[0]; ++dx) {
                    int cc[3] = {c[0] + dx, c[1] + dy, c[2] + dz};
                    for (int d = 0; d < 3; ++d)
                        if (per[d]) cc[d] = (cc[d] + nc[d]) % nc[d];
                    int64_t cell = cc[0] + int64_t(nc[0]) * (cc[1] + int64_t(nc[1]) * cc[2]);
                    for (int k = start[cell]; k < start[cell + 1]; ++k)
                        if (idx[k] != i) fn(int64_t(idx[k]));
                }
    }
};

int g_threads = 0;

/* Map from tag to array index (src/container.h:36-58). */
struct TagMap {
    std::vector<int> m;
    void build(const int *tag, int64_t n) {
        int mx = -1;
        for (int64_t i = 0; i < n; ++i) mx = std::max(mx, tag[i]);
        m.assign(size_t(mx + 1), -1);
        for (int64_t i = 0; i < n; ++i) m[size_t(tag[i])] = int(i);
    }
    int operator[](int t) const { return (t >= 0 && size_t(t) < m.size()) ? m[size_t(t)] : -1; }
};

double present_cut_max(const orc_system *s) {
    bool present[NT] = {false, false, false, false, false, false};
    for (int64_t i = 0; i < s->n; ++i)
        if (s->type[i] >= 0 && s->type[i] < NT) present[s->type[i]] = true;
    const FF<double> &F = ff<double>();
    double c = 0;
    for (int a = 0; a < NT; ++a)
        for (int b = 0; b < NT; ++b)
            if (present[a] && present[b]) c = std::max(c, F.cut_pair[a * NT + b]);
    return c > 0 ? c : 1.0;
}

/* Bond force on i with dx = x_j - x_i: F_i = kappa(r) dx; returns energy.
 * HARMONIC: src/compute_bonded.h:109-115, kappa = K (1 - r0/r). */
template<class R> inline R bond_kappa(int style, R K, R r0, R Rm, R r, double *en, int *flags) {
    if (style == ORC_BOND_HARMONIC) {
        const R rinv = R(1) / r;
        if (en) *en = 0.5 * double(K) * (double(r) - double(r0)) * (double(r) - double(r0));
        return K * (R(1) - r0 * rinv);
    } else if (style == ORC_BOND_FENE) {
        /* U = -K R^2/2 ln(1 - ((r - r0)/R)^2) */
        R s = (r - r0) / Rm;
        R s2 = s * s;
        if (s2 >= R(0.99)) {
            *flags |= 1;
            s2 = R(0.99);
        }
        if (en) *en = -0.5 * double(K) * double(Rm) * double(Rm) * std::log(1.0 - double(s2));
        return K * (r - r0) / (r * (R(1) - s2));
    } else {
        /* WLC + 1/r^2 repulsion, zero net force at r0:
         * F(r) = K [1/(4(1-x)^2) - 1/4 + x] - F_wlc(r0) (r0/r)^2, x = r/lmax,
         * lmax = Rm * r0.  Attractive for r > r0. */
        const R lmax = Rm * r0;
        R x = r / lmax;
        if (x >= R(0.99)) {
            *flags |= 1;
            x = R(0.99);
        }
        const R x0 = r0 / lmax;
        const R omx = R(1) - x, omx0 = R(1) - x0;
        const R fw = K * (R(0.25) / (omx * omx) - R(0.25) + x);
        const R fw0 = K * (R(0.25) / (omx0 * omx0) - R(0.25) + x0);
        const R q = r0 / r;
        const R fr = fw - fw0 * q * q;
        if (en) {
            double xd = double(x), ld = double(lmax);
            double uw = double(K) * ld * (xd * xd / 2.0 + 0.25 / (1.0 - xd) - xd / 4.0 - 0.25);
            double up = double(fw0) * double(r0) * double(r0) / double(r);
            *en = uw + up;
        }
        return fr / r;
    }
}

/* Forces at the current state: pair (cell list, full per-particle loop),
 * bonds (src/compute_bonded.h:89-146), global area/volume constraint. */
template<class R>
int forces_impl(const orc_system *s, double *f3, double *t3, double *e, orc_thermo *th) {
    const int64_t n = s->n;
    const Box b = box_of(s);
    CellList cl;
    cl.build(s->x, n, b, present_cut_max(s) * (1 + 1e-12) + 1e-9);
    /* Work on copies in cell order: the reference re-sorts its particles every
     * freq_voronoi steps for the same memory locality (src/reorder.h:113-149).
     * Results are written back by original index, so the order does not change
     * any sum: each particle's partners are visited cell by cell. */
    std::vector<int> order(static_cast<size_t>(n));
    if (cl.brute)
        for (int64_t k = 0; k < n; ++k) order[size_t(k)] = int(k);
    else
        order = cl.idx;
    std::vector<double> xs(static_cast<size_t>(3 * n));
    std::vector<R> xr(static_cast<size_t>(3 * n)), nr(static_cast<size_t>(3 * n));
    std::vector<int> ts(static_cast<size_t>(n));
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < n; ++k) {
        const int64_t i = order[size_t(k)];
        for (int d = 0; d < 3; ++d) {
            xs[size_t(3 * k + d)] = s->x[3 * i + d];
            xr[size_t(3 * k + d)] = R(s->x[3 * i + d]);
            nr[size_t(3 * k + d)] = R(s->nrm[3 * i + d]);
        }
        ts[size_t(k)] = s->type[i];
    }
    /* Newton's third law inside each thread's contiguous range of sorted
     * particles, evaluated once per pair; pairs that cross ranges are
     * evaluated from both sides (src/compute_pairwise_fused.h:262-275). */
    std::vector<R> fs(static_cast<size_t>(3 * n), R(0)), tq(static_cast<size_t>(3 * n), R(0));
    std::vector<double> es(e ? static_cast<size_t>(n) : 0, 0.0);
    int64_t npairs = 0;
    double epot = 0;
    const int nthr = g_threads > 0 ? g_threads : omp_get_max_threads();
#pragma omp parallel num_threads(nthr) reduction(+ : npairs)
    {
        const int64_t T = omp_get_num_threads(), tid = omp_get_thread_num();
        const int64_t beg = n * tid / T, end = n * (tid + 1) / T;
        for (int64_t k = beg; k < end; ++k) {
            const int typ_i = ts[size_t(k)];
            const int64_t i = order[size_t(k)];
            R *fi = &fs[size_t(3 * k)], *ti_ = &tq[size_t(3 * k)];
            double *ei = e ? &es[size_t(k)] : nullptr;
            cl.for_positions(&xs[size_t(3 * k)], n, k, [&](int64_t k2) {
                const bool inside = k2 >= beg && k2 < end;
                if (inside && k2 < k) return;  // evaluated when k2 was the first particle
                R dx[3];
                for (int d = 0; d < 3; ++d) {
                    if (b.per[d]) {
                        double dd = min_image(xs[size_t(3 * k + d)] - xs[size_t(3 * k2 + d)], b.L[d], 1);
                        dx[d] = R(dd);
                    } else {
                        dx[d] = xr[size_t(3 * k + d)] - xr[size_t(3 * k2 + d)];
                    }
                }
                const R r_sq = dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2];
                int hit;
                if (inside)
                    hit = pair_force<R>(typ_i, ts[size_t(k2)], dx, r_sq, &nr[size_t(3 * k)], &nr[size_t(3 * k2)], fi,
                                        ti_, ei, &fs[size_t(3 * k2)], &tq[size_t(3 * k2)],
                                        e ? &es[size_t(k2)] : nullptr);
                else
                    hit = pair_force<R>(typ_i, ts[size_t(k2)], dx, r_sq, &nr[size_t(3 * k)], &nr[size_t(3 * k2)], fi,
                                        ti_, ei);
                if (hit && (inside || order[size_t(k2)] > i)) npairs++;
            });
        }
    }
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < n; ++k) {
        const int64_t i = order[size_t(k)];
        for (int d = 0; d < 3; ++d) {
            f3[3 * i + d] = double(fs[size_t(3 * k + d)]);
            t3[3 * i + d] = double(tq[size_t(3 * k + d)]);
        }
        if (e) e[i] = es[size_t(k)];
    }
    if (e)
        for (int64_t i = 0; i < n; ++i) epot += e[i];

    int flags = 0;
    /* bonds */
    if (s->nb > 0) {
        TagMap tm;
        tm.build(s->tag, n);
        for (int64_t l = 0; l < s->nb; ++l) {
            const int type = s->bonds[3 * l];
            const int p1 = tm[s->bonds[3 * l + 1]];
            const int p2 = tm[s->bonds[3 * l + 2]];
            if (p1 < 0 || p2 < 0 || type < 0 || type >= ORC_MAX_BOND_TYPES) continue;
            R dx[3];
            for (int d = 0; d < 3; ++d) {
                if (b.per[d])
                    dx[d] = R(min_image(s->x[3 * p2 + d] - s->x[3 * p1 + d], b.L[d], 1));
                else
                    dx[d] = R(s->x[3 * p2 + d]) - R(s->x[3 * p1 + d]);
            }
            const R r = std::sqrt(dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2]);
            const R r0 = s->bond_r0 ? R(s->bond_r0[l]) : R(s->br0[type]);
            double en = 0;
            const R kap = bond_kappa<R>(s->bstyle[type], R(s->bK[type]), r0, R(s->bR[type]), r, &en, &flags);
            for (int d = 0; d < 3; ++d) {
                const R fo = kap * dx[d];
                f3[3 * p1 + d] += double(fo);
                f3[3 * p2 + d] -= double(fo);
            }
            if (e) {
                e[p1] += 0.5 * en;
                e[p2] += 0.5 * en;
            }
            epot += en;
        }
    }

    /* area / volume constraint on the face mesh (FP64 always) */
    double area = 0, volume = 0;
    if (s->nface > 0) {
        TagMap tm;
        tm.build(s->tag, n);
        const int ref = tm[s->faces[0]];
        auto rel = [&](int p, double *out) {
            for (int d = 0; d < 3; ++d) out[d] = min_image(s->x[3 * p + d] - s->x[3 * ref + d], b.L[d], b.per[d]);
        };
        for (int64_t k = 0; k < s->nface; ++k) {
            int pa = tm[s->faces[3 * k]], pb = tm[s->faces[3 * k + 1]], pc = tm[s->faces[3 * k + 2]];
            double A[3], B[3], C[3], e1[3], e2[3], N[3], bc[3];
            rel(pa, A);
            rel(pb, B);
            rel(pc, C);
            for (int d = 0; d < 3; ++d) {
                e1[d] = B[d] - A[d];
                e2[d] = C[d] - A[d];
            }
            cross3(e1, e2, N);
            cross3(B, C, bc);
            area += 0.5 * std::sqrt(dot3(N, N));
            volume += dot3(A, bc) / 6.0;
        }
        const double cv = (s->kv != 0 && s->V0 != 0) ? -s->kv * (volume - s->V0) / s->V0 : 0.0;
        const double ca = (s->ka != 0 && s->A0 != 0) ? -s->ka * (area - s->A0) / s->A0 : 0.0;
        if (cv != 0 || ca != 0) {
            for (int64_t k = 0; k < s->nface; ++k) {
                int p[3] = {tm[s->faces[3 * k]], tm[s->faces[3 * k + 1]], tm[s->faces[3 * k + 2]]};
                double P[3][3];
                for (int q = 0; q < 3; ++q) rel(p[q], P[q]);
                double e1[3], e2[3], N[3];
                for (int d = 0; d < 3; ++d) {
                    e1[d] = P[1][d] - P[0][d];
                    e2[d] = P[2][d] - P[0][d];
                }
                cross3(e1, e2, N);
                const double nn = std::sqrt(dot3(N, N));
                double nh[3] = {N[0] / nn, N[1] / nn, N[2] / nn};
                for (int q = 0; q < 3; ++q) {
                    const double *a = P[q], *bb = P[(q + 1) % 3], *cc = P[(q + 2) % 3];
                    double ba[3], ca_[3], gV[3], bmc[3], gA[3];
                    for (int d = 0; d < 3; ++d) {
                        ba[d] = bb[d] - a[d];
                        ca_[d] = cc[d] - a[d];
                        bmc[d] = bb[d] - cc[d];
                    }
                    cross3(ba, ca_, gV);  // 6 dV/da summed over the closed one-ring
                    cross3(bmc, nh, gA);  // 2 dA/da
                    for (int d = 0; d < 3; ++d) f3[3 * p[q] + d] += cv * gV[d] / 6.0 + ca * gA[d] * 0.5;
                }
            }
        }
    }
    if (th) {
        th->npairs = npairs;
        th->epot = epot;
        th->area = area;
        th->volume = volume;
        th->flags = flags;
    }
    return 0;
}

/* ------------------------------------------------------------------ */
/* Counter-based noise: Philox4x32-10 (Salmon et al., SC'11).          */
/* ------------------------------------------------------------------ */
inline void philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; ++r) {
        const uint64_t p0 = uint64_t(0xD2511F53u) * c0;
        const uint64_t p1 = uint64_t(0xCD9E8D57u) * c2;
        const uint32_t hi0 = uint32_t(p0 >> 32), lo0 = uint32_t(p0);
        const uint32_t hi1 = uint32_t(p1 >> 32), lo1 = uint32_t(p1);
        c0 = hi1 ^ c1 ^ k0;
        c1 = lo1;
        c2 = hi0 ^ c3 ^ k1;
        c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0;
    out[1] = c1;
    out[2] = c2;
    out[3] = c3;
}
inline void noise3(uint64_t seed, int64_t step, int tag, int sys, double r[3]) {
    const uint32_t ctr[4] = {uint32_t(tag), uint32_t(uint64_t(step)), uint32_t(uint64_t(step) >> 32), uint32_t(sys)};
    const uint32_t key[2] = {uint32_t(seed), uint32_t(seed >> 32)};
    uint32_t o[4];
    philox(ctr, key, o);
    for (int k = 0; k < 3; ++k) r[k] = double(o[k] >> 8) * (1.0 / 8388608.0) - 1.0;
}

/* Deterministic chunked FP64 sum. */
template<class FN> double chunked_sum(int64_t n, FN &&term) {
    const int64_t CH = 4096;
    const int64_t nch = (n + CH - 1) / CH;
    std::vector<double> part(size_t(std::max<int64_t>(nch, 1)), 0.0);
#pragma omp parallel for schedule(static)
    for (int64_t c = 0; c < nch; ++c) {
        double acc = 0;
        for (int64_t i = c * CH; i < std::min(n, (c + 1) * CH); ++i) acc += term(i);
        part[size_t(c)] = acc;
    }
    double s = 0;
    for (int64_t c = 0; c < nch; ++c) s += part[size_t(c)];
    return s;
}

/* zero_bulk_velocity (src/zero_bulk_velocity.h:29-56) applied to the lipids
 * as the reference's call site does (src/openrbc.cpp:228): v -= mean lipid v. */
void zero_bulk(orc_system *s) {
    double sum[3] = {0, 0, 0};
    int64_t nl = 0;
    for (int64_t i = 0; i < s->n; ++i)
        if (s->type[i] == 0) {
            for (int d = 0; d < 3; ++d) sum[d] += s->v[3 * i + d];
            ++nl;
        }
    if (!nl) return;
    for (int d = 0; d < 3; ++d) sum[d] /= double(nl);
    for (int64_t i = 0; i < s->n; ++i)
        if (s->type[i] == 0)
            for (int d = 0; d < 3; ++d) s->v[3 * i + d] -= sum[d];
}

/* src/integrate_langevin.h:105-146, per particle, in R. */
template<class R> int langevin_impl(orc_system *s, int nsteps, orc_thermo *th) {
    const int64_t n = s->n;
    const FF<R> &F = ff<R>();
    std::vector<double> f3(3 * n), t3(3 * n);
    R gamma[NT], sigma[NT];
    for (int i = 0; i < NT; ++i) {  // :110-114
        gamma[i] = R(6.0 * M_PI * double(R(s->eta)) * double(F.radius[i]));
        sigma[i] = R(double(std::sqrt(R(2 * R(s->kBT) * gamma[i]))) * std::sqrt(3.0 / s->dt));
    }
    const R dt = R(s->dt);
    const R dt_over_m = dt / R(1);
    for (int st = 0; st < nsteps; ++st) {
        forces_impl<R>(s, f3.data(), t3.data(), nullptr, th);
        if (s->zero_bulk) zero_bulk(s);
        const int64_t step = s->step;
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n; ++i) {
            R x[3], nn[3], v[3], o[3], f[3], t[3], tmp[3];
            for (int d = 0; d < 3; ++d) {
                x[d] = R(s->x[3 * i + d]);
                nn[d] = R(s->nrm[3 * i + d]);
                v[d] = R(s->v[3 * i + d]);
                o[d] = R(s->o[3 * i + d]);
                f[d] = R(f3[3 * i + d]);
                t[d] = R(t3[3 * i + d]);
            }
            // ROTATION (:124-128)
            cross3(nn, t, tmp);
            for (int d = 0; d < 3; ++d) t[d] = tmp[d];
            for (int d = 0; d < 3; ++d) o[d] += dt_over_m * t[d];
            cross3(o, nn, tmp);
            R g[3];
            for (int d = 0; d < 3; ++d) g[d] = nn[d] + tmp[d] * dt;
            const R ginv = R(1) / std::sqrt(dot3(g, g));
            for (int d = 0; d < 3; ++d) nn[d] = g[d] * ginv;
            // TRANSLATION (:138-144)
            double rr[3];
            noise3(s->seed, step, s->tag[i], s->sys, rr);
            const int ty = s->type[i];
            for (int d = 0; d < 3; ++d) {
                f[d] -= gamma[ty] * v[d] + sigma[ty] * R(rr[d]);
                v[d] += f[d] * (dt / F.mass[ty]);
                x[d] += v[d] * dt;
            }
            for (int d = 0; d < 3; ++d) {
                s->x[3 * i + d] = double(x[d]);
                s->nrm[3 * i + d] = double(nn[d]);
                s->v[3 * i + d] = double(v[d]);
                s->o[3 * i + d] = double(o[d]);
                if (s->f) s->f[3 * i + d] = 0;
                if (s->t) s->t[3 * i + d] = 0;
            }
        }
        s->step++;
    }
    if (th) {
        th->ke2 = chunked_sum(n, [&](int64_t i) {
            const double *v = &s->v[3 * i];
            return double(F.mass[s->type[i]]) * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        });
        th->temperature = n ? th->ke2 / (3.0 * double(n)) : 0;
    }
    return 0;
}

/* post_toque_final_update (src/integrate_nh.h:237-273) + zeta update. */
void nh_final(orc_system *s) {
    const int64_t n = s->n;
    const FF<double> &F = ff<double>();
    const double dt = s->dt, zeta = s->zeta;
    const double ke = chunked_sum(n, [&](int64_t i) {
        double *t = &s->t[3 * i], *nn = &s->nrm[3 * i], *v = &s->v[3 * i], *o = &s->o[3 * i], *f = &s->f[3 * i];
        double tmp[3];
        cross3(nn, t, tmp);
        for (int d = 0; d < 3; ++d) t[d] = tmp[d];
        const double m = F.mass[s->type[i]];
        for (int d = 0; d < 3; ++d) v[d] += 0.5 * dt * (f[d] / m - zeta * v[d]);
        for (int d = 0; d < 3; ++d) o[d] += 0.5 * (dt / 1.0) * t[d];
        return 0.5 * m * dot3(v, v);
    });
    if (s->Q == 0) s->Q = double(n) * 0.01;  // runtime_parameter.h:74-76
    s->zeta += 0.5 * s->dt / s->Q * (ke - 0.5 * 3.0 * double(n) * s->kBT);  // :241-244
}

/* verlet_initial_bounce_clearforce_update (src/integrate_nh.h:178-235). */
void nh_initial(orc_system *s) {
    const int64_t n = s->n;
    const FF<double> &F = ff<double>();
    const double dt = s->dt;
    const double gamma = 1.0 / (1.0 + 0.5 * dt * s->zeta);
    const double ke = chunked_sum(n, [&](int64_t i) {
        double *x = &s->x[3 * i], *v = &s->v[3 * i], *o = &s->o[3 * i], *nn = &s->nrm[3 * i];
        double *f = &s->f[3 * i], *t = &s->t[3 * i];
        const double m = F.mass[s->type[i]];
        for (int d = 0; d < 3; ++d) v[d] = (v[d] + 0.5 / m * dt * f[d]) * gamma;
        for (int d = 0; d < 3; ++d) x[d] += v[d] * dt;
        if (s->bounce) {
            for (int d = 0; d < 3; ++d) {
                if (x[d] < s->lo[d]) {
                    x[d] = s->lo[d] + (s->lo[d] - x[d]);
                    v[d] = -v[d];
                } else if (x[d] > s->hi[d]) {
                    x[d] = s->hi[d] - (x[d] - s->hi[d]);
                    v[d] = -v[d];
                }
            }
        }
        const double k = 0.5 * m * dot3(v, v);
        for (int d = 0; d < 3; ++d) o[d] += 0.5 / 1.0 * dt * t[d];
        double tmp[3], g[3];
        cross3(o, nn, tmp);
        for (int d = 0; d < 3; ++d) g[d] = nn[d] + tmp[d] * dt;
        const double gi = 1.0 / std::sqrt(dot3(g, g));
        for (int d = 0; d < 3; ++d) nn[d] = g[d] * gi;
        for (int d = 0; d < 3; ++d) f[d] = t[d] = 0;
        return k;
    });
    if (s->Q == 0) s->Q = double(n) * 0.01;
    s->zeta += 0.5 * s->dt / s->Q * (ke - 0.5 * 3.0 * double(n) * s->kBT);  // :182-185
}

/* ------------------------------------------------------------------ */
/* The timed CPU baseline.                                             */
/* ------------------------------------------------------------------ */
/* Langevin steps with the physics of langevin_impl<float> -- pair, bond and
 * mesh-constraint forces, then src/integrate_langevin.h:105-146 with the
 * counter-based noise -- organised the way the reference's default build runs
 * its main loop (src/openrbc.cpp:189-256), so that its speed stands for the
 * reference's own CPU path:
 *  - particles stay sorted by cell and are re-sorted at every list build, as
 *    the reference re-sorts them every freq_voronoi steps (src/reorder.h:113-149);
 *  - pairs come from a Verlet list (cutoff + skin), rebuilt when a particle has
 *    moved more than skin/2 since the last build, in place of the reference's
 *    Voronoi cell list re-tessellated on a fixed cadence;
 *  - Newton's third law inside each thread's contiguous range of sorted
 *    particles, both sides across ranges (src/compute_pairwise_fused.h:262-275);
 *  - FP32 state and arithmetic (real = float, src/config_static.h:34); mesh
 *    area and volume in FP64.
 * Only the order of each particle's sums differs from langevin_impl<float>. */
struct FastRun {
    int64_t n = 0;
    int T = 1;
    Box b;
    float L[3] = {0, 0, 0};
    float skin = 0.4f;
    std::vector<int> src;      // sorted slot -> caller index
    std::vector<int> slot_of;  // caller index -> sorted slot
    std::vector<float> x, nr, v, o, f, t, xref;
    std::vector<int> ty, tg;
    std::vector<int64_t> nbeg;
    std::vector<int> nl;
    std::vector<int> cid, perm, cs, s1;  // list-build scratch, kept between builds
    std::vector<float> s3;
    std::vector<int64_t> start, cnt;
    std::vector<std::vector<int>> part;
    float rl2[NT * NT];
    float cut2[NT * NT];  // largest interaction range^2 of each type pair
    int64_t builds = 0;

    int64_t range_begin(int r) const { return n * r / T; }
    int range_of(int64_t k) const {
        int r = int((k * T) / std::max<int64_t>(n, 1));
        while (r + 1 < T && k >= range_begin(r + 1)) ++r;
        while (r > 0 && k < range_begin(r)) --r;
        return r;
    }

    void load(const orc_system *s, int threads, double skin_) {
        n = s->n;
        T = std::max(1, threads);
        b = box_of(s);
        for (int d = 0; d < 3; ++d) L[d] = float(b.L[d]);
        skin = float(skin_);
        src.resize(size_t(n));
        slot_of.resize(size_t(n));
        x.resize(size_t(3 * n));
        nr.resize(size_t(3 * n));
        v.resize(size_t(3 * n));
        o.resize(size_t(3 * n));
        f.assign(size_t(3 * n), 0.f);
        t.assign(size_t(3 * n), 0.f);
        xref.resize(size_t(3 * n));
        ty.resize(size_t(n));
        tg.resize(size_t(n));
#pragma omp parallel for schedule(static) num_threads(T)
        for (int64_t i = 0; i < n; ++i) {
            src[size_t(i)] = int(i);
            for (int d = 0; d < 3; ++d) {
                x[size_t(3 * i + d)] = float(s->x[3 * i + d]);
                nr[size_t(3 * i + d)] = float(s->nrm[3 * i + d]);
                v[size_t(3 * i + d)] = float(s->v[3 * i + d]);
                o[size_t(3 * i + d)] = float(s->o[3 * i + d]);
            }
            ty[size_t(i)] = s->type[i];
            tg[size_t(i)] = s->tag[i];
        }
        const FF<double> &F = ff<double>();
        for (int k = 0; k < NT * NT; ++k) {
            const double c = F.cut_pair[k];
            rl2[k] = c > 0 ? float((c + skin_) * (c + skin_)) : 0.f;
            cut2[k] = float(c * c);
        }
    }

    float dxw(float d, int dim) const { return b.per[dim] ? d - L[dim] * std::nearbyint(d / L[dim]) : d; }

    /* re-sort by cell of side (largest cutoff + skin) and rebuild the list */
    void rebuild(double cmax) {
        const double w0 = cmax + skin;
        double lo[3], w[3];
        int nc[3];
        for (int d = 0; d < 3; ++d) {
            double mn = b.lo[d], mx = b.lo[d] + b.L[d];
            if (!b.per[d]) {
                float fmn = 3e38f, fmx = -3e38f;
#pragma omp parallel for schedule(static) num_threads(T) reduction(min : fmn) reduction(max : fmx)
                for (int64_t k = 0; k < n; ++k) {
                    fmn = std::min(fmn, x[size_t(3 * k + d)]);
                    fmx = std::max(fmx, x[size_t(3 * k + d)]);
                }
                mn = double(fmn) - 1e-3;
                mx = double(fmx) + 1e-3;
            }
            nc[d] = std::max(1, int(std::floor((mx - mn) / w0)));
            if (b.per[d] && nc[d] < 3) nc[d] = 1;  // too small to wrap: one cell, all pairs
            nc[d] = std::min(nc[d], 1024);
            lo[d] = mn;
            w[d] = (mx - mn) / nc[d];
        }
        const int64_t ncell = int64_t(nc[0]) * nc[1] * nc[2];
        cid.resize(size_t(n));
        auto coord = [&](double val, int d) {
            int c = int(std::floor((val - lo[d]) / w[d]));
            if (b.per[d]) {
                c %= nc[d];
                if (c < 0) c += nc[d];
            } else {
                c = std::min(std::max(c, 0), nc[d] - 1);
            }
            return c;
        };
#pragma omp parallel for schedule(static) num_threads(T)
        for (int64_t k = 0; k < n; ++k)
            cid[size_t(k)] = coord(x[size_t(3 * k)], 0) +
                             nc[0] * (coord(x[size_t(3 * k + 1)], 1) + nc[1] * coord(x[size_t(3 * k + 2)], 2));
        start.assign(size_t(ncell + 1), 0);
        for (int64_t k = 0; k < n; ++k) start[size_t(cid[size_t(k)] + 1)]++;
        for (int64_t c = 0; c < ncell; ++c) start[size_t(c + 1)] += start[size_t(c)];
        perm.resize(size_t(n));
        {
            std::vector<int64_t> fill(start.begin(), start.end() - 1);
            for (int64_t k = 0; k < n; ++k) perm[size_t(fill[size_t(cid[size_t(k)])]++)] = int(k);
        }
        // gather every per-particle array into the new order (through one
        // scratch buffer per element type, kept between builds)
        auto g3 = [&](std::vector<float> &a) {
            s3.resize(a.size());
#pragma omp parallel for schedule(static) num_threads(T)
            for (int64_t k = 0; k < n; ++k)
                for (int d = 0; d < 3; ++d) s3[size_t(3 * k + d)] = a[size_t(3 * perm[size_t(k)] + d)];
            a.swap(s3);
        };
        auto g1 = [&](std::vector<int> &a) {
            s1.resize(a.size());
#pragma omp parallel for schedule(static) num_threads(T)
            for (int64_t k = 0; k < n; ++k) s1[size_t(k)] = a[size_t(perm[size_t(k)])];
            a.swap(s1);
        };
        g3(x);
        g3(nr);
        g3(v);
        g3(o);
        g1(ty);
        g1(tg);
        g1(src);
        cs.resize(size_t(n));
#pragma omp parallel for schedule(static) num_threads(T)
        for (int64_t k = 0; k < n; ++k) {
            slot_of[size_t(src[size_t(k)])] = int(k);
            cs[size_t(k)] = cid[size_t(perm[size_t(k)])];
        }
        // one pass over the 27 neighbour cells; each thread collects the lists
        // of its own range of slots, which are then laid out in slot order
        // Each thread walks its own range of slots cell by cell: the candidates of
        // the 27 cells around the current cell are staged once (shifted by the
        // periodic image they were reached through), then every particle of the
        // cell is tested against them.  Its lists land in slot order.
        bool wrap_each = false;  // a periodic axis of one or two cells: minimum image per candidate
        for (int d = 0; d < 3; ++d)
            if (b.per[d] && nc[d] < 3) wrap_each = true;
        part.resize(size_t(T));
        cnt.resize(size_t(n) + 1);
        cnt[0] = 0;
#pragma omp parallel num_threads(T)
        {
            const int r = omp_get_thread_num();
            const int64_t rb = range_begin(r), re = range_begin(r + 1);
            std::vector<int> &mine = part[size_t(r)];  // kept between builds: no fresh pages
            mine.clear();
            std::vector<float> sx;
            std::vector<int> sj, st;
            int cur = -1;
            for (int64_t k = rb; k < re; ++k) {
                const int c = cs[size_t(k)];
                if (c != cur) {
                    cur = c;
                    sx.clear();
                    sj.clear();
                    st.clear();
                    const int cc[3] = {c % nc[0], (c / nc[0]) % nc[1], c / (nc[0] * nc[1])};
                    int lo3[3], hi3[3];
                    for (int d = 0; d < 3; ++d) {
                        if (nc[d] < 3 && b.per[d]) {
                            lo3[d] = 0;
                            hi3[d] = nc[d] - 1;  // every cell of the axis once
                        } else if (b.per[d]) {
                            lo3[d] = -1;
                            hi3[d] = 1;
                        } else {
                            lo3[d] = cc[d] > 0 ? -1 : 0;
                            hi3[d] = cc[d] < nc[d] - 1 ? 1 : 0;
                        }
                    }
                    for (int dz = lo3[2]; dz <= hi3[2]; ++dz)
                        for (int dy = lo3[1]; dy <= hi3[1]; ++dy)
                            for (int dx_ = lo3[0]; dx_ <= hi3[0]; ++dx_) {
                                const int dd[3] = {dx_, dy, dz};
                                int q[3];
                                float sh[3] = {0.f, 0.f, 0.f};
                                for (int d = 0; d < 3; ++d) {
                                    q[d] = (nc[d] < 3 && b.per[d]) ? dd[d] : cc[d] + dd[d];
                                    if (b.per[d] && nc[d] >= 3) {
                                        if (q[d] < 0) {
                                            q[d] += nc[d];
                                            sh[d] = -L[d];
                                        } else if (q[d] >= nc[d]) {
                                            q[d] -= nc[d];
                                            sh[d] = L[d];
                                        }
                                    }
                                }
                                const int64_t cell = q[0] + int64_t(nc[0]) * (q[1] + int64_t(nc[1]) * q[2]);
                                for (int64_t j = start[size_t(cell)]; j < start[size_t(cell + 1)]; ++j) {
                                    for (int d = 0; d < 3; ++d) sx.push_back(x[size_t(3 * j + d)] + sh[d]);
                                    sj.push_back(int(j));
                                    st.push_back(ty[size_t(j)]);
                                }
                            }
                }
                const float *rl2k = &rl2[ty[size_t(k)] * NT];
                const float xk0 = x[size_t(3 * k)], xk1 = x[size_t(3 * k + 1)], xk2 = x[size_t(3 * k + 2)];
                const size_t before = mine.size();
                const int m = int(sj.size());
                mine.resize(before + size_t(m));
                int *out = mine.data() + before;
                int acc = 0;
                for (int u = 0; u < m; ++u) {  // branch-free: every candidate is written, the count advances on a hit
                    const int j = sj[size_t(u)];
                    float e0 = xk0 - sx[size_t(3 * u)], e1 = xk1 - sx[size_t(3 * u + 1)], e2 = xk2 - sx[size_t(3 * u + 2)];
                    if (wrap_each) {
                        e0 = dxw(e0, 0);
                        e1 = dxw(e1, 1);
                        e2 = dxw(e2, 2);
                    }
                    // Newton on inside the range: j after k there, any j outside (never k itself)
                    const bool keep = (int64_t(j) > k || int64_t(j) < rb) & (e0 * e0 + e1 * e1 + e2 * e2 < rl2k[st[size_t(u)]]);
                    out[acc] = j;
                    acc += keep ? 1 : 0;
                }
                mine.resize(before + size_t(acc));
                cnt[size_t(k + 1)] = acc;
            }
        }
        nbeg.assign(size_t(n) + 1, 0);
        for (int64_t k = 0; k < n; ++k) nbeg[size_t(k + 1)] = nbeg[size_t(k)] + cnt[size_t(k + 1)];
        nl.resize(size_t(nbeg[size_t(n)]));
#pragma omp parallel num_threads(T)
        {
            const int r = omp_get_thread_num();
            std::copy(part[size_t(r)].begin(), part[size_t(r)].end(), nl.begin() + nbeg[size_t(range_begin(r))]);
        }
        xref = x;
        ++builds;
    }

    float max_disp2() const {
        float m = 0.f;
#pragma omp parallel for schedule(static) num_threads(T) reduction(max : m)
        for (int64_t k = 0; k < n; ++k) {
            float d2 = 0.f;
            for (int d = 0; d < 3; ++d) {
                const float e = x[size_t(3 * k + d)] - xref[size_t(3 * k + d)];
                d2 += e * e;
            }
            m = std::max(m, d2);
        }
        return m;
    }
};

int fast_langevin_f32(orc_system *s, int nsteps, double skin, orc_thermo *th) {
    using R = float;
    const FF<R> &F = ff<R>();
    FastRun z;
    z.load(s, g_threads > 0 ? g_threads : omp_get_max_threads(), skin);
    const int64_t n = z.n;
    const double cmax = present_cut_max(s);
    R gamma[NT], sigma[NT];
    for (int i = 0; i < NT; ++i) {  // src/integrate_langevin.h:110-114
        gamma[i] = R(6.0 * M_PI * double(R(s->eta)) * double(F.radius[i]));
        sigma[i] = R(double(std::sqrt(R(2 * R(s->kBT) * gamma[i]))) * std::sqrt(3.0 / s->dt));
    }
    const R dt = R(s->dt);
    TagMap tm;
    tm.build(s->tag, n);
    int flags = 0;
    for (int st = 0; st < nsteps; ++st) {
        if (z.builds == 0 || z.max_disp2() > 0.25f * z.skin * z.skin) z.rebuild(cmax);
        std::fill(z.f.begin(), z.f.end(), 0.f);
        std::fill(z.t.begin(), z.t.end(), 0.f);
#pragma omp parallel num_threads(z.T)
        {
            const int r = omp_get_thread_num();
            const int64_t beg = z.range_begin(r), end = z.range_begin(r + 1);
            const bool anyper = z.b.per[0] || z.b.per[1] || z.b.per[2];
            const R llcut = F.cutlp[0], llcutsq = F.cutsqlp[0], llrep = F.replp[0], llatt = F.attlp[0],
                    llalpha = F.alphalp[0];
            constexpr int QB = 64;  // list entries filtered per batch
            int qj[QB];
            R qd[QB][3], qr2[QB];
            for (int64_t k = beg; k < end; ++k) {
                const int tk = z.ty[size_t(k)];
                R fk[3] = {0, 0, 0}, tq[3] = {0, 0, 0};
                const float *xk = &z.x[size_t(3 * k)], *nk = &z.nr[size_t(3 * k)];
                const R *cut2k = &z.cut2[size_t(tk * NT)];
                for (int64_t q0 = z.nbeg[size_t(k)]; q0 < z.nbeg[size_t(k + 1)]; q0 += QB) {
                    // the partners inside their pair's range first (branch-free), then their forces
                    const int m = int(std::min<int64_t>(QB, z.nbeg[size_t(k + 1)] - q0));
                    int h = 0;
                    for (int u = 0; u < m; ++u) {
                        const int j = z.nl[size_t(q0 + u)];
                        R d3[3];
                        if (anyper)
                            for (int d = 0; d < 3; ++d) d3[d] = z.dxw(xk[d] - z.x[size_t(3 * j + d)], d);
                        else
                            for (int d = 0; d < 3; ++d) d3[d] = xk[d] - z.x[size_t(3 * j + d)];
                        const R r2 = d3[0] * d3[0] + d3[1] * d3[1] + d3[2] * d3[2];
                        qj[h] = j;
                        qd[h][0] = d3[0];
                        qd[h][1] = d3[1];
                        qd[h][2] = d3[2];
                        qr2[h] = r2;
                        h += (r2 < cut2k[z.ty[size_t(j)]]) ? 1 : 0;
                    }
                    for (int u = 0; u < h; ++u) {
                        const int64_t j = qj[u];
                        const R r2 = qr2[u];
                        const bool inside = j >= beg && j < end;
                        const int tj = z.ty[size_t(j)];
                        if ((tk | tj) == 0) {  // lipid-lipid (src/compute_pairwise_fused.h:109,134)
                            if (r2 > R(1e-5))
                                aniso<R>(qd[u], r2, nk, &z.nr[size_t(3 * j)], llcut, llrep, llatt, llalpha, fk, tq,
                                         nullptr, inside ? &z.f[size_t(3 * j)] : nullptr,
                                         inside ? &z.t[size_t(3 * j)] : nullptr, nullptr);
                        } else {
                            pair_force<R>(tk, tj, qd[u], r2, nk, &z.nr[size_t(3 * j)], fk, tq, nullptr,
                                          inside ? &z.f[size_t(3 * j)] : nullptr,
                                          inside ? &z.t[size_t(3 * j)] : nullptr, nullptr);
                        }
                    }
                }
                for (int d = 0; d < 3; ++d) {  // partners earlier in the range added theirs already
                    z.f[size_t(3 * k + d)] += fk[d];
                    z.t[size_t(3 * k + d)] += tq[d];
                }
            }
        }
        // bonds (src/compute_bonded.h:89-146)
        for (int64_t l = 0; l < s->nb; ++l) {
            const int type = s->bonds[3 * l];
            const int i1 = tm[s->bonds[3 * l + 1]], i2 = tm[s->bonds[3 * l + 2]];
            if (i1 < 0 || i2 < 0 || type < 0 || type >= ORC_MAX_BOND_TYPES) continue;
            const int p1 = z.slot_of[size_t(i1)], p2 = z.slot_of[size_t(i2)];
            R d3[3];
            for (int d = 0; d < 3; ++d) d3[d] = z.dxw(z.x[size_t(3 * p2 + d)] - z.x[size_t(3 * p1 + d)], d);
            const R rr = std::sqrt(d3[0] * d3[0] + d3[1] * d3[1] + d3[2] * d3[2]);
            const R r0 = s->bond_r0 ? R(s->bond_r0[l]) : R(s->br0[type]);
            const R kap = bond_kappa<R>(s->bstyle[type], R(s->bK[type]), r0, R(s->bR[type]), rr, nullptr, &flags);
            for (int d = 0; d < 3; ++d) {
                z.f[size_t(3 * p1 + d)] += kap * d3[d];
                z.f[size_t(3 * p2 + d)] -= kap * d3[d];
            }
        }
        // area / volume constraint (FP64, as in forces_impl)
        if (s->nface > 0 && (s->kv != 0 || s->ka != 0)) {
            const int ref = z.slot_of[size_t(tm[s->faces[0]])];
            auto rel = [&](int p, double *out) {
                for (int d = 0; d < 3; ++d)
                    out[d] = min_image(double(z.x[size_t(3 * p + d)]) - double(z.x[size_t(3 * ref + d)]), z.b.L[d],
                                       z.b.per[d]);
            };
            auto slot = [&](int64_t k, int c) { return z.slot_of[size_t(tm[s->faces[3 * k + c]])]; };
            double area = 0, volume = 0;
            for (int64_t k = 0; k < s->nface; ++k) {
                double A[3], B[3], C[3], e1[3], e2[3], N[3], bc[3];
                rel(slot(k, 0), A);
                rel(slot(k, 1), B);
                rel(slot(k, 2), C);
                for (int d = 0; d < 3; ++d) {
                    e1[d] = B[d] - A[d];
                    e2[d] = C[d] - A[d];
                }
                cross3(e1, e2, N);
                cross3(B, C, bc);
                area += 0.5 * std::sqrt(dot3(N, N));
                volume += dot3(A, bc) / 6.0;
            }
            const double cv = (s->kv != 0 && s->V0 != 0) ? -s->kv * (volume - s->V0) / s->V0 : 0.0;
            const double ca = (s->ka != 0 && s->A0 != 0) ? -s->ka * (area - s->A0) / s->A0 : 0.0;
            for (int64_t k = 0; k < s->nface; ++k) {
                const int p[3] = {slot(k, 0), slot(k, 1), slot(k, 2)};
                double P[3][3];
                for (int q = 0; q < 3; ++q) rel(p[q], P[q]);
                double e1[3], e2[3], N[3];
                for (int d = 0; d < 3; ++d) {
                    e1[d] = P[1][d] - P[0][d];
                    e2[d] = P[2][d] - P[0][d];
                }
                cross3(e1, e2, N);
                const double nn = std::sqrt(dot3(N, N));
                const double nh[3] = {N[0] / nn, N[1] / nn, N[2] / nn};
                for (int q = 0; q < 3; ++q) {
                    const double *a = P[q], *bb = P[(q + 1) % 3], *cc = P[(q + 2) % 3];
                    double ba[3], ca_[3], gV[3], bmc[3], gA[3];
                    for (int d = 0; d < 3; ++d) {
                        ba[d] = bb[d] - a[d];
                        ca_[d] = cc[d] - a[d];
                        bmc[d] = bb[d] - cc[d];
                    }
                    cross3(ba, ca_, gV);
                    cross3(bmc, nh, gA);
                    for (int d = 0; d < 3; ++d) z.f[size_t(3 * p[q] + d)] += R(cv * gV[d] / 6.0 + ca * gA[d] * 0.5);
                }
            }
        }
        // src/integrate_langevin.h:105-146
        const int64_t step = s->step;
#pragma omp parallel for schedule(static) num_threads(z.T)
        for (int64_t k = 0; k < n; ++k) {
            R *xk = &z.x[size_t(3 * k)], *nn = &z.nr[size_t(3 * k)], *vk = &z.v[size_t(3 * k)],
              *ok = &z.o[size_t(3 * k)], *fk = &z.f[size_t(3 * k)];
            R tk[3], tmp[3];
            cross3(nn, &z.t[size_t(3 * k)], tk);
            for (int d = 0; d < 3; ++d) ok[d] += dt * tk[d];
            cross3(ok, nn, tmp);
            R g[3];
            for (int d = 0; d < 3; ++d) g[d] = nn[d] + tmp[d] * dt;
            const R ginv = R(1) / std::sqrt(dot3(g, g));
            for (int d = 0; d < 3; ++d) nn[d] = g[d] * ginv;
            double rr[3];
            noise3(s->seed, step, z.tg[size_t(k)], s->sys, rr);
            const int ty = z.ty[size_t(k)];
            for (int d = 0; d < 3; ++d) {
                const R fd = fk[d] - (gamma[ty] * vk[d] + sigma[ty] * R(rr[d]));
                vk[d] += fd * (dt / F.mass[ty]);
                xk[d] += vk[d] * dt;
            }
        }
        s->step++;
    }
#pragma omp parallel for schedule(static) num_threads(z.T)
    for (int64_t k = 0; k < n; ++k) {
        const int64_t i = z.src[size_t(k)];
        for (int d = 0; d < 3; ++d) {
            s->x[3 * i + d] = double(z.x[size_t(3 * k + d)]);
            s->nrm[3 * i + d] = double(z.nr[size_t(3 * k + d)]);
            s->v[3 * i + d] = double(z.v[size_t(3 * k + d)]);
            s->o[3 * i + d] = double(z.o[size_t(3 * k + d)]);
        }
    }
    if (th) {
        th->ke2 = chunked_sum(n, [&](int64_t i) {
            const double *vv = &s->v[3 * i];
            return double(F.mass[s->type[i]]) * (vv[0] * vv[0] + vv[1] * vv[1] + vv[2] * vv[2]);
        });
        th->temperature = n ? th->ke2 / (3.0 * double(n)) : 0;
        th->flags = flags;
        th->npairs = z.builds;
    }
    return 0;
}

}  // namespace

extern "C" {

void orc_set_threads(int nthreads) {
    g_threads = nthreads;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
}
int orc_get_threads(void) {
#ifdef _OPENMP
    return g_threads > 0 ? g_threads : omp_get_max_threads();
#else
    return 1;
#endif
}

void orc_default_bond_table(orc_system *s) {
    const double r0[4] = {2.25, 1.1225, 2.25, 2.24};
    for (int k = 0; k < ORC_MAX_BOND_TYPES; ++k) {
        s->bstyle[k] = ORC_BOND_HARMONIC;
        s->bK[k] = 57;
        s->br0[k] = k < 4 ? r0[k] : 1.0;
        s->bR[k] = 0;
    }
}

int orc_forces_f64(const orc_system *s, double *f3, double *t3, double *e, orc_thermo *th) {
    return forces_impl<double>(s, f3, t3, e, th);
}
int orc_forces_f32(const orc_system *s, double *f3, double *t3, double *e, orc_thermo *th) {
    return forces_impl<float>(s, f3, t3, e, th);
}
int orc_step_langevin_f64(orc_system *s, int nsteps, orc_thermo *th) { return langevin_impl<double>(s, nsteps, th); }
int orc_step_langevin_f32(orc_system *s, int nsteps, orc_thermo *th) { return langevin_impl<float>(s, nsteps, th); }
int orc_run_langevin_fast_f32(orc_system *s, int nsteps, double skin, orc_thermo *th) {
    if (!(skin >= 0)) return 1;
    return fast_langevin_f32(s, nsteps, skin, th);
}

int orc_nh_prologue_f64(orc_system *s, orc_thermo *th) {
    forces_impl<double>(s, s->f, s->t, nullptr, th);
    nh_final(s);
    return 0;
}
int orc_step_nh_f64(orc_system *s, int nsteps, orc_thermo *th) {
    for (int k = 0; k < nsteps; ++k) {
        nh_initial(s);
        forces_impl<double>(s, s->f, s->t, nullptr, th);
        if (s->zero_bulk) zero_bulk(s);  // src/openrbc.cpp:228, between the forces and the final half
        nh_final(s);
        s->step++;
    }
    if (th) orc_thermo_f64(s, th);
    return 0;
}

int orc_minimize_f64(orc_system *s, int nsteps, double dr_opt, double dn_opt, orc_thermo *th) {
    const int64_t n = s->n;
    const FF<double> &F = ff<double>();
    std::vector<double> f3(static_cast<size_t>(3 * n)), t3(static_cast<size_t>(3 * n));
    for (int it = 0; it < nsteps; ++it) {
        forces_impl<double>(s, f3.data(), t3.data(), nullptr, th);
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n; ++i) {
            double *x = &s->x[3 * i], *nn = &s->nrm[3 * i], *v = &s->v[3 * i];
            const double *f = &f3[size_t(3 * i)];
            double t[3], dn[3], tmp[3];
            cross3(nn, &t3[size_t(3 * i)], t);  // post_torque
            const double m = F.mass[s->type[i]];
            double dx[3];
            for (int d = 0; d < 3; ++d) dx[d] = f[d] / m;
            cross3(t, nn, dn);
            const double ndx = std::sqrt(dot3(dx, dx)), ndn = std::sqrt(dot3(dn, dn));
            const double h = (ndx > dr_opt || ndn > dn_opt) ? std::min(dr_opt / ndx, dn_opt / ndn) : s->dt;
            for (int d = 0; d < 3; ++d) x[d] += f[d] * (h / m);
            cross3(t, nn, tmp);
            for (int d = 0; d < 3; ++d) nn[d] += tmp[d] * h;
            const double inv = 1.0 / std::sqrt(dot3(nn, nn));
            for (int d = 0; d < 3; ++d) nn[d] *= inv;
            if (s->bounce)
                for (int d = 0; d < 3; ++d) {
                    if (s->periodic[d]) continue;
                    if (x[d] < s->lo[d]) {
                        x[d] = s->lo[d] + (s->lo[d] - x[d]);
                        v[d] = -v[d];
                    } else if (x[d] > s->hi[d]) {
                        x[d] = s->hi[d] - (x[d] - s->hi[d]);
                        v[d] = -v[d];
                    }
                }
        }
    }
    if (th) orc_thermo_f64(s, th);
    return 0;
}

int64_t orc_cleanup_marks(const double *x3, const int *type, const int *cell3, const int *sys, int64_t n, int nsys,
                          const int *nc3, const double *L3, int mingen, double tol, int *keep) {
    const int lloyd = 4;
    std::vector<int64_t> cb(static_cast<size_t>(nsys) + 1, 0);
    for (int s = 0; s < nsys; ++s)
        cb[size_t(s) + 1] = cb[size_t(s)] + int64_t(nc3[3 * s]) * nc3[3 * s + 1] * nc3[3 * s + 2];
    auto gid = [&](int s, const int t[3]) {
        return cb[size_t(s)] + t[0] + int64_t(nc3[3 * s]) * (t[1] + int64_t(nc3[3 * s + 1]) * t[2]);
    };
    struct Gen {
        double c[3] = {0, 0, 0};
        double w = 0;  // > 0: a generator
    };
    std::map<int64_t, Gen> gen;
    for (int64_t i = 0; i < n; ++i) {
        keep[i] = 1;
        if (type[i] != 0) continue;
        Gen &g = gen[gid(sys[i], &cell3[3 * i])];
        for (int d = 0; d < 3; ++d) g.c[d] += x3[3 * i + d];
        g.w += 1;
    }
    for (auto &kv : gen) {
        for (int d = 0; d < 3; ++d) kv.second.c[d] /= kv.second.w;
        if (kv.second.w < mingen) kv.second.w = -1;
    }
    std::vector<int64_t> aff(static_cast<size_t>(n), -1);
    std::vector<double> d2(static_cast<size_t>(n), -1.0);
    for (int it = 0; it <= lloyd; ++it) {
        if (it > 0) {  // every generator moves by the mean minimum-image offset of its members
            std::map<int64_t, Gen> acc;
            for (int64_t i = 0; i < n; ++i)
                if (aff[size_t(i)] >= 0) {
                    const Gen &cg = gen[aff[size_t(i)]];
                    Gen &g = acc[aff[size_t(i)]];
                    for (int d = 0; d < 3; ++d) {
                        double q = x3[3 * i + d] - cg.c[d];
                        const double L = L3[3 * sys[i] + d];
                        if (L > 0) q -= L * std::rint(q / L);
                        g.c[d] += q;
                    }
                    g.w += 1;
                }
            for (auto &kv : gen) {
                if (!(kv.second.w > 0)) continue;
                auto f = acc.find(kv.first);
                if (f == acc.end() || f->second.w < mingen) {  // too few members: dissolved
                    kv.second.w = -1;
                    continue;
                }
                for (int d = 0; d < 3; ++d) kv.second.c[d] += f->second.c[d] / f->second.w;
                kv.second.w = f->second.w;
            }
        }
        for (int64_t i = 0; i < n; ++i) {
            if (type[i] != 0) continue;
            const int s = sys[i];
            int64_t best_g = -1;
            double best = 0;
            for (int rad = 1; rad <= 2 && best_g < 0; ++rad)
                for (int dz = -rad; dz <= rad; ++dz)
                    for (int dy = -rad; dy <= rad; ++dy)
                        for (int dx = -rad; dx <= rad; ++dx) {
                            int t[3] = {cell3[3 * i] + dx, cell3[3 * i + 1] + dy, cell3[3 * i + 2] + dz};
                            bool ok = true;
                            for (int d = 0; d < 3; ++d) {
                                const int nt = nc3[3 * s + d];
                                if (L3[3 * s + d] > 0)
                                    t[d] = ((t[d] % nt) + nt) % nt;
                                else
                                    ok = ok && t[d] >= 0 && t[d] < nt;
                            }
                            if (!ok) continue;
                            const int64_t g = gid(s, t);
                            auto f = gen.find(g);
                            if (f == gen.end() || !(f->second.w > 0)) continue;
                            double r2 = 0;
                            for (int d = 0; d < 3; ++d) {
                                double q = x3[3 * i + d] - f->second.c[d];
                                const double L = L3[3 * s + d];
                                if (L > 0) q -= L * std::rint(q / L);
                                r2 += q * q;
                            }
                            if (best_g < 0 || r2 < best || (r2 == best && g < best_g)) {
                                best = r2;
                                best_g = g;
                            }
                        }
            aff[size_t(i)] = best_g;
            d2[size_t(i)] = best;
        }
    }
    std::map<int64_t, std::vector<int64_t>> members;
    int64_t removed = 0;
    for (int64_t i = 0; i < n; ++i) {
        if (type[i] != 0) continue;
        if (aff[size_t(i)] < 0) {  // no generator within two cells: a stray
            keep[i] = 0;
            ++removed;
        } else {
            members[aff[size_t(i)]].push_back(i);
        }
    }
    for (auto &kv : members) {
        if (int64_t(kv.second.size()) < mingen) continue;  // no statistics: all kept
        std::vector<double> v;
        for (int64_t i : kv.second) v.push_back(d2[size_t(i)]);
        std::sort(v.begin(), v.end());
        const double thr = v[v.size() / 2] * tol * tol;
        for (int64_t i : kv.second)
            if (!(d2[size_t(i)] < thr)) {
                keep[i] = 0;
                ++removed;
            }
    }
    return removed;
}

int orc_thermo_f64(const orc_system *s, orc_thermo *th) {
    const FF<double> &F = ff<double>();
    th->ke2 = chunked_sum(s->n, [&](int64_t i) {
        const double *v = &s->v[3 * i];
        return F.mass[s->type[i]] * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    });
    th->temperature = s->n ? th->ke2 / (3.0 * double(s->n)) : 0;
    th->area = th->volume = 0;
    if (s->nface > 0) {
        TagMap tm;
        tm.build(s->tag, s->n);
        const Box b = box_of(s);
        const int ref = tm[s->faces[0]];
        for (int64_t k = 0; k < s->nface; ++k) {
            double P[3][3];
            for (int q = 0; q < 3; ++q) {
                int p = tm[s->faces[3 * k + q]];
                for (int d = 0; d < 3; ++d) P[q][d] = min_image(s->x[3 * p + d] - s->x[3 * ref + d], b.L[d], b.per[d]);
            }
            double e1[3], e2[3], N[3], bc[3];
            for (int d = 0; d < 3; ++d) {
                e1[d] = P[1][d] - P[0][d];
                e2[d] = P[2][d] - P[0][d];
            }
            cross3(e1, e2, N);
            cross3(P[1], P[2], bc);
            th->area += 0.5 * std::sqrt(dot3(N, N));
            th->volume += dot3(P[0], bc) / 6.0;
        }
    }
    return 0;
}

int64_t orc_pairs(const orc_system *s, const double *rcut2, int32_t *pairs, int64_t cap) {
    const int64_t n = s->n;
    const Box b = box_of(s);
    double cmax = 0;
    for (int k = 0; k < NT * NT; ++k) cmax = std::max(cmax, std::sqrt(std::max(0.0, rcut2[k])));
    CellList cl;
    cl.build(s->x, n, b, cmax * (1 + 1e-12) + 1e-9);
    std::vector<std::vector<int32_t>> per(static_cast<size_t>(n));
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < n; ++i) {
        cl.for_candidates(s->x, n, i, [&](int64_t j) {
            if (j <= i) return;
            double r2 = 0;
            for (int d = 0; d < 3; ++d) {
                double dd = min_image(s->x[3 * i + d] - s->x[3 * j + d], b.L[d], b.per[d]);
                r2 += dd * dd;
            }
            if (r2 < rcut2[s->type[i] * NT + s->type[j]] && r2 > 1e-5) per[size_t(i)].push_back(int32_t(j));
        });
        std::sort(per[size_t(i)].begin(), per[size_t(i)].end());
    }
    int64_t cnt = 0;
    for (int64_t i = 0; i < n; ++i)
        for (int32_t j : per[size_t(i)]) {
            if (cnt < cap) {
                pairs[2 * cnt] = int32_t(i);
                pairs[2 * cnt + 1] = j;
            }
            cnt++;
        }
    return cnt;
}

/* src/rdf.h:26-47 (all pairs, dr-wide bins, `static_cast<int>(dx / dr)`) and
 * :49-81 (type filter, cutoff). */
}  // extern "C"

template<class T>
static int64_t rdf_impl(const double *x3, const int *type, int64_t n, int ta, int tb, double dr_, int nbins,
                        double rcut_, const double *c3, const double *L3, uint64_t *counts, int64_t *dropped) {
    std::vector<T> x(static_cast<size_t>(3 * n));
    for (int64_t i = 0; i < n; ++i)
        for (int d = 0; d < 3; ++d) x[size_t(3 * i + d)] = T(x3[3 * i + d] - c3[d]);
    const T dr = T(dr_), rcut = T(rcut_);
    const T L[3] = {T(L3 ? L3[0] : 0), T(L3 ? L3[1] : 0), T(L3 ? L3[2] : 0)};
    auto match = [&](int t, int want) { return want < 0 || t == want; };
    int64_t counted = 0, drop = 0;
    std::vector<uint64_t> h(static_cast<size_t>(nbins), 0);
    for (int64_t i = 0; i < n; ++i)
        for (int64_t j = i + 1; j < n; ++j) {
            const int ti = type[i], tj = type[j];
            if (!((match(ti, ta) && match(tj, tb)) || (match(ti, tb) && match(tj, ta)))) continue;
            T dd[3];
            for (int d = 0; d < 3; ++d) {
                T q = x[size_t(3 * i + d)] - x[size_t(3 * j + d)];
                if (L[d] > T(0)) {
                    const T m = std::rint(q / L[d]);
                    const T sh = L[d] * m;
                    q = q - sh;
                }
                dd[d] = q;
            }
            const T a0 = dd[0] * dd[0], a1 = dd[1] * dd[1], a2 = dd[2] * dd[2];
            const T r = std::sqrt((a0 + a1) + a2);
            if (rcut > T(0) && !(r < rcut)) {
                ++drop;
                continue;
            }
            const T q = r / dr;
            const int64_t b = q < T(2147483647.0) ? int64_t(int(q)) : int64_t(2147483647);
            if (b >= nbins) {
                ++drop;
                continue;
            }
            ++h[size_t(b)];
            ++counted;
        }
    for (int k = 0; k < nbins; ++k) counts[k] = h[size_t(k)];
    if (dropped) *dropped = drop;
    return counted;
}

extern "C" {

int64_t orc_rdf(const double *x3, const int *type, int64_t n, int type_a, int type_b, double dr, int nbins,
                double rcut, const double *centre3, const double *L3, int single, uint64_t *counts, int64_t *dropped) {
    return single ? rdf_impl<float>(x3, type, n, type_a, type_b, dr, nbins, rcut, centre3, L3, counts, dropped)
                  : rdf_impl<double>(x3, type, n, type_a, type_b, dr, nbins, rcut, centre3, L3, counts, dropped);
}

/* src/reorder_morton.h:25-42 */
static inline uint32_t bit_space3(uint32_t x) {
    x = (x | (x << 12)) & 0x00FC003Fu;
    x = (x | (x << 6)) & 0x381C0E07u;
    x = (x | (x << 4)) & 0x190C8643u;
    x = (x | (x << 2)) & 0x49249249u;
    return x;
}
static inline uint32_t to_uint(double v) {
    /* static_cast<unsigned int>(double) for values in [0, 2^32); inputs
     * below zero (outside the reference box) are out of contract. */
    if (!(v >= 0)) return 0;
    if (v >= 4294967296.0) return 0xFFFFFFFFu;
    return uint32_t(v);
}
void orc_morton_encode(const double *p3, int64_t n, const double *bsize, uint32_t *keys) {
    for (int64_t i = 0; i < n; ++i) {
        uint32_t c[3];
        for (int d = 0; d < 3; ++d) c[d] = to_uint(2 * p3[3 * i + d] + bsize[d]);
        keys[i] = bit_space3(c[0]) | (bit_space3(c[1]) << 1) | (bit_space3(c[2]) << 2);
    }
}
void orc_morton_order(const double *p3, int64_t n, const double *bsize, int32_t *order) {
    std::vector<uint32_t> k(static_cast<size_t>(n));
    orc_morton_encode(p3, n, bsize, k.data());
    for (int64_t i = 0; i < n; ++i) order[i] = int32_t(i);
    std::stable_sort(order, order + n, [&](int32_t a, int32_t b) { return k[size_t(a)] < k[size_t(b)]; });
}

void orc_noise(uint64_t seed, int64_t step, int tag, int sys, double r[3]) { noise3(seed, step, tag, sys, r); }

/* Lipid placement of init_rbc (src/init_rbc.h:235-305), the checker of
 * orbc_gpu_place_lipids: face f gets face_nl[f] lipids; for lipid j the
 * attempts k = 0, 1, 2, ... draw (r1, r2) from Philox4x32-10 keyed by the
 * seed with counter (f, j, k, f >> 32 ^ 'LIPI') and the first candidate
 * v1 (1 - sqrt r1) + v2 sqrt r1 (1 - r2) + v3 sqrt r1 r2 that is at least
 * min_dist_lp from v1 and from every protein and at least min_dist from the
 * face's earlier lipids is kept (a brute-force protein scan here, a grid
 * there).  Returns the number of lipids placed, or -(face + 1) when a lipid
 * of that face found no room in 8,192 attempts. */
int64_t orc_place_lipids(const double *vert3, const int *face3, const double *fnorm3, int64_t nface,
                         const int64_t *face_nl, const double *prot3, int64_t nprot, double min_dist,
                         double min_dist_lp, uint64_t seed, double *x3, double *n3) {
    const uint32_t key[2] = {uint32_t(seed), uint32_t(seed >> 32)};
    const double md2 = min_dist * min_dist, mdlp2 = min_dist_lp * min_dist_lp;
    auto sq3 = [](double dx, double dy, double dz) { return dx * dx + dy * dy + dz * dz; };
    int64_t out = 0;
    for (int64_t f = 0; f < nface; ++f) {
        const double *v1 = vert3 + 3 * face3[3 * f], *v2 = vert3 + 3 * face3[3 * f + 1],
                     *v3 = vert3 + 3 * face3[3 * f + 2];
        const int64_t b0 = out;
        for (int64_t j = 0; j < face_nl[f]; ++j) {
            bool placed = false;
            for (uint32_t k = 0; k < 8192u && !placed; ++k) {
                const uint32_t ctr[4] = {uint32_t(f), uint32_t(j), k, uint32_t(uint64_t(f) >> 32) ^ 0x4C495049u};
                uint32_t o[4];
                philox(ctr, key, o);
                const double r1 = double(uint64_t(o[0] >> 5) * 67108864ull + uint64_t(o[1] >> 6)) *
                                  (1.0 / 9007199254740992.0);
                const double r2 = double(uint64_t(o[2] >> 5) * 67108864ull + uint64_t(o[3] >> 6)) *
                                  (1.0 / 9007199254740992.0);
                const double s1 = std::sqrt(r1);
                const double w1 = 1.0 - s1, w2 = s1 * (1.0 - r2), w3 = s1 * r2;
                double r[3];
                for (int d = 0; d < 3; ++d) r[d] = (v1[d] * w1 + v2[d] * w2) + v3[d] * w3;
                bool clean = sq3(r[0] - v1[0], r[1] - v1[1], r[2] - v1[2]) >= mdlp2;
                for (int64_t p = 0; p < nprot && clean; ++p) {
                    const double *q = prot3 + 3 * p;
                    if (sq3(r[0] - q[0], r[1] - q[1], r[2] - q[2]) < mdlp2) clean = false;
                }
                for (int64_t m = b0; m < b0 + j && clean; ++m) {
                    const double *q = x3 + 3 * m;
                    if (sq3(q[0] - r[0], q[1] - r[1], q[2] - r[2]) < md2) clean = false;
                }
                if (clean) {
                    for (int d = 0; d < 3; ++d) {
                        x3[3 * (b0 + j) + d] = r[d];
                        n3[3 * (b0 + j) + d] = fnorm3[3 * f + d];
                    }
                    placed = true;
                }
            }
            if (!placed) return -(f + 1);
        }
        out = b0 + face_nl[f];
    }
    return out;
}

void orc_assign_temperature(orc_system *s, double kT, uint64_t seed) {
    const FF<double> &F = ff<double>();
    for (int64_t i = 0; i < s->n; ++i) {
        const uint32_t ctr[4] = {uint32_t(s->tag[i]), 0x6B8B4567u, 0x327B23C6u, uint32_t(s->sys)};
        const uint32_t key[2] = {uint32_t(seed), uint32_t(seed >> 32)};
        uint32_t o[4];
        philox(ctr, key, o);
        // two Box-Muller pairs from four 32-bit words -> three Gaussians
        double u[4];
        for (int k = 0; k < 4; ++k) u[k] = (double(o[k]) + 0.5) * (1.0 / 4294967296.0);
        const double r0 = std::sqrt(-2.0 * std::log(u[0])), r1 = std::sqrt(-2.0 * std::log(u[2]));
        const double g[3] = {r0 * std::cos(2.0 * M_PI * u[1]), r0 * std::sin(2.0 * M_PI * u[1]),
                             r1 * std::cos(2.0 * M_PI * u[3])};
        const double sc = std::sqrt(2.0 / F.mass[s->type[i]] * kT);
        for (int d = 0; d < 3; ++d) s->v[3 * i + d] = sc * g[d];
    }
}

void orc_ff_tables(double *mass6, double *radius6, double *cutsq36, double *lj_cutsq36) {
    const FF<double> &F = ff<double>();
    for (int t = 0; t < NT; ++t) {
        mass6[t] = F.mass[t];
        radius6[t] = F.radius[t];
    }
    for (int k = 0; k < NT * NT; ++k) {
        const int ti = k / NT, tj = k % NT;
        if (ti == 0 || tj == 0) {
            const int p = std::max(ti, tj);
            cutsq36[k] = F.cutsqlp[p];
            lj_cutsq36[k] = F.lj_cutsq[p];
        } else {
            cutsq36[k] = F.cutsqpp[ti + NT * tj];
            lj_cutsq36[k] = F.lj_cutsq[ti + NT * tj];
        }
    }
}

}  // extern "C"
