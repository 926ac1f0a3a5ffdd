/*
 * TEST INFRASTRUCTURE ONLY.  A thin C ABI over the reference's own headers,
 * compiled by oracle/Makefile (target `ref`) straight from the reference
 * source tree into oracle/_ref/ -- never shipped, never copied.  It exists to
 * generate the golden vectors in tests/golden/ that pin the oracle, and to
 * time the reference's own CPU code where it can be built.
 *
 * Pair forces are produced by the reference's cell-sweep routines applied to
 * one all-enclosing cell -- lipid_lipid::intra_cell, prote_prote::intra_cell
 * and prote_lipid::inter_cell (src/compute_pairwise_fused.h:91-236) -- so
 * every pair inside the cutoff is visited exactly once with the reference's
 * own cut tests and Newton-on accumulation.  Bonds use compute_bonded
 * (src/compute_bonded.h:89-146); integrators use the functors of
 * src/integrate_langevin.h and src/integrate_nh.h driven by integrate()
 * exactly as src/openrbc.cpp:155-242 does.
 */
#include <iostream>
#include <sstream>

#include "compute_bonded.h"
#include "compute_pairwise_fused.h"
#include "compute_temperature.h"
#include "container.h"
#include "forcefield.h"
#include "init_rbc.h"
#include "integrate_langevin.h"
#include "integrate_nh.h"
#include "reorder_morton.h"
#include "runtime_parameter.h"
#include "trajectory.h"
#include "voronoi.h"

using namespace openrbc;
using namespace openrbc::config;

namespace {

struct Quiet {  // RTParameter's constructor and init_rbc print to stdout
    std::stringstream sink;
    std::streambuf *old;
    Quiet() : old(std::cout.rdbuf(sink.rdbuf())) {}
    ~Quiet() { std::cout.rdbuf(old); }
};

RTParameter &params() {
    static RTParameter *p = nullptr;
    if (!p) {
        Quiet q;
        static char arg0[] = "ref";
        static char *argv[] = {arg0, nullptr};
        p = new RTParameter(1, argv);
        p->Q = 0;
        p->zeta = 0;
    }
    return *p;
}

struct State {
    LipidContainer lipid{"lipid"};
    ProteContainer protein{"protein"};
    std::vector<int64_t> lipid_src, prot_src;  // input index of each container slot

    void load(int64_t n, const double *x, const double *nrm, const double *v, const double *o, const int *type,
              const int *tag, int64_t nb, const int *bonds) {
        lipid_src.clear();
        prot_src.clear();
        for (int64_t i = 0; i < n; ++i) (type[i] == 0 ? lipid_src : prot_src).push_back(i);
        lipid.resize(lipid_src.size());
        protein.resize(prot_src.size());
        auto put = [&](Container &c, size_t k, int64_t i) {
            for (int d = 0; d < 3; ++d) {
                c.x[k][d] = real(x[3 * i + d]);
                c.n[k][d] = real(nrm[3 * i + d]);
                c.v[k][d] = v ? real(v[3 * i + d]) : real(0);
                c.o[k][d] = o ? real(o[3 * i + d]) : real(0);
                c.f[k][d] = 0;
                c.t[k][d] = 0;
            }
        };
        for (size_t k = 0; k < lipid_src.size(); ++k) put(lipid, k, lipid_src[k]);
        for (size_t k = 0; k < prot_src.size(); ++k) {
            put(protein, k, prot_src[k]);
            protein.type[k] = type[prot_src[k]];
            protein.tag[k] = tag[prot_src[k]];
        }
        protein.bonds.resize(0);
        for (int64_t l = 0; l < nb; ++l) protein.bonds.emplace_back(bonds[3 * l], bonds[3 * l + 1], bonds[3 * l + 2]);
        Service<BalancerMap>::call()[protein.id() + "-bonds"].set_range(protein.bonds.size());
        protein.tag2idx.build_map(protein);
    }
    template<class FN> void store(FN &&fn) {
        for (size_t k = 0; k < lipid_src.size(); ++k) fn(lipid, k, lipid_src[k]);
        for (size_t k = 0; k < prot_src.size(); ++k) fn(protein, k, prot_src[k]);
    }
    void forces() {
        const int nl = int(lipid.size()), np = int(protein.size());
        lipid_lipid::intra_cell(lipid, 0, nl);
        prote_prote::intra_cell(protein, 0, np);
        prote_lipid::inter_cell(protein, lipid, 0, np, 0, nl, newton_on, newton_on);
        compute_bonded(protein);
    }
    void export_state(double *x, double *nrm, double *v, double *o) {
        store([&](Container &c, size_t k, int64_t i) {
            for (int d = 0; d < 3; ++d) {
                if (x) x[3 * i + d] = double(c.x[k][d]);
                if (nrm) nrm[3 * i + d] = double(c.n[k][d]);
                if (v) v[3 * i + d] = double(c.v[k][d]);
                if (o) o[3 * i + d] = double(c.o[k][d]);
            }
        });
    }
};

}  // namespace

extern "C" {

int ref_real_bytes(void) { return int(sizeof(real)); }

/* Forces and torques at the given state (all pairs inside the cutoff). */
int ref_forces(int64_t n, const double *x, const double *nrm, const int *type, const int *tag, int64_t nb,
               const int *bonds, double *f3, double *t3) {
    omp_set_num_threads(1);
    params();
    State s;
    s.load(n, x, nrm, nullptr, nullptr, type, tag, nb, bonds);
    s.forces();
    s.store([&](Container &c, size_t k, int64_t i) {
        for (int d = 0; d < 3; ++d) {
            f3[3 * i + d] = double(c.f[k][d]);
            t3[3 * i + d] = double(c.t[k][d]);
        }
    });
    return 0;
}

/* nsteps of the default (FUSED_PAIRWISE + LANGEVIN) loop body of
 * src/openrbc.cpp:189-242 without the Voronoi update: forces, then
 * integrate(verlet_langevin).  With kBT = 0 the noise term vanishes. */
int ref_langevin(int64_t n, double *x, double *nrm, double *v, double *o, const int *type, const int *tag, int64_t nb,
                 const int *bonds, double dt, double kBT, double eta, int nsteps) {
    omp_set_num_threads(1);
    RTParameter &p = params();
    p.dt = dt;
    p.kBT = real(kBT);
    p.eta = real(eta);
    State s;
    s.load(n, x, nrm, v, o, type, tag, nb, bonds);
    for (int k = 0; k < nsteps; ++k) {
        s.forces();
        integrate(verlet_langevin(p), s.lipid, s.protein);
    }
    s.export_state(x, nrm, v, o);
    return 0;
}

/* Nose-Hoover path (LANGEVIN undefined, FUSED_INTEGRATOR defined):
 * prologue = forces + post_toque_final_update (src/openrbc.cpp:162-185),
 * then nsteps of verlet_initial_bounce_clearforce_update / forces /
 * post_toque_final_update (src/openrbc.cpp:189-242).  zeta is in/out,
 * Q = 0 means the reference's default 0.01 N. */
int ref_nh(int64_t n, double *x, double *nrm, double *v, double *o, const int *type, const int *tag, int64_t nb,
           const int *bonds, double dt, double kBT, double *zeta, double Q, int nsteps) {
    omp_set_num_threads(1);
    RTParameter &p = params();
    p.dt = dt;
    p.kBT = real(kBT);
    p.zeta = real(*zeta);
    p.Q = real(Q);
    State s;
    s.load(n, x, nrm, v, o, type, tag, nb, bonds);
    s.forces();
    integrate(post_toque_final_update(p), s.lipid, s.protein);
    for (int k = 0; k < nsteps; ++k) {
        integrate(verlet_initial_bounce_clearforce_update(p), s.lipid, s.protein);
        s.forces();
        integrate(post_toque_final_update(p), s.lipid, s.protein);
    }
    s.export_state(x, nrm, v, o);
    *zeta = double(p.zeta);
    return 0;
}

double ref_temperature(int64_t n, const double *x, const double *nrm, const double *v, const int *type,
                       const int *tag) {
    omp_set_num_threads(1);
    RTParameter &p = params();
    State s;
    s.load(n, x, nrm, v, nullptr, type, tag, 0, nullptr);
    return compute_temperature(s.lipid, s.protein, p);
}

/* save_frame (src/trajectory.h:61-105) of the given state: lipids (type 0,
 * implicit tags 1, 2, ... in input order) then proteins, with nstep and the
 * dump_field bits `fields`; affil gives each input particle's cell
 * affiliation, f its force.  Writes at most cap bytes to buf and returns the
 * frame size. */
int64_t ref_save_frame(int64_t n, const double *x, const double *nrm, const double *v, const double *f,
                       const int *type, const int *tag, const int *affil, int nstep, int fields, char *buf,
                       int64_t cap) {
    omp_set_num_threads(1);
    RTParameter &p = params();
    p.nstep = nstep;
    p.dump_field = fields;
    State s;
    s.load(n, x, nrm, v, nullptr, type, tag, 0, nullptr);
    VCellList cl[2];
    cl[0].affiliation.resize(s.lipid.size());
    cl[1].affiliation.resize(s.protein.size());
    for (size_t k = 0; k < s.lipid_src.size(); ++k) {
        cl[0].affiliation[k] = affil[s.lipid_src[k]];
        for (int d = 0; d < 3; ++d) s.lipid.f[k][d] = real(f[3 * s.lipid_src[k] + d]);
    }
    for (size_t k = 0; k < s.prot_src.size(); ++k) {
        cl[1].affiliation[k] = affil[s.prot_src[k]];
        for (int d = 0; d < 3; ++d) s.protein.f[k][d] = real(f[3 * s.prot_src[k] + d]);
    }
    std::ostringstream out;
    save_frame(out, s.lipid, s.protein, cl[0], cl[1], p);
    const std::string b = out.str();
    if (int64_t(b.size()) <= cap) std::memcpy(buf, b.data(), b.size());
    return int64_t(b.size());
}

/* morton_encode (src/reorder_morton.h:35-40) with the reference box. */
void ref_morton_encode(int64_t n, const double *p3, uint32_t *keys) {
    RTParameter &p = params();
    for (int64_t i = 0; i < n; ++i)
        keys[i] = morton_encode(real(p3[3 * i]), real(p3[3 * i + 1]), real(p3[3 * i + 2]), p);
}

/* Wall-clock seconds of the reference's own production loop on the given
 * state: the Voronoi initialisation of src/openrbc.cpp:71-76 (*secs_init),
 * then the main loop of src/openrbc.cpp:153-256 in the default build
 * (FUSED_PAIRWISE + LANGEVIN: Voronoi and cell-list updates every
 * freq_voronoi steps, compute_pairwise_fused, compute_bonded,
 * integrate(verlet_langevin)) for nsteps steps on `threads` OpenMP threads
 * (*secs_loop), without I/O and without the stray-lipid cleanup.  For timing
 * only: the state is not returned. */
int ref_time_production(int64_t n, const double *x, const double *nrm, const double *v, const double *o,
                        const int *type, const int *tag, int64_t nb, const int *bonds, double dt, double kBT,
                        double eta, int nsteps, int threads, double *secs_init, double *secs_loop) {
    omp_set_num_threads(threads);
    RTParameter &p = params();
    if (int(p.prng.size()) < threads) {  // one generator per thread (src/runtime_parameter.h:110-111)
        p.prng.resize(size_t(threads));
        for (auto &r : p.prng) r.init(p.rng.uint());
    }
    p.dt = dt;
    p.kBT = real(kBT);
    p.eta = real(eta);
    p.nstep = 0;
    p.freq_cleanup = 1 << 30;
    State s;
    s.load(n, x, nrm, v, o, type, tag, nb, bonds);
    const double t0 = omp_get_wtime();
    VoronoiDiagram voronoi(std::max<std::size_t>(1, s.lipid.size() / p.voronoi_cell_size));
    VCellList cell_lipid, cell_protein;
    {
        Quiet q;
        voronoi.init(s.lipid, cell_lipid, p, 64);
    }
    cell_lipid.update_particle_affiliation(s.lipid);
    cell_protein.update(s.protein, voronoi, p);
    cell_protein.update_particle_affiliation(s.protein);
    const double t1 = omp_get_wtime();
    voronoi.update(s.lipid, cell_lipid, p);
    cell_lipid.update(s.lipid, voronoi, p);
    cell_protein.update(s.protein, voronoi, p);
    integrate(clear_force(), s.lipid, s.protein);
    compute_pairwise_fused(voronoi, s.lipid, s.protein, cell_lipid, cell_protein);
    compute_bonded(s.protein);
    integrate(verlet_langevin(p), s.lipid, s.protein);
    p.nstep = 0;
    for (int k = 0; k < nsteps; ++k) {
        if (p.nstep % p.freq_voronoi == 0) {
            voronoi.update(s.lipid, cell_lipid, p);
            cell_lipid.update(s.lipid, voronoi, p);
            cell_protein.update(s.protein, voronoi, p);
        }
        compute_pairwise_fused(voronoi, s.lipid, s.protein, cell_lipid, cell_protein);
        compute_bonded(s.protein);
        integrate(verlet_langevin(p), s.lipid, s.protein);
        ++p.nstep;
    }
    const double t2 = omp_get_wtime();
    *secs_init = t1 - t0;
    *secs_loop = t2 - t1;
    return 0;
}

/* init_rbc (src/init_rbc.h:29-337) on a mesh prefix; returns the particle
 * count (proteins first, then lipids) or -1 when cap is too small.  Bonds are
 * written to bonds3 (at most bcap).  Positions are the reference's (real). */
int64_t ref_init_rbc(const char *prefix, int64_t cap, double *x, double *nrm, int *type, int *tag, int64_t bcap,
                     int *bonds3, int64_t *nbonds, double *area) {
    omp_set_num_threads(1);
    RTParameter &p = params();
    p.init = "trimesh";
    p.mesh = prefix;
    LipidContainer lipid("lipid-init");
    ProteContainer protein("protein-init");
    double a;
    {
        Quiet q;
        a = init_rbc(lipid, protein, p, 0);
    }
    const int64_t np = protein.size(), nl = lipid.size();
    *area = a;
    *nbonds = int64_t(protein.bonds.size());
    if (np + nl > cap || int64_t(protein.bonds.size()) > bcap) return -1;
    for (int64_t k = 0; k < np; ++k) {
        for (int d = 0; d < 3; ++d) {
            x[3 * k + d] = double(protein.x[k][d]);
            nrm[3 * k + d] = double(protein.n[k][d]);
        }
        type[k] = protein.type[k];
        tag[k] = protein.tag[k];
    }
    for (int64_t k = 0; k < nl; ++k) {
        for (int d = 0; d < 3; ++d) {
            x[3 * (np + k) + d] = double(lipid.x[k][d]);
            nrm[3 * (np + k) + d] = double(lipid.n[k][d]);
        }
        type[np + k] = 0;
        tag[np + k] = lipid.tag[int(k)];
    }
    for (size_t l = 0; l < protein.bonds.size(); ++l) {
        bonds3[3 * l] = protein.bonds[l].type;
        bonds3[3 * l + 1] = protein.bonds[l].i;
        bonds3[3 * l + 2] = protein.bonds[l].j;
    }
    return np + nl;
}

}  // extern "C"
