// openrbc_gpu -- host driver: the time loop of the reference's main()
// (src/openrbc.cpp:43-264) with its RTParameter command line
// (src/runtime_parameter.h:82-121), where the force + integration block of
// each step (src/openrbc.cpp:191-242) is one orbc_gpu_step call.
//
//   openrbc_gpu [-i lipid|vesicle|trimesh] [-t T] [-k dt] [-e eta] [-T kBT]
//               [-r rho] [--random-seed s] [-Q q] [-D freq_display]
//               [--precision mixed|fp64] [--integrator langevin|nose-hoover]
//               [--skin s] [--n-lipid N] [--mesh-frequency F] [-m mesh] [-E n]
//
// -i lipid builds a spherical lipid vesicle of radius 100 at density rho
// (the reference's init_random_sphere size, src/init_random.h:27-66, placed
// with a 0.55 exclusion so that no energy minimisation is needed);
// -i trimesh -m PREFIX reads PREFIX.{vert,bond,face}.txt as the reference
// does (src/init_rbc.h:44-66) and builds the cell with its init_rbc
// (orbc_init_rbc_network on the host, orbc_gpu_place_lipids on the GPU), then
// minimises for opt-nstep steps and assigns the temperature, as the
// reference's main() does (src/openrbc.cpp:88-160);
// -i vesicle / trimesh without a mesh build the synthetic Evans-Fung
// red-cell membrane with a geodesic spectrin network (include/orbc_workloads.h).
#include <cmath>
#include <cstdio>
#include <fstream>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#include <chrono>

#include "orbc_gpu.h"
#include "orbc_workloads.h"

namespace {

struct Args {
    std::string init = "vesicle", precision = "mixed", integrator = "langevin", mesh;
    int opt_nstep = 1000;
    double t_total = 10, dt = 1e-2, eta = 0.01, kBT = 0.22, rho = 1.05, Q = 0, skin = 0.4;
    int freq_display = 100, rseed = 0xBAD5EED, mesh_freq = 57;
    long long n_lipid = 4000000;
};

bool take(int argc, char **argv, const char *s, const char *l, std::string &out) {
    bool found = false;
    for (int i = 1; i + 1 < argc; ++i)
        if ((s[0] && std::strcmp(argv[i], (std::string("-") + s).c_str()) == 0) ||
            std::strcmp(argv[i], (std::string("--") + l).c_str()) == 0) {
            out = argv[i + 1];
            found = true;
        }
    return found;
}

Args parse(int argc, char **argv) {
    Args a;
    std::string v;
    if (take(argc, argv, "i", "init", v)) a.init = v;
    if (take(argc, argv, "t", "total-time", v)) a.t_total = std::atof(v.c_str());
    if (take(argc, argv, "k", "dt", v)) a.dt = std::atof(v.c_str());
    if (take(argc, argv, "e", "eta", v)) a.eta = std::atof(v.c_str());
    if (take(argc, argv, "D", "display-frequency", v)) a.freq_display = std::atoi(v.c_str());
    if (take(argc, argv, "Q", "nose-hoover-Q", v)) a.Q = std::atof(v.c_str());
    if (take(argc, argv, "r", "rho", v)) a.rho = std::atof(v.c_str());
    if (take(argc, argv, "T", "kBT", v)) a.kBT = std::atof(v.c_str());
    if (take(argc, argv, "r", "random-seed", v)) a.rseed = std::atoi(v.c_str());
    if (take(argc, argv, "", "precision", v)) a.precision = v;
    if (take(argc, argv, "", "integrator", v)) a.integrator = v;
    if (take(argc, argv, "", "skin", v)) a.skin = std::atof(v.c_str());
    if (take(argc, argv, "", "n-lipid", v)) a.n_lipid = std::atoll(v.c_str());
    if (take(argc, argv, "", "mesh-frequency", v)) a.mesh_freq = std::atoi(v.c_str());
    if (take(argc, argv, "m", "mesh", v)) a.mesh = v;
    if (take(argc, argv, "E", "opt-nstep", v)) a.opt_nstep = std::atoi(v.c_str());
    return a;
}

/* PREFIX.vert.txt (x y z), .bond.txt (i j), .face.txt (i j k), whitespace
 * separated, as src/init_rbc.h:44-66 reads them. */
bool read_mesh(const std::string &prefix, std::vector<double> &vert, std::vector<int> &bond, std::vector<int> &face) {
    std::ifstream fv(prefix + ".vert.txt"), fb(prefix + ".bond.txt"), ff(prefix + ".face.txt");
    if (!fv || !fb || !ff) return false;
    double x, y, z;
    while (fv >> x >> y >> z) vert.insert(vert.end(), {x, y, z});
    int i, j, k;
    while (fb >> i >> j) bond.insert(bond.end(), {i, j});
    while (ff >> i >> j >> k) face.insert(face.end(), {i, j, k});
    return !vert.empty() && !bond.empty() && !face.empty();
}

int die(orbc_handle *h, int rc, const char *what) {
    std::fprintf(stderr, "<OpenRBC-GPU> %s failed (%d): %s\n", what, rc, orbc_gpu_error(h));
    return 1;
}

}  // namespace

int main(int argc, char **argv) {
    const Args a = parse(argc, argv);
    if (a.init != "lipid" && a.init != "vesicle" && a.init != "trimesh") {
        std::printf("<OpenRBC-GPU> Initialization mode must be 'lipid', 'vesicle', or 'trimesh'\n");
        return 1;
    }
    orbc_params p;
    orbc_gpu_default_params(&p);
    p.precision = a.precision == "fp64" ? ORBC_PREC_FP64 : ORBC_PREC_MIXED;
    p.integrator = a.integrator == "nose-hoover" ? ORBC_INT_NOSE_HOOVER : ORBC_INT_LANGEVIN;
    p.dt = a.dt;
    p.kBT = a.kBT;
    p.eta = a.eta;
    p.Q = a.Q;
    p.seed = uint64_t(a.rseed);
    p.skin = a.skin;

    std::vector<double> x, n, v, o, r0;
    std::vector<int> type, tag, bonds, faces;
    int64_t N = 0, nb = 0, nf = 0;
    orbc_system_desc sys;
    std::memset(&sys, 0, sizeof(sys));
    for (int d = 0; d < 3; ++d) {
        sys.lo[d] = -1000;
        sys.hi[d] = 1000;
    }
    std::printf("Initializing system ...\n");
    bool minimise = false;
    if (a.init == "trimesh" && !a.mesh.empty()) {
        std::vector<double> vert;
        std::vector<int> bond, face;
        if (!read_mesh(a.mesh, vert, bond, face)) {
            std::printf("<OpenRBC-GPU> cannot read mesh files %s.{vert|bond|face}.txt\n", a.mesh.c_str());
            return 1;
        }
        const int64_t nv = int64_t(vert.size() / 3), ne = int64_t(bond.size() / 2), nfc = int64_t(face.size() / 3);
        int64_t np = 0, nl = 0;
        if (orbc_init_rbc_sizes(nv, ne, &np, &nb)) return die(nullptr, ORBC_ERR_ARG, "orbc_init_rbc_sizes");
        std::vector<double> vs(3 * nv), fn(3 * nfc);
        std::vector<int64_t> fnl(nfc);
        if (orbc_init_rbc_network(vert.data(), nv, bond.data(), ne, face.data(), nfc, a.rho, uint64_t(a.rseed),
                                  vs.data(), fn.data(), nullptr, nullptr, nullptr, nullptr, nullptr, fnl.data(), &nl))
            return die(nullptr, ORBC_ERR_ARG, "orbc_init_rbc_network");
        N = np + nl;
        x.assign(3 * N, 0.0), n.assign(3 * N, 0.0), v.assign(3 * N, 0.0), o.assign(3 * N, 0.0);
        type.assign(N, 0), tag.resize(N), bonds.resize(3 * nb);
        if (orbc_init_rbc_network(vert.data(), nv, bond.data(), ne, face.data(), nfc, a.rho, uint64_t(a.rseed),
                                  nullptr, nullptr, x.data(), n.data(), type.data(), tag.data(), bonds.data(),
                                  nullptr, nullptr))
            return die(nullptr, ORBC_ERR_ARG, "orbc_init_rbc_network");
        const int rcl = orbc_gpu_place_lipids(vs.data(), nv, face.data(), fn.data(), nfc, fnl.data(), x.data(), np,
                                              0.55, 1.685, uint64_t(a.rseed), x.data() + 3 * np, n.data() + 3 * np);
        if (rcl) return die(nullptr, rcl, "orbc_gpu_place_lipids");
        for (int64_t k = np; k < N; ++k) tag[k] = int(k + 1);
        minimise = true;
    } else if (a.init == "lipid") {
        N = int64_t(a.rho * 4 * M_PI * 100.0 * 100.0);
        x.resize(3 * N), n.resize(3 * N), v.resize(3 * N), o.resize(3 * N), type.resize(N), tag.resize(N);
        double R;
        if (orbc_gen_vesicle(N, a.rho, a.kBT, uint64_t(a.rseed), 1, x.data(), n.data(), v.data(), o.data(),
                             type.data(), tag.data(), &R))
            return die(nullptr, 1, "orbc_gen_vesicle");
    } else {
        orbc_gen_rbc_counts(a.n_lipid, a.mesh_freq, &N, &nb, &nf);
        x.resize(3 * N), n.resize(3 * N), v.resize(3 * N), o.resize(3 * N), type.resize(N), tag.resize(N);
        bonds.resize(3 * nb), r0.resize(nb), faces.resize(3 * nf);
        double R, A, V;
        if (orbc_gen_rbc(a.n_lipid, a.mesh_freq, a.kBT, uint64_t(a.rseed), x.data(), n.data(), v.data(), o.data(),
                         type.data(), tag.data(), bonds.data(), r0.data(), faces.data(), &R, &A, &V))
            return die(nullptr, 1, "orbc_gen_rbc");
        p.bond_style[4] = ORBC_BOND_WLC_POW;
        p.bond_K[4] = 1.0;
        p.bond_R[4] = 2.2;
        sys.kv = 10.0;
        sys.V0 = 0.64 * 4.0 / 3.0 * M_PI * std::pow(A / (4 * M_PI), 1.5);
        sys.ka = 10.0;
        sys.A0 = A;
    }
    orbc_handle *h = nullptr;
    int rc = orbc_gpu_create(&p, &h);
    if (rc) return die(nullptr, rc, "orbc_gpu_create");
    const int64_t off[2] = {0, N};
    rc = orbc_gpu_upload_batch(h, 1, &sys, off, x.data(), n.data(), v.data(), o.data(), type.data(), tag.data(),
                               size_t(N), nb ? bonds.data() : nullptr, r0.empty() ? nullptr : r0.data(), size_t(nb),
                               nf ? faces.data() : nullptr, size_t(nf));
    if (rc) return die(h, rc, "orbc_gpu_upload_batch");
    if (minimise) {  // src/openrbc.cpp:88-146 and :160
        rc = orbc_gpu_minimize(h, a.opt_nstep, 5e-2, 5e-2, nullptr);
        if (rc) return die(h, rc, "orbc_gpu_minimize");
        rc = orbc_gpu_assign_temperature(h, a.kBT, uint64_t(a.rseed));
        if (rc) return die(h, rc, "orbc_gpu_assign_temperature");
    }
    std::printf("Done: %lld particles, %lld bonds, %lld faces.\nRun ...\n", (long long)N, (long long)nb,
                (long long)nf);

    const auto t0 = std::chrono::steady_clock::now();
    long long nstep = 0;
    const long long total = (long long)std::llround(a.t_total / a.dt);
    while (nstep < total) {
        const int chunk = int(std::min<long long>(a.freq_display, total - nstep));
        orbc_thermo th;
        rc = orbc_gpu_step(h, chunk, &th);
        if (rc) return die(h, rc, "orbc_gpu_step");
        nstep += chunk;
        const double wall = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        // status line of src/display.h:38-50: time, temperature, wall time
        std::printf("t = %10.3lf  T = %9.6lf  wall = %8.3lf s  A = %.1lf  V = %.1lf  rebuilds = %lld\n",
                    nstep * a.dt, th.temperature, wall, th.area, th.volume, (long long)th.rebuilds);
    }
    const double wall = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    std::printf("%lld steps * %lld particles on 1 GPU: %.3lf s, %.3e particle-steps/s\n", nstep, (long long)N,
                wall, double(nstep) * double(N) / wall);
    orbc_gpu_destroy(h);
    return 0;
}
