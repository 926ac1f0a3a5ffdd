// Whole-cell initialiser, host part: the protein network that init_rbc
// (src/init_rbc.h:29-233) builds on a triangulated mesh, and the lipid count
// of every face.  The lipids themselves are placed on the GPU
// (orbc_gpu_place_lipids, orbc_init_rbc.cu).
//
// Steps, as in the reference:
//   * the mesh is rescaled so that its mean edge is 80 nm in reduced units
//     (1 unit = 4.4545 nm, src/init_rbc.h:69-79);
//   * face normals cross(v0 - v1, v2 - v1), normalised; vertex and edge
//     normals are the normalised sums of the normals of the faces around them
//     (:82-117);
//   * one glycophorin (type 3) per vertex, one actin (type 4) per vertex,
//     layer_dist = r0[0] below it and bonded to it (bond type 0), one band-III
//     (type 2) at the middle of every edge (:119-171);
//   * 19 spectrin beads (type 5) per edge between the two actins, shortened by
//     one unit at each end, with uniform noise of +-0.05 per coordinate; the
//     beads are chained (type 3), the end beads bonded to the actins (type 2)
//     and the middle bead to the edge's band-III (type 1) (:200-233);
//   * face f receives int(area_f * rho) lipids (:262-264).
// The reference draws the spectrin noise from its sequential generator; here
// it is Philox4x32-10 keyed by the seed with counter (edge, bead), so the
// network does not depend on the order of construction.
#include <cmath>
#include <cstdint>
#include <set>
#include <vector>

#include "orbc_gpu.h"

namespace {

constexpr int SPECTRIN_BEADS = 19;           // ForceField::spectrin_resolution
constexpr double LAYER_DIST = 2.25;          // ForceField::r0[0], actin-glycophorin bond length
constexpr double EDGE_NM = 80.0, UNIT_NM = 4.4545;

struct V3 {
    double x, y, z;
};
inline V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 add(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 scale(double s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline double sumsq(V3 a) {
    double s = 0;
    s += a.x * a.x;
    s += a.y * a.y;
    s += a.z * a.z;
    return s;
}
inline double length(V3 a) { return std::sqrt(sumsq(a)); }
inline V3 unit(V3 a) { return scale(1.0 / std::sqrt(sumsq(a)), a); }

/* Philox4x32-10 (Salmon et al., SC'11). */
void philox(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1, uint32_t o[4]) {
    for (int r = 0; r < 10; ++r) {
        const uint64_t p0 = uint64_t(0xD2511F53u) * c0, p1 = uint64_t(0xCD9E8D57u) * c2;
        const uint32_t n0 = uint32_t(p1 >> 32) ^ c1 ^ k0, n2 = uint32_t(p0 >> 32) ^ c3 ^ k1;
        c1 = uint32_t(p1);
        c3 = uint32_t(p0);
        c0 = n0;
        c2 = n2;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    o[0] = c0;
    o[1] = c1;
    o[2] = c2;
    o[3] = c3;
}

bool valid_mesh(const double *vert3, int64_t nvert, const int *bond2, int64_t nbond, const int *face3,
                int64_t nface) {
    if (!vert3 || !bond2 || !face3 || nvert < 3 || nbond < 3 || nface < 1) return false;
    for (int64_t k = 0; k < 2 * nbond; ++k)
        if (bond2[k] < 0 || bond2[k] >= nvert) return false;
    for (int64_t k = 0; k < 3 * nface; ++k)
        if (face3[k] < 0 || face3[k] >= nvert) return false;
    return true;
}

}  // namespace

extern "C" int orbc_init_rbc_sizes(int64_t nvert, int64_t nbond, int64_t *nprotein, int64_t *nbonds) {
    if (nvert < 3 || nbond < 3) return ORBC_ERR_ARG;
    if (nprotein) *nprotein = 2 * nvert + nbond + nbond * SPECTRIN_BEADS;
    if (nbonds) *nbonds = nvert + nbond * (SPECTRIN_BEADS - 1 + 3);
    return ORBC_OK;
}

extern "C" int orbc_init_rbc_network(const double *vert3, int64_t nvert, const int *bond2, int64_t nbond,
                                     const int *face3, int64_t nface, double rho, uint64_t seed, double *vert3_out,
                                     double *fnorm3_out, double *x3, double *n3, int *type, int *tag, int *bonds3,
                                     int64_t *face_nl, int64_t *nlipid) {
    if (!valid_mesh(vert3, nvert, bond2, nbond, face3, nface) || !(rho > 0)) return ORBC_ERR_ARG;
    const size_t nv = size_t(nvert), ne = size_t(nbond), nf = size_t(nface);
    std::vector<V3> v(nv);
    for (size_t i = 0; i < nv; ++i) v[i] = {vert3[3 * i], vert3[3 * i + 1], vert3[3 * i + 2]};
    auto vx = [&](int64_t k) { return v[size_t(k)]; };
    // rescale: mean edge = 80 nm
    double mean_edge = 0;
    for (size_t e = 0; e < ne; ++e) mean_edge += length(sub(vx(bond2[2 * e]), vx(bond2[2 * e + 1])));
    mean_edge /= double(ne);
    const double s = (EDGE_NM / UNIT_NM) / mean_edge;
    for (auto &p : v) p = {p.x * s, p.y * s, p.z * s};
    // normals
    std::vector<V3> fn(nf), vn(nv, V3{0, 0, 0}), en(ne, V3{0, 0, 0});
    std::vector<std::set<int64_t>> vf(nv);
    for (size_t f = 0; f < nf; ++f) {
        const int a = face3[3 * f], b = face3[3 * f + 1], c = face3[3 * f + 2];
        fn[f] = unit(cross(sub(vx(a), vx(b)), sub(vx(c), vx(b))));
        vf[size_t(a)].insert(int64_t(f));
        vf[size_t(b)].insert(int64_t(f));
        vf[size_t(c)].insert(int64_t(f));
    }
    for (size_t e = 0; e < ne; ++e) {
        const auto &f1 = vf[size_t(bond2[2 * e])], &f2 = vf[size_t(bond2[2 * e + 1])];
        int shared = 0;
        for (int64_t f : f1)
            if (f2.count(f)) {
                en[e] = add(en[e], fn[size_t(f)]);
                ++shared;
            }
        if (shared != 2) return ORBC_ERR_ARG;  // every edge borders exactly two faces
    }
    for (size_t i = 0; i < nv; ++i) {
        for (int64_t f : vf[i]) vn[i] = add(vn[i], fn[size_t(f)]);
        if (vf[i].empty()) return ORBC_ERR_ARG;
        vn[i] = unit(vn[i]);
    }
    for (size_t e = 0; e < ne; ++e) en[e] = unit(en[e]);
    // lipid counts per face
    int64_t total = 0;
    for (size_t f = 0; f < nf; ++f) {
        const V3 a = vx(face3[3 * f]), b = vx(face3[3 * f + 1]), c = vx(face3[3 * f + 2]);
        const double area = 0.5 * length(cross(sub(a, b), sub(c, b)));
        const int64_t k = int64_t(area * rho);
        if (face_nl) face_nl[f] = k;
        total += k;
    }
    if (nlipid) *nlipid = total;
    if (vert3_out)
        for (size_t i = 0; i < nv; ++i) {
            vert3_out[3 * i] = v[i].x;
            vert3_out[3 * i + 1] = v[i].y;
            vert3_out[3 * i + 2] = v[i].z;
        }
    if (fnorm3_out)
        for (size_t f = 0; f < nf; ++f) {
            fnorm3_out[3 * f] = fn[f].x;
            fnorm3_out[3 * f + 1] = fn[f].y;
            fnorm3_out[3 * f + 2] = fn[f].z;
        }
    if (!x3 || !n3 || !type || !tag || !bonds3) return ORBC_OK;  // sizes and mesh data only
    int64_t np = 0, nb = 0;
    auto put = [&](V3 p, V3 q, int ty) {
        x3[3 * np] = p.x;
        x3[3 * np + 1] = p.y;
        x3[3 * np + 2] = p.z;
        n3[3 * np] = q.x;
        n3[3 * np + 1] = q.y;
        n3[3 * np + 2] = q.z;
        type[np] = ty;
        tag[np] = int(np + 1);
        return np++;
    };
    auto bond = [&](int ty, int64_t i, int64_t j) {
        bonds3[3 * nb] = ty;
        bonds3[3 * nb + 1] = int(i + 1);  // tags
        bonds3[3 * nb + 2] = int(j + 1);
        ++nb;
    };
    for (size_t i = 0; i < nv; ++i) put(v[i], vn[i], 3);                              // glycophorin
    const int64_t actin0 = np;
    for (size_t i = 0; i < nv; ++i) {                                                 // actin
        const int64_t a = put(sub(v[i], scale(LAYER_DIST, vn[i])), vn[i], 4);
        bond(0, int64_t(i), a);
    }
    const int64_t band0 = np;
    for (size_t e = 0; e < ne; ++e)                                                   // band-III
        put(scale(0.5, add(vx(bond2[2 * e]), vx(bond2[2 * e + 1]))), en[e], 2);
    const double step = double(1.0f / float(SPECTRIN_BEADS + 1));  // the reference's 1.f / (res + 1)
    for (size_t e = 0; e < ne; ++e) {                                                 // spectrin
        const int64_t i0 = bond2[2 * e], i1 = bond2[2 * e + 1];
        V3 beg = sub(v[size_t(i0)], scale(LAYER_DIST, vn[size_t(i0)]));
        V3 end = sub(v[size_t(i1)], scale(LAYER_DIST, vn[size_t(i1)]));
        V3 inc = scale(step, sub(end, beg));
        const double li = length(inc);
        const V3 u = {inc.x / li * 1.0, inc.y / li * 1.0, inc.z / li * 1.0};
        beg = add(beg, u);
        end = sub(end, u);
        inc = scale(step, sub(end, beg));
        int64_t prev = -1;
        for (int j = 0; j < SPECTRIN_BEADS; ++j) {
            const V3 p = add(beg, scale(double(j + 1), inc));
            uint32_t o[4];
            philox(uint32_t(e), uint32_t(j), uint32_t(e >> 32), 0x53504543u, uint32_t(seed), uint32_t(seed >> 32), o);
            const double nx = double(o[0]) * (1.0 / 2147483648.0) - 1.0;
            const double ny = double(o[1]) * (1.0 / 2147483648.0) - 1.0;
            const double nz = double(o[2]) * (1.0 / 2147483648.0) - 1.0;
            const int64_t b = put({p.x + 0.05 * nx, p.y + 0.05 * ny, p.z + 0.05 * nz}, p, 5);  // n = x, as there
            if (j > 0) bond(3, prev, b);
            if (j == 0) bond(2, actin0 + i0, b);
            if (j == SPECTRIN_BEADS / 2) bond(1, band0 + int64_t(e), b);
            if (j == SPECTRIN_BEADS - 1) bond(2, actin0 + i1, b);
            prev = b;
        }
    }
    return ORBC_OK;
}
