/*
 * Synthetic workloads for liborbc_gpu (host code, part of the same library).
 *
 * No reference counterpart: the reference builds its systems with
 * init_random_sphere (src/init_random.h:27-66) and init_rbc
 * (src/init_rbc.h:29-337) from a mesh file.  These generators produce the
 * seeded systems the benchmarks and parity tests run on: a jittered lipid
 * lattice, a biconcave (Evans-Fung) red-cell membrane with a geodesic spectrin
 * network, and spherical vesicles.  Arrays are AoS double[3 n]; tags are
 * 1-based; all randomness comes from a counter-based generator keyed by seed.
 */
#ifndef ORBC_WORKLOADS_H_
#define ORBC_WORKLOADS_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* n lipids on a square lattice of `ncol` columns and spacing `spacing` in
 * the z = 0 plane (row-major), Gaussian jitter `jitter` per coordinate,
 * normals +z tilted by a N(0, tilt^2) angle about a random in-plane axis,
 * Maxwell-Boltzmann velocities at kT (mass 1), zero angular velocity. */
int orbc_gen_lattice(int64_t n, int ncol, double spacing, double jitter, double tilt, double kT, uint64_t seed,
                     double *x3, double *n3, double *v3, double *o3, int *type, int *tag);

/* Sizes of orbc_gen_rbc's output: particles (anchors + lipids), bonds, faces
 * of a geodesic icosahedron of frequency `freq` (10 freq^2 + 2 vertices). */
int orbc_gen_rbc_counts(int64_t n_lipid, int freq, int64_t *n_total, int64_t *n_bonds, int64_t *n_faces);

/* Whole red-cell membrane: an Evans-Fung biconcave surface scaled so that its
 * area holds n_lipid lipids at number density 1.05; lipids placed uniformly
 * by area with a 0.55 Poisson-disk exclusion, normals along the outward
 * surface normal; one anchor particle (type 3) per vertex of a geodesic
 * spectrin mesh mapped equal-area onto the surface; one bond (type 4) per
 * mesh edge with rest length U[0.9, 1.1] x the mean edge; faces are the mesh
 * triangles (counter-clockwise from outside).  Anchors come first.  Outputs
 * the surface radius (reduced units), the mesh area and enclosed volume. */
int orbc_gen_rbc(int64_t n_lipid, int freq, double kT, uint64_t seed, double *x3, double *n3, double *v3,
                 double *o3, int *type, int *tag, int *bonds3, double *bond_r0, int *faces3, double *radius,
                 double *area, double *volume);

/* nves vesicle sizes, log-normal around `median`, clipped to [nmin, nmax],
 * with the spread chosen so that the sizes add up to about `total`. */
int orbc_gen_vesicle_sizes(int nves, int64_t nmin, int64_t nmax, int64_t median, int64_t total, uint64_t seed,
                           int64_t *sizes);

/* One spherical lipid vesicle of n lipids at density rho centred at the
 * origin (radius sqrt(n / (4 pi rho))), Poisson-disk placement, radial
 * normals, Maxwell-Boltzmann velocities; tags start at tag0. */
int orbc_gen_vesicle(int64_t n, double rho, double kT, uint64_t seed, int tag0, double *x3, double *n3, double *v3,
                     double *o3, int *type, int *tag, double *radius);

#ifdef __cplusplus
}
#endif

#endif
