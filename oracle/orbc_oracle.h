/*
 * TEST INFRASTRUCTURE ONLY.  CPU restatement of OpenRBC's per-timestep path.
 *
 * This header declares the C ABI of liborbc_oracle.so, the checker that the
 * parity tests, __graft_entry__.smoke() and bench.py's cpu_baseline / reference
 * arm compare the GPU library against.  Nothing in the shipped package
 * (openrbc_gb300/) includes, links or loads it.
 *
 * Parity status: pinned.  The restatement is checked against golden vectors
 * produced by the reference's own headers (src/pairwise_kernel.h,
 * src/pairwise_kernel_fused.h, src/compute_bonded.h, src/integrate_langevin.h,
 * src/integrate_nh.h, src/compute_temperature.h, src/reorder_morton.h),
 * compiled by oracle/Makefile into oracle/_ref/ and run by
 * tests/golden/make_golden.py.
 */
#ifndef ORBC_ORACLE_H_
#define ORBC_ORACLE_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Bond styles.  HARMONIC is the reference's only bonded potential
 * (src/compute_bonded.h:112-115).  FENE (expand form, shifted by r0) and
 * WLC_POW (worm-like chain + 1/r^2 repulsion with equilibrium at r0) are the
 * spectrin springs of the whole-cell workloads and are restated here. */
enum { ORC_BOND_HARMONIC = 0, ORC_BOND_FENE = 1, ORC_BOND_WLC_POW = 2 };

#define ORC_MAX_BOND_TYPES 8

typedef struct {
    int64_t n;              /* particle count                                  */
    double *x, *nrm, *v, *o;/* AoS [3n]: position, orientation, velocity, omega */
    double *f, *t;          /* AoS [3n]: force / torque (carried between NH halves) */
    const int *type;        /* [n] particle type 0..5 (0 = lipid)               */
    const int *tag;         /* [n] unique tag (bond/face endpoints refer to tags) */
    int64_t nb;             /* bonds                                            */
    const int *bonds;       /* [3nb] (type, tag_i, tag_j) as src/container.h:30-34 */
    const double *bond_r0;  /* [nb] per-bond rest length or NULL (type default) */
    int64_t nface;          /* triangles of the area/volume mesh               */
    const int *faces;       /* [3nface] tags (a, b, c), counter-clockwise seen from outside */
    double lo[3], hi[3];    /* box; used for periodic wrap and NH bounce-back   */
    int periodic[3];
    double dt, kBT, eta;    /* integrator parameters (src/runtime_parameter.h:47-52) */
    double zeta, Q;         /* Nose-Hoover thermostat state (Q == 0 -> 0.01 N)  */
    uint64_t seed;          /* counter-based RNG key                            */
    int64_t step;           /* step counter (RNG counter word)                  */
    int sys;                /* system id (RNG counter word) for batched runs    */
    int bounce;             /* reflective walls at lo/hi (src/integrate_nh.h:124-144) */
    int zero_bulk;          /* subtract the mean lipid velocity before integrating
                               (src/zero_bulk_velocity.h:29-56, src/openrbc.cpp:228) */
    /* global mesh constraints: F = -k (Q - Q0)/Q0 dQ/dx, Q = V or A */
    double kv, V0, ka, A0;
    /* bond-type table */
    int    bstyle[ORC_MAX_BOND_TYPES];
    double bK[ORC_MAX_BOND_TYPES];   /* harmonic K, FENE K, WLC kT/p (force scale) */
    double br0[ORC_MAX_BOND_TYPES];  /* default rest length                        */
    double bR[ORC_MAX_BOND_TYPES];   /* FENE max extension R; WLC lmax / r0         */
} orc_system;

typedef struct {
    double ke2;      /* sum m v^2                                        */
    double temperature; /* sum m v^2 / (3N) (src/compute_temperature.h:24-29) */
    double area, volume;
    double epot;     /* total potential energy (pair + bond)              */
    int64_t npairs;  /* interacting pairs (unordered)                     */
    int flags;       /* bit0: FENE/WLC over-extension                     */
} orc_thermo;

/* Fill the reference force-field bond table (types 0..3 harmonic, K=57,
 * r0={2.25,1.1225,2.25,2.24}; src/forcefield_canonical.h:106-109). */
void orc_default_bond_table(orc_system *s);

/* Pair + bond (+ mesh constraint) forces and torques at the current state,
 * FP64.  f3/t3 are overwritten; e (optional) receives per-particle energy
 * (each pair and bond split half/half).  Returns 0. */
int orc_forces_f64(const orc_system *s, double *f3, double *t3, double *e, orc_thermo *th);
/* Same restatement evaluated in FP32 (reference default precision,
 * src/config_static.h:34); used as the timed CPU baseline. */
int orc_forces_f32(const orc_system *s, double *f3, double *t3, double *e, orc_thermo *th);

/* Langevin step (src/integrate_langevin.h:99-149) with counter-based noise:
 * forces at the current state, then the reference's rotation/translation
 * update.  Runs nsteps; s->step advances. */
int orc_step_langevin_f64(orc_system *s, int nsteps, orc_thermo *th);
int orc_step_langevin_f32(orc_system *s, int nsteps, orc_thermo *th);
/* The timed CPU baseline: nsteps of the same FP32 Langevin step organised as
 * the reference's production loop runs (particles sorted by cell, a Verlet
 * list with the given skin rebuilt when a particle moved more than skin/2,
 * Newton's third law inside each thread's range; see orbc_oracle.cpp).
 * th->npairs receives the number of list builds. */
int orc_run_langevin_fast_f32(orc_system *s, int nsteps, double skin, orc_thermo *th);

/* Nose-Hoover: prologue = forces + post_toque_final_update
 * (src/openrbc.cpp:162-185, src/integrate_nh.h:237-273); step =
 * verlet_initial_bounce_clearforce_update, forces, post_toque_final_update
 * (src/openrbc.cpp:189-242).  zeta in s is updated. */
int orc_nh_prologue_f64(orc_system *s, orc_thermo *th);
int orc_step_nh_f64(orc_system *s, int nsteps, orc_thermo *th);

/* Energy minimisation loop (src/openrbc.cpp:88-146), nsteps iterations of:
 * forces; post_torque t <- n x t (src/integrate_nh.h:146-154); per particle
 * dx = f / m, dn = t x n, h = (|dx| > dr_opt || |dn| > dn_opt) ?
 * min(dr_opt / |dx|, dn_opt / |dn|) : dt; x += f (h / m); n += (t x n) h;
 * n <- n / |n| (:113-130); bounce_back at lo / hi when s->bounce
 * (src/integrate_nh.h:124-144).  FP64.  s->step is not advanced. */
int orc_minimize_f64(orc_system *s, int nsteps, double dr_opt, double dn_opt, orc_thermo *th);

/* assign_temperature (src/assign_temperature.h:26-44): v_d = sqrt(2 kT / m) g
 * with g a unit Gaussian (Box-Muller on Philox4x32-10 keyed by seed and tag;
 * the reference's factor 2 is kept). */
void orc_assign_temperature(orc_system *s, double kT, uint64_t seed);

/* rdf / rdf_1peak_r (src/rdf.h:26-81): histogram of pair distances
 * r = |x_i - x_j| over all unordered pairs i < j of the n points x3 whose
 * types match (type_a, type_b) in either order (-1 matches any type),
 * bin = (int)(r / dr), pairs with r >= rcut (rcut > 0) or bin >= nbins
 * dropped and counted in *dropped.  Coordinates are taken relative to
 * centre3; periodic axes (L[d] > 0) use the minimum image
 * d - L rint(d / L).  single != 0 evaluates everything in FP32 (the
 * reference's default `real`), else FP64; each operation is rounded once
 * (no contraction), so a GPU that performs the same operations produces the
 * same counts.  Returns the number of counted pairs. */
int64_t orc_rdf(const double *x3, const int *type, int64_t n, int type_a, int type_b, double dr, int nbins,
                double rcut, const double *centre3, const double *L3, int single, uint64_t *counts, int64_t *dropped);

/* delete_lipid's marking rule (src/cleanup.h:40-59) with the GPU's
 * stand-in for the Voronoi cells: generators start as the lipid centroids of
 * the partition units (cell3[3i] = unit coordinates of particle i -- the GPU
 * uses 2 x 2 x 2 bricks of grid cells -- in system sys[i], nc3[3s] units per
 * axis) holding at least mingen lipids; each lipid is affiliated with the
 * nearest generator homed in the units within one unit (then two; none: a
 * stray, removed), ties to the lower home unit (numbered x fastest, systems
 * in order), with the minimum image on axes where
 * L3[3s + d] > 0; four Lloyd updates (each generator moves by the mean
 * minimum-image offset of its members, generators left with fewer than
 * mingen members are dissolved, re-affiliate) follow; per generator with at least mingen members the
 * threshold is the sorted dr2[count / 2] times tol^2 and a lipid is kept when
 * dr2 < threshold.  Proteins are always kept.  keep[n] receives 0/1; returns
 * the number removed.  FP64. */
int64_t orc_cleanup_marks(const double *x3, const int *type, const int *cell3, const int *sys, int64_t n, int nsys,
                          const int *nc3, const double *L3, int mingen, double tol, int *keep);

/* Temperature, area and volume of the current state. */
int orc_thermo_f64(const orc_system *s, orc_thermo *th);

/* All unordered pairs (i<j, by array index) with r^2 < rcut2[ti*6+tj] and
 * r^2 > 1e-5, sorted by (i, j).  Returns the pair count; writes at most cap
 * pairs.  Minimum image in periodic dims. */
int64_t orc_pairs(const orc_system *s, const double *rcut2, int32_t *pairs, int64_t cap);

/* Reference Morton key (src/reorder_morton.h:25-42) of n points (AoS [3n]),
 * bsize = box extent per dim (2000 in the reference). */
void orc_morton_encode(const double *p3, int64_t n, const double *bsize, uint32_t *keys);
/* Stable order by (key, index). */
void orc_morton_order(const double *p3, int64_t n, const double *bsize, int32_t *order);

/* Philox4x32-10 uniform noise in [-1,1) for (seed, step, tag, sys) -> r[3]. */
void orc_noise(uint64_t seed, int64_t step, int tag, int sys, double r[3]);

/* Force-field scalar tables in FP64 (for tests): 6 masses, 6 radii. */
void orc_ff_tables(double *mass6, double *radius6, double *cutsq36, double *lj_cutsq36);

/* Number of OpenMP threads the oracle uses (0 = library default). */
void orc_set_threads(int nthreads);
int  orc_get_threads(void);

#ifdef __cplusplus
}
#endif

#endif
