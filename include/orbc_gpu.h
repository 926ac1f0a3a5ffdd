/*
 * liborbc_gpu -- C ABI of the GB300 (sm_103a) implementation of OpenRBC's
 * per-timestep hot path.
 *
 * The reference has no runtime plug-in surface: its main() selects the force
 * and integration routines at compile time (src/openrbc.cpp:162-186 and
 * :191-242, #ifdef FUSED_PAIRWISE / LANGEVIN / FUSED_INTEGRATOR) and calls
 *   compute_pairwise_fused(voronoi, lipid, protein, cell_lipid, cell_protein)
 *       (src/compute_pairwise_fused.h:238-242),
 *   compute_bonded(protein)                        (src/compute_bonded.h:89-90),
 *   integrate(verlet_langevin(param), lipid, protein)
 *       (src/integrate_nh.h:29-55, src/integrate_langevin.h:99-149),
 *   integrate(verlet_initial_bounce_clearforce_update / post_toque_final_update)
 *       (src/integrate_nh.h:178-273),
 *   compute_temperature(lipid, protein, param)     (src/compute_temperature.h:24-29),
 * with the Voronoi / k-d tree / Morton reorder machinery in between
 * (src/voronoi.h:78-237, src/reorder_morton.h:44-122, src/reorder.h:33-149).
 * A host driver that keeps RTParameter and the containers replaces that block
 * of main() by the calls below; the library owns all device state.
 *
 * Conventions: every call returns ORBC_OK (0) or an ORBC_ERR_* code and never
 * exits or traps; orbc_gpu_error() returns the message of the last failure on
 * a handle.  Arrays are host memory, AoS double[3 n] like the reference's
 * vect containers (src/container.h:64-73); bonds are (type, tag_i, tag_j)
 * triples like openrbc::Bond (src/container.h:30-34).  A handle is not
 * re-entrant: use it from one host thread.
 */
#ifndef ORBC_GPU_H_
#define ORBC_GPU_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orbc_handle orbc_handle;

enum {
    ORBC_OK = 0,
    ORBC_ERR_ARG = 1,          /* bad argument (the reference would rt_assert + exit(0)) */
    ORBC_ERR_CUDA = 2,         /* CUDA runtime error                                      */
    ORBC_ERR_NBR_OVERFLOW = 3, /* neighbour list overflowed its capacity                 */
    ORBC_ERR_NAN = 4,          /* non-finite coordinate                                   */
    ORBC_ERR_GRID = 5,         /* particle left an open grid (kept in the edge cell)       */
    ORBC_ERR_BOND = 6,         /* FENE / WLC bond stretched beyond its maximum            */
    ORBC_ERR_STATE = 7,        /* call out of order (e.g. step before upload)             */
    ORBC_ERR_NOMEM = 8,        /* device allocation failed                                */
    ORBC_ERR_NODEV = 9,        /* no CUDA device                                          */
    ORBC_ERR_IO = 10           /* a trajectory or checkpoint file could not be read / written */
};

enum { ORBC_PREC_FP64 = 0, ORBC_PREC_MIXED = 1 };
enum { ORBC_INT_LANGEVIN = 0, ORBC_INT_NOSE_HOOVER = 1 };
enum { ORBC_BOND_HARMONIC = 0, ORBC_BOND_FENE = 1, ORBC_BOND_WLC_POW = 2 };
#define ORBC_MAX_BOND_TYPES 8

/* Run-time parameters.  dt, kBT, eta, Q, seed keep the meaning (and the
 * defaults, see orbc_gpu_default_params) of RTParameter
 * (src/runtime_parameter.h:38-76); the compile-time switches LANGEVIN /
 * FUSED_INTEGRATOR and `real` (src/config_static.h:30-34) become the
 * integrator and precision fields. */
typedef struct {
    int precision;          /* ORBC_PREC_FP64 or ORBC_PREC_MIXED (FP32 forces, FP64 reductions) */
    int integrator;         /* ORBC_INT_LANGEVIN or ORBC_INT_NOSE_HOOVER                          */
    double dt, kBT, eta;    /* time step, thermal energy, solvent viscosity                       */
    double Q;               /* Nose-Hoover mass; 0 -> 0.01 N per system                            */
    uint64_t seed;          /* counter-based RNG key (Langevin noise)                              */
    double skin;            /* neighbour-list skin; rebuild when any particle moved > skin/2      */
    int max_neighbors;      /* initial neighbour capacity per particle (0 = automatic)            */
    int rebuild_every;      /* also rebuild at least every k steps (0 = displacement only)        */
    int bounce;             /* Nose-Hoover reflective walls at the box (src/integrate_nh.h:124-144) */
    int use_graph;          /* capture each step in a CUDA graph                                  */
    int energy;             /* accumulate the potential energy every step                         */
    /* box of a single-system upload; open axes grow to the particles' extent */
    double lo[3], hi[3];
    int periodic[3];
    /* global membrane constraints on the face mesh: F = -k (Q - Q0)/Q0 dQ/dx */
    double kv, V0, ka, A0;
    /* bond-type table: style, stiffness (harmonic K / FENE K / WLC kT/p),
       default rest length, FENE maximum extension / WLC lmax-over-r0 */
    int bond_style[ORBC_MAX_BOND_TYPES];
    double bond_K[ORBC_MAX_BOND_TYPES];
    double bond_r0[ORBC_MAX_BOND_TYPES];
    double bond_R[ORBC_MAX_BOND_TYPES];
    /* kernel forms 0..127 (bits 3 and 4 not both set): bit 0 =
       software-pipelined neighbour pass (else 2-way unrolled), bit 1 =
       non-lipid pair path inlined (else called), bit 2 = Langevin step kernel
       compiled for more resident blocks per SM (20 blocks at 48 registers,
       18 at 56 with bit 5; else 16 blocks at 64 registers), bits 3-4 = how
       the neighbour list is built: 0 per cell of a warp, 32 candidates at a
       time, entries placed by prefix count; 1
       per-particle 27-cell sweeps; 2 per warp in two phases (accept masks per
       particle, then every lane writes its own column) -- all three write the
       same list; bit 5 (32) = merged shell pass: skin-shell rows are
       distance-tested first and their hits evaluated in the loop of the inner
       rows (bit-identical results); bit 6 (64) = compensated (Kahan)
       summation of each particle's force and torque, also in the forces
       hook.  Bits 5 and 6 imply bits 0 and 1.  orbc_gpu_autotune picks the
       forms per workload */
    int kernel_variant;
    /* 1: remove each system's mean lipid velocity between the force
       evaluation and the integrator every step, as the disabled call
       integrate(zero_bulk_velocity(param), lipid) at src/openrbc.cpp:228 would
       (src/zero_bulk_velocity.h:29-56); 0 (default): off, as in the reference */
    int zero_bulk;
    /* orbc_gpu_set_state(_f32) / orbc_gpu_download(_f32): 1 (default) = when the
       caller's arrays are reachable from the GPU -- page-locked and mapped
       (cudaHostAlloc / cudaHostRegister), or ordinary pageable memory on a
       GPU that reads the host's page tables (Grace systems) -- the
       conversion kernels read and write them in place over the host link,
       with no staging copy; 0 = always copy through a device staging buffer */
    int host_direct;
} orbc_params;

/* One independent system of a batched upload (its own box and constraint). */
typedef struct {
    double lo[3], hi[3];
    int periodic[3];
    double kv, V0, ka, A0;
    double zeta;            /* initial Nose-Hoover variable */
} orbc_system_desc;

typedef struct {
    int64_t step;           /* completed steps                                           */
    int64_t n;              /* particles                                                 */
    double temperature;     /* sum m v^2 / 3N (src/compute_temperature.h:24-29)          */
    double ke2;             /* sum m v^2                                                 */
    double epot;            /* potential energy (when params.energy or after forces())  */
    double area, volume;    /* membrane mesh area and enclosed volume (FP64)            */
    double zeta;            /* Nose-Hoover thermostat variable                           */
    int64_t rebuilds;       /* neighbour-list rebuilds so far                            */
    int max_neighbors;      /* largest neighbour count at the last rebuild               */
    int capacity;           /* neighbour-list capacity per particle                      */
    int flags;              /* ORBC_ERR_* bits seen (1 << code)                           */
    int pad;
} orbc_thermo;

/* Defaults of RTParameter (src/runtime_parameter.h:47-64): kBT 0.22,
 * eta 0.01, dt 0.01, seed 0xBAD5EED; reference bond table
 * (src/forcefield_canonical.h:106-109); box +-1000 (:111-115). */
void orbc_gpu_default_params(orbc_params *p);

/* Replaces the set-up in src/openrbc.cpp:43-71 (containers, Voronoi init). */
int orbc_gpu_create(const orbc_params *p, orbc_handle **out);

/* Topology + state of one system.  Lipids are type 0, proteins 1..5
 * (src/forcefield_canonical.h:31-37); bonds3 = (type, tag_i, tag_j) refer to
 * tags (src/compute_bonded.h:109-110).  Replaces LipidContainer/ProteContainer
 * filling and TagIndexMap::build_map (src/container.h:36-58). */
int orbc_gpu_upload(orbc_handle *h, const double *x3, const double *n3, const double *v3, const double *o3,
                    const int *type, const int *tag, size_t n, const int *bonds3, size_t nb);

/* Several independent systems in one launch per step: particles of system s
 * are [offsets[s], offsets[s+1]) of the arrays; tags are unique over all
 * systems; bond_r0 (may be NULL) gives per-bond rest lengths; faces3 (may be
 * NULL) are (tag_a, tag_b, tag_c) triangles, counter-clockwise seen from
 * outside, defining each system's membrane area and volume.  No reference
 * counterpart (the reference runs one cell per process). */
int orbc_gpu_upload_batch(orbc_handle *h, int nsys, const orbc_system_desc *sys, const int64_t *offsets,
                          const double *x3, const double *n3, const double *v3, const double *o3, const int *type,
                          const int *tag, size_t n, const int *bonds3, const double *bond_r0, size_t nb,
                          const int *faces3, size_t nf);

/* Overwrite positions / orientations / velocities / angular velocities of
 * the uploaded particles (same order as the upload) without re-sending the
 * topology.  Particles within skin/2 of where the current neighbour list was
 * built keep their cell; if any moved farther, the list is rebuilt before the
 * next force evaluation.  Used when the host containers stay the source of
 * truth between steps. */
int orbc_gpu_set_state(orbc_handle *h, const double *x3, const double *n3, const double *v3, const double *o3);

/* orbc_gpu_set_state for the upload indices [first, first + count) from host
 * arrays in the reference's own container layout: AoS vectors of
 * `real` = float (src/config_static.h:34) with `stride` floats per particle,
 * 3 (vector<real,3>) or 4 (the padded _VEC4 layout, src/config_static.h:36-44).
 * The containers' x, v, n, o (src/container.h:68-72) can be passed as they
 * are: one call for the lipid range, one for the protein range.  Half the
 * bytes of the FP64 call cross the host link. */
int orbc_gpu_set_state_f32(orbc_handle *h, int64_t first, int64_t count, int stride, const float *x, const float *n,
                           const float *v, const float *o);

/* nsteps of the loop body of src/openrbc.cpp:189-242 (pair forces, bonds,
 * constraint, integrator; neighbour rebuild on demand).  out may be NULL.
 *
 * Two conditions found by a neighbour rebuild inside the call are handled
 * without an error: a list that outgrows its capacity, and a particle of a
 * system with open axes that has left that system's grid (set at upload: the
 * particles' extent plus a margin of at least a quarter of it and five list
 * cutoffs on each side; a stray lipid that leaves the membrane reaches it
 * after enough steps).  The device stops stepping at that build, so no step
 * runs on a truncated list or with a particle clamped into an edge cell; the
 * library grows the list, or re-grids the systems from the current state,
 * rebuilds, finishes the interrupted Nose-Hoover step's second half if its
 * first half ran, and runs the remaining steps, so the call still completes
 * nsteps steps.  The same holds for orbc_gpu_minimize and orbc_gpu_forces, and
 * for particles that orbc_gpu_set_state places outside the grid.
 * ORBC_ERR_NAN and ORBC_ERR_BOND stay recorded (every later step, minimize
 * and forces call returns them, and orbc_thermo.flags shows them) until the
 * next orbc_gpu_upload. */
int orbc_gpu_step(orbc_handle *h, int nsteps, orbc_thermo *out);

/* Current state in upload order (any pointer may be NULL). */
int orbc_gpu_download(orbc_handle *h, double *x3, double *n3, double *v3, double *o3);

/* orbc_gpu_download of the upload indices [first, first + count) into host
 * AoS float vectors with `stride` floats per particle (3, or 4 with the
 * fourth written as 0); the layout of orbc_gpu_set_state_f32. */
int orbc_gpu_download_f32(orbc_handle *h, int64_t first, int64_t count, int stride, float *x, float *n, float *v,
                          float *o);

/* Parity hook: forces, torques and per-particle potential energy at the
 * current state, in upload order (compute_pairwise_fused + compute_bonded,
 * src/compute_pairwise_fused.h:238-320, src/compute_bonded.h:89-146). */
int orbc_gpu_forces(orbc_handle *h, double *f3, double *t3, double *e);

/* Temperature, energy, area, volume, thermostat state of system `sys`. */
int orbc_gpu_thermo(orbc_handle *h, int sys, orbc_thermo *out);

/* Parity hook: the full neighbour list in upload order as CSR (counts[n],
 * then up to cap neighbour indices); returns the total in *total. */
int orbc_gpu_neighbors(orbc_handle *h, int *counts, int *list, int64_t cap, int64_t *total);

/* Parity hook: grid of system `sys` (origin, cell size, cell counts) and, per
 * particle in upload order, its packed cell (x | y << 11 | z << 22), its
 * offset from the cell centre and its slot in the cell-sorted device order. */
int orbc_gpu_cells(orbc_handle *h, int sys, double *lo3, double *lc3, int *nc3, int *cell, double *offset3,
                   int *slot);

/* Measured FMA throughput of the current GPU in TFLOP/s (FP32 and FP64;
 * 8 independent FMA chains per thread, every SM busy, ~10 ms): the ALU
 * roofline denominators of the force kernels.  No counterpart in the
 * reference. */
int orbc_gpu_fma_peak(double *tflops_fp32, double *tflops_fp64);

/* Force a neighbour-list rebuild now (sort + bins + list). */
int orbc_gpu_rebuild(orbc_handle *h);

/* Trajectory frame in the reference's .orbc layout (save_frame,
 * src/trajectory.h:26-105), so its reader and orbc-util read it:
 * FRAMEBEG int32 nstep, NATOM uint64 N, IDENTITY N x (int32 tag, int32 type),
 * then per `fields` bit (the reference's DumpField, src/runtime_parameter.h:
 * 30-36) POSITION (1), VELOCITY (8), ROTATION (2) as N x 3 `real`, VORONOI
 * (4) as N x int32 (the particle's grid-cell id here: there is no Voronoi
 * tessellation), FORCE (16) as N x 3 `real` (evaluated at the current state),
 * then FRAMEEND.  Particles are written lipids first, then proteins, each in
 * upload order, as the reference's save_frame(lipid, protein) does.
 * real_bytes = 4 matches the reference's default build, 8 its FP64 build.
 * append = 0 truncates the file.  async = 1 returns as soon as the frame is
 * queued: the device gathers it into a staging buffer, a second stream copies
 * it to one of two pinned host buffers and a writer thread writes it while
 * the caller goes on stepping (a third frame waits for a free buffer);
 * orbc_gpu_flush waits for the queue and reports write errors.  async = 0
 * writes before returning. */
#define ORBC_DUMP_POSITION 1
#define ORBC_DUMP_ROTATION 2
#define ORBC_DUMP_VORONOI 4
#define ORBC_DUMP_VELOCITY 8
#define ORBC_DUMP_FORCE 16
int orbc_gpu_save_frame(orbc_handle *h, const char *path, int append, int nstep, int fields, int real_bytes,
                        int async);
int orbc_gpu_flush(orbc_handle *h);

/* Checkpoint / restart (no counterpart in the reference, whose trajectory
 * lacks angular velocities, the thermostat and the RNG state): positions,
 * orientations, velocities and angular velocities (FP64, upload order), the
 * step counter that keys the noise, the RNG seed, each system's Nose-Hoover
 * zeta and the carried Nose-Hoover forces and torques.  load_checkpoint needs
 * a handle holding the same topology (orbc_gpu_upload of the same particles,
 * in the same order); the run then continues where the saved one was. */
int orbc_gpu_save_checkpoint(orbc_handle *h, const char *path);
int orbc_gpu_load_checkpoint(orbc_handle *h, const char *path);

/* Stray-lipid cleanup (delete_lipid, src/cleanup.h:29-91, called every
 * freq_cleanup steps at src/openrbc.cpp:201): lipids are affiliated with the
 * nearest generator -- the lipid centroid of a 4 x 4 x 4 tile of grid cells
 * holding at least 8 lipids, standing in for the reference's Voronoi
 * centroids -- among the surrounding tiles; per generator, a lipid is removed
 * unless its squared distance to the generator is below stray_tolerance^2
 * times the median one (a lipid with no generator within two tiles is
 * removed).  Proteins are never removed.  Survivors keep their order and are
 * renumbered 0 .. n' - 1 (upload indices, per system), as the reference's
 * compaction does; *removed receives the count.  The reference's default
 * stray_tolerance is 2.5 (src/runtime_parameter.h:51). */
int orbc_gpu_cleanup(orbc_handle *h, double stray_tolerance, int64_t *removed);

/* Energy minimisation (the loop of src/openrbc.cpp:88-146): nsteps times
 * forces, post_torque t <- n x t (src/integrate_nh.h:146-154), the
 * step-limited steepest-descent move per particle (dx = f / m, dn = t x n,
 * h = (|dx| > dr_max || |dn| > dn_max) ? min(dr_max / |dx|, dn_max / |dn|)
 * : params.dt; x += f h / m; n <- normalize(n + dn h), :113-130) and
 * bounce_back at the box walls on open axes when params.bounce (:132).  The
 * reference's defaults are nsteps = 1000 and dr_max = dn_max = 0.05
 * (src/runtime_parameter.h:56-58).  The step counter does not advance. */
int orbc_gpu_minimize(orbc_handle *h, int nsteps, double dr_max, double dn_max, orbc_thermo *out);

/* assign_temperature (src/assign_temperature.h:26-44, applied to lipids and
 * proteins at src/openrbc.cpp:160): every particle's velocity becomes
 * sqrt(2 kBT / m) g with g three unit Gaussians (the reference's factor 2 is
 * kept; pass kBT * amplify for its amplify argument).  The Gaussians come from
 * Box-Muller on one Philox4x32-10 block keyed by seed with counter (tag,
 * 0x6B8B4567, 0x327B23C6, system index), so they do not depend on the thread
 * count or the slot order (the reference draws from per-thread generators).
 * Orientations and angular velocities are untouched. */
int orbc_gpu_assign_temperature(orbc_handle *h, double kBT, uint64_t seed);

/* rdf / rdf_1peak_r (src/rdf.h:26-81): histogram of the distances of all
 * unordered pairs of system sys whose types match (type_a, type_b) in either
 * order (-1 = any type): counts[(int)(r / dr)] += 1 for r < rcut (rcut <= 0:
 * no cutoff) and bin < nbins; other pairs are counted in *dropped (the
 * reference writes past its 10,000 bins instead).  The reference's `rdf` is
 * type_a = type_b = -1 over one container, dr = 0.1, nbins = 10000;
 * `rdf_1peak_r` is type 4 with itself, dr = 0.5, rcut = 25, 51 bins.
 * Distances are evaluated in the handle's precision (FP32 for
 * ORBC_PREC_MIXED, as the reference's default `real`; FP64 otherwise) from
 * coordinates relative to the centre of the system's box, with the minimum
 * image on periodic axes (the reference has none).  All pairs are visited
 * (O(N^2), as in the reference).  The caller normalises: the reference writes
 * r = dr i and counts[i] / (4 * 3.14 * r^2 * dr) to rdf.txt. */
int orbc_gpu_rdf(orbc_handle *h, int sys, int type_a, int type_b, double dr, int nbins, double rcut,
                 uint64_t *counts, int64_t *dropped);

/* Milliseconds of device time of the last orbc_gpu_step call, and the number
 * of kernel launches it issued (graph nodes included). */
int orbc_gpu_last_timing(orbc_handle *h, double *ms, int64_t *launches);

/* Per-kernel device times over nsteps un-captured steps (CUDA events around
 * each launch group on the library's stream; a synchronisation per step).
 * No reference counterpart (the reference's Timers, src/timer.h:26-69, time
 * whole routines on the host). */
typedef struct {
    int64_t steps;            /* steps profiled                                   */
    int64_t rebuilds;         /* neighbour rebuilds among them                    */
    double step_kernel_ms;    /* mean time of the fused force + integrator kernel */
    double rebuild_ms;        /* mean time of one full rebuild chain              */
    double gate_ms;           /* mean time of the rebuild chain when it was skipped */
    double mesh_ms;           /* mean time of the area / volume kernel            */
    double mean_neighbors;    /* mean neighbour-list length per particle          */
    double pairs_in_cutoff;   /* mean partners inside the interaction range       */
    double rebin_ms, sort_ms, gather_ms, nlist_ms;  /* rebuild stages (mean per rebuild) */
} orbc_profile;
int orbc_gpu_profile(orbc_handle *h, int nsteps, orbc_profile *out);

/* Autotuner: times trial_steps graph-captured steps per candidate from a
 * snapshot of the current state, keeps the fastest, and restores the snapshot
 * (state, step counter, thermostat), so the simulation does not advance.
 * Dimensions, in order: the list-build form (bits 3-4) at the caller's skin;
 * with it, neighbour-list
 * skin (0.3, 0.45, 0.6, 0.8, 1.0) x force-loop form (kernel_variant bits 0-1,
 * and the merged shell pass, bit 5); the two skins half-way to the best one's
 * neighbours; the occupancy form (bit 2); the other list-build forms again;
 * and the rebuild cadence (rebuild_every 0 = only when a particle moved more
 * than skin/2, else also every 5 or 10 steps).  Compensated accumulation (bit 6) is an accuracy
 * choice and is kept as the caller set it.  trials (may be NULL) receives up
 * to max_trials rows.  No reference counterpart (the reference's cadences are
 * fixed command-line values, src/runtime_parameter.h:57-60). */
typedef struct {
    double skin;
    int variant;        /* kernel_variant of the trial */
    int rebuild_every;  /* rebuild cadence of the trial */
    double ms_per_step;
    double rebuilds_per_step;
} orbc_tune_trial;
int orbc_gpu_autotune(orbc_handle *h, int trial_steps, orbc_tune_trial *trials, int max_trials, int *ntrials);

/* Reference Morton key of n points (src/reorder_morton.h:25-42; bsize3 is
 * RTParameter::bsize, 2000 per axis) and the stable order by (key, index)
 * that reorder_morton (src/reorder_morton.h:44-122) sorts by. */
int orbc_gpu_morton_encode(const double *p3, int64_t n, const double *bsize3, uint32_t *keys);
int orbc_gpu_morton_order(const double *p3, int64_t n, const double *bsize3, int32_t *order);

/* orbc_gpu_morton_order for callers that cannot allocate device memory.
 * No counterpart in the reference.  Some callers may not call cudaMalloc /
 * cudaFree: programs whose device memory belongs to another allocator (for
 * example a framework's caching pool that must be the only allocator), and
 * latency-bound loops that cannot afford the device synchronisation those
 * calls imply.  Here the caller passes device pointers: d_p3 holds n points
 * (AoS double[3n]) and d_order receives the stable (key, index) order;
 * bsize3 is host memory.  The sort's scratch lives in one fixed array of
 * about 3.1 MB in the library's device memory, present on every GPU that
 * loads the library until the process exits; nothing is allocated per call.
 * n above ORBC_NOALLOC_MAX_POINTS returns ORBC_ERR_ARG.  The first call on a
 * device looks up that array's device address (with the device current) and
 * caches it with the context's id, so a call after cudaDeviceReset looks it up
 * again; make the first call on a device (and the first after a reset) before
 * any stream capture.  A CUDA error already pending when the call starts is
 * reported (ORBC_ERR_CUDA) and left pending; orbc_gpu_error(NULL) gives the
 * message of any failure.  Work is queued on
 * `stream` (a cudaStream_t, NULL for the default stream) and the call returns
 * without waiting.  All calls share the one scratch array: calls whose work
 * overlaps on the GPU (other streams, other host threads) race and corrupt
 * each other's results, so order them on one stream. */
#define ORBC_NOALLOC_MAX_POINTS 262144
int orbc_gpu_morton_order_noalloc(const double *d_p3, int64_t n, const double *bsize3, int32_t *d_order,
                                  void *stream);

/* Whole-cell initialiser: init_rbc (src/init_rbc.h:29-305) for a
 * triangulated mesh.  The protein network is built on the host and the
 * lipids are placed on the GPU.
 *
 * orbc_init_rbc_sizes: proteins (2 nvert + 20 nbond: glycophorin and actin
 * per vertex, band-III and 19 spectrin beads per edge) and bonds
 * (nvert + 21 nbond) of the network.
 *
 * orbc_init_rbc_network (host, src/init_rbc.h:66-233): rescales the mesh so
 * that its mean edge is 80 nm in reduced units, computes face, vertex and
 * edge normals, and writes the proteins in the reference's order.
 *   - Proteins: x3, n3, type, tag (tags 1 .. nprotein), followed by their
 *     bonds3 (type, tag_i, tag_j).
 *   - face_nl: lipids per face, int(area * rho) (:262-264); nlipid: their sum.
 *   - vert3_out, fnorm3_out: the scaled vertices and the face normals.
 * Any output may be NULL; with x3 NULL only the sizes and mesh data are
 * written.  The spectrin noise (+-0.05 per coordinate) comes from
 * Philox4x32-10 keyed by `seed` with counter (edge, bead), where the
 * reference uses its sequential generator.
 *
 * orbc_gpu_place_lipids (GPU, src/init_rbc.h:235-305): face f receives
 * face_nl[f] lipids, uniform on the triangle. A lipid is redrawn until it is
 *   - at least min_dist_lp (ForceField::reqlp[1] = 1.685 there) from the
 *     face's first vertex and from every protein in prot3, and
 *   - at least min_dist (0.55) from the face's earlier lipids.
 * Its normal is the face normal.  Output is in face order: x3, n3
 * (sum face_nl entries).  Attempt k of lipid j of face f draws from
 * Philox4x32-10 keyed by `seed` with counter (f, j, k), and the first clean
 * attempt wins, so the result does not depend on the parallel layout.  A
 * lipid that finds no room after 8,192 attempts returns ORBC_ERR_ARG, where
 * the reference would retry forever. */
int orbc_init_rbc_sizes(int64_t nvert, int64_t nbond, int64_t *nprotein, int64_t *nbonds);
int orbc_init_rbc_network(const double *vert3, int64_t nvert, const int *bond2, int64_t nbond, const int *face3,
                          int64_t nface, double rho, uint64_t seed, double *vert3_out, double *fnorm3_out,
                          double *x3, double *n3, int *type, int *tag, int *bonds3, int64_t *face_nl,
                          int64_t *nlipid);
int orbc_gpu_place_lipids(const double *vert3, int64_t nvert, const int *face3, const double *fnorm3, int64_t nface,
                          const int64_t *face_nl, const double *prot3, int64_t nprot, double min_dist,
                          double min_dist_lp, uint64_t seed, double *x3, double *n3);

int orbc_gpu_destroy(orbc_handle *h);
const char *orbc_gpu_error(orbc_handle *h);   /* NULL handle -> last create/standalone error */
const char *orbc_gpu_version(void);

#ifdef __cplusplus
}
#endif

#endif
