// Device-side data layout shared by the kernels and the host engine.
//
// Particle state lives on the GPU in "slots": each system (one cell, one
// vesicle, one lattice) owns a contiguous slot range padded to a multiple of
// SYS_PAD so that every 256-slot block belongs to exactly one system.  Padding
// slots are ghosts (type GHOST) that never enter a cell or a neighbour list.
//
// Positions are stored as an integer grid cell (packed 11/11/10 bits) plus an
// offset from that cell's centre in the working precision R (float for the
// mixed form, double for the plain FP64 form).  Neighbour-list entries carry
// the cell shift between the two particles (27 codes, periodic images
// included), so a pair separation is (o_i - o_j) + shift * Lc without ever
// forming an absolute coordinate.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace orbc {

constexpr int NT = 6;            // particle types (src/forcefield_canonical.h:31-37)
constexpr int GHOST = 15;        // type of padding slots
constexpr int SYS_PAD = 256;     // slot padding per system
constexpr int LITE_BS = 64;      // threads per block of the force / integrator kernels
constexpr int MAX_BT = 8;        // bond types
constexpr int MAX_DEG = 15;      // bonds / faces per particle (4-bit fields)
constexpr uint32_t NB_MASK = (1u << 27) - 1u;
constexpr int NB_SHIFT = 27;
constexpr int MAX_SLOTS = 1 << 27;
constexpr int NPART = 8;         // per-warp partial sums: ke2, epot, maxd2, flags, lipid sum v (3), pad
constexpr int RED_GROUP = 256;   // warp partials (of 32 slots) per reduction group
constexpr int MESH_CHUNK = 256;  // faces per block of the area / volume kernel (one per thread: the FP64 work spreads over all SMs)

enum : int {
    ERRB_NBR_OVERFLOW = 1,  // a neighbour list overflowed its capacity
    ERRB_NAN = 2,           // non-finite coordinate after a step
    ERRB_GRID = 4,          // particle outside an open grid (clamped to the edge cell)
    ERRB_BOND = 8,          // FENE / WLC bond beyond its maximum extension
};

enum : int { BOND_HARMONIC = 0, BOND_FENE = 1, BOND_WLC_POW = 2 };
enum : int { PAIR_NONE = 0, PAIR_ANISO = 1, PAIR_REP = 2 };

struct __align__(32) double4a {
    double x, y, z, w;
};
template<class R> struct Vec;
template<> struct Vec<float> {
    using T4 = float4;
};
template<> struct Vec<double> {
    using T4 = double4a;
};

// w word of a position record: type (4 bits) | bond degree << 4 | face degree << 8
__host__ __device__ inline int w_type(int w) { return w & 15; }
__host__ __device__ inline int w_bdeg(int w) { return (w >> 4) & 15; }
__host__ __device__ inline int w_fdeg(int w) { return (w >> 8) & 15; }

__device__ __forceinline__ int wbits(float w) { return __float_as_int(w); }
__device__ __forceinline__ int wbits(double w) { return int(__double_as_longlong(w)); }
__device__ __forceinline__ void wset(float &w, int b) { w = __int_as_float(b); }
__device__ __forceinline__ void wset(double &w, int b) { w = __longlong_as_double((long long)(unsigned)b); }

// packed cell coordinates (x: 11 bits, y: 11 bits, z: 10 bits)
__host__ __device__ inline int cpack(int x, int y, int z) { return x | (y << 11) | (z << 22); }
__host__ __device__ inline int cx_of(int c) { return c & 2047; }
__host__ __device__ inline int cy_of(int c) { return (c >> 11) & 2047; }
__host__ __device__ inline int cz_of(int c) { return (c >> 22) & 1023; }
constexpr int MAX_NC_XY = 2047, MAX_NC_Z = 1023;

/* Neighbour list layout: warp-blocked ELL.  The entries of the 32 slots of a
 * warp form one contiguous block of cap rows x 32 entries, so entry k of slot
 * i is at nbr_index(i, k, cap); a warp's whole list is cap * 128 contiguous bytes. */
__host__ __device__ inline int64_t nbr_index(int i, int k, int cap) {
    return ((int64_t(i >> 5) * cap + k) << 5) | int64_t(i & 31);
}

struct BondSlot {
    int partner;  // slot of the other end
    int type;     // bond type (table index)
    double r0;    // rest length
};

template<class R> struct PairP {
    R cutsq, cut, rep8, att4, alpha, aatt, ljcutsq, lj1, lj2, rep, att;
    R anysq;  // max(cutsq, ljcutsq): the pair interacts somehow inside it
    int kind;
    int pad2;
};

template<class R> struct BondP {
    R K, Rm;
    int style, pad;
};

template<class R> struct FFDev {
    PairP<R> pair[NT * NT];        // by (ti * NT + tj)
    R mass[NT], inv_mass[NT], gamma[NT], sigma[NT];
    BondP<R> bond[MAX_BT];
    float rlist2[16 * 16];          // neighbour-list cutoff^2 (cut + skin)^2, 0 = never
    float rin2[16 * 16];            // interaction range^2: list entries inside it go to the inner rows
};

struct SysDev {
    double lo[3], Lc[3];            // grid origin and cell size
    double wlo[3], whi[3];          // reflective walls (Nose-Hoover bounce-back)
    int nc[3], per[3];
    int ntile[3], pad0;             // 4 x 4 x 4 tiles of cells per axis (cell-id order)
    unsigned cell_base;             // first global cell id; ncell + 1 ids (last = ghost cell)
    int off, npad, nreal;
    int face_begin, face_end;
    int mblk_begin, mblk_end;       // blocks of the area / volume kernel (MESH_CHUNK faces each)
    int nlipid, pad1;               // lipids in the system (bulk-velocity removal)
    int gbase, ngrp;                // reduction groups of RED_GROUP warps (first, count)
    double kv, V0, ka, A0, Q;
    double invLc[3];                // 1 / Lc
    float Lcf[3], invLcf[3];        // Lc and 1 / Lc rounded to float
};

/* Cell size and its inverse in the working precision (the FP32 kernels take
 * them ready-made: a per-particle FP64 division or conversion would run on
 * the FP64 pipe). */
template<class R> __device__ __forceinline__ R lc_of(const SysDev &s, int d);
template<> __device__ __forceinline__ float lc_of<float>(const SysDev &s, int d) { return s.Lcf[d]; }
template<> __device__ __forceinline__ double lc_of<double>(const SysDev &s, int d) { return s.Lc[d]; }
template<class R> __device__ __forceinline__ R inv_lc_of(const SysDev &s, int d);
template<> __device__ __forceinline__ float inv_lc_of<float>(const SysDev &s, int d) { return s.invLcf[d]; }
template<> __device__ __forceinline__ double inv_lc_of<double>(const SysDev &s, int d) { return s.invLc[d]; }

/* Cell id inside a system: 4 x 4 x 4 tiles of cells in row-major tile
 * order, Morton (x, y, z interleaved) inside a tile.  Particles are sorted by
 * cell id, so 32 consecutive slots sit in a compact clump of cells (a warp's
 * neighbourhood), unlike row-major order where a warp strings along a row. */
__host__ __device__ __forceinline__ unsigned tile_spread2(unsigned v) { return (v & 1u) | ((v & 2u) << 2); }
__host__ __device__ __forceinline__ unsigned cell_code(const SysDev &s, int x, int y, int z) {
    const unsigned tile =
        unsigned(x >> 2) + unsigned(s.ntile[0]) * (unsigned(y >> 2) + unsigned(s.ntile[1]) * unsigned(z >> 2));
    return (tile << 6) | tile_spread2(unsigned(x) & 3u) | (tile_spread2(unsigned(y) & 3u) << 1) |
           (tile_spread2(unsigned(z) & 3u) << 2);
}
/* ids per system (tiles x 64); id cell_base + ncell_ids is the ghost id */
__host__ __device__ __forceinline__ unsigned ncell_ids(const SysDev &s) {
    return unsigned(s.ntile[0]) * unsigned(s.ntile[1]) * unsigned(s.ntile[2]) * 64u;
}

struct SysState {
    double zeta;        // Nose-Hoover thermostat variable
    double ke2;         // sum m v^2 after the last integration
    double epot;        // potential energy (when accumulated)
    double area, volume;
    double cv, ca;      // constraint coefficients -k (Q - Q0) / Q0 used by the next forces
    double vcom[3];     // mean lipid velocity removed before the next integration
    double pad;
};

struct Scalars {
    int cur, lp, rebuild, error;
    int max_nnb, out_of_grid, cond_hint;
    int nh_half;          // 1 between a Nose-Hoover first half and its second half
    unsigned int blk_counter, mesh_counter;
    unsigned int iters;   // completed steps or minimisation iterations (k_advance, k_reduce)
    unsigned int pad3;
    long long step, rebuilds, since_rebuild, pad4;
};

/* The last list build found a list longer than its capacity, or a particle
 * outside its system's open grid: the step kernels then leave the state
 * untouched (and the step counters unchanged) until the host has grown the
 * list or re-gridded the system and rebuilt, so that no step is computed on a
 * truncated list or with a particle clamped into an edge cell.  The flags are
 * written only by the list build (and by set_state), so every thread of a step
 * kernel reads the same value. */
__device__ __forceinline__ bool halted(const Scalars *S) {
    return (__ldcg(&S->error) & (ERRB_NBR_OVERFLOW | ERRB_GRID)) != 0;
}

template<class R> struct KArgs {
    using T4 = typename Vec<R>::T4;
    // particle arrays; pos/nrm ping-pong on Scalars::cur, the rest on Scalars::lp
    T4 *pos[2], *nrm[2], *vel[2], *omg[2], *frc[2], *trq[2], *xref[2];
    int *cell[2], *tag[2], *home[2];
    BondSlot *bond[2];
    int2 *fslot[2];
    double *epart;           // per-slot energy (forces hook)
    int4 *faces;             // (a, b, c, sys) slots of the area/volume mesh
    int nfaces;
    int nmblk;               // blocks of the area / volume kernel
    int *mesh_blk_sys;       // system of each of those blocks
    double *mesh_partial;    // [nmblk][2] area, volume
    uint32_t *nbr;           // warp-blocked ELL neighbour list (nbr_index)
    int *nnb;                // inner count | shell count << 16 (see k_nlist)
    int cap;
    int2 *ranges;            // cell -> [begin, end) of its slots
    int *slot_of_home;
    int *blk_sys;            // system of each 256-slot block
    double *partial;         // [npad / 32][NPART]: warp partials
    double *gpartial;        // [ngroups][NPART]: sums of RED_GROUP consecutive warps of one system
    int ngroups;
    Scalars *S;
    SysDev *sys;
    SysState *ss;
    int nsys, npad;
    // radix sort scratch
    uint32_t *skey[2];
    int *sval[2];
    int *counts, *digit_total, *inv;
    int sort_passes, ntiles;
    // parameters
    double dt, kBT;
    R skin_half2;
    uint64_t seed;
    int rebuild_every;
    int variant;             // force-kernel form (see launch_step_langevin)
    int carry_forces;        // forces / torques persist between kernels (Nose-Hoover)
    int zero_bulk;           // remove the mean lipid velocity before integrating
    int nlist_lane;          // list-build form: 0 per cell of a warp, 1 per-lane 27-cell sweep, 2 two-phase
    const FFDev<R> *ff;      // force-field tables (global)
    PairP<R> ll;             // the lipid-lipid pair, in kernel-parameter space: read as constant operands,
                             // so the bulk pair path keeps no registers for its parameters
};

// host-side launchers (explicitly instantiated for float and double)
template<class R> void launch_rebuild(const KArgs<R> &a, cudaStream_t st, bool gated);
// stage 0 rebin, 1 radix sort, 2 ranges + gather, 3 neighbour list
template<class R> void launch_rebuild_stage(const KArgs<R> &a, cudaStream_t st, bool gated, int stage);
template<class R> void launch_mesh(const KArgs<R> &a, cudaStream_t st);
template<class R> void launch_step_langevin(const KArgs<R> &a, cudaStream_t st, bool energy);
template<class R> void launch_nh_final(const KArgs<R> &a, cudaStream_t st, bool energy);
template<class R> void launch_nh_initial(const KArgs<R> &a, cudaStream_t st);
template<class R> void launch_nh_prologue(const KArgs<R> &a, cudaStream_t st);
template<class R> void launch_forces(const KArgs<R> &a, cudaStream_t st);
template<class R> void launch_vcom(const KArgs<R> &a, cudaStream_t st);
template<class R> void launch_minimize(const KArgs<R> &a, double dr_opt, double dn_opt, cudaStream_t st);
template<class R>
void launch_frame_pack(const KArgs<R> &a, const int *file_of_home, int real_bytes, void *pos, void *vel, void *rot,
                       int *cell, void *frc, cudaStream_t st);
template<class R>
int launch_cleanup_mark(const KArgs<R> &a, int mingen, double tol2, double4a *gen, double *dr2, int *gone_home,
                        unsigned long long *removed, cudaStream_t st);
template<class R> void launch_cleanup_apply(const KArgs<R> &a, const int *newidx, int *soh_new, cudaStream_t st);
template<class R> void launch_set_carried(const KArgs<R> &a, const double *f3, const double *t3, int64_t nhome,
                                          cudaStream_t st);
template<class R>
cudaError_t launch_rdf(const double *x3, const int *type, int n, const double centre[3], const double L[3], int ta,
                       int tb, double dr, int nbins, double rcut, unsigned long long *counts,
                       unsigned long long *dropped, void *work, cudaStream_t st);
template<class R> void launch_assign_temperature(const KArgs<R> &a, double kT, uint64_t seed, cudaStream_t st);

// upload indices [k0, k1) of caller-order AoS arrays that start at upload
// index `first`, `stride` values of TH (double or float) per particle
template<class R, class TH>
void launch_set_state(const KArgs<R> &a, const TH *x, const TH *n, const TH *v, const TH *o, int64_t k0, int64_t k1,
                      int64_t first, int stride, cudaStream_t st);
template<class R, class TH>
void launch_download(const KArgs<R> &a, int64_t h0, int64_t h1, int64_t first, int stride, TH *x, TH *n, TH *v, TH *o,
                     TH *f, TH *t, double *e, cudaStream_t st);
// the same two transfers reading / writing host arrays the GPU can reach, in tiles
template<class R, class TH>
void launch_set_state_host(const KArgs<R> &a, const TH *x, const TH *n, const TH *v, const TH *o, int64_t k0,
                           int64_t k1, int64_t first, int stride, cudaStream_t st);
template<class R, class TH>
void launch_download_host(const KArgs<R> &a, int64_t h0, int64_t h1, int64_t first, int stride, TH *x, TH *n, TH *v,
                          TH *o, cudaStream_t st);
// full-size FP64 vectors of 3 (first = 0, stride = 3)
template<class R> void launch_download(const KArgs<R> &a, int64_t h0, int64_t h1, double *x, double *n, double *v,
                                       double *o, double *f, double *t, double *e, cudaStream_t st);
void launch_set_cond(cudaGraphConditionalHandle h, Scalars *S, cudaStream_t st);
void launch_morton(const double *p3, int64_t n, const double *bsize3, uint32_t *keys, cudaStream_t st);
// LSD radix sort of (key, index) pairs, stable; returns the buffer index (0/1) holding the result.
int radix_sort_pairs(uint32_t *keys[2], int *vals[2], int *counts, int *digit_total, int *inv, int64_t n,
                     int passes, int ntiles, const int *gate, cudaStream_t st);
int sort_tiles(int64_t n);
constexpr int SORT_TILE = 4096;
// message of the handle-less entry points, read back by orbc_gpu_error(NULL)
void set_standalone_error(const char *what, const char *detail);

}  // namespace orbc
