// Per-step kernels: the fused force evaluation (anisotropic lipid pair
// potential, lipid-protein, LJ, protein-protein, bonds, global area/volume
// constraint) and the integrators, one thread per particle slot over a full
// neighbour list -- every force and torque is accumulated in registers by the
// thread that owns the particle, so no atomics are needed.
//
//   k_step_langevin   forces + src/integrate_langevin.h:105-146 (one launch per
//                     step; positions ping-pong between two buffers)
//   k_nh_final        forces + post_toque_final_update (src/integrate_nh.h:237-273)
//   k_nh_initial      verlet_initial_bounce_clearforce_update (:178-235)
//   k_forces          forces only (parity hook)
//   k_mesh            FP64 membrane area and enclosed volume per system
//
// Per-system sums are deterministic and take two launches: each warp of a
// step kernel reduces its 32 particles with shuffles and stores one warp
// partial (warp_partials); k_reduce, launched next on the stream, adds the
// warp partials of each reduction group in a fixed tree, and its last block
// adds each system's group sums in a fixed order and applies the thermostat,
// the rebuild rule, the step counter and the buffer parity.  The lite Langevin
// kernel keeps no sums: each warp raises the rebuild flag itself and
// k_advance flips the buffers.
#include "orbc_device.cuh"

namespace orbc {

namespace {

template<class R> struct R3 {
    R x, y, z;
};

template<class R> __device__ __forceinline__ typename Vec<R>::T4 ldg4(const typename Vec<R>::T4 *p);
template<> __device__ __forceinline__ float4 ldg4<float>(const float4 *p) { return __ldg(p); }
template<> __device__ __forceinline__ double4a ldg4<double>(const double4a *p) {
    const double2 a = __ldg(reinterpret_cast<const double2 *>(p));
    const double2 b = __ldg(reinterpret_cast<const double2 *>(p) + 1);
    double4a r;
    r.x = a.x;
    r.y = a.y;
    r.z = b.x;
    r.w = b.y;
    return r;
}

/* Streaming (evict-first) access for data touched once per step -- the
 * velocity / reference-position state and the neighbour rows of the plain
 * loops -- so that it does not push out of L2 the positions and orientations
 * that the next step gathers again.  The skin-shell rows, and the inner rows
 * of the merged loop, which every warp prefetches into L1 first, are read
 * through the read-only path instead (0.735 against 0.744 ms for the merged
 * form on the 4.03M cell). */
template<class R> __device__ __forceinline__ typename Vec<R>::T4 ldcs4(const typename Vec<R>::T4 *p);
template<> __device__ __forceinline__ float4 ldcs4<float>(const float4 *p) { return __ldcs(p); }
template<> __device__ __forceinline__ double4a ldcs4<double>(const double4a *p) {
    const double2 a = __ldcs(reinterpret_cast<const double2 *>(p));
    const double2 b = __ldcs(reinterpret_cast<const double2 *>(p) + 1);
    double4a r;
    r.x = a.x;
    r.y = a.y;
    r.z = b.x;
    r.w = b.y;
    return r;
}
__device__ __forceinline__ void stcs4(float4 *p, const float4 &v) { __stcs(p, v); }
__device__ __forceinline__ void stcs4(double4a *p, const double4a &v) {
    __stcs(reinterpret_cast<double2 *>(p), make_double2(v.x, v.y));
    __stcs(reinterpret_cast<double2 *>(p) + 1, make_double2(v.z, v.w));
}

__device__ __forceinline__ void inv_sqrt(float r2, float &r, float &rinv) {
    rinv = rsqrtf(r2);
    r = r2 * rinv;
}
/* FP64: 1/sqrt(r2) by Newton's iteration for the reciprocal square root,
 * y <- y (3 - r2 y^2) / 2, started from the FP32 hardware estimate.  The
 * relative error e goes to about 1.5 e^2 per step (1e-7 -> 2e-14 -> below
 * the FP64 rounding), so two steps leave only a few ulp of rounding; the
 * callers pass pair distances 1e-5 < r2 < 100, well inside the FP32 range.
 * It takes fewer FP64 operations than a correctly rounded square root and
 * division, which bound the plain FP64 step (3 % of its time on the 4.03M
 * cell; forces change by 9e-16 relative). */
__device__ __forceinline__ void inv_sqrt(double r2, double &r, double &rinv) {
    double y = double(rsqrtf(float(r2)));
    y = y * (1.5 - 0.5 * r2 * y * y);
    y = y * (1.5 - 0.5 * r2 * y * y);
    rinv = y;
    r = r2 * y;
}
__device__ __forceinline__ float rnorm3(float x, float y, float z) { return rsqrtf(x * x + y * y + z * z); }
__device__ __forceinline__ double rnorm3(double x, double y, double z) { return 1.0 / sqrt(x * x + y * y + z * z); }

/* Anisotropic poly 4-8 pair seen from particle i (src/pairwise_kernel.h:30-68,
 * src/pairwise_kernel_fused.h:22-61).  dx = x_i - x_j. */
template<class R, bool E>
__device__ __forceinline__ void aniso(const PairP<R> &P, R dx, R dy, R dz, R r2, R nix, R niy, R niz, R njx, R njy,
                                      R njz, R3<R> &f, R3<R> &t, R &e) {
    R r, rinv;
    inv_sqrt(r2, r, rinv);
    const R ux = dx * rinv, uy = dy * rinv, uz = dz * rinv;
    const R ninj = nix * njx + niy * njy + niz * njz;
    const R niu = nix * ux + niy * uy + niz * uz;
    const R nju = njx * ux + njy * uy + njz * uz;
    const R A = R(1) + P.alpha * (ninj - niu * nju - R(1));
    const R rc = P.cut - r;
    const R rc3 = rc * rc * rc;
    const R rc4 = rc * rc3;
    const R rc7 = rc3 * rc4;
    const R pix = nix - niu * ux, piy = niy - niu * uy, piz = niz - niu * uz;
    const R pjx = njx - nju * ux, pjy = njy - nju * uy, pjz = njz - nju * uz;
    const R alphaua = P.aatt * rc4;
    const R alphauar = alphaua * rinv;
    const R fra = P.rep8 * rc7 + A * P.att4 * rc3;
    f.x += fra * ux + alphauar * (nju * pix + niu * pjx);
    f.y += fra * uy + alphauar * (nju * piy + niu * pjy);
    f.z += fra * uz + alphauar * (nju * piz + niu * pjz);
    t.x -= alphaua * pjx;
    t.y -= alphaua * pjy;
    t.z -= alphaua * pjz;
    if (E) e += R(0.5) * (P.rep * rc4 * rc4 + A * P.att * rc4);
}

/* Lennard-Jones with the WCA cut (src/pairwise_kernel_fused.h:63-77). */
template<class R, bool E>
__device__ __forceinline__ void ljf(const PairP<R> &P, R dx, R dy, R dz, R r2, R3<R> &f, R &e) {
    const R r2inv = R(1) / r2;
    const R r6inv = r2inv * r2inv * r2inv;
    const R fpair = r6inv * (P.lj1 * r6inv - P.lj2) * r2inv;
    f.x += dx * fpair;
    f.y += dy * fpair;
    f.z += dz * fpair;
    if (E) e += R(0.5) * r6inv * (P.lj1 * (R(1) / R(12)) * r6inv - P.lj2 * (R(1) / R(6)));
}

/* Protein-protein repulsion (src/pairwise_kernel_fused.h:79-97). */
template<class R, bool E>
__device__ __forceinline__ void repf(const PairP<R> &P, R dx, R dy, R dz, R r2, R3<R> &f, R &e) {
    R r, rinv;
    inv_sqrt(r2, r, rinv);
    const R rc = P.cut - r;
    const R rc3 = rc * rc * rc;
    const R rc4 = rc * rc3;
    const R fr = P.rep8 * rc3 * rc4 * rinv;
    f.x += fr * dx;
    f.y += fr * dy;
    f.z += fr * dz;
    if (E) e += R(0.5) * P.rep * rc4 * rc4;
}

/* Dispatch of src/compute_pairwise_fused.h:91-236 for a non lipid-lipid pair. */
template<class R, bool E>
__device__ __forceinline__ void pair_general_body(const PairP<R> &P, R dx, R dy, R dz, R r2, R nix, R niy, R niz,
                                                  R njx, R njy, R njz, R3<R> &f, R3<R> &t, R &e) {
    if (!(r2 > R(1e-5))) return;
    if (r2 < P.cutsq) {
        if (P.kind == PAIR_ANISO)
            aniso<R, E>(P, dx, dy, dz, r2, nix, niy, niz, njx, njy, njz, f, t, e);
        else
            repf<R, E>(P, dx, dy, dz, r2, f, e);
    } else if (r2 < P.ljcutsq) {
        ljf<R, E>(P, dx, dy, dz, r2, f, e);
    }
}
template<class R, bool E>
__device__ __noinline__ void pair_general_call(const PairP<R> &P, R dx, R dy, R dz, R r2, R nix, R niy, R niz,
                                               R njx, R njy, R njz, R3<R> &f, R3<R> &t, R &e) {
    pair_general_body<R, E>(P, dx, dy, dz, r2, nix, niy, niz, njx, njy, njz, f, t, e);
}
/* INL: inline the rare non-lipid path (more registers, no call) or call it. */
template<class R, bool E, bool INL>
__device__ __forceinline__ void pair_general(const PairP<R> &P, R dx, R dy, R dz, R r2, R nix, R niy, R niz, R njx,
                                             R njy, R njz, R3<R> &f, R3<R> &t, R &e) {
    if (INL)
        pair_general_body<R, E>(P, dx, dy, dz, r2, nix, niy, niz, njx, njy, njz, f, t, e);
    else
        pair_general_call<R, E>(P, dx, dy, dz, r2, nix, niy, niz, njx, njy, njz, f, t, e);
}

__device__ __forceinline__ int wrap_delta(int d, int n) {
    if (2 * d >= n) return d - n;
    if (2 * d < -n) return d + n;
    return d;
}

/* x_j - x_i from the packed cells and offsets (minimum image on periodic axes). */
template<class R, class T4>
__device__ __forceinline__ void rel_pos(const SysDev &sd, int cj, int ci, const T4 &pj, const T4 &pi, R &dx, R &dy,
                                        R &dz) {
    int d0 = cx_of(cj) - cx_of(ci), d1 = cy_of(cj) - cy_of(ci), d2 = cz_of(cj) - cz_of(ci);
    if (sd.per[0]) d0 = wrap_delta(d0, sd.nc[0]);
    if (sd.per[1]) d1 = wrap_delta(d1, sd.nc[1]);
    if (sd.per[2]) d2 = wrap_delta(d2, sd.nc[2]);
    dx = R(d0) * lc_of<R>(sd, 0) + (pj.x - pi.x);
    dy = R(d1) * lc_of<R>(sd, 1) + (pj.y - pi.y);
    dz = R(d2) * lc_of<R>(sd, 2) + (pj.z - pi.z);
}

/* Bond force on i, F_i = kappa(r) (x_j - x_i):  HARMONIC is
 * src/compute_bonded.h:109-115; FENE (expand form) and WLC + 1/r^2 (zero
 * force at r0) are the spectrin springs of the whole-cell workloads. */
template<class R, bool E>
__device__ __forceinline__ R bond_kappa(const BondP<R> &B, R r0, R r, R &e, int &flags) {
    if (B.style == BOND_HARMONIC) {
        if (E) e += R(0.25) * B.K * (r - r0) * (r - r0);
        return B.K * (R(1) - r0 / r);
    } else if (B.style == BOND_FENE) {
        const R s = (r - r0) / B.Rm;
        R s2 = s * s;
        if (s2 >= R(0.99)) {
            flags |= ERRB_BOND;
            s2 = R(0.99);
        }
        if (E) e += R(-0.25) * B.K * B.Rm * B.Rm * R(log(1.0 - double(s2)));
        return B.K * (r - r0) / (r * (R(1) - s2));
    } else {
        const R lmax = B.Rm * r0;
        R x = r / lmax;
        if (x >= R(0.99)) {
            flags |= ERRB_BOND;
            x = R(0.99);
        }
        const R x0 = r0 / lmax;
        const R omx = R(1) - x, omx0 = R(1) - x0;
        const R fw = B.K * (R(0.25) / (omx * omx) - R(0.25) + x);
        const R fw0 = B.K * (R(0.25) / (omx0 * omx0) - R(0.25) + x0);
        const R q = r0 / r;
        if (E) {
            const R uw = B.K * lmax * (x * x * R(0.5) + R(0.25) / (R(1) - x) - x * R(0.25) - R(0.25));
            e += R(0.5) * (uw + fw0 * r0 * q);
        }
        return (fw - fw0 * q * q) / r;
    }
}

/* Bring the used rows of this warp's block of neighbour entries (read once
 * per step) into L1 ahead of the pair loops, so the loops' entry loads do not
 * wait on DRAM.  packed = inner count | shell count << 16.  All 32 lanes must
 * call it. */
__device__ __forceinline__ void prefetch_warp_list(const uint32_t *nbr, int i, int cap, int packed) {
    const int rin = __reduce_max_sync(0xffffffffu, unsigned(packed & 0xffff));
    const int rout = __reduce_max_sync(0xffffffffu, unsigned(packed >> 16));
    const uint32_t *base = nbr + nbr_index(i & ~31, 0, cap);
    for (int r = int(threadIdx.x & 31); r < rin + rout; r += 32) {
        const int row = r < rin ? r : cap - 1 - (r - rin);
        asm volatile("prefetch.global.L1 [%0];" ::"l"(base + 32 * row));
    }
}

/* The 27 cell shifts of the list entries, already multiplied by the block's
 * cell size: x_i - x_j = (o_i - o_j) + sh[code] (a shift of -1, 0 or +1 cells
 * times Lc is exact, so this rounds as the unscaled product would).  A block
 * never straddles two systems. */
template<class R> __device__ __forceinline__ void init_shift(const KArgs<R> &a, typename Vec<R>::T4 *sh) {
    if (threadIdx.x < 27) {
        const SysDev &sd = a.sys[a.blk_sys[(blockIdx.x * blockDim.x) / SYS_PAD]];
        const int c = threadIdx.x;
        typename Vec<R>::T4 v;
        v.x = R(-(c % 3 - 1)) * lc_of<R>(sd, 0);
        v.y = R(-((c / 3) % 3 - 1)) * lc_of<R>(sd, 1);
        v.z = R(-(c / 9 - 1)) * lc_of<R>(sd, 2);
        v.w = R(0);
        sh[c] = v;
    }
    __syncthreads();
}

/* Resident blocks of LITE_BS threads asked of the force kernels: the FP32
 * count, halved for FP64, whose doubles need twice the registers (the FP64
 * forms are bound by the FP64 pipe, so fewer resident warps cost nothing,
 * while spills would). */
template<class R> constexpr int fp_blocks(int n) { return sizeof(R) == 4 ? n : n / 2; }

/* Form bits of the force loop (orbc_params.kernel_variant; the autotuner
 * picks one per workload):
 *   1  software-pipelined list pass (the next entry's gathers in flight while
 *      the current pair is evaluated) instead of a 2-way unrolled loop;
 *   2  the rare non-lipid pair path inlined instead of called;
 *   4  occupancy form of the lite Langevin kernel (more resident blocks);
 *   32 merged shell pass: the skin-shell rows are only distance-tested, each
 *      lane records its hits in a bit mask, and the hits are evaluated in the
 *      same loop as the inner rows, so a shell row that one lane of a warp
 *      hits no longer costs the whole warp a pair evaluation; and where a
 *      lane's pair involves a protein, all lanes of the warp evaluate their
 *      lipid-lipid and lipid-protein pairs in one anisotropic code path with
 *      per-pair parameters instead of two paths one after the other.  The
 *      pairs are added in the same order as without it: the results are
 *      bit-identical;
 *   64 compensated accumulation: each particle's force and torque are summed
 *      with Kahan compensation (the rounding error of each running sum is
 *      carried into the next addition), for the FP32 form. */
constexpr int FORM_PIPE = 1, FORM_INLINE = 2, FORM_OCC = 4, FORM_MERGED = 32, FORM_KAHAN = 64;

/* s += d with Kahan compensation c (one component). */
template<class R> __device__ __forceinline__ void kahan_add(R &s, R &c, R d) {
    const R y = d - c;
    const R t = s + y;
    c = (t - s) - y;
    s = t;
}

/* All forces and torques on particle slot i: pair terms over its neighbour
 * list (form V, above), bonds, mesh constraint. */
template<class R, bool E, int V>
__device__ __forceinline__ void particle_forces(const KArgs<R> &a, const FFDev<R> &F, int i, int cur, int lp, int w,
                                                const typename Vec<R>::T4 &pi, const typename Vec<R>::T4 &ni,
                                                const SysDev &sd, const SysState &ss,
                                                const typename Vec<R>::T4 *sh, R3<R> &f, R3<R> &t, R &e,
                                                int &flags) {
    using T4 = typename Vec<R>::T4;
    constexpr bool KAHAN = (V & FORM_KAHAN) != 0;
    const int ty = w_type(w);
    const T4 *__restrict__ pos = a.pos[cur];
    const T4 *__restrict__ nrm = a.nrm[cur];
    const uint32_t *__restrict__ nb = a.nbr + nbr_index(i, 0, a.cap);
    const int packed = a.nnb[i];
    const int nin = packed & 0xffff, nout = packed >> 16;
    const uint32_t *__restrict__ shell = nb + int64_t(a.cap - 1) * 32;  // shell rows run downwards
    const int64_t stride = 32;
    const R ll_cutsq = a.ll.cutsq;
    R3<R> cf = {0, 0, 0}, ct = {0, 0, 0};  // Kahan compensations (KAHAN only)
    auto accumulate = [&](const R3<R> &df, const R3<R> &dt) {
        kahan_add(f.x, cf.x, df.x);
        kahan_add(f.y, cf.y, df.y);
        kahan_add(f.z, cf.z, df.z);
        kahan_add(t.x, ct.x, dt.x);
        kahan_add(t.y, ct.y, dt.y);
        kahan_add(t.z, ct.z, dt.z);
    };
    auto pair = [&](uint32_t ent, const T4 &pj, const T4 &nj) {
        const T4 s = sh[ent >> NB_SHIFT];
        const R dx = (pi.x - pj.x) + s.x;
        const R dy = (pi.y - pj.y) + s.y;
        const R dz = (pi.z - pj.z) + s.z;
        const R r2 = dx * dx + dy * dy + dz * dz;
        const int tj = w_type(wbits(pj.w));
        if (KAHAN) {
            R3<R> df = {0, 0, 0}, dt = {0, 0, 0};
            if ((V & FORM_MERGED) && !__all_sync(__activemask(), (ty | tj) == 0) && (ty == 0 || tj == 0) &&
                F.pair[ty | tj].kind == PAIR_ANISO) {
                // one anisotropic path for the warp, as in the uncompensated form
                // below; a lipid-lipid pair is added only inside its range, a
                // protein pair always (as the general path does)
                const PairP<R> &P = F.pair[ty | tj];
                const bool inr = r2 < P.cutsq && r2 > R(1e-5);
                if (inr) aniso<R, E>(P, dx, dy, dz, r2, ni.x, ni.y, ni.z, nj.x, nj.y, nj.z, df, dt, e);
                if (inr || (ty | tj) != 0) accumulate(df, dt);
            } else if ((ty | tj) == 0) {
                if (r2 < ll_cutsq && r2 > R(1e-5)) {
                    aniso<R, E>(a.ll, dx, dy, dz, r2, ni.x, ni.y, ni.z, nj.x, nj.y, nj.z, df, dt, e);
                    accumulate(df, dt);
                }
            } else {
                pair_general<R, E, (V & FORM_INLINE) != 0>(F.pair[ty * NT + tj], dx, dy, dz, r2, ni.x, ni.y, ni.z,
                                                           nj.x, nj.y, nj.z, df, dt, e);
                accumulate(df, dt);
            }
        } else if ((V & FORM_MERGED) && !__all_sync(__activemask(), (ty | tj) == 0)) {
            /* Some lane of the warp has a protein in this pair: every lipid-lipid
             * and lipid-protein pair of the warp goes through the same
             * anisotropic code with its own parameters (row ty | tj of the
             * table: the protein's type, 0 for two lipids), so that the
             * protein's lane does not run after the lipids' lanes.  The
             * parameters are those of the other branches: the results are
             * the same bit for bit. */
            if ((ty == 0 || tj == 0) && F.pair[ty | tj].kind == PAIR_ANISO) {
                const PairP<R> &P = F.pair[ty | tj];
                if (r2 < P.cutsq && r2 > R(1e-5))
                    aniso<R, E>(P, dx, dy, dz, r2, ni.x, ni.y, ni.z, nj.x, nj.y, nj.z, f, t, e);
            } else {
                pair_general<R, E, (V & FORM_INLINE) != 0>(F.pair[ty * NT + tj], dx, dy, dz, r2, ni.x, ni.y, ni.z,
                                                           nj.x, nj.y, nj.z, f, t, e);
            }
        } else if ((ty | tj) == 0) {
            if (r2 < ll_cutsq && r2 > R(1e-5))
                aniso<R, E>(a.ll, dx, dy, dz, r2, ni.x, ni.y, ni.z, nj.x, nj.y, nj.z, f, t, e);
        } else {
            pair_general<R, E, (V & FORM_INLINE) != 0>(F.pair[ty * NT + tj], dx, dy, dz, r2, ni.x, ni.y, ni.z, nj.x,
                                                       nj.y, nj.z, f, t, e);
        }
    };
    // Shell rows: partners in the skin at the last build, mostly still outside
    // the range; returns whether row k's partner has come inside it.
    auto shell_hit = [&](int k, uint32_t &ent, T4 &pj) {
        ent = __ldg(shell - int64_t(k) * stride);  // the rows were prefetched into L1 (read-only path)
        pj = ldg4<R>(pos + int(ent & NB_MASK));
        const T4 s = sh[ent >> NB_SHIFT];
        const R dx = (pi.x - pj.x) + s.x;
        const R dy = (pi.y - pj.y) + s.y;
        const R dz = (pi.z - pj.z) + s.z;
        const R r2 = dx * dx + dy * dy + dz * dz;
        const int tj = w_type(wbits(pj.w));
        const R lim = ((ty | tj) == 0) ? ll_cutsq : F.pair[ty * NT + tj].anysq;
        return r2 < lim;
    };
    if (V & FORM_MERGED) {
        /* shell rows first, distance only: row k's hit is bit k of hm (rows
         * beyond 32 are evaluated on the spot, after the merged pass, as
         * without this form) */
        uint32_t hm = 0;
        const int nq = min(nout, 32);
        for (int k = 0; k < nq; ++k) {
            uint32_t ent;
            T4 pj;
            if (shell_hit(k, ent, pj)) hm |= 1u << k;
        }
        // inner rows, then the shell hits in row order, in one loop
        const int total = nin + __popc(hm);
        auto entry = [&](int k) -> uint32_t {
            if (k < nin) return __ldg(nb + int64_t(k) * stride);
            const int b = __ffs(hm) - 1;
            hm &= hm - 1u;
            return __ldg(shell - int64_t(b) * stride);
        };
        uint32_t e1 = total > 0 ? entry(0) : 0u;
        uint32_t e2 = total > 1 ? entry(1) : 0u;
        T4 pn, nn;
        if (total > 0) {
            pn = ldg4<R>(pos + int(e1 & NB_MASK));
            nn = ldg4<R>(nrm + int(e1 & NB_MASK));
        }
        for (int k = 0; k < total; ++k) {
            const uint32_t ent = e1;
            const T4 pj = pn, nj = nn;
            e1 = e2;
            if (k + 2 < total) e2 = entry(k + 2);
            if (k + 1 < total) {
                pn = ldg4<R>(pos + int(e1 & NB_MASK));
                nn = ldg4<R>(nrm + int(e1 & NB_MASK));
            }
            pair(ent, pj, nj);
        }
        for (int k = 32; k < nout; ++k) {
            uint32_t ent;
            T4 pj;
            if (shell_hit(k, ent, pj)) pair(ent, pj, ldg4<R>(nrm + int(ent & NB_MASK)));
        }
    } else {
        // Inner rows: partners that were inside the interaction range at the last
        // build; almost all still are, so every lane does the pair arithmetic.
        if (V & FORM_PIPE) {
            /* software-pipelined: the entry two ahead and the gathers one ahead
             * are in flight while the current pair is evaluated */
            uint32_t e1 = nin > 0 ? __ldcs(nb) : 0u;
            uint32_t e2 = nin > 1 ? __ldcs(nb + stride) : 0u;
            T4 pn, nn;
            if (nin > 0) {
                pn = ldg4<R>(pos + int(e1 & NB_MASK));
                nn = ldg4<R>(nrm + int(e1 & NB_MASK));
            }
            for (int k = 0; k < nin; ++k) {
                const uint32_t ent = e1;
                const T4 pj = pn, nj = nn;
                e1 = e2;
                if (k + 2 < nin) e2 = __ldcs(nb + int64_t(k + 2) * stride);
                if (k + 1 < nin) {
                    pn = ldg4<R>(pos + int(e1 & NB_MASK));
                    nn = ldg4<R>(nrm + int(e1 & NB_MASK));
                }
                pair(ent, pj, nj);
            }
        } else {
#pragma unroll 2
            for (int k = 0; k < nin; ++k) {
                const uint32_t ent = __ldcs(nb + int64_t(k) * stride);
                const int j = int(ent & NB_MASK);
                pair(ent, ldg4<R>(pos + j), ldg4<R>(nrm + j));
            }
        }
        // the orientation is only gathered for the few shell partners that came in
#pragma unroll 2
        for (int k = 0; k < nout; ++k) {
            uint32_t ent;
            T4 pj;
            if (shell_hit(k, ent, pj)) pair(ent, pj, ldg4<R>(nrm + int(ent & NB_MASK)));
        }
    }
    // bonds
    const int bd = w_bdeg(w);
    if (bd) {
        const int ci = a.cell[lp][i];
        for (int b = 0; b < bd; ++b) {
            const BondSlot bs = a.bond[lp][int64_t(b) * a.npad + i];
            const T4 pj = pos[bs.partner];
            R dx, dy, dz;
            rel_pos<R>(sd, a.cell[lp][bs.partner], ci, pj, pi, dx, dy, dz);
            const R r = sqrt(dx * dx + dy * dy + dz * dz);
            const R kap = bond_kappa<R, E>(F.bond[bs.type], R(bs.r0), r, e, flags);
            if (KAHAN) {
                kahan_add(f.x, cf.x, kap * dx);
                kahan_add(f.y, cf.y, kap * dy);
                kahan_add(f.z, cf.z, kap * dz);
            } else {
                f.x += kap * dx;
                f.y += kap * dy;
                f.z += kap * dz;
            }
        }
    }
    // global area / volume constraint on mesh vertices
    const int fd = w_fdeg(w);
    if (fd && (ss.cv != 0.0 || ss.ca != 0.0)) {
        const int ci = a.cell[lp][i];
        const R cv = R(ss.cv) * R(1.0 / 6.0), ca = R(ss.ca) * R(0.5);
        for (int b = 0; b < fd; ++b) {
            const int2 fs = a.fslot[lp][int64_t(b) * a.npad + i];
            R bx, by, bz, cx, cy, cz;
            rel_pos<R>(sd, a.cell[lp][fs.x], ci, pos[fs.x], pi, bx, by, bz);
            rel_pos<R>(sd, a.cell[lp][fs.y], ci, pos[fs.y], pi, cx, cy, cz);
            const R nx = by * cz - bz * cy, ny = bz * cx - bx * cz, nz = bx * cy - by * cx;  // 6 dV/da
            const R inn = rnorm3(nx, ny, nz);
            const R hx = nx * inn, hy = ny * inn, hz = nz * inn;
            const R ex = bx - cx, ey = by - cy, ez = bz - cz;
            const R gx = ey * hz - ez * hy, gy = ez * hx - ex * hz, gz = ex * hy - ey * hx;  // 2 dA/da
            if (KAHAN) {
                kahan_add(f.x, cf.x, cv * nx + ca * gx);
                kahan_add(f.y, cf.y, cv * ny + ca * gy);
                kahan_add(f.z, cf.z, cv * nz + ca * gz);
            } else {
                f.x += cv * nx + ca * gx;
                f.y += cv * ny + ca * gy;
                f.z += cv * nz + ca * gz;
            }
        }
    }
}

__device__ __forceinline__ void philox4(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1,
                                        uint32_t o[4]) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const uint32_t lo0 = 0xD2511F53u * c0, hi0 = __umulhi(0xD2511F53u, c0);
        const uint32_t lo1 = 0xCD9E8D57u * c2, hi1 = __umulhi(0xCD9E8D57u, c2);
        const uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
        c0 = n0;
        c1 = lo1;
        c2 = n2;
        c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    o[0] = c0;
    o[1] = c1;
    o[2] = c2;
    o[3] = c3;
}
__device__ __forceinline__ void philox3(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1,
                                        uint32_t &o0, uint32_t &o1, uint32_t &o2) {
    uint32_t o[4];
    philox4(c0, c1, c2, c3, k0, k1, o);
    o0 = o[0];
    o1 = o[1];
    o2 = o[2];
}
template<class R> __device__ __forceinline__ R u11(uint32_t u) { return R(u >> 8) * R(1.0 / 8388608.0) - R(1); }


/* Reflective walls (src/integrate_nh.h:124-144) on the axes where the system
 * has them (wlo < whi), applied in the frame of the particle's cell. */
template<class R>
__device__ __forceinline__ void bounce_walls(const SysDev &sd, int c, typename Vec<R>::T4 &p, typename Vec<R>::T4 &v) {
    const int cc[3] = {cx_of(c), cy_of(c), cz_of(c)};
    R *pp[3] = {&p.x, &p.y, &p.z};
    R *vv[3] = {&v.x, &v.y, &v.z};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        if (!(sd.wlo[d] < sd.whi[d])) continue;
        const double center = sd.lo[d] + (double(cc[d]) + 0.5) * sd.Lc[d];
        const R lo = R(sd.wlo[d] - center), hi = R(sd.whi[d] - center);
        if (*pp[d] < lo) {
            *pp[d] = lo + (lo - *pp[d]);
            *vv[d] = -*vv[d];
        } else if (*pp[d] > hi) {
            *pp[d] = hi - (*pp[d] - hi);
            *vv[d] = -*vv[d];
        }
    }
}

enum { MODE_LANGEVIN = 0, MODE_NH_FINAL = 1, MODE_NH_INITIAL = 2, MODE_FORCES = 3, MODE_VCOM = 4 };

/* Per-system sums, first level.  Every warp reduces its particles' values --
 * the sums in the working precision (in mixed mode the FP64 pipe would cost
 * more than the force loop), the maximum and the flags on integers -- and
 * lane 0 stores them in FP64 as the warp's partial.  No barrier, fence or
 * atomic: k_reduce, launched next on the stream, sums each system's partials
 * in a fixed order.  Partial layout: ke2, epot, max displacement^2, error
 * flags, lipid sum v (3).  All 32 lanes of the warp must call it; i is the
 * caller's slot (a warp never straddles two systems). */
template<class R>
__device__ __forceinline__ void warp_partials(const KArgs<R> &a, int i, R ke, R ep, float md2, int flags,
                                              R vx = R(0), R vy = R(0), R vz = R(0)) {
    R v[5] = {ke, ep, vx, vy, vz};
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
        for (int k = 0; k < 5; ++k) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
    }
    // md2 >= 0 (or NaN, flagged separately): the bit order is the value order
    const unsigned wmax = __reduce_max_sync(0xffffffffu, __float_as_uint(md2));
    const int wfl = int(__reduce_or_sync(0xffffffffu, unsigned(flags)));
    if ((threadIdx.x & 31) == 0) {
        double *p = a.partial + int64_t(i >> 5) * NPART;
        p[0] = double(v[0]);
        p[1] = double(v[1]);
        p[2] = double(__uint_as_float(wmax));
        p[3] = double(wfl);
        p[4] = double(v[2]);
        p[5] = double(v[3]);
        p[6] = double(v[4]);
    }
}

__device__ __forceinline__ double combine_part(int k, double x, double y) {
    return k == 2 ? fmax(x, y) : (k == 3 ? double(int(x) | int(y)) : x + y);
}

/* Per-system sums, second and third level, after a kernel that wrote warp
 * partials.  Block g sums the RED_GROUP warp partials of reduction group g
 * (RED_GROUP x 32 consecutive slots of one system) in a fixed-shape tree; the
 * last block to finish (ticket) gives each system to one warp, which adds the
 * system's group partials in a fixed order, and applies the mode's update:
 * thermostat, kinetic energy, potential energy, bulk velocity, rebuild rule,
 * step counter, buffer parity. */
template<class R> __global__ void __launch_bounds__(RED_GROUP) k_reduce(KArgs<R> a, int mode, int count_step) {
    if (halted(a.S)) return;  // the kernel before it did nothing; its partials are stale
    __shared__ double red[7][RED_GROUP];
    __shared__ double wmax[RED_GROUP / 32];
    __shared__ int wfl[RED_GROUP / 32];
    __shared__ int last;
    const int g = blockIdx.x, t = threadIdx.x, lane = t & 31, warp = t >> 5;
    int s = 0;
    while (s + 1 < a.nsys && g >= a.sys[s + 1].gbase) ++s;
    const SysDev &sd = a.sys[s];
    const int gl = g - sd.gbase;
    const int64_t w0 = int64_t(sd.off / 32) + int64_t(gl) * RED_GROUP;
    const int nw = min(RED_GROUP, sd.npad / 32 - gl * RED_GROUP);
    for (int k = 0; k < 7; ++k) red[k][t] = t < nw ? __ldcg(a.partial + (w0 + t) * NPART + k) : 0.0;
    __syncthreads();
    for (int h = RED_GROUP / 2; h > 0; h >>= 1) {
        if (t < h)
            for (int k = 0; k < 7; ++k) red[k][t] = combine_part(k, red[k][t], red[k][t + h]);
        __syncthreads();
    }
    if (t == 0) {
        double *gp = a.gpartial + int64_t(g) * NPART;
        for (int k = 0; k < 7; ++k) gp[k] = red[k][0];
        __threadfence();
        last = atomicAdd(&a.S->blk_counter, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    double mymax = 0.0;
    int myfl = 0;
    for (int q = warp; q < a.nsys; q += RED_GROUP / 32) {
        const SysDev &sq = a.sys[q];
        double v[7];
        for (int k = 0; k < 7; ++k) {
            double acc = 0.0;
            for (int u = lane; u < sq.ngrp; u += 32)
                acc = combine_part(k, acc, __ldcg(a.gpartial + int64_t(sq.gbase + u) * NPART + k));
            v[k] = acc;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            for (int k = 0; k < 7; ++k) v[k] = combine_part(k, v[k], __shfl_xor_sync(0xffffffffu, v[k], o));
        if (lane == 0) {
            SysState &ss = a.ss[q];
            const double k2 = v[0], e = v[1];
            if ((mode == MODE_LANGEVIN || mode == MODE_NH_INITIAL || mode == MODE_VCOM) && sq.nlipid > 0) {
                ss.vcom[0] = v[4] / double(sq.nlipid);
                ss.vcom[1] = v[5] / double(sq.nlipid);
                ss.vcom[2] = v[6] / double(sq.nlipid);
            }
            if (mode == MODE_VCOM) {
                ss.ke2 = k2;
            } else if (mode == MODE_LANGEVIN || mode == MODE_FORCES) {
                if (mode == MODE_LANGEVIN) ss.ke2 = k2;
                ss.epot = e;
            } else {
                // zeta += dt/2Q (sum m v^2 / 2 - 3/2 N kT)  (src/integrate_nh.h:182-185, :241-244)
                const double nreal = double(sq.nreal);
                const double Q = sq.Q > 0 ? sq.Q : 0.01 * nreal;
                ss.zeta += 0.5 * a.dt / Q * (0.5 * k2 - 0.5 * 3.0 * nreal * a.kBT);
                ss.ke2 = k2;
                if (mode == MODE_NH_FINAL) ss.epot = e;
            }
            mymax = fmax(mymax, v[2]);
            myfl |= int(v[3]);
        }
    }
    if (lane == 0) {
        wmax[warp] = mymax;
        wfl[warp] = myfl;
    }
    __syncthreads();
    if (t == 0) {
        double m = 0.0;
        int fl = 0;
        for (int w = 0; w < RED_GROUP / 32; ++w) {
            m = fmax(m, wmax[w]);
            fl |= wfl[w];
        }
        Scalars *S = a.S;
        S->error |= fl;
        if (mode == MODE_LANGEVIN || mode == MODE_NH_INITIAL) {
            S->since_rebuild += 1;
            if (m > double(a.skin_half2) || (a.rebuild_every > 0 && S->since_rebuild >= a.rebuild_every))
                S->rebuild = 1;
        }
        if (mode == MODE_LANGEVIN) {
            S->cur ^= 1;
            S->step += 1;
            S->iters += 1;
        }
        if (mode == MODE_NH_INITIAL) S->nh_half = 1;
        if (mode == MODE_NH_FINAL) {
            S->nh_half = 0;
            if (count_step) {
                S->step += 1;
                S->iters += 1;
            }
        }
        S->blk_counter = 0;
        __threadfence();
    }
}

/* One particle of the fused Langevin step: forces at the current state, then
 * src/integrate_langevin.h:105-146 (rotation, then translation with the
 * counter-based noise).  Writes the new state; returns the squared
 * displacement since the list was built, sum m v^2, the energy and the lipid
 * velocity (for the bulk-velocity removal). */
template<class R, bool E, int V>
__device__ __forceinline__ void langevin_particle(const KArgs<R> &a, const FFDev<R> &F, const typename Vec<R>::T4 *sh,
                                                  int i, int s, int cur, int lp, long long step,
                                                  const typename Vec<R>::T4 &pi, int w, bool zero_bulk, R &ke, R &ep,
                                                  float &md2, int &flags, R &vsx, R &vsy, R &vsz) {
    using T4 = typename Vec<R>::T4;
    const int ty = w_type(w);
    const SysDev &sd = a.sys[s];
    const T4 ni = a.nrm[cur][i];
    R3<R> f = {0, 0, 0}, t = {0, 0, 0};
    R e = 0;
    particle_forces<R, E, V>(a, F, i, cur, lp, w, pi, ni, sd, a.ss[s], sh, f, t, e, flags);
    const R dt = R(a.dt);
    T4 v = ldcs4<R>(&a.vel[lp][i]), o = ldcs4<R>(&a.omg[lp][i]);
    if (zero_bulk && ty == 0) {  // zero_bulk_velocity on the lipids (src/zero_bulk_velocity.h:38-45)
        v.x -= R(__ldcg(&a.ss[s].vcom[0]));
        v.y -= R(__ldcg(&a.ss[s].vcom[1]));
        v.z -= R(__ldcg(&a.ss[s].vcom[2]));
    }
    // ROTATION: t <- n x t; o += dt t; n <- normalize(n + (o x n) dt)
    const R tx = ni.y * t.z - ni.z * t.y, ty_ = ni.z * t.x - ni.x * t.z, tz = ni.x * t.y - ni.y * t.x;
    o.x += dt * tx;
    o.y += dt * ty_;
    o.z += dt * tz;
    const R gx = ni.x + (o.y * ni.z - o.z * ni.y) * dt;
    const R gy = ni.y + (o.z * ni.x - o.x * ni.z) * dt;
    const R gz = ni.z + (o.x * ni.y - o.y * ni.x) * dt;
    const R gi = rnorm3(gx, gy, gz);
    T4 nn = ni;
    nn.x = gx * gi;
    nn.y = gy * gi;
    nn.z = gz * gi;
    // TRANSLATION: f -= gamma v + sigma r; v += f dt/m; x += v dt
    uint32_t r0, r1, r2;
    philox3(uint32_t(__ldcs(&a.tag[lp][i])), uint32_t(step), uint32_t((unsigned long long)step >> 32), uint32_t(s),
            uint32_t(a.seed), uint32_t(a.seed >> 32), r0, r1, r2);
    const R gam = F.gamma[ty], sig = F.sigma[ty];
    const R dtm = dt * F.inv_mass[ty];
    f.x -= gam * v.x + sig * u11<R>(r0);
    f.y -= gam * v.y + sig * u11<R>(r1);
    f.z -= gam * v.z + sig * u11<R>(r2);
    v.x += f.x * dtm;
    v.y += f.y * dtm;
    v.z += f.z * dtm;
    T4 p = pi;
    p.x += v.x * dt;
    p.y += v.y * dt;
    p.z += v.z * dt;
    a.pos[cur ^ 1][i] = p;
    a.nrm[cur ^ 1][i] = nn;
    stcs4(&a.vel[lp][i], v);
    stcs4(&a.omg[lp][i], o);
    const T4 xr = ldcs4<R>(&a.xref[lp][i]);
    const R ddx = p.x - xr.x, ddy = p.y - xr.y, ddz = p.z - xr.z;
    md2 = float(ddx * ddx + ddy * ddy + ddz * ddz);
    if (!isfinite(p.x + p.y + p.z + v.x + v.y + v.z)) flags |= ERRB_NAN;
    ke = F.mass[ty] * (v.x * v.x + v.y * v.y + v.z * v.z);
    ep = e;
    if (ty == 0) {
        vsx = v.x;
        vsy = v.y;
        vsz = v.z;
    }
}

/* Langevin step with the per-system sums (energy, bulk-velocity removal):
 * the structure of the lite kernel below (small blocks, force-field table
 * through the read-only path) plus warp partials, summed per system by
 * k_reduce after the kernel.  Resident blocks as for k_nh_final (20, 18 with
 * the merged shell pass, 16 with compensated sums): 0.82 against 0.92 ms per
 * step with the merged pass on the 4.03M cell, where 20 blocks spilled. */
template<class R, bool E, int V>
__global__ void __launch_bounds__(LITE_BS, fp_blocks<R>((V & FORM_KAHAN) ? 16 : ((V & FORM_MERGED) ? 18 : 20)))
    k_step_langevin(KArgs<R> a) {
    if (halted(a.S)) return;
    using T4 = typename Vec<R>::T4;
    __shared__ T4 sh[27];
    init_shift<R>(a, sh);
    const FFDev<R> *__restrict__ Fp = a.ff;
    const int cur = __ldcg(&a.S->cur), lp = __ldcg(&a.S->lp);
    const long long step = __ldcg(&a.S->step);
    const int i = blockIdx.x * LITE_BS + threadIdx.x;
    const int s = a.blk_sys[i / SYS_PAD];
    const T4 pi = a.pos[cur][i];
    prefetch_warp_list(a.nbr, i, a.cap, a.nnb[i]);
    const int w = wbits(pi.w);
    R ke = 0, ep = 0, vsx = 0, vsy = 0, vsz = 0;
    float md2 = 0.f;
    int flags = 0;
    if (w_type(w) != GHOST)
        langevin_particle<R, E, V>(a, *Fp, sh, i, s, cur, lp, step, pi, w, a.zero_bulk != 0, ke, ep, md2, flags, vsx,
                                   vsy, vsz);
    warp_partials<R>(a, i, ke, ep, md2, flags, vsx, vsy, vsz);
}

/* Langevin step without per-system sums (no energy, no bulk-velocity
 * removal): small blocks that retire independently, the force-field table read
 * through the read-only path, and no end-of-block reduction -- a warp whose
 * particles moved more than skin/2 raises the rebuild flag itself, and
 * k_advance flips the buffers after the kernel.  The temperature is reduced on
 * demand (k_vcom). */
template<class R, int V>
__global__ void __launch_bounds__(LITE_BS, fp_blocks<R>((V & 4) ? ((V & FORM_MERGED) ? 18 : 20) : 16))
    k_step_langevin_lite(KArgs<R> a) {
    if (halted(a.S)) return;
    using T4 = typename Vec<R>::T4;
    __shared__ T4 sh[27];
    init_shift<R>(a, sh);
    const FFDev<R> *__restrict__ Fp = a.ff;
    const int cur = __ldcg(&a.S->cur), lp = __ldcg(&a.S->lp);
    const long long step = __ldcg(&a.S->step);
    const int i = blockIdx.x * LITE_BS + threadIdx.x;
    const int s = a.blk_sys[i / SYS_PAD];
    const T4 pi = a.pos[cur][i];
    prefetch_warp_list(a.nbr, i, a.cap, a.nnb[i]);
    const int w = wbits(pi.w);
    R ke = 0, ep = 0, vsx = 0, vsy = 0, vsz = 0;
    float md2 = 0.f;
    int flags = 0;
    if (w_type(w) != GHOST)
        langevin_particle<R, false, V>(a, *Fp, sh, i, s, cur, lp, step, pi, w, false, ke, ep, md2, flags, vsx, vsy,
                                       vsz);
    const unsigned m = __reduce_max_sync(0xffffffffu, __float_as_uint(md2));  // md2 >= 0: bit order = value order
    const int fl = int(__reduce_or_sync(0xffffffffu, unsigned(flags)));
    if ((threadIdx.x & 31) == 0) {
        if (double(__uint_as_float(m)) > double(a.skin_half2) || !(__uint_as_float(m) == __uint_as_float(m)))
            a.S->rebuild = 1;
        if (fl) atomicOr(&a.S->error, fl);
    }
}

/* After a lite Langevin step (count_step = 1) or a minimisation step (0):
 * flip the position buffers, advance the step counter and apply the
 * every-k-steps rebuild rule. */
__global__ void k_advance(Scalars *S, int rebuild_every, int count_step) {
    if (halted(S)) return;
    S->iters += 1;
    S->cur ^= 1;
    S->step += count_step;
    S->since_rebuild += 1;
    if (rebuild_every > 0 && S->since_rebuild >= rebuild_every) S->rebuild = 1;
}

/* One step of the energy minimisation (src/openrbc.cpp:88-146): forces,
 * post_torque t <- n x t (src/integrate_nh.h:146-154), the step-limited
 * steepest-descent move of :113-130 and bounce_back (:132).  Positions and
 * orientations ping-pong like the Langevin step; the step counter (the noise
 * key) does not advance. */
template<class R, int V>
__global__ void __launch_bounds__(LITE_BS, fp_blocks<R>((V & 2) ? 12 : 16))
    k_minimize(KArgs<R> a, double dr_opt, double dn_opt) {
    if (halted(a.S)) return;
    using T4 = typename Vec<R>::T4;
    __shared__ T4 sh[27];
    init_shift<R>(a, sh);
    const FFDev<R> *__restrict__ Fp = a.ff;
    const int cur = __ldcg(&a.S->cur), lp = __ldcg(&a.S->lp);
    const int i = blockIdx.x * LITE_BS + threadIdx.x;
    const int s = a.blk_sys[i / SYS_PAD];
    const SysDev &sd = a.sys[s];
    const T4 pi = a.pos[cur][i];
    prefetch_warp_list(a.nbr, i, a.cap, a.nnb[i]);
    const int w = wbits(pi.w);
    const int ty = w_type(w);
    float md2 = 0.f;
    int flags = 0;
    if (ty != GHOST) {
        const T4 ni = a.nrm[cur][i];
        R3<R> f = {0, 0, 0}, t = {0, 0, 0};
        R e = 0;
        particle_forces<R, false, V>(a, *Fp, i, cur, lp, w, pi, ni, sd, a.ss[s], sh, f, t, e, flags);
        const R tx = ni.y * t.z - ni.z * t.y, ty_ = ni.z * t.x - ni.x * t.z, tz = ni.x * t.y - ni.y * t.x;
        const R m = Fp->mass[ty];
        const R dxx = f.x / m, dxy = f.y / m, dxz = f.z / m;
        const R dnx = ty_ * ni.z - tz * ni.y, dny = tz * ni.x - tx * ni.z, dnz = tx * ni.y - ty_ * ni.x;
        const R ndx = sqrt(dxx * dxx + dxy * dxy + dxz * dxz), ndn = sqrt(dnx * dnx + dny * dny + dnz * dnz);
        const R dr = R(dr_opt), dn = R(dn_opt);
        const R h = (ndx > dr || ndn > dn) ? min(dr / ndx, dn / ndn) : R(a.dt);
        const R hm = h / m;
        T4 p = pi;
        p.x += f.x * hm;
        p.y += f.y * hm;
        p.z += f.z * hm;
        const R gx = ni.x + dnx * h, gy = ni.y + dny * h, gz = ni.z + dnz * h;
        const R gi = R(1) / sqrt(gx * gx + gy * gy + gz * gz);
        T4 nn = ni;
        nn.x = gx * gi;
        nn.y = gy * gi;
        nn.z = gz * gi;
        T4 v = a.vel[lp][i];
        const T4 v0 = v;
        bounce_walls<R>(sd, a.cell[lp][i], p, v);
        if (v.x != v0.x || v.y != v0.y || v.z != v0.z) a.vel[lp][i] = v;
        a.pos[cur ^ 1][i] = p;
        a.nrm[cur ^ 1][i] = nn;
        const T4 xr = a.xref[lp][i];
        const R ddx = p.x - xr.x, ddy = p.y - xr.y, ddz = p.z - xr.z;
        md2 = float(ddx * ddx + ddy * ddy + ddz * ddz);
        if (!isfinite(p.x + p.y + p.z + nn.x + nn.y + nn.z)) flags |= ERRB_NAN;
    }
    const unsigned mm = __reduce_max_sync(0xffffffffu, __float_as_uint(md2));
    const int fl = int(__reduce_or_sync(0xffffffffu, unsigned(flags)));
    if ((threadIdx.x & 31) == 0) {
        if (double(__uint_as_float(mm)) > double(a.skin_half2) || !(__uint_as_float(mm) == __uint_as_float(mm)))
            a.S->rebuild = 1;
        if (fl) atomicOr(&a.S->error, fl);
    }
}

/* Nose-Hoover second half (post_toque_final_update, src/integrate_nh.h:237-273)
 * fused with the forces: the lite structure plus warp partials for the
 * kinetic-energy sum that k_reduce turns into the thermostat update.  The
 * resident blocks asked for fall with the registers a form needs (20 blocks
 * at 48 registers, 18 at 56 with the merged shell pass, 16 at 64 with
 * compensated sums), so that those two forms do not spill. */
template<class R, bool E, int V>
__global__ void __launch_bounds__(LITE_BS, fp_blocks<R>((V & FORM_KAHAN) ? 16 : ((V & FORM_MERGED) ? 18 : 20)))
    k_nh_final(KArgs<R> a, int count_step) {
    if (halted(a.S)) return;
    using T4 = typename Vec<R>::T4;
    __shared__ T4 sh[27];
    init_shift<R>(a, sh);
    const FFDev<R> &F = *a.ff;
    const int cur = __ldcg(&a.S->cur), lp = __ldcg(&a.S->lp);
    const int i = blockIdx.x * LITE_BS + threadIdx.x;
    const int s = a.blk_sys[i / SYS_PAD];
    const SysDev &sd = a.sys[s];
    const T4 pi = a.pos[cur][i];
    prefetch_warp_list(a.nbr, i, a.cap, a.nnb[i]);
    const int w = wbits(pi.w);
    const int ty = w_type(w);
    R ke = 0, ep = 0;
    int flags = 0;
    if (ty != GHOST) {
        const T4 ni = a.nrm[cur][i];
        R3<R> f = {0, 0, 0}, t = {0, 0, 0};
        R e = 0;
        particle_forces<R, E, V>(a, F, i, cur, lp, w, pi, ni, sd, a.ss[s], sh, f, t, e, flags);
        const R dt = R(a.dt);
        const R zeta = R(__ldcg(&a.ss[s].zeta));
        const R im = F.inv_mass[ty];
        T4 v = a.vel[lp][i], o = a.omg[lp][i];
        if (a.zero_bulk && count_step && ty == 0) {  // between the forces and the final half (src/openrbc.cpp:228)
            v.x -= R(__ldcg(&a.ss[s].vcom[0]));
            v.y -= R(__ldcg(&a.ss[s].vcom[1]));
            v.z -= R(__ldcg(&a.ss[s].vcom[2]));
        }
        T4 tq = v;
        tq.x = ni.y * t.z - ni.z * t.y;  // post_torque: t <- n x t
        tq.y = ni.z * t.x - ni.x * t.z;
        tq.z = ni.x * t.y - ni.y * t.x;
        v.x += R(0.5) * dt * (f.x * im - zeta * v.x);
        v.y += R(0.5) * dt * (f.y * im - zeta * v.y);
        v.z += R(0.5) * dt * (f.z * im - zeta * v.z);
        o.x += R(0.5) * dt * tq.x;
        o.y += R(0.5) * dt * tq.y;
        o.z += R(0.5) * dt * tq.z;
        T4 fo = v;
        fo.x = f.x;
        fo.y = f.y;
        fo.z = f.z;
        a.vel[lp][i] = v;
        a.omg[lp][i] = o;
        a.frc[lp][i] = fo;
        a.trq[lp][i] = tq;
        if (!isfinite(v.x + v.y + v.z)) flags |= ERRB_NAN;
        ke = F.mass[ty] * (v.x * v.x + v.y * v.y + v.z * v.z);
        ep = e;
    }
    warp_partials<R>(a, i, ke, ep, 0.f, flags);
}

template<class R> __global__ void __launch_bounds__(256) k_nh_initial(KArgs<R> a) {
    if (halted(a.S)) return;
    using T4 = typename Vec<R>::T4;
    const int cur = __ldcg(&a.S->cur), lp = __ldcg(&a.S->lp);
    const int i = blockIdx.x * 256 + threadIdx.x;
    const int s = a.blk_sys[i / SYS_PAD];
    const SysDev &sd = a.sys[s];
    T4 p = a.pos[cur][i];
    const int w = wbits(p.w);
    const int ty = w_type(w);
    R ke = 0, vsx = 0, vsy = 0, vsz = 0;
    float md2 = 0.f;
    int flags = 0;
    if (ty != GHOST) {
        const R dt = R(a.dt);
        const R gamma = R(1) / (R(1) + R(0.5) * dt * R(__ldcg(&a.ss[s].zeta)));
        const R hm = R(0.5) * a.ff->inv_mass[ty];
        T4 v = a.vel[lp][i], o = a.omg[lp][i];
        const T4 f = a.frc[lp][i], t = a.trq[lp][i];
        v.x = (v.x + hm * dt * f.x) * gamma;
        v.y = (v.y + hm * dt * f.y) * gamma;
        v.z = (v.z + hm * dt * f.z) * gamma;
        p.x += v.x * dt;
        p.y += v.y * dt;
        p.z += v.z * dt;
        // bounce back at the walls (src/integrate_nh.h:199-208), in the cell frame
        bounce_walls<R>(sd, a.cell[lp][i], p, v);
        ke = a.ff->mass[ty] * (v.x * v.x + v.y * v.y + v.z * v.z);
        if (ty == 0) {
            vsx = v.x;
            vsy = v.y;
            vsz = v.z;
        }
        o.x += R(0.5) * dt * t.x;
        o.y += R(0.5) * dt * t.y;
        o.z += R(0.5) * dt * t.z;
        T4 n = a.nrm[cur][i];
        const R gx = n.x + (o.y * n.z - o.z * n.y) * dt;
        const R gy = n.y + (o.z * n.x - o.x * n.z) * dt;
        const R gz = n.z + (o.x * n.y - o.y * n.x) * dt;
        const R gi = rnorm3(gx, gy, gz);
        n.x = gx * gi;
        n.y = gy * gi;
        n.z = gz * gi;
        a.pos[cur][i] = p;
        a.nrm[cur][i] = n;
        a.vel[lp][i] = v;
        a.omg[lp][i] = o;
        const T4 xr = a.xref[lp][i];
        const R ddx = p.x - xr.x, ddy = p.y - xr.y, ddz = p.z - xr.z;
        md2 = float(ddx * ddx + ddy * ddy + ddz * ddz);
        if (!isfinite(p.x + p.y + p.z)) flags |= ERRB_NAN;
    }
    warp_partials<R>(a, i, ke, R(0), md2, flags, vsx, vsy, vsz);
}

/* Velocity sums of each system after the velocities were replaced (upload,
 * set_state, assign_temperature): sum m v^2 and the mean lipid velocity; the
 * step kernels keep both current afterwards. */
template<class R> __global__ void __launch_bounds__(256) k_vcom(KArgs<R> a) {
    using T4 = typename Vec<R>::T4;
    const int cur = __ldcg(&a.S->cur), lp = __ldcg(&a.S->lp);
    const int i = blockIdx.x * 256 + threadIdx.x;
    R ke = 0, vsx = 0, vsy = 0, vsz = 0;
    const int ty = w_type(wbits(a.pos[cur][i].w));
    if (ty != GHOST) {
        const T4 v = a.vel[lp][i];
        ke = a.ff->mass[ty] * (v.x * v.x + v.y * v.y + v.z * v.z);
        if (ty == 0) {
            vsx = v.x;
            vsy = v.y;
            vsz = v.z;
        }
    }
    warp_partials<R>(a, i, ke, R(0), 0.f, 0, vsx, vsy, vsz);
}

/* assign_temperature (src/assign_temperature.h:26-44, called at
 * src/openrbc.cpp:160): v = sqrt(2 kT / m) g, g three unit Gaussians from
 * Box-Muller on one Philox4x32-10 block keyed by the seed with counter
 * (tag, 0x6B8B4567, 0x327B23C6, system), u = (word + 1/2) / 2^32.  The factor
 * 2 of the reference is kept.  Computed in FP64, stored in R. */
template<class R> __global__ void __launch_bounds__(256) k_assign_temperature(KArgs<R> a, double kT, uint64_t seed) {
    using T4 = typename Vec<R>::T4;
    const int cur = __ldcg(&a.S->cur), lp = __ldcg(&a.S->lp);
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.npad) return;
    const int ty = w_type(wbits(a.pos[cur][i].w));
    if (ty == GHOST) return;
    const int s = a.blk_sys[i / SYS_PAD];
    uint32_t o[4];
    philox4(uint32_t(a.tag[lp][i]), 0x6B8B4567u, 0x327B23C6u, uint32_t(s), uint32_t(seed), uint32_t(seed >> 32), o);
    double u[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) u[k] = (double(o[k]) + 0.5) * (1.0 / 4294967296.0);
    const double r0 = sqrt(-2.0 * log(u[0])), r1 = sqrt(-2.0 * log(u[2]));
    const double twopi = 6.283185307179586;
    const double sc = sqrt(2.0 / double(a.ff->mass[ty]) * kT);
    T4 v = a.vel[lp][i];
    v.x = R(sc * r0 * cos(twopi * u[1]));
    v.y = R(sc * r0 * sin(twopi * u[1]));
    v.z = R(sc * r1 * cos(twopi * u[3]));
    a.vel[lp][i] = v;
}

template<class R, bool E, int V> __global__ void __launch_bounds__(LITE_BS, fp_blocks<R>(16)) k_forces(KArgs<R> a) {
    if (halted(a.S)) return;
    using T4 = typename Vec<R>::T4;
    __shared__ T4 sh[27];
    init_shift<R>(a, sh);
    const FFDev<R> &F = *a.ff;
    const int cur = __ldcg(&a.S->cur), lp = __ldcg(&a.S->lp);
    const int i = blockIdx.x * LITE_BS + threadIdx.x;
    const int s = a.blk_sys[i / SYS_PAD];
    const SysDev &sd = a.sys[s];
    const T4 pi = a.pos[cur][i];
    prefetch_warp_list(a.nbr, i, a.cap, a.nnb[i]);
    const int w = wbits(pi.w);
    R ep = 0;
    int flags = 0;
    if (w_type(w) != GHOST) {
        const T4 ni = a.nrm[cur][i];
        R3<R> f = {0, 0, 0}, t = {0, 0, 0};
        R e = 0;
        particle_forces<R, E, V>(a, F, i, cur, lp, w, pi, ni, sd, a.ss[s], sh, f, t, e, flags);
        T4 q = pi;
        q.x = f.x;
        q.y = f.y;
        q.z = f.z;
        a.frc[lp][i] = q;
        q.x = t.x;
        q.y = t.y;
        q.z = t.z;
        a.trq[lp][i] = q;
        a.epart[i] = double(e);
        ep = e;
    }
    warp_partials<R>(a, i, R(0), ep, 0.f, flags);
}

/* FP64 membrane area and enclosed volume of each system's face mesh, and
 * the constraint coefficients for the next force evaluation.  Each block sums
 * MESH_CHUNK faces of one system; the last block adds the block sums of each
 * system in block order (deterministic). */
template<class R> __global__ void __launch_bounds__(256) k_mesh(KArgs<R> a) {
    using T4 = typename Vec<R>::T4;
    const int b = blockIdx.x;
    const int s = a.mesh_blk_sys[b];
    const SysDev &sd = a.sys[s];
    __shared__ double sa[8], sv[8];
    __shared__ bool last;
    const int cur = __ldcg(&a.S->cur), lp = __ldcg(&a.S->lp);
    double ar = 0, vol = 0;
    const int f0 = sd.face_begin + (b - sd.mblk_begin) * MESH_CHUNK;
    const int f1 = min(sd.face_end, f0 + MESH_CHUNK);
    if (f1 > f0) {
        const int ref = a.faces[sd.face_begin].x;
        const T4 pr = a.pos[cur][ref];
        const int cr = a.cell[lp][ref];
        for (int f = f0 + int(threadIdx.x); f < f1; f += blockDim.x) {
            const int4 q = a.faces[f];
            double P[3][3];
            const int idx[3] = {q.x, q.y, q.z};
            for (int k = 0; k < 3; ++k) {
                const T4 pk = a.pos[cur][idx[k]];
                rel_pos<double>(sd, a.cell[lp][idx[k]], cr, pk, pr, P[k][0], P[k][1], P[k][2]);
            }
            const double e1[3] = {P[1][0] - P[0][0], P[1][1] - P[0][1], P[1][2] - P[0][2]};
            const double e2[3] = {P[2][0] - P[0][0], P[2][1] - P[0][1], P[2][2] - P[0][2]};
            const double nx = e1[1] * e2[2] - e1[2] * e2[1], ny = e1[2] * e2[0] - e1[0] * e2[2],
                         nz = e1[0] * e2[1] - e1[1] * e2[0];
            ar += sqrt(nx * nx + ny * ny + nz * nz);  // twice the area
            const double bx = P[1][1] * P[2][2] - P[1][2] * P[2][1], by = P[1][2] * P[2][0] - P[1][0] * P[2][2],
                         bz = P[1][0] * P[2][1] - P[1][1] * P[2][0];
            vol += P[0][0] * bx + P[0][1] * by + P[0][2] * bz;  // six times the volume
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        ar += __shfl_xor_sync(0xffffffffu, ar, o);
        vol += __shfl_xor_sync(0xffffffffu, vol, o);
    }
    if ((threadIdx.x & 31) == 0) {
        sa[threadIdx.x >> 5] = ar;
        sv[threadIdx.x >> 5] = vol;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double A = 0, V = 0;
        for (int w = 0; w < 8; ++w) {
            A += sa[w];
            V += sv[w];
        }
        a.mesh_partial[2 * b] = A;
        a.mesh_partial[2 * b + 1] = V;
        __threadfence();
        last = atomicAdd(&a.S->mesh_counter, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    const int lane = threadIdx.x & 31;
    for (int q = threadIdx.x >> 5; q < a.nsys; q += 8) {
        const SysDev &sq = a.sys[q];
        double A = 0, V = 0;
        for (int k = sq.mblk_begin + lane; k < sq.mblk_end; k += 32) {
            A += __ldcg(a.mesh_partial + 2 * k);
            V += __ldcg(a.mesh_partial + 2 * k + 1);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            A += __shfl_xor_sync(0xffffffffu, A, o);
            V += __shfl_xor_sync(0xffffffffu, V, o);
        }
        if (lane == 0) {
            A *= 0.5;  // the FP64 division once per system, not per face
            V /= 6.0;
            SysState &ss = a.ss[q];
            ss.area = A;
            ss.volume = V;
            ss.cv = (sq.kv != 0 && sq.V0 != 0) ? -sq.kv * (V - sq.V0) / sq.V0 : 0.0;
            ss.ca = (sq.ka != 0 && sq.A0 != 0) ? -sq.ka * (A - sq.A0) / sq.A0 : 0.0;
        }
    }
    if (threadIdx.x == 0) a.S->mesh_counter = 0;
}

}  // namespace

/* Force-kernel forms: the bits of FORM_* above (the list-build form, bits 3-4
 * of orbc_params.kernel_variant, is handled by the rebuild).  The merged and
 * compensated bits are instantiated on top of the pipelined, inlined loop. */
template<class R> void reduce_sums(const KArgs<R> &a, int mode, int count_step, cudaStream_t st) {
    k_reduce<R><<<a.ngroups, RED_GROUP, 0, st>>>(a, mode, count_step);
}
/* the pair-loop bits of a form (FORM_OCC dropped), rounded to an instantiated one */
constexpr int loop_form(int v) {
    return (v & (FORM_MERGED | FORM_KAHAN)) ? ((v & (FORM_MERGED | FORM_KAHAN)) | FORM_PIPE | FORM_INLINE) : (v & 3);
}
template<class R, int V> void step_langevin_v(const KArgs<R> &a, cudaStream_t st, bool energy) {
    if (energy) {
        k_step_langevin<R, true, loop_form(V)><<<a.npad / LITE_BS, LITE_BS, 0, st>>>(a);
        reduce_sums<R>(a, MODE_LANGEVIN, 1, st);
    } else if (a.zero_bulk) {
        k_step_langevin<R, false, loop_form(V)><<<a.npad / LITE_BS, LITE_BS, 0, st>>>(a);
        reduce_sums<R>(a, MODE_LANGEVIN, 1, st);
    } else {
        k_step_langevin_lite<R, V><<<a.npad / LITE_BS, LITE_BS, 0, st>>>(a);
        k_advance<<<1, 1, 0, st>>>(a.S, a.rebuild_every, 1);
    }
}
template<class R, int V> void nh_final_v(const KArgs<R> &a, cudaStream_t st, bool energy) {
    if (energy)
        k_nh_final<R, true, V><<<a.npad / LITE_BS, LITE_BS, 0, st>>>(a, 1);
    else
        k_nh_final<R, false, V><<<a.npad / LITE_BS, LITE_BS, 0, st>>>(a, 1);
    reduce_sums<R>(a, MODE_NH_FINAL, 1, st);
}
template<class R> void launch_step_langevin(const KArgs<R> &a, cudaStream_t st, bool energy) {
    const int ext = a.variant & (FORM_MERGED | FORM_KAHAN);
    if (ext) {  // the extended forms, with or without the occupancy form
        const bool occ = (a.variant & FORM_OCC) != 0;
        switch (ext | (occ ? FORM_OCC : 0)) {
            case FORM_MERGED: step_langevin_v<R, FORM_MERGED | 3>(a, st, energy); break;
            case FORM_KAHAN: step_langevin_v<R, FORM_KAHAN | 3>(a, st, energy); break;
            case FORM_MERGED | FORM_KAHAN: step_langevin_v<R, FORM_MERGED | FORM_KAHAN | 3>(a, st, energy); break;
            case FORM_MERGED | FORM_OCC: step_langevin_v<R, FORM_MERGED | 7>(a, st, energy); break;
            case FORM_KAHAN | FORM_OCC: step_langevin_v<R, FORM_KAHAN | 7>(a, st, energy); break;
            default: step_langevin_v<R, FORM_MERGED | FORM_KAHAN | 7>(a, st, energy); break;
        }
        return;
    }
    switch (a.variant & 7) {
        case 1: step_langevin_v<R, 1>(a, st, energy); break;
        case 2: step_langevin_v<R, 2>(a, st, energy); break;
        case 3: step_langevin_v<R, 3>(a, st, energy); break;
        case 4: step_langevin_v<R, 4>(a, st, energy); break;
        case 5: step_langevin_v<R, 5>(a, st, energy); break;
        case 6: step_langevin_v<R, 6>(a, st, energy); break;
        case 7: step_langevin_v<R, 7>(a, st, energy); break;
        default: step_langevin_v<R, 0>(a, st, energy); break;
    }
}
template<class R> void launch_nh_final(const KArgs<R> &a, cudaStream_t st, bool energy) {
    switch (loop_form(a.variant)) {
        case 1: nh_final_v<R, 1>(a, st, energy); break;
        case 2: nh_final_v<R, 2>(a, st, energy); break;
        case 3: nh_final_v<R, 3>(a, st, energy); break;
        case FORM_MERGED | 3: nh_final_v<R, FORM_MERGED | 3>(a, st, energy); break;
        case FORM_KAHAN | 3: nh_final_v<R, FORM_KAHAN | 3>(a, st, energy); break;
        case FORM_MERGED | FORM_KAHAN | 3: nh_final_v<R, FORM_MERGED | FORM_KAHAN | 3>(a, st, energy); break;
        default: nh_final_v<R, 0>(a, st, energy); break;
    }
}
template<class R> void launch_nh_prologue(const KArgs<R> &a, cudaStream_t st) {
    if (a.variant & FORM_KAHAN)
        k_nh_final<R, true, FORM_KAHAN | 3><<<a.npad / LITE_BS, LITE_BS, 0, st>>>(a, 0);
    else
        k_nh_final<R, true, 0><<<a.npad / LITE_BS, LITE_BS, 0, st>>>(a, 0);
    reduce_sums<R>(a, MODE_NH_FINAL, 0, st);
}
template<class R> void launch_nh_initial(const KArgs<R> &a, cudaStream_t st) {
    k_nh_initial<R><<<a.npad / 256, 256, 0, st>>>(a);
    reduce_sums<R>(a, MODE_NH_INITIAL, 0, st);
}
/* The forces hook evaluates pairs in the form's accumulation (plain or
 * compensated); the loop structure does not change the sums' order. */
template<class R> void launch_forces(const KArgs<R> &a, cudaStream_t st) {
    if (a.variant & FORM_KAHAN)
        k_forces<R, true, FORM_KAHAN | 3><<<a.npad / LITE_BS, LITE_BS, 0, st>>>(a);
    else
        k_forces<R, true, 0><<<a.npad / LITE_BS, LITE_BS, 0, st>>>(a);
    reduce_sums<R>(a, MODE_FORCES, 0, st);
}
template<class R> void launch_mesh(const KArgs<R> &a, cudaStream_t st) {
    if (a.nmblk > 0) k_mesh<R><<<a.nmblk, 256, 0, st>>>(a);
}
template<class R, int V> void minimize_v(const KArgs<R> &a, double dr_opt, double dn_opt, cudaStream_t st) {
    k_minimize<R, V><<<a.npad / LITE_BS, LITE_BS, 0, st>>>(a, dr_opt, dn_opt);
    k_advance<<<1, 1, 0, st>>>(a.S, a.rebuild_every, 0);
}
template<class R> void launch_minimize(const KArgs<R> &a, double dr_opt, double dn_opt, cudaStream_t st) {
    switch (a.variant & 3) {
        case 1: minimize_v<R, 1>(a, dr_opt, dn_opt, st); break;
        case 2: minimize_v<R, 2>(a, dr_opt, dn_opt, st); break;
        case 3: minimize_v<R, 3>(a, dr_opt, dn_opt, st); break;
        default: minimize_v<R, 0>(a, dr_opt, dn_opt, st); break;
    }
}
template<class R> void launch_vcom(const KArgs<R> &a, cudaStream_t st) {
    k_vcom<R><<<a.npad / 256, 256, 0, st>>>(a);
    reduce_sums<R>(a, MODE_VCOM, 0, st);
}
template<class R> void launch_assign_temperature(const KArgs<R> &a, double kT, uint64_t seed, cudaStream_t st) {
    k_assign_temperature<R><<<(a.npad + 255) / 256, 256, 0, st>>>(a, kT, seed);
}

#define ORBC_INST(R)                                                                   \
    template void launch_step_langevin<R>(const KArgs<R> &, cudaStream_t, bool);      \
    template void launch_nh_final<R>(const KArgs<R> &, cudaStream_t, bool);           \
    template void launch_nh_prologue<R>(const KArgs<R> &, cudaStream_t);              \
    template void launch_nh_initial<R>(const KArgs<R> &, cudaStream_t);               \
    template void launch_forces<R>(const KArgs<R> &, cudaStream_t);                   \
    template void launch_vcom<R>(const KArgs<R> &, cudaStream_t);                     \
    template void launch_minimize<R>(const KArgs<R> &, double, double, cudaStream_t); \
    template void launch_assign_temperature<R>(const KArgs<R> &, double, uint64_t, cudaStream_t); \
    template void launch_mesh<R>(const KArgs<R> &, cudaStream_t);
ORBC_INST(float)
ORBC_INST(double)
#undef ORBC_INST

}  // namespace orbc
