// Stray-lipid cleanup (delete_lipid, src/cleanup.h:29-91) on the device.
//
// The reference affiliates every lipid with its nearest Voronoi centroid
// (cells of ~14 lipids) and, per Voronoi cell, removes the lipids whose
// squared distance to the centroid is not below stray_tolerance^2 times the
// median one, then compacts the lipid container.  Here the Voronoi generators
// start as the lipid centroids of the grid cells holding at least `mingen`
// lipids (a cell of ~3.4 sigma holds ~10 lipids of a membrane); every lipid is
// affiliated with the nearest generator homed among the surrounding cells
// (3^3, then 5^3; none within that is a stray), and four Lloyd updates move each generator to the mean of its
// members (dissolving generators left with too few) and re-affiliate, as the
// reference's Voronoi update does.  The
// (generator, slot) pairs are radix-sorted and one warp per generator finds
// the median squared distance by rank counting and marks the strays.  A
// generator is named by its home cell's first slot.  Removal turns the marked slots into ghosts (the next rebuild
// sorts them behind the live particles) and renumbers the survivors' upload
// indices in order, as the reference's compaction does.
#include "orbc_device.cuh"

namespace orbc {

namespace {

constexpr uint32_t CL_NONE = 0xffffffffu;
constexpr int CL_LLOYD = 4;  // centroid updates after the first affiliation

template<class R>
__device__ __forceinline__ int abs_pos(const KArgs<R> &a, const SysDev &sd, int cur, int lp, int p, double x[3]) {
    const auto q = a.pos[cur][p];
    const int cl = a.cell[lp][p];
    const int cc[3] = {cx_of(cl), cy_of(cl), cz_of(cl)};
    const double off[3] = {double(q.x), double(q.y), double(q.z)};
#pragma unroll
    for (int d = 0; d < 3; ++d) x[d] = __dadd_rn(__dadd_rn(sd.lo[d], __dmul_rn(double(cc[d]) + 0.5, sd.Lc[d])), off[d]);
    return w_type(wbits(q.w));
}

/* Generators: the first slot of each occupied cell holds the cell's lipid
 * centroid and lipid count (FP64, slot order) -- a generator when the cell
 * holds at least mingen lipids. */
template<class R> __global__ void k_cl_gen(KArgs<R> a, double4a *gen, int mingen) {
    const int cur = __ldcg(&a.S->cur), lp = __ldcg(&a.S->lp);
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < a.npad; p += gridDim.x * blockDim.x) {
        const SysDev &sd = a.sys[a.blk_sys[p / SYS_PAD]];
        if (w_type(wbits(a.pos[cur][p].w)) == GHOST) continue;
        const int cl = a.cell[lp][p];
        const int2 rg = a.ranges[sd.cell_base + cell_code(sd, cx_of(cl), cy_of(cl), cz_of(cl))];
        if (rg.x != p) continue;
        double c[3] = {0, 0, 0};
        int cnt = 0;
        for (int q = rg.x; q < rg.y; ++q) {
            double x[3];
            if (abs_pos(a, sd, cur, lp, q, x) != 0) continue;
            for (int d = 0; d < 3; ++d) c[d] += x[d];
            ++cnt;
        }
        double4a G;
        G.x = cnt ? c[0] / cnt : 0.0;
        G.y = cnt ? c[1] / cnt : 0.0;
        G.z = cnt ? c[2] / cnt : 0.0;
        G.w = cnt >= mingen ? double(cnt) : -1.0;  // w > 0: a generator
        gen[p] = G;
    }
}

/* Affiliation of each lipid with its nearest generator; key = generator
 * (first slot of its home cell; CL_NONE for non-lipids, CL_NONE - 1 for a
 * stray with no generator homed within two cells), dr2 = squared distance. */
template<class R>
__global__ void k_cl_assign(KArgs<R> a, const double4a *gen, uint32_t *key, int *val, double *dr2) {
    const int cur = __ldcg(&a.S->cur), lp = __ldcg(&a.S->lp);
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < a.npad; p += gridDim.x * blockDim.x) {
        const SysDev &sd = a.sys[a.blk_sys[p / SYS_PAD]];
        double x[3];
        uint32_t k = CL_NONE;
        double best = -1.0;
        if (abs_pos(a, sd, cur, lp, p, x) == 0) {
            const int cl = a.cell[lp][p];
            const int c0[3] = {cx_of(cl), cy_of(cl), cz_of(cl)};
            double L[3];
            for (int d = 0; d < 3; ++d) L[d] = sd.per[d] ? double(sd.nc[d]) * sd.Lc[d] : 0.0;
            for (int rad = 1; rad <= 2 && k == CL_NONE; ++rad) {
                for (int dz = -rad; dz <= rad; ++dz)
                    for (int dy = -rad; dy <= rad; ++dy)
                        for (int dx = -rad; dx <= rad; ++dx) {
                            int t[3] = {c0[0] + dx, c0[1] + dy, c0[2] + dz};
                            bool ok = true;
                            for (int d = 0; d < 3; ++d) {
                                if (sd.per[d])
                                    t[d] = ((t[d] % sd.nc[d]) + sd.nc[d]) % sd.nc[d];
                                else
                                    ok = ok && t[d] >= 0 && t[d] < sd.nc[d];
                            }
                            if (!ok) continue;
                            const int2 rg = a.ranges[sd.cell_base + cell_code(sd, t[0], t[1], t[2])];
                            if (rg.y <= rg.x) continue;
                            const double4a G = gen[rg.x];
                            if (!(G.w > 0.0)) continue;
                            double q[3] = {x[0] - G.x, x[1] - G.y, x[2] - G.z};
                            for (int d = 0; d < 3; ++d)
                                if (L[d] > 0) q[d] -= L[d] * rint(q[d] / L[d]);
                            const double r2 = q[0] * q[0] + q[1] * q[1] + q[2] * q[2];
                            if (k == CL_NONE || r2 < best || (r2 == best && uint32_t(rg.x) < k)) {
                                best = r2;
                                k = uint32_t(rg.x);
                            }
                        }
            }
            if (k == CL_NONE) k = CL_NONE - 1;
        }
        key[p] = k;
        val[p] = p;
        dr2[p] = best;
    }
}

/* One Lloyd iteration (as the reference's Voronoi update moves each centroid
 * to the mean of its cell's members): every generator moves by the mean
 * minimum-image offset of the lipids now affiliated with it; a generator left
 * with fewer than mingen members is dissolved.  One warp per generator. */
template<class R>
__global__ void k_cl_update(KArgs<R> a, double4a *gen, int mingen, const uint32_t *skey, const int *sval) {
    const int lane = threadIdx.x & 31;
    const int wglob = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    const int cur = __ldcg(&a.S->cur), lp = __ldcg(&a.S->lp);
    const int n = a.npad;
    for (int g = wglob; g < n; g += nwarps) {
        const double4a G0 = gen[g];
        if (!(G0.w > 0.0)) continue;  // not a generator (or dissolved)
        const SysDev &sd = a.sys[a.blk_sys[g / SYS_PAD]];
        int lo = 0, hi = n;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (skey[mid] < uint32_t(g)) lo = mid + 1;
            else hi = mid;
        }
        int e = lo, h2 = n;
        while (e < h2) {
            const int mid = (e + h2) >> 1;
            if (skey[mid] <= uint32_t(g)) e = mid + 1;
            else h2 = mid;
        }
        const double g0[3] = {G0.x, G0.y, G0.z};
        double c[3] = {0, 0, 0};
        for (int q = lo + lane; q < e; q += 32) {
            double x[3];
            abs_pos(a, sd, cur, lp, sval[q], x);
            for (int d = 0; d < 3; ++d) {
                double u = x[d] - g0[d];
                if (sd.per[d]) {
                    const double L = double(sd.nc[d]) * sd.Lc[d];
                    u -= L * rint(u / L);
                }
                c[d] += u;
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            for (int d = 0; d < 3; ++d) c[d] += __shfl_xor_sync(0xffffffffu, c[d], o);
        __syncwarp();
        if (lane == 0) {
            const int cnt = e - lo;
            double4a G = G0;
            if (cnt >= mingen) {
                G.x = g0[0] + c[0] / cnt;
                G.y = g0[1] + c[1] / cnt;
                G.z = g0[2] + c[2] / cnt;
                G.w = double(cnt);
            } else {
                G.w = -1.0;
            }
            gen[g] = G;
        }
    }
}

/* Median per generator (rank counting over its sorted segment) and marks;
 * one warp per candidate generator slot, plus one task for the strays. */
template<class R>
__global__ void k_cl_mark(KArgs<R> a, const double4a *gen, int mingen, const uint32_t *skey, const int *sval,
                          const double *dr2, double tol2, int *gone_home, unsigned long long *removed) {
    const int lane = threadIdx.x & 31;
    const int wglob = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    const int lp = __ldcg(&a.S->lp);
    const int n = a.npad;
    for (int tw = wglob; tw <= n; tw += nwarps) {
        uint32_t g;
        if (tw < n) {
            if (!(gen[tw].w > 0.0)) continue;  // generators sit at their brick's first slot
            g = uint32_t(tw);
        } else {
            g = CL_NONE - 1;
        }
        int lo = 0, hi = n;  // lower bound of g
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (skey[mid] < g) lo = mid + 1;
            else hi = mid;
        }
        int e = lo, h2 = n;  // upper bound of g
        while (e < h2) {
            const int mid = (e + h2) >> 1;
            if (skey[mid] <= g) e = mid + 1;
            else h2 = mid;
        }
        if (e <= lo) continue;
        unsigned long long gone = 0;
        if (g == CL_NONE - 1) {
            for (int q = lo + lane; q < e; q += 32) {
                gone_home[a.home[lp][sval[q]]] = 1;
                ++gone;
            }
        } else if (e - lo >= mingen) {  // fewer members: no statistics, all kept
            const int cnt = e - lo, want = cnt / 2;
            double med = -1.0;
            for (int q = lo + lane; q < e; q += 32) {
                const double v = dr2[sval[q]];
                int rank = 0;
                for (int u = lo; u < e; ++u) {
                    const double w = dr2[sval[u]];
                    rank += (w < v || (w == v && u < q)) ? 1 : 0;
                }
                if (rank == want) med = v;
            }
            const unsigned who = __ballot_sync(0xffffffffu, med >= 0);
            med = __shfl_sync(0xffffffffu, med, __ffs(who) - 1);
            const double thr = med * tol2;
            for (int q = lo + lane; q < e; q += 32) {
                const int p = sval[q];
                if (!(dr2[p] < thr)) {
                    gone_home[a.home[lp][p]] = 1;
                    ++gone;
                }
            }
        }
        gone = __reduce_add_sync(0xffffffffu, unsigned(gone));
        if (lane == 0 && gone) atomicAdd(removed, gone);
    }
}

/* Marked slots become ghosts (their old cells' ranges cleared, so the next
 * rebuild drops them); survivors get their new upload index. */
template<class R> __global__ void k_cleanup_apply(KArgs<R> a, const int *newidx, int *soh_new) {
    const int cur = __ldcg(&a.S->cur), lp = __ldcg(&a.S->lp);
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < a.npad; p += gridDim.x * blockDim.x) {
        const int h = a.home[lp][p];
        if (h < 0) continue;
        const int nh = newidx[h];
        if (nh >= 0) {
            a.home[lp][p] = nh;
            soh_new[nh] = p;
            continue;
        }
        const SysDev &sd = a.sys[a.blk_sys[p / SYS_PAD]];
        const int c = a.cell[lp][p];
        a.ranges[sd.cell_base + cell_code(sd, cx_of(c), cy_of(c), cz_of(c))] = make_int2(0, 0);
        auto q = a.pos[cur][p];
        wset(q.w, GHOST);
        a.pos[cur][p] = q;
        a.home[lp][p] = -1;
        auto z = a.vel[lp][p];
        z.x = z.y = z.z = 0;
        a.vel[lp][p] = z;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) a.S->rebuild = 1;
}

int cl_blocks(int64_t threads) { return int(std::min<int64_t>((threads + 255) / 256, 152 * 16)); }

}  // namespace

/* Marks (gone_home[upload index] = 1, zeroed by the caller) of the strays of
 * the current state.  gen (zeroed by the caller) and dr2 hold npad entries. */
template<class R>
int launch_cleanup_mark(const KArgs<R> &a, int mingen, double tol2, double4a *gen, double *dr2, int *gone_home,
                        unsigned long long *removed, cudaStream_t st) {
    k_cl_gen<R><<<cl_blocks(a.npad), 256, 0, st>>>(a, gen, mingen);
    int fin = 0;
    for (int it = 0; it <= CL_LLOYD; ++it) {
        if (it > 0)
            k_cl_update<R><<<cl_blocks(int64_t(a.npad) * 32), 256, 0, st>>>(a, gen, mingen, a.skey[fin], a.sval[fin]);
        k_cl_assign<R><<<cl_blocks(a.npad), 256, 0, st>>>(a, gen, a.skey[0], a.sval[0], dr2);
        fin = radix_sort_pairs(const_cast<uint32_t **>(a.skey), const_cast<int **>(a.sval), a.counts, a.digit_total,
                               nullptr, a.npad, 4, a.ntiles, nullptr, st);
    }
    k_cl_mark<R><<<cl_blocks((int64_t(a.npad) + 1) * 32), 256, 0, st>>>(a, gen, mingen, a.skey[fin], a.sval[fin],
                                                                        dr2, tol2, gone_home, removed);
    return cudaGetLastError() == cudaSuccess ? 0 : 1;
}
template<class R> void launch_cleanup_apply(const KArgs<R> &a, const int *newidx, int *soh_new, cudaStream_t st) {
    k_cleanup_apply<R><<<cl_blocks(a.npad), 256, 0, st>>>(a, newidx, soh_new);
}

template int launch_cleanup_mark<float>(const KArgs<float> &, int, double, double4a *, double *, int *,
                                        unsigned long long *, cudaStream_t);
template int launch_cleanup_mark<double>(const KArgs<double> &, int, double, double4a *, double *, int *,
                                         unsigned long long *, cudaStream_t);
template void launch_cleanup_apply<float>(const KArgs<float> &, const int *, int *, cudaStream_t);
template void launch_cleanup_apply<double>(const KArgs<double> &, const int *, int *, cudaStream_t);

}  // namespace orbc
