// Spatial sort, cell binning and neighbour-list build (the GPU replacement of
// the reference's Voronoi tessellation + k-d tree + Morton reorder:
// src/voronoi.h:143-237, src/kdtree.h:117-285, src/reorder_morton.h:44-122,
// src/reorder.h:33-149), plus state conversion between the caller's AoS
// double arrays and the device layout.
//
// Rebuild chain (runs only when a particle moved more than skin/2 since the
// last build, or on demand):
//   k_rebin          re-express each position in the cell that now holds it,
//                    clear the old cell ranges, emit (cell key, slot) pairs
//   LSD radix sort   stable, 8-bit digits, (key, slot) -> sorted + inverse map
//   k_ranges_gather  cell [begin, end) ranges and the physical reorder of all
//                    per-particle arrays (bond / face partners remapped)
//   k_nlist          full neighbour list per particle from the 27 cells
//                    around its own; the last block flips buffer parities
#include "orbc_device.cuh"

#include <cstdio>

namespace orbc {

namespace {

__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }


__device__ __forceinline__ int gate_closed(const int *gate) { return gate && !__ldcg(gate); }

}  // namespace

/* ------------------------------------------------------------------------- */
/* LSD radix sort of (uint32 key, int value) pairs, 8-bit digits, stable.     */
/* One 4096-key tile per block: histogram -> per-digit scan over tiles ->    */
/* stable in-tile ranking (warp match + per-warp digit counts) and scatter.  */
/* ------------------------------------------------------------------------- */
__global__ void __launch_bounds__(256) k_rs_hist(const uint32_t *keys, int64_t n, int shift, int *counts,
                                                  int ntiles, const int *gate) {
    if (gate_closed(gate)) return;
    __shared__ int h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const int64_t base = int64_t(blockIdx.x) * SORT_TILE;
#pragma unroll 4
    for (int k = 0; k < SORT_TILE / 256; ++k) {
        const int64_t idx = base + k * 256 + threadIdx.x;
        if (idx < n) atomicAdd(&h[(keys[idx] >> shift) & 255u], 1);
    }
    __syncthreads();
    counts[int64_t(threadIdx.x) * ntiles + blockIdx.x] = h[threadIdx.x];
}

__global__ void __launch_bounds__(1024) k_rs_scan(int *counts, int ntiles, int *digit_total, const int *gate) {
    if (gate_closed(gate)) return;
    __shared__ int wsum[32];
    __shared__ int carry;
    int *row = counts + int64_t(blockIdx.x) * ntiles;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < ntiles; base += 1024) {
        const int i = base + threadIdx.x;
        const int v = i < ntiles ? row[i] : 0;
        int x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) wsum[warp] = x;
        __syncthreads();
        if (warp == 0) {
            int s = wsum[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, s, o);
                if (lane >= o) s += y;
            }
            wsum[lane] = s;
        }
        __syncthreads();
        const int incl = x + (warp > 0 ? wsum[warp - 1] : 0);
        const int c0 = carry;
        if (i < ntiles) row[i] = c0 + incl - v;
        __syncthreads();
        if (threadIdx.x == 1023) carry = c0 + incl;
        __syncthreads();
    }
    if (threadIdx.x == 0) digit_total[blockIdx.x] = carry;
}

__global__ void __launch_bounds__(256) k_rs_scatter(const uint32_t *kin, const int *vin, uint32_t *kout, int *vout,
                                                     int64_t n, int shift, const int *counts, int ntiles,
                                                     const int *digit_total, int *inv, const int *gate) {
    if (gate_closed(gate)) return;
    __shared__ int base_s[256];
    __shared__ int run[256];
    __shared__ int wcnt[8][256];
    __shared__ int wsum[8];
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    // exclusive scan of the digit totals -> global digit base
    {
        const int v = digit_total[t];
        int x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) wsum[warp] = x;
        __syncthreads();
        int off = 0;
        for (int w = 0; w < warp; ++w) off += wsum[w];
        base_s[t] = off + x - v + counts[int64_t(t) * ntiles + blockIdx.x];
        run[t] = 0;
    }
    const unsigned lt = (1u << lane) - 1u;
    const int64_t tb = int64_t(blockIdx.x) * SORT_TILE;
    for (int r = 0; r < SORT_TILE / 256; ++r) {
#pragma unroll
        for (int k = 0; k < 8; ++k) wcnt[k][t] = 0;
        __syncthreads();
        const int64_t idx = tb + r * 256 + t;
        const bool valid = idx < n;
        const uint32_t key = valid ? kin[idx] : 0u;
        const int val = valid ? vin[idx] : 0;
        const int dg = valid ? int((key >> shift) & 255u) : 256;
        const unsigned peers = __match_any_sync(0xffffffffu, dg);
        const int rank = __popc(peers & lt);
        if (valid && lane == __ffs(peers) - 1) wcnt[warp][dg] = __popc(peers);
        __syncthreads();
        {
            int acc = run[t];
#pragma unroll
            for (int w = 0; w < 8; ++w) {
                const int c = wcnt[w][t];
                wcnt[w][t] = acc;
                acc += c;
            }
            run[t] = acc;
        }
        __syncthreads();
        if (valid) {
            const int pos = base_s[dg] + wcnt[warp][dg] + rank;
            kout[pos] = key;
            vout[pos] = val;
            if (inv) inv[val] = pos;
        }
        __syncthreads();
    }
}

int sort_tiles(int64_t n) { return int((n + SORT_TILE - 1) / SORT_TILE); }

int radix_sort_pairs(uint32_t *keys[2], int *vals[2], int *counts, int *digit_total, int *inv, int64_t n,
                     int passes, int ntiles, const int *gate, cudaStream_t st) {
    int cur = 0;
    for (int p = 0; p < passes; ++p) {
        const int shift = 8 * p;
        k_rs_hist<<<ntiles, 256, 0, st>>>(keys[cur], n, shift, counts, ntiles, gate);
        k_rs_scan<<<256, 1024, 0, st>>>(counts, ntiles, digit_total, gate);
        k_rs_scatter<<<ntiles, 256, 0, st>>>(keys[cur], vals[cur], keys[1 - cur], vals[1 - cur], n, shift, counts,
                                             ntiles, digit_total, p == passes - 1 ? inv : nullptr, gate);
        cur = 1 - cur;
    }
    return cur;
}

/* ------------------------------------------------------------------------- */
/* Rebuild chain                                                             */
/* ------------------------------------------------------------------------- */
template<class R> __global__ void __launch_bounds__(256) k_rebin(KArgs<R> a, int gated) {
    using T4 = typename Vec<R>::T4;
    if (gated && !__ldcg(&a.S->rebuild)) return;
    const int cur = __ldcg(&a.S->cur), lp = __ldcg(&a.S->lp);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.S->max_nnb = 0;
        a.S->out_of_grid = 0;
    }
    int out = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.npad; i += gridDim.x * blockDim.x) {
        const SysDev &sd = a.sys[a.blk_sys[i / SYS_PAD]];
        T4 p = a.pos[cur][i];
        const int w = wbits(p.w);
        uint32_t key;
        if (w_type(w) == GHOST) {
            key = sd.cell_base + ncell_ids(sd);
        } else {
            const int c = a.cell[lp][i];
            int cc[3] = {cx_of(c), cy_of(c), cz_of(c)};
            a.ranges[sd.cell_base + cell_code(sd, cc[0], cc[1], cc[2])] = make_int2(0, 0);
            R o[3] = {p.x, p.y, p.z};
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                const R L = lc_of<R>(sd, d);
                const R invL = inv_lc_of<R>(sd, d);
                const int k = int(floor(add_rn(mul_rn(o[d], invL), R(0.5))));
                int nc = cc[d] + k;
                if (sd.per[d]) {
                    o[d] = sub_rn(o[d], mul_rn(R(k), L));
                    nc %= sd.nc[d];
                    if (nc < 0) nc += sd.nc[d];
                } else {
                    const int cl = min(max(nc, 0), sd.nc[d] - 1);
                    if (cl != nc) out = 1;
                    o[d] = sub_rn(o[d], mul_rn(R(cl - cc[d]), L));
                    nc = cl;
                }
                cc[d] = nc;
            }
            p.x = o[0];
            p.y = o[1];
            p.z = o[2];
            a.pos[cur][i] = p;  // the gather that follows sets the displacement reference
            a.cell[lp][i] = cpack(cc[0], cc[1], cc[2]);
            key = sd.cell_base + cell_code(sd, cc[0], cc[1], cc[2]);
        }
        a.skey[0][i] = key;
        a.sval[0][i] = i;
    }
    if (out) {
        atomicOr(&a.S->error, ERRB_GRID);
        atomicAdd(&a.S->out_of_grid, 1);
    }
}

template<class R> __global__ void __launch_bounds__(256) k_ranges_gather(KArgs<R> a, int fin, int gated) {
    if (gated && !__ldcg(&a.S->rebuild)) return;
    const int cur = __ldcg(&a.S->cur), lp = __ldcg(&a.S->lp);
    const int nc = 1 - cur, nl = 1 - lp;
    const uint32_t *sk = a.skey[fin];
    const int *sv = a.sval[fin];
    const int n = a.npad;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        // every load of the slot before its first store: the stores may alias
        // the loads as far as the compiler knows, and would serialise them
        const uint32_t k = sk[p];
        const bool first = p == 0 || sk[p - 1] != k, last = p == n - 1 || sk[p + 1] != k;
        const int src = sv[p];
        const auto ps = a.pos[cur][src];
        const auto ns = a.nrm[cur][src];
        const auto vs = a.vel[lp][src];
        const auto os = a.omg[lp][src];
        const int cs = a.cell[lp][src], ts = a.tag[lp][src], h = a.home[lp][src];
        if (a.carry_forces) {  // Nose-Hoover carries f and t from one half-step to the next
            const auto fs = a.frc[lp][src], qs = a.trq[lp][src];
            a.frc[nl][p] = fs;
            a.trq[nl][p] = qs;
        }
        if (first) a.ranges[k].x = p;
        if (last) a.ranges[k].y = p + 1;
        a.pos[nc][p] = ps;
        a.nrm[nc][p] = ns;
        a.vel[nl][p] = vs;
        a.omg[nl][p] = os;
        a.xref[nl][p] = ps;  // the list about to be built is referenced to these positions
        a.cell[nl][p] = cs;
        a.tag[nl][p] = ts;
        a.home[nl][p] = h;
        if (h >= 0) a.slot_of_home[h] = p;
        const int w = wbits(ps.w);
        const int bd = w_bdeg(w), fd = w_fdeg(w);
        for (int b = 0; b < bd; ++b) {
            BondSlot s = a.bond[lp][int64_t(b) * n + src];
            s.partner = a.inv[s.partner];
            a.bond[nl][int64_t(b) * n + p] = s;
        }
        for (int b = 0; b < fd; ++b) {
            int2 s = a.fslot[lp][int64_t(b) * n + src];
            s.x = a.inv[s.x];
            s.y = a.inv[s.y];
            a.fslot[nl][int64_t(b) * n + p] = s;
        }
    }
    for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < a.nfaces; f += gridDim.x * blockDim.x) {
        int4 q = a.faces[f];
        q.x = a.inv[q.x];
        q.y = a.inv[q.y];
        q.z = a.inv[q.z];
        a.faces[f] = q;
    }
}

/* End of a list build: block max of the candidate counts -> global max and
 * overflow flag; the last block to finish makes the new buffers current and
 * clears the rebuild request. */
template<class R> __device__ __forceinline__ void nlist_finalise(const KArgs<R> &a, int maxc, int cur, int lp) {
    __shared__ int smax[8];
    __shared__ bool last;
    int m = maxc;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) smax[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        int bm = 0;
        for (int w = 0; w < int(blockDim.x >> 5); ++w) bm = max(bm, smax[w]);
        atomicMax(&a.S->max_nnb, bm);
        if (bm > a.cap) atomicOr(&a.S->error, ERRB_NBR_OVERFLOW);
        __threadfence();
        const unsigned ticket = atomicAdd(&a.S->blk_counter, 1u);
        last = (ticket == gridDim.x - 1);
    }
    __syncthreads();
    if (last && threadIdx.x == 0) {
        a.S->cur = cur;
        a.S->lp = lp;
        a.S->rebuild = 0;
        a.S->rebuilds += 1;
        a.S->since_rebuild = 0;
        a.S->blk_counter = 0;
        __threadfence();
    }
}

template<class R> __global__ void __launch_bounds__(128) k_nlist(KArgs<R> a, int gated) {
    using T4 = typename Vec<R>::T4;
    if (gated && !__ldcg(&a.S->rebuild)) return;
    constexpr int CAND = sizeof(T4) == 16 ? 384 : 192;  // staged candidates per warp and pass
    constexpr int NLW = 4;                                // warps per block
    __shared__ float rl2s[256], ri2s[256];
    __shared__ T4 s_pos[NLW][CAND];
    __shared__ int s_j[NLW][CAND];
    __shared__ unsigned char s_code[NLW][CAND];           // shift code of the candidate's cell (0..26)
    __shared__ int s_off[NLW][28], s_beg[NLW][27];
    const int warp = threadIdx.x >> 5;
    for (int k = threadIdx.x; k < 256; k += blockDim.x) {
        rl2s[k] = __ldg(&a.ff->rlist2[k]);
        ri2s[k] = __ldg(&a.ff->rin2[k]);
    }
    __syncthreads();
    const int cur = 1 - __ldcg(&a.S->cur), lp = 1 - __ldcg(&a.S->lp);
    const int n = a.npad;
    int maxc = 0;
    // n is a multiple of the block size, so whole warps stay in the loop together
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const T4 p = a.pos[cur][i];
        const int ty = w_type(wbits(p.w));
        const bool real = ty != GHOST;
        const SysDev &sd = a.sys[a.blk_sys[i / SYS_PAD]];  // one system per warp (SYS_PAD-aligned)
        const int c = a.cell[lp][i];
        const int cc[3] = {cx_of(c), cy_of(c), cz_of(c)};
        const R L[3] = {lc_of<R>(sd, 0), lc_of<R>(sd, 1), lc_of<R>(sd, 2)};
        // Entries inside the pair's interaction range fill rows 0, 1, ... of
        // this slot's column; skin-shell entries fill rows cap-1, cap-2, ...
        int nin = 0, nout = 0, total = 0;
        // Candidate j seen from i's cell: o_j + d * Lc (d = cell_j - cell_i);
        // x_i - x_j = o_i - (o_j + d * Lc).  Both list-build forms use these
        // two functions, so they accept the same pairs.
        auto shifted = [&](const T4 &q, int dx, int dy, int dz) {
            T4 r = q;
            r.x = q.x + R(dx) * L[0];
            r.y = q.y + R(dy) * L[1];
            r.z = q.z + R(dz) * L[2];
            return r;
        };
        auto dist2 = [&](const T4 &pi, const T4 &qs) {
            const R ex = pi.x - qs.x, ey = pi.y - qs.y, ez = pi.z - qs.z;
            return ex * ex + ey * ey + ez * ez;
        };
        auto test = [&](int j, const T4 &q, int dx, int dy, int dz) {
            const int tj = w_type(wbits(q.w));
            const float rl2 = rl2s[ty * 16 + tj];
            if (!(rl2 > 0.f)) return;
            const R r2 = dist2(p, shifted(q, dx, dy, dz));
            if (r2 < R(rl2)) {
                const uint32_t ent = uint32_t(j) | (uint32_t((dx + 1) + 3 * (dy + 1) + 9 * (dz + 1)) << NB_SHIFT);
                if (nin + nout < a.cap) {
                    if (r2 < R(ri2s[ty * 16 + tj]))
                        a.nbr[nbr_index(i, nin++, a.cap)] = ent;
                    else
                        a.nbr[nbr_index(i, a.cap - 1 - nout++, a.cap)] = ent;
                }
                ++total;
            }
        };
        // Form 0 (warp sweep): consecutive slots sit in a few neighbouring
        // cells (cell ids follow tiles).  For each distinct cell of the warp,
        // 27 lanes fetch the ranges of its 27 neighbour cells, a warp scan
        // turns them into offsets and the candidates are staged in shared
        // memory (CAND per pass, all loads issued together); then for each
        // particle in that cell the 32 lanes test 32 candidates at a time and
        // accepted entries are placed by ballot and prefix count.  Form 1
        // (per-lane sweep): every lane walks its own 27 cells.
        bool swept = false;
        if (!a.nlist_lane) {
            swept = true;
            const int kme = cc[0] | (cc[1] << 11) | (cc[2] << 22);
            int *off = s_off[warp];
            int *beg = s_beg[warp];
            unsigned todo = __ballot_sync(0xffffffffu, real);
            while (todo) {
                // the lanes in one cell share its candidates
                const int kd = __shfl_sync(0xffffffffu, kme, __ffs(todo) - 1);
                const unsigned grp = __ballot_sync(0xffffffffu, real && kme == kd);
                todo &= ~grp;
                const int xd = kd & 2047, yd = (kd >> 11) & 2047, zd = (kd >> 22) & 1023;
                int2 rg = make_int2(0, 0);
                if (lane < 27) {
                    int x = xd + lane % 3 - 1, y = yd + (lane / 3) % 3 - 1, z = zd + lane / 9 - 1;
                    bool ok = true;
                    if (sd.per[0]) x = x < 0 ? x + sd.nc[0] : (x >= sd.nc[0] ? x - sd.nc[0] : x);
                    else ok = ok && x >= 0 && x < sd.nc[0];
                    if (sd.per[1]) y = y < 0 ? y + sd.nc[1] : (y >= sd.nc[1] ? y - sd.nc[1] : y);
                    else ok = ok && y >= 0 && y < sd.nc[1];
                    if (sd.per[2]) z = z < 0 ? z + sd.nc[2] : (z >= sd.nc[2] ? z - sd.nc[2] : z);
                    else ok = ok && z >= 0 && z < sd.nc[2];
                    if (ok) rg = a.ranges[sd.cell_base + cell_code(sd, x, y, z)];
                }
                const int cnt = rg.y > rg.x ? rg.y - rg.x : 0;
                int inc = cnt;  // inclusive warp scan
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int t = __shfl_up_sync(0xffffffffu, inc, o);
                    if (lane >= o) inc += t;
                }
                if (lane < 27) {
                    off[lane] = inc - cnt;
                    beg[lane] = rg.x;
                }
                const int total_c = __shfl_sync(0xffffffffu, inc, 31);
                if (lane == 0) off[27] = total_c;
                __syncwarp();
                // per-particle counters of this cell's particles, carried across passes
                int cin = 0, cout = 0, ctot = 0;
                for (int c0 = 0; c0 < total_c; c0 += CAND) {
                    const int nch = min(CAND, total_c - c0);
                    for (int t = lane; t < nch; t += 32) {
                        const int idx = c0 + t;
                        int l = 0;  // last neighbour cell with off[l] <= idx
#pragma unroll
                        for (int step = 16; step > 0; step >>= 1)
                            if (l + step < 27 && off[l + step] <= idx) l += step;
                        const int j = beg[l] + (idx - off[l]);
                        s_pos[warp][t] = shifted(a.pos[cur][j], l % 3 - 1, (l / 3) % 3 - 1, l / 9 - 1);
                        s_j[warp][t] = j;
                        s_code[warp][t] = (unsigned char)l;
                    }
                    __syncwarp();
                    for (unsigned g = grp; g; g &= g - 1u) {
                        const int il = __ffs(g) - 1;
                        T4 pi = p;
                        pi.x = __shfl_sync(0xffffffffu, p.x, il);
                        pi.y = __shfl_sync(0xffffffffu, p.y, il);
                        pi.z = __shfl_sync(0xffffffffu, p.z, il);
                        const int ti = __shfl_sync(0xffffffffu, ty, il);
                        const int gi = i - lane + il;
                        int qin = __shfl_sync(0xffffffffu, cin, il), qout = __shfl_sync(0xffffffffu, cout, il);
                        int qtot = __shfl_sync(0xffffffffu, ctot, il);
                        uint32_t *col = a.nbr + nbr_index(gi, 0, a.cap);  // row k of gi at col[32 k]
                        // lipid-lipid pairs (the bulk) take their cutoffs from registers
                        const float rl2_ll = rl2s[ti * 16], ri2_ll = ri2s[ti * 16];
                        for (int b0 = 0; b0 < nch; b0 += 32) {
                            const int t = b0 + lane;
                            bool acc = false, inner = false;
                            uint32_t ent = 0;
                            if (t < nch) {
                                const int j = s_j[warp][t];
                                const T4 q = s_pos[warp][t];
                                const int tj = w_type(wbits(q.w));
                                const float rl2 = tj == 0 ? rl2_ll : rl2s[ti * 16 + tj];
                                if (j != gi && rl2 > 0.f) {
                                    const R r2 = dist2(pi, q);
                                    if (r2 < R(rl2)) {
                                        acc = true;
                                        inner = r2 < R(tj == 0 ? ri2_ll : ri2s[ti * 16 + tj]);
                                        ent = uint32_t(j) | (uint32_t(s_code[warp][t]) << NB_SHIFT);
                                    }
                                }
                            }
                            const unsigned ma = __ballot_sync(0xffffffffu, acc);
                            const unsigned mi = __ballot_sync(0xffffffffu, acc && inner);
                            // entries past the capacity are counted, not written
                            unsigned mw = ma;
                            if (qin + qout + __popc(ma) > a.cap)
                                mw = __ballot_sync(0xffffffffu, acc && qin + qout + __popc(ma & lt) < a.cap);
                            if ((mw >> lane) & 1u) {
                                const int row = inner ? qin + __popc(mi & mw & lt)
                                                      : a.cap - 1 - (qout + __popc(~mi & mw & lt));
                                col[32 * row] = ent;
                            }
                            const int win = __popc(mi & mw);
                            qin += win;
                            qout += __popc(mw) - win;
                            qtot += __popc(ma);
                        }
                        if (lane == il) {
                            cin = qin;
                            cout = qout;
                            ctot = qtot;
                        }
                    }
                    __syncwarp();
                }
                if (grp & (1u << lane)) {
                    nin = cin;
                    nout = cout;
                    total = ctot;
                }
            }
        }
        if (!swept && real) {
            for (int dz = -1; dz <= 1; ++dz) {
                int z = cc[2] + dz;
                if (sd.per[2]) {
                    z = z < 0 ? z + sd.nc[2] : (z >= sd.nc[2] ? z - sd.nc[2] : z);
                } else if (z < 0 || z >= sd.nc[2]) {
                    continue;
                }
                for (int dy = -1; dy <= 1; ++dy) {
                    int y = cc[1] + dy;
                    if (sd.per[1]) {
                        y = y < 0 ? y + sd.nc[1] : (y >= sd.nc[1] ? y - sd.nc[1] : y);
                    } else if (y < 0 || y >= sd.nc[1]) {
                        continue;
                    }
                    for (int dx = -1; dx <= 1; ++dx) {
                        int x = cc[0] + dx;
                        if (sd.per[0]) {
                            x = x < 0 ? x + sd.nc[0] : (x >= sd.nc[0] ? x - sd.nc[0] : x);
                        } else if (x < 0 || x >= sd.nc[0]) {
                            continue;
                        }
                        const int2 rg = a.ranges[sd.cell_base + cell_code(sd, x, y, z)];
                        for (int j = rg.x; j < rg.y; ++j)
                            if (j != i) test(j, a.pos[cur][j], dx, dy, dz);
                    }
                }
            }
        }
        a.nnb[i] = real ? (nin | (nout << 16)) : 0;
        maxc = max(maxc, total);
    }
    nlist_finalise(a, maxc, cur, lp);
}

/* Form 2 of the list build (two phases per warp).  The distinct cells of a
 * warp's particles are fetched as in form 0 -- 27 lanes fetch a cell's
 * neighbour ranges -- and each cell's candidates are staged pre-shifted into
 * that cell's frame, padded with ghosts (never accepted) to a multiple of
 * 32.  Phase 1: for two particles of the cell at a time the warp tests 32
 * candidates per ballot pair, branch-free (one staged load serves both
 * particles), and each particle's own lane keeps the accept masks (in range
 * at all / inside the interaction range) in registers.  The candidates' list
 * entries stay staged in shared memory for as many cells as fit, so that
 * phase 2 -- every lane expands its masks in candidate order into its own
 * column -- runs for most warps once, with all their lanes.  The candidates,
 * their order and the arithmetic are those of forms 0 and 1, so all three
 * forms write the same rows. */
template<class R> __device__ __forceinline__ R ghost_w_of();  // the w word of a ghost's position
template<> __device__ __forceinline__ float ghost_w_of<float>() { return __int_as_float(GHOST); }
template<> __device__ __forceinline__ double ghost_w_of<double>() { return __longlong_as_double((long long)GHOST); }
// 7 resident blocks per SM: the staging below (about 31 KB per block in FP32)
// and at most 72 registers; more warps in flight beat fewer passes per warp
template<class R> __global__ void __launch_bounds__(128, 7) k_nlist2(KArgs<R> a, int gated) {
    using T4 = typename Vec<R>::T4;
    if (gated && !__ldcg(&a.S->rebuild)) return;
    constexpr int NLW = 4;                                // warps per block
    constexpr int MB = 8;                                 // accept masks (32 candidates each) per lane
    constexpr int REG = 32 * MB;                          // candidates of one cell (or chunk) per phase 1
    constexpr int SE = sizeof(T4) == 16 ? 768 : 512;      // list entries staged per warp until phase 2
    __shared__ float2 s_cut[256];                         // (list cutoff^2, range cutoff^2) per type pair
    __shared__ T4 s_pos[NLW][REG];                        // the current cell's candidates
    __shared__ uint32_t s_ent[NLW][SE];                   // j | shift code of its cell << NB_SHIFT
    __shared__ int s_off[NLW][28], s_beg[NLW][27];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int k = threadIdx.x; k < 256; k += blockDim.x)
        s_cut[k] = make_float2(__ldg(&a.ff->rlist2[k]), __ldg(&a.ff->rin2[k]));
    __syncthreads();
    const int cur = 1 - __ldcg(&a.S->cur), lp = 1 - __ldcg(&a.S->lp);
    // the grid covers npad (a multiple of the block size) once
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const T4 p = a.pos[cur][i];
    const int ty = w_type(wbits(p.w));
    const bool real = ty != GHOST;
    const SysDev &sd = a.sys[a.blk_sys[i / SYS_PAD]];  // one system per warp (SYS_PAD-aligned)
    const int c = a.cell[lp][i];
    const int cc[3] = {cx_of(c), cy_of(c), cz_of(c)};
    const R L[3] = {lc_of<R>(sd, 0), lc_of<R>(sd, 1), lc_of<R>(sd, 2)};
    // the expressions of k_nlist's shifted() and dist2()
    auto shifted = [&](const T4 &q, int dx, int dy, int dz) {
        T4 r = q;
        r.x = q.x + R(dx) * L[0];
        r.y = q.y + R(dy) * L[1];
        r.z = q.z + R(dz) * L[2];
        return r;
    };
    auto dist2 = [&](const T4 &pi, const T4 &qs) {
        const R ex = pi.x - qs.x, ey = pi.y - qs.y, ez = pi.z - qs.z;
        return ex * ex + ey * ey + ez * ez;
    };
    const int kme = cc[0] | (cc[1] << 11) | (cc[2] << 22);
    int *off = s_off[warp];
    int *beg = s_beg[warp];
    T4 *sp = s_pos[warp];
    uint32_t *se = s_ent[warp];
    uint32_t *col = a.nbr + nbr_index(i, 0, a.cap);  // row k of slot i at col[32 k]
    const R ghost_w = ghost_w_of<R>();
    const int cap = a.cap;
    int qin = 0, qout = 0, qtot = 0;
    // neighbour ranges of cell kd -> off/beg; returns the candidate count
    auto fetch = [&](int kd) {
        const int xd = kd & 2047, yd = (kd >> 11) & 2047, zd = (kd >> 22) & 1023;
        int2 rg = make_int2(0, 0);
        if (lane < 27) {
            int x = xd + lane % 3 - 1, y = yd + (lane / 3) % 3 - 1, z = zd + lane / 9 - 1;
            bool ok = true;
            if (sd.per[0]) x = x < 0 ? x + sd.nc[0] : (x >= sd.nc[0] ? x - sd.nc[0] : x);
            else ok = ok && x >= 0 && x < sd.nc[0];
            if (sd.per[1]) y = y < 0 ? y + sd.nc[1] : (y >= sd.nc[1] ? y - sd.nc[1] : y);
            else ok = ok && y >= 0 && y < sd.nc[1];
            if (sd.per[2]) z = z < 0 ? z + sd.nc[2] : (z >= sd.nc[2] ? z - sd.nc[2] : z);
            else ok = ok && z >= 0 && z < sd.nc[2];
            if (ok) rg = a.ranges[sd.cell_base + cell_code(sd, x, y, z)];
        }
        const int cnt = rg.y > rg.x ? rg.y - rg.x : 0;
        int inc = cnt;  // inclusive warp scan
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += t;
        }
        __syncwarp();  // the previous cell's staging is done with off/beg
        if (lane < 27) {
            off[lane] = inc - cnt;
            beg[lane] = rg.x;
        }
        __syncwarp();
        return __shfl_sync(0xffffffffu, inc, 31);
    };
    // candidates [c0, c0 + nch) of the fetched cell -> sp[0 ...] and se[ebase ...]
    auto stage = [&](int c0, int nch, int ebase) {
#pragma unroll 4
        for (int t = lane; t < nch; t += 32) {
            const int idx = c0 + t;
            int l = 0;  // last neighbour cell with off[l] <= idx
#pragma unroll
            for (int step = 16; step > 0; step >>= 1)
                if (l + step < 27 && off[l + step] <= idx) l += step;
            const int j = beg[l] + (idx - off[l]);
            sp[t] = shifted(a.pos[cur][j], l % 3 - 1, (l / 3) % 3 - 1, l / 9 - 1);
            se[ebase + t] = uint32_t(j) | (uint32_t(l) << NB_SHIFT);
        }
        if (nch + lane < ((nch + 31) & ~31)) {  // ghosts up to a multiple of 32: never accepted
            T4 z;
            z.x = z.y = z.z = R(0);
            z.w = ghost_w;
            sp[nch + lane] = z;
        }
        __syncwarp();
    };
    uint32_t macc[MB], minn[MB];
    // phase 1 for the particles grp, two per pass, over the staged candidates [0, nch), nch <= REG;
    // ts: the owning lane's own staged index (self is not a neighbour), -1 if absent
    auto phase1 = [&](unsigned grp, int nch, int ts) {
        for (unsigned g = grp; g;) {
            const int il = __ffs(g) - 1;
            g &= g - 1u;
            const int il2 = g ? __ffs(g) - 1 : il;  // the second particle of the pass (il again if none)
            if (g) g &= g - 1u;
            T4 pi = p, pi2 = p;
            pi.x = __shfl_sync(0xffffffffu, p.x, il);
            pi.y = __shfl_sync(0xffffffffu, p.y, il);
            pi.z = __shfl_sync(0xffffffffu, p.z, il);
            pi2.x = __shfl_sync(0xffffffffu, p.x, il2);
            pi2.y = __shfl_sync(0xffffffffu, p.y, il2);
            pi2.z = __shfl_sync(0xffffffffu, p.z, il2);
            const int ti = __shfl_sync(0xffffffffu, ty, il) * 16;
            const int tsi = __shfl_sync(0xffffffffu, ts, il);
            const int ti2 = __shfl_sync(0xffffffffu, ty, il2) * 16;
            const int tsi2 = __shfl_sync(0xffffffffu, ts, il2);
#pragma unroll
            for (int b = 0; b < MB; ++b) {
                if (b * 32 < nch) {
                    const int t = b * 32 + lane;
                    const T4 q = sp[t];
                    const int tj = w_type(wbits(q.w));
                    const float2 cut = s_cut[ti + tj];
                    const float2 cut2 = s_cut[ti2 + tj];
                    const R r2 = dist2(pi, q);
                    const R r2b = dist2(pi2, q);
                    const bool acc = t != tsi && r2 < R(cut.x);
                    const bool acc2 = t != tsi2 && r2b < R(cut2.x);
                    const unsigned ma = __ballot_sync(0xffffffffu, acc);
                    const unsigned mi = __ballot_sync(0xffffffffu, acc && r2 < R(cut.y));
                    const unsigned ma2 = __ballot_sync(0xffffffffu, acc2);
                    const unsigned mi2 = __ballot_sync(0xffffffffu, acc2 && r2b < R(cut2.y));
                    if (lane == il) {
                        macc[b] = ma;
                        minn[b] = mi;
                    }
                    if (lane == il2) {
                        macc[b] = ma2;
                        minn[b] = mi2;
                    }
                }
            }
        }
    };
    int mybase = 0;  // where this lane's candidates start in se
    // phase 2: this lane's accepted candidates, in order; the masks are cleared
    auto phase2 = [&]() {
#pragma unroll
        for (int b = 0; b < MB; ++b) {
            unsigned m = macc[b];
            const unsigned mi = minn[b];
            while (m) {
                const int bit = __ffs(m) - 1;
                m &= m - 1u;
                const uint32_t e = se[mybase + b * 32 + bit];
                const bool in = (mi >> bit) & 1u;
                if (qin + qout < cap) {
                    col[32 * (in ? qin : cap - 1 - qout)] = e;
                    qin += in;
                    qout += !in;
                }
                ++qtot;
            }
            macc[b] = minn[b] = 0u;
        }
        __syncwarp();  // every lane is done with se before it is restaged
    };
#pragma unroll
    for (int b = 0; b < MB; ++b) macc[b] = minn[b] = 0u;
    unsigned todo = __ballot_sync(0xffffffffu, real);
    unsigned pend = 0u;  // lanes whose masks refer to se
    int eused = 0;       // entries staged in se
    while (todo) {
        const int kd = __shfl_sync(0xffffffffu, kme, __ffs(todo) - 1);
        const unsigned grp = __ballot_sync(0xffffffffu, real && kme == kd) & todo;
        const int total_c = fetch(kd);
        todo &= ~grp;
        const int ts = off[13] + (i - beg[13]);
        if (total_c > REG) {  // in chunks of REG, each placed at once
            if (pend) phase2();
            pend = 0u;
            eused = 0;
            mybase = 0;
            for (int c0 = 0; c0 < total_c; c0 += REG) {
                const int nch = min(REG, total_c - c0);
                stage(c0, nch, 0);
                phase1(grp, nch, (ts >= c0 && ts < c0 + nch) ? ts - c0 : -1);
                phase2();
            }
            continue;
        }
        if (eused + total_c > SE) {  // se is full: place what it holds
            phase2();
            pend = 0u;
            eused = 0;
        }
        stage(0, total_c, eused);
        phase1(grp, total_c, ts);
        if ((grp >> lane) & 1u) mybase = eused;
        eused += total_c;
        pend |= grp;
    }
    if (pend) phase2();
    a.nnb[i] = real ? (qin | (qout << 16)) : 0;
    nlist_finalise(a, real ? qtot : 0, cur, lp);
}

static int grid_for(int64_t n, int per_block = 256) {
    int64_t g = (n + per_block - 1) / per_block;
    const int64_t cap = 152 * 8;
    return int(g < 1 ? 1 : (g > cap ? cap : g));
}

template<class R> void launch_rebuild_stage(const KArgs<R> &a, cudaStream_t st, bool gated, int stage) {
    const int g = grid_for(a.npad);
    switch (stage) {
        case 0:
            k_rebin<R><<<(a.npad + 255) / 256, 256, 0, st>>>(a, gated ? 1 : 0);
            break;
        case 1:
            radix_sort_pairs(const_cast<uint32_t **>(a.skey), const_cast<int **>(a.sval), a.counts, a.digit_total,
                             a.inv, a.npad, a.sort_passes, a.ntiles, gated ? &a.S->rebuild : nullptr, st);
            break;
        case 2:
            k_ranges_gather<R><<<g, 256, 0, st>>>(a, a.sort_passes % 2, gated ? 1 : 0);
            break;
        default:
            if (a.nlist_lane == 2)
                k_nlist2<R><<<(a.npad + 127) / 128, 128, 0, st>>>(a, gated ? 1 : 0);
            else
                k_nlist<R><<<(a.npad + 127) / 128, 128, 0, st>>>(a, gated ? 1 : 0);
            break;
    }
}

template<class R> void launch_rebuild(const KArgs<R> &a, cudaStream_t st, bool gated) {
    for (int k = 0; k < 4; ++k) launch_rebuild_stage<R>(a, st, gated, k);
}

/* ------------------------------------------------------------------------- */
/* State conversion                                                          */
/* ------------------------------------------------------------------------- */
/* Host state -> device slots for upload indices [k0, k1).  The staged host
 * arrays hold the particles from upload index `first` on, `stride` values of
 * type TH per particle (AoS; FP64 vectors of 3, or the reference's own `real`
 * = float vectors of 3, or of 4 under its _VEC4 layout). */
template<class R, class TH>
__device__ __forceinline__ void set_one(const KArgs<R> &a, int cur, int lp, int64_t k, const TH *x, const TH *nv,
                                        const TH *v, const TH *o, int &out, int &moved) {
    using T4 = typename Vec<R>::T4;
    {
        const int p = a.slot_of_home[k];
        const int hk = 0;
        const SysDev &sd = a.sys[a.blk_sys[p / SYS_PAD]];
        T4 q = a.pos[cur][p];
        // A particle still within skin/2 of where the list was built keeps its
        // cell (the list's shift codes stay valid) and no rebuild is needed:
        // the offset is taken from that cell's centre (minimum image on
        // periodic axes).  Otherwise it is binned afresh and the list rebuilt.
        const int c0 = a.cell[lp][p];
        const int cc0[3] = {cx_of(c0), cy_of(c0), cz_of(c0)};
        const T4 xr = a.xref[lp][p];
        const R xrv[3] = {xr.x, xr.y, xr.z};
        R keep[3];
        R md2 = 0;
        for (int d = 0; d < 3; ++d) {
            const double center = __dadd_rn(sd.lo[d], __dmul_rn(double(cc0[d]) + 0.5, sd.Lc[d]));
            double u = __dsub_rn(double(x[hk + d]), center);
            if (sd.per[d]) {
                const double L = double(sd.nc[d]) * sd.Lc[d];
                u -= L * rint(u / L);
            }
            keep[d] = R(u);
            md2 += (keep[d] - xrv[d]) * (keep[d] - xrv[d]);
        }
        if (md2 <= a.skin_half2) {
            q.x = keep[0];
            q.y = keep[1];
            q.z = keep[2];
            a.pos[cur][p] = q;
        } else {
            moved = 1;
            a.ranges[sd.cell_base + cell_code(sd, cc0[0], cc0[1], cc0[2])] = make_int2(0, 0);
            int cc[3];
            R off[3];
            for (int d = 0; d < 3; ++d) {
                const double xd = double(x[hk + d]);
                const int cu = int(floor(__ddiv_rn(__dsub_rn(xd, sd.lo[d]), sd.Lc[d])));
                int c = cu;
                if (sd.per[d]) {
                    c %= sd.nc[d];
                    if (c < 0) c += sd.nc[d];
                } else {
                    c = min(max(cu, 0), sd.nc[d] - 1);
                    if (c != cu) out = 1;
                }
                const int cref = sd.per[d] ? cu : c;
                const double center = __dadd_rn(sd.lo[d], __dmul_rn(double(cref) + 0.5, sd.Lc[d]));
                off[d] = R(__dsub_rn(xd, center));
                cc[d] = c;
            }
            q.x = off[0];
            q.y = off[1];
            q.z = off[2];
            a.pos[cur][p] = q;
            a.xref[lp][p] = q;
            a.cell[lp][p] = cpack(cc[0], cc[1], cc[2]);
        }
        T4 t = a.nrm[cur][p];
        t.x = R(nv[hk]);
        t.y = R(nv[hk + 1]);
        t.z = R(nv[hk + 2]);
        a.nrm[cur][p] = t;
        t = a.vel[lp][p];
        t.x = R(v[hk]);
        t.y = R(v[hk + 1]);
        t.z = R(v[hk + 2]);
        a.vel[lp][p] = t;
        t = a.omg[lp][p];
        t.x = R(o[hk]);
        t.y = R(o[hk + 1]);
        t.z = R(o[hk + 2]);
        a.omg[lp][p] = t;
    }
}

template<class R, class TH>
__global__ void k_set_state(KArgs<R> a, const TH *x, const TH *nv, const TH *v, const TH *o, int64_t k0, int64_t k1,
                            int64_t first, int stride) {
    const int cur = __ldcg(&a.S->cur), lp = __ldcg(&a.S->lp);
    int out = 0, moved = 0;
    for (int64_t k = k0 + blockIdx.x * int64_t(blockDim.x) + threadIdx.x; k < k1; k += int64_t(gridDim.x) * blockDim.x) {
        const int64_t hk = (k - first) * stride;
        set_one<R, TH>(a, cur, lp, k, x + hk, nv + hk, v + hk, o + hk, out, moved);
    }
    if (out) atomicOr(&a.S->error, ERRB_GRID);
    if (__syncthreads_or(moved) && threadIdx.x == 0) a.S->rebuild = 1;
}

/* In-place transfers over the host link (the caller's arrays are reachable
 * from the GPU).  Host memory gives full link bandwidth only to wide, fully
 * coalesced accesses, so each block moves a tile of HOST_TILE particles of
 * each array through shared memory with 16-byte loads or stores (a base that
 * is not 16-byte aligned falls back to contiguous scalar accesses), and the
 * per-particle conversion works on the staged tile. */
constexpr int HOST_TILE = 256;
template<class TH> __device__ __forceinline__ void tile_in(TH *dst, const TH *src, int nvals) {
    const uintptr_t addr = reinterpret_cast<uintptr_t>(src);
    if ((addr & 15u) == 0) {
        const int nv4 = int(nvals * sizeof(TH) / 16);
        const int4 *s4 = reinterpret_cast<const int4 *>(src);
        int4 *d4 = reinterpret_cast<int4 *>(dst);
        for (int t = threadIdx.x; t < nv4; t += blockDim.x) d4[t] = s4[t];
        for (int t = nv4 * int(16 / sizeof(TH)) + threadIdx.x; t < nvals; t += blockDim.x) dst[t] = src[t];
    } else {
        for (int t = threadIdx.x; t < nvals; t += blockDim.x) dst[t] = src[t];
    }
}
template<class TH> __device__ __forceinline__ void tile_out(TH *dst, const TH *src, int nvals) {
    const uintptr_t addr = reinterpret_cast<uintptr_t>(dst);
    if ((addr & 15u) == 0) {
        const int nv4 = int(nvals * sizeof(TH) / 16);
        const int4 *s4 = reinterpret_cast<const int4 *>(src);
        int4 *d4 = reinterpret_cast<int4 *>(dst);
        for (int t = threadIdx.x; t < nv4; t += blockDim.x) d4[t] = s4[t];
        for (int t = nv4 * int(16 / sizeof(TH)) + threadIdx.x; t < nvals; t += blockDim.x) dst[t] = src[t];
    } else {
        for (int t = threadIdx.x; t < nvals; t += blockDim.x) dst[t] = src[t];
    }
}

template<class R, class TH>
__global__ void __launch_bounds__(HOST_TILE) k_set_state_host(KArgs<R> a, const TH *x, const TH *nv, const TH *v,
                                                              const TH *o, int64_t k0, int64_t k1, int64_t first,
                                                              int stride) {
    __shared__ __align__(16) TH buf[4][HOST_TILE * 4];
    const int cur = __ldcg(&a.S->cur), lp = __ldcg(&a.S->lp);
    const int64_t kb = k0 + int64_t(blockIdx.x) * HOST_TILE;
    const int m = int(k1 - kb < HOST_TILE ? k1 - kb : HOST_TILE);
    const TH *src[4] = {x, nv, v, o};
    for (int q = 0; q < 4; ++q) tile_in<TH>(buf[q], src[q] + (kb - first) * stride, m * stride);
    __syncthreads();
    int out = 0, moved = 0;
    const int t = threadIdx.x;
    if (t < m) {
        const int hk = t * stride;
        set_one<R, TH>(a, cur, lp, kb + t, buf[0] + hk, buf[1] + hk, buf[2] + hk, buf[3] + hk, out, moved);
    }
    if (out) atomicOr(&a.S->error, ERRB_GRID);
    if (__syncthreads_or(moved) && threadIdx.x == 0) a.S->rebuild = 1;
}

template<class R, class TH>
void launch_set_state(const KArgs<R> &a, const TH *x, const TH *n, const TH *v, const TH *o, int64_t k0, int64_t k1,
                      int64_t first, int stride, cudaStream_t st) {
    k_set_state<R, TH><<<grid_for(k1 - k0), 256, 0, st>>>(a, x, n, v, o, k0, k1, first, stride);
}
template<class R, class TH>
void launch_set_state_host(const KArgs<R> &a, const TH *x, const TH *n, const TH *v, const TH *o, int64_t k0,
                           int64_t k1, int64_t first, int stride, cudaStream_t st) {
    const int64_t nb = (k1 - k0 + HOST_TILE - 1) / HOST_TILE;
    if (nb > 0) k_set_state_host<R, TH><<<int(nb), HOST_TILE, 0, st>>>(a, x, n, v, o, k0, k1, first, stride);
}

/* Device state -> caller-order AoS vectors of TH for upload indices [h0, h1),
 * written from upload index `first` on with `stride` values per particle (a
 * fourth value, when stride is 4, is written as 0).  One thread per upload
 * index (the slot comes from slot_of_home), so the writes -- the side that
 * streams to the host -- are coalesced; the slot-side reads are gathers. */
template<class R, class TH>
__device__ __forceinline__ void get_one(const KArgs<R> &a, int cur, int lp, int64_t h, int64_t hk, int stride, TH *x,
                                        TH *nv, TH *v, TH *o, TH *f, TH *t, double *e) {
    using T4 = typename Vec<R>::T4;
    {
        const int p = a.slot_of_home[h];
        const SysDev &sd = a.sys[a.blk_sys[p / SYS_PAD]];
        if (x) {
            const T4 q = a.pos[cur][p];
            const int c = a.cell[lp][p];
            const int cc[3] = {cx_of(c), cy_of(c), cz_of(c)};
            const double off[3] = {double(q.x), double(q.y), double(q.z)};
            for (int d = 0; d < 3; ++d)
                x[hk + d] = TH(__dadd_rn(__dadd_rn(sd.lo[d], __dmul_rn(double(cc[d]) + 0.5, sd.Lc[d])), off[d]));
            if (stride == 4) x[hk + 3] = TH(0);
        }
        auto put = [&](TH *dst, const T4 &q) {
            if (!dst) return;
            dst[hk] = TH(q.x);
            dst[hk + 1] = TH(q.y);
            dst[hk + 2] = TH(q.z);
            if (stride == 4) dst[hk + 3] = TH(0);
        };
        if (nv) put(nv, a.nrm[cur][p]);
        if (v) put(v, a.vel[lp][p]);
        if (o) put(o, a.omg[lp][p]);
        if (f) put(f, a.frc[lp][p]);
        if (t) put(t, a.trq[lp][p]);
        if (e) e[h] = a.epart[p];
    }
}

template<class R, class TH>
__global__ void k_download(KArgs<R> a, int64_t h0, int64_t h1, int64_t first, int stride, TH *x, TH *nv, TH *v,
                           TH *o, TH *f, TH *t, double *e) {
    const int cur = __ldcg(&a.S->cur), lp = __ldcg(&a.S->lp);
    for (int64_t h = h0 + blockIdx.x * int64_t(blockDim.x) + threadIdx.x; h < h1; h += int64_t(gridDim.x) * blockDim.x)
        get_one<R, TH>(a, cur, lp, h, (h - first) * stride, stride, x, nv, v, o, f, t, e);
}

/* In-place download: the tile's values are formed in shared memory, then
 * each array's tile is written to the host with 16-byte stores. */
template<class R, class TH>
__global__ void __launch_bounds__(HOST_TILE) k_download_host(KArgs<R> a, int64_t h0, int64_t h1, int64_t first,
                                                             int stride, TH *x, TH *nv, TH *v, TH *o) {
    __shared__ __align__(16) TH buf[4][HOST_TILE * 4];
    const int cur = __ldcg(&a.S->cur), lp = __ldcg(&a.S->lp);
    const int64_t hb = h0 + int64_t(blockIdx.x) * HOST_TILE;
    const int m = int(h1 - hb < HOST_TILE ? h1 - hb : HOST_TILE);
    TH *dst[4] = {x, nv, v, o};
    const int t = threadIdx.x;
    if (t < m)
        get_one<R, TH>(a, cur, lp, hb + t, int64_t(t) * stride, stride, x ? buf[0] : nullptr, nv ? buf[1] : nullptr,
                       v ? buf[2] : nullptr, o ? buf[3] : nullptr, nullptr, nullptr, nullptr);
    __syncthreads();
    for (int q = 0; q < 4; ++q)
        if (dst[q]) tile_out<TH>(dst[q] + (hb - first) * stride, buf[q], m * stride);
}

template<class R, class TH>
void launch_download(const KArgs<R> &a, int64_t h0, int64_t h1, int64_t first, int stride, TH *x, TH *n, TH *v, TH *o,
                     TH *f, TH *t, double *e, cudaStream_t st) {
    k_download<R, TH><<<grid_for(h1 - h0), 256, 0, st>>>(a, h0, h1, first, stride, x, n, v, o, f, t, e);
}
template<class R, class TH>
void launch_download_host(const KArgs<R> &a, int64_t h0, int64_t h1, int64_t first, int stride, TH *x, TH *n, TH *v,
                          TH *o, cudaStream_t st) {
    const int64_t nb = (h1 - h0 + HOST_TILE - 1) / HOST_TILE;
    if (nb > 0) k_download_host<R, TH><<<int(nb), HOST_TILE, 0, st>>>(a, h0, h1, first, stride, x, n, v, o);
}
template<class R> void launch_download(const KArgs<R> &a, int64_t h0, int64_t h1, double *x, double *n, double *v,
                                       double *o, double *f, double *t, double *e, cudaStream_t st) {
    launch_download<R, double>(a, h0, h1, 0, 3, x, n, v, o, f, t, e, st);
}

__global__ void k_set_cond(cudaGraphConditionalHandle h, const Scalars *S) {
    cudaGraphSetConditional(h, __ldcg(&S->rebuild) ? 1u : 0u);
}
void launch_set_cond(cudaGraphConditionalHandle h, Scalars *S, cudaStream_t st) {
    k_set_cond<<<1, 1, 0, st>>>(h, S);
}

/* ------------------------------------------------------------------------- */
/* Reference Morton key (src/reorder_morton.h:25-42).                        */
/* ------------------------------------------------------------------------- */
__device__ __forceinline__ uint32_t bit_space3(uint32_t x) {
    x = (x | (x << 12)) & 0x00FC003Fu;
    x = (x | (x << 6)) & 0x381C0E07u;
    x = (x | (x << 4)) & 0x190C8643u;
    x = (x | (x << 2)) & 0x49249249u;
    return x;
}
__global__ void k_morton(const double *p3, int64_t n, double b0, double b1, double b2, uint32_t *keys) {
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
        const uint32_t cx = __double2uint_rz(__dadd_rn(2.0 * p3[3 * i], b0));
        const uint32_t cy = __double2uint_rz(__dadd_rn(2.0 * p3[3 * i + 1], b1));
        const uint32_t cz = __double2uint_rz(__dadd_rn(2.0 * p3[3 * i + 2], b2));
        keys[i] = bit_space3(cx) | (bit_space3(cy) << 1) | (bit_space3(cz) << 2);
    }
}
void launch_morton(const double *p3, int64_t n, const double *b, uint32_t *keys, cudaStream_t st) {
    k_morton<<<grid_for(n), 256, 0, st>>>(p3, n, b[0], b[1], b[2], keys);
}

template void launch_rebuild<float>(const KArgs<float> &, cudaStream_t, bool);
template void launch_rebuild_stage<float>(const KArgs<float> &, cudaStream_t, bool, int);
template void launch_rebuild_stage<double>(const KArgs<double> &, cudaStream_t, bool, int);
template void launch_rebuild<double>(const KArgs<double> &, cudaStream_t, bool);
#define ORBC_IO_INST(R, TH)                                                                                    \
    template void launch_set_state<R, TH>(const KArgs<R> &, const TH *, const TH *, const TH *, const TH *, int64_t, \
                                          int64_t, int64_t, int, cudaStream_t);                                      \
    template void launch_download<R, TH>(const KArgs<R> &, int64_t, int64_t, int64_t, int, TH *, TH *, TH *, TH *,    \
                                         TH *, TH *, double *, cudaStream_t);                                          \
    template void launch_set_state_host<R, TH>(const KArgs<R> &, const TH *, const TH *, const TH *, const TH *,     \
                                               int64_t, int64_t, int64_t, int, cudaStream_t);                           \
    template void launch_download_host<R, TH>(const KArgs<R> &, int64_t, int64_t, int64_t, int, TH *, TH *, TH *,    \
                                              TH *, cudaStream_t);
ORBC_IO_INST(float, float)
ORBC_IO_INST(float, double)
ORBC_IO_INST(double, float)
ORBC_IO_INST(double, double)
#undef ORBC_IO_INST
template void launch_download<float>(const KArgs<float> &, int64_t, int64_t, double *, double *, double *, double *,
                                     double *, double *, double *, cudaStream_t);
template void launch_download<double>(const KArgs<double> &, int64_t, int64_t, double *, double *, double *,
                                      double *, double *, double *, double *, cudaStream_t);

}  // namespace orbc
