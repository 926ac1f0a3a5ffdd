// Whole-cell initialiser, GPU part: the lipid placement of init_rbc
// (src/init_rbc.h:235-305).  Face f receives face_nl[f] lipids, each drawn
// uniformly on the triangle (square-root barycentric sampling) and redrawn
// until it is at least min_dist_lp from the face's first vertex and from every
// protein, and at least min_dist from the lipids already placed on the same
// face; its normal is the face normal.
//
// One warp per face.  Attempt k of lipid j draws its two uniforms from
// Philox4x32-10 keyed by the seed with counter (face, j, k); the 32 lanes try
// attempts k0 .. k0 + 31 at once and the lowest clean attempt wins, which is
// the candidate a one-by-one loop over k would keep, so the result does not
// depend on the parallel layout.  Distances to proteins come from a uniform
// grid of cell size >= min_dist_lp (27 cells).  Every coordinate is computed
// with explicitly rounded FP64 operations, so the CPU restatement in the
// oracle reproduces the placement bit for bit.  A lipid that finds no room
// after MAX_ROUNDS x 32 attempts stops its face and is reported.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

#include "orbc_gpu.h"
#include "orbc_device.cuh"

namespace {

constexpr int MAX_ROUNDS = 256;

struct PlaceArgs {
    const double *vert;   // [nvert][3] scaled vertices
    const int *face;      // [nface][3]
    const double *fnorm;  // [nface][3]
    const int64_t *base;  // [nface + 1] first lipid of each face
    const double *prot;   // [nprot][3] proteins sorted by grid cell
    const int *cstart;    // [ncell + 1]
    int64_t nface;
    double lo[3], h;
    int nc[3];
    double md2, mdlp2;
    uint32_t k0, k1;
    double *x, *n;
    int *failed;          // first face that ran out of attempts + 1 (0: none)
};

__device__ __forceinline__ void philox4_init(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0,
                                             uint32_t k1, uint32_t o[4]) {
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

// [0, 1) with 53 random bits from two words
__device__ __forceinline__ double u01_53(uint32_t a, uint32_t b) {
    return double(uint64_t(a >> 5) * 67108864ull + uint64_t(b >> 6)) * (1.0 / 9007199254740992.0);
}

__device__ __forceinline__ double sq3(double dx, double dy, double dz) {
    return __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
}

__global__ void __launch_bounds__(128) k_place_lipids(PlaceArgs a) {
    const int lane = threadIdx.x & 31;
    const int64_t wid = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = (int64_t(gridDim.x) * blockDim.x) >> 5;
    for (int64_t f = wid; f < a.nface; f += nw) {
        const int i0 = a.face[3 * f], i1 = a.face[3 * f + 1], i2 = a.face[3 * f + 2];
        const double v1[3] = {a.vert[3 * i0], a.vert[3 * i0 + 1], a.vert[3 * i0 + 2]};
        const double v2[3] = {a.vert[3 * i1], a.vert[3 * i1 + 1], a.vert[3 * i1 + 2]};
        const double v3[3] = {a.vert[3 * i2], a.vert[3 * i2 + 1], a.vert[3 * i2 + 2]};
        const int64_t b0 = a.base[f], nl = a.base[f + 1] - b0;
        for (int64_t j = 0; j < nl; ++j) {
            bool placed = false;
            for (int round = 0; round < MAX_ROUNDS && !placed; ++round) {
                const uint32_t k = uint32_t(round) * 32u + uint32_t(lane);
                uint32_t o[4];
                philox4_init(uint32_t(f), uint32_t(j), k, uint32_t(f >> 32) ^ 0x4C495049u, a.k0, a.k1, o);
                const double r1 = u01_53(o[0], o[1]), r2 = u01_53(o[2], o[3]);
                const double s1 = __dsqrt_rn(r1);
                const double w1 = __dsub_rn(1.0, s1), w2 = __dmul_rn(s1, __dsub_rn(1.0, r2)), w3 = __dmul_rn(s1, r2);
                double r[3];
#pragma unroll
                for (int d = 0; d < 3; ++d)
                    r[d] = __dadd_rn(__dadd_rn(__dmul_rn(v1[d], w1), __dmul_rn(v2[d], w2)), __dmul_rn(v3[d], w3));
                bool clean = sq3(__dsub_rn(r[0], v1[0]), __dsub_rn(r[1], v1[1]), __dsub_rn(r[2], v1[2])) >= a.mdlp2;
                // proteins: the 27 grid cells around r (cell side >= min_dist_lp)
                int c[3];
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    const int cd = int(floor(__ddiv_rn(__dsub_rn(r[d], a.lo[d]), a.h)));
                    c[d] = min(max(cd, 0), a.nc[d] - 1);
                }
                for (int dz = -1; dz <= 1 && clean; ++dz) {
                    const int z = c[2] + dz;
                    if (z < 0 || z >= a.nc[2]) continue;
                    for (int dy = -1; dy <= 1 && clean; ++dy) {
                        const int y = c[1] + dy;
                        if (y < 0 || y >= a.nc[1]) continue;
                        for (int dx = -1; dx <= 1 && clean; ++dx) {
                            const int x = c[0] + dx;
                            if (x < 0 || x >= a.nc[0]) continue;
                            const int cell = x + a.nc[0] * (y + a.nc[1] * z);
                            for (int p = a.cstart[cell]; p < a.cstart[cell + 1]; ++p) {
                                const double *q = a.prot + 3 * int64_t(p);
                                if (sq3(__dsub_rn(r[0], q[0]), __dsub_rn(r[1], q[1]), __dsub_rn(r[2], q[2])) < a.mdlp2) {
                                    clean = false;
                                    break;
                                }
                            }
                        }
                    }
                }
                // the face's earlier lipids (written by this warp, visible after __syncwarp)
                for (int64_t m = 0; m < j && clean; ++m) {
                    const double *q = a.x + 3 * (b0 + m);
                    if (sq3(__dsub_rn(q[0], r[0]), __dsub_rn(q[1], r[1]), __dsub_rn(q[2], r[2])) < a.md2) clean = false;
                }
                const unsigned ok = __ballot_sync(0xffffffffu, clean);
                if (ok) {
                    if (lane == __ffs(ok) - 1) {
                        double *xo = a.x + 3 * (b0 + j), *no = a.n + 3 * (b0 + j);
                        for (int d = 0; d < 3; ++d) {
                            xo[d] = r[d];
                            no[d] = a.fnorm[3 * f + d];
                        }
                    }
                    __syncwarp();
                    placed = true;
                }
            }
            if (!placed) {
                if (lane == 0) atomicCAS(a.failed, 0, int(f) + 1);
                break;
            }
        }
    }
}

}  // namespace

extern "C" int orbc_gpu_place_lipids(const double *vert3, int64_t nvert, const int *face3, const double *fnorm3,
                                     int64_t nface, const int64_t *face_nl, const double *prot3, int64_t nprot,
                                     double min_dist, double min_dist_lp, uint64_t seed, double *x3, double *n3) {
    if (!vert3 || !face3 || !fnorm3 || !face_nl || !x3 || !n3 || nvert < 3 || nface < 1 || nprot < 0 ||
        (nprot > 0 && !prot3) || !(min_dist >= 0) || !(min_dist_lp > 0))
        return ORBC_ERR_ARG;
    for (int64_t k = 0; k < 3 * nface; ++k)
        if (face3[k] < 0 || face3[k] >= nvert) return ORBC_ERR_ARG;
    std::vector<int64_t> base(size_t(nface) + 1, 0);
    for (int64_t f = 0; f < nface; ++f) {
        if (face_nl[f] < 0) return ORBC_ERR_ARG;
        base[size_t(f) + 1] = base[size_t(f)] + face_nl[f];
    }
    const int64_t nl = base[size_t(nface)];
    // protein grid over the bounding box of vertices and proteins
    double lo[3], hi[3];
    for (int d = 0; d < 3; ++d) lo[d] = hi[d] = vert3[d];
    auto grow = [&](const double *p) {
        for (int d = 0; d < 3; ++d) {
            lo[d] = std::min(lo[d], p[d]);
            hi[d] = std::max(hi[d], p[d]);
        }
    };
    for (int64_t i = 0; i < nvert; ++i) grow(vert3 + 3 * i);
    for (int64_t i = 0; i < nprot; ++i) grow(prot3 + 3 * i);
    // cell side min_dist_lp, or larger so that a hollow cell's box stays under 2^26 cells
    double h = min_dist_lp;
    {
        double vol = 1;
        for (int d = 0; d < 3; ++d) vol *= (hi[d] - lo[d]) + 3 * h;
        const double cap = double(int64_t(1) << 26);
        if (vol / (h * h * h) > cap) h = std::cbrt(vol / cap) * 1.01;
    }
    int nc[3];
    int64_t ncell = 1;
    for (int d = 0; d < 3; ++d) {
        lo[d] -= h;
        nc[d] = int((hi[d] + h - lo[d]) / h) + 1;
        ncell *= nc[d];
    }
    if (ncell > (int64_t(1) << 27)) return ORBC_ERR_ARG;
    auto cell_of = [&](const double *p) {
        int c[3];
        for (int d = 0; d < 3; ++d) c[d] = std::min(std::max(int(std::floor((p[d] - lo[d]) / h)), 0), nc[d] - 1);
        return int64_t(c[0]) + nc[0] * (int64_t(c[1]) + int64_t(nc[1]) * c[2]);
    };
    std::vector<int> cstart(size_t(ncell) + 1, 0);
    std::vector<int64_t> pcell(static_cast<size_t>(nprot));
    for (int64_t i = 0; i < nprot; ++i) {
        pcell[size_t(i)] = cell_of(prot3 + 3 * i);
        ++cstart[size_t(pcell[size_t(i)]) + 1];
    }
    for (int64_t c = 0; c < ncell; ++c) cstart[size_t(c) + 1] += cstart[size_t(c)];
    std::vector<double> sorted(size_t(3 * std::max<int64_t>(nprot, 1)));
    {
        std::vector<int> fill(cstart.begin(), cstart.end() - 1);
        for (int64_t i = 0; i < nprot; ++i) {
            const int at = fill[size_t(pcell[size_t(i)])]++;
            for (int d = 0; d < 3; ++d) sorted[size_t(3 * at + d)] = prot3[3 * i + d];
        }
    }
    // device buffers
    double *dv = nullptr, *dfn = nullptr, *dp = nullptr, *dx = nullptr, *dn = nullptr;
    int *df = nullptr, *dcs = nullptr, *dfail = nullptr;
    int64_t *db = nullptr;
    auto cleanup = [&]() {
        cudaFree(dv);
        cudaFree(dfn);
        cudaFree(dp);
        cudaFree(dx);
        cudaFree(dn);
        cudaFree(df);
        cudaFree(dcs);
        cudaFree(dfail);
        cudaFree(db);
    };
    const size_t bx = size_t(3 * std::max<int64_t>(nl, 1)) * sizeof(double);
    if (cudaMalloc(&dv, size_t(3 * nvert) * sizeof(double)) || cudaMalloc(&dfn, size_t(3 * nface) * sizeof(double)) ||
        cudaMalloc(&dp, sorted.size() * sizeof(double)) || cudaMalloc(&dx, bx) || cudaMalloc(&dn, bx) ||
        cudaMalloc(&df, size_t(3 * nface) * sizeof(int)) || cudaMalloc(&dcs, cstart.size() * sizeof(int)) ||
        cudaMalloc(&dfail, sizeof(int)) || cudaMalloc(&db, base.size() * sizeof(int64_t))) {
        cleanup();
        return ORBC_ERR_NOMEM;
    }
    cudaMemcpy(dv, vert3, size_t(3 * nvert) * sizeof(double), cudaMemcpyHostToDevice);
    cudaMemcpy(dfn, fnorm3, size_t(3 * nface) * sizeof(double), cudaMemcpyHostToDevice);
    cudaMemcpy(dp, sorted.data(), sorted.size() * sizeof(double), cudaMemcpyHostToDevice);
    cudaMemcpy(df, face3, size_t(3 * nface) * sizeof(int), cudaMemcpyHostToDevice);
    cudaMemcpy(dcs, cstart.data(), cstart.size() * sizeof(int), cudaMemcpyHostToDevice);
    cudaMemcpy(db, base.data(), base.size() * sizeof(int64_t), cudaMemcpyHostToDevice);
    cudaMemset(dfail, 0, sizeof(int));
    PlaceArgs a;
    a.vert = dv;
    a.face = df;
    a.fnorm = dfn;
    a.base = db;
    a.prot = dp;
    a.cstart = dcs;
    a.nface = nface;
    for (int d = 0; d < 3; ++d) {
        a.lo[d] = lo[d];
        a.nc[d] = nc[d];
    }
    a.h = h;
    a.md2 = min_dist * min_dist;
    a.mdlp2 = min_dist_lp * min_dist_lp;
    a.k0 = uint32_t(seed);
    a.k1 = uint32_t(seed >> 32);
    a.x = dx;
    a.n = dn;
    a.failed = dfail;
    const int64_t warps = std::min<int64_t>(nface, int64_t(152) * 64);
    k_place_lipids<<<unsigned((warps + 3) / 4), 128>>>(a);
    int failed = 0;
    cudaError_t e = cudaMemcpy(&failed, dfail, sizeof(int), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && nl > 0) e = cudaMemcpy(x3, dx, size_t(3 * nl) * sizeof(double), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && nl > 0) e = cudaMemcpy(n3, dn, size_t(3 * nl) * sizeof(double), cudaMemcpyDeviceToHost);
    cleanup();
    if (e != cudaSuccess) return ORBC_ERR_CUDA;
    return failed ? ORBC_ERR_ARG : ORBC_OK;
}
