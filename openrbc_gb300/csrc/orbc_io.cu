// Device side of the trajectory and checkpoint I/O: gathers the state into
// the payload sections of a frame in the reference's .orbc layout
// (src/trajectory.h:61-105; particles in file order, lipids first, then
// proteins) in the file's `real` type, and writes carried Nose-Hoover forces
// back from a checkpoint.
#include "orbc_device.cuh"

namespace orbc {

namespace {

/* One pass over the slots: every live particle writes its fields at its file
 * position.  Positions are reconstructed in FP64 exactly as k_download does,
 * then rounded to T. */
template<class R, class T>
__global__ void k_frame_pack(KArgs<R> a, const int *file_of_home, T *pos, T *vel, T *rot, int *cell, T *frc) {
    const int cur = __ldcg(&a.S->cur), lp = __ldcg(&a.S->lp);
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < a.npad; p += gridDim.x * blockDim.x) {
        const int h = a.home[lp][p];
        if (h < 0) continue;
        const int64_t f = file_of_home[h];
        const SysDev &sd = a.sys[a.blk_sys[p / SYS_PAD]];
        const int c = a.cell[lp][p];
        const int cc[3] = {cx_of(c), cy_of(c), cz_of(c)};
        if (pos) {
            const auto q = a.pos[cur][p];
            const double off[3] = {double(q.x), double(q.y), double(q.z)};
#pragma unroll
            for (int d = 0; d < 3; ++d)
                pos[3 * f + d] =
                    T(__dadd_rn(__dadd_rn(sd.lo[d], __dmul_rn(double(cc[d]) + 0.5, sd.Lc[d])), off[d]));
        }
        auto put = [&](T *dst, const typename Vec<R>::T4 &q) {
            dst[3 * f] = T(q.x);
            dst[3 * f + 1] = T(q.y);
            dst[3 * f + 2] = T(q.z);
        };
        if (vel) put(vel, a.vel[lp][p]);
        if (rot) put(rot, a.nrm[cur][p]);
        if (frc) put(frc, a.frc[lp][p]);
        if (cell) cell[f] = int(cell_code(sd, cc[0], cc[1], cc[2]));
    }
}

template<class R> __global__ void k_set_carried(KArgs<R> a, const double *f3, const double *t3, int64_t nhome) {
    const int lp = __ldcg(&a.S->lp);
    for (int64_t k = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; k < nhome; k += int64_t(gridDim.x) * blockDim.x) {
        const int p = a.slot_of_home[k];
        auto q = a.frc[lp][p];
        q.x = R(f3[3 * k]);
        q.y = R(f3[3 * k + 1]);
        q.z = R(f3[3 * k + 2]);
        a.frc[lp][p] = q;
        q = a.trq[lp][p];
        q.x = R(t3[3 * k]);
        q.y = R(t3[3 * k + 1]);
        q.z = R(t3[3 * k + 2]);
        a.trq[lp][p] = q;
    }
}

int io_grid(int64_t n) {
    const int64_t g = (n + 255) / 256;
    return int(g < 1 ? 1 : (g > 152 * 8 ? 152 * 8 : g));
}

}  // namespace

template<class R>
void launch_frame_pack(const KArgs<R> &a, const int *file_of_home, int real_bytes, void *pos, void *vel, void *rot,
                       int *cell, void *frc, cudaStream_t st) {
    if (real_bytes == 4)
        k_frame_pack<R, float><<<io_grid(a.npad), 256, 0, st>>>(a, file_of_home, static_cast<float *>(pos),
                                                                static_cast<float *>(vel), static_cast<float *>(rot),
                                                                cell, static_cast<float *>(frc));
    else
        k_frame_pack<R, double><<<io_grid(a.npad), 256, 0, st>>>(a, file_of_home, static_cast<double *>(pos),
                                                                 static_cast<double *>(vel),
                                                                 static_cast<double *>(rot), cell,
                                                                 static_cast<double *>(frc));
}

template<class R> void launch_set_carried(const KArgs<R> &a, const double *f3, const double *t3, int64_t nhome,
                                          cudaStream_t st) {
    k_set_carried<R><<<io_grid(nhome), 256, 0, st>>>(a, f3, t3, nhome);
}

template void launch_frame_pack<float>(const KArgs<float> &, const int *, int, void *, void *, void *, int *, void *,
                                       cudaStream_t);
template void launch_frame_pack<double>(const KArgs<double> &, const int *, int, void *, void *, void *, int *,
                                        void *, cudaStream_t);
template void launch_set_carried<float>(const KArgs<float> &, const double *, const double *, int64_t, cudaStream_t);
template void launch_set_carried<double>(const KArgs<double> &, const double *, const double *, int64_t,
                                         cudaStream_t);

}  // namespace orbc
