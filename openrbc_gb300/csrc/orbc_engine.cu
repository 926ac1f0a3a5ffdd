// Host engine of liborbc_gpu: builds the device layout from the caller's
// containers, owns every device buffer, sequences the kernels of one step
// (captured once into a CUDA graph whose neighbour rebuild sits behind a
// device-set conditional node), and implements the C ABI of orbc_gpu.h.
#include "orbc_device.cuh"
#include "orbc_gpu.h"

#include <algorithm>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

namespace orbc {

static thread_local std::string g_last_error;

/* ------------------------------------------------------------------------- */
/* Trajectory frames (src/trajectory.h:26-105): the device gathers a frame's  */
/* payload (POSITION, VELOCITY, ROTATION, VORONOI, FORCE) into a staging      */
/* buffer, a copy stream moves it to one of two pinned host buffers, and a    */
/* writer thread appends titles, header, identity and payload to the file --  */
/* the caller's stream goes on stepping meanwhile.                            */
/* ------------------------------------------------------------------------- */
class FrameWriter {
   public:
    struct Job {
        std::string path;
        bool append = false;
        int nstep = 0, fields = 0, real_bytes = 4;
        uint64_t natom = 0;
        std::shared_ptr<const std::vector<int32_t>> ident;  // (tag, type) pairs in file order
        size_t bytes = 0;                                   // payload bytes in the host buffer
    };
    ~FrameWriter() { stop(); }

    /* A free buffer of at least `bytes` (waits for a pending write to end). */
    int acquire(size_t bytes, int device, std::string &err) {
        std::unique_lock<std::mutex> lk(m_);
        if (!started_) {
            dev_ = device;
            th_ = std::thread([this] { run(); });
            started_ = true;
        }
        cv_.wait(lk, [this] { return !slot_[0].busy || !slot_[1].busy; });
        const int s = slot_[0].busy ? 1 : 0;
        Slot &sl = slot_[s];
        if (!sl.ev && cudaEventCreateWithFlags(&sl.ev, cudaEventDisableTiming) != cudaSuccess) {
            err = "frame writer: cudaEventCreate failed";
            return -1;
        }
        if (sl.cap < bytes) {
            if (sl.h) cudaFreeHost(sl.h);
            sl.h = nullptr;
            sl.cap = 0;
            if (cudaMallocHost(&sl.h, bytes ? bytes : 1) != cudaSuccess) {
                err = "frame writer: pinned allocation of " + std::to_string(bytes) + " bytes failed";
                return -1;
            }
            sl.cap = bytes;
        }
        sl.busy = true;
        return s;
    }
    char *host(int s) { return slot_[s].h; }
    cudaEvent_t event(int s) { return slot_[s].ev; }
    void submit(int s, Job job) {
        std::lock_guard<std::mutex> lk(m_);
        slot_[s].job = std::move(job);
        q_.push_back(s);
        cv_.notify_all();
    }
    /* Wait until every submitted frame is on disk; returns the first write
     * error since the last flush (empty if none). */
    std::string flush() {
        std::unique_lock<std::mutex> lk(m_);
        cv_.wait(lk, [this] { return q_.empty() && !slot_[0].busy && !slot_[1].busy; });
        std::string e;
        e.swap(werr_);
        return e;
    }
    void stop() {
        {
            std::unique_lock<std::mutex> lk(m_);
            if (!started_) return;
            cv_.wait(lk, [this] { return q_.empty() && !slot_[0].busy && !slot_[1].busy; });
            quit_ = true;
            cv_.notify_all();
        }
        th_.join();
        started_ = false;
        for (Slot &sl : slot_) {
            if (sl.h) cudaFreeHost(sl.h);
            if (sl.ev) cudaEventDestroy(sl.ev);
            sl.h = nullptr;
            sl.ev = nullptr;
            sl.cap = 0;
        }
    }

   private:
    struct Slot {
        char *h = nullptr;
        size_t cap = 0;
        cudaEvent_t ev = nullptr;
        bool busy = false;
        Job job;
    };
    Slot slot_[2];
    std::deque<int> q_;
    std::mutex m_;
    std::condition_variable cv_;
    std::thread th_;
    bool started_ = false, quit_ = false;
    int dev_ = 0;
    std::string werr_;

    static bool put_title(FILE *f, const char *t) {
        char b[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        std::memcpy(b, t, std::strlen(t));
        return std::fwrite(b, 1, 8, f) == 8;
    }
    void run() {
        cudaSetDevice(dev_);
        for (;;) {
            int s;
            {
                std::unique_lock<std::mutex> lk(m_);
                cv_.wait(lk, [this] { return quit_ || !q_.empty(); });
                if (q_.empty()) return;
                s = q_.front();
            }
            Slot &sl = slot_[s];
            const Job &j = sl.job;
            std::string e;
            if (cudaEventSynchronize(sl.ev) != cudaSuccess) e = "frame writer: device copy failed";
            FILE *f = e.empty() ? std::fopen(j.path.c_str(), j.append ? "ab" : "wb") : nullptr;
            if (e.empty() && !f) e = "frame writer: cannot open " + j.path;
            if (f) {
                bool ok = put_title(f, "FRAMEBEG") && std::fwrite(&j.nstep, 4, 1, f) == 1 && put_title(f, "NATOM") &&
                          std::fwrite(&j.natom, 8, 1, f) == 1 && put_title(f, "IDENTITY") &&
                          std::fwrite(j.ident->data(), 4, j.ident->size(), f) == j.ident->size();
                static const char *titles[5] = {"POSITION", "VELOCITY", "ROTATION", "VORONOI", "FORCE"};
                static const int bits[5] = {1, 8, 2, 4, 16};
                size_t off = 0;
                for (int k = 0; k < 5 && ok; ++k) {
                    if (!(j.fields & bits[k])) continue;
                    const size_t b = size_t(j.natom) * (k == 3 ? 4 : 3 * size_t(j.real_bytes));
                    ok = put_title(f, titles[k]) && std::fwrite(sl.h + off, 1, b, f) == b;
                    off += b;
                }
                ok = ok && put_title(f, "FRAMEEND");
                if (std::fclose(f) != 0 || !ok) e = "frame writer: write to " + j.path + " failed";
            }
            std::lock_guard<std::mutex> lk(m_);
            if (!e.empty() && werr_.empty()) werr_ = e;
            q_.pop_front();
            sl.busy = false;
            cv_.notify_all();
        }
    }
};

/* ------------------------------------------------------------------------- */
/* Force field in FP64 (src/forcefield_canonical.h:23-156).                  */
/* ------------------------------------------------------------------------- */
struct FFHost {
    double mass[NT], radius[NT];
    double cutsq[NT * NT], cut[NT * NT], rep[NT * NT], att[NT * NT], alpha[NT * NT];
    double ljcutsq[NT * NT], lj1[NT * NT], lj2[NT * NT];
    int kind[NT * NT];
    double range[NT * NT];  // interaction range of the type pair (0 = none)
    FFHost() {
        const double m[NT] = {1, 4, 4, 1, 10, 10};
        const double rad[NT] = {0.56125, 1.12375, 1.12375, 0.56125, 1.5, 0.5};
        // lipid-protein row (by protein type) and protein-protein block (types 1..3)
        const double cl[NT] = {2.6, 2.6, 2.6, 2.6, 0, 0};
        const double rl[NT] = {1.1225, 1.685, 1.685, 1.1225, 0, 0};
        const double el[NT] = {1.2, 1.4, 2.8, 2.8, 0, 0};
        const double al[NT] = {1.55, 5, 5, 5, 0, 0};
        const double rp[4][4] = {{1.1225, 1.685, 1.685, 1.1225}, {1.685, 2.245, 2.245, 1.685},
                                 {1.685, 2.245, 2.245, 1.685}, {1.1225, 1.685, 1.685, 1.1225}};
        const double ep[4][4] = {{1.2, 1.4, 2.8, 2.8}, {1.4, 1, 1, 1}, {2.8, 1, 1, 1}, {2.8, 1, 1, 1}};
        const double lje[NT * NT] = {0, 0, 0, 0, 1, 1, 0, 0, 0, 0, 1, 1, 0, 0, 0, 0, 1, 1,
                                     0, 0, 0, 0, 0, 0, 1, 1, 1, 0, 0, 0, 1, 1, 1, 0, 0, 0};
        const double ljs[NT * NT] = {0, 0, 0, 0, 1, 1, 0, 0, 0, 0, 3.4, 3.4, 0, 0, 0, 0, 3.4, 1,
                                     0, 0, 0, 0, 0, 0, 1, 3.4, 3.4, 0, 3, 1.8, 1, 3.4, 1, 0, 1.8, 1};
        const double w = 3.4 * 1.1225;
        const double ljc[NT * NT] = {0, 0, 0, 0, 1.1225, 1.1225, 0, 0, 0, 0, w, w, 0, 0, 0, 0, w, 1.1225,
                                     0, 0, 0, 0, 0, 0, 1.1225, w, w, 0, 0, 0, 1.1225, w, 1.1225, 0, 0, 0};
        auto pw = [](double b, int e) {
            double p = 1;
            for (int k = 0; k < e; ++k) p = b * p;
            return p;
        };
        for (int t = 0; t < NT; ++t) {
            mass[t] = m[t];
            radius[t] = rad[t];
        }
        for (int ti = 0; ti < NT; ++ti)
            for (int tj = 0; tj < NT; ++tj) {
                const int k = ti * NT + tj;
                double c = 0, req = 0, eps = 0, a = 0;
                int lj_idx, kd;
                if (ti == 0 || tj == 0) {  // lipid-lipid / lipid-protein: table index = protein type
                    const int p = std::max(ti, tj);
                    c = cl[p];
                    req = rl[p];
                    eps = el[p];
                    a = al[p];
                    kd = c > 0 ? PAIR_ANISO : PAIR_NONE;
                    lj_idx = p;
                } else {  // protein-protein: type12 = t1 + 6 t2
                    lj_idx = ti + NT * tj;
                    if (ti < 4 && tj < 4) {
                        c = 2.6;
                        req = rp[ti][tj];
                        eps = ep[ti][tj];
                        kd = PAIR_REP;
                    } else {
                        kd = PAIR_NONE;
                    }
                }
                kind[k] = kd;
                cut[k] = kd ? c : 0;
                cutsq[k] = kd ? c * c : 0;
                rep[k] = kd ? eps / pw(c - req, 8) : 0;
                att[k] = kd == PAIR_ANISO ? -2.0 * eps / pw(c - req, 4) : 0;
                alpha[k] = kd == PAIR_ANISO ? a : 0;
                ljcutsq[k] = ljc[lj_idx] * ljc[lj_idx];
                lj1[k] = 48.0 * lje[lj_idx] * std::pow(ljs[lj_idx], 12);
                lj2[k] = 24.0 * lje[lj_idx] * std::pow(ljs[lj_idx], 6);
                range[k] = std::sqrt(std::max(cutsq[k], ljcutsq[k]));
            }
    }
};
static const FFHost &ffh() {
    static const FFHost f;
    return f;
}

/* ------------------------------------------------------------------------- */
template<class T> struct DevBuf {
    T *p = nullptr;
    size_t n = 0;
    cudaError_t alloc(size_t count) {
        release();
        n = count;
        if (count == 0) count = 1;
        return cudaMalloc(&p, count * sizeof(T));
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    ~DevBuf() { release(); }
};

struct HostSys {
    orbc_system_desc desc;
    int64_t begin, end;  // caller index range
};

class EngineBase {
   public:
    virtual ~EngineBase() {}
    std::string err;
    orbc_params P;
    int fail(int code, const std::string &msg) {
        err = msg;
        g_last_error = msg;
        return code;
    }
    virtual int upload(int nsys, const orbc_system_desc *sys, const int64_t *offsets, const double *x3,
                       const double *n3, const double *v3, const double *o3, const int *type, const int *tag, size_t n,
                       const int *bonds3, const double *bond_r0, size_t nb, const int *faces3, size_t nf) = 0;
    virtual int set_state(const double *x3, const double *n3, const double *v3, const double *o3) = 0;
    virtual int set_state_f32(int64_t first, int64_t count, int stride, const float *x, const float *n,
                              const float *v, const float *o) = 0;
    virtual int assign_temperature(double kT, uint64_t seed) = 0;
    virtual int minimize(int nsteps, double dr_opt, double dn_opt, orbc_thermo *out) = 0;
    virtual int save_frame(const char *path, int append, int nstep, int fields, int real_bytes, int async) = 0;
    virtual int flush_frames() = 0;
    virtual int save_checkpoint(const char *path) = 0;
    virtual int cleanup(double tol, int64_t *removed) = 0;
    virtual int load_checkpoint(const char *path) = 0;
    virtual int step(int nsteps, orbc_thermo *out) = 0;
    virtual int download(double *x3, double *n3, double *v3, double *o3) = 0;
    virtual int download_f32(int64_t first, int64_t count, int stride, float *x, float *n, float *v, float *o) = 0;
    virtual int forces(double *f3, double *t3, double *e) = 0;
    virtual int thermo(int sys, orbc_thermo *out) = 0;
    virtual int neighbors(int *counts, int *list, int64_t cap, int64_t *total) = 0;
    virtual int cells(int sys, double *lo3, double *lc3, int *nc3, int *cell, double *off3, int *slot) = 0;
    virtual int rebuild() = 0;
    virtual int rdf(int sys, int ta, int tb, double dr, int nbins, double rcut, uint64_t *counts,
                    int64_t *dropped) = 0;
    virtual int profile(int nsteps, orbc_profile *out) = 0;
    virtual int autotune(int trial_steps, orbc_tune_trial *trials, int max_trials, int *ntrials) = 0;
    double last_ms = 0;
    int64_t last_launches = 0;
};

#define CK(x)                                                                                  \
    do {                                                                                       \
        cudaError_t e_ = (x);                                                                  \
        if (e_ != cudaSuccess) return fail(ORBC_ERR_CUDA, std::string(#x) + ": " + cudaGetErrorString(e_)); \
    } while (0)

static int err_code_of(int bits) {
    if (bits & ERRB_NBR_OVERFLOW) return ORBC_ERR_NBR_OVERFLOW;
    if (bits & ERRB_NAN) return ORBC_ERR_NAN;
    if (bits & ERRB_BOND) return ORBC_ERR_BOND;
    if (bits & ERRB_GRID) return ORBC_ERR_GRID;
    return ORBC_OK;
}
static int flag_bits(int bits) {
    int f = 0;
    if (bits & ERRB_NBR_OVERFLOW) f |= 1 << ORBC_ERR_NBR_OVERFLOW;
    if (bits & ERRB_NAN) f |= 1 << ORBC_ERR_NAN;
    if (bits & ERRB_BOND) f |= 1 << ORBC_ERR_BOND;
    if (bits & ERRB_GRID) f |= 1 << ORBC_ERR_GRID;
    return f;
}

template<class R> class Engine : public EngineBase {
    using T4 = typename Vec<R>::T4;

   public:
    explicit Engine(const orbc_params &p) { P = p; }
    ~Engine() override {
        fw.stop();  // pending frames reach the disk before the buffers go
        drop_graph();
        if (ev0) cudaEventDestroy(ev0);
        if (ev1) cudaEventDestroy(ev1);
        if (hsc) cudaFreeHost(hsc);
        for (cudaEvent_t &e : fpack)
            if (e) cudaEventDestroy(e);
        for (cudaEvent_t &e : xev)
            if (e) cudaEventDestroy(e);
        for (cudaEvent_t &e : pev)
            if (e) cudaEventDestroy(e);
        if (cs) cudaStreamDestroy(cs);
        if (st) cudaStreamDestroy(st);
    }

    int init() {
        int ndev = 0;
        if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(ORBC_ERR_NODEV, "no CUDA device");
        CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        CK(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
        CK(cudaEventCreate(&ev0));
        CK(cudaEventCreate(&ev1));
        CK(cudaMallocHost(&hsc, 2 * sizeof(Scalars)));
        for (cudaEvent_t &e : fpack) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        for (cudaEvent_t &e : xev) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        for (cudaEvent_t &e : pev) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        CK(cudaGetDevice(&device));
        int pma = 0;
        CK(cudaDeviceGetAttribute(&pma, cudaDevAttrPageableMemoryAccess, device));
        pageable_access = pma != 0;
        return ORBC_OK;
    }
    bool pageable_access = false;  // the GPU reads pageable host memory (host page tables)
    int64_t direct_transfers = 0;  // set_state_f32 / download_f32 calls served in place

    /* --------------------------------------------------------------------- */
    int upload(int nsys, const orbc_system_desc *descs, const int64_t *offsets, const double *x3, const double *n3,
               const double *v3, const double *o3, const int *type, const int *tag, size_t n_, const int *bonds3,
               const double *bond_r0, size_t nb, const int *faces3, size_t nf) override {
        const int64_t n = int64_t(n_);
        if (nsys < 1 || n < 1 || !x3 || !n3 || !type || !tag) return fail(ORBC_ERR_ARG, "upload: empty system");
        if (offsets[0] != 0 || offsets[nsys] != n) return fail(ORBC_ERR_ARG, "upload: offsets must span [0, n)");
        for (int s = 0; s < nsys; ++s)
            if (offsets[s + 1] <= offsets[s]) return fail(ORBC_ERR_ARG, "upload: empty system in batch");
        for (int64_t i = 0; i < n; ++i) {
            if (type[i] < 0 || type[i] >= NT) return fail(ORBC_ERR_ARG, "upload: particle type outside 0..5");
            if (tag[i] < 0) return fail(ORBC_ERR_ARG, "upload: negative tag");
        }
        drop_graph();
        nh_primed = false;
        vcom_valid = false;
        if (!relayout_in_progress) {  // topology copy for re-layouts (autotune)
            topo.descs.assign(descs, descs + nsys);
            topo.offsets.assign(offsets, offsets + nsys + 1);
            topo.type.assign(type, type + n);
            topo.tag.assign(tag, tag + n);
            topo.bonds.assign(bonds3 ? bonds3 : nullptr, bonds3 ? bonds3 + 3 * nb : nullptr);
            topo.bond_r0.assign(bond_r0 ? bond_r0 : nullptr, bond_r0 ? bond_r0 + nb : nullptr);
            topo.faces.assign(faces3 ? faces3 : nullptr, faces3 ? faces3 + 3 * nf : nullptr);
        }
        this->nsys = nsys;
        nhome = n;
        {
            int rc = build_file_order(type, tag, n);
            if (rc) return rc;
        }
        const FFHost &F = ffh();
        // tag -> caller index
        int maxtag = 0;
        for (int64_t i = 0; i < n; ++i) maxtag = std::max(maxtag, tag[i]);
        std::vector<int> t2i(size_t(maxtag) + 1, -1);
        for (int64_t i = 0; i < n; ++i) {
            if (t2i[size_t(tag[i])] >= 0) return fail(ORBC_ERR_ARG, "upload: duplicate tag");
            t2i[size_t(tag[i])] = int(i);
        }
        auto idx_of = [&](int t) { return (t >= 0 && t <= maxtag) ? t2i[size_t(t)] : -1; };

        // ---- per-system grid and slot layout
        hsys.assign(size_t(nsys), SysDev());
        ngroups_total = 0;
        std::vector<int> sys_of(static_cast<size_t>(n));
        int64_t off = 0;
        uint64_t cbase = 0;
        for (int s = 0; s < nsys; ++s) {
            SysDev &sd = hsys[size_t(s)];
            std::memset(&sd, 0, sizeof(sd));
            const orbc_system_desc &d = descs[s];
            const int64_t b = offsets[s], e = offsets[s + 1];
            bool present[NT] = {false, false, false, false, false, false};
            for (int64_t i = b; i < e; ++i) {
                present[type[i]] = true;
                sys_of[size_t(i)] = s;
            }
            double rmax = 0;
            for (int ta = 0; ta < NT; ++ta)
                for (int tc = 0; tc < NT; ++tc)
                    if (present[ta] && present[tc] && F.range[ta * NT + tc] > 0)
                        rmax = std::max(rmax, F.range[ta * NT + tc]);
            const double rl = (rmax > 0 ? rmax : 1.0) + P.skin;
            for (int dd = 0; dd < 3; ++dd) {
                const int maxnc = dd < 2 ? MAX_NC_XY : MAX_NC_Z;
                sd.per[dd] = d.periodic[dd] ? 1 : 0;
                if (sd.per[dd]) {
                    const double L = d.hi[dd] - d.lo[dd];
                    int nc = int(std::floor(L / rl));
                    if (nc < 3) return fail(ORBC_ERR_ARG, "upload: periodic box shorter than 3 list cutoffs");
                    nc = std::min(nc, maxnc);
                    sd.nc[dd] = nc;
                    sd.Lc[dd] = L / nc;
                    sd.lo[dd] = d.lo[dd];
                } else {
                    double mn = 1e300, mx = -1e300;
                    for (int64_t i = b; i < e; ++i) {
                        mn = std::min(mn, x3[3 * i + dd]);
                        mx = std::max(mx, x3[3 * i + dd]);
                    }
                    const double ext = mx - mn;
                    const double margin = std::max(0.25 * ext, 4.0 * rl) + rl;
                    double Lc = rl;
                    int nc = int(std::ceil((ext + 2 * margin) / Lc));
                    if (nc > maxnc) {
                        nc = maxnc;
                        Lc = (ext + 2 * margin) / nc;
                    }
                    sd.nc[dd] = std::max(nc, 1);
                    sd.Lc[dd] = Lc;
                    sd.lo[dd] = 0.5 * (mn + mx) - 0.5 * nc * Lc;
                }
                if (P.bounce && !sd.per[dd]) {  // walls (Nose-Hoover step, minimisation) on open axes
                    sd.wlo[dd] = d.lo[dd];
                    sd.whi[dd] = d.hi[dd];
                }
                // the kernels' copies: no FP64 division or conversion per particle
                sd.invLc[dd] = 1.0 / sd.Lc[dd];
                sd.Lcf[dd] = float(sd.Lc[dd]);
                sd.invLcf[dd] = float(sd.invLc[dd]);
            }
            const int64_t ns = e - b;
            const int64_t npad_s = std::max<int64_t>(SYS_PAD, (ns + SYS_PAD - 1) / SYS_PAD * SYS_PAD);
            sd.gbase = ngroups_total;
            sd.ngrp = int((npad_s / 32 + RED_GROUP - 1) / RED_GROUP);
            ngroups_total += sd.ngrp;
            sd.off = int(off);
            sd.npad = int(npad_s);
            sd.nreal = int(ns);
            sd.nlipid = 0;
            for (int64_t i = b; i < e; ++i) sd.nlipid += type[i] == 0 ? 1 : 0;
            sd.cell_base = unsigned(cbase);
            sd.kv = d.kv;
            sd.V0 = d.V0;
            sd.ka = d.ka;
            sd.A0 = d.A0;
            sd.Q = P.Q;
            off += npad_s;
            for (int dd = 0; dd < 3; ++dd) sd.ntile[dd] = (sd.nc[dd] + 3) / 4;
            cbase += uint64_t(sd.ntile[0]) * uint64_t(sd.ntile[1]) * uint64_t(sd.ntile[2]) * 64u + 1;
        }
        if (off >= MAX_SLOTS) return fail(ORBC_ERR_ARG, "upload: more than 2^27 particle slots");
        if (cbase >= (uint64_t(1) << 32) - 1) return fail(ORBC_ERR_ARG, "upload: more than 2^32 cells");
        npad = int(off);
        const int nb256 = npad / SYS_PAD;
        total_cells = cbase;

        // ---- slots
        std::vector<T4> hpos(static_cast<size_t>(npad)), hnrm(static_cast<size_t>(npad)), hvel(static_cast<size_t>(npad)), homg(static_cast<size_t>(npad)),
            hzero(static_cast<size_t>(npad));
        std::vector<int> hcell(size_t(npad), 0), htag(size_t(npad), -1), hhome(size_t(npad), -1),
            hsoh(static_cast<size_t>(n)), hbs(static_cast<size_t>(nb256));
        std::vector<int> wbitsv(size_t(npad), GHOST);
        std::memset(hzero.data(), 0, hzero.size() * sizeof(T4));
        for (int s = 0; s < nsys; ++s) {
            const SysDev &sd = hsys[size_t(s)];
            for (int b = sd.off / SYS_PAD; b < (sd.off + sd.npad) / SYS_PAD; ++b) hbs[size_t(b)] = s;
            for (int64_t i = offsets[s]; i < offsets[s + 1]; ++i) {
                const int p = sd.off + int(i - offsets[s]);
                hhome[size_t(p)] = int(i);
                hsoh[size_t(i)] = p;
                htag[size_t(p)] = tag[i];
                wbitsv[size_t(p)] = type[i];
                int cc[3];
                double o[3];
                bin_point(sd, &x3[3 * i], cc, o);
                hcell[size_t(p)] = cpack(cc[0], cc[1], cc[2]);
                hpos[size_t(p)] = mk4(R(o[0]), R(o[1]), R(o[2]));
                hnrm[size_t(p)] = mk4(R(n3[3 * i]), R(n3[3 * i + 1]), R(n3[3 * i + 2]));
                hvel[size_t(p)] = v3 ? mk4(R(v3[3 * i]), R(v3[3 * i + 1]), R(v3[3 * i + 2])) : mk4(0, 0, 0);
                homg[size_t(p)] = o3 ? mk4(R(o3[3 * i]), R(o3[3 * i + 1]), R(o3[3 * i + 2])) : mk4(0, 0, 0);
            }
        }
        for (int p = 0; p < npad; ++p)
            if (hhome[size_t(p)] < 0) {
                hpos[size_t(p)] = mk4(0, 0, 0);
                hnrm[size_t(p)] = mk4(0, 0, 1);
                hvel[size_t(p)] = mk4(0, 0, 0);
                homg[size_t(p)] = mk4(0, 0, 0);
            }
        // ---- bonds (ELL by slot, both ends)
        std::vector<int> bdeg(size_t(npad), 0);
        for (size_t l = 0; l < nb; ++l) {
            const int bt = bonds3[3 * l], ki = idx_of(bonds3[3 * l + 1]), kj = idx_of(bonds3[3 * l + 2]);
            if (bt < 0 || bt >= MAX_BT) return fail(ORBC_ERR_ARG, "upload: bond type outside 0..7");
            if (ki < 0 || kj < 0) return fail(ORBC_ERR_ARG, "upload: bond endpoint tag not found");
            if (ki == kj) return fail(ORBC_ERR_ARG, "upload: bond to itself");
            if (sys_of[size_t(ki)] != sys_of[size_t(kj)]) return fail(ORBC_ERR_ARG, "upload: bond across systems");
            bdeg[size_t(hsoh[size_t(ki)])]++;
            bdeg[size_t(hsoh[size_t(kj)])]++;
        }
        maxb = 0;
        for (int d : bdeg) maxb = std::max(maxb, d);
        if (maxb > MAX_DEG) return fail(ORBC_ERR_ARG, "upload: more than 15 bonds on one particle");
        std::vector<BondSlot> hb(size_t(std::max(maxb, 1)) * size_t(npad));
        std::fill(bdeg.begin(), bdeg.end(), 0);
        for (size_t l = 0; l < nb; ++l) {
            const int bt = bonds3[3 * l];
            const int pi = hsoh[size_t(idx_of(bonds3[3 * l + 1]))], pj = hsoh[size_t(idx_of(bonds3[3 * l + 2]))];
            const double r0 = bond_r0 ? bond_r0[l] : P.bond_r0[bt];
            hb[size_t(bdeg[size_t(pi)]++) * npad + size_t(pi)] = BondSlot{pj, bt, r0};
            hb[size_t(bdeg[size_t(pj)]++) * npad + size_t(pj)] = BondSlot{pi, bt, r0};
        }
        // ---- faces
        std::vector<int> fdeg(size_t(npad), 0);
        std::vector<int4> hfaces;
        hfaces.reserve(nf);
        for (int s = 0; s < nsys; ++s) {
            hsys[size_t(s)].face_begin = int(hfaces.size());
            for (size_t k = 0; k < nf; ++k) {
                int q[3];
                for (int c = 0; c < 3; ++c) {
                    const int ki = idx_of(faces3[3 * k + c]);
                    if (ki < 0) return fail(ORBC_ERR_ARG, "upload: face vertex tag not found");
                    q[c] = ki;
                }
                if (sys_of[size_t(q[0])] != s) continue;
                if (sys_of[size_t(q[1])] != s || sys_of[size_t(q[2])] != s)
                    return fail(ORBC_ERR_ARG, "upload: face across systems");
                const int a = hsoh[size_t(q[0])], b = hsoh[size_t(q[1])], c = hsoh[size_t(q[2])];
                hfaces.push_back(make_int4(a, b, c, s));
                fdeg[size_t(a)]++;
                fdeg[size_t(b)]++;
                fdeg[size_t(c)]++;
            }
            hsys[size_t(s)].face_end = int(hfaces.size());
        }
        // blocks of the area / volume kernel: MESH_CHUNK faces of one system each
        std::vector<int> hmbs;
        for (int s = 0; s < nsys; ++s) {
            SysDev &sd = hsys[size_t(s)];
            const int nfs = sd.face_end - sd.face_begin;
            sd.mblk_begin = int(hmbs.size());
            for (int k = 0; k < (nfs + MESH_CHUNK - 1) / MESH_CHUNK; ++k) hmbs.push_back(s);
            sd.mblk_end = int(hmbs.size());
        }
        nmblk = int(hmbs.size());
        maxf = 0;
        for (int d : fdeg) maxf = std::max(maxf, d);
        if (maxf > MAX_DEG) return fail(ORBC_ERR_ARG, "upload: more than 15 faces on one vertex");
        std::vector<int2> hfs(size_t(std::max(maxf, 1)) * size_t(npad));
        std::fill(fdeg.begin(), fdeg.end(), 0);
        for (const int4 &q : hfaces) {
            hfs[size_t(fdeg[size_t(q.x)]++) * npad + size_t(q.x)] = make_int2(q.y, q.z);
            hfs[size_t(fdeg[size_t(q.y)]++) * npad + size_t(q.y)] = make_int2(q.z, q.x);
            hfs[size_t(fdeg[size_t(q.z)]++) * npad + size_t(q.z)] = make_int2(q.x, q.y);
        }
        for (int p = 0; p < npad; ++p) {
            const int w = hhome[size_t(p)] < 0 ? GHOST : (wbitsv[size_t(p)] | (bdeg[size_t(p)] << 4) | (fdeg[size_t(p)] << 8));
            setw(hpos[size_t(p)], w);
        }
        has_mesh = !hfaces.empty();
        nfaces = int(hfaces.size());

        // ---- device allocation
        for (int k = 0; k < 2; ++k) {
            if (pos[k].alloc(size_t(npad)) || nrm[k].alloc(size_t(npad)) || vel[k].alloc(size_t(npad)) ||
                omg[k].alloc(size_t(npad)) || frc[k].alloc(size_t(npad)) || trq[k].alloc(size_t(npad)) ||
                xref[k].alloc(size_t(npad)) || cell[k].alloc(size_t(npad)) || tagd[k].alloc(size_t(npad)) ||
                home[k].alloc(size_t(npad)) || bond[k].alloc(hb.size()) || fslot[k].alloc(hfs.size()) ||
                skey[k].alloc(size_t(npad)) || sval[k].alloc(size_t(npad)))
                return fail(ORBC_ERR_NOMEM, "upload: device allocation failed");
        }
        ntiles = sort_tiles(npad);
        if (epart.alloc(size_t(npad)) || faces.alloc(hfaces.size()) || ranges.alloc(size_t(total_cells)) ||
            soh.alloc(size_t(n)) || blk_sys.alloc(size_t(nb256)) || partial.alloc(size_t(npad / 32) * NPART) || gpartial.alloc(size_t(ngroups_total) * NPART) ||
            Sd.alloc(1) || sysd.alloc(size_t(nsys)) || ssd.alloc(size_t(nsys)) || counts.alloc(size_t(256) * ntiles) ||
            dtot.alloc(256) || invd.alloc(size_t(npad)) || ffd.alloc(1) || nnb.alloc(size_t(npad)) ||
            stage.alloc(size_t(n) * 12) || mesh_bs.alloc(hmbs.size()) || mesh_part.alloc(hmbs.size() * 2 + 2))
            return fail(ORBC_ERR_NOMEM, "upload: device allocation failed");
        cap = P.max_neighbors > 0 ? P.max_neighbors : 64;

        if (nbr.alloc(size_t(cap) * size_t(npad))) return fail(ORBC_ERR_NOMEM, "upload: neighbour list allocation failed");

        CK(cudaMemcpyAsync(pos[0].p, hpos.data(), hpos.size() * sizeof(T4), cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(nrm[0].p, hnrm.data(), hnrm.size() * sizeof(T4), cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(vel[0].p, hvel.data(), hvel.size() * sizeof(T4), cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(omg[0].p, homg.data(), homg.size() * sizeof(T4), cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(frc[0].p, hzero.data(), hzero.size() * sizeof(T4), cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(trq[0].p, hzero.data(), hzero.size() * sizeof(T4), cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(xref[0].p, hpos.data(), hpos.size() * sizeof(T4), cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(cell[0].p, hcell.data(), hcell.size() * sizeof(int), cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(tagd[0].p, htag.data(), htag.size() * sizeof(int), cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(home[0].p, hhome.data(), hhome.size() * sizeof(int), cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(bond[0].p, hb.data(), hb.size() * sizeof(BondSlot), cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(fslot[0].p, hfs.data(), hfs.size() * sizeof(int2), cudaMemcpyHostToDevice, st));
        if (!hfaces.empty())
            CK(cudaMemcpyAsync(faces.p, hfaces.data(), hfaces.size() * sizeof(int4), cudaMemcpyHostToDevice, st));
        if (!hmbs.empty())
            CK(cudaMemcpyAsync(mesh_bs.p, hmbs.data(), hmbs.size() * sizeof(int), cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(soh.p, hsoh.data(), hsoh.size() * sizeof(int), cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(blk_sys.p, hbs.data(), hbs.size() * sizeof(int), cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(sysd.p, hsys.data(), hsys.size() * sizeof(SysDev), cudaMemcpyHostToDevice, st));
        CK(cudaMemsetAsync(ranges.p, 0, size_t(total_cells) * sizeof(int2), st));
        CK(cudaMemsetAsync(partial.p, 0, size_t(npad / 32) * NPART * sizeof(double), st));
        CK(cudaMemsetAsync(gpartial.p, 0, size_t(ngroups_total) * NPART * sizeof(double), st));
        CK(cudaMemsetAsync(epart.p, 0, size_t(npad) * sizeof(double), st));
        CK(cudaMemsetAsync(nnb.p, 0, size_t(npad) * sizeof(int), st));
        // other parity copies start equal (gather overwrites them before use)
        Scalars hs;
        std::memset(&hs, 0, sizeof(hs));
        hs.rebuild = 1;
        CK(cudaMemcpyAsync(Sd.p, &hs, sizeof(hs), cudaMemcpyHostToDevice, st));
        std::vector<SysState> hss(static_cast<size_t>(nsys));
        std::memset(hss.data(), 0, hss.size() * sizeof(SysState));
        for (int s = 0; s < nsys; ++s) hss[size_t(s)].zeta = descs[s].zeta;
        CK(cudaMemcpyAsync(ssd.p, hss.data(), hss.size() * sizeof(SysState), cudaMemcpyHostToDevice, st));
        build_ff();
        CK(cudaMemcpyAsync(ffd.p, &hff, sizeof(hff), cudaMemcpyHostToDevice, st));
        // key bits -> radix passes
        int bits = 1;
        while (bits < 32 && (uint64_t(1) << bits) < total_cells) ++bits;
        passes = (bits + 7) / 8;
        fill_args();
        CK(cudaStreamSynchronize(st));
        uploaded = true;
        // first neighbour build; grow the capacity if the guess was short
        int rc = build_lists(true);
        if (rc) return rc;
        if (has_mesh) launch_mesh<R>(a, st);
        launch_vcom<R>(a, st);  // temperature and lipid mean of the uploaded velocities
        CK(cudaGetLastError());
        CK(cudaStreamSynchronize(st));
        vcom_valid = true;
        return ORBC_OK;
    }

    /* --------------------------------------------------------------------- */
    int set_state(const double *x3, const double *n3, const double *v3, const double *o3) override {
        if (!uploaded) return fail(ORBC_ERR_STATE, "set_state before upload");
        if (!x3 || !n3 || !v3 || !o3) return fail(ORBC_ERR_ARG, "set_state: all four arrays are required");
        return set_state_t<double>(0, nhome, 3, x3, n3, v3, o3);
    }
    int set_state_f32(int64_t first, int64_t count, int stride, const float *x, const float *n, const float *v,
                      const float *o) override {
        if (!uploaded) return fail(ORBC_ERR_STATE, "set_state before upload");
        if (!x || !n || !v || !o) return fail(ORBC_ERR_ARG, "set_state_f32: all four arrays are required");
        if (first < 0 || count < 0 || first + count > nhome || (stride != 3 && stride != 4))
            return fail(ORBC_ERR_ARG, "set_state_f32: need 0 <= first, first + count <= n and stride 3 or 4");
        if (count == 0) return ORBC_OK;
        return set_state_t<float>(first, count, stride, x, n, v, o);
    }
    /* upload indices [first, first + count) from host AoS arrays of TH with
     * `stride` values per particle; chunked: the copy stream moves chunk c + 1
     * while the step stream converts chunk c */
    /* Whether the GPU can read / write host arrays in place: page-locked
     * memory mapped at the same address (cudaHostAlloc / cudaHostRegister under
     * unified addressing), or pageable memory on a GPU that reads the host's
     * page tables.  Device and managed memory take the staged path. */
    bool host_reachable(const void *p) {
        if (!P.host_direct || !p) return false;
        cudaPointerAttributes at;
        if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        if (at.type == cudaMemoryTypeHost) return at.devicePointer == p;
        if (at.type == cudaMemoryTypeUnregistered) return pageable_access;
        return false;
    }
    template<class TH>
    int set_state_t(int64_t first, int64_t count, int stride, const TH *x, const TH *n, const TH *v, const TH *o) {
        if (host_reachable(x) && host_reachable(n) && host_reachable(v) && host_reachable(o)) {
            // one pass over the host link: the conversion kernel reads the caller's arrays
            launch_set_state_host<R, TH>(a, x, n, v, o, first, first + count, first, stride, st);
            vcom_valid = !lite();
            if (vcom_valid) launch_vcom<R>(a, st);
            CK(cudaGetLastError());
            CK(cudaStreamSynchronize(st));  // the caller may reuse its arrays on return
            nh_primed = false;
            ++direct_transfers;
            return ORBC_OK;
        }
        TH *d = reinterpret_cast<TH *>(stage.p);
        const TH *src[4] = {x, n, v, o};
        const int64_t m = count * stride;  // values per array
        const int nch = count >= (int64_t(1) << 20) ? NXCH : 1;
        CK(cudaEventRecord(pev[0], st));  // earlier work on the staging buffer
        CK(cudaStreamWaitEvent(cs, pev[0], 0));
        for (int c = 0; c < nch; ++c) {
            const int64_t k0 = count * c / nch, k1 = count * (c + 1) / nch;
            for (int q = 0; q < 4; ++q)
                CK(cudaMemcpyAsync(d + m * q + k0 * stride, src[q] + k0 * stride, size_t(k1 - k0) * stride * sizeof(TH),
                                   cudaMemcpyHostToDevice, cs));
            CK(cudaEventRecord(xev[c], cs));
            CK(cudaStreamWaitEvent(st, xev[c], 0));
            launch_set_state<R, TH>(a, d, d + m, d + 2 * m, d + 3 * m, first + k0, first + k1, first, stride, st);
        }
        // temperature and lipid mean of the new velocities; the lite Langevin
        // step needs neither (thermo() reduces them on demand)
        vcom_valid = !lite();
        if (vcom_valid) launch_vcom<R>(a, st);
        CK(cudaStreamSynchronize(cs));  // the caller may reuse its arrays on return
        CK(cudaGetLastError());
        nh_primed = false;
        return ORBC_OK;
    }

    int minimize(int nsteps, double dr_opt, double dn_opt, orbc_thermo *out) override {
        if (!uploaded) return fail(ORBC_ERR_STATE, "minimize before upload");
        if (nsteps < 0 || !(dr_opt > 0) || !(dn_opt > 0))
            return fail(ORBC_ERR_ARG, "minimize: need nsteps >= 0 and positive move limits");
        for (int attempt = 0;; ++attempt) {
            Scalars before;
            CK(cudaMemcpy(&before, Sd.p, sizeof(Scalars), cudaMemcpyDeviceToHost));
            for (int k = 0; k < nsteps; ++k) {
                launch_rebuild<R>(a, st, true);
                if (has_mesh) launch_mesh<R>(a, st);
                launch_minimize<R>(a, dr_opt, dn_opt, st);
            }
            CK(cudaGetLastError());
            CK(cudaStreamSynchronize(st));
            Scalars hs;
            CK(cudaMemcpy(&hs, Sd.p, sizeof(Scalars), cudaMemcpyDeviceToHost));
            if (!(hs.error & (ERRB_NBR_OVERFLOW | ERRB_GRID))) break;
            // a halting build: the iterations after it did nothing; grow the
            // list or re-grid, rebuild from the current state and run the rest
            if (attempt == 4) return fail(ORBC_ERR_NBR_OVERFLOW, "minimize: neighbour capacity could not be sized");
            const int rc = recover(hs);
            if (rc) return rc;
            nsteps -= int(hs.iters - before.iters);
        }
        nh_primed = false;   // forces of the new configuration are not carried
        vcom_valid = false;  // walls may have reversed velocities
        Scalars hs;
        CK(cudaMemcpy(&hs, Sd.p, sizeof(Scalars), cudaMemcpyDeviceToHost));
        if (out) {
            int rc = thermo(-1, out);
            if (rc) return rc;
        }
        if (hs.max_nnb > cap * 0.85) {
            int rc = grow_capacity(hs.max_nnb);
            if (rc) return rc;
        }
        const int code = err_code_of(hs.error);
        if (code) return fail(code, "minimize: device reported error bits " + std::to_string(hs.error));
        return ORBC_OK;
    }

    /* After a halting build (see halted(): a list overflowed, or a particle
     * left its system's open grid; the step kernels that followed left the
     * state untouched): re-grid the systems from the current state if a
     * particle left a grid -- a full re-layout, which also sizes the lists --
     * else grow the capacity to the need the build reported, clear the flag
     * and rebuild. */
    int recover(const Scalars &hs) {
        if (hs.error & ERRB_GRID) return regrid();
        int rc = grow_capacity(hs.max_nnb, false);
        if (rc) return rc;
        const int clr = hs.error & ~ERRB_NBR_OVERFLOW;
        CK(cudaMemcpy(&Sd.p->error, &clr, sizeof(int), cudaMemcpyHostToDevice));
        return build_lists(false);
    }
    /* New grids for the current positions: the open axes are sized again from
     * the particles' extent (the state, the step counter and each system's
     * thermostat variable are kept; carried Nose-Hoover forces are not). */
    int regrid() {
        const size_t m = size_t(nhome) * 3;
        std::vector<double> x(m), nv(m), v(m), o(m);
        int rc = download(x.data(), nv.data(), v.data(), o.data());
        if (rc) return rc;
        Scalars hs;
        CK(cudaMemcpy(&hs, Sd.p, sizeof(Scalars), cudaMemcpyDeviceToHost));
        std::vector<SysState> hss(topo.descs.size());
        CK(cudaMemcpy(hss.data(), ssd.p, hss.size() * sizeof(SysState), cudaMemcpyDeviceToHost));
        for (size_t k = 0; k < hss.size(); ++k) topo.descs[k].zeta = hss[k].zeta;
        rc = relayout(x, nv, v, o, hs.step);
        if (rc) return rc;
        ++regrids;
        return ORBC_OK;
    }
    int64_t regrids = 0;

    /* Frame order (src/trajectory.h:75-77): lipids, then proteins, each in
     * upload order; fmap = file position of each upload index. */
    int build_file_order(const int *type, const int *tag, int64_t n) {
        std::vector<int> hf(static_cast<size_t>(n));
        auto id = std::make_shared<std::vector<int32_t>>(static_cast<size_t>(2 * n));
        int64_t k = 0;
        for (int pass = 0; pass < 2; ++pass)
            for (int64_t q = 0; q < n; ++q)
                if ((type[q] == 0) == (pass == 0)) {
                    hf[size_t(q)] = int(k);
                    (*id)[size_t(2 * k)] = tag[q];
                    (*id)[size_t(2 * k + 1)] = type[q];
                    ++k;
                }
        ident = id;
        CK(fmap.alloc(size_t(n)));
        CK(cudaMemcpy(fmap.p, hf.data(), hf.size() * sizeof(int), cudaMemcpyHostToDevice));
        return ORBC_OK;
    }

    /* delete_lipid (src/cleanup.h:29-91): see orbc_cleanup.cu. */
    int cleanup(double tol, int64_t *removed_out) override {
        if (!uploaded) return fail(ORBC_ERR_STATE, "cleanup before upload");
        if (!(tol > 0)) return fail(ORBC_ERR_ARG, "cleanup: stray tolerance must be positive");
        const int mingen = 4;
        DevBuf<int> gone;
        DevBuf<double4a> gen;
        DevBuf<double> dr2;
        DevBuf<unsigned long long> cnt;
        CK(gen.alloc(size_t(npad)));
        CK(dr2.alloc(size_t(npad)));
        CK(gone.alloc(size_t(nhome)));
        CK(cnt.alloc(1));
        // the cells and ranges of the current positions
        launch_rebuild<R>(a, st, true);
        CK(cudaMemsetAsync(gone.p, 0, size_t(nhome) * sizeof(int), st));
        CK(cudaMemsetAsync(cnt.p, 0, sizeof(unsigned long long), st));
        CK(cudaMemsetAsync(gen.p, 0, size_t(npad) * sizeof(double4a), st));
        if (launch_cleanup_mark<R>(a, mingen, tol * tol, gen.p, dr2.p, gone.p, cnt.p, st))
            return fail(ORBC_ERR_CUDA, "cleanup: kernel launch failed");
        unsigned long long nrem = 0;
        CK(cudaMemcpyAsync(&nrem, cnt.p, sizeof(nrem), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        if (removed_out) *removed_out = int64_t(nrem);
        if (nrem == 0) return ORBC_OK;
        std::vector<int> hg(static_cast<size_t>(nhome)), newidx(static_cast<size_t>(nhome));
        CK(cudaMemcpy(hg.data(), gone.p, hg.size() * sizeof(int), cudaMemcpyDeviceToHost));
        // survivors keep their order (the reference compacts with a prefix sum)
        int64_t k = 0;
        std::vector<int64_t> offs(static_cast<size_t>(nsys) + 1, 0);
        std::vector<int> ntype, ntag;
        ntype.reserve(size_t(nhome));
        ntag.reserve(size_t(nhome));
        for (int sy = 0; sy < nsys; ++sy) {
            int gone_here = 0;
            for (int64_t h = topo.offsets[size_t(sy)]; h < topo.offsets[size_t(sy) + 1]; ++h) {
                if (hg[size_t(h)]) {
                    newidx[size_t(h)] = -1;
                    ++gone_here;
                    continue;
                }
                newidx[size_t(h)] = int(k++);
                ntype.push_back(topo.type[size_t(h)]);
                ntag.push_back(topo.tag[size_t(h)]);
            }
            offs[size_t(sy) + 1] = k;
            hsys[size_t(sy)].nreal -= gone_here;
            hsys[size_t(sy)].nlipid -= gone_here;
        }
        const int64_t nnew = k;
        CK(gone.alloc(size_t(nhome)));  // reused for the new numbering
        CK(cudaMemcpyAsync(gone.p, newidx.data(), newidx.size() * sizeof(int), cudaMemcpyHostToDevice, st));
        DevBuf<int> soh2;
        CK(soh2.alloc(size_t(std::max<int64_t>(nnew, 1))));
        launch_cleanup_apply<R>(a, gone.p, soh2.p, st);
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(sysd.p, hsys.data(), hsys.size() * sizeof(SysDev), cudaMemcpyHostToDevice, st));
        CK(cudaStreamSynchronize(st));
        std::swap(soh.p, soh2.p);
        std::swap(soh.n, soh2.n);
        a.slot_of_home = soh.p;
        topo.type.swap(ntype);
        topo.tag.swap(ntag);
        topo.offsets = offs;
        nhome = nnew;
        int rc = build_file_order(topo.type.data(), topo.tag.data(), nhome);
        if (rc) return rc;
        drop_graph();
        vcom_valid = false;
        return ORBC_OK;
    }

    int save_frame(const char *path, int append, int nstep, int fields, int real_bytes, int async) override {
        if (!uploaded) return fail(ORBC_ERR_STATE, "save_frame before upload");
        if (!path || (fields & ~31) || (real_bytes != 4 && real_bytes != 8))
            return fail(ORBC_ERR_ARG, "save_frame: need a path, fields within 0..31 and real_bytes 4 or 8");
        const size_t n = size_t(nhome), vec = 3 * n * size_t(real_bytes);
        // payload in file order: POSITION, VELOCITY, ROTATION, VORONOI, FORCE
        size_t off[5], bytes = 0;
        const int bits[5] = {1, 8, 2, 4, 16};
        for (int k = 0; k < 5; ++k) {
            off[k] = bytes;
            if (fields & bits[k]) bytes += k == 3 ? 4 * n : vec;
        }
        if (fields & 16) {
            // Nose-Hoover carries the forces of the current positions; otherwise evaluate them
            if (!(P.integrator == ORBC_INT_NOSE_HOOVER && nh_primed)) {
                launch_rebuild<R>(a, st, true);
                if (has_mesh) launch_mesh<R>(a, st);
                launch_forces<R>(a, st);
                nh_primed = false;
            }
        }
        std::string err;
        const int sl = fw.acquire(bytes, device, err);
        if (sl < 0) return fail(ORBC_ERR_NOMEM, err);
        if (fstage[sl].n < bytes) CK(fstage[sl].alloc(bytes));
        char *d = fstage[sl].p;
        auto at = [&](int k) -> void * { return (fields & bits[k]) ? d + off[k] : nullptr; };
        launch_frame_pack<R>(a, fmap.p, real_bytes, at(0), at(1), at(2), static_cast<int *>(at(3)), at(4), st);
        CK(cudaGetLastError());
        CK(cudaEventRecord(fpack[sl], st));
        CK(cudaStreamWaitEvent(cs, fpack[sl], 0));
        if (bytes) CK(cudaMemcpyAsync(fw.host(sl), d, bytes, cudaMemcpyDeviceToHost, cs));
        CK(cudaEventRecord(fw.event(sl), cs));
        FrameWriter::Job job;
        job.path = path;
        job.append = append != 0;
        job.nstep = nstep;
        job.fields = fields;
        job.real_bytes = real_bytes;
        job.natom = uint64_t(n);
        job.ident = ident;
        job.bytes = bytes;
        fw.submit(sl, std::move(job));
        if (!async) return flush_frames();
        return ORBC_OK;
    }

    int flush_frames() override {
        const std::string e = fw.flush();
        if (!e.empty()) return fail(ORBC_ERR_IO, e);
        return ORBC_OK;
    }

    /* Checkpoint: the caller-order state in FP64 plus everything a bitwise
     * continuation of the step needs beyond it -- step counter (the noise
     * counter), RNG key, per-system Nose-Hoover zeta and the carried forces
     * and torques of the Nose-Hoover step. */
    int save_checkpoint(const char *path) override {
        if (!uploaded) return fail(ORBC_ERR_STATE, "save_checkpoint before upload");
        if (!path) return fail(ORBC_ERR_ARG, "save_checkpoint: no path");
        const size_t m = size_t(nhome) * 3;
        std::vector<double> buf(6 * m);
        int rc = download(buf.data(), buf.data() + m, buf.data() + 2 * m, buf.data() + 3 * m);
        if (rc) return rc;
        const int carried = (P.integrator == ORBC_INT_NOSE_HOOVER && nh_primed) ? 1 : 0;
        if (carried) {
            double *dd = stage.p;
            launch_download<R>(a, 0, nhome, nullptr, nullptr, nullptr, nullptr, dd, dd + m, nullptr, st);
            CK(cudaGetLastError());
            CK(cudaMemcpyAsync(buf.data() + 4 * m, dd, 2 * m * sizeof(double), cudaMemcpyDeviceToHost, st));
        }
        std::vector<SysState> hss(static_cast<size_t>(nsys));
        Scalars hs;
        CK(cudaMemcpyAsync(hss.data(), ssd.p, hss.size() * sizeof(SysState), cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(&hs, Sd.p, sizeof(Scalars), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        FILE *f = std::fopen(path, "wb");
        if (!f) return fail(ORBC_ERR_IO, std::string("save_checkpoint: cannot open ") + path);
        const char magic[8] = {'O', 'R', 'B', 'C', 'C', 'K', 'P', 'T'};
        const int32_t hdr[4] = {1, P.precision, nsys, carried};
        const int64_t counts[2] = {nhome, int64_t(hs.step)};
        const uint64_t seed = P.seed;
        bool ok = std::fwrite(magic, 1, 8, f) == 8 && std::fwrite(hdr, 4, 4, f) == 4 &&
                  std::fwrite(counts, 8, 2, f) == 2 && std::fwrite(&seed, 8, 1, f) == 1;
        for (int k = 0; ok && k < nsys; ++k) ok = std::fwrite(&hss[size_t(k)].zeta, 8, 1, f) == 1;
        const size_t nd = (carried ? 6 : 4) * m;
        ok = ok && std::fwrite(buf.data(), sizeof(double), nd, f) == nd;
        if (std::fclose(f) != 0 || !ok) return fail(ORBC_ERR_IO, std::string("save_checkpoint: write failed: ") + path);
        return ORBC_OK;
    }

    int load_checkpoint(const char *path) override {
        if (!uploaded) return fail(ORBC_ERR_STATE, "load_checkpoint before upload (the topology comes from upload)");
        if (!path) return fail(ORBC_ERR_ARG, "load_checkpoint: no path");
        FILE *f = std::fopen(path, "rb");
        if (!f) return fail(ORBC_ERR_IO, std::string("load_checkpoint: cannot open ") + path);
        char magic[8];
        int32_t hdr[4];
        int64_t counts[2];
        uint64_t seed;
        bool ok = std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, "ORBCCKPT", 8) == 0 &&
                  std::fread(hdr, 4, 4, f) == 4 && std::fread(counts, 8, 2, f) == 2 && std::fread(&seed, 8, 1, f) == 1;
        if (!ok || hdr[0] != 1 || hdr[2] != nsys || counts[0] != nhome) {
            std::fclose(f);
            return fail(ORBC_ERR_ARG, "load_checkpoint: not a checkpoint of this topology (particles / systems differ)");
        }
        const int carried = hdr[3];
        std::vector<double> zeta(static_cast<size_t>(nsys));
        const size_t m = size_t(nhome) * 3, nd = (carried ? 6 : 4) * m;
        std::vector<double> buf(nd);
        ok = std::fread(zeta.data(), 8, zeta.size(), f) == zeta.size() && std::fread(buf.data(), 8, nd, f) == nd;
        std::fclose(f);
        if (!ok) return fail(ORBC_ERR_IO, std::string("load_checkpoint: truncated file ") + path);
        int rc = set_state(buf.data(), buf.data() + m, buf.data() + 2 * m, buf.data() + 3 * m);
        if (rc) return rc;
        std::vector<SysState> hss(static_cast<size_t>(nsys));
        CK(cudaMemcpyAsync(hss.data(), ssd.p, hss.size() * sizeof(SysState), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        for (int k = 0; k < nsys; ++k) hss[size_t(k)].zeta = zeta[size_t(k)];
        CK(cudaMemcpyAsync(ssd.p, hss.data(), hss.size() * sizeof(SysState), cudaMemcpyHostToDevice, st));
        const long long stepv = counts[1];
        CK(cudaMemcpyAsync(&Sd.p->step, &stepv, sizeof(stepv), cudaMemcpyHostToDevice, st));
        P.seed = seed;
        a.seed = seed;
        drop_graph();  // the captured graph holds the kernel arguments (seed)
        if (carried && P.integrator == ORBC_INT_NOSE_HOOVER) {
            double *dd = stage.p;
            CK(cudaMemcpyAsync(dd, buf.data() + 4 * m, 2 * m * sizeof(double), cudaMemcpyHostToDevice, st));
            launch_set_carried<R>(a, dd, dd + m, nhome, st);
            CK(cudaGetLastError());
            nh_primed = true;
        }
        CK(cudaStreamSynchronize(st));
        return ORBC_OK;
    }

    int assign_temperature(double kT, uint64_t seed) override {
        if (!uploaded) return fail(ORBC_ERR_STATE, "assign_temperature before upload");
        if (!(kT >= 0)) return fail(ORBC_ERR_ARG, "assign_temperature: kT must be >= 0");
        launch_assign_temperature<R>(a, kT, seed, st);
        launch_vcom<R>(a, st);  // temperature and lipid mean of the new velocities
        CK(cudaGetLastError());
        CK(cudaStreamSynchronize(st));
        nh_primed = false;
        vcom_valid = true;
        return ORBC_OK;
    }

    /* --------------------------------------------------------------------- */
    void enqueue_step(bool gated_rebuild) {
        if (P.integrator == ORBC_INT_NOSE_HOOVER) {
            launch_nh_initial<R>(a, st);
            launch_rebuild<R>(a, st, gated_rebuild);
            if (has_mesh) launch_mesh<R>(a, st);
            launch_nh_final<R>(a, st, P.energy != 0);
        } else {
            launch_rebuild<R>(a, st, gated_rebuild);
            if (has_mesh) launch_mesh<R>(a, st);
            launch_step_langevin<R>(a, st, P.energy != 0);
        }
    }
    /* Langevin without energy or bulk-velocity removal: no per-step sums */
    bool lite() const { return P.integrator == ORBC_INT_LANGEVIN && !P.energy && !P.zero_bulk; }
    /* per step: the force kernel and k_advance (lite) or k_reduce; Nose-Hoover
     * adds k_nh_initial and its k_reduce; the mesh kernel; the condition kernel */
    int fixed_launches_per_step() const {
        int k = (P.integrator == ORBC_INT_NOSE_HOOVER ? 4 : 2) + (has_mesh ? 1 : 0);
        return k + (graph_cond ? 1 : 0);
    }
    int rebuild_launches() const { return 1 + 3 * passes + 1 + 1; }

    /* Capture steps_per_graph steps into *exec (cond: the rebuild sits behind
     * a conditional node; otherwise the rebuild kernels are device-gated). */
    int capture_graph(int steps_per_graph, cudaGraphExec_t *exec, bool *cond) {
        cudaGraphExec_t gexec = nullptr;
        cudaGraph_t g = nullptr;
        // conditional rebuild: [pre] -> set_cond -> IF{rebuild} -> [mesh] -> step kernel
        bool ok = cudaGraphCreate(&g, 0) == cudaSuccess;
        std::vector<cudaGraph_t> bodies;
        if (ok) {
            ok = cudaStreamBeginCaptureToGraph(st, g, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal) ==
                 cudaSuccess;
            for (int k = 0; ok && k < steps_per_graph; ++k) {
                cudaGraphConditionalHandle hc;
                if (cudaGraphConditionalHandleCreate(&hc, g, 0, 0) != cudaSuccess) {
                    ok = false;
                    break;
                }
                if (P.integrator == ORBC_INT_NOSE_HOOVER) launch_nh_initial<R>(a, st);
                launch_set_cond(hc, a.S, st);
                cudaStreamCaptureStatus cst;
                cudaGraph_t cg;
                const cudaGraphNode_t *deps = nullptr;
                size_t nd = 0;
                if (cudaStreamGetCaptureInfo(st, &cst, nullptr, &cg, &deps, nullptr, &nd) != cudaSuccess) {
                    ok = false;
                    break;
                }
                cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};
                cp.conditional.handle = hc;
                cp.conditional.type = cudaGraphCondTypeIf;
                cp.conditional.size = 1;
                cudaGraphNode_t cn;
                if (cudaGraphAddNode(&cn, cg, deps, nullptr, nd, &cp) != cudaSuccess) {
                    ok = false;
                    break;
                }
                bodies.push_back(cp.conditional.phGraph_out[0]);
                if (cudaStreamUpdateCaptureDependencies(st, &cn, nullptr, 1, cudaStreamSetCaptureDependencies) !=
                    cudaSuccess) {
                    ok = false;
                    break;
                }
                if (has_mesh) launch_mesh<R>(a, st);
                if (P.integrator == ORBC_INT_NOSE_HOOVER)
                    launch_nh_final<R>(a, st, P.energy != 0);
                else
                    launch_step_langevin<R>(a, st, P.energy != 0);
            }
            cudaGraph_t out = nullptr;
            cudaError_t e = cudaStreamEndCapture(st, &out);
            ok = ok && e == cudaSuccess;
            for (size_t k = 0; ok && k < bodies.size(); ++k) {
                ok = cudaStreamBeginCaptureToGraph(st, bodies[k], nullptr, nullptr, 0,
                                                   cudaStreamCaptureModeThreadLocal) == cudaSuccess;
                if (!ok) break;
                launch_rebuild<R>(a, st, false);
                cudaGraph_t b2 = nullptr;
                ok = cudaStreamEndCapture(st, &b2) == cudaSuccess;
            }
            if (ok) ok = cudaGraphInstantiate(&gexec, g, 0) == cudaSuccess;
        }
        cudaGetLastError();
        if (g) cudaGraphDestroy(g);
        if (ok) {
            *exec = gexec;
            *cond = true;
            return ORBC_OK;
        }
        // fallback: plain capture with device-gated rebuild kernels
        if (gexec) cudaGraphExecDestroy(gexec);
        gexec = nullptr;
        cudaStreamCaptureStatus cst;
        if (cudaStreamIsCapturing(st, &cst) == cudaSuccess && cst != cudaStreamCaptureStatusNone) {
            cudaGraph_t junk;
            cudaStreamEndCapture(st, &junk);
            if (junk) cudaGraphDestroy(junk);
        }
        cudaGetLastError();
        g = nullptr;
        CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        for (int k = 0; k < steps_per_graph; ++k) enqueue_step(true);
        CK(cudaStreamEndCapture(st, &g));
        CK(cudaGraphInstantiate(&gexec, g, 0));
        cudaGraphDestroy(g);
        *exec = gexec;
        *cond = false;
        return ORBC_OK;
    }

    int step(int nsteps, orbc_thermo *out) override {
        if (!uploaded) return fail(ORBC_ERR_STATE, "step before upload");
        if (nsteps < 0) return fail(ORBC_ERR_ARG, "step: negative step count");
        const int G = 4;  // steps per graph launch; single steps use a one-step graph
        if (P.use_graph && nsteps > 0) {
            if (!gexec) {
                int rc = capture_graph(G, &gexec, &graph_cond);
                if (rc) return rc;
                graph_steps = G;
            }
            if (nsteps % G && !gexec1) {
                bool c1 = false;
                int rc = capture_graph(1, &gexec1, &c1);
                if (rc) return rc;
            }
        }
        // the counters before and after come back through pinned memory, with
        // one wait at the end of the call
        CK(cudaMemcpyAsync(&hsc[0], Sd.p, sizeof(Scalars), cudaMemcpyDeviceToHost, st));
        int64_t extra = 0;
        if (P.zero_bulk && P.integrator == ORBC_INT_LANGEVIN && !vcom_valid) {
            launch_vcom<R>(a, st);
            CK(cudaGetLastError());
            vcom_valid = true;
            extra += 2;  // k_vcom + k_reduce
        }
        if (P.integrator == ORBC_INT_NOSE_HOOVER && !nh_primed) {
            launch_rebuild<R>(a, st, true);
            if (has_mesh) launch_mesh<R>(a, st);
            launch_nh_prologue<R>(a, st);
            CK(cudaGetLastError());
            nh_primed = true;
            extra += rebuild_launches() + (has_mesh ? 1 : 0) + 2;  // gated rebuild, mesh, k_nh_final + k_reduce
        }
        CK(cudaEventRecord(ev0, st));
        if (P.use_graph && nsteps > 0) {
            int k = 0;
            for (; k + graph_steps <= nsteps; k += graph_steps) CK(cudaGraphLaunch(gexec, st));
            for (; k < nsteps; ++k) CK(cudaGraphLaunch(gexec1, st));
        } else {
            for (int k = 0; k < nsteps; ++k) enqueue_step(true);
        }
        CK(cudaGetLastError());
        CK(cudaEventRecord(ev1, st));
        CK(cudaMemcpyAsync(&hsc[1], Sd.p, sizeof(Scalars), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        float ms = 0;
        CK(cudaEventElapsedTime(&ms, ev0, ev1));
        last_ms = ms;
        const Scalars before = hsc[0], hs = hsc[1];
        const int64_t nreb = hs.rebuilds - before.rebuilds;
        const int per_step = P.use_graph && gexec ? fixed_launches_per_step() : (fixed_launches_per_step() - (graph_cond ? 1 : 0) + rebuild_launches());
        last_launches = extra + int64_t(nsteps) * per_step + (P.use_graph && graph_cond ? nreb * rebuild_launches() : 0);
        if (out) {
            int rc = thermo(-1, out);
            if (rc) return rc;
        }
        if (hs.error & (ERRB_NBR_OVERFLOW | ERRB_GRID)) {
            /* A list build inside the call halted the steps (a list
             * overflowed, or a particle left an open grid): the steps after it
             * left the state untouched.  Grow the list or re-grid, rebuild
             * from the current state, finish the interrupted Nose-Hoover step
             * if its first half ran, and run the steps that remain. */
            if (overflow_depth >= 4) return fail(ORBC_ERR_NBR_OVERFLOW, "step: neighbour capacity could not be sized");
            int rc = recover(hs);
            if (rc) return rc;
            int remaining = nsteps - int(hs.iters - before.iters);
            if (P.integrator == ORBC_INT_NOSE_HOOVER) {
                if (hs.nh_half) {  // the second half of the interrupted step (it also carries the forces)
                    if (has_mesh) launch_mesh<R>(a, st);
                    launch_nh_final<R>(a, st, P.energy != 0);
                    CK(cudaGetLastError());
                    nh_primed = true;
                    --remaining;
                } else {
                    nh_primed = false;  // the overflow hit the prologue's build: prime again
                }
            }
            ++overflow_depth;
            rc = step(std::max(remaining, 0), out);
            --overflow_depth;
            return rc;
        }
        // keep headroom in the neighbour capacity
        if (hs.max_nnb > cap * 0.85) {
            int rc = grow_capacity(hs.max_nnb);
            if (rc) return rc;
        }
        const int code = err_code_of(hs.error);
        if (code) return fail(code, "step: device reported error bits " + std::to_string(hs.error));
        return ORBC_OK;
    }
    int overflow_depth = 0;

    int download(double *x3, double *n3, double *v3, double *o3) override {
        if (!uploaded) return fail(ORBC_ERR_STATE, "download before upload");
        return download_t<double>(0, nhome, 3, x3, n3, v3, o3);
    }
    int download_f32(int64_t first, int64_t count, int stride, float *x, float *n, float *v, float *o) override {
        if (!uploaded) return fail(ORBC_ERR_STATE, "download before upload");
        if (first < 0 || count < 0 || first + count > nhome || (stride != 3 && stride != 4))
            return fail(ORBC_ERR_ARG, "download_f32: need 0 <= first, first + count <= n and stride 3 or 4");
        if (count == 0) return ORBC_OK;
        return download_t<float>(first, count, stride, x, n, v, o);
    }
    /* upload indices [first, first + count) to host AoS arrays of TH; chunked:
     * the copy stream moves chunk c to the host while the step stream converts
     * chunk c + 1 */
    template<class TH> int download_t(int64_t first, int64_t count, int stride, TH *x, TH *n, TH *v, TH *o) {
        if ((x || n || v || o) && (!x || host_reachable(x)) && (!n || host_reachable(n)) &&
            (!v || host_reachable(v)) && (!o || host_reachable(o))) {
            // the conversion kernel writes the caller's arrays over the host link
            launch_download_host<R, TH>(a, first, first + count, first, stride, x, n, v, o, st);
            CK(cudaGetLastError());
            CK(cudaStreamSynchronize(st));
            ++direct_transfers;
            return ORBC_OK;
        }
        TH *d = reinterpret_cast<TH *>(stage.p);
        const int64_t m = count * stride;
        TH *dst[4] = {x, n, v, o};
        const int nch = count >= (int64_t(1) << 20) ? NXCH : 1;
        for (int c = 0; c < nch; ++c) {
            const int64_t h0 = count * c / nch, h1 = count * (c + 1) / nch;
            launch_download<R, TH>(a, first + h0, first + h1, first, stride, x ? d : nullptr, n ? d + m : nullptr,
                                   v ? d + 2 * m : nullptr, o ? d + 3 * m : nullptr, nullptr, nullptr, nullptr, st);
            CK(cudaGetLastError());
            CK(cudaEventRecord(xev[c], st));
            CK(cudaStreamWaitEvent(cs, xev[c], 0));
            for (int q = 0; q < 4; ++q)
                if (dst[q])
                    CK(cudaMemcpyAsync(dst[q] + h0 * stride, d + m * q + h0 * stride,
                                       size_t(h1 - h0) * stride * sizeof(TH), cudaMemcpyDeviceToHost, cs));
        }
        CK(cudaStreamSynchronize(cs));
        return ORBC_OK;
    }

    int forces(double *f3, double *t3, double *e) override {
        if (!uploaded) return fail(ORBC_ERR_STATE, "forces before upload");
        Scalars hs;
        for (int attempt = 0;; ++attempt) {
            launch_rebuild<R>(a, st, true);
            if (has_mesh) launch_mesh<R>(a, st);
            launch_forces<R>(a, st);
            CK(cudaGetLastError());
            CK(cudaMemcpyAsync(&hsc[0], Sd.p, sizeof(Scalars), cudaMemcpyDeviceToHost, st));
            CK(cudaStreamSynchronize(st));
            hs = hsc[0];
            if (!(hs.error & (ERRB_NBR_OVERFLOW | ERRB_GRID))) break;
            if (attempt == 4) return fail(ORBC_ERR_NBR_OVERFLOW, "forces: neighbour capacity could not be sized");
            const int rc = recover(hs);  // the forces kernel did nothing: grow, rebuild, again
            if (rc) return rc;
        }
        double *d = stage.p;
        const size_t m = size_t(nhome) * 3;
        launch_download<R>(a, 0, nhome, nullptr, nullptr, nullptr, nullptr, d, d + m, d + 2 * m, st);
        CK(cudaGetLastError());
        if (f3) CK(cudaMemcpyAsync(f3, d, m * sizeof(double), cudaMemcpyDeviceToHost, st));
        if (t3) CK(cudaMemcpyAsync(t3, d + m, m * sizeof(double), cudaMemcpyDeviceToHost, st));
        if (e) CK(cudaMemcpyAsync(e, d + 2 * m, size_t(nhome) * sizeof(double), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        // the forces kernel overwrote the carried Nose-Hoover forces
        nh_primed = false;
        const int code = err_code_of(hs.error);
        if (code) return fail(code, "forces: device reported error bits " + std::to_string(hs.error));
        return ORBC_OK;
    }

    int thermo(int s, orbc_thermo *out) override {
        if (!uploaded) return fail(ORBC_ERR_STATE, "thermo before upload");
        if (s >= nsys) return fail(ORBC_ERR_ARG, "thermo: no such system");
        // area / volume of the current state (recomputing them is idempotent:
        // the next step's mesh kernel sees the same positions)
        if (has_mesh) {
            launch_mesh<R>(a, st);
            CK(cudaGetLastError());
        }
        // the lite Langevin step keeps no per-step sums: reduce sum m v^2 now
        if (lite()) {
            launch_vcom<R>(a, st);
            CK(cudaGetLastError());
        }
        std::vector<SysState> hss(static_cast<size_t>(nsys));
        Scalars hs;
        CK(cudaMemcpyAsync(hss.data(), ssd.p, hss.size() * sizeof(SysState), cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(&hs, Sd.p, sizeof(Scalars), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        std::memset(out, 0, sizeof(*out));
        double ke = 0, ep = 0;
        int64_t nn = 0;
        for (int k = 0; k < nsys; ++k) {
            if (s >= 0 && k != s) continue;
            const double half = P.integrator == ORBC_INT_NOSE_HOOVER ? 1.0 : 1.0;
            ke += hss[size_t(k)].ke2 * half;
            ep += hss[size_t(k)].epot;
            nn += hsys[size_t(k)].nreal;
        }
        const int k0 = s >= 0 ? s : 0;
        out->step = hs.step;
        out->n = nn;
        out->ke2 = ke;
        out->temperature = nn ? ke / (3.0 * double(nn)) : 0;
        out->epot = ep;
        out->area = hss[size_t(k0)].area;
        out->volume = hss[size_t(k0)].volume;
        out->zeta = hss[size_t(k0)].zeta;
        out->rebuilds = hs.rebuilds;
        out->max_neighbors = hs.max_nnb;
        out->capacity = cap;
        out->flags = flag_bits(hs.error);
        return ORBC_OK;
    }

    int neighbors(int *counts_o, int *list, int64_t capl, int64_t *total) override {
        if (!uploaded) return fail(ORBC_ERR_STATE, "neighbors before upload");
        launch_rebuild<R>(a, st, true);
        CK(cudaGetLastError());
        std::vector<int> hn(static_cast<size_t>(npad)), hh(static_cast<size_t>(npad));
        std::vector<uint32_t> hl(size_t(cap) * size_t(npad));
        Scalars hs;
        CK(cudaMemcpyAsync(&hs, Sd.p, sizeof(Scalars), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        CK(cudaMemcpy(hn.data(), nnb.p, hn.size() * sizeof(int), cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(hh.data(), home[hs.lp].p, hh.size() * sizeof(int), cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(hl.data(), nbr.p, hl.size() * sizeof(uint32_t), cudaMemcpyDeviceToHost));
        std::vector<std::vector<int>> per(static_cast<size_t>(nhome));
        for (int p = 0; p < npad; ++p) {
            const int h = hh[size_t(p)];
            if (h < 0) continue;
            const int nin = hn[size_t(p)] & 0xffff, nout = hn[size_t(p)] >> 16;
            for (int k = 0; k < nin + nout; ++k) {
                const int row = k < nin ? k : cap - 1 - (k - nin);
                const uint32_t ent = hl[size_t(nbr_index(p, row, cap))];
                per[size_t(h)].push_back(hh[size_t(ent & NB_MASK)]);
            }
            std::sort(per[size_t(h)].begin(), per[size_t(h)].end());
        }
        int64_t tot = 0;
        for (int64_t i = 0; i < nhome; ++i) {
            if (counts_o) counts_o[i] = int(per[size_t(i)].size());
            for (int j : per[size_t(i)]) {
                if (list && tot < capl) list[tot] = j;
                ++tot;
            }
        }
        if (total) *total = tot;
        return ORBC_OK;
    }

    int cells(int s, double *lo3, double *lc3, int *nc3, int *cello, double *off3, int *slot) override {
        if (!uploaded) return fail(ORBC_ERR_STATE, "cells before upload");
        if (s < 0 || s >= nsys) return fail(ORBC_ERR_ARG, "cells: no such system");
        const SysDev &sd = hsys[size_t(s)];
        for (int d = 0; d < 3; ++d) {
            if (lo3) lo3[d] = sd.lo[d];
            if (lc3) lc3[d] = sd.Lc[d];
            if (nc3) nc3[d] = sd.nc[d];
        }
        Scalars hs;
        CK(cudaMemcpyAsync(&hs, Sd.p, sizeof(Scalars), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        std::vector<int> hc(static_cast<size_t>(npad)), hh(static_cast<size_t>(npad));
        std::vector<T4> hp(static_cast<size_t>(npad));
        CK(cudaMemcpy(hc.data(), cell[hs.lp].p, hc.size() * sizeof(int), cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(hh.data(), home[hs.lp].p, hh.size() * sizeof(int), cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(hp.data(), pos[hs.cur].p, hp.size() * sizeof(T4), cudaMemcpyDeviceToHost));
        for (int p = 0; p < npad; ++p) {
            const int h = hh[size_t(p)];
            if (h < 0) continue;
            if (cello) cello[h] = hc[size_t(p)];
            if (off3) {
                off3[3 * int64_t(h)] = double(hp[size_t(p)].x);
                off3[3 * int64_t(h) + 1] = double(hp[size_t(p)].y);
                off3[3 * int64_t(h) + 2] = double(hp[size_t(p)].z);
            }
            if (slot) slot[h] = p;
        }
        return ORBC_OK;
    }

    int rebuild() override {
        if (!uploaded) return fail(ORBC_ERR_STATE, "rebuild before upload");
        return build_lists(false);
    }

    int rdf(int s, int ta, int tb, double dr, int nbins, double rcut, uint64_t *counts, int64_t *dropped) override {
        if (!uploaded) return fail(ORBC_ERR_STATE, "rdf before upload");
        if (s < 0 || s >= nsys) return fail(ORBC_ERR_ARG, "rdf: no such system");
        if (!(dr > 0) || nbins < 1 || nbins > (1 << 24) || !counts || ta < -1 || ta >= NT || tb < -1 || tb >= NT)
            return fail(ORBC_ERR_ARG, "rdf: need dr > 0, 1 <= nbins <= 2^24, types in -1..5 and a counts array");
        const int64_t b = topo.offsets[size_t(s)], e = topo.offsets[size_t(s) + 1];
        const int n = int(e - b);
        const orbc_system_desc &d = topo.descs[size_t(s)];
        double centre[3], L[3];
        for (int k = 0; k < 3; ++k) {
            centre[k] = 0.5 * (d.lo[k] + d.hi[k]);
            L[k] = d.periodic[k] ? d.hi[k] - d.lo[k] : 0.0;
        }
        launch_download<R>(a, 0, nhome, stage.p, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, st);
        CK(cudaGetLastError());
        DevBuf<int> td;
        DevBuf<T4> work;
        DevBuf<unsigned long long> cnt;
        CK(td.alloc(size_t(n)));
        CK(work.alloc(size_t(n)));
        CK(cnt.alloc(size_t(nbins) + 1));
        CK(cudaMemcpyAsync(td.p, topo.type.data() + b, size_t(n) * sizeof(int), cudaMemcpyHostToDevice, st));
        CK(cudaMemsetAsync(cnt.p, 0, (size_t(nbins) + 1) * sizeof(unsigned long long), st));
        CK(launch_rdf<R>(stage.p + 3 * b, td.p, n, centre, L, ta, tb, dr, nbins, rcut, cnt.p, cnt.p + nbins, work.p,
                         st));
        std::vector<unsigned long long> h(size_t(nbins) + 1);
        CK(cudaMemcpyAsync(h.data(), cnt.p, h.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        for (int k = 0; k < nbins; ++k) counts[k] = uint64_t(h[size_t(k)]);
        if (dropped) *dropped = int64_t(h[size_t(nbins)]);
        return ORBC_OK;
    }

    int profile(int nsteps, orbc_profile *out) override {
        if (!uploaded) return fail(ORBC_ERR_STATE, "profile before upload");
        if (nsteps < 1 || !out) return fail(ORBC_ERR_ARG, "profile: need nsteps >= 1");
        std::memset(out, 0, sizeof(*out));
        if (P.integrator == ORBC_INT_NOSE_HOOVER && !nh_primed) {
            int rc = step(0, nullptr);
            if (rc) return rc;
        }
        cudaEvent_t ev[5], er[5];
        for (auto &e : ev) CK(cudaEventCreate(&e));
        for (auto &e : er) CK(cudaEventCreate(&e));
        double t_step = 0, t_reb = 0, t_gate = 0, t_mesh = 0, t_stage[4] = {0, 0, 0, 0};
        int64_t nreb = 0;
        for (int k = 0; k < nsteps; ++k) {
            Scalars b4;
            CK(cudaMemcpy(&b4, Sd.p, sizeof(Scalars), cudaMemcpyDeviceToHost));
            CK(cudaEventRecord(ev[0], st));
            if (P.integrator == ORBC_INT_NOSE_HOOVER) launch_nh_initial<R>(a, st);
            CK(cudaEventRecord(ev[1], st));
            for (int g = 0; g < 4; ++g) {
                CK(cudaEventRecord(er[g], st));
                launch_rebuild_stage<R>(a, st, true, g);
            }
            CK(cudaEventRecord(er[4], st));
            CK(cudaEventRecord(ev[2], st));
            if (has_mesh) launch_mesh<R>(a, st);
            CK(cudaEventRecord(ev[3], st));
            if (P.integrator == ORBC_INT_NOSE_HOOVER)
                launch_nh_final<R>(a, st, P.energy != 0);
            else
                launch_step_langevin<R>(a, st, P.energy != 0);
            CK(cudaEventRecord(ev[4], st));
            CK(cudaEventSynchronize(ev[4]));
            CK(cudaGetLastError());
            float m01, m12, m23, m34;
            CK(cudaEventElapsedTime(&m01, ev[0], ev[1]));
            CK(cudaEventElapsedTime(&m12, ev[1], ev[2]));
            CK(cudaEventElapsedTime(&m23, ev[2], ev[3]));
            CK(cudaEventElapsedTime(&m34, ev[3], ev[4]));
            Scalars af;
            CK(cudaMemcpy(&af, Sd.p, sizeof(Scalars), cudaMemcpyDeviceToHost));
            if (af.rebuilds > b4.rebuilds) {
                t_reb += m12;
                ++nreb;
                for (int g = 0; g < 4; ++g) {
                    float mg;
                    CK(cudaEventElapsedTime(&mg, er[g], er[g + 1]));
                    t_stage[g] += mg;
                }
            } else {
                t_gate += m12;
            }
            t_mesh += m23;
            t_step += m34 + m01;
        }
        for (auto &e : er) cudaEventDestroy(e);
        for (auto &e : ev) cudaEventDestroy(e);
        out->steps = nsteps;
        out->rebuilds = nreb;
        out->step_kernel_ms = t_step / nsteps;
        out->rebuild_ms = nreb ? t_reb / nreb : 0.0;
        out->gate_ms = nsteps > nreb ? t_gate / double(nsteps - nreb) : 0.0;
        out->mesh_ms = t_mesh / nsteps;
        out->rebin_ms = nreb ? t_stage[0] / nreb : 0.0;
        out->sort_ms = nreb ? t_stage[1] / nreb : 0.0;
        out->gather_ms = nreb ? t_stage[2] / nreb : 0.0;
        out->nlist_ms = nreb ? t_stage[3] / nreb : 0.0;
        // neighbour statistics of the current list
        Scalars hs;
        CK(cudaMemcpy(&hs, Sd.p, sizeof(Scalars), cudaMemcpyDeviceToHost));
        std::vector<int> hn(static_cast<size_t>(npad)), hh(static_cast<size_t>(npad));
        CK(cudaMemcpy(hn.data(), nnb.p, hn.size() * sizeof(int), cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(hh.data(), home[hs.lp].p, hh.size() * sizeof(int), cudaMemcpyDeviceToHost));
        double tot = 0, tin = 0;
        int64_t cnt = 0;
        for (int p = 0; p < npad; ++p)
            if (hh[size_t(p)] >= 0) {
                tot += (hn[size_t(p)] & 0xffff) + (hn[size_t(p)] >> 16);
                tin += hn[size_t(p)] & 0xffff;
                ++cnt;
            }
        out->mean_neighbors = cnt ? tot / double(cnt) : 0.0;
        out->pairs_in_cutoff = cnt ? tin / double(cnt) : 0.0;  // inner entries at the last build
        return ORBC_OK;
    }

    /* Pick the neighbour-list skin and the force-kernel form by timing short
     * trials from one snapshot of the state; the snapshot (positions,
     * orientations, velocities, angular velocities, step counter, thermostat)
     * is restored afterwards, so tuning does not advance the simulation. */
    int autotune(int trial_steps, orbc_tune_trial *trials, int max_trials, int *ntrials) override {
        if (!uploaded) return fail(ORBC_ERR_STATE, "autotune before upload");
        if (trial_steps < 1) return fail(ORBC_ERR_ARG, "autotune: need trial_steps >= 1");
        const size_t m = size_t(nhome) * 3;
        std::vector<double> x(m), nv(m), v(m), o(m);
        int rc = download(x.data(), nv.data(), v.data(), o.data());
        if (rc) return rc;
        Scalars hs;
        CK(cudaMemcpy(&hs, Sd.p, sizeof(Scalars), cudaMemcpyDeviceToHost));
        std::vector<SysState> hss(topo.descs.size());
        CK(cudaMemcpy(hss.data(), ssd.p, hss.size() * sizeof(SysState), cudaMemcpyDeviceToHost));
        for (size_t k = 0; k < hss.size(); ++k) topo.descs[k].zeta = hss[k].zeta;
        const double skins[] = {0.3, 0.45, 0.6, 0.8, 1.0};
        double best_ms = 1e300, best_skin = P.skin;
        int best_var = P.kernel_variant, best_every = P.rebuild_every, nt = 0;
        const int keep = P.kernel_variant & 64;  // compensated accumulation: the caller's accuracy choice
        auto trial = [&](double sk, int var, int every) -> int {
            P.skin = sk;
            P.kernel_variant = var | keep;
            P.rebuild_every = every;
            int r = relayout(x, nv, v, o, hs.step);
            if (r) return r;
            r = step(3, nullptr);  // warm: builds the graph
            if (r) return r;
            Scalars b4;
            CK(cudaMemcpy(&b4, Sd.p, sizeof(Scalars), cudaMemcpyDeviceToHost));
            r = step(trial_steps, nullptr);
            if (r) return r;
            Scalars af;
            CK(cudaMemcpy(&af, Sd.p, sizeof(Scalars), cudaMemcpyDeviceToHost));
            const double ms = last_ms / trial_steps;
            if (trials && nt < max_trials) {
                trials[nt].skin = sk;
                trials[nt].variant = var | keep;
                trials[nt].rebuild_every = every;
                trials[nt].ms_per_step = ms;
                trials[nt].rebuilds_per_step = double(af.rebuilds - b4.rebuilds) / trial_steps;
            }
            ++nt;
            if (ms < best_ms) {
                best_ms = ms;
                best_skin = sk;
                best_var = var | keep;
                best_every = every;
            }
            return ORBC_OK;
        };
        // the list-build form first (bits 3-4, at the caller's skin and the
        // pipelined, inlined loop); then skin x force-loop form (bits 0-1, and
        // the merged shell pass) with it; the skins half-way to the best one's
        // grid neighbours; at the best pair the occupancy form (bit 2), the
        // other list-build forms and two fixed rebuild cadences
        const int occ0 = P.kernel_variant & 4, every0 = P.rebuild_every;
        const double skin0 = P.skin;
        for (int f = 0; f < 3; ++f)
            if ((rc = trial(skin0, 3 | occ0 | (f << 3), every0))) return rc;
        const int rest = (best_var & 24) | occ0;
        const int loops[] = {0, 1, 2, 3, 3 | 32};
        for (double sk : skins)
            for (int lf : loops)
                if ((rc = trial(sk, lf | rest, every0))) return rc;
        const int nsk = int(sizeof(skins) / sizeof(skins[0]));
        int bi = 0;
        while (bi + 1 < nsk && skins[bi] != best_skin) ++bi;
        const double lo_sk = 0.5 * (skins[bi > 0 ? bi - 1 : 0] + best_skin);
        const double hi_sk = 0.5 * (skins[bi + 1 < nsk ? bi + 1 : nsk - 1] + best_skin);
        const int bv = best_var & ~64;
        if ((rc = trial(lo_sk, bv, every0))) return rc;
        if ((rc = trial(hi_sk, bv, every0))) return rc;
        if ((rc = trial(best_skin, (best_var & ~64) ^ 4, every0))) return rc;
        const int lf = (best_var >> 3) & 3;
        for (int f = 0; f < 3; ++f)
            if (f != lf && (rc = trial(best_skin, (best_var & (7 | 32)) | (f << 3), every0))) return rc;
        for (int every : {5, 10})
            if (every != every0 && (rc = trial(best_skin, best_var & ~64, every))) return rc;
        if (ntrials) *ntrials = nt;
        P.skin = best_skin;
        P.kernel_variant = best_var;
        P.rebuild_every = best_every;
        return relayout(x, nv, v, o, hs.step);
    }

   private:
    struct Topology {
        std::vector<orbc_system_desc> descs;
        std::vector<int64_t> offsets;
        std::vector<int> type, tag, bonds, faces;
        std::vector<double> bond_r0;
    } topo;
    bool relayout_in_progress = false;

    /* Rebuild the whole device layout for the current parameters from a host
     * snapshot of the state, then restore the step counter. */
    int relayout(const std::vector<double> &x, const std::vector<double> &nv, const std::vector<double> &v,
                 const std::vector<double> &o, long long step_counter) {
        relayout_in_progress = true;
        const size_t nb = topo.bonds.size() / 3, nf = topo.faces.size() / 3;
        int rc = upload(int(topo.descs.size()), topo.descs.data(), topo.offsets.data(), x.data(), nv.data(), v.data(),
                        o.data(), topo.type.data(), topo.tag.data(), topo.type.size(),
                        nb ? topo.bonds.data() : nullptr, topo.bond_r0.empty() ? nullptr : topo.bond_r0.data(), nb,
                        nf ? topo.faces.data() : nullptr, nf);
        relayout_in_progress = false;
        if (rc) return rc;
        CK(cudaMemcpy(&Sd.p->step, &step_counter, sizeof(step_counter), cudaMemcpyHostToDevice));
        return ORBC_OK;
    }

    static T4 mk4(R x, R y, R z) {
        T4 v;
        v.x = x;
        v.y = y;
        v.z = z;
        v.w = R(0);
        return v;
    }
    static void setw(float4 &v, int w) { std::memcpy(&v.w, &w, 4); }
    static void setw(double4a &v, int w) {
        long long b = (long long)(unsigned)w;
        std::memcpy(&v.w, &b, 8);
    }
    /* cell of a point and its offset from the cell centre (same formula as k_set_state) */
    static void bin_point(const SysDev &sd, const double *x, int cc[3], double o[3]) {
        for (int d = 0; d < 3; ++d) {
            const int cu = int(std::floor((x[d] - sd.lo[d]) / sd.Lc[d]));
            int c = cu;
            if (sd.per[d]) {
                c %= sd.nc[d];
                if (c < 0) c += sd.nc[d];
            } else {
                c = std::min(std::max(cu, 0), sd.nc[d] - 1);
            }
            const int cref = sd.per[d] ? cu : c;
            const double center = sd.lo[d] + (double(cref) + 0.5) * sd.Lc[d];
            o[d] = x[d] - center;
            cc[d] = c;
        }
    }

    void build_ff() {
        const FFHost &F = ffh();
        std::memset(&hff, 0, sizeof(hff));
        for (int k = 0; k < NT * NT; ++k) {
            PairP<R> &q = hff.pair[k];
            q.kind = F.kind[k];
            q.cutsq = R(F.cutsq[k]);
            q.cut = R(F.cut[k]);
            q.rep = R(F.rep[k]);
            q.att = R(F.att[k]);
            q.rep8 = R(8.0 * F.rep[k]);
            q.att4 = R(4.0 * F.att[k]);
            q.alpha = R(F.alpha[k]);
            q.aatt = R(F.alpha[k] * F.att[k]);
            q.ljcutsq = R(F.ljcutsq[k]);
            q.lj1 = R(F.lj1[k]);
            q.lj2 = R(F.lj2[k]);
            q.anysq = R(std::max(F.cutsq[k], F.ljcutsq[k]));
        }
        for (int t = 0; t < NT; ++t) {
            const double gam = 6.0 * M_PI * P.eta * F.radius[t];  // src/integrate_langevin.h:110-114
            const double sig = std::sqrt(2.0 * P.kBT * gam) * std::sqrt(3.0 / P.dt);
            hff.mass[t] = R(F.mass[t]);
            hff.inv_mass[t] = R(1.0 / F.mass[t]);
            hff.gamma[t] = R(gam);
            hff.sigma[t] = R(sig);
        }
        for (int b = 0; b < MAX_BT; ++b) {
            hff.bond[b].K = R(P.bond_K[b]);
            hff.bond[b].Rm = R(P.bond_R[b]);
            hff.bond[b].style = P.bond_style[b];
        }
        for (int ti = 0; ti < 16; ++ti)
            for (int tj = 0; tj < 16; ++tj) {
                float v = 0.f;
                float vin = 0.f;
                if (ti < NT && tj < NT && F.range[ti * NT + tj] > 0) {
                    const double rl = F.range[ti * NT + tj] + P.skin;
                    v = float(rl * rl);
                    vin = float(F.range[ti * NT + tj] * F.range[ti * NT + tj]);
                }
                hff.rlist2[ti * 16 + tj] = v;
                hff.rin2[ti * 16 + tj] = vin;
            }
    }

    void fill_args() {
        std::memset(&a, 0, sizeof(a));
        for (int k = 0; k < 2; ++k) {
            a.pos[k] = pos[k].p;
            a.nrm[k] = nrm[k].p;
            a.vel[k] = vel[k].p;
            a.omg[k] = omg[k].p;
            a.frc[k] = frc[k].p;
            a.trq[k] = trq[k].p;
            a.xref[k] = xref[k].p;
            a.cell[k] = cell[k].p;
            a.tag[k] = tagd[k].p;
            a.home[k] = home[k].p;
            a.bond[k] = bond[k].p;
            a.fslot[k] = fslot[k].p;
            a.skey[k] = skey[k].p;
            a.sval[k] = sval[k].p;
        }
        a.epart = epart.p;
        a.faces = faces.p;
        a.nfaces = nfaces;
        a.nmblk = nmblk;
        a.mesh_blk_sys = mesh_bs.p;
        a.mesh_partial = mesh_part.p;
        a.nbr = nbr.p;
        a.nnb = nnb.p;
        a.cap = cap;
        a.ranges = ranges.p;
        a.slot_of_home = soh.p;
        a.blk_sys = blk_sys.p;
        a.partial = partial.p;
        a.gpartial = gpartial.p;
        a.ngroups = ngroups_total;
        a.S = Sd.p;
        a.sys = sysd.p;
        a.ss = ssd.p;
        a.nsys = nsys;
        a.npad = npad;
        a.counts = counts.p;
        a.digit_total = dtot.p;
        a.inv = invd.p;
        a.sort_passes = passes;
        a.ntiles = ntiles;
        a.dt = P.dt;
        a.kBT = P.kBT;
        a.skin_half2 = R(0.25 * P.skin * P.skin);
        a.seed = P.seed;
        a.rebuild_every = P.rebuild_every;
        a.variant = P.kernel_variant & (7 | 32 | 64);
        a.nlist_lane = (P.kernel_variant >> 3) & 3;
        a.carry_forces = P.integrator == ORBC_INT_NOSE_HOOVER ? 1 : 0;
        a.zero_bulk = P.zero_bulk ? 1 : 0;
        a.ff = ffd.p;
        a.ll = hff.pair[0];
    }

    int build_lists(bool first) {
        for (int attempt = 0; attempt < 4; ++attempt) {
            int one = 1;
            CK(cudaMemcpyAsync(&Sd.p->rebuild, &one, sizeof(int), cudaMemcpyHostToDevice, st));
            int zero = 0;
            CK(cudaMemcpyAsync(&Sd.p->max_nnb, &zero, sizeof(int), cudaMemcpyHostToDevice, st));
            launch_rebuild<R>(a, st, false);
            CK(cudaGetLastError());
            Scalars hs;
            CK(cudaMemcpyAsync(&hs, Sd.p, sizeof(Scalars), cudaMemcpyDeviceToHost, st));
            CK(cudaStreamSynchronize(st));
            if (hs.max_nnb <= cap && !(first && hs.max_nnb > cap * 0.8)) {
                if (hs.error & ERRB_NBR_OVERFLOW) {
                    int clr = hs.error & ~ERRB_NBR_OVERFLOW;
                    CK(cudaMemcpy(&Sd.p->error, &clr, sizeof(int), cudaMemcpyHostToDevice));
                }
                return ORBC_OK;
            }
            int rc = grow_capacity(hs.max_nnb, false);
            if (rc) return rc;
            int clr = hs.error & ~ERRB_NBR_OVERFLOW;
            CK(cudaMemcpy(&Sd.p->error, &clr, sizeof(int), cudaMemcpyHostToDevice));
        }
        return fail(ORBC_ERR_NBR_OVERFLOW, "neighbour capacity could not be sized");
    }

    int grow_capacity(int need, bool rebuild_now = true) {
        int nc = std::max(cap, int(std::ceil(need * 1.3 / 8.0)) * 8);
        if (nc <= cap) nc = cap + 16;

        drop_graph();
        if (nbr.alloc(size_t(nc) * size_t(npad))) return fail(ORBC_ERR_NOMEM, "neighbour list allocation failed");
        cap = nc;
        a.nbr = nbr.p;
        a.cap = cap;
        if (rebuild_now) {  // the next step rebuilds into the larger list
            int one = 1;
            CK(cudaMemcpyAsync(&Sd.p->rebuild, &one, sizeof(int), cudaMemcpyHostToDevice, st));
            CK(cudaStreamSynchronize(st));
        }
        return ORBC_OK;
    }

    void drop_graph() {
        if (gexec) cudaGraphExecDestroy(gexec);
        if (gexec1) cudaGraphExecDestroy(gexec1);
        gexec = nullptr;
        gexec1 = nullptr;
        graph_cond = false;
    }

    cudaStream_t st = nullptr, cs = nullptr;  // step stream, frame-copy stream
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, fpack[2] = {nullptr, nullptr};
    Scalars *hsc = nullptr;  // pinned: the counters before and after step()
    static constexpr int NXCH = 4;  // chunks of the host <-> device state transfers
    cudaEvent_t xev[NXCH] = {}, pev[1] = {};
    int device = 0;
    FrameWriter fw;
    DevBuf<char> fstage[2];
    DevBuf<int> fmap;                                    // file position of each upload index
    std::shared_ptr<const std::vector<int32_t>> ident;  // (tag, type) pairs in file order
    cudaGraphExec_t gexec = nullptr, gexec1 = nullptr;
    bool graph_cond = false;
    int graph_steps = 0;
    bool uploaded = false, nh_primed = false, has_mesh = false, vcom_valid = false;
    int nsys = 0, npad = 0, cap = 0, passes = 4, ntiles = 1, maxb = 0, maxf = 0, nfaces = 0, nmblk = 0;
    int64_t nhome = 0;
    uint64_t total_cells = 0;
    std::vector<SysDev> hsys;
    DevBuf<T4> pos[2], nrm[2], vel[2], omg[2], frc[2], trq[2], xref[2];
    DevBuf<int> cell[2], tagd[2], home[2];
    DevBuf<BondSlot> bond[2];
    DevBuf<int2> fslot[2];
    DevBuf<uint32_t> skey[2];
    DevBuf<int> sval[2];
    DevBuf<double> epart, partial, stage, gpartial;
    int ngroups_total = 0;
    DevBuf<int4> faces;
    DevBuf<int2> ranges;
    DevBuf<int> soh, blk_sys, counts, dtot, invd, nnb, mesh_bs;
    DevBuf<double> mesh_part;
    DevBuf<uint32_t> nbr;
    DevBuf<Scalars> Sd;
    DevBuf<SysDev> sysd;
    DevBuf<SysState> ssd;
    DevBuf<FFDev<R>> ffd;
    FFDev<R> hff;
    KArgs<R> a;
};

}  // namespace orbc

using namespace orbc;

struct orbc_handle {
    std::unique_ptr<EngineBase> e;
};

namespace orbc {
void set_standalone_error(const char *what, const char *detail) {
    g_last_error = std::string(what) + ": " + detail;
}
}  // namespace orbc

extern "C" {

void orbc_gpu_default_params(orbc_params *p) {
    std::memset(p, 0, sizeof(*p));
    p->precision = ORBC_PREC_MIXED;
    p->integrator = ORBC_INT_LANGEVIN;
    p->dt = 0.01;
    p->kBT = 0.22;
    p->eta = 0.01;
    p->Q = 0;
    p->seed = 0xBAD5EED;
    p->skin = 0.4;
    p->max_neighbors = 0;
    p->rebuild_every = 0;
    p->bounce = 1;
    p->use_graph = 1;
    p->energy = 0;
    p->host_direct = 1;
    for (int d = 0; d < 3; ++d) {
        p->lo[d] = -1000;
        p->hi[d] = 1000;
        p->periodic[d] = 0;
    }
    const double r0[4] = {2.25, 1.1225, 2.25, 2.24};
    for (int b = 0; b < ORBC_MAX_BOND_TYPES; ++b) {
        p->bond_style[b] = ORBC_BOND_HARMONIC;
        p->bond_K[b] = 57;
        p->bond_r0[b] = b < 4 ? r0[b] : 1.0;
        p->bond_R[b] = 0;
    }
}

int orbc_gpu_create(const orbc_params *p, orbc_handle **out) {
    if (!p || !out) {
        g_last_error = "create: null argument";
        return ORBC_ERR_ARG;
    }
    *out = nullptr;
    if (!(p->dt > 0) || p->skin < 0 || (p->precision != ORBC_PREC_FP64 && p->precision != ORBC_PREC_MIXED) ||
        (p->integrator != ORBC_INT_LANGEVIN && p->integrator != ORBC_INT_NOSE_HOOVER) ||
        (p->kernel_variant < 0 || p->kernel_variant > 127 || (p->kernel_variant & 24) == 24) || (p->zero_bulk != 0 && p->zero_bulk != 1) ||
        (p->host_direct != 0 && p->host_direct != 1)) {
        g_last_error = "create: invalid parameters";
        return ORBC_ERR_ARG;
    }
    for (int b = 0; b < ORBC_MAX_BOND_TYPES; ++b) {
        if (p->bond_style[b] < 0 || p->bond_style[b] > 2 ||
            (p->bond_style[b] != ORBC_BOND_HARMONIC && !(p->bond_R[b] > 0))) {
            g_last_error = "create: invalid bond table (FENE / WLC need bond_R > 0)";
            return ORBC_ERR_ARG;
        }
    }
    std::unique_ptr<orbc_handle> h(new orbc_handle);
    int rc;
    if (p->precision == ORBC_PREC_FP64) {
        auto *e = new Engine<double>(*p);
        h->e.reset(e);
        rc = e->init();
    } else {
        auto *e = new Engine<float>(*p);
        h->e.reset(e);
        rc = e->init();
    }
    if (rc) {
        g_last_error = h->e->err;
        return rc;
    }
    *out = h.release();
    return ORBC_OK;
}

int orbc_gpu_upload(orbc_handle *h, const double *x3, const double *n3, const double *v3, const double *o3,
                    const int *type, const int *tag, size_t n, const int *bonds3, size_t nb) {
    if (!h) return ORBC_ERR_ARG;
    orbc_system_desc d;
    std::memset(&d, 0, sizeof(d));
    const orbc_params &P = h->e->P;
    for (int k = 0; k < 3; ++k) {
        d.lo[k] = P.lo[k];
        d.hi[k] = P.hi[k];
        d.periodic[k] = P.periodic[k];
    }
    d.kv = P.kv;
    d.V0 = P.V0;
    d.ka = P.ka;
    d.A0 = P.A0;
    const int64_t off[2] = {0, int64_t(n)};
    return h->e->upload(1, &d, off, x3, n3, v3, o3, type, tag, n, bonds3, nullptr, nb, nullptr, 0);
}

int orbc_gpu_upload_batch(orbc_handle *h, int nsys, const orbc_system_desc *sys, const int64_t *offsets,
                          const double *x3, const double *n3, const double *v3, const double *o3, const int *type,
                          const int *tag, size_t n, const int *bonds3, const double *bond_r0, size_t nb,
                          const int *faces3, size_t nf) {
    if (!h || !sys || !offsets) return ORBC_ERR_ARG;
    return h->e->upload(nsys, sys, offsets, x3, n3, v3, o3, type, tag, n, bonds3, bond_r0, nb, faces3, nf);
}

int orbc_gpu_set_state(orbc_handle *h, const double *x3, const double *n3, const double *v3, const double *o3) {
    return h ? h->e->set_state(x3, n3, v3, o3) : ORBC_ERR_ARG;
}
int orbc_gpu_set_state_f32(orbc_handle *h, int64_t first, int64_t count, int stride, const float *x, const float *n,
                           const float *v, const float *o) {
    return h ? h->e->set_state_f32(first, count, stride, x, n, v, o) : ORBC_ERR_ARG;
}
int orbc_gpu_download_f32(orbc_handle *h, int64_t first, int64_t count, int stride, float *x, float *n, float *v,
                          float *o) {
    return h ? h->e->download_f32(first, count, stride, x, n, v, o) : ORBC_ERR_ARG;
}
int orbc_gpu_step(orbc_handle *h, int nsteps, orbc_thermo *out) { return h ? h->e->step(nsteps, out) : ORBC_ERR_ARG; }
int orbc_gpu_download(orbc_handle *h, double *x3, double *n3, double *v3, double *o3) {
    return h ? h->e->download(x3, n3, v3, o3) : ORBC_ERR_ARG;
}
int orbc_gpu_forces(orbc_handle *h, double *f3, double *t3, double *e) {
    return h ? h->e->forces(f3, t3, e) : ORBC_ERR_ARG;
}
int orbc_gpu_thermo(orbc_handle *h, int sys, orbc_thermo *out) {
    return (h && out) ? h->e->thermo(sys, out) : ORBC_ERR_ARG;
}
int orbc_gpu_neighbors(orbc_handle *h, int *counts, int *list, int64_t cap, int64_t *total) {
    return h ? h->e->neighbors(counts, list, cap, total) : ORBC_ERR_ARG;
}
int orbc_gpu_cells(orbc_handle *h, int sys, double *lo3, double *lc3, int *nc3, int *cell, double *offset3,
                   int *slot) {
    return h ? h->e->cells(sys, lo3, lc3, nc3, cell, offset3, slot) : ORBC_ERR_ARG;
}
int orbc_gpu_rebuild(orbc_handle *h) { return h ? h->e->rebuild() : ORBC_ERR_ARG; }
int orbc_gpu_rdf(orbc_handle *h, int sys, int type_a, int type_b, double dr, int nbins, double rcut,
                 uint64_t *counts, int64_t *dropped) {
    return h ? h->e->rdf(sys, type_a, type_b, dr, nbins, rcut, counts, dropped) : ORBC_ERR_ARG;
}
int orbc_gpu_save_frame(orbc_handle *h, const char *path, int append, int nstep, int fields, int real_bytes,
                        int async) {
    return h ? h->e->save_frame(path, append, nstep, fields, real_bytes, async) : ORBC_ERR_ARG;
}
int orbc_gpu_flush(orbc_handle *h) { return h ? h->e->flush_frames() : ORBC_ERR_ARG; }
int orbc_gpu_cleanup(orbc_handle *h, double stray_tolerance, int64_t *removed) {
    return h ? h->e->cleanup(stray_tolerance, removed) : ORBC_ERR_ARG;
}
int orbc_gpu_save_checkpoint(orbc_handle *h, const char *path) {
    return h ? h->e->save_checkpoint(path) : ORBC_ERR_ARG;
}
int orbc_gpu_load_checkpoint(orbc_handle *h, const char *path) {
    return h ? h->e->load_checkpoint(path) : ORBC_ERR_ARG;
}
int orbc_gpu_minimize(orbc_handle *h, int nsteps, double dr_max, double dn_max, orbc_thermo *out) {
    return h ? h->e->minimize(nsteps, dr_max, dn_max, out) : ORBC_ERR_ARG;
}
int orbc_gpu_assign_temperature(orbc_handle *h, double kBT, uint64_t seed) {
    return h ? h->e->assign_temperature(kBT, seed) : ORBC_ERR_ARG;
}
int orbc_gpu_last_timing(orbc_handle *h, double *ms, int64_t *launches) {
    if (!h) return ORBC_ERR_ARG;
    if (ms) *ms = h->e->last_ms;
    if (launches) *launches = h->e->last_launches;
    return ORBC_OK;
}

int orbc_gpu_profile(orbc_handle *h, int nsteps, orbc_profile *out) {
    return h ? h->e->profile(nsteps, out) : ORBC_ERR_ARG;
}

int orbc_gpu_autotune(orbc_handle *h, int trial_steps, orbc_tune_trial *trials, int max_trials, int *ntrials) {
    return h ? h->e->autotune(trial_steps, trials, max_trials, ntrials) : ORBC_ERR_ARG;
}

int orbc_gpu_destroy(orbc_handle *h) {
    delete h;
    return ORBC_OK;
}
const char *orbc_gpu_error(orbc_handle *h) { return h ? h->e->err.c_str() : g_last_error.c_str(); }
const char *orbc_gpu_version(void) { return "orbc_gpu 0.1 sm_103a"; }

static int standalone_fail(const char *what, cudaError_t e) {
    g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
    return ORBC_ERR_CUDA;
}

int orbc_gpu_morton_encode(const double *p3, int64_t n, const double *bsize3, uint32_t *keys) {
    if (n < 0 || (n > 0 && (!p3 || !bsize3 || !keys))) return ORBC_ERR_ARG;
    if (n == 0) return ORBC_OK;
    double *dp = nullptr;
    uint32_t *dk = nullptr;
    cudaError_t e = cudaMalloc(&dp, size_t(n) * 3 * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&dk, size_t(n) * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMemcpy(dp, p3, size_t(n) * 3 * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        launch_morton(dp, n, bsize3, dk, 0);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(keys, dk, size_t(n) * sizeof(uint32_t), cudaMemcpyDeviceToHost);
    cudaFree(dp);
    cudaFree(dk);
    return e == cudaSuccess ? ORBC_OK : standalone_fail("morton_encode", e);
}

__global__ static void k_iota(int *v, int64_t n) {
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
        v[i] = int(i);
}

int orbc_gpu_morton_order(const double *p3, int64_t n, const double *bsize3, int32_t *order) {
    if (n < 0 || (n > 0 && (!p3 || !bsize3 || !order))) return ORBC_ERR_ARG;
    if (n == 0) return ORBC_OK;
    if (n >= (int64_t(1) << 31)) return ORBC_ERR_ARG;
    const int ntiles = sort_tiles(n);
    double *dp = nullptr;
    uint32_t *k[2] = {nullptr, nullptr};
    int *v[2] = {nullptr, nullptr}, *cnt = nullptr, *tot = nullptr;
    cudaError_t e = cudaMalloc(&dp, size_t(n) * 3 * sizeof(double));
    for (int b = 0; b < 2 && e == cudaSuccess; ++b) {
        e = cudaMalloc(&k[b], size_t(n) * sizeof(uint32_t));
        if (e == cudaSuccess) e = cudaMalloc(&v[b], size_t(n) * sizeof(int));
    }
    if (e == cudaSuccess) e = cudaMalloc(&cnt, size_t(256) * ntiles * sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&tot, 256 * sizeof(int));
    if (e == cudaSuccess) e = cudaMemcpy(dp, p3, size_t(n) * 3 * sizeof(double), cudaMemcpyHostToDevice);
    int fin = 0;
    if (e == cudaSuccess) {
        launch_morton(dp, n, bsize3, k[0], 0);
        k_iota<<<1216, 256>>>(v[0], n);
        fin = radix_sort_pairs(k, v, cnt, tot, nullptr, n, 4, ntiles, nullptr, 0);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(order, v[fin], size_t(n) * sizeof(int), cudaMemcpyDeviceToHost);
    cudaFree(dp);
    for (int b = 0; b < 2; ++b) {
        cudaFree(k[b]);
        cudaFree(v[b]);
    }
    cudaFree(cnt);
    cudaFree(tot);
    return e == cudaSuccess ? ORBC_OK : standalone_fail("morton_order", e);
}

}  // extern "C"
