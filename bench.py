"""Benchmark: particle-steps/s of the OpenRBC step on the 4M-particle red-cell
membrane, mixed precision vs plain FP64 on one GB300.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Workload: Evans-Fung biconcave membrane with 4.0M lipids (Poisson-disk by
area, density 1.05) plus 32,492 spectrin anchors on a frequency-57 geodesic
mesh, 97,470 WLC-POW bonds (rest length U[0.9, 1.1] x mean edge), global
area / volume constraint at reduced volume 0.64, Langevin dt = 0.01, kT = 1,
eta = 0.01.  Seeded synthetic data (the reference ships no dataset).

value      mixed-precision particle-steps/s, device time of K steps (inputs
           resident in HBM; working set several GB, larger than L2).
e2e        the same metric through the C ABI the reference host would call
           each step with its own containers (AoS vector<real,3>, real =
           float): orbc_gpu_set_state_f32 from pinned host buffers + one
           orbc_gpu_step + orbc_gpu_download_f32 back to the host buffers,
           restarted from the state the timed steps started from, so that
           it covers the same stretch of the run as `value`.
roofline   the fused step kernel: compulsory bytes (104 B per particle-step,
           mixed) / its CUDA-event time vs measured HBM bandwidth; the FP32
           ALU fraction of its algorithmic flops is reported beside it.
cpu_baseline  the oracle's CPU baseline -- the reference's FP32 step organised
           as its production loop, measured within a few per cent of the
           reference's own main loop on x86 (oracle/port_vs_reference.py) --
           on the host cores, a bounded sample; it also checks the GPU's
           mixed-precision forces against the oracle's FP64 forces.
--impl reference  times that CPU implementation for the same metric on the
           same workload, exactly --warmup + --steps steps, without loading
           the GPU library.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s, 4M-particle RBC: mixed vs FP64 GPU at force err<=1e-5"
N_LIPID = 4_000_000
FREQ = 57
KT = 1.0
DT = 0.01
SKIN = 0.4
# algorithmic counts per particle-step (mixed): state read + written once
BYTES_PER_PSTEP = 104.0
FLOP_PER_PAIR = 106.0


def workload(n_lipid=N_LIPID, lib=None):
    """The membrane; `lib` is the library that generates it (default the GPU
    library; the CPU-only reference arm passes the oracle's build of the same
    host generators, so that it never loads the GPU library)."""
    from openrbc_gb300 import workloads
    freq = FREQ if n_lipid == N_LIPID else max(4, int(round(FREQ * (n_lipid / N_LIPID) ** 0.5)))
    return workloads.rbc(n_lipid=n_lipid, freq=freq, kT=KT, seed=2, lib=lib)


def bench_config(w, n_lipid):
    """The workload description, identical in both arms."""
    n = len(w["x"])
    return {"workload": f"rbc-evans-fung-{n}", "n_particles": n, "n_lipid": n_lipid, "anchors": n - n_lipid,
            "bonds": int(len(w["bonds"])), "faces": int(len(w["faces"])), "integrator": "langevin", "dt": DT,
            "kT": KT, "eta": 0.01, "reduced_volume": 0.64,
            "l2": "inputs larger than L2 (state + neighbour list > 1 GB)", "parallelism": "one system per rank"}


def log(*a):
    print("[bench]", *a, file=sys.stderr, flush=True)


def make_sim(w, precision, **kw):
    from openrbc_gb300 import RTParameter, Simulation, workloads
    p = RTParameter(init="trimesh", mesh="synthetic", kBT=KT, dt=DT, eta=0.01, precision=precision)
    s = Simulation(p, skin=kw.pop("skin", SKIN), bond_table=workloads.RBC_BOND_TABLE, **kw)
    c = w["constraint"]
    sysdesc = [{"lo": (-1000.0,) * 3, "hi": (1000.0,) * 3, "periodic": (0, 0, 0), "kv": c["kv"], "V0": c["V0"],
                "ka": c["ka"], "A0": c["A0"]}]
    s.upload_batch(sysdesc, w["x"], w["n"], w["v"], w["o"], w["type"], w["tag"], [0, len(w["x"])],
                   bonds=w["bonds"], bond_r0=w["bond_r0"], faces=w["faces"])
    return s


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    def __init__(self, index=0):
        self.samples = []
        self.stop = threading.Event()
        self.index = index
        self.t = threading.Thread(target=self.run, daemon=True)

    def run(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        while not self.stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True,
                                     timeout=5).stdout.strip()
                if out:
                    self.samples.append([s.strip() for s in out.split(",")])
            except Exception:
                pass
            self.stop.wait(0.2)

    def __enter__(self):
        self.t.start()
        return self

    def __exit__(self, *a):
        self.stop.set()
        self.t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in self.samples for k in range(4) if s[3 + k].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


TRAFFIC_PROFILE = "profiles/k_step_langevin_lite_float_rbc1M.md"


def profiled_traffic_per_particle():
    """DRAM bytes per particle of one launch of the step kernel, from the
    committed ncu summary (the capture cannot run inside the benchmark)."""
    path = os.path.join(ROOT, TRAFFIC_PROFILE)
    try:
        with open(path) as f:
            for line in f:
                if "traffic_bytes_per_particle:" in line:
                    return float(line.split("traffic_bytes_per_particle:")[1].split("|")[0].strip())
    except OSError:
        pass
    return None


def fma_peaks(L):
    """Measured FP32 / FP64 FMA throughput of this GPU (TFLOP/s)."""
    import ctypes as C
    a, b = C.c_double(), C.c_double()
    try:
        if L.orbc_gpu_fma_peak(C.byref(a), C.byref(b)) == 0:
            return a.value, b.value
    except Exception:
        pass
    return None, None


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


CPU_SKIN = 0.6  # neighbour skin of the CPU baseline's Verlet list


def oracle_state(w, orc):
    st = orc.State(x=w["x"], nrm=w["n"], v=w["v"], o=w["o"], type=w["type"], tag=w["tag"], bonds=w["bonds"],
                   bond_r0=w["bond_r0"], faces=w["faces"], kBT=KT, dt=DT, eta=0.01, seed=0xBAD5EED,
                   kv=w["constraint"]["kv"], V0=w["constraint"]["V0"], ka=w["constraint"]["ka"],
                   A0=w["constraint"]["A0"])
    st.bstyle[4], st.bK[4], st.br0[4], st.bR[4] = 2, 1.0, 1.0, 2.2
    return st


CPU_KIND = ("the oracle's CPU baseline (orc_run_langevin_fast_f32): the reference's FP32 Langevin step "
            "(src/compute_pairwise_fused.h, src/compute_bonded.h, src/integrate_langevin.h) organised as its "
            "production loop -- cell-sorted particles, Verlet list, Newton's third law inside each thread's "
            "range -- built with the reference's -O3 -ffast-math native flags; on x86 it runs within a few "
            "per cent of the reference's own main loop on the same states (oracle/port_vs_reference.py)")


def cpu_baseline(w, nsteps=20, f_mixed=None):
    """The oracle's CPU baseline on all host cores (bounded sample), and --
    as the checker -- the oracle's FP64 forces of the same state against the
    GPU's mixed-precision forces."""
    from oracle import oracle as orc
    threads = os.cpu_count() or 1
    orc.set_threads(threads)
    out = {}
    if f_mixed is not None:
        f64, _, _, _ = orc.forces(oracle_state(w, orc), "f64")
        out["force_rel_err_mixed_vs_oracle_fp64"] = float(np.linalg.norm(f_mixed - f64) / np.linalg.norm(f64))
    st = oracle_state(w, orc)
    orc.cpu_baseline_run(st, 1, CPU_SKIN)  # warm-up
    t0 = time.perf_counter()
    th = orc.cpu_baseline_run(st, nsteps, CPU_SKIN)
    dt = time.perf_counter() - t0
    n = len(w["x"])
    out.update({"value": n * nsteps / dt, "unit": "particle-steps/s", "cores": orc.get_threads(), "kind": "port",
                "sample": f"{nsteps} Langevin steps of the full {n}-particle membrane ({th['npairs']} list builds), "
                          f"FP32; " + CPU_KIND})
    return out


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    return rank, ws


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def allreduce_max(v, ws):
    if ws <= 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_reference(args, rank, ws):
    """The reference arm: the oracle's CPU baseline (the reference's CPU step,
    see CPU_KIND) on the host cores, exactly --warmup untimed then --steps
    timed steps of the same workload.  Loads no GPU library: the workload
    comes from the oracle's build of the host generators."""
    if rank != 0:
        return 0
    from oracle import oracle as orc
    orc.build()
    w = workload(args.n_lipid, lib=orc.workloads_lib())
    n = len(w["x"])
    threads = os.cpu_count() or 1
    orc.set_threads(threads)
    st = oracle_state(w, orc)
    if args.warmup > 0:
        orc.cpu_baseline_run(st, args.warmup, CPU_SKIN)
    t0 = time.perf_counter()
    th = orc.cpu_baseline_run(st, args.steps, CPU_SKIN)
    secs = time.perf_counter() - t0
    value = n * args.steps / secs
    cb = {"value": value, "unit": "particle-steps/s", "cores": orc.get_threads(), "kind": "port",
          "sample": f"the full workload: {args.warmup} warm-up + {args.steps} timed Langevin steps "
                    f"({th['npairs']} list builds in the timed steps), FP32; " + CPU_KIND}
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "particle-steps/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * secs / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "precision": "fp32 (the reference's real)", "config": bench_config(w, args.n_lipid),
            "cpu_baseline": cb, "e2e": {"value": value, "unit": "particle-steps/s", "h2d_bytes_per_step": 0,
                                        "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# The other workloads of the configuration list, one JSON line each
# (python bench.py --config NAME); the default line is the 4M-particle
# membrane above.
# ---------------------------------------------------------------------------
def _roof(prof, n, bytes_per_pstep=BYTES_PER_PSTEP):
    peak, kind = measured_peaks()
    kt = prof["step_kernel_ms"]
    achieved = bytes_per_pstep * n / (kt * 1e-3) / 1e9
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": None, "kernel_ms": kt, "bytes_per_particle_step": bytes_per_pstep,
            "peak_source": f"{kind} (MEASURED_PEAKS.json hbm_gbs)"}


def _line(metric_value, args, cfg, **extra):
    line = {"metric": METRIC, "value": metric_value, "unit": "particle-steps/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": cfg}
    line.update(extra)
    return line


def run_config_lattice(args):
    """Plain method, small: 32,768 lipids on the 182-column square lattice of
    spacing 1.1 in a periodic 200 x 200 x 40 box, Langevin dt 0.01, kT 1, 100
    steps: plain FP64 and mixed on the GPU, the oracle's FP64 restatement and
    FP32 CPU baseline on the host cores."""
    from openrbc_gb300 import RTParameter, Simulation, workloads
    from oracle import oracle as orc
    w = workloads.lattice(n=32768, ncol=182, spacing=1.1, jitter=0.05, tilt=0.05, kT=1.0, seed=1)
    n = len(w["x"])
    box, per = ((0.0, 200.0), (0.0, 200.0), (-20.0, 20.0)), (1, 1, 1)
    steps = args.steps
    out = {}
    f_gpu = {}
    for prec, form in (("fp64", 3 | 16 | 32), ("mixed", 7 | 16 | 32)):
        p = RTParameter(init="lipid", kBT=KT, dt=DT, eta=0.01, precision=prec)
        with Simulation(p, box=box, periodic=per, kernel_variant=form, skin=0.5) as s:
            s.upload(w["x"], w["n"], w["v"], w["o"], w["type"], w["tag"])
            f_gpu[prec], _, _ = s.forces()
            s.step(args.warmup)
            s.step(steps)
            ms, launches = s.last_timing()
            prof = s.profile(20)
        out[prec] = {"value": n * steps / (ms * 1e-3), "ms_per_step": ms / steps, "kernel_form": form,
                     "gpu_launches": launches, "profile": prof}
        log(f"lattice {prec}: {ms / steps:.4f} ms/step")
    threads = os.cpu_count() or 1
    orc.set_threads(threads)
    st = orc.State(x=w["x"], nrm=w["n"], v=w["v"], o=w["o"], type=w["type"], tag=w["tag"], kBT=KT, dt=DT, eta=0.01,
                   lo=tuple(b[0] for b in box), hi=tuple(b[1] for b in box), periodic=per, seed=1)
    f_ref, _, _, _ = orc.forces(st, "f64")
    t0 = time.perf_counter()
    orc.langevin(st.copy(), steps, "f64")
    cpu64 = n * steps / (time.perf_counter() - t0)
    st32 = st.copy()
    t0 = time.perf_counter()
    orc.cpu_baseline_run(st32, steps, CPU_SKIN)
    cpu32 = n * steps / (time.perf_counter() - t0)
    cfg = {"workload": "lattice-32768", "n_particles": n, "lattice": "182 columns, spacing 1.1, jitter 0.05, "
           "tilt 0.05 rad", "box": "200 x 200 x 40, periodic", "integrator": "langevin", "dt": DT, "kT": KT,
           "l2": "working set below L2: the state stays in L2 between steps"}
    return _line(out["fp64"]["value"], args, cfg, dtype="f64", precision="fp64 (the plain FP64 GPU form)",
                 ms_per_step=out["fp64"]["ms_per_step"], mixed=out["mixed"], fp64=out["fp64"],
                 force_rel_err_fp64_vs_oracle=float(np.linalg.norm(f_gpu["fp64"] - f_ref) / np.linalg.norm(f_ref)),
                 force_rel_err_mixed_vs_oracle=float(np.linalg.norm(f_gpu["mixed"] - f_ref) / np.linalg.norm(f_ref)),
                 cpu_fp64={"value": cpu64, "cores": threads, "kind": "port", "what": "the oracle's FP64 restatement"},
                 cpu_baseline={"value": cpu32, "unit": "particle-steps/s", "cores": threads, "kind": "port",
                               "sample": f"{steps} steps, FP32; " + CPU_KIND},
                 roofline=_roof(out["fp64"]["profile"], n, 192.0), gpu_launches=out["fp64"]["gpu_launches"])


def run_config_nh(args):
    """The 4M-particle membrane in mixed precision under Nose-Hoover at kT 1:
    --steps steps in chunks of --check-every; after each chunk the mixed state
    is loaded into a plain FP64 handle of the same system and its forces,
    torques, potential energy, area and volume are compared with the mixed
    handle's own at that state."""
    from openrbc_gb300 import RTParameter, Simulation, workloads
    w = workload(args.n_lipid)
    n = len(w["x"])
    c = w["constraint"]
    sysdesc = [{"lo": (-1000.0,) * 3, "hi": (1000.0,) * 3, "periodic": (0, 0, 0), "kv": c["kv"], "V0": c["V0"],
                "ka": c["ka"], "A0": c["A0"]}]

    def handle(prec, form):
        p = RTParameter(init="trimesh", mesh="synthetic", kBT=KT, dt=DT, precision=prec, integrator="nose-hoover")
        s = Simulation(p, skin=0.8, bond_table=workloads.RBC_BOND_TABLE, kernel_variant=form, energy=True)
        s.upload_batch(sysdesc, w["x"], w["n"], w["v"], w["o"], w["type"], w["tag"], [0, n], bonds=w["bonds"],
                       bond_r0=w["bond_r0"], faces=w["faces"])
        return s

    form = args.form if args.form else (3 | 16 | 32 | 64)
    # the running handle, and two probes that receive its state at each check:
    # calling forces() on the running handle would re-prime its carried forces
    mixed, probe, ref = handle("mixed", form), handle("mixed", form), handle("fp64", 3 | 16 | 32)
    mixed.step(args.warmup)
    checks, total_ms, done = [], 0.0, 0
    while done < args.steps:
        k = min(args.check_every, args.steps - done)
        mixed.step(k)
        ms, _ = mixed.last_timing()
        total_ms += ms
        done += k
        thm = mixed.thermo()
        x, nv, v, o = mixed.download()
        probe.set_state(x, nv, v, o)
        ref.set_state(x, nv, v, o)
        fm, tm, em = probe.forces()
        fr, tr, er = ref.forces()
        thp, thr = probe.thermo(), ref.thermo()
        row = {"step": thm["step"], "force_rel_err": float(np.linalg.norm(fm - fr) / np.linalg.norm(fr)),
               "torque_rel_err": float(np.linalg.norm(tm - tr) / np.linalg.norm(tr)),
               "energy_rel_err": float(abs(em.sum() - er.sum()) / abs(er.sum())),
               "area_rel_err": abs(thp["area"] - thr["area"]) / thr["area"],
               "volume_rel_err": abs(thp["volume"] - thr["volume"]) / thr["volume"],
               "area": thm["area"], "volume": thm["volume"], "temperature": thm["temperature"], "zeta": thm["zeta"]}
        checks.append(row)
        log(f"nh step {row['step']}: force err {row['force_rel_err']:.2e}, area err {row['area_rel_err']:.2e}, "
            f"volume err {row['volume_rel_err']:.2e}, T {row['temperature']:.4f}")
    probe.close()
    ref.close()
    prof = mixed.profile(20)
    value = n * args.steps / (total_ms * 1e-3)
    mixed.close()
    cfg = dict(bench_config(w, args.n_lipid), integrator="nose-hoover", workload=f"rbc-evans-fung-{n}-nh")
    return _line(value, args, cfg, ms_per_step=total_ms / args.steps, precision="mixed", kernel_form=form,
                 checks=checks, check_every=args.check_every,
                 max_force_rel_err=max(r["force_rel_err"] for r in checks),
                 max_area_rel_err=max(r["area_rel_err"] for r in checks),
                 max_volume_rel_err=max(r["volume_rel_err"] for r in checks), profile=prof,
                 roofline=_roof(prof, n))


def _tuned(sim, args):
    if args.no_autotune:
        return None
    trials = sim.autotune(trial_steps=20)
    best = min(trials, key=lambda r: r["ms_per_step"])
    return {"chosen": best, "trials": len(trials)}


def run_config_vesicles(args):
    """96 spherical vesicles, log-normal sizes between 10k and 250k lipids
    (median 40k, about 5M in all), each in its own periodic box of edge 2.5
    diameters, advanced together in one launch per step (mixed, Langevin)."""
    from openrbc_gb300 import RTParameter, Simulation, workloads
    w = workloads.vesicles()
    n = len(w["x"])
    p = RTParameter(init="vesicle", kBT=KT, dt=DT, eta=0.01, precision="mixed")
    with Simulation(p, skin=0.8, kernel_variant=args.form or (7 | 16 | 32)) as s:
        s.upload_batch(w["systems"], w["x"], w["n"], w["v"], w["o"], w["type"], w["tag"], w["offsets"])
        tune = _tuned(s, args)
        s.step(args.warmup)
        th = s.step(args.steps)
        ms, launches = s.last_timing()
        prof = s.profile(20)
    value = n * args.steps / (ms * 1e-3)
    sizes = w["sizes"]
    cfg = {"workload": f"vesicles-96-{n}", "n_particles": n, "systems": 96, "size_min": int(sizes.min()),
           "size_median": int(np.median(sizes)), "size_max": int(sizes.max()), "integrator": "langevin", "dt": DT,
           "kT": KT, "l2": "inputs larger than L2", "parallelism": "one launch per step for all systems"}
    return _line(value, args, cfg, ms_per_step=ms / args.steps, precision="mixed", tuning=tune, profile=prof,
                 roofline=_roof(prof, n), gpu_launches=launches, temperature=th["temperature"])


ENSEMBLE_KV = 0.05  # volume-constraint stiffness of the ensemble's cells


def run_config_ensemble(args):
    """8 whole red cells of about 4.0M particles each (32M in all), reduced
    volumes 0.60, 0.65, ..., 0.95, each with its own spectrin network (seeds
    5..12) and volume constraint, Nose-Hoover at kT 1, mixed, one
    graph-captured step for all cells.  Every cell starts from the same
    biconcave shape (reduced volume about 0.64), so the cells far from their
    target are pulled towards it by a soft constraint (kv = ENSEMBLE_KV; with
    the single cell's kv = 10 the 0.95 cell's spectrin bonds pass their
    maximum extension within a few hundred steps)."""
    from openrbc_gb300 import RTParameter, Simulation, workloads
    cells, sysd, base = [], [], 0
    for i in range(8):
        v0 = 0.60 + 0.05 * i
        wi = workloads.rbc(n_lipid=args.n_lipid, freq=FREQ if args.n_lipid == N_LIPID else
                           max(4, int(round(FREQ * (args.n_lipid / N_LIPID) ** 0.5))), kT=KT, seed=5 + i,
                           reduced_volume=v0, kv=ENSEMBLE_KV)
        shift = base - int(wi["tag"].min()) + 1
        wi["tag"] = wi["tag"] + shift
        wi["bonds"] = wi["bonds"].copy()
        wi["bonds"][:, 1:] += shift
        wi["faces"] = wi["faces"] + shift
        base = int(wi["tag"].max())
        c = wi["constraint"]
        sysd.append({"lo": (-1000.0,) * 3, "hi": (1000.0,) * 3, "periodic": (0, 0, 0), "kv": c["kv"], "V0": c["V0"],
                     "ka": c["ka"], "A0": c["A0"]})
        cells.append(wi)
        log(f"cell {i}: {len(wi['x'])} particles, reduced volume {v0:.2f}")
    cat = {k: np.concatenate([c[k] for c in cells]) for k in ("x", "n", "v", "o", "type", "tag", "bonds", "bond_r0",
                                                             "faces")}
    offs = np.concatenate([[0], np.cumsum([len(c["x"]) for c in cells])])
    n = int(offs[-1])
    p = RTParameter(init="trimesh", mesh="synthetic", kBT=KT, dt=DT, precision="mixed", integrator="nose-hoover")
    with Simulation(p, skin=0.8, bond_table=workloads.RBC_BOND_TABLE,
                    kernel_variant=args.form or (3 | 16 | 32 | 64)) as s:
        s.upload_batch(sysd, cat["x"], cat["n"], cat["v"], cat["o"], cat["type"], cat["tag"], offs,
                       bonds=cat["bonds"], bond_r0=cat["bond_r0"], faces=cat["faces"])
        s.step(args.warmup)
        th = s.step(args.steps)
        ms, launches = s.last_timing()
        per_cell = [s.thermo(k) for k in range(8)]
        prof = s.profile(10)
    value = n * args.steps / (ms * 1e-3)
    cfg = {"workload": f"rbc-ensemble-8x{args.n_lipid}", "n_particles": n, "systems": 8,
           "reduced_volumes": [round(0.60 + 0.05 * i, 2) for i in range(8)], "kv": ENSEMBLE_KV,
           "integrator": "nose-hoover", "dt": DT,
           "kT": KT, "l2": "inputs larger than L2", "parallelism": "one graph-captured step for all cells"}
    return _line(value, args, cfg, ms_per_step=ms / args.steps, precision="mixed", profile=prof,
                 roofline=_roof(prof, n), gpu_launches=launches,
                 cells=[{"area": c["area"], "volume": c["volume"], "temperature": c["temperature"], "zeta": c["zeta"]}
                        for c in per_cell])


CONFIGS = {"lattice32k": run_config_lattice, "nh4m": run_config_nh, "vesicles96": run_config_vesicles,
           "ensemble8": run_config_ensemble}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--fp64-steps", type=int, default=10)
    ap.add_argument("--n-lipid", type=int, default=N_LIPID, help="smaller membranes for profiling runs")
    ap.add_argument("--skip-fp64", action="store_true")
    ap.add_argument("--skip-e2e", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default skin / kernel form")
    ap.add_argument("--skin", type=float, default=None, help="neighbour skin when not autotuning")
    ap.add_argument("--form", type=int, default=0, help="kernel form 0..127 (orbc_params.kernel_variant)")
    ap.add_argument("--rebuild-every", type=int, default=0, help="fixed rebuild cadence when not autotuning")
    ap.add_argument("--config", default="rbc4m", choices=["rbc4m"] + sorted(CONFIGS),
                    help="workload: rbc4m (default, the headline line), lattice32k, nh4m, vesicles96, ensemble8")
    ap.add_argument("--check-every", type=int, default=1000, help="nh4m: steps between FP64 comparisons")
    ap.add_argument("--host-direct", type=int, default=1, choices=[0, 1],
                    help="e2e: 1 = in-place host transfers where the arrays are reachable, 0 = staged copies")
    args = ap.parse_args()
    rank, ws = dist_setup()
    if args.impl == "reference":
        return run_reference(args, rank, ws)
    if "LOCAL_RANK" in os.environ:
        os.environ.setdefault("CUDA_VISIBLE_DEVICES", os.environ["LOCAL_RANK"])
    if args.config != "rbc4m":
        line = CONFIGS[args.config](args)
        if rank == 0:
            print(json.dumps(line), flush=True)
        return 0

    from openrbc_gb300 import _native as N
    L = N.lib()
    t_gen = time.perf_counter()
    w = workload(args.n_lipid)
    n = len(w["x"])
    log(f"workload: {n} particles, {len(w['bonds'])} bonds, {len(w['faces'])} faces "
        f"({time.perf_counter() - t_gen:.1f} s)")

    # ---- mixed precision, device-resident
    sim = make_sim(w, "mixed", skin=args.skin if args.skin is not None else SKIN, kernel_variant=args.form,
                   rebuild_every=args.rebuild_every, host_direct=bool(args.host_direct))
    f_mixed, _, _ = sim.forces()
    tune = None
    if not args.no_autotune:
        t_tune = time.perf_counter()
        trials = sim.autotune(trial_steps=20)
        best = min(trials, key=lambda r: r["ms_per_step"])
        tune = {"chosen": best, "trials": trials, "seconds": time.perf_counter() - t_tune}
        log(f"autotune: skin {best['skin']}, form {best['variant']}, rebuild every {best['rebuild_every']}, "
            f"{best['ms_per_step']:.4f} ms/step "
            f"({len(trials)} trials, {tune['seconds']:.1f} s)")
    sim.step(args.warmup)
    # the state the timed steps start from: the profiled pass and the end-to-end
    # passes restart from it, so that every figure covers the same stretch of
    # the run (at kT = 1 the lipid film thins out as a run goes on)
    snap = sim.download()
    barrier(ws)
    th0 = sim.thermo()
    with ClockSampler() as clk:
        th = sim.step(args.steps)
        ms, launches = sim.last_timing()
    ms = allreduce_max(ms, ws)
    value = ws * n * args.steps / (ms * 1e-3)
    log(f"mixed: {ms / args.steps:.4f} ms/step, {value:.4e} particle-steps/s, "
        f"rebuilds {th['rebuilds'] - th0['rebuilds']}, T = {th['temperature']:.4f}")

    # ---- dominant kernel timing (profiled pass: CUDA events around each launch group)
    sim.set_state(*snap)
    prof = sim.profile(20)
    log(f"profile: {prof}")

    # ---- plain FP64 on the same workload
    fp64 = None
    ferr = None
    if not args.skip_fp64 and args.fp64_steps > 0:
        # the mixed run's force-loop and list-build forms and skin; the
        # occupancy form (bit 2) is sized for FP32 registers and compensated
        # accumulation (bit 6) is an FP32 remedy: both are left out
        form = (tune["chosen"]["variant"] if tune else args.form) & ~(4 | 64)
        skin = tune["chosen"]["skin"] if tune else (args.skin if args.skin is not None else SKIN)
        sim64 = make_sim(w, "fp64", skin=skin, kernel_variant=form)
        f64, _, _ = sim64.forces()
        sim64.step(2)
        sim64.step(args.fp64_steps)
        ms64, _ = sim64.last_timing()
        value64 = n * args.fp64_steps / (ms64 * 1e-3)
        sim64.close()
        ferr = float(np.linalg.norm(f_mixed - f64) / np.linalg.norm(f64))
        fp64 = {"value": value64, "ms_per_step": ms64 / args.fp64_steps, "steps": args.fp64_steps,
                "skin": skin, "kernel_form": form}
        log(f"fp64: {ms64 / args.fp64_steps:.4f} ms/step; mixed force rel err vs fp64 {ferr:.3e}")

    # ---- end to end through the C ABI with pinned host buffers
    e2e = None
    if not args.skip_e2e:
        import torch
        # the reference's containers: AoS float vectors of 3 (src/config_static.h:34-44)
        host = [torch.empty((n, 3), dtype=torch.float32, pin_memory=True).numpy() for _ in range(4)]
        sim.set_state(*snap)
        for h, arr in zip(host, snap):
            h[:] = arr
        e2e_steps = max(100, args.steps)

        def e2e_step():
            N.check(L.orbc_gpu_set_state_f32(sim.h, 0, n, 3, *[h.ctypes.data for h in host]), sim.h)
            N.check(L.orbc_gpu_step(sim.h, 1, None), sim.h)
            N.check(L.orbc_gpu_download_f32(sim.h, 0, n, 3, *[h.ctypes.data for h in host]), sim.h)

        for _ in range(3):  # warm-up (first use captures the one-step graph)
            e2e_step()
        barrier(ws)
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            e2e_step()
        e2e_s = allreduce_max(time.perf_counter() - t0, ws)
        # where an e2e step's time goes (a separate pass after the timed one)
        ph = np.zeros(3)
        for _ in range(20):
            t1 = time.perf_counter()
            N.check(L.orbc_gpu_set_state_f32(sim.h, 0, n, 3, *[h.ctypes.data for h in host]), sim.h)
            t2 = time.perf_counter()
            N.check(L.orbc_gpu_step(sim.h, 1, None), sim.h)
            t3 = time.perf_counter()
            N.check(L.orbc_gpu_download_f32(sim.h, 0, n, 3, *[h.ctypes.data for h in host]), sim.h)
            ph += [t2 - t1, t3 - t2, time.perf_counter() - t3]
        e2e = {"value": ws * n * e2e_steps / e2e_s, "unit": "particle-steps/s",
               "h2d_bytes_per_step": 4 * 3 * 4 * n, "d2h_bytes_per_step": 4 * 3 * 4 * n, "steps": e2e_steps,
               "phases_ms": {"set_state_f32": 1e3 * ph[0] / 20, "step": 1e3 * ph[1] / 20,
                             "download_f32": 1e3 * ph[2] / 20},
               "note": "per step: orbc_gpu_set_state_f32 (pinned H2D of the x, n, v, o float containers; the "
                       "list is rebuilt only when a particle moved more than skin/2) + "
                       "orbc_gpu_step(1) + orbc_gpu_download_f32 (D2H of x, n, v, o)"}
        # the same through ordinary pageable arrays, as the reference's own
        # containers are allocated (in place where the GPU reads host page tables)
        sim.set_state(*snap)
        pg = [np.array(a, dtype=np.float32) for a in snap]
        for _ in range(3):
            N.check(L.orbc_gpu_set_state_f32(sim.h, 0, n, 3, *[h.ctypes.data for h in pg]), sim.h)
            N.check(L.orbc_gpu_step(sim.h, 1, None), sim.h)
            N.check(L.orbc_gpu_download_f32(sim.h, 0, n, 3, *[h.ctypes.data for h in pg]), sim.h)
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            N.check(L.orbc_gpu_set_state_f32(sim.h, 0, n, 3, *[h.ctypes.data for h in pg]), sim.h)
            N.check(L.orbc_gpu_step(sim.h, 1, None), sim.h)
            N.check(L.orbc_gpu_download_f32(sim.h, 0, n, 3, *[h.ctypes.data for h in pg]), sim.h)
        e2e["pageable_value"] = n * e2e_steps / (time.perf_counter() - t0)
        log(f"e2e: {e2e['value']:.4e} particle-steps/s (pageable containers {e2e['pageable_value']:.4e}); "
            f"phases {e2e['phases_ms']}")

    peak, peak_kind = measured_peaks()
    kt = prof["step_kernel_ms"]
    achieved = BYTES_PER_PSTEP * n / (kt * 1e-3) / 1e9
    pairs = prof["pairs_in_cutoff"]
    flops = 0.5 * pairs * FLOP_PER_PAIR * n
    tpp = profiled_traffic_per_particle()
    fma32, fma64 = fma_peaks(L)
    alu_tf = flops / (kt * 1e-3) / 1e12
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": tpp * n if tpp else None, "kernel": "k_step_langevin_lite<float>", "kernel_ms": kt,
            "bytes_per_particle_step": BYTES_PER_PSTEP,
            "traffic_source": f"{TRAFFIC_PROFILE}: ncu dram__bytes_read.sum + dram__bytes_write.sum of one "
                              f"launch on the 1.0M-lipid cell, {tpp} B per particle, scaled to {n} particles",
            "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else peak_kind,
            "alu": {"achieved": alu_tf, "peak": fma32, "frac": (alu_tf / fma32) if fma32 else None,
                    "unit": "TFLOP/s FP32",
                    "counts": "106 flop per interacting pair (src/compute_pairwise.h:64-65,129), "
                              "half the inner list entries",
                    "peak_source": "orbc_gpu_fma_peak on this GPU (FFMA chains, all SMs)", "fp64_peak": fma64}}
    line = {"metric": METRIC, "value": value, "unit": "particle-steps/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "precision": "mixed (FP32 pair / bond arithmetic, positions as int32 cell + FP32 offset, FP64 "
                         "area / volume / kinetic-energy sums)",
            "config": bench_config(w, args.n_lipid),
            "tuning": {"skin": tune["chosen"]["skin"] if tune else (args.skin if args.skin is not None else SKIN),
                       "kernel_form": tune["chosen"]["variant"] if tune else args.form,
                       "rebuild_every": tune["chosen"]["rebuild_every"] if tune else args.rebuild_every},
            "fp64": fp64, "mixed_over_fp64": (value / ws / fp64["value"]) if fp64 else None,
            "force_rel_err_mixed_vs_fp64": ferr, "rebuilds_in_timed_region": th["rebuilds"] - th0["rebuilds"],
            "roofline": roof, "e2e": e2e, "gpu_launches": launches, "clocks": clk.summary(), "profile": prof,
            "autotune": tune}
    sim.close()
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(w, f_mixed=f_mixed)
        line["force_rel_err_mixed_vs_oracle_fp64"] = line["cpu_baseline"].pop("force_rel_err_mixed_vs_oracle_fp64")
        log(f"cpu baseline: {line['cpu_baseline']}")
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
