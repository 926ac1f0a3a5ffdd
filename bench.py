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
           orbc_gpu_step + orbc_gpu_download_f32 back to the host buffers.
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
    args = ap.parse_args()
    rank, ws = dist_setup()
    if args.impl == "reference":
        return run_reference(args, rank, ws)
    if "LOCAL_RANK" in os.environ:
        os.environ.setdefault("CUDA_VISIBLE_DEVICES", os.environ["LOCAL_RANK"])

    from openrbc_gb300 import _native as N
    L = N.lib()
    t_gen = time.perf_counter()
    w = workload(args.n_lipid)
    n = len(w["x"])
    log(f"workload: {n} particles, {len(w['bonds'])} bonds, {len(w['faces'])} faces "
        f"({time.perf_counter() - t_gen:.1f} s)")

    # ---- mixed precision, device-resident
    sim = make_sim(w, "mixed", skin=args.skin if args.skin is not None else SKIN, kernel_variant=args.form,
                   rebuild_every=args.rebuild_every)
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
        for h, arr in zip(host, sim.download()):
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
        e2e = {"value": ws * n * e2e_steps / e2e_s, "unit": "particle-steps/s",
               "h2d_bytes_per_step": 4 * 3 * 4 * n, "d2h_bytes_per_step": 4 * 3 * 4 * n, "steps": e2e_steps,
               "note": "per step: orbc_gpu_set_state_f32 (pinned H2D of the x, n, v, o float containers; the "
                       "list is rebuilt only when a particle moved more than skin/2) + "
                       "orbc_gpu_step(1) + orbc_gpu_download_f32 (D2H of x, n, v, o)"}
        log(f"e2e: {e2e['value']:.4e} particle-steps/s")

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
