"""TEST INFRASTRUCTURE ONLY -- times the oracle's CPU baseline against the
reference's own CPU code on the same machine and the same states, so that
the port can stand in for the reference where the reference cannot be built
(its source tree does not travel with this repository).

    python oracle/port_vs_reference.py --ref-src /path/to/reference/src [--threads 8] [--n-lipid 1000000]

Builds (oracle/Makefile `refbin`, the reference's Makefile flags
-O3 -march=native -mrecip -ffast-math, default FUSED_PAIRWISE + LANGEVIN mode,
real = float) the reference's program oracle/_ref/openrbc and the harness
oracle/_ref/libref_prod.so, whose ref_time_production runs the reference's
production loop (Voronoi initialisation, then src/openrbc.cpp:153-256 without
I/O: Voronoi and cell-list updates every freq_voronoi = 2 steps,
compute_pairwise_fused, compute_bonded, integrate(verlet_langevin)) on a
given state.  Then, on `--threads` OpenMP threads:

1. sphere: the reference's program on its own lipid sphere (`-i lipid`,
   about 131,740 lipids; `--opt` minimisation steps relax its random
   placement) for 100 steps, read from its `+main-loop` timer
   (src/openrbc.cpp:153,261); the state after its first step (a trajectory
   dump) through ref_time_production and through the oracle's CPU baseline
   (orc_run_langevin_fast_f32), 100 steps each.
2. membrane: the benchmark's Evans-Fung membrane at `--n-lipid` lipids
   (lipids and spectrin anchors, without bonds or the area / volume
   constraint, which the reference does not have in this form) through
   ref_time_production and through the oracle's CPU baseline, `--steps`
   steps each.

Prints one JSON line with every rate in particle-steps/s.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import re
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
# run as a script, this directory is first on the path and would shadow the
# oracle package with oracle/oracle.py
sys.path = [ROOT] + [p for p in sys.path if os.path.abspath(p or ".") != HERE]

import numpy as np  # noqa: E402


def ref_prod():
    L = C.CDLL(os.path.join(HERE, "_ref", "libref_prod.so"))
    vp, i64, d = C.c_void_p, C.c_int64, C.c_double
    L.ref_time_production.argtypes = [i64, vp, vp, vp, vp, vp, vp, i64, vp, d, d, d, C.c_int, C.c_int,
                                      C.POINTER(d), C.POINTER(d)]
    return L


def time_reference(L, x, n, v, o, ty, tg, steps, threads, dt=0.01, kBT=0.22, eta=0.01):
    arr = [np.ascontiguousarray(a, np.float64) for a in (x, n, v, o)]
    ty = np.ascontiguousarray(ty, np.int32)
    tg = np.ascontiguousarray(tg, np.int32)
    si, sl = C.c_double(), C.c_double()
    L.ref_time_production(len(ty), *[a.ctypes.data for a in arr], ty.ctypes.data, tg.ctypes.data, 0, None, dt, kBT,
                          eta, steps, threads, C.byref(si), C.byref(sl))
    return {"particle_steps_per_s": len(ty) * steps / sl.value, "loop_s": sl.value, "voronoi_init_s": si.value,
            "steps": steps, "particles": int(len(ty)), "threads": threads,
            "what": "ref_time_production: the reference's main loop (src/openrbc.cpp:153-256) on this state"}


def time_port(x, n, v, o, ty, tg, steps, threads, dt=0.01, kBT=0.22, eta=0.01):
    from oracle import oracle as orc
    st = orc.State(x=x, nrm=n, v=v, o=o, type=ty, tag=tg, kBT=kBT, dt=dt, eta=eta, seed=1)
    orc.set_threads(threads)
    t0 = time.perf_counter()
    th = orc.cpu_baseline_run(st, steps)
    s = time.perf_counter() - t0
    return {"particle_steps_per_s": len(ty) * steps / s, "s": s, "steps": steps, "particles": int(len(ty)),
            "threads": orc.get_threads(), "list_builds": th["npairs"],
            "what": "orc_run_langevin_fast_f32, the oracle's CPU baseline, skin 0.4"}


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref-src", required=True, help="the reference's src/ directory")
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--opt", type=int, default=300, help="minimisation steps of the sphere before its timed loop")
    ap.add_argument("--n-lipid", type=int, default=1_000_000)
    args = ap.parse_args()
    subprocess.run(["make", "-s", "-C", HERE, "refbin", "liborbc_oracle_fast.so", "liborbc_workloads.so",
                    f"REF={args.ref_src}"], check=True, stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    exe = os.path.join(HERE, "_ref", "openrbc")
    env = dict(os.environ, OMP_NUM_THREADS=str(args.threads), OMP_PROC_BIND="close", OMP_PLACES="cores")
    dt, nsph = 0.01, 100
    out = {"host": subprocess.run(["uname", "-m"], capture_output=True, text=True).stdout.strip(),
           "threads": args.threads}
    with tempfile.TemporaryDirectory() as tmp:
        common = ["-i", "lipid", "-E", str(args.opt), "--cleanup-frequency", "1000000",
                  "-o", os.path.join(tmp, "topo.txt")]
        log = subprocess.run([exe, *common, "-t", str(nsph * dt), "-d", "1000000", "-x", os.path.join(tmp, "a.orbc")],
                             env=env, cwd=tmp, capture_output=True, text=True, check=True).stdout
        # display_timing prints "<t> ms on ..." or "<t> s on ..." by magnitude
        m = re.search(r"([0-9.]+)\s+(ms|s) on (\d+) steps \* (\d+) particles on (\d+) threads", log)
        if not m:
            raise RuntimeError("the reference printed no main-loop timing:\n" + log[-2000:])
        ms = float(m.group(1)) * (1.0 if m.group(2) == "ms" else 1e3)
        steps, npart = int(m.group(3)), int(m.group(4))
        prog = {"particle_steps_per_s": npart * steps / (ms * 1e-3), "ms": ms, "steps": steps, "particles": npart,
                "threads": int(m.group(5)), "timer": "+main-loop (src/openrbc.cpp:153,261)",
                "command": f"openrbc {' '.join(common[:-2])} -t {nsph * dt} -d 1000000"}
        subprocess.run([exe, *common, "-t", str(dt), "-d", "1", "--dump-field", "11",
                        "-x", os.path.join(tmp, "b.orbc")], env=env, cwd=tmp, capture_output=True, check=True)
        with open(os.path.join(tmp, "b.orbc"), "rb") as f:
            data = f.read()
    from openrbc_gb300.frames import iter_frames
    fr = list(iter_frames(data, 4))[-1]
    zero = np.zeros_like(fr["x"])
    L = ref_prod()
    out["sphere"] = {
        "program": prog,
        "reference_loop": time_reference(L, fr["x"], fr["n"], fr["v"], zero, fr["type"], fr["tag"], nsph,
                                         args.threads),
        "port": time_port(fr["x"], fr["n"], fr["v"], zero, fr["type"], fr["tag"], nsph, args.threads)}
    from openrbc_gb300 import workloads
    from oracle import oracle as orc
    freq = max(4, int(round(57 * (args.n_lipid / 4_000_000) ** 0.5)))
    w = workloads.rbc(n_lipid=args.n_lipid, freq=freq, kT=1.0, seed=2, lib=orc.workloads_lib())
    ref_m = time_reference(L, w["x"], w["n"], w["v"], w["o"], w["type"], w["tag"], args.steps, args.threads,
                           kBT=1.0)
    port_m = time_port(w["x"], w["n"], w["v"], w["o"], w["type"], w["tag"], args.steps, args.threads, kBT=1.0)
    out["membrane"] = {"n_lipid": args.n_lipid, "reference_loop": ref_m, "port": port_m,
                       "port_over_reference": port_m["particle_steps_per_s"] / ref_m["particle_steps_per_s"]}
    out["sphere"]["port_over_reference_loop"] = (out["sphere"]["port"]["particle_steps_per_s"]
                                                 / out["sphere"]["reference_loop"]["particle_steps_per_s"])
    print(json.dumps(out))
    return 0


if __name__ == "__main__":
    sys.exit(main())
