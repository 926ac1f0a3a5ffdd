"""The benchmark's reference arm (bench.py --impl reference) runs the oracle's
CPU baseline on the host cores: it must time exactly the steps it reports and
never load the GPU library -- its inputs come from the oracle's build of the
host generators, which must produce the library's workload bit for bit."""
import json
import os
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROBE = r"""
import json, sys, io, contextlib
sys.argv = ["bench.py", "--impl", "reference", "--n-lipid", "20000", "--steps", "3", "--warmup", "2"]
sys.path.insert(0, ".")
import bench
buf = io.StringIO()
with contextlib.redirect_stdout(buf):
    rc = bench.main()
maps = open("/proc/self/maps").read()
print(json.dumps({"rc": rc, "line": buf.getvalue().strip().splitlines()[-1],
                  "gpu_lib_loaded": "liborbc_gpu" in maps,
                  "oracle_loaded": "liborbc_oracle_fast" in maps}))
"""


def test_reference_arm_loads_no_gpu_library_and_times_its_steps():
    r = subprocess.run([sys.executable, "-c", PROBE], cwd=ROOT, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    out = json.loads(r.stdout.strip().splitlines()[-1])
    assert out["rc"] == 0
    assert not out["gpu_lib_loaded"]
    assert out["oracle_loaded"]
    line = json.loads(out["line"])
    assert line["impl"] == "reference" and line["steps"] == 3 and line["warmup"] == 2
    assert line["value"] > 0 and abs(line["ms_per_step"] * 1e-3 * line["value"] - line["config"]["n_particles"]) \
        < 1e-6 * line["config"]["n_particles"]
    assert line["e2e"]["value"] == line["value"]


def test_oracle_generators_match_the_library_bit_for_bit():
    sys.path.insert(0, ROOT)
    from openrbc_gb300 import workloads
    from oracle import oracle as orc
    a = workloads.rbc(n_lipid=15000, freq=6)
    b = workloads.rbc(n_lipid=15000, freq=6, lib=orc.workloads_lib())
    for k in ("x", "n", "v", "o", "type", "tag", "bonds", "bond_r0", "faces"):
        assert np.array_equal(a[k], b[k]), k
    assert a["area"] == b["area"] and a["volume"] == b["volume"]
    a = workloads.lattice(n=3000, ncol=55)
    b = workloads.lattice(n=3000, ncol=55, lib=orc.workloads_lib())
    for k in a:
        assert np.array_equal(a[k], b[k]), k
