"""Statistical agreement of thermostatted runs: the GPU's mixed-precision
step against the oracle's FP64 step from the same start and the same noise
key.  The trajectories separate (the dynamics is chaotic and the two
evaluate forces in different precisions), so the checks are on equilibrium
averages: the temperature (src/compute_temperature.h:24-29), the pair-distance
histogram (src/rdf.h:26-47) and the membrane area and enclosed volume.

Acceptance: block means agree within 4 combined standard errors (plus a small
absolute floor for nearly constant observables); histograms of the sampled
frames agree to a Kolmogorov-Smirnov distance below 0.02 with the first peak
in the same bin.
"""
import numpy as np
import pytest

from conftest import rel_l2
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def _blocks(a, nb=4):
    a = np.asarray(a, np.float64)
    m = len(a) // nb * nb
    b = a[:m].reshape(nb, -1).mean(axis=1)
    return b.mean(), b.std(ddof=1) / np.sqrt(nb)


def _agree(a, b, floor):
    (ma, ea), (mb, eb) = _blocks(a), _blocks(b)
    return abs(ma - mb) <= 4.0 * np.hypot(ea, eb) + floor, (ma, ea, mb, eb)


def _ks(h1, h2):
    c1 = np.cumsum(h1, dtype=np.float64)
    c2 = np.cumsum(h2, dtype=np.float64)
    return float(np.abs(c1 / c1[-1] - c2 / c2[-1]).max())


def test_lattice_temperature_and_rdf_mixed_vs_fp64_oracle():
    from openrbc_gb300 import RTParameter, Simulation, workloads
    ncol, n, kT, seed = 64, 4096, 0.5, 31
    w = workloads.lattice(n=n, ncol=ncol, kT=kT, seed=3)
    box = ((0.0, ncol * 1.1), (0.0, (n // ncol) * 1.1), (-20.0, 20.0))
    per = (1, 1, 0)
    centre = [0.5 * (b[0] + b[1]) for b in box]
    L = (box[0][1] - box[0][0], box[1][1] - box[1][0], 0.0)
    equil, every, frames = 200, 25, 16
    rdf_kw = dict(dr=0.05, nbins=100, rcut=5.0)

    st = orc.State(x=w["x"], nrm=w["n"], v=w["v"], o=w["o"], type=w["type"], tag=w["tag"], lo=[b[0] for b in box],
                   hi=[b[1] for b in box], periodic=per, kBT=kT, seed=seed)
    T_ref, h_ref = [], np.zeros(rdf_kw["nbins"])
    orc.langevin(st, equil)
    for _ in range(frames):
        th = orc.langevin(st, every)
        T_ref.append(th["temperature"])
        h_ref += orc.rdf(st.x, st.type, centre=centre, L=L, **rdf_kw)[0]

    p = RTParameter(init="lipid", kBT=kT, precision="mixed", rseed=seed)
    T_gpu, h_gpu = [], np.zeros(rdf_kw["nbins"])
    with Simulation(p, box=box, periodic=per, skin=0.4) as s:
        s.upload(w["x"], w["n"], w["v"], w["o"], w["type"], w["tag"])
        s.step(equil)
        for _ in range(frames):
            th = s.step(every)
            T_gpu.append(th["temperature"])
            h_gpu += s.rdf(**rdf_kw)[0]
        x = s.download()[0]

    ok, info = _agree(T_gpu, T_ref, 0.0)
    assert ok, info
    assert _ks(h_gpu, h_ref) < 0.02
    assert int(np.argmax(h_gpu)) == int(np.argmax(h_ref))
    # the two runs did separate, so this is a statistical (not a trajectory) check
    assert rel_l2(x, st.x) > 1e-6


def test_whole_cell_area_volume_temperature_mixed_vs_fp64_oracle():
    from openrbc_gb300 import RTParameter, Simulation, workloads
    w = workloads.rbc(n_lipid=30_000, freq=5, kT=1.0, seed=3)
    table = workloads.RBC_BOND_TABLE
    c = w["constraint"]
    st = orc.State(x=w["x"], nrm=w["n"], v=w["v"], o=w["o"], type=w["type"], tag=w["tag"], bonds=w["bonds"],
                   bond_r0=w["bond_r0"], faces=w["faces"], kBT=1.0, seed=17)
    for t, spec in table.items():
        st.bstyle[t], st.bK[t], st.br0[t], st.bR[t] = spec["style"], spec["K"], spec["r0"], spec["R"]
    st.kv, st.V0, st.ka, st.A0 = c["kv"], c["V0"], c["ka"], c["A0"]
    equil, every, frames = 60, 15, 12
    ref = {"T": [], "A": [], "V": []}
    orc.langevin(st, equil)
    for _ in range(frames):
        orc.langevin(st, every)
        th = orc.thermo(st)
        ref["T"].append(th["temperature"])
        ref["A"].append(th["area"])
        ref["V"].append(th["volume"])

    gpu = {"T": [], "A": [], "V": []}
    p = RTParameter(init="lipid", kBT=1.0, precision="mixed", rseed=17)
    with Simulation(p, bond_table=table) as s:
        sysd = [{"lo": (-1000.0,) * 3, "hi": (1000.0,) * 3, "kv": c["kv"], "V0": c["V0"], "ka": c["ka"],
                 "A0": c["A0"]}]
        s.upload_batch(sysd, w["x"], w["n"], w["v"], w["o"], w["type"], w["tag"], [0, len(w["x"])],
                       bonds=w["bonds"], bond_r0=w["bond_r0"], faces=w["faces"])
        s.step(equil)
        for _ in range(frames):
            th = s.step(every)
            gpu["T"].append(th["temperature"])
            gpu["A"].append(th["area"])
            gpu["V"].append(th["volume"])
    for key, floor in (("T", 0.0), ("A", 2e-4 * ref["A"][0]), ("V", 2e-4 * ref["V"][0])):
        ok, info = _agree(gpu[key], ref[key], floor)
        assert ok, (key, info)
