"""Mixed precision along a long Nose-Hoover run of a whole cell (the shape of
the 10,000-step mixed-precision configuration, scaled to a test): every few
hundred steps the mixed state is handed to an FP64 handle of the same cell
and the force, energy, area and volume of both are compared at that state.
The FP64 path is itself pinned to the oracle (test_gpu_parity,
test_gpu_systems), so this bounds the mixed error against FP64 arithmetic
along the trajectory, not only at the start."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def _cell():
    from openrbc_gb300 import workloads
    return workloads.rbc(n_lipid=200_000, freq=13, kT=1.0, seed=8)


def _sim(w, precision):
    from openrbc_gb300 import RTParameter, Simulation, workloads
    p = RTParameter(init="trimesh", kBT=1.0, dt=0.01, precision=precision, integrator="nose-hoover")
    s = Simulation(p, skin=0.8, bond_table=workloads.RBC_BOND_TABLE, energy=True)
    c = w["constraint"]
    s.upload_batch([{"lo": (-1000.0,) * 3, "hi": (1000.0,) * 3, "kv": c["kv"], "V0": c["V0"], "ka": c["ka"],
                     "A0": c["A0"]}], w["x"], w["n"], w["v"], w["o"], w["type"], w["tag"], [0, len(w["x"])],
                   bonds=w["bonds"], bond_r0=w["bond_r0"], faces=w["faces"])
    return s


def test_mixed_forces_energy_area_volume_track_fp64_along_the_run():
    w = _cell()
    checks = []
    with _sim(w, "mixed") as sm, _sim(w, "fp64") as sd:
        for block in range(4):
            sm.step(250)
            x, n, v, o = sm.download()
            fm, tm, em = sm.forces()
            thm = sm.thermo(0)
            sd.set_state(x, n, v, o)
            fd, td, ed = sd.forces()
            thd = sd.thermo(0)
            checks.append((rel_l2(fm, fd), rel_l2(tm, td), abs(em.sum() - ed.sum()) / np.abs(ed).sum(),
                           abs(thm["area"] - thd["area"]) / thd["area"],
                           abs(thm["volume"] - thd["volume"]) / thd["volume"]))
        assert sm.thermo(0)["step"] == 1000 and np.isfinite(sm.thermo(0)["zeta"])
    for ferr, terr, eerr, aerr, verr in checks:
        assert ferr < 1e-5 and terr < 1e-5
        assert eerr < 1e-5
        assert aerr < 1e-6 and verr < 1e-6
