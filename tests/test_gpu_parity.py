"""GPU parity: liborbc_gpu (through its C ABI) against the golden vectors made
by the reference's own code and against the oracle on the same inputs.

Tolerances (relative L2 over all particles unless stated):
  FP64 forces / torques vs reference FP64 ........ 1e-10
  mixed forces / torques vs reference FP64 ....... 1e-5  (the stated force-error bound)
  FP64 100-step noise-free trajectory ............ 1e-9
  mixed trajectories, 10-100 steps ............... 2e-5 to 3e-5 (FP32 state; about 20 times
                                                   the largest difference seen on a GB300)
Integer / index work (neighbour sets, Morton keys and order) is bit-exact.
"""
import numpy as np
import pytest

from conftest import load_golden, rel_l2
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

REF_BOX = ((-1000.0, 1000.0),) * 3


def sim_for(g, precision, integrator="langevin", kBT=0.22, dt=0.01, eta=0.01, skin=0.4, energy=False, **kw):
    from openrbc_gb300 import RTParameter, Simulation
    p = RTParameter(init="lipid", kBT=kBT, dt=dt, eta=eta, precision=precision, integrator=integrator)
    s = Simulation(p, skin=skin, energy=energy, box=REF_BOX, **kw)
    s.upload(g["x"], g["nrm"], g["v"], g["o"], g["type"], g["tag"], g.get("bonds"))
    return s


@pytest.mark.parametrize("name", ["lattice_576.npz", "cell_ico12.npz"])
def test_forces_fp64_vs_reference(name):
    g = load_golden(name)
    with sim_for(g, "fp64") as s:
        f, t, e = s.forces()
    assert rel_l2(f, g["f64"]) < 1e-10
    assert rel_l2(t, g["t64"]) < 1e-10


@pytest.mark.parametrize("name", ["lattice_576.npz", "cell_ico12.npz"])
def test_forces_mixed_vs_reference(name):
    g = load_golden(name)
    with sim_for(g, "mixed") as s:
        f, t, e = s.forces()
    assert rel_l2(f, g["f64"]) < 1e-5, rel_l2(f, g["f64"])
    assert rel_l2(t, g["t64"]) < 1e-5, rel_l2(t, g["t64"])


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("mixed", 1e-5)])
def test_energy_vs_oracle(precision, tol):
    g = load_golden("cell_ico12.npz")
    st = orc.State(x=g["x"], nrm=g["nrm"], v=g["v"], o=g["o"], type=g["type"], tag=g["tag"], bonds=g["bonds"])
    _, _, e_ref, _ = orc.forces(st, energy=True)
    with sim_for(g, precision) as s:
        _, _, e = s.forces()
    assert abs(e.sum() - e_ref.sum()) < tol * np.abs(e_ref).sum()
    assert rel_l2(e, e_ref) < 10 * tol


@pytest.mark.parametrize("name", ["lattice_576.npz", "cell_ico12.npz"])
def test_noise_free_langevin_fp64(name):
    g = load_golden(name)
    with sim_for(g, "fp64", kBT=0.0, dt=float(g["lang_dt"]), eta=float(g["lang_eta"])) as s:
        s.step(int(g["lang_steps"]))
        x, n, v, o = s.download()
    assert rel_l2(x - g["x"], g["lang_x"] - g["x"]) < 1e-8
    assert rel_l2(n, g["lang_n"]) < 1e-9
    assert rel_l2(v, g["lang_v"]) < 1e-8
    assert rel_l2(o, g["lang_o"]) < 1e-8


@pytest.mark.parametrize("name", ["lattice_576.npz", "cell_ico12.npz"])
def test_noise_free_langevin_mixed(name):
    g = load_golden(name)
    with sim_for(g, "mixed", kBT=0.0, dt=float(g["lang_dt"]), eta=float(g["lang_eta"])) as s:
        s.step(int(g["lang_steps"]))
        x, n, v, o = s.download()
    assert rel_l2(x - g["x"], g["lang_x"] - g["x"]) < 3e-5
    assert rel_l2(v, g["lang_v"]) < 3e-5


@pytest.mark.parametrize("name", ["lattice_576.npz", "cell_ico12.npz"])
def test_nose_hoover_fp64(name):
    g = load_golden(name)
    with sim_for(g, "fp64", integrator="nose-hoover", kBT=float(g["nh_kBT"]), dt=float(g["nh_dt"])) as s:
        th = s.step(int(g["nh_steps"]))
        x, n, v, o = s.download()
    assert rel_l2(x - g["x"], g["nh_x"] - g["x"]) < 1e-8
    assert rel_l2(v, g["nh_v"]) < 1e-8
    assert rel_l2(o, g["nh_o"]) < 1e-8
    assert abs(th["zeta"] - float(g["nh_zeta"])) < 1e-8 * max(1.0, abs(float(g["nh_zeta"])))


@pytest.mark.parametrize("name", ["lattice_576.npz", "cell_ico12.npz"])
def test_nose_hoover_mixed(name):
    """The mixed form along the reference's own Nose-Hoover trajectory."""
    g = load_golden(name)
    with sim_for(g, "mixed", integrator="nose-hoover", kBT=float(g["nh_kBT"]), dt=float(g["nh_dt"])) as s:
        th = s.step(int(g["nh_steps"]))
        x, n, v, o = s.download()
    assert rel_l2(x - g["x"], g["nh_x"] - g["x"]) < 3e-5
    assert rel_l2(v, g["nh_v"]) < 3e-5
    assert rel_l2(o, g["nh_o"]) < 3e-5
    assert abs(th["zeta"] - float(g["nh_zeta"])) < 3e-5 * max(1.0, abs(float(g["nh_zeta"])))


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-9), ("mixed", 2e-5)])
def test_langevin_with_noise_vs_oracle(precision, tol):
    """Same counter-based noise on both sides, kT = 1, 10 steps."""
    g = load_golden("cell_ico12.npz")
    st = orc.State(x=g["x"], nrm=g["nrm"], v=g["v"], o=g["o"], type=g["type"], tag=g["tag"], bonds=g["bonds"],
                   kBT=1.0, dt=0.01, eta=0.01, seed=0xBAD5EED)
    orc.langevin(st, 10)
    with sim_for(g, precision, kBT=1.0) as s:
        th = s.step(10)
        x, n, v, o = s.download()
    assert rel_l2(x - g["x"], st.x - g["x"]) < tol
    assert rel_l2(v, st.v) < tol
    m = np.array([1, 4, 4, 1, 10, 10.0])[g["type"]]
    T = (m[:, None] * st.v ** 2).sum() / (3 * len(m))
    assert abs(th["temperature"] - T) < 10 * tol * T


@pytest.mark.parametrize("name", ["lattice_576.npz", "cell_ico12.npz"])
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("mixed", 1e-6)])
def test_temperature_matches_reference(name, precision, tol):
    """compute_temperature (src/compute_temperature.h:24-29) of the uploaded
    velocities: sum m v^2 / 3N against the reference's own value, before and
    after a zero-step call."""
    g = load_golden(name)
    T_ref = float(g["temperature"])
    with sim_for(g, precision) as s:
        th = s.thermo()
        assert th["n"] == len(g["x"])
        assert abs(th["temperature"] - T_ref) < tol * T_ref, (th["temperature"], T_ref)
        th0 = s.step(0)
        assert abs(th0["temperature"] - T_ref) < tol * T_ref, (th0["temperature"], T_ref)


def test_neighbour_sets_match_brute_force():
    g = load_golden("cell_ico12.npz")
    skin = 0.4
    _, _, c2, l2 = orc.ff_tables()
    rng = np.sqrt(np.maximum(c2, l2))
    rl2 = np.where(rng > 0, (rng + skin) ** 2, 0.0)
    st = orc.State(x=g["x"], nrm=g["nrm"], v=g["v"], o=g["o"], type=g["type"], tag=g["tag"])
    ref = orc.pairs(st, rl2)
    with sim_for(g, "fp64", skin=skin) as s:
        counts, lst = s.neighbors()
    rows = np.repeat(np.arange(len(counts)), counts)
    got = np.stack([rows, lst], 1)
    got = got[got[:, 0] < got[:, 1]]
    got = got[np.lexsort((got[:, 1], got[:, 0]))]
    # the oracle also drops pairs closer than 1e-5; the list keeps them (none exist here)
    a = set(map(tuple, ref))
    b = set(map(tuple, got))
    diff = a ^ b
    if diff:
        x = g["x"]
        for i, j in diff:
            r2 = ((x[i] - x[j]) ** 2).sum()
            lim = rl2[g["type"][i], g["type"][j]]
            assert abs(r2 - lim) < 1e-9 * lim, (i, j, r2, lim)
    # full list is symmetric
    assert np.array_equal(np.sort(rows), np.sort(lst)) or counts.sum() == len(lst)


def test_morton_keys_and_order_bit_exact():
    from openrbc_gb300 import morton_encode, morton_order
    g = load_golden("morton.npz")
    assert np.array_equal(morton_encode(g["p"]), g["keys64"])
    assert np.array_equal(morton_encode(g["p32"]), g["keys32"])
    keys = g["keys64"]
    assert np.array_equal(morton_order(g["p"]), np.lexsort((np.arange(len(keys)), keys)))


def test_morton_order_large_and_empty():
    from openrbc_gb300 import morton_order
    rng = np.random.default_rng(11)
    p = rng.uniform(-1000, 1000, (300_000, 3))
    p[::7] = p[3]  # many equal keys: stability matters
    keys = orc.morton_encode(p)
    assert np.array_equal(morton_order(p), np.lexsort((np.arange(len(keys)), keys)))
    assert len(morton_order(np.zeros((0, 3)))) == 0


# ---- the benchmark configurations' own fixtures ------------------------------
def _f64(a):
    return np.asarray(a, np.float64)


@pytest.mark.parametrize("precision,form,tol", [("fp64", 0, 1e-10), ("mixed", 0, 1e-5), ("mixed", 3 | 16 | 32, 1e-5),
                                                ("mixed", 3 | 16 | 32 | 64, 1e-5)])
def test_example_large_patch_forces(precision, form, tol):
    """A patch of the reference's own whole cell (init_rbc on example-large:
    lipids, band-III, actin, spectrin beads and their harmonic bonds) against
    the reference's FP64 forces and torques."""
    from openrbc_gb300 import RTParameter, Simulation
    g = load_golden("example_large_patch.npz")
    p = RTParameter(init="lipid", kBT=0.22, precision=precision)
    with Simulation(p, box=REF_BOX, kernel_variant=form) as s:
        s.upload(g["x"], g["nrm"], np.zeros_like(g["x"]), np.zeros_like(g["x"]), g["type"], g["tag"], g["bonds"])
        f, t, _ = s.forces()
    c = g["check"]
    assert rel_l2(f[c], g["f64"][c]) < tol, rel_l2(f[c], g["f64"][c])
    assert rel_l2(t[c], g["t64"][c]) < tol, rel_l2(t[c], g["t64"][c])


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-9), ("mixed", 3e-5)])
def test_example_large_patch_langevin_vs_oracle(precision, tol):
    """Ten Langevin steps of the same patch at the reference's default kT =
    0.22, against the oracle on the same input with the same counter-based
    noise (bonds, every protein type of the whole cell, list rebuilds)."""
    g = load_golden("example_large_patch.npz")
    z = np.zeros_like(np.asarray(g["x"], np.float64))
    st = orc.State(x=g["x"], nrm=g["nrm"], v=z, o=z, type=g["type"], tag=g["tag"], bonds=g["bonds"], kBT=0.22,
                   dt=0.01, eta=0.01, seed=0xBAD5EED)
    orc.langevin(st, 10)
    gg = {"x": g["x"], "nrm": g["nrm"], "v": z, "o": z, "type": g["type"], "tag": g["tag"], "bonds": g["bonds"]}
    with sim_for(gg, precision, kBT=0.22) as s:
        th = s.step(10)
        x, n, v, o = s.download()
    assert th["rebuilds"] >= 1
    assert rel_l2(x - g["x"], st.x - g["x"]) < tol
    assert rel_l2(v, st.v) < tol
    assert rel_l2(o, st.o) < 3 * tol  # angular velocities: the largest relative differences (6.4e-6 mixed)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("mixed", 1e-5)])
def test_config1_lattice_forces(precision, tol):
    """The plain small workload (32,768 lipids on the 182-column lattice)."""
    g = load_golden("lattice_32768.npz")
    gg = {k: (_f64(g[k]) if k in ("x", "nrm", "v", "o") else g[k]) for k in g}
    with sim_for(gg, precision) as s:
        f, t, _ = s.forces()
        th = s.thermo()
    assert rel_l2(f, g["f64"]) < tol
    assert rel_l2(t, g["t64"]) < tol
    T_ref = float(g["temperature"])
    assert abs(th["temperature"] - T_ref) < (1e-12 if precision == "fp64" else 1e-6) * T_ref


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-8), ("mixed", 3e-5)])
def test_config1_lattice_noise_free_langevin(precision, tol):
    """100 noise-free Langevin steps of the 32,768-lipid lattice against the
    reference's FP64 trajectory (every fourth particle kept in the fixture)."""
    g = load_golden("lattice_32768.npz")
    gg = {k: (_f64(g[k]) if k in ("x", "nrm", "v", "o") else g[k]) for k in g}
    with sim_for(gg, precision, kBT=0.0, dt=float(g["lang_dt"]), eta=float(g["lang_eta"])) as s:
        s.step(int(g["lang_steps"]))
        x, n, v, o = s.download()
    k = g["lang_keep"]
    x0 = gg["x"][k]
    assert rel_l2(x[k] - x0, g["lang_x"] - x0) < tol
    assert rel_l2(v[k], g["lang_v"]) < tol
    if precision == "fp64":
        assert rel_l2(n[k], g["lang_n"]) < 1e-9
        assert rel_l2(o[k], g["lang_o"]) < tol
