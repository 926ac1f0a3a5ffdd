"""Pin the oracle (CPU restatement) against golden vectors produced by the
reference's own code (tests/golden/make_golden.py).  CPU only."""
import numpy as np
import pytest

from conftest import load_golden, rel_l2
from oracle import oracle as orc


def state_from(g, **kw):
    return orc.State(x=g["x"], nrm=g["nrm"], v=g["v"], o=g["o"], type=g["type"], tag=g["tag"],
                     bonds=g.get("bonds", np.zeros((0, 3), np.int32)), **kw)


@pytest.mark.parametrize("name", ["lattice_576.npz", "cell_ico12.npz"])
def test_forces_fp64_match_reference(name):
    g = load_golden(name)
    st = state_from(g)
    f, t, _, th = orc.forces(st, "f64")
    assert rel_l2(f, g["f64"]) < 1e-12
    assert rel_l2(t, g["t64"]) < 1e-12
    assert np.abs(f - g["f64"]).max() < 1e-10 * max(1.0, np.abs(g["f64"]).max())


@pytest.mark.parametrize("name", ["lattice_576.npz", "cell_ico12.npz"])
def test_forces_fp32_match_reference_fp32(name):
    g = load_golden(name)
    st = state_from(g)
    f, t, _, _ = orc.forces(st, "f32")
    assert rel_l2(f, g["f32"]) < 2e-5
    assert rel_l2(t, g["t32"]) < 2e-5


def test_newton_third_law_and_zero_torque_sum():
    g = load_golden("lattice_576.npz")
    f, t, _, _ = orc.forces(state_from(g), "f64")
    assert np.abs(f.sum(0)).max() < 1e-9


@pytest.mark.parametrize("name", ["lattice_576.npz", "cell_ico12.npz"])
def test_noise_free_langevin_trajectory(name):
    g = load_golden(name)
    st = state_from(g, dt=float(g["lang_dt"]), kBT=0.0, eta=float(g["lang_eta"]))
    orc.langevin(st, int(g["lang_steps"]))
    for k, ref in (("x", "lang_x"), ("nrm", "lang_n"), ("v", "lang_v"), ("o", "lang_o")):
        assert rel_l2(getattr(st, k), g[ref]) < 1e-9, k


@pytest.mark.parametrize("name", ["lattice_576.npz", "cell_ico12.npz"])
def test_nose_hoover_trajectory(name):
    g = load_golden(name)
    st = state_from(g, dt=float(g["nh_dt"]), kBT=float(g["nh_kBT"]), Q=0.0, zeta=0.0, bounce=1)
    orc.nh_prologue(st)
    orc.nh_steps(st, int(g["nh_steps"]))
    for k, ref in (("x", "nh_x"), ("nrm", "nh_n"), ("v", "nh_v"), ("o", "nh_o")):
        assert rel_l2(getattr(st, k), g[ref]) < 1e-9, k
    assert abs(st.zeta - float(g["nh_zeta"])) < 1e-9 * max(1.0, abs(float(g["nh_zeta"])))


@pytest.mark.parametrize("name", ["lattice_576.npz", "cell_ico12.npz"])
def test_temperature(name):
    g = load_golden(name)
    th = orc.thermo(state_from(g))
    assert abs(th["temperature"] - float(g["temperature"])) < 1e-12 * float(g["temperature"])


def test_morton_keys_bit_exact():
    g = load_golden("morton.npz")
    assert np.array_equal(orc.morton_encode(g["p"]), g["keys64"])
    assert np.array_equal(orc.morton_encode(g["p32"]), g["keys32"])


def test_morton_aliasing_pinned():
    # bit_space3 (src/reorder_morton.h:25-31) spreads the low 11 bits of x;
    # 2x+2000 = 1024 lands on bit 30, x-inputs >= 2048 alias, and the z word
    # (shifted by 2) loses bit 10 already.
    def raw(v):  # coordinate whose 2x + 2000 equals v
        return (v - 2000.0) / 2.0
    k = orc.morton_encode(np.array([[raw(0), raw(0), raw(0)], [raw(1024), raw(0), raw(0)],
                                    [raw(2048 + 5), raw(0), raw(0)], [raw(5), raw(0), raw(0)],
                                    [raw(0), raw(0), raw(1024 + 3)], [raw(0), raw(0), raw(3)]]))
    assert k[0] == 0 and k[1] == 0x40000000
    assert k[2] == k[3] and k[4] == k[5]


def test_morton_order_is_stable_sort():
    g = load_golden("morton.npz")
    order = orc.morton_order(g["p"])
    keys = g["keys64"]
    ref = np.lexsort((np.arange(len(keys)), keys))
    assert np.array_equal(order, ref)


def test_pair_set_matches_brute_force():
    g = load_golden("cell_ico12.npz")
    st = state_from(g)
    rc2 = np.full(36, 3.0 ** 2)
    pairs = orc.pairs(st, rc2)
    x = st.x
    d2 = ((x[:, None, :] - x[None, :, :]) ** 2).sum(-1)
    iu = np.triu_indices(len(x), 1)
    mask = (d2[iu] < 9.0) & (d2[iu] > 1e-5)
    ref = np.stack([iu[0][mask], iu[1][mask]], 1)
    assert np.array_equal(pairs, ref)


def test_periodic_minimum_image_forces():
    # a lattice that tiles its periodic box: forces are translation invariant
    n = 20
    sp = 1.1
    ix, iy = np.meshgrid(np.arange(n), np.arange(n), indexing="xy")
    x = np.stack([ix.ravel() * sp, iy.ravel() * sp, np.zeros(n * n)], 1)
    rng = np.random.default_rng(0)
    x += rng.normal(0, 0.05, x.shape)
    nrm = np.tile([0.0, 0.0, 1.0], (n * n, 1))
    st = orc.State(x=x, nrm=nrm, v=np.zeros_like(x), o=np.zeros_like(x), type=np.zeros(n * n),
                   tag=np.arange(1, n * n + 1), lo=(0, 0, -10), hi=(n * sp, n * sp, 10), periodic=(1, 1, 0))
    f0, _, _, _ = orc.forces(st)
    st2 = st.copy()
    st2.x[:, 0] = (st2.x[:, 0] + 7.3) % (n * sp)
    f1, _, _, _ = orc.forces(st2)
    assert rel_l2(f1, f0) < 1e-12


def test_noise_is_uniform_and_deterministic():
    r = np.array([orc.noise(1234, s, t) for s in range(20) for t in range(200)])
    assert np.all(r >= -1) and np.all(r < 1)
    assert abs(r.mean()) < 0.02 and abs(r.var() - 1 / 3) < 0.02
    assert np.array_equal(orc.noise(5, 6, 7, 8), orc.noise(5, 6, 7, 8))
    assert not np.array_equal(orc.noise(5, 6, 7, 8), orc.noise(5, 6, 7, 9))


def test_energy_is_minus_gradient():
    g = load_golden("cell_ico12.npz")
    st = state_from(g)
    f, _, e, _ = orc.forces(st, energy=True)
    rng = np.random.default_rng(1)
    for i in rng.choice(st.n, 6, replace=False):
        for d in range(3):
            h = 1e-6
            sp, sm = st.copy(), st.copy()
            sp.x[i, d] += h
            sm.x[i, d] -= h
            ep = orc.forces(sp, energy=True)[2].sum()
            em = orc.forces(sm, energy=True)[2].sum()
            num = -(ep - em) / (2 * h)
            assert abs(num - f[i, d]) < 1e-5 * max(1.0, abs(f[i, d])), (i, d, num, f[i, d])


# ---- the benchmark configurations' own fixtures ------------------------------
def _f64(a):
    return np.asarray(a, np.float64)


def test_example_large_patch_forces_match_reference():
    """A patch of the reference's own whole cell (init_rbc on example-large,
    every particle type it holds, its harmonic spectrin bonds)."""
    g = load_golden("example_large_patch.npz")
    st = orc.State(x=g["x"], nrm=g["nrm"], v=np.zeros_like(g["x"]), o=np.zeros_like(g["x"]), type=g["type"],
                   tag=g["tag"], bonds=g["bonds"])
    f, t, _, _ = orc.forces(st, "f64")
    assert rel_l2(f, g["f64"]) < 1e-12
    assert rel_l2(t, g["t64"]) < 1e-12
    assert g["check"].sum() > 15000 and set(np.unique(g["type"])) == {0, 2, 3, 4, 5}


def test_config1_lattice_matches_reference():
    """The plain small workload (32,768 lipids): forces, temperature and 100
    noise-free Langevin steps against the reference's FP64 code."""
    g = load_golden("lattice_32768.npz")
    st = orc.State(x=_f64(g["x"]), nrm=_f64(g["nrm"]), v=_f64(g["v"]), o=_f64(g["o"]), type=g["type"], tag=g["tag"])
    f, t, _, _ = orc.forces(st, "f64")
    assert rel_l2(f, g["f64"]) < 1e-12
    assert rel_l2(t, g["t64"]) < 1e-12
    f32, t32, _, _ = orc.forces(st, "f32")
    assert rel_l2(f32, g["f32"]) < 2e-5
    T = orc.thermo(st)["temperature"]
    assert abs(T - float(g["temperature"])) < 1e-12 * float(g["temperature"])
    st = orc.State(x=_f64(g["x"]), nrm=_f64(g["nrm"]), v=_f64(g["v"]), o=_f64(g["o"]), type=g["type"], tag=g["tag"],
                   dt=float(g["lang_dt"]), kBT=0.0, eta=float(g["lang_eta"]))
    orc.set_threads(8)
    orc.langevin(st, int(g["lang_steps"]))
    keep = g["lang_keep"]
    x0 = _f64(g["x"])[keep]
    assert rel_l2(st.x[keep] - x0, g["lang_x"] - x0) < 1e-9
    for k, ref in (("nrm", "lang_n"), ("v", "lang_v"), ("o", "lang_o")):
        assert rel_l2(getattr(st, k)[keep], g[ref]) < 1e-9, k
