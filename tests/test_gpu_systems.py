"""GPU parity on the benchmark-shaped systems: periodic lipid lattice, whole
cell with WLC / FENE spectrin bonds and the area / volume constraint, batched
vesicles; plus determinism, graph / no-graph equivalence, state round trips
and bit-exact binning.  Everything goes through the C ABI and is checked
against the oracle on the same inputs."""
import numpy as np
import pytest

from conftest import rel_l2
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def lattice_sys(n=4096, ncol=64, kT=1.0, seed=5):
    from openrbc_gb300 import workloads
    w = workloads.lattice(n=n, ncol=ncol, kT=kT, seed=seed)
    L = ncol * 1.1
    box = ((0.0, L), (0.0, (n // ncol) * 1.1), (-20.0, 20.0))
    return w, box


def oracle_state(w, box=None, periodic=(0, 0, 0), **kw):
    lo = tuple(b[0] for b in box) if box else (-1000.0,) * 3
    hi = tuple(b[1] for b in box) if box else (1000.0,) * 3
    st = orc.State(x=w["x"], nrm=w["n"], v=w["v"], o=w["o"], type=w["type"], tag=w["tag"],
                   bonds=w.get("bonds", np.zeros((0, 3), np.int32)), bond_r0=w.get("bond_r0"),
                   faces=w.get("faces"), lo=lo, hi=hi, periodic=periodic, **kw)
    return st


def min_image_diff(a, b, box, periodic):
    d = a - b
    for k in range(3):
        if periodic[k]:
            L = box[k][1] - box[k][0]
            d[:, k] -= L * np.round(d[:, k] / L)
    return d


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("mixed", 1e-5)])
def test_periodic_lattice_forces(precision, tol):
    from openrbc_gb300 import RTParameter, Simulation
    w, box = lattice_sys()
    per = (1, 1, 0)
    st = oracle_state(w, box, per)
    f_ref, t_ref, _, _ = orc.forces(st)
    p = RTParameter(init="lipid", kBT=1.0, precision=precision)
    with Simulation(p, box=box, periodic=per) as s:
        s.upload(w["x"], w["n"], w["v"], w["o"], w["type"], w["tag"])
        f, t, _ = s.forces()
    assert rel_l2(f, f_ref) < tol
    assert rel_l2(t, t_ref) < tol


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-9), ("mixed", 1e-5)])
def test_periodic_lattice_langevin(precision, tol):
    from openrbc_gb300 import RTParameter, Simulation
    w, box = lattice_sys()
    per = (1, 1, 0)
    st = oracle_state(w, box, per, kBT=1.0, seed=77)
    orc.langevin(st, 20)
    p = RTParameter(init="lipid", kBT=1.0, precision=precision, rseed=77)
    with Simulation(p, box=box, periodic=per, skin=0.3) as s:
        s.upload(w["x"], w["n"], w["v"], w["o"], w["type"], w["tag"])
        s.step(20)
        x, n, v, o = s.download()
    d_gpu = min_image_diff(x, w["x"], box, per)
    d_ref = min_image_diff(st.x, w["x"], box, per)
    assert rel_l2(d_gpu, d_ref) < tol
    assert rel_l2(v, st.v) < tol


def small_rbc(style="wlc"):
    from openrbc_gb300 import workloads
    w = workloads.rbc(n_lipid=30_000, freq=5, kT=1.0, seed=3)
    if style == "wlc":
        table = {4: {"style": 2, "K": 1.0, "r0": 1.0, "R": 2.2}}
    else:
        table = {4: {"style": 1, "K": 5.0, "r0": 1.0, "R": 6.0}}
    return w, table


def upload_rbc(s, w, with_constraint=True):
    c = w["constraint"] if with_constraint else {"kv": 0, "V0": 0, "ka": 0, "A0": 0}
    sysd = [{"lo": (-1000.0,) * 3, "hi": (1000.0,) * 3, "kv": c["kv"], "V0": c["V0"], "ka": c["ka"], "A0": c["A0"]}]
    s.upload_batch(sysd, w["x"], w["n"], w["v"], w["o"], w["type"], w["tag"], [0, len(w["x"])], bonds=w["bonds"],
                   bond_r0=w["bond_r0"], faces=w["faces"])


def oracle_rbc(w, table, with_constraint=True, **kw):
    st = oracle_state(w, **kw)
    for t, spec in table.items():
        st.bstyle[t], st.bK[t], st.br0[t], st.bR[t] = spec["style"], spec["K"], spec["r0"], spec["R"]
    if with_constraint:
        c = w["constraint"]
        st.kv, st.V0, st.ka, st.A0 = c["kv"], c["V0"], c["ka"], c["A0"]
    return st


@pytest.mark.parametrize("style", ["wlc", "fene"])
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("mixed", 1e-5)])
def test_whole_cell_forces_with_bonds_and_constraint(style, precision, tol):
    from openrbc_gb300 import RTParameter, Simulation
    w, table = small_rbc(style)
    # squeeze the anchors slightly so both constraints are active
    w["constraint"]["V0"] *= 1.02
    w["constraint"]["A0"] *= 0.99
    st = oracle_rbc(w, table)
    f_ref, t_ref, e_ref, th_ref = orc.forces(st, energy=True)
    p = RTParameter(init="lipid", kBT=1.0, precision=precision)
    with Simulation(p, bond_table=table) as s:
        upload_rbc(s, w)
        f, t, e = s.forces()
        th = s.thermo(0)
    assert rel_l2(f, f_ref) < tol
    assert rel_l2(t, t_ref) < tol
    assert abs(e.sum() - e_ref.sum()) < 10 * tol * np.abs(e_ref).sum()
    assert abs(th["area"] - th_ref["area"]) < 1e-9 * th_ref["area"]
    assert abs(th["volume"] - th_ref["volume"]) < 1e-9 * th_ref["volume"]
    # bonded / constrained anchors specifically
    nv = int((w["type"] == 3).sum())
    assert rel_l2(f[:nv], f_ref[:nv]) < 10 * tol


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-9), ("mixed", 1e-5)])
def test_whole_cell_langevin_with_constraint(precision, tol):
    from openrbc_gb300 import RTParameter, Simulation
    w, table = small_rbc("wlc")
    st = oracle_rbc(w, table, kBT=1.0, seed=9)
    th_ref = orc.langevin(st, 10)
    p = RTParameter(init="lipid", kBT=1.0, precision=precision, rseed=9)
    with Simulation(p, bond_table=table) as s:
        upload_rbc(s, w)
        th = s.step(10)
        x, n, v, o = s.download()
    assert rel_l2(x - w["x"], st.x - w["x"]) < tol
    assert rel_l2(v, st.v) < tol
    ref = orc.thermo(st)
    assert abs(th["volume"] - ref["volume"]) < 1e-6 * ref["volume"] or precision == "mixed"


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-9), ("mixed", 1e-5)])
def test_batched_vesicles_match_independent_systems(precision, tol):
    from openrbc_gb300 import RTParameter, Simulation, workloads
    vs = workloads.vesicles(nves=5, nmin=1500, nmax=6000, median=3000, total=15000, kT=1.0, seed=6)
    p = RTParameter(init="lipid", kBT=1.0, precision=precision, rseed=21)
    with Simulation(p) as s:
        s.upload_batch(vs["systems"], vs["x"], vs["n"], vs["v"], vs["o"], vs["type"], vs["tag"], vs["offsets"])
        f, t, _ = s.forces()
        s.step(5)
        x, _, v, _ = s.download()
        th = [s.thermo(k) for k in range(5)]
    for k in range(5):
        a, b = int(vs["offsets"][k]), int(vs["offsets"][k + 1])
        sysd = vs["systems"][k]
        sub = {key: vs[key][a:b] for key in ("x", "n", "v", "o", "type", "tag")}
        box = tuple(zip(sysd["lo"], sysd["hi"]))
        st = oracle_state(sub, box, (1, 1, 1), kBT=1.0, seed=21, sys=k)
        fr, tr, _, _ = orc.forces(st)
        assert rel_l2(f[a:b], fr) < tol
        orc.langevin(st, 5)
        d = min_image_diff(x[a:b], sub["x"], box, (1, 1, 1))
        dr = min_image_diff(st.x, sub["x"], box, (1, 1, 1))
        assert rel_l2(d, dr) < (1e-9 if precision == "fp64" else 2e-5)
        m = 1.0
        T = m * (st.v ** 2).sum() / (3 * (b - a))
        assert abs(th[k]["temperature"] - T) < (1e-9 if precision == "fp64" else 1e-4) * T


def test_graph_and_direct_launch_are_bit_identical():
    from openrbc_gb300 import RTParameter, Simulation
    w, box = lattice_sys(n=8192, ncol=90)
    outs = []
    for graph in (True, False):
        p = RTParameter(init="lipid", kBT=1.0, precision="mixed", rseed=3)
        with Simulation(p, box=box, periodic=(1, 1, 0), use_graph=graph) as s:
            s.upload(w["x"], w["n"], w["v"], w["o"], w["type"], w["tag"])
            th = s.step(37)
            outs.append((s.download(), th))
    (a, tha), (b, thb) = outs
    for u, v in zip(a, b):
        assert np.array_equal(u, v)
    assert tha["rebuilds"] == thb["rebuilds"] and tha["ke2"] == thb["ke2"]


def test_runs_are_deterministic_and_rebuild():
    from openrbc_gb300 import RTParameter, Simulation
    w, box = lattice_sys(n=8192, ncol=90)
    res = []
    for _ in range(2):
        p = RTParameter(init="lipid", kBT=1.0, precision="mixed", rseed=4)
        with Simulation(p, box=box, periodic=(1, 1, 0), skin=0.2) as s:
            s.upload(w["x"], w["n"], w["v"], w["o"], w["type"], w["tag"])
            th = s.step(60)
            res.append((s.download()[0], th))
    assert np.array_equal(res[0][0], res[1][0])
    assert res[0][1]["rebuilds"] > 2  # the skin trigger fired during the run


def test_state_round_trip_and_set_state():
    from openrbc_gb300 import RTParameter, Simulation
    w, box = lattice_sys()
    p = RTParameter(init="lipid", kBT=1.0, precision="fp64")
    with Simulation(p, box=box, periodic=(1, 1, 0)) as s:
        s.upload(w["x"], w["n"], w["v"], w["o"], w["type"], w["tag"])
        x, n, v, o = s.download()
        d = min_image_diff(x, w["x"], box, (1, 1, 0))
        assert np.abs(d).max() < 1e-12
        assert np.abs(n - w["n"]).max() == 0 and np.abs(v - w["v"]).max() == 0
        f0, _, _ = s.forces()
        s.step(10)
        s.set_state(w["x"], w["n"], w["v"], w["o"])
        f1, _, _ = s.forces()
    assert rel_l2(f1, f0) < 1e-12


def test_binning_and_sort_bit_exact():
    """Cells, the cell-sorted slot order and offsets restated from the
    exported grid: cell = floor((x - lo) / Lc), offset = x - centre."""
    from openrbc_gb300 import RTParameter, Simulation
    w, box = lattice_sys(n=6000, ncol=77)
    per = (1, 1, 0)
    p = RTParameter(init="lipid", kBT=1.0, precision="fp64")
    with Simulation(p, box=box, periodic=per) as s:
        s.upload(w["x"], w["n"], w["v"], w["o"], w["type"], w["tag"])
        c = s.cells(0)
    lo, Lc, nc = c["lo"], c["Lc"], c["nc"]
    x = w["x"]
    cu = np.floor((x - lo) / Lc).astype(np.int64)
    cc = cu.copy()
    for d in range(3):
        if per[d]:
            cc[:, d] %= nc[d]
        else:
            cc[:, d] = np.clip(cu[:, d], 0, nc[d] - 1)
    packed = cc[:, 0] | (cc[:, 1] << 11) | (cc[:, 2] << 22)
    assert np.array_equal(c["cell"], packed.astype(np.int32))
    ref = np.where(np.array(per)[None, :] == 1, cu, cc)
    off = x - (lo + (ref + 0.5) * Lc)
    assert np.array_equal(c["offset"], off)
    # slots are the stable order by (cell id, upload index) within the system; the
    # cell id walks 4 x 4 x 4 tiles of cells row-major, Morton order inside a tile
    nt = (nc + 3) // 4
    t = cc // 4
    r = cc % 4

    def spread2(v):
        return (v & 1) | ((v & 2) << 2)

    cid = (t[:, 0] + nt[0] * (t[:, 1] + nt[1] * t[:, 2])) * 64 + (spread2(r[:, 0]) | (spread2(r[:, 1]) << 1) |
                                                                  (spread2(r[:, 2]) << 2))
    order = np.lexsort((np.arange(len(cid)), cid))
    assert np.array_equal(np.argsort(c["slot"]), order)


def test_nose_hoover_mixed_tracks_fp64():
    from openrbc_gb300 import RTParameter, Simulation
    w, box = lattice_sys()
    res = {}
    for prec in ("fp64", "mixed"):
        p = RTParameter(init="lipid", kBT=1.0, precision=prec, integrator="nose-hoover")
        with Simulation(p, box=box, periodic=(1, 1, 0)) as s:
            s.upload(w["x"], w["n"], w["v"], w["o"], w["type"], w["tag"])
            res[prec] = s.step(50)
    assert abs(res["mixed"]["zeta"] - res["fp64"]["zeta"]) < 1e-3 * max(1e-3, abs(res["fp64"]["zeta"]))
    assert abs(res["mixed"]["temperature"] - res["fp64"]["temperature"]) < 1e-3 * res["fp64"]["temperature"]


@pytest.mark.parametrize("variant", [1, 2, 3, 4, 7, 8, 15, 16, 19, 23])
def test_force_kernel_forms_agree(variant):
    """The force-kernel forms evaluate the same pairs in the same order; the
    three list-build forms (bits 3-4) find the same pairs."""
    from openrbc_gb300 import RTParameter
    from openrbc_gb300 import Simulation
    w, table = small_rbc("wlc")
    out = {}
    for v in (0, variant):
        p = RTParameter(init="lipid", kBT=1.0, precision="mixed", rseed=5)
        with Simulation(p, bond_table=table, kernel_variant=v) as s:
            upload_rbc(s, w)
            f, t, _ = s.forces()
            s.step(20)
            out[v] = (f, s.download()[0])
    assert rel_l2(out[variant][0], out[0][0]) < 1e-6
    assert rel_l2(out[variant][1] - w["x"], out[0][1] - w["x"]) < 1e-4


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_list_build_forms_find_the_same_pairs(precision):
    """The three list-build forms write the same rows (same entries, same
    order) on the open whole cell and on a periodic sheet."""
    from openrbc_gb300 import RTParameter, Simulation
    w, table = small_rbc("wlc")
    lat, box = lattice_sys(n=8192, ncol=90)
    for case in ("cell", "sheet"):
        sets = []
        for v in (0, 8, 16):
            p = RTParameter(init="lipid", kBT=1.0, precision=precision, rseed=5)
            if case == "cell":
                with Simulation(p, bond_table=table, kernel_variant=v) as s:
                    upload_rbc(s, w)
                    s.step(7)
                    s.set_state(w["x"], w["n"], w["v"], w["o"])
                    s.rebuild()
                    sets.append(s.neighbors())
            else:
                with Simulation(p, box=box, periodic=(1, 1, 0), kernel_variant=v) as s:
                    s.upload(lat["x"], lat["n"], lat["v"], lat["o"], lat["type"], lat["tag"])
                    s.step(9)
                    s.rebuild()
                    sets.append(s.neighbors())
        for counts, lst in sets[1:]:
            assert np.array_equal(sets[0][0], counts)
            assert np.array_equal(sets[0][1], lst)


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
@pytest.mark.parametrize("density", [0.15, 0.9])
def test_list_build_forms_on_periodic_3d_gases(precision, density):
    """Uniform gases in a periodic cube, against brute-force minimum-image
    pairs.  At density 0.15 a warp's 32 particles span about seven cells of
    about 150 candidates each, more than form 2 keeps staged at once; at 0.9
    every cell has more than 256 candidates and form 2 takes them in chunks.
    The three forms must still write the same rows."""
    from openrbc_gb300 import RTParameter, Simulation
    n, skin = 4000, 0.4
    L = (n / density) ** (1.0 / 3.0)
    rng = np.random.default_rng(21)
    x = rng.uniform(0.0, L, (n, 3))
    nv = rng.normal(size=(n, 3))
    nv /= np.linalg.norm(nv, axis=1, keepdims=True)
    zero = np.zeros((n, 3))
    ty = np.zeros(n, np.int32)
    tag = np.arange(1, n + 1, dtype=np.int32)
    sets = []
    for v in (0, 8, 16):
        p = RTParameter(init="lipid", kBT=1.0, precision=precision, rseed=5)
        with Simulation(p, box=((0.0, L),) * 3, periodic=(1, 1, 1), skin=skin, kernel_variant=v) as s:
            s.upload(x, nv, zero, zero, ty, tag)
            sets.append(s.neighbors())
    for counts, lst in sets[1:]:
        assert np.array_equal(sets[0][0], counts)
        assert np.array_equal(sets[0][1], lst)
    counts, lst = sets[0]
    rl2 = (2.6 + skin) ** 2
    ref = set()
    for a in range(0, n, 500):
        d = x[a:a + 500, None, :] - x[None, :, :]
        d -= L * np.round(d / L)
        r2 = (d * d).sum(-1)
        ii, jj = np.nonzero(r2 < rl2)
        ref.update((int(i) + a, int(j)) for i, j in zip(ii, jj) if int(i) + a != int(j))
    rows = np.repeat(np.arange(n), counts)
    got = set(zip(rows.tolist(), lst.tolist()))
    assert len(got) == len(lst)  # no pair twice
    tol = 1e-9 if precision == "fp64" else 2e-6
    for i, j in got ^ ref:  # only pairs on the cutoff sphere may differ
        d = x[i] - x[j]
        d -= L * np.round(d / L)
        assert abs((d * d).sum() - rl2) < tol * rl2, (i, j)


def test_autotune_restores_state_and_keeps_stepping():
    from openrbc_gb300 import RTParameter, Simulation
    w, box = lattice_sys(n=8192, ncol=90)
    p = RTParameter(init="lipid", kBT=1.0, precision="mixed", rseed=8)
    with Simulation(p, box=box, periodic=(1, 1, 0)) as s:
        s.upload(w["x"], w["n"], w["v"], w["o"], w["type"], w["tag"])
        s.step(5)
        before = s.download()
        step0 = s.thermo()["step"]
        trials = s.autotune(trial_steps=4)
        after = s.download()
        # 3 list-build forms, 5 skins x 5 loop forms, 2 skins, the occupancy form, 2 list-build forms,
        # 2 rebuild cadences
        assert len(trials) == 35 and all(t["ms_per_step"] > 0 for t in trials)
        assert {(t["variant"] >> 3) & 3 for t in trials} == {0, 1, 2}
        assert {t["rebuild_every"] for t in trials} == {0, 5, 10}
        assert any(t["variant"] & 32 for t in trials)
        assert s.thermo()["step"] == step0
        d = min_image_diff(after[0], before[0], box, (1, 1, 0))
        assert np.abs(d).max() < 1e-5
        for u, v in zip(after[1:], before[1:]):
            assert np.abs(u - v).max() < 1e-6
        th = s.step(10)
        assert th["step"] == step0 + 10 and np.isfinite(th["temperature"])


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("rebuild_every", [1, None])
def test_batched_cell_ensemble_matches_each_cell_alone(precision, rebuild_every):
    """Whole-cell ensemble (several red cells, each with its own spectrin
    network and its own volume target) in one handle: every cell evolves as it
    does alone (Nose-Hoover, no noise), with its own thermostat, area and
    volume.  The batch shares one rebuild decision (a rebuild re-sorts every
    cell, which reorders the force sums of the cells that did not need it), so
    with a list rebuilt every step the runs agree bit for bit, and with the
    displacement rule to rounding."""
    from openrbc_gb300 import RTParameter, Simulation, workloads
    table = {4: {"style": 2, "K": 1.0, "r0": 1.0, "R": 2.2}}
    cells, base = [], 0
    for k, vf in enumerate((0.97, 1.0, 1.03)):
        w = workloads.rbc(n_lipid=20_000, freq=5, kT=1.0, seed=40 + k)
        shift = base - int(w["tag"].min())
        w["tag"] = w["tag"] + shift
        w["bonds"] = w["bonds"].copy()
        w["bonds"][:, 1:] += shift
        w["faces"] = w["faces"] + shift
        base = int(w["tag"].max()) + 1
        c = dict(w["constraint"])
        c["V0"] *= vf
        cells.append((w, {"lo": (-1000.0,) * 3, "hi": (1000.0,) * 3, "kv": c["kv"], "V0": c["V0"],
                          "ka": c["ka"], "A0": c["A0"]}))

    def run(group):
        p = RTParameter(init="lipid", kBT=1.0, precision=precision, integrator="nose-hoover")
        cat = lambda key: np.concatenate([w[key] for w, _ in group])
        off = np.cumsum([0] + [len(w["x"]) for w, _ in group])
        with Simulation(p, bond_table=table, rebuild_every=rebuild_every) as s:
            s.upload_batch([d for _, d in group], cat("x"), cat("n"), cat("v"), cat("o"), cat("type"), cat("tag"),
                           off, bonds=cat("bonds"), bond_r0=cat("bond_r0"), faces=cat("faces"))
            s.step(12)
            return s.download(), [s.thermo(k) for k in range(len(group))], off

    state, th, off = run(cells)
    tol = 0.0 if rebuild_every == 1 else (1e-12 if precision == "fp64" else 1e-5)
    for k in range(len(cells)):
        alone, th1, _ = run([cells[k]])
        a, b = int(off[k]), int(off[k + 1])
        w = cells[k][0]
        if tol == 0.0:
            for u, v in zip(state, alone):
                assert np.array_equal(u[a:b], v)
        else:
            assert rel_l2(state[0][a:b] - w["x"], alone[0] - w["x"]) < tol
            assert rel_l2(state[2][a:b], alone[2]) < tol
        for key in ("zeta", "ke2", "area", "volume"):
            assert abs(th[k][key] - th1[0][key]) <= tol * max(1.0, abs(th1[0][key]))
    assert len({t["volume"] for t in th}) == len(cells)  # the volume targets differ
