"""Edge cases through the C ABI: malformed topologies are refused with a
status (the reference's rt_assert would exit), the handle stays usable after
a refused call, the neighbour capacity grows when a dense state overflows it
(forces still match the oracle), and ragged batches with very small systems
step like the oracle."""
import numpy as np
import pytest

from conftest import rel_l2
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def _lattice(n=1024, ncol=32, spacing=1.1, seed=3):
    from openrbc_gb300 import workloads
    w = workloads.lattice(n=n, ncol=ncol, spacing=spacing, kT=1.0, seed=seed)
    box = ((0.0, ncol * spacing), (0.0, (n // ncol) * spacing), (-20.0, 20.0))
    return w, box


def _bad_inputs():
    w, _ = _lattice()
    cases = {}
    cases["empty"] = {k: w[k][:0] for k in ("x", "n", "v", "o", "type", "tag")}
    d = {k: w[k].copy() for k in ("x", "n", "v", "o", "type", "tag")}
    d["tag"][5] = d["tag"][6]
    cases["duplicate tag"] = d
    d = {k: w[k].copy() for k in ("x", "n", "v", "o", "type", "tag")}
    d["type"][7] = 6
    cases["type outside 0..5"] = d
    d = {k: w[k].copy() for k in ("x", "n", "v", "o", "type", "tag")}
    d["tag"][3] = -1
    cases["negative tag"] = d
    t = w["tag"]
    for name, b in (("bond to a missing tag", [4, int(t[0]), int(t.max()) + 10]),
                    ("bond to itself", [4, int(t[0]), int(t[0])]),
                    ("bond type outside 0..7", [9, int(t[0]), int(t[1])])):
        d = {k: w[k].copy() for k in ("x", "n", "v", "o", "type", "tag")}
        d["type"][:2] = 3
        d["bonds"] = np.array([b], np.int32)
        cases[name] = d
    return cases


@pytest.mark.parametrize("case", ["empty", "duplicate tag", "type outside 0..5", "negative tag",
                                  "bond to a missing tag", "bond to itself", "bond type outside 0..7"])
def test_malformed_upload_is_refused_and_the_handle_stays_usable(case):
    from openrbc_gb300 import OrbcError, RTParameter, Simulation
    d = _bad_inputs()[case]
    w, _ = _lattice()
    with Simulation(RTParameter(init="lipid", kBT=1.0, precision="mixed")) as s:
        with pytest.raises(OrbcError):
            s.upload(d["x"], d["n"], d["v"], d["o"], d["type"], d["tag"], d.get("bonds"))
        s.upload(w["x"], w["n"], w["v"], w["o"], w["type"], w["tag"])
        th = s.step(5)
    assert th["step"] == 5 and np.isfinite(th["temperature"])


def test_calls_before_upload_and_short_periodic_boxes_are_refused():
    from openrbc_gb300 import OrbcError, RTParameter, Simulation
    w, box = _lattice()
    with Simulation(RTParameter(init="lipid", precision="mixed")) as s:
        with pytest.raises(OrbcError):
            s.step(1)
        with pytest.raises(OrbcError):
            s.download()
    tiny = ((0.0, 6.0), (0.0, 6.0), (-20.0, 20.0))  # shorter than three list cutoffs
    sel = (w["x"][:, 0] < 6.0) & (w["x"][:, 1] < 6.0)
    with Simulation(RTParameter(init="lipid", precision="mixed"), box=tiny, periodic=(1, 1, 0)) as s:
        with pytest.raises(OrbcError):
            s.upload(w["x"][sel], w["n"][sel], w["v"][sel], w["o"][sel], w["type"][sel], w["tag"][sel])


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("mixed", 1e-5)])
def test_neighbour_capacity_grows_past_a_small_start(precision, tol):
    """A lattice at spacing 0.8 has about twice the neighbours of the 1.1
    sheet; starting from a capacity of 16 the library must grow it and still
    produce the oracle's forces and trajectory."""
    from openrbc_gb300 import RTParameter, Simulation
    w, box = _lattice(n=2048, ncol=32, spacing=0.8)
    per = (1, 1, 0)
    lo, hi = tuple(b[0] for b in box), tuple(b[1] for b in box)
    st = orc.State(x=w["x"], nrm=w["n"], v=w["v"], o=w["o"], type=w["type"], tag=w["tag"],
                   bonds=np.zeros((0, 3), np.int32), lo=lo, hi=hi, periodic=per, kBT=1.0, seed=17)
    f_ref, t_ref, _, _ = orc.forces(st)
    with Simulation(RTParameter(init="lipid", kBT=1.0, precision=precision, rseed=17), box=box, periodic=per,
                    max_neighbors=16) as s:
        s.upload(w["x"], w["n"], w["v"], w["o"], w["type"], w["tag"])
        f, t, _ = s.forces()
        th = s.step(5)
        x = s.download()[0]
    assert th["capacity"] > 16 and th["max_neighbors"] > 16
    assert rel_l2(f, f_ref) < tol and rel_l2(t, t_ref) < tol
    orc.langevin(st, 5)
    d = x - w["x"]
    d_ref = st.x - w["x"]
    for k in range(2):
        L = box[k][1] - box[k][0]
        d[:, k] -= L * np.round(d[:, k] / L)
        d_ref[:, k] -= L * np.round(d_ref[:, k] / L)
    assert rel_l2(d, d_ref) < (1e-9 if precision == "fp64" else 2e-5)


def test_ragged_batch_with_tiny_systems_matches_the_oracle():
    """One, two and three-particle systems next to a 1,000-particle sheet:
    each system is padded to its own slot range and steps like the oracle."""
    from openrbc_gb300 import RTParameter, Simulation
    w, box = _lattice(n=1024, ncol=32)
    parts = [(0, 1024)]
    xs = [w["x"]]
    for m, k in ((1, 0), (2, 1), (3, 2)):  # small clusters far from the sheet, each its own system
        xs.append(np.array([[500.0 + 200 * k + 0.9 * j, 500.0, 0.0] for j in range(m)]))
        parts.append((parts[-1][1], parts[-1][1] + m))
    n = parts[-1][1]
    x = np.concatenate(xs)
    rng = np.random.default_rng(4)
    nv = np.concatenate([w["n"], np.tile([0.0, 0.0, 1.0], (n - 1024, 1))])
    v = np.concatenate([w["v"], rng.normal(0, 1, (n - 1024, 3))])
    o = np.concatenate([w["o"], np.zeros((n - 1024, 3))])
    ty = np.zeros(n, np.int32)
    tag = np.arange(1, n + 1, dtype=np.int32)
    systems = [{"lo": (-1000.0,) * 3, "hi": (1000.0,) * 3} for _ in parts]
    offsets = [0] + [b for _, b in parts]
    with Simulation(RTParameter(init="lipid", kBT=1.0, precision="fp64", rseed=9)) as s:
        s.upload_batch(systems, x, nv, v, o, ty, tag, offsets)
        f, t, _ = s.forces()
        s.step(6)
        x1, _, v1, _ = s.download()
    for k, (a, b) in enumerate(parts):
        sub = {"x": x[a:b], "n": nv[a:b], "v": v[a:b], "o": o[a:b], "type": ty[a:b], "tag": tag[a:b]}
        st = orc.State(x=sub["x"], nrm=sub["n"], v=sub["v"], o=sub["o"], type=sub["type"], tag=sub["tag"],
                       bonds=np.zeros((0, 3), np.int32), lo=(-1000.0,) * 3, hi=(1000.0,) * 3,
                       periodic=(0, 0, 0), kBT=1.0, seed=9, sys=k)
        fr, tr, _, _ = orc.forces(st)
        assert np.allclose(f[a:b], fr, rtol=1e-10, atol=1e-12)
        orc.langevin(st, 6)
        assert np.allclose(x1[a:b], st.x, rtol=1e-10, atol=1e-10)
        assert np.allclose(v1[a:b], st.v, rtol=1e-9, atol=1e-10)
