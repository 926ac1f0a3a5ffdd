"""GPU parity for the velocity rows of the step: zero_bulk_velocity
(src/zero_bulk_velocity.h:29-56, at its call site src/openrbc.cpp:228) and
assign_temperature (src/assign_temperature.h:26-44, src/openrbc.cpp:160),
through the C ABI against the oracle on the same inputs.

Tolerances (relative L2):
  assign_temperature FP64 ............. 1e-12 (FP64 Box-Muller, libm vs CUDA log/sin/cos)
  assign_temperature mixed ............ 1e-7  (stored as FP32)
  zero-bulk Langevin / NH FP64 ........ 1e-9  (10 steps, same counter-based noise)
  zero-bulk Langevin mixed ............ 2e-5  (FP32 state; about 20 times the largest
                                         difference seen on a GB300)
"""
import numpy as np
import pytest

from conftest import load_golden, rel_l2
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

REF_BOX = ((-1000.0, 1000.0),) * 3


def _sim(g, precision, integrator="langevin", kBT=1.0, seed=0xBAD5EED, **kw):
    from openrbc_gb300 import RTParameter, Simulation
    p = RTParameter(init="lipid", kBT=kBT, dt=0.01, eta=0.01, precision=precision, integrator=integrator,
                    rseed=seed)
    s = Simulation(p, skin=0.4, box=REF_BOX, **kw)
    s.upload(g["x"], g["nrm"], g["v"], g["o"], g["type"], g["tag"], g.get("bonds"))
    return s


def _state(g, **kw):
    return orc.State(x=g["x"], nrm=g["nrm"], v=g["v"], o=g["o"], type=g["type"], tag=g["tag"],
                     bonds=g.get("bonds", np.zeros((0, 3), np.int32)), dt=0.01, eta=0.01, **kw)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("mixed", 1e-7)])
def test_assign_temperature_matches_oracle(precision, tol):
    g = load_golden("cell_ico12.npz")
    st = _state(g)
    orc.assign_temperature(st, 0.7, 1234567)
    with _sim(g, precision) as s:
        s.assign_temperature(kBT=0.7, seed=1234567)
        x, n, v, o = s.download()
    assert rel_l2(v, st.v) < tol
    # positions and angular velocities untouched (up to the storage precision)
    assert np.abs(o - g["o"]).max() < 1e-6
    assert np.abs(x - g["x"]).max() < 1e-4


def test_assign_temperature_statistics():
    """v_d = sqrt(2 kT / m) g: the instantaneous temperature sum m v^2 / 3N is
    2 kT (the reference's factor 2), each component has unit-Gaussian shape."""
    from openrbc_gb300 import RTParameter, Simulation, workloads
    w = workloads.lattice(n=65536, ncol=256, kT=0.0, seed=2)
    L = 256 * 1.1
    box = ((0.0, L), (0.0, 256 * 1.1), (-20.0, 20.0))
    p = RTParameter(init="lipid", kBT=0.5, precision="mixed", rseed=99)
    with Simulation(p, box=box, periodic=(1, 1, 0)) as s:
        s.upload(w["x"], w["n"], w["v"], w["o"], w["type"], w["tag"])
        s.assign_temperature()
        th = s.thermo(0)
        _, _, v, _ = s.download()
    assert abs(th["temperature"] - 1.0) < 0.02
    g = v.ravel() / np.sqrt(2 * 0.5)
    assert abs(g.mean()) < 0.01 and abs(g.std() - 1.0) < 0.01
    assert abs((g ** 4).mean() - 3.0) < 0.05      # Gaussian kurtosis


def test_assign_temperature_is_order_independent():
    """The draw is keyed by tag, so permuting the upload order permutes the result."""
    g = load_golden("cell_ico12.npz")
    perm = np.random.default_rng(3).permutation(len(g["x"]))
    h = dict(g)
    for k in ("x", "nrm", "v", "o", "type", "tag"):
        h[k] = np.ascontiguousarray(g[k][perm])
    with _sim(g, "fp64") as s:
        s.assign_temperature(kBT=1.0, seed=5)
        v1 = s.download()[2]
    with _sim(h, "fp64") as s:
        s.assign_temperature(kBT=1.0, seed=5)
        v2 = s.download()[2]
    assert np.array_equal(v1[perm], v2)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-9), ("mixed", 2e-5)])
def test_zero_bulk_langevin_matches_oracle(precision, tol):
    g = load_golden("cell_ico12.npz")
    v0 = g["v"] + np.array([0.3, -0.2, 0.1])   # give the lipids a bulk drift to remove
    h = dict(g)
    h["v"] = v0
    st = _state(h, kBT=1.0, seed=0xBAD5EED, zero_bulk=1)
    orc.langevin(st, 10)
    with _sim(h, precision, zero_bulk=True) as s:
        s.step(10)
        x, n, v, o = s.download()
    assert rel_l2(x - g["x"], st.x - g["x"]) < tol
    assert rel_l2(v, st.v) < tol
    # without the removal the drift survives (the option is really on)
    st2 = _state(h, kBT=1.0, seed=0xBAD5EED)
    orc.langevin(st2, 10)
    assert rel_l2(v, st2.v) > 0.05


def test_zero_bulk_langevin_across_set_state():
    """set_state invalidates the stored lipid mean; the next step recomputes it."""
    g = load_golden("cell_ico12.npz")
    h = dict(g)
    h["v"] = g["v"] + np.array([0.0, 0.5, 0.0])
    st = _state(h, kBT=1.0, seed=0xBAD5EED, zero_bulk=1, step=2)   # the noise counter is at step 2
    orc.langevin(st, 3)
    with _sim(g, "fp64", zero_bulk=True) as s:
        s.step(2)                                  # some other state first
        s.set_state(h["x"], h["nrm"], h["v"], h["o"])
        s.step(3)
        x, n, v, o = s.download()
    assert rel_l2(v, st.v) < 1e-9


def test_zero_bulk_nose_hoover_matches_oracle():
    g = load_golden("lattice_576.npz")
    h = dict(g)
    h["v"] = g["v"] + np.array([0.05, 0.0, -0.05])
    st = _state(h, kBT=0.22, zero_bulk=1)
    orc.nh_prologue(st)
    orc.nh_steps(st, 10)
    with _sim(h, "fp64", integrator="nose-hoover", kBT=0.22, zero_bulk=True) as s:
        th = s.step(10)
        x, n, v, o = s.download()
    assert rel_l2(x - g["x"], st.x - g["x"]) < 1e-9
    assert rel_l2(v, st.v) < 1e-9
    assert abs(th["zeta"] - st.zeta) < 1e-9 * max(1.0, abs(st.zeta))
