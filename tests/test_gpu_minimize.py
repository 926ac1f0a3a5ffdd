"""GPU energy minimisation (orbc_gpu_minimize; the loop of
src/openrbc.cpp:88-146) against the oracle's restatement on the same inputs.

Tolerances (relative L2 of the displacement from the start):
  FP64 ........ 1e-9
  mixed ....... 3e-2 (FP32 forces; every step moves a particle by exactly the
                cap along its force, so where the force is small its direction,
                and the path, depend on the last bits) and the final energy
                within 1e-3
"""
import numpy as np
import pytest

from conftest import load_golden, rel_l2
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

REF_BOX = ((-1000.0, 1000.0),) * 3


def _jittered(name, sigma=0.08, seed=1):
    g = load_golden(name)
    x = g["x"] + np.random.default_rng(seed).normal(0.0, sigma, g["x"].shape)
    return dict(g, x=x)


def _sim(g, precision, box=REF_BOX, **kw):
    from openrbc_gb300 import RTParameter, Simulation
    p = RTParameter(init="lipid", precision=precision, dt=0.01)
    s = Simulation(p, box=box, **kw)
    s.upload(g["x"], g["nrm"], g["v"], g["o"], g["type"], g["tag"], g.get("bonds"))
    return s


def _state(g, box=REF_BOX, bounce=1):
    return orc.State(x=g["x"], nrm=g["nrm"], v=g["v"], o=g["o"], type=g["type"], tag=g["tag"],
                     bonds=g.get("bonds", np.zeros((0, 3), np.int32)), lo=tuple(b[0] for b in box),
                     hi=tuple(b[1] for b in box), bounce=bounce, dt=0.01)


@pytest.mark.parametrize("name", ["lattice_576.npz", "cell_ico12.npz"])
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-9), ("mixed", 3e-2)])
def test_minimize_matches_oracle(name, precision, tol):
    g = _jittered(name)
    st = _state(g)
    orc.minimize(st, 40, 0.05, 0.05)
    e_ref = orc.forces(st, energy=True)[2].sum()
    with _sim(g, precision) as s:
        th = s.minimize(40, 0.05, 0.05)
        x, n, v, o = s.download()
        e_gpu = s.forces()[2].sum()
    assert abs(e_gpu - e_ref) < 1e-3 * abs(e_ref)
    assert th["step"] == 0                      # the noise key does not advance
    assert rel_l2(x - g["x"], st.x - g["x"]) < tol
    assert rel_l2(n - g["nrm"], st.nrm - g["nrm"]) < tol
    assert np.abs(np.linalg.norm(n, axis=1) - 1.0).max() < 1e-5


def test_minimize_lowers_the_energy_and_limits_each_move():
    g = _jittered("lattice_576.npz", sigma=0.15, seed=4)
    with _sim(g, "fp64", energy=True) as s:
        _, _, e0 = s.forces()
        x0 = s.download()[0]
        s.minimize(1, 0.02, 0.05)
        x1 = s.download()[0]
        s.minimize(60, 0.02, 0.05)
        _, _, e1 = s.forces()
    assert e1.sum() < e0.sum()
    # one step moves no particle further than dr_max (up to rounding)
    assert np.linalg.norm(x1 - x0, axis=1).max() <= 0.02 * (1 + 1e-9)


def test_minimize_bounces_at_the_walls_like_the_oracle():
    g = _jittered("lattice_576.npz", sigma=0.05, seed=2)
    g["x"][:, 2] *= 0.2
    box = ((-1000.0, 1000.0), (-1000.0, 1000.0), (-0.004, 0.004))
    st = _state(g, box)
    orc.minimize(st, 10, 0.05, 0.05)
    with _sim(g, "fp64", box=box) as s:
        s.minimize(10, 0.05, 0.05)
        x, n, v, o = s.download()
    flipped = np.sign(st.v) != np.sign(g["v"])
    assert flipped.any()                        # some particles did hit a wall
    assert np.array_equal(np.sign(v), np.sign(st.v))
    assert rel_l2(x - g["x"], st.x - g["x"]) < 1e-9
