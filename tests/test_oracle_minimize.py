"""Oracle (CPU) checks of the energy-minimisation restatement
(src/openrbc.cpp:88-146).  These run without a GPU."""
import numpy as np

from conftest import load_golden
from oracle import oracle as orc


def _jittered_state(sigma, seed, **kw):
    g = load_golden("lattice_576.npz")
    x = g["x"] + np.random.default_rng(seed).normal(0.0, sigma, g["x"].shape)
    return orc.State(x=x, nrm=g["nrm"], v=g["v"], o=g["o"], type=g["type"], tag=g["tag"], **kw)


def test_minimisation_descends_and_keeps_unit_normals():
    st = _jittered_state(0.1, 3)
    e0 = orc.forces(st, energy=True)[2].sum()
    orc.minimize(st, 30, 0.05, 0.05)
    e1 = orc.forces(st, energy=True)[2].sum()
    assert e1 < e0
    assert np.abs(np.linalg.norm(st.nrm, axis=1) - 1.0).max() < 1e-12
    assert st.step == 0


def test_minimisation_step_is_limited():
    st = _jittered_state(0.2, 5)
    x0 = st.x.copy()
    orc.minimize(st, 1, 0.01, 0.05)
    assert np.linalg.norm(st.x - x0, axis=1).max() <= 0.01 * (1 + 1e-12)
