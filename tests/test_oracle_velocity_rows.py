"""Oracle (CPU) checks of the velocity rows: zero_bulk_velocity
(src/zero_bulk_velocity.h:29-56) and assign_temperature
(src/assign_temperature.h:26-44).  These run without a GPU."""
import numpy as np

from conftest import load_golden
from oracle import oracle as orc


def _state(g, **kw):
    return orc.State(x=g["x"], nrm=g["nrm"], v=g["v"], o=g["o"], type=g["type"], tag=g["tag"],
                     bonds=g.get("bonds", np.zeros((0, 3), np.int32)), **kw)


def test_assign_temperature_gives_twice_kT():
    """The reference draws sqrt(2 kT / m) g per component, so the measured
    temperature sum m v^2 / 3N is 2 kT."""
    n = 40000
    x = np.zeros((n, 3))
    x[:, 0] = np.arange(n) * 3.0 - 1000.0 + 0.5
    st = orc.State(x=x, nrm=np.tile([0.0, 0.0, 1.0], (n, 1)), v=np.zeros((n, 3)), o=np.zeros((n, 3)),
                   type=np.zeros(n, np.int32), tag=np.arange(n, dtype=np.int32))
    orc.assign_temperature(st, 0.35, 11)
    T = (st.v ** 2).sum() / (3 * n)
    assert abs(T / 0.7 - 1.0) < 0.02
    g = st.v.ravel() / np.sqrt(0.7)
    assert abs(g.mean()) < 0.01 and abs(g.std() - 1.0) < 0.01


def test_assign_temperature_uses_mass_and_tag():
    g = load_golden("cell_ico12.npz")
    a = _state(g)
    orc.assign_temperature(a, 1.0, 5)
    b = _state(g)
    orc.assign_temperature(b, 1.0, 5)
    assert np.array_equal(a.v, b.v)                      # deterministic
    c = _state(g)
    orc.assign_temperature(c, 1.0, 6)
    assert not np.array_equal(a.v, c.v)                  # keyed by the seed
    m = np.array([1.0, 4.0, 4.0, 1.0, 10.0, 10.0])[g["type"]]
    heavy, light = m == 10.0, m == 1.0
    # per-particle scale sqrt(2 kT / m): heavy particles move sqrt(10) slower on average
    r = np.sqrt((a.v[light] ** 2).mean() / (a.v[heavy] ** 2).mean())
    assert 2.0 < r < 5.0


def test_zero_bulk_removes_lipid_drift():
    """With noise off and only lipids, the pair forces sum to zero, so the
    lipid mean after a step is the removed drift times nothing: ~0."""
    g = load_golden("lattice_576.npz")
    v = g["v"] + np.array([0.4, -0.3, 0.2])
    on = _state(dict(g, v=v), kBT=0.0, zero_bulk=1)
    orc.langevin(on, 1)
    off = _state(dict(g, v=v), kBT=0.0, zero_bulk=0)
    orc.langevin(off, 1)
    assert np.abs(on.v[on.type == 0].mean(0)).max() < 1e-12
    assert np.abs(off.v[off.type == 0].mean(0)).max() > 0.1
