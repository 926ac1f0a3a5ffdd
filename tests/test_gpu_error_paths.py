"""Error paths of the step, made on the host with small systems:

* a neighbour list that outgrows its capacity at a rebuild inside a
  multi-step call: the device stops stepping at that build, the library grows
  the list, rebuilds from the current state and runs the remaining steps, so
  the call returns the same state as a run whose capacity was large enough
  from the start (Langevin with and without per-step sums, Nose-Hoover whose
  interrupted step is finished, minimisation, the forces hook);
* a particle placed or drifted outside an open system's grid: the rebuild
  that finds it halts the step, the library re-grids the system from the
  current state and runs the remaining steps; the particle then moves as a
  free particle and the rest of the system as if it were not there.

The overflow is provoked by uploading a sparse lattice into a small list
capacity and then setting a dense state: the builds only ever write inside
the capacity they were given, and report the need."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

BOX = ((-200.0, 200.0), (-200.0, 200.0), (-50.0, 50.0))


def lattices(n=3000, ncol=60):
    from openrbc_gb300 import workloads
    dense = workloads.lattice(n=n, ncol=ncol, spacing=1.1, kT=1.0, seed=31)
    sparse = workloads.lattice(n=n, ncol=ncol, spacing=2.2, kT=1.0, seed=31)
    return sparse, dense


def sim(precision, integrator, cap, energy=False):
    from openrbc_gb300 import RTParameter, Simulation
    p = RTParameter(init="lipid", kBT=1.0, precision=precision, integrator=integrator, rseed=5)
    return Simulation(p, box=BOX, max_neighbors=cap, energy=energy, skin=0.4)


def dense_run(precision, integrator, cap, action, energy=False):
    sparse, dense = lattices()
    with sim(precision, integrator, cap, energy) as s:
        s.upload(sparse["x"], sparse["n"], sparse["v"], sparse["o"], sparse["type"], sparse["tag"])
        th0 = s.thermo()
        s.set_state(dense["x"], dense["n"], dense["v"], dense["o"])
        out = action(s)
        th = s.thermo()
        return out, s.download(), th0, th


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("integrator,energy", [("langevin", False), ("langevin", True), ("nose-hoover", False)])
def test_overflow_inside_a_multi_step_call_is_recovered(precision, integrator, energy):
    tol = 1e-10 if precision == "fp64" else 1e-5
    _, small, th0, th = dense_run(precision, integrator, 16, lambda s: s.step(12), energy)
    _, big, _, thb = dense_run(precision, integrator, 96, lambda s: s.step(12), energy)
    assert th0["capacity"] == 16 and th["capacity"] > 16  # it overflowed and grew
    assert th["step"] == thb["step"] == 12
    for u, v in zip(small, big):
        assert rel_l2(u, v) < tol
    assert abs(th["temperature"] - thb["temperature"]) < tol * thb["temperature"]
    if integrator == "nose-hoover":
        assert abs(th["zeta"] - thb["zeta"]) < tol * max(1.0, abs(thb["zeta"]))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_overflow_in_minimize_and_forces_is_recovered(precision):
    tol = 1e-10 if precision == "fp64" else 1e-5
    f_small, _, _, th = dense_run(precision, "langevin", 16, lambda s: s.forces())
    f_big, _, _, _ = dense_run(precision, "langevin", 96, lambda s: s.forces())
    assert th["capacity"] > 16
    for u, v in zip(f_small[:2], f_big[:2]):
        assert rel_l2(u, v) < tol
    _, small, _, th = dense_run(precision, "langevin", 16, lambda s: s.minimize(6, 0.05, 0.05))
    _, big, _, _ = dense_run(precision, "langevin", 96, lambda s: s.minimize(6, 0.05, 0.05))
    assert th["capacity"] > 16
    for u, v in zip(small, big):
        assert rel_l2(u, v) < tol


def test_particle_outside_an_open_grid_is_regridded():
    """One lipid moved 900 sigma away from the lattice, far beyond the grid's
    margin and every interaction range (noise-free Langevin): the step
    re-grids from the current state and completes, and the run agrees with
    one that uploads the moved state directly."""
    from openrbc_gb300 import RTParameter, Simulation
    _, dense = lattices()

    def noise_free():
        p = RTParameter(init="lipid", kBT=0.0, precision="fp64", rseed=5)
        return Simulation(p, box=BOX, skin=0.4)

    with noise_free() as s:
        s.upload(dense["x"], dense["n"], dense["v"], dense["o"], dense["type"], dense["tag"])
        s.step(3)
        x, n, v, o = s.download()
        x[17] += np.array([900.0, 0.0, 0.0])
        s.set_state(x, n, v, o)
        th = s.step(5)
        assert th["step"] == 8 and not th["flags"]
        got = s.download()
    with noise_free() as s:
        s.upload(x, n, v, o, dense["type"], dense["tag"])
        s.step(5)
        ref = s.download()
    for u, w in zip(got, ref):
        assert rel_l2(u, w) < 1e-12
    assert np.linalg.norm(got[0][17] - x[17]) < 1.0  # a free particle, friction only


def test_forces_after_placing_a_particle_outside_the_grid():
    """forces() re-grids too: the moved particle feels nothing and the others
    feel what they feel without it."""
    _, dense = lattices()
    x = dense["x"].copy()
    keep = np.arange(len(x)) != 17
    with sim("fp64", "langevin", 0) as s:
        s.upload(dense["x"], dense["n"], dense["v"], dense["o"], dense["type"], dense["tag"])
        x[17] += np.array([0.0, 0.0, -700.0])
        s.set_state(x, dense["n"], dense["v"], dense["o"])
        f, t, _ = s.forces()
    assert np.abs(f[17]).max() == 0.0 and np.abs(t[17]).max() == 0.0
    with sim("fp64", "langevin", 0) as s:
        s.upload(x[keep], dense["n"][keep], dense["v"][keep], dense["o"][keep], dense["type"][keep],
                 dense["tag"][keep])
        f2, t2, _ = s.forces()
    assert rel_l2(f[keep], f2) < 1e-12 and rel_l2(t[keep], t2) < 1e-12
