"""Error paths of the step, made on the host with small systems:

* a neighbour list that outgrows its capacity at a rebuild inside a
  multi-step call: the device stops stepping at that build, the library grows
  the list, rebuilds from the current state and runs the remaining steps, so
  the call returns the same state as a run whose capacity was large enough
  from the start (Langevin with and without per-step sums, Nose-Hoover whose
  interrupted step is finished, minimisation, the forces hook);
* a particle that leaves an open system's grid makes step / minimize /
  forces return ORBC_ERR_GRID, and keeps doing so until the next upload.

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


def test_particle_leaving_an_open_grid_is_an_error_until_upload():
    from openrbc_gb300 import OrbcError
    _, dense = lattices()
    with sim("mixed", "langevin", 0) as s:
        s.upload(dense["x"], dense["n"], dense["v"], dense["o"], dense["type"], dense["tag"])
        s.step(3)
        x, n, v, o = s.download()
        x[17] += np.array([900.0, 0.0, 0.0])  # far beyond the grid's margin
        s.set_state(x, n, v, o)
        with pytest.raises(OrbcError) as ei:
            s.step(1)
        assert ei.value.code == 5  # ORBC_ERR_GRID
        assert s.thermo()["flags"] & (1 << 5)
        with pytest.raises(OrbcError) as ei:
            s.forces()
        assert ei.value.code == 5
        # a fresh upload clears it
        s.upload(dense["x"], dense["n"], dense["v"], dense["o"], dense["type"], dense["tag"])
        th = s.step(2)
        assert th["step"] == 2 and not th["flags"]
