"""Whole-cell initialiser on the GPU (orbc_gpu_place_lipids,
src/init_rbc.h:235-305): the placement equals the oracle's one-attempt-at-a-
time restatement bit for bit, and it builds a cell of millions of lipids in
well under a second (the reference takes seconds on all host cores)."""
import time

import numpy as np
import pytest

from conftest import geodesic_mesh

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("freq,seed", [(1, 0), (1, 7), (3, 2)])
def test_gpu_placement_is_the_oracle_placement(freq, seed):
    from openrbc_gb300 import workloads
    from oracle import oracle as orc
    v, e, f = geodesic_mesh(freq)
    net = workloads.init_rbc_network(v, e, f, rho=1.05, seed=seed)
    xg, ng = workloads.place_lipids(net, seed=seed)
    xo, no = orc.place_lipids(net, seed=seed)
    assert len(xg) == net["n_lipid"] > 0
    assert np.array_equal(xg, xo)
    assert np.array_equal(ng, no)


def test_whole_cell_from_a_large_mesh_steps():
    """A frequency-16 geodesic cell (about 0.9M lipids): built, uploaded with
    the reference's bond table and stepped."""
    from openrbc_gb300 import RTParameter, Simulation, workloads
    v, e, f = geodesic_mesh(16)
    t0 = time.perf_counter()
    w = workloads.init_rbc(v, e, f, rho=1.05, seed=1)
    dt = time.perf_counter() - t0
    npr = w["n_protein"]
    n = len(w["x"])
    print(f"init_rbc: {n} particles ({n - npr} lipids) in {dt:.2f} s")
    assert n - npr > 500_000
    # spot check of the protein exclusion on a sample of lipids
    rng = np.random.default_rng(0)
    prot = w["x"][:npr]
    for k in rng.choice(np.arange(npr, n), 300, replace=False):
        assert np.sqrt(((prot - w["x"][k]) ** 2).sum(1)).min() >= 1.685
    p = RTParameter(init="trimesh", kBT=0.22, precision="mixed")
    with Simulation(p) as s:
        s.upload(w["x"], w["n"], w["v"], w["o"], w["type"], w["tag"], w["bonds"])
        s.minimize(50, 0.01, 0.01)
        th = s.step(10)
    assert np.isfinite(th["temperature"]) and th["n"] == n
