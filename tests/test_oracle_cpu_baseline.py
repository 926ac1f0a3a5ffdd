"""The timed CPU baseline (orc_run_langevin_fast_f32: cell-sorted particles,
Verlet list, Newton's third law inside each thread's range) computes the same
FP32 Langevin step as the oracle's plain restatement: after a few steps with
the same counter-based noise the two agree to FP32 rounding of the summation
order, on an open whole cell (bonds, area / volume constraint) and on a
periodic lattice."""
import numpy as np
import pytest

from conftest import rel_l2
from oracle import oracle as orc


def _cell_state():
    from openrbc_gb300 import workloads
    w = workloads.rbc(n_lipid=12000, freq=6, kT=1.0, seed=2, lib=orc.workloads_lib())
    st = orc.State(x=w["x"], nrm=w["n"], v=w["v"], o=w["o"], type=w["type"], tag=w["tag"], bonds=w["bonds"],
                   bond_r0=w["bond_r0"], faces=w["faces"], kBT=1.0, dt=0.01, eta=0.01, seed=11,
                   kv=w["constraint"]["kv"], V0=w["constraint"]["V0"], ka=w["constraint"]["ka"],
                   A0=w["constraint"]["A0"])
    st.bstyle[4], st.bK[4], st.br0[4], st.bR[4] = 2, 1.0, 1.0, 2.2
    return st


def _lattice_state():
    from openrbc_gb300 import workloads
    w = workloads.lattice(n=4096, ncol=64, kT=1.0, seed=3, lib=orc.workloads_lib())
    return orc.State(x=w["x"], nrm=w["n"], v=w["v"], o=w["o"], type=w["type"], tag=w["tag"], kBT=1.0, dt=0.01,
                     eta=0.01, seed=12, lo=(-0.55, -0.55, -20.0), hi=(64 * 1.1 - 0.55, 64 * 1.1 - 0.55, 20.0),
                     periodic=(1, 1, 0))


@pytest.mark.parametrize("make", [_cell_state, _lattice_state])
@pytest.mark.parametrize("threads", [1, 4])
def test_cpu_baseline_matches_the_plain_restatement(make, threads):
    orc.set_threads(threads)
    a, b, ref = make(), make(), make()
    x0 = a.x.copy()
    orc.langevin(a, 6, "f32")
    th = orc.cpu_baseline_run(b, 6, 0.4)
    orc.langevin(ref, 6, "f64")
    assert th["npairs"] >= 1
    # both FP32 runs sit at the same distance from FP64, and much closer to each other
    e_plain = rel_l2(a.x - x0, ref.x - x0)
    e_fast = rel_l2(b.x - x0, ref.x - x0)
    assert e_fast < 2 * e_plain + 1e-6
    assert rel_l2(b.x - x0, a.x - x0) < 1e-4
    assert rel_l2(b.v, a.v) < 1e-4
    assert rel_l2(b.nrm, a.nrm) < 1e-6
    assert b.step == a.step == 6
