"""Force-loop forms (orbc_params.kernel_variant):

* the merged shell pass (bit 5) adds every pair in the same order as the
  plain pipelined loop, so whole trajectories with list rebuilds are
  bit-identical to it, in both precisions, for every integrator;
* compensated accumulation (bit 6) sums each particle's force and torque
  with Kahan compensation: its FP32 forces are at least as close to the
  reference's FP64 forces as plain FP32 sums, and well inside the 1e-5 bound;
  its trajectories stay within the mixed tolerance of the oracle.
"""
import numpy as np
import pytest

from conftest import load_golden, rel_l2
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

REF_BOX = ((-1000.0, 1000.0),) * 3


def run(w, precision, form, steps, integrator="langevin", box=REF_BOX, periodic=(0, 0, 0), table=None,
        faces=None, constraint=None, skin=0.5, kBT=1.0, energy=False):
    from openrbc_gb300 import RTParameter, Simulation
    p = RTParameter(init="lipid", kBT=kBT, precision=precision, integrator=integrator, rseed=77)
    kw = {"bond_table": table} if table else {}
    with Simulation(p, box=box, periodic=periodic, skin=skin, kernel_variant=form, energy=energy, **kw) as s:
        if faces is not None:
            c = constraint
            sysd = [{"lo": tuple(b[0] for b in box), "hi": tuple(b[1] for b in box), "periodic": periodic,
                     "kv": c["kv"], "V0": c["V0"], "ka": c["ka"], "A0": c["A0"]}]
            s.upload_batch(sysd, w["x"], w["n"], w["v"], w["o"], w["type"], w["tag"], [0, len(w["x"])],
                           bonds=w["bonds"], bond_r0=w["bond_r0"], faces=faces)
        else:
            s.upload(w["x"], w["n"], w["v"], w["o"], w["type"], w["tag"], w.get("bonds"))
        th = s.step(steps)
        return s.download(), th


def cell():
    from openrbc_gb300 import workloads
    return workloads.rbc(n_lipid=30_000, freq=6, kT=1.0, seed=21)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("integrator", ["langevin", "nose-hoover"])
@pytest.mark.parametrize("base", [3 | 16, 7 | 16, 3])
def test_merged_shell_pass_is_bit_identical(precision, integrator, base):
    from openrbc_gb300 import workloads
    if precision == "fp64" and base & 4:
        pytest.skip("the occupancy form is an FP32 form")
    w = cell()
    kw = dict(table=workloads.RBC_BOND_TABLE, faces=w["faces"], constraint=w["constraint"])
    a, tha = run(w, precision, base, 40, integrator, **kw)
    b, thb = run(w, precision, base | 32, 40, integrator, **kw)
    assert tha["rebuilds"] >= 2  # rebuilds happened inside the run
    for u, v in zip(a, b):
        assert np.array_equal(u, v)
    assert tha["zeta"] == thb["zeta"]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("integrator", ["langevin", "nose-hoover"])
@pytest.mark.parametrize("base", [3 | 16 | 64, 7 | 16 | 64])
def test_merged_shell_pass_is_bit_identical_with_compensated_sums(precision, integrator, base):
    """With compensated sums too: in the merged form a warp whose pairs involve
    a protein (the cell's anchors) evaluates its lipid and protein pairs in one
    path, and each pair must still enter the sums exactly as without it."""
    from openrbc_gb300 import workloads
    if precision == "fp64" and base & 4:
        pytest.skip("the occupancy form is an FP32 form")
    w = cell()
    assert (w["type"] != 0).sum() > 100  # anchors in the cell
    kw = dict(table=workloads.RBC_BOND_TABLE, faces=w["faces"], constraint=w["constraint"])
    a, tha = run(w, precision, base, 40, integrator, **kw)
    b, thb = run(w, precision, base | 32, 40, integrator, **kw)
    assert tha["rebuilds"] >= 2
    for u, v in zip(a, b):
        assert np.array_equal(u, v)
    assert tha["zeta"] == thb["zeta"]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("base", [3, 3 | 64])
def test_merged_shell_pass_is_bit_identical_with_every_protein_type(precision, base):
    """The reference's 3,544-particle cell: lipids and band-III, actin,
    spectrin and glycophorin-type particles, so warps meet lipid-protein
    anisotropic pairs, protein-protein repulsion and WCA pairs together; the
    merged form's single anisotropic path must leave every sum as it was."""
    g = load_golden("cell_ico12.npz")
    assert len(set(g["type"].tolist())) >= 5
    w = {"x": g["x"], "n": g["nrm"], "v": g["v"], "o": g["o"], "type": g["type"], "tag": g["tag"],
         "bonds": g["bonds"]}
    a, tha = run(w, precision, base, 30, skin=0.4)
    b, thb = run(w, precision, base | 32, 30, skin=0.4)
    assert tha["rebuilds"] >= 2
    for u, v in zip(a, b):
        assert np.array_equal(u, v)


def test_merged_shell_pass_periodic_lattice_with_energy():
    from openrbc_gb300 import workloads
    w = workloads.lattice(n=6000, ncol=80, kT=1.0, seed=9)
    box = ((0.0, 88.0), (0.0, 75 * 1.1), (-20.0, 20.0))
    a, tha = run(w, "mixed", 3 | 16, 30, box=box, periodic=(1, 1, 0), energy=True)
    b, thb = run(w, "mixed", 35 | 16, 30, box=box, periodic=(1, 1, 0), energy=True)
    for u, v in zip(a, b):
        assert np.array_equal(u, v)
    assert tha["epot"] == thb["epot"]


@pytest.mark.parametrize("name", ["lattice_576.npz", "cell_ico12.npz"])
def test_compensated_forces_vs_reference(name):
    from openrbc_gb300 import RTParameter, Simulation
    g = load_golden(name)
    errs = {}
    for form in (3, 3 | 64):
        p = RTParameter(init="lipid", kBT=0.22, precision="mixed")
        with Simulation(p, box=REF_BOX, kernel_variant=form) as s:
            s.upload(g["x"], g["nrm"], g["v"], g["o"], g["type"], g["tag"], g.get("bonds"))
            f, t, _ = s.forces()
        errs[form] = (rel_l2(f, g["f64"]), rel_l2(t, g["t64"]))
    plain, comp = errs[3], errs[3 | 64]
    assert comp[0] < 1e-5 and comp[1] < 1e-5
    assert comp[0] <= plain[0] * 1.05 + 1e-9 and comp[1] <= plain[1] * 1.05 + 1e-9, errs


def test_compensated_forces_on_a_whole_cell_vs_oracle():
    from openrbc_gb300 import RTParameter, Simulation, workloads
    w = cell()
    st = orc.State(x=w["x"], nrm=w["n"], v=w["v"], o=w["o"], type=w["type"], tag=w["tag"], bonds=w["bonds"],
                   bond_r0=w["bond_r0"], faces=w["faces"], kv=w["constraint"]["kv"], V0=w["constraint"]["V0"],
                   ka=w["constraint"]["ka"], A0=w["constraint"]["A0"])
    st.bstyle[4], st.bK[4], st.br0[4], st.bR[4] = 2, 1.0, 1.0, 2.2
    f_ref, t_ref, _, _ = orc.forces(st)
    errs = {}
    for form in (3 | 16, 3 | 16 | 64):
        p = RTParameter(init="lipid", kBT=1.0, precision="mixed")
        c = w["constraint"]
        with Simulation(p, box=REF_BOX, kernel_variant=form, bond_table=workloads.RBC_BOND_TABLE) as s:
            s.upload_batch([{"lo": (-1000.0,) * 3, "hi": (1000.0,) * 3, "periodic": (0, 0, 0), "kv": c["kv"],
                             "V0": c["V0"], "ka": c["ka"], "A0": c["A0"]}], w["x"], w["n"], w["v"], w["o"],
                           w["type"], w["tag"], [0, len(w["x"])], bonds=w["bonds"], bond_r0=w["bond_r0"],
                           faces=w["faces"])
            f, t, _ = s.forces()
        errs[form] = (rel_l2(f, f_ref), rel_l2(t, t_ref))
    assert errs[3 | 16 | 64][0] < 1e-5 and errs[3 | 16 | 64][1] < 1e-5
    assert errs[3 | 16 | 64][0] <= errs[3 | 16][0] * 1.05 + 1e-9, errs


@pytest.mark.parametrize("form", [3 | 64, 3 | 32 | 64, 7 | 32 | 64])
def test_compensated_langevin_vs_oracle(form):
    """Same counter-based noise on both sides, kT = 1, 10 steps."""
    from openrbc_gb300 import RTParameter, Simulation
    g = load_golden("cell_ico12.npz")
    st = orc.State(x=g["x"], nrm=g["nrm"], v=g["v"], o=g["o"], type=g["type"], tag=g["tag"], bonds=g["bonds"],
                   kBT=1.0, dt=0.01, eta=0.01, seed=0xBAD5EED)
    orc.langevin(st, 10)
    p = RTParameter(init="lipid", kBT=1.0, precision="mixed")
    with Simulation(p, box=REF_BOX, kernel_variant=form, skin=0.4) as s:
        s.upload(g["x"], g["nrm"], g["v"], g["o"], g["type"], g["tag"], g["bonds"])
        s.step(10)
        x, n, v, o = s.download()
    assert rel_l2(x - g["x"], st.x - g["x"]) < 2e-5
    assert rel_l2(v, st.v) < 2e-5
