"""GPU pair-distance histogram (orbc_gpu_rdf; src/rdf.h:26-81) against the
oracle's restatement on the same coordinates.  Counts are integers and both
sides round every operation once in the same order, so the histograms are
compared bit for bit."""
import numpy as np
import pytest

from conftest import load_golden
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

REF_BOX = ((-1000.0, 1000.0),) * 3


def _sim(g, precision, box=REF_BOX, periodic=(0, 0, 0)):
    from openrbc_gb300 import RTParameter, Simulation
    p = RTParameter(init="lipid", precision=precision)
    s = Simulation(p, box=box, periodic=periodic)
    s.upload(g["x"], g.get("nrm", g.get("n")), g["v"], g["o"], g["type"], g["tag"], g.get("bonds"))
    return s


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_rdf_all_pairs_bit_exact(precision):
    """The reference's `rdf`: all pairs, dr = 0.1, 10,000 bins."""
    g = load_golden("cell_ico12.npz")
    with _sim(g, precision) as s:
        s.step(5)
        x = s.download()[0]
        counts, dropped = s.rdf()
    ref, counted, ref_drop = orc.rdf(x, g["type"], dr=0.1, nbins=10000, single=precision == "mixed")
    n = len(x)
    assert counted + ref_drop == n * (n - 1) // 2
    assert dropped == ref_drop
    assert np.array_equal(counts, ref)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_rdf_type_filter_and_cutoff_bit_exact(precision):
    """`rdf_1peak_r`: type-4 pairs only, dr = 0.5, r < 25 (51 bins)."""
    g = load_golden("cell_ico12.npz")
    with _sim(g, precision) as s:
        x = s.download()[0]
        counts, dropped = s.rdf(type_a=4, type_b=4, dr=0.5, nbins=51, rcut=25.0)
        mixed_counts, _ = s.rdf(type_a=0, type_b=3, dr=0.25, nbins=40)
    ref, counted, ref_drop = orc.rdf(x, g["type"], 4, 4, dr=0.5, nbins=51, rcut=25.0, single=precision == "mixed")
    assert counted > 0 and np.array_equal(counts, ref) and dropped == ref_drop
    ref2, _, _ = orc.rdf(x, g["type"], 0, 3, dr=0.25, nbins=40, single=precision == "mixed")
    assert np.array_equal(mixed_counts, ref2)
    n4 = int((g["type"] == 4).sum())
    assert counted + ref_drop == n4 * (n4 - 1) // 2


def test_rdf_periodic_minimum_image():
    from openrbc_gb300 import RTParameter, Simulation, workloads
    w = workloads.lattice(n=2048, ncol=32, kT=1.0, seed=8)
    box = ((0.0, 32 * 1.1), (0.0, 64 * 1.1), (-10.0, 10.0))
    with Simulation(RTParameter(init="lipid", precision="mixed"), box=box, periodic=(1, 1, 0)) as s:
        s.upload(w["x"], w["n"], w["v"], w["o"], w["type"], w["tag"])
        s.step(3)
        x = s.download()[0]
        counts, dropped = s.rdf(dr=0.05, nbins=200, rcut=10.0)
    centre = [0.5 * (b[0] + b[1]) for b in box]
    L = (box[0][1] - box[0][0], box[1][1] - box[1][0], 0.0)
    ref, counted, ref_drop = orc.rdf(x, w["type"], dr=0.05, nbins=200, rcut=10.0, centre=centre, L=L, single=True)
    assert np.array_equal(counts, ref) and dropped == ref_drop
    # the first shell sits at the lattice spacing (1.1), also across the seam
    assert 19 <= int(np.argmax(ref[:27])) <= 25


def test_rdf_of_second_system_in_a_batch():
    from openrbc_gb300 import RTParameter, Simulation, workloads
    ves = workloads.vesicles(nves=3, nmin=1500, nmax=6000, median=3000, total=9000, kT=1.0, seed=6)
    with Simulation(RTParameter(init="lipid", precision="fp64")) as s:
        s.upload_batch(ves["systems"], ves["x"], ves["n"], ves["v"], ves["o"], ves["type"], ves["tag"],
                       ves["offsets"])
        x = s.download()[0]
        counts, dropped = s.rdf(sys=1, dr=0.2, nbins=300)
    b, e = ves["offsets"][1], ves["offsets"][2]
    d = ves["systems"][1]
    centre = [0.5 * (d["lo"][k] + d["hi"][k]) for k in range(3)]
    L = [d["hi"][k] - d["lo"][k] for k in range(3)]   # periodic box
    ref, _, ref_drop = orc.rdf(x[b:e], ves["type"][b:e], dr=0.2, nbins=300, centre=centre, L=L)
    assert np.array_equal(counts, ref) and dropped == ref_drop


def test_rdf_rejects_bad_arguments():
    from openrbc_gb300 import OrbcError
    g = load_golden("lattice_576.npz")
    with _sim(g, "mixed") as s:
        for kw in ({"dr": 0.0}, {"nbins": 0}, {"sys": 3}, {"type_a": 9}):
            with pytest.raises(OrbcError):
                s.rdf(**kw)
