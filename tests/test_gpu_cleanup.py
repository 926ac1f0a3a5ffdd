"""GPU stray-lipid cleanup (orbc_gpu_cleanup; delete_lipid,
src/cleanup.h:29-91) against the oracle's marking rule on the same partition
(the grid cells the library reports), and the compaction
that follows: survivors keep their order and renumbering, the run goes on."""
import numpy as np
import pytest

from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def _lattice_with_strays(strays, lift):
    from openrbc_gb300 import workloads
    w = workloads.lattice(n=4096, ncol=64, kT=0.2, seed=11)
    for k, i in enumerate(strays):
        w["x"][i, 2] += lift[k]
    box = ((0.0, 64 * 1.1), (0.0, 64 * 1.1), (-20.0, 20.0))
    return w, box


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_cleanup_removes_exactly_the_strays_like_the_oracle(precision):
    from openrbc_gb300 import RTParameter, Simulation
    strays = [100, 901, 2047, 3000, 4095]
    w, box = _lattice_with_strays(strays, [5.0, 6.0, 9.0, 7.0, 14.0])
    p = RTParameter(init="lipid", kBT=0.2, precision=precision)
    with Simulation(p, box=box, periodic=(1, 1, 0)) as s:
        s.upload(w["x"], w["n"], w["v"], w["o"], w["type"], w["tag"])
        x = s.download()[0]
        c = s.cells(0)
        cell3 = np.stack([c["cell"] & 2047, (c["cell"] >> 11) & 2047, (c["cell"] >> 22) & 1023], 1)
        L3 = [[c["nc"][0] * c["Lc"][0], c["nc"][1] * c["Lc"][1], 0.0]]
        keep, n_ref = orc.cleanup_marks(x, w["type"], cell3, np.zeros(len(x), np.int32), [c["nc"]], L3, mingen=4,
                                        tol=2.5)
        removed = s.cleanup(2.5)
        x2, n2, v2, o2 = s.download()
        th = s.step(20)
    assert set(strays) <= set(np.flatnonzero(~keep).tolist())   # every stray is caught
    assert removed == n_ref
    assert len(x2) == len(x) - removed and th["n"] == len(x2)
    assert np.array_equal(x2, x[keep])          # survivors untouched, renumbered in order
    assert np.isfinite(th["temperature"])


def test_cleanup_on_a_clean_membrane_removes_nothing():
    from openrbc_gb300 import RTParameter, Simulation
    w, box = _lattice_with_strays([], [])
    with Simulation(RTParameter(init="lipid", kBT=0.2, precision="mixed"), box=box, periodic=(1, 1, 0)) as s:
        s.upload(w["x"], w["n"], w["v"], w["o"], w["type"], w["tag"])
        s.step(10)
        before = s.download()
        assert s.cleanup(2.5) == 0
        after = s.download()
    for u, v in zip(before, after):
        assert np.array_equal(u, v)


def test_cleanup_renumbers_survivors_per_system_and_frames_follow(tmp_path):
    from openrbc_gb300 import RTParameter, Simulation, workloads
    from openrbc_gb300.frames import read_frames
    vs = workloads.vesicles(nves=3, nmin=2000, nmax=4000, median=3000, total=9000, kT=0.5, seed=7)
    off = vs["offsets"]
    # throw two lipids of the second vesicle far out of its membrane
    for i in (int(off[1]) + 10, int(off[1]) + 500):
        vs["x"][i] *= 1.6
    gone = {int(vs["tag"][int(off[1]) + 10]), int(vs["tag"][int(off[1]) + 500])}
    with Simulation(RTParameter(init="lipid", kBT=0.5, precision="mixed")) as s:
        s.upload_batch(vs["systems"], vs["x"], vs["n"], vs["v"], vs["o"], vs["type"], vs["tag"], off)
        x0 = s.download()[0]
        cells = [s.cells(k) for k in range(3)]
        removed = s.cleanup(2.5)
        th = [s.thermo(k) for k in range(3)]
        s.step(5)
        path = str(tmp_path / "after.orbc")
        s.save_frame(path, nstep=5, fields=1, append=False)
    # the oracle on each system's partition
    keep = np.ones(len(vs["x"]), bool)
    for k in range(3):
        a, b = int(off[k]), int(off[k + 1])
        c = cells[k]
        sel = c["cell"][a:b]
        cell3 = np.stack([sel & 2047, (sel >> 11) & 2047, (sel >> 22) & 1023], 1)
        L3 = [[c["nc"][d] * c["Lc"][d] for d in range(3)]]           # vesicle boxes are periodic
        kk, _ = orc.cleanup_marks(x0[a:b], vs["type"][a:b], cell3, np.zeros(b - a, np.int32), [c["nc"]], L3,
                                  mingen=4, tol=2.5)
        keep[a:b] = kk
    assert removed == int((~keep).sum()) and gone <= set(vs["tag"][~keep].tolist())
    assert [t["n"] for t in th] == [int(keep[off[k]:off[k + 1]].sum()) for k in range(3)]
    fr = read_frames(path)[0]
    assert fr["natom"] == int(keep.sum())
    assert np.array_equal(np.sort(fr["tag"]), np.sort(vs["tag"][keep]))
