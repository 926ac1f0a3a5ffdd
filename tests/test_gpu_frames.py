"""GPU trajectory frames and checkpoints through the C ABI.

Frames (orbc_gpu_save_frame) must be byte-identical to the restated .orbc
serializer (pinned to the reference's own save_frame by
tests/test_frames_format.py) applied to the state the library reports through
download / forces / cells.  Checkpoints must let a fresh handle continue a run
where it was saved: FP64 to 1e-10, mixed to 1e-4 (relative L2 of the
displacement).
"""
import os

import numpy as np
import pytest

from conftest import load_golden, orbc_frame, rel_l2

pytestmark = pytest.mark.gpu

REF_BOX = ((-1000.0, 1000.0),) * 3


def _sim(g, precision, integrator="langevin", **kw):
    from openrbc_gb300 import RTParameter, Simulation
    p = RTParameter(init="lipid", precision=precision, integrator=integrator, kBT=0.5, rseed=12)
    s = Simulation(p, box=REF_BOX, **kw)
    s.upload(g["x"], g["nrm"], g["v"], g["o"], g["type"], g["tag"], g.get("bonds"))
    return s


def _cell_ids(c):
    """Cell id of each particle from the exported grid (4 x 4 x 4 tiles, Morton inside)."""
    cc = np.stack([c["cell"] & 2047, (c["cell"] >> 11) & 2047, (c["cell"] >> 22) & 1023], 1).astype(np.int64)
    nt = (c["nc"] + 3) // 4
    t, r = cc // 4, cc % 4

    def spread2(v):
        return (v & 1) | ((v & 2) << 2)

    return ((t[:, 0] + nt[0] * (t[:, 1] + nt[1] * t[:, 2])) * 64 +
            (spread2(r[:, 0]) | (spread2(r[:, 1]) << 1) | (spread2(r[:, 2]) << 2))).astype(np.int32)


def _expected(s, g, nstep, fields, real_bytes):
    x, n, v, o = s.download()
    f = s.forces()[0] if fields & 16 else None
    cell = _cell_ids(s.cells(0))
    lip = g["type"] == 0
    order = np.concatenate([np.flatnonzero(lip), np.flatnonzero(~lip)])
    sel = (lambda a: None if a is None else a[order])
    return orbc_frame(nstep, g["tag"][order], g["type"][order], fields, real_bytes, x=x[order], v=v[order],
                      n=n[order], cell=cell[order], f=sel(f))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("real_bytes,fields", [(4, 31), (8, 31), (4, 7)])
def test_frame_bytes_match_the_reference_layout(tmp_path, precision, real_bytes, fields):
    g = load_golden("cell_ico12.npz")
    path = str(tmp_path / "t.orbc")
    with _sim(g, precision) as s:
        s.step(5)
        s.save_frame(path, nstep=5, fields=fields, append=False, real_bytes=real_bytes)
        want = _expected(s, g, 5, fields, real_bytes)
    with open(path, "rb") as fh:
        got = fh.read()
    assert len(got) == len(want)
    assert got == want


def test_async_frames_overlap_stepping_and_arrive_in_order(tmp_path):
    from openrbc_gb300.frames import read_frames
    g = load_golden("cell_ico12.npz")
    path = str(tmp_path / "traj.orbc")
    snaps = []
    with _sim(g, "mixed") as s:
        for k in range(6):
            s.step(4)
            s.save_frame(path, nstep=4 * (k + 1), fields=1 + 2 + 8, append=k > 0, asynchronous=True)
            snaps.append(s.download()[0])
        s.flush()
    fr = read_frames(path)
    assert [f["step"] for f in fr] == [4, 8, 12, 16, 20, 24]
    lip = g["type"] == 0
    order = np.concatenate([np.flatnonzero(lip), np.flatnonzero(~lip)])
    for f, x in zip(fr, snaps):
        assert np.array_equal(f["x"], x[order].astype(np.float32).astype(np.float64))


def test_frame_errors_are_reported(tmp_path):
    from openrbc_gb300 import OrbcError
    g = load_golden("lattice_576.npz")
    with _sim(g, "mixed") as s:
        with pytest.raises(OrbcError):
            s.save_frame(str(tmp_path / "no_such_dir" / "t.orbc"), nstep=0, fields=1)
        with pytest.raises(OrbcError):
            s.save_frame(str(tmp_path / "t.orbc"), nstep=0, fields=64)


@pytest.mark.parametrize("precision,integrator,tol", [("fp64", "langevin", 1e-10), ("fp64", "nose-hoover", 1e-10),
                                                      ("mixed", "langevin", 1e-4)])
def test_checkpoint_restart_continues_the_run(tmp_path, precision, integrator, tol):
    g = load_golden("cell_ico12.npz")
    ck = str(tmp_path / "run.ckpt")
    with _sim(g, precision, integrator) as s:
        s.step(10)
        s.save_checkpoint(ck)
        x_mid = s.download()[0]
        th_a = s.step(10)
        x_a, n_a, v_a, o_a = s.download()
    assert os.path.getsize(ck) > 0
    with _sim(g, precision, integrator) as s:
        s.load_checkpoint(ck)
        th_b = s.step(10)
        x_b, n_b, v_b, o_b = s.download()
    assert th_b["step"] == th_a["step"] == 20
    assert rel_l2(x_b - x_mid, x_a - x_mid) < tol
    assert rel_l2(v_b, v_a) < tol and rel_l2(o_b, o_a) < tol
    if integrator == "nose-hoover":
        assert abs(th_b["zeta"] - th_a["zeta"]) < tol * max(1.0, abs(th_a["zeta"]))


def test_checkpoint_of_another_topology_is_refused(tmp_path):
    from openrbc_gb300 import OrbcError
    ck = str(tmp_path / "a.ckpt")
    g = load_golden("lattice_576.npz")
    with _sim(g, "mixed") as s:
        s.save_checkpoint(ck)
    h = load_golden("cell_ico12.npz")
    with _sim(h, "mixed") as s:
        with pytest.raises(OrbcError):
            s.load_checkpoint(ck)
