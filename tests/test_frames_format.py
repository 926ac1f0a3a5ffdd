"""The .orbc frame layout (src/trajectory.h:61-105), pinned to frames written
by the reference's own save_frame (tests/golden/frames.npz, made by
tests/golden/make_golden.py): the restated serializer in conftest reproduces
them byte for byte, and the package's reader parses them.  No GPU needed."""
import numpy as np
import pytest

from conftest import load_golden, orbc_frame


def _file_order(type_):
    lip = type_ == 0
    return np.concatenate([np.flatnonzero(lip), np.flatnonzero(~lip)])


@pytest.mark.parametrize("key,real_bytes,fields,nstep", [("frame_f32_31_120", 4, 31, 120),
                                                          ("frame_f64_31_120", 8, 31, 120),
                                                          ("frame_f32_7_0", 4, 7, 0)])
def test_serializer_reproduces_reference_frames(key, real_bytes, fields, nstep):
    g = load_golden("frames.npz")
    o = _file_order(g["type"])
    ref = bytes(g[key])
    mine = orbc_frame(nstep, g["tag"][o], g["type"][o], fields, real_bytes, x=g["x"][o], v=g["v"][o],
                      n=g["nrm"][o], cell=g["affil"][o], f=g["f"][o])
    assert mine == ref


def test_reader_parses_reference_frames():
    from openrbc_gb300.frames import iter_frames
    g = load_golden("frames.npz")
    o = _file_order(g["type"])
    fr = list(iter_frames(bytes(g["frame_f64_31_120"]) * 2, real_bytes=8))
    assert len(fr) == 2 and fr[1]["step"] == 120 and fr[0]["natom"] == len(o) and fr[0]["fields"] == 31
    assert np.array_equal(fr[0]["tag"], g["tag"][o]) and np.array_equal(fr[0]["type"], g["type"][o])
    assert np.array_equal(fr[0]["x"], g["x"][o]) and np.array_equal(fr[0]["cell"], g["affil"][o])
    assert np.array_equal(fr[0]["f"], g["f"][o])
