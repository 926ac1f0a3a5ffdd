import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) and the CUDA library")


def load_golden(name):
    return dict(np.load(os.path.join(GOLDEN, name), allow_pickle=False))


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    den = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (den if den > 0 else 1.0))


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as orc
    orc.lib()
    return orc


def orbc_frame(nstep, tag, type_, fields, real_bytes, x=None, v=None, n=None, cell=None, f=None):
    """Bytes of one .orbc frame (src/trajectory.h:61-105) for particles given in
    file order (lipids first): the layout the reference's save_frame writes,
    restated independently of the library's writer."""
    import struct
    rdt = np.float32 if real_bytes == 4 else np.float64

    def title(t):
        return t.encode().ljust(8, b"\0")

    out = [title("FRAMEBEG"), struct.pack("<i", int(nstep)), title("NATOM"), struct.pack("<Q", len(tag)),
           title("IDENTITY"), np.stack([tag, type_], 1).astype("<i4").tobytes()]
    for bit, name, arr in ((1, "POSITION", x), (8, "VELOCITY", v), (2, "ROTATION", n), (4, "VORONOI", cell),
                           (16, "FORCE", f)):
        if fields & bit:
            out.append(title(name))
            out.append(np.asarray(arr, np.int32 if bit == 4 else rdt).tobytes())
    out.append(title("FRAMEEND"))
    return b"".join(out)
