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


def geodesic_mesh(freq=1):
    """Icosahedron (freq 1) or its geodesic subdivision on the unit sphere:
    vertices, edges (i < j, sorted) and faces counter-clockwise seen from
    outside.  freq 1 with vertices rounded to 9 decimals is the mesh the
    golden whole cell was built from by the reference's init_rbc
    (tests/golden/make_golden.py writes it with %.9f)."""
    t = (1 + 5 ** 0.5) / 2
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t],
                  [0, -1, -t], [0, 1, -t], [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], float)
    v /= np.linalg.norm(v, axis=1)[:, None]
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4],
                  [11, 10, 2], [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8],
                  [3, 8, 9], [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]])
    if freq > 1:
        verts = [tuple(p) for p in v]
        index = {}

        def vid(p):
            q = p / np.linalg.norm(p)
            key = tuple(np.round(q, 12))
            if key not in index:
                index[key] = len(verts)
                verts.append(tuple(q))
            return index[key]
        for k, p in enumerate(v):
            index[tuple(np.round(p, 12))] = k
        faces = []
        for a, b, c in f:
            A, B, C = v[a], v[b], v[c]
            grid = {}
            for i in range(freq + 1):
                for j in range(freq + 1 - i):
                    p = A + (B - A) * i / freq + (C - A) * j / freq
                    grid[i, j] = vid(p)
            for i in range(freq):
                for j in range(freq - i):
                    faces.append((grid[i, j], grid[i + 1, j], grid[i, j + 1]))
                    if i + j < freq - 1:
                        faces.append((grid[i + 1, j], grid[i + 1, j + 1], grid[i, j + 1]))
        v = np.array(verts)
        f = np.array(faces)
    c = v[f].mean(1)
    nn = np.cross(v[f[:, 1]] - v[f[:, 0]], v[f[:, 2]] - v[f[:, 0]])
    flip = np.sum(nn * c, 1) < 0
    f[flip] = f[flip][:, ::-1]
    e = sorted({(min(p, q), max(p, q)) for a, b, cc in f for p, q in ((a, b), (b, cc), (cc, a))})
    if freq == 1:
        v = np.array([[float(f"{x:.9f}") for x in row] for row in v])
    return v, np.array(e, np.int32), f.astype(np.int32)
