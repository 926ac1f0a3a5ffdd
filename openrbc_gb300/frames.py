"""Reader for trajectory frames in the reference's .orbc layout
(src/trajectory.h:26-150: Serializer / save_frame / read_frame).

A frame is a sequence of sections, each an 8-byte zero-padded title followed
by raw native-endian data:

  FRAMEBEG  int32 step
  NATOM     uint64 particle count N
  IDENTITY  N x (int32 tag, int32 type), lipids first, then proteins
  POSITION  N x 3 real        (dump_field bit 1)
  VELOCITY  N x 3 real        (bit 8)
  ROTATION  N x 3 real        (bit 2)
  VORONOI   N x int32 cell    (bit 4)
  FORCE     N x 3 real        (bit 16)
  FRAMEEND

`real` is float32 in the reference's default build and float64 in its FP64
build; the reader takes it as an argument, as the reference's reader does
through its compile-time `real`.
"""
from __future__ import annotations

from typing import Iterator, List

import numpy as np

DUMP_POSITION, DUMP_ROTATION, DUMP_VORONOI, DUMP_VELOCITY, DUMP_FORCE = 1, 2, 4, 8, 16

_VEC = {"POSITION": "x", "VELOCITY": "v", "ROTATION": "n", "FORCE": "f"}


def iter_frames(data: bytes, real_bytes: int = 4) -> Iterator[dict]:
    """Frames of an .orbc byte string, in order (read_frame, src/trajectory.h:109-150)."""
    rdt = np.float32 if real_bytes == 4 else np.float64
    off, size = 0, len(data)
    frame: dict = {}
    natom = 0
    while off + 8 <= size:
        title = data[off:off + 8].rstrip(b"\0").decode("ascii", "replace")
        off += 8
        if title == "FRAMEBEG":
            frame = {"step": int(np.frombuffer(data, np.int32, 1, off)[0]), "fields": 0}
            off += 4
        elif title == "NATOM":
            natom = int(np.frombuffer(data, np.uint64, 1, off)[0])
            frame["natom"] = natom
            off += 8
        elif title == "IDENTITY":
            ident = np.frombuffer(data, np.int32, 2 * natom, off).reshape(natom, 2)
            frame["tag"], frame["type"] = ident[:, 0].copy(), ident[:, 1].copy()
            off += 8 * natom
        elif title in _VEC:
            nbytes = 3 * natom * real_bytes
            frame[_VEC[title]] = np.frombuffer(data, rdt, 3 * natom, off).reshape(natom, 3).astype(np.float64)
            frame["fields"] |= {"POSITION": DUMP_POSITION, "VELOCITY": DUMP_VELOCITY, "ROTATION": DUMP_ROTATION,
                                "FORCE": DUMP_FORCE}[title]
            off += nbytes
        elif title == "VORONOI":
            frame["cell"] = np.frombuffer(data, np.int32, natom, off).copy()
            frame["fields"] |= DUMP_VORONOI
            off += 4 * natom
        elif title == "FRAMEEND":
            yield frame
            frame = {}
        else:
            raise ValueError(f"unknown section {title!r} at byte {off - 8}")


def read_frames(path: str, real_bytes: int = 4) -> List[dict]:
    """All frames of an .orbc trajectory file."""
    with open(path, "rb") as f:
        return list(iter_frames(f.read(), real_bytes))
