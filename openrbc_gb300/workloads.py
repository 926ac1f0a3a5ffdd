"""Seeded synthetic systems (thin wrappers over include/orbc_workloads.h).

lattice     flat jittered lipid lattice (the plain small workload)
rbc         whole red-cell membrane: Evans-Fung surface, lipids by area,
            geodesic spectrin mesh with WLC-POW bonds and area/volume mesh
vesicles    a batch of spherical vesicles with log-normal sizes

The generators are host code.  Each function takes an optional `lib`: any
ctypes library that exports them (declared with _native.declare_generators);
the default is liborbc_gpu.so, which contains them.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N

# Spectrin spring of the whole-cell workloads: bond type 4, worm-like chain +
# 1/r^2 repulsion balanced at each bond's own rest length, lmax = 2.2 r0.
RBC_BOND_TABLE = {4: {"style": N.BOND_WLC_POW, "K": 1.0, "r0": 1.0, "R": 2.2}}


def _gen(lib):
    return lib if lib is not None else N.lib()


def lattice(n=32768, ncol=182, spacing=1.1, jitter=0.05, tilt=0.05, kT=1.0, seed=1, lib=None):
    x, nn, v, o = (np.zeros((n, 3)) for _ in range(4))
    ty, tg = np.zeros(n, np.int32), np.zeros(n, np.int32)
    rc = _gen(lib).orbc_gen_lattice(n, ncol, spacing, jitter, tilt, kT, seed, x.ctypes.data, nn.ctypes.data,
                                  v.ctypes.data, o.ctypes.data, ty.ctypes.data, tg.ctypes.data)
    if rc:
        raise ValueError("orbc_gen_lattice failed")
    return {"x": x, "n": nn, "v": v, "o": o, "type": ty, "tag": tg}


def rbc(n_lipid=4_000_000, freq=57, kT=1.0, seed=2, reduced_volume=0.64, kv=10.0, ka=10.0, lib=None):
    L = _gen(lib)
    nt, nb, nf = C.c_int64(), C.c_int64(), C.c_int64()
    L.orbc_gen_rbc_counts(n_lipid, freq, C.byref(nt), C.byref(nb), C.byref(nf))
    n = nt.value
    x, nn, v, o = (np.zeros((n, 3)) for _ in range(4))
    ty, tg = np.zeros(n, np.int32), np.zeros(n, np.int32)
    bonds = np.zeros((nb.value, 3), np.int32)
    r0 = np.zeros(nb.value)
    faces = np.zeros((nf.value, 3), np.int32)
    R, A, V = C.c_double(), C.c_double(), C.c_double()
    rc = L.orbc_gen_rbc(n_lipid, freq, kT, seed, x.ctypes.data, nn.ctypes.data, v.ctypes.data, o.ctypes.data,
                        ty.ctypes.data, tg.ctypes.data, bonds.ctypes.data, r0.ctypes.data, faces.ctypes.data,
                        C.byref(R), C.byref(A), C.byref(V))
    if rc:
        raise ValueError("orbc_gen_rbc failed")
    area = A.value
    # target volume at the requested reduced volume v = V / (4/3 pi (A/4pi)^{3/2})
    V0 = reduced_volume * 4.0 / 3.0 * np.pi * (area / (4.0 * np.pi)) ** 1.5
    return {"x": x, "n": nn, "v": v, "o": o, "type": ty, "tag": tg, "bonds": bonds, "bond_r0": r0, "faces": faces,
            "radius": R.value, "area": area, "volume": V.value,
            "constraint": {"kv": kv, "V0": V0, "ka": ka, "A0": area}}


def vesicles(nves=96, nmin=10_000, nmax=250_000, median=40_000, total=5_000_000, kT=1.0, seed=4, rho=1.05,
             lib=None):
    L = _gen(lib)
    sizes = np.zeros(nves, np.int64)
    if L.orbc_gen_vesicle_sizes(nves, nmin, nmax, median, total, seed, sizes.ctypes.data):
        raise ValueError("orbc_gen_vesicle_sizes failed")
    ntot = int(sizes.sum())
    x, nn, v, o = (np.zeros((ntot, 3)) for _ in range(4))
    ty, tg = np.zeros(ntot, np.int32), np.zeros(ntot, np.int32)
    offsets = np.zeros(nves + 1, np.int64)
    offsets[1:] = np.cumsum(sizes)
    systems = []
    for k in range(nves):
        a, b = int(offsets[k]), int(offsets[k + 1])
        R = C.c_double()
        rc = L.orbc_gen_vesicle(b - a, rho, kT, seed * 1000 + k, a + 1, x[a:].ctypes.data, nn[a:].ctypes.data,
                                v[a:].ctypes.data, o[a:].ctypes.data, ty[a:].ctypes.data, tg[a:].ctypes.data,
                                C.byref(R))
        if rc:
            raise ValueError("orbc_gen_vesicle failed")
        half = 1.25 * 2.0 * R.value  # box edge = 2.5 x diameter
        systems.append({"lo": (-half, -half, -half), "hi": (half, half, half), "periodic": (1, 1, 1)})
    return {"x": x, "n": nn, "v": v, "o": o, "type": ty, "tag": tg, "offsets": offsets, "systems": systems,
            "sizes": sizes}


def init_rbc_network(vert, bond, face, rho=1.05, seed=0):
    """The protein network init_rbc builds on a triangulated mesh
    (orbc_init_rbc_network, src/init_rbc.h:66-233; host): rescaled vertices,
    face normals, proteins, bonds and the lipid count of every face."""
    vert = np.ascontiguousarray(vert, np.float64).reshape(-1, 3)
    bond = np.ascontiguousarray(bond, np.int32).reshape(-1, 2)
    face = np.ascontiguousarray(face, np.int32).reshape(-1, 3)
    L = N.lib()
    npr, nb = C.c_int64(), C.c_int64()
    if L.orbc_init_rbc_sizes(len(vert), len(bond), C.byref(npr), C.byref(nb)):
        raise ValueError("orbc_init_rbc_sizes failed")
    x, nn = np.zeros((npr.value, 3)), np.zeros((npr.value, 3))
    ty, tg = np.zeros(npr.value, np.int32), np.zeros(npr.value, np.int32)
    b3 = np.zeros((nb.value, 3), np.int32)
    vs, fn = np.zeros_like(vert), np.zeros((len(face), 3))
    fnl = np.zeros(len(face), np.int64)
    nl = C.c_int64()
    rc = L.orbc_init_rbc_network(vert.ctypes.data, len(vert), bond.ctypes.data, len(bond), face.ctypes.data,
                                 len(face), float(rho), int(seed) & 0xFFFFFFFFFFFFFFFF, vs.ctypes.data,
                                 fn.ctypes.data, x.ctypes.data, nn.ctypes.data, ty.ctypes.data, tg.ctypes.data,
                                 b3.ctypes.data, fnl.ctypes.data, C.byref(nl))
    if rc:
        raise ValueError(f"orbc_init_rbc_network failed ({rc})")
    return {"x": x, "n": nn, "type": ty, "tag": tg, "bonds": b3, "vert": vs, "face": face, "face_normal": fn,
            "face_nl": fnl, "n_lipid": nl.value}


def place_lipids(net, min_dist=0.55, min_dist_lp=1.685, seed=0):
    """Lipid placement of init_rbc on the GPU (orbc_gpu_place_lipids,
    src/init_rbc.h:235-305) for a network from init_rbc_network."""
    L = N.lib()
    nl = int(net["face_nl"].sum())
    x, nn = np.zeros((nl, 3)), np.zeros((nl, 3))
    fnl = np.ascontiguousarray(net["face_nl"], np.int64)
    prot = np.ascontiguousarray(net["x"], np.float64)
    rc = L.orbc_gpu_place_lipids(net["vert"].ctypes.data, len(net["vert"]), net["face"].ctypes.data,
                                 net["face_normal"].ctypes.data, len(net["face"]), fnl.ctypes.data, prot.ctypes.data,
                                 len(prot), float(min_dist), float(min_dist_lp), int(seed) & 0xFFFFFFFFFFFFFFFF,
                                 x.ctypes.data, nn.ctypes.data)
    if rc:
        raise ValueError(f"orbc_gpu_place_lipids failed ({rc})")
    return x, nn


def init_rbc(vert, bond, face, rho=1.05, seed=0):
    """init_rbc (src/init_rbc.h:29-305) on a triangulated mesh: proteins from
    the host network, lipids placed on the GPU; proteins first (tags 1 ..),
    then lipids, zero velocities, as the reference leaves them."""
    net = init_rbc_network(vert, bond, face, rho=rho, seed=seed)
    xl, nl = place_lipids(net, seed=seed)
    npr = len(net["x"])
    x = np.concatenate([net["x"], xl])
    n = np.concatenate([net["n"], nl])
    ty = np.concatenate([net["type"], np.zeros(len(xl), np.int32)])
    tg = np.concatenate([net["tag"], np.arange(npr + 1, npr + 1 + len(xl), dtype=np.int32)])
    return {"x": x, "n": n, "v": np.zeros_like(x), "o": np.zeros_like(x), "type": ty, "tag": tg,
            "bonds": net["bonds"], "n_protein": npr}
