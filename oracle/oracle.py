"""TEST INFRASTRUCTURE ONLY -- Python binding of the oracle.

ctypes binding of ``liborbc_oracle.so`` (the CPU restatement in
``orbc_oracle.cpp``) and of the reference harness in ``_ref/`` (built from the
reference's own headers where its source tree is present).  Only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU baseline / reference arm
import this module; the shipped package never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liborbc_oracle.so")
LIB_FAST = os.path.join(HERE, "liborbc_oracle_fast.so")
LIB_WORKLOADS = os.path.join(HERE, "liborbc_workloads.so")
REF_DIR = os.path.join(HERE, "_ref")

BOND_HARMONIC, BOND_FENE, BOND_WLC_POW = 0, 1, 2
MAX_BOND_TYPES = 8

_lock = threading.Lock()
_lib = None
_lib_fast = None
_ref = {}
_workloads = None


def build(ref_src: Optional[str] = None) -> None:
    """Compile the oracle, and the reference harness when the reference's
    source directory is given (argument, or the ORBC_REF_SRC environment
    variable) and exists."""
    subprocess.run(["make", "-s", "-C", HERE, "liborbc_oracle.so", "liborbc_oracle_fast.so", "liborbc_workloads.so"],
                   check=True)
    src = ref_src or os.environ.get("ORBC_REF_SRC")
    if src and os.path.isdir(src):
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={src}"], check=True,
                       stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)


class OrcSystemC(C.Structure):
    _fields_ = [
        ("n", C.c_int64),
        ("x", C.c_void_p), ("nrm", C.c_void_p), ("v", C.c_void_p), ("o", C.c_void_p),
        ("f", C.c_void_p), ("t", C.c_void_p),
        ("type", C.c_void_p), ("tag", C.c_void_p),
        ("nb", C.c_int64), ("bonds", C.c_void_p), ("bond_r0", C.c_void_p),
        ("nface", C.c_int64), ("faces", C.c_void_p),
        ("lo", C.c_double * 3), ("hi", C.c_double * 3), ("periodic", C.c_int * 3),
        ("dt", C.c_double), ("kBT", C.c_double), ("eta", C.c_double),
        ("zeta", C.c_double), ("Q", C.c_double),
        ("seed", C.c_uint64), ("step", C.c_int64), ("sys", C.c_int), ("bounce", C.c_int),
        ("zero_bulk", C.c_int),
        ("kv", C.c_double), ("V0", C.c_double), ("ka", C.c_double), ("A0", C.c_double),
        ("bstyle", C.c_int * MAX_BOND_TYPES), ("bK", C.c_double * MAX_BOND_TYPES),
        ("br0", C.c_double * MAX_BOND_TYPES), ("bR", C.c_double * MAX_BOND_TYPES),
    ]


class OrcThermoC(C.Structure):
    _fields_ = [("ke2", C.c_double), ("temperature", C.c_double), ("area", C.c_double),
                ("volume", C.c_double), ("epot", C.c_double), ("npairs", C.c_int64),
                ("flags", C.c_int)]


def reference_bond_table():
    """Bond types 0..3 of src/forcefield_canonical.h:106-109 (harmonic, K=57)."""
    style = np.zeros(MAX_BOND_TYPES, np.int32)
    K = np.full(MAX_BOND_TYPES, 57.0)
    r0 = np.ones(MAX_BOND_TYPES)
    r0[:4] = [2.25, 1.1225, 2.25, 2.24]
    R = np.zeros(MAX_BOND_TYPES)
    return style, K, r0, R


@dataclass
class State:
    """Particle state in the caller's order (AoS float64 like the C ABI)."""
    x: np.ndarray
    nrm: np.ndarray
    v: np.ndarray
    o: np.ndarray
    type: np.ndarray
    tag: np.ndarray
    bonds: np.ndarray = field(default_factory=lambda: np.zeros((0, 3), np.int32))
    bond_r0: Optional[np.ndarray] = None
    faces: Optional[np.ndarray] = None
    lo: tuple = (-1000.0, -1000.0, -1000.0)
    hi: tuple = (1000.0, 1000.0, 1000.0)
    periodic: tuple = (0, 0, 0)
    dt: float = 0.01
    kBT: float = 0.22
    eta: float = 0.01
    zeta: float = 0.0
    Q: float = 0.0
    seed: int = 0
    step: int = 0
    sys: int = 0
    bounce: int = 0
    zero_bulk: int = 0
    kv: float = 0.0
    V0: float = 0.0
    ka: float = 0.0
    A0: float = 0.0
    bstyle: np.ndarray = None
    bK: np.ndarray = None
    br0: np.ndarray = None
    bR: np.ndarray = None
    f: np.ndarray = None
    t: np.ndarray = None

    def __post_init__(self):
        # private copies: the integrators update x, nrm, v, o in place
        self.x = np.array(self.x, np.float64, order="C", copy=True).reshape(-1, 3)
        n = len(self.x)
        self.nrm = np.array(self.nrm, np.float64, order="C", copy=True).reshape(n, 3)
        self.v = np.array(self.v, np.float64, order="C", copy=True).reshape(n, 3)
        self.o = np.array(self.o, np.float64, order="C", copy=True).reshape(n, 3)
        self.type = np.ascontiguousarray(self.type, np.int32).reshape(n)
        self.tag = np.ascontiguousarray(self.tag, np.int32).reshape(n)
        self.bonds = np.ascontiguousarray(self.bonds, np.int32).reshape(-1, 3)
        if self.bond_r0 is not None:
            self.bond_r0 = np.ascontiguousarray(self.bond_r0, np.float64).reshape(-1)
        if self.faces is not None:
            self.faces = np.ascontiguousarray(self.faces, np.int32).reshape(-1, 3)
        if self.bstyle is None:
            self.bstyle, self.bK, self.br0, self.bR = reference_bond_table()
        if self.f is None:
            self.f = np.zeros((n, 3))
        if self.t is None:
            self.t = np.zeros((n, 3))

    @property
    def n(self):
        return len(self.x)

    def copy(self) -> "State":
        kw = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in self.__dict__.items()}
        return State(**kw)

    def _c(self) -> OrcSystemC:
        s = OrcSystemC()
        s.n = self.n
        for name in ("x", "nrm", "v", "o", "f", "t", "type", "tag"):
            setattr(s, name, getattr(self, name).ctypes.data)
        s.nb = len(self.bonds)
        s.bonds = self.bonds.ctypes.data if len(self.bonds) else None
        s.bond_r0 = self.bond_r0.ctypes.data if self.bond_r0 is not None else None
        s.nface = 0 if self.faces is None else len(self.faces)
        s.faces = self.faces.ctypes.data if self.faces is not None and len(self.faces) else None
        for d in range(3):
            s.lo[d], s.hi[d], s.periodic[d] = self.lo[d], self.hi[d], int(self.periodic[d])
        for name in ("dt", "kBT", "eta", "zeta", "Q", "kv", "V0", "ka", "A0"):
            setattr(s, name, float(getattr(self, name)))
        s.seed, s.step, s.sys, s.bounce = int(self.seed), int(self.step), int(self.sys), int(self.bounce)
        s.zero_bulk = int(self.zero_bulk)
        for k in range(MAX_BOND_TYPES):
            s.bstyle[k] = int(self.bstyle[k])
            s.bK[k] = float(self.bK[k])
            s.br0[k] = float(self.br0[k])
            s.bR[k] = float(self.bR[k])
        return s


def lib(fast: bool = False):
    """The checker (strict IEEE build) or, with fast=True, the same source
    built with the reference's optimisation flags for the timed baseline."""
    global _lib, _lib_fast
    with _lock:
        if (_lib_fast if fast else _lib) is None:
            path = LIB_FAST if fast else LIB
            if not os.path.exists(path):
                build()
            L = C.CDLL(path)
            P = C.POINTER
            for name in ("orc_forces_f64", "orc_forces_f32"):
                getattr(L, name).argtypes = [P(OrcSystemC), C.c_void_p, C.c_void_p, C.c_void_p, P(OrcThermoC)]
            for name in ("orc_step_langevin_f64", "orc_step_langevin_f32", "orc_step_nh_f64"):
                getattr(L, name).argtypes = [P(OrcSystemC), C.c_int, P(OrcThermoC)]
            L.orc_run_langevin_fast_f32.argtypes = [P(OrcSystemC), C.c_int, C.c_double, P(OrcThermoC)]
            L.orc_nh_prologue_f64.argtypes = [P(OrcSystemC), P(OrcThermoC)]
            L.orc_thermo_f64.argtypes = [P(OrcSystemC), P(OrcThermoC)]
            L.orc_pairs.argtypes = [P(OrcSystemC), C.c_void_p, C.c_void_p, C.c_int64]
            L.orc_pairs.restype = C.c_int64
            L.orc_morton_encode.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]
            L.orc_morton_order.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]
            L.orc_noise.argtypes = [C.c_uint64, C.c_int64, C.c_int, C.c_int, C.c_void_p]
            L.orc_ff_tables.argtypes = [C.c_void_p] * 4
            L.orc_assign_temperature.argtypes = [P(OrcSystemC), C.c_double, C.c_uint64]
            L.orc_set_threads.argtypes = [C.c_int]
            L.orc_get_threads.restype = C.c_int
            if fast:
                _lib_fast = L
            else:
                _lib = L
    return _lib_fast if fast else _lib


def workloads_lib():
    """The library's host-only input generators built by this directory's
    Makefile (same sources and flags as the library), so that a CPU-only
    process makes the benchmark's inputs without loading the GPU library.
    Pass it as `lib=` to openrbc_gb300.workloads."""
    global _workloads
    with _lock:
        if _workloads is None:
            if not os.path.exists(LIB_WORKLOADS):
                subprocess.run(["make", "-s", "-C", HERE, "liborbc_workloads.so"], check=True)
            from openrbc_gb300._native import declare_generators
            _workloads = declare_generators(C.CDLL(LIB_WORKLOADS))
    return _workloads


def _thermo(th: OrcThermoC) -> dict:
    return {k: getattr(th, k) for k, _ in OrcThermoC._fields_}


def set_threads(n: int) -> None:
    lib().orc_set_threads(int(n))
    lib(True).orc_set_threads(int(n))


def get_threads() -> int:
    return int(lib().orc_get_threads())


def forces(st: State, precision: str = "f64", energy: bool = False):
    """(f, t, e_or_None, thermo) at the current state."""
    L = lib()
    f = np.zeros((st.n, 3))
    t = np.zeros((st.n, 3))
    e = np.zeros(st.n) if energy else None
    th = OrcThermoC()
    c = st._c()
    fn = L.orc_forces_f64 if precision == "f64" else L.orc_forces_f32
    fn(C.byref(c), f.ctypes.data, t.ctypes.data, e.ctypes.data if energy else None, C.byref(th))
    return f, t, e, _thermo(th)


def _sync_back(st: State, c: OrcSystemC):
    st.zeta, st.Q, st.step = c.zeta, c.Q, c.step


def langevin(st: State, nsteps: int, precision: str = "f64", fast: bool = False) -> dict:
    L = lib(fast)
    c = st._c()
    th = OrcThermoC()
    fn = L.orc_step_langevin_f64 if precision == "f64" else L.orc_step_langevin_f32
    fn(C.byref(c), int(nsteps), C.byref(th))
    _sync_back(st, c)
    return _thermo(th)


def cpu_baseline_run(st: State, nsteps: int, skin: float = 0.4) -> dict:
    """nsteps FP32 Langevin steps organised as the reference's production
    loop runs (orc_run_langevin_fast_f32, built with the reference's
    optimisation flags): the timed CPU baseline.  thermo['npairs'] holds the
    number of neighbour-list builds."""
    L = lib(True)
    c = st._c()
    th = OrcThermoC()
    if L.orc_run_langevin_fast_f32(C.byref(c), int(nsteps), float(skin), C.byref(th)):
        raise ValueError("orc_run_langevin_fast_f32: bad argument")
    _sync_back(st, c)
    return _thermo(th)


def nh_prologue(st: State) -> dict:
    c = st._c()
    th = OrcThermoC()
    lib().orc_nh_prologue_f64(C.byref(c), C.byref(th))
    _sync_back(st, c)
    return _thermo(th)


def nh_steps(st: State, nsteps: int) -> dict:
    c = st._c()
    th = OrcThermoC()
    lib().orc_step_nh_f64(C.byref(c), int(nsteps), C.byref(th))
    _sync_back(st, c)
    return _thermo(th)


def minimize(st: State, nsteps: int, dr_opt: float = 0.05, dn_opt: float = 0.05) -> dict:
    c = st._c()
    th = OrcThermoC()
    lib().orc_minimize_f64(C.byref(c), int(nsteps), C.c_double(dr_opt), C.c_double(dn_opt), C.byref(th))
    _sync_back(st, c)
    return _thermo(th)


def assign_temperature(st: State, kT: float, seed: int) -> None:
    lib().orc_assign_temperature(C.byref(st._c()), float(kT), int(seed))


def rdf(x, type, type_a=-1, type_b=-1, dr=0.1, nbins=10000, rcut=0.0, centre=(0.0, 0.0, 0.0),
        L=(0.0, 0.0, 0.0), single=False):
    """Pair-distance histogram (orc_rdf; src/rdf.h:26-81).  Returns
    (counts, counted, dropped)."""
    x = np.ascontiguousarray(x, np.float64).reshape(-1, 3)
    t = np.ascontiguousarray(type, np.int32).reshape(-1)
    c = np.ascontiguousarray(centre, np.float64)
    Lb = np.ascontiguousarray(L, np.float64)
    counts = np.zeros(int(nbins), np.uint64)
    dropped = C.c_int64()
    L_ = lib()
    L_.orc_rdf.restype = C.c_int64
    n = L_.orc_rdf(x.ctypes.data_as(C.c_void_p), t.ctypes.data_as(C.c_void_p), C.c_int64(len(x)), int(type_a),
                   int(type_b), C.c_double(dr), int(nbins), C.c_double(rcut), c.ctypes.data_as(C.c_void_p),
                   Lb.ctypes.data_as(C.c_void_p), 1 if single else 0, counts.ctypes.data_as(C.c_void_p),
                   C.byref(dropped))
    return counts, int(n), dropped.value


def cleanup_marks(x, type, cell3, sys, nc3, L3, mingen=4, tol=2.5):
    """delete_lipid's marking rule with grid-cell centroids as generators
    (orc_cleanup_marks; src/cleanup.h:40-59).  Returns (keep flags, removed)."""
    x = np.ascontiguousarray(x, np.float64).reshape(-1, 3)
    t = np.ascontiguousarray(type, np.int32)
    tl = np.ascontiguousarray(cell3, np.int32).reshape(-1, 3)
    sy = np.ascontiguousarray(sys, np.int32)
    nt = np.ascontiguousarray(nc3, np.int32).reshape(-1, 3)
    Lb = np.ascontiguousarray(L3, np.float64).reshape(-1, 3)
    keep = np.zeros(len(x), np.int32)
    L = lib()
    L.orc_cleanup_marks.restype = C.c_int64
    vp = C.c_void_p
    r = L.orc_cleanup_marks(x.ctypes.data_as(vp), t.ctypes.data_as(vp), tl.ctypes.data_as(vp), sy.ctypes.data_as(vp),
                            C.c_int64(len(x)), C.c_int(len(nt)), nt.ctypes.data_as(vp), Lb.ctypes.data_as(vp),
                            C.c_int(mingen), C.c_double(tol), keep.ctypes.data_as(vp))
    return keep.astype(bool), int(r)


def place_lipids(net, min_dist=0.55, min_dist_lp=1.685, seed=0):
    """init_rbc's lipid placement (orc_place_lipids; src/init_rbc.h:235-305)
    for a network from openrbc_gb300.workloads.init_rbc_network: the checker
    of the GPU placement, one attempt at a time."""
    L = lib()
    L.orc_place_lipids.restype = C.c_int64
    vp = C.c_void_p
    vert = np.ascontiguousarray(net["vert"], np.float64)
    face = np.ascontiguousarray(net["face"], np.int32)
    fn = np.ascontiguousarray(net["face_normal"], np.float64)
    fnl = np.ascontiguousarray(net["face_nl"], np.int64)
    prot = np.ascontiguousarray(net["x"], np.float64)
    nl = int(fnl.sum())
    x, n = np.zeros((nl, 3)), np.zeros((nl, 3))
    r = L.orc_place_lipids(vert.ctypes.data_as(vp), face.ctypes.data_as(vp), fn.ctypes.data_as(vp),
                           C.c_int64(len(face)), fnl.ctypes.data_as(vp), prot.ctypes.data_as(vp),
                           C.c_int64(len(prot)), C.c_double(min_dist), C.c_double(min_dist_lp),
                           C.c_uint64(int(seed) & 0xFFFFFFFFFFFFFFFF), x.ctypes.data_as(vp), n.ctypes.data_as(vp))
    if r != nl:
        raise ValueError(f"orc_place_lipids: face {-r - 1} found no room")
    return x, n


def thermo(st: State) -> dict:
    th = OrcThermoC()
    lib().orc_thermo_f64(C.byref(st._c()), C.byref(th))
    return _thermo(th)


def pairs(st: State, rcut2: np.ndarray) -> np.ndarray:
    """Unordered pairs (i<j) with r^2 < rcut2[ti, tj], sorted, shape (m, 2)."""
    L = lib()
    r2 = np.ascontiguousarray(rcut2, np.float64).reshape(36)
    c = st._c()
    m = L.orc_pairs(C.byref(c), r2.ctypes.data, None, 0)
    out = np.zeros((max(m, 1), 2), np.int32)
    L.orc_pairs(C.byref(c), r2.ctypes.data, out.ctypes.data, m)
    return out[:m]


def morton_encode(p: np.ndarray, bsize=(2000.0, 2000.0, 2000.0)) -> np.ndarray:
    p = np.ascontiguousarray(p, np.float64).reshape(-1, 3)
    b = np.ascontiguousarray(bsize, np.float64)
    k = np.zeros(len(p), np.uint32)
    lib().orc_morton_encode(p.ctypes.data, len(p), b.ctypes.data, k.ctypes.data)
    return k


def morton_order(p: np.ndarray, bsize=(2000.0, 2000.0, 2000.0)) -> np.ndarray:
    p = np.ascontiguousarray(p, np.float64).reshape(-1, 3)
    b = np.ascontiguousarray(bsize, np.float64)
    o = np.zeros(len(p), np.int32)
    lib().orc_morton_order(p.ctypes.data, len(p), b.ctypes.data, o.ctypes.data)
    return o


def noise(seed: int, step: int, tag: int, sys: int = 0) -> np.ndarray:
    r = np.zeros(3)
    lib().orc_noise(int(seed), int(step), int(tag), int(sys), r.ctypes.data)
    return r


def ff_tables():
    m, r = np.zeros(6), np.zeros(6)
    c2, l2 = np.zeros(36), np.zeros(36)
    lib().orc_ff_tables(m.ctypes.data, r.ctypes.data, c2.ctypes.data, l2.ctypes.data)
    return m, r, c2.reshape(6, 6), l2.reshape(6, 6)


# ---------------------------------------------------------------------------
# Reference harness (built from the reference's own headers; present only
# where the reference source tree was available at build time).
# ---------------------------------------------------------------------------
def ref_available(precision: str = "f64") -> bool:
    return os.path.exists(os.path.join(REF_DIR, f"libref_{precision}.so"))


def ref(precision: str = "f64"):
    with _lock:
        if precision not in _ref:
            L = C.CDLL(os.path.join(REF_DIR, f"libref_{precision}.so"))
            vp, i64, d = C.c_void_p, C.c_int64, C.c_double
            L.ref_forces.argtypes = [i64, vp, vp, vp, vp, i64, vp, vp, vp]
            L.ref_langevin.argtypes = [i64, vp, vp, vp, vp, vp, vp, i64, vp, d, d, d, C.c_int]
            L.ref_nh.argtypes = [i64, vp, vp, vp, vp, vp, vp, i64, vp, d, d, vp, d, C.c_int]
            L.ref_temperature.argtypes = [i64, vp, vp, vp, vp, vp]
            L.ref_temperature.restype = d
            L.ref_morton_encode.argtypes = [i64, vp, vp]
            L.ref_init_rbc.argtypes = [C.c_char_p, i64, vp, vp, vp, vp, i64, vp, vp, vp]
            L.ref_init_rbc.restype = i64
            _ref[precision] = L
    return _ref[precision]
