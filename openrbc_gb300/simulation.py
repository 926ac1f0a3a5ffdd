"""Host-side driver of the GPU step: the Python mirror of the block of
src/openrbc.cpp:155-256 that the C ABI replaces.

A `Simulation` owns one liborbc_gpu handle.  Containers are plain numpy
arrays in the reference's AoS layout (x, n, v, o as (N, 3) float64; type and
tag as int32; bonds as (type, tag_i, tag_j) rows, src/container.h:30-34).
Every call goes through include/orbc_gpu.h; errors raise OrbcError.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional, Sequence

import numpy as np

from . import _native as N
from .runtime_parameter import RTParameter

# reference bond table (src/forcefield_canonical.h:106-109): types 0..3 harmonic, K = 57
REFERENCE_BOND_R0 = (2.25, 1.1225, 2.25, 2.24)


def _ptr(a):
    return None if a is None else a.ctypes.data


def _f64(a, n=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a.reshape(-1, 3) if n is None else a.reshape(n, 3)


class Simulation:
    def __init__(self, param: Optional[RTParameter] = None, *, precision: Optional[str] = None,
                 integrator: Optional[str] = None, skin: Optional[float] = None, use_graph: bool = True,
                 energy: bool = False, box: Optional[Sequence[Sequence[float]]] = None,
                 periodic: Sequence[int] = (0, 0, 0), bond_table: Optional[dict] = None,
                 max_neighbors: int = 0, rebuild_every: Optional[int] = None, bounce: bool = True,
                 mesh_constraint: Optional[dict] = None, kernel_variant: int = 0, zero_bulk: bool = False,
                 host_direct: bool = True):
        self.param = param or RTParameter(init="lipid")
        p = N.Params()
        L = N.lib()
        L.orbc_gpu_default_params(C.byref(p))
        prm = self.param
        p.precision = N.PREC_FP64 if (precision or prm.precision) == "fp64" else N.PREC_MIXED
        p.integrator = N.INT_NOSE_HOOVER if (integrator or prm.integrator) == "nose-hoover" else N.INT_LANGEVIN
        p.dt, p.kBT, p.eta, p.Q = prm.dt, prm.kBT, prm.eta, prm.Q
        p.seed = int(prm.rseed) & 0xFFFFFFFFFFFFFFFF
        p.skin = prm.skin if skin is None else skin
        p.max_neighbors = int(max_neighbors)
        p.rebuild_every = prm.rebuild_every if rebuild_every is None else int(rebuild_every)
        p.bounce = 1 if bounce else 0
        p.use_graph = 1 if use_graph else 0
        p.energy = 1 if energy else 0
        p.kernel_variant = int(kernel_variant)
        p.zero_bulk = 1 if zero_bulk else 0
        p.host_direct = 1 if host_direct else 0
        bx = box if box is not None else prm.box
        for d in range(3):
            p.lo[d], p.hi[d] = float(bx[d][0]), float(bx[d][1])
            p.periodic[d] = int(periodic[d])
        if mesh_constraint:
            p.kv = mesh_constraint.get("kv", 0.0)
            p.V0 = mesh_constraint.get("V0", 0.0)
            p.ka = mesh_constraint.get("ka", 0.0)
            p.A0 = mesh_constraint.get("A0", 0.0)
        if bond_table:
            for t, spec in bond_table.items():
                p.bond_style[t] = spec.get("style", N.BOND_HARMONIC)
                p.bond_K[t] = spec.get("K", 57.0)
                p.bond_r0[t] = spec.get("r0", 1.0)
                p.bond_R[t] = spec.get("R", 0.0)
        self.params = p
        h = C.c_void_p()
        N.check(L.orbc_gpu_create(C.byref(p), C.byref(h)))
        self.h = h
        self.n = 0

    # ------------------------------------------------------------------
    def close(self):
        if getattr(self, "h", None):
            N.lib().orbc_gpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, rc):
        N.check(rc, self.h)

    # ------------------------------------------------------------------
    def upload(self, x, n, v, o, type, tag, bonds=None):
        """Single system (orbc_gpu_upload)."""
        x = _f64(x)
        self.n = len(x)
        self._keep = [x, _f64(n, self.n), _f64(v, self.n), _f64(o, self.n),
                      np.ascontiguousarray(type, np.int32), np.ascontiguousarray(tag, np.int32)]
        b = None if bonds is None or len(bonds) == 0 else np.ascontiguousarray(bonds, np.int32).reshape(-1, 3)
        self._check(N.lib().orbc_gpu_upload(self.h, *[_ptr(a) for a in self._keep], self.n, _ptr(b),
                                            0 if b is None else len(b)))

    def upload_batch(self, systems: Sequence[dict], x, n, v, o, type, tag, offsets, bonds=None, bond_r0=None,
                     faces=None):
        """Several independent systems (orbc_gpu_upload_batch).  Each entry of
        `systems` has lo, hi, periodic and optionally kv, V0, ka, A0, zeta."""
        x = _f64(x)
        self.n = len(x)
        descs = (N.SystemDesc * len(systems))()
        for k, s in enumerate(systems):
            for d in range(3):
                descs[k].lo[d], descs[k].hi[d] = s["lo"][d], s["hi"][d]
                descs[k].periodic[d] = int(s.get("periodic", (0, 0, 0))[d])
            for key in ("kv", "V0", "ka", "A0", "zeta"):
                setattr(descs[k], key, float(s.get(key, 0.0)))
        off = np.ascontiguousarray(offsets, np.int64)
        arrs = [x, _f64(n, self.n), _f64(v, self.n), _f64(o, self.n), np.ascontiguousarray(type, np.int32),
                np.ascontiguousarray(tag, np.int32)]
        b = None if bonds is None or len(bonds) == 0 else np.ascontiguousarray(bonds, np.int32).reshape(-1, 3)
        r0 = None if bond_r0 is None else np.ascontiguousarray(bond_r0, np.float64)
        fc = None if faces is None or len(faces) == 0 else np.ascontiguousarray(faces, np.int32).reshape(-1, 3)
        self._check(N.lib().orbc_gpu_upload_batch(
            self.h, len(systems), descs, off.ctypes.data, *[_ptr(a) for a in arrs], self.n, _ptr(b), _ptr(r0),
            0 if b is None else len(b), _ptr(fc), 0 if fc is None else len(fc)))

    def set_state(self, x, n, v, o):
        arrs = [_f64(a, self.n) for a in (x, n, v, o)]
        self._check(N.lib().orbc_gpu_set_state(self.h, *[_ptr(a) for a in arrs]))

    def set_state_f32(self, x, n, v, o, first: int = 0):
        """set_state from float32 arrays of shape (count, 3) or (count, 4) (the
        reference's vector<real,3> / _VEC4 containers) for upload indices
        [first, first + count)."""
        arrs = [np.ascontiguousarray(a, dtype=np.float32) for a in (x, n, v, o)]
        count, stride = arrs[0].shape
        if any(a.shape != (count, stride) for a in arrs):
            raise ValueError("set_state_f32: the four arrays need the same (count, 3|4) shape")
        self._check(N.lib().orbc_gpu_set_state_f32(self.h, int(first), int(count), int(stride),
                                                   *[a.ctypes.data for a in arrs]))

    def download_f32(self, first: int = 0, count: Optional[int] = None, stride: int = 3):
        """download into float32 arrays of shape (count, stride) for upload
        indices [first, first + count)."""
        count = self.n - first if count is None else count
        out = [np.zeros((count, stride), np.float32) for _ in range(4)]
        self._check(N.lib().orbc_gpu_download_f32(self.h, int(first), int(count), int(stride),
                                                  *[a.ctypes.data for a in out]))
        return tuple(out)

    def step(self, nsteps: int = 1) -> dict:
        th = N.Thermo()
        self._check(N.lib().orbc_gpu_step(self.h, int(nsteps), C.byref(th)))
        return th.as_dict()

    def thermo(self, sys: int = -1) -> dict:
        th = N.Thermo()
        self._check(N.lib().orbc_gpu_thermo(self.h, int(sys), C.byref(th)))
        return th.as_dict()

    def download(self):
        out = [np.zeros((self.n, 3)) for _ in range(4)]
        self._check(N.lib().orbc_gpu_download(self.h, *[a.ctypes.data for a in out]))
        return tuple(out)

    def forces(self):
        f, t, e = np.zeros((self.n, 3)), np.zeros((self.n, 3)), np.zeros(self.n)
        self._check(N.lib().orbc_gpu_forces(self.h, f.ctypes.data, t.ctypes.data, e.ctypes.data))
        return f, t, e

    def neighbors(self):
        """CSR (counts, indices) of the full neighbour list in upload order."""
        counts = np.zeros(self.n, np.int32)
        tot = C.c_int64()
        self._check(N.lib().orbc_gpu_neighbors(self.h, counts.ctypes.data, None, 0, C.byref(tot)))
        lst = np.zeros(max(tot.value, 1), np.int32)
        self._check(N.lib().orbc_gpu_neighbors(self.h, counts.ctypes.data, lst.ctypes.data, tot.value,
                                               C.byref(tot)))
        return counts, lst[:tot.value]

    def cells(self, sys: int = 0):
        lo, lc = np.zeros(3), np.zeros(3)
        nc = np.zeros(3, np.int32)
        cell = np.zeros(self.n, np.int32)
        off = np.zeros((self.n, 3))
        slot = np.zeros(self.n, np.int32)
        self._check(N.lib().orbc_gpu_cells(self.h, int(sys), lo.ctypes.data, lc.ctypes.data, nc.ctypes.data,
                                           cell.ctypes.data, off.ctypes.data, slot.ctypes.data))
        return {"lo": lo, "Lc": lc, "nc": nc, "cell": cell, "offset": off, "slot": slot}

    def rebuild(self):
        self._check(N.lib().orbc_gpu_rebuild(self.h))

    def save_frame(self, path: str, nstep: Optional[int] = None, fields: Optional[int] = None, append: bool = True,
                   real_bytes: int = 4, asynchronous: bool = False):
        """save_frame (src/trajectory.h:61-105) through orbc_gpu_save_frame:
        fields default to the parameter's dump_field, nstep to the step
        counter; real_bytes 4 is the reference's default `real`."""
        if nstep is None:
            nstep = int(self.thermo()["step"])
        f = int(self.param.dump_field if fields is None else fields)
        self._check(N.lib().orbc_gpu_save_frame(self.h, str(path).encode(), 1 if append else 0, int(nstep), f,
                                                int(real_bytes), 1 if asynchronous else 0))

    def flush(self):
        """Wait until every queued frame is written (orbc_gpu_flush)."""
        self._check(N.lib().orbc_gpu_flush(self.h))

    def cleanup(self, stray_tolerance: Optional[float] = None) -> int:
        """delete_lipid (src/cleanup.h:29-91) through orbc_gpu_cleanup; returns
        the number of lipids removed (survivors are renumbered in order)."""
        tol = float(self.param.stray_tolerance if stray_tolerance is None else stray_tolerance)
        removed = C.c_int64()
        self._check(N.lib().orbc_gpu_cleanup(self.h, tol, C.byref(removed)))
        self.n -= removed.value
        return removed.value

    def save_checkpoint(self, path: str):
        self._check(N.lib().orbc_gpu_save_checkpoint(self.h, str(path).encode()))

    def load_checkpoint(self, path: str):
        self._check(N.lib().orbc_gpu_load_checkpoint(self.h, str(path).encode()))

    def minimize(self, nsteps: Optional[int] = None, dr_max: Optional[float] = None,
                 dn_max: Optional[float] = None) -> dict:
        """Energy minimisation (orbc_gpu_minimize; src/openrbc.cpp:88-146) with
        the parameter's opt_nstep, dr_opt and dn_opt by default."""
        th = N.Thermo()
        self._check(N.lib().orbc_gpu_minimize(
            self.h, int(self.param.opt_nstep if nsteps is None else nsteps),
            float(self.param.dr_opt if dr_max is None else dr_max),
            float(self.param.dn_opt if dn_max is None else dn_max), C.byref(th)))
        return th.as_dict()

    def assign_temperature(self, kBT: Optional[float] = None, seed: Optional[int] = None, amplify: float = 1.0):
        """integrate(assign_temperature(param, amplify), lipid, protein)
        (src/assign_temperature.h:26-44, src/openrbc.cpp:160) on the device:
        v = sqrt(2 kBT amplify / m) g.  Defaults: the parameter's kBT and rseed."""
        kT = (self.param.kBT if kBT is None else float(kBT)) * float(amplify)
        sd = (int(self.param.rseed) if seed is None else int(seed)) & 0xFFFFFFFFFFFFFFFF
        self._check(N.lib().orbc_gpu_assign_temperature(self.h, kT, sd))

    def rdf(self, sys: int = 0, type_a: int = -1, type_b: int = -1, dr: float = 0.1, nbins: int = 10000,
            rcut: float = 0.0):
        """Pair-distance histogram of one system (orbc_gpu_rdf; src/rdf.h:26-81).
        Returns (counts[nbins] as uint64, dropped pair count)."""
        counts = np.zeros(int(nbins), np.uint64)
        dropped = C.c_int64()
        self._check(N.lib().orbc_gpu_rdf(self.h, int(sys), int(type_a), int(type_b), float(dr), int(nbins),
                                         float(rcut), counts.ctypes.data, C.byref(dropped)))
        return counts, dropped.value

    def profile(self, nsteps: int = 20) -> dict:
        """Per-kernel CUDA-event times over nsteps un-captured steps (orbc_gpu_profile)."""
        pr = N.Profile()
        self._check(N.lib().orbc_gpu_profile(self.h, int(nsteps), C.byref(pr)))
        return pr.as_dict()

    def autotune(self, trial_steps: int = 30):
        """Pick skin, force-kernel and list-build forms and rebuild cadence by
        timing trials (orbc_gpu_autotune); the state is restored afterwards.
        Returns the trial table."""
        rows = (N.TuneTrial * 64)()
        nt = C.c_int()
        self._check(N.lib().orbc_gpu_autotune(self.h, int(trial_steps), rows, 64, C.byref(nt)))
        return [{"skin": r.skin, "variant": r.variant, "rebuild_every": r.rebuild_every, "ms_per_step": r.ms_per_step,
                 "rebuilds_per_step": r.rebuilds_per_step} for r in rows[:nt.value]]

    def last_timing(self):
        ms = C.c_double()
        launches = C.c_int64()
        self._check(N.lib().orbc_gpu_last_timing(self.h, C.byref(ms), C.byref(launches)))
        return ms.value, launches.value


def rdf_table(counts, dr: float = 0.1):
    """The reference's rdf.txt rows (src/rdf.h:39-43): r = dr i and
    counts[i] / (4 * 3.14 * r^2 * dr), including its literal 3.14 and the
    infinite first row."""
    c = np.asarray(counts, np.float64)
    r = dr * np.arange(len(c))
    with np.errstate(divide="ignore", invalid="ignore"):
        g = c / (4.0 * 3.14 * r * r * dr)
    return r, g


def write_rdf(path, counts, dr: float = 0.1):
    """Write rdf.txt as the reference does: one `r value` line per bin."""
    r, g = rdf_table(counts, dr)
    with open(path, "w") as f:
        for a, b in zip(r, g):
            f.write(f"{a:g} {b:g}\n")


def morton_encode(points, bsize=(2000.0, 2000.0, 2000.0)) -> np.ndarray:
    p = _f64(points)
    b = np.ascontiguousarray(bsize, np.float64)
    k = np.zeros(len(p), np.uint32)
    N.check(N.lib().orbc_gpu_morton_encode(p.ctypes.data, len(p), b.ctypes.data, k.ctypes.data))
    return k


def morton_order(points, bsize=(2000.0, 2000.0, 2000.0)) -> np.ndarray:
    p = _f64(points)
    b = np.ascontiguousarray(bsize, np.float64)
    o = np.zeros(len(p), np.int32)
    N.check(N.lib().orbc_gpu_morton_order(p.ctypes.data, len(p), b.ctypes.data, o.ctypes.data))
    return o
