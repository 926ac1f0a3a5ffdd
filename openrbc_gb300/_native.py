"""ctypes binding of liborbc_gpu.so (include/orbc_gpu.h, include/orbc_workloads.h).

The library is the product: this module only declares its C ABI.  Loading
fails loudly when the library is missing -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "liborbc_gpu.so")

ORBC_OK = 0
ERRORS = {1: "ORBC_ERR_ARG", 2: "ORBC_ERR_CUDA", 3: "ORBC_ERR_NBR_OVERFLOW", 4: "ORBC_ERR_NAN",
          5: "ORBC_ERR_GRID", 6: "ORBC_ERR_BOND", 7: "ORBC_ERR_STATE", 8: "ORBC_ERR_NOMEM", 9: "ORBC_ERR_NODEV",
          10: "ORBC_ERR_IO"}
PREC_FP64, PREC_MIXED = 0, 1
INT_LANGEVIN, INT_NOSE_HOOVER = 0, 1
BOND_HARMONIC, BOND_FENE, BOND_WLC_POW = 0, 1, 2
MAX_BOND_TYPES = 8
NOALLOC_MAX_POINTS = 262144

# Every symbol include/*.h declares (checked by the CPU test suite).
EXPORTS = [
    "orbc_gpu_default_params", "orbc_gpu_create", "orbc_gpu_upload", "orbc_gpu_upload_batch",
    "orbc_gpu_set_state", "orbc_gpu_set_state_f32", "orbc_gpu_step", "orbc_gpu_download", "orbc_gpu_download_f32",
    "orbc_gpu_forces", "orbc_gpu_thermo",
    "orbc_gpu_neighbors", "orbc_gpu_cells", "orbc_gpu_rebuild", "orbc_gpu_last_timing",
    "orbc_gpu_morton_encode", "orbc_gpu_morton_order", "orbc_gpu_destroy", "orbc_gpu_error",
    "orbc_gpu_version", "orbc_gpu_profile", "orbc_gpu_morton_order_noalloc", "orbc_gpu_autotune",
    "orbc_gpu_assign_temperature", "orbc_gpu_rdf", "orbc_gpu_minimize", "orbc_gpu_save_frame", "orbc_gpu_flush",
    "orbc_gpu_save_checkpoint", "orbc_gpu_load_checkpoint", "orbc_gpu_cleanup", "orbc_gpu_fma_peak",
    "orbc_gen_lattice", "orbc_gen_rbc_counts", "orbc_gen_rbc", "orbc_gen_vesicle_sizes", "orbc_gen_vesicle",
    "orbc_init_rbc_sizes", "orbc_init_rbc_network", "orbc_gpu_place_lipids",
]


class OrbcError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class Params(C.Structure):
    _fields_ = [
        ("precision", C.c_int), ("integrator", C.c_int),
        ("dt", C.c_double), ("kBT", C.c_double), ("eta", C.c_double), ("Q", C.c_double),
        ("seed", C.c_uint64), ("skin", C.c_double),
        ("max_neighbors", C.c_int), ("rebuild_every", C.c_int), ("bounce", C.c_int),
        ("use_graph", C.c_int), ("energy", C.c_int),
        ("lo", C.c_double * 3), ("hi", C.c_double * 3), ("periodic", C.c_int * 3),
        ("kv", C.c_double), ("V0", C.c_double), ("ka", C.c_double), ("A0", C.c_double),
        ("bond_style", C.c_int * MAX_BOND_TYPES), ("bond_K", C.c_double * MAX_BOND_TYPES),
        ("bond_r0", C.c_double * MAX_BOND_TYPES), ("bond_R", C.c_double * MAX_BOND_TYPES),
        ("kernel_variant", C.c_int), ("zero_bulk", C.c_int), ("host_direct", C.c_int),
    ]


class SystemDesc(C.Structure):
    _fields_ = [("lo", C.c_double * 3), ("hi", C.c_double * 3), ("periodic", C.c_int * 3),
                ("kv", C.c_double), ("V0", C.c_double), ("ka", C.c_double), ("A0", C.c_double),
                ("zeta", C.c_double)]


class Thermo(C.Structure):
    _fields_ = [("step", C.c_int64), ("n", C.c_int64), ("temperature", C.c_double), ("ke2", C.c_double),
                ("epot", C.c_double), ("area", C.c_double), ("volume", C.c_double), ("zeta", C.c_double),
                ("rebuilds", C.c_int64), ("max_neighbors", C.c_int), ("capacity", C.c_int),
                ("flags", C.c_int), ("pad", C.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "pad"}


class Profile(C.Structure):
    _fields_ = [("steps", C.c_int64), ("rebuilds", C.c_int64), ("step_kernel_ms", C.c_double),
                ("rebuild_ms", C.c_double), ("gate_ms", C.c_double), ("mesh_ms", C.c_double),
                ("mean_neighbors", C.c_double), ("pairs_in_cutoff", C.c_double), ("rebin_ms", C.c_double),
                ("sort_ms", C.c_double), ("gather_ms", C.c_double), ("nlist_ms", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class TuneTrial(C.Structure):
    _fields_ = [("skin", C.c_double), ("variant", C.c_int), ("rebuild_every", C.c_int), ("ms_per_step", C.c_double),
                ("rebuilds_per_step", C.c_double)]


_lib = None
_lock = threading.Lock()


def lib():
    """Load the library (building it first when absent in a source checkout)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            from . import build as _b
            _b.build()
        if not os.path.exists(LIB_PATH):
            raise OSError(f"liborbc_gpu.so not found at {LIB_PATH}; run openrbc_gb300.build.build()")
        L = C.CDLL(LIB_PATH)
        vp, i64, i32, d, sz = C.c_void_p, C.c_int64, C.c_int, C.c_double, C.c_size_t
        P = C.POINTER
        H = C.c_void_p
        L.orbc_gpu_default_params.argtypes = [P(Params)]
        L.orbc_gpu_default_params.restype = None
        L.orbc_gpu_create.argtypes = [P(Params), P(H)]
        L.orbc_gpu_upload.argtypes = [H, vp, vp, vp, vp, vp, vp, sz, vp, sz]
        L.orbc_gpu_upload_batch.argtypes = [H, i32, P(SystemDesc), vp, vp, vp, vp, vp, vp, vp, sz, vp, vp, sz, vp, sz]
        L.orbc_gpu_set_state.argtypes = [H, vp, vp, vp, vp]
        L.orbc_gpu_step.argtypes = [H, i32, P(Thermo)]
        L.orbc_gpu_download.argtypes = [H, vp, vp, vp, vp]
        L.orbc_gpu_set_state_f32.argtypes = [H, i64, i64, i32, vp, vp, vp, vp]
        L.orbc_init_rbc_sizes.argtypes = [i64, i64, P(i64), P(i64)]
        L.orbc_init_rbc_network.argtypes = [vp, i64, vp, i64, vp, i64, d, C.c_uint64, vp, vp, vp, vp, vp, vp, vp, vp,
                                            P(i64)]
        L.orbc_gpu_place_lipids.argtypes = [vp, i64, vp, vp, i64, vp, vp, i64, d, d, C.c_uint64, vp, vp]
        L.orbc_gpu_download_f32.argtypes = [H, i64, i64, i32, vp, vp, vp, vp]
        L.orbc_gpu_forces.argtypes = [H, vp, vp, vp]
        L.orbc_gpu_thermo.argtypes = [H, i32, P(Thermo)]
        L.orbc_gpu_neighbors.argtypes = [H, vp, vp, i64, P(i64)]
        L.orbc_gpu_cells.argtypes = [H, i32, vp, vp, vp, vp, vp, vp]
        L.orbc_gpu_rebuild.argtypes = [H]
        L.orbc_gpu_assign_temperature.argtypes = [H, d, C.c_uint64]
        L.orbc_gpu_rdf.argtypes = [H, i32, i32, i32, d, i32, d, vp, P(i64)]
        L.orbc_gpu_minimize.argtypes = [H, i32, d, d, P(Thermo)]
        L.orbc_gpu_save_frame.argtypes = [H, C.c_char_p, i32, i32, i32, i32, i32]
        L.orbc_gpu_flush.argtypes = [H]
        L.orbc_gpu_cleanup.argtypes = [H, d, P(i64)]
        L.orbc_gpu_fma_peak.argtypes = [P(d), P(d)]
        L.orbc_gpu_save_checkpoint.argtypes = [H, C.c_char_p]
        L.orbc_gpu_load_checkpoint.argtypes = [H, C.c_char_p]
        L.orbc_gpu_last_timing.argtypes = [H, P(d), P(i64)]
        L.orbc_gpu_morton_encode.argtypes = [vp, i64, vp, vp]
        L.orbc_gpu_morton_order.argtypes = [vp, i64, vp, vp]
        L.orbc_gpu_profile.argtypes = [H, i32, P(Profile)]
        L.orbc_gpu_morton_order_noalloc.argtypes = [vp, i64, vp, vp, vp]
        L.orbc_gpu_autotune.argtypes = [H, i32, P(TuneTrial), i32, P(i32)]
        L.orbc_gpu_destroy.argtypes = [H]
        L.orbc_gpu_error.argtypes = [H]
        L.orbc_gpu_error.restype = C.c_char_p
        L.orbc_gpu_version.restype = C.c_char_p
        declare_generators(L)
        _lib = L
        return L


def declare_generators(L):
    """Argument types of the host-only workload generators
    (include/orbc_workloads.h) on a library that exports them."""
    vp, i64, i32, d = C.c_void_p, C.c_int64, C.c_int, C.c_double
    P = C.POINTER
    L.orbc_gen_lattice.argtypes = [i64, i32, d, d, d, d, C.c_uint64, vp, vp, vp, vp, vp, vp]
    L.orbc_gen_rbc_counts.argtypes = [i64, i32, P(i64), P(i64), P(i64)]
    L.orbc_gen_rbc.argtypes = [i64, i32, d, C.c_uint64, vp, vp, vp, vp, vp, vp, vp, vp, vp, P(d), P(d), P(d)]
    L.orbc_gen_vesicle_sizes.argtypes = [i32, i64, i64, i64, i64, C.c_uint64, vp]
    L.orbc_gen_vesicle.argtypes = [i64, d, d, C.c_uint64, i32, vp, vp, vp, vp, vp, vp, P(d)]
    return L


def check(rc, handle=None):
    if rc != ORBC_OK:
        msg = lib().orbc_gpu_error(handle)
        raise OrbcError(rc, msg.decode() if msg else "")
