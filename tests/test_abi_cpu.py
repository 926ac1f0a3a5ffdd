"""CPU-only checks of the C ABI library: it loads without a GPU, exports every
symbol include/*.h declares, reports errors instead of exiting, and its host
workload generators and parameter parser behave."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import ROOT


def declared_symbols():
    names = set()
    for h in ("orbc_gpu.h", "orbc_workloads.h"):
        src = open(os.path.join(ROOT, "include", h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"\b(orbc_[a-z0-9_]+)\s*\(", src):
            names.add(m.group(1))
    return names


def test_library_exports_every_declared_symbol():
    from openrbc_gb300 import _native as N
    L = N.lib()
    decl = declared_symbols()
    assert decl, "no declarations found"
    missing = [s for s in sorted(decl) if not hasattr(L, s)]
    assert not missing, missing
    assert set(N.EXPORTS) >= decl


def test_default_params_match_rtparameter():
    from openrbc_gb300 import RTParameter
    from openrbc_gb300 import _native as N
    p = N.Params()
    N.lib().orbc_gpu_default_params(C.byref(p))
    r = RTParameter()
    assert (p.dt, p.kBT, p.eta, p.seed) == (r.dt, pytest.approx(r.kBT), pytest.approx(r.eta), r.rseed)
    assert list(p.bond_r0)[:4] == [2.25, 1.1225, 2.25, 2.24] and p.bond_K[0] == 57
    assert list(p.lo) == [-1000.0] * 3 and list(p.hi) == [1000.0] * 3


def test_create_rejects_bad_params_without_exiting():
    from openrbc_gb300 import _native as N
    L = N.lib()
    p = N.Params()
    L.orbc_gpu_default_params(C.byref(p))
    p.dt = -1
    h = C.c_void_p()
    rc = L.orbc_gpu_create(C.byref(p), C.byref(h))
    assert rc == 1 and not h.value
    assert b"invalid" in L.orbc_gpu_error(None)


@pytest.mark.parametrize("field,value", [("kernel_variant", -1), ("kernel_variant", 128), ("kernel_variant", 24),
                                         ("kernel_variant", 24 | 3), ("host_direct", 2), ("zero_bulk", -1)])
def test_create_rejects_out_of_range_forms_and_switches(field, value):
    """Kernel forms are 0..127 with list-build bits 3 and 4 not both set; the
    switches are 0 or 1: anything else is an argument error, not a guess."""
    from openrbc_gb300 import _native as N
    L = N.lib()
    p = N.Params()
    L.orbc_gpu_default_params(C.byref(p))
    setattr(p, field, value)
    h = C.c_void_p()
    assert L.orbc_gpu_create(C.byref(p), C.byref(h)) == 1 and not h.value
    assert b"invalid" in L.orbc_gpu_error(None)


def test_create_without_gpu_reports_nodev():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from openrbc_gb300 import _native as N
    L = N.lib()
    p = N.Params()
    L.orbc_gpu_default_params(C.byref(p))
    h = C.c_void_p()
    rc = L.orbc_gpu_create(C.byref(p), C.byref(h))
    assert rc in (2, 9) and not h.value


def test_null_handle_calls_return_arg_error():
    from openrbc_gb300 import _native as N
    L = N.lib()
    assert L.orbc_gpu_step(None, 1, None) == 1
    assert L.orbc_gpu_download(None, None, None, None, None) == 1
    assert L.orbc_gpu_morton_encode(None, -1, None, None) == 1


def test_lattice_generator():
    from openrbc_gb300 import workloads
    w = workloads.lattice()
    x = w["x"]
    assert x.shape == (32768, 3)
    assert abs(np.linalg.norm(w["n"], axis=1) - 1).max() < 1e-12
    assert abs(x[:, 2]).max() < 0.5 and x[:, 0].max() < 200.2
    assert abs(w["v"].std() - 1.0) < 0.02
    assert np.array_equal(w["tag"], np.arange(1, 32769))


def test_rbc_generator_small():
    from openrbc_gb300 import workloads
    w = workloads.rbc(n_lipid=40_000, freq=6, kT=1.0, seed=2)
    nv = 10 * 36 + 2
    assert (w["type"][:nv] == 3).all() and (w["type"][nv:] == 0).all()
    assert len(w["bonds"]) == 30 * 36 and len(w["faces"]) == 20 * 36
    v_red = w["volume"] / (4 / 3 * np.pi * (w["area"] / (4 * np.pi)) ** 1.5)
    assert 0.6 < v_red < 0.7
    # outward normals: volume from faces is positive and lipid normals point away from the centre
    assert w["volume"] > 0
    x, n = w["x"][nv:], w["n"][nv:]
    assert np.mean(np.sum(x * n, 1) > 0) > 0.7
    from scipy.spatial import cKDTree
    d, _ = cKDTree(x).query(x, 2)
    assert d[:, 1].min() >= 0.55 - 1e-9


def test_vesicle_sizes_lognormal():
    from openrbc_gb300 import _native as N
    s = np.zeros(96, np.int64)
    assert N.lib().orbc_gen_vesicle_sizes(96, 10_000, 250_000, 40_000, 5_000_000, 4, s.ctypes.data) == 0
    assert s.min() >= 10_000 and s.max() <= 250_000
    assert abs(s.sum() - 5_000_000) < 0.02 * 5_000_000


def test_rtparameter_cli_mirrors_reference():
    from openrbc_gb300 import ParameterError, RTParameter
    p = RTParameter.from_argv(["-i", "lipid", "-k", "0.005", "-T", "1", "--eta", "0.02", "-E", "0"])
    assert (p.init, p.dt, p.kBT, p.eta, p.opt_nstep) == ("lipid", 0.005, 1.0, 0.02, 0)
    q = RTParameter.from_argv(["-r", "1.5"])  # registered for rho and random-seed alike
    assert q.rho == 1.5 and q.rseed == 1
    with pytest.raises(ParameterError):
        RTParameter.from_argv(["-i", "bogus"])
    with pytest.raises(ParameterError):
        RTParameter.from_argv(["-i", "lipid", "--cleanup-frequency", "61"])
