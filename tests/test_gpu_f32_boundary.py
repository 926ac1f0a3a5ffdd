"""FP32 host boundary (orbc_gpu_set_state_f32 / orbc_gpu_download_f32).

The reference's containers hold AoS `vector<real,3>` with real = float
(src/config_static.h:34-44, src/container.h:68-72).  These calls accept those
arrays as they are, by upload-index range and stride.  An FP32 state must land
on the device exactly as the same values sent through the FP64 call, ranges
must compose, the padded stride-4 layout must equal stride 3, and the FP32
download must be the FP64 download rounded to float.
"""
import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu

REF_BOX = ((-1000.0, 1000.0),) * 3


def _sim(g, precision="mixed"):
    from openrbc_gb300 import RTParameter, Simulation
    p = RTParameter(init="lipid", precision=precision, kBT=0.5, rseed=21)
    s = Simulation(p, box=REF_BOX)
    s.upload(g["x"], g["nrm"], g["v"], g["o"], g["type"], g["tag"], g.get("bonds"))
    return s


def _f32_state(g, shift=0.0):
    x = (g["x"] + shift).astype(np.float32)
    return x, g["nrm"].astype(np.float32), g["v"].astype(np.float32), g["o"].astype(np.float32)


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_f32_download_is_the_rounded_fp64_download(precision):
    g = load_golden("cell_ico12.npz")
    with _sim(g, precision) as s:
        s.step(5)
        ref = s.download()
        got3 = s.download_f32()
        got4 = s.download_f32(stride=4)
        n = s.n
        a = n // 3
        part = s.download_f32(first=a, count=n - 2 * a)
    for r, u, w, q in zip(ref, got3, got4, part):
        want = r.astype(np.float32)
        assert np.array_equal(u, want)
        assert np.array_equal(w[:, :3], want) and not w[:, 3].any()
        assert np.array_equal(q, want[a:n - a])


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_f32_state_lands_like_the_same_values_in_fp64(precision):
    g = load_golden("cell_ico12.npz")
    x, nv, v, o = _f32_state(g, shift=0.03)
    outs = []
    for mode in ("fp64", "f32", "ranges", "stride4"):
        with _sim(g, precision) as s:
            s.step(3)
            if mode == "fp64":
                s.set_state(*[a.astype(np.float64) for a in (x, nv, v, o)])
            elif mode == "f32":
                s.set_state_f32(x, nv, v, o)
            elif mode == "ranges":
                a = 1000
                s.set_state_f32(x[a:], nv[a:], v[a:], o[a:], first=a)
                s.set_state_f32(x[:a], nv[:a], v[:a], o[:a], first=0)
            else:
                pad = [np.concatenate([q, np.full((len(q), 1), 7.0, np.float32)], 1) for q in (x, nv, v, o)]
                s.set_state_f32(*pad)
            th = s.step(10)
            outs.append((s.download(), th["temperature"]))
    for state, temp in outs[1:]:
        for u, w in zip(state, outs[0][0]):
            assert np.array_equal(u, w)
        assert temp == outs[0][1]


def test_f32_boundary_rejects_bad_ranges():
    from openrbc_gb300 import OrbcError
    g = load_golden("lattice_576.npz")
    with _sim(g) as s:
        x, nv, v, o = _f32_state(g)
        with pytest.raises(OrbcError):
            s.set_state_f32(x, nv, v, o, first=1)             # runs past the last particle
        with pytest.raises(OrbcError):
            s.download_f32(first=-1, count=10)
        with pytest.raises(OrbcError):
            s.download_f32(stride=5)
        s.set_state_f32(x[:0], nv[:0], v[:0], o[:0], first=0)  # empty range is a no-op


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_in_place_host_transfers_equal_staged_copies(precision):
    """With host_direct the conversion kernels read and write the caller's
    arrays in place when the GPU can reach them (mapped page-locked memory;
    pageable memory on GPUs that read the host's page tables): the states and
    downloads must equal those of the staged copies, for pageable numpy arrays
    and page-locked ones, in FP32 (stride 3 and 4, index ranges, one of them
    starting off a 16-byte boundary) and FP64."""
    import torch
    from openrbc_gb300 import RTParameter, Simulation
    g = load_golden("cell_ico12.npz")
    x, nv, v, o = _f32_state(g, shift=0.02)

    def pinned(a):
        t = torch.empty(a.shape, dtype=torch.float32 if a.dtype == np.float32 else torch.float64, pin_memory=True)
        t.numpy()[:] = a
        return t.numpy()

    results = []
    for direct in (False, True):
        for kind in ("pageable", "pinned"):
            conv = pinned if kind == "pinned" else (lambda a: np.ascontiguousarray(a))
            p = RTParameter(init="lipid", precision=precision, kBT=0.5, rseed=21)
            with Simulation(p, box=REF_BOX, host_direct=direct) as s:
                s.upload(g["x"], g["nrm"], g["v"], g["o"], g["type"], g["tag"], g.get("bonds"))
                s.step(2)
                a = 1001  # x[a:] starts 12 bytes past a 16-byte boundary: the unaligned path
                s.set_state_f32(*[conv(q[a:]) for q in (x, nv, v, o)], first=a)
                s.set_state_f32(*[conv(q[:a]) for q in (x, nv, v, o)], first=0)
                s.step(4)
                f32 = s.download_f32()
                f32s4 = s.download_f32(stride=4)
                d64 = [conv(q) for q in s.download()]
                s.set_state(*[conv(q.astype(np.float64) + 0.001) for q in d64])
                th = s.step(3)
                results.append((f32, f32s4, s.download(), th["temperature"]))
    ref = results[0]
    for r in results[1:]:
        for u, w in zip(r[0], ref[0]):
            assert np.array_equal(u, w)
        for u, w in zip(r[1], ref[1]):
            assert np.array_equal(u, w)
        for u, w in zip(r[2], ref[2]):
            assert np.array_equal(u, w)
        assert r[3] == ref[3]
