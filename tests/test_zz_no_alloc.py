"""The Morton-order sort for callers that cannot allocate device memory
(orbc_gpu_morton_order_noalloc) must give exactly the order of the
allocating entry point, orbc_gpu_morton_order, call after call: its scratch
is one fixed device array shared by all calls and reused as left by the
previous one.  The order is integer output, so the comparison is exact.
Runs last (file name) so that a failure here leaves every other test run."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _sort_on_device(L, points, bsize, stream=None):
    import torch
    n = len(points)
    dp = torch.from_numpy(np.ascontiguousarray(points)).to("cuda")
    dout = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    rc = L.orbc_gpu_morton_order_noalloc(dp.data_ptr(), n, bsize.ctypes.data, dout.data_ptr(),
                                         stream.cuda_stream if stream is not None else None)
    if stream is not None:
        stream.synchronize()
    torch.cuda.synchronize()
    return rc, dout.cpu().numpy()


def test_noalloc_order_matches_allocating_entry_point_twice():
    from openrbc_gb300 import _native as N
    from openrbc_gb300 import morton_order
    L = N.lib()
    bsize = np.array([2000.0, 2000.0, 2000.0])
    rng = np.random.default_rng(20261203)
    # two calls in a row; the second is larger, so it reads scratch the first left behind
    for n in (150_000, N.NOALLOC_MAX_POINTS):
        p = rng.uniform(-1000.0, 1000.0, (n, 3))
        p[::9] = p[4]  # many equal keys: the order must stay stable
        rc, got = _sort_on_device(L, p, bsize)
        assert rc == 0
        assert np.array_equal(got, morton_order(p, bsize))


def test_noalloc_on_a_caller_stream():
    """Work queued on the caller's own (non-default) stream."""
    import torch
    from openrbc_gb300 import _native as N
    from openrbc_gb300 import morton_order
    L = N.lib()
    bsize = np.array([2000.0, 2000.0, 2000.0])
    rng = np.random.default_rng(7)
    s = torch.cuda.Stream()
    for n in (40_000, 70_001):
        p = rng.uniform(-1000.0, 1000.0, (n, 3))
        rc, got = _sort_on_device(L, p, bsize, stream=s)
        assert rc == 0
        assert np.array_equal(got, morton_order(p, bsize))


def test_noalloc_rejects_sizes_beyond_its_scratch():
    from openrbc_gb300 import _native as N
    L = N.lib()
    bsize = np.array([2000.0, 2000.0, 2000.0])
    assert L.orbc_gpu_morton_order_noalloc(None, N.NOALLOC_MAX_POINTS + 1, bsize.ctypes.data, None, None) == 1
    assert b"ORBC_NOALLOC_MAX_POINTS" in L.orbc_gpu_error(None)
    assert L.orbc_gpu_morton_order_noalloc(None, 0, bsize.ctypes.data, None, None) == 0
