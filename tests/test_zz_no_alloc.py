"""The no-allocation pricing entry point.

Some callers cannot allocate device memory when they need prices (code under
an allocator that owns the GPU, or with a fixed memory budget), so the library
offers mango_gpu_price_american_batch_noalloc, which runs a bounded batch in
one static device array instead of allocating.  This file checks, through the
C ABI, that it gives the same results as the allocating entry point
(mango_gpu_price_american_batch) on two calls in a row -- the second call
reuses the array the first one left behind -- and that over-limit requests
are refused.  It is named to be collected last: if it fails, a run that stops
at the first failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-9
ATOL = 1e-11


def _noalloc(pkg):
    lib = pkg.library()
    f = lib.mango_gpu_price_american_batch_noalloc
    f.argtypes = [ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p,
                  ctypes.c_uint64, ctypes.POINTER(pkg.MangoGpuTrbdf2), ctypes.c_void_p,
                  ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(pkg.MangoError)]
    f.restype = ctypes.c_int32
    return f


def _workload(pkg, n, seed):
    rng = np.random.default_rng(seed)
    params = pkg.pricing_array(np.full(n, 100.0), rng.uniform(80, 120, n), rng.uniform(0.1, 2.0, n),
                               rng.uniform(0.1, 0.5, n), rng.uniform(0.0, 0.08, n), rng.uniform(0.0, 0.04, n),
                               (np.arange(n) % 2 == 0).astype(np.int32))
    grids = pkg.grid_array(n, pkg.GRID_FIXED_N, rng.integers(51, 202, n), rng.integers(100, 401, n))
    return params, grids


def _call(pkg, f, params, grids):
    n = params.size
    out = np.zeros(n, dtype=pkg.OUT_DTYPE)
    failed = ctypes.c_uint64()
    err = pkg.MangoError()
    tr = pkg.MangoGpuTrbdf2(0.0, 1, 0)
    st = f(0, None, params.ctypes.data, n, grids.ctypes.data, 1, ctypes.byref(tr), out.ctypes.data,
           ctypes.byref(failed), ctypes.byref(err))
    return st, out, failed.value, err.message.decode(errors="replace")


def test_noalloc_matches_allocating_entry_point_twice(pkg):
    f = _noalloc(pkg)
    params, grids = _workload(pkg, 512, 31)
    with pkg.Engine(0) as eng:
        want = eng.price_arrays(params, grids)
    assert (want["status"] == 0).all()
    for call in range(2):
        # a different batch in between leaves other contents in the shared array
        other_p, other_g = _workload(pkg, 96, 100 + call)
        st, _, _, _ = _call(pkg, f, other_p, other_g)
        assert st == 0
        st, got, failed, msg = _call(pkg, f, params, grids)
        assert st == 0, msg
        assert failed == 0
        assert (got["status"] == want["status"]).all()
        assert (got["n_space"] == want["n_space"]).all() and (got["n_time"] == want["n_time"]).all()
        for k in ("value", "delta", "gamma", "theta"):
            bad = np.abs(got[k] - want[k]) > RTOL * np.abs(want[k]) + ATOL
            assert not bad.any(), f"call {call}: {k} differs at {np.nonzero(bad)[0][:5]}"


def test_noalloc_rejects_requests_beyond_its_limits(pkg):
    f = _noalloc(pkg)
    params, grids = _workload(pkg, 4097, 5)
    st, _, _, msg = _call(pkg, f, params, grids)
    assert st == pkg.MANGO_ERR_VALIDATION and "4096" in msg
    big = pkg.grid_array(64, pkg.GRID_FIXED_N, 3001, 10)
    st, out, failed, msg = _call(pkg, f, params[:64].copy(), big)
    assert st == pkg.MANGO_ERR_VALIDATION and "131072" in msg
    # a call refused as a whole still fills every slot
    assert failed == 64 and (out["status"] == pkg.MANGO_ERR_VALIDATION).all()
    assert np.isnan(out["value"]).all() and (out["n_space"] == 0).all()
    # per-slot validation still works inside the limits
    p = pkg.pricing_array([100.0, -5.0], [100.0, 100.0], 1.0, 0.2, 0.05, 0.0, 1)
    st, out, failed, _ = _call(pkg, f, p, pkg.grid_array(2, pkg.GRID_FIXED_N, 101, 50))
    assert st == 0 and failed == 1 and out["status"].tolist() == [0, 1]


def test_noalloc_grid_sized_at_a_given_volatility(pkg):
    """MANGO_GPU_GRID_FIXED_N_AT_VOL (the grid an IV caller fixes) gives the
    allocating entry point's results."""
    f = _noalloc(pkg)
    params, _ = _workload(pkg, 96, 12)
    grids = pkg.grid_array(96, pkg.GRID_FIXED_N_AT_VOL, 101, 200, alpha=np.linspace(0.1, 0.6, 96))
    with pkg.Engine(0) as eng:
        want = eng.price_arrays(params, grids)
    st, got, failed, msg = _call(pkg, f, params, grids)
    assert st == 0 and failed == 0, msg
    assert (got["n_space"] == want["n_space"]).all() and (got["n_time"] == want["n_time"]).all()
    for k in ("value", "delta", "gamma", "theta"):
        assert np.allclose(got[k], want[k], rtol=RTOL, atol=ATOL), k


def test_noalloc_allocates_no_device_memory(pkg):
    """Once the first call has set up the array, calls of different sizes
    leave the device's free memory unchanged."""
    torch = pytest.importorskip("torch")
    f = _noalloc(pkg)
    params, grids = _workload(pkg, 512, 7)
    assert _call(pkg, f, params, grids)[0] == 0  # set-up call
    torch.cuda.mem_get_info(0)
    free0, _ = torch.cuda.mem_get_info(0)
    for n, seed in ((512, 8), (64, 9), (300, 10), (1, 11)):
        p, g = _workload(pkg, n, seed)
        st, _, failed, msg = _call(pkg, f, p, g)
        assert st == 0 and failed == 0, msg
    free1, _ = torch.cuda.mem_get_info(0)
    assert free1 == free0
