"""The warp-per-option march (wmarch.cu) against the thread-per-option march
and the reference's golden vectors.

A batch small enough for one wave of resident warps is marched one warp per
option (scans across the lanes); MANGO_GPU_WARP_MARCH forces either layout.
Both must meet the 1e-9 bar against the reference's goldens (edge cases with
and without the Rannacher start included), and the two layouts agree to
rounding (only the association of the recurrences at the 32 lane
boundaries differs).  The price-table sweep (200 slices) runs on the warp
march by default and is covered by test_gpu_table.py."""
import numpy as np
import pytest

from conftest import golden, rel_err

pytestmark = pytest.mark.gpu

RTOL = 1e-9
ATOL = 1e-11


def greeks(out):
    return np.stack([out["value"], out["delta"], out["gamma"], out["theta"]], 1)


def check(got, want, rtol=RTOL, atol=ATOL):
    bad = np.abs(got - want) > rtol * np.abs(want) + atol
    assert not bad.any(), f"max rel {rel_err(got, want).max():.3e}; rows {np.argwhere(bad)[:8].tolist()}"


def price(engine, pkg, g, grid, rannacher=True, sel=slice(None)):
    p = pkg.pricing_array(g["S"][sel], g["K"][sel], g["T"][sel], g["sigma"][sel], g["r"][sel], g["q"][sel],
                          g["is_put"][sel])
    return engine.price_arrays(p, grid, rannacher=rannacher)


@pytest.mark.parametrize("layout", ["0", "1"])
@pytest.mark.parametrize("name", ["pricing_cfg0.npz", "pricing_mixed.npz", "pricing_uneven.npz"])
def test_layouts_vs_reference(engine, pkg, monkeypatch, layout, name):
    monkeypatch.setenv("MANGO_GPU_WARP_MARCH", layout)
    g = golden(name)
    grid = pkg.grid_array(len(g["S"]), pkg.GRID_FIXED_N, g["nx"], g["nt"])
    out = price(engine, pkg, g, grid)
    assert (out["status"] == 0).all()
    check(greeks(out), g["out"])


@pytest.mark.parametrize("layout", ["0", "1"])
def test_layouts_edge_cases(engine, pkg, monkeypatch, layout):
    monkeypatch.setenv("MANGO_GPU_WARP_MARCH", layout)
    g = golden("pricing_edge.npz")
    for rann in (0, 1):
        sel = np.nonzero(g["rannacher"] == rann)[0]
        grid = pkg.grid_array(len(sel), pkg.GRID_FIXED_N, g["nx"][sel], g["nt"][sel])
        out = price(engine, pkg, g, grid, rannacher=bool(rann), sel=sel)
        assert (out["status"] == g["status"][sel]).all()
        check(greeks(out), g["out"][sel])


@pytest.mark.parametrize("layout", ["0", "1"])
def test_layouts_auto_grids(engine, pkg, monkeypatch, layout):
    monkeypatch.setenv("MANGO_GPU_WARP_MARCH", layout)
    g = golden("pricing_auto.npz")
    out = price(engine, pkg, g, None)
    assert (out["status"] == 0).all()
    check(greeks(out), g["out"])


def test_warp_matches_thread_layout(engine, pkg, monkeypatch):
    """512 puts and calls on uneven grids (51..401 points, 100..600 steps):
    the two layouts agree to 1e-11 relative on value, delta and gamma;
    theta, a one-step difference over dt, amplifies that rounding by 1/dt
    and agrees to 1e-9."""
    rng = np.random.default_rng(99)
    n = 512
    p = pkg.pricing_array(np.full(n, 100.0), rng.uniform(70, 130, n), rng.uniform(0.05, 2.0, n),
                          rng.uniform(0.05, 0.6, n), rng.uniform(0.0, 0.08, n), rng.uniform(0.0, 0.05, n),
                          (np.arange(n) % 2 == 0).astype(np.int32))
    grid = pkg.grid_array(n, pkg.GRID_FIXED_N, rng.integers(51, 402, n), rng.integers(100, 601, n))
    outs = {}
    for layout in ("0", "1"):
        monkeypatch.setenv("MANGO_GPU_WARP_MARCH", layout)
        outs[layout] = engine.price_arrays(p, grid)
        assert (outs[layout]["status"] == 0).all()
    a, b = greeks(outs["1"]), greeks(outs["0"])
    check(a[:, :3], b[:, :3], rtol=1e-11, atol=1e-13)
    check(a[:, 3], b[:, 3], rtol=1e-9, atol=1e-11)


def test_uneven_batch_binned_equals_single_queue(engine, pkg, monkeypatch):
    """An uneven batch (N_x ~ U{51..401}, N_t ~ U{100..1000}; 24,576 options,
    768 tiles) has its thread-march tiles assigned to SM sub-partitions, then
    a second launch marches anything left.  Which warp marches a tile changes
    nothing: results equal the single-queue launch (MANGO_GPU_BINS=0) bit for
    bit, with and without the warp march for the long poles."""
    n = 24576
    rng = np.random.default_rng(31)
    p = pkg.pricing_array(np.full(n, 100.0), rng.uniform(80, 120, n), rng.uniform(0.1, 2.0, n),
                          rng.uniform(0.1, 0.5, n), rng.uniform(0.0, 0.08, n),
                          rng.uniform(0.0, 0.04, n), (np.arange(n) % 2 == 0).astype(np.int32))
    g = pkg.grid_array(n, pkg.GRID_FIXED_N, rng.integers(51, 402, n), rng.integers(100, 1001, n))
    for long_poles in ("0", "1216"):
        monkeypatch.setenv("MANGO_GPU_WARP_LONG", long_poles)
        monkeypatch.setenv("MANGO_GPU_BINS", "1")
        binned = engine.price_arrays(p, g)
        monkeypatch.setenv("MANGO_GPU_BINS", "0")
        queue = engine.price_arrays(p, g)
        assert (binned["status"] == 0).all() and (queue["status"] == 0).all()
        for k in ("value", "delta", "gamma", "theta"):
            assert np.array_equal(binned[k], queue[k]), (long_poles, k)
