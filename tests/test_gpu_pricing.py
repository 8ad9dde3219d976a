"""GPU parity: the sm_103a march through the C ABI against the reference's
golden vectors and the CPU oracle.  Bar (the benchmark spec): prices and Greeks
within 1e-9 relative (plus a 1e-11 absolute floor for values that are
zero up to rounding)."""
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


def run(engine, pkg, g, grid, rannacher=True, sel=slice(None)):
    p = pkg.pricing_array(g["S"][sel], g["K"][sel], g["T"][sel], g["sigma"][sel], g["r"][sel], g["q"][sel],
                          g["is_put"][sel])
    return engine.price_arrays(p, grid, rannacher=rannacher)


@pytest.mark.parametrize("name", ["pricing_cfg0.npz", "pricing_mixed.npz", "pricing_uneven.npz"])
def test_fixed_grid_vs_reference(engine, pkg, name):
    g = golden(name)
    grid = pkg.grid_array(len(g["S"]), pkg.GRID_FIXED_N, g["nx"], g["nt"])
    out = run(engine, pkg, g, grid)
    assert (out["status"] == 0).all()
    assert (out["n_space"] == g["dims"][:, 0]).all() and (out["n_time"] == g["dims"][:, 1]).all()
    check(greeks(out), g["out"])


def test_auto_grid_vs_reference(engine, pkg):
    g = golden("pricing_auto.npz")
    out = run(engine, pkg, g, None)
    assert (out["status"] == 0).all()
    assert (out["n_space"] == g["dims"][:, 0]).all() and (out["n_time"] == g["dims"][:, 1]).all()
    check(greeks(out), g["out"])


def test_edge_cases_vs_reference(engine, pkg):
    g = golden("pricing_edge.npz")
    for rann in (0, 1):
        sel = np.nonzero(g["rannacher"] == rann)[0]
        grid = pkg.grid_array(len(sel), pkg.GRID_FIXED_N, g["nx"][sel], g["nt"][sel])
        out = run(engine, pkg, g, grid, rannacher=bool(rann), sel=sel)
        assert (out["status"] == g["status"][sel]).all()
        check(greeks(out), g["out"][sel])


def test_explicit_grids_vs_reference(engine, pkg):
    g = golden("pricing_explicit.npz")
    n = len(g["S"])
    grid = pkg.grid_array(n, 0, g["nx"], g["nt"], g["x_min"], g["x_max"], g["alpha"])
    grid["kind"] = g["kind"]
    out = run(engine, pkg, g, grid)
    assert (out["status"] == 0).all()
    check(greeks(out), g["out"])


def test_config1_sample_vs_oracle(engine, pkg, oracle):
    """2,048 options from the uneven-grid batch workload (N_x ~ U{51..401},
    N_t ~ U{100..1000}, puts/calls alternating) against the oracle."""
    rng = np.random.default_rng(2024)
    n = 2048
    S = np.full(n, 100.0)
    K = rng.uniform(80, 120, n)
    T = rng.uniform(0.1, 2.0, n)
    s = rng.uniform(0.1, 0.5, n)
    r = rng.uniform(0.0, 0.08, n)
    q = rng.uniform(0.0, 0.04, n)
    put = (np.arange(n) % 2 == 0).astype(np.int32)
    nx = rng.integers(51, 402, n)
    nt = rng.integers(100, 1001, n)
    out = engine.price_arrays(pkg.pricing_array(S, K, T, s, r, q, put),
                              pkg.grid_array(n, pkg.GRID_FIXED_N, nx, nt))
    ref, dims, st = oracle.price_batch(S, K, T, s, r, q, put, nx, nt)
    assert (st == 0).all() and (out["status"] == 0).all()
    assert (out["n_space"] == dims[:, 0]).all()
    check(greeks(out), ref)


def test_per_slot_validation_and_empty_batch(engine, pkg):
    p = pkg.pricing_array([100, -1, 100, 100], [100, 100, 100, 100], [1, 1, 0, 1], [0.2, 0.2, 0.2, 0.0],
                          0.05, 0.0, 1)
    out = engine.price_arrays(p, pkg.grid_array(1, pkg.GRID_FIXED_N, 101, 100))
    assert out["status"].tolist() == [0, 1, 1, 1]
    assert np.isfinite(out["value"][0]) and np.isnan(out["value"][1:]).all()
    empty = engine.price_arrays(pkg.pricing_array([], [], [], [], [], [], []))
    assert empty.size == 0


def test_batch_composition_does_not_change_results(engine, pkg):
    """Batch equals single (american_option_test.cc:119-143), bit for bit,
    whatever the batch's order and neighbours."""
    g = golden("pricing_mixed.npz")
    grid = pkg.grid_array(1, pkg.GRID_FIXED_N, 101, 498)
    full = run(engine, pkg, g, grid)
    perm = np.random.default_rng(3).permutation(len(g["S"]))
    shuffled = run(engine, pkg, g, grid, sel=perm)
    assert np.array_equal(greeks(shuffled), greeks(full)[perm])
    one = run(engine, pkg, g, grid, sel=slice(5, 6))
    assert np.array_equal(greeks(one)[0], greeks(full)[5])


def test_american_option_price_single(pkg):
    p = pkg.PricingParams(spot=100, strike=100, maturity=1.0, rate=0.05, dividend_yield=0.02,
                          option_type=pkg.OptionType.PUT, volatility=0.2)
    res = pkg.american_option_price(p)
    # reference solve_american_option on the auto grid (101 x 120)
    assert res.n_space == 101 and res.n_time == 120
    assert abs(res.value() - 6.65445228390427) < 1e-9 * 6.65
    assert abs(res.delta() - -0.422923644193511) < 1e-9
    batch = pkg.BatchAmericanOptionSolver().solve_batch([p, p])
    assert batch.failed_count == 0 and batch.results[1].value() == res.value()


@pytest.mark.parametrize("n", [70000, 270000])
def test_chunked_batch_matches_resident_batch(engine, pkg, n):
    """Batches of 65,536 options or more run as 2 to 4 chunks on two
    streams; every option equals its price from one resident (unchunked)
    batch."""
    rng = np.random.default_rng(n)
    p = pkg.pricing_array(100.0, rng.uniform(80, 120, n), rng.uniform(0.1, 2.0, n), rng.uniform(0.1, 0.5, n),
                          rng.uniform(0.0, 0.08, n), rng.uniform(0.0, 0.04, n), (np.arange(n) % 3 != 0))
    grid = pkg.grid_array(1, pkg.GRID_FIXED_N, 51, 60)
    out = engine.price_arrays(p, grid)
    b = engine.batch(p, grid)
    b.run()
    ref = b.results()
    b.close()
    assert (out["status"] == 0).all() and (ref["status"] == 0).all()
    check(greeks(out), greeks(ref), rtol=1e-13, atol=1e-14)
    again = engine.price_arrays(p, grid)  # buffers reused
    assert np.array_equal(again["value"], out["value"])


def test_tile_handoff_does_not_change_results(engine, pkg, monkeypatch):
    """The thread march hands a tile's remaining steps to a warp whose queue
    ran dry (the tile's state is in device memory between steps): 65,536
    options at 101 x 498, where the sub-partitions holding four warps hand
    tiles to those that finished, price bit for bit as with the hand-off
    off."""
    rng = np.random.default_rng(77)
    n = 65536
    p = pkg.pricing_array(100.0, rng.uniform(80, 120, n), rng.uniform(0.1, 2.0, n), rng.uniform(0.1, 0.5, n),
                          rng.uniform(0.0, 0.08, n), rng.uniform(0.0, 0.04, n), (np.arange(n) % 2 == 0))
    grid = pkg.grid_array(1, pkg.GRID_FIXED_N, 101, 498)
    res = {}
    for ho in ("0", "1"):
        monkeypatch.setenv("MANGO_GPU_HANDOFF", ho)
        b = engine.batch(p, grid)
        b.run()
        res[ho] = b.results()
        b.close()
    for k in ("value", "delta", "gamma", "theta", "status"):
        assert np.array_equal(res["0"][k], res["1"][k]), k


def test_value_at_vs_reference(engine, pkg):
    """AmericanOptionResult::value_at at other spots (tests/golden/value_at.npz:
    below, inside and above each grid), through the resident batch."""
    g = golden("value_at.npz")
    p = pkg.pricing_array(g["S"], g["K"], g["T"], g["sigma"], g["r"], g["q"], g["is_put"])
    b = engine.batch(p, pkg.grid_array(len(g["S"]), pkg.GRID_FIXED_N, g["nx"], g["nt"]))
    b.run()
    res = b.results()
    n = len(g["S"])
    got = b.value_at(np.arange(n), g["spot2"])
    want = g["value"]
    assert np.abs(got[:, 0] - want).max() <= 1e-9 * np.abs(want).max()
    own = b.value_at(np.arange(n), g["S"])  # at the option's own spot: the batch's results
    check(own, greeks(res), rtol=1e-15, atol=0.0)
    b.close()


@pytest.mark.parametrize("warp", ["0", "1"])
def test_singular_pivot_reports_solver_error(engine, pkg, monkeypatch, warp):
    """A singular Thomas pivot (thomas_solver.hpp:386-388) fails that option
    alone with MANGO_ERR_SOLVER and NaN results, on the thread march and on
    the warp march.  The pivot is made singular by the host-side hook
    MANGO_GPU_SINGULAR_PIVOT (row 1's diagonals zeroed in the coefficients
    of caller slot 5); the other slots keep their results bit for bit."""
    g = golden("pricing_mixed.npz")
    grid = pkg.grid_array(1, pkg.GRID_FIXED_N, 101, 498)
    monkeypatch.setenv("MANGO_GPU_WARP_MARCH", warp)
    clean = run(engine, pkg, g, grid)
    assert (clean["status"] == 0).all()
    monkeypatch.setenv("MANGO_GPU_SINGULAR_PIVOT", "5")
    out = run(engine, pkg, g, grid)
    assert out["status"][5] == pkg.MANGO_ERR_SOLVER
    assert np.isnan(greeks(out)[5]).all()
    keep = np.arange(len(out)) != 5
    assert (out["status"][keep] == 0).all()
    assert np.array_equal(greeks(out)[keep], greeks(clean)[keep])
    p = pkg.PricingParams(spot=float(g["S"][5]), strike=float(g["K"][5]), maturity=float(g["T"][5]),
                          rate=float(g["r"][5]), dividend_yield=float(g["q"][5]),
                          option_type=pkg.OptionType.PUT if g["is_put"][5] else pkg.OptionType.CALL,
                          volatility=float(g["sigma"][5]))
    monkeypatch.setenv("MANGO_GPU_SINGULAR_PIVOT", "0")
    with pytest.raises(pkg.SolverError):
        pkg.american_option_price(p)
