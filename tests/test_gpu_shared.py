"""Shared-grid batches on the GPU against the reference's
BatchAmericanOptionSolver::solve_batch(use_shared_grid = true)
(tests/golden/shared.npz): option chains on the normalized route (one
S = K = 1 march per (sigma, r, q, T) group, every strike read from it) and
batches the route rejects on one shared grid, with the batch-estimated grid
and with custom grids.  Bar: prices and Greeks within 1e-9 relative (1e-11
absolute floor); grid sizes identical.  Theta is the one-step difference
(V_prev - V) K / dt: the shared grid takes the batch's largest step count
(5000 here, dt = 5e-5 for the shortest maturity), which amplifies
value-level rounding by 1/dt, so theta also gets an absolute allowance of
1e-13 K / dt (a value-level disagreement of 1e-13 of the strike)."""
import numpy as np
import pytest

from conftest import golden, rel_err

pytestmark = pytest.mark.gpu

RTOL = 1e-9
ATOL = 1e-11

# case -> (maturity key, volatility key, type key, use_normalized, chain route expected)
CASES = {
    "chain": ("T", "sig", "put", True, 1),
    "chain_sinh": ("T", "sig", "put", True, 1),
    "chain_fixed_n": ("T", "sig", "put", True, 1),
    "chain_regular": ("T", "sig", "put", False, 0),
    "mixed": ("T", "sig", "mixed", True, 0),
    "mixed_fixed_n": ("T", "sig", "mixed", True, 0),
    "mixed_uniform": ("T", "sig", "mixed", True, 0),
    "wide": ("wide_T", "wide_sig", "put", True, 0),
}


def greeks(out):
    return np.stack([out["value"], out["delta"], out["gamma"], out["theta"]], 1)


def check(got, want, theta_atol=None):
    tol = RTOL * np.abs(want) + ATOL
    if theta_atol is not None:
        tol[:, 3] += theta_atol
    bad = np.abs(got - want) > tol
    assert not bad.any(), f"max rel {rel_err(got, want).max():.3e}; rows {np.argwhere(bad)[:8].tolist()}"


def custom_grid(pkg, spec):
    kind, x_min, x_max, nx, alpha, nt = spec
    kind = int(kind)
    if kind == 0:
        return None
    if kind == 1:
        return pkg.grid_array(1, pkg.GRID_FIXED_N, int(nx), 0)
    return pkg.grid_array(1, pkg.GRID_SINH if kind == 2 else pkg.GRID_UNIFORM, int(nx), int(nt), x_min, x_max,
                          alpha)


def params_of(pkg, g, tkey, skey, ptype):
    return pkg.pricing_array(g["S"], g["K"], g[tkey], g[skey], g["r"], g["q"], g[ptype])


@pytest.mark.parametrize("name", list(CASES))
def test_shared_grid_vs_reference(engine, pkg, name):
    g = golden("shared.npz")
    tkey, skey, ptype, normalized, route = CASES[name]
    out, got_route = engine.price_shared_arrays(params_of(pkg, g, tkey, skey, ptype),
                                                custom_grid(pkg, g[f"{name}_grid"]), use_normalized=normalized)
    assert got_route == route
    assert (out["status"] == 0).all()
    dims = g[f"{name}_dims"]
    assert (out["n_space"] == dims[:, 0]).all() and (out["n_time"] == dims[:, 1]).all()
    dt = g[tkey] / dims[:, 1]
    check(greeks(out), g[f"{name}_out"], 1e-13 * g["K"] / dt)


def test_chain_skips_invalid_options(engine, pkg):
    """A slot that fails validation is reported MANGO_ERR_VALIDATION and
    forms no group; the rest of the chain is priced as without it."""
    g = golden("shared.npz")
    p = params_of(pkg, g, "T", "sig", "put")
    bad = pkg.pricing_array(100.0, 100.0, 1.0, -0.2, 0.03, 0.01, 1)
    both = np.concatenate([p[:5], bad, p[5:]])
    out, route = engine.price_shared_arrays(both)
    assert route == 1
    assert out["status"][5] == pkg.MANGO_ERR_VALIDATION and np.isnan(out["value"][5])
    keep = np.r_[0:5, 6:both.size]
    assert (out["status"][keep] == 0).all()
    check(greeks(out[keep]), g["chain_out"])


def test_empty_batch(engine, pkg):
    out, route = engine.price_shared_arrays(pkg.pricing_array([], [], [], [], [], [], []))
    assert out.size == 0 and route == 0


def test_batch_solver_mirror(engine, pkg):
    g = golden("shared.npz")
    plist = [pkg.PricingParams(spot=float(g["S"][i]), strike=float(g["K"][i]), maturity=float(g["T"][i]),
                               rate=float(g["r"][i]), dividend_yield=float(g["q"][i]),
                               option_type=pkg.OptionType.PUT, volatility=float(g["sig"][i]))
             for i in range(g["S"].size)]
    solver = pkg.BatchAmericanOptionSolver(engine)
    res = solver.solve_batch(plist, use_shared_grid=True)
    assert solver.last_route == 1 and res.failed_count == 0
    vals = np.array([r.value() for r in res.results])
    check(vals, g["chain_out"][:, 0])
    solver.set_use_normalized(False)
    res = solver.solve_batch(plist, use_shared_grid=True)
    assert solver.last_route == 0
    check(np.array([r.value() for r in res.results]), g["chain_regular_out"][:, 0])
    # a custom grid without a shared grid: the grid resolved for the first
    # option serves every option (the regular route)
    res = solver.set_use_normalized(True).solve_batch(plist, custom_grid=pkg.PDEGridConfig(-2.5, 2.5, 181, 300, 2.0))
    assert solver.last_route == 0 and res.failed_count == 0


# Yield curves and dividends on the shared routes (tests/golden/shared_tv.npz):
# chains grouped by curve on the normalized route, dividend batches on the
# regular shared grid with each option's dividend times as mandatory points.
TV_CASES = {"chain_curve": 1, "chain_curve_sinh": 1, "divs": 0, "divs_uniform": 0, "divs_fixed_n": 0}


@pytest.mark.parametrize("name", list(TV_CASES))
def test_shared_grid_schedules_vs_reference(engine, pkg, name):
    import json
    g = golden("shared_tv.npz")
    rows = [json.loads(str(s)) for s in g[f"{name}_rows"]]
    p = pkg.pricing_array([r["S"] for r in rows], [r["K"] for r in rows], [r["T"] for r in rows],
                          [r["sigma"] for r in rows], [r["r"] for r in rows], [r["q"] for r in rows],
                          [r["put"] for r in rows])
    keep = pkg.attach_schedules(p, [r.get("curve") for r in rows], [r.get("divs") for r in rows])
    out, route = engine.price_shared_arrays(p, custom_grid(pkg, g[f"{name}_grid"]))
    assert route == TV_CASES[name]
    assert (out["status"] == 0).all()
    dims = g[f"{name}_dims"]
    assert (out["n_space"] == dims[:, 0]).all() and (out["n_time"] == dims[:, 1]).all()
    dt = np.array([r["T"] for r in rows]) / dims[:, 1]
    check(greeks(out), g[f"{name}_out"], 1e-13 * np.array([r["K"] for r in rows]) / dt)
    del keep
