"""Yield curves and discrete dividends on the GPU's time-varying march
against the reference's AmericanOptionSolver on the same options
(tests/golden/tv.npz): the solver's own grid (dividend-widened, mandatory
time points), pinned-size, sinh and uniform grids with the dividends as
mandatory times, Rannacher on and off, and edge schedules (dividends at
t = 0 and T, zero and same-date amounts, a dividend larger than the grid's
lower bound, a single-point curve, flat extrapolation past the last tenor).

Bar: prices and Greeks within 1e-9 relative (1e-11 absolute floor), grid
sizes identical.  Theta is (V_prev - V) K / dt with dt the time domain's
mean step; with up to 5000 steps it amplifies value-level rounding by 1/dt,
so it gets an extra absolute allowance of 1e-13 K / dt."""
import json

import numpy as np
import pytest

from conftest import golden, rel_err

pytestmark = pytest.mark.gpu

RTOL = 1e-9
ATOL = 1e-11


def records(pkg, rows):
    p = pkg.pricing_array([r["S"] for r in rows], [r["K"] for r in rows], [r["T"] for r in rows],
                          [r["sigma"] for r in rows], [r["r"] for r in rows], [r["q"] for r in rows],
                          [r["put"] for r in rows])
    keep = pkg.attach_schedules(p, [r.get("curve") for r in rows], [r.get("divs") for r in rows])
    return p, keep


def grids(pkg, rows):
    g = pkg.grid_array(len(rows))
    for i, r in enumerate(rows):
        k = r.get("kind", 0)
        if k == 1:
            g[i] = pkg.grid_array(1, pkg.GRID_FIXED_N, r["nx"], r["nt"])[0]
        elif k == 2:
            g[i] = pkg.grid_array(1, pkg.GRID_SINH, r["nx"], r["nt"], r["x_min"], r["x_max"], r["alpha"])[0]
        elif k == 3:
            g[i] = pkg.grid_array(1, pkg.GRID_UNIFORM, r["nx"], r["nt"], r["x_min"], r["x_max"])[0]
    return g


def check(out, want, rows, dims):
    got = np.stack([out["value"], out["delta"], out["gamma"], out["theta"]], 1)
    tol = RTOL * np.abs(want) + ATOL
    dt = np.array([r["T"] for r in rows]) / dims[:, 1]
    tol[:, 3] += 1e-13 * np.array([r["K"] for r in rows]) / dt
    bad = np.abs(got - want) > tol
    assert not bad.any(), f"max rel {rel_err(got, want).max():.3e}; rows {np.argwhere(bad)[:8].tolist()}"


@pytest.mark.parametrize("case", ["auto", "explicit", "no_rannacher", "edge"])
def test_tv_vs_reference(engine, pkg, case):
    g = golden("tv.npz")
    rows = [json.loads(str(s)) for s in g[f"{case}_rows"]]
    p, keep = records(pkg, rows)
    out = engine.price_arrays(p, grids(pkg, rows), rannacher=bool(g[f"{case}_rannacher"]))
    assert (out["status"] == 0).all(), np.nonzero(out["status"])[0][:8]
    dims = g[f"{case}_dims"]
    assert (out["n_space"] == dims[:, 0]).all(), np.nonzero(out["n_space"] != dims[:, 0])[0][:8]
    assert (out["n_time"] == dims[:, 1]).all(), np.nonzero(out["n_time"] != dims[:, 1])[0][:8]
    check(out, g[f"{case}_out"], rows, dims)
    del keep


def test_tv_mixed_with_constant_options(engine, pkg):
    """A batch whose tiles hold constant-rate and time-varying options: each
    option priced as when alone."""
    g = golden("tv.npz")
    rows = [json.loads(str(s)) for s in g["auto_rows"]][:40]
    p, keep = records(pkg, rows)
    plain = pkg.pricing_array(100.0, np.linspace(85, 115, 45), 1.0, 0.25, 0.03, 0.0, 1)
    alone = engine.price_arrays(plain)
    both = np.concatenate([plain[:20], p, plain[20:]])
    out = engine.price_arrays(both)
    assert (out["status"] == 0).all()
    v = out["value"][np.r_[0:20, 60:85]]
    assert np.abs(v - alone["value"]).max() <= 1e-13 * np.abs(alone["value"]).max()
    dims = g["auto_dims"][:40]
    check(out[20:60], g["auto_out"][:40], rows, dims)
    del keep


def test_tv_validation(engine, pkg):
    base = pkg.pricing_array(100.0, 100.0, 1.0, 0.2, 0.03, 0.0, 1)
    cases = [
        ([[0.5, -0.01], [1.0, -0.03]], None),          # no t = 0 point
        ([[0.0, 0.01], [1.0, -0.03]], None),           # log discount at 0 != 0
        ([[0.0, 0.0], [1.0, -0.03], [1.0, -0.04]], None),  # repeated tenor
        (None, [[1.5, 1.0]]),                          # dividend after expiry
        (None, [[0.5, -1.0]]),                         # negative amount
        (None, [[float("nan"), 1.0]]),
    ]
    for curve, divs in cases:
        p = base.copy()
        keep = pkg.attach_schedules(p, [curve] if curve is not None else None, [divs] if divs is not None else None)
        out = engine.price_arrays(p)
        assert out["status"][0] == pkg.MANGO_ERR_VALIDATION, (curve, divs)
        del keep
    # unsorted tenor points are sorted, as YieldCurve::from_points does
    pts = [[0.0, 0.0], [0.5, -0.01], [1.0, -0.03]]
    a, ka = records(pkg, [{"S": 100.0, "K": 100.0, "T": 1.0, "sigma": 0.2, "r": 0.0, "q": 0.0, "put": 1,
                           "curve": pts}])
    b, kb = records(pkg, [{"S": 100.0, "K": 100.0, "T": 1.0, "sigma": 0.2, "r": 0.0, "q": 0.0, "put": 1,
                           "curve": pts[::-1]}])
    assert engine.price_arrays(a)["value"][0] == engine.price_arrays(b)["value"][0]


def test_tv_mirror(engine, pkg):
    g = golden("tv.npz")
    r = json.loads(str(g["auto_rows"][6]))
    p = pkg.PricingParams(spot=r["S"], strike=r["K"], maturity=r["T"], volatility=r["sigma"],
                          rate=pkg.YieldCurve.from_points(r["curve"]) if "curve" in r else r["r"],
                          dividend_yield=r["q"], option_type=pkg.OptionType.PUT if r["put"] else pkg.OptionType.CALL,
                          discrete_dividends=[pkg.Dividend(t, a) for t, a in r.get("divs", [])])
    res = pkg.BatchAmericanOptionSolver(engine).solve_batch([p, p])
    want = g["auto_out"][6]
    for x in res.results:
        assert abs(x.value() - want[0]) <= RTOL * abs(want[0])


def test_tv_in_chunked_batch(engine, pkg):
    """A one-shot batch large enough to run in chunks, with time-varying
    options in every chunk: each option equals its price from one resident
    (unchunked) batch."""
    n = 70000
    rng = np.random.default_rng(12)
    p = pkg.pricing_array(100.0, rng.uniform(85, 115, n), rng.uniform(0.2, 1.5, n), rng.uniform(0.15, 0.4, n),
                          0.03, 0.0, (np.arange(n) % 2 == 0))
    curve = [(0.0, 0.0), (0.5, -0.012), (1.0, -0.027), (2.0, -0.06)]
    tv = np.arange(n) % 7 == 0
    keep = pkg.attach_schedules(p, [curve if t else None for t in tv],
                                [[(0.4 * T, 1.0)] if t else None for t, T in zip(tv, p["maturity"])])
    grid = pkg.grid_array(1, pkg.GRID_FIXED_N, 51, 60)
    out = engine.price_arrays(p, grid)
    b = engine.batch(p, grid)
    b.run()
    ref = b.results()
    b.close()
    assert (out["status"] == 0).all() and (ref["status"] == 0).all()
    got = np.stack([out["value"], out["delta"], out["gamma"], out["theta"]], 1)
    want = np.stack([ref["value"], ref["delta"], ref["gamma"], ref["theta"]], 1)
    assert np.abs(got - want).max() <= 1e-13 * np.abs(want).max()
    assert (out["n_time"][tv] != 60).any()  # dividend points were added
    del keep


@pytest.mark.parametrize("method", ["brent", "secant", "newton"])
def test_iv_with_schedules_vs_reference(engine, pkg, method):
    """FDM implied volatility for quotes with yield curves and dividends
    against the reference's IVSolver::solve (tests/golden/iv_tv.npz): grid
    sized at 0.3 (PDEGridConfig), dividend times as mandatory points.  Brent
    replays the reference's iterates: roots within 1e-8 and the same
    iteration count (the time-varying march agrees with the reference to
    ~1e-12, so a count may differ on a quote whose last step lands within
    rounding of the tolerance: at most 2 of 96 allowed).  The secant method
    stops elsewhere inside the same price tolerance, so its roots agree
    within 1e-6 in volatility; so do Newton's (its quotes with schedules take
    the secant path, the others Newton's)."""
    g = golden("iv_tv.npz")
    rows = [json.loads(str(s)) for s in g["rows"]]
    n = len(rows)
    q = pkg.query_array([r["S"] for r in rows], [r["K"] for r in rows], [r["T"] for r in rows],
                        [r["r"] for r in rows], [r["q"] for r in rows], [r["put"] for r in rows], g["price"])
    keep = pkg.attach_schedules(q, [r.get("curve") for r in rows], [r.get("divs") for r in rows])
    grids = pkg.grid_array(n, pkg.GRID_FIXED_N_AT_VOL, 101, 200, alpha=g["grid_sigma"])
    out = engine.solve_iv_arrays(q, grids, method={"brent": pkg.IV_BRENT, "secant": pkg.IV_SECANT,
                                                   "newton": pkg.IV_NEWTON}[method])
    ok = g["status"] == 0
    assert (out["status"][ok] == 0).all(), np.nonzero(out["status"][ok])[0][:8]
    err = np.abs(out["implied_vol"][ok] - g["out"][ok, 0])
    if method == "brent":
        assert err.max() < 1e-8, err.max()
        assert np.count_nonzero(out["iterations"][ok] != g["out"][ok, 1]) <= 2
    else:
        # another root finder stopping anywhere |V - P| < 1e-6: the roots
        # agree to that price tolerance over vega (1e-6 in volatility here)
        assert err.max() < 1e-6, err.max()
    del keep


def test_greeks_with_schedules(engine, pkg):
    """Frozen-grid sensitivities of options with a yield curve and
    dividends equal central differences of the pricing path on the same
    explicit grid: vega and dV/dK by bumped inputs, rho by a parallel shift
    of the zero curve (ln D(t) - h t)."""
    curve = np.array([(0.0, 0.0), (0.5, -0.012), (1.0, -0.027), (2.0, -0.06)])
    n = 8
    K = np.linspace(90, 110, n)
    T = np.linspace(0.4, 1.6, n)
    sig = np.full(n, 0.25)
    put = (np.arange(n) % 2 == 0)
    divs = [[(0.5 * t, 1.5)] for t in T]
    grid = pkg.grid_array(1, pkg.GRID_SINH, 141, 300, -2.5, 2.5, 2.0)

    def price(K_, sig_, curves):
        p = pkg.pricing_array(100.0, K_, T, sig_, 0.0, 0.0, put)
        keep = pkg.attach_schedules(p, curves, divs)
        v = engine.price_arrays(p, grid)["value"]
        del keep
        return v

    p = pkg.pricing_array(100.0, K, T, sig, 0.0, 0.0, put)
    keep = pkg.attach_schedules(p, [curve] * n, divs)
    g = engine.greeks_arrays(p, grid)
    assert (g["status"] == 0).all()
    h = 1e-5
    hv, hr, hk = h * sig, h * 1e-2, h * K
    vega = (price(K, sig + hv, [curve] * n) - price(K, sig - hv, [curve] * n)) / (2 * hv)
    up = [np.column_stack([curve[:, 0], curve[:, 1] - hr * curve[:, 0]])] * n
    dn = [np.column_stack([curve[:, 0], curve[:, 1] + hr * curve[:, 0]])] * n
    rho = (price(K, sig, up) - price(K, sig, dn)) / (2 * hr)
    dk = (price(K + hk, sig, [curve] * n) - price(K - hk, sig, [curve] * n)) / (2 * hk)
    for got, want in ((g["vega"], vega), (g["rho"], rho), (g["dstrike"], dk)):
        assert np.abs(got - want).max() <= 1e-9 * np.abs(want).max() + 1e-12
    assert (g["rho"][put] < 0).all() and (g["rho"][~put] > 0).all()
    del keep
