"""GPU FDM implied volatility with the safeguarded secant root finder.

The secant path stops on Brent's own test (|V(sigma) - P| < tol), so its
root and Brent's both lie within tol / vega of the exact root of the same
discrete objective: the bar is |sigma_secant - sigma_brent| <= 2 tol / vega
(plus 1e-8), |V(sigma_secant) - P| < tol checked by re-pricing on the GPU,
and failure statuses identical to the reference Brent's (quotes the secant
does not settle are re-solved by Brent), except where Brent finds no sign
change over its bracket and the secant still finds |V - P| < tol."""
import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu

TOL = 1e-6


def per_quote_grid(pkg, vol, nx=101, nt=498):
    return pkg.grid_array(len(vol), pkg.GRID_FIXED_N_AT_VOL, nx, nt, alpha=vol)


def vega_on_grid(engine, pkg, S, K, T, r, q, put, sig, grids, h=1e-4):
    up = engine.price_arrays(pkg.pricing_array(S, K, T, sig + h, r, q, put), grids)["value"]
    dn = engine.price_arrays(pkg.pricing_array(S, K, T, np.maximum(sig - h, 1e-3), r, q, put), grids)["value"]
    return np.abs(up - dn) / (sig + h - np.maximum(sig - h, 1e-3))


def test_secant_vs_reference_golden(engine, pkg):
    g = golden("iv.npz")
    q = pkg.query_array(g["S"], g["K"], g["T"], g["r"], g["q"], g["is_put"], g["price"])
    grids = per_quote_grid(pkg, g["true_vol"])
    out = engine.solve_iv_arrays(q, grids, method=pkg.IV_SECANT)
    assert (out["status"] == 0).all()
    sig = out["implied_vol"]
    vega = vega_on_grid(engine, pkg, g["S"], g["K"], g["T"], g["r"], g["q"], g["is_put"], sig, grids)
    d = np.abs(sig - g["out"][:, 0])
    assert (d <= 2 * TOL / vega + 1e-8).all(), f"worst {d.max():.3e}"
    assert np.abs(sig - g["true_vol"]).max() < 1e-6
    # fewer evaluations than the reference's Brent iterations + 2 endpoints
    assert out["iterations"].mean() < (g["out"][:, 1] + 2).mean()


def test_secant_vs_oracle_sample(engine, pkg, oracle):
    rng = np.random.default_rng(78)
    n = 512
    S = np.full(n, 100.0)
    K = S * rng.uniform(0.8, 1.2, n)
    T = rng.uniform(0.02, 2.0, n)
    r = rng.uniform(0.0, 0.08, n)
    q = rng.uniform(0.0, 0.04, n)
    vt = rng.uniform(0.05, 0.8, n)
    put = (np.arange(n) % 3 != 0).astype(np.int32)
    grids = per_quote_grid(pkg, vt)
    px = engine.price_arrays(pkg.pricing_array(S, K, T, vt, r, q, put), grids)
    assert (px["status"] == 0).all()
    quotes = pkg.query_array(S, K, T, r, q, put, px["value"])
    out = engine.solve_iv_arrays(quotes, grids, method=pkg.IV_SECANT)
    ref, st = oracle.iv_batch(S, K, T, r, q, put, px["value"], vt, 101, 498)
    # Status categories are Brent's, except that a quote Brent rejects with a
    # bracketing error (no sign change of V - P over [0.01, upper]: V flat
    # within rounding of P at low vol, or not monotone at high vol on a
    # narrow grid) may still get a root with |V - P| < tol from the secant.
    brk = st == 10
    assert ((out["status"] != 0) == (st != 0))[~brk].all()
    assert np.isin(out["status"][brk], (0, pkg.MANGO_ERR_BRACKETING)).all()
    extra = brk & (out["status"] == 0)
    if extra.any():
        sel2 = lambda a: np.asarray(a)[extra]
        v2 = engine.price_arrays(pkg.pricing_array(sel2(S), sel2(K), sel2(T), out["implied_vol"][extra], sel2(r),
                                                   sel2(q), sel2(put)), grids[extra])["value"]
        assert np.abs(v2 - sel2(px["value"])).max() < TOL
    ok = st == 0
    sig = out["implied_vol"][ok]
    sel = lambda a: np.asarray(a)[ok]
    # the defining property, re-priced on the GPU at the returned vol
    v = engine.price_arrays(pkg.pricing_array(sel(S), sel(K), sel(T), sig, sel(r), sel(q), sel(put)),
                            grids[ok])["value"]
    assert np.abs(v - sel(px["value"])).max() < TOL
    vega = vega_on_grid(engine, pkg, sel(S), sel(K), sel(T), sel(r), sel(q), sel(put), sig, grids[ok])
    d = np.abs(sig - ref[ok, 0])
    far = d > 2 * TOL / np.maximum(vega, 1e-12) + 1e-8
    # Roots further apart than 2 tol / vega mean the discrete objective has
    # more than one root: both points solve |V - P| < tol, and between them V
    # is either flat (within 20 tol of P: the price barely depends on the
    # vol there) or not monotone (it leaves the range of its end values).
    for j in np.nonzero(far)[0]:
        i = np.nonzero(ok)[0][j]
        seg = np.linspace(sig[j], ref[i, 0], 17)
        vs = engine.price_arrays(pkg.pricing_array(S[i], K[i], T[i], seg, r[i], q[i], put[i]),
                                 grids[i:i + 1])["value"] - px["value"][i]
        assert abs(vs[0]) < TOL and abs(vs[-1]) < TOL, (i, vs[0], vs[-1])
        flat = np.abs(vs).max() < 20 * TOL
        lo_end, hi_end = min(vs[0], vs[-1]), max(vs[0], vs[-1])
        bumpy = (vs[1:-1] < lo_end - TOL).any() or (vs[1:-1] > hi_end + TOL).any()
        assert flat or bumpy, (i, sig[j], ref[i, 0], vs)
    assert far.mean() < 0.02
    assert np.mean(np.abs(sig - vt[ok]) < 1e-6) > 0.95


def test_secant_fallback_statuses(engine, pkg):
    # Quotes whose roots fall outside Brent's bracket [0.01, upper] go to
    # Brent, which reports them exactly as the reference does.
    S = np.array([100.0, 100.0, 100.0, 100.0])
    K = np.array([100.0, 100.0, 60.0, 100.0])
    T = np.array([1.0, 1.0, 1.0, 0.5])
    put = np.array([1, 1, 0, 0], dtype=np.int32)
    grids = pkg.grid_array(4, pkg.GRID_FIXED_N_AT_VOL, 101, 300, alpha=np.full(4, 0.3))
    # 0: ordinary put; 1: put priced near its upper bound K, above the value at
    # every vol in [0.01, 3]; 2: ITM call priced between intrinsic and the
    # vol-0.01 value S - K e^{-rT}; 3: ordinary call
    px = engine.price_arrays(pkg.pricing_array(S, K, T, np.array([0.3, 0.3, 0.3, 0.2]), 0.03, 0.0, put), grids)
    prices = px["value"].copy()
    prices[1] = 99.0
    prices[2] = 40.5
    quotes = pkg.query_array(S, K, T, 0.03, 0.0, put, prices)
    a = engine.solve_iv_arrays(quotes, grids, method=pkg.IV_BRENT)
    b = engine.solve_iv_arrays(quotes, grids, method=pkg.IV_SECANT)
    assert (a["status"] == b["status"]).all(), (a["status"], b["status"])
    fail = a["status"] != 0
    assert fail[1] and fail[2]
    assert (a["iterations"][fail] == b["iterations"][fail]).all()
    assert abs(b["implied_vol"][0] - 0.3) < 1e-6 and abs(b["implied_vol"][3] - 0.2) < 1e-6


def test_secant_error_slots_and_mirror(engine, pkg):
    q = pkg.query_array([100, -1, 100], [100, 100, 100], 1.0, 0.05, 0.0, [1, 1, 1], [5.0, 5.0, 150.0])
    out = engine.solve_iv_arrays(q, pkg.grid_array(1, pkg.GRID_FIXED_N_AT_VOL, 101, 200, alpha=0.3),
                                 method=pkg.IV_SECANT)
    assert out["status"][0] == 0
    assert out["status"][1] == pkg.MANGO_ERR_VALIDATION
    assert out["status"][2] == pkg.MANGO_ERR_ARBITRAGE
    solver = pkg.IVSolver(pkg.IVSolverConfig(grid=pkg.FixedGrid(101, 300), grid_vol=0.25, method=pkg.IV_SECANT),
                          engine=engine)
    px = engine.price_arrays(pkg.pricing_array(100, 95, 0.75, 0.35, 0.03, 0.01, 1),
                             pkg.grid_array(1, pkg.GRID_FIXED_N_AT_VOL, 101, 300, alpha=0.25))
    res = solver.solve(pkg.IVQuery(spot=100, strike=95, maturity=0.75, rate=0.03, dividend_yield=0.01,
                                   option_type=pkg.OptionType.PUT, market_price=float(px["value"][0])))
    assert abs(res.implied_vol - 0.35) < 1e-6
    with pytest.raises(Exception):
        engine.solve_iv_arrays(q[:1], pkg.grid_array(1, pkg.GRID_FIXED_N_AT_VOL, 101, 200, alpha=0.3), method=7)
