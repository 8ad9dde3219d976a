"""Interpolated implied volatility and vega on a GPU price table, against
the reference's InterpolatedIVSolver<BSplinePriceTable>::solve_batch and
PriceTable vega on the same coefficients (tests/golden/interp_iv.npz: a real
EEP table from the reference's own sweep).

Bars: vega 1e-11 relative (the analytic partial uses precomputed reciprocal
knot gaps where the reference divides); statuses identical (the C ABI's
map_iv_error categories); implied vols within 1e-9 with identical Brent
iteration counts (the same iterate sequence on prices that agree to
~1e-13)."""
import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu


def table_from(engine, g):
    axes = np.split(g["grids"], np.cumsum(g["sizes"])[:-1])
    return engine.price_table_create(axes, g["coeffs"], 100.0, 0.0, 1, eep=True)


def test_table_vega_vs_reference(engine, pkg):
    g = golden("interp_iv.npz")
    t = table_from(engine, g)
    p = g["vega_params"]
    v = t.vega_arrays(pkg.pricing_array(p[:, 0], p[:, 1], p[:, 2], p[:, 3], p[:, 4], 0.0, 1))
    ref = g["vega"]
    assert np.abs(v - ref).max() <= 1e-11 * np.abs(ref).max()
    t.close()


def test_interpolated_iv_vs_reference(engine, pkg):
    g = golden("interp_iv.npz")
    t = table_from(engine, g)
    q = g["quotes"]
    queries = pkg.query_array(q[:, 0], q[:, 1], q[:, 2], q[:, 3], q[:, 4], q[:, 5].astype(np.int32), q[:, 6])
    cfg = pkg.InterpolatedIVSolverConfig(*[float(x) for x in g["cfg"]])
    cfg.max_iter = int(cfg.max_iter)
    out = t.iv_arrays(queries, cfg)
    st = g["status"]
    assert (out["status"] == st).all(), np.nonzero(out["status"] != st)[0][:10]
    ok = st == 0
    assert ok.sum() > 900
    ref = g["out"]
    assert np.abs(out["implied_vol"][ok] - ref[ok, 0]).max() < 1e-9
    assert (out["iterations"][ok] == ref[ok, 1]).all()
    # default config equals the reference defaults
    out2 = t.iv_arrays(queries)
    assert np.array_equal(out2["status"], out["status"])
    assert np.array_equal(out2["implied_vol"][ok], out["implied_vol"][ok])
    t.close()


def test_vega_threshold_rejects_flat_quotes(engine, pkg):
    g = golden("interp_iv.npz")
    t = table_from(engine, g)
    # a short-dated deep-OTM put inside the table's range: vega ~ 0
    q = pkg.query_array(100.0, 100.0 / 1.29, 0.03, 0.02, 0.0, 1, 1e-12)
    hi = pkg.InterpolatedIVSolverConfig(vega_threshold=1e3)
    assert t.iv_arrays(q, hi)["status"][0] == pkg.MANGO_ERR_SOLVER
    t.close()


def test_interpolated_iv_mirror(engine, pkg):
    cfg = pkg.IVSolverFactoryConfig(option_type=pkg.OptionType.PUT, spot=100.0, dividend_yield=0.0,
                                    grid=pkg.IVGrid(moneyness=np.linspace(0.8, 1.2, 9), vol=[0.1, 0.2, 0.3, 0.4, 0.5],
                                                    rate=[0.0, 0.02, 0.04, 0.06]),
                                    backend=pkg.BSplineBackend(maturity_grid=[0.25, 0.5, 0.75, 1.0, 1.5]))
    solver = pkg.make_interpolated_iv_solver(cfg, engine)
    p = pkg.PricingParams(spot=100.0, strike=105.0, maturity=0.8, rate=0.03, dividend_yield=0.0,
                          option_type=pkg.OptionType.PUT, volatility=0.27)
    px = solver.table.price(p)
    r = solver.solve(pkg.IVQuery(spot=100.0, strike=105.0, maturity=0.8, rate=0.03, dividend_yield=0.0,
                                 option_type=pkg.OptionType.PUT, market_price=px))
    assert abs(r.implied_vol - 0.27) < 1e-5
    batch = solver.solve_batch([pkg.IVQuery(spot=100.0, strike=105.0, maturity=0.8, rate=0.03, dividend_yield=0.01,
                                            option_type=pkg.OptionType.PUT, market_price=px)])
    assert batch.failed_count == 1
    solver.table.close()
