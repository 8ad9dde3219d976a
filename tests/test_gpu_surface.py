"""GPU price-table surface: the separable collocation fit, the EEP step, the
standard table's price query and the whole device-resident build, against the
reference's golden outputs (surface.npz) and the CPU restatement
(oracle/fit_oracle.py, pinned in test_oracle_surface.py).

Bars: prices 1e-12 relative against the reference on the same coefficients;
EEP 1e-12 absolute; fit coefficients 1e-13 of the largest against the
reference's own fit (fit.npz) and within cond(B) x 1e-14 of the dense
restatement; cubic reproduction 1e-11."""
import sys

import numpy as np
import pytest

from conftest import ROOT, golden

sys.path.insert(0, str(ROOT / "oracle"))
import fit_oracle  # noqa: E402

pytestmark = pytest.mark.gpu


def axes_of(g):
    return np.split(g["grids"], np.cumsum(g["sizes"])[:-1])


def records(pkg, p, put, q):
    return pkg.pricing_array(p[:, 0], p[:, 1], p[:, 2], p[:, 3], p[:, 4], q, put)


def test_table_price_vs_reference(engine, pkg):
    g = golden("surface.npz")
    axes = axes_of(g)
    for name, put in (("put", 1), ("call", 0)):
        q = float(g[f"{name}_q"])
        t = engine.price_table_create(axes, g["coeffs"], 100.0, q, put, eep=True)
        v = t.price_arrays(records(pkg, g["params"], put, q))
        ref = g[f"{name}_price"]
        assert np.abs(v - ref).max() <= 1e-12 * np.abs(ref).max() + 1e-13, name
        t.close()


def test_table_without_eep_is_the_transform_leaf(engine, pkg, oracle):
    g = golden("surface.npz")
    axes = axes_of(g)
    t = engine.price_table_create(axes, g["coeffs"], 100.0, 0.0, 1, eep=False)
    v = t.price_arrays(records(pkg, g["params"], 1, 0.0))
    ref = oracle.surface_price(axes, g["coeffs"], g["params"], 100.0, 0.0, 1, eep=False)
    assert np.abs(v - ref).max() <= 1e-13 * np.abs(ref).max() + 1e-14
    assert (v >= 0).all()


def test_eep_decompose_vs_reference(engine):
    g = golden("surface.npz")
    axes = axes_of(g)
    out = engine.eep_decompose(*axes, g["eep_in"], K_ref=100.0, dividend_yield=0.015, option_type=1)
    assert np.abs(out.ravel() - g["eep_out"]).max() < 1e-12


def cubic(a, b, c, d):
    return 1 + a - 2 * a ** 3 + 0.5 * b ** 2 * c - c ** 3 + 3 * d * a ** 2 + b ** 3 * d


def test_fit_reproduces_cubics(engine, oracle):
    axes = [np.linspace(-0.4, 0.3, 11) + 0.01 * np.arange(11) ** 2, np.linspace(0.02, 2.0, 9),
            np.linspace(0.05, 0.8, 7), np.linspace(0.0, 0.08, 5)]
    mesh = np.meshgrid(*axes, indexing="ij")
    coeffs, stats = engine.bspline4d_fit(axes, cubic(*mesh))
    assert stats["failed_slices"] == [0, 0, 0, 0]
    assert max(stats["max_residual"]) < 1e-12
    rng = np.random.default_rng(11)
    q = np.stack([rng.uniform(a[0], a[-1], 2000) for a in axes], 1)
    surf = engine.bspline4d(axes, coeffs)
    assert np.abs(surf.eval(q) - cubic(*q.T)).max() < 1e-11
    assert np.abs(oracle.bspline4d_eval(axes, coeffs, q) - cubic(*q.T)).max() < 1e-11


def test_fit_vs_dense_restatement(engine):
    g = golden("surface.npz")
    axes = axes_of(g)
    vals = np.random.default_rng(3).standard_normal([a.size for a in axes])
    coeffs, stats = engine.bspline4d_fit(axes, vals)
    ref = fit_oracle.fit4d(axes, vals)
    conds = [np.linalg.cond(fit_oracle.collocation_matrix(a), 1) for a in axes]
    assert np.allclose(stats["condition"], conds, rtol=1e-9)
    bound = np.prod(conds) * 1e-14 * np.abs(ref).max()
    assert np.abs(coeffs - ref).max() <= bound, (np.abs(coeffs - ref).max(), bound)


def test_fit_vs_reference_fit(engine):
    """The device fit against the reference's BSplineNDSeparable<double,4>::fit
    (fit.npz): every coefficient on the 12 x 8 x 6 x 5 surface axes, 4096
    sampled coefficients and the sum of all on the full 50 x 30 x 20 x 10
    table axes, at 1e-13 of the largest coefficient; per-axis condition
    numbers against the reference's dgbcon estimates (rtol 1e-9)."""
    g = golden("fit.npz")
    axes = np.split(g["rand_grids"], np.cumsum(g["rand_sizes"])[:-1])
    coeffs, stats = engine.bspline4d_fit(axes, g["rand_values"].reshape([a.size for a in axes]))
    ref = g["rand_coeffs"]
    assert np.abs(coeffs.ravel() - ref).max() <= 1e-13 * np.abs(ref).max()
    assert np.allclose(stats["condition"], g["rand_cond"], rtol=1e-9)
    axes = np.split(g["table_grids"], np.cumsum(g["table_sizes"])[:-1])
    vals = np.random.default_rng(int(g["table_seed"])).standard_normal(int(np.prod(g["table_sizes"])))
    coeffs, stats = engine.bspline4d_fit(axes, vals.reshape([a.size for a in axes]))
    c = coeffs.ravel()
    amax = float(g["table_coeff_absmax"])
    assert np.abs(c[g["table_idx"]] - g["table_coeffs"]).max() <= 1e-13 * amax
    assert abs(c.sum() - float(g["table_coeff_sum"])) <= 1e-13 * amax * c.size
    assert np.allclose(stats["condition"], g["table_cond"], rtol=1e-9)


def test_fit_failure_and_validation(engine, pkg):
    axes = [np.linspace(0, 1, 6), np.linspace(0, 1, 5), np.linspace(0, 1, 4), np.linspace(0, 1, 4)]
    vals = np.random.default_rng(1).standard_normal([6, 5, 4, 4])
    with pytest.raises(pkg.EngineError) as e:
        engine.bspline4d_fit(axes, vals, tolerance=1e-300)
    assert e.value.status == pkg.MANGO_ERR_SOLVER and sum(e.value.stats["failed_slices"]) > 0
    bad = vals.copy()
    bad[1, 2, 3, 0] = np.nan
    with pytest.raises(pkg.EngineError) as e:
        engine.bspline4d_fit(axes, bad)
    assert e.value.status == pkg.MANGO_ERR_VALIDATION
    with pytest.raises(pkg.EngineError):
        engine.bspline4d_fit([np.linspace(0, 1, 3)] + axes[1:], np.zeros([3, 5, 4, 4]))


TABLE_AXES = (np.linspace(np.log(0.7), np.log(1.3), 10), np.linspace(0.05, 1.5, 7),
              np.linspace(0.1, 0.6, 5), np.linspace(0.0, 0.06, 4))


def test_table_build_vs_restated_pipeline(engine, pkg, oracle):
    """Device build (sweep -> EEP -> fit -> surface) against the CPU
    composition of the same stages: the GPU sweep tensor (pinned to the
    reference in test_gpu_table.py), the restated EEP and fit, the C
    B-spline evaluation and the European add-back."""
    grid = pkg.PDEGridConfig(-3.0, 3.0, 101, 200)
    q = 0.01
    table, stats = engine.price_table_build(*TABLE_AXES, K_ref=100.0, dividend_yield=q, option_type=1,
                                            grid=grid, eep=True)
    assert stats["failed_slices"] == [0, 0, 0, 0] and stats["failed_pde_slices"] == 0
    tensor, _, failed = engine.price_table_sweep(*TABLE_AXES, 100.0, q, 1, grid)
    assert failed == 0
    eep = fit_oracle.eep_decompose(TABLE_AXES, tensor, 100.0, q, True)
    coeffs = fit_oracle.fit4d(TABLE_AXES, eep)
    rng = np.random.default_rng(9)
    n = 512
    p = np.stack([np.full(n, 100.0), 100.0 / np.exp(rng.uniform(TABLE_AXES[0][0], TABLE_AXES[0][-1], n)),
                  rng.uniform(0.05, 1.5, n), rng.uniform(0.1, 0.6, n), rng.uniform(0.0, 0.06, n)], 1)
    got = table.price_arrays(records(pkg, p, 1, q))
    ref = oracle.surface_price(TABLE_AXES, coeffs, p, 100.0, q, 1)
    assert np.abs(got - ref).max() <= 1e-9 * np.abs(ref).max()
    # the mirror's validated scalar price
    pp = pkg.PricingParams(spot=100.0, strike=float(p[0, 1]), maturity=float(p[0, 2]), rate=float(p[0, 4]),
                           dividend_yield=q, option_type=pkg.OptionType.PUT, volatility=float(p[0, 3]))
    assert abs(table.price(pp) - got[0]) < 1e-12 * abs(got[0]) + 1e-14
    with pytest.raises(ValueError):
        table.price(pkg.PricingParams(spot=100.0, strike=100.0, maturity=5.0, rate=0.01, dividend_yield=q,
                                      option_type=pkg.OptionType.PUT, volatility=0.2))
    table.close()


def test_table_build_failure_rate_and_repair(engine, pkg, oracle, monkeypatch):
    """PriceTableBuilderND<4>'s failure handling (bspline_builder.cpp:95-101,
    773-959) driven by the host-side hook MANGO_GPU_TABLE_FAIL, which reports
    slice 5 (sigma 1, r 1) failed as a whole and slice 17 (sigma 4, r 1) at
    maturity 3 only.  max_failure_rate 0 (strict, the reference's default)
    and 0.03 refuse the build (1 of 20 slices = 0.05); 0.05 builds it after
    the repair: the whole slice becomes a copy of its nearest valid neighbour
    in the search order (dsigma -1 first: sigma 0, r 1), the failed maturity
    the index-weighted interpolation of maturities 2 and 4.  The repaired
    table equals the restated pipeline run on the tensor repaired the same
    way."""
    grid = pkg.PDEGridConfig(-3.0, 3.0, 101, 200)
    args = (*TABLE_AXES, 100.0, 0.0, 1, grid)
    with pytest.raises(pkg.EngineError, match="max_failure_rate"):
        engine.price_table_build(*args, max_failure_rate=1.5)
    monkeypatch.setenv("MANGO_GPU_TABLE_FAIL", "5,17:3")
    for rate in (0.0, 0.03):
        with pytest.raises(pkg.EngineError, match="above max_failure_rate"):
            engine.price_table_build(*args, max_failure_rate=rate)
    table, info = engine.price_table_build(*args, max_failure_rate=0.05)
    assert info["failed_pde_slices"] == 1
    assert info["repaired_slices"] == 1 and info["repaired_points"] == 1
    monkeypatch.delenv("MANGO_GPU_TABLE_FAIL")
    tensor, _, failed = engine.price_table_sweep(*args)
    assert failed == 0
    rep = tensor.copy()
    rep[:, :, 1, 1] = tensor[:, :, 0, 1]
    rep[:, 3, 4, 1] = 0.5 * (tensor[:, 2, 4, 1] + tensor[:, 4, 4, 1])
    coeffs = fit_oracle.fit4d(TABLE_AXES, fit_oracle.eep_decompose(TABLE_AXES, rep, 100.0, 0.0, True))
    rng = np.random.default_rng(17)
    n = 512
    p = np.stack([np.full(n, 100.0), 100.0 / np.exp(rng.uniform(TABLE_AXES[0][0], TABLE_AXES[0][-1], n)),
                  rng.uniform(0.05, 1.5, n), rng.uniform(0.1, 0.6, n), rng.uniform(0.0, 0.06, n)], 1)
    got = table.price_arrays(records(pkg, p, 1, 0.0))
    ref = oracle.surface_price(TABLE_AXES, coeffs, p, 100.0, 0.0, 1)
    assert np.abs(got - ref).max() <= 1e-9 * np.abs(ref).max()
    clean, info = engine.price_table_build(*args)
    assert info["repaired_slices"] == 0 and info["repaired_points"] == 0
    assert np.abs(clean.price_arrays(records(pkg, p, 1, 0.0)) - got).max() > 1e-6
    table.close()
    clean.close()


def test_table_build_interpolates_at_nodes(engine, pkg):
    """At the table's nodes the surface returns the PDE price it was built
    from, through the EEP floor: K/K_ref (eep_floor(K_ref u - E) + E), with
    u the normalised PDE price and E the European price at K_ref."""
    grid = pkg.PDEGridConfig(-3.0, 3.0, 101, 200)
    table, _ = engine.price_table_build(*TABLE_AXES, K_ref=100.0, dividend_yield=0.0, option_type=1, grid=grid)
    tensor, _, _ = engine.price_table_sweep(*TABLE_AXES, 100.0, 0.0, 1, grid)
    for mi, ti, vi, ri in ((0, 3, 2, 1), (5, 3, 2, 1), (9, 6, 4, 3), (2, 0, 0, 0)):
        m, tau, sig, r = (TABLE_AXES[d][i] for d, i in enumerate((mi, ti, vi, ri)))
        K = 100.0 / np.exp(m)
        e = fit_oracle.european_price(100.0 * np.exp(m), 100.0, tau, sig, r, 0.0, True)
        want = K / 100.0 * (fit_oracle.eep_floor(100.0 * tensor[mi, ti, vi, ri] - e) + e)
        v = table.price_arrays(pkg.pricing_array(100.0, K, tau, sig, r, 0.0, 1))[0]
        assert abs(v - want) < 1e-9 * K, (mi, ti, vi, ri, v, want)
    table.close()


def test_make_price_table_mirror(engine, pkg):
    cfg = pkg.IVSolverFactoryConfig(option_type=pkg.OptionType.PUT, spot=100.0, dividend_yield=0.0,
                                    grid=pkg.IVGrid(moneyness=np.linspace(0.8, 1.2, 8), vol=[0.15, 0.25, 0.35, 0.45],
                                                    rate=[0.0, 0.02, 0.04, 0.06]),
                                    backend=pkg.BSplineBackend(maturity_grid=[0.25, 0.5, 0.75, 1.0, 1.5]))
    t = pkg.make_price_table(cfg, engine)
    assert t.surface_type == "bspline" and t.option_type == pkg.OptionType.PUT
    p = pkg.PricingParams(spot=100.0, strike=100.0, maturity=1.0, rate=0.03, dividend_yield=0.0,
                          option_type=pkg.OptionType.PUT, volatility=0.25)
    direct = pkg.american_option_price(p).value()
    assert abs(t.price(p) - direct) < 0.02 * direct
    t.close()


def test_table_data_round_trip(engine, pkg):
    """to_data / from_data (the reference's PriceTableData for bspline_4d):
    a built table exported and reconstructed prices identically; knots that
    are not the grids' clamped knots and bounds off the grids are refused."""
    grid = pkg.PDEGridConfig(-3.0, 3.0, 101, 200)
    table, _ = engine.price_table_build(*TABLE_AXES, K_ref=100.0, dividend_yield=0.01, option_type=1, grid=grid)
    d = table.to_data()
    assert d.surface_type == "bspline_4d" and len(d.segments) == 1
    s = d.segments[0]
    assert s.num_pts == [a.size for a in TABLE_AXES] and s.K_ref == 100.0
    for a, g, k in zip(TABLE_AXES, s.grids, s.knots):
        assert np.array_equal(a, g) and np.array_equal(k, fit_oracle.clamped_knots(a))
    t2 = pkg.from_data(d, engine)
    p = records(pkg, np.stack([np.full(64, 100.0), 100.0 / np.exp(np.linspace(-0.3, 0.2, 64)),
                               np.full(64, 0.8), np.full(64, 0.25), np.full(64, 0.03)], 1), 1, 0.01)
    assert np.array_equal(table.price_arrays(p), t2.price_arrays(p))
    s.knots[2] = s.knots[2] + 1e-9
    with pytest.raises(pkg.SerializationError):
        pkg.from_data(d, engine)
    s.knots[2] = s.knots[2] - 1e-9
    d.bounds_sigma_max = 0.7
    with pytest.raises(pkg.SerializationError):
        pkg.from_data(d, engine)
    table.close()
    t2.close()


@pytest.mark.parametrize("name,q,put", [("put", 0.0, 1), ("put_q", 0.02, 1), ("call_q", 0.01, 0)])
def test_table_greeks_vs_reference(engine, pkg, name, q, put):
    """delta / gamma / theta / rho of the standard table (EEPLayer over
    TransformLeaf with analytic spline partials) against the reference's
    PriceTable on the same coefficients (tests/golden/table_greeks.npz).
    Bar: 1e-11 of each Greek's largest magnitude (the reference divides by
    knot spans where the kernel multiplies by their reciprocals)."""
    g = golden("table_greeks.npz")
    t = engine.price_table_create(axes_of(g), g["coeffs"], 100.0, q, put, eep=True)
    out, status = t.greeks_arrays(records(pkg, g["params"], put, q))
    assert (status == 0).all()
    ref = g[f"{name}_greeks"]
    for j in range(4):
        scale = np.abs(ref[:, j]).max()
        assert np.abs(out[:, j] - ref[:, j]).max() <= 1e-11 * scale + 1e-13, (name, j)
    # the single-record mirror of mango_price_table_delta etc.
    p0 = pkg.PricingParams(spot=100.0, strike=float(g["params"][5, 1]), maturity=float(g["params"][5, 2]),
                           volatility=float(g["params"][5, 3]), rate=float(g["params"][5, 4]),
                           dividend_yield=q, option_type=pkg.OptionType(put))
    for j, f in enumerate((t.delta, t.gamma, t.theta, t.rho)):
        assert f(p0) == out[5, j]


def test_table_greeks_validation(engine, pkg):
    """Records failing AnyPriceTable::validate_pricing_params get NaN and
    MANGO_ERR_VALIDATION; the rest of the batch is still computed."""
    g = golden("table_greeks.npz")
    t = engine.price_table_create(axes_of(g), g["coeffs"], 100.0, 0.0, 1, eep=True)
    p = g["params"][:8].copy()
    recs = records(pkg, p, 1, 0.0)
    recs["maturity"][1] = 5.0          # outside the maturity axis
    recs["option_type"][2] = 0         # call on a put table
    recs["dividend_yield"][3] = 0.01   # yield mismatch
    recs["volatility"][4] = -0.2       # not positive
    recs["strike"][5] = 10.0           # log-moneyness outside the axis
    out, status = t.greeks_arrays(recs)
    bad = [1, 2, 3, 4, 5]
    assert (status[bad] == pkg.MANGO_ERR_VALIDATION).all()
    assert np.isnan(out[bad]).all()
    good = [0, 6, 7]
    assert (status[good] == 0).all()
    assert np.abs(out[good] - g["put_greeks"][good]).max() <= 1e-11 * np.abs(g["put_greeks"]).max()
    with pytest.raises(ValueError):
        t.delta(pkg.PricingParams(spot=100.0, strike=100.0, maturity=5.0, volatility=0.2, rate=0.02,
                                  dividend_yield=0.0, option_type=pkg.OptionType.PUT))
