"""Forward-mode (tangent-linear) sensitivities of the march
(mango_gpu_price_american_tangent_batch) against central differences of
the pricing kernel on the same frozen grid (mango_gpu_price_american_greeks_
batch), plus the value against the pricing batch.

The discrete price is piecewise smooth in each parameter: a node of the
obstacle's active set (or a deep-ITM lock row) flips at some time step when
the parameter moves far enough, and a central difference whose bump
straddles such a flip differs from the exact derivative at the point.  As
the bump shrinks from 1e-5 to 1e-7 relative the differences converge onto
the tangent, so each sensitivity is compared with the closest of the
differences at 1e-5, 1e-6 and 1e-7 (until the smallest bump's rounding
error dominates).

Bars: value 1e-11 relative to the pricing batch (same algorithm, different
kernel: rounding only); delta 1e-9; sensitivities on 101 x 498 grids 2e-6
relative + 1e-6 absolute for 99% of the options and 1e-3 relative for all,
with a median relative error at h = 1e-5 below 1e-7; on the automatic grids
(up to 5000 steps, so more flips per bump) 2e-5 relative + 1e-5 absolute for
95% of the options."""
import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu


def inputs(pkg, n, seed, mixed):
    rng = np.random.default_rng(seed)
    S = np.full(n, 100.0)
    K = rng.uniform(80, 120, n)
    T = rng.uniform(0.1, 2.0, n)
    sig = rng.uniform(0.1, 0.5, n)
    r = rng.uniform(0.0, 0.08, n)
    q = rng.uniform(0.0, 0.04, n)
    put = (np.arange(n) % 2 == 0).astype(np.int32) if mixed else np.ones(n, np.int32)
    return pkg.pricing_array(S, K, T, sig, r, q, put)


@pytest.mark.parametrize("mixed", [False, True])
def test_tangent_vs_central_differences(engine, pkg, mixed):
    params = inputs(pkg, 512, 7 + mixed, mixed)
    grid = pkg.grid_array(1, pkg.GRID_FIXED_N, 101, 498)
    tan = engine.tangent_arrays(params, grid)
    fds = [engine.greeks_arrays(params, grid, h) for h in (1e-5, 1e-6, 1e-7)]
    fd = fds[0]
    assert (tan["status"] == 0).all()
    assert (tan["n_space"] == fd["n_space"]).all() and (tan["n_time"] == fd["n_time"]).all()
    v = fd["value"]
    assert np.abs(tan["value"] - v).max() <= 1e-11 * np.abs(v).max()
    assert np.abs(tan["delta"] - fd["delta"]).max() <= 1e-9
    for k in ("vega", "rho", "dividend_rho", "dstrike"):
        err = np.min([np.abs(tan[k] - f[k]) for f in fds], axis=0)
        bar = 2e-6 * np.abs(fd[k]) + 1e-6
        assert (err <= bar).mean() >= 0.99, (k, err.max())
        assert (err <= 1e-3 * np.abs(fd[k]) + 1e-6).all(), (k, err.max())
        assert np.median(np.abs(tan[k] - fd[k]) / (np.abs(fd[k]) + 1e-12)) <= 1e-7, k
    assert np.isnan(tan["gamma"]).all() and np.isnan(tan["theta"]).all()


def test_tangent_auto_grid_and_validation(engine, pkg):
    params = inputs(pkg, 64, 3, True)
    params["volatility"][5] = -0.1          # invalid
    tan = engine.tangent_arrays(params)
    fd = engine.greeks_arrays(params, None, 1e-5)
    ok = np.arange(64) != 5
    assert tan["status"][5] == pkg.MANGO_ERR_VALIDATION and np.isnan(tan["vega"][5])
    assert (tan["status"][ok] == 0).all()
    assert np.abs(tan["value"][ok] - fd["value"][ok]).max() <= 1e-11 * np.abs(fd["value"][ok]).max()
    fd7 = engine.greeks_arrays(params, None, 1e-7)
    for k in ("vega", "rho", "dividend_rho", "dstrike"):
        err = np.minimum(np.abs(tan[k][ok] - fd[k][ok]), np.abs(tan[k][ok] - fd7[k][ok]))
        assert (err <= 2e-5 * np.abs(fd[k][ok]) + 1e-5).mean() >= 0.95, (k, err.max())


def test_tangent_vs_oracle_tangent(engine, pkg, oracle):
    """The GPU march and the oracle's restatement of the same forward-mode
    derivative on the same 101 x 498 grids.  Bars: value 1e-11, the
    sensitivities 1e-8 relative + 1e-9 (rounding of the precomputed row
    coefficients against the per-stage ones, through 998 stages)."""
    params = inputs(pkg, 24, 21, True)
    grid = pkg.grid_array(1, pkg.GRID_FIXED_N, 101, 498)
    tan = engine.tangent_arrays(params, grid)
    one = engine.tangent_arrays(params, grid, vega_only=True)
    assert (tan["status"] == 0).all() and (one["status"] == 0).all()
    for i in range(params.size):
        x, _ = pkg.resolve_grid(params[i:i + 1], pkg.FixedGrid(101, 498))
        p = params[i]
        rc, t6 = oracle.price_tangent_on_grid(p["spot"], p["strike"], p["maturity"], p["volatility"],
                                              p["rate_const"], p["dividend_yield"], p["option_type"], x, 498)
        assert rc == 0
        assert abs(tan["value"][i] - t6[0]) <= 1e-11 * abs(t6[0]) + 1e-13, i
        assert abs(tan["delta"][i] - t6[1]) <= 1e-9, i
        for col, k in ((2, "vega"), (3, "rho"), (4, "dividend_rho"), (5, "dstrike")):
            assert abs(tan[k][i] - t6[col]) <= 1e-8 * abs(t6[col]) + 1e-9, (i, k, tan[k][i], t6[col])
        assert abs(one["vega"][i] - t6[2]) <= 1e-8 * abs(t6[2]) + 1e-9, (i, one["vega"][i], t6[2])


def test_vega_batch_matches_three_direction_tangent(engine, pkg):
    """mango_gpu_price_american_vega_batch carries the volatility tangent
    alone: its value and delta equal the three-direction march's bit for bit
    (the same primal), its vega and dV/dK to 1e-10 relative (the same
    formulas, compiled with another contraction order)."""
    params = inputs(pkg, 256, 5, True)
    for grid in (pkg.grid_array(1, pkg.GRID_FIXED_N, 101, 498), None):
        full = engine.tangent_arrays(params, grid)
        one = engine.tangent_arrays(params, grid, vega_only=True)
        assert (one["status"] == 0).all() and (full["status"] == 0).all()
        for k in ("value", "delta"):
            assert (one[k] == full[k]).all(), k
        for k in ("vega", "dstrike"):
            assert np.allclose(one[k], full[k], rtol=1e-10, atol=1e-12), (k, np.abs(one[k] - full[k]).max())
        assert np.isnan(one["rho"]).all() and np.isnan(one["dividend_rho"]).all()


def test_tangent_vs_reference_frozen_grid_differences(engine, pkg):
    """1,024 puts of the differentiation workload against the reference's
    own central differences on each option's frozen 101 x 498 grid
    (greeks_fd.npz: h = 1e-5, 1e-6, 1e-7).  The same bars as against the
    engine's own differences: the closest difference within 2e-6 relative +
    1e-6 for 99 % of the options and 1e-3 relative for all (a difference that
    straddles a change of the obstacle's active set is not the derivative at
    the point); and the engine's own h = 1e-5 differences reproduce the
    reference's (same bumps, same flips) to 1e-5 relative."""
    g = golden("greeks_fd.npz")
    params = pkg.pricing_array(g["S"], g["K"], g["T"], g["sigma"], g["r"], g["q"], g["is_put"])
    grid = pkg.grid_array(1, pkg.GRID_FIXED_N, 101, 498)
    tan = engine.tangent_arrays(params, grid)
    assert (tan["status"] == 0).all()
    assert np.abs(tan["value"] - g["value"]).max() <= 1e-9 * np.abs(g["value"]).max()
    for k in ("vega", "rho", "dividend_rho", "dstrike"):
        err = np.min(np.abs(tan[k][None, :] - g[k]), axis=0)
        ref = np.abs(g[k][0])
        assert (err <= 2e-6 * ref + 1e-6).mean() >= 0.99, (k, err.max())
        assert (err <= 1e-3 * ref + 1e-6).all(), (k, err.max())
    fd = engine.greeks_arrays(params, grid, 1e-5)
    for k in ("vega", "rho", "dividend_rho", "dstrike"):
        assert np.allclose(fd[k], g[k][0], rtol=1e-5, atol=1e-6), (k, np.abs(fd[k] - g[k][0]).max())


def test_large_batch_single_launch_matches_split_marches(engine, pkg):
    """A three-direction batch small enough to fit one wave runs as three
    single-direction marches side by side; a large one (40,000 options) as
    one three-direction march.  Both are the same differentiation of the
    same march: the first 512 options agree to rounding (value and delta
    1e-12 relative, the sensitivities 1e-10)."""
    params = inputs(pkg, 40000, 11, True)
    grid = pkg.grid_array(1, pkg.GRID_FIXED_N, 101, 498)
    big = engine.tangent_arrays(params, grid)
    small = engine.tangent_arrays(params[:512], grid)
    assert (big["status"] == 0).all() and (small["status"] == 0).all()
    for k in ("value", "delta"):
        assert np.allclose(big[k][:512], small[k], rtol=1e-12, atol=1e-14), k
    for k in ("vega", "rho", "dividend_rho", "dstrike"):
        assert np.allclose(big[k][:512], small[k], rtol=1e-10, atol=1e-12), (k, np.abs(big[k][:512] - small[k]).max())
