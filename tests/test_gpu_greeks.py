"""Frozen-grid sensitivities (vega, rho, dividend rho, dV/dK) on the GPU
against the same central differences of the CPU oracle on the same grids
(the reference's bump-and-reprice definition), plus structural checks."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_greeks_vs_oracle_central_differences(engine, pkg, oracle):
    rng = np.random.default_rng(99)
    n = 48
    S = np.full(n, 100.0)
    K = rng.uniform(80, 120, n)
    T = rng.uniform(0.1, 2.0, n)
    sig = rng.uniform(0.1, 0.5, n)
    r = rng.uniform(0.005, 0.08, n)
    q = rng.uniform(0.01, 0.04, n)
    put = (np.arange(n) % 2 == 0).astype(np.int32)
    params = pkg.pricing_array(S, K, T, sig, r, q, put)
    grid = pkg.grid_array(1, pkg.GRID_FIXED_N, 101, 498)
    h = 1e-5
    out = engine.greeks_arrays(params, grid, h)
    assert (out["status"] == 0).all()
    for i in range(0, n, 6):
        x, _ = pkg.resolve_grid(params[i:i + 1], pkg.FixedGrid(101, 498))
        base = dict(S=S[i], K=K[i], T=T[i], sigma=sig[i], r=r[i], q=q[i])

        def v(**kw):
            p = dict(base, **kw)
            rc, o4, _, _ = oracle.price_on_grid(p["S"], p["K"], p["T"], p["sigma"], p["r"], p["q"], put[i], x, 498)
            assert rc == 0
            return o4[0]
        hv, hr, hq, hk = h * sig[i], h * max(abs(r[i]), 1e-2), h * max(q[i], 1e-2), h * K[i]
        want = {
            "vega": (v(sigma=sig[i] + hv) - v(sigma=sig[i] - hv)) / (2 * hv),
            "rho": (v(r=r[i] + hr) - v(r=r[i] - hr)) / (2 * hr),
            "dividend_rho": (v(q=q[i] + hq) - v(q=q[i] - hq)) / (2 * hq),
            "dstrike": (v(K=K[i] + hk) - v(K=K[i] - hk)) / (2 * hk),
        }
        for k, w in want.items():
            assert abs(out[k][i] - w) <= 1e-6 * abs(w) + 1e-7, (i, k, out[k][i], w)
    # American puts: positive vega, negative rho, positive dividend rho, dV/dK > 0
    p = put == 1
    assert (out["vega"] > 0).all()
    assert (out["rho"][p] < 0).all() and (out["dividend_rho"][p] > 0).all() and (out["dstrike"][p] > 0).all()
    base = engine.price_arrays(params, grid)
    assert np.array_equal(out["value"], base["value"])
