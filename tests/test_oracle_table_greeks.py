"""The reference's table Greeks (tests/golden/table_greeks.npz, from
PriceTable::delta / gamma / theta / rho) against central differences of the
oracle's restated table price (AnyPriceTable::price: spline value floored at
0, times K/K_ref, plus the closed-form European) on the same coefficients.
Interior records only (no bump across an axis end or across the floor at 0).
Bars: 1e-6 of each Greek's largest magnitude (the differences' truncation
error with the bumps below)."""
import sys

import numpy as np

from conftest import ROOT, golden

sys.path.insert(0, str(ROOT / "oracle"))


def test_reference_table_greeks_match_oracle_differences(oracle):
    g = golden("table_greeks.npz")
    axes = np.split(g["grids"], np.cumsum(g["sizes"])[:-1])
    p = g["params"]
    q, put = 0.02, 1
    ref = g["put_q_greeks"]
    x = np.stack([np.log(p[:, 0] / p[:, 1]), p[:, 2], p[:, 3], p[:, 4]], 1)
    raw = oracle.bspline4d_eval(axes, g["coeffs"], x)
    hs, ht, hr = 1e-3, 1e-5, 1e-5
    lo = np.array([a[0] for a in axes])
    hi = np.array([a[-1] for a in axes])
    margin = np.array([2 * hs / 80.0, 2 * ht, 0.0, 2 * hr])
    inside = ((x[:, [0, 1, 3]] > (lo + margin)[[0, 1, 3]]) & (x[:, [0, 1, 3]] < (hi - margin)[[0, 1, 3]])).all(1)
    sel = np.flatnonzero(inside & (np.abs(raw) > 1e-3))
    assert sel.size > 300
    P = p[sel]

    def price(dS=0.0, dt=0.0, dr=0.0):
        m = P.copy()
        m[:, 0] += dS
        m[:, 2] += dt
        m[:, 4] += dr
        return oracle.surface_price(axes, g["coeffs"], m, 100.0, q, put)

    v0 = price()
    fd = np.stack([(price(dS=hs) - price(dS=-hs)) / (2 * hs),
                   (price(dS=hs) - 2 * v0 + price(dS=-hs)) / (hs * hs),
                   -(price(dt=ht) - price(dt=-ht)) / (2 * ht),
                   (price(dr=hr) - price(dr=-hr)) / (2 * hr)], 1)
    for j in range(4):
        scale = np.abs(ref[sel, j]).max()
        assert np.abs(fd[:, j] - ref[sel, j]).max() <= 1e-6 * scale + 1e-9, (j, np.abs(fd[:, j] - ref[sel, j]).max())
