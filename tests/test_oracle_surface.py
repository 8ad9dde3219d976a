"""Pin the CPU restatement of the price-table surface (oracle/fit_oracle.py
plus the C B-spline evaluation) to the reference's own outputs: the
standard table's price (EEPLayer over TransformLeaf, make_bspline_surface)
and eep_decompose with AnalyticalEEP, from tests/golden/surface.npz.  The fit
itself needs LAPACKE in the reference (absent here); it is checked by
polynomial reproduction, the reference's own test strategy
(tests/bspline_collocation_1d_test.cc, tests/bspline_fitter_4d_separable_test.cc)."""
import sys

import numpy as np

from conftest import ROOT, golden

sys.path.insert(0, str(ROOT / "oracle"))
import fit_oracle  # noqa: E402


def axes_of(g):
    sizes = g["sizes"]
    cuts = np.cumsum(sizes)[:-1]
    return np.split(g["grids"], cuts)


def test_surface_price_restatement_vs_reference(oracle):
    g = golden("surface.npz")
    axes = axes_of(g)
    for name, put in (("put", 1), ("call", 0)):
        v = oracle.surface_price(axes, g["coeffs"], g["params"], 100.0, float(g[f"{name}_q"]), put)
        ref = g[f"{name}_price"]
        assert np.abs(v - ref).max() <= 1e-12 * np.abs(ref).max() + 1e-13


def test_eep_restatement_vs_reference():
    g = golden("surface.npz")
    axes = axes_of(g)
    out = fit_oracle.eep_decompose(axes, g["eep_in"], 100.0, 0.015, True).ravel()
    assert np.abs(out - g["eep_out"]).max() < 1e-12


def test_knots_restatement_vs_reference():
    g = golden("bspline.npz")
    cuts = np.cumsum(g["sizes"])[:-1]
    knots = np.concatenate([fit_oracle.clamped_knots(a) for a in np.split(g["grids"], cuts)])
    assert np.array_equal(knots, g["knots"])


def test_fit_restatement_reproduces_cubics(oracle):
    axes = [np.linspace(-0.4, 0.3, 9) ** 1 + 0.01 * np.arange(9) ** 2, np.linspace(0.02, 2.0, 7),
            np.linspace(0.05, 0.8, 6), np.linspace(0.0, 0.08, 5)]
    f = lambda a, b, c, d: 1 + a - 2 * a ** 3 + 0.5 * b ** 2 * c - c ** 3 + 3 * d * a ** 2 + b ** 3 * d
    mesh = np.meshgrid(*axes, indexing="ij")
    coeffs = fit_oracle.fit4d(axes, f(*mesh))
    rng = np.random.default_rng(5)
    q = np.stack([rng.uniform(a[0], a[-1], 500) for a in axes], 1)
    got = oracle.bspline4d_eval(axes, coeffs, q)
    assert np.abs(got - f(*q.T)).max() < 1e-11
