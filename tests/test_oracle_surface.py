"""Pin the CPU restatement of the price-table surface (oracle/fit_oracle.py
plus the C B-spline evaluation) to the reference's own outputs: the
standard table's price (EEPLayer over TransformLeaf, make_bspline_surface)
and eep_decompose with AnalyticalEEP, from tests/golden/surface.npz; and the
separable collocation fit, against the reference's own
BSplineNDSeparable<double,4>::fit (tests/golden/fit.npz, its LAPACKE calls
served by the LAPACK scipy bundles), besides polynomial reproduction, the
reference's own test strategy (tests/bspline_collocation_1d_test.cc,
tests/bspline_fitter_4d_separable_test.cc)."""
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


def fit_axes(g, name):
    return np.split(g[f"{name}_grids"], np.cumsum(g[f"{name}_sizes"])[:-1])


def fit_table_values(g):
    """The full-axes case's values, regenerated from the stored seed as the
    golden generator made them."""
    return np.random.default_rng(int(g["table_seed"])).standard_normal(int(np.prod(g["table_sizes"])))


def test_fit_restatement_vs_reference_fit():
    """The dense restatement against the reference's banded-LU fit: 1e-13 of
    the largest coefficient on the surface axes (every coefficient) and on
    the full 50 x 30 x 20 x 10 table axes (4096 sampled coefficients and the
    sum of all); the reference's dgbcon estimates equal the exact 1-norm
    condition numbers."""
    g = golden("fit.npz")
    axes = fit_axes(g, "rand")
    c = fit_oracle.fit4d(axes, g["rand_values"].reshape([a.size for a in axes])).ravel()
    ref = g["rand_coeffs"]
    assert np.abs(c - ref).max() <= 1e-13 * np.abs(ref).max()
    axes = fit_axes(g, "table")
    c = fit_oracle.fit4d(axes, fit_table_values(g).reshape([a.size for a in axes])).ravel()
    amax = float(g["table_coeff_absmax"])
    assert np.abs(c[g["table_idx"]] - g["table_coeffs"]).max() <= 1e-13 * amax
    assert abs(c.sum() - float(g["table_coeff_sum"])) <= 1e-13 * amax * c.size
    for name in ("rand", "table"):
        conds = [np.linalg.cond(fit_oracle.collocation_matrix(a), 1) for a in fit_axes(g, name)]
        assert np.allclose(g[f"{name}_cond"], conds, rtol=1e-9), name
