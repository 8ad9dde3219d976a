"""GPU price-table sweep and 4D B-spline query against the reference.

Table: PriceTableBuilderND<4> sweep + extraction on reduced axes, explicit
201 x 1000 grid (the per-slice fallback route) and the default accuracy route,
and the full 50 x 30 x 20 x 10 sweep of the table-build workload; bar 1e-9
relative on the normalized prices, identical per-slice grids.
Query: BSplineND<double,4>::eval on the 50x30x20x10 axes; bar 1e-12 relative
(plus 1e-14 of the largest coefficient for results near zero), knots exact."""
import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("route", ["explicit", "auto"])
def test_table_sweep_vs_reference(engine, pkg, route):
    g = golden("table.npz")
    grid = pkg.PDEGridConfig(-3.0, 3.0, 201, 1000) if route == "explicit" else None
    tensor, dims, failed = engine.price_table_sweep(g["m"], g["tau"], g["sigma"], g["r"], 100.0, 0.0, 1, grid)
    assert failed == 0
    assert (dims == g[f"{route}_dims"]).all()
    want = g[f"{route}_tensor"]
    bad = np.abs(tensor - want) > 1e-9 * np.abs(want) + 1e-12
    assert not bad.any(), f"max abs diff {np.abs(tensor - want).max():.3e}"


def test_table_sweep_full_axes_vs_reference(engine, pkg):
    """The table-build workload's sweep at full size (50 x 30 x 20 x 10 axes,
    200 slices on the explicit 201 x 1000 grid, the reference's per-slice
    fallback route) against the reference's own tensor (table_full.npz):
    identical per-slice grids, every entry within 1e-9 relative (+1e-12)."""
    g = golden("table_full.npz")
    tensor, dims, failed = engine.price_table_sweep(g["m"], g["tau"], g["sigma"], g["r"], 100.0, 0.0, 1,
                                                    pkg.PDEGridConfig(-3.0, 3.0, 201, 1000))
    assert failed == 0
    assert (dims == g["dims"]).all()
    want = g["tensor"]
    bad = np.abs(tensor - want) > 1e-9 * np.abs(want) + 1e-12
    assert not bad.any(), f"{bad.sum()} entries; max abs diff {np.abs(tensor - want).max():.3e}"


def test_bspline_query_vs_reference(engine, pkg):
    g = golden("bspline.npz")
    sizes = g["sizes"]
    coeffs = np.random.default_rng(int(g["seed"])).standard_normal(int(np.prod(sizes)))
    grids = np.split(g["grids"], np.cumsum(sizes)[:-1])
    surf = engine.bspline4d(grids, coeffs)
    assert np.array_equal(surf.knots(), g["knots"][: int(sizes.sum()) + 16])
    out = surf.eval(g["q"])
    bound = 1e-12 * np.abs(g["out"]) + 1e-14 * np.abs(coeffs).max()
    assert (np.abs(out - g["out"]) <= bound).all(), f"max diff {np.abs(out - g['out']).max():.3e}"


def test_bspline_linear_reproduction(engine, pkg):
    """Coefficients of a function linear in each axis reproduce it exactly
    at the grid corners (bspline_nd_test.cc linear-function case)."""
    axes = [np.linspace(0, 1, 6), np.linspace(-1, 2, 7), np.linspace(0.5, 1.5, 5), np.linspace(0, 3, 8)]
    # For clamped cubic B-splines the Greville abscissae reproduce linear data;
    # at the domain corners the spline equals the corner coefficients.
    C = np.fromfunction(lambda a, b, c, d: 1.0 + 2 * a + 3 * b - c + 0.5 * d, [len(a) for a in axes])
    surf = engine.bspline4d(axes, C)
    corners = np.array([[a[0] if (k >> d) & 1 == 0 else a[-1] for d, a in enumerate(axes)] for k in range(16)])
    want = np.array([C[tuple(0 if (k >> d) & 1 == 0 else len(axes[d]) - 1 for d in range(4))] for k in range(16)])
    assert np.allclose(surf.eval(corners), want, rtol=0, atol=1e-10)

