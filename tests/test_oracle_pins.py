"""Pin the CPU oracle (oracle/mango_oracle.c) to the reference's own outputs.

The golden .npz files were produced by the unmodified reference sources
(tests/golden/make_golden.py).  The reference compiles its stencil loops with
target_clones (avx2/avx512f), so its last-bit rounding depends on the CPU it
ran on; the oracle (plain IEEE, explicit fma only where the reference writes
std::fma) therefore agrees to ~1e-12 relative, not bit for bit.  Grids, which
involve no such loops, must match exactly.
"""
import numpy as np
import pytest

from conftest import golden, rel_err

RTOL = 1e-10   # oracle vs reference, prices and Greeks
ATOL = 1e-12   # dollars / per-unit Greeks near zero


def check(got, want, rtol=RTOL, atol=ATOL):
    got = np.asarray(got)
    want = np.asarray(want)
    bad = np.abs(got - want) > rtol * np.abs(want) + atol
    assert not bad.any(), f"max rel {rel_err(got, want).max():.3e} at {np.argwhere(bad)[:5].ravel()}"


@pytest.mark.parametrize("name", ["pricing_cfg0.npz", "pricing_mixed.npz", "pricing_uneven.npz"])
def test_oracle_fixed_grids(oracle, name):
    g = golden(name)
    out, dims, st = oracle.price_batch(g["S"], g["K"], g["T"], g["sigma"], g["r"], g["q"], g["is_put"],
                                       g["nx"], g["nt"])
    assert (st == 0).all() and (g["status"] == 0).all()
    assert (dims == g["dims"]).all()
    check(out, g["out"])


def test_oracle_auto_grid(oracle):
    g = golden("pricing_auto.npz")
    out, dims, st = oracle.price_batch(g["S"], g["K"], g["T"], g["sigma"], g["r"], g["q"], g["is_put"], 0, 0)
    assert (st == 0).all()
    assert (dims == g["dims"]).all(), "auto grid sizes (Nx, Nt) must equal the reference's"
    check(out, g["out"])


def test_oracle_edge_cases(oracle):
    g = golden("pricing_edge.npz")
    for rann in (0, 1):
        sel = g["rannacher"] == rann
        out, dims, st = oracle.price_batch(*(g[k][sel] for k in ("S", "K", "T", "sigma", "r", "q", "is_put", "nx", "nt")),
                                           rannacher=rann)
        assert (st == g["status"][sel]).all()
        check(out, g["out"][sel])


def test_oracle_explicit_grids(oracle):
    g = golden("pricing_explicit.npz")
    for i in range(len(g["S"])):
        x = oracle.explicit_grid(int(g["kind"][i]), g["x_min"][i], g["x_max"][i], g["nx"][i], g["alpha"][i])
        rc, out, _, _ = oracle.price_on_grid(g["S"][i], g["K"][i], g["T"][i], g["sigma"][i], g["r"][i], g["q"][i],
                                             g["is_put"][i], x, g["nt"][i])
        assert rc == 0
        check(out, g["out"][i])


def test_oracle_grids_bitwise(oracle):
    g = golden("grids.npz")
    for i, (S, K, T, s, nx) in enumerate(g["params"]):
        x, nt = oracle.grid(S, K, T, s, int(nx))
        assert x.size == g["n"][i]
        assert nt == g["nt"][i]
        assert np.array_equal(x, g["x"][i, : x.size])


def test_oracle_solution_vectors(oracle):
    g = golden("solutions.npz")
    for i, (S, K, T, s, r, q, put, nx, nt) in enumerate(g["params"]):
        n = int(g["n"][i])
        x, _ = oracle.grid(S, K, T, s, int(nx))
        assert np.array_equal(x, g["x"][i, :n])
        rc, _, u, up = oracle.price_on_grid(S, K, T, s, r, q, int(put), x, int(nt))
        assert rc == 0
        assert np.abs(u - g["u"][i, :n]).max() < 1e-13
        assert np.abs(up - g["u_prev"][i, :n]).max() < 1e-13


def test_oracle_iv_brent(oracle):
    g = golden("iv.npz")
    out, st = oracle.iv_batch(g["S"], g["K"], g["T"], g["r"], g["q"], g["is_put"], g["price"], g["true_vol"],
                              g["nx"], g["nt"])
    assert (st == g["status"]).all()
    # Brent replays the same iterate sequence; prices agree to ~1e-12 so the
    # roots agree far inside the 1e-8 vol bar.
    assert np.abs(out[:, 0] - g["out"][:, 0]).max() < 1e-9
    assert (out[:, 1] == g["out"][:, 1]).all(), "Brent iteration counts must match"


def test_oracle_thomas_projected_known_answers(oracle):
    """Known answers in the spirit of the reference's tridiagonal tests
    (tests/tridiagonal_solver_test.cc): no constraint active reproduces the
    plain solve; an obstacle above the solution is returned exactly."""
    import ctypes
    lib = oracle.lib()
    P = oracle.P
    n = 5
    lower = np.full(n - 1, -1.0)
    diag = np.full(n, 4.0)
    upper = np.full(n - 1, -1.0)
    x_true = np.array([1.0, 2.0, 3.0, 2.0, 1.0])
    A = np.diag(diag) + np.diag(lower, -1) + np.diag(upper, 1)
    rhs = A @ x_true
    ws = np.zeros(2 * n)
    x = np.zeros(n)
    psi = np.full(n, -10.0)
    assert lib.mo_thomas_projected(P(lower), P(diag), P(upper), P(rhs), P(psi), P(x), ctypes.c_int64(n), P(ws)) == 0
    assert np.allclose(x, x_true, rtol=0, atol=1e-14)
    psi = np.full(n, 5.0)
    assert lib.mo_thomas_projected(P(lower), P(diag), P(upper), P(rhs), P(psi), P(x), ctypes.c_int64(n), P(ws)) == 0
    assert np.array_equal(x, psi)
    diag0 = diag.copy()
    diag0[0] = 0.0
    assert lib.mo_thomas_projected(P(lower), P(diag0), P(upper), P(rhs), P(psi), P(x), ctypes.c_int64(n), P(ws)) == 1


def test_oracle_bspline_vs_reference(oracle):
    import ctypes
    g = golden("bspline.npz")
    sizes = g["sizes"]
    coeffs = np.random.default_rng(int(g["seed"])).standard_normal(int(np.prod(sizes)))
    knots = np.zeros(int(sizes.sum()) + 16)
    off = 0
    goff = 0
    for d in range(4):
        n = int(sizes[d])
        t = np.zeros(n + 4)
        oracle.lib().mo_clamped_knots(oracle.P(np.ascontiguousarray(g["grids"][goff:goff + n])), ctypes.c_int64(n),
                                      oracle.P(t))
        knots[off:off + n + 4] = t
        off += n + 4
        goff += n
    assert np.array_equal(knots, g["knots"]), "clamped knots must match the reference exactly"
    q = np.ascontiguousarray(g["q"])
    out = np.zeros(q.shape[0])
    assert oracle.lib().mo_bspline4d_eval(oracle.P(sizes), oracle.P(g["grids"]), oracle.P(coeffs), oracle.P(q),
                                          ctypes.c_int64(q.shape[0]), oracle.P(out)) == 0
    bound = 1e-12 * np.abs(g["out"]) + 1e-14 * np.abs(coeffs).max()
    assert (np.abs(out - g["out"]) <= bound).all()


def test_oracle_iv_config4_sample(oracle):
    """256 quotes of iv_config4.npz: the oracle's Brent finds the reference's
    roots with the same iteration counts, and fails where it fails."""
    g = golden("iv_config4.npz")
    sel = np.arange(0, 4096, 16)
    out, st = oracle.iv_batch(*(g[k][sel] for k in ("S", "K", "T", "r", "q", "is_put", "price", "true_vol",
                                                     "nx", "nt")))
    ok = g["status"][sel] == 0
    assert ((st == 0) == ok).all()
    assert np.abs(out[ok, 0] - g["out"][sel][ok, 0]).max() < 1e-9
    assert (out[ok, 1] == g["out"][sel][ok, 1]).all()


def test_oracle_frozen_grid_prices(oracle):
    """The reference's prices of greeks_fd.npz on each option's frozen grid,
    for 16 options: the oracle on the same grid agrees to 1e-10, and so do
    the h = 1e-5 volatility differences to the oracle's own (to 1e-5, the
    difference amplifying price rounding by 1 / 2h)."""
    import ctypes

    from oracle_lib import Accuracy, P, Spec, lib

    g = golden("greeks_fd.npz")
    for i in range(0, 1024, 64):
        S, K, T, s, r, q = (float(g[k][i]) for k in ("S", "K", "T", "sigma", "r", "q"))
        acc = Accuracy()
        lib().mo_default_accuracy(ctypes.byref(acc))
        acc.min_spatial_points = acc.max_spatial_points = 101
        spec = Spec()
        nt = ctypes.c_int64()
        c = ctypes.c_double
        lib().mo_estimate_grid(c(S), c(K), c(T), c(s), ctypes.byref(acc), ctypes.byref(spec), ctypes.byref(nt))
        x = np.zeros(spec.n_points)
        lib().mo_generate_grid(ctypes.byref(spec), P(x))
        rc, out, _, _ = oracle.price_on_grid(S, K, T, s, r, q, 1, x, 498)
        assert rc == 0 and abs(out[0] - g["value"][i]) <= 1e-10 * abs(g["value"][i]) + 1e-12
        hs = s * 1e-5
        up = oracle.price_on_grid(S, K, T, s + hs, r, q, 1, x, 498)[1][0]
        dn = oracle.price_on_grid(S, K, T, s - hs, r, q, 1, x, 498)[1][0]
        vega = (up - dn) / (2 * hs)
        assert abs(vega - g["vega"][0, i]) <= 1e-5 * abs(vega) + 1e-6, (i, vega, g["vega"][0, i])
