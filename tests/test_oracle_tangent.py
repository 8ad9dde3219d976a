"""The oracle's forward-mode march (mo_price_tangent_on_grid) on the CPU:
its value and delta equal mo_price_on_grid's (the primal is the same
restatement), and each sensitivity equals the closest of the oracle's own
central differences at 1e-5, 1e-6 and 1e-7 relative on the same grid (the
differences converge onto the exact discrete derivative as the bump shrinks,
unless a bump straddles a flip of the obstacle's active set).
Bars: value/delta 1e-14 relative; sensitivities 2e-6 relative + 1e-6."""
import numpy as np


def test_oracle_tangent_matches_its_central_differences(oracle):
    rng = np.random.default_rng(5)
    for k in range(6):
        S, K = 100.0, float(rng.uniform(80, 120))
        T, sig = float(rng.uniform(0.1, 2.0)), float(rng.uniform(0.1, 0.5))
        r, q = float(rng.uniform(0.005, 0.08)), float(rng.uniform(0.005, 0.04))
        put = k % 2 == 0
        x, _ = oracle.grid(S, K, T, sig, nx=101)
        nt = 498
        rc, t6 = oracle.price_tangent_on_grid(S, K, T, sig, r, q, put, x, nt)
        assert rc == 0
        rc, o4, _, _ = oracle.price_on_grid(S, K, T, sig, r, q, put, x, nt)
        assert rc == 0
        assert abs(t6[0] - o4[0]) <= 1e-14 * abs(o4[0]) and abs(t6[1] - o4[1]) <= 1e-14 * abs(o4[1]) + 1e-16

        def v(**kw):
            p = dict(S=S, K=K, T=T, sigma=sig, r=r, q=q)
            p.update(kw)
            rc, o, _, _ = oracle.price_on_grid(p["S"], p["K"], p["T"], p["sigma"], p["r"], p["q"], put, x, nt)
            assert rc == 0
            return o[0]

        for col, name, base in ((2, "sigma", sig), (3, "r", r), (4, "q", q), (5, "K", K)):
            errs = []
            for h in (1e-5, 1e-6, 1e-7):
                d = h * base
                fd = (v(**{name: base + d}) - v(**{name: base - d})) / (2 * d)
                errs.append(abs(t6[col] - fd))
            assert min(errs) <= 2e-6 * abs(t6[col]) + 1e-6, (k, name, t6[col], errs)
