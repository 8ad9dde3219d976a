"""torch.autograd over the forward-mode march
(american_option_price_autograd -> mango_gpu_price_american_tangent_batch).

The backward pass multiplies the incoming gradient by the exact discrete
derivatives of the march.  Checked gradcheck-style: the gradient of a
weighted sum of prices against central differences of that sum taken
through the function itself on volatility-independent grids (each option's
101 x 498 grid sized at its base volatility, so the bumps do not move the
grid), with the closest of h = 1e-5, 1e-6, 1e-7 relative (a difference that
straddles a change of the obstacle's active set is not the derivative at the
point); and the strike gradient against the engine's frozen-grid difference
in the strike."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def inputs(n, seed):
    rng = np.random.default_rng(seed)
    return (np.full(n, 100.0), rng.uniform(80, 120, n), rng.uniform(0.1, 2.0, n), rng.uniform(0.1, 0.5, n),
            rng.uniform(0.0, 0.08, n), rng.uniform(0.0, 0.04, n), (np.arange(n) % 2 == 0).astype(np.int32))


def test_values_and_gradients_match_the_tangent_batch(engine, pkg):
    S, K, T, sig, r, q, put = inputs(64, 5)
    grid = pkg.grid_array(64, pkg.GRID_FIXED_N_AT_VOL, 101, 498, alpha=sig)
    ts = {k: torch.tensor(v, dtype=torch.float64, device="cuda", requires_grad=True)
          for k, v in (("sig", sig), ("r", r), ("q", q), ("K", K))}
    V = pkg.american_option_price_autograd(S, ts["K"], T, ts["sig"], ts["r"], ts["q"], put, grid=grid,
                                           engine=engine)
    assert V.device.type == "cuda" and V.dtype == torch.float64
    w = torch.linspace(0.5, 1.5, 64, dtype=torch.float64, device="cuda")
    (w * V).sum().backward()
    tan = engine.tangent_arrays(pkg.pricing_array(S, K, T, sig, r, q, put), grid)
    assert np.array_equal(V.detach().cpu().numpy(), tan["value"])
    wn = w.cpu().numpy()
    for k, f in (("sig", "vega"), ("r", "rho"), ("q", "dividend_rho"), ("K", "dstrike")):
        assert np.allclose(ts[k].grad.cpu().numpy(), wn * tan[f], rtol=1e-14, atol=0), k


def test_gradients_against_central_differences(engine, pkg):
    n = 256
    S, K, T, sig, r, q, put = inputs(n, 11)
    grid = pkg.grid_array(n, pkg.GRID_FIXED_N_AT_VOL, 101, 498, alpha=sig)
    w = np.random.default_rng(3).uniform(0.5, 1.5, n)
    x = {k: torch.tensor(v, dtype=torch.float64, requires_grad=True) for k, v in (("sig", sig), ("r", r),
                                                                                  ("q", q))}
    V = pkg.american_option_price_autograd(S, K, T, x["sig"], x["r"], x["q"], put, grid=grid, engine=engine)
    (torch.from_numpy(w) * V).sum().backward()

    def loss(s_, r_, q_):
        with torch.no_grad():
            v = pkg.american_option_price_autograd(S, K, T, s_, r_, q_, put, grid=grid, engine=engine)
        return w * v.numpy()

    for name, base, scale in (("sig", sig, sig), ("r", r, np.maximum(np.abs(r), 1e-2)),
                              ("q", q, np.maximum(q, 1e-2))):
        g = x[name].grad.numpy() / w
        errs = []
        for h in (1e-5, 1e-6, 1e-7):
            hh = scale * h
            up, dn = base + hh, np.maximum(base - hh, 0.0)
            args = {"sig": sig, "r": r, "q": q}
            a_up, a_dn = dict(args), dict(args)
            a_up[name], a_dn[name] = up, dn
            fd = (loss(a_up["sig"], a_up["r"], a_up["q"]) - loss(a_dn["sig"], a_dn["r"], a_dn["q"])) / (up - dn) / w
            errs.append(np.abs(g - fd))
        err = np.min(errs, axis=0)
        assert (err <= 2e-6 * np.abs(g) + 1e-6).mean() >= 0.99, (name, err.max())
        assert (err <= 1e-3 * np.abs(g) + 1e-6).all(), (name, err.max())
    # strike: against the engine's frozen-grid central difference
    k = torch.tensor(K, dtype=torch.float64, requires_grad=True)
    V = pkg.american_option_price_autograd(S, k, T, sig, r, q, put, grid=grid, engine=engine)
    V.sum().backward()
    fds = [engine.greeks_arrays(pkg.pricing_array(S, K, T, sig, r, q, put), grid, h)["dstrike"]
           for h in (1e-5, 1e-6, 1e-7)]
    err = np.min([np.abs(k.grad.numpy() - f) for f in fds], axis=0)
    assert (err <= 2e-6 * np.abs(fds[0]) + 1e-6).mean() >= 0.99, err.max()
