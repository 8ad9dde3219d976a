"""Generate the golden fixtures in this directory from the reference itself.

Runs the UNMODIFIED reference sources, compiled by oracle/ref/Makefile into
oracle/_ref/libmango_ref.so (needs the reference tree, so this script runs on
the development host only; the .npz outputs are committed and travel).

    python tests/golden/make_golden.py

Workloads (seeded numpy generators; the reference's CPU path is the source of
every output value):
  pricing_cfg0.npz   64 American puts, spot 100, K~U[80,120], T~U[0.1,2],
                     sigma~U[0.1,0.5], r~U[0,0.08], q~U[0,0.04]; grid rule
                     101 x 498 (estimate_pde_grid with min=max=101 points)
  pricing_mixed.npz  64 options, same distributions, puts/calls alternating
  pricing_auto.npz   32 options on the reference auto grid (GridAccuracyParams{})
  pricing_uneven.npz 256 options, Nx~U{51..401}, Nt~U{100..1000}, puts/calls
  pricing_edge.npz   hand-picked edge cases (deep ITM/OTM, r=0, q>r calls,
                     tiny grids, 1-3 steps, Rannacher off, extreme vol/maturity)
  pricing_explicit.npz explicit sinh / uniform PDEGridConfig grids
  grids.npz          reference grids (bit-exact host grid generation)
  solutions.npz      full final and previous solution vectors for 4 options
  iv.npz             16 FDM implied vols (Brent) on per-quote 101 x 498 grids
  bspline.npz        BSplineND<double,4>::eval on the 50x30x20x10 table axes with
                     seeded standard-normal coefficients (regenerated from the
                     stored seed), 4096 random + edge queries, and the knots
  table.npz          PriceTableBuilderND<4> sweep + extraction on reduced axes
                     (12 x 6 x 5 x 3) for the explicit 201 x 1000 grid (the
                     reference's per-slice fallback route) and the default
                     accuracy route, with each slice's (N_x, N_t)
  surface.npz        the standard price table (make_bspline_surface: EEPLayer
                     over TransformLeaf) on 12 x 8 x 6 x 5 axes with seeded
                     coefficients: 2048 price queries (some outside the axes)
                     for a put and a call table; and eep_decompose
                     (AnalyticalEEP) of a seeded V/K_ref tensor on the same axes
  fit.npz            BSplineNDSeparable<double,4>::fit (the reference's own
                     collocation fit, its LAPACKE dgbtrf/dgbtrs/dgbcon calls
                     forwarded to the LAPACK that scipy bundles, see
                     oracle/ref/lapacke_stubs.c): on the full 50 x 30 x 20 x 10
                     table axes, values from a stored seed (regenerated by the
                     test) and 4096 of the 300,000 coefficients at stored
                     indices; on the 12 x 8 x 6 x 5 surface axes, seeded values
                     and every coefficient; per-axis residuals and condition
                     estimates
  interp_iv.npz      a real EEP table: the reference's own sweep tensor on
                     12 x 6 x 5 x 4 axes (auto grid), its eep_decompose, fitted by the
                     reference's own fit (BSplineNDSeparable, see fit.npz); on it the
                     reference's vega at 1024 points
                     and InterpolatedIVSolver::solve_batch for 1024 quotes
                     (prices from the table at seeded vols, plus invalid,
                     out-of-range and mismatched quotes)
"""
from __future__ import annotations

import ctypes
import os
import json
import pathlib
import subprocess
import sys

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
ROOT = HERE.parent.parent
REF_SO = ROOT / "oracle" / "_ref" / "libmango_ref.so"


def _lib():
    import importlib.util
    spec = importlib.util.spec_from_file_location("_b", ROOT / "mango-option_gb300" / "build.py")
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    ref = b.reference_dir()
    if ref is None:
        sys.exit("the reference tree is needed (MANGO_REFERENCE_DIR or a checkout beside the repository)")
    subprocess.run(["make", "-s", "-C", str(ROOT / "oracle" / "ref"), f"REF={ref}", "-j8"], check=True)
    return ctypes.CDLL(str(REF_SO))


def P(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def price(lib, S, K, T, sig, r, q, put, nx, nt, rannacher=1):
    n = len(S)
    args = [np.ascontiguousarray(a, dtype=np.float64) for a in (S, K, T, sig, r, q)]
    put = np.ascontiguousarray(put, dtype=np.int32)
    nx = np.ascontiguousarray(nx, dtype=np.int64)
    nt = np.ascontiguousarray(nt, dtype=np.int64)
    out = np.full(4 * n, np.nan)
    dims = np.zeros(2 * n, np.int64)
    st = np.zeros(n, np.int32)
    lib.ref_price_batch(ctypes.c_int64(n), *(P(a) for a in args), P(put), P(nx), P(nt),
                        ctypes.c_int32(rannacher), ctypes.c_int32(8), P(out), P(dims), P(st))
    return out.reshape(n, 4), dims.reshape(n, 2), st


def config0_inputs(n, seed, mixed):
    rng = np.random.default_rng(seed)
    S = np.full(n, 100.0)
    K = rng.uniform(80, 120, n)
    T = rng.uniform(0.1, 2.0, n)
    sig = rng.uniform(0.1, 0.5, n)
    r = rng.uniform(0.0, 0.08, n)
    q = rng.uniform(0.0, 0.04, n)
    put = (np.arange(n) % 2 == 0).astype(np.int32) if mixed else np.ones(n, np.int32)
    return S, K, T, sig, r, q, put


def save(name, **kw):
    np.savez_compressed(HERE / name, **kw)
    print("wrote", name, {k: v.shape for k, v in kw.items()})


def main():
    lib = _lib()

    for name, mixed in (("pricing_cfg0.npz", False), ("pricing_mixed.npz", True)):
        S, K, T, sig, r, q, put = config0_inputs(64, 42, mixed)
        nx = np.full(64, 101)
        nt = np.full(64, 498)
        out, dims, st = price(lib, S, K, T, sig, r, q, put, nx, nt)
        save(name, S=S, K=K, T=T, sigma=sig, r=r, q=q, is_put=put, nx=nx, nt=nt, out=out,
             dims=dims, status=st)

    S, K, T, sig, r, q, put = config0_inputs(32, 11, True)
    out, dims, st = price(lib, S, K, T, sig, r, q, put, np.zeros(32), np.zeros(32))
    save("pricing_auto.npz", S=S, K=K, T=T, sigma=sig, r=r, q=q, is_put=put, out=out,
         dims=dims, status=st)

    rng = np.random.default_rng(1234)
    n = 256
    S, K, T, sig, r, q, put = config0_inputs(n, 99, True)
    nx = rng.integers(51, 402, n)
    nt = rng.integers(100, 1001, n)
    out, dims, st = price(lib, S, K, T, sig, r, q, put, nx, nt)
    save("pricing_uneven.npz", S=S, K=K, T=T, sigma=sig, r=r, q=q, is_put=put, nx=nx, nt=nt,
         out=out, dims=dims, status=st)

    # Edge cases: (S, K, T, sigma, r, q, put, nx, nt, rannacher)
    edge = [
        (25.0, 100.0, 1.0, 0.2, 0.05, 0.0, 1, 101, 498, 1),   # deep ITM put (locks)
        (0.25, 100.0, 1.0, 0.2, 0.05, 0.0, 1, 101, 200, 1),   # extremely deep ITM put
        (400.0, 100.0, 1.0, 0.2, 0.05, 0.0, 1, 101, 200, 1),  # deep OTM put
        (100.0, 100.0, 1.0, 0.3, 0.0, 0.0, 1, 101, 300, 1),   # r = 0 put (never locks)
        (100.0, 100.0, 1.0, 0.3, 0.02, 0.08, 0, 101, 300, 1),  # call, q > r: early exercise
        (250.0, 100.0, 1.0, 0.3, 0.02, 0.08, 0, 101, 300, 1),  # deep ITM call, q > r
        (100.0, 100.0, 1.0, 0.3, 0.05, 0.0, 0, 101, 300, 1),  # call, q = 0 (European)
        (100.0, 100.0, 0.02, 0.3, 0.05, 0.02, 1, 101, 50, 1),  # very short maturity
        (100.0, 100.0, 2.0, 0.8, 0.08, 0.04, 1, 101, 500, 1),  # high vol, long
        (100.0, 100.0, 2.0, 0.05, 0.08, 0.0, 1, 101, 500, 1),  # low vol
        (100.0, 95.0, 1.0, 0.25, 0.05, 0.01, 1, 5, 3, 1),     # tiny grid
        (100.0, 95.0, 1.0, 0.25, 0.05, 0.01, 1, 7, 2, 1),
        (100.0, 95.0, 1.0, 0.25, 0.05, 0.01, 0, 9, 1, 1),     # one step (Rannacher only)
        (100.0, 95.0, 1.0, 0.25, 0.05, 0.01, 1, 9, 1, 0),     # one TR-BDF2 step
        (100.0, 105.0, 1.0, 0.25, 0.05, 0.01, 1, 101, 100, 0),  # Rannacher off
        (100.0, 105.0, 1.0, 0.25, 0.05, 0.01, 0, 101, 100, 0),
        (100.0, 100.0, 1.0, 0.2, -0.01, 0.0, 1, 101, 200, 1),  # negative rate
        (100.0, 80.0, 0.5, 0.4, 0.08, 0.04, 1, 401, 1000, 1),  # large grid
    ]
    cols = list(zip(*edge))
    out = np.full((len(edge), 4), np.nan)
    st = np.zeros(len(edge), np.int32)
    dims = np.zeros((len(edge), 2), np.int64)
    for rann in (0, 1):
        sel = [i for i, e in enumerate(edge) if e[9] == rann]
        o, d, s = price(lib, *(np.array(c)[sel] for c in cols[:9]), rannacher=rann)
        out[sel], dims[sel], st[sel] = o, d, s
    save("pricing_edge.npz", S=np.array(cols[0]), K=np.array(cols[1]), T=np.array(cols[2]),
         sigma=np.array(cols[3]), r=np.array(cols[4]), q=np.array(cols[5]),
         is_put=np.array(cols[6], np.int32), nx=np.array(cols[7]), nt=np.array(cols[8]),
         rannacher=np.array(cols[9], np.int32), out=out, dims=dims, status=st)

    # Explicit grids: sinh_spaced and uniform PDEGridConfig.
    alpha = 2.0 * np.arcsinh(5.0 / np.sqrt(2.0))
    ex = [
        (100.0, 100.0, 2.0, 0.3, 0.05, 0.0, 1, 2, -3.0, 3.0, 201, alpha, 1000),
        (100.0, 90.0, 1.0, 0.2, 0.03, 0.01, 1, 2, -1.5, 1.5, 101, 3.0, 300),
        (100.0, 110.0, 1.0, 0.2, 0.03, 0.05, 0, 2, -1.5, 1.5, 101, 1.0, 300),
        (100.0, 100.0, 1.0, 0.25, 0.04, 0.0, 1, 3, -2.0, 2.0, 161, 0.0, 400),
        (100.0, 100.0, 1.0, 0.25, 0.04, 0.06, 0, 3, -2.0, 2.0, 161, 0.0, 400),
    ]
    c = [np.array(v) for v in zip(*ex)]
    n = len(ex)
    o = np.full(4 * n, np.nan)
    s = np.zeros(n, np.int32)
    f = [np.ascontiguousarray(a, dtype=np.float64) for a in c[:6]]
    lib.ref_price_explicit(ctypes.c_int64(n), *(P(a) for a in f),
                           P(np.ascontiguousarray(c[6], np.int32)),
                           P(np.ascontiguousarray(c[7], np.int32)),
                           P(np.ascontiguousarray(c[8], np.float64)),
                           P(np.ascontiguousarray(c[9], np.float64)),
                           P(np.ascontiguousarray(c[10], np.int64)),
                           P(np.ascontiguousarray(c[11], np.float64)),
                           P(np.ascontiguousarray(c[12], np.int64)), ctypes.c_int32(1), P(o), P(s))
    save("pricing_explicit.npz", S=c[0], K=c[1], T=c[2], sigma=c[3], r=c[4], q=c[5],
         is_put=c[6].astype(np.int32), kind=c[7].astype(np.int32), x_min=c[8], x_max=c[9],
         nx=c[10], alpha=c[11], nt=c[12], out=o.reshape(n, 4), status=s)

    # Grids (bitwise): mix of auto and pinned sizes.
    gs = [(100, 100, 1, 0.2, 0), (100, 93, 1.3, 0.3, 101), (100, 120, 0.1, 0.1, 0),
          (100, 80, 2.0, 0.5, 401), (100, 100, 0.5, 0.8, 51), (100, 300, 1.0, 0.2, 101)]
    xs = np.full((len(gs), 2048), np.nan)
    ns = np.zeros(len(gs), np.int64)
    nts = np.zeros(len(gs), np.int64)
    for i, (S_, K_, T_, s_, nx_) in enumerate(gs):
        x = np.zeros(2048)
        nn = np.zeros(1, np.int64)
        ntt = np.zeros(1, np.int64)
        lib.ref_make_grid(ctypes.c_double(S_), ctypes.c_double(K_), ctypes.c_double(T_),
                          ctypes.c_double(s_), ctypes.c_int64(nx_), ctypes.c_int64(2048), P(x),
                          P(nn), P(ntt))
        xs[i] = x
        ns[i], nts[i] = nn[0], ntt[0]
    save("grids.npz", params=np.array(gs, np.float64), x=xs, n=ns, nt=nts)

    # Solutions for element-wise checks.
    sol = [(100, 93, 1.3, 0.3, 0.05, 0.02, 1, 101, 498), (100, 110, 1.0, 0.2, 0.03, 0.06, 0, 101, 300),
           (25, 100, 1.0, 0.2, 0.05, 0.0, 1, 101, 498), (100, 100, 0.5, 0.4, 0.02, 0.01, 1, 201, 250)]
    U = np.full((4, 512), np.nan)
    UP = np.full((4, 512), np.nan)
    X = np.full((4, 512), np.nan)
    NS = np.zeros(4, np.int64)
    for i, (S_, K_, T_, s_, r_, q_, p_, nx_, nt_) in enumerate(sol):
        x = np.zeros(512)
        u = np.zeros(512)
        up = np.zeros(512)
        nn = np.zeros(1, np.int64)
        rc = lib.ref_price_solution(*(ctypes.c_double(v) for v in (S_, K_, T_, s_, r_, q_)),
                                    ctypes.c_int32(p_), ctypes.c_int64(nx_), ctypes.c_int64(nt_),
                                    ctypes.c_int64(512), P(x), P(u), P(up), P(nn))
        assert rc == 0
        X[i], U[i], UP[i], NS[i] = x, u, up, nn[0]
    save("solutions.npz", params=np.array(sol, np.float64), x=X, u=U, u_prev=UP, n=NS)

    # IV: prices from the reference at a true vol, recovered by reference Brent.
    rng = np.random.default_rng(4242)
    n = 16
    S = np.full(n, 100.0)
    K = S * rng.uniform(0.8, 1.2, n)
    T = rng.uniform(0.02, 2.0, n)
    r = rng.uniform(0.0, 0.08, n)
    q = rng.uniform(0.0, 0.04, n)
    vt = rng.uniform(0.05, 0.8, n)
    put = (np.arange(n) % 4 != 3).astype(np.int32)
    nx = np.full(n, 101)
    nt = np.full(n, 498)
    out, _, _ = price(lib, S, K, T, vt, r, q, put, nx, nt)
    px = out[:, 0].copy()
    o3 = np.full(3 * n, np.nan)
    st = np.zeros(n, np.int32)
    f = [np.ascontiguousarray(a, dtype=np.float64) for a in (S, K, T, r, q)]
    lib.ref_iv_batch(ctypes.c_int64(n), *(P(a) for a in f), P(put), P(px), P(vt),
                     P(np.ascontiguousarray(nx, np.int64)), P(np.ascontiguousarray(nt, np.int64)),
                     ctypes.c_int32(8), P(o3), P(st))
    save("iv.npz", S=S, K=K, T=T, r=r, q=q, is_put=put, price=px, true_vol=vt, nx=nx, nt=nt,
         out=o3.reshape(n, 3), status=st)

    golden_bspline(lib)
    golden_table(lib)
    golden_table_full(lib)
    golden_iv_config4(lib)
    golden_greeks_fd(lib)
    golden_surface(lib)
    golden_interp_iv(lib)
    golden_shared(lib)
    golden_tv(lib)
    golden_shared_tv(lib)
    golden_iv_tv(lib)
    golden_value_at(lib)
    golden_table_greeks(lib)
    golden_fit(lib)


def table_axes(nm, ntau, ns, nr):
    return (np.linspace(np.log(0.7), np.log(1.3), nm), np.linspace(0.02, 2.0, ntau),
            np.linspace(0.05, 0.8, ns), np.linspace(0.0, 0.08, nr))


BSPLINE_SEED = 2025


def bspline_coeffs(sizes):
    return np.random.default_rng(BSPLINE_SEED).standard_normal(int(np.prod(sizes)))


def golden_bspline(lib):
    axes = table_axes(50, 30, 20, 10)
    sizes = np.array([a.size for a in axes], np.int64)
    grids = np.concatenate(axes)
    coeffs = bspline_coeffs(sizes)
    rng = np.random.default_rng(7)
    q = np.stack([rng.uniform(a[0], a[-1], 4096) for a in axes], 1)
    edge = []
    for a in axes:
        edge.append([a[0], a[-1], a[0] - 0.1, a[-1] + 0.1, a[1], a[-2], 0.5 * (a[3] + a[4]), a[len(a) // 2]])
    edge = np.array(edge).T  # 8 x 4 combos along the diagonal
    e2 = np.array([[axes[0][i % 50], axes[1][(3 * i) % 30], axes[2][(7 * i) % 20], axes[3][(11 * i) % 10]]
                   for i in range(56)])
    q = np.ascontiguousarray(np.vstack([q, edge, e2]))
    out = np.zeros(q.shape[0])
    knots = np.zeros(int(sizes.sum()) + 16)
    rc = lib.ref_bspline4d_eval(P(sizes), P(grids), P(coeffs), P(q), ctypes.c_int64(q.shape[0]), P(out), P(knots))
    assert rc == 0
    save("bspline.npz", sizes=sizes, grids=grids, seed=np.array(BSPLINE_SEED), q=q, out=out, knots=knots)


def golden_table(lib):
    res = {}
    axes = table_axes(12, 6, 5, 3)
    alpha = 2.0 * np.arcsinh(5.0 / np.sqrt(2.0))
    for name, kind in (("explicit", 1), ("auto", 0)):
        nm, nt, ns, nr = (a.size for a in axes)
        out = np.zeros(nm * nt * ns * nr)
        dims = np.zeros(2 * ns * nr, np.int64)
        rc = lib.ref_table_sweep(P(axes[0]), ctypes.c_int64(nm), P(axes[1]), ctypes.c_int64(nt), P(axes[2]),
                                 ctypes.c_int64(ns), P(axes[3]), ctypes.c_int64(nr), ctypes.c_double(100.0),
                                 ctypes.c_double(0.0), ctypes.c_int32(1), ctypes.c_int32(kind),
                                 ctypes.c_double(-3.0), ctypes.c_double(3.0), ctypes.c_int64(201),
                                 ctypes.c_double(alpha), ctypes.c_int64(1000), P(out), P(dims))
        assert rc == 0
        res[f"{name}_tensor"] = out.reshape(nm, nt, ns, nr)
        res[f"{name}_dims"] = dims.reshape(ns * nr, 2)
    save("table.npz", m=axes[0], tau=axes[1], sigma=axes[2], r=axes[3], **res)


def golden_surface(lib):
    axes = table_axes(12, 8, 6, 5)
    sizes = np.array([a.size for a in axes], np.int64)
    grids = np.concatenate(axes)
    rng = np.random.default_rng(2026)
    coeffs = rng.standard_normal(int(np.prod(sizes))) * 2.0 + 0.5
    n = 2048
    p = np.stack([rng.uniform(80, 120, n), rng.uniform(80, 120, n), rng.uniform(0.005, 2.1, n),
                  rng.uniform(0.04, 0.85, n), rng.uniform(-0.005, 0.085, n)], 1)
    p = np.ascontiguousarray(p)
    res = {}
    for name, put, q in (("put", 1, 0.015), ("call", 0, 0.03)):
        out = np.zeros(n)
        rc = lib.ref_surface_price(P(sizes), P(grids), P(coeffs), ctypes.c_double(100.0), ctypes.c_double(q),
                                   ctypes.c_int32(put), P(p), ctypes.c_int64(n), P(out))
        assert rc == 0
        res[f"{name}_price"] = out
        res[f"{name}_q"] = np.array(q)
    nm, nt, ns, nr = (a.size for a in axes)
    ten = np.ascontiguousarray(rng.uniform(0.0, 0.45, nm * nt * ns * nr))
    eep = ten.copy()
    rc = lib.ref_eep_decompose(P(axes[0]), ctypes.c_int64(nm), P(axes[1]), ctypes.c_int64(nt), P(axes[2]),
                               ctypes.c_int64(ns), P(axes[3]), ctypes.c_int64(nr), ctypes.c_double(100.0),
                               ctypes.c_double(0.015), ctypes.c_int32(1), P(eep))
    assert rc == 0
    save("surface.npz", sizes=sizes, grids=grids, coeffs=coeffs, params=p, eep_in=ten, eep_out=eep, **res)


def golden_interp_iv(lib):
    sys.path.insert(0, str(ROOT / "oracle"))
    import fit_oracle
    axes = list(table_axes(12, 6, 5, 4))
    nm, nt, ns, nr = (a.size for a in axes)
    ten = np.zeros(nm * nt * ns * nr)
    dims = np.zeros(2 * ns * nr, np.int64)
    rc = lib.ref_table_sweep(P(axes[0]), ctypes.c_int64(nm), P(axes[1]), ctypes.c_int64(nt), P(axes[2]),
                             ctypes.c_int64(ns), P(axes[3]), ctypes.c_int64(nr), ctypes.c_double(100.0),
                             ctypes.c_double(0.0), ctypes.c_int32(1), ctypes.c_int32(0), ctypes.c_double(0.0),
                             ctypes.c_double(0.0), ctypes.c_int64(0), ctypes.c_double(0.0), ctypes.c_int64(0),
                             P(ten), P(dims))
    assert rc == 0
    rc = lib.ref_eep_decompose(P(axes[0]), ctypes.c_int64(nm), P(axes[1]), ctypes.c_int64(nt), P(axes[2]),
                               ctypes.c_int64(ns), P(axes[3]), ctypes.c_int64(nr), ctypes.c_double(100.0),
                               ctypes.c_double(0.0), ctypes.c_int32(1), P(ten))
    assert rc == 0
    sizes = np.array([nm, nt, ns, nr], np.int64)
    grids = np.ascontiguousarray(np.concatenate(axes))
    # the reference's own fit (BSplineNDSeparable<double,4>, LAPACKE forwarded)
    os.environ["MANGO_REF_LAPACKE"] = scipy_lapacke()
    lib.ref_bspline4d_fit.restype = ctypes.c_int32
    coeffs = np.zeros_like(ten)
    assert lib.ref_bspline4d_fit(P(sizes), P(grids), P(ten), ctypes.c_double(1e-6), P(coeffs), P(np.zeros(4)),
                                 P(np.zeros(4))) == 0
    dense = fit_oracle.fit4d(axes, ten.reshape(nm, nt, ns, nr)).ravel()
    assert np.abs(coeffs - dense).max() <= 1e-13 * np.abs(coeffs).max()
    rng = np.random.default_rng(31)
    n = 1024
    # vega at random in-range points
    vp = np.ascontiguousarray(np.stack([np.full(n, 100.0), 100.0 / np.exp(rng.uniform(axes[0][0], axes[0][-1], n)),
                                        rng.uniform(0.02, 2.0, n), rng.uniform(0.05, 0.8, n),
                                        rng.uniform(0.0, 0.08, n)], 1))
    vega = np.zeros(n)
    assert lib.ref_surface_vega(P(sizes), P(grids), P(coeffs), ctypes.c_double(100.0), ctypes.c_double(0.0),
                                ctypes.c_int32(1), P(vp), ctypes.c_int64(n), P(vega)) == 0
    # quotes priced from the table itself at seeded vols
    vt = rng.uniform(0.08, 0.7, n)
    K = 100.0 / np.exp(rng.uniform(axes[0][0], axes[0][-1], n))
    tau = rng.uniform(0.05, 1.9, n)
    r = rng.uniform(0.0, 0.08, n)
    pp = np.ascontiguousarray(np.stack([np.full(n, 100.0), K, tau, vt, r], 1))
    px = np.zeros(n)
    assert lib.ref_surface_price(P(sizes), P(grids), P(coeffs), ctypes.c_double(100.0), ctypes.c_double(0.0),
                                 ctypes.c_int32(1), P(pp), ctypes.c_int64(n), P(px)) == 0
    qs = np.stack([np.full(n, 100.0), K, tau, r, np.zeros(n), np.ones(n), px], 1)
    # invalid and edge quotes in the last rows
    qs[-1] = [100.0, 100.0, 1.0, 0.03, 0.0, 1.0, 150.0]       # above the put bound K -> arbitrage
    qs[-2] = [100.0, 100.0, 5.0, 0.03, 0.0, 1.0, 8.0]         # maturity outside the table
    qs[-3] = [100.0, 100.0, 1.0, 0.03, 0.01, 1.0, 8.0]        # dividend yield mismatch
    qs[-4] = [100.0, 100.0, 1.0, 0.03, 0.0, 0.0, 8.0]         # option type mismatch
    qs[-5] = [100.0, 130.0, 0.05, 0.03, 0.0, 1.0, 29.9]       # below intrinsic -> arbitrage
    qs[-6] = [100.0, 71.0, 0.03, 0.0, 0.0, 1.0, 1e-9]         # deep OTM, tiny vega
    qs[-7] = [100.0, 100.0, 1.0, 0.03, 0.0, 1.0, 45.0]        # no root in the bracket
    qs = np.ascontiguousarray(qs)
    cfg = np.array([50.0, 1e-6, 0.01, 3.0, 1e-4])
    out = np.zeros(3 * n)
    st = np.zeros(n, np.int32)
    assert lib.ref_surface_iv(P(sizes), P(grids), P(coeffs), ctypes.c_double(100.0), ctypes.c_double(0.0),
                              ctypes.c_int32(1), P(cfg), P(qs), ctypes.c_int64(n), P(out), P(st)) == 0
    save("interp_iv.npz", sizes=sizes, grids=grids, coeffs=coeffs, vega_params=vp, vega=vega, quotes=qs,
         true_vol=vt, cfg=cfg, out=out.reshape(n, 3), status=st)



def shared_batch(lib, S, K, T, sig, r, q, put, use_normalized, kind=0, x_min=0.0, x_max=0.0, nx=0,
                 alpha=0.0, nt=0):
    n = len(S)
    args = [np.ascontiguousarray(a, dtype=np.float64) for a in (S, K, T, sig, r, q)]
    put = np.ascontiguousarray(put, dtype=np.int32)
    out = np.full(4 * n, np.nan)
    dims = np.zeros(2 * n, np.int64)
    st = np.zeros(n, np.int32)
    rc = lib.ref_batch_shared(ctypes.c_int64(n), *(P(a) for a in args), P(put), ctypes.c_int32(use_normalized),
                              ctypes.c_int32(kind), ctypes.c_double(x_min), ctypes.c_double(x_max),
                              ctypes.c_int64(nx), ctypes.c_double(alpha), ctypes.c_int64(nt), ctypes.c_int32(8),
                              P(out), P(dims), P(st))
    assert rc == 0
    return out.reshape(n, 4), dims.reshape(n, 2), st


def golden_shared(lib):
    """BatchAmericanOptionSolver::solve_batch(use_shared_grid = true): option
    chains (several strikes per (sigma, r, q, T) group) on the normalized
    route, and batches the route rejects (mixed types, a wide grid) on the
    regular shared grid, with and without custom grids."""
    rng = np.random.default_rng(41)
    groups = [(0.2, 0.03, 0.01, 1.0), (0.25, 0.05, 0.0, 0.5), (0.3, 0.02, 0.02, 1.5), (0.15, 0.04, 0.01, 0.25),
              (0.35, 0.0, 0.0, 0.75), (0.22, 0.06, 0.03, 2.0)]
    rows = []
    for g in groups:
        for K in rng.uniform(86.0, 116.0, 9):
            rows.append((100.0, K) + g)
    rows.append((97.0, 101.0) + groups[0])            # a different spot in group 0
    rows.append((100.0, 100.0, 0.2 + 5e-11, 0.03, 0.01, 1.0))  # within the 1e-10 grouping tolerance
    chain = np.array(rows)
    n = len(chain)
    S, K, sig, r, q, T = (np.ascontiguousarray(chain[:, i]) for i in range(6))
    put = np.ones(n, np.int32)
    none = (0, 0.0, 0.0, 0, 0.0, 0)
    mixed = (np.arange(n) % 3 == 0).astype(np.int32)
    wide_sig = sig.copy()
    wide_sig[0] = 0.6
    wide_T = T.copy()
    wide_T[0] = 2.0
    cases = {
        "chain": (T, sig, put, 1, none),
        "chain_sinh": (T, sig, put, 1, (2, -2.5, 2.5, 181, 2.0, 300)),
        "chain_fixed_n": (T, sig, put, 1, (1, 0.0, 0.0, 141, 0.0, 0)),
        "chain_regular": (T, sig, put, 0, none),
        "mixed": (T, sig, mixed, 1, none),
        "mixed_fixed_n": (T, sig, mixed, 1, (1, 0.0, 0.0, 151, 0.0, 0)),
        "mixed_uniform": (T, sig, mixed, 1, (3, -3.0, 3.0, 201, 0.0, 250)),
        "wide": (wide_T, wide_sig, put, 1, none),
    }
    kw = {"S": S, "K": K, "T": T, "sig": sig, "r": r, "q": q, "put": put, "mixed": mixed, "wide_sig": wide_sig,
          "wide_T": wide_T}
    for name, (T_, sg, p_, un, grid) in cases.items():
        out, dims, st = shared_batch(lib, S, K, T_, sg, r, q, p_, un, *grid)
        assert (st == 0).all(), name
        kw[f"{name}_out"] = out
        kw[f"{name}_dims"] = dims
        kw[f"{name}_grid"] = np.array(grid, dtype=np.float64)
    save("shared.npz", **kw)


def tv_batch(lib, rows, rannacher=1):
    """Price rows (dicts) through ref_price_tv."""
    n = len(rows)
    col = lambda k, d=0.0: np.ascontiguousarray([r.get(k, d) for r in rows], dtype=np.float64)
    icol = lambda k, d=0: np.ascontiguousarray([r.get(k, d) for r in rows], dtype=np.int64)
    curves = [np.asarray(r.get("curve") or np.zeros((0, 2)), np.float64).reshape(-1, 2) for r in rows]
    divs = [np.asarray(r.get("divs") or np.zeros((0, 2)), np.float64).reshape(-1, 2) for r in rows]
    def flat(blocks):
        cnt = np.array([b.shape[0] for b in blocks], np.int64)
        off = np.concatenate([[0], np.cumsum(cnt)[:-1]]).astype(np.int64)
        allp = np.concatenate(blocks + [np.zeros((1, 2))])
        return off, cnt, np.ascontiguousarray(allp[:, 0]), np.ascontiguousarray(allp[:, 1])
    co, cn, ct, cl = flat(curves)
    do, dn, dt, da = flat(divs)
    put = np.ascontiguousarray([r["put"] for r in rows], dtype=np.int32)
    kind = np.ascontiguousarray([r.get("kind", 0) for r in rows], dtype=np.int32)
    out = np.full(4 * n, np.nan)
    dims = np.zeros(2 * n, np.int64)
    st = np.zeros(n, np.int32)
    args = [col("S"), col("K"), col("T"), col("sigma"), col("r"), col("q")]
    rest = [icol("nx"), icol("nt"), col("x_min"), col("x_max"), col("alpha")]
    rc = lib.ref_price_tv(ctypes.c_int64(n), *(P(a) for a in args), P(put), P(co), P(cn), P(ct), P(cl), P(do),
                          P(dn), P(dt), P(da), P(kind), *(P(a) for a in rest), ctypes.c_int32(rannacher),
                          ctypes.c_int32(8), P(out), P(dims), P(st))
    assert rc == 0
    return out.reshape(n, 4), dims.reshape(n, 2), st


def zero_curve(tenors, zeros):
    return [(0.0, 0.0)] + [(t, -z * t) for t, z in zip(tenors, zeros)]


TV_CURVES = {
    "up": zero_curve([0.25, 0.5, 1.0, 2.0, 3.0, 5.0], [0.02, 0.025, 0.03, 0.035, 0.038, 0.04]),
    "down": zero_curve([0.25, 0.5, 1.0, 2.0, 5.0], [0.06, 0.055, 0.05, 0.04, 0.03]),
    "short": [(0.0, 0.0), (1.0, -0.05)],
    "negative": zero_curve([0.5, 1.0, 2.0], [-0.005, -0.002, 0.004]),
    "single": [(0.0, 0.0)],
}


def tv_rows(seed, n, kinds):
    rng = np.random.default_rng(seed)
    rows = []
    curve_names = [None, "up", "down", "short", "negative"]
    for i in range(n):
        T = float(rng.uniform(0.3, 2.0))
        r = {"S": 100.0, "K": float(rng.uniform(80, 120)), "T": T, "sigma": float(rng.uniform(0.15, 0.45)),
             "r": float(rng.uniform(0.0, 0.06)), "q": float(rng.choice([0.0, 0.01, 0.025])),
             "put": int(i % 3 != 2)}
        c = curve_names[i % 5]
        if c:
            r["curve"] = TV_CURVES[c]
        d = (i // 5) % 6
        if d == 1:
            r["divs"] = [(0.25 * T, 1.0), (0.75 * T, 1.0)]
        elif d == 2:
            r["divs"] = [(0.5 * T, 3.0)]
        elif d == 3:
            r["divs"] = [(t, 0.5) for t in np.arange(0.25, T, 0.25)]
        elif d == 4:
            r["divs"] = [(0.3 * T, 0.0), (0.6 * T, 1.5)]
        elif d == 5:
            r["divs"] = [(0.4 * T, 1.0), (0.4 * T, 1.5)]
        if "curve" not in r and "divs" not in r:
            r["divs"] = [(0.5 * T, 2.0)]
        k = kinds[i % len(kinds)]
        r["kind"] = k
        if k == 1:
            r["nx"], r["nt"] = (101, 200) if i % 2 else (121, 0)
        elif k == 2:
            r.update(nx=121, nt=300, x_min=-3.0, x_max=3.0, alpha=2.0)
        elif k == 3:
            r.update(nx=151, nt=250, x_min=-3.0, x_max=3.0)
        rows.append(r)
    return rows


def golden_tv(lib):
    """Yield curves and discrete dividends through AmericanOptionSolver:
    the solver's own grid, pinned-size, sinh and uniform grids, Rannacher on
    and off, and edge schedules."""
    cases = {
        "auto": (tv_rows(51, 96, [0]), 1),
        "explicit": (tv_rows(52, 96, [1, 2, 3]), 1),
        "no_rannacher": (tv_rows(53, 32, [0, 2]), 0),
    }
    edge = [
        # dividends at t = 0 and t = T: no event, no mandatory point
        {"S": 100.0, "K": 100.0, "T": 1.0, "sigma": 0.25, "r": 0.04, "q": 0.0, "put": 1,
         "divs": [(0.0, 2.0), (1.0, 2.0)], "curve": TV_CURVES["up"]},
        # a dividend larger than e^{x_min} K: the conservative grid extension
        {"S": 100.0, "K": 100.0, "T": 1.0, "sigma": 0.2, "r": 0.03, "q": 0.0, "put": 1, "divs": [(0.5, 60.0)]},
        {"S": 100.0, "K": 100.0, "T": 1.0, "sigma": 0.2, "r": 0.03, "q": 0.0, "put": 0, "divs": [(0.5, 60.0)]},
        # single-point curve: rate 0 everywhere
        {"S": 100.0, "K": 110.0, "T": 0.7, "sigma": 0.3, "r": 0.05, "q": 0.0, "put": 1, "curve": TV_CURVES["single"]},
        # deep ITM call before a large dividend (early exercise), and a deep ITM put
        {"S": 150.0, "K": 100.0, "T": 0.5, "sigma": 0.2, "r": 0.02, "q": 0.0, "put": 0, "divs": [(0.25, 8.0)]},
        {"S": 60.0, "K": 100.0, "T": 1.5, "sigma": 0.25, "r": 0.05, "q": 0.0, "put": 1, "divs": [(0.5, 1.0)],
         "curve": TV_CURVES["down"]},
        # curve beyond its last tenor (flat forward extrapolation)
        {"S": 100.0, "K": 95.0, "T": 2.0, "sigma": 0.2, "r": 0.0, "q": 0.01, "put": 0, "curve": TV_CURVES["short"]},
        # a dividend on the first step and one on the last
        {"S": 100.0, "K": 100.0, "T": 1.0, "sigma": 0.2, "r": 0.03, "q": 0.0, "put": 1,
         "divs": [(0.999, 1.0), (0.001, 1.0)]},
    ]
    cases["edge"] = (edge, 1)
    kw = {}
    for name, (rows, rann) in cases.items():
        out, dims, st = tv_batch(lib, rows, rann)
        assert (st == 0).all(), (name, st)
        kw[f"{name}_rows"] = np.array([json.dumps(r) for r in rows])
        kw[f"{name}_out"] = out
        kw[f"{name}_dims"] = dims
        kw[f"{name}_rannacher"] = np.int32(rann)
    save("tv.npz", **kw)


def shared_tv_batch(lib, rows, use_normalized, grid=(0, 0.0, 0.0, 0, 0.0, 0)):
    n = len(rows)
    col = lambda k, d=0.0: np.ascontiguousarray([r.get(k, d) for r in rows], dtype=np.float64)
    curves = [np.asarray(r.get("curve") or np.zeros((0, 2)), np.float64).reshape(-1, 2) for r in rows]
    divs = [np.asarray(r.get("divs") or np.zeros((0, 2)), np.float64).reshape(-1, 2) for r in rows]
    def flat(blocks):
        cnt = np.array([b.shape[0] for b in blocks], np.int64)
        off = np.concatenate([[0], np.cumsum(cnt)[:-1]]).astype(np.int64)
        allp = np.concatenate(blocks + [np.zeros((1, 2))])
        return off, cnt, np.ascontiguousarray(allp[:, 0]), np.ascontiguousarray(allp[:, 1])
    co, cn, ct, cl = flat(curves)
    do, dn, dt, da = flat(divs)
    put = np.ascontiguousarray([r["put"] for r in rows], dtype=np.int32)
    out = np.full(4 * n, np.nan)
    dims = np.zeros(2 * n, np.int64)
    st = np.zeros(n, np.int32)
    kind, x_min, x_max, nx, alpha, nt = grid
    args = [col("S"), col("K"), col("T"), col("sigma"), col("r"), col("q")]
    rc = lib.ref_batch_shared_tv(ctypes.c_int64(n), *(P(a) for a in args), P(put), P(co), P(cn), P(ct), P(cl),
                                 P(do), P(dn), P(dt), P(da), ctypes.c_int32(use_normalized), ctypes.c_int32(kind),
                                 ctypes.c_double(x_min), ctypes.c_double(x_max), ctypes.c_int64(nx),
                                 ctypes.c_double(alpha), ctypes.c_int64(nt), ctypes.c_int32(8), P(out), P(dims),
                                 P(st))
    assert rc == 0
    return out.reshape(n, 4), dims.reshape(n, 2), st


def golden_shared_tv(lib):
    """solve_batch(use_shared_grid = true) with yield curves (normalized
    chains grouped by curve) and discrete dividends (regular shared grid
    with per-option mandatory times)."""
    rng = np.random.default_rng(61)
    chain = []
    for ci, c in enumerate(["up", "down", "up"]):
        for K in rng.uniform(88.0, 114.0, 8):
            chain.append({"S": 100.0, "K": float(K), "T": [1.0, 0.5, 1.0][ci], "sigma": [0.2, 0.3, 0.2][ci],
                          "r": 0.0, "q": 0.01, "put": 1, "curve": TV_CURVES[c]})
    chain.append({"S": 100.0, "K": 100.0, "T": 1.0, "sigma": 0.2, "r": 0.03, "q": 0.01, "put": 1})
    divs = []
    for i in range(40):
        T = float(rng.uniform(0.4, 1.5))
        r = {"S": 100.0, "K": float(rng.uniform(85, 115)), "T": T, "sigma": float(rng.uniform(0.15, 0.4)),
             "r": 0.03, "q": 0.0, "put": int(i % 4 != 3)}
        if i % 3 == 0:
            r["divs"] = [(0.5 * T, 1.5)]
        elif i % 3 == 1:
            r["divs"] = [(0.3 * T, 1.0), (0.7 * T, 1.0)]
            r["curve"] = TV_CURVES["up"]
        divs.append(r)
    cases = {
        "chain_curve": (chain, 1, (0, 0.0, 0.0, 0, 0.0, 0)),
        "chain_curve_sinh": (chain, 1, (2, -2.5, 2.5, 161, 2.0, 250)),
        "divs": (divs, 1, (0, 0.0, 0.0, 0, 0.0, 0)),
        "divs_uniform": (divs, 1, (3, -3.0, 3.0, 181, 0.0, 300)),
        "divs_fixed_n": (divs, 1, (1, 0.0, 0.0, 131, 0.0, 0)),
    }
    kw = {}
    for name, (rows, un, grid) in cases.items():
        out, dims, st = shared_tv_batch(lib, rows, un, grid)
        assert (st == 0).all(), name
        kw[f"{name}_rows"] = np.array([json.dumps(r) for r in rows])
        kw[f"{name}_out"] = out
        kw[f"{name}_dims"] = dims
        kw[f"{name}_grid"] = np.array(grid, dtype=np.float64)
    save("shared_tv.npz", **kw)


def golden_iv_tv(lib):
    """IVSolver::solve with yield curves and dividends: market prices from
    the reference's own solver at the true volatility, implied vols on a
    grid sized at 0.3 (PDEGridConfig, dividend times added by the solver)."""
    rows = tv_rows(71, 96, [1])
    rng = np.random.default_rng(72)
    for r in rows:
        r["nx"], r["nt"] = 101, 200
        r["sigma"] = float(rng.uniform(0.12, 0.6))
    out, dims, st = tv_batch(lib, rows, 1)
    assert (st == 0).all()
    price = np.ascontiguousarray(out[:, 0])
    n = len(rows)
    col = lambda k: np.ascontiguousarray([r.get(k, 0.0) for r in rows], dtype=np.float64)
    curves = [np.asarray(r.get("curve") or np.zeros((0, 2)), np.float64).reshape(-1, 2) for r in rows]
    divs = [np.asarray(r.get("divs") or np.zeros((0, 2)), np.float64).reshape(-1, 2) for r in rows]
    def flat(blocks):
        cnt = np.array([b.shape[0] for b in blocks], np.int64)
        off = np.concatenate([[0], np.cumsum(cnt)[:-1]]).astype(np.int64)
        allp = np.concatenate(blocks + [np.zeros((1, 2))])
        return off, cnt, np.ascontiguousarray(allp[:, 0]), np.ascontiguousarray(allp[:, 1])
    co, cn, ct, cl = flat(curves)
    do, dn, dt, da = flat(divs)
    put = np.ascontiguousarray([r["put"] for r in rows], dtype=np.int32)
    gsig = np.full(n, 0.3)
    nx = np.full(n, 101, np.int64)
    nt = np.full(n, 200, np.int64)
    o3 = np.full(3 * n, np.nan)
    ist = np.zeros(n, np.int32)
    lib.ref_iv_batch_tv(ctypes.c_int64(n), P(col("S")), P(col("K")), P(col("T")), P(col("r")), P(col("q")), P(put),
                        P(price), P(gsig), P(nx), P(nt), P(co), P(cn), P(ct), P(cl), P(do), P(dn), P(dt), P(da),
                        ctypes.c_int32(8), P(o3), P(ist))
    save("iv_tv.npz", rows=np.array([json.dumps(r) for r in rows]), price=price, grid_sigma=gsig, nx=nx, nt=nt,
         out=o3.reshape(n, 3), status=ist)


def golden_value_at(lib):
    """AmericanOptionResult::value_at at other spots, below, inside and
    above each option's grid."""
    S, K, T, sig, r, q, put = config0_inputs(64, 81, True)
    rng = np.random.default_rng(82)
    spot2 = rng.uniform(40.0, 160.0, 64)
    spot2[:4] = [1e-3, 5.0, 1e4, 100.0]  # below / far below / above the grid, at the spot
    nx = np.full(64, 101, np.int64)
    nt = np.full(64, 498, np.int64)
    out = np.zeros(64)
    st = np.zeros(64, np.int32)
    a = [np.ascontiguousarray(v, dtype=np.float64) for v in (S, K, T, sig, r, q)]
    lib.ref_value_at(ctypes.c_int64(64), *(P(v) for v in a), P(np.ascontiguousarray(put, np.int32)), P(nx), P(nt),
                     P(spot2), ctypes.c_int32(8), P(out), P(st))
    assert (st == 0).all()
    save("value_at.npz", S=S, K=K, T=T, sigma=sig, r=r, q=q, is_put=put, nx=nx, nt=nt, spot2=spot2, value=out)


def golden_table_greeks(lib):
    """The standard table's delta / gamma / theta / rho (PriceTable over
    EEPLayer<TransformLeaf>) on interp_iv.npz's coefficients, as a put table
    with q = 0 (the one the coefficients were fitted for), a put table with
    q = 0.02 and a call table with q = 0.01 (the same spline reused, so the
    European terms with a dividend yield are exercised)."""
    g = np.load(HERE / "interp_iv.npz")
    sizes, grids, coeffs = g["sizes"], g["grids"], g["coeffs"]
    axes = np.split(grids, np.cumsum(sizes)[:-1])
    rng = np.random.default_rng(57)
    n = 512
    m = rng.uniform(axes[0][0], axes[0][-1], n)
    p = np.stack([np.full(n, 100.0), 100.0 / np.exp(m), rng.uniform(axes[1][0], axes[1][-1], n),
                  rng.uniform(axes[2][0], axes[2][-1], n), rng.uniform(axes[3][0], axes[3][-1], n)], 1)
    # the axis ends and a deep out-of-the-money corner (spline value <= 0)
    p[0] = [100.0, 100.0 / np.exp(axes[0][0]), axes[1][0], axes[2][0], axes[3][0]]
    p[1] = [100.0, 100.0 / np.exp(axes[0][-1]), axes[1][-1], axes[2][-1], axes[3][-1]]
    p[2] = [100.0, 100.0 / np.exp(axes[0][-1]), axes[1][0], axes[2][0], axes[3][-1]]
    p = np.ascontiguousarray(p)
    kw = {}
    for name, q, put in (("put", 0.0, 1), ("put_q", 0.02, 1), ("call_q", 0.01, 0)):
        out = np.zeros(4 * n)
        st = np.zeros(n, np.int32)
        assert lib.ref_surface_greeks(P(sizes), P(grids), P(coeffs), ctypes.c_double(100.0), ctypes.c_double(q),
                                      ctypes.c_int32(put), P(p), ctypes.c_int64(n), P(out), P(st)) == 0
        assert (st == 0).all()
        kw[f"{name}_greeks"] = out.reshape(n, 4)
    save("table_greeks.npz", sizes=sizes, grids=grids, coeffs=coeffs, params=p, **kw)


def golden_table_full(lib):
    """The table-build workload's sweep at full size: 50 x 30 x 20 x 10 axes,
    200 (vol, rate) slices, the explicit 201 x 1000 grid (the reference's
    per-slice fallback route)."""
    axes = table_axes(50, 30, 20, 10)
    alpha = 2.0 * np.arcsinh(5.0 / np.sqrt(2.0))
    nm, nt, ns, nr = (a.size for a in axes)
    out = np.zeros(nm * nt * ns * nr)
    dims = np.zeros(2 * ns * nr, np.int64)
    rc = lib.ref_table_sweep(P(axes[0]), ctypes.c_int64(nm), P(axes[1]), ctypes.c_int64(nt), P(axes[2]),
                             ctypes.c_int64(ns), P(axes[3]), ctypes.c_int64(nr), ctypes.c_double(100.0),
                             ctypes.c_double(0.0), ctypes.c_int32(1), ctypes.c_int32(1),
                             ctypes.c_double(-3.0), ctypes.c_double(3.0), ctypes.c_int64(201),
                             ctypes.c_double(alpha), ctypes.c_int64(1000), P(out), P(dims))
    assert rc == 0
    save("table_full.npz", m=axes[0], tau=axes[1], sigma=axes[2], r=axes[3], alpha=np.array(alpha),
         tensor=out.reshape(nm, nt, ns, nr), dims=dims.reshape(ns * nr, 2))


def scipy_lapacke():
    """The OpenBLAS that scipy bundles, which exports LAPACKE's banded
    routines (with a scipy_ prefix): the reference's fit calls them through
    oracle/ref/lapacke_stubs.c."""
    import glob
    import scipy
    libs = glob.glob(str(pathlib.Path(scipy.__file__).parent.parent / "scipy.libs" / "libscipy_openblas*.so"))
    if not libs:
        sys.exit("no LAPACKE-providing library found for the reference's fit")
    return libs[0]


FIT_SEED = 2028


def fit_table_values(sizes):
    """Values of the full-axes fit case (regenerated by the tests from
    FIT_SEED)."""
    return np.random.default_rng(FIT_SEED).standard_normal(int(np.prod(sizes)))


def golden_fit(lib):
    """The reference's separable fit on the full table axes and on the
    surface axes."""
    os.environ["MANGO_REF_LAPACKE"] = scipy_lapacke()
    lib.ref_bspline4d_fit.restype = ctypes.c_int32
    res = {"table_seed": np.array(FIT_SEED)}
    big = table_axes(50, 30, 20, 10)
    small = table_axes(12, 8, 6, 5)
    cases = (("table", big, fit_table_values([a.size for a in big])),
             ("rand", small, np.random.default_rng(2027).standard_normal(12 * 8 * 6 * 5)))
    for name, ax, vals in cases:
        sizes = np.array([a.size for a in ax], np.int64)
        grids = np.ascontiguousarray(np.concatenate(ax))
        vals = np.ascontiguousarray(vals, dtype=np.float64)
        co = np.zeros_like(vals)
        resid, cond = np.zeros(4), np.zeros(4)
        rc = lib.ref_bspline4d_fit(P(sizes), P(grids), P(vals), ctypes.c_double(1e-6), P(co), P(resid), P(cond))
        assert rc == 0, name
        res.update({f"{name}_sizes": sizes, f"{name}_grids": grids, f"{name}_residual": resid,
                    f"{name}_cond": cond})
        if name == "table":
            idx = np.sort(np.random.default_rng(FIT_SEED + 1).choice(vals.size, 4096, replace=False))
            res.update({"table_idx": idx, "table_coeffs": co[idx], "table_coeff_sum": np.array(co.sum()),
                        "table_coeff_absmax": np.array(np.abs(co).max())})
        else:
            res.update({f"{name}_values": vals, f"{name}_coeffs": co})
    save("fit.npz", **res)


def golden_iv_config4(lib):
    """4,096 quotes of the batched-IV workload's distributions (true vol
    U[0.05, 0.8], K/S U[0.8, 1.2], T U[0.02, 2], r U[0, 0.08], q U[0, 0.04],
    3 in 4 puts), priced by the reference at the true vol on the 101 x 498
    grid rule sized at that vol, and inverted by the reference's IVSolver
    (Brent) on the same grid."""
    rng = np.random.default_rng(4244)
    n = 4096
    S = np.full(n, 100.0)
    K = S * rng.uniform(0.8, 1.2, n)
    T = rng.uniform(0.02, 2.0, n)
    r = rng.uniform(0.0, 0.08, n)
    q = rng.uniform(0.0, 0.04, n)
    vt = rng.uniform(0.05, 0.8, n)
    put = (np.arange(n) % 4 != 3).astype(np.int32)
    nx = np.full(n, 101)
    nt = np.full(n, 498)
    out, _, pst = price(lib, S, K, T, vt, r, q, put, nx, nt)
    assert (pst == 0).all()
    px = out[:, 0].copy()
    o3 = np.full(3 * n, np.nan)
    st = np.zeros(n, np.int32)
    f = [np.ascontiguousarray(a, dtype=np.float64) for a in (S, K, T, r, q)]
    lib.ref_iv_batch(ctypes.c_int64(n), *(P(a) for a in f), P(put), P(px), P(vt),
                     P(np.ascontiguousarray(nx, np.int64)), P(np.ascontiguousarray(nt, np.int64)),
                     ctypes.c_int32(0), P(o3), P(st))
    save("iv_config4.npz", S=S, K=K, T=T, r=r, q=q, is_put=put, price=px, true_vol=vt, nx=nx, nt=nt,
         out=o3.reshape(n, 3), status=st)


def golden_greeks_fd(lib):
    """1,024 American puts of the differentiation workload (config-0
    distributions, 101 x 498 grid rule): the reference's prices at the
    option and at the eight bumped parameter sets of a central difference
    for h = 1e-5, 1e-6 and 1e-7 (sigma h, max(|r|, 1e-2) h, max(q, 1e-2) h
    clipped at q = 0, K h), all on the option's own frozen grid; and the
    differences themselves, per h."""
    n = 1024
    S, K, T, sig, r, q, put = config0_inputs(n, 3, False)
    nx = np.full(n, 101, np.int64)
    nt = np.full(n, 498, np.int64)

    def prices(s_, r_, q_, k_):
        out = np.zeros(4 * n)
        st = np.zeros(n, np.int32)
        f = [np.ascontiguousarray(a, dtype=np.float64) for a in (S, k_, T, s_, r_, q_, S, K, T, sig)]
        lib.ref_price_frozen(ctypes.c_int64(n), *(P(a) for a in f[:6]), P(put), *(P(a) for a in f[6:]),
                             P(nx), P(nt), ctypes.c_int32(0), P(out), P(st))
        assert (st == 0).all()
        return out.reshape(n, 4)[:, 0]

    base = prices(sig, r, q, K)
    hs_all = np.array([1e-5, 1e-6, 1e-7])
    kw = {k: np.zeros((3, n)) for k in ("vega", "rho", "dividend_rho", "dstrike")}
    for j, h in enumerate(hs_all):
        hs, hr = sig * h, np.maximum(np.abs(r), 1e-2) * h
        hq, hk = np.maximum(q, 1e-2) * h, K * h
        qdn = np.maximum(q - hq, 0.0)
        kw["vega"][j] = (prices(sig + hs, r, q, K) - prices(sig - hs, r, q, K)) / (2 * hs)
        kw["rho"][j] = (prices(sig, r + hr, q, K) - prices(sig, r - hr, q, K)) / (2 * hr)
        kw["dividend_rho"][j] = (prices(sig, r, q + hq, K) - prices(sig, r, qdn, K)) / (q + hq - qdn)
        kw["dstrike"][j] = (prices(sig, r, q, K + hk) - prices(sig, r, q, K - hk)) / (2 * hk)
    save("greeks_fd.npz", S=S, K=K, T=T, sigma=sig, r=r, q=q, is_put=put, h=hs_all, value=base, **kw)


if __name__ == "__main__":
    if len(sys.argv) > 1:  # regenerate the named fixtures only
        _l = _lib()
        for _name in sys.argv[1:]:
            globals()[f"golden_{_name}"](_l)
    else:
        sys.exit(main())
