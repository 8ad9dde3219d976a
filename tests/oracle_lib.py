"""ctypes wrapper over the CPU oracle (oracle/mango_oracle.c), for tests only.

The oracle is the checker: tests compare the GPU engine with it and with the
reference's golden vectors; nothing in the engine imports this module.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from __graft_entry__ import _build_module

_lib = None
c = ctypes.c_double


class Spec(ctypes.Structure):
    _fields_ = [("type", ctypes.c_int32), ("n_clusters", ctypes.c_int32), ("x_min", c), ("x_max", c),
                ("n_points", ctypes.c_int64), ("concentration", c), ("c_center", c * 4),
                ("c_alpha", c * 4), ("c_weight", c * 4)]


class Accuracy(ctypes.Structure):
    _fields_ = [("n_sigma", c), ("alpha", c), ("tol", c), ("c_t", c), ("min_spatial_points", ctypes.c_int64),
                ("max_spatial_points", ctypes.c_int64), ("max_time_steps", ctypes.c_int64)]


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(str(_build_module().build_oracle()))
    return _lib


def P(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _f(a, n=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return np.broadcast_to(a, (n,)).copy() if n is not None and a.ndim == 0 else a


def price_batch(S, K, T, sigma, r, q, is_put, nx, nt, rannacher=1, threads=0):
    """value/delta/gamma/theta (n x 4), dims (n x 2), status (n)."""
    n = len(S)
    f = [np.ascontiguousarray(np.broadcast_to(np.asarray(a, np.float64), (n,))) for a in (S, K, T, sigma, r, q)]
    put = np.ascontiguousarray(np.broadcast_to(np.asarray(is_put, np.int32), (n,)))
    nx = np.ascontiguousarray(np.broadcast_to(np.asarray(nx, np.int64), (n,)))
    nt = np.ascontiguousarray(np.broadcast_to(np.asarray(nt, np.int64), (n,)))
    out = np.full(4 * n, np.nan)
    dims = np.zeros(2 * n, np.int64)
    st = np.zeros(n, np.int32)
    threads = threads or (os.cpu_count() or 1)
    lib().mo_price_batch(ctypes.c_int64(n), *(P(a) for a in f), P(put), P(nx), P(nt),
                         ctypes.c_int32(rannacher), ctypes.c_int32(threads), P(out), P(dims), P(st))
    return out.reshape(n, 4), dims.reshape(n, 2), st


def price_on_grid(S, K, T, sigma, r, q, is_put, x, nt, rannacher=1):
    x = np.ascontiguousarray(x, np.float64)
    out = np.full(4, np.nan)
    u = np.zeros(x.size)
    up = np.zeros(x.size)
    rc = lib().mo_price_on_grid(c(S), c(K), c(T), c(sigma), c(r), c(q), ctypes.c_int32(int(is_put)), P(x),
                                ctypes.c_int64(x.size), ctypes.c_int64(int(nt)), ctypes.c_int32(rannacher),
                                P(out), P(u), P(up))
    return rc, out, u, up


def price_tangent_on_grid(S, K, T, sigma, r, q, is_put, x, nt):
    """mo_price_tangent_on_grid: {value, delta, dV/dsigma, dV/drate, dV/dq, dV/dK}."""
    x = np.ascontiguousarray(x, np.float64)
    out = np.full(6, np.nan)
    rc = lib().mo_price_tangent_on_grid(c(S), c(K), c(T), c(sigma), c(r), c(q), ctypes.c_int32(int(is_put)),
                                        P(x), ctypes.c_int64(x.size), ctypes.c_int64(int(nt)), P(out))
    return rc, out


def grid(S, K, T, sigma, nx=0):
    acc = Accuracy()
    lib().mo_default_accuracy(ctypes.byref(acc))
    if nx:
        acc.min_spatial_points = acc.max_spatial_points = int(nx)
    sp = Spec()
    nt = ctypes.c_int64()
    lib().mo_estimate_grid(c(S), c(K), c(T), c(sigma), ctypes.byref(acc), ctypes.byref(sp), ctypes.byref(nt))
    x = np.zeros(sp.n_points)
    lib().mo_generate_grid(ctypes.byref(sp), P(x))
    return x, nt.value


def explicit_grid(kind, x_min, x_max, n, alpha):
    """GridSpec::sinh_spaced (kind 2) or uniform (kind 3), generated."""
    sp = Spec()
    sp.type = 2 if kind == 2 else 0
    sp.x_min, sp.x_max, sp.n_points, sp.concentration = x_min, x_max, int(n), alpha
    x = np.zeros(int(n))
    lib().mo_generate_grid(ctypes.byref(sp), P(x))
    return x


def iv_batch(S, K, T, r, q, is_put, price, grid_sigma, nx, nt, threads=0):
    n = len(S)
    f = [np.ascontiguousarray(np.broadcast_to(np.asarray(a, np.float64), (n,))) for a in (S, K, T, r, q)]
    put = np.ascontiguousarray(np.broadcast_to(np.asarray(is_put, np.int32), (n,)))
    px = np.ascontiguousarray(price, np.float64)
    gs = np.ascontiguousarray(grid_sigma, np.float64)
    nx = np.ascontiguousarray(np.broadcast_to(np.asarray(nx, np.int64), (n,)))
    nt = np.ascontiguousarray(np.broadcast_to(np.asarray(nt, np.int64), (n,)))
    out = np.full(3 * n, np.nan)
    st = np.zeros(n, np.int32)
    threads = threads or (os.cpu_count() or 1)
    lib().mo_iv_batch(ctypes.c_int64(n), *(P(a) for a in f), P(put), P(px), P(gs), P(nx), P(nt),
                      ctypes.c_int32(threads), P(out), P(st))
    return out.reshape(n, 3), st


def bspline4d_eval(axes, coeffs, q):
    """BSplineND<double,4>::eval of the C restatement (mo_bspline4d_eval)."""
    sizes = np.array([len(a) for a in axes], np.int64)
    grids = np.ascontiguousarray(np.concatenate([np.asarray(a, np.float64) for a in axes]))
    c = np.ascontiguousarray(coeffs, dtype=np.float64).ravel()
    q = np.ascontiguousarray(q, dtype=np.float64).reshape(-1, 4)
    out = np.zeros(q.shape[0])
    rc = lib().mo_bspline4d_eval(P(sizes), P(grids), P(c), P(q), ctypes.c_int64(q.shape[0]), P(out))
    assert rc == 0
    return out


def surface_price(axes, coeffs, params, K_ref, q, put, eep=True):
    """AnyPriceTable::price restated: max(0, spline(log(S/K), tau, sigma, r)) K/K_ref
    plus the European price (params: n x 5 {S, K, tau, sigma, r})."""
    import fit_oracle
    p = np.asarray(params, np.float64).reshape(-1, 5)
    x = np.stack([np.log(p[:, 0] / p[:, 1]), p[:, 2], p[:, 3], p[:, 4]], 1)
    raw = bspline4d_eval(axes, coeffs, x)
    v = np.maximum(0.0, raw) * p[:, 1] / K_ref
    if eep:
        v = v + np.array([fit_oracle.european_price(*row, q, bool(put)) for row in p])
    return v
