"""mango-option GB300 engine: Python surface over the C ABI in include/mango_gpu.h.

The names mirror the reference's pybind11 module ``mango_option``
(src/python/mango_bindings.cpp): ``OptionType``, ``PricingParams``,
``american_option_price`` (mango_bindings.cpp:580), ``BatchAmericanOptionSolver``
with ``solve_batch`` (mango_bindings.cpp:681-745) and the result accessors
``value``/``delta``/``gamma``/``theta``.  Batches may also be passed as numpy
arrays (``price_arrays``), which is how large workloads avoid per-option Python
objects.

Everything runs through ``libmango_gpu.so`` (built in-tree by build.py).  There
is no CPU fallback: if the library is missing or no GB300 is present, the calls
raise.
"""
from __future__ import annotations

import ctypes
import dataclasses
import enum
import pathlib
from typing import Iterable, Optional, Sequence, Tuple

import numpy as np

_PKG = pathlib.Path(__file__).resolve().parent
LIB_PATH = _PKG / "_build" / "libmango_gpu.so"

MANGO_OK = 0
MANGO_ERR_VALIDATION = 1
MANGO_ERR_ARBITRAGE = 2
MANGO_ERR_NO_CONVERGENCE = 3
MANGO_ERR_BRACKETING = 4
MANGO_ERR_SOLVER = 5

GRID_AUTO = 0
GRID_FIXED_N = 1
GRID_SINH = 2
GRID_UNIFORM = 3
GRID_FIXED_N_AT_VOL = 4

# Root finders of mango_gpu_solve_iv_batch_method.
IV_BRENT = 0
IV_SECANT = 1
IV_NEWTON = 2

# C layouts (include/mango_gpu.h); sizes are asserted there and in tests.
PRICING_DTYPE = np.dtype([
    ("spot", "f8"), ("strike", "f8"), ("maturity", "f8"), ("dividend_yield", "f8"),
    ("volatility", "f8"), ("rate_const", "f8"), ("tenor_points", "u8"),
    ("n_tenor_points", "u8"), ("dividends", "u8"), ("n_dividends", "u8"),
    ("option_type", "i4"), ("_pad", "i4")])
IVQUERY_DTYPE = np.dtype([
    ("spot", "f8"), ("strike", "f8"), ("maturity", "f8"), ("dividend_yield", "f8"),
    ("market_price", "f8"), ("rate_const", "f8"), ("tenor_points", "u8"),
    ("n_tenor_points", "u8"), ("dividends", "u8"), ("n_dividends", "u8"),
    ("option_type", "i4"), ("_pad", "i4")])
GRID_DTYPE = np.dtype([
    ("kind", "i4"), ("reserved", "i4"), ("n_space", "i8"), ("n_time", "i8"),
    ("x_min", "f8"), ("x_max", "f8"), ("alpha", "f8")])
GREEKS_DTYPE = np.dtype([
    ("value", "f8"), ("delta", "f8"), ("gamma", "f8"), ("theta", "f8"),
    ("status", "i4"), ("n_space", "i4"), ("n_time", "i4"), ("reserved", "i4"),
    ("vega", "f8"), ("rho", "f8"), ("dividend_rho", "f8"), ("dstrike", "f8")])
IVSLOT_DTYPE = np.dtype([
    ("status", "i4"), ("_pad", "i4"), ("implied_vol", "f8"), ("iterations", "u8"),
    ("final_error", "f8"), ("vega", "f8"), ("has_vega", "i4"), ("used_rate_approximation", "i4")])
OUT_DTYPE = np.dtype([
    ("value", "f8"), ("delta", "f8"), ("gamma", "f8"), ("theta", "f8"),
    ("status", "i4"), ("n_space", "i4"), ("n_time", "i4"), ("reserved", "i4")])


class MangoError(ctypes.Structure):
    _fields_ = [("code", ctypes.c_int32), ("message", ctypes.c_char * 256)]


class MangoIvConfig(ctypes.Structure):
    _fields_ = [("brent_tol_abs", ctypes.c_double), ("max_iter", ctypes.c_int32)]


class MangoGpuTrbdf2(ctypes.Structure):
    _fields_ = [("gamma", ctypes.c_double), ("rannacher_startup", ctypes.c_int32),
                ("reserved", ctypes.c_int32)]


class MangoGpuStats(ctypes.Structure):
    _fields_ = [(k, ctypes.c_double) for k in (
        "host_prep_ms", "h2d_ms", "prep_ms", "march_ms", "outputs_ms", "d2h_ms", "total_ms",
        "algo_flops", "h2d_bytes", "d2h_bytes")] + [
        ("options", ctypes.c_int64), ("tiles", ctypes.c_int64), ("kernel_launches", ctypes.c_int64),
        ("iv_evals", ctypes.c_int64 * 2)]


class MangoInterpSolverConfig(ctypes.Structure):
    _fields_ = [("max_iter", ctypes.c_uint64), ("tolerance", ctypes.c_double), ("sigma_min", ctypes.c_double),
                ("sigma_max", ctypes.c_double), ("vega_threshold", ctypes.c_double)]


class MangoGpuFitStats(ctypes.Structure):
    _fields_ = [("max_residual", ctypes.c_double * 4), ("condition", ctypes.c_double * 4),
                ("failed_slices", ctypes.c_uint64 * 4)]


class EngineError(RuntimeError):
    """Raised when the engine call itself fails (no device, CUDA error)."""


_lib = None
_P = ctypes.c_void_p


def library() -> ctypes.CDLL:
    """Load libmango_gpu.so (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise ImportError(f"{LIB_PATH} is missing: run __graft_entry__.build() first")
        lib = ctypes.CDLL(str(LIB_PATH))
        lib.mango_gpu_context_create.argtypes = [ctypes.c_int32, ctypes.POINTER(_P), ctypes.POINTER(MangoError)]
        lib.mango_gpu_context_create.restype = ctypes.c_int32
        lib.mango_gpu_context_destroy.argtypes = [_P]
        lib.mango_gpu_context_destroy.restype = None
        lib.mango_gpu_price_american_batch.argtypes = [
            _P, _P, ctypes.c_uint64, _P, ctypes.c_uint64, ctypes.POINTER(MangoGpuTrbdf2), _P,
            ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(MangoError)]
        lib.mango_gpu_price_american_batch.restype = ctypes.c_int32
        lib.mango_gpu_price_american_batch_shared.argtypes = [
            _P, _P, ctypes.c_uint64, _P, ctypes.c_int32, ctypes.POINTER(MangoGpuTrbdf2), _P,
            ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(MangoError)]
        lib.mango_gpu_price_american_batch_shared.restype = ctypes.c_int32
        lib.mango_gpu_resolve_grid.argtypes = [_P, _P, _P, ctypes.c_int64,
                                               ctypes.POINTER(ctypes.c_int64),
                                               ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(MangoError)]
        lib.mango_gpu_resolve_grid.restype = ctypes.c_int32
        lib.mango_gpu_last_stats.argtypes = [_P, ctypes.POINTER(MangoGpuStats)]
        lib.mango_gpu_last_stats.restype = ctypes.c_int32
        lib.mango_gpu_batch_create.argtypes = [_P, _P, ctypes.c_uint64, _P, ctypes.c_uint64,
                                               ctypes.POINTER(MangoGpuTrbdf2), ctypes.POINTER(_P),
                                               ctypes.POINTER(MangoError)]
        lib.mango_gpu_batch_create.restype = ctypes.c_int32
        lib.mango_gpu_batch_run.argtypes = [_P, ctypes.POINTER(MangoError)]
        lib.mango_gpu_batch_run.restype = ctypes.c_int32
        lib.mango_gpu_batch_value_at.argtypes = [_P, _P, _P, ctypes.c_uint64, _P, ctypes.POINTER(MangoError)]
        lib.mango_gpu_batch_value_at.restype = ctypes.c_int32
        lib.mango_gpu_batch_results.argtypes = [_P, _P, ctypes.POINTER(ctypes.c_uint64),
                                                ctypes.POINTER(MangoError)]
        lib.mango_gpu_batch_results.restype = ctypes.c_int32
        lib.mango_gpu_batch_destroy.argtypes = [_P]
        lib.mango_gpu_batch_destroy.restype = None
        lib.mango_gpu_batch_timings.argtypes = [_P, ctypes.c_int32] + [ctypes.POINTER(ctypes.c_double)] * 3 + [
            ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(MangoError)]
        lib.mango_gpu_batch_timings.restype = ctypes.c_int32
        lib.mango_gpu_context_set_stream.argtypes = [_P, _P]
        lib.mango_gpu_context_set_stream.restype = ctypes.c_int32
        lib.mango_gpu_fp64_probe.argtypes = [_P, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(MangoError)]
        lib.mango_gpu_fp64_probe.restype = ctypes.c_int32
        lib.mango_gpu_solve_iv_batch.argtypes = [_P, _P, ctypes.c_uint64, _P, ctypes.c_uint64,
                                                 ctypes.POINTER(MangoIvConfig), _P,
                                                 ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(MangoError)]
        lib.mango_gpu_solve_iv_batch.restype = ctypes.c_int32
        lib.mango_gpu_solve_iv_batch_method.argtypes = [_P, _P, ctypes.c_uint64, _P, ctypes.c_uint64,
                                                        ctypes.POINTER(MangoIvConfig), ctypes.c_int32, _P,
                                                        ctypes.POINTER(ctypes.c_uint64),
                                                        ctypes.POINTER(MangoError)]
        lib.mango_gpu_solve_iv_batch_method.restype = ctypes.c_int32
        lib.mango_gpu_price_table_sweep.argtypes = [
            _P, _P, ctypes.c_uint64, _P, ctypes.c_uint64, _P, ctypes.c_uint64, _P, ctypes.c_uint64,
            ctypes.c_double, ctypes.c_double, ctypes.c_int32, _P, _P, _P, ctypes.POINTER(ctypes.c_uint64),
            ctypes.POINTER(MangoError)]
        lib.mango_gpu_price_table_sweep.restype = ctypes.c_int32
        lib.mango_gpu_bspline4d_create.argtypes = [_P, _P, _P, _P, ctypes.POINTER(_P), ctypes.POINTER(MangoError)]
        lib.mango_gpu_bspline4d_create.restype = ctypes.c_int32
        lib.mango_gpu_bspline4d_destroy.argtypes = [_P]
        lib.mango_gpu_bspline4d_destroy.restype = None
        lib.mango_gpu_bspline4d_eval.argtypes = [_P, _P, ctypes.c_uint64, _P, ctypes.POINTER(MangoError)]
        lib.mango_gpu_bspline4d_eval.restype = ctypes.c_int32
        lib.mango_gpu_bspline4d_eval_device.argtypes = [_P, _P, ctypes.c_uint64, _P, ctypes.POINTER(MangoError)]
        lib.mango_gpu_bspline4d_eval_device.restype = ctypes.c_int32
        lib.mango_gpu_bspline4d_knots.argtypes = [_P, _P, ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint64)]
        lib.mango_gpu_bspline4d_knots.restype = ctypes.c_int32
        lib.mango_gpu_bspline4d_export.argtypes = [_P, _P, _P, ctypes.c_uint64, _P, ctypes.c_uint64,
                                                   ctypes.POINTER(MangoError)]
        lib.mango_gpu_bspline4d_export.restype = ctypes.c_int32
        lib.mango_gpu_crc64_update.argtypes = [ctypes.c_uint64, ctypes.c_char_p, ctypes.c_uint64]
        lib.mango_gpu_crc64_update.restype = ctypes.c_uint64
        lib.mango_gpu_bspline4d_fit.argtypes = [_P, _P, _P, _P, ctypes.c_double, _P,
                                                ctypes.POINTER(MangoGpuFitStats), ctypes.POINTER(MangoError)]
        lib.mango_gpu_bspline4d_fit.restype = ctypes.c_int32
        lib.mango_gpu_price_table_create.argtypes = [_P, _P, _P, _P, ctypes.c_double, ctypes.c_double,
                                                     ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(_P),
                                                     ctypes.POINTER(MangoError)]
        lib.mango_gpu_price_table_create.restype = ctypes.c_int32
        lib.mango_gpu_price_table_build.argtypes = [
            _P, _P, ctypes.c_uint64, _P, ctypes.c_uint64, _P, ctypes.c_uint64, _P, ctypes.c_uint64,
            ctypes.c_double, ctypes.c_double, ctypes.c_int32, _P, ctypes.c_int32, ctypes.c_double,
            ctypes.POINTER(_P), ctypes.POINTER(MangoGpuFitStats), ctypes.POINTER(ctypes.c_uint64),
            ctypes.POINTER(MangoError)]
        lib.mango_gpu_price_table_build.restype = ctypes.c_int32
        lib.mango_gpu_price_table_build_ex.argtypes = \
            lib.mango_gpu_price_table_build.argtypes[:15] + [ctypes.c_double] + \
            lib.mango_gpu_price_table_build.argtypes[15:18] + [_P] + \
            lib.mango_gpu_price_table_build.argtypes[18:]
        lib.mango_gpu_price_table_build_ex.restype = ctypes.c_int32
        lib.mango_gpu_eep_decompose.argtypes = [_P, _P, ctypes.c_uint64, _P, ctypes.c_uint64, _P, ctypes.c_uint64,
                                                _P, ctypes.c_uint64, ctypes.c_double, ctypes.c_double,
                                                ctypes.c_int32, _P, ctypes.POINTER(MangoError)]
        lib.mango_gpu_eep_decompose.restype = ctypes.c_int32
        lib.mango_gpu_price_table_destroy.argtypes = [_P]
        lib.mango_gpu_price_table_destroy.restype = None
        lib.mango_gpu_price_table_spline.argtypes = [_P]
        lib.mango_gpu_price_table_spline.restype = _P
        lib.mango_gpu_price_table_info.argtypes = [_P, ctypes.POINTER(ctypes.c_double),
                                                   ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int32),
                                                   ctypes.POINTER(ctypes.c_int32), _P]
        lib.mango_gpu_price_table_info.restype = ctypes.c_int32
        lib.mango_gpu_price_table_price.argtypes = [_P, _P, ctypes.c_uint64, _P, ctypes.POINTER(MangoError)]
        lib.mango_gpu_price_table_price.restype = ctypes.c_int32
        lib.mango_gpu_price_table_price_device.argtypes = [_P, _P, ctypes.c_uint64, _P, ctypes.POINTER(MangoError)]
        lib.mango_gpu_price_table_price_device.restype = ctypes.c_int32
        lib.mango_gpu_price_table_vega.argtypes = [_P, _P, ctypes.c_uint64, _P, ctypes.POINTER(MangoError)]
        lib.mango_gpu_price_table_vega.restype = ctypes.c_int32
        lib.mango_gpu_price_table_greeks.argtypes = [_P, _P, ctypes.c_uint64, _P, _P, ctypes.POINTER(MangoError)]
        lib.mango_gpu_price_table_greeks.restype = ctypes.c_int32
        lib.mango_gpu_price_table_iv_batch.argtypes = [_P, ctypes.POINTER(MangoInterpSolverConfig), _P,
                                                       ctypes.c_uint64, _P, ctypes.POINTER(ctypes.c_uint64),
                                                       ctypes.POINTER(MangoError)]
        lib.mango_gpu_price_table_iv_batch.restype = ctypes.c_int32
        lib.mango_gpu_price_table_iv_batch_device.argtypes = [_P, ctypes.POINTER(MangoInterpSolverConfig), _P,
                                                              ctypes.c_uint64, _P, ctypes.POINTER(MangoError)]
        lib.mango_gpu_price_table_iv_batch_device.restype = ctypes.c_int32
        lib.mango_gpu_price_american_greeks_batch.argtypes = [
            _P, _P, ctypes.c_uint64, _P, ctypes.c_uint64, ctypes.c_double, _P,
            ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(MangoError)]
        lib.mango_gpu_price_american_greeks_batch.restype = ctypes.c_int32
        lib.mango_gpu_price_american_tangent_batch.argtypes = [
            _P, _P, ctypes.c_uint64, _P, ctypes.c_uint64, _P, ctypes.POINTER(ctypes.c_uint64),
            ctypes.POINTER(MangoError)]
        lib.mango_gpu_price_american_tangent_batch.restype = ctypes.c_int32
        lib.mango_gpu_price_american_vega_batch.argtypes = \
            lib.mango_gpu_price_american_tangent_batch.argtypes
        lib.mango_gpu_price_american_vega_batch.restype = ctypes.c_int32
        lib.mango_gpu_build_info.argtypes = []
        lib.mango_gpu_build_info.restype = ctypes.c_char_p
        _lib = lib
    return _lib


def _ptr(a: Optional[np.ndarray]):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


class OptionType(enum.IntEnum):
    """Reference OptionType; values are the C ABI's (MANGO_CALL=0, MANGO_PUT=1)."""
    CALL = 0
    PUT = 1


@dataclasses.dataclass
class Dividend:
    """Reference Dividend (src/option/option_spec.hpp:158-161): a cash
    amount paid at calendar_time years from the valuation date."""
    calendar_time: float = 0.0
    amount: float = 0.0


class YieldCurve:
    """Reference YieldCurve (src/option/yield_curve.hpp): tenor points
    (tenor, ln D(tenor)) sorted by tenor, the first at t = 0; ln D linear
    between tenors, so the forward rate is constant on each interval."""

    def __init__(self, points):
        self.points = [(float(t), float(ld)) for t, ld in points]

    @staticmethod
    def flat(rate: float) -> "YieldCurve":
        return YieldCurve([(0.0, 0.0), (100.0, -rate * 100.0)])

    @staticmethod
    def from_points(points) -> "YieldCurve":
        pts = sorted(((float(t), float(ld)) for t, ld in points), key=lambda p: p[0])
        if not pts:
            raise ValueError("Empty points vector")
        if pts[0][0] != 0.0:
            raise ValueError("First point must have t=0")
        if abs(pts[0][1]) > 1e-10:
            raise ValueError("log_discount at t=0 must be 0")
        for a, b in zip(pts, pts[1:]):
            if b[0] <= a[0] + 1e-10:
                raise ValueError("Tenors must be strictly increasing")
        return YieldCurve(pts)

    @staticmethod
    def from_discounts(tenors, discounts) -> "YieldCurve":
        if len(tenors) != len(discounts):
            raise ValueError("Tenors and discounts must have same size")
        if any(d <= 0.0 for d in discounts):
            raise ValueError("Discount factors must be positive")
        return YieldCurve.from_points([(t, float(np.log(d))) for t, d in zip(tenors, discounts)])

    def log_discount(self, t: float) -> float:
        p = self.points
        if len(p) < 2 or t <= 0.0:
            return 0.0
        j = next((k for k, q in enumerate(p) if t < q[0]), len(p))
        if j == 0:
            return 0.0
        if j == len(p):
            rate = -(p[-1][1] - p[-2][1]) / (p[-1][0] - p[-2][0])
            return p[-1][1] - rate * (t - p[-1][0])
        a = (t - p[j - 1][0]) / (p[j][0] - p[j - 1][0])
        return p[j - 1][1] + a * (p[j][1] - p[j - 1][1])

    def discount(self, t: float) -> float:
        return float(np.exp(self.log_discount(t)))

    def rate(self, t: float) -> float:
        p = self.points
        if len(p) < 2:
            return 0.0
        j = 0 if t <= 0.0 else next((k for k, q in enumerate(p) if t < q[0]), len(p))
        idx = 0 if j == 0 else (len(p) - 2 if j == len(p) else j - 1)
        return -(p[idx + 1][1] - p[idx][1]) / (p[idx + 1][0] - p[idx][0])

    def zero_rate(self, t: float) -> float:
        return self.rate(0.0) if t <= 0.0 else -self.log_discount(t) / t


@dataclasses.dataclass
class PricingParams:
    """Reference PricingParams (src/option/option_spec.hpp:262-281): rate is
    a constant or a YieldCurve; discrete_dividends a list of Dividend on top
    of the continuous dividend_yield."""
    spot: float = 0.0
    strike: float = 0.0
    maturity: float = 0.0
    rate: object = 0.0
    dividend_yield: float = 0.0
    option_type: OptionType = OptionType.CALL
    volatility: float = 0.0
    discrete_dividends: list = dataclasses.field(default_factory=list)


@dataclasses.dataclass
class PDEGridConfig:
    """Explicit grid: sinh (alpha > 0) or uniform (alpha == 0) over
    [x_min, x_max] in ln(S/K), n_space points, n_time steps
    (src/option/grid_spec_types.hpp:55-59)."""
    x_min: float = -3.0
    x_max: float = 3.0
    n_space: int = 101
    n_time: int = 1000
    alpha: float = 2.0 * float(np.arcsinh(5.0 / np.sqrt(2.0)))


@dataclasses.dataclass
class FixedGrid:
    """The reference's sinh-clustered auto grid pinned to n_space points,
    with n_time steps (estimate_pde_grid with min = max = n_space)."""
    n_space: int = 101
    n_time: int = 498


def pricing_array(spot, strike, maturity, volatility, rate, dividend_yield, is_put) -> np.ndarray:
    """Pack per-option arrays (broadcast) into the C MangoPricingParams layout."""
    cols = np.broadcast_arrays(*(np.asarray(v, dtype=np.float64) for v in
                                 (spot, strike, maturity, volatility, rate, dividend_yield, is_put)))
    n = cols[0].size
    a = np.zeros(n, dtype=PRICING_DTYPE)
    a["spot"], a["strike"], a["maturity"] = cols[0].ravel(), cols[1].ravel(), cols[2].ravel()
    a["volatility"], a["rate_const"], a["dividend_yield"] = cols[3].ravel(), cols[4].ravel(), cols[5].ravel()
    a["option_type"] = np.where(cols[6].ravel() != 0, 1, 0).astype(np.int32)
    return a


class _Records(np.ndarray):
    """PRICING_DTYPE records that own the schedules their pointers reach."""


def attach_schedules(records: np.ndarray, curves=None, dividends=None):
    """Point MangoPricingParams records at yield curves and dividend
    schedules (the C struct's tenor_points / dividends pointers).
    curves[i]: None, a YieldCurve or (k, 2) (tenor, log discount) pairs;
    dividends[i]: None, a list of Dividend or (k, 2) (calendar time, amount)
    pairs.  Returns the buffers the pointers reach: keep them alive while the
    records are in use."""
    n = records.size
    def pairs(v, kind):
        if v is None:
            return np.zeros((0, 2))
        if isinstance(v, YieldCurve):
            return np.asarray(v.points, dtype=np.float64).reshape(-1, 2)
        if kind == "div" and len(v) and isinstance(v[0], Dividend):
            return np.asarray([(d.calendar_time, d.amount) for d in v], dtype=np.float64).reshape(-1, 2)
        return np.asarray(v, dtype=np.float64).reshape(-1, 2)
    keep = []
    for key, cnt, vals, kind in (("tenor_points", "n_tenor_points", curves, "curve"),
                                 ("dividends", "n_dividends", dividends, "div")):
        if vals is None:
            continue
        blocks = [pairs(v, kind) for v in vals]
        if len(blocks) != n:
            raise ValueError(f"{key}: one entry per record required")
        counts = np.array([b.shape[0] for b in blocks], dtype=np.uint64)
        flat = np.ascontiguousarray(np.concatenate(blocks + [np.zeros((1, 2))]), dtype=np.float64)
        offs = np.concatenate([[0], np.cumsum(counts)[:-1]]).astype(np.uint64)
        base = flat.ctypes.data
        records[key] = np.where(counts > 0, base + 16 * offs, 0).astype(np.uint64)
        records[cnt] = counts
        keep.append(flat)
    return keep


def query_array(spot, strike, maturity, rate, dividend_yield, is_put, market_price) -> np.ndarray:
    """Pack per-quote arrays (broadcast) into the C MangoIvQuery layout."""
    cols = np.broadcast_arrays(*(np.asarray(v, dtype=np.float64) for v in
                                 (spot, strike, maturity, rate, dividend_yield, is_put, market_price)))
    n = cols[0].size
    a = np.zeros(n, dtype=IVQUERY_DTYPE)
    a["spot"], a["strike"], a["maturity"] = cols[0].ravel(), cols[1].ravel(), cols[2].ravel()
    a["rate_const"], a["dividend_yield"] = cols[3].ravel(), cols[4].ravel()
    a["option_type"] = np.where(cols[5].ravel() != 0, 1, 0).astype(np.int32)
    a["market_price"] = cols[6].ravel()
    return a


def grid_array(n: int, kind: int = GRID_AUTO, n_space=0, n_time=0, x_min=0.0, x_max=0.0,
               alpha=0.0) -> np.ndarray:
    g = np.zeros(n, dtype=GRID_DTYPE)
    g["kind"] = kind
    g["n_space"] = n_space
    g["n_time"] = n_time
    g["x_min"] = x_min
    g["x_max"] = x_max
    g["alpha"] = alpha
    return g


def _grid_entry(grid) -> np.ndarray:
    if grid is None:
        return grid_array(1, GRID_AUTO)
    if isinstance(grid, FixedGrid):
        return grid_array(1, GRID_FIXED_N, grid.n_space, grid.n_time)
    if isinstance(grid, PDEGridConfig):
        kind = GRID_SINH if grid.alpha > 0 else GRID_UNIFORM
        return grid_array(1, kind, grid.n_space, grid.n_time, grid.x_min, grid.x_max, grid.alpha)
    raise TypeError(f"unsupported grid {grid!r}")


class Engine:
    """One CUDA context of the engine (include/mango_gpu.h MangoGpuContext)."""

    def __init__(self, device: int = 0):
        lib = library()
        self._ctx = _P()
        err = MangoError()
        st = lib.mango_gpu_context_create(device, ctypes.byref(self._ctx), ctypes.byref(err))
        if st != MANGO_OK:
            self._ctx = None
            raise EngineError(f"mango_gpu_context_create: {err.message.decode(errors='replace')}")

    def close(self) -> None:
        if self._ctx:
            library().mango_gpu_context_destroy(self._ctx)
            self._ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def price_arrays(self, params: np.ndarray, grids: Optional[np.ndarray] = None,
                     rannacher: bool = True, gamma: float = 0.0) -> np.ndarray:
        """Batched pricing.  params: PRICING_DTYPE array; grids: GRID_DTYPE array
        of length len(params) or 1 (applied to all) or None (auto grid).
        Returns an OUT_DTYPE array (value, delta, gamma, theta, status, n_space, n_time)."""
        params = np.ascontiguousarray(params, dtype=PRICING_DTYPE)
        n = params.size
        out = np.zeros(n, dtype=OUT_DTYPE)
        stride = 0
        if grids is not None:
            grids = np.ascontiguousarray(grids, dtype=GRID_DTYPE)
            if grids.size == n and n != 1:
                stride = 1
            elif grids.size != 1:
                raise ValueError("grids must have length 1 or len(params)")
        tr = MangoGpuTrbdf2(gamma, 1 if rannacher else 0, 0)
        failed = ctypes.c_uint64()
        err = MangoError()
        st = library().mango_gpu_price_american_batch(
            self._ctx, _ptr(params), n, _ptr(grids), stride, ctypes.byref(tr), _ptr(out),
            ctypes.byref(failed), ctypes.byref(err))
        if st != MANGO_OK:
            raise EngineError(f"mango_gpu_price_american_batch: {err.message.decode(errors='replace')}")
        return out

    def price_shared_arrays(self, params: np.ndarray, custom_grid: Optional[np.ndarray] = None,
                            use_normalized: bool = True, rannacher: bool = True,
                            gamma: float = 0.0):
        """Shared-grid batch (mango_gpu_price_american_batch_shared): the
        normalized chain when use_normalized and the batch is eligible, else
        one grid for the whole batch.  custom_grid: one GRID_DTYPE record
        resolved for the first option of the solve, or None for the
        batch-estimated grid.  Returns (OUT_DTYPE records, route) with route
        1 for the chain, 0 for the regular shared grid."""
        params = np.ascontiguousarray(params, dtype=PRICING_DTYPE)
        n = params.size
        out = np.zeros(n, dtype=OUT_DTYPE)
        if custom_grid is not None:
            custom_grid = np.ascontiguousarray(custom_grid, dtype=GRID_DTYPE)
            if custom_grid.size != 1:
                raise ValueError("custom_grid must be a single grid record")
        tr = MangoGpuTrbdf2(gamma, 1 if rannacher else 0, 0)
        failed = ctypes.c_uint64()
        route = ctypes.c_int32()
        err = MangoError()
        st = library().mango_gpu_price_american_batch_shared(
            self._ctx, _ptr(params), n, _ptr(custom_grid), 1 if use_normalized else 0, ctypes.byref(tr),
            _ptr(out), ctypes.byref(failed), ctypes.byref(route), ctypes.byref(err))
        if st != MANGO_OK:
            e = EngineError(f"mango_gpu_price_american_batch_shared: {err.message.decode(errors='replace')}")
            e.status = st
            raise e
        return out, int(route.value)

    def solve_iv_arrays(self, queries: np.ndarray, grids: np.ndarray, tol: float = 0.0,
                        max_iter: int = 0, method: int = 0) -> np.ndarray:
        """Batched FDM implied volatility (mango_gpu_solve_iv_batch_method).
        queries: IVQUERY_DTYPE; grids: GRID_DTYPE (length 1 or len(queries)),
        each a volatility-independent grid; method IV_BRENT (the reference's
        Brent), IV_SECANT or IV_NEWTON (Newton on the exact discrete vega).  Returns IVSLOT_DTYPE records."""
        queries = np.ascontiguousarray(queries, dtype=IVQUERY_DTYPE)
        grids = np.ascontiguousarray(grids, dtype=GRID_DTYPE)
        n = queries.size
        stride = 1 if (grids.size == n and n != 1) else 0
        out = np.zeros(n, dtype=IVSLOT_DTYPE)
        cfg = MangoIvConfig(tol, max_iter)
        failed = ctypes.c_uint64()
        err = MangoError()
        st = library().mango_gpu_solve_iv_batch_method(self._ctx, _ptr(queries), n, _ptr(grids), stride,
                                                       ctypes.byref(cfg), int(method), _ptr(out),
                                                       ctypes.byref(failed), ctypes.byref(err))
        if st != MANGO_OK:
            raise EngineError(f"mango_gpu_solve_iv_batch: {err.message.decode(errors='replace')}")
        return out

    def price_table_sweep(self, moneyness, maturity, volatility, rate, K_ref: float = 100.0,
                          dividend_yield: float = 0.0, option_type: int = 1, grid=None):
        """PriceTableBuilderND<4> sweep + extraction (mango_gpu_price_table_sweep).
        Returns (tensor [m][tau][sigma][r] of V/K_ref, slice dims (n_slices x 2),
        failed slice count).  grid: None (GridAccuracyParams{}) or PDEGridConfig."""
        axes = [np.ascontiguousarray(a, dtype=np.float64) for a in (moneyness, maturity, volatility, rate)]
        shape = tuple(a.size for a in axes)
        tensor = np.zeros(shape)
        dims = np.zeros((shape[2] * shape[3], 2), np.int64)
        g = None if grid is None else _grid_entry(grid)
        failed = ctypes.c_uint64()
        err = MangoError()
        st = library().mango_gpu_price_table_sweep(
            self._ctx, _ptr(axes[0]), shape[0], _ptr(axes[1]), shape[1], _ptr(axes[2]), shape[2],
            _ptr(axes[3]), shape[3], K_ref, dividend_yield, int(option_type), _ptr(g), _ptr(tensor),
            _ptr(dims), ctypes.byref(failed), ctypes.byref(err))
        if st != MANGO_OK:
            raise EngineError(f"mango_gpu_price_table_sweep: {err.message.decode(errors='replace')}")
        return tensor, dims, failed.value

    def bspline4d(self, grids, coeffs) -> "BSpline4D":
        return BSpline4D(self, grids, coeffs)

    def bspline4d_fit(self, grids, values, tolerance: float = 0.0):
        """BSplineNDSeparable<double,4>::fit (mango_gpu_bspline4d_fit): the
        coefficients (same shape as values) and per-axis diagnostics.  Raises
        EngineError when a slice fails the residual check."""
        gs = [np.ascontiguousarray(g, dtype=np.float64) for g in grids]
        sizes = np.array([g.size for g in gs], np.int64)
        v = np.ascontiguousarray(values, dtype=np.float64)
        coeffs = np.zeros(v.size)
        stats = MangoGpuFitStats()
        err = MangoError()
        st = library().mango_gpu_bspline4d_fit(self._ctx, _ptr(np.concatenate(gs)), _ptr(sizes), _ptr(v),
                                               tolerance, _ptr(coeffs), ctypes.byref(stats), ctypes.byref(err))
        info = _fit_stats(stats)
        if st != MANGO_OK:
            e = EngineError(err.message.decode(errors="replace"))
            e.status, e.stats = st, info
            raise e
        return coeffs.reshape(v.shape), info

    def eep_decompose(self, moneyness, maturity, volatility, rate, tensor, K_ref: float = 100.0,
                      dividend_yield: float = 0.0, option_type: int = 1) -> np.ndarray:
        """eep_decompose with AnalyticalEEP of a V/K_ref tensor (mango_gpu_eep_decompose)."""
        axes = [np.ascontiguousarray(a, dtype=np.float64) for a in (moneyness, maturity, volatility, rate)]
        t = np.ascontiguousarray(tensor, dtype=np.float64).copy()
        err = MangoError()
        st = library().mango_gpu_eep_decompose(self._ctx, _ptr(axes[0]), axes[0].size, _ptr(axes[1]),
                                               axes[1].size, _ptr(axes[2]), axes[2].size, _ptr(axes[3]),
                                               axes[3].size, K_ref, dividend_yield, int(option_type), _ptr(t),
                                               ctypes.byref(err))
        if st != MANGO_OK:
            raise EngineError(err.message.decode(errors="replace"))
        return t

    def price_table_create(self, grids, coeffs, K_ref: float, dividend_yield: float = 0.0,
                           option_type: int = 1, eep: bool = True) -> "GpuPriceTable":
        """Standard price table over given spline coefficients
        (make_bspline_surface; mango_gpu_price_table_create)."""
        gs = [np.ascontiguousarray(g, dtype=np.float64) for g in grids]
        sizes = np.array([g.size for g in gs], np.int64)
        c = np.ascontiguousarray(coeffs, dtype=np.float64).ravel()
        h = _P()
        err = MangoError()
        st = library().mango_gpu_price_table_create(self._ctx, _ptr(np.concatenate(gs)), _ptr(sizes), _ptr(c),
                                                    K_ref, dividend_yield, int(option_type), int(bool(eep)),
                                                    ctypes.byref(h), ctypes.byref(err))
        if st != MANGO_OK:
            raise EngineError(err.message.decode(errors="replace"))
        return GpuPriceTable(self, h)

    def price_table_build(self, moneyness, maturity, volatility, rate, K_ref: float = 100.0,
                          dividend_yield: float = 0.0, option_type: int = 1, grid=None, eep: bool = True,
                          tolerance: float = 0.0, max_failure_rate: float = 0.0):
        """PriceTableBuilderND<4>::build on the device (mango_gpu_price_table_build_ex):
        sweep, failure check and repair (max_failure_rate as PriceTableConfig's,
        0 = strict), EEP decomposition, fit.  moneyness is log-moneyness.
        Returns (GpuPriceTable, fit diagnostics with the failed and repaired
        counts)."""
        axes = [np.ascontiguousarray(a, dtype=np.float64) for a in (moneyness, maturity, volatility, rate)]
        g = None if grid is None else _grid_entry(grid)
        h = _P()
        stats = MangoGpuFitStats()
        failed = ctypes.c_uint64()
        repaired = (ctypes.c_uint64 * 2)()
        err = MangoError()
        st = library().mango_gpu_price_table_build_ex(
            self._ctx, _ptr(axes[0]), axes[0].size, _ptr(axes[1]), axes[1].size, _ptr(axes[2]), axes[2].size,
            _ptr(axes[3]), axes[3].size, K_ref, dividend_yield, int(option_type), _ptr(g), int(bool(eep)),
            tolerance, float(max_failure_rate), ctypes.byref(h), ctypes.byref(stats), ctypes.byref(failed),
            repaired, ctypes.byref(err))
        if st != MANGO_OK:
            raise EngineError(err.message.decode(errors="replace"))
        info = _fit_stats(stats)
        info["failed_pde_slices"] = int(failed.value)
        info["repaired_slices"] = int(repaired[0])
        info["repaired_points"] = int(repaired[1])
        return GpuPriceTable(self, h), info

    def greeks_arrays(self, params: np.ndarray, grids: Optional[np.ndarray] = None,
                      h_rel: float = 1e-5) -> np.ndarray:
        """Prices, delta/gamma/theta and frozen-grid central differences for
        vega, rho, dividend rho and dV/dK (mango_gpu_price_american_greeks_batch)."""
        params = np.ascontiguousarray(params, dtype=PRICING_DTYPE)
        n = params.size
        stride = 0
        if grids is not None:
            grids = np.ascontiguousarray(grids, dtype=GRID_DTYPE)
            stride = 1 if (grids.size == n and n != 1) else 0
        out = np.zeros(n, dtype=GREEKS_DTYPE)
        failed = ctypes.c_uint64()
        err = MangoError()
        st = library().mango_gpu_price_american_greeks_batch(self._ctx, _ptr(params), n, _ptr(grids), stride,
                                                             h_rel, _ptr(out), ctypes.byref(failed),
                                                             ctypes.byref(err))
        if st != MANGO_OK:
            raise EngineError(err.message.decode(errors="replace"))
        return out

    def tangent_arrays(self, params: np.ndarray, grids: Optional[np.ndarray] = None,
                       vega_only: bool = False) -> np.ndarray:
        """Value, delta and the exact discrete dV/dvolatility, dV/drate,
        dV/ddividend_yield, dV/dK of the march in one forward-mode pass
        (mango_gpu_price_american_tangent_batch); GREEKS_DTYPE records with
        gamma and theta NaN.  vega_only: the volatility direction alone
        (mango_gpu_price_american_vega_batch; rho and dividend_rho NaN)."""
        params = np.ascontiguousarray(params, dtype=PRICING_DTYPE)
        n = params.size
        stride = 0
        if grids is not None:
            grids = np.ascontiguousarray(grids, dtype=GRID_DTYPE)
            stride = 1 if (grids.size == n and n != 1) else 0
        out = np.zeros(n, dtype=GREEKS_DTYPE)
        failed = ctypes.c_uint64()
        err = MangoError()
        fn = (library().mango_gpu_price_american_vega_batch if vega_only
              else library().mango_gpu_price_american_tangent_batch)
        st = fn(self._ctx, _ptr(params), n, _ptr(grids), stride, _ptr(out), ctypes.byref(failed),
                ctypes.byref(err))
        if st != MANGO_OK:
            raise EngineError(err.message.decode(errors="replace"))
        return out

    def set_stream(self, stream_handle: Optional[int]) -> None:
        """Enqueue on a caller's cudaStream_t (e.g. torch.cuda.current_stream().cuda_stream)."""
        library().mango_gpu_context_set_stream(self._ctx, _P(stream_handle) if stream_handle else None)

    def fp64_probe(self) -> float:
        """Measured FP64 FMA throughput of the device, TFLOP/s."""
        v = ctypes.c_double()
        err = MangoError()
        if library().mango_gpu_fp64_probe(self._ctx, ctypes.byref(v), ctypes.byref(err)) != MANGO_OK:
            raise EngineError(err.message.decode(errors="replace"))
        return v.value

    def batch(self, params: np.ndarray, grids: Optional[np.ndarray] = None, rannacher: bool = True,
              gamma: float = 0.0) -> "ResidentBatch":
        return ResidentBatch(self, params, grids, rannacher, gamma)

    def stats(self) -> dict:
        s = MangoGpuStats()
        library().mango_gpu_last_stats(self._ctx, ctypes.byref(s))
        d = {k: getattr(s, k) for k, _ in MangoGpuStats._fields_}
        d["iv_evals"] = list(d["iv_evals"])
        return d


class BSpline4D:
    """Device-resident 4D cubic B-spline surface (mango_gpu_bspline4d_*),
    the counterpart of BSplineND<double,4>."""

    def __init__(self, engine: Engine, grids, coeffs):
        self._engine = engine
        gs = [np.ascontiguousarray(g, dtype=np.float64) for g in grids]
        self.sizes = np.array([g.size for g in gs], np.int64)
        packed = np.concatenate(gs)
        c = np.ascontiguousarray(coeffs, dtype=np.float64).ravel()
        self._s = _P()
        err = MangoError()
        st = library().mango_gpu_bspline4d_create(engine._ctx, _ptr(packed), _ptr(self.sizes), _ptr(c),
                                                  ctypes.byref(self._s), ctypes.byref(err))
        if st != MANGO_OK:
            self._s = None
            raise EngineError(err.message.decode(errors="replace"))

    def eval(self, queries: np.ndarray) -> np.ndarray:
        q = np.ascontiguousarray(queries, dtype=np.float64).reshape(-1, 4)
        out = np.zeros(q.shape[0])
        err = MangoError()
        if library().mango_gpu_bspline4d_eval(self._s, _ptr(q), q.shape[0], _ptr(out), ctypes.byref(err)) != MANGO_OK:
            raise EngineError(err.message.decode(errors="replace"))
        return out

    def eval_device(self, d_queries: int, n: int, d_out: int) -> None:
        err = MangoError()
        if library().mango_gpu_bspline4d_eval_device(self._s, _P(d_queries), n, _P(d_out), ctypes.byref(err)) != MANGO_OK:
            raise EngineError(err.message.decode(errors="replace"))

    def knots(self) -> np.ndarray:
        n = ctypes.c_uint64()
        library().mango_gpu_bspline4d_knots(self._s, None, 0, ctypes.byref(n))
        out = np.zeros(n.value)
        library().mango_gpu_bspline4d_knots(self._s, _ptr(out), n.value, ctypes.byref(n))
        return out

    def close(self):
        if self._s:
            library().mango_gpu_bspline4d_destroy(self._s)
            self._s = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _fit_stats(s: MangoGpuFitStats) -> dict:
    return {"max_residual": list(s.max_residual), "condition": list(s.condition),
            "failed_slices": [int(x) for x in s.failed_slices]}


class GpuPriceTable:
    """Device-resident standard price table (mango_gpu_price_table_*): the
    counterpart of the reference's PriceTable (AnyPriceTable) for the 4D
    B-spline surface with EEP decomposition."""

    surface_type = "bspline"

    def __init__(self, engine: Engine, handle):
        self._engine = engine
        self._t = handle
        K, q = ctypes.c_double(), ctypes.c_double()
        ot, eep = ctypes.c_int32(), ctypes.c_int32()
        b = np.zeros(8)
        library().mango_gpu_price_table_info(self._t, ctypes.byref(K), ctypes.byref(q), ctypes.byref(ot),
                                             ctypes.byref(eep), _ptr(b))
        self.K_ref, self.dividend_yield = K.value, q.value
        self.option_type = OptionType(ot.value)
        self.eep = bool(eep.value)
        self.bounds = b.reshape(4, 2)

    def price_arrays(self, params: np.ndarray) -> np.ndarray:
        """AnyPriceTable::price for PRICING_DTYPE records (no range checks)."""
        params = np.ascontiguousarray(params, dtype=PRICING_DTYPE)
        out = np.zeros(params.size)
        err = MangoError()
        if library().mango_gpu_price_table_price(self._t, _ptr(params), params.size, _ptr(out),
                                                 ctypes.byref(err)) != MANGO_OK:
            raise EngineError(err.message.decode(errors="replace"))
        return out

    def price_device(self, d_params: int, n: int, d_out: int) -> None:
        err = MangoError()
        if library().mango_gpu_price_table_price_device(self._t, _P(d_params), n, _P(d_out),
                                                        ctypes.byref(err)) != MANGO_OK:
            raise EngineError(err.message.decode(errors="replace"))

    def vega_arrays(self, params: np.ndarray) -> np.ndarray:
        """AnyPriceTable::vega for PRICING_DTYPE records (no range checks)."""
        params = np.ascontiguousarray(params, dtype=PRICING_DTYPE)
        out = np.zeros(params.size)
        err = MangoError()
        if library().mango_gpu_price_table_vega(self._t, _ptr(params), params.size, _ptr(out),
                                                ctypes.byref(err)) != MANGO_OK:
            raise EngineError(err.message.decode(errors="replace"))
        return out

    def vega(self, params: PricingParams) -> float:
        self.validate(params)
        return float(self.vega_arrays(_to_array([params]))[0])

    def greeks_arrays(self, params: np.ndarray) -> Tuple[np.ndarray, np.ndarray]:
        """delta, gamma, theta, rho (columns of an n x 4 array) and per-record
        statuses for PRICING_DTYPE records (mango_gpu_price_table_greeks):
        records that fail validation hold NaN and MANGO_ERR_VALIDATION."""
        params = np.ascontiguousarray(params, dtype=PRICING_DTYPE)
        out = np.zeros((params.size, 4))
        status = np.zeros(params.size, dtype=np.int32)
        err = MangoError()
        rc = library().mango_gpu_price_table_greeks(self._t, _ptr(params), params.size, _ptr(out),
                                                    _ptr(status), ctypes.byref(err))
        if rc not in (MANGO_OK, MANGO_ERR_VALIDATION):
            raise EngineError(err.message.decode(errors="replace"))
        return out, status

    def _greek(self, params: PricingParams, col: int) -> float:
        """greek_call (mango_c_api.cpp:272-300): validate, then one Greek."""
        self.validate(params)
        out, status = self.greeks_arrays(_to_array([params]))
        if status[0] != MANGO_OK:
            raise ValueError("pricing params fail the table's validation")
        return float(out[0, col])

    def delta(self, params: PricingParams) -> float:
        return self._greek(params, 0)

    def gamma(self, params: PricingParams) -> float:
        return self._greek(params, 1)

    def theta(self, params: PricingParams) -> float:
        return self._greek(params, 2)

    def rho(self, params: PricingParams) -> float:
        return self._greek(params, 3)

    def iv_arrays(self, queries: np.ndarray, config: Optional["InterpolatedIVSolverConfig"] = None) -> np.ndarray:
        """InterpolatedIVSolver::solve_batch (mango_gpu_price_table_iv_batch):
        IVQUERY_DTYPE in, IVSLOT_DTYPE out."""
        queries = np.ascontiguousarray(queries, dtype=IVQUERY_DTYPE)
        out = np.zeros(queries.size, dtype=IVSLOT_DTYPE)
        cfg = None if config is None else ctypes.byref(config._c())
        failed = ctypes.c_uint64()
        err = MangoError()
        if library().mango_gpu_price_table_iv_batch(self._t, cfg, _ptr(queries), queries.size, _ptr(out),
                                                    ctypes.byref(failed), ctypes.byref(err)) != MANGO_OK:
            raise EngineError(err.message.decode(errors="replace"))
        return out

    def iv_device(self, d_queries: int, n: int, d_slots: int,
                  config: Optional["InterpolatedIVSolverConfig"] = None) -> None:
        cfg = None if config is None else ctypes.byref(config._c())
        err = MangoError()
        if library().mango_gpu_price_table_iv_batch_device(self._t, cfg, _P(d_queries), n, _P(d_slots),
                                                           ctypes.byref(err)) != MANGO_OK:
            raise EngineError(err.message.decode(errors="replace"))

    def make_iv_solver(self, solver_config: Optional["InterpolatedIVSolverConfig"] = None):
        """PriceTable.make_iv_solver of the reference's bindings."""
        return InterpolatedIVSolver(self, solver_config)

    def validate(self, p: PricingParams) -> None:
        """AnyPriceTable::validate_pricing_params (price_table_factory.cpp:700-744)."""
        if p.option_type != self.option_type:
            raise ValueError("option type does not match the table")
        if abs(p.dividend_yield - self.dividend_yield) > 1e-10:
            raise ValueError("dividend yield does not match the table")
        coords = (np.log(p.spot / p.strike), p.maturity, p.volatility, p.rate)
        for d, x in enumerate(coords):
            if x < self.bounds[d, 0] or x > self.bounds[d, 1]:
                raise ValueError(f"axis {d} value {x} outside the table")

    def price(self, params: PricingParams) -> float:
        """PriceTable.price of the reference's bindings: validate, then price."""
        self.validate(params)
        return float(self.price_arrays(_to_array([params]))[0])

    def spline_knots(self) -> np.ndarray:
        """The spline's packed clamped knots (n_d + 4 per axis)."""
        s = library().mango_gpu_price_table_spline(self._t)
        n = ctypes.c_uint64()
        library().mango_gpu_bspline4d_knots(s, None, 0, ctypes.byref(n))
        out = np.zeros(n.value)
        library().mango_gpu_bspline4d_knots(s, _ptr(out), n.value, ctypes.byref(n))
        return out

    def to_data(self) -> "PriceTableData":
        """to_data: the reference's PriceTableData of this table."""
        return to_data(self)

    def save(self, path, compression: str = "zstd") -> None:
        """write_parquet(to_data(table), path): the reference's Parquet file."""
        write_parquet(to_data(self), path, compression)

    def spline_eval(self, queries: np.ndarray) -> np.ndarray:
        q = np.ascontiguousarray(queries, dtype=np.float64).reshape(-1, 4)
        out = np.zeros(q.shape[0])
        err = MangoError()
        s = library().mango_gpu_price_table_spline(self._t)
        if library().mango_gpu_bspline4d_eval(s, _ptr(q), q.shape[0], _ptr(out), ctypes.byref(err)) != MANGO_OK:
            raise EngineError(err.message.decode(errors="replace"))
        return out

    def close(self):
        if self._t:
            library().mango_gpu_price_table_destroy(self._t)
            self._t = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


@dataclasses.dataclass
class InterpolatedIVSolverConfig:
    """Reference InterpolatedIVSolverConfig (src/option/interpolated_iv_solver.hpp:44-57)."""
    max_iter: int = 50
    tolerance: float = 1e-6
    sigma_min: float = 0.01
    sigma_max: float = 3.0
    vega_threshold: float = 1e-4

    def _c(self) -> MangoInterpSolverConfig:
        return MangoInterpSolverConfig(self.max_iter, self.tolerance, self.sigma_min, self.sigma_max,
                                       self.vega_threshold)


class InterpolatedIVSolver:
    """Reference InterpolatedIVSolver on a GPU price table: all quotes of
    solve_batch solved together on the device."""

    def __init__(self, table: "GpuPriceTable", config: Optional[InterpolatedIVSolverConfig] = None):
        self.table = table
        self.config = config or InterpolatedIVSolverConfig()

    def solve_batch(self, queries) -> "BatchIVResult":
        qs = list(queries)
        if any(isinstance(q.rate, YieldCurve) or getattr(q, "discrete_dividends", None) for q in qs):
            raise ValueError("the interpolated IV solver takes constant rates and continuous dividend yields")
        arr = query_array([q.spot for q in qs], [q.strike for q in qs], [q.maturity for q in qs],
                          [q.rate for q in qs], [q.dividend_yield for q in qs],
                          [int(q.option_type == OptionType.PUT) for q in qs], [q.market_price for q in qs])
        out = self.table.iv_arrays(arr, self.config)
        res = []
        for row in out:
            if row["status"] == MANGO_OK:
                res.append(IVSuccess(float(row["implied_vol"]), int(row["iterations"]), float(row["final_error"])))
            else:
                res.append(IVError(int(row["status"]), int(row["iterations"]), float(row["final_error"])))
        return BatchIVResult(res, int(np.count_nonzero(out["status"])))

    def solve(self, query):
        r = self.solve_batch([query]).results[0]
        if isinstance(r, IVError):
            raise r
        return r


@dataclasses.dataclass
class IVGrid:
    """Reference IVGrid (moneyness S/K, volatility and rate axes)."""
    moneyness: Sequence[float]
    vol: Sequence[float]
    rate: Sequence[float]


@dataclasses.dataclass
class BSplineBackend:
    """Reference BSplineBackend (maturity axis)."""
    maturity_grid: Sequence[float]


@dataclasses.dataclass
class IVSolverFactoryConfig:
    """Reference IVSolverFactoryConfig for the standard B-spline path
    (continuous dividend yield)."""
    option_type: OptionType = OptionType.PUT
    spot: float = 100.0
    dividend_yield: float = 0.0
    grid: Optional[IVGrid] = None
    backend: Optional[BSplineBackend] = None


def make_interpolated_iv_solver(config: IVSolverFactoryConfig, engine: Optional[Engine] = None,
                                solver_config: Optional[InterpolatedIVSolverConfig] = None) -> InterpolatedIVSolver:
    """make_interpolated_iv_solver, standard B-spline path: build the table,
    then wrap it in an interpolated IV solver."""
    return make_price_table(config, engine).make_iv_solver(solver_config)


def make_price_table(config: IVSolverFactoryConfig, engine: Optional[Engine] = None) -> GpuPriceTable:
    """make_price_table, standard B-spline path (price_table_factory.cpp:
    294-325): log-moneyness from the moneyness axis, K_ref = spot, the default
    accuracy PDE grid, EEP decomposition.  Axes are sorted and de-duplicated
    as PriceTableBuilder::from_vectors does."""
    if config.grid is None or config.backend is None:
        raise ValueError("config needs grid and backend")
    m = np.asarray(config.grid.moneyness, dtype=np.float64)
    if (m <= 0).any():
        raise ValueError("moneyness must be positive")
    axes = [np.unique(np.log(m)), np.unique(np.asarray(config.backend.maturity_grid, dtype=np.float64)),
            np.unique(np.asarray(config.grid.vol, dtype=np.float64)),
            np.unique(np.asarray(config.grid.rate, dtype=np.float64))]
    eng = engine or default_engine()
    table, _ = eng.price_table_build(*axes, K_ref=config.spot, dividend_yield=config.dividend_yield,
                                     option_type=int(config.option_type), grid=None, eep=True)
    return table


class ResidentBatch:
    """A batch uploaded once and re-run on the device (mango_gpu_batch_*)."""

    def __init__(self, engine: Engine, params: np.ndarray, grids: Optional[np.ndarray], rannacher: bool,
                 gamma: float):
        self._engine = engine
        self.params = np.ascontiguousarray(params, dtype=PRICING_DTYPE)
        n = self.params.size
        stride = 0
        if grids is not None:
            grids = np.ascontiguousarray(grids, dtype=GRID_DTYPE)
            stride = 1 if (grids.size == n and n != 1) else 0
        self._grids = grids
        self._b = _P()
        err = MangoError()
        tr = MangoGpuTrbdf2(gamma, 1 if rannacher else 0, 0)
        st = library().mango_gpu_batch_create(engine._ctx, _ptr(self.params), n, _ptr(grids), stride,
                                              ctypes.byref(tr), ctypes.byref(self._b), ctypes.byref(err))
        if st != MANGO_OK:
            self._b = None
            raise EngineError(err.message.decode(errors="replace"))
        self.n = n

    def run(self) -> None:
        err = MangoError()
        if library().mango_gpu_batch_run(self._b, ctypes.byref(err)) != MANGO_OK:
            raise EngineError(err.message.decode(errors="replace"))

    def results(self) -> np.ndarray:
        out = np.zeros(self.n, dtype=OUT_DTYPE)
        failed = ctypes.c_uint64()
        err = MangoError()
        if library().mango_gpu_batch_results(self._b, _ptr(out), ctypes.byref(failed), ctypes.byref(err)) != MANGO_OK:
            raise EngineError(err.message.decode(errors="replace"))
        return out

    def value_at(self, slots, spots) -> np.ndarray:
        """AmericanOptionResult::value_at (mango_american_value_at) and the
        functionals at other spots: the option in slots[j] read at spots[j]
        with its own strike; returns (n, 4) value, delta, gamma, theta."""
        sl = np.ascontiguousarray(np.broadcast_to(np.asarray(slots, np.uint64), np.shape(spots)), np.uint64).ravel()
        sp = np.ascontiguousarray(spots, dtype=np.float64).ravel()
        out = np.zeros((sp.size, 4))
        err = MangoError()
        if library().mango_gpu_batch_value_at(self._b, _ptr(sl), _ptr(sp), sp.size, _ptr(out),
                                              ctypes.byref(err)) != MANGO_OK:
            raise EngineError(err.message.decode(errors="replace"))
        return out

    def timings(self, reset: bool = False) -> dict:
        a, m, o = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        runs = ctypes.c_int64()
        err = MangoError()
        if library().mango_gpu_batch_timings(self._b, 1 if reset else 0, ctypes.byref(a), ctypes.byref(m),
                                             ctypes.byref(o), ctypes.byref(runs), ctypes.byref(err)) != MANGO_OK:
            raise EngineError(err.message.decode(errors="replace"))
        return {"prep_ms": a.value, "march_ms": m.value, "outputs_ms": o.value, "runs": runs.value}

    def close(self) -> None:
        if self._b:
            library().mango_gpu_batch_destroy(self._b)
            self._b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def resolve_grid(params: np.ndarray, grid=None):
    """Host-only: the grid (x, n_time) the engine uses for one option."""
    params = np.ascontiguousarray(params, dtype=PRICING_DTYPE).reshape(1)
    g = grid if isinstance(grid, np.ndarray) else _grid_entry(grid)
    g = np.ascontiguousarray(g, dtype=GRID_DTYPE).reshape(1)
    x = np.zeros(1 << 16)
    n = ctypes.c_int64()
    nt = ctypes.c_int64()
    err = MangoError()
    st = library().mango_gpu_resolve_grid(_ptr(params), _ptr(g), _ptr(x), x.size, ctypes.byref(n),
                                          ctypes.byref(nt), ctypes.byref(err))
    if st != MANGO_OK:
        raise ValueError(err.message.decode(errors="replace"))
    return x[: n.value].copy(), nt.value


_default_engine: Optional[Engine] = None


def default_engine() -> Engine:
    global _default_engine
    if _default_engine is None:
        _default_engine = Engine(0)
    return _default_engine


def _to_array(params: Sequence[PricingParams]) -> np.ndarray:
    curve = [p.rate if isinstance(p.rate, YieldCurve) else None for p in params]
    divs = [p.discrete_dividends or None for p in params]
    a = pricing_array([p.spot for p in params], [p.strike for p in params],
                      [p.maturity for p in params], [p.volatility for p in params],
                      [0.0 if c is not None else p.rate for c, p in zip(curve, params)],
                      [p.dividend_yield for p in params],
                      [int(p.option_type == OptionType.PUT) for p in params])
    if not any(c is not None for c in curve) and not any(divs):
        return a
    rec = a.view(_Records)
    rec._keep = attach_schedules(rec, curve if any(c is not None for c in curve) else None,
                                 divs if any(divs) else None)
    return rec


@dataclasses.dataclass
class AmericanOptionResult:
    """Reference AmericanOptionResult accessors (american_option_result.hpp)."""
    _row: np.void
    params: PricingParams

    def value(self) -> float:
        return float(self._row["value"])

    def delta(self) -> float:
        return float(self._row["delta"])

    def gamma(self) -> float:
        return float(self._row["gamma"])

    def theta(self) -> float:
        return float(self._row["theta"])

    @property
    def n_space(self) -> int:
        return int(self._row["n_space"])

    @property
    def n_time(self) -> int:
        return int(self._row["n_time"])


class SolverError(RuntimeError):
    def __init__(self, status: int, message: str = ""):
        super().__init__(message or f"status {status}")
        self.status = status


def american_option_price(params: PricingParams, grid=None) -> AmericanOptionResult:
    """Single option (mango_bindings.cpp:580; american_option.cpp:440-450)."""
    out = default_engine().price_arrays(_to_array([params]), _grid_entry(grid))
    if out[0]["status"] != MANGO_OK:
        raise SolverError(int(out[0]["status"]))
    return AmericanOptionResult(out[0], params)


def american_option_price_autograd(spot, strike, maturity, volatility, rate, dividend_yield, is_put,
                                   grid=None, engine: Optional[Engine] = None):
    """Differentiable American prices for torch: the values of a batch of
    options (mango_gpu_price_american_tangent_batch), with gradients with
    respect to volatility, rate, dividend_yield and strike from the exact
    discrete derivatives of the march (the same grid; the active obstacle
    set frozen).  Arguments are scalars or 1-D tensors / arrays broadcast to
    one length; any of volatility, rate, dividend_yield and strike may be a
    tensor that requires grad.  The result is a float64 tensor on the device
    of the first tensor argument.  A failed option raises SolverError.

    This is the torch counterpart of the reference's american_option_price
    binding (src/python/mango_bindings.cpp:580) for a batch, with backward
    grad_output * [dV/dsigma, dV/dr, dV/dq, dV/dK]."""
    import torch

    class _AmericanPrice(torch.autograd.Function):
        @staticmethod
        def forward(ctx, sig, r, q, k, S, T, put):
            eng = engine or default_engine()
            host = [np.ascontiguousarray(t.detach().cpu().numpy(), np.float64) for t in (S, k, T, sig, r, q)]
            params = pricing_array(*host, np.ascontiguousarray(put.detach().cpu().numpy(), np.int32))
            out = eng.tangent_arrays(params, _grid_entry(grid) if not isinstance(grid, np.ndarray) else grid)
            bad = np.nonzero(out["status"] != MANGO_OK)[0]
            if bad.size:
                raise SolverError(int(out["status"][bad[0]]))
            dev = sig.device
            ctx.save_for_backward(*(torch.from_numpy(np.ascontiguousarray(out[f])).to(dev)
                                    for f in ("vega", "rho", "dividend_rho", "dstrike")))
            return torch.from_numpy(np.ascontiguousarray(out["value"])).to(dev)

        @staticmethod
        def backward(ctx, g):
            vega, rho, drho, dk = ctx.saved_tensors
            return g * vega, g * rho, g * drho, g * dk, None, None, None

    args = [spot, strike, maturity, volatility, rate, dividend_yield, is_put]
    dev = next((a.device for a in args if isinstance(a, torch.Tensor)), torch.device("cpu"))
    ts = [a if isinstance(a, torch.Tensor) else torch.as_tensor(np.asarray(a, np.float64), device=dev)
          for a in args]
    n = max(t.numel() for t in ts)
    S, K, T, sig, r, q, put = (t.to(torch.float64).reshape(-1).expand(n) if t.numel() == 1
                               else t.to(torch.float64).reshape(-1) for t in ts)
    return _AmericanPrice.apply(sig, r, q, K, S, T, put)


@dataclasses.dataclass
class BatchAmericanOptionResult:
    results: list
    failed_count: int


class BatchAmericanOptionSolver:
    """Reference BatchAmericanOptionSolver (american_option_batch.hpp:114).
    solve_batch without a shared grid prices every option on its own grid in
    one GPU batch; with use_shared_grid it takes the reference's routing
    (american_option_batch.cpp:272-302): the normalized chain when
    use_normalized (default on) and the batch is eligible, else one grid for
    the whole batch.  A custom_grid is resolved once, for the first option,
    as the reference's solve_regular_batch does."""

    def __init__(self, engine: Optional[Engine] = None):
        self._engine = engine
        self._grid = None
        self._use_normalized = True
        self._rannacher = True
        self._gamma = 0.0
        self.last_route = None

    def set_grid(self, grid) -> None:
        """Per-option grid for batches without a shared or custom grid."""
        self._grid = grid

    def set_use_normalized(self, enable: bool) -> "BatchAmericanOptionSolver":
        self._use_normalized = bool(enable)
        return self

    def use_normalized(self) -> bool:
        return self._use_normalized

    def set_trbdf2_config(self, gamma: float = 0.0, rannacher_startup: bool = True) -> "BatchAmericanOptionSolver":
        self._gamma = float(gamma)
        self._rannacher = bool(rannacher_startup)
        return self

    def solve_batch(self, params: Iterable[PricingParams], use_shared_grid: bool = False,
                    custom_grid=None) -> BatchAmericanOptionResult:
        plist = list(params)
        eng = self._engine or default_engine()
        arr = _to_array(plist)
        if use_shared_grid or custom_grid is not None:
            # Without a shared grid, a custom grid resolved for the first
            # option serves every option: the shared route minus the chain.
            cg = None if custom_grid is None else _grid_entry(custom_grid)
            out, self.last_route = eng.price_shared_arrays(
                arr, cg, use_normalized=self._use_normalized and use_shared_grid,
                rannacher=self._rannacher, gamma=self._gamma)
        else:
            out = eng.price_arrays(arr, _grid_entry(self._grid), rannacher=self._rannacher, gamma=self._gamma)
            self.last_route = None
        results = []
        for row, p in zip(out, plist):
            if row["status"] == MANGO_OK:
                results.append(AmericanOptionResult(row, p))
            else:
                results.append(SolverError(int(row["status"])))
        return BatchAmericanOptionResult(results, int(np.count_nonzero(out["status"])))


@dataclasses.dataclass
class IVQuery:
    """Reference IVQuery (src/option/option_spec.hpp:208-228): rate is a
    constant or a YieldCurve; discrete_dividends a list of Dividend."""
    spot: float = 0.0
    strike: float = 0.0
    maturity: float = 0.0
    rate: object = 0.0
    dividend_yield: float = 0.0
    option_type: OptionType = OptionType.CALL
    market_price: float = 0.0
    discrete_dividends: list = dataclasses.field(default_factory=list)


@dataclasses.dataclass
class IVSuccess:
    implied_vol: float
    iterations: int
    final_error: float
    vega: Optional[float] = None


class IVError(RuntimeError):
    def __init__(self, status: int, iterations: int = 0, final_error: float = float("nan")):
        super().__init__(f"status {status}")
        self.status = status
        self.iterations = iterations
        self.final_error = final_error


@dataclasses.dataclass
class BatchIVResult:
    results: list
    failed_count: int


@dataclasses.dataclass
class IVSolverConfig:
    """Reference IVSolverConfig (src/option/iv_solver.hpp:48-68); `grid` must
    not depend on the unknown volatility: a PDEGridConfig, or FixedGrid
    sized at `grid_vol`."""
    grid: object = None
    grid_vol: float = 0.0
    brent_tol_abs: float = 1e-6
    max_iter: int = 100
    method: int = 0  # IV_BRENT (the reference's root finder), IV_SECANT or IV_NEWTON


class IVSolver:
    """Reference IVSolver (src/option/iv_solver.hpp:134): Brent FDM IV, all
    quotes of solve_batch solved together on the GPU."""

    def __init__(self, config: Optional[IVSolverConfig] = None, engine: Optional[Engine] = None):
        self.config = config or IVSolverConfig(grid=PDEGridConfig())
        self._engine = engine

    def _grid(self):
        g = self.config.grid
        if isinstance(g, FixedGrid):
            if not self.config.grid_vol > 0:
                raise ValueError("FixedGrid for IV needs IVSolverConfig.grid_vol > 0")
            return grid_array(1, GRID_FIXED_N_AT_VOL, g.n_space, g.n_time, alpha=self.config.grid_vol)
        if isinstance(g, PDEGridConfig):
            return _grid_entry(g)
        raise ValueError("IVSolver on the GPU needs a fixed grid (PDEGridConfig or FixedGrid)")

    def solve_batch(self, queries) -> BatchIVResult:
        qs = list(queries)
        curves = [q.rate if isinstance(q.rate, YieldCurve) else None for q in qs]
        divs = [q.discrete_dividends or None for q in qs]
        arr = query_array([q.spot for q in qs], [q.strike for q in qs], [q.maturity for q in qs],
                          [0.0 if c is not None else q.rate for c, q in zip(curves, qs)],
                          [q.dividend_yield for q in qs],
                          [int(q.option_type == OptionType.PUT) for q in qs], [q.market_price for q in qs])
        keep = attach_schedules(arr, curves if any(c is not None for c in curves) else None,
                                divs if any(divs) else None)
        eng = self._engine or default_engine()
        out = eng.solve_iv_arrays(arr, self._grid(), self.config.brent_tol_abs, self.config.max_iter,
                                  self.config.method)
        del keep
        res = []
        for row in out:
            if row["status"] == MANGO_OK:
                res.append(IVSuccess(float(row["implied_vol"]), int(row["iterations"]), float(row["final_error"])))
            else:
                res.append(IVError(int(row["status"]), int(row["iterations"]), float(row["final_error"])))
        return BatchIVResult(res, int(np.count_nonzero(out["status"])))

    def solve(self, query):
        r = self.solve_batch([query]).results[0]
        if isinstance(r, IVError):
            raise r
        return r


from .persistence import (PriceTableData, PriceTableSegment, SerializationError,  # noqa: E402
                          from_data, read_parquet, to_data, write_parquet)


def load_price_table(path, engine: Optional[Engine] = None) -> "GpuPriceTable":
    """read_parquet + from_data: a saved bspline_4d table on the device."""
    return from_data(read_parquet(path), engine)
