#!/usr/bin/env python
"""Benchmark: batched American-option pricing, options/s at 101 x 498, FP64.

Workload (one "step" = one pass of the hot path over the batch):
  65,536 American options, puts and calls alternating, spot 100,
  K~U[80,120], T~U[0.1,2], sigma~U[0.1,0.5], r~U[0,0.08], q~U[0,0.04]
  (seeded), each on the reference's sinh-clustered grid pinned to
  101 space points x 498 time steps (estimate_pde_grid with
  min = max = 101, PDEGridConfig n_time = 498).  Synthetic data.

  value : options/s with the batch resident in device memory (setup +
          march + outputs kernels per step; ~1.5 GB of per-option state,
          far above the 129 MB L2, so no flush is needed between steps).
  e2e   : options/s through the C ABI call mango_gpu_price_american_batch
          with host arrays: validation, grid generation, H2D, kernels, D2H.
  roofline: the march kernel against the FP64 FMA rate measured live on the
          same GPU (mango_gpu_fp64_probe).
  cpu_baseline: the oracle's C restatement of the reference's per-option
          loop (OpenMP over all host cores) on a bounded sample.

--impl reference: the reference's CPU implementation of the same path on
the host cores (the C restatement; the reference's own build is not
available on the GPU host), same metric and config.

Multi-GPU (--gpus N under torchrun): replicas only -- every option is
independent, each rank prices its own copy of the batch, no collective on
the data path; value = options priced by all ranks / max rank time.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import pathlib
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

N_OPTIONS = 65536
NX, NT = 101, 498
METRIC = "options/s @101x498 FP64 (batched American pricing with value/delta/gamma/theta)"


def make_workload(pkg, n, seed=20251203, uneven=False):
    rng = np.random.default_rng(seed)
    S = np.full(n, 100.0)
    K = rng.uniform(80, 120, n)
    T = rng.uniform(0.1, 2.0, n)
    sig = rng.uniform(0.1, 0.5, n)
    r = rng.uniform(0.0, 0.08, n)
    q = rng.uniform(0.0, 0.04, n)
    put = (np.arange(n) % 2 == 0).astype(np.int32)
    params = pkg.pricing_array(S, K, T, sig, r, q, put)
    if uneven:
        nx = rng.integers(51, 402, n)
        nt = rng.integers(100, 1001, n)
        grids = pkg.grid_array(n, pkg.GRID_FIXED_N, nx, nt)
    else:
        grids = pkg.grid_array(1, pkg.GRID_FIXED_N, NX, NT)
    return params, grids, (S, K, T, sig, r, q, put)


def measured_hbm_gbs():
    """Measured HBM copy bandwidth of the GB300s (MEASURED_PEAKS.json), or None."""
    f = ROOT / "MEASURED_PEAKS.json"
    try:
        return float(json.loads(f.read_text())["hbm_gbs"])
    except Exception:
        return None


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def reduce_max(x, ws):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def load_oracle():
    """The CPU implementation of the reference's path for the baseline legs:
    the reference's own build when it is loadable here, else the C
    restatement (the GPU host never has the reference tree)."""
    import importlib.util
    ref = ROOT / "oracle" / "_ref" / "libmango_ref.so"
    try:
        if ref.exists():
            return ctypes.CDLL(str(ref)), "reference", "ref_price_batch"
    except OSError:
        pass
    spec = importlib.util.spec_from_file_location("_b", ROOT / "mango-option_gb300" / "build.py")
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    return ctypes.CDLL(str(b.build_oracle())), "port", "mo_price_batch"


def load_port():
    """The C restatement of the reference's path (oracle/), built in place."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("_b", ROOT / "mango-option_gb300" / "build.py")
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    return ctypes.CDLL(str(b.build_oracle()))


def cpu_price(lib, fn, cols, nx, nt, threads):
    S, K, T, sig, r, q, put = (np.ascontiguousarray(c) for c in cols)
    n = len(S)
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    nxa = np.full(n, nx, np.int64)
    nta = np.full(n, nt, np.int64)
    out = np.zeros(4 * n)
    st = np.zeros(n, np.int32)
    t0 = time.perf_counter()
    getattr(lib, fn)(ctypes.c_int64(n), P(S), P(K), P(T), P(sig), P(r), P(q), P(put.astype(np.int32)), P(nxa),
                     P(nta), ctypes.c_int32(1), ctypes.c_int32(threads), P(out), None, P(st))
    return time.perf_counter() - t0, out.reshape(n, 4)


def cpu_sample(lib, fn, cols, threads, target_s=2.0):
    """Options/s of the CPU path on a bounded sample sized to ~target_s wall."""
    m = 64
    while True:
        sub = [c[:m] for c in cols]
        t, _ = cpu_price(lib, fn, sub, NX, NT, threads)
        if t > target_s / 4 or m >= len(cols[0]):
            break
        m = min(len(cols[0]), m * 4)
    return m / t, m, t


def _cpu_threads():
    return os.cpu_count() or 1


def _P(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def cpu_uneven(lib, n=None, target_s=2.0):
    """The uneven-grid workload on the CPU restatement (OpenMP, all host
    cores): options of the 65,536-option batch's distributions, N_x ~
    U{51..401}, N_t ~ U{100..1000}, growing samples until ~target_s."""
    threads = _cpu_threads()
    m = 64
    while True:
        rng = np.random.default_rng(77)
        S = np.full(m, 100.0)
        K, T, sig = rng.uniform(80, 120, m), rng.uniform(0.1, 2.0, m), rng.uniform(0.1, 0.5, m)
        r, q = rng.uniform(0.0, 0.08, m), rng.uniform(0.0, 0.04, m)
        put = (np.arange(m) % 2 == 0).astype(np.int32)
        nx = rng.integers(51, 402, m).astype(np.int64)
        nt = rng.integers(100, 1001, m).astype(np.int64)
        out = np.zeros(4 * m)
        st = np.zeros(m, np.int32)
        t0 = time.perf_counter()
        lib.mo_price_batch(ctypes.c_int64(m), *(_P(np.ascontiguousarray(a)) for a in (S, K, T, sig, r, q)), _P(put),
                           _P(nx), _P(nt), ctypes.c_int32(1), ctypes.c_int32(threads), _P(out), None, _P(st))
        t = time.perf_counter() - t0
        if t > target_s / 4 or m >= 16384:
            break
        m *= 4
    return {"value": m / t, "unit": "options/s", "cores": threads, "kind": "port",
            "sample": f"{m} options of the uneven-grid distributions, {t:.2f} s on {threads} threads"}


def cpu_iv(lib, pkg, target_s=2.0):
    """Brent FDM IV (the reference's IVSolver restated) on quotes of the
    batched-IV distributions, OpenMP over quotes on all host cores."""
    threads = _cpu_threads()
    m = 32
    while True:
        S, K, T, r, q, vt, put, _ = make_iv_workload(pkg, m, seed=4245)
        out4 = np.zeros(4 * m)
        dims = np.zeros(2 * m, np.int64)
        pst = np.zeros(m, np.int32)
        nx = np.full(m, NX, np.int64)
        ntv = np.full(m, NT, np.int64)
        f = [np.ascontiguousarray(a, np.float64) for a in (S, K, T, vt, r, q)]
        lib.mo_price_batch(ctypes.c_int64(m), *(_P(a) for a in f), _P(put), _P(nx), _P(ntv), ctypes.c_int32(1),
                           ctypes.c_int32(threads), _P(out4), _P(dims), _P(pst))
        px = np.ascontiguousarray(out4.reshape(m, 4)[:, 0])
        o3 = np.zeros(3 * m)
        st = np.zeros(m, np.int32)
        g = [np.ascontiguousarray(a, np.float64) for a in (S, K, T, r, q)]
        t0 = time.perf_counter()
        lib.mo_iv_batch(ctypes.c_int64(m), *(_P(a) for a in g), _P(put), _P(px), _P(np.ascontiguousarray(vt)),
                        _P(nx), _P(ntv), ctypes.c_int32(threads), _P(o3), _P(st))
        t = time.perf_counter() - t0
        if t > target_s / 4 or m >= 8192:
            break
        m *= 4
    return {"value": m / t, "unit": "IV/s", "cores": threads, "kind": "port",
            "sample": f"{m} quotes of the batched-IV distributions, Brent on 101x498, {t:.2f} s on {threads} threads"}


def cpu_sweep(lib, slices=16):
    """The table sweep's PDE solves on the CPU restatement, on one core as the
    reference routes them (its per-slice fallback solves the (vol, rate) groups
    one after the other): `slices` of the 200 (vol, rate) solves at
    S = K = 100, T = 2 on 201 points x 1000 steps (the explicit grid's sizes,
    an upper bound of the per-slice grids), scaled to solves/s."""
    sig = np.repeat(TABLE_AXES[2], TABLE_AXES[3].size)[:: 200 // slices][:slices]
    rr = np.tile(TABLE_AXES[3], TABLE_AXES[2].size)[:: 200 // slices][:slices]
    m = sig.size
    out = np.zeros(4 * m)
    st = np.zeros(m, np.int32)
    t0 = time.perf_counter()
    lib.mo_price_batch(ctypes.c_int64(m), _P(np.full(m, 100.0)), _P(np.full(m, 100.0)), _P(np.full(m, 2.0)),
                       _P(np.ascontiguousarray(sig)), _P(np.ascontiguousarray(rr)), _P(np.zeros(m)),
                       _P(np.ones(m, np.int32)), _P(np.full(m, 201, np.int64)), _P(np.full(m, 1000, np.int64)),
                       ctypes.c_int32(1), ctypes.c_int32(1), _P(out), None, _P(st))
    t = time.perf_counter() - t0
    return {"value": m / t, "unit": "PDE solves/s", "cores": 1, "kind": "port",
            "sample": f"{m} of the 200 (vol, rate) solves at 201x1000, {t:.2f} s on 1 thread "
                      "(the reference solves the slices serially)"}


def cpu_query(lib, nq=2_000_000):
    """BSplineND<double,4>::eval restated, OpenMP over queries on all host
    cores, on the same table and query distribution."""
    threads = _cpu_threads()
    sizes = np.array([a.size for a in TABLE_AXES], np.int64)
    grids = np.ascontiguousarray(np.concatenate(TABLE_AXES))
    coeffs = np.random.default_rng(2025).standard_normal(int(np.prod(sizes)))
    rng = np.random.default_rng(7)
    q = np.ascontiguousarray(np.stack([rng.uniform(a[0], a[-1], nq) for a in TABLE_AXES], 1))
    out = np.zeros(nq)
    t0 = time.perf_counter()
    lib.mo_bspline4d_eval(_P(sizes), _P(grids), _P(coeffs), _P(q), ctypes.c_int64(nq), _P(out))
    t = time.perf_counter() - t0
    return {"value": nq / t, "unit": "queries/s", "cores": threads, "kind": "port",
            "sample": f"{nq} queries, {t:.2f} s on {threads} threads"}


def make_iv_workload(pkg, n, seed=4242):
    """Batched-IV workload: true vol~U[0.05,0.8], K/S~U[0.8,1.2], T~U[0.02,2],
    r~U[0,0.08], q~U[0,0.04], puts (3 in 4) and calls, spot 100; each quote
    on the 101 x 498 grid rule sized at its true vol."""
    rng = np.random.default_rng(seed)
    S = np.full(n, 100.0)
    K = S * rng.uniform(0.8, 1.2, n)
    T = rng.uniform(0.02, 2.0, n)
    r = rng.uniform(0.0, 0.08, n)
    q = rng.uniform(0.0, 0.04, n)
    vt = rng.uniform(0.05, 0.8, n)
    put = (np.arange(n) % 4 != 3).astype(np.int32)
    grids = pkg.grid_array(n, pkg.GRID_FIXED_N_AT_VOL, NX, NT, alpha=vt)
    return S, K, T, r, q, vt, put, grids


VEGA_FLOOR = 1e-4  # the reference InterpolatedIVSolver's default vega_threshold


def bench_iv(pkg, eng, n):
    """Batched IV (262,144 quotes): the reference's Brent, the secant and
    Newton (coarse-grid Newton on the exact discrete vega, then the secant on
    the own grid), end to end through
    mango_gpu_solve_iv_batch_method.  The quotes are priced at their true vol
    with the forward-mode march (which also gives the discrete vega at the true
    vol) on each quote's 101 x 498 grid sized at that vol -- the grid the
    synthetic generator used; inverting on the generator's grid makes the
    round trip exact, so |sigma - sigma_true| measures the root finder alone.
    (A caller without the true vol sizes every grid at some other fixed vol;
    the solver's accuracy on its own discrete objective is the same.)

    Accuracy per arm, over the quotes outside two named classes, each counted:
    validation/arbitrage statuses (the price is not a valid American price
    for the quote, e.g. below intrinsic after rounding), and a discrete vega
    at the true vol below VEGA_FLOOR (the volatility barely moves the price,
    so it is not determined to 1e-6 by a price; the reference's
    InterpolatedIVSolver rejects such quotes for the same reason).  A quote
    outside 1e-6 whose returned vol re-prices to within half of what the true
    vol's vega implies, |V(returned) - P| < |vega(true)| |returned - true| / 2,
    has an objective that is flat or not monotone between the two vols (the
    price does not determine the vol there); those are counted as a third
    class, separately from the misses."""
    S, K, T, r, q, vt, put, grids = make_iv_workload(pkg, n)
    truth = eng.tangent_arrays(pkg.pricing_array(S, K, T, vt, r, q, put), grids, vega_only=True)
    px = truth["value"]
    quotes = pkg.query_array(S, K, T, r, q, put, px)
    low_vega = np.abs(truth["vega"]) < VEGA_FLOOR
    res = {"workload": f"{n} American quotes (3/4 puts), true vol~U[0.05,0.8], K/S~U[0.8,1.2], "
                       f"T~U[0.02,2], 101x498 per-quote grids sized at the true vol (the generator's "
                       f"grid), prices from the forward solver",
           "vega_floor": VEGA_FLOOR}
    arms = (("brent", pkg.IV_BRENT, "Brent, the reference iterate sequence"),
            ("secant", pkg.IV_SECANT, "secant from the Black-Scholes IV, Brent fallback"),
            ("newton", pkg.IV_NEWTON, "Newton on the exact discrete vega of a coarse grid, then the secant "
                                      "on the own grid (3e-6 secant stop), k-section and Brent fallback"))
    for name, method, desc in arms:
        # warm the context's buffers with a solve of the same size (steady state of repeated
        # batches; the first solve of a context also page-locks its staging and allocates)
        eng.solve_iv_arrays(quotes, grids, method=method)
        t0 = time.perf_counter()
        out = eng.solve_iv_arrays(quotes, grids, method=method)
        t = time.perf_counter() - t0
        st = eng.stats()
        invalid = np.isin(out["status"], (pkg.MANGO_ERR_VALIDATION, pkg.MANGO_ERR_ARBITRAGE))
        eligible = ~invalid & ~low_vega
        ok = out["status"] == 0
        err = np.abs(out["implied_vol"] - vt)
        within = eligible & ok & (err <= 1e-6)
        miss = eligible & ~within
        other_root = np.zeros(n, bool)
        if miss.any():
            idx = np.nonzero(miss & ok)[0]
            if idx.size:
                sel = lambda a: np.asarray(a)[idx]
                v = eng.price_arrays(pkg.pricing_array(sel(S), sel(K), sel(T), out["implied_vol"][idx], sel(r),
                                                       sel(q), sel(put)), grids[idx])["value"]
                other_root[idx] = np.abs(v - px[idx]) < 0.5 * np.abs(truth["vega"][idx]) * err[idx]
        codes, counts = np.unique(out["status"], return_counts=True)
        res[name] = {
            "method": desc, "value": n / t,
            "unit": "IV/s (end to end through mango_gpu_solve_iv_batch_method)", "seconds": t,
            "buffers": "warm: one solve of the same batch before the timed one",
            "status_counts": {int(c): int(k) for c, k in zip(codes, counts)},
            "iterations_mean": float(out["iterations"][ok].mean()) if ok.any() else None,
            "excluded_invalid": int(invalid.sum()), "excluded_low_vega": int((~invalid & low_vega).sum()),
            "eligible": int(eligible.sum()),
            "frac_within_1e-6_vol": float(within.sum() / max(eligible.sum(), 1)),
            "misses": int((miss & ~other_root).sum()), "flat_or_non_monotone": int(other_root.sum()),
            "misses_settled_by_newton": int((miss & ~other_root & (out["has_vega"] == 1)).sum()),
            "settled_by_newton": int(((out["has_vega"] == 1) & ok).sum()),
            "frac_within_1e-6_vol_excluding_flat": float(within.sum() / max((eligible & ~other_root).sum(), 1)),
            "max_abs_vol_error_eligible": float(err[eligible & ok].max()) if (eligible & ok).any() else None,
            "quote_evaluations": int(st["options"]),
            "evaluations_by_grid": {"coarse_tangent": int(st["iv_evals"][0]), "own": int(st["iv_evals"][1])},
            "rounds": int(st["tiles"]), "kernel_launches": int(st["kernel_launches"]),
            "breakdown_ms": {"host_prep": round(st["host_prep_ms"], 2), "repack": round(st["prep_ms"], 2),
                             "evaluations_device": round(st["march_ms"], 2), "total": round(st["total_ms"], 2)}}
    res["value"] = res["newton"]["value"]
    res["unit"] = res["newton"]["unit"]
    res["speedup_newton_vs_brent"] = res["newton"]["value"] / res["brent"]["value"]
    res["speedup_secant_vs_brent"] = res["secant"]["value"] / res["brent"]["value"]
    return res


def bench_greeks(pkg, eng, n=16384):
    """Sensitivity workload: 16,384 American puts (spot 100, strike, maturity,
    volatility, rate and dividend yield drawn as in the pricing workload,
    101 x 498 grid rule), value/delta/gamma/theta plus frozen-grid vega, rho,
    dividend rho and dV/dK (8 bumped copies each, one device batch)."""
    rng = np.random.default_rng(3)
    params = pkg.pricing_array(np.full(n, 100.0), rng.uniform(80, 120, n), rng.uniform(0.1, 2.0, n),
                               rng.uniform(0.1, 0.5, n), rng.uniform(0.0, 0.08, n), rng.uniform(0.0, 0.04, n), 1)
    grid = pkg.grid_array(1, pkg.GRID_FIXED_N, NX, NT)
    eng.greeks_arrays(params, grid)
    t0 = time.perf_counter()
    out = eng.greeks_arrays(params, grid)
    t = time.perf_counter() - t0
    return {"workload": f"{n} American puts, 101x498, value+delta+gamma+theta+vega+rho+dq+dK "
                        "(central differences on the frozen grid, 9 prices per option)",
            "value": n / t, "unit": "options with full Greeks/s (end to end)", "seconds": t,
            "failed": int(np.count_nonzero(out["status"])),
            "tangent": bench_tangent(pkg, eng, params, grid)}


def bench_tangent(pkg, eng, params, grid):
    """The same 16,384 puts through the forward-mode march
    (mango_gpu_price_american_tangent_batch): value, delta and the exact
    discrete dV/dvolatility, dV/drate, dV/ddividend_yield, dV/dK in one pass."""
    eng.tangent_arrays(params, grid)
    t0 = time.perf_counter()
    out = eng.tangent_arrays(params, grid)
    t = time.perf_counter() - t0
    return {"workload": f"{params.size} American puts, 101x498, value+delta+exact discrete vega/rho/dq/dK "
                        "(forward-mode march, 3 tangents; three single-direction marches side by side at this size)",
            "value": params.size / t, "unit": "options with sensitivities/s (end to end)", "seconds": t,
            "failed": int(np.count_nonzero(out["status"]))}


def bench_schedules(pkg, eng, torch, stream, n, fp64_peak):
    """Time-varying march: n puts and calls (the pricing workload's
    distributions) on the
    101 x 498 grid rule with a 7-point yield curve, then with the curve plus
    two cash dividends per option (mandatory time points, two spline
    shifts).  Resident batches, device time of two runs."""
    rng = np.random.default_rng(5)
    T = rng.uniform(0.1, 2.0, n)
    params = pkg.pricing_array(np.full(n, 100.0), rng.uniform(80, 120, n), T, rng.uniform(0.1, 0.5, n), 0.0,
                               rng.uniform(0.0, 0.04, n), (np.arange(n) % 2 == 0).astype(np.int32))
    tenors = [0.25, 0.5, 1.0, 2.0, 3.0, 5.0]
    zeros = [0.02, 0.025, 0.03, 0.035, 0.038, 0.04]
    curve = [(0.0, 0.0)] + [(t, -z * t) for t, z in zip(tenors, zeros)]
    grid = pkg.grid_array(1, pkg.GRID_FIXED_N, NX, NT)
    out = {}
    for name, divs in (("yield_curve", None), ("curve_and_dividends",
                                               [[(0.3 * t, 1.0), (0.7 * t, 1.0)] for t in T])):
        p = params.copy()
        keep = pkg.attach_schedules(p, [curve] * n, divs)
        b = eng.batch(p, grid)
        del keep
        b.run()
        torch.cuda.synchronize()
        b.timings(reset=True)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(2):
            b.run()
        e1.record(stream)
        torch.cuda.synchronize()
        t = e0.elapsed_time(e1) / 1e3
        res = b.results()
        kt = b.timings()
        algo = eng.stats()["algo_flops"]
        out[name] = {
            "workload": f"{n} puts/calls, 101 points, 498 steps (+ dividend points), 7-point curve"
                        + (", 2 cash dividends each" if divs else ""),
            "value": 2 * n / t, "unit": "options/s", "failed": int(np.count_nonzero(res["status"])),
            "march_ms": kt["march_ms"],
            "fp64_frac": algo / (kt["march_ms"] / 1e3) / 1e12 / fp64_peak if fp64_peak else None,
            "mean_steps": float(np.mean(res["n_time"]))}
        b.close()
    # FDM IV of quotes carrying the curve and dividends: prices from the
    # forward solver at seeded vols, then Brent on a grid sized at 0.3.
    m = min(n, 16384)
    vt = rng.uniform(0.1, 0.6, m)
    p = pkg.pricing_array(np.full(m, 100.0), rng.uniform(85, 115, m), T[:m], vt, 0.0, 0.0, 1)
    divs = [[(0.3 * t, 1.0), (0.7 * t, 1.0)] for t in T[:m]]
    keep = pkg.attach_schedules(p, [curve] * m, divs)
    ivgrid = pkg.grid_array(1, pkg.GRID_FIXED_N_AT_VOL, NX, NT, alpha=0.3)
    px = eng.price_arrays(p, ivgrid)["value"]
    q = pkg.query_array(100.0, p["strike"], p["maturity"], 0.0, 0.0, 1, px)
    qkeep = pkg.attach_schedules(q, [curve] * m, divs)
    t0 = time.perf_counter()
    iv = eng.solve_iv_arrays(q, ivgrid, method=pkg.IV_BRENT)
    t_iv = time.perf_counter() - t0
    ok = iv["status"] == 0
    out["iv_curve_and_dividends"] = {
        "workload": f"{m} American puts, 7-point curve and 2 cash dividends each, 101x498 grid sized at 0.3, "
                    "Brent (the reference iterate sequence)",
        "value": m / t_iv, "unit": "IV/s (end to end through mango_gpu_solve_iv_batch_method)",
        "solved": int(np.count_nonzero(ok)),
        "max_abs_vol_error": float(np.abs(iv["implied_vol"][ok] - vt[ok]).max()) if ok.any() else None}
    del keep, qkeep
    return out


def bench_chain(pkg, eng, n):
    """Shared-grid batch on the normalized-chain route: n American puts as
    n/64 parameter groups (volatility, rate, yield, maturity) of 64 strikes
    each, one S = K = 1 march per group, every strike read from it
    (BatchAmericanOptionSolver::solve_batch with use_shared_grid)."""
    rng = np.random.default_rng(9)
    groups = max(1, n // 64)
    per = n // groups
    g_sig = rng.uniform(0.15, 0.45, groups)
    g_r = rng.uniform(0.0, 0.06, groups)
    g_q = rng.uniform(0.0, 0.03, groups)
    g_T = rng.uniform(0.25, 1.5, groups)
    # is_normalized_eligible tests the first option's grid (spacing <= 0.05)
    g_sig[0], g_T[0] = 0.2, 1.0
    K = np.tile(np.linspace(88.0, 112.0, per), groups)
    rep = lambda a: np.repeat(a, per)
    p = pkg.pricing_array(100.0, K, rep(g_T), rep(g_sig), rep(g_r), rep(g_q), 1)
    eng.price_shared_arrays(p)
    t0 = time.perf_counter()
    out, route = eng.price_shared_arrays(p)
    t = time.perf_counter() - t0
    return {"workload": f"{p.size} American puts, {groups} groups of {per} strikes, estimated shared grid",
            "value": p.size / t, "unit": "options/s (end to end through mango_gpu_price_american_batch_shared)",
            "route": "normalized chain" if route == 1 else "regular shared grid",
            "failed": int(np.count_nonzero(out["status"]))}


TABLE_AXES = (np.linspace(np.log(0.7), np.log(1.3), 50), np.linspace(0.02, 2.0, 30),
              np.linspace(0.05, 0.8, 20), np.linspace(0.0, 0.08, 10))


def bench_table(pkg, eng, torch, stream, nq, fp64_peak):
    """Price-table workload: 50 x 30 x 20 x 10 axes, 200 (sigma, r) PDE solves
    on the explicit 201 x 1000 sinh grid (the reference falls back to
    per-slice grids), then nq uniform random in-range 4D queries."""
    grid = pkg.PDEGridConfig(-3.0, 3.0, 201, 1000)
    eng.price_table_sweep(*TABLE_AXES, 100.0, 0.0, 1, grid)  # warm-up
    t0 = time.perf_counter()
    tensor, dims, failed = eng.price_table_sweep(*TABLE_AXES, 100.0, 0.0, 1, grid)
    t_sweep = time.perf_counter() - t0
    st = eng.stats()
    sweep = {"workload": "PriceTableBuilderND<4> sweep+extraction, 50x30x20x10 axes, 200 PDE solves, "
                         "explicit 201x1000 grid (per-slice fallback grids)",
             "seconds": t_sweep, "value": 200 / t_sweep, "unit": "PDE solves/s (end to end)",
             "failed": int(failed), "max_n_time": int(dims[:, 1].max()),
             "breakdown_ms": {k: round(float(st[k]), 3) for k in
                              ("host_prep_ms", "h2d_ms", "prep_ms", "march_ms", "outputs_ms", "d2h_ms")
                              if k in st}}
    sizes = [a.size for a in TABLE_AXES]
    coeffs = np.random.default_rng(2025).standard_normal(int(np.prod(sizes)))
    surf = eng.bspline4d(TABLE_AXES, coeffs)
    rng = np.random.default_rng(7)
    q = np.stack([rng.uniform(a[0], a[-1], nq) for a in TABLE_AXES], 1)
    dq = torch.from_numpy(q).to("cuda")
    dout = torch.empty(nq, dtype=torch.float64, device="cuda")
    for _ in range(3):
        surf.eval_device(dq.data_ptr(), nq, dout.data_ptr())
    torch.cuda.synchronize()
    reps = 10
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        surf.eval_device(dq.data_ptr(), nq, dout.data_ptr())
    e1.record(stream)
    torch.cuda.synchronize()
    t = e0.elapsed_time(e1) / 1e3 / reps
    t0 = time.perf_counter()
    host_out = surf.eval(q)
    t_e2e = time.perf_counter() - t0
    assert np.isfinite(host_out).all()
    flops_per_query = 780.0  # algorithmic count: 4 x (span + Cox-de Boor) + 256 FMA + partial sums
    query = {"workload": f"{nq} uniform random in-range 4D queries, 50x30x20x10 cubic B-spline (2.4 MB coeffs)",
             "value": nq / t, "unit": "queries/s (device-resident)",
             "e2e": {"value": nq / t_e2e, "unit": "queries/s", "h2d_bytes_per_step": int(q.nbytes),
                     "d2h_bytes_per_step": int(host_out.nbytes)},
             "hbm_gbs": 40.0 * nq / t / 1e9,
             "fp64_frac": flops_per_query * nq / t / 1e12 / fp64_peak, "ms": 1e3 * t}
    surf.close()
    # Whole table build on the device (sweep -> EEP -> fit -> surface) and
    # the standard table's price query (EEPLayer over TransformLeaf).
    eng.price_table_build(*TABLE_AXES, K_ref=100.0, dividend_yield=0.0, option_type=1, grid=grid)[0].close()
    t0 = time.perf_counter()
    table, fstats = eng.price_table_build(*TABLE_AXES, K_ref=100.0, dividend_yield=0.0, option_type=1, grid=grid)
    t_build = time.perf_counter() - t0
    sweep["build"] = {"workload": "PriceTableBuilderND<4>::build on the device: sweep + EEP + fit + surface",
                      "seconds": t_build, "fit_max_residual": max(fstats["max_residual"]),
                      "fit_failed_slices": int(sum(fstats["failed_slices"]))}
    nrec = min(nq, 2_000_000)
    rng = np.random.default_rng(8)
    recs = pkg.pricing_array(np.full(nrec, 100.0), 100.0 / np.exp(rng.uniform(TABLE_AXES[0][0], TABLE_AXES[0][-1], nrec)),
                             rng.uniform(0.02, 2.0, nrec), rng.uniform(0.05, 0.8, nrec), rng.uniform(0.0, 0.08, nrec),
                             0.0, 1)
    d_rec = torch.from_numpy(recs.view(np.uint8)).to("cuda")
    d_val = torch.empty(nrec, dtype=torch.float64, device="cuda")
    for _ in range(3):
        table.price_device(d_rec.data_ptr(), nrec, d_val.data_ptr())
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(reps):
        table.price_device(d_rec.data_ptr(), nrec, d_val.data_ptr())
    e1.record(stream)
    torch.cuda.synchronize()
    t_price = e0.elapsed_time(e1) / 1e3 / reps
    t0 = time.perf_counter()
    host_vals = table.price_arrays(recs)
    t_price_e2e = time.perf_counter() - t0
    assert np.isfinite(host_vals).all()
    query["table_price"] = {
        "workload": f"{nrec} American put prices from the 50x30x20x10 EEP table "
                    "(spline + max(0, .) K/K_ref + closed-form European)",
        "value": nrec / t_price, "unit": "prices/s (device-resident)",
        "e2e": {"value": nrec / t_price_e2e, "unit": "prices/s", "h2d_bytes_per_step": int(recs.nbytes),
                "d2h_bytes_per_step": int(host_vals.nbytes)}}
    # delta / gamma / theta / rho on the table (mango_gpu_price_table_greeks),
    # end to end from host records; in-range records so every status is 0.
    ng = min(nrec, 1_000_000)
    grng = np.random.default_rng(13)
    gp = pkg.pricing_array(np.full(ng, 100.0), 100.0 / np.exp(grng.uniform(-0.3, 0.2, ng)),
                           grng.uniform(0.1, 1.9, ng), grng.uniform(0.1, 0.7, ng), grng.uniform(0.005, 0.075, ng),
                           0.0, 1)
    table.greeks_arrays(gp)
    t0 = time.perf_counter()
    g4, gst = table.greeks_arrays(gp)
    t_g = time.perf_counter() - t0
    query["table_greeks"] = {
        "workload": f"{ng} American put delta/gamma/theta/rho from the 50x30x20x10 EEP table "
                    "(analytic spline partials + closed-form European Greeks)",
        "value": ng / t_g, "unit": "records with 4 Greeks/s (end to end)",
        "failed": int(np.count_nonzero(gst))}
    # Interpolated IV on the table (InterpolatedIVSolver::solve_batch): quotes
    # priced from the table at seeded vols, solved back on the device.
    niv = min(nq, 1_000_000)
    rng = np.random.default_rng(12)
    ivp = pkg.pricing_array(np.full(niv, 100.0), 100.0 / np.exp(rng.uniform(-0.3, 0.2, niv)),
                            rng.uniform(0.1, 1.9, niv), rng.uniform(0.1, 0.7, niv), rng.uniform(0.005, 0.075, niv),
                            0.0, 1)
    ivpx = table.price_arrays(ivp)
    ivq = pkg.query_array(ivp["spot"], ivp["strike"], ivp["maturity"], ivp["rate_const"], 0.0, 1, ivpx)
    d_q = torch.from_numpy(ivq.view(np.uint8)).to("cuda")
    d_s = torch.empty(niv * pkg.IVSLOT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    for _ in range(2):
        table.iv_device(d_q.data_ptr(), niv, d_s.data_ptr())
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(3):
        table.iv_device(d_q.data_ptr(), niv, d_s.data_ptr())
    e1.record(stream)
    torch.cuda.synchronize()
    t_iv = e0.elapsed_time(e1) / 1e3 / 3
    t0 = time.perf_counter()
    slots = table.iv_arrays(ivq)
    t_iv_e2e = time.perf_counter() - t0
    okv = slots["status"] == 0
    query["interp_iv"] = {
        "workload": f"{niv} American put quotes priced from the 50x30x20x10 EEP table, implied vol by "
                    "InterpolatedIVSolver (Brent on the table, vega pre-check)",
        "value": niv / t_iv, "unit": "IV/s (device-resident)",
        "e2e": {"value": niv / t_iv_e2e, "unit": "IV/s", "h2d_bytes_per_step": int(ivq.nbytes),
                "d2h_bytes_per_step": int(slots.nbytes)},
        "solved": int(okv.sum()), "iterations_mean": float(slots["iterations"][okv].mean()),
        "max_abs_vol_error": float(np.abs(slots["implied_vol"][okv] - ivp["volatility"][okv]).max())}
    table.close()
    return sweep, query


def run_reference(args, ws, rank):
    if rank != 0:
        return 0
    import __graft_entry__ as ge
    pkg = ge.load_package()  # record packing only; the timed work is the CPU implementation
    _, _, cols = make_workload(pkg, N_OPTIONS)
    lib, kind, fn = load_oracle()
    threads = os.cpu_count() or 1
    _, m, _ = cpu_sample(lib, fn, cols, threads, target_s=1.0)
    for _ in range(args.warmup):
        cpu_price(lib, fn, [c[:m] for c in cols], NX, NT, threads)
    times = []
    for _ in range(args.steps):
        t, _ = cpu_price(lib, fn, [c[:m] for c in cols], NX, NT, threads)
        times.append(t)
    total = sum(times)
    value = m * args.steps / total
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "options/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"{N_OPTIONS} American puts/calls, 101x498 grid rule (bounded sample of {m} per step)",
                   "options_per_step": m},
        "cpu_baseline": {"value": value, "unit": "options/s", "cores": threads, "kind": kind,
                         "sample": f"first {m} options of the {N_OPTIONS}-option workload per step"},
        "e2e": {"value": value, "unit": "options/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def bench_layouts(pkg, eng, torch):
    """The engine's layout choice (thread-per-option or warp-per-option march,
    plan_warp_tiles) against both layouts forced with MANGO_GPU_WARP_MARCH, on
    the pricing workload at several batch sizes, the uneven batch, and the
    table sweep.  Device march time of the batch's run after a warm-up run;
    the table sweep end to end.  One JSON line per workload."""
    def batch_ms(p, g):
        b = eng.batch(p, g)
        b.run()
        torch.cuda.synchronize()
        b.timings(reset=True)
        for _ in range(3):
            b.run()
        torch.cuda.synchronize()
        ms = b.timings()["march_ms"]
        b.close()
        return ms

    def sweep_ms():
        grid = pkg.PDEGridConfig(-3.0, 3.0, 201, 1000)
        eng.price_table_sweep(*TABLE_AXES, 100.0, 0.0, 1, grid)
        t0 = time.perf_counter()
        for _ in range(3):
            eng.price_table_sweep(*TABLE_AXES, 100.0, 0.0, 1, grid)
        return (time.perf_counter() - t0) / 3 * 1e3

    work = []
    for n in (65536, 8192, 4096, 512):
        p, g, _ = make_workload(pkg, n)
        work.append((f"{n} options, 101x498", lambda p=p, g=g: batch_ms(p, g)))
    p, g, _ = make_workload(pkg, 200)
    work.append(("200 options, 201x1000", lambda p=p: batch_ms(p, pkg.grid_array(1, pkg.GRID_FIXED_N, 201, 1000))))
    p, g, _ = make_workload(pkg, 65536, seed=77, uneven=True)
    work.append(("65536 options, N_x~U{51..401}, N_t~U{100..1000}", lambda p=p, g=g: batch_ms(p, g)))
    work.append(("table sweep, 200 solves at 201x1000 (end to end)", sweep_ms))
    for name, fn in work:
        row = {}
        for label, val in (("auto", None), ("thread", "0"), ("warp", "1")):
            if val is None:
                os.environ.pop("MANGO_GPU_WARP_MARCH", None)
            else:
                os.environ["MANGO_GPU_WARP_MARCH"] = val
            row[label] = round(fn(), 3)
        os.environ.pop("MANGO_GPU_WARP_MARCH", None)
        best = min(("thread", "warp"), key=lambda k: row[k])
        print(json.dumps({"workload": name, "ms": row, "faster": best,
                          "auto_within_3pct_of_faster": row["auto"] <= 1.03 * row[best]}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--options", type=int, default=N_OPTIONS)
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-extra", action="store_true",
                    help="skip the uneven-grid and schedule side measurements")
    ap.add_argument("--no-uneven", action="store_true", help="skip the uneven-grid side measurement")
    ap.add_argument("--no-schedules", action="store_true", help="skip the yield-curve / dividend measurement")
    ap.add_argument("--no-iv", action="store_true", help="skip the batched-IV side measurement")
    ap.add_argument("--iv-quotes", type=int, default=262144)
    ap.add_argument("--no-table", action="store_true", help="skip the table sweep / query side measurement")
    ap.add_argument("--queries", type=int, default=10_000_000)
    ap.add_argument("--layouts", action="store_true",
                    help="only compare the engine's thread/warp march choice with both layouts forced")
    args = ap.parse_args()
    ws, rank, local = dist_setup()
    if args.impl == "reference":
        return run_reference(args, ws, rank)

    import torch
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import __graft_entry__ as ge
    pkg = ge.load_package()
    eng = pkg.Engine(local)
    # A dedicated (non-default) stream: the engine enqueues on it and the
    # CUDA events below are recorded on it, so they bracket exactly its work.
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    assert stream.cuda_stream != 0
    eng.set_stream(stream.cuda_stream)
    if args.layouts:
        return bench_layouts(pkg, eng, torch)
    fp64_peak = eng.fp64_probe()

    n = args.options
    params, grids, cols = make_workload(pkg, n)
    batch = eng.batch(params, grids)
    for _ in range(max(3, args.warmup)):
        batch.run()
    torch.cuda.synchronize()
    warm = batch.results()
    assert (warm["status"] == 0).all(), "warm-up batch reported failures"
    batch.timings(reset=True)

    clk = ClockSampler(local)
    clk.start()
    time.sleep(0.3)
    barrier(ws)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        batch.run()
    e1.record(stream)
    torch.cuda.synchronize()
    barrier(ws)
    clocks = clk.stop()
    t_dev = reduce_max(e0.elapsed_time(e1) / 1e3, ws)
    kt = batch.timings()
    value = n * ws * args.steps / t_dev

    # End to end through the C ABI with host arrays.
    for _ in range(2):
        eng.price_arrays(params, grids)
    torch.cuda.synchronize()
    barrier(ws)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        out = eng.price_arrays(params, grids)
    t_e2e = reduce_max(time.perf_counter() - t0, ws)
    st = eng.stats()
    e2e = {"value": n * ws * args.steps / t_e2e, "unit": "options/s",
           "h2d_bytes_per_step": int(st["h2d_bytes"]), "d2h_bytes_per_step": int(st["d2h_bytes"]),
           "ms_per_step": 1e3 * t_e2e / args.steps,
           "breakdown_ms": {k: round(st[k], 3) for k in ("host_prep_ms", "h2d_ms", "prep_ms", "march_ms",
                                                        "outputs_ms", "d2h_ms", "total_ms")}}
    assert (out["status"] == 0).all()

    # Roofline of the dominant kernel (the march).
    algo = st["algo_flops"]
    march_s = kt["march_ms"] / 1e3
    achieved = algo / march_s / 1e12
    # DRAM traffic of one launch from the committed ncu capture of this
    # workload (dram__bytes_read + dram__bytes_write), scaled by row-steps
    # when the option count differs from the captured one.
    traffic, hbm = None, None
    tf = ROOT / "profiles" / "march_kernel_traffic.json"
    if tf.exists():
        try:
            cap = json.loads(tf.read_text())
            traffic = cap["bytes_per_row_step"] * n * (NT - 1) * (NX - 2)
        except Exception:
            traffic = None
    if traffic is not None:
        hbm_peak = measured_hbm_gbs()
        hbm = {"traffic_gbs": traffic / march_s / 1e9, "peak_gbs": hbm_peak,
               "frac": (traffic / march_s / 1e9 / hbm_peak) if hbm_peak else None,
               "note": "per-option working state (23 KB) re-streamed every step; 1.5 GB >> L2"}
    # FP64 pipe: the kernel's FP64 warp instructions per warp row-step
    # (ncu sm__inst_executed_pipe_fp64.sum of a captured launch) times this
    # launch's row-steps, per second, against the probe's DFMA issue rate
    # (TFLOP/s / 2 flops / 32 lanes): the pipe fraction beside the
    # algorithmic one.
    pipe = None
    pf = ROOT / "profiles" / "march_kernel_fp64.json"
    if pf.exists():
        try:
            per = json.loads(pf.read_text())["fp64_warp_inst_per_warp_row_step"]
            inst = per * n * (NT - 1) * (NX - 2) / 32.0
            probe_inst = fp64_peak * 1e12 / 2.0 / 32.0
            pipe = {"fp64_warp_inst_per_warp_row_step": per, "achieved_ginst_s": inst / march_s / 1e9,
                    "probe_ginst_s": probe_inst / 1e9, "frac": inst / march_s / probe_inst,
                    "source": "profiles/march_kernel_fp64.json"}
        except Exception:
            pipe = None
    roofline = {"bound": "fp64", "achieved": achieved, "peak": fp64_peak, "unit": "TFLOP/s",
                "frac": achieved / fp64_peak, "traffic": traffic,
                "peak_source": "measured live: mango_gpu_fp64_probe (independent DFMA chains, all SMs)",
                "kernel": "march_kernel", "kernel_ms": kt["march_ms"],
                "algo_flops_per_launch": algo, "fp64_pipe": pipe, "hbm_streaming": hbm}

    extra = {}
    if not args.no_extra and not args.no_uneven and rank == 0:
        p2, g2, _ = make_workload(pkg, n, seed=77, uneven=True)
        b2 = eng.batch(p2, g2)
        b2.run()
        torch.cuda.synchronize()
        b2.timings(reset=True)
        f0 = torch.cuda.Event(enable_timing=True)
        f1 = torch.cuda.Event(enable_timing=True)
        f0.record(stream)
        for _ in range(2):
            b2.run()
        f1.record(stream)
        torch.cuda.synchronize()
        tu = f0.elapsed_time(f1) / 1e3
        o2 = b2.results()
        kt2 = b2.timings()
        algo2 = eng.stats()["algo_flops"]
        extra["uneven_grids"] = {
            "workload": f"{n} puts/calls, N_x~U{{51..401}}, N_t~U{{100..1000}}, one persistent launch",
            "value": 2 * n / tu, "unit": "options/s", "failed": int(np.count_nonzero(o2["status"])),
            "march_ms": kt2["march_ms"], "fp64_frac": algo2 / (kt2["march_ms"] / 1e3) / 1e12 / fp64_peak}
        b2.close()

    if not args.no_extra and not args.no_schedules and rank == 0:
        extra["schedules"] = bench_schedules(pkg, eng, torch, stream, n, fp64_peak)
    if not args.no_extra and rank == 0:
        extra["shared_chain"] = bench_chain(pkg, eng, n)
    if not args.no_iv and rank == 0:
        extra["iv"] = bench_iv(pkg, eng, args.iv_quotes)
    if not args.no_iv and rank == 0:
        extra["greeks"] = bench_greeks(pkg, eng)
    if not args.no_table and rank == 0:
        extra["table_sweep"], extra["bspline_query"] = bench_table(pkg, eng, torch, stream,
                                                                   args.queries, fp64_peak)

    if rank == 0 and ws == 1 and not args.no_cpu:
        # CPU baselines of the side workloads (the reference's paths restated,
        # bounded samples, after every GPU measurement)
        port = load_port()
        if "uneven_grids" in extra:
            extra["uneven_grids"]["cpu_baseline"] = cpu_uneven(port)
        if "iv" in extra:
            extra["iv"]["cpu_baseline"] = cpu_iv(port, pkg)
        if "table_sweep" in extra:
            extra["table_sweep"]["cpu_baseline"] = cpu_sweep(port)
        if "bspline_query" in extra:
            extra["bspline_query"]["cpu_baseline"] = cpu_query(port)
    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        lib, kind, fn = load_oracle()
        threads = os.cpu_count() or 1
        v, m, t = cpu_sample(lib, fn, cols, threads)
        cpu = {"value": v, "unit": "options/s", "cores": threads, "kind": kind,
               "sample": f"first {m} options of the workload, 101x498, {t:.2f} s wall on {threads} threads"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "options/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * t_dev / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"{n} American puts/calls (50/50), 101x498 sinh grid rule, FP64",
                       "options": n, "n_space": NX, "n_time": NT, "parallelism": f"replicas x{ws}",
                       "l2": "no flush: per-step device state ~1.5 GB >> 129 MB L2"},
            "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "clocks": clocks,
            "gpu_launches": 3 * args.steps,
            "kernel_ms_per_step": {k: round(kt[k], 4) for k in ("prep_ms", "march_ms", "outputs_ms")},
            **extra,
        }
        print(json.dumps(line), flush=True)
    batch.close()
    eng.close()
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
