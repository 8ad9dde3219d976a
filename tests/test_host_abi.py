"""C-ABI and host-logic checks that need no GPU: the library loads and
exports every symbol include/mango_gpu.h declares, struct layouts match the
reference ABI, host grid selection reproduces the reference's grids bit for
bit, and the no-device failure path reports an error instead of crashing."""
import ctypes
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT, golden


def header_functions():
    text = (ROOT / "include" / "mango_gpu.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(mango_gpu_\w+)\s*\(", text)))


def test_library_exports_every_declared_symbol(pkg):
    lib = pkg.library()
    names = header_functions()
    assert len(names) >= 6
    for name in names:
        assert hasattr(lib, name), f"{name} declared in include/mango_gpu.h but not exported"
    nm = subprocess.run(["nm", "-D", "--defined-only", str(pkg.LIB_PATH)], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\b(mango_gpu_\w+)\b", nm))
    assert exported == set(names), f"undeclared exports: {exported - set(names)}"


def test_struct_layouts_match_reference_abi(pkg):
    # src/ffi/mango_c_api.h:195-329 asserts these sizes/offsets.
    assert pkg.PRICING_DTYPE.itemsize == 88
    assert pkg.PRICING_DTYPE.fields["rate_const"][1] == 40
    assert pkg.PRICING_DTYPE.fields["tenor_points"][1] == 48
    assert pkg.PRICING_DTYPE.fields["n_dividends"][1] == 72
    assert pkg.PRICING_DTYPE.fields["option_type"][1] == 80
    assert pkg.IVQUERY_DTYPE.itemsize == 88
    assert pkg.IVQUERY_DTYPE.fields["market_price"][1] == 32
    assert ctypes.sizeof(pkg.MangoError) == 260
    assert pkg.GRID_DTYPE.itemsize == 48
    assert pkg.OUT_DTYPE.itemsize == 48


def test_header_compiles_as_c_and_cpp(tmp_path):
    src = tmp_path / "t.c"
    src.write_text('#include "mango_gpu.h"\nint main(void){MangoGpuGrid g; (void)g; return (int)sizeof(MangoPricingParams) - 88;}\n')
    for cc, ext in (("gcc", "c"), ("g++", "cpp")):
        f = tmp_path / f"t.{ext}"
        f.write_text(src.read_text())
        r = subprocess.run([cc, "-std=c11" if ext == "c" else "-std=c++17", "-I", str(ROOT / "include"), "-o",
                            str(tmp_path / f"t_{ext}"), str(f)], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        assert subprocess.run([str(tmp_path / f"t_{ext}")]).returncode == 0


def test_host_grids_match_reference_bitwise(pkg):
    g = golden("grids.npz")
    for i, (S, K, T, s, nx) in enumerate(g["params"]):
        p = pkg.pricing_array(S, K, T, s, 0.05, 0.0, 1)
        grid = pkg.FixedGrid(int(nx), 123) if nx > 0 else None
        x, nt = pkg.resolve_grid(p, grid)
        assert x.size == g["n"][i]
        if nx == 0:
            assert nt == g["nt"][i]
        assert np.array_equal(x, g["x"][i, : x.size]), f"grid {i} differs"


def test_host_grids_match_oracle_for_config1_sizes(pkg, oracle):
    rng = np.random.default_rng(5)
    for _ in range(40):
        S, K, T, s = 100.0, rng.uniform(80, 120), rng.uniform(0.02, 2.0), rng.uniform(0.05, 0.8)
        nx = int(rng.integers(51, 402))
        x, _ = pkg.resolve_grid(pkg.pricing_array(S, K, T, s, 0.03, 0.01, 0), pkg.FixedGrid(nx, 200))
        xo, _ = oracle.grid(S, K, T, s, nx)
        assert np.array_equal(x, xo)


def test_resolve_grid_rejects_invalid_params(pkg):
    with pytest.raises(ValueError):
        pkg.resolve_grid(pkg.pricing_array(-1.0, 100.0, 1.0, 0.2, 0.05, 0.0, 1))
    with pytest.raises(ValueError):
        pkg.resolve_grid(pkg.pricing_array(100.0, 100.0, 1.0, 0.0, 0.05, 0.0, 1))
    with pytest.raises(ValueError):
        pkg.resolve_grid(pkg.pricing_array(100.0, 100.0, 1.0, 0.2, 0.05, 0.0, 1), pkg.FixedGrid(2, 10))


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_has_gpu(), reason="exercises the no-device error path")
def test_context_create_without_device_reports_error(pkg):
    with pytest.raises(pkg.EngineError):
        pkg.Engine(0)
