"""Price-table persistence: the CRC64 against the reference's own
src/support/crc64.cpp (compiled into the reference library), and the
Parquet format of src/option/table/parquet/parquet_io.cpp: a file written
and read back, and the reference's own writer and reader (compiled against
the Arrow C++ libraries pyarrow bundles into oracle/_ref/
libmango_ref_parquet.so, where the reference tree is present) reading the
engine's files and writing files the engine reads.  The device round trip
(table -> file -> table) is in the GPU test at the end."""
import ctypes
import sys

import numpy as np
import pytest

from conftest import ROOT

sys.path.insert(0, str(ROOT / "oracle"))
import fit_oracle  # noqa: E402

pa = pytest.importorskip("pyarrow")
pq = pytest.importorskip("pyarrow.parquet")


def ref_lib():
    so = ROOT / "oracle" / "_ref" / "libmango_ref.so"
    if not so.exists():
        pytest.skip("reference library not built here")
    lib = ctypes.CDLL(str(so))
    lib.ref_crc64_update.restype = ctypes.c_uint64
    lib.ref_crc64_update.argtypes = [ctypes.c_uint64, ctypes.c_char_p, ctypes.c_uint64]
    return lib


def test_crc64_matches_reference(pkg):
    lib = ref_lib()
    ours = pkg.library().mango_gpu_crc64_update
    rng = np.random.default_rng(7)
    crc_r = crc_o = 0
    for n in (0, 1, 7, 8, 255, 4096, 100001):
        b = rng.integers(0, 256, n, dtype=np.uint8).tobytes()
        crc_r = lib.ref_crc64_update(crc_r, b, n)
        crc_o = ours(crc_o, b, n)
        assert crc_r == crc_o, n
    assert ours(0, b"123456789", 9) == lib.ref_crc64_update(0, b"123456789", 9)


def sample_data(pkg, seed=3):
    rng = np.random.default_rng(seed)
    axes = [np.linspace(-0.3, 0.3, 9), np.linspace(0.05, 1.5, 6), np.linspace(0.1, 0.6, 5),
            np.linspace(0.0, 0.06, 4)]
    knots = [fit_oracle.clamped_knots(a) for a in axes]  # as the device derives them
    seg = pkg.PriceTableSegment(segment_id=0, K_ref=100.0, tau_start=0.0, tau_end=1.5, tau_min=0.05, tau_max=1.5,
                                domain_lo=[a[0] for a in axes], domain_hi=[a[-1] for a in axes],
                                num_pts=[a.size for a in axes], grids=axes, knots=knots,
                                values=rng.standard_normal(9 * 6 * 5 * 4))
    return pkg.PriceTableData(option_type=1, dividend_yield=0.01, maturity=1.5, bounds_m_min=-0.3,
                              bounds_m_max=0.3, bounds_tau_min=0.05, bounds_tau_max=1.5, bounds_sigma_min=0.1,
                              bounds_sigma_max=0.6, bounds_rate_min=0.0, bounds_rate_max=0.06, segments=[seg],
                              n_pde_solves=20, precompute_time_seconds=0.125)


@pytest.mark.parametrize("compression", ["zstd", "snappy", "none"])
def test_parquet_round_trip_and_layout(pkg, tmp_path, compression):
    d = sample_data(pkg)
    f = tmp_path / "t.parquet"
    pkg.write_parquet(d, f, compression)
    t = pq.read_table(f)
    assert t.column_names == ["segment_id", "K_ref", "tau_start", "tau_end", "tau_min", "tau_max", "interp_type",
                              "ndim", "domain_lo", "domain_hi", "num_pts", "grid_0", "grid_1", "grid_2", "grid_3",
                              "knots_0", "knots_1", "knots_2", "knots_3", "values", "checksum_values"]
    assert all(not f.nullable for f in t.schema)
    meta = {k.decode(): v.decode() for k, v in t.schema.metadata.items()}
    assert meta["mango.format_version"] == "2.0" and meta["mango.surface_type"] == "bspline_4d"
    assert meta["mango.option_type"] == "PUT" and meta["mango.dividend_yield"] == "0.01"
    assert meta["mango.precompute_time_seconds"] == "0.125" and meta["mango.n_pde_solves"] == "20"
    back = pkg.read_parquet(f)
    s0, s1 = d.segments[0], back.segments[0]
    assert back.bounds_rate_max == 0.06 and back.option_type == 1
    for g0, g1 in zip(s0.grids + s0.knots, s1.grids + s1.knots):
        assert np.array_equal(g0, g1)
    assert np.array_equal(s0.values, s1.values)


def ref_parquet():
    so = ROOT / "oracle" / "_ref" / "libmango_ref_parquet.so"
    if not so.exists():
        pytest.skip("the reference's Parquet writer is not built here")
    lib = ctypes.CDLL(str(so))
    lib.ref_parquet_write_bspline4d.restype = ctypes.c_int32
    lib.ref_parquet_read.restype = ctypes.c_int32
    return lib


def P(a):
    return a.ctypes.data_as(ctypes.c_void_p)


COMPRESSION = {"none": 0, "snappy": 1, "zstd": 2}


@pytest.mark.parametrize("compression", ["zstd", "snappy", "none"])
def test_reference_reads_engine_file(pkg, tmp_path, compression):
    """read_parquet of the reference accepts the engine's file (format
    version, keys, column types, both checksum levels) and returns its
    fields."""
    lib = ref_parquet()
    d = sample_data(pkg)
    f = tmp_path / "engine.parquet"
    pkg.write_parquet(d, f, compression)
    kind = ctypes.create_string_buffer(64)
    sc, b8, s4 = np.zeros(8), np.zeros(8), np.zeros(4, np.int64)
    vals = np.zeros(d.segments[0].values.size)
    assert lib.ref_parquet_read(str(f).encode(), kind, P(sc), P(b8), P(s4), P(vals), ctypes.c_int64(vals.size)) == 0
    assert kind.value == b"bspline_4d"
    assert list(sc) == [1.0, 0.01, 1.5, 20.0, 0.125, 1.0, 100.0, 4.0]
    assert list(b8) == [-0.3, 0.3, 0.05, 1.5, 0.1, 0.6, 0.0, 0.06]
    assert list(s4) == d.segments[0].num_pts
    assert np.array_equal(vals, d.segments[0].values)


@pytest.mark.parametrize("compression", ["zstd", "snappy", "none"])
def test_engine_reads_reference_file(pkg, tmp_path, compression):
    """The reference's write_parquet output is read by the engine with every
    field and both checksums as written."""
    lib = ref_parquet()
    d = sample_data(pkg)
    s = d.segments[0]
    f = tmp_path / "reference.parquet"
    sizes = np.array(s.num_pts, np.int64)
    grids, knots = np.concatenate(s.grids), np.concatenate(s.knots)
    b8 = np.array([d.bounds_m_min, d.bounds_m_max, d.bounds_tau_min, d.bounds_tau_max, d.bounds_sigma_min,
                   d.bounds_sigma_max, d.bounds_rate_min, d.bounds_rate_max])
    lo, hi = np.array(s.domain_lo, float), np.array(s.domain_hi, float)
    rc = lib.ref_parquet_write_bspline4d(
        str(f).encode(), P(sizes), P(grids), P(knots), P(np.ascontiguousarray(s.values)), ctypes.c_double(s.K_ref),
        ctypes.c_int32(1), ctypes.c_double(d.dividend_yield), ctypes.c_double(d.maturity), P(b8), P(lo), P(hi),
        ctypes.c_double(s.tau_start), ctypes.c_double(s.tau_end), ctypes.c_double(s.tau_min),
        ctypes.c_double(s.tau_max), ctypes.c_int64(d.n_pde_solves), ctypes.c_double(d.precompute_time_seconds),
        ctypes.c_int32(COMPRESSION[compression]))
    assert rc == 0
    back = pkg.read_parquet(f)
    assert back.option_type == 1 and back.dividend_yield == 0.01 and back.maturity == 1.5
    assert back.n_pde_solves == 20 and back.precompute_time_seconds == 0.125
    assert (back.bounds_m_min, back.bounds_rate_max) == (-0.3, 0.06)
    s1 = back.segments[0]
    assert (s1.K_ref, s1.tau_start, s1.tau_end, s1.tau_min, s1.tau_max) == (100.0, 0.0, 1.5, 0.05, 1.5)
    assert s1.interp_type == "bspline" and s1.ndim == 4 and list(s1.num_pts) == s.num_pts
    for g0, g1 in zip(s.grids + s.knots, s1.grids + s1.knots):
        assert np.array_equal(g0, g1)
    assert np.array_equal(s.values, s1.values)


def test_parquet_rejects_corruption(pkg, tmp_path):
    d = sample_data(pkg)
    f = tmp_path / "t.parquet"
    pkg.write_parquet(d, f)
    t = pq.read_table(f)
    # a changed coefficient: segment checksum mismatch
    vals = t.column("values").to_pylist()
    vals[0][5] += 1e-12
    bad = t.set_column(t.column_names.index("values"), t.schema.field("values"), pa.array(vals, t.schema.field("values").type))
    pq.write_table(bad.replace_schema_metadata(t.schema.metadata), tmp_path / "bad.parquet")
    with pytest.raises(pkg.SerializationError):
        pkg.read_parquet(tmp_path / "bad.parquet")
    # a changed file field: metadata checksum mismatch
    meta = dict(t.schema.metadata)
    meta[b"mango.dividend_yield"] = b"0.02"
    pq.write_table(t.replace_schema_metadata(meta), tmp_path / "bad2.parquet")
    with pytest.raises(pkg.SerializationError):
        pkg.read_parquet(tmp_path / "bad2.parquet")
    # a wrong version and a missing key
    for k, v in ((b"mango.format_version", b"1.0"), (b"mango.maturity", None)):
        meta = dict(t.schema.metadata)
        if v is None:
            meta.pop(k)
        else:
            meta[k] = v
        pq.write_table(t.replace_schema_metadata(meta), tmp_path / "bad3.parquet")
        with pytest.raises(pkg.SerializationError):
            pkg.read_parquet(tmp_path / "bad3.parquet")
    # invalid data is refused before writing
    d.bounds_m_min = d.bounds_m_max
    with pytest.raises(pkg.SerializationError):
        pkg.write_parquet(d, tmp_path / "never.parquet")


@pytest.mark.gpu
def test_table_save_load_prices_identically(engine, pkg, tmp_path):
    d = sample_data(pkg)
    t = pkg.from_data(d, engine)
    f = tmp_path / "table.parquet"
    t.save(f)
    t2 = pkg.load_price_table(f, engine)
    p = pkg.pricing_array(100.0, 100.0 / np.exp(np.linspace(-0.25, 0.25, 64)), 0.7, 0.3, 0.03, 0.01, 1)
    assert np.array_equal(t.price_arrays(p), t2.price_arrays(p))
    rd = t2.to_data()
    assert np.array_equal(rd.segments[0].values, d.segments[0].values)
    t.close()
    t2.close()
