"""Price-table persistence: the reference's PriceTableData model and its
Parquet format (src/option/table/serialization/price_table_data.hpp,
to_data.cpp, from_data.cpp; src/option/table/parquet/parquet_io.cpp), for
the standard EEP B-spline table ("bspline_4d").

File layout (format version "2.0"), restated from parquet_io.cpp:
  * one row per segment with columns segment_id (int32), K_ref, tau_start,
    tau_end, tau_min, tau_max (float64), interp_type (utf8), ndim (int32),
    domain_lo, domain_hi (list<float64>), num_pts (list<int32>),
    grid_0..grid_3, knots_0..knots_3, values (list<float64>) and
    checksum_values (uint64), none nullable;
  * file metadata keys mango.format_version, mango.surface_type,
    mango.option_type ("PUT" / "CALL"), mango.dividend_yield,
    mango.maturity, mango.bounds_{m,tau,sigma,rate}_{min,max},
    mango.n_pde_solves, mango.precompute_time_seconds (doubles printed with
    17 significant digits) and mango.metadata_checksum;
  * checksum_values = CRC64 over the segment's fields in order (integers
    and doubles as little-endian 8-byte or 4-byte words, strings and vectors
    prefixed by their length); mango.metadata_checksum = CRC64 over the file
    fields and the (segment_id, checksum) pairs sorted by segment_id.
Reading rejects a wrong version, a missing key or column, a wrong column
type, nulls and any checksum mismatch.

The Parquet container is written and read through pyarrow (present where
the tables are built offline; not needed by the pricing path)."""
from __future__ import annotations

import ctypes
import dataclasses
import struct
import sys
from typing import List, Optional

import numpy as np

FORMAT_VERSION = "2.0"
SURFACE_BSPLINE_4D = "bspline_4d"


class SerializationError(ValueError):
    """PriceTableErrorCode::SerializationFailed / InvalidConfig."""


def _pkg():
    return sys.modules[__package__]


@dataclasses.dataclass
class PriceTableSegment:
    """PriceTableData::Segment."""
    segment_id: int = 0
    K_ref: float = 0.0
    tau_start: float = 0.0
    tau_end: float = 0.0
    tau_min: float = 0.0
    tau_max: float = 0.0
    interp_type: str = "bspline"
    ndim: int = 4
    domain_lo: List[float] = dataclasses.field(default_factory=list)
    domain_hi: List[float] = dataclasses.field(default_factory=list)
    num_pts: List[int] = dataclasses.field(default_factory=list)
    grids: List[np.ndarray] = dataclasses.field(default_factory=list)
    knots: List[np.ndarray] = dataclasses.field(default_factory=list)
    values: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros(0))


@dataclasses.dataclass
class PriceTableData:
    """PriceTableData (price_table_data.hpp): a table's file-level fields and
    its segments."""
    surface_type: str = SURFACE_BSPLINE_4D
    option_type: int = 1  # OptionType (MANGO_CALL 0, MANGO_PUT 1)
    dividend_yield: float = 0.0
    maturity: float = 0.0
    bounds_m_min: float = 0.0
    bounds_m_max: float = 0.0
    bounds_tau_min: float = 0.0
    bounds_tau_max: float = 0.0
    bounds_sigma_min: float = 0.0
    bounds_sigma_max: float = 0.0
    bounds_rate_min: float = 0.0
    bounds_rate_max: float = 0.0
    segments: List[PriceTableSegment] = dataclasses.field(default_factory=list)
    n_pde_solves: int = 0
    precompute_time_seconds: float = 0.0


# ------------------------------------------------------------- checksums --

class _Crc:
    """CRCHasher of parquet_io.cpp over the library's CRC64."""

    def __init__(self):
        self.crc = 0
        self._lib = _pkg().library()

    def _bytes(self, b: bytes):
        self.crc = int(self._lib.mango_gpu_crc64_update(ctypes.c_uint64(self.crc), b, len(b)))

    def u64(self, v: int):
        self._bytes(struct.pack("<Q", int(v) & 0xFFFFFFFFFFFFFFFF))

    def i32(self, v: int):
        self._bytes(struct.pack("<i", int(v)))

    def f64(self, v: float):
        self._bytes(struct.pack("<d", float(v)))

    def string(self, s: str):
        b = s.encode()
        self.u64(len(b))
        self._bytes(b)

    def f64_vec(self, v):
        a = np.ascontiguousarray(v, dtype="<f8")
        self.u64(a.size)
        self._bytes(a.tobytes())

    def i32_vec(self, v):
        a = np.ascontiguousarray(v, dtype="<i4")
        self.u64(a.size)
        self._bytes(a.tobytes())


def segment_checksum(seg: PriceTableSegment) -> int:
    """segment_checksum (parquet_io.cpp:150-175)."""
    h = _Crc()
    h.i32(seg.segment_id)
    h.f64(seg.K_ref)
    h.f64(seg.tau_start)
    h.f64(seg.tau_end)
    h.f64(seg.tau_min)
    h.f64(seg.tau_max)
    h.string(seg.interp_type)
    h.u64(seg.ndim)
    h.f64_vec(seg.domain_lo)
    h.f64_vec(seg.domain_hi)
    h.i32_vec(seg.num_pts)
    h.u64(len(seg.grids))
    for g in seg.grids:
        h.f64_vec(g)
    h.u64(len(seg.knots))
    for k in seg.knots:
        h.f64_vec(k)
    h.f64_vec(seg.values)
    return h.crc


def metadata_checksum(data: PriceTableData, seg_crcs) -> int:
    """metadata_checksum (parquet_io.cpp:177-211)."""
    h = _Crc()
    h.string(data.surface_type)
    h.i32(data.option_type)
    for v in (data.dividend_yield, data.maturity, data.bounds_m_min, data.bounds_m_max, data.bounds_tau_min,
              data.bounds_tau_max, data.bounds_sigma_min, data.bounds_sigma_max, data.bounds_rate_min,
              data.bounds_rate_max):
        h.f64(v)
    h.u64(data.n_pde_solves)
    h.f64(data.precompute_time_seconds)
    pairs = sorted(seg_crcs)
    h.u64(len(pairs))
    for sid, crc in pairs:
        h.i32(sid)
        h.u64(crc)
    return h.crc


def _d2s(v: float) -> str:
    # std::ostringstream with precision 17 (default float field): %.17g
    return format(float(v), ".17g")


def _parse_double(s: str) -> float:
    try:
        v = float(s)
    except ValueError as e:
        raise SerializationError(f"bad number {s!r}") from e
    if not np.isfinite(v):
        raise SerializationError(f"non-finite {s!r}")
    return v


def _parse_uint(s: str) -> int:
    if not s or s[0] == "-" or not s.isdigit():
        raise SerializationError(f"bad integer {s!r}")
    return int(s)


# ---------------------------------------------------------- Parquet I/O --

def _arrow():
    try:
        import pyarrow as pa
        import pyarrow.parquet as pq
    except ImportError as e:  # the pricing path never needs it
        raise ImportError("price-table persistence needs pyarrow") from e
    return pa, pq


def _schema(pa, metadata):
    ld = pa.list_(pa.float64())  # arrow::list(arrow::float64()): child "item", nullable
    li = pa.list_(pa.int32())
    f = [pa.field("segment_id", pa.int32(), False), pa.field("K_ref", pa.float64(), False),
         pa.field("tau_start", pa.float64(), False), pa.field("tau_end", pa.float64(), False),
         pa.field("tau_min", pa.float64(), False), pa.field("tau_max", pa.float64(), False),
         pa.field("interp_type", pa.utf8(), False), pa.field("ndim", pa.int32(), False),
         pa.field("domain_lo", ld, False), pa.field("domain_hi", ld, False), pa.field("num_pts", li, False)]
    f += [pa.field(f"grid_{d}", ld, False) for d in range(4)]
    f += [pa.field(f"knots_{d}", ld, False) for d in range(4)]
    f += [pa.field("values", ld, False), pa.field("checksum_values", pa.uint64(), False)]
    return pa.schema(f, metadata=metadata)


def write_parquet(data: PriceTableData, path, compression: str = "zstd") -> None:
    """write_parquet (parquet_io.cpp:364-600): validation, metadata,
    per-segment checksums, one row per segment.  compression: "zstd"
    (default), "snappy" or "none"."""
    pa, pq = _arrow()
    scalars = (data.dividend_yield, data.maturity, data.precompute_time_seconds, data.bounds_m_min,
               data.bounds_m_max, data.bounds_tau_min, data.bounds_tau_max, data.bounds_sigma_min,
               data.bounds_sigma_max, data.bounds_rate_min, data.bounds_rate_max)
    if not all(np.isfinite(v) for v in scalars):
        raise SerializationError("non-finite file field")
    if (data.bounds_m_min >= data.bounds_m_max or data.bounds_tau_min >= data.bounds_tau_max
            or data.bounds_sigma_min >= data.bounds_sigma_max or data.bounds_rate_min >= data.bounds_rate_max):
        raise SerializationError("empty bounds")
    if data.option_type not in (0, 1):
        raise SerializationError("option type")
    for seg in data.segments:
        if not 1 <= seg.ndim <= 4 or len(seg.grids) > seg.ndim or len(seg.knots) > seg.ndim:
            raise SerializationError("ndim")
        if not np.isfinite(seg.K_ref) or seg.K_ref <= 0.0:
            raise SerializationError("K_ref")
        if not all(np.isfinite(v) for v in (seg.tau_start, seg.tau_end, seg.tau_min, seg.tau_max)):
            raise SerializationError("tau range")
        if seg.tau_start > seg.tau_end or seg.tau_min > seg.tau_max:
            raise SerializationError("tau range")
        if len(seg.values) == 0:
            raise SerializationError("empty values")
    meta = {
        "mango.format_version": FORMAT_VERSION,
        "mango.surface_type": data.surface_type,
        "mango.option_type": "PUT" if data.option_type == 1 else "CALL",
        "mango.dividend_yield": _d2s(data.dividend_yield),
        "mango.maturity": _d2s(data.maturity),
        "mango.bounds_m_min": _d2s(data.bounds_m_min),
        "mango.bounds_m_max": _d2s(data.bounds_m_max),
        "mango.bounds_tau_min": _d2s(data.bounds_tau_min),
        "mango.bounds_tau_max": _d2s(data.bounds_tau_max),
        "mango.bounds_sigma_min": _d2s(data.bounds_sigma_min),
        "mango.bounds_sigma_max": _d2s(data.bounds_sigma_max),
        "mango.bounds_rate_min": _d2s(data.bounds_rate_min),
        "mango.bounds_rate_max": _d2s(data.bounds_rate_max),
        "mango.n_pde_solves": str(int(data.n_pde_solves)),
        "mango.precompute_time_seconds": _d2s(data.precompute_time_seconds),
    }
    crcs = [segment_checksum(s) for s in data.segments]
    meta["mango.metadata_checksum"] = str(metadata_checksum(data, [(s.segment_id, c) for s, c in
                                                                   zip(data.segments, crcs)]))
    segs = data.segments
    pad = lambda lst, d: [np.asarray(x[d], np.float64) if d < len(x) else np.zeros(0) for x in lst]
    cols = {
        "segment_id": pa.array([s.segment_id for s in segs], pa.int32()),
        "K_ref": pa.array([s.K_ref for s in segs], pa.float64()),
        "tau_start": pa.array([s.tau_start for s in segs], pa.float64()),
        "tau_end": pa.array([s.tau_end for s in segs], pa.float64()),
        "tau_min": pa.array([s.tau_min for s in segs], pa.float64()),
        "tau_max": pa.array([s.tau_max for s in segs], pa.float64()),
        "interp_type": pa.array([s.interp_type for s in segs], pa.utf8()),
        "ndim": pa.array([s.ndim for s in segs], pa.int32()),
        "domain_lo": [np.asarray(s.domain_lo, np.float64) for s in segs],
        "domain_hi": [np.asarray(s.domain_hi, np.float64) for s in segs],
        "num_pts": [np.asarray(s.num_pts, np.int32) for s in segs],
    }
    for d in range(4):
        cols[f"grid_{d}"] = pad([s.grids for s in segs], d)
    for d in range(4):
        cols[f"knots_{d}"] = pad([s.knots for s in segs], d)
    cols["values"] = [np.asarray(s.values, np.float64) for s in segs]
    cols["checksum_values"] = pa.array(crcs, pa.uint64())
    schema = _schema(pa, meta)
    arrays = [pa.array(cols[f.name], f.type) if not isinstance(cols[f.name], pa.Array) else cols[f.name]
              for f in schema]
    table = pa.Table.from_arrays(arrays, schema=schema)
    comp = {"zstd": "zstd", "snappy": "snappy", "none": "none"}[compression]
    pq.write_table(table, str(path), compression=comp, row_group_size=1024, store_schema=True)


def read_parquet(path) -> PriceTableData:
    """read_parquet (parquet_io.cpp:604-947)."""
    pa, pq = _arrow()
    try:
        table = pq.read_table(str(path))
    except Exception as e:
        raise SerializationError(f"cannot read {path}: {e}") from e
    raw = table.schema.metadata or {}
    kv = {k.decode(): v.decode() for k, v in raw.items()}

    def meta(key):
        if key not in kv:
            raise SerializationError(f"missing {key}")
        return kv[key]

    if meta("mango.format_version") != FORMAT_VERSION:
        raise SerializationError("format version")
    data = PriceTableData()
    data.surface_type = meta("mango.surface_type")
    ot = meta("mango.option_type")
    if ot not in ("PUT", "CALL"):
        raise SerializationError("option type")
    data.option_type = 1 if ot == "PUT" else 0
    for name in ("dividend_yield", "maturity", "bounds_m_min", "bounds_m_max", "bounds_tau_min", "bounds_tau_max",
                 "bounds_sigma_min", "bounds_sigma_max", "bounds_rate_min", "bounds_rate_max"):
        setattr(data, name, _parse_double(meta(f"mango.{name}")))
    data.n_pde_solves = _parse_uint(meta("mango.n_pde_solves"))
    data.precompute_time_seconds = _parse_double(meta("mango.precompute_time_seconds"))
    scalar = {"segment_id": pa.int32(), "K_ref": pa.float64(), "tau_start": pa.float64(), "tau_end": pa.float64(),
              "tau_min": pa.float64(), "tau_max": pa.float64(), "interp_type": pa.string(), "ndim": pa.int32(),
              "checksum_values": pa.uint64()}
    lists = {"domain_lo": pa.float64(), "domain_hi": pa.float64(), "num_pts": pa.int32(), "values": pa.float64()}
    lists.update({f"grid_{d}": pa.float64() for d in range(4)})
    lists.update({f"knots_{d}": pa.float64() for d in range(4)})
    cols = {}
    for name, typ in list(scalar.items()) + list(lists.items()):
        if name not in table.column_names:
            raise SerializationError(f"missing column {name}")
        col = table.column(name).combine_chunks()
        if col.null_count:
            raise SerializationError(f"nulls in {name}")
        if name in scalar:
            if col.type != typ:
                raise SerializationError(f"type of {name}")
        else:
            if not pa.types.is_list(col.type) or col.type.value_type != typ or col.values.null_count:
                raise SerializationError(f"type of {name}")
        cols[name] = col
    seg_crcs = []
    for i in range(table.num_rows):
        s = PriceTableSegment()
        s.segment_id = cols["segment_id"][i].as_py()
        for name in ("K_ref", "tau_start", "tau_end", "tau_min", "tau_max"):
            setattr(s, name, cols[name][i].as_py())
        s.interp_type = cols["interp_type"][i].as_py()
        s.ndim = cols["ndim"][i].as_py()
        lst = lambda name, dt: np.asarray(cols[name][i].values.to_numpy(zero_copy_only=False), dtype=dt)
        s.domain_lo = lst("domain_lo", np.float64).tolist()
        s.domain_hi = lst("domain_hi", np.float64).tolist()
        s.num_pts = lst("num_pts", np.int32).tolist()
        s.grids = [g for g in (lst(f"grid_{d}", np.float64) for d in range(min(s.ndim, 4))) if g.size]
        s.knots = [k for k in (lst(f"knots_{d}", np.float64) for d in range(min(s.ndim, 4))) if k.size]
        s.values = lst("values", np.float64)
        stored = cols["checksum_values"][i].as_py()
        if stored != segment_checksum(s):
            raise SerializationError(f"segment {s.segment_id} checksum mismatch")
        seg_crcs.append((s.segment_id, stored))
        data.segments.append(s)
    if _parse_uint(meta("mango.metadata_checksum")) != metadata_checksum(data, seg_crcs):
        raise SerializationError("metadata checksum mismatch")
    return data


# ------------------------------------------------- table <-> data model --

def to_data(table) -> PriceTableData:
    """to_data for the standard EEP B-spline table (to_data.cpp,
    extract_segments.hpp:38-58, 89-110): one segment with the table's
    K_ref, tau range [0, tau_max], the spline's grids, knots and
    coefficients."""
    if not table.eep:
        raise SerializationError("only the EEP B-spline table (bspline_4d) is serialisable")
    pkg = _pkg()
    lib = pkg.library()
    s = lib.mango_gpu_price_table_spline(table._t)
    sizes = np.zeros(4, np.int64)
    err = pkg.MangoError()
    if lib.mango_gpu_bspline4d_export(s, sizes.ctypes.data_as(ctypes.c_void_p), None, 0, None, 0,
                                      ctypes.byref(err)) != pkg.MANGO_OK:
        raise pkg.EngineError(err.message.decode(errors="replace"))
    grids = np.zeros(int(sizes.sum()))
    coeffs = np.zeros(int(np.prod(sizes)))
    if lib.mango_gpu_bspline4d_export(s, sizes.ctypes.data_as(ctypes.c_void_p), grids.ctypes.data_as(ctypes.c_void_p),
                                      grids.size, coeffs.ctypes.data_as(ctypes.c_void_p), coeffs.size,
                                      ctypes.byref(err)) != pkg.MANGO_OK:
        raise pkg.EngineError(err.message.decode(errors="replace"))
    n = ctypes.c_uint64()
    lib.mango_gpu_bspline4d_knots(s, None, 0, ctypes.byref(n))
    knots = np.zeros(n.value)
    lib.mango_gpu_bspline4d_knots(s, knots.ctypes.data_as(ctypes.c_void_p), n.value, ctypes.byref(n))
    axes = np.split(grids, np.cumsum(sizes)[:-1])
    kax = np.split(knots, np.cumsum(sizes + 4)[:-1])
    b = np.asarray(table.bounds).reshape(4, 2)
    seg = PriceTableSegment(segment_id=0, K_ref=table.K_ref, tau_start=0.0, tau_end=float(b[1, 1]),
                            tau_min=float(b[1, 0]), tau_max=float(b[1, 1]), interp_type="bspline", ndim=4,
                            domain_lo=[float(a[0]) for a in axes], domain_hi=[float(a[-1]) for a in axes],
                            num_pts=[int(a.size) for a in axes], grids=[a.copy() for a in axes],
                            knots=[k.copy() for k in kax], values=coeffs)
    return PriceTableData(surface_type=SURFACE_BSPLINE_4D, option_type=int(table.option_type),
                          dividend_yield=table.dividend_yield, maturity=float(b[1, 1]),
                          bounds_m_min=float(b[0, 0]), bounds_m_max=float(b[0, 1]), bounds_tau_min=float(b[1, 0]),
                          bounds_tau_max=float(b[1, 1]), bounds_sigma_min=float(b[2, 0]),
                          bounds_sigma_max=float(b[2, 1]), bounds_rate_min=float(b[3, 0]),
                          bounds_rate_max=float(b[3, 1]), segments=[seg])


def from_data(data: PriceTableData, engine=None):
    """from_data<BSplineLeaf> (from_data.cpp:53-79, reconstruct.hpp:41-71,
    136-148): one "bspline" segment of dimension 4 whose knots are the
    clamped cubic knots of its grids, reconstructed as the device table."""
    pkg = _pkg()
    if data.surface_type != SURFACE_BSPLINE_4D:
        raise SerializationError(f"surface type {data.surface_type!r} is not {SURFACE_BSPLINE_4D!r}")
    if len(data.segments) != 1:
        raise SerializationError("bspline_4d holds exactly one segment")
    seg = data.segments[0]
    if seg.interp_type != "bspline" or seg.ndim != 4 or len(seg.grids) != 4 or len(seg.knots) != 4:
        raise SerializationError("segment is not a 4D B-spline")
    if not np.isfinite(seg.K_ref) or seg.K_ref <= 0.0:
        raise SerializationError("K_ref")
    sizes = [np.asarray(g).size for g in seg.grids]
    if np.asarray(seg.values).size != int(np.prod(sizes)):
        raise SerializationError("coefficient count does not match the grids")
    b = [(data.bounds_m_min, data.bounds_m_max), (data.bounds_tau_min, data.bounds_tau_max),
         (data.bounds_sigma_min, data.bounds_sigma_max), (data.bounds_rate_min, data.bounds_rate_max)]
    for d, (lo, hi) in enumerate(b):
        g = np.asarray(seg.grids[d], np.float64)
        if not (lo < hi) or lo != g[0] or hi != g[-1]:
            # make_bspline_surface takes its bounds from the grids
            raise SerializationError(f"bounds of axis {d} are not its grid's range")
    eng = engine or pkg.default_engine()
    table = eng.price_table_create([np.asarray(g, np.float64) for g in seg.grids],
                                   np.asarray(seg.values, np.float64).reshape(sizes), seg.K_ref,
                                   data.dividend_yield, data.option_type, eep=True)
    # The device spline derives its knots from the grids; a file whose knots
    # differ describes another spline.
    got = np.split(table.spline_knots(), np.cumsum(np.array(sizes) + 4)[:-1])
    for d in range(4):
        if not np.array_equal(got[d], np.asarray(seg.knots[d], np.float64)):
            table.close()
            raise SerializationError(f"knots of axis {d} are not the clamped knots of its grid")
    return table
