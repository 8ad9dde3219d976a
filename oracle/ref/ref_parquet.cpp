// Test infrastructure only: a thin extern "C" driver over the UNMODIFIED
// reference Parquet writer and reader (src/option/table/parquet/
// parquet_io.cpp), compiled against the Arrow C++ libraries and headers that
// pyarrow bundles (the reference's own Arrow dependency is not installed
// here).  Used by tests/golden/make_golden.py to write a table file with the
// reference, and by tests/test_persistence.py (in the container that has the
// reference tree) to read the engine's files with the reference.
#include "mango/option/table/parquet/parquet_io.hpp"

#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

using namespace mango;

extern "C" {

// One-segment "bspline_4d" PriceTableData (the layout to_data writes for the
// standard EEP table): sizes[4], grids and knots concatenated per axis,
// values = the coefficients; scalars as named.  compression 0 none, 1
// snappy, 2 zstd.  Returns 0 on success.
int32_t ref_parquet_write_bspline4d(const char* path, const int64_t* sizes, const double* grids,
                                    const double* knots, const double* values, double K_ref,
                                    int32_t is_put, double dividend_yield, double maturity,
                                    const double* bounds8, const double* domain_lo4,
                                    const double* domain_hi4, double tau_start, double tau_end,
                                    double tau_min, double tau_max, int64_t n_pde_solves,
                                    double precompute_s, int32_t compression) {
  PriceTableData d;
  d.surface_type = "bspline_4d";
  d.option_type = is_put ? OptionType::PUT : OptionType::CALL;
  d.dividend_yield = dividend_yield;
  d.maturity = maturity;
  d.bounds_m_min = bounds8[0];
  d.bounds_m_max = bounds8[1];
  d.bounds_tau_min = bounds8[2];
  d.bounds_tau_max = bounds8[3];
  d.bounds_sigma_min = bounds8[4];
  d.bounds_sigma_max = bounds8[5];
  d.bounds_rate_min = bounds8[6];
  d.bounds_rate_max = bounds8[7];
  d.n_pde_solves = static_cast<size_t>(n_pde_solves);
  d.precompute_time_seconds = precompute_s;
  PriceTableData::Segment s;
  s.segment_id = 0;
  s.K_ref = K_ref;
  s.tau_start = tau_start;
  s.tau_end = tau_end;
  s.tau_min = tau_min;
  s.tau_max = tau_max;
  s.interp_type = "bspline";
  s.ndim = 4;
  size_t go = 0, ko = 0, total = 1;
  for (int k = 0; k < 4; ++k) {
    s.domain_lo.push_back(domain_lo4[k]);
    s.domain_hi.push_back(domain_hi4[k]);
    s.num_pts.push_back(static_cast<int32_t>(sizes[k]));
    s.grids.emplace_back(grids + go, grids + go + sizes[k]);
    s.knots.emplace_back(knots + ko, knots + ko + sizes[k] + 4);
    go += static_cast<size_t>(sizes[k]);
    ko += static_cast<size_t>(sizes[k]) + 4;
    total *= static_cast<size_t>(sizes[k]);
  }
  s.values.assign(values, values + total);
  d.segments.push_back(std::move(s));
  ParquetWriteOptions o;
  o.compression = compression == 0   ? ParquetCompression::NONE
                  : compression == 1 ? ParquetCompression::SNAPPY
                                     : ParquetCompression::ZSTD;
  return write_parquet(d, path, o) ? 0 : 1;
}

// Read a file with the reference reader.  Fills scalars8 = {option_type (1
// put), dividend_yield, maturity, n_pde_solves, precompute_time_seconds,
// segments, K_ref of segment 0, ndim of segment 0}, bounds8, sizes4 and up
// to cap values of segment 0; surface type into type_out (64 bytes).
// Returns 0 on success, 1 when the reader rejects the file.
int32_t ref_parquet_read(const char* path, char* type_out, double* scalars8, double* bounds8,
                         int64_t* sizes4, double* values, int64_t cap) {
  auto r = read_parquet(path);
  if (!r) return 1;
  const PriceTableData& d = *r;
  std::strncpy(type_out, d.surface_type.c_str(), 63);
  type_out[63] = 0;
  scalars8[0] = d.option_type == OptionType::PUT ? 1.0 : 0.0;
  scalars8[1] = d.dividend_yield;
  scalars8[2] = d.maturity;
  scalars8[3] = static_cast<double>(d.n_pde_solves);
  scalars8[4] = d.precompute_time_seconds;
  scalars8[5] = static_cast<double>(d.segments.size());
  scalars8[6] = d.segments.empty() ? 0.0 : d.segments[0].K_ref;
  scalars8[7] = d.segments.empty() ? 0.0 : static_cast<double>(d.segments[0].ndim);
  const double b[8] = {d.bounds_m_min,     d.bounds_m_max,     d.bounds_tau_min,
                       d.bounds_tau_max,   d.bounds_sigma_min, d.bounds_sigma_max,
                       d.bounds_rate_min,  d.bounds_rate_max};
  for (int k = 0; k < 8; ++k) bounds8[k] = b[k];
  if (!d.segments.empty()) {
    const auto& s = d.segments[0];
    for (size_t k = 0; k < 4 && k < s.num_pts.size(); ++k) sizes4[k] = s.num_pts[k];
    const int64_t n = std::min<int64_t>(cap, static_cast<int64_t>(s.values.size()));
    for (int64_t i = 0; i < n; ++i) values[i] = s.values[static_cast<size_t>(i)];
  }
  return 0;
}

}  // extern "C"
