// grid_host.hpp -- host-side grid selection and generation for the march.
//
// The spatial grid must be the reference's grid to the last bit (prices are
// compared at 1e-9 relative and the auto grid's time-step count is a ceil()
// of a grid spacing), so this file evaluates the reference's formulas in the
// reference's order with the host libm:
//   estimate_pde_grid            src/option/grid_spec_types.cpp:37-118
//   GridSpec::multi_sinh_spaced  src/pde/core/grid.hpp:110-160 (validation)
//   merge_nearby_clusters        src/pde/core/grid.hpp:191-234
//   enforce_monotonicity         src/pde/core/grid.hpp:240-262
//   GridSpec::generate           src/pde/core/grid.hpp:364-498
// Compiled with -ffp-contract=off so no fused multiply-add appears that the
// reference does not write.
#pragma once
#include <cstdint>
#include <vector>

namespace mgpu {

// GridAccuracyParams (src/option/grid_spec_types.hpp:23-53).
struct Accuracy {
  double n_sigma = 5.0;
  double alpha = 0.0;  // filled by default_accuracy(): 2*asinh(5/sqrt 2)
  double tol = 1e-2;
  double c_t = 0.75;
  int64_t min_points = 100;
  int64_t max_points = 1200;
  int64_t max_steps = 5000;
};
Accuracy default_accuracy();

// GridSpec value type (src/pde/core/grid.hpp:50-183).
struct GridSpec {
  enum Type : int32_t { Uniform = 0, Log = 1, Sinh = 2, MultiSinh = 3 };
  int32_t type = Uniform;
  int32_t n_clusters = 0;
  double x_min = 0, x_max = 0;
  int64_t n = 0;
  double concentration = 1.0;
  double c_center[4] = {0, 0, 0, 0};
  double c_alpha[4] = {0, 0, 0, 0};
  double c_weight[4] = {0, 0, 0, 0};
};

// estimate_pde_grid for a constant-rate, continuous-dividend option.
// Writes the spec and the auto step count (needs one grid generation, like
// the reference, to find the smallest spacing).
void estimate_grid(double spot, double strike, double maturity, double sigma,
                   const Accuracy& acc, GridSpec* spec, int64_t* n_time,
                   std::vector<double>* scratch);

// The spatial GridSpec of estimate_grid alone, for callers that give the
// step count themselves.
void estimate_spec(double spot, double strike, double maturity, double sigma,
                   const Accuracy& acc, GridSpec* spec);

// Same, with caller-provided scratch of `cap` doubles (no heap use); a grid
// larger than cap is not generated and *n_time is left at 0.
void estimate_grid(double spot, double strike, double maturity, double sigma,
                   const Accuracy& acc, GridSpec* spec, int64_t* n_time, double* scratch,
                   int64_t cap);

// TimeDomain::with_mandatory_points(t0, t1, dt, mandatory): the explicit
// points (n_steps + 1 of them) in *pts, or *pts empty when no mandatory
// point falls inside (t0, t1), the domain then being from_n_steps with
// *n_steps = ceil((t1 - t0) / dt).
void time_points(double t0, double t1, double dt, std::vector<double> mandatory,
                 std::vector<double>* pts, int64_t* n_steps);

// estimate_pde_grid for an option with discrete dividends: taus are the
// times to expiry of its dividends inside (0, T) (any amount), max_dk the
// largest amount / strike among them.  The lower bound is widened for the
// dividend shift; the time domain is from_n_steps when taus is empty (tp
// cleared), else with_mandatory_points at the capped step (points in *tp).
void estimate_grid_div(double spot, double strike, double maturity, double sigma,
                       const Accuracy& acc, const std::vector<double>& taus, double max_dk,
                       GridSpec* spec, int64_t* n_time, std::vector<double>* tp,
                       std::vector<double>* scratch);

// GridSpec::sinh_spaced / uniform factories (no validation; callers check).
GridSpec sinh_spec(double x_min, double x_max, int64_t n, double alpha);
GridSpec uniform_spec(double x_min, double x_max, int64_t n);

// GridSpec::generate into x[0..spec.n).
void generate_grid(const GridSpec& spec, double* x);

}  // namespace mgpu
