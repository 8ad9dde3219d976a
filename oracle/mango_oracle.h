/* mango_oracle.h -- CPU restatement of the reference's American-option hot
 * path, in plain C.  TEST INFRASTRUCTURE ONLY: tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline leg may call it, as the checker; the product
 * (mango-option_gb300/) never links, loads or calls it.
 *
 * Every function cites the reference file:line it restates.  Arithmetic order
 * follows the reference expression by expression (fma where the reference
 * writes std::fma, plain ops elsewhere, compiled with -ffp-contract=off).
 * The reference compiles its stencil loops with target_clones
 * (avx2/avx512f), so its own last bits depend on the CPU it runs on; this
 * port agrees with it to ~1e-12 relative on prices and bit for bit on grids.
 * That is pinned by tests/test_oracle_pins.py against golden vectors produced
 * by the reference itself (tests/golden/make_golden.py).
 */
#ifndef MANGO_ORACLE_H
#define MANGO_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* GridAccuracyParams (src/option/grid_spec_types.hpp:23-53). */
typedef struct {
  double n_sigma;
  double alpha;
  double tol;
  double c_t;
  int64_t min_spatial_points;
  int64_t max_spatial_points;
  int64_t max_time_steps;
} mo_accuracy;

/* GridSpec (src/pde/core/grid.hpp:50-183): type 0 uniform, 1 log, 2 sinh,
 * 3 multi-sinh.  Clusters are stored after merge_nearby_clusters. */
typedef struct {
  int32_t type;
  int32_t n_clusters;
  double x_min, x_max;
  int64_t n_points;
  double concentration;
  double c_center[4], c_alpha[4], c_weight[4];
} mo_grid_spec;

void mo_default_accuracy(mo_accuracy* acc);

/* estimate_pde_grid (src/option/grid_spec_types.cpp:37-118), continuous
 * dividends only.  Returns the spec and the number of time steps. */
int32_t mo_estimate_grid(double spot, double strike, double maturity, double sigma,
                         const mo_accuracy* acc, mo_grid_spec* spec, int64_t* n_time);

/* GridSpec::generate (src/pde/core/grid.hpp:364-498). */
int32_t mo_generate_grid(const mo_grid_spec* spec, double* x);

/* One American option: AmericanOptionSolver::solve
 * (src/option/american_option.cpp:354-438) on grid x[0..nx) with nt steps,
 * then AmericanOptionResult value/delta/gamma/theta
 * (src/option/american_option_result.cpp:25-121).
 * out4 = {value, delta, gamma, theta}.  u_final/u_prev may be NULL.
 * Returns 0 ok, 5 linear-solve failure, 1 validation failure. */
int32_t mo_price_on_grid(double spot, double strike, double maturity, double sigma,
                         double rate, double dividend_yield, int32_t is_put,
                         const double* x, int64_t nx, int64_t nt, int32_t rannacher,
                         double* out4, double* u_final, double* u_prev);

/* Forward-mode derivative of mo_price_on_grid (Rannacher start) along
 * volatility, rate and dividend yield, the primal's active obstacle set and
 * deep-ITM lock rows frozen; dV/dK from the final spline on the
 * strike-independent grid.  out6 = {value, delta, dV/dsigma, dV/drate,
 * dV/dq, dV/dK}.  The checker of the GPU tangent march.  Returns as
 * mo_price_on_grid. */
int32_t mo_price_tangent_on_grid(double spot, double strike, double maturity, double sigma,
                                 double rate, double dividend_yield, int32_t is_put,
                                 const double* x, int64_t nx, int64_t nt, double* out6);

/* Batch over options, each with its own grid rule (nx > 0: estimate_pde_grid
 * with min = max = nx, and nt steps; nx == 0: default auto grid).  OpenMP over
 * options when compiled with -fopenmp, n_threads <= 0 means all.
 * out_dims (nullable) = {nx, nt} per option. */
int32_t mo_price_batch(int64_t n, const double* S, const double* K, const double* T,
                       const double* sigma, const double* r, const double* q,
                       const int32_t* is_put, const int64_t* nx, const int64_t* nt,
                       int32_t rannacher, int32_t n_threads, double* out4,
                       int64_t* out_dims, int32_t* status);

/* FDM implied volatility by Brent (src/option/iv_solver.cpp:133-242,
 * src/math/root_finding.hpp:145-302) with a fixed per-quote grid built by the
 * grid rule at grid_sigma[i].  out3 = {iv, iterations, final_error}.
 * status: 0 ok, 1 validation, 11 max-iter, 10 bracket, 12 numerical. */
int32_t mo_iv_batch(int64_t n, const double* S, const double* K, const double* T,
                    const double* r, const double* q, const int32_t* is_put,
                    const double* price, const double* grid_sigma, const int64_t* nx,
                    const int64_t* nt, int32_t n_threads, double* out3, int32_t* status);

/* Natural cubic spline evaluation helpers (src/math/cubic_spline_solver.hpp),
 * exported for tests: value and first derivative of the spline through
 * (x, y) at xe. */
int32_t mo_spline_eval(const double* x, const double* y, int64_t n, double xe,
                       double* value, double* deriv);

/* Projected Thomas (src/math/thomas_solver.hpp:321-420); returns 0 ok,
 * 1 singular.  ws must hold 2n doubles. */
int32_t mo_thomas_projected(const double* lower, const double* diag, const double* upper,
                            const double* rhs, const double* psi, double* x, int64_t n,
                            double* ws);

/* clamped_knots_cubic (src/math/bspline/bspline_basis.hpp:47-91): n + 4 knots. */
void mo_clamped_knots(const double* x, int64_t n, double* t);

/* BSplineND<double,4>::eval (src/math/bspline/bspline_nd.hpp:133-157,
 * 314-346) with knots from mo_clamped_knots on each axis.  grids: the four
 * axes concatenated (sizes[d] points each); coeffs row-major; q: n x 4. */
int32_t mo_bspline4d_eval(const int64_t* sizes, const double* grids, const double* coeffs,
                          const double* q, int64_t n, double* out);

#ifdef __cplusplus
}
#endif
#endif
