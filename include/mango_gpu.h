/* mango_gpu.h -- C ABI of the GB300 (sm_103a) batched American-option engine.
 *
 * Additive to the reference's stable C ABI (src/ffi/mango_c_api.h): the value
 * types below are the reference's own (same names, same layout, asserted at
 * the end of this file), so a caller that already fills MangoPricingParams /
 * MangoIvQuery for mango_price_american / mango_solve_iv passes the same
 * arrays here.  Include src/ffi/mango_c_api.h FIRST when using both headers;
 * its include guard then suppresses the duplicate type definitions below.
 *
 * Conventions follow the reference ABI (src/ffi/mango_c_api.h:16-28,
 * src/ffi/mango_c_api.cpp:23-31, 354-366, 523-576): functions return a
 * MangoStatus, an optional MangoError* receives a code and a 256-byte
 * message, batch calls never abort the whole batch (a per-slot status plus a
 * failed count), and no exception crosses the boundary.  Every batch call is
 * synchronous with respect to the caller's host buffers.
 *
 * Rates and dividends: the American-pricing batch calls
 * (mango_gpu_price_american_batch, _batch_shared, mango_gpu_batch_create)
 * and the FDM implied-volatility calls accept the reference's yield curves
 * (tenor_points, validated as YieldCurve::from_points does) and discrete
 * dividends (validated as validate_pricing_params / validate_iv_query do)
 * and march those options on a kernel whose stage matrices follow r(t), the
 * mandatory dividend times and the dividend shift; so do the frozen-grid
 * Greeks.  The other entry points (table sweep, table queries, the
 * no-allocation batch) take
 * constant rates and continuous dividend yields only and reject the rest per
 * slot with MANGO_ERR_VALIDATION and a message naming the unsupported
 * feature.
 */
#ifndef MANGO_GPU_H
#define MANGO_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#ifndef MANGO_C_API_H
/* ---- value types shared with src/ffi/mango_c_api.h:16-139 ---- */
typedef int32_t MangoStatus;
#define MANGO_OK 0
#define MANGO_ERR_VALIDATION 1
#define MANGO_ERR_ARBITRAGE 2
#define MANGO_ERR_NO_CONVERGENCE 3
#define MANGO_ERR_BRACKETING 4
#define MANGO_ERR_SOLVER 5

typedef int32_t MangoOptionType;
#define MANGO_CALL 0
#define MANGO_PUT 1

typedef struct { int32_t code; char message[256]; } MangoError;
typedef struct { double calendar_time; double amount; } MangoDividend;
typedef struct { double tenor; double log_discount; } MangoTenorPoint;

typedef struct {
  double spot;
  double strike;
  double maturity;
  double dividend_yield;
  double volatility;
  double rate_const;
  const MangoTenorPoint* tenor_points;
  uint64_t n_tenor_points;
  const MangoDividend* dividends;
  uint64_t n_dividends;
  MangoOptionType option_type;
} MangoPricingParams;

typedef struct {
  double spot;
  double strike;
  double maturity;
  double dividend_yield;
  double market_price;
  double rate_const;
  const MangoTenorPoint* tenor_points;
  uint64_t n_tenor_points;
  const MangoDividend* dividends;
  uint64_t n_dividends;
  MangoOptionType option_type;
} MangoIvQuery;

typedef struct {
  double implied_vol;
  uint64_t iterations;
  double final_error;
  double vega;
  int32_t has_vega;
  int32_t used_rate_approximation;
} MangoIvSuccess;

typedef struct { double brent_tol_abs; int32_t max_iter; } MangoIvConfig;

typedef struct {
  uint64_t max_iter;
  double tolerance;
  double sigma_min;
  double sigma_max;
  double vega_threshold;
} MangoInterpSolverConfig;

typedef struct {
  int32_t status;
  MangoIvSuccess success;
} MangoIvBatchSlot;
#endif /* MANGO_C_API_H */

/* ---- engine-specific types ---- */

/* Grid selection for one option, the C form of the reference's PDEGridSpec
 * variant (src/option/grid_spec_types.hpp:55-61):
 *   MANGO_GPU_GRID_AUTO     estimate_pde_grid(params, GridAccuracyParams{})
 *                           (src/option/grid_spec_types.cpp:37-118);
 *   MANGO_GPU_GRID_FIXED_N  estimate_pde_grid with min_spatial_points ==
 *                           max_spatial_points == n_space, then
 *                           PDEGridConfig{spec, n_time}: the reference's own
 *                           sinh-clustered grid at a pinned size; n_time == 0
 *                           keeps the estimate's own step count (the
 *                           GridAccuracyParams alternative of PDEGridSpec);
 *   MANGO_GPU_GRID_SINH     PDEGridConfig{GridSpec::sinh_spaced(x_min, x_max,
 *                           n_space, alpha), n_time};
 *   MANGO_GPU_GRID_UNIFORM  PDEGridConfig{GridSpec::uniform(x_min, x_max,
 *                           n_space), n_time};
 *   MANGO_GPU_GRID_FIXED_N_AT_VOL  as FIXED_N, but the grid is sized with the
 *                           volatility given in `alpha` instead of the
 *                           option's own -- a fixed per-quote PDEGridConfig
 *                           for implied-volatility solves, where the
 *                           volatility is the unknown.
 * x_min/x_max are log-moneyness ln(S/K). */
#define MANGO_GPU_GRID_AUTO 0
#define MANGO_GPU_GRID_FIXED_N 1
#define MANGO_GPU_GRID_SINH 2
#define MANGO_GPU_GRID_UNIFORM 3
#define MANGO_GPU_GRID_FIXED_N_AT_VOL 4
typedef struct {
  int32_t kind;
  int32_t reserved;
  int64_t n_space;
  int64_t n_time;
  double x_min;
  double x_max;
  double alpha;
} MangoGpuGrid;

/* TRBDF2Config subset honoured by the march (src/pde/core/trbdf2_config.hpp:
 * 18-49): gamma (default 2 - sqrt 2) and the Rannacher start-up flag
 * (default on, as AmericanOptionSolver sets it). Pass NULL for defaults. */
typedef struct {
  double gamma;
  int32_t rannacher_startup;
  int32_t reserved;
} MangoGpuTrbdf2;

/* Per-option result: AmericanOptionResult::value/delta/gamma/theta
 * (src/option/american_option_result.cpp:25-121).  status is a MangoStatus;
 * n_space/n_time report the grid the option was solved on. */
typedef struct {
  double value;
  double delta;
  double gamma;
  double theta;
  int32_t status;
  int32_t n_space;
  int32_t n_time;
  int32_t reserved;
} MangoGpuAmericanOut;

/* Opaque engine context: one CUDA device, one stream, grow-only device
 * buffers reused across calls.  Not thread-safe: use one context per host
 * thread (contexts on the same device share nothing). */
typedef struct MangoGpuContext MangoGpuContext;

/* Create a context on CUDA device `device`.  Fails (MANGO_ERR_SOLVER) when
 * the device is absent or is not an sm_103 part this library was built for. */
MangoStatus mango_gpu_context_create(int32_t device, MangoGpuContext** out,
                                     MangoError* err);
void mango_gpu_context_destroy(MangoGpuContext* ctx);

/* Batched American pricing with Greeks.  Replaces a loop of
 * mango_price_american (src/ffi/mango_c_api.h:141-150) and the C++
 * BatchAmericanOptionSolver::solve_batch regular path
 * (src/option/american_option_batch.cpp:384-518), which has no C export.
 * grids: NULL => MANGO_GPU_GRID_AUTO for every option; else one per option,
 * or a single entry applied to all when grid_stride == 0.
 * out: n slots.  *out_failed (nullable) = slots whose status != MANGO_OK.
 * Returns MANGO_OK unless the call itself could not run (bad pointers, CUDA
 * failure), in which case err says why and no slot is meaningful.
 * The call is synchronous.  Its device and pinned host buffers (up to 4 GB
 * of device state per batch) stay in the context for the next call; batches of 65,536 options or more run as 2 to
 * 4 chunks (at least 32,768 options each) on two internal streams, ordered
 * after the context's stream, so that the host preparation of a chunk
 * overlaps the device work of the one before. */
MangoStatus mango_gpu_price_american_batch(MangoGpuContext* ctx,
                                           const MangoPricingParams* params,
                                           uint64_t n, const MangoGpuGrid* grids,
                                           uint64_t grid_stride,
                                           const MangoGpuTrbdf2* trbdf2,
                                           MangoGpuAmericanOut* out,
                                           uint64_t* out_failed, MangoError* err);

/* BatchAmericanOptionSolver::solve_batch(params, use_shared_grid = true,
 * no setup callback, custom_grid) (src/option/american_option_batch.cpp:
 * 272-302).  With use_normalized != 0 and a batch that is_normalized_eligible
 * accepts (american_option_batch.cpp:26-107: one option type, positive spot
 * and strike, the first option's estimated grid no wider than 5.8 with
 * spacing <= 0.05 and margins >= max(0.35, 6 dx) around ln(S/K) of every
 * option), options are grouped by (volatility, rate, dividend yield,
 * maturity, type) within 1e-10, each group is solved once at S = K = 1 and
 * every option is read from its group's solution with its own spot and
 * strike (solve_normalized_chain, american_option_batch.cpp:313-382);
 * otherwise every option is marched on one grid shared by the batch
 * (solve_regular_batch, american_option_batch.cpp:384-518).
 * custom_grid: NULL => the shared grid is estimate_batch_pde_grid over the
 * batch (src/option/grid_spec_types.cpp:120-177; over the normalised group
 * option on the chain route); else it is resolved, any kind, for the first
 * option of the solve (the normalised group option on the chain route).
 * Options that fail validation do not shape the shared grid and are
 * reported MANGO_ERR_VALIDATION.  *out_route (nullable) = 1 when the chain
 * route ran, 0 otherwise.  Other arguments and returns as
 * mango_gpu_price_american_batch. */
MangoStatus mango_gpu_price_american_batch_shared(MangoGpuContext* ctx,
                                                  const MangoPricingParams* params, uint64_t n,
                                                  const MangoGpuGrid* custom_grid,
                                                  int32_t use_normalized,
                                                  const MangoGpuTrbdf2* trbdf2,
                                                  MangoGpuAmericanOut* out, uint64_t* out_failed,
                                                  int32_t* out_route, MangoError* err);

/* Batched FDM implied volatility: IVSolver::solve (src/option/iv_solver.cpp:
 * 133-242) with Brent (src/math/root_finding.hpp:145-302) for every quote,
 * the batch analogue of mango_solve_iv (src/ffi/mango_c_api.h:154-157) and
 * of IVSolver::solve_batch.  Each quote needs a grid that does not depend on
 * the unknown volatility: MANGO_GPU_GRID_FIXED_N_AT_VOL, _SINH or _UNIFORM
 * (the reference's IVSolverConfig.grid = PDEGridConfig); grid_stride as for
 * pricing.  config NULL or zero fields => brent_tol_abs 1e-6, max_iter 100.
 * Slot status: MANGO_OK, _VALIDATION, _ARBITRAGE (price outside
 * [intrinsic, upper bound]), _BRACKETING, _NO_CONVERGENCE, _SOLVER.  Each
 * evaluation re-prices the quotes still iterating on the device: the host
 * re-packs their trial points into full tiles (finished quotes leave the
 * working set), then one gather, setup, march, outputs and root-finder step
 * launch run on the context's stream.  After the call, mango_gpu_last_stats
 * reports options = quote evaluations (marches), tiles = evaluations (rounds
 * of those launches), algo_flops = their work, march_ms = device time of the
 * evaluations, prep_ms = host time of the re-packing, host_prep_ms =
 * validation and grid generation, total_ms = the whole call. */
MangoStatus mango_gpu_solve_iv_batch(MangoGpuContext* ctx, const MangoIvQuery* queries,
                                     uint64_t n, const MangoGpuGrid* grids, uint64_t grid_stride,
                                     const MangoIvConfig* config, MangoIvBatchSlot* out,
                                     uint64_t* out_failed, MangoError* err);

/* Root finders for mango_gpu_solve_iv_batch_method. */
enum {
  MANGO_GPU_IV_BRENT = 0,   /* the reference's Brent, iterate for iterate */
  MANGO_GPU_IV_SECANT = 1,  /* safeguarded secant, Brent fallback (below) */
  MANGO_GPU_IV_NEWTON = 2   /* coarse-grid Newton, own-grid secant (below) */
};

/* mango_gpu_solve_iv_batch with a choice of root finder.  MANGO_GPU_IV_BRENT
 * is mango_gpu_solve_iv_batch.  MANGO_GPU_IV_SECANT starts every quote at the
 * Black-Scholes implied volatility of its price, takes one Newton step along
 * the Black-Scholes vega, then secant steps kept inside the bracket seen so
 * far (bisection otherwise); it stops on the same test as Brent (|V - P| <
 * brent_tol_abs, or a bracket narrower than brent_tol_abs).  A quote not
 * settled within 10 evaluations, or whose root lies outside the Brent
 * bracket, is solved again from scratch by Brent, so failure statuses are
 * Brent's, with one exception: where V - P has no sign change over Brent's
 * bracket [0.01, upper] (Brent: MANGO_ERR_BRACKETING) but the secant reaches
 * |V - P| < brent_tol_abs inside it, the quote is reported settled at that
 * point.  Converged roots of the two methods differ by at most about
 * 2 brent_tol_abs / vega.  iterations = evaluations for secant-settled
 * quotes, Brent's count otherwise.
 *
 * MANGO_GPU_IV_NEWTON starts on a coarse grid of the quote's grid kind (2/5
 * of the space points, an eighth of the time steps): two Newton steps from
 * the Black-Scholes implied volatility with the exact discrete vega of that
 * grid (the forward-mode march of mango_gpu_price_american_vega_batch), whose
 * two vegas also give the curvature d(vega)/d(sigma).  On the quote's own
 * grid it then evaluates prices only: one step from the coarse root along the
 * coarse vega and curvature, then secant steps corrected by the curvature of
 * the last three values, kept inside the bracket seen so far.  The quote
 * settles when the secant step through its last two own-grid values is at
 * most 3e-6 in volatility, at that step's end (a volatility-space stop: the
 * error left is that step times the relative change of the slope over it),
 * or, where the objective is flat, on the reference's test |V - P| <
 * brent_tol_abs.  A quote not settled after 6 own-grid evaluations, or whose
 * slope is not positive, goes on with the k-section finder of
 * MANGO_GPU_IV_SECANT inside what Newton has bracketed (settling at |V - P|
 * below 1e-7 times the slope, or a bracket narrower than 1e-7, or, where two
 * points below brent_tol_abs show the objective flat, on the reference's
 * test), then Brent from scratch as that finder does.  Quotes with yield curves or discrete
 * dividends use the secant path.  iterations = coarse plus own-grid
 * evaluations for Newton-settled quotes; final_error = |V - P| at the last
 * evaluated point; has_vega = 1 and vega = the slope of that last secant
 * (dV/dsigma of the discrete objective over the last step) for quotes settled
 * by the secant stop.  No counterpart in the reference ABI. */
MangoStatus mango_gpu_solve_iv_batch_method(MangoGpuContext* ctx, const MangoIvQuery* queries,
                                            uint64_t n, const MangoGpuGrid* grids,
                                            uint64_t grid_stride, const MangoIvConfig* config,
                                            int32_t method, MangoIvBatchSlot* out,
                                            uint64_t* out_failed, MangoError* err);

/* Price-table PDE sweep: PriceTableBuilderND<4>::make_batch + solve_batch +
 * extract_tensor (src/option/table/bspline/bspline_builder.cpp:198-480).  One
 * American option per (volatility, rate) pair at spot = strike = K_ref and
 * maturity = the last maturity-axis point, marched with snapshots at the
 * maturity axis and resampled onto the log-moneyness axis by natural cubic
 * splines.  grid: NULL or MANGO_GPU_GRID_AUTO => GridAccuracyParams{} (one
 * shared grid); MANGO_GPU_GRID_SINH / _UNIFORM => PDEGridConfig, used as is
 * when it meets the reference's width / spacing limits, else the reference's
 * fallback (auto estimation pinned to n_space, per-slice grids through the
 * normalized-chain route).  tensor: nm*ntau*nsig*nr doubles, layout
 * [moneyness][maturity][volatility][rate], normalized prices V/K_ref; NaN for
 * failed slices.  slice_dims (nullable): {n_space, n_time} per slice, slices
 * ordered volatility-major.  No C export in the reference (C++ API only). */
MangoStatus mango_gpu_price_table_sweep(MangoGpuContext* ctx, const double* moneyness,
                                        uint64_t nm, const double* maturity, uint64_t ntau,
                                        const double* volatility, uint64_t nsig,
                                        const double* rate, uint64_t nr, double K_ref,
                                        double dividend_yield, MangoOptionType option_type,
                                        const MangoGpuGrid* grid, double* tensor,
                                        int64_t* slice_dims, uint64_t* out_failed_slices,
                                        MangoError* err);

/* 4D cubic B-spline surface: BSplineND<double,4> (src/math/bspline/
 * bspline_nd.hpp:66-157) with knots from clamped_knots_cubic
 * (src/math/bspline/bspline_basis.hpp:47-91) on each axis grid.  grids:
 * the four axis grids concatenated (sizes[4] points each, 4..512, strictly
 * increasing); coeffs: row-major [axis0][axis1][axis2][axis3].  The surface
 * keeps knots, reciprocal tables and coefficients in device memory. */
typedef struct MangoGpuBSpline4D MangoGpuBSpline4D;
MangoStatus mango_gpu_bspline4d_create(MangoGpuContext* ctx, const double* grids,
                                       const int64_t* sizes, const double* coeffs,
                                       MangoGpuBSpline4D** out, MangoError* err);
void mango_gpu_bspline4d_destroy(MangoGpuBSpline4D* surface);
/* BSplineND::eval for n query points (queries: n x 4, host arrays; out: n). */
MangoStatus mango_gpu_bspline4d_eval(MangoGpuBSpline4D* surface, const double* queries,
                                     uint64_t n, double* out, MangoError* err);
/* Same with device-resident queries and output, enqueued on the context's
 * stream without waiting. */
MangoStatus mango_gpu_bspline4d_eval_device(MangoGpuBSpline4D* surface, const double* d_queries,
                                            uint64_t n, double* d_out, MangoError* err);
/* The packed knot vectors (axis 0..3, sizes[d] + 4 each), for inspection. */
MangoStatus mango_gpu_bspline4d_knots(const MangoGpuBSpline4D* surface, double* out, uint64_t cap,
                                      uint64_t* n_out);
/* The surface's data for serialisation (BSplineND grid(d) / coefficients(),
 * src/option/table/serialization/extract_segments.hpp:38-58): sizes[4], the
 * packed axes (sum of sizes doubles; NULL to skip) and the coefficients in
 * row-major order (product of sizes doubles, copied from the device; NULL to
 * skip). */
MangoStatus mango_gpu_bspline4d_export(const MangoGpuBSpline4D* surface, int64_t* sizes,
                                       double* grids, uint64_t grid_cap, double* coeffs,
                                       uint64_t coeff_cap, MangoError* err);

/* CRC64::update (src/support/crc64.hpp): reflected ECMA-182 polynomial
 * 0xC96C5795D7870F42 over n bytes from crc (0 to start), no final
 * inversion; the checksum of the Parquet price-table format.  Host only. */
uint64_t mango_gpu_crc64_update(uint64_t crc, const void* data, uint64_t n);

/* Separable collocation fit: BSplineNDSeparable<double,4>::fit
 * (src/math/bspline/bspline_nd_separable.hpp:153-384) with
 * BSplineCollocation1D (src/math/bspline/bspline_collocation.hpp:326-390):
 * coefficients whose BSplineND interpolates values (row-major, same layout
 * as coeffs) at the grid points.  Axes 3, 2, 1, 0 in turn; every slice along
 * an axis solves the axis's cubic collocation system (banded LU with partial
 * pivoting, factored once per axis) and is accepted when max |B c - f| <=
 * tolerance (0 => 1e-6, BSplineNDSeparableConfig).  A rejected slice keeps
 * its input values and counts in failed_slices; any failure makes the call
 * return MANGO_ERR_SOLVER ("fitting failed"), as the reference's fit does.
 * NaN or infinite values: MANGO_ERR_VALIDATION.  condition[d] is the exact
 * 1-norm condition number of the axis's collocation matrix (the reference
 * reports LAPACK dgbcon's estimate of it). */
typedef struct {
  double max_residual[4];
  double condition[4];
  uint64_t failed_slices[4];
} MangoGpuFitStats;
MangoStatus mango_gpu_bspline4d_fit(MangoGpuContext* ctx, const double* grids,
                                    const int64_t* sizes, const double* values, double tolerance,
                                    double* coeffs, MangoGpuFitStats* stats, MangoError* err);

/* Price table: the reference's standard 4D B-spline price table
 * (make_bspline_surface, src/option/table/bspline/bspline_surface.cpp:9-37):
 * axes log-moneyness, maturity, volatility, rate; price(S, K, tau, sigma, r)
 * = max(0, spline(log(S/K), tau, sigma, r)) * K / K_ref (TransformLeaf,
 * src/option/table/transform_leaf.hpp:28-33) plus, when eep != 0, the
 * closed-form European price with the table's option type and dividend yield
 * (EEPLayer + AnalyticalEEP, src/option/table/eep/eep_layer.hpp:21-25).
 * Queries are clamped into the axes as BSplineND::eval clamps them. */
typedef struct MangoGpuPriceTable MangoGpuPriceTable;
/* From given spline coefficients (grids, sizes, coeffs as for
 * mango_gpu_bspline4d_create). */
MangoStatus mango_gpu_price_table_create(MangoGpuContext* ctx, const double* grids,
                                         const int64_t* sizes, const double* coeffs, double K_ref,
                                         double dividend_yield, MangoOptionType option_type,
                                         int32_t eep, MangoGpuPriceTable** out, MangoError* err);
/* Whole build on the device: PriceTableBuilderND<4>::build
 * (src/option/table/bspline/bspline_builder.cpp:140-196) = the sweep of
 * mango_gpu_price_table_sweep (same arguments), then, when eep != 0, the EEP
 * decomposition of the tensor (eep_decompose with AnalyticalEEP,
 * src/option/table/eep/eep_decomposer.hpp:60-80: entry = softplus floor of
 * K_ref V - European), then the fit (tolerance as for
 * mango_gpu_bspline4d_fit).  A build with failed PDE slices is refused
 * (MANGO_ERR_SOLVER), as the reference's strict default max_failure_rate = 0
 * refuses it; mango_gpu_price_table_build_ex takes the rate and repairs. */
MangoStatus mango_gpu_price_table_build(
    MangoGpuContext* ctx, const double* moneyness, uint64_t n_moneyness, const double* maturity,
    uint64_t n_maturity, const double* volatility, uint64_t n_volatility, const double* rate,
    uint64_t n_rate, double K_ref, double dividend_yield, MangoOptionType option_type,
    const MangoGpuGrid* grid, int32_t eep, double tolerance, MangoGpuPriceTable** out,
    MangoGpuFitStats* stats, uint64_t* out_failed_slices, MangoError* err);
/* mango_gpu_price_table_build with PriceTableBuilderND<4>'s failure handling
 * (src/option/table/bspline/bspline_builder.cpp:95-101, 773-959):
 * max_failure_rate in [0, 1] (PriceTableConfig, bspline_builder.hpp:101; 0 =
 * strict, the reference's default) bounds the fraction of (volatility, rate)
 * slices whose PDE solve failed; below it the swept tensor is repaired before
 * the EEP step and the fit -- maturities where a slice's resampling failed
 * are interpolated along tau, whole failed slices are copied from the
 * nearest valid slice in (volatility, rate) index distance -- and above it
 * the build fails (MANGO_ERR_SOLVER).  out_repaired (nullable, 2 entries):
 * whole slices and single maturity points repaired.
 * mango_gpu_price_table_build is this call with max_failure_rate = 0.  No
 * counterpart in the reference ABI. */
MangoStatus mango_gpu_price_table_build_ex(
    MangoGpuContext* ctx, const double* moneyness, uint64_t n_moneyness, const double* maturity,
    uint64_t n_maturity, const double* volatility, uint64_t n_volatility, const double* rate,
    uint64_t n_rate, double K_ref, double dividend_yield, MangoOptionType option_type,
    const MangoGpuGrid* grid, int32_t eep, double tolerance, double max_failure_rate,
    MangoGpuPriceTable** out, MangoGpuFitStats* stats, uint64_t* out_failed_slices,
    uint64_t* out_repaired, MangoError* err);
void mango_gpu_price_table_destroy(MangoGpuPriceTable* table);
/* The EEP step alone (the TensorTransformFn of the standard build,
 * eep_decompose with AnalyticalEEP over BSplineTensorAccessor,
 * src/option/table/bspline/bspline_tensor_accessor.hpp:16-56): tensor
 * [m][tau][sigma][r] of V/K_ref in, EEP in price units out, in place. */
MangoStatus mango_gpu_eep_decompose(MangoGpuContext* ctx, const double* moneyness,
                                    uint64_t n_moneyness, const double* maturity,
                                    uint64_t n_maturity, const double* volatility,
                                    uint64_t n_volatility, const double* rate, uint64_t n_rate,
                                    double K_ref, double dividend_yield,
                                    MangoOptionType option_type, double* tensor, MangoError* err);
/* The table's spline (owned by the table): eval / knots as above. */
MangoGpuBSpline4D* mango_gpu_price_table_spline(MangoGpuPriceTable* table);
/* K_ref, dividend yield, option type, eep flag and the axis bounds
 * (m, tau, sigma, rate: min, max); any output may be NULL. */
MangoStatus mango_gpu_price_table_info(const MangoGpuPriceTable* table, double* K_ref,
                                       double* dividend_yield, int32_t* option_type, int32_t* eep,
                                       double* bounds8);
/* AnyPriceTable::price (src/option/price_table_factory.cpp:746-751) for n
 * parameter records (host arrays).  Constant rates only: a record with
 * tenor points prices as NaN. */
MangoStatus mango_gpu_price_table_price(MangoGpuPriceTable* table, const MangoPricingParams* params,
                                        uint64_t n, double* out, MangoError* err);
/* Same with device-resident records and output, enqueued without waiting. */
MangoStatus mango_gpu_price_table_price_device(MangoGpuPriceTable* table,
                                               const MangoPricingParams* d_params, uint64_t n,
                                               double* d_out, MangoError* err);
/* AnyPriceTable::vega (EEPLayer::vega over TransformLeaf::vega,
 * src/option/table/eep/eep_layer.hpp:27-31, transform_leaf.hpp:35-47): the
 * spline's analytic partial along the volatility axis times K/K_ref where
 * the spline value is positive, plus the closed-form European vega when
 * the table has EEP.  Constant rates only (NaN otherwise). */
MangoStatus mango_gpu_price_table_vega(MangoGpuPriceTable* table, const MangoPricingParams* params,
                                       uint64_t n, double* out, MangoError* err);

/* The table's delta, gamma, theta and rho for n records: the batch analogue
 * of mango_price_table_delta / _gamma / _theta / _rho
 * (src/ffi/mango_c_api.cpp:652-682, greek_call at 272-300).  Each record is
 * validated first as AnyPriceTable::validate_pricing_params does
 * (src/option/price_table_factory.cpp:700-745: positive finite inputs, the
 * table's option type and dividend yield within 1e-10, every coordinate
 * inside the table's axis ranges; constant rates only), then EEPLayer::greek
 * / gamma (src/option/table/eep/eep_layer.hpp:33-76) over the analytic spline
 * partials.  out4[4i .. 4i+3] = {delta, gamma, theta, rho}; a record that
 * fails validation gets NaN there and MANGO_ERR_VALIDATION in status[i]
 * (status may be NULL), and the call returns MANGO_ERR_VALIDATION with the
 * count and the first failing index in err.  The other records are still
 * computed. */
MangoStatus mango_gpu_price_table_greeks(MangoGpuPriceTable* table, const MangoPricingParams* params,
                                         uint64_t n, double* out4, int32_t* status,
                                         MangoError* err);

/* Interpolated implied volatility on the table:
 * InterpolatedIVSolver::solve_batch (src/option/interpolated_iv_solver.hpp:
 * 427-560), the batch analogue of mango_interp_iv_solve_batch
 * (src/ffi/mango_c_api.cpp:523-576).  Per quote: the reference's checks
 * (option type and dividend yield must match the table; validate_iv_query),
 * the adaptive volatility bracket, the axis-range check, the vega pre-check
 * at volatilities 0.10 / 0.25 / 0.50 against vega_threshold, then Brent on
 * table price - market price.  config NULL => the reference defaults
 * (max_iter 50, tolerance 1e-6, sigma 0.01 .. 3.0, vega_threshold 1e-4);
 * fields are applied verbatim otherwise.  Slot statuses follow the
 * reference's map_iv_error (mango_c_api.cpp:124-141): range and
 * type/dividend mismatches MANGO_ERR_VALIDATION, vega too small
 * MANGO_ERR_SOLVER. */
MangoStatus mango_gpu_price_table_iv_batch(MangoGpuPriceTable* table,
                                           const MangoInterpSolverConfig* config,
                                           const MangoIvQuery* queries, uint64_t n,
                                           MangoIvBatchSlot* out, uint64_t* out_failed,
                                           MangoError* err);
/* Same with device-resident queries and slots, enqueued without waiting
 * (no failed count). */
MangoStatus mango_gpu_price_table_iv_batch_device(MangoGpuPriceTable* table,
                                                  const MangoInterpSolverConfig* config,
                                                  const MangoIvQuery* d_queries, uint64_t n,
                                                  MangoIvBatchSlot* d_out, MangoError* err);

/* Sensitivities on a frozen grid: value, delta, gamma, theta as in
 * mango_gpu_price_american_batch plus dV/dvolatility, dV/drate,
 * dV/ddividend_yield and dV/dstrike, each a central difference with a
 * relative bump h_rel (0 => 1e-5) of that parameter, all bumped copies
 * priced on the unbumped option's grid (the grid of the reference's
 * estimate_pde_grid moves with volatility and strike, so derivatives through
 * it are discontinuous; this is the reference's bump-and-reprice definition
 * of these Greeks).  One device batch of 9 x n options.  Options with yield
 * curves and discrete dividends are accepted; for a yield curve dV/drate is
 * the derivative along a parallel shift of the zero rates (every log
 * discount ln D(t) moves by -h t).  No counterpart in the reference ABI. */
typedef struct {
  MangoGpuAmericanOut base;
  double vega;
  double rho;
  double dividend_rho;
  double dstrike;
} MangoGpuGreeksOut;
MangoStatus mango_gpu_price_american_greeks_batch(MangoGpuContext* ctx,
                                                  const MangoPricingParams* params, uint64_t n,
                                                  const MangoGpuGrid* grids, uint64_t grid_stride,
                                                  double h_rel, MangoGpuGreeksOut* out,
                                                  uint64_t* out_failed, MangoError* err);

/* Exact discrete sensitivities in one pass: the march of each option's own
 * grid (the reference's plain method with the Rannacher start, as
 * solve_american_option; constant rates and continuous dividends only)
 * differentiated in forward mode with respect to volatility, rate and
 * dividend yield, the active obstacle set frozen; dV/dK from the final
 * spline on the strike-independent grid.  These are the derivatives of the
 * discrete price that the central differences of
 * mango_gpu_price_american_greeks_batch approximate on the same grid.
 * Fills value, delta, vega, rho, dividend_rho, dstrike, status, n_space and
 * n_time; gamma and theta are NaN (mango_gpu_price_american_batch gives
 * them).  Returns MANGO_ERR_VALIDATION only when every option failed; per
 * option statuses otherwise. */
MangoStatus mango_gpu_price_american_tangent_batch(MangoGpuContext* ctx,
                                                   const MangoPricingParams* params, uint64_t n,
                                                   const MangoGpuGrid* grids, uint64_t grid_stride,
                                                   MangoGpuGreeksOut* out, uint64_t* out_failed,
                                                   MangoError* err);

/* mango_gpu_price_american_tangent_batch along volatility alone: value,
 * delta, vega and dstrike (rho and dividend_rho NaN) at about a third of the
 * tangent work; the derivative a Newton step on the implied volatility
 * needs.  No counterpart in the reference ABI. */
MangoStatus mango_gpu_price_american_vega_batch(MangoGpuContext* ctx,
                                                const MangoPricingParams* params, uint64_t n,
                                                const MangoGpuGrid* grids, uint64_t grid_stride,
                                                MangoGpuGreeksOut* out, uint64_t* out_failed,
                                                MangoError* err);

/* Resident batch: the same pipeline as mango_gpu_price_american_batch split
 * so that inputs can stay in device memory across runs (repeat pricing of a
 * book, IV iterations, benchmarking).  _create validates, resolves grids and
 * uploads; _run enqueues the device work (setup, march, outputs) on the
 * context's stream and returns without waiting; _results waits and copies the
 * per-option results to the caller.  No counterpart in the reference ABI. */
typedef struct MangoGpuBatch MangoGpuBatch;
MangoStatus mango_gpu_batch_create(MangoGpuContext* ctx, const MangoPricingParams* params,
                                   uint64_t n, const MangoGpuGrid* grids, uint64_t grid_stride,
                                   const MangoGpuTrbdf2* trbdf2, MangoGpuBatch** out,
                                   MangoError* err);
MangoStatus mango_gpu_batch_run(MangoGpuBatch* batch, MangoError* err);
/* AmericanOptionResult::value_at and the functionals at another spot, the
 * batch counterpart of mango_american_value_at (src/ffi/mango_c_api.h:
 * 148-149; american_option_result.cpp:29-45): for each j, the option in
 * slot slots[j] of a batch that has run, read at spots[j] with its own
 * strike: out4[4j..4j+3] = value, delta, gamma, theta (NaN for a slot that
 * failed or never ran).  Waits for the batch's work. */
MangoStatus mango_gpu_batch_value_at(MangoGpuBatch* batch, const uint64_t* slots,
                                     const double* spots, uint64_t n, double* out4,
                                     MangoError* err);
MangoStatus mango_gpu_batch_results(MangoGpuBatch* batch, MangoGpuAmericanOut* out,
                                    uint64_t* out_failed, MangoError* err);
void mango_gpu_batch_destroy(MangoGpuBatch* batch);
/* Mean device time (CUDA events on the launching stream) of the setup,
 * march and outputs kernels over the runs since the last reset (at most the
 * last 256); waits for the stream.  reset != 0 starts a new window. */
MangoStatus mango_gpu_batch_timings(MangoGpuBatch* batch, int32_t reset, double* prep_ms,
                                    double* march_ms, double* outputs_ms, int64_t* runs,
                                    MangoError* err);

/* Make the context enqueue its work on `stream` (a cudaStream_t of the same
 * device, e.g. a framework's current stream), or on its own stream when
 * NULL.  No counterpart in the reference ABI. */
MangoStatus mango_gpu_context_set_stream(MangoGpuContext* ctx, void* stream);

/* Diagnostic: FP64 FMA throughput of this device in TFLOP/s (an FMA counts
 * 2), measured with independent FMA chains on every SM; the denominator the
 * engine's FP64 roofline fractions are quoted against.  No counterpart in
 * the reference ABI. */
MangoStatus mango_gpu_fp64_probe(MangoGpuContext* ctx, double* tflops, MangoError* err);

/* Batched pricing for callers that cannot allocate device memory (for
 * example code running under an allocator that owns the whole GPU, or with a
 * fixed memory budget).  Same inputs, outputs and per-slot semantics as
 * mango_gpu_price_american_batch, but no context is needed and nothing is
 * allocated: the work runs in one static device array of about 32 MB that
 * every GPU loading this library holds until the process exits.  Limits: at
 * most 4096 options per call and at most 131072 grid rows (sum over
 * 32-option tiles of 32 x the tile's largest n_space); larger requests are
 * rejected with MANGO_ERR_VALIDATION.  The first call on a device looks up
 * the array's address (make it outside any stream capture).  Calls share
 * the array: GPU work of overlapping calls races, so keep them on one stream
 * or synchronise between them.  stream may be NULL (legacy default stream).
 * The calling thread's current device is restored before the call returns.
 * A call rejected or failed as a whole still fills every slot (NaN results,
 * the call's status).  No counterpart in the reference ABI. */
MangoStatus mango_gpu_price_american_batch_noalloc(int32_t device, void* stream,
                                                   const MangoPricingParams* params, uint64_t n,
                                                   const MangoGpuGrid* grids, uint64_t grid_stride,
                                                   const MangoGpuTrbdf2* trbdf2,
                                                   MangoGpuAmericanOut* out, uint64_t* out_failed,
                                                   MangoError* err);

/* Host only (no device needed): the grid the engine would solve `params` on
 * for `grid`, i.e. resolve_grid + GridSpec::generate
 * (src/option/american_option.cpp:54-73, src/pde/core/grid.hpp:364-498).
 * Writes up to `cap` points to x_out and the sizes to *n_space / *n_time. */
MangoStatus mango_gpu_resolve_grid(const MangoPricingParams* params, const MangoGpuGrid* grid,
                                   double* x_out, int64_t cap, int64_t* n_space,
                                   int64_t* n_time, MangoError* err);

/* Timings and work counters of the context's last batch call.  Device
 * times come from CUDA events on the context's stream.  algo_flops counts
 * the reference algorithm's FP64 work: 28 flops per interior row per TR-BDF2
 * step, 18 per row for the Rannacher start, 20 per row for the outputs (an
 * FMA counts 2, a divide 1).  No counterpart in the reference ABI. */
typedef struct {
  double host_prep_ms;
  double h2d_ms;
  double prep_ms;
  double march_ms;
  double outputs_ms;
  double d2h_ms;
  double total_ms;
  double algo_flops;
  double h2d_bytes;
  double d2h_bytes;
  int64_t options;
  int64_t tiles;
  int64_t kernel_launches;
  /* FDM IV: quote evaluations on the coarse grids with the volatility
   * tangent (MANGO_GPU_IV_NEWTON only) and on the quotes' own grids. */
  int64_t iv_evals[2];
} MangoGpuStats;
MangoStatus mango_gpu_last_stats(const MangoGpuContext* ctx, MangoGpuStats* out);

/* Library build information (never NULL). */
const char* mango_gpu_build_info(void);

#ifdef __cplusplus
}  /* extern "C" */
#endif

#ifdef __cplusplus
static_assert(sizeof(MangoPricingParams) == 88, "MangoPricingParams size");
static_assert(offsetof(MangoPricingParams, rate_const) == 40, "rate_const off");
static_assert(offsetof(MangoPricingParams, option_type) == 80, "option_type off");
static_assert(sizeof(MangoIvQuery) == 88, "MangoIvQuery size");
static_assert(sizeof(MangoGpuGrid) == 48, "MangoGpuGrid size");
static_assert(sizeof(MangoGpuAmericanOut) == 48, "MangoGpuAmericanOut size");
static_assert(sizeof(MangoGpuGreeksOut) == 80, "MangoGpuGreeksOut size");
static_assert(sizeof(MangoGpuFitStats) == 96, "MangoGpuFitStats size");
static_assert(sizeof(MangoInterpSolverConfig) == 40, "MangoInterpSolverConfig size");
static_assert(sizeof(MangoIvBatchSlot) == 48, "MangoIvBatchSlot size");
#endif

#endif /* MANGO_GPU_H */
