/*
 * weno_gb300.h -- C ABI of the GB300 (sm_103a) 2D Euler finite-volume step.
 *
 * The entry points replace the reference's PyO3 extension `weno_ext`
 * (weno_ext/src/lib.rs, weno_ext/weno_ext.pyi).  Each function cites the
 * reference interface it replaces.  All arrays are float64 unless stated;
 * strides are in ELEMENTS and may be any (including negative) values.  Device
 * entry points take device pointers and a cudaStream_t passed as void*; they
 * only enqueue work (stream-ordered, asynchronous).  The caller owns every
 * input, output and workspace buffer; the library allocates nothing on these
 * paths (the *_host helpers and the solver own their device buffers).
 *
 * Arithmetic policy (`mode`):
 *   WENO_EXACT  the reference's operation order with no FMA contraction: the
 *               doubles are bit-identical to the Rust core's.
 *   WENO_FAST   the same scheme with fewer FP64 operations and FMA
 *               contraction: reciprocals / square roots within 1-2 ulp
 *               (seeded Newton steps, see weno_fast_math_eval), the WENO
 *               weight normalisations within 2^-41; agrees with WENO_EXACT
 *               to rounding (about 1e-16 relative L1 on a step, within 1e-10
 *               over multi-step runs).
 *
 * Return value: WENO_OK (0) or an error code; weno_last_error() describes the
 * last error of the calling thread.
 */
#ifndef WENO_GB300_H
#define WENO_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  WENO_OK = 0,
  WENO_ERR_SHAPE = 1,     /* array too small / inconsistent shape (the reference panics) */
  WENO_ERR_ARG = 2,       /* invalid argument value */
  WENO_ERR_CUDA = 3,      /* a CUDA call failed */
  WENO_ERR_WORKSPACE = 4, /* workspace missing or too small */
  WENO_ERR_NUMERIC = 5    /* non-finite or non-positive wave speed met by the solver */
};

enum { WENO_EXACT = 0, WENO_FAST = 1 };

/* Riemann solver selector of weno_riemann. */
enum { WENO_HLLC = 0, WENO_HLLE = 1, WENO_BLEND = 2 };

const char* weno_last_error(void);
int weno_abi_version(void);

/* Euler flux of channels 0..3 of q (m, n, c>=4), normal to x (ydir=0) or y.
 * out: dense (m, n, 4).  Replaces flux_x_py / flux_y_py (lib.rs:18-30,
 * utils.rs:74-109). */
int weno_flux(const double* q, int64_t m, int64_t n, int64_t c, int64_t s0, int64_t s1, int64_t s2, double gamma,
              int ydir, int mode, double* out, void* stream);

/* Primitive variables of q (m, n, c>=4): six dense (m, n) planes p, a (sound
 * speed), rho (clamped), u, v, h (total enthalpy).  Replaces con2primi_py
 * (lib.rs:32-38, utils.rs:9-35). */
int weno_con2primi(const double* q, int64_t m, int64_t n, int64_t c, int64_t s0, int64_t s1, int64_t s2,
                   double gamma, int mode, double* p, double* a, double* rho, double* u, double* v, double* h,
                   void* stream);

/* WENO5 reconstruction with the 2-point Gauss-quadrature transverse pass.
 * u: (m, n, c>=4), m, n >= 6.  Outputs q_l, f_l, q_r, f_r dense
 * (m-5, n-6, 4) for ydir=0 and (m-6, n-5, 4) for ydir=1.  cons=0:
 * characteristic projection (weno_x_py / weno_y_py, lib.rs:40-52,
 * weno.rs:367-632); cons=1: component-wise (weno.rs:635-1071).
 * Workspace: weno_reconstruct_workspace(m, n, ydir) bytes. */
size_t weno_reconstruct_workspace(int64_t m, int64_t n, int ydir);
int weno_reconstruct(const double* u, int64_t m, int64_t n, int64_t c, int64_t s0, int64_t s1, int64_t s2,
                     double gamma, int ydir, int cons, int mode, double* q_l, double* f_l, double* q_r, double* f_r,
                     void* ws, size_t ws_bytes, void* stream);

/* Interface flux from dense (m, n, 4) face states and fluxes, in the order of
 * lib.rs (q_l, f_l, q_r, f_r).  kind WENO_HLLC: hllc_x_rs_py / hllc_y_rs_py
 * (lib.rs:54-74); WENO_HLLE: hlle_*_rs_py (lib.rs:76-96); WENO_BLEND: the
 * pressure-gradient blend of hllc_hlle_*_rs_py with force_hlle=false
 * (lib.rs:98-132, riemann.rs:352-486; requires m, n >= 2).  out: dense
 * (m, n, 4).  Workspace: weno_riemann_workspace(m, n, kind) bytes (0 for
 * HLLC/HLLE). */
size_t weno_riemann_workspace(int64_t m, int64_t n, int kind);
int weno_riemann(const double* q_l, const double* f_l, const double* q_r, const double* f_r, int64_t m, int64_t n,
                 double gamma, int ydir, int kind, double jp_lo, double jp_hi, int mode, double* out, void* ws,
                 size_t ws_bytes, void* stream);

/* Residual L(U) = -(dF/dx + dG/dy) of u (m, n, c>=4) with 3 ghost cells on
 * every side; out: dense (m-6, n-6, 4).  force_hlle selects HLLE, otherwise
 * the HLLC/HLLE sensor blend with thresholds (jp_lo, jp_hi) (needs m, n >= 8).
 * cons selects the component-wise reconstruction.  Replaces l_local_py
 * (lib.rs:134-153, riemann.rs:489-541).  Workspace:
 * weno_l_local_workspace(m, n, force_hlle) bytes. */
size_t weno_l_local_workspace(int64_t m, int64_t n, int force_hlle);
int weno_l_local(const double* u, int64_t m, int64_t n, int64_t c, int64_t s0, int64_t s1, int64_t s2, double dx,
                 double gamma, int force_hlle, double jp_lo, double jp_hi, int cons, int mode, double* out, void* ws,
                 size_t ws_bytes, void* stream);

/* weno_l_local without a caller workspace and without any allocation: the
 * scratch is a 64 MiB array owned by the library (a static device array that
 * every GPU loading the library holds until exit).  No counterpart in the
 * reference.  For callers that cannot allocate device memory -- a host that
 * owns all device memory through its own pool, a loop that must not pay
 * cudaMalloc's device-wide synchronisation, code recorded into a CUDA graph.
 * Limit: weno_l_local_workspace(m, n, force_hlle) <= 64 MiB, i.e. about
 * 720 x 720 cells with HLLE and 560 x 560 with the blend (FP64); larger arrays
 * return WENO_ERR_WORKSPACE.  All calls on a device share the array: calls
 * that overlap on the GPU race and must be ordered by the caller.  The first
 * call on a device looks up the array's address (may load the module): make
 * it before any stream capture. */
int weno_l_local_noalloc(const double* u, int64_t m, int64_t n, int64_t c, int64_t s0, int64_t s1, int64_t s2,
                         double dx, double gamma, int force_hlle, double jp_lo, double jp_hi, int cons, int mode,
                         double* out, void* stream);

/* weno_l_local on HOST memory: copies u to the device, runs the residual and
 * copies the (m-6, n-6, 4) result back; synchronous.  u must be C-contiguous
 * (s0 = n*c, s1 = c, s2 = 1).  The library keeps one grow-only device buffer
 * set per device for these calls and serialises them with a lock.  This is the
 * call a Rust/C host of the reference would make in place of l_local_py. */
int weno_l_local_host(const double* u, int64_t m, int64_t n, int64_t c, double dx, double gamma, int force_hlle,
                      double jp_lo, double jp_hi, int cons, int mode, double* out);

/* ------------------------------------------------------------------------
 * Device-resident SSP-RK3 solver: the time loop of Rie_prob_2d_rs.py:169-207,
 * 311-365 (bc_kind WENO_BC_TRANSMISSIVE) or double_mach_reflection.py:97-134,
 * 229-260 (WENO_BC_DMR, unitest.py:207-227) with the state resident in HBM as
 * four conserved planes of (nx+6) x (ny+6).  precision 64 (IEEE double), 48
 * (double-float: pairs of floats with about 48 significant bits, run on the
 * FP32 pipes, several times the FP64 rate on GB300) or 32 (FP32 bulk); dt,
 * the positivity check and the conservation sums are FP64 in every mode.  The
 * solver owns its device memory.
 * ---------------------------------------------------------------------- */
enum { WENO_BC_TRANSMISSIVE = 0, WENO_BC_DMR = 1 };

typedef struct weno_solver weno_solver;

/* weno_eps: the WENO5 smoothness epsilon (<= 0: the reference's 1e-12,
 * weno.rs:223 / utils.rs:3); the density and pressure floors stay 1e-12.
 * Debugging aid: with the environment variable WENO_DEBUG_NAN_FILL=1 the
 * solver's (and weno_batch_create's) internal buffers start as NaN bit
 * patterns instead of zeros, so reads of data a step did not write show up. */
int weno_solver_create(weno_solver** out, int64_t nx, int64_t ny, double dx, double gamma, int precision, int mode,
                       int cons, int force_hlle, double jp_lo, double jp_hi, double cfl, double weno_eps, int bc_kind,
                       int64_t bound, const double* post8, void* stream);
int weno_solver_destroy(weno_solver* s);
/* Load the state from a device array (nx+6, ny+6, c>=4).  With c >= 8 the
 * first step's dt uses the primitive channels 5..7 as the driver does. */
int weno_solver_set_state(weno_solver* s, const double* q, int64_t c, int64_t s0, int64_t s1, int64_t s2);
int weno_solver_set_state_host(weno_solver* s, const double* q, int64_t c);
/* Enqueue nsteps steps.  t_final < 0: step-count mode; otherwise steps stop
 * (as device-side no-ops) once t >= t_final - 1e-12, dt clipped to the time
 * left.  use_graph=1 replays a captured CUDA graph of one step. */
int weno_solver_run(weno_solver* s, int64_t nsteps, double t_final, int use_graph);
/* The driver's (nx+6, ny+6, 8) array: conserved channels and the primitive
 * sync (rho_safe, u, v, p), then the boundary fill on all eight channels. */
int weno_solver_get_state(weno_solver* s, double* out);
int weno_solver_get_state_host(weno_solver* s, double* out);
/* Synchronise and read the clock: simulated time, completed steps and the
 * status bits seen so far (0 ok; 1 a non-finite wave speed; 2 a non-positive
 * recovered density or pressure, checked in FP64 at every CFL reduction). */
int weno_solver_info(weno_solver* s, double* t, int64_t* steps, int* status);
/* FP64 sums of the four conserved variables over the interior (synchronises). */
int weno_solver_totals(weno_solver* s, double* out4);
/* CUDA-event timing of kernel groups, recorded on the solver's stream during
 * runs with use_graph=0.  Classes: 0 CFL reduction + dt, 1 boundary fills,
 * 2 x pass 1, 3 x pass 2, 4 sensor blends, 5 y pass 1, 6 y pass 2,
 * 7 residual + stage combination.  Enabling resets the record; the report
 * synchronises and returns the summed milliseconds and launch-group counts. */
int weno_solver_enable_timing(weno_solver* s, int on);
int weno_solver_timing_report(weno_solver* s, double* ms, int64_t* launches, int nclasses);
/* Number of kernel launches one step enqueues (for launch accounting). */
int weno_solver_launches_per_step(weno_solver* s);

/* ------------------------------------------------------------------------
 * Batched solver: many independent problems of uneven size stepped together.
 * Each solve is the loop of weno_solver_* (same scheme, boundary kinds and
 * per-solve dt = CFL*dx/(max(c+|u|)+1e-16) clipped to its own t_end), with
 * only its interior cells stored in a packed pool of `pool_cells` cells per RK
 * buffer.  One step of ALL active solves is five launches: the per-solve dt,
 * three persistent stage kernels that walk a packed list of TX x TY tiles
 * (tile shape `tile_config`, 0..3) and fuse the whole residual with the stage
 * combination in shared memory, and the clock update; the boundary fill is
 * applied while tiles load.  tile_config 4 is the staged variant: each stage
 * is three launches (pass 1 of every face, pass 2 with the Riemann solvers,
 * residual with the combination) over 16 x 32 tiles, with the face states and
 * fluxes in a device workspace the batch owns (weno_batch_bytes_per_cell), so
 * no face is computed twice -- faster where the arithmetic pipe binds and
 * HBM has room (FP64).  Solves can be
 * added and removed between runs (continuous batching).  Results of a solve
 * do not depend on the other solves in the batch.
 * ---------------------------------------------------------------------- */
typedef struct weno_batch weno_batch;

int weno_batch_tile_config_count(void);
/* Device bytes one pool cell costs in a batch of this precision, flux choice and
 * tile configuration: the three RK pools, plus (staged configuration) the
 * share of the face workspace reserved per cell.  pool_cells x this is about
 * what weno_batch_create allocates. */
double weno_batch_bytes_per_cell(int precision, int force_hlle, int tile_config);
int weno_batch_create(weno_batch** out, int64_t pool_cells, int max_solves, int precision, int mode, int cons,
                      int force_hlle, double gamma, double jp_lo, double jp_hi, double cfl, double weno_eps,
                      int tile_config, void* stream);
int weno_batch_destroy(weno_batch* b);
/* Add a solve from a device array (nx+6, ny+6, c>=4) (ghost cells ignored);
 * t_end < 0 for step-count only; max_steps <= 0 for no cap; cfl <= 0 takes the
 * batch's CFL number.  Returns its slot. */
int weno_batch_add(weno_batch* b, int64_t nx, int64_t ny, double dx, int bc_kind, int64_t bound, const double* post8,
                   double t_end, int64_t max_steps, double cfl, const double* q, int64_t c, int64_t s0, int64_t s1,
                   int64_t s2, int* slot_out);
int weno_batch_remove(weno_batch* b, int slot);
/* Enqueue nsteps steps of every active solve (finished solves are no-ops). */
int weno_batch_run(weno_batch* b, int64_t nsteps, int use_graph);
/* The driver's (nx+6, ny+6, 8) array of one solve (device pointer); synchronises. */
int weno_batch_get_state(weno_batch* b, int slot, double* out);
/* status: WENO_OK, WENO_ERR_NUMERIC (a non-finite wave speed stopped the solve) or
 * WENO_ERR_CUDA (a tile's staging copy did not complete within its time limit). */
int weno_batch_info(weno_batch* b, int slot, double* t, int64_t* steps, int* active, int* status);
/* Synchronise and copy every slot's active flag, time and step count (arrays of max_solves). */
int weno_batch_poll(weno_batch* b, int* active, double* t, int64_t* steps);
int weno_batch_stats(weno_batch* b, int64_t* ntiles, int64_t* free_cells, int* launches_per_step);
/* Test hook of the bounded staging waits (no counterpart in the reference).
 * From the next run on, the TMA copy of packed tile `tile` is not issued, so
 * its wait gives up after wait_ns nanoseconds; the CTA then flags the solve of
 * that tile and of every later tile it would have walked (status
 * WENO_ERR_CUDA, and the solve stops at the end of the step) and leaves.  The
 * tile list holds each added solve's tiles in slot order, rows then columns;
 * grid > 0 fixes the stage kernels' persistent grid (CTA k walks tiles k,
 * k + grid, ...).  tile < 0 restores normal operation (1 s waits, grid from
 * occupancy).  No copy is left in flight and no GPU fault is involved.  The
 * staged configuration (tile_config 4) stages nothing by TMA: there only the
 * fixed grid applies. */
int weno_batch_debug_skip_copy(weno_batch* b, int tile, int64_t wait_ns, int grid);

/* ------------------------------------------------------------------------
 * Device generators of the seeded initial data, written straight into a
 * device array (nx+6, ny+6, 8) in the drivers' layout (no counterpart in the
 * reference's extension; they restate Rie_prob_2d_rs.py:213-263 and
 * unitest.py:169-205 with seeded states).
 * ---------------------------------------------------------------------- */
/* Four quadrants split at padded indices si, sj; prim16 = 4 x (rho, u, v, p)
 * for (i<si, j<sj), (i>=si, j<sj), (i<si, j>=sj), (i>=si, j>=sj). */
int weno_init_quadrant(double* out, int64_t nx, int64_t ny, int64_t si, int64_t sj, const double* prim16,
                       double gamma, void* stream);
/* Planar shock at angle theta through (x0, 0) on [0,lx]x[0,ly], Mach `mach`
 * into gas at rest (rho1, p1), post-shock state from Rankine-Hugoniot, then
 * the oblique-shock boundary; returns the boundary's bound row and 8-channel
 * inflow vector for weno_solver_create / weno_batch_add. */
int weno_init_oblique_shock(double* out, int64_t nx, int64_t ny, double lx, double ly, double x0, double mach,
                            double theta, double rho1, double p1, double gamma, int64_t* bound_out, double* post8_out,
                            void* stream);

/* Rie_prob_2d_rs.py:37-120 apply_bc_reflecting, in place on a device array
 * (n, n, 8) in the drivers' layout: edge ghosts mirror the interior with the
 * wall-normal momentum and velocity negated, then the four 3x3 corner blocks
 * are taken from interior blocks with both pairs negated, as the reference
 * does.  The reference indexes axis 0 with the axis-1 extent, so only square
 * arrays (n >= 9) with 8 channels are accepted (WENO_ERR_SHAPE otherwise). */
int weno_bc_reflecting(double* q, int64_t m, int64_t n, int64_t c, int64_t s0, int64_t s1, int64_t s2, void* stream);
/* unitest.py:169-205 init_refac, the double-Mach set-up of
 * double_mach_reflection.py, into a dense device array (nx+6, ny+6, 8): gas at
 * rest (1.4, 0, 0, 1), the post-shock state (8, 4.125, -7.1447, 116.5) above
 * the line y = sqrt(3) x - sqrt(3)/6 rounded to cell rows as the reference
 * rounds them, then apply_bc_refac.  Returns the boundary's `bound` row; the
 * inflow vector is the driver's literal (weno_solver_create with post8 NULL). */
int weno_init_refac(double* out, int64_t nx, int64_t ny, double lx, double ly, double gamma, int64_t* bound_out,
                    void* stream);

/* Diagnostics: measured FP64 FMA (TFLOP/s), FP64 divide (per s) and FP32 FMA
 * (TFLOP/s) throughput of the current device -- the compute-roofline
 * denominators, with no counterpart in the reference. */
int weno_probe_rates(double* fp64_tflops, double* fp64_div_per_s, double* fp32_tflops, void* stream);

/* Diagnostics: the FAST-mode FP64 reciprocal, reciprocal square root and
 * square root (an FP32 hardware seed and one third-order Newton step; within
 * 1, 1 and 2 ulp) and the second-order reciprocal (relative error below
 * 2^-41) of n device doubles x, written to the device array out as
 * [1/x | 1/sqrt(x) | sqrt(x) | 1/x second order] (4n doubles), for tests of
 * their error bounds. */
int weno_fast_math_eval(const double* x, double* out, int64_t n, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* WENO_GB300_H */
