/*
 * hacc_pm.h -- C ABI of the long-range particle-mesh (PM) kick on one GPU.
 *
 * The other half of HACC's TreePM step next to the short-range kick of
 * hacc_sr.h: CIC deposit of the particles, spectral Poisson solve with the
 * quiet solver's filtered 6th-order Green's function and 4th-order gradient,
 * inverse CIC interpolation of the three gradient components and the
 * velocity kick.  Runs on an hsr_ctx (its stream and device).
 *
 * Reference interfaces replaced (paths inside the reference project):
 *   hsr_pm_kick    <- map2_poisson_forward + map2_poisson_backward_gradient
 *                     src/simulation/mc3.cxx:304-374, i.e. Particles::cic
 *                     (src/cpu/Particles.cxx:589-643), fft_copy_arr_forward
 *                     (mc3.cxx:206-225), SolverQuiet::forward_solve and
 *                     backward_solve_gradient (src/dfft/solver.hpp:91-160,
 *                     506-547, 707-820), fft_copy_arr_backward (mc3.cxx:
 *                     228-245), GridExchange::exchangeGrid and
 *                     Particles::inverse_cic (Particles.cxx:647-714) for the
 *                     three components
 *   hsr_treepm_step <- one pass of the time-step loop of
 *                     src/simulation/driver_hires.cxx:320-447: PM half kick,
 *                     Particles::subCycle, PM kick
 *   hsr_pm_fields  <- the grids those calls leave behind: the alive block of
 *                     the density after cic + fft_copy_arr_forward and of
 *                     each gradient component after backward_solve_gradient +
 *                     fft_copy_arr_backward
 *
 * One GPU holds the whole periodic box: the reference's run on one rank.
 * Particle coordinates are the rank's local grid coordinates (Particles with
 * m_coords_localQ == 1): the alive block is [ngo, ngo + ng) per axis and
 * overloaded copies may lie anywhere in the local grid [0, ng + 2 ngo + 1).
 * As in the reference, deposits outside the alive block are dropped and the
 * interpolation reads each local cell's periodic image (cells outside the
 * local grid read 0).  Requires even ng >= 2 and 0 <= ngo < ng.
 */
#ifndef HACC_PM_H
#define HACC_PM_H

#include <stdint.h>

#include "hacc_sr.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Arithmetic of the transforms and the spectra.  F64: double, as the
 * reference's FFTW solve (complex_t double); F32: single precision (half the
 * HBM traffic and none of the FP64 pipe, at single-precision rounding of the
 * gradient fields). */
enum { HSR_PM_F64 = 0, HSR_PM_F32 = 1 };

typedef struct hsr_pm_params {
  int32_t ng;         /* grid cells per side of the periodic box (Domain::m_ng) */
  int32_t ngo;        /* overload width in cells (Domain::ng_overload())        */
  float gpscal;       /* Particles::m_gpscal: each particle deposits gpscal^3   */
  float fscal;        /* TimeStepper::fscal()                                   */
  float tau;          /* inverse_cic's tau: TimeStepper::tau() * stepFraction   */
  int32_t precision;  /* HSR_PM_F64 or HSR_PM_F32                               */
} hsr_pm_params;

typedef struct hsr_pm_stats {
  double t_total_ms;        /* wall time of the call                        */
  double t_h2d_ms;          /* host arrays: copies to the device (events)   */
  double t_deposit_ms;      /* CIC deposit (CUDA events)                    */
  double t_solve_ms;        /* transforms, spectra and gradient grids       */
  double t_interp_ms;       /* inverse CIC and kick                         */
  double t_d2h_ms;          /* host arrays: velocities back (events)        */
  int64_t h2d_bytes, d2h_bytes;
  int64_t kernel_launches;  /* this library's kernels                       */
  int64_t fft_execs;        /* cuFFT executions (one forward, one batched
                               inverse of the three components)             */
} hsr_pm_stats;

/* The PM kick: v_d += fscal * tau * (inverse CIC of the d-th gradient
 * component of the solved potential), d = x, y, z, for the n particles.
 * Positions are read only.  mem: HSR_MEM_HOST or HSR_MEM_DEVICE (device
 * pointers on the context's device).  Synchronous.  The plans and the Green's
 * function are made on the first call for an (ng, precision) and kept.
 * Replaces map2_poisson_forward + map2_poisson_backward_gradient and the
 * inverse CIC kick (src/simulation/mc3.cxx:304-374). */
hsr_status hsr_pm_kick(hsr_ctx *ctx, const hsr_pm_params *p, int64_t n, const float *x,
                       const float *y, const float *z, float *vx, float *vy, float *vz,
                       int32_t mem);

/* The density (ng^3 floats) and the three gradient components (3 x ng^3
 * floats, component-major) of the alive block for these positions, each
 * grid with x the slowest and z the fastest index, like the reference's
 * (i*ng + j)*ng + k.  Either output may be NULL.  Same `mem` rule as
 * hsr_pm_kick, for all five pointers.  The grids the reference's
 * map2_poisson_forward and map2_poisson_backward_gradient leave in the
 * solver (src/simulation/mc3.cxx:304-374). */
hsr_status hsr_pm_fields(hsr_ctx *ctx, const hsr_pm_params *p, int64_t n, const float *x,
                         const float *y, const float *z, float *rho, float *grad, int32_t mem);

hsr_status hsr_pm_get_stats(const hsr_ctx *ctx, hsr_pm_stats *st);

/* Vector-Jacobian product of the PM kick with respect to the positions: for
 * the velocity change dv = fscal tau F(x) that hsr_pm_kick adds and a
 * cotangent vbar of it, writes xbar = (d dv / d x)^T vbar (n entries each,
 * caller's order).  The density, the solve and both halves of the chain rule
 * run on the device: the interpolation's derivative at each particle and,
 * through the density, the cotangents deposited by CIC, the transposed solve
 * (the conjugate spectrum) and the CIC derivative at each depositor.  CIC
 * weights are piecewise linear: the product is the derivative away from cell
 * faces.  Same `mem` rule as hsr_pm_kick for all nine arrays.  No
 * counterpart in the reference (differentiation is new in this library). */
hsr_status hsr_pm_vjp(hsr_ctx *ctx, const hsr_pm_params *p, int64_t n, const float *x,
                      const float *y, const float *z, const float *vbx, const float *vby,
                      const float *vbz, float *xbx, float *xby, float *xbz, int32_t mem);

/* One time step of HACC's TreePM loop on the device (the body of the step
 * loop in src/simulation/driver_hires.cxx:320-447 on one rank):
 *   open   if pm_open.tau != 0: the PM kick with pm_open (the loop's half
 *          kick, stepFraction 0.5, at the step's start; tau == 0 stands for
 *          doHalfKick == 0 and skips it),
 *   sub    hsr_subcycle with `sub` (the stepper at mid-step: map1's and
 *          map2's arguments),
 *   close  the PM kick with pm_close (at the step's end; stepFraction 1, or
 *          0.5 on the last step).
 * The PM kicks see all n particles (the reference's cic and inverse_cic run
 * over every local particle, overloaded ones included); the sub-cycle
 * resorts them and kicks the in-box ones, as hsr_subcycle does.  The arrays
 * stay on the device for the whole step.  hsr_get_stats reports the
 * sub-cycle, hsr_pm_get_stats the two PM kicks summed (t_total_ms: the whole
 * step).  *n_inbox receives the in-box count of the last resort. */
typedef struct hsr_treepm_params {
  hsr_subcycle_params sub;
  hsr_pm_params pm_open;
  hsr_pm_params pm_close;
} hsr_treepm_params;

hsr_status hsr_treepm_step(hsr_ctx *ctx, const hsr_treepm_params *tp, int64_t n, float *x,
                           float *y, float *z, float *vx, float *vy, float *vz, float *mass,
                           float *phi, int64_t *id, uint16_t *mask, int32_t mem,
                           int64_t *n_inbox);

/* SolverQuiet's 1-D tables (src/dfft/solver.hpp:726-790) as this library
 * computes them on the host in double: the filter W(k), the denominator term
 * a0 + a1 cos + a2 cos 2 + a3 cos 4 and the gradient factor b1 sin + b2 sin 2,
 * each ng entries indexed by wave number (no device needed). */
hsr_status hsr_pm_tables(int32_t ng, double *filter, double *denom, double *gradient);

#ifdef __cplusplus
}
#endif
#endif /* HACC_PM_H */
