// pm.cuh -- the long-range particle-mesh kick on one GPU: CIC deposit,
// spectral Poisson solve with the reference's quiet Green's function and
// 4th-order gradient, inverse CIC kick.
//
// Reference (paths inside the reference project):
//   map2_poisson_forward / map2_poisson_backward_gradient
//       src/simulation/mc3.cxx:304-374
//   Particles::cic, Particles::inverse_cic        src/cpu/Particles.cxx:589-714
//   fft_copy_arr_forward / fft_copy_arr_backward  src/simulation/mc3.cxx:206-245
//   SolverQuiet::initialize_greens_function, SolverBase::kspace_solve_gradient,
//   forward_solve / backward_solve_gradient
//       src/dfft/solver.hpp:91-160, 506-547, 707-820
//   GridExchange (dead zones ngo below, ngo + 1 above the alive block)
//       src/halo_finder/GridExchange.cxx:68-99, 139-470;
//       src/simulation/driver_hires.cxx:258
//
// The whole periodic box lives on one GPU, so the reference's distributed
// pieces collapse:
//   * the rank's local grid (ng + 2 ngo + 1 cells a side, Domain.cxx:69) is
//     never stored.  A deposit into a cell outside the alive block is dropped
//     (fft_copy_arr_forward copies only the alive block), and a read of a
//     cell of the local grid is a read of its periodic image in the alive
//     block (what GridExchange::exchangeGrid puts in every dead cell on one
//     rank); cells outside the local grid read 0 (array_index's safe slot);
//   * the distributed complex FFT of a real field becomes a real-to-complex
//     transform on the half spectrum (cuFFT).  The reference keeps the real
//     part of a complex inverse transform, which is the inverse transform of
//     the spectrum's Hermitian part.  The Green's function is even and the
//     gradient factor odd in k, except on the planes k_a = 0 (where the
//     reference sets the factor to 1) and k_a = ng/2 of the gradient axis a,
//     where both k and -k carry the same factor: there the spectrum is
//     anti-Hermitian and its real part is zero, so the factor is 0 on those
//     planes and the half-spectrum inverse gives the reference's real part;
//   * the three gradient components are solved in one batched inverse
//     transform and interpolated in one pass over the particles (the
//     reference's three inverse_cic passes update different components from
//     the same positions).
#pragma once

#include <cstdint>
#include <string>

#include <cuda_runtime.h>
#include <cufft.h>

namespace hsr_pm {

enum { PREC_F64 = 0, PREC_F32 = 1 };

struct Params {
  int ng = 0;        // alive cells per side (the whole box)
  int ngo = 0;       // overload cells below the alive block
  float gpscal = 1;  // deposit per particle: gpscal^3
  float fscal = 1;
  float tau = 0;
  int prec = PREC_F64;
};

struct Timing {
  double deposit_ms = 0, solve_ms = 0, interp_ms = 0;
  int64_t launches = 0;   // this library's kernels
  int64_t fft_execs = 0;  // cuFFT executions
};

// Plans, Green's function and grids for one (ng, precision); rebuilt when
// either changes.  Everything runs on the stream given to each call.
class Solver {
 public:
  ~Solver();
  // Plans and tables for ng and prec (no-op when they are current).
  bool prepare(int ng, int prec, cudaStream_t s, std::string *err);
  // Density of the alive block (cic + fft_copy_arr_forward), into rho_ (ng^3
  // floats, x slowest).
  bool deposit(const Params &p, int64_t n, const float *x, const float *y, const float *z,
               cudaStream_t s, std::string *err);
  // Forward transform and the three gradient fields into grad_ (ng^3 float4:
  // components x, y, z, 0), i.e. the alive block after each
  // backward_solve_gradient + fft_copy_arr_backward.
  bool solve(cudaStream_t s, std::string *err);
  // v_d += (sum_corners grad_d w) * fscal * tau for the three components.
  bool interp(const Params &p, int64_t n, const float *x, const float *y, const float *z,
              float *vx, float *vy, float *vz, cudaStream_t s, std::string *err);
  // Copies rho_ (ng^3) and the three gradient components (3 x ng^3, planar).
  bool export_fields(float *rho, float *grad, bool to_host, cudaStream_t s, std::string *err);

  // The kick's vector-Jacobian product for positions x and the cotangent
  // vbar of its velocity change: xbar = (d dv / d x)^T vbar, written to xb*
  // (recomputes the deposit and the solve of these positions first).
  bool vjp(const Params &p, int64_t n, const float *x, const float *y, const float *z,
           const float *vbx, const float *vby, const float *vbz, float *xbx, float *xby,
           float *xbz, cudaStream_t s, std::string *err);

  // Deposit, solve and interpolation with event timings (the context's
  // events ev[0..3] on stream s).
  bool kick(const Params &p, int64_t n, const float *x, const float *y, const float *z, float *vx,
            float *vy, float *vz, cudaStream_t s, cudaEvent_t *ev, Timing *t, std::string *err);

  int ng() const { return ng_; }
  int64_t launches = 0, fft_execs = 0;

 private:
  void release();
  int ng_ = 0, prec_ = -1;
  cufftHandle fwd_ = 0, inv_ = 0;
  bool have_fwd_ = false, have_inv_ = false;
  // adjoint: batched forward of the three deposited cotangent fields, single
  // inverse of the combined spectrum (made on the first vjp)
  cufftHandle fwd3_ = 0, inv1_ = 0;
  bool have_fwd3_ = false, have_inv1_ = false;
  float *adj_ = nullptr;     // 3 x ng^3: deposited cotangents (float atomics)
  bool prepare_vjp(std::string *err);
  float *rho_ = nullptr;     // ng^3
  void *real_ = nullptr;     // ng^3 real (T): transform input (double only)
  void *spec_ = nullptr;     // ng^2 (ng/2+1) complex (T)
  void *gspec_ = nullptr;    // 3 x ng^2 (ng/2+1) complex (T)
  void *greal_ = nullptr;    // 3 x ng^3 real (T)
  void *green_ = nullptr;    // ng^2 (ng/2+1) real (T)
  void *gtab_ = nullptr;     // ng real (T): gradient factor per wave index
  float4 *grad_ = nullptr;   // ng^3
};

// The reference's 1-D tables of SolverQuiet::initialize_greens_function in
// double (host): filter W(k), the denominator term a0 + a1 cos + a2 cos2 +
// a3 cos4 and the gradient factor b1 sin + b2 sin2, per wave index.
void quiet_tables(int ng, double *filter, double *denom, double *gradient);

}  // namespace hsr_pm
